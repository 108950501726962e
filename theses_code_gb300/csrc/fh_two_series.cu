// fh_two_series.cu -- two-series approximation of the 2D history sums
// (TG_solver_ with dt_alg 4, psi = t; fr_d_t_g_2d.cpp:246-745 and the Om1
// branch 3438-3469).
//
// Per point the sum S(x) = sum_r g(x, r) F[r], g(x, r) = (x - r + a)^A -
// (x - r + b)^A, A = 1 - alpha, F[r] = C^r - C^(r-1), is carried by "long"
// approximations sum_k c_k x^(A-k) (valid for x >= min) and "short" ones
// sum_k c_k (x - b0)^k (valid for min <= x <= max), whose coefficients are
// linear in F.  Each step evaluates the sum at x = j from the approximations
// and the newest layer, then folds the newest F into them, creating,
// splitting and retiring approximations (calc_va, 477-745).  The ranges,
// term counts and splits depend on A, a, b and the step only, never on F, so
// the whole bookkeeping runs once on the host, when the scheme is enabled,
// for every step of the solve: it emits per step a list of items, each an
// evaluation (coefficient slot, basis values), a copy between slots, or the
// addition / initialisation of a slot with the newest layer's coefficients
// ak_k (F g_k).  The device keeps the coefficients of every live slot per
// point (slot-major, coalesced over points) and runs one step's items in
// order, one point per thread, in the reference's operation order (no
// contraction into FMAs), so its sums follow the reference's roundings.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "fh_common.cuh"
#include "fh_internal.h"
#include "fh_two_series.h"

namespace {

constexpr int kAK = 10;     // terms of a new approximation (AK)
constexpr int kMaxAK = 20;  // largest term count (MAXAK)
constexpr double kApproxEps = 1e-7, kEps = 1e-9;

enum : int { kEval = 0, kCopy = 1, kAddIa = 2, kAddIbk = 3, kInitIa = 4, kInitIbk = 5 };

// prod_{i=1}^{n-1} (A - i + 1) / i in the reference's order
double ak_of(double A, int n) {
  double ak = 1;
  for (int i = 1; i < n; i++) ak *= (A - i + 1) / i;
  return ak;
}
// ia_mini (fr_d_t_g_2d.cpp:255-266), integer time grid
double ia_mini(double A, double r, int nterms, double a, double b) {
  const double ak = ak_of(A, nterms);
  return pow(fabs(ak * (pow(a - r, (double)nterms) - pow(b - r, (double)nterms)) / kApproxEps), 1.0 / (nterms - A));
}
// ibk_i2 (fr_d_t_g_2d.cpp:337-371), integer time grid
double ibk_i2(double A, double r, double b, int nterms, double a, double c) {
  const double ak = ak_of(A, nterms);
  if (fabs(b - r) < 1e-10) return pow(fabs(kApproxEps / ak), 1.0 / nterms);
  const double p1 = pow((a + b - r), A) / pow((a + b - r), nterms);
  const double p2 = pow((c + b - r), A) / pow((c + b - r), nterms);
  return pow(fabs(kApproxEps / (ak * (p1 - p2))), 1.0 / nterms);
}

struct LongApx {
  double min;
  int nterms, slot;
};
struct ShortApx {
  double min, max, b;
  int nterms, old, slot;
};

// The bookkeeping of one direction (offsets a, b of g), emitting items.
struct Planner {
  double A, a, b;
  std::vector<LongApx> ia;
  std::vector<ShortApx> ibk;
  std::vector<int> free_slots;
  int nslots = 0;
  std::vector<int4> items;     // {kind | nt << 8, slot, src, coefficient offset}
  std::vector<double> coef;

  int alloc() {
    if (!free_slots.empty()) {
      const int s = *std::min_element(free_slots.begin(), free_slots.end());
      free_slots.erase(std::find(free_slots.begin(), free_slots.end(), s));
      return s;
    }
    return nslots++;
  }
  void release(int s) { free_slots.push_back(s); }
  void item(int kind, int nt, int slot, int src, int off) { items.push_back(make_int4(kind | (nt << 8), slot, src, off)); }

  // coefficients of the newest layer r as ak_k, g_k pairs (k < nt):
  // long: g_k = (a - r)^k - (b - r)^k, k >= 1 (c_0 = 0);
  // short around b0: g_k = (a + b0 - r)^(A-k) - (b + b0 - r)^(A-k)
  int layer_coefs(bool is_long, int r, double b0, int nt) {
    const int off = (int)coef.size();
    coef.resize(coef.size() + 2 * (size_t)nt, 0.0);
    double ak = 1;
    for (int i = is_long ? 1 : 0; i < nt; i++) {
      if (i != 0) ak *= (A - i + 1) / i;
      coef[off + i] = ak;
      coef[off + nt + i] = is_long ? (pow(a - (double)r, (double)i) - pow(b - (double)r, (double)i))
                                   : (pow(a + b0 - (double)r, A - (double)i) - pow(b + b0 - (double)r, A - (double)i));
    }
    return off;
  }
  // a new short approximation of layer r around b0 (min given, or from i2)
  ShortApx new_short(int r, double rmax, double b0, double min_given, int nt) {
    ShortApx q;
    q.b = b0;
    q.min = min_given != -1 ? min_given : b0 - floor(ibk_i2(A, rmax, b0, nt, a, b));
    q.max = b0;
    q.nterms = nt;
    q.old = 0;
    q.slot = -1;
    return q;
  }
  void push_short_init(ShortApx q, int r) {
    q.slot = alloc();
    item(kInitIbk, q.nterms, q.slot, 0, layer_coefs(false, r, q.b, q.nterms));
    ibk.push_back(q);
  }
  void erase_short(int j) {
    release(ibk[j].slot);
    ibk.erase(ibk.begin() + j);
  }
  // series of short approximations of layer r covering [rr, upto]
  double series(int r, double rr, double r2, double upto, bool cap, bool cmp_ceil) {
    double bb0 = rr, bb = rr;
    do {
      bb = rr + 1;
      do {
        bb0 = bb;
        bb = rr + ibk_i2(A, r2, bb, kAK, a, b) + 1;
      } while ((bb - bb0) > kEps);
      if (!std::isfinite(bb)) {
        bb = bb0;
        if (!std::isfinite(bb)) bb = rr;
      }
      ShortApx q = new_short(r, r + 1, floor(bb), rr, kAK);
      rr = floor(bb) + 1;
      if (cap && floor(bb) > upto) q.max = upto;
      push_short_init(q, r);
    } while (floor(bb) < (cmp_ceil ? ceil(upto) : upto));
    return rr;
  }

  // calc_va for block `block` (x = block + 1): evaluation items, then the
  // updates with layer r = block + 1
  void step(int block) {
    const int r = block + 1;
    const double rmax = (double)(block + 2);
    const int rmaxidx = block + 2;
    const double ii = r;
    for (auto &q : ia)
      if (ii >= q.min) {
        const int off = (int)coef.size();
        for (int i = 0; i < q.nterms; i++) coef.push_back(pow(ii, A - (double)i));
        item(kEval, q.nterms, q.slot, 0, off);
      }
    for (auto &q : ibk)
      if ((ii >= q.min) && (ii <= q.max)) {
        const int off = (int)coef.size();
        double xbk = 1;
        for (int i = 0; i < q.nterms; i++) {
          coef.push_back(xbk);
          xbk *= (ii - q.b);
        }
        item(kEval, q.nterms, q.slot, 0, off);
      }
    // 1) retire
    for (int j = 0; j < (int)ibk.size(); j++)
      if (ibk[j].max < rmax) {
        erase_short(j);
        j--;
      }
    // 2) fold the layer into the short approximations ahead of it; split
    int ss = (int)ibk.size();
    for (int j = 0; j < ss; j++)
      if (ibk[j].min >= rmax && ibk[j].old == 0) {
        bool spl = false;
        ShortApx i2{};
        ShortApx add = new_short(r, rmax, ibk[j].b, -1.0, kAK);
        const double add_min = add.min;
        if (add.min > ibk[j].min) {
          int t;
          for (t = kAK; t < kMaxAK; t++)
            if ((ibk[j].b - ibk_i2(A, rmaxidx, ibk[j].b, t, a, b)) < ibk[j].min) break;
          if (t == kMaxAK)
            spl = true;
          else
            add = new_short(r, rmax, ibk[j].b, -1.0, t);
          if (spl) {
            i2 = ibk[j];
            i2.slot = alloc();
            item(kCopy, kMaxAK, i2.slot, ibk[j].slot, 0);
          }
        }
        item(kAddIbk, add.nterms, ibk[j].slot, 0, layer_coefs(false, r, ibk[j].b, add.nterms));
        if (ibk[j].nterms < add.nterms) ibk[j].nterms = add.nterms;
        if (spl && add_min > ibk[j].min) {
          i2.max = ceil(add_min);
          ibk[j].min = i2.max + 1;
          i2.old = 1;
          if (ibk[j].min > ibk[j].max) {
            i2.max = ibk[j].max;
            erase_short(j);
            j--;
            ss--;
          }
          ibk.push_back(i2);
          series(r, i2.min, i2.min, i2.max, true, false);
        }
      }
    // 3) the newest approximation straddling rmax gets this layer's series
    double bm1 = -1;
    for (auto &q : ibk)
      if (q.max >= rmax && q.min < rmax && q.max > bm1 && q.old == 0) {
        bm1 = q.max;
        q.old = 1;
      }
    if (bm1 != -1) {
      for (auto &q : ibk)
        if (q.max < bm1) q.old = 1;
      series(r, rmax, rmaxidx, bm1, true, false);
    }
    // 4) the long approximation of this layer joins the newest one
    double bia_min = ceil(ia_mini(A, rmax, kAK, a, b));
    if (!std::isfinite(bia_min)) bia_min = rmax;
    if (!ia.empty() && bia_min < ia.back().min) {
      item(kAddIa, kAK, ia.back().slot, 0, layer_coefs(true, r, 0.0, kAK));
      if (ia.back().nterms < kAK) ia.back().nterms = kAK;
      return;
    }
    // 5) or short approximations bridge to its minimum and it is added
    bm1 = rmax;
    for (auto &q : ibk)
      if ((q.max + 1) > bm1) bm1 = q.max + 1;
    // the long approximation's coefficients are those of layer r, whatever
    // its final minimum; its slot is initialised before the bridge's
    LongApx q;
    q.slot = alloc();
    q.nterms = kAK;
    item(kInitIa, kAK, q.slot, 0, layer_coefs(true, r, 0.0, kAK));
    q.min = series(r, bm1, rmaxidx, bia_min, false, true);
    ia.push_back(q);
  }
};

// One step of both directions (blockIdx.y: 0 = x sums, 1 = y sums): the
// evaluation items span[dir].x .. .y, the sum with the newest layer written to
// part[dir][p] (scaled by sc = Da tau^A / A), then the updates .y .. .z.
__global__ void __launch_bounds__(256) k_tg_two_series(const double *__restrict__ Dn, int df, long long P,
                                                       const int4 *__restrict__ items, const int4 *__restrict__ span,
                                                       const double *__restrict__ coef, double *__restrict__ cbuf,
                                                       long long nslots, double dterm_x, double dterm_y, double sc,
                                                       double *__restrict__ part) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int dir = blockIdx.y;
  double F;
  if (df) {
    const float2 v = reinterpret_cast<const float2 *>(Dn)[p];
    F = (double)v.x + (double)v.y;
  } else {
    F = Dn[p];
  }
  double *c = cbuf + (long long)dir * nslots * kMaxAK * P;  // slot s, term k: c[(s kMaxAK + k) P + p]
  auto at = [&](int s, int k) -> double & { return c[((long long)s * kMaxAK + k) * P + p]; };
  const int4 sp = span[dir];
  double V = 0.0;
  for (int it = sp.x; it < sp.y; ++it) {  // long approximations, then short ones, in list order
    const int4 q = __ldg(items + it);
    const int nt = q.x >> 8;
    const double *cf = coef + q.w;
    double r = 0.0;
    for (int i = 0; i < nt; ++i) r = __dadd_rn(r, __dmul_rn(at(q.y, i), __ldg(cf + i)));
    V = __dadd_rn(V, r);
  }
  // the newest layer directly: ((0 + a)^A - (0 + b)^A) F
  part[(long long)dir * P + p] = __dmul_rn(__dadd_rn(V, __dmul_rn(dir ? dterm_y : dterm_x, F)), sc);
  for (int it = sp.y; it < sp.z; ++it) {
    const int4 q = __ldg(items + it);
    const int kind = q.x & 0xff, nt = q.x >> 8;
    const double *cf = coef + q.w;
    if (kind == kCopy) {
      for (int i = 0; i < kMaxAK; ++i) at(q.y, i) = at(q.z, i);
    } else {
      const bool add = kind == kAddIa || kind == kAddIbk;
      const int i0 = (kind == kAddIa || kind == kInitIa) ? 1 : 0;
      if (!add) {
        for (int i = 0; i < i0; ++i) at(q.y, i) = 0.0;
        for (int i = nt; i < kMaxAK; ++i) at(q.y, i) = 0.0;
      }
      for (int i = i0; i < nt; ++i) {
        const double v = __dmul_rn(__ldg(cf + i), __dmul_rn(F, __ldg(cf + nt + i)));
        at(q.y, i) = add ? __dadd_rn(at(q.y, i), v) : v;
      }
    }
  }
}

}  // namespace

struct fh_ta {
  int max_steps = 0;
  int nslots[2] = {0, 0};
  // per step j: items of the x sums span[2j] = {first, first update, end}, of
  // the y sums span[2j + 1]
  double dterm[2] = {0.0, 0.0};
  fh_dbuf items, spans, coef, cbuf;
};

namespace {
// The tables of every step 1 .. max_steps - 1 of both directions.
void ta_plan(double alpha, int max_steps, std::vector<int4> &items, std::vector<double> &coef,
             std::vector<int4> &span, int nslots[2], double dterm[2]) {
  const double A = 1.0 - alpha;
  const double offs[2][2] = {{1.5, 0.5}, {2.0, 1.0}};  // x sums (Happ1), y sums (Happ2)
  items.clear();
  coef.clear();
  span.assign((size_t)2 * (max_steps + 1), make_int4(0, 0, 0, 0));
  Planner pl[2];
  for (int d = 0; d < 2; ++d) {
    pl[d].A = A;
    pl[d].a = offs[d][0];
    pl[d].b = offs[d][1];
    dterm[d] = pow(0.0 + offs[d][0], A) - pow(0.0 + offs[d][1], A);
  }
  // step j >= 1 evaluates at x = j and folds layer j in (block j - 1)
  for (int j = 1; j < max_steps; ++j)
    for (int d = 0; d < 2; ++d) {
      Planner &q = pl[d];
      q.step(j - 1);
      // into the shared tables, coefficient offsets rebased; the evaluation
      // items come first
      const int ib = (int)items.size(), cb = (int)coef.size();
      int ne = 0;
      while (ne < (int)q.items.size() && (q.items[ne].x & 0xff) == kEval) ++ne;
      for (int4 v : q.items) {
        v.w += cb;
        items.push_back(v);
      }
      coef.insert(coef.end(), q.coef.begin(), q.coef.end());
      q.coef.clear();
      q.items.clear();
      span[2 * j + d] = make_int4(ib, ib + ne, (int)items.size(), 0);
    }
  nslots[0] = pl[0].nslots;
  nslots[1] = pl[1].nslots;
}
}  // namespace

int fh_ta_create(fh_ctx *ctx, double alpha, int max_steps, long long P, fh_ta **out) {
  *out = nullptr;
  fh_ta *t = new fh_ta;
  t->max_steps = max_steps;
  std::vector<int4> items, span;
  std::vector<double> coef;
  ta_plan(alpha, max_steps, items, coef, span, t->nslots, t->dterm);
  const long long ns = std::max(t->nslots[0], t->nslots[1]);
  int rc;
  if ((rc = fh_alloc(ctx, t->items, sizeof(int4) * std::max<size_t>(items.size(), 1), false)) ||
      (rc = fh_alloc(ctx, t->spans, sizeof(int4) * span.size(), false)) ||
      (rc = fh_alloc(ctx, t->coef, sizeof(double) * std::max<size_t>(coef.size(), 1), false)) ||
      (rc = fh_alloc(ctx, t->cbuf, sizeof(double) * 2 * (size_t)std::max<long long>(ns, 1) * kMaxAK * (size_t)P,
                     false))) {
    delete t;
    return rc;
  }
  cudaError_t e = items.empty() ? cudaSuccess
                                : cudaMemcpy(t->items.p, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(t->spans.p, span.data(), sizeof(int4) * span.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !coef.empty()) e = cudaMemcpy(t->coef.p, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete t;
    return fh_set_error(ctx, FH_ECUDA, "two-series tables: %s", cudaGetErrorString(e));
  }
  t->nslots[0] = t->nslots[1] = (int)std::max<long long>(ns, 1);
  *out = t;
  return FH_OK;
}

void fh_ta_delete(fh_ta *t) { delete t; }

size_t fh_ta_bytes(const fh_ta *t) {
  return t ? t->items.bytes + t->spans.bytes + t->coef.bytes + t->cbuf.bytes : 0;
}

int fh_ta_step(fh_ctx *ctx, const fh_ta *t, int j, const double *Dn, int df, long long P, double sc, double *part,
               cudaStream_t st) {
  FH_REQUIRE(ctx, j >= 1 && j < t->max_steps, FH_EINVAL, "two-series step %d outside 1..%d", j, t->max_steps - 1);
  k_tg_two_series<<<dim3((unsigned)fh_ceil_div(P, 256), 2), 256, 0, st>>>(
      Dn, df, P, t->items.as<int4>(), t->spans.as<int4>() + 2LL * j, t->coef.as<double>(), t->cbuf.as<double>(),
      (long long)t->nslots[0], t->dterm[0], t->dterm[1], sc, part);
  return fh_after_launch(ctx, "k_tg_two_series");
}

extern "C" int fh_tg_two_series_plan(double alpha, int max_steps, int *nslots, double *dterm, int *n_items,
                                     int *items, int *n_coef, double *coef, int *spans) {
  if (!(alpha > 0.0 && alpha < 1.0) || max_steps < 1 || !nslots || !dterm || !n_items || !n_coef) return FH_EINVAL;
  std::vector<int4> it, sp;
  std::vector<double> cf;
  ta_plan(alpha, max_steps, it, cf, sp, nslots, dterm);
  if (items) {
    if (*n_items < (int)it.size()) return FH_EINVAL;
    std::memcpy(items, it.data(), sizeof(int4) * it.size());
  }
  if (coef) {
    if (*n_coef < (int)cf.size()) return FH_EINVAL;
    std::memcpy(coef, cf.data(), sizeof(double) * cf.size());
  }
  if (spans) std::memcpy(spans, sp.data(), sizeof(int4) * sp.size());
  *n_items = (int)it.size();
  *n_coef = (int)cf.size();
  return FH_OK;
}
