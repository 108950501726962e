// fh_ab.cu -- 1D Atangana-Baleanu convection-diffusion solve of
// MF_int_series.cpp:875-958 (solve_and_check, simple = 1): per step i
//   Rp_j = (Ii/(1-a)) C_j + f_j - (1/(1-a)) sum_{tt<=i-2} dC_tt/tau * I(i-tt)
//   A C_{j-1} + Bd C_j + Cc C_{j+1} = Rp_j, Dirichlet at both ends.
// The lag weights I(.) are computed once on the device (fh_weights_ab); the
// history stores dC_t/tau = (C^{t+1}-C^t)/tau per node.  The matrix is the same
// every step, so its elimination coefficients are built once and every step
// runs the two affine recurrences with one warp (see fh_linescan.cuh).
#include <cmath>

#include "fh_internal.h"
#include "fh_common.cuh"
#include "fh_linescan.cuh"
#include "fh_df.cuh"

// blocked contraction helpers (fh_blocked.cu)
struct fh_blk;
fh_blk *fh_blk_new();
void fh_blk_delete(fh_blk *b);
int fh_blk_init(fh_ctx *ctx, fh_blk &b, long long P, int Kcap);
int fh_blk_convert(fh_ctx *ctx, fh_blk &b, const double *D, long long ldd, int k0, int df);
int fh_blk_toeplitz_weights(fh_ctx *ctx, fh_blk &b, const double *w, int base, int K, int mrows);
int fh_blk_gemm(fh_ctx *ctx, fh_blk &b, int K, float2 *out, long long ldo, int gbeg = 0);
long long fh_blk_ppad(const fh_blk &b);
static constexpr int kAbBlock = 128;  // steps per block: one weight row each

struct fh_ab_solver {
  fh_ctx *ctx = nullptr;
  int m = 0, max_steps = 0, step = 0, nrows = 0, max_splits = 1024;
  long long P = 0;  // m+1 rounded up to even
  double tau = 0, alpha = 0, A = 0, Bd = 0, Cc = 0;
  fh_dbuf w, ii, al, den, inv, sl, pf, pb, C, D, W, part, S, src, bl, br;
  fh_graph_cache graph;
  int mode = FH_AB_FP64;
  fh_blk *blk = nullptr;  // blocked mode: bf16 slice planes of the history entries older than T0
  fh_dbuf far;            // far rows ((hi, lo) pairs) of the steps T0+1 .. T0+128
  long long ldfar = 0;
  int T0 = 0;
  // blocked mode with the line in shared memory: 8-step launches of
  // k_ab_line_fused in double-float; history entries, lag weights, source rows
  // and elimination tables as (hi, lo) FP32 pairs
  bool fused = false;
  fh_dbuf mid;            // history rows of the current 8-step sub-block (pairs)
  fh_dbuf w2, src2, tab2; // pairs: lag weights, source rows, tables sl, pf, -al, pb, inv
  ~fh_ab_solver() {
    if (blk) fh_blk_delete(blk);
  }
};

constexpr int kAbThreads = 256;
constexpr int kAbSolveWarps = 8;  // the solve runs on eight warps (two per SM sub-partition), 8-equation chunks
constexpr int kAbSolveThreads = 32 * kAbSolveWarps;

// al[j] = Cc/(Bd - A al[j-1]), den[j] = Bd - A al[j-1], al[0] = 0 (MF_int_series.cpp:933-940).
// The matrix is fixed, so the step-independent parts of both recurrences are
// tabulated here once: inv[j] = 1/den[j], the forward slope sl[j] = -A inv[j],
// and the per-lane chunk prefix products of the forward slopes (pf) and of the
// backward slopes -al[j] (pb) in the chunking of k_ab_line.
__global__ void k_ab_factor(int m, double A, double Bd, double Cc, double *__restrict__ al, double *__restrict__ den,
                            double *__restrict__ inv, double *__restrict__ sl, double *__restrict__ pf,
                            double *__restrict__ pb) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double a = 0.0;
  al[0] = 0.0;
  den[0] = 1.0;
  for (int j = 1; j <= m; ++j) {
    const double d = Bd - A * a;
    a = Cc / d;
    al[j] = a;
    den[j] = d;
    inv[j] = 1.0 / d;
    sl[j] = -A * inv[j];
  }
  const int ch = (m + kAbSolveThreads - 1) / kAbSolveThreads;
  double p = 1.0;
  for (int j = 1; j <= m; ++j) {
    p = ((j - 1) % ch == 0) ? sl[j] : p * sl[j];
    pf[j] = p;
  }
  double q = 1.0;
  for (int j = m - 1; j >= 0; --j) {
    const int b1 = min(m, (j / ch + 1) * ch);
    q = (j == b1 - 1) ? -al[j] : q * -al[j];
    pb[j] = q;
  }
}

// W[t] = w[i - (k0 + t)] for the history entries k0 + t, t < n
__global__ void k_ab_stepweights(int i, int k0, int n, const double *__restrict__ w, double *__restrict__ W) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) W[t] = w[i - k0 - t];
}

// One step of the tridiagonal solve (the line has m+1 nodes):
//   forward   bt[j] = (Rp_j - A bt[j-1]) / den_j = sl_j bt[j-1] + Rp_j inv_j
//   backward  C[j]  = bt[j] - al[j] C[j+1],  C[m] = right boundary value
// All threads stage the right parts and the tabulated coefficients into
// shared memory with coalesced loads (skewed by i / chunk so that the
// threads' chunks fall on distinct banks), kAbSolveWarps warps walk their
// threads' chunks from a zero start and add
// prefix * start value after a group scan of the chunk maps
// (fh_line_solve_prefix scheme), then all threads write C and the new history
// entry.
__global__ void __launch_bounds__(kAbThreads) k_ab_line(int m, double oma, const double *__restrict__ ii,
                                                        const double *__restrict__ alg,
                                                        const double *__restrict__ invg,
                                                        const double *__restrict__ slg,
                                                        const double *__restrict__ pfg,
                                                        const double *__restrict__ pbg,
                                                        const double *__restrict__ src,
                                                        const double *__restrict__ blp,
                                                        const double *__restrict__ brp, double *C,
                                                        const double *__restrict__ S,
                                                        const float2 *__restrict__ far, double *__restrict__ Dnew,
                                                        double tau) {
  extern __shared__ double sm[];
  const int ch = (m + kAbSolveThreads - 1) / kAbSolveThreads;
  const int Lm = m + 2 + m / ch + 1;
  double *rb = sm, *sl = rb + Lm, *pf = sl + Lm, *al = pf + Lm, *pb = al + Lm, *bt = pb + Lm, *cv = bt + Lm;
  auto sk = [ch](int j) { return j + j / ch; };
  // step constants computed once per CTA (FP64 divisions are scarce on this GPU)
  __shared__ double cst[3];
  if (threadIdx.x == 0) {
    cst[0] = ii[0] / oma;  // Ii/(1-a)
    cst[1] = 1.0 / oma;
    cst[2] = 1.0 / tau;
  }
  __syncthreads();
  const double cI = cst[0], ioma = cst[1], itau = cst[2];
  for (int j = threadIdx.x; j <= m; j += kAbThreads) {
    double r = fma(cI, C[j], src[j]);
    if (S || far) {  // MF_intF_simple returns ret/(1-a)
      double sv = S ? S[j] : 0.0;
      if (far) sv += (double)far[j].x + (double)far[j].y;
      r -= sv * ioma;
    }
    rb[sk(j)] = r * invg[j];
    sl[sk(j)] = slg[j];
    pf[sk(j)] = pfg[j];
    al[sk(j)] = alg[j];
    pb[sk(j)] = pbg[j];
  }
  __syncthreads();
  __shared__ fh_aff scan_sm[kAbSolveWarps];
  if (threadIdx.x < kAbSolveThreads) {
    const int t = threadIdx.x;
    const double bl = blp[0], br = brp[0];
    const int f0 = 1 + t * ch, f1 = min(m + 1, f0 + ch);
    double b = 0.0;
    for (int j = f0; j < f1; ++j) {
      b = fma(sl[sk(j)], b, rb[sk(j)]);
      bt[sk(j)] = b;
    }
    const fh_aff Pf =
        fh_group_exclusive_affine<kAbSolveWarps>(f1 > f0 ? fh_aff{pf[sk(f1 - 1)], b} : fh_aff{1.0, 0.0}, scan_sm, 1);
    const double s0 = fma(Pf.a, bl, Pf.b);  // bt[f0 - 1]
    for (int j = f0; j < f1; ++j) bt[sk(j)] = fma(pf[sk(j)], s0, bt[sk(j)]);
    if (t == 0) bt[sk(0)] = bl;
    fh_group_bar(1, kAbSolveThreads);
    const int b0 = t * ch, b1 = min(m, b0 + ch);
    double c = 0.0;
    for (int j = b1 - 1; j >= b0; --j) {
      c = fma(-al[sk(j)], c, bt[sk(j)]);
      cv[sk(j)] = c;
    }
    const fh_aff Pb = fh_group_exclusive_affine_rev<kAbSolveWarps>(b1 > b0 ? fh_aff{pb[sk(b0)], c} : fh_aff{1.0, 0.0},
                                                                   scan_sm, 1);
    const double tv = fma(Pb.a, br, Pb.b);  // C[b1]
    for (int j = b0; j < b1; ++j) cv[sk(j)] = fma(pb[sk(j)], tv, cv[sk(j)]);
    if (t == 0) cv[sk(m)] = br;
  }
  __syncthreads();
  for (int j = threadIdx.x; j <= m; j += kAbThreads) {
    const double v = cv[sk(j)];
    const double old = C[j];
    C[j] = v;
    if (Dnew) Dnew[j] = (v - old) * itau;
  }
}

// ------------------------------------------------ blocked mode: 8-step sub-blocks
// The history of step i (entries tt < K = i - 1) splits into the far rows of
// the current 128-step block (tt < T0, tensor cores), the sub-block rows
// (T0 <= tt < K8, k_ab_mid, once per 8 steps) and the at most 7 entries of the
// sub-block itself (K8 <= tt < K), which k_ab_line_fused adds while it runs
// the 8 steps of the sub-block in one launch.
static constexpr int kAbSub = 8;
static constexpr int kAbFuseThreads = 512;
static constexpr int kAbFuseMaxNodes = 5;  // nodes per thread: m + 1 <= 2560

// mid[r][j] = far row of step K8 + r + sum_{T0 <= tt < K8} w[K8 + r + 1 - tt] D[tt][j], r < nr,
// in double-float (D and w as (hi, lo) pairs, TwoSum accumulation as in
// k_hist_sum_df), one node and one row per thread.
__global__ void k_ab_mid(int m, long long P, int T0, int K8, int nr, const float2 *__restrict__ w2,
                         const float2 *__restrict__ D, const float2 *__restrict__ far, long long ldfar,
                         float2 *__restrict__ mid) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (j > m || r >= nr) return;
  const int i = K8 + r + 1;  // reference step index of row r
  fh_df acc{0.f, 0.f};
  if (far) acc = fh_df_from_pair(far[(long long)(K8 + r - T0) * ldfar + j]);
  float sh = acc.h, sl = acc.l;
  for (int tt = T0; tt < K8; ++tt) {
    const float2 w = __ldg(w2 + i - tt);
    const float2 d = D[(long long)tt * P + j];
    const float ph = w.x * d.x;
    float pl = fmaf(w.x, d.x, -ph);
    pl = fmaf(w.x, d.y, pl);
    pl = fmaf(w.y, d.x, pl);
    const float t = sh + ph;
    const float bb = t - sh;
    const float e = (sh - (t - bb)) + (ph - bb);
    sh = t;
    sl += e + pl;
    if ((tt & 15) == 15) {  // renormalise
      const float u = sh + sl;
      sl = sl - (u - sh);
      sh = u;
    }
  }
  const float h = sh + sl;
  mid[(long long)r * P + j] = make_float2(h, sl - (h - sh));
}

// Steps K8 + s0 .. K8 + s0 + ns - 1 of one sub-block in one CTA, in
// double-float: the elimination tables and the field stay in shared memory
// for the whole launch; per step the right parts (source row, sub-block row or
// far row, the sub-block's own entries), the solve of k_ab_line
// (kAbSolveWarps warps, double-float group scans) and the new history entry
// dC/tau.  FP64 only
// converts the field at the start and the end of the launch.  Every thread
// keeps the right-part loads of all its nodes (j = tid + 512 k) in flight at
// once, the sub-block's entries two per round trip.
__global__ void __launch_bounds__(kAbFuseThreads, 1)
    k_ab_line_fused(int m, double oma, const double *__restrict__ ii, const float2 *__restrict__ tab,
                    long long ldt, const float2 *__restrict__ src2, int nrows, const double *__restrict__ blp,
                    const double *__restrict__ brp, double *C, float2 *D, long long P,
                    const float2 *__restrict__ w2, const float2 *__restrict__ mid, const float2 *__restrict__ far8,
                    long long ldfar, int K8, int s0, int ns, double tau) {
  constexpr int NMAX = kAbFuseMaxNodes;  // nodes per thread
  extern __shared__ float2 smf[];
  const int ch = (m + kAbSolveThreads - 1) / kAbSolveThreads;
  const int Lm = m + 2 + m / ch + 1;
  float2 *rb = smf, *sl = rb + Lm, *pf = sl + Lm, *nal = pf + Lm, *pb = nal + Lm, *bt = pb + Lm, *cv = bt + Lm,
         *inv = cv + Lm, *Cs = inv + Lm;
  auto sk = [ch](int j) { return j + j / ch; };
  __shared__ float2 cst[3], wts[kAbSub][kAbSub], bnd[kAbSub][2];
  for (int j = threadIdx.x; j <= m; j += kAbFuseThreads) {
    sl[sk(j)] = tab[j];
    pf[sk(j)] = tab[ldt + j];
    nal[sk(j)] = tab[2 * ldt + j];
    pb[sk(j)] = tab[3 * ldt + j];
    inv[j] = tab[4 * ldt + j];
    Cs[j] = fh_df_pair(fh_df_from_double(C[j]));
  }
  // step constants (one FP64 conversion per thread), the weights of the
  // sub-block's entries wts[s][t] = w[(K8 + s + 1) - (K8 + t)] and the
  // boundary values of every step
  if (threadIdx.x == 0) cst[0] = fh_df_pair(fh_df_from_double(ii[0] / oma));  // Ii/(1-a)
  if (threadIdx.x == 1) cst[1] = fh_df_pair(fh_df_from_double(-1.0 / oma));
  if (threadIdx.x == 2) cst[2] = fh_df_pair(fh_df_from_double(1.0 / tau));
  if (threadIdx.x >= 32 && threadIdx.x < 32 + kAbSub * kAbSub) {
    const int v = threadIdx.x - 32, ss = v / kAbSub, t = v % kAbSub;
    wts[ss][t] = t < ss ? w2[ss + 1 - t] : make_float2(0.f, 0.f);
  }
  if (threadIdx.x >= 128 && threadIdx.x < 128 + 2 * kAbSub) {
    const int v = threadIdx.x - 128, ss = v >> 1;
    if (ss >= s0 && ss < s0 + ns) {
      const int K = K8 + ss, row = K < nrows - 1 ? K : nrows - 1;
      bnd[ss][v & 1] = fh_df_pair(fh_df_from_double((v & 1) ? brp[row] : blp[row]));
    }
  }
  __syncthreads();
  const fh_df cI = fh_df_from_pair(cst[0]), nioma = fh_df_from_pair(cst[1]), itau = fh_df_from_pair(cst[2]);
  const fh_daff I{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}};
  __shared__ fh_daff scan_sm[kAbSolveWarps];
  for (int s = s0; s < s0 + ns; ++s) {
    const int K = K8 + s;  // history entries of this step (reference step i = K + 1)
    const int row = K < nrows - 1 ? K : nrows - 1;
    const float2 *srow = src2 + (long long)row * (m + 1);
    const float2 *mrow = mid ? mid + (long long)s * P : nullptr;
    const float2 *frow = far8 ? far8 + (long long)s * ldfar : nullptr;
    const bool hist = mrow || frow || s > 0;
    {
      // right parts: all of the thread's loads in flight together
      float2 sr[NMAX], hv[NMAX];
#pragma unroll
      for (int k = 0; k < NMAX; ++k) {
        const int j = threadIdx.x + k * kAbFuseThreads;
        if (j <= m) {
          sr[k] = srow[j];
          hv[k] = mrow ? mrow[j] : (frow ? frow[j] : make_float2(0.f, 0.f));
        }
      }
      fh_df hs[NMAX];
#pragma unroll
      for (int k = 0; k < NMAX; ++k) hs[k] = fh_df_from_pair(hv[k]);
      if (mrow && frow) {
#pragma unroll
        for (int k = 0; k < NMAX; ++k) {
          const int j = threadIdx.x + k * kAbFuseThreads;
          if (j <= m) hs[k] = fh_df_add(fh_df_from_pair(mrow[j]), fh_df_from_pair(frow[j]));
        }
      }
      for (int t0 = 0; t0 < s; t0 += 2) {  // the sub-block's own entries, two per round trip
        float2 d[2][NMAX];
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int k = 0; k < NMAX; ++k) {
            const int j = threadIdx.x + k * kAbFuseThreads;
            if (t0 + u < s && j <= m) d[u][k] = __ldcg(D + (long long)(K8 + t0 + u) * P + j);
          }
#pragma unroll
        for (int u = 0; u < 2; ++u)
          if (t0 + u < s) {
            const fh_df w = fh_df_from_pair(wts[s][t0 + u]);
#pragma unroll
            for (int k = 0; k < NMAX; ++k) hs[k] = fh_df_fma(w, fh_df_from_pair(d[u][k]), hs[k]);
          }
      }
#pragma unroll
      for (int k = 0; k < NMAX; ++k) {
        const int j = threadIdx.x + k * kAbFuseThreads;
        if (j <= m) {
          fh_df r = fh_df_fma(cI, fh_df_from_pair(Cs[j]), fh_df_from_pair(sr[k]));
          if (hist) r = fh_df_fma(nioma, hs[k], r);  // MF_intF_simple returns ret/(1-a)
          rb[sk(j)] = fh_df_pair(fh_df_mul(r, fh_df_from_pair(inv[j])));
        }
      }
    }
    __syncthreads();
    if (threadIdx.x < kAbSolveThreads) {
      const int t = threadIdx.x;
      const fh_df bl = fh_df_from_pair(bnd[s][0]), br = fh_df_from_pair(bnd[s][1]);
      const int f0 = 1 + t * ch, f1 = min(m + 1, f0 + ch);
      fh_df b{0.f, 0.f};
      for (int j = f0; j < f1; ++j) {
        b = fh_df_fma(fh_df_from_pair(sl[sk(j)]), b, fh_df_from_pair(rb[sk(j)]));
        bt[sk(j)] = fh_df_pair(b);
      }
      const fh_daff Pf = fh_group_exclusive_daff<kAbSolveWarps>(
          f1 > f0 ? fh_daff{fh_df_from_pair(pf[sk(f1 - 1)]), b} : I, scan_sm, 1);
      const fh_df s0v = fh_df_fma(Pf.a, bl, Pf.b);  // bt[f0 - 1]
      for (int j = f0; j < f1; ++j)
        bt[sk(j)] = fh_df_pair(fh_df_fma(fh_df_from_pair(pf[sk(j)]), s0v, fh_df_from_pair(bt[sk(j)])));
      if (t == 0) bt[sk(0)] = fh_df_pair(bl);
      fh_group_bar(1, kAbSolveThreads);
      const int b0 = t * ch, b1 = min(m, b0 + ch);
      fh_df c{0.f, 0.f};
      for (int j = b1 - 1; j >= b0; --j) {
        c = fh_df_fma(fh_df_from_pair(nal[sk(j)]), c, fh_df_from_pair(bt[sk(j)]));
        cv[sk(j)] = fh_df_pair(c);
      }
      const fh_daff Pb = fh_group_exclusive_daff_rev<kAbSolveWarps>(
          b1 > b0 ? fh_daff{fh_df_from_pair(pb[sk(b0)]), c} : I, scan_sm, 1);
      const fh_df tv = fh_df_fma(Pb.a, br, Pb.b);  // C[b1]
      for (int j = b0; j < b1; ++j)
        cv[sk(j)] = fh_df_pair(fh_df_fma(fh_df_from_pair(pb[sk(j)]), tv, fh_df_from_pair(cv[sk(j)])));
      if (t == 0) cv[sk(m)] = fh_df_pair(br);
    }
    __syncthreads();
    float2 *Dk = D + (long long)K * P;
    for (int j = threadIdx.x; j <= m; j += kAbFuseThreads) {
      const fh_df v = fh_df_from_pair(cv[sk(j)]);
      Dk[j] = fh_df_pair(fh_df_mul(fh_df_sub(v, fh_df_from_pair(Cs[j])), itau));
      Cs[j] = fh_df_pair(v);
    }
    __syncthreads();
  }
  for (int j = threadIdx.x; j <= m; j += kAbFuseThreads) C[j] = fh_df_to_double(fh_df_from_pair(Cs[j]));
}

// (hi, lo) pairs of n doubles; neg: of their negatives
__global__ void k_ab_pairs(const double *__restrict__ x, float2 *__restrict__ y, long long n, int neg) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = fh_df_pair(fh_df_from_double(neg ? -x[i] : x[i]));
}

static size_t ab_fused_smem(int m) {
  const int ch = (m + kAbSolveThreads - 1) / kAbSolveThreads;
  return sizeof(float2) * (8 * (size_t)(m + 2 + m / ch + 1) + (size_t)m + 1);
}

// Pair copies for the double-float launches: elimination tables (after every
// factorization), lag weights, source rows.
static int ab_pairs(fh_ctx *ctx, const double *x, float2 *y, long long n, int neg) {
  k_ab_pairs<<<(unsigned)fh_ceil_div(n, 256), 256, 0, ctx->stream>>>(x, y, n, neg);
  return fh_after_launch(ctx, "k_ab_pairs");
}
static int ab_table_pairs(fh_ab_solver *s) {
  if (!s->fused) return FH_OK;
  const long long n = s->m + 1;
  float2 *t = s->tab2.as<float2>();
  int rc;
  if ((rc = ab_pairs(s->ctx, s->sl.as<double>(), t, n, 0)) || (rc = ab_pairs(s->ctx, s->pf.as<double>(), t + s->P, n, 0)) ||
      (rc = ab_pairs(s->ctx, s->al.as<double>(), t + 2 * s->P, n, 1)) ||
      (rc = ab_pairs(s->ctx, s->pb.as<double>(), t + 3 * s->P, n, 0)) ||
      (rc = ab_pairs(s->ctx, s->inv.as<double>(), t + 4 * s->P, n, 0)))
    return rc;
  return FH_OK;
}
static int ab_src_pairs(fh_ab_solver *s) {
  if (!s->fused || s->nrows < 1) return FH_OK;
  int rc = fh_alloc(s->ctx, s->src2, sizeof(float2) * (size_t)s->nrows * (s->m + 1), false);
  if (rc) return rc;
  return ab_pairs(s->ctx, s->src.as<double>(), s->src2.as<float2>(), (long long)s->nrows * (s->m + 1), 0);
}

static size_t ab_line_smem(int m) {
  const int ch = (m + kAbSolveThreads - 1) / kAbSolveThreads;
  return sizeof(double) * 7 * (size_t)(m + 2 + m / ch + 1);
}

static int ab_fused_steps(fh_ab_solver *s, int max_n, int *done);

static int ab_one_step(fh_ab_solver *s, int max_n, int *done) {
  *done = 1;
  fh_ctx *ctx = s->ctx;
  const int i = s->step + 1;  // reference step index (1-based)
  const int K = i - 1;        // history entries dC_0 .. dC_{i-2}
  const int row = (i - 1 < s->nrows - 1) ? i - 1 : s->nrows - 1;
  int rc;
  if (s->blk && K > 0 && K % kAbBlock == 0) {
    // new block: entries [K-128, K) into the slice planes, Toeplitz rows of the
    // next 128 steps, far rows S_far[r] = sum_{tt<K} w[K+1+r-tt] dC_tt
    const int dfh = s->fused ? 1 : 0;  // fused launches store the entries as (hi, lo) pairs
    if ((rc = fh_blk_convert(ctx, *s->blk, s->D.as<double>(), s->P, K - kAbBlock, dfh)) ||
        (rc = fh_blk_convert(ctx, *s->blk, s->D.as<double>(), s->P, K - kAbBlock / 2, dfh)))
      return rc;
    const int mrows = s->max_steps - K < kAbBlock ? s->max_steps - K : kAbBlock;
    if ((rc = fh_blk_toeplitz_weights(ctx, *s->blk, s->w.as<double>(), K + 1, K, mrows))) return rc;
    if ((rc = fh_blk_gemm(ctx, *s->blk, K, s->far.as<float2>(), s->ldfar))) return rc;
    s->T0 = K;
  }
  if (s->fused) return ab_fused_steps(s, max_n, done);
  const int k0 = s->blk ? s->T0 : 0;  // entries summed on the CUDA cores this step
  const int kn = K - k0;
  const float2 *far = (s->blk && s->T0 > 0) ? s->far.as<float2>() + (long long)(K - s->T0) * s->ldfar : nullptr;
  const double *S = nullptr;
  if (kn > 0) {
    k_ab_stepweights<<<(unsigned)fh_ceil_div(kn, 256), 256, 0, ctx->stream>>>(i, k0, kn, s->w.as<double>(),
                                                                             s->W.as<double>());
    if ((rc = fh_after_launch(ctx, "k_ab_stepweights"))) return rc;
    int splits, kchunk;
    fh_hist_plan(s->P, kn, s->max_splits, &splits, &kchunk);
    if ((rc = fh_launch_hist_sum_partials(ctx, 1, kn, s->P, s->W.as<double>(), s->max_steps + 1,
                                          s->D.as<double>() + (long long)k0 * s->P, s->P, splits, kchunk,
                                          s->part.as<double>(), s->P)))
      return rc;
    if ((rc = fh_launch_reduce_splits(ctx, splits, s->P, s->part.as<double>(), s->P, s->S.as<double>()))) return rc;
    S = s->S.as<double>();
  }
  fh_prof_mark(ctx, FH_PROF_SWEEP, false);
  k_ab_line<<<1, kAbThreads, ab_line_smem(s->m), ctx->stream>>>(
      s->m, 1.0 - s->alpha, s->ii.as<double>(), s->al.as<double>(), s->inv.as<double>(), s->sl.as<double>(),
      s->pf.as<double>(), s->pb.as<double>(), s->src.as<double>() + (long long)row * (s->m + 1),
      s->bl.as<double>() + row, s->br.as<double>() + row, s->C.as<double>(), S, far,
      s->D.as<double>() + (long long)s->step * s->P, s->tau);
  fh_prof_mark(ctx, FH_PROF_SWEEP, true);
  if ((rc = fh_after_launch(ctx, "k_ab_line"))) return rc;
  s->step++;
  return FH_OK;
}

// Blocked mode: the block-start work of step K is already enqueued; runs up to
// max_n steps of the current 8-step sub-block (k_ab_mid first at its start).
static int ab_fused_steps(fh_ab_solver *s, int max_n, int *done) {
  fh_ctx *ctx = s->ctx;
  const int K = s->step;
  const int T0 = s->blk ? s->T0 : 0;
  const int K8 = (K / kAbSub) * kAbSub;  // >= T0: blocks are whole sub-blocks
  int rc;
  if (K == K8 && K8 > T0) {
    const int nr = min(kAbSub, s->max_steps - K8);
    fh_prof_mark(ctx, FH_PROF_HISTORY, false);
    k_ab_mid<<<dim3((unsigned)fh_ceil_div(s->m + 1, 128), (unsigned)nr), 128, 0, ctx->stream>>>(
        s->m, s->P, T0, K8, nr, s->w2.as<float2>(), reinterpret_cast<const float2 *>(s->D.as<double>()),
        (s->blk && T0 > 0) ? s->far.as<float2>() : nullptr, s->ldfar, s->mid.as<float2>());
    fh_prof_mark(ctx, FH_PROF_HISTORY, true);
    if ((rc = fh_after_launch(ctx, "k_ab_mid"))) return rc;
  }
  const float2 *mid = K8 > T0 ? s->mid.as<float2>() : nullptr;
  const float2 *far8 = (!mid && s->blk && T0 > 0) ? s->far.as<float2>() + (long long)(K8 - T0) * s->ldfar : nullptr;
  const int ns = min(max_n, kAbSub - (K - K8));
  fh_prof_mark(ctx, FH_PROF_SWEEP, false);
  k_ab_line_fused<<<1, kAbFuseThreads, ab_fused_smem(s->m), ctx->stream>>>(
      s->m, 1.0 - s->alpha, s->ii.as<double>(), s->tab2.as<float2>(), s->P, s->src2.as<float2>(), s->nrows,
      s->bl.as<double>(), s->br.as<double>(), s->C.as<double>(), reinterpret_cast<float2 *>(s->D.as<double>()),
      s->P, s->w2.as<float2>(), mid, far8, s->ldfar, K8, K - K8, ns, s->tau);
  fh_prof_mark(ctx, FH_PROF_SWEEP, true);
  if ((rc = fh_after_launch(ctx, "k_ab_line_fused"))) return rc;
  s->step += ns;
  *done = ns;
  return FH_OK;
}

extern "C" {

int fh_ab_create(fh_ctx *ctx, int m, int max_steps, double tau, double alpha, fh_ab_solver **out) {
  FH_REQUIRE(ctx, ctx && out, FH_EINVAL, "fh_ab_create: null argument");
  *out = nullptr;
  FH_REQUIRE(ctx, m >= 2 && m <= 3500 && max_steps >= 1 && tau > 0 && alpha > 0 && alpha < 1, FH_EINVAL,
             "fh_ab_create: need 2 <= m <= 3500, max_steps >= 1, tau > 0, 0 < alpha < 1");
  {
    const size_t sm = ab_line_smem(m);
    FH_REQUIRE(ctx, sm <= 200 * 1024, FH_EINVAL, "fh_ab_create: m too large for the staged line (m <= 3500)");
    FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_ab_line, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_ab_line_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  }
  fh_ab_solver *s = new fh_ab_solver();
  s->ctx = ctx;
  s->m = m;
  s->max_steps = max_steps;
  s->tau = tau;
  s->alpha = alpha;
  s->P = ((long long)m + 1 + 1) & ~1LL;
  const double h = 1.0 / m;
  s->A = -(1.0 / (h * h)) - (1.0 / (2.0 * h));
  s->Cc = -(1.0 / (h * h)) + (1.0 / (2.0 * h));
  int rc;
  const size_t fld = sizeof(double) * (size_t)s->P;
  if ((rc = fh_alloc(ctx, s->w, sizeof(double) * (size_t)(max_steps + 2))) || (rc = fh_alloc(ctx, s->ii, 16)) ||
      (rc = fh_alloc(ctx, s->al, fld)) || (rc = fh_alloc(ctx, s->den, fld)) || (rc = fh_alloc(ctx, s->inv, fld)) ||
      (rc = fh_alloc(ctx, s->sl, fld)) || (rc = fh_alloc(ctx, s->pf, fld)) || (rc = fh_alloc(ctx, s->pb, fld)) ||
      (rc = fh_alloc(ctx, s->C, fld)) ||
      (rc = fh_alloc(ctx, s->D, fld * (size_t)max_steps)) ||
      (rc = fh_alloc(ctx, s->W, sizeof(double) * (size_t)(max_steps + 1))) ||
      (rc = fh_alloc(ctx, s->part, fld * (size_t)s->max_splits, false)) || (rc = fh_alloc(ctx, s->S, fld))) {
    delete s;
    return rc;
  }
  if ((rc = fh_weights_ab(ctx, max_steps + 1, tau, alpha, s->w.as<double>()))) {
    delete s;
    return rc;
  }
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->ii.p, s->w.p, sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  // Bd = Ii/(1-a) + 2/h^2 with Ii from the device weights
  double ii_h = 0.0;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(&ii_h, s->w.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  s->Bd = (ii_h / (1.0 - alpha)) + (2.0 / (h * h));
  k_ab_factor<<<1, 1, 0, ctx->stream>>>(m, s->A, s->Bd, s->Cc, s->al.as<double>(), s->den.as<double>(),
                                        s->inv.as<double>(), s->sl.as<double>(), s->pf.as<double>(),
                                        s->pb.as<double>());
  if ((rc = fh_after_launch(ctx, "k_ab_factor"))) {
    delete s;
    return rc;
  }
  *out = s;
  return FH_OK;
}

int fh_ab_destroy(fh_ab_solver *s) {
  if (!s) return FH_OK;
  if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
  delete s;
  return FH_OK;
}

int fh_ab_set_source_host(fh_ab_solver *s, int nrows, const double *src_host, const double *bl_host,
                          const double *br_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, nrows >= 1 && src_host && bl_host && br_host, FH_EINVAL, "fh_ab_set_source_host: bad args");
  int rc;
  if ((rc = fh_alloc(ctx, s->src, sizeof(double) * (size_t)nrows * (s->m + 1), false)) ||
      (rc = fh_alloc(ctx, s->bl, sizeof(double) * nrows, false)) ||
      (rc = fh_alloc(ctx, s->br, sizeof(double) * nrows, false)))
    return rc;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->src.p, src_host, sizeof(double) * (size_t)nrows * (s->m + 1),
                                   cudaMemcpyHostToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->bl.p, bl_host, sizeof(double) * nrows, cudaMemcpyHostToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->br.p, br_host, sizeof(double) * nrows, cudaMemcpyHostToDevice, ctx->stream));
  s->nrows = nrows;
  if ((rc = ab_src_pairs(s))) return rc;
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FH_OK;
}

int fh_ab_set_c_host(fh_ab_solver *s, const double *C_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, C_host, FH_EINVAL, "fh_ab_set_c_host: null pointer");
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->C.p, C_host, sizeof(double) * (s->m + 1), cudaMemcpyHostToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  s->step = 0;
  s->T0 = 0;
  return FH_OK;
}

int fh_ab_set_c(fh_ab_solver *s, const double *C) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, C, FH_EINVAL, "fh_ab_set_c: null pointer");
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->C.p, C, sizeof(double) * (s->m + 1), cudaMemcpyDeviceToDevice, ctx->stream));
  s->step = 0;
  s->T0 = 0;
  return FH_OK;
}

int fh_ab_set_current_coef(fh_ab_solver *s, double Ii) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "null solver");
  fh_ctx *ctx = s->ctx;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->ii.p, &Ii, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const double h = 1.0 / s->m;
  s->Bd = (Ii / (1.0 - s->alpha)) + (2.0 / (h * h));
  k_ab_factor<<<1, 1, 0, ctx->stream>>>(s->m, s->A, s->Bd, s->Cc, s->al.as<double>(), s->den.as<double>(),
                                        s->inv.as<double>(), s->sl.as<double>(), s->pf.as<double>(),
                                        s->pb.as<double>());
  const int rc = fh_after_launch(ctx, "k_ab_factor");
  return rc ? rc : ab_table_pairs(s);
}

int fh_ab_set_lag_weights_host(fh_ab_solver *s, int n, const double *w_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, w_host && n >= 1 && n <= s->max_steps + 1, FH_EINVAL,
             "fh_ab_set_lag_weights_host: need 1 <= n <= max_steps + 1 and a table");
  FH_REQUIRE(ctx, s->step == 0, FH_EINVAL, "fh_ab_set_lag_weights_host: only before the first step");
  for (int l = 0; l < n; ++l)
    FH_REQUIRE(ctx, std::isfinite(w_host[l]), FH_ENONFINITE, "fh_ab_set_lag_weights_host: weight of lag %d", l + 1);
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->w.as<double>() + 1, w_host, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice,
                                   ctx->stream));
  int rc;
  if (s->w2.p && (rc = ab_pairs(ctx, s->w.as<double>(), s->w2.as<float2>(), s->max_steps + 2, 0))) return rc;
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  s->graph.reset();
  return FH_OK;
}

int fh_ab_set_mode(fh_ab_solver *s, int mode) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, mode == FH_AB_FP64 || mode == FH_AB_BLOCKED, FH_EINVAL, "fh_ab_set_mode: unknown mode %d", mode);
  FH_REQUIRE(ctx, s->step == 0, FH_EINVAL, "fh_ab_set_mode: only before the first step");
  s->mode = mode;
  if (mode == FH_AB_BLOCKED && !s->blk && s->max_steps > kAbBlock) {
    s->blk = fh_blk_new();
    const int kcap = (int)fh_ceil_div(s->max_steps, kAbBlock) * kAbBlock;
    int rc = fh_blk_init(ctx, *s->blk, s->P, kcap);
    if (!rc) {
      s->ldfar = fh_blk_ppad(*s->blk);
      rc = fh_alloc(ctx, s->far, sizeof(float2) * kAbBlock * (size_t)s->ldfar, false);
    }
    if (rc) {
      fh_blk_delete(s->blk);
      s->blk = nullptr;
      return rc;
    }
  }
  if (mode == FH_AB_FP64 && s->blk) {
    fh_blk_delete(s->blk);
    s->blk = nullptr;
  }
  // 8-step launches when the tables and the field fit in shared memory
  s->fused = mode == FH_AB_BLOCKED && ab_fused_smem(s->m) <= 200 * 1024 &&
             s->m + 1 <= kAbFuseThreads * kAbFuseMaxNodes;
  if (s->fused) {
    int rc;
    if (!s->mid.p && (rc = fh_alloc(ctx, s->mid, sizeof(float2) * kAbSub * (size_t)s->P))) return rc;
    if (!s->tab2.p && (rc = fh_alloc(ctx, s->tab2, sizeof(float2) * 5 * (size_t)s->P))) return rc;
    if (!s->w2.p) {
      if ((rc = fh_alloc(ctx, s->w2, sizeof(float2) * (size_t)(s->max_steps + 2)))) return rc;
      if ((rc = ab_pairs(ctx, s->w.as<double>(), s->w2.as<float2>(), s->max_steps + 2, 0))) return rc;
    }
    if ((rc = ab_table_pairs(s)) || (rc = ab_src_pairs(s))) return rc;
  }
  s->graph.reset();
  return FH_OK;
}

int fh_ab_step(fh_ab_solver *s, int nsteps) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, s->nrows >= 1, FH_EINVAL, "fh_ab_step: source not set");
  FH_REQUIRE(ctx, nsteps >= 0 && s->step + nsteps <= s->max_steps, FH_ENOMEM, "fh_ab_step: history full");
  if (ctx->graphs && s->step == 0 && nsteps > 1) {
    int rc = fh_graph_run(ctx, s->graph, nsteps, [&]() {
      for (int n = 0, d = 1; n < nsteps; n += d) {
        int r = ab_one_step(s, nsteps - n, &d);
        if (r) return r;
      }
      return (int)FH_OK;
    });
    if (rc) return rc;
    s->step = nsteps;
    return FH_OK;
  }
  for (int n = 0, d = 1; n < nsteps; n += d) {
    int rc = ab_one_step(s, nsteps - n, &d);
    if (rc) return rc;
  }
  return FH_OK;
}

int fh_ab_get_c_host(fh_ab_solver *s, double *C_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, C_host, FH_EINVAL, "fh_ab_get_c_host: null pointer");
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(C_host, s->C.p, sizeof(double) * (s->m + 1), cudaMemcpyDeviceToHost, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FH_OK;
}

}  // extern "C"
