// fh_tg.cu -- 2D ADI solver with full fractional history, the TG_solver_<.,1,.>
// path of fr_d_t_g_2d.cpp with dt_alg 0 (fr_d_t_g_2d.cpp:2552-2718, 3242-3553).
//
// Per time step j (launches on the context stream):
//   1. k_tg_weights   x/y history weights for k < j and the three current weights
//   2. history sum    S_x, S_y over the j stored full-step differences, one pass
//                     (the reference reads the layers once per half step)
//   3. k_tg_xsweep    one warp per x line (j = 1..M-1), unknowns along i
//   4. k_tg_ysweep    one warp per y line (i = 1..sN-1), unknowns along j; also
//                     appends the new full-step difference to the history and
//                     keeps a copy of the full-step field
// The Thomas factorization of both sweep directions depends only on V2, d and
// the current weight; for psi = t that weight is the same every step, so the
// factorization is built once (k_tg_factor) and each step only runs the two
// affine recurrences (fh_linescan.cuh).  For psi != t it is rebuilt per step.
//
// Storage (HBM): C, Cfull, V2 and the factor tables are (sN+2)(M+2) doubles in
// the reference layout idx = i + j*(sN+2); the history holds one difference
// layer per full step, D[k] = C^{k+1} - C^k (the half-step layers the
// reference also stores are only read through C itself).
#include "fh_internal.h"
#include "fh_common.cuh"
#include "fh_linescan.cuh"
#include "fh_weights.cuh"

struct fh_tg_dev {
  int sN, M, ld;
  long long P;
  double tau, alpha, beta, Da, st, d, C1, S, dL, dLx;
};

struct fh_tg_solver {
  fh_ctx *ctx = nullptr;
  fh_tg_params p{};
  fh_tg_dev dv{};
  int mode = FH_TG_FP64;
  int max_steps = 0;
  int tstep = 0;
  bool have_state = false;
  bool factor_fixed = false;
  int max_splits = 8;
  fh_dbuf C, Cfull, V2, D, W, cw, part, alx, gx, aly, gy;
};

// ---------------------------------------------------------------- kernels

// W[0][k] = kb(k,0.5,0.0,1.0), W[1][k] = kb(k,1.0,0.0,1.0) for k < j;
// cw = {kb(j,0.5,0.0,0.5), kb(j,1.0,0.5,0.5), kb(j,1.0,0.0,0.5)} (TG_solver_::kb).
__global__ void k_tg_weights(fh_tg_dev g, int j, double *__restrict__ W, int ldw, double *__restrict__ cw) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < j) {
    const double s0 = (double)k + 0.0;
    W[k] = g.Da * fh_psi_int(s0, s0 + 1.0, (double)j + 0.5, g.tau, g.alpha, g.beta);
    W[ldw + k] = g.Da * fh_psi_int(s0, s0 + 1.0, (double)j + 1.0, g.tau, g.alpha, g.beta);
  }
  if (k == 0) {
    const double jj = (double)j;
    cw[0] = g.Da * fh_psi_int(jj + 0.0, jj + 0.0 + 0.5, jj + 0.5, g.tau, g.alpha, g.beta);
    cw[1] = g.Da * fh_psi_int(jj + 0.5, jj + 0.5 + 0.5, jj + 1.0, g.tau, g.alpha, g.beta);
    cw[2] = g.Da * fh_psi_int(jj + 0.0, jj + 0.0 + 0.5, jj + 1.0, g.tau, g.alpha, g.beta);
  }
}

// Serial factorization of every line (one thread per line): Al[i+1] and g_i,
// stored at the point of equation i.  dir 0: x lines, dir 1: y lines.
__global__ void k_tg_factor(fh_tg_dev g, int dir, const double *__restrict__ V2, const double *__restrict__ cw,
                            double *__restrict__ al, double *__restrict__ gg) {
  const int line = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int nlines = dir == 0 ? g.M : g.sN;
  if (line >= nlines) return;
  const int N = dir == 0 ? g.sN : g.M;
  const long long base = dir == 0 ? (long long)line * g.ld : line;
  const long long stride = dir == 0 ? 1 : g.ld;
  const double dl = dir == 0 ? g.dL : g.dLx;
  const double kcur = dir == 0 ? cw[0] : cw[1];
  double alv = dir == 0 ? 0.0 : 1.0;
  for (int i = 1; i < N; ++i) {
    const long long id = base + i * stride;
    const double v2 = V2[id];
    double A, B;
    if (dir == 0) {
      A = (v2 / dl) * ((0.5 * (g.d + g.d) / dl) + 0.5);
      B = (v2 / dl) * ((0.5 * (g.d + g.d) / dl) - 0.5);
    } else {
      A = (v2 / (dl * dl)) * 0.5 * (g.d + g.d);
      B = A;
    }
    const double R = g.st * (kcur + 0.0) + A + B;
    const double den = R - A * alv;
    const double aln = B / den;
    al[id] = aln;
    gg[id] = (aln == 0.0 && B == 0.0) ? 1.0 / den : aln / B;
    alv = aln;
  }
}

struct TgXLine {
  long long base;  // line j: point i at base + i
  const double *V2, *C, *part, *gg;
  double *Cw;
  long long ldp;
  int splits;
  double dl, d, st, S, kx;
  __device__ double A(int i) const { return (V2[base + i] / dl) * ((0.5 * (d + d) / dl) + 0.5); }
  __device__ double om(int i) const {
    const long long id = base + i;
    double ts = 0.0;
    for (int s = 0; s < splits; ++s) ts += part[(long long)(2 * s) * ldp + id];
    double o = -st * (kx + 0.0) * C[id];
    o += S * 0.5;
    o += st * ts;
    return o;
  }
  __device__ double g(int i) const { return gg[base + i]; }
  __device__ double al(int i) const { return al_[base + i]; }
  const double *al_;
  __device__ void store(int i, double u) const { Cw[base + i] = u; }
};

__global__ void k_tg_xsweep(fh_tg_dev g, const double *__restrict__ V2, double *C,
                            const double *__restrict__ part, long long ldp, int splits,
                            const double *__restrict__ al, const double *__restrict__ gg,
                            const double *__restrict__ cw) {
  extern __shared__ double sbuf[];
  const int warp = threadIdx.x >> 5;
  const int line = 1 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (line >= g.M) return;  // whole warp exits together
  double *buf = sbuf + (size_t)warp * (g.sN + 1);
  TgXLine L;
  L.base = (long long)line * g.ld;
  L.V2 = V2;
  L.C = C;
  L.part = part;
  L.al_ = al;
  L.gg = gg;
  L.Cw = C;
  L.ldp = ldp;
  L.splits = splits;
  L.dl = g.dL;
  L.d = g.d;
  L.st = g.st;
  L.S = g.S;
  L.kx = cw[0];
  fh_line_solve_cached(L, g.sN, 0.0, g.C1, buf);
}

struct TgYLine {
  long long base, ld;  // line i: element q at base + q*ld
  const double *V2, *C, *part, *al_, *gg;
  double *Cw, *Cfull, *Dj;
  long long ldp;
  int splits, M;
  double dl, d, st, S, ky, kyh;
  __device__ long long id(int q) const { return base + (long long)q * ld; }
  __device__ double A(int q) const { return (V2[id(q)] / (dl * dl)) * 0.5 * (d + d); }
  __device__ double om(int q) const {
    const long long k = id(q);
    double ts = 0.0;
    for (int s = 0; s < splits; ++s) ts += part[(long long)(2 * s + 1) * ldp + k];
    const double c = C[k];
    ts += (kyh + 0.0) * (Cfull[k] - c);  // old[size-2] - old[size-1] (fr_d_t_g_2d.cpp:3478-3481)
    double o = -st * (ky + 0.0) * c;
    o += S * 0.5;
    o += st * ts;
    return o;
  }
  __device__ double g(int q) const { return gg[id(q)]; }
  __device__ double al(int q) const { return al_[id(q)]; }
  __device__ void store(int q, double u) const {
    const long long k = id(q);
    if (q >= 1 && q < M) {
      Dj[k] = u - Cfull[k];
      Cfull[k] = u;
    }
    Cw[k] = u;
  }
};

__global__ void k_tg_ysweep(fh_tg_dev g, const double *__restrict__ V2, double *C,
                            double *Cfull, double *__restrict__ Dj, const double *__restrict__ part,
                            long long ldp, int splits, const double *__restrict__ al,
                            const double *__restrict__ gg, const double *__restrict__ cw) {
  extern __shared__ double sbuf[];
  const int warp = threadIdx.x >> 5;
  const int line = 1 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (line >= g.sN) return;
  double *buf = sbuf + (size_t)warp * (g.M + 1);
  TgYLine L;
  L.base = line;
  L.ld = g.ld;
  L.V2 = V2;
  L.C = C;
  L.part = part;
  L.al_ = al;
  L.gg = gg;
  L.Cw = C;
  L.Cfull = Cfull;
  L.Dj = Dj;
  L.ldp = ldp;
  L.splits = splits;
  L.M = g.M;
  L.dl = g.dLx;
  L.d = g.d;
  L.st = g.st;
  L.S = g.S;
  L.ky = cw[1];
  L.kyh = cw[2];
  fh_line_solve_cached(L, g.M, 1.0, 0.0, buf);
}

// ------------------------------------------------------------------ host

static constexpr int kSweepWarps = 4;

static int tg_factor(fh_tg_solver *s) {
  fh_ctx *ctx = s->ctx;
  const fh_tg_dev &g = s->dv;
  k_tg_factor<<<(unsigned)fh_ceil_div(g.M, 64), 64, 0, ctx->stream>>>(g, 0, s->V2.as<double>(), s->cw.as<double>(),
                                                                     s->alx.as<double>(), s->gx.as<double>());
  int rc = fh_after_launch(ctx, "k_tg_factor(x)");
  if (rc) return rc;
  k_tg_factor<<<(unsigned)fh_ceil_div(g.sN, 64), 64, 0, ctx->stream>>>(g, 1, s->V2.as<double>(), s->cw.as<double>(),
                                                                      s->aly.as<double>(), s->gy.as<double>());
  return fh_after_launch(ctx, "k_tg_factor(y)");
}

static int tg_one_step(fh_tg_solver *s) {
  fh_ctx *ctx = s->ctx;
  const fh_tg_dev &g = s->dv;
  const int j = s->tstep;
  const int ldw = s->max_steps;
  int rc;
  fh_prof_mark(ctx, FH_PROF_WEIGHTS, false);
  k_tg_weights<<<(unsigned)fh_ceil_div(j > 0 ? j : 1, 128), 128, 0, ctx->stream>>>(g, j, s->W.as<double>(), ldw,
                                                                                   s->cw.as<double>());
  fh_prof_mark(ctx, FH_PROF_WEIGHTS, true);
  if ((rc = fh_after_launch(ctx, "k_tg_weights"))) return rc;
  if (!s->factor_fixed || j == 0)
    if ((rc = tg_factor(s))) return rc;
  int splits = 0, kchunk = 0;
  if (j >= 1) {
    fh_hist_plan(g.P, j, s->max_splits, &splits, &kchunk);
    if ((rc = fh_launch_hist_sum_partials(ctx, 2, j, g.P, s->W.as<double>(), ldw, s->D.as<double>(), g.P, splits,
                                          kchunk, s->part.as<double>(), g.P)))
      return rc;
  }
  const unsigned thr = 32 * kSweepWarps;
  fh_prof_mark(ctx, FH_PROF_SWEEP, false);
  size_t smx = sizeof(double) * (size_t)kSweepWarps * (g.sN + 1);
  k_tg_xsweep<<<(unsigned)fh_ceil_div(g.M - 1, kSweepWarps), thr, smx, ctx->stream>>>(
      g, s->V2.as<double>(), s->C.as<double>(), s->part.as<double>(), g.P, splits, s->alx.as<double>(),
      s->gx.as<double>(), s->cw.as<double>());
  if ((rc = fh_after_launch(ctx, "k_tg_xsweep"))) return rc;
  size_t smy = sizeof(double) * (size_t)kSweepWarps * (g.M + 1);
  k_tg_ysweep<<<(unsigned)fh_ceil_div(g.sN - 1, kSweepWarps), thr, smy, ctx->stream>>>(
      g, s->V2.as<double>(), s->C.as<double>(), s->Cfull.as<double>(), s->D.as<double>() + (long long)j * g.P,
      s->part.as<double>(), g.P, splits, s->aly.as<double>(), s->gy.as<double>(), s->cw.as<double>());
  fh_prof_mark(ctx, FH_PROF_SWEEP, true);
  if ((rc = fh_after_launch(ctx, "k_tg_ysweep"))) return rc;
  s->tstep++;
  return FH_OK;
}

extern "C" {

int fh_tg_create(fh_ctx *ctx, const fh_tg_params *p, int max_steps, int mode, fh_tg_solver **out) {
  FH_REQUIRE(ctx, ctx && p && out, FH_EINVAL, "fh_tg_create: null argument");
  *out = nullptr;
  FH_REQUIRE(ctx, p->sN >= 2 && p->M >= 2 && p->sN <= 4096 && p->M <= 4096, FH_EINVAL,
             "fh_tg_create: need 2 <= sN, M <= 4096");
  FH_REQUIRE(ctx, p->alpha > 0.0 && p->alpha < 1.0 && p->beta > 0.0 && p->tau > 0.0, FH_EINVAL,
             "fh_tg_create: need 0 < alpha < 1, beta > 0, tau > 0");
  FH_REQUIRE(ctx, p->dL > 0.0 && p->dLx > 0.0 && p->sigma > 0.0, FH_EINVAL, "fh_tg_create: bad geometry");
  FH_REQUIRE(ctx, max_steps >= 1, FH_EINVAL, "fh_tg_create: max_steps >= 1");
  FH_REQUIRE(ctx, mode == FH_TG_FP64, FH_ENOTSUP, "fh_tg_create: mode %d not available in this build", mode);
  fh_tg_solver *s = new fh_tg_solver();
  s->ctx = ctx;
  s->p = *p;
  s->mode = mode;
  s->max_steps = max_steps;
  fh_tg_dev &g = s->dv;
  g.sN = p->sN;
  g.M = p->M;
  g.ld = p->sN + 2;
  g.P = (long long)(p->sN + 2) * (p->M + 2);
  if (g.P & 1) g.P += 1;  // even pitch for 16-byte history loads
  g.tau = p->tau;
  g.alpha = p->alpha;
  g.beta = p->beta;
  g.Da = 1.0 / tgamma(1.0 - p->alpha);  // TG_solver ctor (fr_d_t_g_2d.cpp:2391-2394)
  g.st = p->sigma / p->tau;
  g.d = p->d;
  g.C1 = p->C1;
  g.S = p->S;
  g.dL = p->dL;
  g.dLx = p->dLx;
  s->factor_fixed = (p->beta == 1.0);
  const size_t fld = sizeof(double) * (size_t)g.P;
  int rc;
  if ((rc = fh_alloc(ctx, s->C, fld)) || (rc = fh_alloc(ctx, s->Cfull, fld)) || (rc = fh_alloc(ctx, s->V2, fld)) ||
      (rc = fh_alloc(ctx, s->alx, fld)) || (rc = fh_alloc(ctx, s->gx, fld)) || (rc = fh_alloc(ctx, s->aly, fld)) ||
      (rc = fh_alloc(ctx, s->gy, fld)) || (rc = fh_alloc(ctx, s->D, fld * (size_t)max_steps)) ||
      (rc = fh_alloc(ctx, s->W, sizeof(double) * 2 * (size_t)max_steps)) ||
      (rc = fh_alloc(ctx, s->cw, sizeof(double) * 4)) ||
      (rc = fh_alloc(ctx, s->part, fld * 2 * (size_t)s->max_splits, false))) {
    delete s;
    return rc;
  }
  *out = s;
  return FH_OK;
}

int fh_tg_destroy(fh_tg_solver *s) {
  if (!s) return FH_OK;
  if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
  delete s;
  return FH_OK;
}

int fh_tg_set_state(fh_tg_solver *s, const double *V2, const double *C) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_state: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, V2 && C, FH_EINVAL, "fh_tg_set_state: null pointer");
  const size_t n = sizeof(double) * (size_t)(s->p.sN + 2) * (s->p.M + 2);
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->V2.p, V2, n, cudaMemcpyDeviceToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->C.p, C, n, cudaMemcpyDeviceToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->Cfull.p, C, n, cudaMemcpyDeviceToDevice, ctx->stream));
  s->tstep = 0;
  s->have_state = true;
  return FH_OK;
}

int fh_tg_set_state_host(fh_tg_solver *s, const double *V2_host, const double *C_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_state_host: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, V2_host && C_host, FH_EINVAL, "fh_tg_set_state_host: null pointer");
  const size_t n = sizeof(double) * (size_t)(s->p.sN + 2) * (s->p.M + 2);
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->V2.p, V2_host, n, cudaMemcpyHostToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->C.p, C_host, n, cudaMemcpyHostToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->Cfull.p, s->C.p, n, cudaMemcpyDeviceToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  s->tstep = 0;
  s->have_state = true;
  return FH_OK;
}

int fh_tg_step(fh_tg_solver *s, int nsteps) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_step: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, s->have_state, FH_EINVAL, "fh_tg_step: state not set");
  FH_REQUIRE(ctx, nsteps >= 0, FH_EINVAL, "fh_tg_step: nsteps < 0");
  FH_REQUIRE(ctx, s->tstep + nsteps <= s->max_steps, FH_ENOMEM, "fh_tg_step: history full (%d + %d > %d)", s->tstep,
             nsteps, s->max_steps);
  for (int n = 0; n < nsteps; ++n) {
    int rc = tg_one_step(s);
    if (rc) return rc;
  }
  return FH_OK;
}

int fh_tg_get_c_host(fh_tg_solver *s, double *C_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_get_c_host: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, C_host, FH_EINVAL, "fh_tg_get_c_host: null pointer");
  const size_t n = sizeof(double) * (size_t)(s->p.sN + 2) * (s->p.M + 2);
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(C_host, s->C.p, n, cudaMemcpyDeviceToHost, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FH_OK;
}

const double *fh_tg_field(const fh_tg_solver *s) { return s ? s->C.as<double>() : nullptr; }

int fh_tg_tstep(const fh_tg_solver *s) { return s ? s->tstep : -1; }

}  // extern "C"
