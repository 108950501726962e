// fh_weights.cu -- history-weight kernels: psi-Caputo, L1 Caputo-Gerasimov,
// Atangana-Baleanu (Mittag-Leffler) and the Mittag-Leffler function itself.
#include "fh_internal.h"
#include "fh_weights.cuh"

__global__ void k_weights_psi(int K, double x0, double len, double X, double tau, double alpha, double beta,
                              double scale, double *__restrict__ w) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const double s0 = (double)k + x0;  // (i + _sa) of TG_solver_::kb
  w[k] = scale * fh_psi_int(s0, s0 + len, X, tau, alpha, beta);
}

// H_solver::Om1 L1 coefficients (mt_minimal.cpp:926-934).
__global__ void k_weights_l1(int os, double alpha, double *__restrict__ w) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= os - 1) return;
  w[t] = pow((double)(os - t), 1.0 - alpha) - pow((double)(os - t - 1), 1.0 - alpha);
}

// I(lag) = sum_k (-lam)^k / Gamma(a k + 2) * (x1^(a k+1) - x0^(a k+1)),
// lam = a/(1-a): the Mittag-Leffler series of MF_int integrated term by term,
// with 1 - (x0/x1)^p taken through expm1/log1p.
__global__ void k_weights_ab(int n, double tau, double alpha, double *__restrict__ w, int *__restrict__ flag) {
  const int lag = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (lag > n) return;
  const double a = alpha, lam = a / (1.0 - a);
  const double x1 = (double)lag * tau, lx1 = log(x1), llam = log(lam);
  const double lr = (lag >= 2) ? log1p(-1.0 / (double)lag) : 0.0;
  double s = 0.0, mx = 0.0;
  for (int k = 0; k < 2000; ++k) {
    const double p = a * k + 1.0;
    const double frac = (lag >= 2) ? -expm1(p * lr) : 1.0;
    double t = exp((double)k * llam + p * lx1 - lgamma(p + 1.0)) * frac;
    if (k & 1) t = -t;
    s += t;
    mx = fmax(mx, fabs(t));
    if (k > 4 && fabs(t) <= 1e-17 * fabs(s) && fabs(t) < mx) break;
  }
  if (!(mx <= 1e6 * fabs(s))) atomicOr(flag, 1);
  w[lag] = s;
  if (lag == 1) w[0] = s;
}

__global__ void k_mittag_leffler(int n, double a, double b, const double *__restrict__ z, double *__restrict__ out,
                                 int *__restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double zi = z[i];
  double s = 0.0, mx = 0.0;
  if (zi == 0.0) {
    s = 1.0 / tgamma(b);
    mx = fabs(s);
  } else {
    const double lz = log(fabs(zi));
    for (int k = 0; k < 4000; ++k) {
      double t = exp((double)k * lz - lgamma(a * k + b));
      if (zi < 0.0 && (k & 1)) t = -t;
      s += t;
      mx = fmax(mx, fabs(t));
      if (k > 4 && fabs(t) <= 1e-17 * fabs(s) && fabs(t) < mx) break;
    }
  }
  if (!(mx <= 1e6 * fabs(s))) atomicOr(flag, 1);
  out[i] = s;
}

int fh_launch_weights_psi(fh_ctx *ctx, int K, double x0, double len, double X, double tau, double alpha,
                          double beta, double scale, double *w) {
  if (K <= 0) return FH_OK;
  k_weights_psi<<<(unsigned)fh_ceil_div(K, 128), 128, 0, ctx->stream>>>(K, x0, len, X, tau, alpha, beta, scale, w);
  return fh_after_launch(ctx, "k_weights_psi");
}

static int check_flag(fh_ctx *ctx, int *dflag, const char *what) {
  int h = 0;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(&h, dflag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (h) return fh_set_error(ctx, FH_ERANGE, "%s: series cancellation beyond 6 digits", what);
  return FH_OK;
}

extern "C" {

int fh_weights_psi(fh_ctx *ctx, int K, double x0, double len, double X, double tau, double alpha, double beta,
                   double scale, double *w) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, K >= 0 && (K == 0 || w), FH_EINVAL, "fh_weights_psi: bad K/w");
  FH_REQUIRE(ctx, alpha > 0.0 && alpha < 1.0 && beta > 0.0 && tau > 0.0 && X > 0.0, FH_EINVAL,
             "fh_weights_psi: need 0<alpha<1, beta>0, tau>0, X>0");
  FH_REQUIRE(ctx, x0 >= 0.0 && len > 0.0 && x0 + (K - 1) + len <= X, FH_EINVAL,
             "fh_weights_psi: intervals must lie in [0, X]");
  return fh_launch_weights_psi(ctx, K, x0, len, X, tau, alpha, beta, scale, w);
}

int fh_weights_l1(fh_ctx *ctx, int os, double alpha, double *w) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, alpha > 0.0 && alpha < 1.0, FH_EINVAL, "fh_weights_l1: need 0<alpha<1");
  if (os < 2) return FH_OK;
  FH_REQUIRE(ctx, w, FH_EINVAL, "fh_weights_l1: w is NULL");
  k_weights_l1<<<(unsigned)fh_ceil_div(os - 1, 128), 128, 0, ctx->stream>>>(os, alpha, w);
  return fh_after_launch(ctx, "k_weights_l1");
}

int fh_weights_ab(fh_ctx *ctx, int n, double tau, double alpha, double *w) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, n >= 1 && w && tau > 0.0 && alpha > 0.0 && alpha < 1.0, FH_EINVAL, "fh_weights_ab: bad args");
  fh_dbuf flag;
  int rc = fh_alloc(ctx, flag, sizeof(int));
  if (rc) return rc;
  k_weights_ab<<<(unsigned)fh_ceil_div(n, 128), 128, 0, ctx->stream>>>(n, tau, alpha, w, flag.as<int>());
  if ((rc = fh_after_launch(ctx, "k_weights_ab"))) return rc;
  return check_flag(ctx, flag.as<int>(), "fh_weights_ab");
}

int fh_mittag_leffler(fh_ctx *ctx, int n, double a, double b, const double *z, double *out) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, n >= 0 && a > 0.0 && b > 0.0, FH_EINVAL, "fh_mittag_leffler: bad args");
  if (n == 0) return FH_OK;
  FH_REQUIRE(ctx, z && out, FH_EINVAL, "fh_mittag_leffler: null pointer");
  fh_dbuf flag;
  int rc = fh_alloc(ctx, flag, sizeof(int));
  if (rc) return rc;
  k_mittag_leffler<<<(unsigned)fh_ceil_div(n, 128), 128, 0, ctx->stream>>>(n, a, b, z, out, flag.as<int>());
  if ((rc = fh_after_launch(ctx, "k_mittag_leffler"))) return rc;
  return check_flag(ctx, flag.as<int>(), "fh_mittag_leffler");
}

}  // extern "C"
