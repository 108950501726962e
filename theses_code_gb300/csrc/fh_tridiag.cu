// fh_tridiag.cu -- batched tridiagonal solvers.
//  * k_tridiag_batched: the reference Thomas sweep (alpha/beta form) with one
//    thread per system; the alpha coefficients live in a scratch array and
//    beta is kept in the solution array shifted by one slot.
//  * k_pcr: parallel cyclic reduction in shared memory, one CTA per system
//    (the published algorithm of Hockney / Zhang-Cohen-Owens 2010).
#include "fh_internal.h"
#include "fh_common.cuh"

__global__ void k_tridiag_batched(int nsys, int N, const double *__restrict__ A, const double *__restrict__ R,
                                  const double *__restrict__ B, const double *__restrict__ Om, long long lds,
                                  const double *__restrict__ al1, const double *__restrict__ bt1, int right_mode,
                                  const double *__restrict__ u_right, double *__restrict__ u, long long ldu,
                                  double *__restrict__ Al) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const double *a = A + s * lds, *r = R + s * lds, *b = B + s * lds, *om = Om + s * lds;
  double *x = u + s * ldu;
  double *al = Al + (long long)s * (N + 1);
  // forward sweep: Al[i+1] = B/(R - A Al[i]); Bt[i+1] = (Al[i+1]/B)(A Bt[i] - Om)
  // (H_solver::al1/bt1, mt_minimal.cpp:829-858, 942-980; TG_solver_::bt1 zero-B case fr_d_t_g_2d.cpp:3519-3522)
  double alv = al1[s], btv = bt1[s];
  al[1] = alv;
  x[0] = btv;  // x[i] holds Bt[i+1]
  for (int i = 1; i < N; ++i) {
    const double ai = a[i], bi = b[i], ri = r[i];
    const double den = ri - ai * alv;
    const double aln = bi / den;
    double btn;
    if (aln == 0.0 && bi == 0.0)
      btn = (ai * btv - om[i]) / den;
    else
      btn = (aln / bi) * (ai * btv - om[i]);
    al[i + 1] = aln;
    x[i] = btn;
    alv = aln;
    btv = btn;
  }
  double un = right_mode == 0 ? u_right[s] : btv / (1.0 - alv);
  x[N] = un;
  for (int i = N - 1; i >= 0; --i) {
    un = al[i + 1] * un + x[i];
    x[i] = un;
  }
  x[N + 1] = x[N];
}

// PCR: each level eliminates the couplings at distance s, after log2 levels
// every equation stands alone.  Rows outside [0, n) act as identity rows.
__global__ void k_pcr(const double *__restrict__ A, const double *__restrict__ Bd, const double *__restrict__ C,
                      const double *__restrict__ D, double *__restrict__ X, int n) {
  extern __shared__ double sm[];
  double *a = sm, *b = sm + n, *c = sm + 2 * n, *d = sm + 3 * n;
  const long long base = (long long)blockIdx.x * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    a[i] = (i == 0) ? 0.0 : A[base + i];
    b[i] = Bd[base + i];
    c[i] = (i == n - 1) ? 0.0 : C[base + i];
    d[i] = D[base + i];
  }
  __syncthreads();
  constexpr int kMaxPer = 8;  // n <= 8 * blockDim
  for (int s = 1; s < n; s <<= 1) {
    double na[kMaxPer], nb[kMaxPer], nc[kMaxPer], nd[kMaxPer];
    int cnt = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x, ++cnt) {
      const int lo = i - s, hi = i + s;
      double ai = a[i], bi = b[i], ci = c[i], di = d[i];
      double k1 = 0.0, k2 = 0.0, alo = 0.0, clo = 0.0, dlo = 0.0, ahi = 0.0, chi = 0.0, dhi = 0.0;
      if (lo >= 0) {
        k1 = ai / b[lo];
        alo = a[lo];
        clo = c[lo];
        dlo = d[lo];
      }
      if (hi < n) {
        k2 = ci / b[hi];
        ahi = a[hi];
        chi = c[hi];
        dhi = d[hi];
      }
      na[cnt] = -alo * k1;
      nb[cnt] = bi - clo * k1 - ahi * k2;
      nc[cnt] = -chi * k2;
      nd[cnt] = di - dlo * k1 - dhi * k2;
    }
    __syncthreads();
    cnt = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x, ++cnt) {
      a[i] = na[cnt];
      b[i] = nb[cnt];
      c[i] = nc[cnt];
      d[i] = nd[cnt];
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) X[base + i] = d[i] / b[i];
}

extern "C" {

int fh_tridiag_batched(fh_ctx *ctx, int nsys, int N, const double *A, const double *R, const double *B,
                       const double *Om, long long lds, const double *al1, const double *bt1, int right_mode,
                       const double *u_right, double *u, long long ldu) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, nsys >= 0 && N >= 1 && lds >= N + 1 && ldu >= N + 2, FH_EINVAL, "fh_tridiag_batched: bad sizes");
  FH_REQUIRE(ctx, right_mode == 0 || right_mode == 1, FH_EINVAL, "fh_tridiag_batched: right_mode must be 0 or 1");
  if (nsys == 0) return FH_OK;
  FH_REQUIRE(ctx, A && R && B && Om && al1 && bt1 && u && (right_mode == 1 || u_right), FH_EINVAL,
             "fh_tridiag_batched: null pointer");
  // Al in the context's workspace: allocated (with a synchronisation) only
  // when a call needs more than earlier calls did
  void *al = nullptr;
  int rc = fh_ctx_work(ctx, sizeof(double) * (size_t)nsys * (size_t)(N + 1), &al);
  if (rc) return rc;
  k_tridiag_batched<<<(unsigned)fh_ceil_div(nsys, 128), 128, 0, ctx->stream>>>(
      nsys, N, A, R, B, Om, lds, al1, bt1, right_mode, u_right, u, ldu, static_cast<double *>(al));
  return fh_after_launch(ctx, "k_tridiag_batched");
}

int fh_pcr_solver(fh_ctx *ctx, const double *a, const double *b, const double *c, const double *d, double *x, int n,
                  int nsys) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, n >= 1 && n <= 2048 && nsys >= 0, FH_EINVAL, "fh_pcr_solver: need 1 <= n <= 2048");
  if (nsys == 0) return FH_OK;
  FH_REQUIRE(ctx, a && b && c && d && x, FH_EINVAL, "fh_pcr_solver: null pointer");
  const int threads = n < 256 ? ((n + 31) / 32) * 32 : 256;
  const size_t smem = sizeof(double) * 4 * (size_t)n;
  if (smem > 48 * 1024)  // opt-in on this context's device
    FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_pcr, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
  k_pcr<<<(unsigned)nsys, threads, smem, ctx->stream>>>(a, b, c, d, x, n);
  return fh_after_launch(ctx, "k_pcr");
}

}  // extern "C"
