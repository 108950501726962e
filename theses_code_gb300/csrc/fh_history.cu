// fh_history.cu -- FP64 history sums S_m[p] = sum_k W[m][k] * D[k][p].
//
// Layout: D is layer-major (layer k at D + k*ldd), point index contiguous, so a
// warp reads 32 consecutive double2 (512 B) per layer.  Each CTA owns a tile of
// 2*blockDim points and one K-chunk ("split"); it stages its chunk of weights
// in shared memory and writes one partial sum per (split, m, point).  The
// consumer adds the partials in split order, so results do not depend on
// scheduling (no atomics).
//
// Cost model: every element of D is read once per step and used in M FMAs.
// On GB300 the FP64 pipe, not HBM, bounds this loop once M >= 1.
#include "fh_internal.h"
#include "fh_common.cuh"

static constexpr int kHistThreads = 256;

// Weights of at most kHistStage layers per row are staged in shared memory at
// a time (32 KiB for M = 2): a split of any length walks its layers in
// stages, in order, so the sum is the same as with one stage and the kernel
// never needs more than the default 48 KiB of dynamic shared memory.
static constexpr int kHistStage = 2048;

template <int M>
__global__ void __launch_bounds__(kHistThreads) k_hist_sum(const double *__restrict__ D, long long ldd, long long P,
                                                           int K, const double *__restrict__ W, int ldw, int kchunk,
                                                           double *__restrict__ part, long long ldpart) {
  extern __shared__ double ws[];  // [M][min(kchunk, kHistStage)]
  const int s = blockIdx.y;
  const int k0 = s * kchunk;
  const int nk = min(K, k0 + kchunk) - k0;
  const int ldws = min(kchunk, kHistStage);
  const long long p = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 2;
  const bool live = p < P;
  double acc0[M], acc1[M];
#pragma unroll
  for (int m = 0; m < M; ++m) acc0[m] = acc1[m] = 0.0;
  const double *d = D + (long long)k0 * ldd + (live ? p : 0);
  for (int kb = 0; kb < nk; kb += ldws) {
    const int ns = min(ldws, nk - kb);
    if (kb > 0) __syncthreads();  // every thread is done with the previous stage
    for (int i = threadIdx.x; i < M * ns; i += blockDim.x) {
      const int m = i / ns, k = i - m * ns;
      ws[m * ldws + k] = W[(long long)m * ldw + k0 + kb + k];
    }
    __syncthreads();
    if (!live) continue;
    int k = 0;
    for (; k + 4 <= ns; k += 4) {
      const double2 v0 = fh_ld_stream2(d);
      const double2 v1 = fh_ld_stream2(d + ldd);
      const double2 v2 = fh_ld_stream2(d + 2 * ldd);
      const double2 v3 = fh_ld_stream2(d + 3 * ldd);
      d += 4 * ldd;
#pragma unroll
      for (int m = 0; m < M; ++m) {
        const double *wm = ws + m * ldws + k;
        acc0[m] = fma(wm[0], v0.x, acc0[m]);
        acc1[m] = fma(wm[0], v0.y, acc1[m]);
        acc0[m] = fma(wm[1], v1.x, acc0[m]);
        acc1[m] = fma(wm[1], v1.y, acc1[m]);
        acc0[m] = fma(wm[2], v2.x, acc0[m]);
        acc1[m] = fma(wm[2], v2.y, acc1[m]);
        acc0[m] = fma(wm[3], v3.x, acc0[m]);
        acc1[m] = fma(wm[3], v3.y, acc1[m]);
      }
    }
    for (; k < ns; ++k) {
      const double2 v = fh_ld_stream2(d);
      d += ldd;
#pragma unroll
      for (int m = 0; m < M; ++m) {
        acc0[m] = fma(ws[m * ldws + k], v.x, acc0[m]);
        acc1[m] = fma(ws[m * ldws + k], v.y, acc1[m]);
      }
    }
  }
  if (!live) return;
#pragma unroll
  for (int m = 0; m < M; ++m) {
    double2 o;
    o.x = acc0[m];
    o.y = acc1[m];
    *reinterpret_cast<double2 *>(part + ((long long)s * M + m) * ldpart + p) = o;
  }
}

// Double-float variant: D holds (hi, lo) FP32 pairs (value = hi + lo, 2^-48
// relative), the weights are split into pairs in shared memory, and the M sums
// are carried as double-float with TwoSum on the FP32 pipe; partials are
// written as FP64 (hi + lo).  On GB300 the FP32 pipe delivers ~56x the FP64
// FMA rate, so this form streams the history at HBM speed.
template <int M>
__global__ void __launch_bounds__(kHistThreads) k_hist_sum_df(const float2 *__restrict__ D, long long ldd, long long P,
                                                              int K, const double *__restrict__ W, int ldw,
                                                              int kchunk, double *__restrict__ part,
                                                              long long ldpart, const float2 *__restrict__ far,
                                                              long long ldfar, int pair_out) {
  extern __shared__ float2 wsf[];  // [M][kchunk] (hi, lo)
  const int s = blockIdx.y;
  const int k0 = s * kchunk;
  const int nk = min(K, k0 + kchunk) - k0;
  for (int i = threadIdx.x; i < M * nk; i += blockDim.x) {
    const int m = i / nk, k = i - m * nk;
    const double w = W[(long long)m * ldw + k0 + k];
    const float wh = __double2float_rn(w);
    wsf[m * kchunk + k] = make_float2(wh, __double2float_rn(w - (double)wh));
  }
  __syncthreads();
  const long long p = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 2;
  if (p >= P) return;
  float ah[M][2], al[M][2];
#pragma unroll
  for (int m = 0; m < M; ++m) {
    if (far && s == 0) {  // split 0 starts from the far-history pair of row m
      const float4 f = *reinterpret_cast<const float4 *>(far + (long long)m * ldfar + p);
      ah[m][0] = f.x;
      al[m][0] = f.y;
      ah[m][1] = f.z;
      al[m][1] = f.w;
    } else {
      ah[m][0] = ah[m][1] = al[m][0] = al[m][1] = 0.f;
    }
  }
  const float4 *d = reinterpret_cast<const float4 *>(D + (long long)k0 * ldd + p);
  const long long ld4 = ldd / 2;  // float4 = two points
  auto acc = [&](const float2 w, const float dh, const float dl, float &sh, float &sl) {
    const float ph = w.x * dh;
    float pl = fmaf(w.x, dh, -ph);
    pl = fmaf(w.x, dl, pl);
    pl = fmaf(w.y, dh, pl);
    const float t = sh + ph;
    const float bb = t - sh;
    const float e = (sh - (t - bb)) + (ph - bb);
    sh = t;
    sl += e + pl;
  };
  int k = 0;
  for (; k + 8 <= nk; k += 8) {  // eight layers (128 B per thread) in flight
    float4 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldcs(d + u * ld4);
    d += 8 * ld4;
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int m = 0; m < M; ++m) {
        const float2 w = wsf[m * kchunk + k + u];
        acc(w, v[u].x, v[u].y, ah[m][0], al[m][0]);
        acc(w, v[u].z, v[u].w, ah[m][1], al[m][1]);
      }
    if ((k & 15) == 8) {
#pragma unroll
      for (int m = 0; m < M; ++m)
#pragma unroll
        for (int q = 0; q < 2; ++q) {  // renormalise (fast two-sum, |ah| >= |al|)
          const float t = ah[m][q] + al[m][q];
          al[m][q] = al[m][q] - (t - ah[m][q]);
          ah[m][q] = t;
        }
    }
  }
  for (; k < nk; ++k) {
    const float4 v = __ldcs(d);
    d += ld4;
#pragma unroll
    for (int m = 0; m < M; ++m) {
      const float2 w = wsf[m * kchunk + k];
      acc(w, v.x, v.y, ah[m][0], al[m][0]);
      acc(w, v.z, v.w, ah[m][1], al[m][1]);
    }
  }
#pragma unroll
  for (int m = 0; m < M; ++m) {
    if (pair_out) {  // renormalised (hi, lo) pairs for double-float consumers
      float4 o;
      o.x = ah[m][0] + al[m][0];
      o.y = al[m][0] - (o.x - ah[m][0]);
      o.z = ah[m][1] + al[m][1];
      o.w = al[m][1] - (o.z - ah[m][1]);
      *reinterpret_cast<float4 *>(reinterpret_cast<float2 *>(part) + ((long long)s * M + m) * ldpart + p) = o;
    } else {
      double2 o;
      o.x = (double)ah[m][0] + (double)al[m][0];
      o.y = (double)ah[m][1] + (double)al[m][1];
      *reinterpret_cast<double2 *>(part + ((long long)s * M + m) * ldpart + p) = o;
    }
  }
}

int fh_launch_hist_sum_df_partials(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw,
                                   const float2 *D, long long ldd, int splits, int kchunk, double *part,
                                   long long ldpart, const float2 *far, long long ldfar, int pair_out) {
  if (K <= 0 || P <= 0) return FH_OK;
  // short sums are a single wave: smaller CTAs even out the load per SM
  const int threads = K <= 64 ? kHistThreads / 2 : kHistThreads;
  dim3 grid((unsigned)fh_ceil_div(P, 2LL * threads), (unsigned)splits);
  const size_t smem = sizeof(float2) * (size_t)M * (size_t)kchunk;
  FH_REQUIRE(ctx, smem <= 48 * 1024, FH_EINVAL, "history chunk too large (%d layers)", kchunk);
  fh_prof_mark(ctx, FH_PROF_HISTORY, false);
  if (M == 1)
    k_hist_sum_df<1><<<grid, threads, smem, ctx->stream>>>(D, ldd, P, K, W, ldw, kchunk, part, ldpart, far, ldfar,
                                                             pair_out);
  else
    k_hist_sum_df<2><<<grid, threads, smem, ctx->stream>>>(D, ldd, P, K, W, ldw, kchunk, part, ldpart, far, ldfar,
                                                             pair_out);
  fh_prof_mark(ctx, FH_PROF_HISTORY, true);
  return fh_after_launch(ctx, "k_hist_sum_df");
}

// out[m*ldS + p] = sum_s part[(s*M+m)*ldpart + p]
__global__ void k_hist_reduce(int M, int splits, long long P, const double *__restrict__ part, long long ldpart,
                              double *__restrict__ S, long long ldS) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  for (int m = 0; m < M; ++m) {
    double acc = 0.0;
    for (int s = 0; s < splits; ++s) acc += part[((long long)s * M + m) * ldpart + p];
    S[(long long)m * ldS + p] = acc;
  }
}

// Layer form: S[p] = sum_t w[t] * (H[(t+1) ldh + p] - H[t ldh + p]) (reference Sum kernel semantics).
// Split y sums the layers [y kchunk, (y + 1) kchunk) into part[y][p]
// (coalesced over p; the split's first difference reads its lower layer).
__global__ void k_hist_sum_layers(int K, long long P, const double *__restrict__ w, const double *__restrict__ H,
                                  long long ldh, int kchunk, double *__restrict__ part, long long ldpart) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int t0 = blockIdx.y * kchunk, t1 = min(K, t0 + kchunk);
  double acc = 0.0;
  double prev = t0 < t1 ? H[(long long)t0 * ldh + p] : 0.0;
  for (int t = t0; t < t1; ++t) {
    const double cur = __ldcs(H + (long long)(t + 1) * ldh + p);
    acc = fma(__ldg(w + t), cur - prev, acc);
    prev = cur;
  }
  part[(long long)blockIdx.y * ldpart + p] = acc;
}

// S[p] = sum_s part[s][p] in split order: 8 warps take every 8th split for 32
// points (coalesced), then the 8 warp sums are added in warp order.
__global__ void __launch_bounds__(256) k_reduce_splits(int splits, long long P, const double *part,
                                                       long long ldpart, double *S) {
  __shared__ double acc8[8][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long p = (long long)blockIdx.x * 32 + lane;
  double a0 = 0.0, a1 = 0.0;
  if (p < P) {
    int s = warp;
    for (; s + 8 < splits; s += 16) {
      a0 += part[(long long)s * ldpart + p];
      a1 += part[(long long)(s + 8) * ldpart + p];
    }
    if (s < splits) a0 += part[(long long)s * ldpart + p];
  }
  acc8[warp][lane] = a0 + a1;
  __syncthreads();
  if (warp == 0 && p < P) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += acc8[w][lane];
    S[p] = t;
  }
}

int fh_launch_reduce_splits(fh_ctx *ctx, int splits, long long P, const double *part, long long ldpart, double *S) {
  fh_prof_mark(ctx, FH_PROF_HISTORY, false);
  k_reduce_splits<<<(unsigned)fh_ceil_div(P, 32), 256, 0, ctx->stream>>>(splits, P, part, ldpart, S);
  fh_prof_mark(ctx, FH_PROF_HISTORY, true);
  return fh_after_launch(ctx, "k_reduce_splits");
}

void fh_hist_plan(long long P, int K, int max_splits, int *splits, int *kchunk) {
  // Enough CTAs for ~3 waves of 8 resident 256-thread CTAs on 152 SMs, but at
  // least 32 layers per split so the partial traffic stays small.
  const long long tiles = fh_ceil_div(P, 2LL * kHistThreads);
  const long long target = 3LL * 152 * 8;
  int s = (int)fh_ceil_div(target, tiles);
  if (s > max_splits) s = max_splits;
  if (s > K / 32) s = K / 32;
  if (s < 1) s = 1;
  int kc = (int)fh_ceil_div(K, s);
  kc = (int)fh_ceil_div(kc, 4) * 4;
  s = (int)fh_ceil_div(K, kc);
  *splits = s;
  *kchunk = kc;
}

int fh_launch_hist_sum_partials(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw, const double *D,
                                long long ldd, int splits, int kchunk, double *part, long long ldpart) {
  if (K <= 0 || P <= 0) return FH_OK;
  dim3 grid((unsigned)fh_ceil_div(P, 2LL * kHistThreads), (unsigned)splits);
  FH_REQUIRE(ctx, kchunk >= 1, FH_EINVAL, "history chunk of %d layers", kchunk);
  const size_t smem = sizeof(double) * (size_t)M * (size_t)(kchunk < kHistStage ? kchunk : kHistStage);
  fh_prof_mark(ctx, FH_PROF_HISTORY, false);
  if (M == 1)
    k_hist_sum<1><<<grid, kHistThreads, smem, ctx->stream>>>(D, ldd, P, K, W, ldw, kchunk, part, ldpart);
  else
    k_hist_sum<2><<<grid, kHistThreads, smem, ctx->stream>>>(D, ldd, P, K, W, ldw, kchunk, part, ldpart);
  fh_prof_mark(ctx, FH_PROF_HISTORY, true);
  return fh_after_launch(ctx, "k_hist_sum");
}

extern "C" {

int fh_history_sum(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw, const double *D, long long ldd,
                   double *S, long long ldS) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, M == 1 || M == 2, FH_EINVAL, "fh_history_sum: M must be 1 or 2");
  FH_REQUIRE(ctx, K >= 0 && P >= 0 && ldS >= P && ldd >= P, FH_EINVAL, "fh_history_sum: bad sizes");
  FH_REQUIRE(ctx, (P % 2) == 0 && (ldd % 2) == 0, FH_EINVAL, "fh_history_sum: P and ldd must be even");
  FH_REQUIRE(ctx, ((uintptr_t)D % 16) == 0, FH_EINVAL, "fh_history_sum: D must be 16-byte aligned");
  if (P == 0) return FH_OK;
  FH_REQUIRE(ctx, S && (K == 0 || (W && D && ldw >= K)), FH_EINVAL, "fh_history_sum: null pointer");
  if (K == 0) {
    for (int m = 0; m < M; ++m)
      FH_CUDA_TRY(ctx, cudaMemsetAsync(S + (long long)m * ldS, 0, sizeof(double) * P, ctx->stream));
    return FH_OK;
  }
  int splits, kchunk;
  fh_hist_plan(P, K, 16, &splits, &kchunk);
  // the split partials in the context's workspace: allocated (with a
  // synchronisation) only when a call needs more than earlier calls did
  void *work = nullptr;
  int rc = fh_ctx_work(ctx, sizeof(double) * (size_t)splits * M * (size_t)P, &work);
  if (rc) return rc;
  double *part = static_cast<double *>(work);
  if ((rc = fh_launch_hist_sum_partials(ctx, M, K, P, W, ldw, D, ldd, splits, kchunk, part, P))) return rc;
  k_hist_reduce<<<(unsigned)fh_ceil_div(P, 256), 256, 0, ctx->stream>>>(M, splits, P, part, P, S, ldS);
  return fh_after_launch(ctx, "k_hist_reduce");
}

// Series accumulators of the irrigation model's sum_alg 2 (time_summing,
// irrigation_fractional.cpp:4150-4164): per point H[n] += c[n] d (the newest
// layer difference d) for n < J, then S = (sum_n e[n] H[n]) / tau, in the
// reference's operation order (no contraction into FMAs).  The step's
// coefficients travel by value.
struct fh_series_coefs {
  double c[FH_SERIES_MAX_TERMS], e[FH_SERIES_MAX_TERMS];
};
__global__ void __launch_bounds__(256) k_series_sum(int J, long long P, const fh_series_coefs cf, double tau,
                                                    const double *__restrict__ Dn, double *__restrict__ H,
                                                    long long ldh, double *__restrict__ S) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const double d = Dn[p];
  double sum = 0.0;
  double *h = H + p;
  for (int n = 0; n < J; ++n, h += ldh) {
    const double v = __dadd_rn(*h, __dmul_rn(cf.c[n], d));
    *h = v;
    sum = __dadd_rn(sum, __dmul_rn(cf.e[n], v));
  }
  S[p] = __ddiv_rn(sum, tau);
}

int fh_series_sum(fh_ctx *ctx, int J, long long P, const double *c_host, const double *e_host, double tau,
                  const double *Dn, double *H, long long ldh, double *S) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, J >= 1 && J <= FH_SERIES_MAX_TERMS && P >= 0 && ldh >= P, FH_EINVAL,
             "fh_series_sum: J = %d (1..%d), P = %lld, ldh = %lld", J, FH_SERIES_MAX_TERMS, P, ldh);
  FH_REQUIRE(ctx, c_host && e_host && tau != 0.0, FH_EINVAL, "fh_series_sum: coefficients or tau");
  if (P == 0) return FH_OK;
  FH_REQUIRE(ctx, Dn && H && S, FH_EINVAL, "fh_series_sum: null pointer");
  fh_series_coefs cf;
  for (int n = 0; n < FH_SERIES_MAX_TERMS; ++n) {
    cf.c[n] = n < J ? c_host[n] : 0.0;
    cf.e[n] = n < J ? e_host[n] : 0.0;
  }
  k_series_sum<<<(unsigned)fh_ceil_div(P, 256), 256, 0, ctx->stream>>>(J, P, cf, tau, Dn, H, ldh, S);
  return fh_after_launch(ctx, "k_series_sum");
}

int fh_history_sum_layers(fh_ctx *ctx, int K, long long P, const double *w, const double *H, long long ldh,
                          double *S) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, K >= 0 && P >= 0 && ldh >= P, FH_EINVAL, "fh_history_sum_layers: bad sizes");
  if (P == 0) return FH_OK;
  FH_REQUIRE(ctx, S && H && (K == 0 || w), FH_EINVAL, "fh_history_sum_layers: null pointer");
  // K splits when the points alone give too few CTAs: ~3 waves of 8 resident
  // CTAs on 152 SMs, at least 64 layers per split, at most 64 splits; the
  // splits' partial sums are added in split order
  const long long nb = fh_ceil_div(P, 256);
  long long s = fh_ceil_div(3LL * 152 * 8, nb);
  if (s > K / 64) s = K / 64;
  if (s > 64) s = 64;
  if (s < 1) s = 1;
  const int kchunk = (int)fh_ceil_div((long long)(K > 0 ? K : 1), s);
  const int splits = (int)fh_ceil_div((long long)(K > 0 ? K : 1), (long long)kchunk);
  double *part = S;
  if (splits > 1) {
    void *work = nullptr;
    int rc = fh_ctx_work(ctx, sizeof(double) * (size_t)splits * (size_t)P, &work);
    if (rc) return rc;
    part = static_cast<double *>(work);
  }
  k_hist_sum_layers<<<dim3((unsigned)nb, (unsigned)splits), 256, 0, ctx->stream>>>(K, P, w, H, ldh, kchunk, part, P);
  int rc = fh_after_launch(ctx, "k_hist_sum_layers");
  if (rc || splits == 1) return rc;
  return fh_launch_reduce_splits(ctx, splits, P, part, P, S);
}

}  // extern "C"
