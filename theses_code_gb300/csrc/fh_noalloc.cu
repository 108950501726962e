// fh_noalloc.cu -- fh_history_sum_noalloc: the split-K history sum of
// fh_history_sum without any device allocation.
//
// Some callers cannot call cudaMalloc at the point where they need the history
// sum: applications that have handed all device memory to their own pool or
// that admit work against a fixed memory budget, and latency-critical step
// loops in which a cudaMalloc/cudaFree pair would synchronise the whole device.
// For them the split-K partial sums go to a fixed array reserved in device
// memory when the library is loaded (every GPU that loads the library holds it
// until the process exits).  The caller still passes W, D and S.
//
// The array is shared by every call of this entry point on a device and keeps
// the partials of the last call; each call overwrites every partial it reads,
// so nothing needs clearing.  Calls whose work overlaps on the GPU (two
// streams or contexts on the same device) race on the array and must be
// serialised by the caller.
#include <mutex>

#include "fh_common.cuh"
#include "fh_internal.h"

// Scratch for splits x M x P partial sums (16 MiB).
static __device__ __align__(256) double g_fh_noalloc_scratch[FH_NOALLOC_SCRATCH_DOUBLES];

static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[256];  // device address of the array, per device ordinal

// Once per device, with that device current: the host-side name of the array
// is only a stand-in, so its device address is looked up here and passed to
// the kernels.  This first lookup also loads the module on that device.
static int noalloc_scratch(fh_ctx *ctx, double **out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  FH_REQUIRE(ctx, ctx->device >= 0 && ctx->device < 256, FH_EINVAL, "device ordinal %d out of range", ctx->device);
  if (!g_noalloc_ptr[ctx->device]) {
    int cur = -1;
    FH_CUDA_TRY(ctx, cudaGetDevice(&cur));
    if (cur != ctx->device) FH_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_fh_noalloc_scratch);
    if (cur != ctx->device) cudaSetDevice(cur);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return fh_set_error(ctx, FH_ECUDA, "fh_history_sum_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    }
    g_noalloc_ptr[ctx->device] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[ctx->device];
  return FH_OK;
}

// S[m*ldS + p] = sum_s part[(s*M+m)*P + p], splits added in order.
__global__ void k_noalloc_reduce(int M, int splits, long long P, const double *__restrict__ part,
                                 double *__restrict__ S, long long ldS) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  for (int m = 0; m < M; ++m) {
    double acc = 0.0;
    for (int s = 0; s < splits; ++s) acc += part[((long long)s * M + m) * P + p];
    S[(long long)m * ldS + p] = acc;
  }
}

extern "C" int fh_history_sum_noalloc(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw,
                                      const double *D, long long ldd, double *S, long long ldS) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, M == 1 || M == 2, FH_EINVAL, "fh_history_sum_noalloc: M must be 1 or 2");
  FH_REQUIRE(ctx, K >= 0 && P >= 0 && ldS >= P && ldd >= P, FH_EINVAL, "fh_history_sum_noalloc: bad sizes");
  FH_REQUIRE(ctx, (P % 2) == 0 && (ldd % 2) == 0, FH_EINVAL, "fh_history_sum_noalloc: P and ldd must be even");
  FH_REQUIRE(ctx, ((uintptr_t)D % 16) == 0, FH_EINVAL, "fh_history_sum_noalloc: D must be 16-byte aligned");
  FH_REQUIRE(ctx, (long long)M * P <= FH_NOALLOC_SCRATCH_DOUBLES, FH_ERANGE,
             "fh_history_sum_noalloc: M*P = %lld exceeds the fixed scratch of %lld doubles", (long long)M * P,
             (long long)FH_NOALLOC_SCRATCH_DOUBLES);
  if (P == 0) return FH_OK;
  FH_REQUIRE(ctx, S && (K == 0 || (W && D && ldw >= K)), FH_EINVAL, "fh_history_sum_noalloc: null pointer");
  if (K == 0) {
    for (int m = 0; m < M; ++m)
      FH_CUDA_TRY(ctx, cudaMemsetAsync(S + (long long)m * ldS, 0, sizeof(double) * P, ctx->stream));
    return FH_OK;
  }
  double *scratch = nullptr;
  int rc = noalloc_scratch(ctx, &scratch);
  if (rc) return rc;
  long long cap = FH_NOALLOC_SCRATCH_DOUBLES / ((long long)M * P);
  const int max_splits = (int)(cap < 16 ? cap : 16);
  int splits, kchunk;
  fh_hist_plan(P, K, max_splits, &splits, &kchunk);
  if ((rc = fh_launch_hist_sum_partials(ctx, M, K, P, W, ldw, D, ldd, splits, kchunk, scratch, P))) return rc;
  k_noalloc_reduce<<<(unsigned)fh_ceil_div(P, 256), 256, 0, ctx->stream>>>(M, splits, P, scratch, S, ldS);
  return fh_after_launch(ctx, "k_noalloc_reduce");
}
