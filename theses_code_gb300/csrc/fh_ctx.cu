// fh_ctx.cu -- context, error reporting and allocation for libfhist.
#include "fh_internal.h"

static char g_noctx_err[512];

int fh_set_error(const fh_ctx *ctx, int code, const char *fmt, ...) {
  char *dst = ctx ? const_cast<fh_ctx *>(ctx)->err : g_noctx_err;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(dst, 512, fmt, ap);
  va_end(ap);
  return code;
}

int fh_after_launch(fh_ctx *ctx, const char *what) {
  ctx->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fh_set_error(ctx, FH_ECUDA, "launch %s: %s", what, cudaGetErrorString(e));
  return FH_OK;
}

int fh_ctx_work(fh_ctx *ctx, size_t bytes, void **out) {
  if (ctx->work.bytes < bytes) {
    FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // earlier calls may still use the old buffer
    const int rc = fh_alloc(ctx, ctx->work, bytes + bytes / 4, false);
    if (rc) return rc;
  }
  *out = ctx->work.p;
  return FH_OK;
}

int fh_alloc(fh_ctx *ctx, fh_dbuf &b, size_t bytes, bool zero) {
  b.release();
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    b.p = nullptr;
    cudaGetLastError();
    return fh_set_error(ctx, FH_ENOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  b.bytes = bytes;
  if (zero) FH_CUDA_TRY(ctx, cudaMemsetAsync(b.p, 0, bytes, ctx->stream));
  return FH_OK;
}

void fh_prof_mark(fh_ctx *ctx, int kind, bool stop, cudaStream_t stream) {
  if (!ctx->prof) return;
  if (!stream) stream = ctx->stream;
  if (ctx->capturing) {
    // inside a capture: a fresh event per mark, recorded as a graph node
    std::vector<cudaEvent_t> &v = ctx->capturing->pev[kind];
    if (stop != ((v.size() & 1) == 1)) return;  // unbalanced mark: ignore
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    v.push_back(e);
    cudaEventRecordWithFlags(e, stream, cudaEventRecordExternal);
    return;
  }
  fh_prof_kind &k = ctx->pk[kind];
  if (k.used == k.ev.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    k.ev.push_back(e);
  }
  if (!stop && (k.used & 1)) return;  // unbalanced start: ignore
  cudaEventRecord(k.ev[k.used++], stream);
}

static void prof_collect(fh_ctx *ctx, int kind) {
  fh_prof_kind &k = ctx->pk[kind];
  for (size_t i = 0; i + 1 < k.used; i += 2) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, k.ev[i], k.ev[i + 1]) == cudaSuccess) {
      k.total_ms += ms;
      k.count++;
    } else {
      cudaGetLastError();
    }
  }
  k.used = 0;
}

void fh_prof_collect_graph(fh_ctx *ctx, fh_graph_cache &gc) {
  for (int kind = 0; kind < FH_PROF_KINDS; ++kind) {
    const std::vector<cudaEvent_t> &v = gc.pev[kind];
    for (size_t i = 0; i + 1 < v.size(); i += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, v[i], v[i + 1]) == cudaSuccess) {
        ctx->pk[kind].total_ms += ms;
        ctx->pk[kind].count++;
      } else {
        cudaGetLastError();
      }
    }
  }
}

static void prof_free(fh_ctx *ctx) {
  for (auto &k : ctx->pk) {
    for (auto e : k.ev) cudaEventDestroy(e);
    k.ev.clear();
    k.used = 0;
  }
}

extern "C" {

int fh_version(void) { return 10000; }

int fh_ctx_profile(fh_ctx *ctx, int enable) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (auto &k : ctx->pk) {
    k.used = 0;
    k.total_ms = 0.0;
    k.count = 0;
  }
  ctx->prof = enable != 0;
  return FH_OK;
}

int fh_ctx_profile_read(fh_ctx *ctx, int kind, double *total_ms, long long *launches) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, kind >= 0 && kind < FH_PROF_KINDS, FH_EINVAL, "fh_ctx_profile_read: bad kind");
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < FH_PROF_KINDS; ++k) prof_collect(ctx, k);
  if (total_ms) *total_ms = ctx->pk[kind].total_ms;
  if (launches) *launches = ctx->pk[kind].count;
  return FH_OK;
}

int fh_ctx_create(int device, fh_ctx **out) {
  if (!out) return fh_set_error(nullptr, FH_EINVAL, "fh_ctx_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fh_set_error(nullptr, FH_ECUDA, "no CUDA device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return fh_set_error(nullptr, FH_EINVAL, "device %d of %d", device, ndev);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return fh_set_error(nullptr, FH_ECUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  fh_ctx *c = new fh_ctx();
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fh_set_error(nullptr, FH_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  c->own_stream = true;
  *out = c;
  return FH_OK;
}

int fh_ctx_destroy(fh_ctx *ctx) {
  if (!ctx) return FH_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  prof_free(ctx);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return FH_OK;
}

const char *fh_last_error(const fh_ctx *ctx) { return ctx ? ctx->err : g_noctx_err; }

int fh_ctx_sync(fh_ctx *ctx) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FH_OK;
}

int fh_ctx_set_graphs(fh_ctx *ctx, int enable) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  ctx->graphs = enable != 0;
  return FH_OK;
}

int fh_ctx_query(fh_ctx *ctx) {
  if (!ctx) return -FH_EINVAL;
  const cudaError_t e = cudaStreamQuery(ctx->stream);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) {
    cudaGetLastError();
    return 0;
  }
  fh_set_error(ctx, FH_ECUDA, "cudaStreamQuery: %s", cudaGetErrorString(e));
  return -FH_ECUDA;
}

int fh_ctx_set_stream(fh_ctx *ctx, void *stream) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  if (ctx->own_stream && ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  ctx->stream = static_cast<cudaStream_t>(stream);
  ctx->own_stream = false;
  return FH_OK;
}

void *fh_ctx_get_stream(fh_ctx *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

long long fh_ctx_launch_count(const fh_ctx *ctx) { return ctx ? ctx->launches : 0; }

}  // extern "C"
