// fh_internal.h -- host-side internals shared by the libfhist translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fhist.h"

struct fh_prof_kind {
  std::vector<cudaEvent_t> ev;  // start/stop pairs, recycled across reads
  size_t used = 0;               // events recorded since the last read
  double total_ms = 0.0;
  long long count = 0;
};

struct fh_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  long long launches = 0;
  bool prof = false;
  fh_prof_kind pk[3];
  char err[512] = {0};
};

// Records the start (stop = false) or stop event of a timed launch of `kind`.
void fh_prof_mark(fh_ctx *ctx, int kind, bool stop);

int fh_set_error(const fh_ctx *ctx, int code, const char *fmt, ...);

// Checks the last CUDA error after a launch and counts the launch.
int fh_after_launch(fh_ctx *ctx, const char *what);

#define FH_CUDA_TRY(ctx, call)                                                              \
  do {                                                                                      \
    cudaError_t _e = (call);                                                                \
    if (_e != cudaSuccess)                                                                  \
      return fh_set_error((ctx), FH_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), \
                          __FILE__, __LINE__);                                              \
  } while (0)

#define FH_REQUIRE(ctx, cond, code, ...)                      \
  do {                                                        \
    if (!(cond)) return fh_set_error((ctx), (code), __VA_ARGS__); \
  } while (0)

// Device allocation owned by an object; freed in its destructor.
struct fh_dbuf {
  void *p = nullptr;
  size_t bytes = 0;
  ~fh_dbuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T *as() const { return static_cast<T *>(p); }
};

int fh_alloc(fh_ctx *ctx, fh_dbuf &b, size_t bytes, bool zero = true);

// ---- launch helpers implemented in the kernel translation units ----
int fh_launch_weights_psi(fh_ctx *ctx, int K, double x0, double len, double X, double tau, double alpha,
                          double beta, double scale, double *w);
int fh_launch_hist_sum_partials(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw,
                                const double *D, long long ldd, int splits, int kchunk, double *part,
                                long long ldpart);
// Chooses the split count for a K x P history sum given a partial-buffer capacity.
void fh_hist_plan(long long P, int K, int max_splits, int *splits, int *kchunk);
