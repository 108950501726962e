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

struct fh_graph_cache;

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

struct fh_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  long long launches = 0;
  bool prof = false;
  bool graphs = true;  // whole solves from the initial state replay a captured graph
  fh_prof_kind pk[FH_PROF_KINDS];
  fh_graph_cache *capturing = nullptr;  // graph being captured (profiling marks become graph nodes)
  fh_dbuf work;  // scratch of the stateless entry points (fh_ctx_work)
  char err[512] = {0};
};

// Scratch of at least `bytes` for work enqueued on ctx->stream: the context's
// buffer, grown when too small (the stream is synchronised before the old
// buffer is freed), so repeated calls of one size neither allocate nor
// synchronise.
int fh_ctx_work(fh_ctx *ctx, size_t bytes, void **out);

// Records the start (stop = false) or stop event of a timed launch of `kind`
// on `stream` (the context stream when null).
void fh_prof_mark(fh_ctx *ctx, int kind, bool stop, cudaStream_t stream = nullptr);

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

// Replays a captured launch sequence: the first run of `nsteps` steps from the
// initial state is recorded by stream capture and instantiated; later runs
// from the same initial state launch the graph.  With profiling on, the
// start/stop marks are captured as external event-record nodes; after every
// replay the stream is synchronised and their intervals are added to the
// context's totals.
struct fh_graph_cache {
  cudaGraphExec_t exec = nullptr;
  int nsteps = -1;
  bool prof = false;                        // captured with profiling marks
  long long kernels = 0;                    // kernel launches in the graph
  std::vector<cudaEvent_t> pev[FH_PROF_KINDS];  // start/stop pairs baked into the graph
  void release_events() {
    for (auto &v : pev) {
      for (auto e : v) cudaEventDestroy(e);
      v.clear();
    }
  }
  void reset() {  // forget the captured graph (the launch sequence changed)
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    nsteps = -1;
    release_events();
  }
  ~fh_graph_cache() {
    if (exec) cudaGraphExecDestroy(exec);
    release_events();
  }
};

// Adds the intervals of the graph's profiling pairs (after a synchronised replay).
void fh_prof_collect_graph(fh_ctx *ctx, fh_graph_cache &gc);

// Runs body() (which enqueues the launches of `nsteps` steps on ctx->stream)
// under capture the first time and replays it afterwards.  body must only
// enqueue work (no synchronisation, no allocation).
template <class Body>
int fh_graph_run(fh_ctx *ctx, fh_graph_cache &gc, int nsteps, Body body) {
  if (!(gc.exec && gc.nsteps == nsteps && gc.prof == ctx->prof)) {
    if (gc.exec) {
      cudaGraphExecDestroy(gc.exec);
      gc.exec = nullptr;
    }
    gc.release_events();
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fh_set_error(ctx, FH_ECUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e));
    const long long l0 = ctx->launches;
    ctx->capturing = &gc;
    const int rc = body();
    ctx->capturing = nullptr;
    e = cudaStreamEndCapture(ctx->stream, &graph);
    gc.kernels = ctx->launches - l0;
    ctx->launches = l0;  // counted when the graph runs
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      gc.release_events();
      return rc;
    }
    if (e != cudaSuccess) {
      gc.release_events();
      return fh_set_error(ctx, FH_ECUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(&gc.exec, graph, cudaGraphInstantiateFlagUseNodePriority);  // launch priorities hold
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      gc.exec = nullptr;
      gc.release_events();
      return fh_set_error(ctx, FH_ECUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    }
    gc.nsteps = nsteps;
    gc.prof = ctx->prof;
  }
  cudaError_t e = cudaGraphLaunch(gc.exec, ctx->stream);
  if (e != cudaSuccess) return fh_set_error(ctx, FH_ECUDA, "cudaGraphLaunch: %s", cudaGetErrorString(e));
  ctx->launches += gc.kernels;
  if (gc.prof) {
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fh_set_error(ctx, FH_ECUDA, "graph replay: %s", cudaGetErrorString(e));
    fh_prof_collect_graph(ctx, gc);
  }
  return FH_OK;
}

int fh_alloc(fh_ctx *ctx, fh_dbuf &b, size_t bytes, bool zero = true);

// ---- launch helpers implemented in the kernel translation units ----
int fh_launch_weights_psi(fh_ctx *ctx, int K, double x0, double len, double X, double tau, double alpha,
                          double beta, double scale, double *w);
int fh_launch_hist_sum_partials(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw,
                                const double *D, long long ldd, int splits, int kchunk, double *part,
                                long long ldpart);
// S[p] = sum_s part[s*ldpart + p] in split order (S may alias split 0).
int fh_launch_reduce_splits(fh_ctx *ctx, int splits, long long P, const double *part, long long ldpart, double *S);
// History stored as (hi, lo) FP32 pairs, double-float accumulation; split 0
// starts from far[m*ldfar + p] (a (hi, lo) pair per point) when far != null.
// The partial sums are doubles, or (hi, lo) pairs when pair_out.
int fh_launch_hist_sum_df_partials(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw,
                                   const float2 *D, long long ldd, int splits, int kchunk, double *part,
                                   long long ldpart, const float2 *far, long long ldfar, int pair_out);
// Chooses the split count for a K x P history sum given a partial-buffer capacity.
void fh_hist_plan(long long P, int K, int max_splits, int *splits, int *kchunk);
