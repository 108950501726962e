// fh_common.cuh -- shared device helpers for libfhist (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fhist.h"

#define FH_WARP 32

// ---------------------------------------------------------------- loads
// History layers are read once per step and are far larger than L2 in the
// large configurations: stream them past L1.
__device__ __forceinline__ double2 fh_ld_stream2(const double *p) {
  return __ldcs(reinterpret_cast<const double2 *>(p));
}
__device__ __forceinline__ double fh_ld_stream(const double *p) { return __ldcs(p); }

// ------------------------------------------------------ affine warp scan
// Affine map x -> a*x + b.  compose(f2, f1) = f2 o f1 (apply f1 first).
struct fh_aff {
  double a, b;
};
__device__ __forceinline__ fh_aff fh_aff_compose(fh_aff f2, fh_aff f1) {
  return fh_aff{f2.a * f1.a, fma(f2.a, f1.b, f2.b)};
}

// Exclusive scan over the warp: lane l receives f_{l-1} o ... o f_0 (identity
// for lane 0).  All 32 lanes must participate.
__device__ __forceinline__ fh_aff fh_warp_exclusive_affine(fh_aff f) {
  const unsigned lane = threadIdx.x & 31u;
  // inclusive scan (Hillis-Steele): g_l = f_l o f_{l-1} o ... o f_0
  fh_aff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    double pa = __shfl_up_sync(0xffffffffu, g.a, d);
    double pb = __shfl_up_sync(0xffffffffu, g.b, d);
    if (lane >= (unsigned)d) g = fh_aff_compose(g, fh_aff{pa, pb});
  }
  double ea = __shfl_up_sync(0xffffffffu, g.a, 1);
  double eb = __shfl_up_sync(0xffffffffu, g.b, 1);
  if (lane == 0) {
    ea = 1.0;
    eb = 0.0;
  }
  return fh_aff{ea, eb};
}

// ----------------------------------------------------------- misc
__host__ __device__ __forceinline__ long long fh_ceil_div(long long a, long long b) { return (a + b - 1) / b; }
