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

// ------------------------------------------------------ Moebius maps
// x -> (m00 x + m01) / (m10 x + m11) as a 2x2 matrix acting on (x, 1).  The
// Thomas alpha recurrence Al[i+1] = B_i / (R_i - A_i Al[i]) is the matrix
// [[0, B_i], [-A_i, R_i]]; chunks compose by matrix products, rescaled by a
// power of two (exact) to keep the entries in range.
struct fh_mob {
  double m00, m01, m10, m11;
};
__device__ __forceinline__ fh_mob fh_mob_normalise(fh_mob t) {
  const double mx = fmax(fmax(fabs(t.m00), fabs(t.m01)), fmax(fabs(t.m10), fabs(t.m11)));
  if (!(mx > 0.0) || !isfinite(mx)) return t;
  int e;
  frexp(mx, &e);
  return fh_mob{ldexp(t.m00, -e), ldexp(t.m01, -e), ldexp(t.m10, -e), ldexp(t.m11, -e)};
}
// f2 o f1 (f1 applied first) = M2 * M1
__device__ __forceinline__ fh_mob fh_mob_compose(fh_mob f2, fh_mob f1) {
  return fh_mob{fma(f2.m00, f1.m00, f2.m01 * f1.m10), fma(f2.m00, f1.m01, f2.m01 * f1.m11),
                fma(f2.m10, f1.m00, f2.m11 * f1.m10), fma(f2.m10, f1.m01, f2.m11 * f1.m11)};
}
// Exclusive warp scan: lane l receives f_{l-1} o ... o f_0 (identity for lane 0).
__device__ __forceinline__ fh_mob fh_warp_exclusive_mob(fh_mob f) {
  const unsigned lane = threadIdx.x & 31u;
  fh_mob g = fh_mob_normalise(f);
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    fh_mob p;
    p.m00 = __shfl_up_sync(0xffffffffu, g.m00, d);
    p.m01 = __shfl_up_sync(0xffffffffu, g.m01, d);
    p.m10 = __shfl_up_sync(0xffffffffu, g.m10, d);
    p.m11 = __shfl_up_sync(0xffffffffu, g.m11, d);
    if (lane >= (unsigned)d) g = fh_mob_normalise(fh_mob_compose(g, p));
  }
  fh_mob e;
  e.m00 = __shfl_up_sync(0xffffffffu, g.m00, 1);
  e.m01 = __shfl_up_sync(0xffffffffu, g.m01, 1);
  e.m10 = __shfl_up_sync(0xffffffffu, g.m10, 1);
  e.m11 = __shfl_up_sync(0xffffffffu, g.m11, 1);
  if (lane == 0) e = fh_mob{1.0, 0.0, 0.0, 1.0};
  return e;
}

// ----------------------------------------------------------- misc
__host__ __device__ __forceinline__ long long fh_ceil_div(long long a, long long b) { return (a + b - 1) / b; }
