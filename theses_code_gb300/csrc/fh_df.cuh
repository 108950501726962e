// fh_df.cuh -- double-float ("df") arithmetic on the FP32 pipe: a value is an
// unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2, ~2^-47
// relative precision.  GB300 runs FP32 at ~56x its FP64 rate, so FP64-heavy
// recurrences that can live with ~1e-14 relative error per operation run
// several times faster in this form.  Algorithms: Dekker / Knuth two-sum and
// FMA-based two-product (e.g. Hida, Li, Bailey, "Library for double-double and
// quad-double arithmetic", 2000, the "sloppy" add and the FMA product).
#pragma once
#include <cuda_runtime.h>

struct fh_df {
  float h, l;
};

__device__ __forceinline__ fh_df fh_df_make(float h, float l) { return fh_df{h, l}; }
__device__ __forceinline__ fh_df fh_df_from_pair(float2 p) { return fh_df{p.x, p.y}; }
__device__ __forceinline__ float2 fh_df_pair(fh_df a) { return make_float2(a.h, a.l); }

// Nearest double-float of a double (only off the hot path: uses FP64).
__device__ __forceinline__ fh_df fh_df_from_double(double x) {
  const float h = __double2float_rn(x);
  return fh_df{h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double fh_df_to_double(fh_df a) { return (double)a.h + (double)a.l; }

// s + e = a + b exactly (Knuth two-sum)
__device__ __forceinline__ void fh_two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ fh_df fh_df_renorm(float s, float e) {
  const float h = s + e;
  return fh_df{h, e - (h - s)};
}

__device__ __forceinline__ fh_df fh_df_add(fh_df a, fh_df b) {
  float s, e;
  fh_two_sum(a.h, b.h, s, e);
  e += a.l + b.l;
  return fh_df_renorm(s, e);
}

__device__ __forceinline__ fh_df fh_df_neg(fh_df a) { return fh_df{-a.h, -a.l}; }
__device__ __forceinline__ fh_df fh_df_sub(fh_df a, fh_df b) { return fh_df_add(a, fh_df_neg(b)); }

__device__ __forceinline__ fh_df fh_df_mul(fh_df a, fh_df b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return fh_df_renorm(p, e);
}

// a * b + c
__device__ __forceinline__ fh_df fh_df_fma(fh_df a, fh_df b, fh_df c) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  float s, e2;
  fh_two_sum(p, c.h, s, e2);
  e += e2 + c.l;
  return fh_df_renorm(s, e);
}

// a / b: quotient of the leading parts corrected once with the remainder
__device__ __forceinline__ fh_df fh_df_div(fh_df a, fh_df b) {
  const float q1 = a.h / b.h;
  const fh_df r = fh_df_sub(a, fh_df_mul(fh_df{q1, 0.f}, b));
  const float q2 = r.h / b.h;
  return fh_df_renorm(q1, q2);
}

// Affine map x -> a x + b with double-float coefficients; compose(f2, f1) = f2 o f1.
struct fh_daff {
  fh_df a, b;
};
__device__ __forceinline__ fh_daff fh_daff_compose(fh_daff f2, fh_daff f1) {
  return fh_daff{fh_df_mul(f2.a, f1.a), fh_df_fma(f2.a, f1.b, f2.b)};
}
__device__ __forceinline__ fh_df fh_df_shfl_up(fh_df v, int d) {
  return fh_df{__shfl_up_sync(0xffffffffu, v.h, d), __shfl_up_sync(0xffffffffu, v.l, d)};
}
__device__ __forceinline__ fh_df fh_df_shfl_down(fh_df v, int d) {
  return fh_df{__shfl_down_sync(0xffffffffu, v.h, d), __shfl_down_sync(0xffffffffu, v.l, d)};
}
// Exclusive warp scan: lane l receives f_{l-1} o ... o f_0 (identity for lane 0).
__device__ __forceinline__ fh_daff fh_warp_exclusive_daff(fh_daff f) {
  const unsigned lane = threadIdx.x & 31u;
  fh_daff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const fh_daff p{fh_df_shfl_up(g.a, d), fh_df_shfl_up(g.b, d)};
    if (lane >= (unsigned)d) g = fh_daff_compose(g, p);
  }
  fh_daff e{fh_df_shfl_up(g.a, 1), fh_df_shfl_up(g.b, 1)};
  if (lane == 0) e = fh_daff{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}};
  return e;
}
// Reverse exclusive scan: lane l receives G_{l+1} o ... o G_31 (identity for lane 31).
__device__ __forceinline__ fh_daff fh_warp_exclusive_daff_rev(fh_daff f) {
  const unsigned lane = threadIdx.x & 31u;
  fh_daff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const fh_daff p{fh_df_shfl_down(g.a, d), fh_df_shfl_down(g.b, d)};
    if (lane + d < 32u) g = fh_daff_compose(g, p);
  }
  fh_daff e{fh_df_shfl_down(g.a, 1), fh_df_shfl_down(g.b, 1)};
  if (lane == 31u) e = fh_daff{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}};
  return e;
}
