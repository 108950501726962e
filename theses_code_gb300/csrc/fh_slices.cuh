// fh_slices.cuh -- exact bf16 slicing of FP64 operands for the blocked
// history contractions on the tensor cores.
//
// Every chunk of 64 layers has a power-of-two scale per weight row (2^Ew) and
// per history point (2^Ed); a scaled value |y| < 128 is cut into four integer
// slices y = a0 + a1/2^8 + a2/2^16 + a3/2^24 with |a_i| <= 128, which bf16
// holds exactly, so the slice products are exact in FP32 and so are their
// level sums over a group of two chunks (both chunks of a group share their
// exponents).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "fh_common.cuh"

constexpr int kSlcK = 64;  // layers per chunk (one 128-byte K-major row of bf16)
constexpr int kSlcN = 4;   // bf16 slices per value

// Chunk groups (pairs of 64-layer chunks; the last group holds one chunk when
// the chunk count is odd).
__host__ __device__ inline int fh_ngroups(int nchunks) { return (nchunks + 1) / 2; }

// x = 2^E (a0 + a1/2^8 + a2/2^16 + a3/2^24) with integer |a_i| <= 128 given |x| < 2^(E+7).
__device__ __forceinline__ void fh_slice4(double x, int E, __nv_bfloat16 (&b)[kSlcN]) {
  double r = ldexp(x, -E);
#pragma unroll
  for (int i = 0; i < kSlcN; ++i) {
    const double a = rint(r);
    b[i] = __double2bfloat16(a);
    r = (r - a) * 256.0;
  }
}

// 2^e as float (0 below the normal range; e stays far below the overflow range here).
__device__ __forceinline__ float fh_exp2i(int e) {
  if (e < -126) return 0.0f;
  return __int_as_float((e + 127) << 23);
}

// 2^e as float for -126 <= e <= 127.
__device__ __forceinline__ float fh_exp2f_int(int e) { return __int_as_float((e + 127) << 23); }

// Per-point exponent E (frexp exponent q of the largest |value|, floored at
// -100; E = q - 7) of a double-float chunk group: every scaled value is below
// 2^7 in magnitude.
__device__ __forceinline__ int fh_point_exp(float mx) {
  int q = -100;
  if (mx >= 7.888609052210118e-31f) q = ((__float_as_int(mx) >> 23) & 0xff) - 126;  // 2^-100
  return q - 7;
}

// Slices of a double-float value (hi, lo) scaled by 2^-E, |hi + lo| < 2^(E+7):
// NS integer bf16 slices a_i with |a_i| <= 128 and (hi + lo) 2^-E =
// sum_i a_i / 2^(8 i) + r, |r| <= 2^(-8 NS + 7) (+ the pair's own rounding).
// FP32 arithmetic only: the scaling is exact, each remainder is kept exactly as
// a renormalised pair.
template <int NS>
__device__ __forceinline__ void fh_slice_pair(float hi, float lo, float scale, __nv_bfloat16 (&b)[NS]) {
  float rh = hi * scale, rl = lo * scale;
#pragma unroll
  for (int i = 0; i < NS; ++i) {
    const float a = rintf(rh);
    b[i] = __float2bfloat16_rn(a);
    const float th = (rh - a) * 256.0f;  // exact: |rh - a| <= 1/2 and a is the integer nearest rh
    const float tl = rl * 256.0f;
    rh = th + tl;                        // fast two-sum (|th| >= |tl| or th == 0)
    rl = tl - (rh - th);
  }
}

// Byte offset of element (row R, k) in a K-major bf16 tile of 64-element
// (128-byte) rows with the 128-byte swizzle (8-row atoms of 1024 B; the 16-byte
// chunk k/8 of row R sits at chunk (k/8) ^ (R % 8)), the layout TMA writes with
// CU_TENSOR_MAP_SWIZZLE_128B and the tcgen05 descriptors of fh_sm100.cuh read.
__host__ __device__ __forceinline__ uint32_t fh_sw128_off(int R, int k) {
  return (uint32_t)(R >> 3) * 1024u + (uint32_t)(R & 7) * 128u + ((uint32_t)(((k >> 3) ^ R) & 7) << 4) +
         (uint32_t)(k & 7) * 2u;
}

// Exponent E with max|x| < 2^(E+7); 0 for an all-zero chunk.
__device__ __forceinline__ int fh_chunk_exp(double mx) {
  if (!(mx > 0.0)) return 0;
  int q;
  frexp(mx, &q);  // mx = f 2^q, f in [0.5, 1)
  return q - 7;
}

// One warp slices the weights w[h] (h < 4: layer 128 G + lane + 32 h) of row m
// in chunk group G: exponent Ew[c][m] for the group's chunks, slices in the
// K-major planes A3[s][m][k] (plane pitch nrows * Kcap).
__device__ __forceinline__ void fh_slice_group_values(const double (&w)[4], int G, int nchunks, long long m,
                                                      long long nrows, int Kcap, __nv_bfloat16 *__restrict__ A3,
                                                      int8_t *__restrict__ Ew) {
  const int lane = threadIdx.x & 31;
  const int c0 = 2 * G, nc = min(2, nchunks - c0);
  double mx = 0.0;
#pragma unroll
  for (int h = 0; h < 4; ++h) mx = fmax(mx, fabs(w[h]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const int E = fh_chunk_exp(mx);
  if (lane == 0)
    for (int c = c0; c < c0 + nc; ++c) Ew[(long long)c * nrows + m] = (int8_t)E;
  const long long plane = nrows * (long long)Kcap;
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    if (h >= 2 * nc) break;
    const int k = c0 * kSlcK + lane + 32 * h;
    __nv_bfloat16 bs[kSlcN];
    fh_slice4(w[h], E, bs);
    const long long o = m * Kcap + k;
#pragma unroll
    for (int i = 0; i < kSlcN; ++i) A3[i * plane + o] = bs[i];
  }
}

// One warp slices row m of group G: val(k) is the weight of layer k.
template <class Val>
__device__ __forceinline__ void fh_slice_row_group(const Val &val, int G, int nchunks, long long m, long long nrows,
                                                   int Kcap, __nv_bfloat16 *__restrict__ A3,
                                                   int8_t *__restrict__ Ew) {
  const int lane = threadIdx.x & 31;
  const int c0 = 2 * G, nc = min(2, nchunks - c0);
  double w[4];
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    const int k = c0 * kSlcK + lane + 32 * h;
    w[h] = h < 2 * nc ? val(k) : 0.0;
  }
  fh_slice_group_values(w, G, nchunks, m, nrows, Kcap, A3, Ew);
}
