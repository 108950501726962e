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
