// fh_blocked.cu -- blocked history contraction on the 5th-generation tensor
// cores (tcgen05 + TMEM + TMA), the far part of the history sum for a block of
// 64 future steps:
//
//   S_far[m][p] = sum_{k<K} W[m][k] * D[k][p],   m < 128 (x/y weights of 64 steps)
//
// Exact-product scheme (Ozaki-style, bf16 slices): every chunk of 64 layers
// has a power-of-two scale per weight row (2^Ew[m][c]) and per point
// (2^Ed[c][p]); scaled values have |y| < 128 and are cut into four integer
// slices y = a0 + a1/2^8 + a2/2^16 + a3/2^24 with |a_i| <= 128, which bf16
// holds exactly.  Products a_i*b_j are exact in FP32 and so are the sums of
// each level l = i + j <= 3 over a group of two chunks (|sum| <= 4*128*2^14 =
// 2^23; both chunks of a group share their exponents): the tensor-core
// accumulation cannot round or truncate.  Per group the epilogue combines the
// four level sums exactly (double-float with one renormalisation), scales by
// 2^(Ew+Ed) and adds into a double-float running sum.  The only approximation is the slicing (~2^-32 of the chunk maxima,
// round to nearest, unbiased) relative to the group maxima; the near layers of
// the block are summed separately in double-float.
//
// Data layout: K-major planes (point p holds its layers contiguously; one
// 64-layer chunk = one 128-byte swizzle row), loaded by TMA with 128-byte
// swizzle; exponents as int8 tables Ed[c][Ppad], Ew[c][128].
//
// Persistent CTAs (320 threads, one per SM, looping over 64-point tiles): warp
// 0 issues TMA loads into a 2-stage ring
// (96 KiB per stage: 4 weight tiles 128x64 + 4 history tiles 64x64 bf16), warp
// 1 owns TMEM (512 columns; 2 buffers x 4 levels x 64 columns) and issues the
// MMAs from one thread, warps 2-9 run the epilogue (two warps per TMEM lane
// quarter, 32 columns each).  Every mbarrier wait is bounded by a %globaltimer
// deadline; on expiry the kernel records FH_ETIMEOUT, waits (bounded) for its
// own copies and MMAs, frees TMEM and returns.
#include <cuda.h>

#include <vector>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "fh_common.cuh"
#include "fh_internal.h"
#include "fh_sm100.cuh"
#include "fh_slices.cuh"
#include "fh_weights.cuh"

namespace {
constexpr int kBM = 128;  // weight rows per block (2 x 64 steps)
constexpr int kBN = 64;   // points per CTA
constexpr int kBK = 64;   // layers per chunk / pipeline stage (one 128-byte row)
constexpr int kStages = 2;
constexpr uint32_t kTileA = kBM * kBK * 2;          // 16 KiB
constexpr uint32_t kTileB = kBN * kBK * 2;          // 8 KiB
constexpr int kSlices = kSlcN;
constexpr int kLevels = kSlices;                     // levels l = i + j <= 3
constexpr uint32_t kStageBytes = kSlices * (kTileA + kTileB);  // 96 KiB
constexpr int kEpiWarps = 8;
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr uint32_t kTmemCols = 512;
constexpr size_t kSmemBytes = kStages * kStageBytes + 1024 + 256;
}  // namespace

__global__ void __launch_bounds__(kThreads, 1)
    k_far_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int K, long long P,
               const int8_t *__restrict__ Ew, const int8_t *__restrict__ Ed, long long Ppad,
               float2 *__restrict__ out, long long ldo, int splits, int gbeg, float2 *__restrict__ part,
               int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  const uint32_t raw = fh_smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t *gbase = smem_raw + (base - raw);
  const uint32_t bars = base + kStages * kStageBytes;
  uint8_t *gbars = gbase + kStages * kStageBytes;
  auto full = [&](int s) { return bars + 8u * s; };
  auto empty = [&](int s) { return bars + 8u * (kStages + s); };
  auto accfull = [&](int b) { return bars + 8u * (2 * kStages + b); };
  auto accempty = [&](int b) { return bars + 8u * (2 * kStages + 2 + b); };
  const uint32_t mmadone = bars + 8u * (2 * kStages + 4);
  const uint32_t tslot = bars + 8u * (2 * kStages + 5);
  volatile uint32_t *tslot_g = reinterpret_cast<volatile uint32_t *>(gbars + 8 * (2 * kStages + 5));
  volatile int *sh_err = reinterpret_cast<volatile int *>(gbars + 8 * (2 * kStages + 6));

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunks = K / kBK;
  // persistent: this CTA owns the work items blockIdx.x, blockIdx.x +
  // gridDim.x, ...; item v = (tile v / splits, group range v % splits): with
  // few tiles (narrow lines) the chunk groups of a tile are split across CTAs
  // (split-K; the partial rows go to part[sp] and k_blk_reduce_splits adds
  // them in split order).  The stage ring and the accumulator buffers run on
  // counters across the items, so loads of the next item overlap the current
  // epilogue.
  const int ntiles = (int)(Ppad / kBN);
  const int ngroups = fh_ngroups(nchunks);  // accumulator buffers cycle per chunk group
  // groups [gbeg, ngroups) are contracted (the older ones have zero weights)
  const int gps = (ngroups - gbeg + splits - 1) / splits;  // groups per split
  const int nitems = ntiles * splits;
  const int my_items = (int)blockIdx.x < nitems ? (nitems - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  // item k of this CTA: tile, first and last group
  auto item = [&](int k, int &tile, int &sp, int &G0, int &G1) {
    const int v = (int)blockIdx.x + k * (int)gridDim.x;
    tile = v / splits;
    sp = v % splits;
    G0 = min(ngroups, gbeg + sp * gps);
    G1 = min(ngroups, G0 + gps);
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      fh_mbar_init(full(s), 1);
      fh_mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      fh_mbar_init(accfull(b), 1);
      fh_mbar_init(accempty(b), 32 * kEpiWarps);
    }
    fh_mbar_init(mmadone, 1);
    *sh_err = 0;
    fh_fence_mbar_init();
  }
  if (warp == 1) {
    fh_tmem_alloc(tslot, kTmemCols);
    fh_tmem_relinquish();
  }
  fh_tc_fence_before();
  __syncthreads();
  fh_tc_fence_after();
  const uint32_t tmem = *tslot_g;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      int last_issued[kStages];
      for (int s = 0; s < kStages; ++s) last_issued[s] = -1;
      int g = 0;  // stage counter
      for (int k = 0; k < my_items && ok; ++k) {
        int tile, sp, G0, G1;
        item(k, tile, sp, G0, G1);
        const int c1 = min(nchunks, 2 * G1);
        for (int c = 2 * G0; c < c1; ++c, ++g) {
          const int s = g % kStages;
          if (g >= kStages && !fh_mbar_wait(empty(s), ((g / kStages) - 1) & 1)) {
            ok = false;
            break;
          }
          fh_mbar_arrive_expect_tx(full(s), kStageBytes);
          const uint32_t sb = base + s * kStageBytes;
          for (int pl = 0; pl < kSlices; ++pl) fh_tma_load_3d(sb + pl * kTileA, &tmA, c * kBK, 0, pl, full(s));
          for (int pl = 0; pl < kSlices; ++pl)
            fh_tma_load_3d(sb + kSlices * kTileA + pl * kTileB, &tmB, c * kBK, tile * kBN, pl, full(s));
          last_issued[s] = g;
        }
      }
      if (!ok) {
        *sh_err = 1;
        for (int s = 0; s < kStages; ++s)
          if (last_issued[s] >= 0) fh_mbar_wait(full(s), (last_issued[s] / kStages) & 1);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int gc = 0;  // chunk counter (stage ring)
      int gg = 0;  // group counter (accumulator buffers)
      for (int k = 0; k < my_items && ok; ++k) {
       int tile, sp, G0, G1;
       item(k, tile, sp, G0, G1);
       for (int G = G0; G < G1 && ok; ++G, ++gg) {
        const int nc = min(2, nchunks - 2 * G);
        const int b = gg & 1;
        if (gg >= 2 && !fh_mbar_wait(accempty(b), ((gg >> 1) - 1) & 1)) {
          ok = false;
          break;
        }
        const uint32_t lv0 = tmem + (uint32_t)(b * kLevels * kBN);
        uint32_t first = 0;
        for (int cc = 0; cc < nc; ++cc, ++gc) {
          const int s = gc % kStages;
          if (!fh_mbar_wait(full(s), (gc / kStages) & 1)) {
            ok = false;
            break;
          }
          fh_tc_fence_after();
          const uint32_t sb = base + s * kStageBytes;
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk) {
            // level l = i + j collects the slice products a_i b_j (exact
            // integers).  The data planes are consecutive in the stage, so B
            // rows 64 ib + n are data slice ib: the MMA of weight slice ia
            // takes data slices 0 .. 3 - ia and writes columns 64 (ia + ib),
            // the accumulator of level ia + ib (the ia = 0 MMA of the group's
            // first 16 layers initialises all four levels).
            const uint64_t bd = fh_desc_kmajor_sw128(sb + kSlices * kTileA + kk * 32);
#pragma unroll
            for (int ia = 0; ia < kSlices; ++ia) {
              const uint64_t ad = fh_desc_kmajor_sw128(sb + ia * kTileA + kk * 32);
              fh_mma_bf16(lv0 + (uint32_t)(ia * kBN), ad, bd, fh_idesc_bf16_f32(kBM, (kSlices - ia) * kBN),
                          (ia > 0 || first) ? 1u : 0u);
            }
            first = 1;
          }
          fh_mma_commit(empty(s));
        }
        if (!ok) break;
        fh_mma_commit(accfull(b));
       }
      }
      fh_mma_commit(mmadone);
      if (!fh_mbar_wait(mmadone, 0)) ok = false;
      if (!ok) *sh_err = 1;
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4)..+31 (row m); the two warps of
    // a lane quarter split the 64 columns
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const uint32_t lanebase = (uint32_t)(32 * q) << 16;
    const int m = 32 * q + lane;
    const int col0 = 32 * half;
    int gg = 0;  // group counter (accumulator buffers)
    for (int k = 0; k < my_items && ok; ++k) {
      int tile, sp, G0, G1;
      item(k, tile, sp, G0, G1);
      const long long p0 = (long long)tile * kBN;
      float HI[32], LO[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) HI[i] = LO[i] = 0.f;
      for (int G = G0; G < G1; ++G, ++gg) {
        const int b = gg & 1;
        // exponents of this group (loaded before the wait: they do not depend on it)
        const int ew = (int)Ew[(long long)(2 * G) * kBM + m];
        const uint4 *edv = reinterpret_cast<const uint4 *>(Ed + (long long)(2 * G) * Ppad + p0 + col0);
        const uint4 ev0 = __ldg(edv), ev1 = __ldg(edv + 1);
        const uint32_t ew32[8] = {ev0.x, ev0.y, ev0.z, ev0.w, ev1.x, ev1.y, ev1.z, ev1.w};
        if (!__all_sync(0xffffffffu, fh_mbar_wait(accfull(b), (gg >> 1) & 1))) {
          ok = false;
          break;
        }
        fh_tc_fence_after();
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          float L0[16], L1[16], L2[16], L3[16];
          const uint32_t cb = tmem + lanebase + (uint32_t)(b * kLevels * kBN + col0 + 16 * t);
          fh_tmem_ld16(cb, L0);
          fh_tmem_ld16(cb + kBN, L1);
          fh_tmem_ld16(cb + 2 * kBN, L2);
          fh_tmem_ld16(cb + 3 * kBN, L3);
          fh_tmem_wait_ld();
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            // T = L0 + L1/2^8 + L2/2^16 + L3/2^24 (|L_l| <= 2^23) exactly as (th, tl):
            // TwoSum of the first two levels, L2 joins the error term exactly,
            // a fast two-sum renormalises, then L3 joins exactly.
            const float x1 = L1[i] * 0.00390625f;
            float th = L0[i] + x1;
            const float bb = th - L0[i];
            float tl = (L0[i] - (th - bb)) + (x1 - bb);
            tl += L2[i] * 1.52587890625e-05f;
            const float tr = th + tl;
            tl = tl - (tr - th);
            th = tr;
            tl += L3[i] * 5.9604644775390625e-08f;
            const int kk = 16 * t + i;
            const float sc = fh_exp2i(ew + (int)(int8_t)(ew32[kk >> 2] >> (8 * (kk & 3))));
            const float vh = th * sc, vl = tl * sc;
            // (HI, LO) += (vh, vl)
            const int k = 16 * t + i;
            const float s2 = HI[k] + vh;
            const float bs = s2 - HI[k];
            const float e = (HI[k] - (s2 - bs)) + (vh - bs);
            HI[k] = s2;
            LO[k] += e + vl;
          }
        }
        fh_tc_fence_before();
        fh_mbar_arrive(accempty(b));
      }
      if (ok && nchunks > 0) {
        // row m, 32 consecutive points: (hi, lo) pairs as 16-byte stores
        float4 *o = reinterpret_cast<float4 *>(
            (splits > 1 ? part + ((long long)sp * kBM + m) * Ppad : out + (long long)m * ldo) + p0 + col0);
#pragma unroll
        for (int k = 0; k < 16; ++k) o[k] = make_float4(HI[2 * k], LO[2 * k], HI[2 * k + 1], LO[2 * k + 1]);
      }
    }
    if (!ok) *sh_err = 1;
  }
  fh_tc_fence_before();
  __syncthreads();
  fh_tc_fence_after();
  if (threadIdx.x == 0 && *sh_err) atomicOr(err, 1);
  if (warp == 1) fh_tmem_dealloc(tmem, kTmemCols);
}

// ----------------------------------------------------------------------------
// Batched form (1D instances of a batch, each with its own weights): the far
// history of the next 64 steps of every instance,
//   far[n][p] = sum_{k<K} W_inst(p)[n][k] * H[k][p],   n < 64,
// with the roles of the operands swapped against k_far_gemm: A = 128
// consecutive history points of one instance (K-major planes H3[s][p][k]),
// B = that instance's 64 weight rows (planes W3[s][inst*64 + n][k]), so the
// TMEM accumulator holds 128 points (lanes) x 64 steps (columns) x 4 levels,
// double-buffered (512 columns).  The tiles come from a list (first point,
// instance, valid points); a tile may reach into the next instance's points,
// whose results are not stored.  Exponents: Ed[c][p] per point, Ew[c][row]
// per weight row.  Same pipeline, exactness argument and bounded waits as
// k_far_gemm.
struct fh_hb_tile {
  long long p0;  // first point (concatenated point index)
  int inst;      // instance: weight rows inst*64 .. inst*64 + 63
  int np;        // valid points of the instance in this tile (<= 128)
};

__global__ void __launch_bounds__(kThreads, 1)
    k_hb_gemm(const __grid_constant__ CUtensorMap tmH, const __grid_constant__ CUtensorMap tmW, int K,
              const fh_hb_tile *__restrict__ tiles, int ntiles, const int8_t *__restrict__ Ew, long long R,
              const int8_t *__restrict__ Ed, long long Ppad, float2 *__restrict__ far, long long ldf,
              int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  const uint32_t raw = fh_smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t *gbase = smem_raw + (base - raw);
  const uint32_t bars = base + kStages * kStageBytes;
  uint8_t *gbars = gbase + kStages * kStageBytes;
  auto full = [&](int s) { return bars + 8u * s; };
  auto empty = [&](int s) { return bars + 8u * (kStages + s); };
  auto accfull = [&](int b) { return bars + 8u * (2 * kStages + b); };
  auto accempty = [&](int b) { return bars + 8u * (2 * kStages + 2 + b); };
  const uint32_t mmadone = bars + 8u * (2 * kStages + 4);
  const uint32_t tslot = bars + 8u * (2 * kStages + 5);
  volatile uint32_t *tslot_g = reinterpret_cast<volatile uint32_t *>(gbars + 8 * (2 * kStages + 5));
  volatile int *sh_err = reinterpret_cast<volatile int *>(gbars + 8 * (2 * kStages + 6));
  constexpr uint32_t kTileH = 128 * kBK * 2;  // 128 points x 64 layers bf16
  constexpr uint32_t kTileW = kBN * kBK * 2;  // 64 rows x 64 layers bf16
  static_assert(kSlices * (kTileH + kTileW) == kStageBytes, "stage layout");

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunks = K / kBK;
  const int ngroups = fh_ngroups(nchunks);
  const int my_items = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      fh_mbar_init(full(s), 1);
      fh_mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      fh_mbar_init(accfull(b), 1);
      fh_mbar_init(accempty(b), 32 * kEpiWarps);
    }
    fh_mbar_init(mmadone, 1);
    *sh_err = 0;
    fh_fence_mbar_init();
  }
  if (warp == 1) {
    fh_tmem_alloc(tslot, kTmemCols);
    fh_tmem_relinquish();
  }
  fh_tc_fence_before();
  __syncthreads();
  fh_tc_fence_after();
  const uint32_t tmem = *tslot_g;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      int last_issued[kStages];
      for (int s = 0; s < kStages; ++s) last_issued[s] = -1;
      int g = 0;  // stage counter
      for (int k = 0; k < my_items && ok; ++k) {
        const fh_hb_tile T = tiles[(int)blockIdx.x + k * (int)gridDim.x];
        for (int c = 0; c < nchunks; ++c, ++g) {
          const int s = g % kStages;
          if (g >= kStages && !fh_mbar_wait(empty(s), ((g / kStages) - 1) & 1)) {
            ok = false;
            break;
          }
          fh_mbar_arrive_expect_tx(full(s), kStageBytes);
          const uint32_t sb = base + s * kStageBytes;
          for (int pl = 0; pl < kSlices; ++pl)
            fh_tma_load_3d(sb + pl * kTileH, &tmH, c * kBK, (int)T.p0, pl, full(s));
          for (int pl = 0; pl < kSlices; ++pl)
            fh_tma_load_3d(sb + kSlices * kTileH + pl * kTileW, &tmW, c * kBK, T.inst * kBN, pl, full(s));
          last_issued[s] = g;
        }
      }
      if (!ok) {
        *sh_err = 1;
        for (int s = 0; s < kStages; ++s)
          if (last_issued[s] >= 0) fh_mbar_wait(full(s), (last_issued[s] / kStages) & 1);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int gc = 0;  // chunk counter (stage ring)
      int gg = 0;  // group counter (accumulator buffers)
      for (int k = 0; k < my_items && ok; ++k) {
        for (int G = 0; G < ngroups && ok; ++G, ++gg) {
          const int nc = min(2, nchunks - 2 * G);
          const int b = gg & 1;
          if (gg >= 2 && !fh_mbar_wait(accempty(b), ((gg >> 1) - 1) & 1)) {
            ok = false;
            break;
          }
          const uint32_t lv0 = tmem + (uint32_t)(b * kLevels * kBN);
          uint32_t first = 0;
          for (int cc = 0; cc < nc; ++cc, ++gc) {
            const int s = gc % kStages;
            if (!fh_mbar_wait(full(s), (gc / kStages) & 1)) {
              ok = false;
              break;
            }
            fh_tc_fence_after();
            const uint32_t sb = base + s * kStageBytes;
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
              // weight planes consecutive in the stage: B rows 64 ib + n are
              // weight slice ib, so the MMA of history slice ia writes the
              // level accumulators ia + ib (as in k_far_gemm)
              const uint64_t bd = fh_desc_kmajor_sw128(sb + kSlices * kTileH + kk * 32);
#pragma unroll
              for (int ia = 0; ia < kSlices; ++ia) {
                const uint64_t ad = fh_desc_kmajor_sw128(sb + ia * kTileH + kk * 32);
                fh_mma_bf16(lv0 + (uint32_t)(ia * kBN), ad, bd, fh_idesc_bf16_f32(128, (kSlices - ia) * kBN),
                            (ia > 0 || first) ? 1u : 0u);
              }
              first = 1;
            }
            fh_mma_commit(empty(s));
          }
          if (!ok) break;
          fh_mma_commit(accfull(b));
        }
      }
      fh_mma_commit(mmadone);
      if (!fh_mbar_wait(mmadone, 0)) ok = false;
      if (!ok) *sh_err = 1;
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4)..+31 (points), the two warps
    // of a lane quarter split the 64 columns (steps)
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const uint32_t lanebase = (uint32_t)(32 * q) << 16;
    const int col0 = 32 * half;
    int gg = 0;
    for (int k = 0; k < my_items && ok; ++k) {
      const fh_hb_tile T = tiles[(int)blockIdx.x + k * (int)gridDim.x];
      const int pt = 32 * q + lane;
      const long long p = T.p0 + pt;
      const long long row0 = (long long)T.inst * kBN + col0;
      float HI[32], LO[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) HI[i] = LO[i] = 0.f;
      for (int G = 0; G < ngroups; ++G, ++gg) {
        const int b = gg & 1;
        // exponents of this group (loaded before the wait: they do not depend on it)
        const int ed = p < Ppad ? (int)Ed[(long long)(2 * G) * Ppad + p] : 0;
        const uint4 *ewv = reinterpret_cast<const uint4 *>(Ew + (long long)(2 * G) * R + row0);
        const uint4 ev0 = __ldg(ewv), ev1 = __ldg(ewv + 1);
        const uint32_t ew32[8] = {ev0.x, ev0.y, ev0.z, ev0.w, ev1.x, ev1.y, ev1.z, ev1.w};
        if (!__all_sync(0xffffffffu, fh_mbar_wait(accfull(b), (gg >> 1) & 1))) {
          ok = false;
          break;
        }
        fh_tc_fence_after();
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          float L0[16], L1[16], L2[16], L3[16];
          const uint32_t cb = tmem + lanebase + (uint32_t)(b * kLevels * kBN + col0 + 16 * t);
          fh_tmem_ld16(cb, L0);
          fh_tmem_ld16(cb + kBN, L1);
          fh_tmem_ld16(cb + 2 * kBN, L2);
          fh_tmem_ld16(cb + 3 * kBN, L3);
          fh_tmem_wait_ld();
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            // T = L0 + L1/2^8 + L2/2^16 + L3/2^24 exactly as (th, tl) (see k_far_gemm)
            const float x1 = L1[i] * 0.00390625f;
            float th = L0[i] + x1;
            const float bb = th - L0[i];
            float tl = (L0[i] - (th - bb)) + (x1 - bb);
            tl += L2[i] * 1.52587890625e-05f;
            const float tr = th + tl;
            tl = tl - (tr - th);
            th = tr;
            tl += L3[i] * 5.9604644775390625e-08f;
            const int kk = 16 * t + i;
            const float sc = fh_exp2i(ed + (int)(int8_t)(ew32[kk >> 2] >> (8 * (kk & 3))));
            const float vh = th * sc, vl = tl * sc;
            const float s2 = HI[kk] + vh;
            const float bs = s2 - HI[kk];
            const float e = (HI[kk] - (s2 - bs)) + (vh - bs);
            HI[kk] = s2;
            LO[kk] += e + vl;
          }
        }
        fh_tc_fence_before();
        fh_mbar_arrive(accempty(b));
      }
      if (ok && nchunks > 0 && pt < T.np) {
#pragma unroll
        for (int kk = 0; kk < 32; ++kk) {
          const float h = HI[kk] + LO[kk];
          far[(long long)(col0 + kk) * ldf + p] = make_float2(h, LO[kk] - (h - HI[kk]));
        }
      }
    }
    if (!ok) *sh_err = 1;
  }
  fh_tc_fence_before();
  __syncthreads();
  fh_tc_fence_after();
  if (threadIdx.x == 0 && *sh_err) atomicOr(err, 1);
  if (warp == 1) fh_tmem_dealloc(tmem, kTmemCols);
}

// Chunk groups: group G covers the 64-layer chunks 2G and 2G+1 (the last group
// holds one chunk when the chunk count is odd).  All chunks of a group share
// the row exponent Ew and the history exponent Ed, so the tensor cores can
// accumulate a whole group (128 layers: level sums <= 4*128*2^14 = 2^23, still
// exact in FP32) before the epilogue combines it (fh_slices.cuh).

// Weight planes of a TG block: row m = 2r + {0: x, 1: y} of step j0 + r,
// A3[s][m][k] (K-major) and Ew[c][m]; one warp per (row, chunk group).
__global__ void k_blk_weights(int j0, int K, int Kcap, double Da, double tau, double alpha, double beta, double cut,
                              __nv_bfloat16 *__restrict__ A3, int8_t *__restrict__ Ew) {
  const int m = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (m >= kBM) return;
  const double X = (double)(j0 + (m >> 1)) + ((m & 1) ? 1.0 : 0.5);
  auto val = [&](int k) {  // weights below `cut` are 0 (restricted summing)
    const double w = k < K ? Da * fh_psi_int((double)k + 0.0, (double)k + 1.0, X, tau, alpha, beta) : 0.0;
    return fabs(w) < cut ? 0.0 : w;
  };
  fh_slice_row_group(val, blockIdx.x, K / kBK, m, kBM, Kcap, A3, Ew);
}

// Toeplitz weight rows (1D solvers with lag weights): row m = step T0 + 1 + m
// weighs history entry k with w[base + m - k] (base = T0 + 1); rows m >= mrows
// are zero.
__global__ void k_blk_toeplitz_rows(const double *__restrict__ w, int base, int K, int Kcap, int mrows,
                                    __nv_bfloat16 *__restrict__ A3, int8_t *__restrict__ Ew) {
  const int m = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (m >= kBM) return;
  auto val = [&](int k) { return (k < K && m < mrows) ? w[base + m - k] : 0.0; };
  fh_slice_row_group(val, blockIdx.x, K / kBK, m, kBM, Kcap, A3, Ew);
}

// Weight rows W[m*ldw + k], k < K, rows m >= mrows are zero (standalone
// contraction, or a block of the per-solve weight table).
__global__ void k_blk_split_rows(const double *__restrict__ W, long long ldw, int K, int Kcap, int mrows,
                                 __nv_bfloat16 *__restrict__ A3, int8_t *__restrict__ Ew) {
  const int m = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (m >= kBM) return;
  auto val = [&](int k) { return (k < K && m < mrows) ? W[(long long)m * ldw + k] : 0.0; };
  fh_slice_row_group(val, blockIdx.x, K / kBK, m, kBM, Kcap, A3, Ew);
}

// The even chunk of a chunk pair, layers [kg0, kg0 + 64) of the double-float
// history (layer-major (hi, lo) pairs, layer k at row k - kd0, pitch ldd, P
// valid points), into the K-major planes H3[s][p][k] and the per-point
// exponents Ed[c][p] of its own maximum (k_blk_convert_df_odd raises them to
// the pair's).  64 points per CTA, 4 threads per point (16 layers each):
// coalesced pair loads, FP32 slicing in registers, the 64 x 64 bf16 tile of
// each plane staged in shared memory (pitch 66: conflict-free) and written as
// full 128-byte rows.  Points whose maximum is below 2^-100 are scaled as if
// it were 2^-100 (their slices carry the value to 2^-132).
constexpr int kCvPts = 64;
constexpr int kCvPitch = kBK + 2;  // bf16 per staged row
constexpr size_t kCvSmemPerChunk = sizeof(__nv_bfloat16) * kSlices * kCvPts * kCvPitch;
__global__ void __launch_bounds__(256) k_blk_convert_df(const float2 *__restrict__ D, long long ldd, int kd0, long long P,
                                                        long long Ppad, int kg0, int Kcap,
                                                        __nv_bfloat16 *__restrict__ H3, int8_t *__restrict__ Ed) {
  constexpr int NCH = 1;
  extern __shared__ __align__(16) __nv_bfloat16 cvout[];  // [kSlices][kCvPts * kCvPitch]
  __shared__ float qmax[4][kCvPts];
  constexpr int kL = 16 * NCH;  // layers per thread
  const long long p0 = (long long)blockIdx.x * kCvPts;
  const int pt = threadIdx.x & (kCvPts - 1);
  const int qh = threadIdx.x >> 6;  // layers qh*kL .. qh*kL + kL - 1 of the group
  const long long p = p0 + pt;
  float hi[kL], lo[kL];
  float mx = 0.f;
#pragma unroll
  for (int i = 0; i < kL; ++i) {
    float2 v = make_float2(0.f, 0.f);
    if (p < P) v = __ldcs(D + (long long)(kg0 - kd0 + qh * kL + i) * ldd + p);
    hi[i] = v.x;
    lo[i] = v.y;
    mx = fmaxf(mx, fabsf(v.x));
  }
  qmax[qh][pt] = mx;
  __syncthreads();
  mx = fmaxf(fmaxf(qmax[0][pt], qmax[1][pt]), fmaxf(qmax[2][pt], qmax[3][pt]));
  const int E = fh_point_exp(mx);
  if (qh < NCH && p < Ppad) Ed[(long long)(kg0 / kBK + qh) * Ppad + p] = (int8_t)E;
  const float scale = fh_exp2f_int(-E);  // -E <= 107
#pragma unroll
  for (int i = 0; i < kL; i += 2) {
    __nv_bfloat16 s0[kSlices], s1[kSlices];
    fh_slice_pair<kSlices>(hi[i], lo[i], scale, s0);
    fh_slice_pair<kSlices>(hi[i + 1], lo[i + 1], scale, s1);
    const int l = qh * kL + i;  // layer within the group
    const int ch = l / kBK, kk = l % kBK;
#pragma unroll
    for (int c = 0; c < kSlices; ++c) {
      __nv_bfloat162 w;
      w.x = s0[c];
      w.y = s1[c];
      *reinterpret_cast<__nv_bfloat162 *>(
          &cvout[((size_t)ch * kSlices + c) * kCvPts * kCvPitch + pt * kCvPitch + kk]) = w;
    }
  }
  __syncthreads();
  // rows of 64 layers (128 B) per point, plane and chunk; a warp writes 4 rows per pass
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long plane = Ppad * (long long)Kcap;
  for (int r = warp * 4 + (lane >> 3); r < NCH * kSlices * kCvPts; r += 8 * 4) {
    const int chc = r / kCvPts, row = r - chc * kCvPts;  // chc = chunk * kSlices + plane
    const int ch = chc / kSlices, c = chc - ch * kSlices;
    const long long pr = p0 + row;
    if (pr >= Ppad) continue;
    const uint32_t *src =
        reinterpret_cast<const uint32_t *>(&cvout[(size_t)chc * kCvPts * kCvPitch + row * kCvPitch + (lane & 7) * 8]);
    uint4 v;
    v.x = src[0];
    v.y = src[1];
    v.z = src[2];
    v.w = src[3];
    reinterpret_cast<uint4 *>(H3 + c * plane + pr * Kcap + kg0 + ch * kBK)[lane & 7] = v;
  }
}

// The odd chunk c of a chunk pair (layers [kc0, kc0 + 64) of the
// double-float history, layer k at row k - kd0 of D):
// both chunks of the pair take the exponent of their joint maximum, which is
// max(Ed[c-1][p], E(odd maximum)) since the even chunk was converted alone
// with its own.  The odd chunk is sliced with it, and the even chunk is read
// and sliced again only at the points where the odd chunk raised it; the
// planes and exponents equal those of slicing both chunks with the pair's
// exponent, with half the traffic wherever nothing is raised.
__global__ void __launch_bounds__(256) k_blk_convert_df_odd(const float2 *__restrict__ D, long long ldd, int kd0,
                                                          long long P, long long Ppad, int kc0, int Kcap,
                                                          __nv_bfloat16 *__restrict__ H3, int8_t *__restrict__ Ed) {
  extern __shared__ __align__(16) __nv_bfloat16 cvout[];  // [2][kSlices][kCvPts * kCvPitch]
  __shared__ float qmax[4][kCvPts];
  __shared__ int Es[kCvPts], redo[kCvPts];
  constexpr int kL = 16;  // layers per thread
  const int c = kc0 / kBK, kg0 = kc0 - kBK;
  const long long p0 = (long long)blockIdx.x * kCvPts;
  const int pt = threadIdx.x & (kCvPts - 1);
  const int qh = threadIdx.x >> 6;  // layers qh*kL .. qh*kL + kL - 1 of a chunk
  const long long p = p0 + pt;
  float hi[kL], lo[kL];
  float mx = 0.f;
#pragma unroll
  for (int i = 0; i < kL; ++i) {
    float2 v = make_float2(0.f, 0.f);
    if (p < P) v = __ldcs(D + (long long)(kc0 - kd0 + qh * kL + i) * ldd + p);
    hi[i] = v.x;
    lo[i] = v.y;
    mx = fmaxf(mx, fabsf(v.x));
  }
  qmax[qh][pt] = mx;
  __syncthreads();
  if (qh == 0) {
    const int Eo = fh_point_exp(fmaxf(fmaxf(qmax[0][pt], qmax[1][pt]), fmaxf(qmax[2][pt], qmax[3][pt])));
    const int Ee = p < Ppad ? (int)Ed[(long long)(c - 1) * Ppad + p] : Eo;
    const int E = Eo > Ee ? Eo : Ee;
    Es[pt] = E;
    redo[pt] = Eo > Ee;
    if (p < Ppad) {
      Ed[(long long)c * Ppad + p] = (int8_t)E;
      if (Eo > Ee) Ed[(long long)(c - 1) * Ppad + p] = (int8_t)E;
    }
  }
  __syncthreads();
  const int E = Es[pt];
  const bool rd = redo[pt] != 0;
  const float scale = fh_exp2f_int(-E);  // -E <= 107
  auto slice_to = [&](int ch) {
#pragma unroll
    for (int i = 0; i < kL; i += 2) {
      __nv_bfloat16 s0[kSlices], s1[kSlices];
      fh_slice_pair<kSlices>(hi[i], lo[i], scale, s0);
      fh_slice_pair<kSlices>(hi[i + 1], lo[i + 1], scale, s1);
      const int kk = qh * kL + i;
#pragma unroll
      for (int q = 0; q < kSlices; ++q) {
        __nv_bfloat162 w;
        w.x = s0[q];
        w.y = s1[q];
        *reinterpret_cast<__nv_bfloat162 *>(
            &cvout[((size_t)ch * kSlices + q) * kCvPts * kCvPitch + pt * kCvPitch + kk]) = w;
      }
    }
  };
  slice_to(1);
  if (rd) {
#pragma unroll
    for (int i = 0; i < kL; ++i) {
      float2 v = make_float2(0.f, 0.f);
      if (p < P) v = __ldcs(D + (long long)(kg0 - kd0 + qh * kL + i) * ldd + p);
      hi[i] = v.x;
      lo[i] = v.y;
    }
    slice_to(0);
  }
  __syncthreads();
  // rows of 64 layers (128 B) per point, plane and chunk; a warp writes 4 rows
  // per pass; the even chunk's rows only where it was sliced again
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long plane = Ppad * (long long)Kcap;
  for (int r = warp * 4 + (lane >> 3); r < 2 * kSlices * kCvPts; r += 8 * 4) {
    const int chc = r / kCvPts, row = r - chc * kCvPts;  // chc = chunk * kSlices + plane
    const int ch = chc / kSlices, q = chc - ch * kSlices;
    const long long pr = p0 + row;
    if (pr >= Ppad || (ch == 0 && !redo[row])) continue;
    const uint32_t *src =
        reinterpret_cast<const uint32_t *>(&cvout[(size_t)chc * kCvPts * kCvPitch + row * kCvPitch + (lane & 7) * 8]);
    uint4 v;
    v.x = src[0];
    v.y = src[1];
    v.z = src[2];
    v.w = src[3];
    reinterpret_cast<uint4 *>(H3 + q * plane + pr * Kcap + kg0 + ch * kBK)[lane & 7] = v;
  }
}

// FP64 history (standalone contraction): layers [kg0, kg0 + 64 nch) of D
// (layer-major, pitch ldd) into the planes and per-point exponents, one thread
// per point (64 points per CTA), the values through a shared tile.
__global__ void __launch_bounds__(64) k_blk_convert(const double *__restrict__ D, long long ldd, long long P,
                                                    long long Ppad, int kg0, int nch, int Kcap,
                                                    __nv_bfloat16 *__restrict__ H3, int8_t *__restrict__ Ed) {
  extern __shared__ double tile[];  // [64 nch][64]
  const int t = threadIdx.x;
  const long long p = (long long)blockIdx.x * 64 + t;
  const int nl = kBK * nch;
  double mx = 0.0;
  for (int k = 0; k < nl; ++k) {
    const double v = p < P ? __ldcs(D + (long long)(kg0 + k) * ldd + p) : 0.0;
    tile[k * 64 + t] = v;
    mx = fmax(mx, fabs(v));
  }
  const int E = fh_chunk_exp(mx);
  if (p >= Ppad) return;
  for (int c = 0; c < nch; ++c) Ed[(long long)(kg0 / kBK + c) * Ppad + p] = (int8_t)E;
  const long long plane = Ppad * (long long)Kcap;
#pragma unroll 1
  for (int v = 0; v < nl / 8; ++v) {
    __align__(16) __nv_bfloat16 c[kSlices][8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      __nv_bfloat16 bs[kSlices];
      fh_slice4(tile[(v * 8 + i) * 64 + t], E, bs);
#pragma unroll
      for (int q = 0; q < kSlices; ++q) c[q][i] = bs[q];
    }
#pragma unroll
    for (int q = 0; q < kSlices; ++q)
      reinterpret_cast<uint4 *>(H3 + q * plane + p * Kcap + kg0)[v] = *reinterpret_cast<const uint4 *>(c[q]);
  }
}

// ------------------------------------------------------------------- host

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static int get_encode(fh_ctx *ctx) {
  if (g_encode) return FH_OK;
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
    return fh_set_error(ctx, FH_ECUDA, "cuTensorMapEncodeTiled unavailable");
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return FH_OK;
}

// 3D bf16 tensor {d0 (contiguous), d1, 3 planes}, box {64, rows, 1}, 128-byte swizzle.
static int make_map(fh_ctx *ctx, CUtensorMap *map, void *base, unsigned long long d0, unsigned long long d1,
                    unsigned rows) {
  int rc = get_encode(ctx);
  if (rc) return rc;
  cuuint64_t dims[3] = {d0, d1, (cuuint64_t)kSlices};
  cuuint64_t strides[2] = {d0 * 2, d0 * d1 * 2};
  cuuint32_t box[3] = {(cuuint32_t)kBK, (cuuint32_t)rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fh_set_error(ctx, FH_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return FH_OK;
}

// Plane storage, exponent tables and tensor maps of one blocked contraction.
struct fh_blk {
  long long P = 0, Ppad = 0;
  int Kcap = 0;
  int nsm = 1;  // SMs of the device: one persistent CTA each
  fh_dbuf H3, A3, Ed, Ew, err;
  fh_dbuf part;        // split-K partial rows (narrow lines: fewer tiles than SMs)
  int max_splits = 1;
  CUtensorMap mapA, mapB;
};

fh_blk *fh_blk_new() { return new fh_blk(); }
void fh_blk_delete(fh_blk *b) { delete b; }
size_t fh_blk_bytes(const fh_blk &b) {
  return b.H3.bytes + b.A3.bytes + b.Ed.bytes + b.Ew.bytes + b.err.bytes + b.part.bytes;
}
long long fh_blk_ppad(const fh_blk &b) { return b.Ppad; }

int fh_blk_init(fh_ctx *ctx, fh_blk &b, long long P, int Kcap) {
  FH_REQUIRE(ctx, Kcap % kBK == 0 && Kcap > 0, FH_EINVAL, "blocked contraction: capacity must be a multiple of 64");
  b.P = P;
  b.Ppad = fh_ceil_div(P, 128) * 128;
  b.Kcap = Kcap;
  FH_CUDA_TRY(ctx, cudaDeviceGetAttribute(&b.nsm, cudaDevAttrMultiProcessorCount, ctx->device));
  int rc;
  if ((rc = fh_alloc(ctx, b.H3, sizeof(__nv_bfloat16) * kSlices * (size_t)b.Ppad * Kcap)) ||
      (rc = fh_alloc(ctx, b.A3, sizeof(__nv_bfloat16) * kSlices * (size_t)kBM * Kcap)) ||
      (rc = fh_alloc(ctx, b.Ed, (size_t)b.Ppad * (Kcap / kBK))) ||
      (rc = fh_alloc(ctx, b.Ew, (size_t)kBM * (Kcap / kBK))) || (rc = fh_alloc(ctx, b.err, sizeof(int))))
    return rc;
  const long long ntiles = b.Ppad / kBN;
  b.max_splits = ntiles < b.nsm ? (int)(b.nsm / ntiles) : 1;
  if (b.max_splits > 8) b.max_splits = 8;
  if (b.max_splits > 1 &&
      (rc = fh_alloc(ctx, b.part, sizeof(float2) * (size_t)b.max_splits * kBM * (size_t)b.Ppad, false)))
    return rc;
  if ((rc = make_map(ctx, &b.mapA, b.A3.p, (unsigned long long)Kcap, kBM, kBM))) return rc;
  if ((rc = make_map(ctx, &b.mapB, b.H3.p, (unsigned long long)Kcap, (unsigned long long)b.Ppad, kBN))) return rc;
  // shared-memory opt-ins on this context's device (per device, so on every init)
  FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_far_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes));
  FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_blk_convert, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(sizeof(double) * 2 * kBK * 64)));
  FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_blk_convert_df_odd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(2 * kCvSmemPerChunk)));
  return FH_OK;
}

// Converts layers [k0, k0+64) of the history (FP64, or (hi, lo) pairs when df)
// into the planes and exponents; chunks must be converted in order.  An odd
// chunk completes the group (k0 - 64, k0): both chunks are (re)converted with
// the group's per-point exponents.
int fh_blk_convert(fh_ctx *ctx, fh_blk &b, const double *D, long long ldd, int k0, int df) {
  FH_REQUIRE(ctx, k0 % kBK == 0 && k0 + kBK <= b.Kcap, FH_EINVAL, "blocked contraction: bad layer block %d", k0);
  const int c = k0 / kBK;
  const int kg0 = (c & 1) ? k0 - kBK : k0;
  const int nch = (c & 1) ? 2 : 1;
  if (df) {
    const float2 *Dp = reinterpret_cast<const float2 *>(D);
    if (nch == 2)
      k_blk_convert_df_odd<<<(unsigned)(b.Ppad / kCvPts), 256, 2 * kCvSmemPerChunk, ctx->stream>>>(
          Dp, ldd, 0, b.P, b.Ppad, k0, b.Kcap, b.H3.as<__nv_bfloat16>(), b.Ed.as<int8_t>());
    else
      k_blk_convert_df<<<(unsigned)(b.Ppad / kCvPts), 256, kCvSmemPerChunk, ctx->stream>>>(
          Dp, ldd, 0, b.P, b.Ppad, kg0, b.Kcap, b.H3.as<__nv_bfloat16>(), b.Ed.as<int8_t>());
    return fh_after_launch(ctx, "k_blk_convert_df");
  }
  k_blk_convert<<<(unsigned)(b.Ppad / 64), 64, sizeof(double) * nch * kBK * 64, ctx->stream>>>(
      D, ldd, b.P, b.Ppad, kg0, nch, b.Kcap, b.H3.as<__nv_bfloat16>(), b.Ed.as<int8_t>());
  return fh_after_launch(ctx, "k_blk_convert");
}

// Weight planes of the TG block starting at step j0 (K = j0 history layers).
// With a weight table (row 2j: x weights of step j, row 2j+1: y weights, pitch
// ldw, nsteps steps) the rows are taken from it instead of being recomputed.
int fh_blk_tg_weights(fh_ctx *ctx, fh_blk &b, int j0, double Da, double tau, double alpha, double beta, double cut,
                      const double *table, int ldw, int nsteps) {
  dim3 g((unsigned)fh_ngroups(j0 / kBK), kBM / 8);
  if (table) {
    const int mrows = 2 * (nsteps - j0) < kBM ? 2 * (nsteps - j0) : kBM;
    k_blk_split_rows<<<g, 256, 0, ctx->stream>>>(table + (long long)j0 * 2 * ldw, ldw, j0, b.Kcap, mrows,
                                                 b.A3.as<__nv_bfloat16>(), b.Ew.as<int8_t>());
    return fh_after_launch(ctx, "k_blk_split_rows");
  }
  k_blk_weights<<<g, 256, 0, ctx->stream>>>(j0, j0, b.Kcap, Da, tau, alpha, beta, cut, b.A3.as<__nv_bfloat16>(),
                                           b.Ew.as<int8_t>());
  return fh_after_launch(ctx, "k_blk_weights");
}

// Toeplitz weight planes for K history entries (k_blk_toeplitz_rows).
int fh_blk_toeplitz_weights(fh_ctx *ctx, fh_blk &b, const double *w, int base, int K, int mrows) {
  FH_REQUIRE(ctx, K % kBK == 0 && K > 0 && K <= b.Kcap, FH_EINVAL, "blocked contraction: K=%d", K);
  dim3 g((unsigned)fh_ngroups(K / kBK), kBM / 8);
  k_blk_toeplitz_rows<<<g, 256, 0, ctx->stream>>>(w, base, K, b.Kcap, mrows, b.A3.as<__nv_bfloat16>(),
                                                  b.Ew.as<int8_t>());
  return fh_after_launch(ctx, "k_blk_toeplitz_rows");
}

// out[m][p] = sum_sp part[sp][m][p] in split order (double-float adds)
__global__ void k_blk_reduce_splits(const float2 *__restrict__ part, int splits, long long Ppad,
                                    float2 *__restrict__ out, long long ldo) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y;
  if (p >= Ppad) return;
  float2 v = part[(long long)m * Ppad + p];
  float h = v.x, l = v.y;
  for (int sp = 1; sp < splits; ++sp) {
    const float2 u = part[((long long)sp * kBM + m) * Ppad + p];
    const float t = h + u.x, bb = t - h;
    const float e = (h - (t - bb)) + (u.x - bb);
    l += e + u.y;
    h = t;
  }
  const float t = h + l;
  out[(long long)m * ldo + p] = make_float2(t, l - (t - h));
}

// S_far = A3 (128 x K) * planes (K x P) -> out[m*ldo + p] as (hi, lo) pairs.
// Narrow lines (fewer 64-point tiles than SMs) split the chunk groups of each
// tile across CTAs and add the partial rows afterwards.
int fh_blk_gemm(fh_ctx *ctx, fh_blk &b, int K, float2 *out, long long ldo, int gbeg) {
  FH_REQUIRE(ctx, K % kBK == 0 && K > 0 && K <= b.Kcap, FH_EINVAL, "blocked contraction: K=%d", K);
  fh_prof_mark(ctx, FH_PROF_GEMM, false);
  const long long ntiles = b.Ppad / kBN;
  const int ngroups = fh_ngroups(K / kBK);
  if (gbeg < 0) gbeg = 0;
  if (gbeg > ngroups - 1) gbeg = ngroups - 1;  // at least one group: every output row is written
  const int splits = b.max_splits < ngroups - gbeg ? b.max_splits : ngroups - gbeg;
  const long long items = ntiles * splits;
  k_far_gemm<<<(unsigned)(items < b.nsm ? items : b.nsm), kThreads, kSmemBytes, ctx->stream>>>(
      b.mapA, b.mapB, K, b.P, b.Ew.as<int8_t>(), b.Ed.as<int8_t>(), b.Ppad, out, ldo, splits, gbeg,
      b.part.as<float2>(), b.err.as<int>());
  int rc = fh_after_launch(ctx, "k_far_gemm");
  if (!rc && splits > 1) {
    k_blk_reduce_splits<<<dim3((unsigned)fh_ceil_div(b.Ppad, 256), kBM), 256, 0, ctx->stream>>>(
        b.part.as<float2>(), splits, b.Ppad, out, ldo);
    rc = fh_after_launch(ctx, "k_blk_reduce_splits");
  }
  fh_prof_mark(ctx, FH_PROF_GEMM, true);
  return rc;
}

// ------------------------------------------------------------ batched form
// Planes, exponents, weight planes, tile list and tensor maps of the batched
// far contraction (k_hb_gemm).  History planes H3[s][Ppad][Kcap] over the
// concatenated points; weight planes W3[s][R][Kcap], R = 64 rows per instance.
struct fh_hblk {
  long long P = 0, Ppad = 0, R = 0;
  int Kcap = 0, ntiles = 0, nsm = 1;
  fh_dbuf H3, Ed, W3, Ew, tiles, err;
  CUtensorMap mapH, mapW;
};

fh_hblk *fh_hblk_new() { return new fh_hblk(); }
void fh_hblk_delete(fh_hblk *b) { delete b; }
__nv_bfloat16 *fh_hblk_wplanes(fh_hblk &b) { return b.W3.as<__nv_bfloat16>(); }
int8_t *fh_hblk_wexp(fh_hblk &b) { return b.Ew.as<int8_t>(); }
int fh_hblk_kcap(const fh_hblk &b) { return b.Kcap; }
size_t fh_hblk_bytes(const fh_hblk &b) {
  return b.H3.bytes + b.Ed.bytes + b.W3.bytes + b.Ew.bytes + b.tiles.bytes + b.err.bytes;
}

// tiles: (first point, instance, valid points) of every 128-point tile
int fh_hblk_init(fh_ctx *ctx, fh_hblk &b, long long P, int Kcap, int ninst, const long long *tile_p0,
                 const int *tile_inst, const int *tile_np, int ntiles) {
  FH_REQUIRE(ctx, Kcap % kBK == 0 && Kcap > 0 && ninst > 0 && ntiles > 0, FH_EINVAL, "batched contraction: sizes");
  b.P = P;
  b.Ppad = fh_ceil_div(P + 128, 128) * 128;  // a tile starting at any point stays inside
  b.R = (long long)ninst * kBN;
  b.Kcap = Kcap;
  b.ntiles = ntiles;
  FH_CUDA_TRY(ctx, cudaDeviceGetAttribute(&b.nsm, cudaDevAttrMultiProcessorCount, ctx->device));
  int rc;
  if ((rc = fh_alloc(ctx, b.H3, sizeof(__nv_bfloat16) * kSlices * (size_t)b.Ppad * Kcap)) ||
      (rc = fh_alloc(ctx, b.Ed, (size_t)b.Ppad * (Kcap / kBK))) ||
      (rc = fh_alloc(ctx, b.W3, sizeof(__nv_bfloat16) * kSlices * (size_t)b.R * Kcap)) ||
      (rc = fh_alloc(ctx, b.Ew, (size_t)b.R * (Kcap / kBK))) ||
      (rc = fh_alloc(ctx, b.tiles, sizeof(fh_hb_tile) * (size_t)ntiles, false)) ||
      (rc = fh_alloc(ctx, b.err, sizeof(int))))
    return rc;
  std::vector<fh_hb_tile> t((size_t)ntiles);
  for (int i = 0; i < ntiles; ++i) {
    FH_REQUIRE(ctx, tile_p0[i] >= 0 && tile_p0[i] < P && tile_np[i] >= 1 && tile_np[i] <= 128 && tile_inst[i] >= 0 &&
                        tile_inst[i] < ninst,
               FH_EINVAL, "batched contraction: tile %d", i);
    t[(size_t)i] = fh_hb_tile{tile_p0[i], tile_inst[i], tile_np[i]};
  }
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(b.tiles.p, t.data(), sizeof(fh_hb_tile) * t.size(), cudaMemcpyHostToDevice,
                                   ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // t is a local buffer
  if ((rc = make_map(ctx, &b.mapH, b.H3.p, (unsigned long long)Kcap, (unsigned long long)b.Ppad, 128))) return rc;
  if ((rc = make_map(ctx, &b.mapW, b.W3.p, (unsigned long long)Kcap, (unsigned long long)b.R, kBN))) return rc;
  FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_hb_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes));
  FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_blk_convert_df_odd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(2 * kCvSmemPerChunk)));
  return FH_OK;
}

// Converts history chunk c (layers [64c, 64c + 64)) held in a ring of
// (hi, lo) pairs (ring row r = layer r mod 128, pitch ldd); an odd chunk
// completes its group and raises the group's per-point exponents, the even
// partner sliced again where they rise, so the ring must still hold it.
int fh_hblk_convert(fh_ctx *ctx, fh_hblk &b, const float2 *ring, long long ldd, int c) {
  FH_REQUIRE(ctx, c >= 0 && (c + 1) * kBK <= b.Kcap, FH_EINVAL, "batched contraction: chunk %d", c);
  const int kg0 = ((c & 1) ? c - 1 : c) * kBK;
  const int kd0 = (kg0 / 128) * 128;  // layer held in ring row 0
  if (c & 1)
    k_blk_convert_df_odd<<<(unsigned)(b.Ppad / kCvPts), 256, 2 * kCvSmemPerChunk, ctx->stream>>>(
        ring, ldd, kd0, b.P, b.Ppad, c * kBK, b.Kcap, b.H3.as<__nv_bfloat16>(), b.Ed.as<int8_t>());
  else
    k_blk_convert_df<<<(unsigned)(b.Ppad / kCvPts), 256, kCvSmemPerChunk, ctx->stream>>>(
        ring, ldd, kd0, b.P, b.Ppad, kg0, b.Kcap, b.H3.as<__nv_bfloat16>(), b.Ed.as<int8_t>());
  return fh_after_launch(ctx, "k_blk_convert_df");
}

// far[n*ldf + p] = sum_{k<K} W3[inst(p)*64 + n][k] H[k][p] as (hi, lo) pairs,
// for the valid points of every tile.
int fh_hblk_gemm(fh_ctx *ctx, fh_hblk &b, int K, float2 *far, long long ldf) {
  FH_REQUIRE(ctx, K % kBK == 0 && K > 0 && K <= b.Kcap, FH_EINVAL, "batched contraction: K=%d", K);
  fh_prof_mark(ctx, FH_PROF_GEMM, false);
  k_hb_gemm<<<(unsigned)(b.ntiles < b.nsm ? b.ntiles : b.nsm), kThreads, kSmemBytes, ctx->stream>>>(
      b.mapH, b.mapW, K, b.tiles.as<fh_hb_tile>(), b.ntiles, b.Ew.as<int8_t>(), b.R, b.Ed.as<int8_t>(), b.Ppad, far,
      ldf, b.err.as<int>());
  const int rc = fh_after_launch(ctx, "k_hb_gemm");
  fh_prof_mark(ctx, FH_PROF_GEMM, true);
  return rc;
}

int fh_hblk_check(fh_ctx *ctx, fh_hblk &b) {
  int h = 0;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(&h, b.err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (h) return fh_set_error(ctx, FH_ETIMEOUT, "batched contraction: a bounded wait expired");
  return FH_OK;
}

__global__ void k_pairs_to_double(const float2 *__restrict__ in, long long ldi, long long P, double *__restrict__ out,
                                  long long ldo) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const float2 v = in[(long long)blockIdx.y * ldi + p];
  out[(long long)blockIdx.y * ldo + p] = (double)v.x + (double)v.y;
}

int fh_blk_check(fh_ctx *ctx, fh_blk &b) {
  int h = 0;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(&h, b.err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (h) return fh_set_error(ctx, FH_ETIMEOUT, "blocked contraction: a bounded wait expired");
  return FH_OK;
}

extern "C" int fh_history_contract_bf16(fh_ctx *ctx, int K, long long P, const double *W, int ldw,
                                          const double *D, long long ldd, double *S, long long ldS) {
  FH_REQUIRE(ctx, ctx, FH_EINVAL, "null context");
  FH_REQUIRE(ctx, K > 0 && K % kBK == 0 && K <= 65536, FH_EINVAL,
             "fh_history_contract_bf16: K must be a positive multiple of 64");
  FH_REQUIRE(ctx, P > 0 && ldd >= P && ldS >= P && ldw >= K, FH_EINVAL, "fh_history_contract_bf16: bad sizes");
  FH_REQUIRE(ctx, W && D && S, FH_EINVAL, "fh_history_contract_bf16: null pointer");
  fh_blk b;
  int rc = fh_blk_init(ctx, b, P, K);
  if (rc) return rc;
  dim3 g((unsigned)fh_ngroups(K / kBK), kBM / 8);
  k_blk_split_rows<<<g, 256, 0, ctx->stream>>>(W, ldw, K, K, kBM, b.A3.as<__nv_bfloat16>(), b.Ew.as<int8_t>());
  if ((rc = fh_after_launch(ctx, "k_blk_split_rows"))) return rc;
  for (int k0 = 0; k0 < K; k0 += kBK)
    if ((rc = fh_blk_convert(ctx, b, D, ldd, k0, 0))) return rc;
  fh_dbuf pairs;
  if ((rc = fh_alloc(ctx, pairs, sizeof(float2) * (size_t)kBM * b.Ppad, false))) return rc;
  if ((rc = fh_blk_gemm(ctx, b, K, pairs.as<float2>(), b.Ppad, 0))) return rc;
  k_pairs_to_double<<<dim3((unsigned)fh_ceil_div(P, 256), kBM), 256, 0, ctx->stream>>>(pairs.as<float2>(), b.Ppad, P,
                                                                                      S, ldS);
  if ((rc = fh_after_launch(ctx, "k_pairs_to_double"))) return rc;
  return fh_blk_check(ctx, b);
}
