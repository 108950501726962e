// fh_linescan.cuh -- one warp solves one grid line whose Thomas factorization
// (the alpha coefficients and the pivots) is already known.  Both remaining
// recurrences are affine maps:
//   forward   Bt[i+1] = g_i (A_i Bt[i] - Om_i)          i = 1..N-1
//   backward  u_i     = Al[i+1] u_{i+1} + Bt[i+1]       i = N-1..0
// Each lane composes the maps of a contiguous chunk, a warp scan gives every
// lane its starting value, and the lane then walks its chunk with the
// reference's own arithmetic.  The serial chain per line drops from ~2N to
// ~2N/32 + 10 dependent steps.
#pragma once
#include "fh_common.cuh"
#include "fh_df.cuh"

// Reverse exclusive scan: lane l receives G_{l+1} o G_{l+2} o ... o G_31
// (identity for lane 31), i.e. the maps of all higher lanes applied first.
__device__ __forceinline__ fh_aff fh_warp_exclusive_affine_rev(fh_aff f) {
  const unsigned lane = threadIdx.x & 31u;
  fh_aff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    double pa = __shfl_down_sync(0xffffffffu, g.a, d);
    double pb = __shfl_down_sync(0xffffffffu, g.b, d);
    if (lane + d < 32u) g = fh_aff_compose(g, fh_aff{pa, pb});
  }
  double ea = __shfl_down_sync(0xffffffffu, g.a, 1);
  double eb = __shfl_down_sync(0xffffffffu, g.b, 1);
  if (lane == 31u) {
    ea = 1.0;
    eb = 0.0;
  }
  return fh_aff{ea, eb};
}

// Line accessor contract (all lanes call with the same line):
//   double om(int i)      right part Om_i, i = 1..N-1
//   double A(int i)       sub-diagonal A_i
//   double g(int i)       pivot factor g_i = Al[i+1]/B_i (or 1/(R_i - A_i Al_i) when Al[i+1] = B_i = 0)
//   double al(int i)      Al[i+1] for i = 1..N-1
//   void   store(int i, double u)   writes u_i, i = 0..N+1
// buf: per-warp shared scratch of N+1 doubles.
template <class Line>
__device__ __forceinline__ void fh_line_solve_cached(const Line &L, int N, double al1, double bt1, double *buf) {
  const int lane = threadIdx.x & 31;
  // ---- forward: Bt[i+1] for i = 1..N-1, stored at buf[i]; buf[0] = Bt[1]
  const int nf = N - 1;
  const int chf = (nf + 31) / 32;
  const int f0 = 1 + lane * chf, f1 = min(N, f0 + chf);
  fh_aff F{1.0, 0.0};
  for (int i = f0; i < f1; ++i) {
    const double om = L.om(i), a = L.A(i), g = L.g(i);
    buf[i] = om;
    F = fh_aff_compose(fh_aff{g * a, -g * om}, F);
  }
  const fh_aff Pf = fh_warp_exclusive_affine(F);
  double bt = fma(Pf.a, bt1, Pf.b);
  for (int i = f0; i < f1; ++i) {
    bt = L.g(i) * (L.A(i) * bt - buf[i]);
    buf[i] = bt;
  }
  if (lane == 0) buf[0] = bt1;
  __syncwarp();
  // ---- u_N = Bt[N] / (1 - Al[N])
  const double alN = (N >= 2) ? L.al(N - 1) : al1;
  const double uN = buf[N - 1] / (1.0 - alN);
  // ---- backward: u_i = Al[i+1] u_{i+1} + Bt[i+1], i = N-1..0
  const int chb = (N + 31) / 32;
  const int b0 = lane * chb, b1 = min(N, b0 + chb);
  // chunk map G = h_{b0} o h_{b0+1} o ... o h_{b1-1} (h_{b1-1} applied first)
  fh_aff G{1.0, 0.0};
  for (int i = b1 - 1; i >= b0; --i) {
    const double ali = (i >= 1) ? L.al(i) : al1;
    G = fh_aff_compose(fh_aff{ali, buf[i]}, G);
  }
  const fh_aff Pb = fh_warp_exclusive_affine_rev(G);
  double u = fma(Pb.a, uN, Pb.b);  // u at index b1
  for (int i = b1 - 1; i >= b0; --i) {
    const double ali = (i >= 1) ? L.al(i) : al1;
    u = ali * u + buf[i];
    L.store(i, u);
  }
  if (lane == 0) {
    L.store(N, uN);
    L.store(N + 1, uN);
  }
  __syncwarp();
}

// ------------------------------------------------------------------------
// Staged variant: the line's coefficients already sit in shared memory.
// Index skew sk(i) = i + i/16 keeps the per-lane chunks (16 consecutive
// equations per lane for lines up to 513 nodes) on distinct bank pairs.
__device__ __forceinline__ int fh_sk(int i) { return i + (i >> 4); }

// fa/fb: forward maps Bt[i+1] = fa_i Bt[i] + fb_i (i = 1..N-1); al: Al[i+1]
// (i = 1..N-1).  bt: scratch; u: result u_i (i = 0..N+1), may alias fa.
__device__ __forceinline__ void fh_line_solve_staged(int N, const double *fa, const double *fb, const double *al,
                                                     double al1, double bt1, double *bt, double *u) {
  const int lane = threadIdx.x & 31;
  const int nf = N - 1;
  const int chf = (nf + 31) / 32;
  const int f0 = 1 + lane * chf, f1 = min(N, f0 + chf);
  fh_aff F{1.0, 0.0};
  for (int i = f0; i < f1; ++i) F = fh_aff_compose(fh_aff{fa[fh_sk(i)], fb[fh_sk(i)]}, F);
  const fh_aff Pf = fh_warp_exclusive_affine(F);
  double b = fma(Pf.a, bt1, Pf.b);
  for (int i = f0; i < f1; ++i) {
    b = fma(fa[fh_sk(i)], b, fb[fh_sk(i)]);
    bt[fh_sk(i)] = b;
  }
  if (lane == 0) bt[fh_sk(0)] = bt1;
  __syncwarp();
  const double alN = (N >= 2) ? al[fh_sk(N - 1)] : al1;
  const double uN = bt[fh_sk(N - 1)] / (1.0 - alN);
  const int chb = (N + 31) / 32;
  const int b0 = lane * chb, b1 = min(N, b0 + chb);
  fh_aff G{1.0, 0.0};
  for (int i = b1 - 1; i >= b0; --i) G = fh_aff_compose(fh_aff{(i >= 1) ? al[fh_sk(i)] : al1, bt[fh_sk(i)]}, G);
  const fh_aff Pb = fh_warp_exclusive_affine_rev(G);
  double v = fma(Pb.a, uN, Pb.b);
  __syncwarp();  // u may alias fa: all forward reads are done
  for (int i = b1 - 1; i >= b0; --i) {
    v = fma((i >= 1) ? al[fh_sk(i)] : al1, v, bt[fh_sk(i)]);
    u[fh_sk(i)] = v;
  }
  if (lane == 0) {
    u[fh_sk(N)] = uN;
    u[fh_sk(N + 1)] = uN;
  }
  __syncwarp();
}

// ------------------------------------------------------------------------
// Prefix variant for a factorization that is fixed over many solves: the
// per-lane chunk products of the forward slopes (pf) and of the backward
// slopes (pb) are precomputed (fh_line_prefix_products), so each phase walks
// its chunk once from a zero start and then adds prefix * start value:
//   forward   Bt[i+1] = b0_i + pf_i Bt[f0]       pf_i = fa_{f0} ... fa_i
//   backward  u_i     = v0_i + pb_i u_{b1}       pb_i = al'_i ... al'_{b1-1}
// Two FP64 operations per equation and phase instead of three.  Chunking as in
// fh_line_solve_staged: lane l owns forward equations [1 + l chf, 1 + (l+1) chf)
// and backward nodes [l chb, (l+1) chb), chf = ceil((N-1)/32), chb = ceil(N/32).
__host__ __device__ inline int fh_chunk_f(int N) { return (N - 1 + 31) / 32; }
__host__ __device__ inline int fh_chunk_b(int N) { return (N + 31) / 32; }

// fa, fb, al, pf, pb: staged (skewed) arrays of the line; bt: scratch;
// u: result u_i (i = 0..N+1), may alias fa.
__device__ __forceinline__ void fh_line_solve_prefix(int N, const double *fa, const double *fb, const double *al,
                                                     const double *pf, const double *pb, double al1, double bt1,
                                                     double *bt, double *u) {
  const int lane = threadIdx.x & 31;
  const int chf = fh_chunk_f(N);
  const int f0 = 1 + lane * chf, f1 = min(N, f0 + chf);
  double b = 0.0;
  for (int i = f0; i < f1; ++i) {
    b = fma(fa[fh_sk(i)], b, fb[fh_sk(i)]);
    bt[fh_sk(i)] = b;
  }
  const fh_aff Pf = fh_warp_exclusive_affine(f1 > f0 ? fh_aff{pf[fh_sk(f1 - 1)], b} : fh_aff{1.0, 0.0});
  const double s = fma(Pf.a, bt1, Pf.b);  // Bt[f0]
  for (int i = f0; i < f1; ++i) bt[fh_sk(i)] = fma(pf[fh_sk(i)], s, bt[fh_sk(i)]);
  if (lane == 0) bt[fh_sk(0)] = bt1;
  __syncwarp();
  const double alN = (N >= 2) ? al[fh_sk(N - 1)] : al1;
  const double uN = bt[fh_sk(N - 1)] / (1.0 - alN);
  const int chb = fh_chunk_b(N);
  const int b0 = lane * chb, b1 = min(N, b0 + chb);
  double v = 0.0;
  __syncwarp();  // u may alias fa: all forward reads are done
  for (int i = b1 - 1; i >= b0; --i) {
    v = fma((i >= 1) ? al[fh_sk(i)] : al1, v, bt[fh_sk(i)]);
    u[fh_sk(i)] = v;
  }
  const fh_aff Pb = fh_warp_exclusive_affine_rev(b1 > b0 ? fh_aff{pb[fh_sk(b0)], v} : fh_aff{1.0, 0.0});
  const double t = fma(Pb.a, uN, Pb.b);  // u_{b1}
  for (int i = b0; i < b1; ++i) u[fh_sk(i)] = fma(pb[fh_sk(i)], t, u[fh_sk(i)]);
  if (lane == 0) {
    u[fh_sk(N)] = uN;
    u[fh_sk(N + 1)] = uN;
  }
  __syncwarp();
}

// ------------------------------------------------------------------------
// Double-float variant of fh_line_solve_prefix (arrays of (hi, lo) pairs,
// fh_df.cuh arithmetic on the FP32 pipe); same chunking and scheme.
__device__ __forceinline__ void fh_line_solve_prefix_df(int N, const float2 *fa, const float2 *fb, const float2 *al,
                                                        const float2 *pf, const float2 *pb, fh_df al1, fh_df bt1,
                                                        float2 *bt, float2 *u) {
  const int lane = threadIdx.x & 31;
  const int chf = fh_chunk_f(N);
  const int f0 = 1 + lane * chf, f1 = min(N, f0 + chf);
  fh_df b{0.f, 0.f};
  for (int i = f0; i < f1; ++i) {
    b = fh_df_fma(fh_df_from_pair(fa[fh_sk(i)]), b, fh_df_from_pair(fb[fh_sk(i)]));
    bt[fh_sk(i)] = fh_df_pair(b);
  }
  const fh_daff Pf = fh_warp_exclusive_daff(f1 > f0 ? fh_daff{fh_df_from_pair(pf[fh_sk(f1 - 1)]), b}
                                                    : fh_daff{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}});
  const fh_df s = fh_df_fma(Pf.a, bt1, Pf.b);  // Bt[f0]
  for (int i = f0; i < f1; ++i)
    bt[fh_sk(i)] = fh_df_pair(fh_df_fma(fh_df_from_pair(pf[fh_sk(i)]), s, fh_df_from_pair(bt[fh_sk(i)])));
  if (lane == 0) bt[fh_sk(0)] = fh_df_pair(bt1);
  __syncwarp();
  const fh_df alN = (N >= 2) ? fh_df_from_pair(al[fh_sk(N - 1)]) : al1;
  const fh_df uN = fh_df_div(fh_df_from_pair(bt[fh_sk(N - 1)]), fh_df_sub(fh_df{1.f, 0.f}, alN));
  const int chb = fh_chunk_b(N);
  const int b0 = lane * chb, b1 = min(N, b0 + chb);
  fh_df v{0.f, 0.f};
  __syncwarp();  // u may alias fa: all forward reads are done
  for (int i = b1 - 1; i >= b0; --i) {
    v = fh_df_fma((i >= 1) ? fh_df_from_pair(al[fh_sk(i)]) : al1, v, fh_df_from_pair(bt[fh_sk(i)]));
    u[fh_sk(i)] = fh_df_pair(v);
  }
  const fh_daff Pb = fh_warp_exclusive_daff_rev(b1 > b0 ? fh_daff{fh_df_from_pair(pb[fh_sk(b0)]), v}
                                                        : fh_daff{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}});
  const fh_df t = fh_df_fma(Pb.a, uN, Pb.b);  // u_{b1}
  for (int i = b0; i < b1; ++i)
    u[fh_sk(i)] = fh_df_pair(fh_df_fma(fh_df_from_pair(pb[fh_sk(i)]), t, fh_df_from_pair(u[fh_sk(i)])));
  if (lane == 0) {
    u[fh_sk(N)] = fh_df_pair(uN);
    u[fh_sk(N + 1)] = fh_df_pair(uN);
  }
  __syncwarp();
}

// ------------------------------------------------------------------------
// Group scans: NW warps (threads 0 .. 32 NW - 1 of the CTA) scan one chain
// of 32 NW chunk maps; warp totals pass through shared memory sm[NW] and a
// named barrier (id bar, the NW warps only).  The caller's threads must all
// call with the same NW and bar.
__device__ __forceinline__ void fh_group_bar(int bar, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
}

// Thread t receives f_{t-1} o ... o f_0 (identity for thread 0).
template <int NW>
__device__ __forceinline__ fh_aff fh_group_exclusive_affine(fh_aff f, fh_aff *sm, int bar) {
  const unsigned lane = threadIdx.x & 31u;
  const int w = threadIdx.x >> 5;
  fh_aff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const double pa = __shfl_up_sync(0xffffffffu, g.a, d);
    const double pb = __shfl_up_sync(0xffffffffu, g.b, d);
    if (lane >= (unsigned)d) g = fh_aff_compose(g, fh_aff{pa, pb});
  }
  if (lane == 31u) sm[w] = g;
  double ea = __shfl_up_sync(0xffffffffu, g.a, 1);
  double eb = __shfl_up_sync(0xffffffffu, g.b, 1);
  if (lane == 0u) {
    ea = 1.0;
    eb = 0.0;
  }
  fh_group_bar(bar, 32 * NW);
  fh_aff P{1.0, 0.0};
  for (int k = 0; k < w; ++k) P = fh_aff_compose(sm[k], P);
  fh_group_bar(bar, 32 * NW);  // sm may be reused after this
  return fh_aff_compose(fh_aff{ea, eb}, P);
}

// Thread t receives G_{t+1} o ... o G_{T-1} (identity for the last thread).
template <int NW>
__device__ __forceinline__ fh_aff fh_group_exclusive_affine_rev(fh_aff f, fh_aff *sm, int bar) {
  const unsigned lane = threadIdx.x & 31u;
  const int w = threadIdx.x >> 5;
  fh_aff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const double pa = __shfl_down_sync(0xffffffffu, g.a, d);
    const double pb = __shfl_down_sync(0xffffffffu, g.b, d);
    if (lane + d < 32u) g = fh_aff_compose(g, fh_aff{pa, pb});
  }
  if (lane == 0u) sm[w] = g;
  double ea = __shfl_down_sync(0xffffffffu, g.a, 1);
  double eb = __shfl_down_sync(0xffffffffu, g.b, 1);
  if (lane == 31u) {
    ea = 1.0;
    eb = 0.0;
  }
  fh_group_bar(bar, 32 * NW);
  fh_aff Q{1.0, 0.0};
  for (int k = NW - 1; k > w; --k) Q = fh_aff_compose(sm[k], Q);
  fh_group_bar(bar, 32 * NW);
  return fh_aff_compose(fh_aff{ea, eb}, Q);
}


// Moebius maps (FP64, rescaled by powers of two): thread t receives
// f_{t-1} o ... o f_0 (identity for thread 0).
template <int NW>
__device__ __forceinline__ fh_mob fh_group_exclusive_mob(fh_mob f, fh_mob *sm, int bar) {
  const unsigned lane = threadIdx.x & 31u;
  const int w = threadIdx.x >> 5;
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
  if (lane == 31u) sm[w] = g;
  fh_mob e;
  e.m00 = __shfl_up_sync(0xffffffffu, g.m00, 1);
  e.m01 = __shfl_up_sync(0xffffffffu, g.m01, 1);
  e.m10 = __shfl_up_sync(0xffffffffu, g.m10, 1);
  e.m11 = __shfl_up_sync(0xffffffffu, g.m11, 1);
  if (lane == 0u) e = fh_mob{1.0, 0.0, 0.0, 1.0};
  fh_group_bar(bar, 32 * NW);
  fh_mob P{1.0, 0.0, 0.0, 1.0};
  for (int k = 0; k < w; ++k) P = fh_mob_normalise(fh_mob_compose(sm[k], P));
  fh_group_bar(bar, 32 * NW);  // sm may be reused after this
  return fh_mob_normalise(fh_mob_compose(e, P));
}

// ------------------------------------------------------------------------
// Double-float group scans: NW warps (threads 0 .. 32 NW - 1 of the CTA) scan
// one chain of 32 NW chunk maps in double-float; warp totals pass through
// shared memory sm[NW] and the named barrier bar (NW warps only).
template <int NW>
__device__ __forceinline__ fh_daff fh_group_exclusive_daff(fh_daff f, fh_daff *sm, int bar) {
  const unsigned lane = threadIdx.x & 31u;
  const int w = threadIdx.x >> 5;
  fh_daff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const fh_daff p{fh_df_shfl_up(g.a, d), fh_df_shfl_up(g.b, d)};
    if (lane >= (unsigned)d) g = fh_daff_compose(g, p);
  }
  if (lane == 31u) sm[w] = g;
  fh_daff e{fh_df_shfl_up(g.a, 1), fh_df_shfl_up(g.b, 1)};
  if (lane == 0u) e = fh_daff{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}};
  fh_group_bar(bar, 32 * NW);
  fh_daff P{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}};
  for (int k = 0; k < w; ++k) P = fh_daff_compose(sm[k], P);
  fh_group_bar(bar, 32 * NW);  // sm may be reused after this
  return fh_daff_compose(e, P);
}

template <int NW>
__device__ __forceinline__ fh_daff fh_group_exclusive_daff_rev(fh_daff f, fh_daff *sm, int bar) {
  const unsigned lane = threadIdx.x & 31u;
  const int w = threadIdx.x >> 5;
  fh_daff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const fh_daff p{fh_df_shfl_down(g.a, d), fh_df_shfl_down(g.b, d)};
    if (lane + d < 32u) g = fh_daff_compose(g, p);
  }
  if (lane == 0u) sm[w] = g;
  fh_daff e{fh_df_shfl_down(g.a, 1), fh_df_shfl_down(g.b, 1)};
  if (lane == 31u) e = fh_daff{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}};
  fh_group_bar(bar, 32 * NW);
  fh_daff Q{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}};
  for (int k = NW - 1; k > w; --k) Q = fh_daff_compose(sm[k], Q);
  fh_group_bar(bar, 32 * NW);
  return fh_daff_compose(e, Q);
}
