// fh_h.cu -- batched 1D H_solver path (mt_minimal.cpp:276-1048 and
// mt_psi_caputo.cpp:369-1507 with gamma = 1): per step
//   1. k_h_weights      per-instance history weights and current weight
//   2. k_hist_tiles     history sum per instance segment (split-K partials)
//   3. k_h_line_warp    one warp per instance: coefficients, right part,
//                       Thomas sweep as warp scans, back substitution,
//                       history append
//
// All instances advance in lock step.  The concatenated state holds each
// instance's N_i+2 nodes in a segment padded to an even length; the history
// stores layer differences d_t = layer[t+1] - layer[t] at slot t for the
// concatenated state (layer-major), so the history loads coalesce across
// neighbouring nodes and instances.
#include <cooperative_groups.h>

#include <utility>
#include <vector>

#include "fh_internal.h"
#include "fh_common.cuh"
#include "fh_linescan.cuh"
#include "fh_df.cuh"
#include "fh_slices.cuh"
#include "fh_weights.cuh"

// batched far contraction on the tensor cores (fh_blocked.cu)
struct fh_hblk;
fh_hblk *fh_hblk_new();
void fh_hblk_delete(fh_hblk *b);
int fh_hblk_init(fh_ctx *ctx, fh_hblk &b, long long P, int Kcap, int ninst, const long long *tile_p0,
                 const int *tile_inst, const int *tile_np, int ntiles);
int fh_hblk_convert(fh_ctx *ctx, fh_hblk &b, const float2 *ring, long long ldd, int c);
int fh_hblk_gemm(fh_ctx *ctx, fh_hblk &b, int K, float2 *far, long long ldf);
int fh_hblk_check(fh_ctx *ctx, fh_hblk &b);
__nv_bfloat16 *fh_hblk_wplanes(fh_hblk &b);
int8_t *fh_hblk_wexp(fh_hblk &b);
int fh_hblk_kcap(const fh_hblk &b);
size_t fh_hblk_bytes(const fh_hblk &b);

struct fh_h_dev_inst {
  int N, weights, kmodel, gravity;
  int fixed;  // coefficients independent of u and of the step: factor once
  // the instance's own clock (fh_h_batch_restart): its step is tstep - tb and
  // its saved-layer count nsaved - ob; history slots below ob belong to an
  // earlier occupant and are never read
  int tb, ob;
  long long off;  // segment start in the concatenated state
  double dL, Dg, Da, tau, alpha, beta, kc, kgam, cinv, al_left, bt_left, u_right;
  // space-fractional derivative in z (fh_h_batch_set_space_order): order
  // spg, spA = 1 - spg (0: classical second derivative), kbf = the
  // mt_psi_caputo factor kb(gamma, i-1, i, i) of A, B, R
  double spg, spA, kbf;
};

struct fh_h_tile {
  int inst;
  int start;  // first node of the tile inside the segment
  int len;    // nodes in the tile (even)
};

struct fh_h_batch {
  fh_ctx *ctx = nullptr;
  int n = 0, max_steps = 0, tstep = 1, nsaved = 0, max_splits = 64, max_weights = 0;
  // history-sum launch shape (fh_h_batch_autotune): threads per tile CTA (two
  // nodes each) and the cap on K splits; one tile list per candidate shape
  int tile_threads = 256, split_cap = 64;
  std::vector<fh_h_tile> tiles_by[3];
  fh_dbuf tl_by[3];
  long long Ptot = 0;
  std::vector<fh_h_params> hp;
  std::vector<long long> off;
  fh_dbuf inst, U, D, W, Lb, ibt, lgt, wc, part, Al, Bt, sA, sB, sR, sOm;
  fh_graph_cache graph;
  bool use_graph = true;
  int mode = FH_H_FP64;  // FH_H_DF64: history as (hi, lo) FP32 pairs; FH_H_BLOCKED: below
  // Al of the variable-coefficient instances serially in the reference order
  // (h_alpha_serial); varcoef: the batch has such instances
  bool serial_al = true, varcoef = false;
  bool persistent = true;  // small FP64 batches: one launch per call (k_h_persistent)
  std::vector<fh_h_dev_inst> di;  // host copy of inst
  std::vector<int> cap;           // nodes a restarted occupant of each instance may have (segment - 2)
  // space-fractional instances: Toeplitz weights wsp and the sums sV per
  // node (state layout), shared memory of k_h_space_v
  bool space = false;
  size_t space_smem = 0;
  fh_dbuf wsp, sV;
  // weights of the next step on hs (h_one_step): two buffer pairs of W and
  // wc, selected by the parity of the step; w_ready = step whose weights
  // are pending on hs behind ev_w
  cudaStream_t hs = nullptr;
  cudaEvent_t ev_main = nullptr, ev_w = nullptr;
  int w_ready = -1;
  // FH_H_BLOCKED: history slots older than the current 64-step block in bf16
  // slice planes (hb), contracted once per block for its 64 steps into far
  // rows; the slots of the last two chunks as (hi, lo) pairs in a 128-layer
  // ring (slot t in row t mod 128)
  fh_hblk *hb = nullptr;
  fh_dbuf ring, far, cheb;  // cheb: interpolation tables of k_hb_wcheb
  bool has_l1 = false;      // some instance has L1 weights (k_hb_weights covers every group)
  double *Wp(int par) const { return W.as<double>() + (long long)par * n * max_weights; }
  double *wcp(int par) const { return wc.as<double>() + (long long)par * n; }
  ~fh_h_batch() {
    if (hb) fh_hblk_delete(hb);
    if (hs) cudaStreamDestroy(hs);
    if (ev_main) cudaEventDestroy(ev_main);
    if (ev_w) cudaEventDestroy(ev_w);
  }
};

static constexpr int kTileThreads = 512;  // largest tile CTA (1024 nodes)
static constexpr int kTileShapes[3] = {128, 256, 512};  // candidate tile CTAs
static inline int tile_shape_index(int threads) { return threads == 128 ? 0 : threads == 256 ? 1 : 2; }
static constexpr int kLineCtaMaxInst = 152;  // batches below this many instances solve one CTA per instance
static constexpr int kSpaceMaxN = 2048;  // nodes of a space-fractional instance (shared-memory sums)
static constexpr int kHWeightThreads = 128;                 // slots per weights CTA
// per psi instance: Lc[kIbTerms] | Uc[kIbTerms] | B(a, b) | kIbLowMax^(1/beta) |
// log tau | 1/beta
static constexpr int kIbStride = 2 * kIbTerms + 4;

// ------------------------------------------------------------------ kernels

// Row b of W: the weights of instance b for the history slots t = 0..os-2,
// and wc[b], the weight of the current slot [tstep, tstep + 1].  The
// reference's t = 0 term multiplies layer1 - layer1 (its layer pointer starts
// at old[1], mt_minimal.cpp:913-917), so slot 0 carries weight 0.
// Thread i of CTA (x, b) owns slot i = t_lo + x*128 + threadIdx.x (slots below
// t_lo are not computed); i = max(os - 1, 0) is the current slot.
// Weight of slot i of instance b at its step tstep with os saved layers
// (cur: the current slot's weight, the factor of the newest difference);
// invX = 1 / (tstep + 1).  The arithmetic of every weight kind as described
// at k_h_weights.
__device__ __forceinline__ double h_slot_weight(const fh_h_dev_inst &I, int b, int i, bool cur, int tstep, int os,
                                                double invX, int ldw, const double *__restrict__ Lb,
                                                const double *__restrict__ ibt, const double2 *__restrict__ lgt) {
  if (I.weights == FH_W_PSI && I.beta != 1.0) {
    // psi = t^beta: the interval [x0, x0 + 1] in the divided-difference form of
    // fh_ib_diff, with the per-instance series tables and the logs as
    // double-doubles from the table of log(x)
    if (i == 0 && !cur) return 0.0;
    const double *Lc = ibt + (long long)b * kIbStride, *Uc = Lc + kIbTerms;
    const int X = tstep + 1, x0 = cur ? tstep : i, x1 = x0 + 1;
    // p - q as a double-double for log values 0 <= p <= q (fast two-sum)
    auto dd_sub = [](double2 p, double2 q, double &h, double &l) {
      h = p.x - q.x;
      l = (p.x - (h + q.x)) + (p.y - q.y);
    };
    const double2 lX = lgt[X], l0 = lgt[x0], l1 = lgt[x1];
    fh_ib_slot q;
    q.zero0 = x0 == 0;
    q.top = x1 == X;
    q.r0 = (double)x0 * invX;
    q.r1 = (double)x1 * invX;
    q.dr = invX;
    dd_sub(l1, lX, q.l1h, q.l1l);  // log(x1/X)
    dd_sub(l0, lX, q.l0h, q.l0l);  // log(x0/X)
    dd_sub(l0, l1, q.ldh, q.ldl);  // log(x0/x1) = -log(x1/x0)
    q.ldh = -q.ldh;
    q.ldl = -q.ldl;
    const double bb = 1.0 - I.alpha;
    const double diff = fh_ib_diff(q, I.beta, bb, Lc[2 * kIbTerms + 1], [&] { return Lc[2 * kIbTerms]; },
                                   fh_ib_coef_tab{Lc}, fh_ib_coef_tab{Uc});
    // (X tau)^(1 - alpha beta) / beta with log X from the table: one exp
    const double sc = exp((1.0 - I.alpha * I.beta) * (lX.x + Lc[2 * kIbTerms + 2])) * Lc[2 * kIbTerms + 3];
    return sc * diff * (1 - I.alpha);
  }
  if (cur)
    return (I.weights == FH_W_L1)
               ? 1.0
               : fh_psi_int_t((double)tstep, (double)tstep + 1.0, (double)(tstep + 1), I.tau, I.alpha) *
                     (1 - I.alpha);
  const int t = i;
  if (t == 0) return 0.0;
  if (I.weights == FH_W_L1) return Lb[(long long)b * ldw + (os - t - 1)];  // L1 weights depend on the lag only
  return fh_psi_int_t((double)t, (double)t + 1.0, (double)(tstep + 1), I.tau, I.alpha) * (1 - I.alpha);
}

__global__ void k_h_weights(const fh_h_dev_inst *__restrict__ inst, int n, int tstep_g, int os_g, int t_lo,
                            double *__restrict__ W_g, int ldw, double *__restrict__ wc, const double *__restrict__ Lb,
                            const double *__restrict__ ibt, const double2 *__restrict__ lgt, double invX_g) {
  const int b = blockIdx.y;
  const fh_h_dev_inst I = inst[b];
  // the instance's own step and slot numbers; its slot i is column I.ob + i
  const int tstep = tstep_g - I.tb, os = os_g - I.ob;
  double *W = W_g + I.ob;
  const double invX = I.tb == 0 ? invX_g : 1.0 / (double)(tstep + 1);
  const int i = t_lo + blockIdx.x * kHWeightThreads + threadIdx.x;
  const int nh = os > 1 ? os - 1 : 0;  // history slots
  if (i > nh) return;
  const bool cur = i == nh;
  const double w = h_slot_weight(I, b, i, cur, tstep, os, invX, ldw, Lb, ibt, lgt);
  if (cur)
    wc[b] = w;
  else
    W[(long long)b * ldw + i] = w;
}

// Incomplete-beta series coefficients of every psi instance (fh_ib_tables).
__global__ void k_h_ibtab(const fh_h_dev_inst *__restrict__ inst, int n, double *__restrict__ ibt) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const fh_h_dev_inst I = inst[b];
  if (I.weights != FH_W_PSI) return;
  const double a = 1.0 / I.beta, bb = 1.0 - I.alpha;
  double *row = ibt + (long long)b * kIbStride;
  fh_ib_tables(a, bb, row, row + kIbTerms);
  row[2 * kIbTerms] = exp(lgamma(a) + lgamma(bb) - lgamma(a + bb));  // B(a, b)
  row[2 * kIbTerms + 1] = pow(kIbLowMax, a);                         // y <= kIbLowMax <=> x/X <= this
  row[2 * kIbTerms + 2] = log(I.tau);
  row[2 * kIbTerms + 3] = a;                                          // 1/beta
}

// Lag table of the L1 instances: Lb[b][l] = (l+1)^(1-a) - l^(1-a) (mt_minimal.cpp:930),
// the weight of the layer difference l steps back.
__global__ void k_h_lagtab(const fh_h_dev_inst *__restrict__ inst, int nlag, double *__restrict__ Lb, int ldw) {
  const int b = blockIdx.y;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const fh_h_dev_inst I = inst[b];
  if (I.weights != FH_W_L1 || l >= nlag) return;
  Lb[(long long)b * ldw + l] = pow((double)(l + 1), 1.0 - I.alpha) - pow((double)l, 1.0 - I.alpha);
}

// part[s][p] = sum_{k in split s} W[inst][k] * D[k][p] over one tile of one instance.
__global__ void __launch_bounds__(kTileThreads) k_hist_tiles(const fh_h_tile *__restrict__ tiles,
                                                             const fh_h_dev_inst *__restrict__ inst,
                                                             const double *__restrict__ D, long long ldd, int K,
                                                             const double *__restrict__ W, int ldw, int kchunk,
                                                             double *__restrict__ part, long long ldpart) {
  extern __shared__ double ws[];
  const fh_h_tile T = tiles[blockIdx.x];
  const int s = blockIdx.y;
  const int k0 = s * kchunk;
  const int nk = min(K, k0 + kchunk) - k0;
  const double *wrow = W + (long long)T.inst * ldw + k0;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) ws[i] = wrow[i];
  __syncthreads();
  const int q = threadIdx.x * 2;
  if (q >= T.len) return;
  const fh_h_dev_inst &I = inst[T.inst];
  const long long p = I.off + T.start + q;
  double a0 = 0.0, a1 = 0.0;
  int k = max(0, I.ob - k0);  // slots of the instance's current occupant only
  const double *d = D + (long long)(k0 + k) * ldd + p;
  for (; k + 4 <= nk; k += 4) {
    const double2 v0 = fh_ld_stream2(d), v1 = fh_ld_stream2(d + ldd);
    const double2 v2 = fh_ld_stream2(d + 2 * ldd), v3 = fh_ld_stream2(d + 3 * ldd);
    d += 4 * ldd;
    a0 = fma(ws[k], v0.x, a0);
    a1 = fma(ws[k], v0.y, a1);
    a0 = fma(ws[k + 1], v1.x, a0);
    a1 = fma(ws[k + 1], v1.y, a1);
    a0 = fma(ws[k + 2], v2.x, a0);
    a1 = fma(ws[k + 2], v2.y, a1);
    a0 = fma(ws[k + 3], v3.x, a0);
    a1 = fma(ws[k + 3], v3.y, a1);
  }
  for (; k < nk; ++k) {
    const double2 v = fh_ld_stream2(d);
    d += ldd;
    a0 = fma(ws[k], v.x, a0);
    a1 = fma(ws[k], v.y, a1);
  }
  double2 o;
  o.x = a0;
  o.y = a1;
  *reinterpret_cast<double2 *>(part + (long long)s * ldpart + p) = o;
}

// Double-float history ((hi, lo) FP32 pairs): the same tile sum with the
// weights split into pairs in shared memory and the sums carried in
// double-float on the FP32 pipe (2^-48 storage precision, HBM-bound).
__global__ void __launch_bounds__(kTileThreads) k_hist_tiles_df(const fh_h_tile *__restrict__ tiles,
                                                                const fh_h_dev_inst *__restrict__ inst,
                                                                const float2 *__restrict__ D, long long ldd, int K,
                                                                const double *__restrict__ W, int ldw, int kchunk,
                                                                double *__restrict__ part, long long ldpart) {
  extern __shared__ float2 wsf2[];
  const fh_h_tile T = tiles[blockIdx.x];
  const int s = blockIdx.y;
  const int k0 = s * kchunk;
  const int nk = min(K, k0 + kchunk) - k0;
  const double *wrow = W + (long long)T.inst * ldw + k0;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) wsf2[i] = fh_df_pair(fh_df_from_double(wrow[i]));
  __syncthreads();
  const int q = threadIdx.x * 2;
  if (q >= T.len) return;
  const fh_h_dev_inst &I = inst[T.inst];
  const long long p = I.off + T.start + q;
  fh_df a0{0.f, 0.f}, a1{0.f, 0.f};
  int k = max(0, I.ob - k0);  // slots of the instance's current occupant only
  const float4 *d = reinterpret_cast<const float4 *>(D + (long long)(k0 + k) * ldd + p);
  const long long ld4 = ldd / 2;
  for (; k + 4 <= nk; k += 4) {
    float4 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = __ldcs(d + u * ld4);
    d += 4 * ld4;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const fh_df w = fh_df_from_pair(wsf2[k + u]);
      a0 = fh_df_fma(w, fh_df{v[u].x, v[u].y}, a0);
      a1 = fh_df_fma(w, fh_df{v[u].z, v[u].w}, a1);
    }
  }
  for (; k < nk; ++k) {
    const float4 v = __ldcs(d);
    d += ld4;
    const fh_df w = fh_df_from_pair(wsf2[k]);
    a0 = fh_df_fma(w, fh_df{v.x, v.y}, a0);
    a1 = fh_df_fma(w, fh_df{v.z, v.w}, a1);
  }
  double2 o;
  o.x = fh_df_to_double(a0);
  o.y = fh_df_to_double(a1);
  *reinterpret_cast<double2 *>(part + (long long)s * ldpart + p) = o;
}

// Space-fractional Caputo derivative in z (gamma < 1): H_solver::Om1 adds
// -Dg/(dw/dh) (K_i V_i - K_{i-1} V_{i-1}) with V_i = sum_{j<i} w_{i-j} F_j over
// the first differences F_j = u_{j+1} - u_j of the current state
// (calc_v, mt_minimal.cpp:228-271, mt_psi_caputo.cpp:749-777, with_zero 1).
// The weights depend on i - j only: mt_minimal (m+1)^A - m^A, mt_psi_caputo
// A kb_space of one interval at distance m+1 (1461-1472; psi = x in space;
// the reference tabulates kb_space[i][j-1], equal up to rounding).
// wsp[off + m], m = 1..N-1, per instance.
__global__ void k_h_spw(const fh_h_dev_inst *__restrict__ inst, double *__restrict__ wsp) {
  const fh_h_dev_inst I = inst[blockIdx.y];
  if (I.spA == 0.0) return;
  for (int m = 1 + blockIdx.x * blockDim.x + threadIdx.x; m < I.N; m += gridDim.x * blockDim.x)
    wsp[I.off + m] = I.weights == FH_W_L1
                         ? pow((double)m + 1, I.spA) - pow((double)m, I.spA)
                         : I.spA * fh_psi_int_t(0.0, 1.0, (double)m + 1.0, I.dL, I.spg);
}

// V_i of one instance per CTA (F and the weights in shared memory), i =
// 1..N-1; V_0 = 0.  O(N^2) FP64 FMAs per instance and step, as the reference
// (FP64-pipe-bound; a double-float form on the FP32 pipe ran 3.4x faster but
// the flux difference K_i V_i - K_{i-1} V_{i-1} amplified its 2^-48 products
// to 1e-10 of the solution at N ~ 1000).  Rows go to threads in snake order
// (t, 2T-1-t, 2T+t, ...) so that every thread sums about as many terms.
__global__ void __launch_bounds__(256) k_h_space_v(const fh_h_dev_inst *__restrict__ inst, const double *__restrict__ U,
                                                   const double *__restrict__ wsp, double *__restrict__ V) {
  extern __shared__ double spm[];
  const fh_h_dev_inst I = inst[blockIdx.x];
  if (I.spA == 0.0) return;
  const int N = I.N;
  const double *u = U + I.off;
  double *F = spm, *w = spm + N;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    F[j] = u[j + 1] - u[j];
    w[j] = wsp[I.off + j];
  }
  __syncthreads();
  const int T = blockDim.x;
  for (int r = 0; r * T < N - 1; ++r) {
    const int i = 1 + r * T + ((r & 1) ? T - 1 - (int)threadIdx.x : (int)threadIdx.x);
    if (i >= N) continue;
    double v = 0.0;
    for (int j = 0; j < i; ++j) v = fma(w[i - j], F[j], v);
    V[I.off + i] = v;
  }
  if (threadIdx.x == 0) V[I.off] = 0.0;
}

__device__ __forceinline__ double fh_h_K(const fh_h_dev_inst &I, double u) {
  return I.kmodel == FH_K_CONST ? I.kc : I.kc * exp(I.kgam * u);
}

// New history entry: FP64, or a (hi, lo) FP32 pair in the double-float mode.
__device__ __forceinline__ void fh_h_store_diff(double *D, long long i, double d, int dfstore) {
  if (dfstore)
    reinterpret_cast<float2 *>(D)[i] = fh_df_pair(fh_df_from_double(d));
  else
    D[i] = d;
}

// H_solver::U1 with one warp per instance (al1, Om1, bt1, bottom Dirichlet,
// back substitution, history append).  The serial recurrences become warp
// scans over per-lane chunks of consecutive equations:
//   Al[i+1] = B_i / (R_i - A_i Al[i])            Moebius maps (matrix scan)
//   Bt[i+1] = (Al[i+1]/B_i)(A_i Bt[i] - Om_i)    affine maps
//   u_i     = Al[i+1] u_{i+1} + Bt[i+1]           affine maps, reverse order
// after which every lane re-walks its chunk from the scanned start value with
// one reciprocal per equation (Al[i+1] = B_i g, g = 1 / (R_i - A_i Al[i])).  The coefficients are kept in the scratch
// arrays sA, sB, sR (reused for Al[i+1]/B_i) and sOm at the equation's node.
// Scans and syncs of one instance's group of threads: one warp (NW = 1) or
// the whole CTA (NW warps, named barrier 1).
template <int NW>
struct HGroup {
  static __device__ __forceinline__ fh_mob mob(fh_mob f, fh_mob *sm) { return fh_group_exclusive_mob<NW>(f, sm, 1); }
  static __device__ __forceinline__ fh_aff aff(fh_aff f, fh_aff *sm) { return fh_group_exclusive_affine<NW>(f, sm, 1); }
  static __device__ __forceinline__ fh_aff aff_rev(fh_aff f, fh_aff *sm) {
    return fh_group_exclusive_affine_rev<NW>(f, sm, 1);
  }
  static __device__ __forceinline__ void sync() { __syncthreads(); }
};
template <>
struct HGroup<1> {
  static __device__ __forceinline__ fh_mob mob(fh_mob f, fh_mob *) { return fh_warp_exclusive_mob(f); }
  static __device__ __forceinline__ fh_aff aff(fh_aff f, fh_aff *) { return fh_warp_exclusive_affine(f); }
  static __device__ __forceinline__ fh_aff aff_rev(fh_aff f, fh_aff *) { return fh_warp_exclusive_affine_rev(f); }
  static __device__ __forceinline__ void sync() { __syncwarp(); }
};

// Parts of the line solve one launch runs: everything (kLineAll), the
// coefficients and right parts only (kLineCoef), or the sweeps from an Al
// already in memory (kLineSolve; k_h_alpha_lanes writes it in between).
enum { kLineAll = 0, kLineCoef = 1, kLineSolve = 2 };

// Al[i+1] = B_i / (R_i - A_i Al[i]) for i = 1..N-1 from Al[1], serially in the
// order and arithmetic of H_solver::al1 (mt_psi_caputo.cpp:1262-1292,
// mt_minimal.cpp:829-858): the product, the difference and the quotient are
// each rounded once (no contraction), so the factors are those of the
// reference for the same coefficients.  The Thomas factors of a diffusion line
// are a weakly contracting recurrence: any re-association of it (a parallel
// scan) changes every factor by a few ulps, and over hundreds of steps of a
// 1000-node line those changes grew to 1e-10 of the solution.
__device__ __forceinline__ void h_alpha_serial(int N, double al_left, const double *__restrict__ A,
                                               const double *__restrict__ B, const double *__restrict__ R,
                                               double *__restrict__ Al) {
  double a = al_left;
  Al[1] = a;
  int i = 1;
  for (; i + 4 <= N; i += 4) {  // coefficient loads ahead of the dependent chain
    double Aq[4], Bq[4], Rq[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      Aq[k] = A[i + k];
      Bq[k] = B[i + k];
      Rq[k] = R[i + k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a = __ddiv_rn(Bq[k], __dsub_rn(Rq[k], __dmul_rn(Aq[k], a)));
      Al[i + k + 1] = a;
    }
  }
  for (; i < N; ++i) {
    a = __ddiv_rn(B[i], __dsub_rn(R[i], __dmul_rn(A[i], a)));
    Al[i + 1] = a;
  }
}

// One instance by a group of 32 NW threads; `lane` is the thread's index in
// the group (its chunk of consecutive equations).  serial: Al of the
// variable-coefficient instances serially (h_alpha_serial, by lane 0 in
// kLineAll launches); otherwise by the Moebius scan (kLineAll only).
template <int NW, bool SPACE, int PH>
__device__ __forceinline__ void h_line(const fh_h_dev_inst &I, int b, int lane, double *__restrict__ U,
                                       const double *__restrict__ wc, const double *__restrict__ part,
                                       long long ldpart, int splits, double *__restrict__ Al,
                                       double *__restrict__ Bt, double *__restrict__ sA, double *__restrict__ sB,
                                       double *__restrict__ sR, double *__restrict__ sOm, double *__restrict__ Dnew,
                                       int append, int os, int dfstore, const double *__restrict__ sV,
                                       fh_mob *smm, fh_aff *sma, int serial) {
  constexpr int TG = 32 * NW;
  const bool first = os == I.ob;  // the instance's first step (saved-layer count os)
  const long long o = I.off;
  double *u = U + o;
  const int N = I.N;
  const double DaW = I.Da * wc[b];
  // ---- pass 1: coefficients of equations i in [f0, f1), chunk Moebius map;
  // the products and sums in the reference's order, each rounded once
  const int chf = (N - 1 + TG - 1) / TG;
  const int f0 = 1 + lane * chf, f1 = min(N, f0 + chf);
  fh_mob T{1.0, 0.0, 0.0, 1.0};
  if (PH != kLineSolve && f0 < f1) {
    double Km = fh_h_K(I, u[f0 - 1]), Kc = fh_h_K(I, u[f0]);
    for (int i = f0; i < f1; ++i) {
      const double Kp = fh_h_K(I, u[i + 1]);
      double A = I.Dg * Km * I.cinv;
      double B = I.Dg * Kp * I.cinv;
      double R = I.cinv * (Kp + Km) * I.Dg;
      double om = -DaW * u[i];
      if (SPACE && I.spA != 0.0) {  // space-fractional derivative (k_h_space_v)
        if (I.weights == FH_W_PSI) {
          A = A * I.kbf * I.spA;
          B = B * I.kbf * I.spA;
          R = R * I.kbf * I.spA;
        }
        const double flux = __dsub_rn(__dmul_rn(Kc, sV[o + i]), __dmul_rn(Km, sV[o + i - 1]));
        om = __dsub_rn(-I.Dg * I.cinv * flux, DaW * u[i]);
      }
      R = __dadd_rn(R, DaW);
      if (I.gravity) om = __dadd_rn(om, __ddiv_rn(Kc - Km, I.dL));
      double ts = 0.0;
      for (int s = 0; s < splits; ++s) ts += part[(long long)s * ldpart + o + i];
      om = __dadd_rn(om, __dmul_rn(I.Da, ts));
      sOm[o + i] = om;
      if (!I.fixed || first) {
        sA[o + i] = A;
        sB[o + i] = B;
        sR[o + i] = R;
      }
      if (!I.fixed && !serial) {
        T = fh_mob_compose(fh_mob{0.0, B, -A, R}, T);
        if (((i - f0) & 7) == 7) T = fh_mob_normalise(T);
      }
      Km = Kc;
      Kc = Kp;
    }
  }
  if (PH == kLineCoef) return;
  fh_aff F{1.0, 0.0};
  if (I.fixed || serial) {
    // Al serially in the reference order (h_alpha_serial): once for constant
    // coefficients (kept for later steps), every step otherwise; then
    // sR[i] = Al[i+1] / B_i, the reference's factor of the Bt recurrence
    const bool need = I.fixed ? first : PH == kLineAll;
    if (need) {
      HGroup<NW>::sync();
      if (lane == 0) h_alpha_serial(N, I.al_left, sA + o, sB + o, sR + o, Al + o);
      HGroup<NW>::sync();
    }
    if (!I.fixed || first)
      for (int i = f0; i < f1; ++i) sR[o + i] = __ddiv_rn(Al[o + i + 1], sB[o + i]);
    for (int i = f0; i < f1; ++i) {
      const double gq = sR[o + i];
      F = fh_aff_compose(fh_aff{gq * sA[o + i], -(gq * sOm[o + i])}, F);
    }
  } else {
    // ---- Al: Moebius scan, re-walk with the reference arithmetic, chunk affine map of Bt
    const fh_mob PT = HGroup<NW>::mob(T, smm);
    double alv = (lane == 0) ? I.al_left : fma(PT.m00, I.al_left, PT.m01) / fma(PT.m10, I.al_left, PT.m11);
    for (int i = f0; i < f1; ++i) {
      const double A = sA[o + i], B = sB[o + i], R = sR[o + i], om = sOm[o + i];
      const double gq = 1.0 / (R - A * alv);  // Al[i+1] / B_i
      const double aln = B * gq;
      Al[o + i + 1] = aln;
      sR[o + i] = gq;
      F = fh_aff_compose(fh_aff{gq * A, -(gq * om)}, F);
      alv = aln;
    }
    if (lane == 0) Al[o + 1] = I.al_left;
  }
  // ---- Bt: scan, re-walk Bt[i+1] = (Al[i+1]/B)(A Bt[i] - Om)
  const fh_aff PF = HGroup<NW>::aff(F, sma);
  double btv = (lane == 0) ? I.bt_left : fma(PF.a, I.bt_left, PF.b);
  for (int i = f0; i < f1; ++i) {
    btv = sR[o + i] * (sA[o + i] * btv - sOm[o + i]);
    Bt[o + i + 1] = btv;
  }
  if (lane == 0) Bt[o + 1] = I.bt_left;
  HGroup<NW>::sync();
  // ---- back substitution u_i = Al[i+1] u_{i+1} + Bt[i+1], i = N-1..0; u_N = u_right
  const double uN = I.u_right;
  const int chb = (N + TG - 1) / TG;
  const int b0 = lane * chb, b1 = min(N, b0 + chb);
  fh_aff G{1.0, 0.0};
  for (int i = b1 - 1; i >= b0; --i) G = fh_aff_compose(fh_aff{Al[o + i + 1], Bt[o + i + 1]}, G);
  const fh_aff PG = HGroup<NW>::aff_rev(G, sma);
  double un = fma(PG.a, uN, PG.b);  // u at node b1
  // every lane reads the old values of its own nodes before writing them
  for (int i = b1 - 1; i >= b0; --i) {
    un = Al[o + i + 1] * un + Bt[o + i + 1];
    const double old = u[i];
    u[i] = un;
    if (append) fh_h_store_diff(Dnew, o + i, un - old, dfstore);
  }
  if (lane == 0) {
    const double oldN = u[N], oldG = u[N + 1];
    u[N] = uN;
    u[N + 1] = uN;
    if (append) {
      fh_h_store_diff(Dnew, o + N, uN - oldN, dfstore);
      fh_h_store_diff(Dnew, o + N + 1, uN - oldG, dfstore);
    }
  }
}

// SPACE: the batch has space-fractional instances (a separate instantiation
// keeps the registers of the classical path).  PH: the part of the line solve
// (kLineAll with the Moebius scan for Al, or kLineCoef / kLineSolve around
// k_h_alpha_lanes).  Seven resident CTAs per SM (registers <= 73) keep 4096
// instances (1024 CTAs) in one wave on 152 SMs.
template <bool SPACE, int PH>
__global__ void __launch_bounds__(128, 7) k_h_line_warp(const fh_h_dev_inst *__restrict__ inst, int n,
                                                     double *__restrict__ U, const double *__restrict__ wc,
                                                     const double *__restrict__ part, long long ldpart, int splits,
                                                     double *__restrict__ Al, double *__restrict__ Bt,
                                                     double *__restrict__ sA, double *__restrict__ sB,
                                                     double *__restrict__ sR, double *__restrict__ sOm,
                                                     double *__restrict__ Dnew, int append, int os,
                                                     int dfstore, const double *__restrict__ sV) {
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (b >= n) return;  // whole warp
  h_line<1, SPACE, PH>(inst[b], b, threadIdx.x & 31, U, wc, part, ldpart, splits, Al, Bt, sA, sB, sR, sOm, Dnew,
                       append, os, dfstore, sV, nullptr, nullptr, PH != kLineAll);
}

// Al of every variable-coefficient instance (h_alpha_serial), one lane per
// instance: the chain is FP64 latency (~650 cycles per equation on GB300), so
// 32 instances share each warp instruction, and one warp per CTA spreads the
// chains over the SMs.
__global__ void __launch_bounds__(32) k_h_alpha_lanes(const fh_h_dev_inst *__restrict__ inst, int n,
                                                      const double *__restrict__ sA, const double *__restrict__ sB,
                                                      const double *__restrict__ sR, double *__restrict__ Al) {
  const int b = blockIdx.x * 32 + threadIdx.x;
  if (b >= n) return;
  const fh_h_dev_inst I = inst[b];
  if (I.fixed) return;
  h_alpha_serial(I.N, I.al_left, sA + I.off, sB + I.off, sR + I.off, Al + I.off);
}

// Small batches (fewer instances than SMs): one CTA of kLineCtaWarps warps per
// instance, so that each thread walks ~N/256 equations instead of ~N/32; Al
// serially by thread 0 (serial != 0) or by the Moebius scan.
static constexpr int kLineCtaWarps = 8;
template <bool SPACE>
__global__ void __launch_bounds__(32 * kLineCtaWarps) k_h_line_cta(
    const fh_h_dev_inst *__restrict__ inst, double *__restrict__ U, const double *__restrict__ wc,
    const double *__restrict__ part, long long ldpart, int splits, double *__restrict__ Al, double *__restrict__ Bt,
    double *__restrict__ sA, double *__restrict__ sB, double *__restrict__ sR, double *__restrict__ sOm,
    double *__restrict__ Dnew, int append, int os, int dfstore, const double *__restrict__ sV, int serial) {
  __shared__ fh_mob smm[kLineCtaWarps];
  __shared__ fh_aff sma[kLineCtaWarps];
  h_line<kLineCtaWarps, SPACE, kLineAll>(inst[blockIdx.x], blockIdx.x, threadIdx.x, U, wc, part, ldpart, splits, Al,
                                         Bt, sA, sB, sR, sOm, Dnew, append, os, dfstore, sV, smm, sma, serial);
}

// ------------------------------------------- persistent solves of small batches
// Batches of few instances run all the steps of a call in one launch: one
// cluster of kPersCtas CTAs per instance.  Per step CTA r computes the
// weights of its share of the instance's history slots and their sum over the
// instance's nodes into its shared memory; after a cluster barrier CTA 0 adds
// the CTAs' partial sums in rank order (distributed shared memory), solves the
// line (h_line on eight warps, as k_h_line_cta) and appends the new layer; a
// second cluster barrier publishes the layer (and frees the partial sums) for
// the next step.  No kernel boundary and no grid-wide synchronisation: the
// instances are independent, and a cluster barrier is a hardware barrier that
// every CTA of the cluster reaches the same number of times.
constexpr int kPersCtas = 8;
constexpr int kPersThreads = 32 * kLineCtaWarps;
constexpr int kPersMaxNodes = 2048;  // nodes of an instance (N + 2) in the partial sums
constexpr int kPersMaxInst = 32;     // larger batches step kernel by kernel
constexpr int kPersMaxChunk = 3800;  // history slots of one CTA (weights in shared memory, < 48 KiB in all)

// Phase stamps of the persistent solve for profiling builds (-DFH_H_STAMPS):
// %clock64 at the phase boundaries of the first 1024 steps of CTA 0 of
// instance 0, read with fh_h_stamps_read.  Empty otherwise.
#ifdef FH_H_STAMPS
__device__ long long g_h_stamps[1024 * 8];
#define H_STAMP(p)                                                              \
  if (b == 0 && r == 0 && threadIdx.x == 0 && s < 1024) g_h_stamps[s * 8 + (p)] = clock64();
extern "C" int fh_h_stamps_read(long long *h) {
  return (int)cudaMemcpyFromSymbol(h, g_h_stamps, sizeof(g_h_stamps));
}
#else
#define H_STAMP(p)
#endif

__global__ void __cluster_dims__(kPersCtas, 1, 1) __launch_bounds__(kPersThreads)
    k_h_persistent(const fh_h_dev_inst *__restrict__ inst, int tstep0, int os0, int nsteps, double *D,
                   long long ldd, int ldw, double *wc, const double *__restrict__ Lb,
                   const double *__restrict__ ibt, const double2 *__restrict__ lgt, double *U, double *part,
                   double *Al, double *Bt, double *sA, double *sB, double *sR, double *sOm, int serial) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double wsh[];  // this CTA's weights of the step (kPersMaxChunk at most)
  __shared__ double psum[kPersMaxNodes];
  __shared__ fh_mob smm[kLineCtaWarps];
  __shared__ fh_aff sma[kLineCtaWarps];
  const int b = blockIdx.x / kPersCtas;
  const int r = (int)cl.block_rank();
  const fh_h_dev_inst I = inst[b];
  const int np = I.N + 2;
  for (int s = 0; s < nsteps; ++s) {
    const int os_g = os0 + s;
    const int tstep = tstep0 + s - I.tb, os = os_g - I.ob;
    const int K = os >= 2 ? os - 1 : 0;  // history slots
    const double invX = 1.0 / (double)(tstep + 1);
    const int kch = (K + kPersCtas - 1) / kPersCtas;
    const int k0 = min(K, r * kch), k1 = min(K, k0 + kch), nk = k1 - k0;
    H_STAMP(0);
    for (int k = (int)threadIdx.x; k < nk; k += blockDim.x)
      wsh[k] = h_slot_weight(I, b, k0 + k, false, tstep, os, invX, ldw, Lb, ibt, lgt);
    if (r == 0 && threadIdx.x == 0)
      wc[b] = h_slot_weight(I, b, os > 1 ? os - 1 : 0, true, tstep, os, invX, ldw, Lb, ibt, lgt);
    __syncthreads();
    H_STAMP(1);
    // slots of the instance's occupant start at global slot I.ob; eight
    // independent loads ahead of the multiply-adds
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
      double acc = 0.0;
      const double *d = D + (long long)(I.ob + k0) * ldd + I.off + p;
      int k = 0;
      for (; k + 8 <= nk; k += 8, d += 8 * ldd) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = __ldcg(d + u * ldd);
#pragma unroll
        for (int u = 0; u < 8; ++u) acc = fma(wsh[k + u], v[u], acc);
      }
      for (; k < nk; ++k, d += ldd) acc = fma(wsh[k], __ldcg(d), acc);
      psum[p] = acc;
    }
    H_STAMP(2);
    cl.sync();
    H_STAMP(3);
    if (r == 0) {
      for (int p = threadIdx.x; p < np; p += blockDim.x) {
        double t = 0.0;
        for (int q = 0; q < kPersCtas; ++q) t += cl.map_shared_rank(psum, q)[p];
        part[I.off + p] = t;
      }
      __syncthreads();
      H_STAMP(4);
      const int append = os_g >= 1;
      double *Dnew = append ? D + (long long)(os_g - 1) * ldd : nullptr;
      h_line<kLineCtaWarps, false, kLineAll>(I, b, threadIdx.x, U, wc, part, 0, 1, Al, Bt, sA, sB, sR, sOm, Dnew,
                                             append, os_g, 0, nullptr, smm, sma, serial);
      H_STAMP(5);
    }
    cl.sync();
    H_STAMP(6);
  }
}

// ---------------------------------------------------- blocked history mode
// psi = t^beta node value F(x) = B(y(x); 1/beta, 1-alpha) at X (lower series
// r P(y), flag low = 1) or its upper tail U(c) = c^b Q(c) (low = 0), from the
// per-instance tables and the log table: one exp or expm1 + log + exp and one
// Horner polynomial per node.  A slot weight is the difference of its two
// nodes; the difference loses ~log10(X) digits, which is far below the 2^-32
// of the bf16 slices the blocked contraction uses these weights at.
// h_psi_node_at: the same at a real X (0 < x < X) given log x and log X as
// double-doubles and r = x/X.
__device__ __forceinline__ void h_psi_node_at(const fh_h_dev_inst &I, const double *__restrict__ Lc, double2 lx,
                                              double2 lX, double r, double &v, int &low) {
  const double *Uc = Lc + kIbTerms;
  const double sh = lx.x - lX.x;
  const double sl = (lx.x - (sh + lX.x)) + (lx.y - lX.y);
  const double th = I.beta * sh;
  const double tl = fma(I.beta, sh, -th) + I.beta * sl;
  if (r <= Lc[2 * kIbTerms + 1]) {  // y <= kIbLowMax: lower series in y
    const double ey = exp(th);
    const double y = fma(ey, tl, ey);
    v = r * fh_series(fh_ib_coef_tab{Lc}, fh_ib_nterms(y), y);
    low = 1;
  } else {  // upper tail in c = 1 - y
    const double em = expm1(th);
    const double c = -fma(em + 1.0, tl, em);
    v = c <= 0.0 ? 0.0 : exp((1.0 - I.alpha) * log(c)) * fh_series(fh_ib_coef_tab{Uc}, fh_ib_nterms(c), c);
    low = 0;
  }
}

__device__ __forceinline__ void h_psi_node(const fh_h_dev_inst &I, const double *__restrict__ Lc,
                                           const double2 *__restrict__ lgt, int x, int X, double invX, double &v,
                                           int &low) {
  if (x <= 0) {
    v = 0.0;
    low = 1;
    return;
  }
  if (x >= X) {  // c = 0
    v = 0.0;
    low = 0;
    return;
  }
  h_psi_node_at(I, Lc, lgt[x], lgt[X], (double)x * invX, v, low);
}

// Far slots by interpolation across the block's steps.  For a fixed slot
// [t, t + 1] the weight w(X) over the block's X in [K + 3, K + 66] is
// analytic off the branch points X = t, t + 1, so within the Bernstein
// ellipse of the interval with parameter rho = D + sqrt(D^2 - 1),
// D = 1 + 2 d / 63, d = K + 2 - t the distance of the nearer branch point:
// the interpolant at m first-kind Chebyshev points is within ~rho^-m of w
// (Trefethen, Approximation Theory and Approximation Practice, ch. 8).  A
// chunk group takes the order of its last slot for kHbChebBits bits (2^-38,
// far below the 2^-31 of the group's bf16 slices); groups that would need
// more than kHbChebMax points are evaluated exactly per step.
constexpr int kHbChebMax = 16;
constexpr double kHbChebBits = 38.0;
constexpr int kHbGroupSlots = 2 * kSlcK;  // slots of a chunk group
__host__ __device__ inline int hb_cheb_order(int d) {
  const double D = 1.0 + 2.0 * (double)d / 63.0;
  const double rho = D + sqrt(D * D - 1.0);
  return (int)ceil(kHbChebBits * 0.6931471805599453 / log(rho)) + 1;
}
// The same in the slot direction: the group's slot starts t in
// [t0, t0 + 127] (half length 63.5) with the nearer of the branch points
// t = 0 (at t0) and t = X - 1 (beyond the group's last slot by at least d).
__host__ __device__ inline int hb_cheb_order_t(int dt) {
  const double D = 1.0 + (double)dt / 63.5;
  const double rho = D + sqrt(D * D - 1.0);
  return (int)ceil(kHbChebBits * 0.6931471805599453 / log(rho)) + 1;
}
// Leading chunk groups of the block at K that are interpolated.
static int hb_cheb_groups(int K) {
  const int ng = fh_ngroups(K / kSlcK);
  int g = 0;
  while (g < ng - 1 && hb_cheb_order(K + 2 - (g * kHbGroupSlots + kHbGroupSlots - 1)) <= kHbChebMax) ++g;
  return g;
}
// Interpolation tables for m = 1..kHbChebMax points: block m holds the
// Lagrange basis L[r][j] at the block's steps r < 64 (x_r = -1 + 2 r / 63;
// row stride kHbChebMax) and, in row 64, the X offsets 31.5 (1 + x_j) of the
// points x_j = cos((2 j + 1) pi / (2 m)) from K + 3.
static constexpr size_t kHbChebBlock = (size_t)(kSlcK + 1) * kHbChebMax;
// Slot-direction tables after them: block m holds L[k][i] at the group's 128
// slots (x_k = -1 + 2 k / 127) and, in row 128, the slot offsets
// 63.5 (1 + x_i) from the group's first slot.
static constexpr size_t kHbChebTBlock = (size_t)(kHbGroupSlots + 1) * kHbChebMax;
static constexpr size_t kHbChebTBase = (kHbChebMax + 1) * kHbChebBlock;
static void hb_cheb_table(std::vector<double> &t) {
  t.assign(kHbChebTBase + (kHbChebMax + 1) * kHbChebTBlock, 0.0);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int m = 1; m <= kHbChebMax; ++m) {
    double *T = t.data() + (size_t)m * kHbChebBlock;
    long double xj[kHbChebMax];
    for (int j = 0; j < m; ++j) {
      xj[j] = cosl((long double)(2 * j + 1) * pi / (long double)(2 * m));
      T[kSlcK * kHbChebMax + j] = (double)(31.5L * (1.0L + xj[j]));
    }
    for (int r = 0; r < kSlcK; ++r) {
      const long double x = -1.0L + 2.0L * (long double)r / 63.0L;
      for (int j = 0; j < m; ++j) {
        long double l = 1.0L;
        for (int i = 0; i < m; ++i)
          if (i != j) l *= (x - xj[i]) / (xj[j] - xj[i]);
        T[r * kHbChebMax + j] = (double)l;
      }
    }
    double *Tt = t.data() + kHbChebTBase + (size_t)m * kHbChebTBlock;
    for (int j = 0; j < m; ++j) Tt[kHbGroupSlots * kHbChebMax + j] = (double)(63.5L * (1.0L + xj[j]));
    for (int k = 0; k < kHbGroupSlots; ++k) {
      const long double x = -1.0L + 2.0L * (long double)k / 127.0L;
      for (int j = 0; j < m; ++j) {
        long double l = 1.0L;
        for (int i = 0; i < m; ++i)
          if (i != j) l *= (x - xj[i]) / (xj[j] - xj[i]);
        Tt[k * kHbChebMax + j] = (double)l;
      }
    }
  }
}

// Weight planes of the interpolated chunk groups G < gridDim.x of the psi
// instances (one CTA per (group, instance)): the group's 129 node values at
// each of the m points X_j (h_psi_node_at; psi = t: (1 - x/X)^(1 - alpha)),
// the 128 slot weights at each X_j, then per step r of the block the
// interpolated weights sum_j L[r][j] w_j, sliced into W3/Ew as k_hb_weights
// does.  Rows past the last step are zero.
__global__ void __launch_bounds__(256) k_hb_wcheb(const fh_h_dev_inst *__restrict__ inst, int K, int max_steps,
                                                  const double *__restrict__ ibt, const double2 *__restrict__ lgt,
                                                  const double *__restrict__ cheb, long long R, int Kcap,
                                                  __nv_bfloat16 *__restrict__ W3, int8_t *__restrict__ Ew) {
  __shared__ double sv[kHbChebMax][kHbGroupSlots + 1];
  __shared__ double sw[kHbChebMax][kHbGroupSlots];
  __shared__ double sL[kSlcK * kHbChebMax];
  __shared__ double sX[kHbChebMax][3];  // log X_j, 1/X_j, scale of X_j
  __shared__ double sn[kHbChebMax][kHbChebMax];  // 2D path: weights at the (slot, step) points
  __shared__ unsigned char slo[kHbChebMax][kHbGroupSlots + 1];
  const int b = blockIdx.y, G = blockIdx.x;
  const fh_h_dev_inst I = inst[b];
  if (I.weights != FH_W_PSI) return;  // whole CTA
  const int x0 = G * kHbGroupSlots;
  const int m = min(hb_cheb_order(K + 2 - (x0 + kHbGroupSlots - 1)), kHbChebMax);
  const double *tab = cheb + (size_t)m * kHbChebBlock;
  for (int i = threadIdx.x; i < kSlcK * kHbChebMax; i += blockDim.x) sL[i] = tab[i];
  const double *Lc = ibt + (long long)b * kIbStride;
  const bool psi_t = I.beta == 1.0;
  if (threadIdx.x < m) {
    const int j = threadIdx.x;
    const double X = (double)(K + 3) + tab[kSlcK * kHbChebMax + j];
    const double lX = log(X);
    sX[j][0] = lX;
    sX[j][1] = 1.0 / X;
    // (X tau)^(1 - alpha beta) (1 - alpha) / beta; psi = t: (X tau)^(1 - alpha)
    sX[j][2] = psi_t ? exp((1.0 - I.alpha) * (lX + Lc[2 * kIbTerms + 2]))
                     : exp((1.0 - I.alpha * I.beta) * (lX + Lc[2 * kIbTerms + 2])) * Lc[2 * kIbTerms + 3] *
                           (1.0 - I.alpha);
  }
  __syncthreads();
  // Groups after the first (slot starts t >= 128, away from the branch point
  // t = 0) are interpolated in the slot direction too: the weights at
  // mt x m points (t_i, X_j) of the interval [t_i, t_i + 1] (the
  // divided-difference form at real t), then the group's 128 slots at each
  // X_j from those
  const int mt = G >= 1 ? hb_cheb_order_t(min(K + 2 - (x0 + kHbGroupSlots - 1), x0)) : kHbChebMax + 1;
  if (mt <= kHbChebMax) {
    const double *tabt = cheb + kHbChebTBase + (size_t)mt * kHbChebTBlock;
    double *sLt = &sv[0][0];  // L[k][i], 128 x kHbChebMax (fits in sv)
    for (int i = threadIdx.x; i < kHbGroupSlots * kHbChebMax; i += blockDim.x) sLt[i] = tabt[i];
    const double *Uc = Lc + kIbTerms;
    for (int i = threadIdx.x; i < mt * m; i += blockDim.x) {
      const int ti = i / m, j = i - ti * m;
      const double t = (double)x0 + tabt[kHbGroupSlots * kHbChebMax + ti];
      const double X = (double)(K + 3) + tab[kSlcK * kHbChebMax + j];
      double w;
      if (psi_t) {
        w = fh_psi_int_t(t, t + 1.0, X, I.tau, I.alpha) * (1.0 - I.alpha);
      } else {
        auto lrat = [](double x, double Xv) { return 2.0 * x <= Xv ? log(x / Xv) : log1p((x - Xv) / Xv); };
        fh_ib_slot q;
        q.zero0 = false;
        q.top = false;
        q.r0 = t * sX[j][1];
        q.r1 = (t + 1.0) * sX[j][1];
        q.dr = sX[j][1];
        q.l1h = lrat(t + 1.0, X);
        q.l1l = 0.0;
        q.l0h = lrat(t, X);
        q.l0l = 0.0;
        q.ldh = log1p(1.0 / t);
        q.ldl = 0.0;
        const double diff = fh_ib_diff(q, I.beta, 1.0 - I.alpha, Lc[2 * kIbTerms + 1],
                                       [&] { return Lc[2 * kIbTerms]; }, fh_ib_coef_tab{Lc}, fh_ib_coef_tab{Uc});
        w = sX[j][2] * diff;
      }
      sn[ti][j] = w;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m * kHbGroupSlots; i += blockDim.x) {
      const int j = i / kHbGroupSlots, k = i - j * kHbGroupSlots;
      const double *Lk = sLt + k * kHbChebMax;
      double acc = 0.0;
      for (int ti = 0; ti < mt; ++ti) acc = fma(Lk[ti], sn[ti][j], acc);
      sw[j][k] = acc;
    }
    __syncthreads();
  } else {
  for (int i = threadIdx.x; i < m * (kHbGroupSlots + 1); i += blockDim.x) {
    const int j = i / (kHbGroupSlots + 1), k = i - j * (kHbGroupSlots + 1);
    const int x = x0 + k;  // x < K + 3 <= X_j
    double v;
    int lo;
    if (psi_t) {
      v = exp((1.0 - I.alpha) * log1p(-(double)x * sX[j][1]));
      lo = 0;
    } else if (x == 0) {
      v = 0.0;
      lo = 1;
    } else {
      h_psi_node_at(I, Lc, lgt[x], make_double2(sX[j][0], 0.0), (double)x * sX[j][1], v, lo);
    }
    sv[j][k] = v;
    slo[j][k] = (unsigned char)lo;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < m * kHbGroupSlots; i += blockDim.x) {
    const int j = i / kHbGroupSlots, k = i - j * kHbGroupSlots;
    const double v0 = sv[j][k], v1 = sv[j][k + 1];
    const int l0 = slo[j][k], l1 = slo[j][k + 1];
    double diff;
    if (l0 && l1)
      diff = v1 - v0;
    else if (!l0)
      diff = v0 - v1;
    else
      diff = (Lc[2 * kIbTerms] - v1) - v0;
    sw[j][k] = x0 + k >= 1 ? sX[j][2] * diff : 0.0;  // slot 0 weighs nothing
  }
  __syncthreads();
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunks = K / kSlcK;
  for (int r = warp; r < kSlcK; r += blockDim.x >> 5) {
    double w[4] = {0.0, 0.0, 0.0, 0.0};
    if (K + r + 2 <= max_steps) {
      const double *Lr = sL + r * kHbChebMax;
      for (int j = 0; j < m; ++j) {
        const double l = Lr[j];
#pragma unroll
        for (int h = 0; h < 4; ++h) w[h] = fma(l, sw[j][lane + 32 * h], w[h]);
      }
    }
    fh_slice_group_values(w, G, nchunks, (long long)b * kSlcK + r, R, Kcap, W3, Ew);
  }
}

// Weight planes of the block whose first step has K = 64 blk history slots:
// row m = 64 inst + r is step tstep = K + r + 2 (X = K + r + 3) of instance
// inst, weighing the slots t < K (slot 0: weight 0, as in k_h_weights); rows
// past the last step are zero.  One warp per (row, chunk group G >= G0), sliced
// into W3/Ew (fh_slices.cuh); the groups below gcheb of the psi instances are
// k_hb_wcheb's.
__global__ void k_hb_weights(const fh_h_dev_inst *__restrict__ inst, int K, int max_steps, int G0, int gcheb,
                             const double *__restrict__ Lb, int ldw, const double *__restrict__ ibt,
                             const double2 *__restrict__ lgt, long long R, int Kcap, __nv_bfloat16 *__restrict__ W3,
                             int8_t *__restrict__ Ew) {
  const long long m = (long long)blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (m >= R) return;  // whole warp
  const int lane = threadIdx.x & 31;
  const int b = (int)(m / kSlcK), r = (int)(m % kSlcK);
  const fh_h_dev_inst I = inst[b];
  const int G = G0 + blockIdx.x, nchunks = K / kSlcK;
  if (I.weights == FH_W_PSI && G < gcheb) return;  // interpolated (k_hb_wcheb); whole warp
  const int tstep = K + r + 2, X = tstep + 1, os = K + r + 1;
  const bool live = tstep <= max_steps;
  double w[4];
  const int k0 = 2 * G * kSlcK + lane;
  if (I.weights == FH_W_L1) {
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int k = k0 + 32 * h;
      w[h] = (live && k >= 1 && k < K) ? Lb[(long long)b * ldw + (os - k - 1)] : 0.0;
    }
  } else if (I.beta == 1.0) {
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int k = k0 + 32 * h;
      w[h] = (live && k >= 1 && k < K)
                 ? fh_psi_int_t((double)k, (double)k + 1.0, (double)X, I.tau, I.alpha) * (1 - I.alpha)
                 : 0.0;
    }
  } else {
    const double *Lc = ibt + (long long)b * kIbStride;
    const double invX = 1.0 / (double)X;
    double v[5];
    int lo[5];
    // nodes k0 + 32 h (h < 4) and, for lane 31, the upper node 128 G + 128 of
    // the group's last slot
#pragma unroll
    for (int h = 0; h < 5; ++h) {
      v[h] = 0.0;
      lo[h] = 1;
      if (live && (h < 4 || lane == 31))
        h_psi_node(I, Lc, lgt, h < 4 ? k0 + 32 * h : 2 * G * kSlcK + 128, X, invX, v[h], lo[h]);
    }
    const double sc = live ? exp((1.0 - I.alpha * I.beta) * (lgt[X].x + Lc[2 * kIbTerms + 2])) *
                                 Lc[2 * kIbTerms + 3] * (1 - I.alpha)
                           : 0.0;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      // upper node of slot k = k0 + 32 h: node k + 1 (the next lane, or lane 0 of the next h)
      double v1 = __shfl_down_sync(0xffffffffu, v[h], 1);
      int l1 = __shfl_down_sync(0xffffffffu, lo[h], 1);
      const double vn = __shfl_sync(0xffffffffu, v[h + 1], 0);
      const int ln = __shfl_sync(0xffffffffu, lo[h + 1], 0);
      if (lane == 31) {
        v1 = h < 3 ? vn : v[4];
        l1 = h < 3 ? ln : lo[4];
      }
      const int k = k0 + 32 * h;
      double diff;
      if (lo[h] && l1)
        diff = v1 - v[h];
      else if (!lo[h])
        diff = v[h] - v1;
      else
        diff = (Lc[2 * kIbTerms] - v1) - v[h];
      w[h] = (live && k >= 1 && k < K) ? sc * diff : 0.0;
    }
  }
  fh_slice_group_values(w, G, nchunks, m, R, Kcap, W3, Ew);
}

// History sum of the blocked mode at one step: part[p] = far[p] + sum over
// the near slots t in [t_lo, K) of W[inst][t] * ring[t mod 128][p], in
// double-float (the far row holds the contraction of the older slots; null
// before the first block has one), two points per thread over the
// per-instance tiles; written as FP64 for the line kernels.
__global__ void __launch_bounds__(kTileThreads) k_h_near_df(const fh_h_tile *__restrict__ tiles,
                                                            const fh_h_dev_inst *__restrict__ inst,
                                                            const float2 *__restrict__ ring, long long ldr, int t_lo,
                                                            int K, const double *__restrict__ W, int ldw,
                                                            const float2 *__restrict__ far,
                                                            double *__restrict__ part) {
  __shared__ float2 wsf2[kSlcK];
  const fh_h_tile T = tiles[blockIdx.x];
  const int nk = K - t_lo;  // < 64
  const double *wrow = W + (long long)T.inst * ldw + t_lo;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) wsf2[i] = fh_df_pair(fh_df_from_double(wrow[i]));
  __syncthreads();
  const int q = threadIdx.x * 2;
  if (q >= T.len) return;
  const long long p = inst[T.inst].off + T.start + q;
  fh_df a0{0.f, 0.f}, a1{0.f, 0.f};
  if (far) {
    const float4 f = *reinterpret_cast<const float4 *>(far + p);
    a0 = fh_df{f.x, f.y};
    a1 = fh_df{f.z, f.w};
  }
  for (int k = 0; k < nk; ++k) {
    const int t = t_lo + k;
    const float4 v = __ldcs(reinterpret_cast<const float4 *>(ring + (long long)(t & 127) * ldr + p));
    const fh_df w = fh_df_from_pair(wsf2[k]);
    a0 = fh_df_fma(w, fh_df{v.x, v.y}, a0);
    a1 = fh_df_fma(w, fh_df{v.z, v.w}, a1);
  }
  double2 o;
  o.x = fh_df_to_double(a0);
  o.y = fh_df_to_double(a1);
  *reinterpret_cast<double2 *>(part + p) = o;
}

// ------------------------------------------------------------------- host

// K splits of the batch history sum: enough CTAs for ~3 waves of 8 resident
// CTAs on 152 SMs, at least 32 layers per split, at most `cap` splits.
// Chunks of at most kHistMaxChunk layers in any case: the chunk's weights sit
// in shared memory, and larger chunks cost resident CTAs (4096 instances at
// K = 5000 without splits: 40 KB per CTA, 5 CTAs per SM, 71 % of HBM).
static constexpr int kHistMaxChunk = 512;
static constexpr int kHistMaxSplits = 64;  // partial-sum buffers of a batch
static void h_plan(size_t ntiles, int K, int cap, int *splits, int *kchunk) {
  const long long target = 3LL * 152 * 8;
  int s = (int)fh_ceil_div(target, (long long)(ntiles > 0 ? ntiles : 1));
  if (s > cap) s = cap;
  if (s > K / 32) s = K / 32;
  const int smin = (int)fh_ceil_div(K, kHistMaxChunk);
  if (s < smin) s = smin < kHistMaxSplits ? smin : kHistMaxSplits;
  if (s < 1) s = 1;
  int kc = (int)fh_ceil_div(K, s);
  kc = (int)fh_ceil_div(kc, 4) * 4;
  *splits = (int)fh_ceil_div(K, kc);
  *kchunk = kc;
}

// History sum over K layers with the weights W into part (tile shape ti).
static int h_hist(fh_h_batch *B, int ti, int K, int splits, int kchunk, const double *W, cudaStream_t st) {
  fh_ctx *ctx = B->ctx;
  const dim3 g((unsigned)B->tiles_by[ti].size(), (unsigned)splits);
  const size_t smem = sizeof(double) * (size_t)kchunk;
  FH_REQUIRE(ctx, smem <= 48 * 1024, FH_EINVAL, "history chunk too large");
  if (B->mode == FH_H_DF64)
    k_hist_tiles_df<<<g, kTileShapes[ti], smem, st>>>(  // float2 weights: same bytes as FP64
        B->tl_by[ti].as<fh_h_tile>(), B->inst.as<fh_h_dev_inst>(), reinterpret_cast<const float2 *>(B->D.as<double>()),
        B->Ptot, K, W, B->max_weights, kchunk, B->part.as<double>(), B->Ptot);
  else
    k_hist_tiles<<<g, kTileShapes[ti], smem, st>>>(B->tl_by[ti].as<fh_h_tile>(), B->inst.as<fh_h_dev_inst>(),
                                                   B->D.as<double>(), B->Ptot, K, W, B->max_weights, kchunk,
                                                   B->part.as<double>(), B->Ptot);
  return fh_after_launch(ctx, "k_hist_tiles");
}

// Weights of step `tstep` (os saved layers) into the buffer pair `par`: the
// history slots from t_lo on and the current weight.
static int h_weights(fh_h_batch *B, int tstep, int os, int par, cudaStream_t st, int t_lo = 0) {
  fh_ctx *ctx = B->ctx;
  FH_REQUIRE(ctx, tstep + 1 < B->max_steps + 2, FH_EINVAL, "h_weights: step %d beyond the log table", tstep);
  const int nh = os > 1 ? os - 1 : 0;
  if (t_lo > nh) t_lo = nh;
  dim3 gw((unsigned)((nh - t_lo) / kHWeightThreads + 1), (unsigned)B->n);  // slots t_lo .. nh
  fh_prof_mark(ctx, FH_PROF_WEIGHTS, false, st);
  k_h_weights<<<gw, kHWeightThreads, 0, st>>>(B->inst.as<fh_h_dev_inst>(), B->n, tstep, os, t_lo, B->Wp(par),
                                              B->max_weights, B->wcp(par), B->Lb.as<double>(), B->ibt.as<double>(),
                                              B->lgt.as<double2>(), 1.0 / (double)(tstep + 1));
  fh_prof_mark(ctx, FH_PROF_WEIGHTS, true, st);
  return fh_after_launch(ctx, "k_h_weights");
}

// One step.  The weights depend on the step number only, so with `next` (and
// a small batch) the weights of the following step are computed on the side
// stream hs (high priority) beside this step's history sum and line solves,
// into the other buffer pair; the following call waits for them.
static int h_one_step(fh_h_batch *B, bool next) {
  fh_ctx *ctx = B->ctx;
  const int os = B->nsaved;
  const int K = os >= 2 ? os - 1 : 0;
  const int par = B->tstep & 1;
  const bool blk = B->mode == FH_H_BLOCKED;
  // blocked mode: slots below t_lo (whole 64-slot chunks) are in the far rows
  auto near_lo = [&](int k) { return blk ? (k / kSlcK) * kSlcK : 0; };
  const int t_lo = near_lo(K);
  int rc;
  if (B->w_ready == B->tstep) {
    FH_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, B->ev_w, 0));
  } else if ((rc = h_weights(B, B->tstep, os, par, ctx->stream, t_lo))) {
    return rc;
  }
  B->w_ready = -1;
  // only for small batches: in large ones the FP64-bound weights take SM
  // slots from the HBM-bound history sum (measured: 4096 instances, 5000
  // steps, the history sum fell from 92 % to 58 % of HBM beside them)
  if (next && B->hs && B->n < kLineCtaMaxInst) {
    FH_CUDA_TRY(ctx, cudaEventRecord(B->ev_main, ctx->stream));
    FH_CUDA_TRY(ctx, cudaStreamWaitEvent(B->hs, B->ev_main, 0));
    if ((rc = h_weights(B, B->tstep + 1, os + 1, par ^ 1, B->hs, near_lo(os + 1 >= 2 ? os : 0)))) return rc;
    FH_CUDA_TRY(ctx, cudaEventRecord(B->ev_w, B->hs));
    B->w_ready = B->tstep + 1;
  }
  int splits = 0, kchunk = 0;
  if (blk) {
    float2 *ring = B->ring.as<float2>(), *far = B->far.as<float2>();
    if (K >= kSlcK && K == t_lo) {
      // first step of a block: the chunk just completed into the planes, the
      // weight planes of the block's 64 steps, and their far rows
      fh_prof_mark(ctx, FH_PROF_HISTORY, false);
      rc = fh_hblk_convert(ctx, *B->hb, ring, B->Ptot, K / kSlcK - 1);
      fh_prof_mark(ctx, FH_PROF_HISTORY, true);
      if (rc) return rc;
      fh_prof_mark(ctx, FH_PROF_WEIGHTS, false);
      const long long R = (long long)B->n * kSlcK;
      const int ng = fh_ngroups(K / kSlcK), gcheb = hb_cheb_groups(K), G0 = B->has_l1 ? 0 : gcheb;
      if (gcheb > 0) {
        k_hb_wcheb<<<dim3((unsigned)gcheb, (unsigned)B->n), 256, 0, ctx->stream>>>(
            B->inst.as<fh_h_dev_inst>(), K, B->max_steps, B->ibt.as<double>(), B->lgt.as<double2>(),
            B->cheb.as<double>(), R, fh_hblk_kcap(*B->hb), fh_hblk_wplanes(*B->hb), fh_hblk_wexp(*B->hb));
        if ((rc = fh_after_launch(ctx, "k_hb_wcheb"))) return rc;
      }
      k_hb_weights<<<dim3((unsigned)(ng - G0), (unsigned)fh_ceil_div(R, 8)), 256, 0, ctx->stream>>>(
          B->inst.as<fh_h_dev_inst>(), K, B->max_steps, G0, gcheb, B->Lb.as<double>(), B->max_weights,
          B->ibt.as<double>(), B->lgt.as<double2>(), R, fh_hblk_kcap(*B->hb), fh_hblk_wplanes(*B->hb),
          fh_hblk_wexp(*B->hb));
      fh_prof_mark(ctx, FH_PROF_WEIGHTS, true);
      if ((rc = fh_after_launch(ctx, "k_hb_weights"))) return rc;
      if ((rc = fh_hblk_gemm(ctx, *B->hb, K, far, B->Ptot))) return rc;
    }
    const int ti = tile_shape_index(B->tile_threads);
    fh_prof_mark(ctx, FH_PROF_HISTORY, false);
    k_h_near_df<<<(unsigned)B->tiles_by[ti].size(), kTileShapes[ti], 0, ctx->stream>>>(
        B->tl_by[ti].as<fh_h_tile>(), B->inst.as<fh_h_dev_inst>(), ring, B->Ptot, t_lo, K, B->Wp(par),
        B->max_weights, t_lo >= kSlcK ? far + (long long)(K - t_lo) * B->Ptot : nullptr, B->part.as<double>());
    fh_prof_mark(ctx, FH_PROF_HISTORY, true);
    if ((rc = fh_after_launch(ctx, "k_h_near_df"))) return rc;
    splits = 1;
  } else if (K > 0) {
    const int ti = tile_shape_index(B->tile_threads);
    h_plan(B->tiles_by[ti].size(), K, B->split_cap, &splits, &kchunk);
    fh_prof_mark(ctx, FH_PROF_HISTORY, false);
    rc = h_hist(B, ti, K, splits, kchunk, B->Wp(par), ctx->stream);
    fh_prof_mark(ctx, FH_PROF_HISTORY, true);
    if (rc) return rc;
    // fold the partial sums into split 0 (in split order) for the warp-per-
    // instance lines; the CTA-per-instance lines of small batches read all
    // splits themselves (one launch less per step)
    if (splits > 2 && B->n >= kLineCtaMaxInst) {
      if ((rc = fh_launch_reduce_splits(ctx, splits, B->Ptot, B->part.as<double>(), B->Ptot, B->part.as<double>())))
        return rc;
      splits = 1;
    }
  }
  fh_prof_mark(ctx, FH_PROF_SWEEP, false);  // right parts (incl. the space-fractional sums) and line solves
  if (B->space) {
    k_h_space_v<<<(unsigned)B->n, 256, B->space_smem, ctx->stream>>>(B->inst.as<fh_h_dev_inst>(), B->U.as<double>(),
                                                                   B->wsp.as<double>(), B->sV.as<double>());
    if ((rc = fh_after_launch(ctx, "k_h_space_v"))) return rc;
  }
  const int append = os >= 1;
  double *Dnew = !append ? nullptr
                 : blk   ? reinterpret_cast<double *>(B->ring.as<float2>() + (long long)((os - 1) & 127) * B->Ptot)
                         : B->D.as<double>() + (long long)(os - 1) * B->Ptot;
  {
    const int fst = os, dfs = (B->mode == FH_H_DF64 || blk) ? 1 : 0;  // first step per instance: os == its base
    const dim3 gc((unsigned)B->n), gw((unsigned)fh_ceil_div(B->n, 4));
    const fh_h_dev_inst *in = B->inst.as<fh_h_dev_inst>();
    double *Al = B->Al.as<double>(), *Bt = B->Bt.as<double>(), *sA = B->sA.as<double>(), *sB = B->sB.as<double>();
    double *sR = B->sR.as<double>(), *sOm = B->sOm.as<double>(), *U = B->U.as<double>();
    const double *part = B->part.as<double>(), *wcp = B->wcp(par), *sV = B->sV.as<double>();
    const int serial = B->serial_al ? 1 : 0;
    if (B->n < kLineCtaMaxInst) {
      if (B->space)
        k_h_line_cta<true><<<gc, 32 * kLineCtaWarps, 0, ctx->stream>>>(in, U, wcp, part, B->Ptot, splits, Al, Bt, sA, sB,
                                                                      sR, sOm, Dnew, append, fst, dfs, sV, serial);
      else
        k_h_line_cta<false><<<gc, 32 * kLineCtaWarps, 0, ctx->stream>>>(in, U, wcp, part, B->Ptot, splits, Al, Bt, sA,
                                                                       sB, sR, sOm, Dnew, append, fst, dfs, sV, serial);
    } else if (!serial || !B->varcoef) {
      if (B->space)
        k_h_line_warp<true, kLineAll><<<gw, 128, 0, ctx->stream>>>(in, B->n, U, wcp, part, B->Ptot, splits, Al, Bt, sA,
                                                                   sB, sR, sOm, Dnew, append, fst, dfs, sV);
      else
        k_h_line_warp<false, kLineAll><<<gw, 128, 0, ctx->stream>>>(in, B->n, U, wcp, part, B->Ptot, splits, Al, Bt,
                                                                    sA, sB, sR, sOm, Dnew, append, fst, dfs, sV);
    } else {
      // coefficients, serial Al one lane per instance, sweeps
      if (B->space)
        k_h_line_warp<true, kLineCoef><<<gw, 128, 0, ctx->stream>>>(in, B->n, U, wcp, part, B->Ptot, splits, Al, Bt,
                                                                    sA, sB, sR, sOm, Dnew, append, fst, dfs, sV);
      else
        k_h_line_warp<false, kLineCoef><<<gw, 128, 0, ctx->stream>>>(in, B->n, U, wcp, part, B->Ptot, splits, Al, Bt,
                                                                     sA, sB, sR, sOm, Dnew, append, fst, dfs, sV);
      if ((rc = fh_after_launch(ctx, "k_h_line_warp"))) return rc;
      k_h_alpha_lanes<<<(unsigned)fh_ceil_div(B->n, 32), 32, 0, ctx->stream>>>(in, B->n, sA, sB, sR, Al);
      if ((rc = fh_after_launch(ctx, "k_h_alpha_lanes"))) return rc;
      if (B->space)
        k_h_line_warp<true, kLineSolve><<<gw, 128, 0, ctx->stream>>>(in, B->n, U, wcp, part, B->Ptot, splits, Al, Bt,
                                                                     sA, sB, sR, sOm, Dnew, append, fst, dfs, sV);
      else
        k_h_line_warp<false, kLineSolve><<<gw, 128, 0, ctx->stream>>>(in, B->n, U, wcp, part, B->Ptot, splits, Al,
                                                                      Bt, sA, sB, sR, sOm, Dnew, append, fst, dfs, sV);
    }
  }
  fh_prof_mark(ctx, FH_PROF_SWEEP, true);
  if ((rc = fh_after_launch(ctx, "k_h_line_warp"))) return rc;
  B->nsaved++;
  B->tstep++;
  return FH_OK;
}

// A new solve of the whole batch: every instance on the batch's clock again.
static int h_reset_clocks(fh_h_batch *b) {
  bool any = false;
  for (auto &I : b->di)
    if (I.tb || I.ob) {
      I.tb = I.ob = 0;
      any = true;
    }
  if (!any) return FH_OK;
  FH_CUDA_TRY(b->ctx, cudaMemcpyAsync(b->inst.p, b->di.data(), sizeof(fh_h_dev_inst) * b->n, cudaMemcpyHostToDevice,
                                      b->ctx->stream));
  FH_CUDA_TRY(b->ctx, cudaStreamSynchronize(b->ctx->stream));
  b->w_ready = -1;
  b->graph.reset();
  return FH_OK;
}

static bool h_params_ok(const fh_h_params &p) {
  return p.N >= 2 && p.N <= (1 << 20) && p.L > 0 && p.tau > 0 && p.alpha > 0 && p.alpha < 1 &&
         (p.weights == FH_W_L1 || p.weights == FH_W_PSI) && (p.kmodel == FH_K_CONST || p.kmodel == FH_K_EXP) &&
         (p.weights == FH_W_L1 || p.beta > 0);
}

// Device record of one instance (segment at `off`, own clock at zero).
static void h_fill_inst(const fh_h_params &p, long long off, fh_h_dev_inst &I) {
  I.N = p.N;
  I.weights = p.weights;
  I.kmodel = p.kmodel;
  I.gravity = p.gravity;
  I.fixed = (p.kmodel == FH_K_CONST) && (p.weights == FH_W_L1 || p.beta == 1.0);
  I.tb = 0;
  I.ob = 0;
  I.off = off;
  I.dL = p.L / p.N;
  I.Dg = pow(I.dL, -2.0);
  I.Da = p.weights == FH_W_L1 ? pow(p.tau, -p.alpha) / tgamma(2.0 - p.alpha) : pow(p.tau, -1.0) / tgamma(2.0 - p.alpha);
  I.tau = p.tau;
  I.alpha = p.alpha;
  I.beta = p.beta;
  I.kc = p.kc;
  I.kgam = p.kgam;
  I.cinv = p.cinv;
  I.al_left = p.al_left;
  I.bt_left = p.bt_left;
  I.u_right = p.u_right;
  I.spg = 1.0;
  I.spA = 0.0;
  I.kbf = 1.0;
}

extern "C" {

int fh_h_batch_create(fh_ctx *ctx, int ninst, const fh_h_params *params_host, int max_steps, fh_h_batch **out) {
  FH_REQUIRE(ctx, ctx && params_host && out, FH_EINVAL, "fh_h_batch_create: null argument");
  *out = nullptr;
  FH_REQUIRE(ctx, ninst >= 1 && max_steps >= 1, FH_EINVAL, "fh_h_batch_create: need ninst >= 1, max_steps >= 1");
  fh_h_batch *B = new fh_h_batch();
  B->ctx = ctx;
  B->n = ninst;
  B->max_steps = max_steps;
  B->max_weights = max_steps + 1;
  B->hp.assign(params_host, params_host + ninst);
  std::vector<fh_h_dev_inst> di(ninst);
  long long off = 0;
  for (int b = 0; b < ninst; ++b) {
    const fh_h_params &p = params_host[b];
    if (!h_params_ok(p)) {
      delete B;
      return fh_set_error(ctx, FH_EINVAL, "fh_h_batch_create: bad parameters for instance %d", b);
    }
    fh_h_dev_inst &I = di[b];
    h_fill_inst(p, off, I);
    if (!I.fixed) B->varcoef = true;
    if (I.weights == FH_W_L1) B->has_l1 = true;
    B->off.push_back(off);
    const int seg = ((p.N + 2) + 1) & ~1;
    B->cap.push_back(seg - 2);
    for (int k = 0; k < 3; ++k) {
      const int tn = 2 * kTileShapes[k];
      for (int st = 0; st < seg; st += tn) B->tiles_by[k].push_back({b, st, seg - st < tn ? seg - st : tn});
    }
    off += seg;
  }
  B->Ptot = off;
  int rc;
  const size_t st = sizeof(double) * (size_t)B->Ptot;
  if ((rc = fh_alloc(ctx, B->inst, sizeof(fh_h_dev_inst) * ninst, false)) ||
      (rc = fh_alloc(ctx, B->tl_by[0], sizeof(fh_h_tile) * B->tiles_by[0].size(), false)) ||
      (rc = fh_alloc(ctx, B->tl_by[1], sizeof(fh_h_tile) * B->tiles_by[1].size(), false)) ||
      (rc = fh_alloc(ctx, B->tl_by[2], sizeof(fh_h_tile) * B->tiles_by[2].size(), false)) || (rc = fh_alloc(ctx, B->U, st)) ||
      (rc = fh_alloc(ctx, B->Al, st)) || (rc = fh_alloc(ctx, B->Bt, st)) || (rc = fh_alloc(ctx, B->sA, st)) ||
      (rc = fh_alloc(ctx, B->sB, st)) || (rc = fh_alloc(ctx, B->sR, st)) || (rc = fh_alloc(ctx, B->sOm, st)) ||
      (rc = fh_alloc(ctx, B->D, st * (size_t)max_steps)) ||
      (rc = fh_alloc(ctx, B->W, sizeof(double) * 2 * (size_t)ninst * B->max_weights)) ||
      (rc = fh_alloc(ctx, B->Lb, sizeof(double) * (size_t)ninst * B->max_weights, false)) ||
      (rc = fh_alloc(ctx, B->ibt, sizeof(double) * kIbStride * (size_t)ninst, false)) ||
      (rc = fh_alloc(ctx, B->lgt, sizeof(double2) * (size_t)(max_steps + 2), false)) ||
      (rc = fh_alloc(ctx, B->wc, sizeof(double) * 2 * (size_t)ninst)) ||
      (rc = fh_alloc(ctx, B->part, st * (size_t)B->max_splits, false))) {
    delete B;
    return rc;
  }
  {
    int plo = 0, phi = 0;
    cudaError_t es = cudaDeviceGetStreamPriorityRange(&plo, &phi);
    if (es == cudaSuccess) es = cudaStreamCreateWithPriority(&B->hs, cudaStreamNonBlocking, phi);
    if (es == cudaSuccess) es = cudaEventCreateWithFlags(&B->ev_main, cudaEventDisableTiming);
    if (es == cudaSuccess) es = cudaEventCreateWithFlags(&B->ev_w, cudaEventDisableTiming);
    if (es != cudaSuccess) {
      delete B;
      return fh_set_error(ctx, FH_ECUDA, "fh_h_batch_create: weights stream: %s", cudaGetErrorString(es));
    }
  }
  // log(x) as (head, tail) doubles for x = 0..max_steps+1: the psi weights form
  // beta log(x/X) from it as a double-double; long double carries the tail
  std::vector<double2> lg((size_t)max_steps + 2);
  lg[0] = make_double2(0.0, 0.0);
  for (int x = 1; x < max_steps + 2; ++x) {
    const long double l = logl((long double)x);
    const double h = (double)l;
    lg[x] = make_double2(h, (double)(l - (long double)h));
  }
  B->di = di;
  cudaError_t e1 = cudaMemcpyAsync(B->inst.p, di.data(), sizeof(fh_h_dev_inst) * ninst, cudaMemcpyHostToDevice, ctx->stream);
  if (e1 == cudaSuccess)
    e1 = cudaMemcpyAsync(B->lgt.p, lg.data(), sizeof(double2) * lg.size(), cudaMemcpyHostToDevice, ctx->stream);
  cudaError_t e2 = cudaSuccess;
  for (int k = 0; k < 3 && e2 == cudaSuccess; ++k)
    e2 = cudaMemcpyAsync(B->tl_by[k].p, B->tiles_by[k].data(), sizeof(fh_h_tile) * B->tiles_by[k].size(),
                         cudaMemcpyHostToDevice, ctx->stream);
  cudaError_t e3 = cudaStreamSynchronize(ctx->stream);
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    delete B;
    return fh_set_error(ctx, FH_ECUDA, "fh_h_batch_create: upload failed");
  }
  k_h_lagtab<<<dim3((unsigned)fh_ceil_div(B->max_weights, 128), (unsigned)ninst), 128, 0, ctx->stream>>>(
      B->inst.as<fh_h_dev_inst>(), B->max_weights, B->Lb.as<double>(), B->max_weights);
  if ((rc = fh_after_launch(ctx, "k_h_lagtab"))) {
    delete B;
    return rc;
  }
  k_h_ibtab<<<(unsigned)fh_ceil_div(ninst, 128), 128, 0, ctx->stream>>>(B->inst.as<fh_h_dev_inst>(), ninst,
                                                                        B->ibt.as<double>());
  if ((rc = fh_after_launch(ctx, "k_h_ibtab"))) {
    delete B;
    return rc;
  }
  *out = B;
  return FH_OK;
}

int fh_h_batch_destroy(fh_h_batch *b) {
  if (!b) return FH_OK;
  if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return FH_OK;
}

long long fh_h_batch_device_bytes(const fh_h_batch *b) {
  if (!b) return -1;
  const fh_dbuf *bufs[] = {&b->inst, &b->U, &b->D, &b->W, &b->Lb, &b->ibt, &b->lgt, &b->wc, &b->part, &b->Al,
                           &b->Bt, &b->sA, &b->sB, &b->sR, &b->sOm, &b->wsp, &b->sV, &b->ring, &b->far, &b->cheb,
                           &b->tl_by[0], &b->tl_by[1], &b->tl_by[2]};
  size_t s = 0;
  for (const fh_dbuf *d : bufs) s += d->bytes;
  if (b->hb) s += fh_hblk_bytes(*b->hb);
  return (long long)s;
}

long long fh_h_batch_state_size(const fh_h_batch *b) {
  if (!b) return -1;
  long long s = 0;
  for (const auto &p : b->hp) s += p.N + 2;
  return s;
}

int fh_h_batch_set_u_host(fh_h_batch *b, const double *U_host) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, U_host, FH_EINVAL, "fh_h_batch_set_u_host: null pointer");
  long long src = 0;
  for (int i = 0; i < b->n; ++i) {
    const size_t cnt = (size_t)b->hp[i].N + 2;
    FH_CUDA_TRY(ctx, cudaMemcpyAsync(b->U.as<double>() + b->off[i], U_host + src, sizeof(double) * cnt,
                                     cudaMemcpyHostToDevice, ctx->stream));
    src += (long long)cnt;
  }
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  b->tstep = 1;
  b->nsaved = 0;
  return h_reset_clocks(b);
}

int fh_h_batch_restart(fh_h_batch *b, int i, const fh_h_params *p, const double *U0_host) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, p && U0_host && i >= 0 && i < b->n, FH_EINVAL, "fh_h_batch_restart: bad arguments");
  FH_REQUIRE(ctx, h_params_ok(*p), FH_EINVAL, "fh_h_batch_restart: bad parameters");
  FH_REQUIRE(ctx, p->N <= b->cap[i], FH_EINVAL, "fh_h_batch_restart: N = %d above the instance's %d nodes", p->N,
             b->cap[i]);
  FH_REQUIRE(ctx, b->mode != FH_H_BLOCKED && !b->space, FH_EINVAL,
             "fh_h_batch_restart: FP64 or DF64 history, no space-fractional instances");
  FH_REQUIRE(ctx, b->nsaved + 1 < b->max_steps, FH_ENOMEM, "fh_h_batch_restart: no history slots left (%d of %d)",
             b->nsaved, b->max_steps);
  fh_h_dev_inst I;
  h_fill_inst(*p, b->off[i], I);
  I.tb = b->tstep - 1;  // the occupant's first step is its step 1
  I.ob = b->nsaved;
  b->di[i] = I;
  b->hp[i] = *p;
  if (!I.fixed) b->varcoef = true;
  if (I.weights == FH_W_L1) b->has_l1 = true;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(b->U.as<double>() + b->off[i], U0_host, sizeof(double) * ((size_t)p->N + 2),
                                   cudaMemcpyHostToDevice, ctx->stream));
  fh_h_dev_inst *di = b->inst.as<fh_h_dev_inst>() + i;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(di, &b->di[i], sizeof(fh_h_dev_inst), cudaMemcpyHostToDevice, ctx->stream));
  // the occupant's lag and series tables
  k_h_lagtab<<<dim3((unsigned)fh_ceil_div(b->max_weights, 128), 1), 128, 0, ctx->stream>>>(
      di, b->max_weights, b->Lb.as<double>() + (long long)i * b->max_weights, b->max_weights);
  int rc = fh_after_launch(ctx, "k_h_lagtab");
  if (rc) return rc;
  k_h_ibtab<<<1, 32, 0, ctx->stream>>>(di, 1, b->ibt.as<double>() + (long long)i * kIbStride);
  if ((rc = fh_after_launch(ctx, "k_h_ibtab"))) return rc;
  // the host copy of the initial state and the records are read before return
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  b->w_ready = -1;  // weights prepared ahead used the previous occupant's clock
  b->graph.reset();
  return FH_OK;
}

int fh_h_batch_set_u(fh_h_batch *b, const double *U) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, U, FH_EINVAL, "fh_h_batch_set_u: null pointer");
  long long src = 0;
  for (int i = 0; i < b->n; ++i) {
    const size_t cnt = (size_t)b->hp[i].N + 2;
    FH_CUDA_TRY(ctx, cudaMemcpyAsync(b->U.as<double>() + b->off[i], U + src, sizeof(double) * cnt,
                                     cudaMemcpyDeviceToDevice, ctx->stream));
    src += (long long)cnt;
  }
  b->tstep = 1;
  b->nsaved = 0;
  return h_reset_clocks(b);
}

int fh_h_batch_get_u_host(fh_h_batch *b, double *U_host) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, U_host, FH_EINVAL, "fh_h_batch_get_u_host: null pointer");
  long long dst = 0;
  for (int i = 0; i < b->n; ++i) {
    const size_t cnt = (size_t)b->hp[i].N + 2;
    FH_CUDA_TRY(ctx, cudaMemcpyAsync(U_host + dst, b->U.as<double>() + b->off[i], sizeof(double) * cnt,
                                     cudaMemcpyDeviceToHost, ctx->stream));
    dst += (long long)cnt;
  }
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FH_OK;
}

int fh_h_batch_get_u_range_host(fh_h_batch *b, int first, int count, double *U_host) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, U_host && first >= 0 && count >= 0 && first + count <= b->n, FH_EINVAL,
             "fh_h_batch_get_u_range_host: bad range");
  long long dst = 0;
  for (int i = first; i < first + count; ++i) {
    const size_t cnt = (size_t)b->hp[i].N + 2;
    FH_CUDA_TRY(ctx, cudaMemcpyAsync(U_host + dst, b->U.as<double>() + b->off[i], sizeof(double) * cnt,
                                     cudaMemcpyDeviceToHost, ctx->stream));
    dst += (long long)cnt;
  }
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FH_OK;
}

// The persistent path: FP64 history, no space-fractional instances, few
// instances of at most kPersMaxNodes nodes each.
static bool h_persistent_ok(const fh_h_batch *b) {
  if (!b->persistent || b->mode != FH_H_FP64 || b->space || b->n > kPersMaxInst) return false;
  if ((b->max_steps + kPersCtas - 1) / kPersCtas > kPersMaxChunk) return false;
  for (const auto &p : b->hp)
    if (p.N + 2 > kPersMaxNodes) return false;
  return true;
}

static int h_persistent_run(fh_h_batch *b, int nsteps) {
  fh_ctx *ctx = b->ctx;
  b->w_ready = -1;
  fh_prof_mark(ctx, FH_PROF_HISTORY, false);
  const size_t smem = sizeof(double) * (size_t)((b->max_steps + kPersCtas - 1) / kPersCtas);
  k_h_persistent<<<(unsigned)(b->n * kPersCtas), kPersThreads, smem, ctx->stream>>>(
      b->inst.as<fh_h_dev_inst>(), b->tstep, b->nsaved, nsteps, b->D.as<double>(), b->Ptot, b->max_weights,
      b->wcp(0), b->Lb.as<double>(), b->ibt.as<double>(), b->lgt.as<double2>(), b->U.as<double>(),
      b->part.as<double>(), b->Al.as<double>(), b->Bt.as<double>(), b->sA.as<double>(), b->sB.as<double>(),
      b->sR.as<double>(), b->sOm.as<double>(), b->serial_al ? 1 : 0);
  fh_prof_mark(ctx, FH_PROF_HISTORY, true);
  int rc = fh_after_launch(ctx, "k_h_persistent");
  if (rc) return rc;
  b->nsaved += nsteps;
  b->tstep += nsteps;
  return FH_OK;
}

int fh_h_batch_step(fh_h_batch *b, int nsteps) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, nsteps >= 0, FH_EINVAL, "fh_h_batch_step: nsteps < 0");
  FH_REQUIRE(ctx, b->nsaved + nsteps <= b->max_steps, FH_ENOMEM, "fh_h_batch_step: history full (%d + %d > %d)",
             b->nsaved, nsteps, b->max_steps);
  if (nsteps >= 1 && h_persistent_ok(b)) return h_persistent_run(b, nsteps);
  if (b->use_graph && ctx->graphs && b->nsaved == 0 && nsteps > 1) {
    // whole solve from the initial state: capture once, replay afterwards
    b->w_ready = -1;
    int rc = fh_graph_run(ctx, b->graph, nsteps, [&]() {
      for (int i = 0; i < nsteps; ++i) {
        int r = h_one_step(b, i + 1 < nsteps);
        if (r) return r;
      }
      return (int)FH_OK;
    });
    if (rc) return rc;
    b->tstep = 1 + nsteps;
    b->nsaved = nsteps;
    return FH_OK;
  }
  b->w_ready = -1;
  for (int i = 0; i < nsteps; ++i) {
    int rc = h_one_step(b, i + 1 < nsteps);
    if (rc) return rc;
  }
  return FH_OK;
}



int fh_h_batch_tstep(const fh_h_batch *b) { return b ? b->tstep : -1; }

int fh_h_batch_set_persistent(fh_h_batch *b, int enable) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  b->persistent = enable != 0;
  b->graph.reset();
  return FH_OK;
}

int fh_h_batch_set_space_order(fh_h_batch *b, const double *gamma_host) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, gamma_host, FH_EINVAL, "fh_h_batch_set_space_order: null pointer");
  FH_REQUIRE(ctx, b->nsaved == 0, FH_EINVAL, "fh_h_batch_set_space_order: only before the first step");
  int maxN = 0;
  for (int i = 0; i < b->n; ++i) {
    const double g = gamma_host[i];
    FH_REQUIRE(ctx, g > 0.0 && g <= 1.0, FH_EINVAL, "fh_h_batch_set_space_order: gamma[%d] = %g not in (0, 1]", i, g);
    FH_REQUIRE(ctx, g == 1.0 || b->hp[i].N <= kSpaceMaxN, FH_EINVAL,
               "fh_h_batch_set_space_order: instance %d: N = %d > %d with gamma < 1", i, b->hp[i].N, kSpaceMaxN);
    if (g != 1.0 && b->hp[i].N > maxN) maxN = b->hp[i].N;
  }
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  // new buffers first: on failure the batch keeps its previous configuration
  fh_dbuf nw, nv;
  int rc;
  if (maxN > 0 && ((rc = fh_alloc(ctx, nw, sizeof(double) * (size_t)b->Ptot)) ||
                   (rc = fh_alloc(ctx, nv, sizeof(double) * (size_t)b->Ptot))))
    return rc;
  std::swap(b->wsp.p, nw.p);
  std::swap(b->wsp.bytes, nw.bytes);
  std::swap(b->sV.p, nv.p);
  std::swap(b->sV.bytes, nv.bytes);
  for (int i = 0; i < b->n; ++i) {
    fh_h_dev_inst &I = b->di[i];
    const double g = gamma_host[i];
    I.spg = g;
    I.spA = g == 1.0 ? 0.0 : 1.0 - g;
    if (g == 1.0) {
      I.Dg = pow(I.dL, -2.0);
      I.kbf = 1.0;
    } else {
      // reset_D: mt_minimal.cpp:744-749 dL^(-1-gamma)/Gamma(2-gamma),
      // mt_psi_caputo.cpp:1176-1181 dL^-2/Gamma(2-gamma)
      I.Dg = (I.weights == FH_W_L1 ? pow(I.dL, -1.0 - g) : pow(I.dL, -2.0)) / tgamma(2.0 - g);
      // kb(gamma, i-1, i, i, dL) of one interval at distance 1 (psi = x)
      const double gtj = I.dL, v = (gtj / gtj) * pow(gtj, 1.0 - g);
      const double v4 = pow(fabs(1.0 - 0.0 / gtj), 1.0 - g), v3 = pow(fabs(1.0 - gtj / gtj), 1.0 - g);
      I.kbf = (-(v3 - v4) / (1.0 - g)) * v;
    }
  }
  b->space = maxN > 0;
  b->space_smem = sizeof(double) * 2 * (size_t)maxN;
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(b->inst.p, b->di.data(), sizeof(fh_h_dev_inst) * b->n, cudaMemcpyHostToDevice,
                                   ctx->stream));
  if (b->space) {
    k_h_spw<<<dim3((unsigned)fh_ceil_div(maxN, 128), (unsigned)b->n), 128, 0, ctx->stream>>>(
        b->inst.as<fh_h_dev_inst>(), b->wsp.as<double>());
    if ((rc = fh_after_launch(ctx, "k_h_spw"))) return rc;
  }
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  b->graph.reset();
  return FH_OK;
}

// Times the batch history sum for every candidate launch shape (tile CTA of
// 128/256/512 threads, K split cap 1/8/64) at a probe depth of
// min(max_steps - 1, 512) layers on the batch's own buffers (history contents
// do not change the timing) and keeps the fastest.
int fh_h_batch_autotune(fh_h_batch *b, float *best_ms) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, !ctx->capturing, FH_EINVAL, "fh_h_batch_autotune: not during a capture");
  FH_REQUIRE(ctx, b->mode != FH_H_BLOCKED, FH_EINVAL, "fh_h_batch_autotune: the blocked mode has no split history sum");
  const int K = b->max_steps - 1 < 512 ? b->max_steps - 1 : 512;
  if (K < 32) return FH_OK;
  static const int caps[3] = {1, 8, 64};
  cudaEvent_t e0, e1;
  FH_CUDA_TRY(ctx, cudaEventCreate(&e0));
  FH_CUDA_TRY(ctx, cudaEventCreate(&e1));
  float best = 1e30f;
  int bt = b->tile_threads, bc = b->split_cap;
  for (int ti = 0; ti < 3; ++ti)
    for (int ci = 0; ci < 3; ++ci) {
      int splits, kchunk;
      h_plan(b->tiles_by[ti].size(), K, caps[ci] < b->max_splits ? caps[ci] : b->max_splits, &splits, &kchunk);
      if ((size_t)kchunk * sizeof(double) > 48 * 1024) continue;
      float ms = 0.f;
      for (int rep = 0; rep < 3; ++rep) {  // first repetition warms up
        cudaEventRecord(e0, ctx->stream);
        int rc = h_hist(b, ti, K, splits, kchunk, b->W.as<double>(), ctx->stream);
        if (rc) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          return rc;
        }
        cudaEventRecord(e1, ctx->stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          return fh_set_error(ctx, FH_ECUDA, "fh_h_batch_autotune: %s", cudaGetErrorString(e));
        }
        if (rep > 0) {
          float t = 0.f;
          cudaEventElapsedTime(&t, e0, e1);
          ms += t;
        }
      }
      if (ms < best) {
        best = ms;
        bt = kTileShapes[ti];
        bc = caps[ci];
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->tile_threads = bt;
  b->split_cap = bc;
  b->graph.reset();
  if (best_ms) *best_ms = best / 2;
  return FH_OK;
}

int fh_h_batch_launch_shape(const fh_h_batch *b, int *tile_threads, int *split_cap) {
  if (!b) return FH_EINVAL;
  if (tile_threads) *tile_threads = b->tile_threads;
  if (split_cap) *split_cap = b->split_cap;
  return FH_OK;
}

int fh_h_batch_set_mode(fh_h_batch *b, int mode) {
  FH_REQUIRE(nullptr, b, FH_EINVAL, "null batch");
  fh_ctx *ctx = b->ctx;
  FH_REQUIRE(ctx, mode == FH_H_FP64 || mode == FH_H_DF64 || mode == FH_H_BLOCKED, FH_EINVAL,
             "fh_h_batch_set_mode: unknown mode %d", mode);
  FH_REQUIRE(ctx, b->nsaved == 0, FH_EINVAL, "fh_h_batch_set_mode: only before the first step");
  int rc;
  if (mode == FH_H_BLOCKED && !b->hb) {
    // the weight-plane grids have n (interpolated groups) and 8 n rows
    FH_REQUIRE(ctx, (long long)b->n * 8 <= 65535, FH_EINVAL,
               "fh_h_batch_set_mode: the blocked mode takes at most 8191 instances (%d)", b->n);
    // 128-point tiles of every instance's segment
    std::vector<long long> tp0;
    std::vector<int> tin, tnp;
    for (int i = 0; i < b->n; ++i) {
      const int seg = b->hp[i].N + 2;
      for (int k = 0; k < seg; k += 128) {
        tp0.push_back(b->off[i] + k);
        tin.push_back(i);
        tnp.push_back(seg - k < 128 ? seg - k : 128);
      }
    }
    const int kcap = (int)fh_ceil_div(b->max_steps, kSlcK) * kSlcK;
    std::vector<double> ct;
    hb_cheb_table(ct);
    b->hb = fh_hblk_new();
    if ((rc = fh_hblk_init(ctx, *b->hb, b->Ptot, kcap, b->n, tp0.data(), tin.data(), tnp.data(), (int)tp0.size())) ||
        (rc = fh_alloc(ctx, b->ring, sizeof(float2) * 128 * (size_t)b->Ptot)) ||
        (rc = fh_alloc(ctx, b->far, sizeof(float2) * kSlcK * (size_t)b->Ptot, false)) ||
        (rc = fh_alloc(ctx, b->cheb, sizeof(double) * ct.size(), false)) ||
        (rc = cudaMemcpy(b->cheb.p, ct.data(), sizeof(double) * ct.size(), cudaMemcpyHostToDevice) != cudaSuccess
                  ? fh_set_error(ctx, FH_ECUDA, "fh_h_batch_set_mode: upload of the interpolation tables failed")
                  : FH_OK)) {
      fh_hblk_delete(b->hb);
      b->hb = nullptr;
      b->ring.release();
      b->far.release();
      b->cheb.release();
      return rc;
    }
    b->D.release();  // the full-precision history is not kept in this mode
  }
  if (mode != FH_H_BLOCKED && b->hb) {
    fh_hblk_delete(b->hb);
    b->hb = nullptr;
    b->ring.release();
    b->far.release();
    b->cheb.release();
    if ((rc = fh_alloc(ctx, b->D, sizeof(double) * (size_t)b->Ptot * (size_t)b->max_steps))) return rc;
  }
  b->mode = mode;
  // the blocked mode's bound is 1e-9: Al by the parallel Moebius scan (within
  // ~1e-10), not by the serial reference-order chain the 1e-12 modes need
  b->serial_al = mode != FH_H_BLOCKED;
  b->graph.reset();
  return FH_OK;
}

}  // extern "C"
