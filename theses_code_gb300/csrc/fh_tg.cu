// fh_tg.cu -- 2D ADI solver with full fractional history, the TG_solver_<.,1,.>
// path of fr_d_t_g_2d.cpp with dt_alg 0 (fr_d_t_g_2d.cpp:2552-2718, 3242-3553).
//
// Per time step j (launches on the context stream):
//   1. weights        x/y history weights for k < j and the three current
//                     weights (a per-solve table when it fits, else per step)
//   2. history sum    S_x, S_y over the stored full-step differences, one pass
//                     (the reference reads the layers once per half step);
//                     in blocked mode only the layers of the current 64-step
//                     block, the older ones come from the tensor-core rows
//   3. k_tg_xsweep    one CTA per x line (j = 1..M-1), unknowns along i; writes
//                     the half-step field Ch
//   4. k_tg_ysweep    four y lines per CTA (i = 1..sN-1), unknowns along j;
//                     writes the new full-step field C and appends the new
//                     full-step difference to the history
// The Thomas factorization of both sweep directions depends only on V2, d and
// the current weight; for psi = t that weight is the same every step, so the
// factorization is built once (k_tg_factor) and each step only runs the two
// affine recurrences (fh_linescan.cuh).  For psi != t it is rebuilt per step.
//
// Storage (HBM): C, Ch, V2 and the factor tables are (sN+2)(M+2) doubles in
// the reference layout idx = i + j*(sN+2); the history holds one difference
// layer per full step, D[k] = C^{k+1} - C^k (the half-step layers the
// reference also stores are only read through Ch).
#include <algorithm>
#include <cmath>
#include <vector>
#include <mutex>

#include "fh_internal.h"
#include "fh_common.cuh"
#include "fh_linescan.cuh"
#include "fh_sm100.cuh"
#include "fh_slices.cuh"
#include "fh_weights.cuh"
#include "fh_two_series.h"

// blocked contraction helpers (fh_blocked.cu)
struct fh_blk;
fh_blk *fh_blk_new();
void fh_blk_delete(fh_blk *b);
size_t fh_blk_bytes(const fh_blk &b);
int fh_blk_init(fh_ctx *ctx, fh_blk &b, long long P, int Kcap);
int fh_blk_convert(fh_ctx *ctx, fh_blk &b, const double *D, long long ldd, int k0, int df);
int fh_blk_tg_weights(fh_ctx *ctx, fh_blk &b, int j0, double Da, double tau, double alpha, double beta, double cut,
                      const double *table, int ldw, int nsteps);
int fh_blk_gemm(fh_ctx *ctx, fh_blk &b, int K, float2 *out, long long ldo, int gbeg = 0);
long long fh_blk_ppad(const fh_blk &b);
static constexpr int kTgBlock = 64;  // steps per block (128 weight rows)

struct fh_tg_dev {
  int sN, M, ld;
  long long P;
  double tau, alpha, beta, Da, st, d, C1, S, dL, dLx;
  double hcut;  // restricted summing: history weights below hcut are 0 (0: full history)
  // diffusion coefficient: d (fixed_d), else lambda |v| (ka0 / kk) per node
  // (TG_solver_<func,0,0>::D, fr_d_t_g_2d.cpp:2787-2800)
  int fixed_d = 1;
  double lam = 0.0, ka0 = 0.0, kk = 1.0;
};

// D at a node of |v|^2 = v2.
__device__ __forceinline__ double tg_D(const fh_tg_dev &g, double v2) {
  if (g.fixed_d) return g.d;
  const double v = sqrt(v2);
  const double k_ = g.ka0 / g.kk;
  return g.lam * v * k_;
}

// History weight w with restricted summing (dt_alg 2, fr_d_t_g_2d.cpp:3356-3380):
// the reference's sums run from the newest layer pair back and stop at the
// first weight below dt_eps.  The weights fall monotonically with the lag
// (psi increasing), so zeroing every weight below dt_eps drops exactly the
// layers the reference leaves out.
__device__ __forceinline__ double tg_hw(const fh_tg_dev &g, double w) { return fabs(w) < g.hcut ? 0.0 : w; }

struct fh_tg_solver {
  fh_ctx *ctx = nullptr;
  fh_tg_params p{};
  fh_tg_dev dv{};
  int mode = FH_TG_FP64;
  bool df = false;        // history stored as (hi, lo) FP32 pairs
  int max_steps = 0;
  int tstep = 0;
  bool have_state = false;
  bool factor_fixed = false;
  int max_splits = 8;
  fh_dbuf C, Ch, V2, D, W, cw, part, alx, gx, fax, pfx, pbx, aly, gy, fay, pfy, pby, far;
  // blocked mode: the sweeps run in double-float; fields and factor tables as (hi, lo) pairs
  bool dfsweep = false;
  fh_dbuf Cd, Chd, fax2, gx2, alx2, pfx2, pbx2, fay2, gy2, aly2, pfy2, pby2;
  // fused sub-block sweeps (k_tg_sweeps_fused): grid-barrier counter, error flag
  bool fused = false;
  int fuse_blocks = 0;
  fh_dbuf bar, derr;
  // blocked mode with a per-solve weight table: mid rows on the tensor cores
  // (k_tg_mid_tc); mws / mwe: every sub-block's weight slices and row exponents
  bool mid_tc = false;
  fh_dbuf mws, mwe;
  bool wtab = false;      // Wall/cwall hold every step's weights (computed at step 0)
  fh_blk *blk = nullptr;  // blocked mode: bf16 slice planes and tensor maps
  int j0 = 0;             // first step of the current block (far rows valid when j0 > 0)
  long long ldfar = 0;
  fh_graph_cache graph;
  // restricted summing with psi = t: every history weight of a lag beyond
  // rs_lag is below the cut (-1: unknown or full history)
  int rs_lag = -1;
  // series expansion (dt_alg 3): ser_J terms, accumulators H[n][p], per-step
  // coefficient rows ser_tab[j] = c[J] | ex[J] | ey[J]; the history store
  // keeps only the newest layer pair
  int ser_J = 0;
  fh_dbuf H, ser_tab;
  // two-series approximation (dt_alg 4): planned tables and coefficient
  // slots; the history store keeps only the newest layer pair
  fh_ta *two = nullptr;
  bool one_layer() const { return ser_J || two; }
  // mass exchange (TG_solver::N1): N per node and the right-part term dN of
  // the current half step; c1 = 1/(2 + tau a b), tsb = tau sigma b
  bool massN = false;
  double mass_c1 = 0.0, mass_tsb = 0.0;
  fh_dbuf Nn, dN;
  ~fh_tg_solver() {
    if (two) fh_ta_delete(two);
    if (blk) fh_blk_delete(blk);
  }
};

// ---------------------------------------------------------------- kernels

// W[0][k] = kb(k,0.5,0.0,1.0), W[1][k] = kb(k,1.0,0.0,1.0) for k < j;
// cw = {kb(j,0.5,0.0,0.5), kb(j,1.0,0.5,0.5), kb(j,1.0,0.0,0.5)} (TG_solver_::kb).
__global__ void k_tg_weights(fh_tg_dev g, int j, int kstart, double *__restrict__ W, int ldw,
                             double *__restrict__ cw) {
  const int k = kstart + blockIdx.x * blockDim.x + threadIdx.x;
  if (k < j) {
    const double s0 = (double)k + 0.0;
    W[k] = tg_hw(g, g.Da * fh_psi_int(s0, s0 + 1.0, (double)j + 0.5, g.tau, g.alpha, g.beta));
    W[ldw + k] = tg_hw(g, g.Da * fh_psi_int(s0, s0 + 1.0, (double)j + 1.0, g.tau, g.alpha, g.beta));
  }
  if (k == kstart) {
    const double jj = (double)j;
    cw[0] = g.Da * fh_psi_int(jj + 0.0, jj + 0.0 + 0.5, jj + 0.5, g.tau, g.alpha, g.beta);
    cw[1] = g.Da * fh_psi_int(jj + 0.5, jj + 0.5 + 0.5, jj + 1.0, g.tau, g.alpha, g.beta);
    cw[2] = g.Da * fh_psi_int(jj + 0.0, jj + 0.0 + 0.5, jj + 1.0, g.tau, g.alpha, g.beta);
  }
}

// Mass exchange with the non-soluble phase, TG_solver::N1 (fr_d_t_g_2d.cpp:
// 2503-2521) before each half step over the nodes i <= sN, j <= M:
// N' = c1 (2 N + tsb C) with c1 = 1/(2 + tau a b), tsb = tau sigma b; the
// half step's right parts add dN = (1/tau) (N' - N) (3330-3332).  Before the
// y half step C is the half-step field: Ch on the x lines (rows 1..M-1), C on
// rows 0 and M, which the x half step leaves alone.
__global__ void k_tg_n1(fh_tg_dev g, int half, const double *__restrict__ C, const double *__restrict__ Ch,
                        double c1, double tsb, double *__restrict__ Nn, double *__restrict__ dN) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nn = (long long)(g.sN + 1) * (g.M + 1);
  if (t >= nn) return;
  const int i = (int)(t % (g.sN + 1)), j = (int)(t / (g.sN + 1));
  const long long id = i + (long long)j * g.ld;
  const double c = (half && j >= 1 && j < g.M) ? Ch[id] : C[id];
  const double prev = Nn[id];
  const double nw = c1 * (2 * prev + tsb * c);
  Nn[id] = nw;
  dN[id] = (1.0 / g.tau) * (nw - prev);
}

// Coefficients of the factorization, one thread per node (coalesced in both
// directions): A and B of node i of every line into Ao and Bo (the pf and pb
// arrays of the direction, which k_tg_factor reads in its serial pass and then
// overwrites with its prefix products).  dir 0: x lines, dir 1: y lines.  A, B
// in the reference's arithmetic (fr_d_t_g_2d.cpp:2579-2584, 2636-2641).
__global__ void k_tg_factor_coef(fh_tg_dev g, int dir, const double *__restrict__ V2, double *__restrict__ Ao,
                                 double *__restrict__ Bo) {
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= g.P) return;
  const int row = (int)(id / g.ld), col = (int)(id % g.ld);
  const int line = dir == 0 ? row : col, i = dir == 0 ? col : row;
  const int nlines = dir == 0 ? g.M : g.sN, N = dir == 0 ? g.sN : g.M;
  if (line < 1 || line >= nlines || i < 1 || i >= N) return;
  const long long stride = dir == 0 ? 1 : g.ld;
  const double dl = dir == 0 ? g.dL : g.dLx;
  const double v2 = V2[id];
  // A_ and B (fr_d_t_g_2d.cpp:3242-3257): D(i-1) + D(i) and D(i+1) + D(i)
  const double Dc = tg_D(g, v2), Dm = tg_D(g, V2[id - stride]), Dp = tg_D(g, V2[id + stride]);
  double A, B;
  if (dir == 0) {
    A = (v2 / dl) * ((0.5 * (Dm + Dc) / dl) + 0.5);
    B = (v2 / dl) * ((0.5 * (Dp + Dc) / dl) - 0.5);
  } else {
    A = (v2 / (dl * dl)) * 0.5 * (Dm + Dc);
    B = (v2 / (dl * dl)) * 0.5 * (Dp + Dc);
  }
  Ao[id] = A;
  Bo[id] = B;
}

// Serial pass of the factorization (one thread per line).  The reference's
// pivot recurrence Al_{i+1} = B_i / den_i, den_i = R_i - A_i Al_i, g_i =
// Al_{i+1} / B_i (= 1 / den_i) runs as its continuant, Al_i = P_i / Q_i:
//   P_{i+1} = B_i Q_i,  Q_{i+1} = R_i Q_i - A_i P_i  (= den_i Q_i),
// two FP64 operations per node on the serial path instead of an FP64
// division (whose latency set the pace: ~1.3 us per node); P and Q are
// rescaled by a power of two when |Q| leaves [2^-400, 2^400] (exact, the
// ratios stay).  Stores P_{i+1} (al), Q_{i+1} (gg) and Q_i (fa) of node i;
// k_tg_factor_ratio turns them into Al, g and fa = g A.  pf and pb hold A
// and B (k_tg_factor_coef) and are not written here.
__global__ void k_tg_factor(fh_tg_dev g, int dir, const double *__restrict__ cw, double *__restrict__ al,
                            double *__restrict__ gg, double *__restrict__ fa, const double *__restrict__ pf,
                            const double *__restrict__ pb) {
  const int line = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int nlines = dir == 0 ? g.M : g.sN;
  if (line >= nlines) return;
  const int N = dir == 0 ? g.sN : g.M;
  const long long base = dir == 0 ? (long long)line * g.ld : line;
  const long long stride = dir == 0 ? 1 : g.ld;
  const double kcur = dir == 0 ? cw[0] : cw[1];
  double P = dir == 0 ? 0.0 : 1.0, Q = 1.0;
#pragma unroll 4
  for (int i = 1; i < N; ++i) {
    const long long id = base + i * stride;
    const double A = pf[id], B = pb[id];
    const double R = g.st * (kcur + 0.0) + A + B;
    const double Pn = B * Q, Qn = R * Q - A * P;
    al[id] = Pn;
    gg[id] = Qn;
    fa[id] = Q;
    P = Pn;
    Q = Qn;
    const double m = fabs(Q);
    if (m > 0x1p400 || m < 0x1p-400) {
      const int e = ilogb(Q);
      P = scalbn(P, -e);
      Q = scalbn(Q, -e);
    }
  }
}

// Ratios of the serial pass, one thread per node: Al_{i+1} = P_{i+1} / Q_{i+1},
// g_i = Q_i / Q_{i+1}, fa_i = g_i A_i.
__global__ void k_tg_factor_ratio(fh_tg_dev g, int dir, double *__restrict__ al, double *__restrict__ gg,
                                  double *__restrict__ fa, const double *__restrict__ pf) {
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= g.P) return;
  const int row = (int)(id / g.ld), col = (int)(id % g.ld);
  const int line = dir == 0 ? row : col, i = dir == 0 ? col : row;
  const int nlines = dir == 0 ? g.M : g.sN, N = dir == 0 ? g.sN : g.M;
  if (line < 1 || line >= nlines || i < 1 || i >= N) return;
  const double Qn = gg[id];
  const double gi = fa[id] / Qn;
  al[id] = al[id] / Qn;
  gg[id] = gi;
  fa[id] = gi * pf[id];
}

// The whole factorization of one line per warp, for lines whose five
// per-node arrays fit in shared memory: the coefficients A, B (lanes over the
// nodes, as k_tg_factor_coef), the continuant chain (lane 0, as k_tg_factor,
// from shared memory instead of global loads on the serial path), the ratios
// (lanes, as k_tg_factor_ratio) and the chunk prefix products (lane c its
// chunk c, as k_tg_factor_prefix); the same operations, so the same values.
constexpr int kFactorLineArrays = 5;
__global__ void __launch_bounds__(32) k_tg_factor_line(fh_tg_dev g, int dir, const double *__restrict__ V2,
                                                       const double *__restrict__ cw, double *__restrict__ al,
                                                       double *__restrict__ gg, double *__restrict__ fa,
                                                       double *__restrict__ pf, double *__restrict__ pb) {
  extern __shared__ double fsm[];
  const int line = 1 + blockIdx.x, lane = threadIdx.x;
  const int N = dir == 0 ? g.sN : g.M;
  const long long base = dir == 0 ? (long long)line * g.ld : line;
  const long long stride = dir == 0 ? 1 : g.ld;
  double *sA = fsm, *sB = sA + N, *sP = sB + N, *sQn = sP + N, *sQ = sQn + N;
  const double dl = dir == 0 ? g.dL : g.dLx;
  for (int i = 1 + lane; i < N; i += 32) {
    const long long id = base + i * stride;
    const double v2 = V2[id];
    const double Dc = tg_D(g, v2), Dm = tg_D(g, V2[id - stride]), Dp = tg_D(g, V2[id + stride]);
    double A, B;
    if (dir == 0) {
      A = (v2 / dl) * ((0.5 * (Dm + Dc) / dl) + 0.5);
      B = (v2 / dl) * ((0.5 * (Dp + Dc) / dl) - 0.5);
    } else {
      A = (v2 / (dl * dl)) * 0.5 * (Dm + Dc);
      B = (v2 / (dl * dl)) * 0.5 * (Dp + Dc);
    }
    sA[i] = A;
    sB[i] = B;
  }
  __syncwarp();
  if (lane == 0) {
    const double kcur = dir == 0 ? cw[0] : cw[1];
    double P = dir == 0 ? 0.0 : 1.0, Q = 1.0;
    for (int i = 1; i < N; ++i) {
      const double A = sA[i], B = sB[i];
      const double R = g.st * (kcur + 0.0) + A + B;
      const double Pn = B * Q, Qn = R * Q - A * P;
      sP[i] = Pn;
      sQn[i] = Qn;
      sQ[i] = Q;
      P = Pn;
      Q = Qn;
      const double m = fabs(Q);
      if (m > 0x1p400 || m < 0x1p-400) {
        const int e = ilogb(Q);
        P = scalbn(P, -e);
        Q = scalbn(Q, -e);
      }
    }
  }
  __syncwarp();
  for (int i = 1 + lane; i < N; i += 32) {
    const long long id = base + i * stride;
    const double Qn = sQn[i];
    const double gi = sQ[i] / Qn;
    const double aln = sP[i] / Qn;
    const double fai = gi * sA[i];
    al[id] = aln;
    gg[id] = gi;
    fa[id] = fai;
    sP[i] = aln;
    sQ[i] = fai;
  }
  __syncwarp();
  const int chf = fh_chunk_f(N), chb = fh_chunk_b(N);
  const int f0 = 1 + lane * chf, f1 = min(N, f0 + chf);
  double p = 1.0;
  for (int i = f0; i < f1; ++i) {
    p = (i == f0) ? sQ[i] : p * sQ[i];
    pf[base + i * stride] = p;
  }
  const double al1 = dir == 0 ? 0.0 : 1.0;
  const int b0 = lane * chb, b1 = min(N, b0 + chb);
  double q = 1.0;
  for (int i = b1 - 1; i >= b0; --i) {
    const double a = (i >= 1) ? sP[i] : al1;
    q = (i == b1 - 1) ? a : q * a;
    pb[base + i * stride] = q;
  }
}

// Chunk prefix products of the forward slopes fa and of the backward slopes
// Al in the lane chunking of fh_line_solve_prefix (one thread per line).
__global__ void k_tg_factor_prefix(fh_tg_dev g, int dir, const double *__restrict__ al, const double *__restrict__ fa,
                                   double *__restrict__ pf, double *__restrict__ pb) {
  const int line = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int nlines = dir == 0 ? g.M : g.sN;
  if (line >= nlines) return;
  const int N = dir == 0 ? g.sN : g.M;
  const long long base = dir == 0 ? (long long)line * g.ld : line;
  const long long stride = dir == 0 ? 1 : g.ld;
  const int chf = fh_chunk_f(N), chb = fh_chunk_b(N);
  double p = 1.0;
  for (int i = 1; i < N; ++i) {
    const long long id = base + i * stride;
    p = ((i - 1) % chf == 0) ? fa[id] : p * fa[id];
    pf[id] = p;
  }
  const double al1 = dir == 0 ? 0.0 : 1.0;
  double q = 1.0;
  for (int i = N - 1; i >= 0; --i) {
    const long long id = base + i * stride;
    const int b1 = min(N, (i / chb + 1) * chb);
    const double a = (i >= 1) ? al[id] : al1;
    q = (i == b1 - 1) ? a : q * a;
    pb[id] = q;
  }
}

// All step weights of a solve in one launch: row j of Wall holds
// [kb(k,0.5,0,1) for k < j | kb(k,1,0,1) for k < j] (x and y rows, pitch ldw),
// cwall[4j..4j+2] the three current weights of step j.
// psi = t (beta 1): slot [k, k+1] of row j takes fh_psi_int_t's bound terms
// pow(|1 - tau x / gtj|, 1 - alpha) at x = k and x = k + 1, and its row factor
// gtj / gtj * pow(gtj, 1 - alpha): each is computed once per CTA (the same
// operations, so the same values) instead of once per slot.
constexpr int kWallThreads = 128;
__global__ void __launch_bounds__(kWallThreads) k_tg_weights_all(fh_tg_dev g, int nsteps, double *__restrict__ Wall,
                                                                 int ldw, double *__restrict__ cwall) {
  __shared__ double bnd[2][kWallThreads + 1], rowf[2];
  const int k = blockIdx.x * kWallThreads + threadIdx.x;
  const int j = blockIdx.y;
  if (j >= nsteps) return;
  double *W = Wall + (long long)j * 2 * ldw;
  const int k0 = blockIdx.x * kWallThreads;
  if (g.beta == 1.0) {
    if (k0 < j) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const double gtj = g.tau * ((double)j + (h ? 1.0 : 0.5));
        for (int b = threadIdx.x; b <= kWallThreads; b += kWallThreads) {
          const int x = k0 + b;
          bnd[h][b] = x <= j ? pow(fabs(1.0 - (g.tau * (double)x) / gtj), 1 - g.alpha) : 0.0;
        }
        if (threadIdx.x == 0) {
          double v = gtj / gtj;
          v *= pow(gtj, 1 - g.alpha);
          rowf[h] = v;
        }
      }
      __syncthreads();
      if (k < j) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const double v2 = -(bnd[h][threadIdx.x + 1] - bnd[h][threadIdx.x]) / (1 - g.alpha);
          double sum = 0.0;
          sum += v2 * rowf[h];
          W[(long long)h * ldw + k] = tg_hw(g, g.Da * sum);
        }
      }
    }
  } else if (k0 < j) {
    // psi = t^beta: the series tables of a = 1/beta, b = 1 - alpha, once per CTA
    __shared__ double Lc[kIbTerms], Uc[kIbTerms], cst[2];
    const double a = 1.0 / g.beta, b = 1.0 - g.alpha;
    if (threadIdx.x == 0) {
      fh_ib_tables(a, b, Lc, Uc);
      cst[0] = pow(kIbLowMax, a);
      cst[1] = exp(lgamma(a) + lgamma(b) - lgamma(a + b));
    }
    __syncthreads();
    if (k < j) {
      const double s0 = (double)k + 0.0;
      W[k] = tg_hw(g, g.Da * fh_psi_int_pre(s0, s0 + 1.0, (double)j + 0.5, g.tau, g.alpha, g.beta, Lc, Uc, cst[0],
                                            cst[1]));
      W[ldw + k] = tg_hw(g, g.Da * fh_psi_int_pre(s0, s0 + 1.0, (double)j + 1.0, g.tau, g.alpha, g.beta, Lc, Uc,
                                                  cst[0], cst[1]));
    }
  }
  if (k == 0) {
    const double jj = (double)j;
    cwall[4 * j + 0] = g.Da * fh_psi_int(jj + 0.0, jj + 0.0 + 0.5, jj + 0.5, g.tau, g.alpha, g.beta);
    cwall[4 * j + 1] = g.Da * fh_psi_int(jj + 0.5, jj + 0.5 + 0.5, jj + 1.0, g.tau, g.alpha, g.beta);
    cwall[4 * j + 2] = g.Da * fh_psi_int(jj + 0.0, jj + 0.0 + 0.5, jj + 1.0, g.tau, g.alpha, g.beta);
  }
}

// Series expansion of the history sums (dt_alg 3, psi = t; fr_d_t_g_2d.cpp:
// 3384-3429): per point the accumulators gain the newest layer pair,
// H[n] += c[n] (C^j - C^(j-1)) (one FMA: FP64-pipe-bound kernel), and the
// x and y sums are Da sum_n e[n] H[n] with the per-step coefficients
// e[n] = (alpha)_n / n! gtj^(-alpha-n) of the two half-step times (zero after
// the reference's cut at the first non-finite one).  Writes the sums where
// the sweeps read one K split (part[0][p], part[1][p]).  One point per
// thread; the step's coefficient row staged in shared memory.
static constexpr int kSerMaxTerms = 256;
__global__ void __launch_bounds__(256) k_tg_series(const double *__restrict__ Dn, int df, double *__restrict__ H, int J,
                                                   long long P, const double *__restrict__ tab, double Da,
                                                   double *__restrict__ part) {
  __shared__ double ct[3 * kSerMaxTerms];
  for (int i = threadIdx.x; i < 3 * J; i += blockDim.x) ct[i] = tab[i];
  __syncthreads();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  double d;
  if (df) {
    const float2 v = reinterpret_cast<const float2 *>(Dn)[p];
    d = (double)v.x + (double)v.y;
  } else {
    d = Dn[p];
  }
  double sx = 0.0, sy = 0.0;
  double *h = H + p;
  for (int n = 0; n < J; ++n, h += P) {
    const double v = fma(ct[n], d, *h);
    *h = v;
    sx = fma(ct[J + n], v, sx);
    sy = fma(ct[2 * J + n], v, sy);
  }
  part[p] = Da * sx;
  part[P + p] = Da * sy;
}

// Shared-memory footprint of one staged line array: fh_sk(N+1)+1 doubles.
__host__ __device__ inline int tg_line_stride(int N) { return (N + 2) + ((N + 2) >> 4) + 2; }

static constexpr int kXLines = 4;       // x lines per CTA, one solving warp each
static constexpr int kXGroup = 128;     // threads staging / writing one line
static constexpr int kXThreads = kXGroup * kXLines;
static constexpr int kYThreads = 512;  // four adjacent y lines per CTA
static constexpr int kUnroll = 4;      // equations staged per thread per round

// x half-step (fr_d_t_g_2d.cpp:2577-2590): four lines j per CTA.  A group of
// 128 threads per line stages its forward maps into shared memory with
// independent, coalesced loads (all four lines in one round trip), then warp
// w solves line w (the four solving warps sit on the SM's four
// sub-partitions, so the solves run in parallel), then the groups write the
// half-step field Ch.  The boundary
// nodes i = 0, N, N+1 are also written into C, which otherwise keeps the
// full-step field.
__global__ void __launch_bounds__(kXThreads) k_tg_xsweep(fh_tg_dev g, double *C, double *__restrict__ Ch,
                                                        const double *__restrict__ part, long long ldp, int splits,
                                                        const double *__restrict__ fax,
                                                        const double *__restrict__ gx,
                                                        const double *__restrict__ alx,
                                                        const double *__restrict__ pfx,
                                                        const double *__restrict__ pbx,
                                                        const double *__restrict__ cw,
                                                        const float2 *__restrict__ far,
                                                        const double *__restrict__ dN) {
  extern __shared__ double sbuf[];
  const int warp = threadIdx.x >> 5;
  const int line0 = 1 + blockIdx.x * kXLines;
  const int N = g.sN;
  const int L = tg_line_stride(N);
  const double kst = -g.st * (cw[0] + 0.0), S2 = g.S * 0.5, st = g.st;
  {
    const int ln = threadIdx.x / kXGroup, tg = threadIdx.x % kXGroup;
    const int line = line0 + ln;
    double *fa = sbuf + (size_t)ln * 5 * L, *fb = fa + L, *al = fb + L, *pf = al + L, *pb = pf + L;
    const long long base = (long long)line * g.ld;
    for (int r0 = 1; line < g.M && r0 < N; r0 += kXGroup * kUnroll) {
      double ts[kUnroll], c[kUnroll], a[kUnroll], gi[kUnroll], l[kUnroll], qf[kUnroll], qb[kUnroll];
#pragma unroll
      for (int e = 0; e < kUnroll; ++e) {
        const int i = r0 + tg + e * kXGroup;
        const long long id = base + (i < N ? i : 1);
        c[e] = C[id];
        a[e] = fax[id];
        gi[e] = gx[id];
        l[e] = alx[id];
        qf[e] = pfx[id];
        qb[e] = pbx[id];
        ts[e] = 0.0;
        if (far) {
          const float2 fp = far[id];
          ts[e] = (double)fp.x + (double)fp.y;
        }
      }
      for (int s = 0; s < splits; ++s)
#pragma unroll
        for (int e = 0; e < kUnroll; ++e) {
          const int i = r0 + tg + e * kXGroup;
          ts[e] += part[(long long)(2 * s) * ldp + base + (i < N ? i : 1)];
        }
#pragma unroll
      for (int e = 0; e < kUnroll; ++e) {
        const int i = r0 + tg + e * kXGroup;
        if (i < N) {
          double om = kst * c[e];
          om += S2;
          if (dN) om += dN[base + i];  // mass exchange
          om += st * ts[e];
          fa[fh_sk(i)] = a[e];
          fb[fh_sk(i)] = -gi[e] * om;
          al[fh_sk(i)] = l[e];
          pf[fh_sk(i)] = qf[e];
          pb[fh_sk(i)] = qb[e];
        }
      }
    }
    // node 0 belongs to lane 0's backward chunk: its prefix product
    if (tg == 0 && line < g.M) pb[fh_sk(0)] = pbx[base];
  }
  __syncthreads();
  if (warp < kXLines && line0 + warp < g.M) {
    double *fa = sbuf + (size_t)warp * 5 * L;
    // bt scratch reuses pf's slots only after pf is consumed: use a separate
    // region, the fb array, which the forward walk overwrites in place
    fh_line_solve_prefix(N, fa, fa + L, fa + 2 * L, fa + 3 * L, fa + 4 * L, 0.0, g.C1, fa + L, fa);
  }
  __syncthreads();
  {
    const int ln = threadIdx.x / kXGroup, tg = threadIdx.x % kXGroup;
    const int line = line0 + ln;
    const double *u = sbuf + (size_t)ln * 5 * L;
    const long long base = (long long)line * g.ld;
    for (int i = tg; line < g.M && i <= N + 1; i += kXGroup) {
      const double v = u[fh_sk(i)];
      Ch[base + i] = v;
      if (i == 0 || i >= N) C[base + i] = v;
    }
  }
}

// y half-step (fr_d_t_g_2d.cpp:2634-2648): four adjacent lines i per CTA so
// that the strided column loads share 32-byte sectors; 128 threads stage each
// line (kUnroll rows per thread in flight), warp w solves line w.  Reads the
// half-step field Ch and the full-step field C, writes the new full-step field
// into C and appends the difference D_j = C^{j+1} - C^j.
__global__ void __launch_bounds__(kYThreads) k_tg_ysweep(fh_tg_dev g, double *C, const double *__restrict__ Ch,
                                                        double *__restrict__ Dj, const double *__restrict__ part,
                                                        long long ldp, int splits, const double *__restrict__ fay,
                                                        const double *__restrict__ gy,
                                                        const double *__restrict__ aly,
                                                        const double *__restrict__ pfy,
                                                        const double *__restrict__ pby,
                                                        const double *__restrict__ cw,
                                                        const float2 *__restrict__ far, int dfstore,
                                                        const double *__restrict__ dN) {
  extern __shared__ double sbuf[];
  const int warp = threadIdx.x >> 5;
  const int N = g.M;
  const int L = tg_line_stride(N);
  const int i0 = 1 + blockIdx.x * 4;
  const double kst = -g.st * (cw[1] + 0.0), kyh = cw[2], S2 = g.S * 0.5, st = g.st;
  const int col = threadIdx.x & 3;
  const int rg = threadIdx.x >> 2;  // row group 0..127
  constexpr int kRows = kYThreads / 4;
  const int line = i0 + col;
  const bool live = line < g.sN;
  double *fa = sbuf + (size_t)col * 6 * L, *fb = fa + L, *al = fb + L, *pf = al + L, *pb = pf + L, *cf = pb + L;
  for (int r0 = 1; r0 < N; r0 += kRows * kUnroll) {
    double ts[kUnroll], c[kUnroll], f[kUnroll], a[kUnroll], gi[kUnroll], l[kUnroll], qf[kUnroll], qb[kUnroll];
#pragma unroll
    for (int e = 0; e < kUnroll; ++e) {
      const int q = r0 + rg + e * kRows;
      const long long id = (live ? line : 1) + (long long)(q < N ? q : 1) * g.ld;
      c[e] = Ch[id];
      f[e] = C[id];
      a[e] = fay[id];
      gi[e] = gy[id];
      l[e] = aly[id];
      qf[e] = pfy[id];
      qb[e] = pby[id];
      ts[e] = 0.0;
      if (far) {
        const float2 fp = far[id];
        ts[e] = (double)fp.x + (double)fp.y;
      }
    }
    for (int s = 0; s < splits; ++s)
#pragma unroll
      for (int e = 0; e < kUnroll; ++e) {
        const int q = r0 + rg + e * kRows;
        ts[e] += part[(long long)(2 * s + 1) * ldp + (live ? line : 1) + (long long)(q < N ? q : 1) * g.ld];
      }
#pragma unroll
    for (int e = 0; e < kUnroll; ++e) {
      const int q = r0 + rg + e * kRows;
      if (live && q < N) {
        double t = ts[e];
        t += (kyh + 0.0) * (f[e] - c[e]);  // old[size-2] - old[size-1] (fr_d_t_g_2d.cpp:3478-3481)
        double om = kst * c[e];
        om += S2;
        if (dN) om += dN[line + (long long)q * g.ld];  // mass exchange
        om += st * t;
        fa[fh_sk(q)] = a[e];
        fb[fh_sk(q)] = -gi[e] * om;
        al[fh_sk(q)] = l[e];
        pf[fh_sk(q)] = qf[e];
        pb[fh_sk(q)] = qb[e];
        cf[fh_sk(q)] = f[e];
      }
    }
  }
  if (live && rg == 0) pb[fh_sk(0)] = pby[line];  // node 0: lane 0's backward chunk
  __syncthreads();
  if (warp < 4 && i0 + warp < g.sN) {
    double *wfa = sbuf + (size_t)warp * 6 * L;
    fh_line_solve_prefix(N, wfa, wfa + L, wfa + 2 * L, wfa + 3 * L, wfa + 4 * L, 1.0, 0.0, wfa + L, wfa);
  }
  __syncthreads();
  if (live) {
    for (int q = rg; q <= N + 1; q += kRows) {
      const long long id = line + (long long)q * g.ld;
      const double u = fa[fh_sk(q)];
      C[id] = u;
      if (q >= 1 && q < N) {
        const double dd = u - cf[fh_sk(q)];
        if (dfstore) {  // (hi, lo) FP32 pair, 2^-48 relative
          const float h = __double2float_rn(dd);
          reinterpret_cast<float2 *>(Dj)[id] = make_float2(h, __double2float_rn(dd - (double)h));
        } else {
          Dj[id] = dd;
        }
      }
    }
  }
}

// ---------------------------------------------------- double-float sweeps
// Blocked mode runs both half steps in double-float arithmetic on the FP32
// pipe (fh_df.cuh): fields, factor tables, history sums and far rows are
// (hi, lo) FP32 pairs, so no FP64 instruction is left in the sweeps.  Same
// structure as k_tg_xsweep / k_tg_ysweep.
//
// History right part of step j at a point: one precomputed row rb (the mid
// row of step j, or its far row, or the near sum) plus the newest nt <= 7
// layers D[j8 .. j-1] of the current 8-step sub-block weighted by
// w_j(j8 + t), which the sweeps sum themselves (k_tg_mid_tc below).
static constexpr int kSub = 8;  // steps per sub-block of the near history

__device__ __forceinline__ void tg_tiny_weights(const double *__restrict__ wt, int nt, float2 *wsm) {
  if (threadIdx.x >= 32 && threadIdx.x < 32 + nt) wsm[threadIdx.x - 32] = fh_df_pair(fh_df_from_double(wt[threadIdx.x - 32]));
}

__global__ void __launch_bounds__(kXThreads) k_tg_xsweep_df(fh_tg_dev g, float2 *Cd, float2 *__restrict__ Chd,
                                                           const float2 *__restrict__ rb,
                                                           const float2 *__restrict__ tiny, int nt,
                                                           const double *__restrict__ wt,
                                                           const float2 *__restrict__ fax,
                                                           const float2 *__restrict__ gx,
                                                           const float2 *__restrict__ alx,
                                                           const float2 *__restrict__ pfx,
                                                           const float2 *__restrict__ pbx,
                                                           const double *__restrict__ cw) {
  extern __shared__ float2 sbf[];
  const int warp = threadIdx.x >> 5;
  const int line0 = 1 + blockIdx.x * kXLines;
  const int N = g.sN;
  const int L = tg_line_stride(N);
  const int ln = threadIdx.x / kXGroup, tg = threadIdx.x % kXGroup;
  const int line = line0 + ln;
  const bool live = line < g.M;
  float2 *fa = sbf + (size_t)ln * 5 * L, *fb = fa + L, *al = fb + L, *pf = al + L, *pb = pf + L;
  const long long base = (long long)line * g.ld;
  // factor tables first; the pivot factor waits in the fb slot until the
  // right part is known
  if (live) {
    for (int i = 1 + tg; i < N; i += kXGroup) {
      const long long id = base + i;
      fa[fh_sk(i)] = fax[id];
      fb[fh_sk(i)] = gx[id];
      al[fh_sk(i)] = alx[id];
      pf[fh_sk(i)] = pfx[id];
      pb[fh_sk(i)] = pbx[id];
    }
    if (tg == 0) pb[fh_sk(0)] = pbx[base];
  }
  // step constants as double-float, split once per CTA (FP64 instructions are
  // scarce on this GPU: one per thread would stall every warp at the start)
  __shared__ float2 cst[4], wsm[kSub];
  if (threadIdx.x == 0) {
    cst[0] = fh_df_pair(fh_df_from_double(-g.st * (cw[0] + 0.0)));
    cst[1] = fh_df_pair(fh_df_from_double(g.S * 0.5));
    cst[2] = fh_df_pair(fh_df_from_double(g.st));
    cst[3] = fh_df_pair(fh_df_from_double(g.C1));
  }
  tg_tiny_weights(wt, nt, wsm);
  __syncthreads();
  const fh_df kst = fh_df_from_pair(cst[0]), S2 = fh_df_from_pair(cst[1]), st = fh_df_from_pair(cst[2]);
  for (int r0 = 1; live && r0 < N; r0 += kXGroup * kUnroll) {
    float2 c[kUnroll];
    fh_df ts[kUnroll];
#pragma unroll
    for (int e = 0; e < kUnroll; ++e) {
      const int i = r0 + tg + e * kXGroup;
      const long long id = base + (i < N ? i : 1);
      c[e] = Cd[id];
      ts[e] = rb ? fh_df_from_pair(rb[id]) : fh_df{0.f, 0.f};
    }
#pragma unroll
    for (int t = 0; t < kSub - 1; ++t)
      if (t < nt) {
        const fh_df w = fh_df_from_pair(wsm[t]);
#pragma unroll
        for (int e = 0; e < kUnroll; ++e) {
          const int i = r0 + tg + e * kXGroup;
          ts[e] = fh_df_fma(w, fh_df_from_pair(tiny[(long long)t * g.P + base + (i < N ? i : 1)]), ts[e]);
        }
      }
#pragma unroll
    for (int e = 0; e < kUnroll; ++e) {
      const int i = r0 + tg + e * kXGroup;
      if (i < N) {
        fh_df om = fh_df_fma(kst, fh_df_from_pair(c[e]), S2);
        om = fh_df_fma(st, ts[e], om);
        fb[fh_sk(i)] = fh_df_pair(fh_df_neg(fh_df_mul(fh_df_from_pair(fb[fh_sk(i)]), om)));
      }
    }
  }
  __syncthreads();
  if (warp < kXLines && line0 + warp < g.M) {
    float2 *fa = sbf + (size_t)warp * 5 * L;
    fh_line_solve_prefix_df(N, fa, fa + L, fa + 2 * L, fa + 3 * L, fa + 4 * L, fh_df{0.f, 0.f},
                            fh_df_from_pair(cst[3]), fa + L, fa);
  }
  __syncthreads();
  {
    const int ln = threadIdx.x / kXGroup, tg = threadIdx.x % kXGroup;
    const int line = line0 + ln;
    const float2 *u = sbf + (size_t)ln * 5 * L;
    const long long base = (long long)line * g.ld;
    for (int i = tg; line < g.M && i <= N + 1; i += kXGroup) {
      const float2 v = u[fh_sk(i)];
      Chd[base + i] = v;
      if (i == 0 || i >= N) Cd[base + i] = v;
    }
  }
}

__global__ void __launch_bounds__(kYThreads) k_tg_ysweep_df(fh_tg_dev g, float2 *Cd, const float2 *__restrict__ Chd,
                                                           float2 *__restrict__ Dj, const float2 *__restrict__ rb,
                                                           const float2 *__restrict__ tiny, int nt,
                                                           const double *__restrict__ wt,
                                                           const float2 *__restrict__ fay,
                                                           const float2 *__restrict__ gy,
                                                           const float2 *__restrict__ aly,
                                                           const float2 *__restrict__ pfy,
                                                           const float2 *__restrict__ pby,
                                                           const double *__restrict__ cw) {
  extern __shared__ float2 sbf[];
  const int warp = threadIdx.x >> 5;
  const int N = g.M;
  const int L = tg_line_stride(N);
  const int i0 = 1 + blockIdx.x * 4;
  const int col = threadIdx.x & 3;
  const int rg = threadIdx.x >> 2;  // row group 0..127
  constexpr int kRows = kYThreads / 4;
  const int line = i0 + col;
  const bool live = line < g.sN;
  float2 *fa = sbf + (size_t)col * 6 * L, *fb = fa + L, *al = fb + L, *pf = al + L, *pb = pf + L, *cf = pb + L;
  // factor tables first; the pivot factor waits in the fb slot (see k_tg_xsweep_df)
  if (live) {
    for (int q = 1 + rg; q < N; q += kRows) {
      const long long id = line + (long long)q * g.ld;
      fa[fh_sk(q)] = fay[id];
      fb[fh_sk(q)] = gy[id];
      al[fh_sk(q)] = aly[id];
      pf[fh_sk(q)] = pfy[id];
      pb[fh_sk(q)] = pby[id];
    }
  }
  __shared__ float2 cst[4], wsm[kSub];  // step constants, split once per CTA (see k_tg_xsweep_df)
  if (threadIdx.x == 0) {
    cst[0] = fh_df_pair(fh_df_from_double(-g.st * (cw[1] + 0.0)));
    cst[1] = fh_df_pair(fh_df_from_double(cw[2] + 0.0));
    cst[2] = fh_df_pair(fh_df_from_double(g.S * 0.5));
    cst[3] = fh_df_pair(fh_df_from_double(g.st));
  }
  tg_tiny_weights(wt, nt, wsm);
  __syncthreads();
  const fh_df kst = fh_df_from_pair(cst[0]), kyh = fh_df_from_pair(cst[1]), S2 = fh_df_from_pair(cst[2]),
              st = fh_df_from_pair(cst[3]);
  for (int r0 = 1; live && r0 < N; r0 += kRows * kUnroll) {
    float2 c[kUnroll], f[kUnroll];
    fh_df ts[kUnroll];
#pragma unroll
    for (int e = 0; e < kUnroll; ++e) {
      const int q = r0 + rg + e * kRows;
      const long long id = line + (long long)(q < N ? q : 1) * g.ld;
      c[e] = Chd[id];
      f[e] = Cd[id];
      ts[e] = rb ? fh_df_from_pair(rb[id]) : fh_df{0.f, 0.f};
    }
#pragma unroll
    for (int t = 0; t < kSub - 1; ++t)
      if (t < nt) {
        const fh_df w = fh_df_from_pair(wsm[t]);
#pragma unroll
        for (int e = 0; e < kUnroll; ++e) {
          const int q = r0 + rg + e * kRows;
          ts[e] = fh_df_fma(w, fh_df_from_pair(tiny[(long long)t * g.P + line + (long long)(q < N ? q : 1) * g.ld]),
                            ts[e]);
        }
      }
#pragma unroll
    for (int e = 0; e < kUnroll; ++e) {
      const int q = r0 + rg + e * kRows;
      if (q < N) {
        const fh_df cc = fh_df_from_pair(c[e]);
        // old[size-2] - old[size-1] (fr_d_t_g_2d.cpp:3478-3481)
        const fh_df t = fh_df_fma(kyh, fh_df_sub(fh_df_from_pair(f[e]), cc), ts[e]);
        fh_df om = fh_df_fma(kst, cc, S2);
        om = fh_df_fma(st, t, om);
        fb[fh_sk(q)] = fh_df_pair(fh_df_neg(fh_df_mul(fh_df_from_pair(fb[fh_sk(q)]), om)));
        cf[fh_sk(q)] = f[e];
      }
    }
  }
  if (live && rg == 0) pb[fh_sk(0)] = pby[line];  // node 0: lane 0's backward chunk
  __syncthreads();
  if (warp < 4 && i0 + warp < g.sN) {
    float2 *wfa = sbf + (size_t)warp * 6 * L;
    fh_line_solve_prefix_df(N, wfa, wfa + L, wfa + 2 * L, wfa + 3 * L, wfa + 4 * L, fh_df{1.f, 0.f},
                            fh_df{0.f, 0.f}, wfa + L, wfa);
  }
  __syncthreads();
  if (live) {
    for (int q = rg; q <= N + 1; q += kRows) {
      const long long id = line + (long long)q * g.ld;
      const float2 u = fa[fh_sk(q)];
      Cd[id] = u;
      if (q >= 1 && q < N) Dj[id] = fh_df_pair(fh_df_sub(fh_df_from_pair(u), fh_df_from_pair(cf[fh_sk(q)])));
    }
  }
}


// ------------------------------------------------ mid rows on the tensor cores
// Blocked mode, per-solve weight table: the mid rows of sub-block jb over the
// block's layers [j0, jb) (K = jb - j0 <= 56) as exact bf16-slice products on
// the tensor cores, like the far rows, with five slices per value (a value is
// kept to 2^-40 of its point's or row's maximum) and one exponent per point
// for all K layers.  Per CTA: A = 128 points x 64 layers in five K-major
// planes that the CTA slices itself from the double-float layers; B = the
// sub-block's weight slices stacked as 80 rows (slice ib, row n at 16 ib + n,
// n = 2r + m: x and y rows of step jb + r).  The MMA of data slice ia takes
// the first (5 - ia) * 16 rows of B and writes TMEM columns 16 ia .. 79, so
// the product (ia, ib) lands on the columns 16 (ia + ib) of its level: the
// tensor cores form every product of level <= 4 (15 of 25) with five MMAs
// per 16 layers and add up each level in the FP32 accumulator.  Slices are
// integers of magnitude <= 192 (data) and <= 128 (weights), so a level sum
// (<= 5 products per layer, K <= 64 layers) is an integer below 2^24: exact.
// The epilogue turns the five level sums into a double-float value, scales
// it by 2^(Ed + Ew) and adds the base row (far rows of the block).
constexpr int kMtSl = 5;                           // slices per value
constexpr int kMtRows = 2 * kSub;                  // x and y rows of 8 steps
constexpr uint32_t kMtTileA = 128 * 128;           // 128 points x 64 layers bf16
constexpr uint32_t kMtTileB = kMtRows * 128;       // 16 rows x 64 layers bf16
constexpr uint32_t kMtWBytes = kMtSl * kMtTileB;   // one sub-block's weight slices (10 KiB)
constexpr size_t kMtSmem = 1024 + kMtSl * kMtTileA + kMtWBytes + 64;
constexpr uint32_t kMtTmemCols = 128;              // levels 0..4 x 16 rows = 80 used

// Weight slices of every sub-block's mid rows: CTA sb slices the rows of
// steps 8 sb .. 8 sb + 7 over the layers [j0, 8 sb) of their block (W: the
// per-solve table, x row then y row per step, pitch ldw) into the stacked
// layout above (ws + sb * kMtWBytes) and the row exponents we[16 sb + n].
// Eight threads per row, eight layers each; FP64 slicing (a0 .. a4 of
// w 2^-E, E from the row's largest |w|).
__global__ void __launch_bounds__(128) k_tg_mid_wslice(const double *__restrict__ W, int ldw, int max_steps,
                                                       uint8_t *__restrict__ ws, int8_t *__restrict__ we) {
  const int sb = blockIdx.x, jb = sb * kSub, j0 = (jb / kTgBlock) * kTgBlock, K = jb - j0;
  const int nr = min(kSub, max_steps - jb);
  const int n = threadIdx.x >> 3, c = threadIdx.x & 7;  // row, 8-layer chunk
  const int r = n >> 1, m = n & 1;
  double w[8];
  double mx = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int k = 8 * c + i;
    w[i] = (r < nr && k < K) ? W[(long long)(jb + r) * 2 * ldw + (long long)m * ldw + j0 + k] : 0.0;
    mx = fmax(mx, fabs(w[i]));
  }
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const int E = fh_chunk_exp(mx);
  uint32_t pk[kMtSl][4];
#pragma unroll
  for (int i = 0; i < 8; i += 2) {
    double x0 = ldexp(w[i], -E), x1 = ldexp(w[i + 1], -E);
#pragma unroll
    for (int q = 0; q < kMtSl; ++q) {
      const double a0 = rint(x0), a1 = rint(x1);
      __nv_bfloat162 b2;
      b2.x = __double2bfloat16(a0);
      b2.y = __double2bfloat16(a1);
      pk[q][i >> 1] = *reinterpret_cast<const uint32_t *>(&b2);
      x0 = (x0 - a0) * 256.0;
      x1 = (x1 - a1) * 256.0;
    }
  }
  uint8_t *dst = ws + (size_t)sb * kMtWBytes;
#pragma unroll
  for (int q = 0; q < kMtSl; ++q)
    *reinterpret_cast<uint4 *>(dst + q * kMtTileB + fh_sw128_off(n, 8 * c)) =
        make_uint4(pk[q][0], pk[q][1], pk[q][2], pk[q][3]);
  if (c == 0) we[(size_t)sb * kMtRows + n] = (int8_t)E;
}

// Slices a0..a4 of a double-float value (hi, lo) scaled by 2^-E (|scaled| <
// 2^7), as bf16 bit patterns in the high halves of floats: a0..a2 come from
// hi alone (its 24 bits end at slice 2's scale), then the low word joins
// (the one FP32 add drops bits below 2^-47 of the point's maximum).  Each a_i
// is an integer of magnitude <= 192 (a3 takes the low word's share), so its
// float's high half is its exact bf16 pattern.
__device__ __forceinline__ void mt_slice5(float hi, float lo, float scale, float (&a)[kMtSl]) {
  float r = hi * scale;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    a[i] = rintf(r);
    r = (r - a[i]) * 256.0f;  // exact
  }
  r = fmaf(lo * scale, 16777216.0f, r);
  a[3] = rintf(r);
  r = (r - a[3]) * 256.0f;
  a[4] = rintf(r);
}

// Mid rows of one sub-block: out[n][p] = base[n][p] + sum_{k < K} w_n(k) D[k][p]
// for the nr * 2 rows n of the sub-block (weights ws / we from
// k_tg_mid_wslice), 128 points per CTA, two threads per point (layers
// [32 h, 32 h + 32) of the point for thread half h); KS = ceil(K/16).  Warp w
// reads TMEM lanes 32 (w % 4) .. + 31 and rows 8 (w / 4) .. + 7 in the
// epilogue.  The MMA completion wait is bounded; on expiry the CTA stores
// nothing and sets *err.
template <int KS>
__global__ void __launch_bounds__(256, 2) k_tg_mid_tc(const float2 *__restrict__ D, long long P, int K,
                                                  const uint8_t *__restrict__ ws, const int8_t *__restrict__ we,
                                                  int nr, const float2 *__restrict__ base, long long ldbase,
                                                  float2 *__restrict__ out, long long ldo, int *__restrict__ err) {
  extern __shared__ uint8_t mt_raw[];
  __shared__ float mxs[2][128];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int pt = tid & 127, h = tid >> 7;
  const long long p = (long long)blockIdx.x * 128 + pt;
  // the point's layers first (the longest latency), then this warp's base rows
  constexpr int KH = KS >= 2 ? 32 : 16;  // layers per thread half
  const int k0 = KH * h;
  const bool mine = 16 * KS > k0;        // this half holds layers of the tile
  float hi[KH], lo[KH];
#pragma unroll
  for (int i = 0; i < KH; ++i) {
    float2 v = make_float2(0.f, 0.f);
    if (mine && k0 + i < K && p < P) v = __ldcs(D + (long long)(k0 + i) * P + p);
    hi[i] = v.x;
    lo[i] = v.y;
  }
  const int r0 = 8 * (warp >> 2);  // epilogue rows of this warp
  float2 bv[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
    bv[i] = (base && p < P && ((r0 + i) >> 1) < nr) ? __ldcs(base + (long long)(r0 + i) * ldbase + p)
                                                    : make_float2(0.f, 0.f);
  const uint32_t raw = fh_smem_u32(mt_raw);
  const uint32_t sA = (raw + 1023u) & ~1023u;
  uint8_t *gA = mt_raw + (sA - raw);
  const uint32_t sB = sA + kMtSl * kMtTileA;
  uint8_t *gB = gA + kMtSl * kMtTileA;
  const uint32_t bar = sB + kMtWBytes, tslot = bar + 8;
  volatile uint32_t *tslot_g = reinterpret_cast<volatile uint32_t *>(gB + kMtWBytes + 8);
  if (tid == 0) {
    fh_mbar_init(bar, 1);
    fh_fence_mbar_init();
  }
  if (warp == 0) {
    fh_tmem_alloc(tslot, kMtTmemCols);
    fh_tmem_relinquish();
  }
  const uint4 *wsrc = reinterpret_cast<const uint4 *>(ws);
  for (int i = tid; i < (int)(kMtWBytes / 16); i += 256) reinterpret_cast<uint4 *>(gB)[i] = __ldg(wsrc + i);
  float mx = 0.f;
#pragma unroll
  for (int i = 0; i < KH; ++i) mx = fmaxf(mx, fabsf(hi[i]));
  mxs[h][pt] = mx;
  __syncthreads();
  const int E = fh_point_exp(fmaxf(mxs[0][pt], mxs[1][pt]));
  if (mine) {
    const float scale = fh_exp2f_int(-E);  // -E <= 107
#pragma unroll
    for (int c = 0; c < KH / 8; ++c) {
      uint32_t pk[kMtSl][4];
#pragma unroll
      for (int i = 0; i < 8; i += 2) {
        float a0[kMtSl], a1[kMtSl];
        mt_slice5(hi[8 * c + i], lo[8 * c + i], scale, a0);
        mt_slice5(hi[8 * c + i + 1], lo[8 * c + i + 1], scale, a1);
#pragma unroll
        for (int q = 0; q < kMtSl; ++q)
          pk[q][i >> 1] = __byte_perm(__float_as_uint(a0[q]), __float_as_uint(a1[q]), 0x7632);
      }
      const uint32_t off = fh_sw128_off(pt, k0 + 8 * c);
#pragma unroll
      for (int q = 0; q < kMtSl; ++q)
        *reinterpret_cast<uint4 *>(gA + q * kMtTileA + off) = make_uint4(pk[q][0], pk[q][1], pk[q][2], pk[q][3]);
    }
  }
  fh_fence_proxy_async_smem();
  fh_tc_fence_before();
  __syncthreads();
  fh_tc_fence_after();
  const uint32_t tmem = *tslot_g;
  if (tid == 0) {
#pragma unroll
    for (int ia = 0; ia < kMtSl; ++ia) {
      const uint32_t idesc = fh_idesc_bf16_f32(128, (kMtSl - ia) * kMtRows);
#pragma unroll
      for (int kk = 0; kk < KS; ++kk)
        fh_mma_bf16(tmem + (uint32_t)(kMtRows * ia), fh_desc_kmajor_sw128(sA + ia * kMtTileA + kk * 32),
                    fh_desc_kmajor_sw128(sB + kk * 32), idesc, (ia > 0 || kk > 0) ? 1u : 0u);
    }
    fh_mma_commit(bar);
  }
  __syncwarp();  // lanes 1..31 of warp 0 must not spin in the wait while lane 0 issues
  // bounded wait for the MMAs, sleeping between polls (the other CTA on the SM keeps the issue slots)
  bool done = false;
  {
    const uint64_t t0 = fh_globaltimer();
    for (;;) {
      uint32_t d;
      asm volatile(
          "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], 0;\n selp.u32 %0, 1, 0, q;\n}\n"
          : "=r"(d)
          : "r"(bar)
          : "memory");
      if (d) {
        done = true;
        break;
      }
      if (fh_globaltimer() - t0 > FH_WAIT_NS) break;
      __nanosleep(200);
    }
  }
  const bool ok = __all_sync(0xffffffffu, done);
  fh_tc_fence_after();
  // level sums of rows r0 .. r0 + 7 (TMEM lane 32 (warp % 4) + lane is this thread's point)
  const uint32_t lanes = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)r0;
  float L[kMtSl][8];
#pragma unroll
  for (int l = 0; l < kMtSl; ++l) fh_tmem_ld8(lanes + (uint32_t)(kMtRows * l), L[l]);
  fh_tmem_wait_ld();
  if (ok && p < P) {
    const uint2 ev = __ldg(reinterpret_cast<const uint2 *>(we + r0));
    const uint32_t ew32[2] = {ev.x, ev.y};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int n = r0 + i;
      if ((n >> 1) >= nr) continue;
      // T = L0 + L1/2^8 + L2/2^16 + L3/2^24 + L4/2^32 as (th, tl)
      const float x1 = L[1][i] * 0.00390625f;
      float th = L[0][i] + x1;
      const float bb = th - L[0][i];
      float tl = (L[0][i] - (th - bb)) + (x1 - bb);
      tl += L[2][i] * 1.52587890625e-05f;
      const float tr = th + tl;
      tl = tl - (tr - th);
      th = tr;
      tl += L[3][i] * 5.9604644775390625e-08f + L[4][i] * 2.3283064365386963e-10f;
      const float sc = fh_exp2i(E + (int)(int8_t)(ew32[i >> 2] >> (8 * (i & 3))));
      const float vh = th * sc, vl = tl * sc;
      const float2 b = bv[i];
      const float s2 = b.x + vh;
      const float bs = s2 - b.x;
      const float e = ((b.x - (s2 - bs)) + (vh - bs)) + (b.y + vl);
      const float hh = s2 + e;
      out[(long long)n * ldo + p] = make_float2(hh, e - (hh - s2));
    }
  }
  fh_tc_fence_before();
  __syncthreads();
  if (warp == 0) fh_tmem_dealloc(tmem, kMtTmemCols);
  if (!ok && (tid & 31) == 0) atomicOr(err, 1);
}

// ------------------------------------------------ fused sub-block sweeps
// One cooperative launch runs both half steps of up to kSub consecutive steps
// of one sub-block.  Every CTA owns four x lines and four y columns; the
// fixed factor tables of both (fa, al in the solve layout, g in the node
// layout; 96 KiB) stay in shared memory for the whole launch.  The half
// steps are separated by grid barriers (every CTA is resident: one CTA per
// SM, launched cooperatively); data written by other CTAs within the launch
// is read through L2 (ld.global.cg), never from L1.  Each barrier wait is
// bounded by FH_WAIT_NS of %globaltimer: on expiry the CTA sets *err and
// returns (the other CTAs then time out at their next barrier).
//
// Two thread mappings per half step:
//  * node mapping (coalesced global traffic): thread tid holds node 1 + tid of
//    each x line (k = line), or row 1 + tid/4 + 128 k of column tid % 4 (the
//    four columns of a row are adjacent in memory); it loads the fields and
//    history layers, keeps the history partial sums of its nodes in
//    registers, forms the right parts -g om and stores the results;
//  * solve mapping: the 128 threads of group l (warps 4l..4l+3) solve line l,
//    thread t the equations 1 + 4t .. 4 + 4t, exchanging right parts and
//    solutions with the node mapping through shared memory.
// The grid barriers are split: a CTA arrives when its results are stored and
// computes the history partial sums of the next half step (one round trip of
// loads) before it waits, so those loads overlap the barrier.  Arithmetic per
// node as in
// k_tg_xsweep_df / k_tg_ysweep_df (double-float).
static constexpr int kFuseGroup = 128;                        // threads per line (four warps)
static constexpr int kFuseEq = 4;                             // equations per solving thread
static constexpr int kFuseLines = 4;                          // x lines and y columns per CTA
static constexpr int kFuseThreads = kFuseGroup * kFuseLines;  // 512
static constexpr int kFuseMaxN = kFuseGroup * kFuseEq + 1;    // lines of at most 513 nodes
static constexpr int kFuseSE = kFuseGroup + 4;                // solve-layout stride of one equation slot
static constexpr int kFuseSL = kFuseEq * kFuseSE;             // solve-layout slots per line
static constexpr int kFuseNL = kFuseMaxN - 1;                 // node-layout slots per line (nodes 1..512)
static constexpr int kBarWarp = kFuseThreads / 32 - 1;

struct tg_fuse_args {
  fh_tg_dev g;
  float2 *Cd, *Chd, *D;  // D: history layers (pairs), layer k at D + k P
  const float2 *fax, *gx, *alx, *fay, *gy, *aly;
  const double *W;       // per-solve weight table, row j at W + 2 j ldw
  const double *cwall;   // current weights, 4 per step
  const float2 *rb0;     // history row of step j8 + s: x at rb0 + s rb_step, y at + rb_xy (null: none)
  long long rb_step, rb_xy;
  int ldw, j8, s0, ns;   // steps j8 + s0 .. j8 + s0 + ns - 1
  unsigned *bar;
  int *err;
};

// Per-thread shared-memory state of the y mapping ([slot][k][thread], each
// thread reads only its own entries): the sub-block layers it produced in
// this launch (ycache, the first kYCache of them) and the history row of the
// current step's y sums, prefetched by cp.async at the start of the step
// (ypre).  The field at its y nodes stays in registers across the steps.
static constexpr int kYCache = 5;
// dynamic shared memory: fa, al (solve layout) and g (node layout) of both
// directions, the right-part / solution exchange of four lines, then
// ycache, ypre
static constexpr size_t kFuseSmem =
    sizeof(float2) * (2 * 2 * kFuseLines * (size_t)kFuseSL + 2 * kFuseLines * (size_t)kFuseNL +
                      kFuseLines * (size_t)kFuseSL + (size_t)(kYCache + 1) * kFuseLines * kFuseThreads);

// solve-layout slot of equation i (1 <= i <= 512): thread (i-1)/4, entry (i-1)%4
__device__ __forceinline__ int tg_fslot(int i) { return ((i - 1) & 3) * kFuseSE + ((i - 1) >> 2); }

__device__ __forceinline__ void tg_grid_arrive(unsigned *bar) {
  __syncthreads();  // every store of the CTA precedes the release
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
  }
}

// Waits until the barrier counter reaches `target` (warp kBarWarp polls, lane 0
// loading and broadcasting the count); false (and *err set) on expiry.
__device__ __forceinline__ bool tg_grid_wait(const unsigned *bar, unsigned target, int *err) {
  __shared__ int gs_ok;
  if ((threadIdx.x >> 5) == kBarWarp) {
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t deadline = fh_globaltimer() + FH_WAIT_NS;
    int ok = 1;
    for (unsigned it = 0;; ++it) {
      int st = 0;
      if (lane == 0) {
        unsigned v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
        // the deadline and the error flag are checked every 64 polls
        st = v >= target ? 1 : (((it & 63u) == 63u && (*(volatile int *)err || fh_globaltimer() > deadline)) ? 2 : 0);
      }
      st = __shfl_sync(0xffffffffu, st, 0);
      if (st == 1) break;
      if (st == 2) {
        ok = 0;
        if (lane == 0) atomicOr(err, 1);
        break;
      }
      if (it >= 2048u) __nanosleep(64);  // tight polling first: a barrier usually completes within ~2 us
    }
    if (lane == 0) gs_ok = ok;
    __syncwarp();
  }
  __syncthreads();
  return gs_ok != 0;
}

// Phase stamps of the fused sweeps for profiling builds (-DFH_TG_STAMPS):
// %clock64 of every phase boundary of every step, taken by warp kBarWarp,
// read with fh_tg_stamps_read.  Empty otherwise.
#ifdef FH_TG_STAMPS
constexpr int kTgStamps = 12;  // stamps per step
__device__ long long g_tg_stamps[256 * kSub * kTgStamps];
#define TG_STAMP(p)                                                                   \
  if (warp == kBarWarp) {                                                             \
    const long long c_ = clock64();                                                   \
    if ((threadIdx.x & 31) == 0) g_tg_stamps[(blockIdx.x * kSub + s) * kTgStamps + (p)] = c_; \
    __syncwarp();                                                                     \
  }
extern "C" int fh_tg_stamps_read(long long *h) {
  return (int)cudaMemcpyFromSymbol(h, g_tg_stamps, sizeof(g_tg_stamps));
}
#else
#define TG_STAMP(p)
#endif

// Exclusive scan of the chunk maps of one line's 128 threads (four warps,
// named barrier `bar`, warp totals in sm[4]): forward, thread t receives
// f_{t-1} o ... o f_0; reverse, G_{t+1} o ... o G_127.
template <bool REV>
__device__ __forceinline__ fh_daff tg_group_scan(fh_daff f, fh_daff *sm, int bar, int w4) {
  const unsigned lane = threadIdx.x & 31u;
  fh_daff g = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    if (!REV) {
      const fh_daff p{fh_df_shfl_up(g.a, d), fh_df_shfl_up(g.b, d)};
      if (lane >= (unsigned)d) g = fh_daff_compose(g, p);
    } else {
      const fh_daff p{fh_df_shfl_down(g.a, d), fh_df_shfl_down(g.b, d)};
      if (lane + d < 32u) g = fh_daff_compose(g, p);
    }
  }
  const fh_daff id{fh_df{1.f, 0.f}, fh_df{0.f, 0.f}};
  fh_daff e;
  if (!REV) {
    if (lane == 31u) sm[w4] = g;
    e = fh_daff{fh_df_shfl_up(g.a, 1), fh_df_shfl_up(g.b, 1)};
    if (lane == 0u) e = id;
  } else {
    if (lane == 0u) sm[w4] = g;
    e = fh_daff{fh_df_shfl_down(g.a, 1), fh_df_shfl_down(g.b, 1)};
    if (lane == 31u) e = id;
  }
  fh_group_bar(bar, kFuseGroup);
  fh_daff P = id;
  if (!REV)
    for (int k = 0; k < w4; ++k) P = fh_daff_compose(sm[k], P);
  else
    for (int k = 3; k > w4; --k) P = fh_daff_compose(sm[k], P);
  fh_group_bar(bar, kFuseGroup);  // sm may be reused after this
  return fh_daff_compose(e, P);
}

// One line of N nodes by the 128 threads of its group: Thomas in the
// reference form from the fixed factors, u_i = al_i u_{i+1} + bt_i with
// bt_i = fa_i bt_{i-1} + fb_i, bt_0 = bt1, al_0 = al1, u_N = u_{N+1} =
// bt_{N-1} / (1 - al_{N-1}).  Each thread walks its four equations from zero
// (keeping the prefix slope products), the chunk maps are scanned across the
// group, and the start value finishes each chunk.  fb (solve layout) is
// replaced by u; ub receives u_0 and u_N.
__device__ __forceinline__ void tg_group_solve(int N, const float2 *fa, const float2 *al, float2 *xch, float2 *ub,
                                               fh_df al1, fh_df bt1, fh_daff *sm, fh_df *uNs, int bar, int t, int w4) {
  const fh_df one{1.f, 0.f}, zero{0.f, 0.f};
  fh_df B[kFuseEq], P[kFuseEq];
  fh_df b = zero, p = one;
#pragma unroll
  for (int e = 0; e < kFuseEq; ++e) {
    const int i = 1 + kFuseEq * t + e;
    if (i < N) {
      const int sl = e * kFuseSE + t;
      const fh_df f = fh_df_from_pair(fa[sl]);
      b = fh_df_fma(f, b, fh_df_from_pair(xch[sl]));
      p = fh_df_mul(p, f);
    }
    B[e] = b;
    P[e] = p;
  }
  const fh_daff Pf = tg_group_scan<false>(fh_daff{p, b}, sm, bar, w4);
  const fh_df s = fh_df_fma(Pf.a, bt1, Pf.b);  // bt at equation 4t (bt1 for t = 0)
  fh_df bt[kFuseEq];
#pragma unroll
  for (int e = 0; e < kFuseEq; ++e) bt[e] = fh_df_fma(P[e], s, B[e]);
  // u_N from the thread of equation N - 1
  {
    const int e = (N - 2) - kFuseEq * t;
    if (e >= 0 && e < kFuseEq) {
      const fh_df aN = fh_df_from_pair(al[e * kFuseSE + t]);
      *uNs = fh_df_div(bt[e], fh_df_sub(one, aN));
    }
  }
  fh_group_bar(bar, kFuseGroup);
  const fh_df uN = *uNs;
  fh_df V[kFuseEq], Q[kFuseEq];
  fh_df v = zero, q = one;
#pragma unroll
  for (int e = kFuseEq - 1; e >= 0; --e) {
    const int i = 1 + kFuseEq * t + e;
    if (i < N) {
      const fh_df a = fh_df_from_pair(al[e * kFuseSE + t]);
      v = fh_df_fma(a, v, bt[e]);
      q = fh_df_mul(q, a);
    }
    V[e] = v;
    Q[e] = q;
  }
  const fh_daff Pb = tg_group_scan<true>(fh_daff{q, v}, sm, bar, w4);
  const fh_df u1 = fh_df_fma(Pb.a, uN, Pb.b);  // u at equation 4t + 5 (u_N past the last chunk)
#pragma unroll
  for (int e = 0; e < kFuseEq; ++e) {
    const int i = 1 + kFuseEq * t + e;
    if (i < N) xch[e * kFuseSE + t] = fh_df_pair(fh_df_fma(Q[e], u1, V[e]));
  }
  if (t == 0) {
    const fh_df u0 = fh_df_fma(al1, fh_df_fma(Q[0], u1, V[0]), bt1);
    ub[0] = fh_df_pair(u0);
    ub[1] = fh_df_pair(uN);
  }
}

__global__ void __launch_bounds__(kFuseThreads, 1) k_tg_sweeps_fused(const tg_fuse_args a) {
  extern __shared__ float2 sbf[];
  // cx/cy: step constants; wx/wy[s][t]: weight of layer j8 + t in step j8 + s
  __shared__ float2 cx[kSub][4], cy[kSub][4], wx[kSub][kSub], wy[kSub][kSub];
  __shared__ fh_daff scan_sm[kFuseLines][4];
  __shared__ fh_df uN_sm[kFuseLines];
  __shared__ float2 ub_sm[kFuseLines][2];
  const fh_tg_dev &g = a.g;
  const int Nx = g.sN, Ny = g.M;
  const int tid = threadIdx.x;
  [[maybe_unused]] const int warp = tid >> 5;  // read by the phase stamps of profiling builds
  float2 *fa_x = sbf, *al_x = fa_x + kFuseLines * kFuseSL;  // solve layout, [line][slot]
  float2 *fa_y = al_x + kFuseLines * kFuseSL, *al_y = fa_y + kFuseLines * kFuseSL;
  float2 *g_x = al_y + kFuseLines * kFuseSL, *g_y = g_x + kFuseLines * kFuseNL;  // node layout, [line][i-1]
  float2 *xch = g_y + kFuseLines * kFuseNL;       // [line][slot]: -g om, then u
  float2 *ycache = xch + kFuseLines * kFuseSL;    // [layer][k][thread]
  float2 *ypre = ycache + kYCache * kFuseLines * kFuseThreads;
  auto ys = [&](float2 *base, int k) -> float2 & { return base[k * kFuseThreads + tid]; };
  // lines line0 .. line0 + 3 (rows j of the x sweep, columns i of the y sweep),
  // aligned to four so that a row of the CTA's columns is one 32-byte sector;
  // line 0 (a boundary) is not solved
  const int line0 = kFuseLines * blockIdx.x;
  auto xl_ok = [&](int l) { return line0 + l >= 1 && line0 + l < g.M; };
  auto yl_ok = [&](int l) { return line0 + l >= 1 && line0 + l < g.sN; };
  // fixed factor tables: every load of the thread issued at once (the
  // launch's first step waits for them); x rows coalesced along the row, y
  // columns with four adjacent columns (one 32-byte sector) per four threads
  {
    constexpr int kIt = kFuseLines * kFuseNL / kFuseThreads;
    float2 vx[kIt][3], vy[kIt][3];
#pragma unroll
    for (int u = 0; u < kIt; ++u) {
      const int v = tid + u * kFuseThreads;
      const int lx = v / kFuseNL, ix = 1 + v % kFuseNL;
      const int ly = v % kFuseLines, iy = 1 + v / kFuseLines;
      const float2 z = make_float2(0.f, 0.f);
      const bool okx = xl_ok(lx) && ix < Nx, oky = yl_ok(ly) && iy < Ny;
      const long long idx = (long long)(line0 + lx) * g.ld + ix;
      const long long idy = line0 + ly + (long long)iy * g.ld;
      vx[u][0] = okx ? __ldg(a.fax + idx) : z;
      vx[u][1] = okx ? __ldg(a.alx + idx) : z;
      vx[u][2] = okx ? __ldg(a.gx + idx) : z;
      vy[u][0] = oky ? __ldg(a.fay + idy) : z;
      vy[u][1] = oky ? __ldg(a.aly + idy) : z;
      vy[u][2] = oky ? __ldg(a.gy + idy) : z;
    }
#pragma unroll
    for (int u = 0; u < kIt; ++u) {
      const int v = tid + u * kFuseThreads;
      const int lx = v / kFuseNL, ix = 1 + v % kFuseNL;
      const int ly = v % kFuseLines, iy = 1 + v / kFuseLines;
      if (xl_ok(lx) && ix < Nx) {
        fa_x[lx * kFuseSL + tg_fslot(ix)] = vx[u][0];
        al_x[lx * kFuseSL + tg_fslot(ix)] = vx[u][1];
        g_x[lx * kFuseNL + ix - 1] = vx[u][2];
      }
      if (yl_ok(ly) && iy < Ny) {
        fa_y[ly * kFuseSL + tg_fslot(iy)] = vy[u][0];
        al_y[ly * kFuseSL + tg_fslot(iy)] = vy[u][1];
        g_y[ly * kFuseNL + iy - 1] = vy[u][2];
      }
    }
  }
  // double-float step constants and sub-block weights, one FP64 conversion per thread
  constexpr int kPer = 8 + 2 * kSub;
  for (int v = tid; v < a.ns * kPer; v += blockDim.x) {
    const int s = a.s0 + v / kPer, r = v % kPer;
    const int j = a.j8 + s;
    const double *cw = a.cwall + 4LL * j;
    const double *Wj = a.W + (long long)j * 2 * a.ldw + a.j8;
    double val;
    float2 *dst;
    if (r < 4) {
      dst = &cx[s][r];
      val = r == 0 ? -g.st * (cw[0] + 0.0) : r == 1 ? g.S * 0.5 : r == 2 ? g.st : g.C1;
    } else if (r < 8) {
      dst = &cy[s][r - 4];
      val = r == 4 ? -g.st * (cw[1] + 0.0) : r == 5 ? cw[2] + 0.0 : r == 6 ? g.S * 0.5 : g.st;
    } else if (r < 8 + kSub) {
      dst = &wx[s][r - 8];
      val = (r - 8) < s ? Wj[r - 8] : 0.0;
    } else {
      dst = &wy[s][r - 8 - kSub];
      val = (r - 8 - kSub) < s ? Wj[a.ldw + (r - 8 - kSub)] : 0.0;
    }
    *dst = fh_df_pair(fh_df_from_double(val));
  }
  __syncthreads();

  // node mapping: x node 1 + tid of line k; y row 1 + tid/4 + 128 k of column tid % 4
  const int xi = 1 + tid;
  const int yc = tid & 3, yq0 = 1 + (tid >> 2);
  const bool ycol_live = yl_ok(yc);
  auto xlive = [&](int k) { return xl_ok(k) && xi < Nx; };
  auto xid = [&](int k) { return (long long)(line0 + k) * g.ld + xi; };
  auto yq = [&](int k) { return yq0 + 128 * k; };
  auto ylive = [&](int k) { return ycol_live && yq(k) < Ny; };
  auto yid = [&](int k) { return (long long)(line0 + yc) + (long long)yq(k) * g.ld; };
  // solve mapping
  const int grp = tid / kFuseGroup, gt = tid % kFuseGroup, w4 = gt >> 5;
  const float2 *tiny = a.D + (long long)a.j8 * g.P;  // layers of the sub-block
  const unsigned nblk = gridDim.x;
  unsigned nb = 0;

  fh_df tsx[kFuseLines], tsy[kFuseLines];  // history parts of the thread's x / y nodes
  float2 f[kFuseLines];                    // old field at the thread's y nodes
  // x history part of step s without its newest layer: row + sum_{t < s-1} w(t) D[j8 + t]
  // history part of step s at the thread's x nodes without the newest layer,
  // row + sum_{t < s-1} w(t) D[j8 + t], and at its y nodes, row + sum_{t < s}
  // w(t) D[j8 + t], with the old field there: every load of a part is issued
  // at once (*_load), then summed (*_sum).
  auto x_load = [&](int s, float2 (&r)[kFuseLines], float2 (&d)[kSub - 1][kFuseLines]) {
    const float2 *rbx = a.rb0 ? a.rb0 + (long long)s * a.rb_step : nullptr;
#pragma unroll
    for (int k = 0; k < kFuseLines; ++k) r[k] = (rbx && xlive(k)) ? __ldcg(rbx + xid(k)) : make_float2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < kSub - 1; ++t)
#pragma unroll
      for (int k = 0; k < kFuseLines; ++k)
        d[t][k] = (t < s - 1 && xlive(k)) ? __ldcg(tiny + (long long)t * g.P + xid(k)) : make_float2(0.f, 0.f);
  };
  auto x_sum = [&](int s, const float2 (&r)[kFuseLines], const float2 (&d)[kSub - 1][kFuseLines]) {
#pragma unroll
    for (int k = 0; k < kFuseLines; ++k) tsx[k] = fh_df_from_pair(r[k]);
#pragma unroll
    for (int t = 0; t < kSub - 1; ++t)
      if (t < s - 1) {
        const fh_df w = fh_df_from_pair(wx[s][t]);
#pragma unroll
        for (int k = 0; k < kFuseLines; ++k) tsx[k] = fh_df_fma(w, fh_df_from_pair(d[t][k]), tsx[k]);
      }
  };
  // the y sums read the field and the layers this thread produced from
  // shared memory, older layers from L2, and the prefetched history row
  auto y_load = [&](int s, float2 (&r)[kFuseLines], float2 (&d)[kSub - 1][kFuseLines]) {
#pragma unroll
    for (int t = 0; t < kSub - 1; ++t)
#pragma unroll
      for (int k = 0; k < kFuseLines; ++k) {
        const int c = t - a.s0;
        d[t][k] = (t >= s || !ylive(k))     ? make_float2(0.f, 0.f)
                  : (c >= 0 && c < kYCache) ? ys(ycache + c * kFuseLines * kFuseThreads, k)
                                            : __ldcg(tiny + (long long)t * g.P + yid(k));
      }
    asm volatile("cp.async.wait_all;" ::: "memory");
#pragma unroll
    for (int k = 0; k < kFuseLines; ++k) r[k] = ys(ypre, k);
  };
  // history row of the step's y sums into ypre (asynchronous; zero without rows)
  auto y_prefetch = [&](int s) {
    const float2 *rby = a.rb0 ? a.rb0 + (long long)s * a.rb_step + a.rb_xy : nullptr;
#pragma unroll
    for (int k = 0; k < kFuseLines; ++k) {
      if (rby && ylive(k)) {
        const unsigned dst = (unsigned)__cvta_generic_to_shared(&ys(ypre, k));
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(rby + yid(k)) : "memory");
      } else {
        ys(ypre, k) = make_float2(0.f, 0.f);
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  auto y_sum = [&](int s, const float2 (&r)[kFuseLines], const float2 (&d)[kSub - 1][kFuseLines]) {
#pragma unroll
    for (int k = 0; k < kFuseLines; ++k) tsy[k] = fh_df_from_pair(r[k]);
#pragma unroll
    for (int t = 0; t < kSub - 1; ++t)
      if (t < s) {
        const fh_df w = fh_df_from_pair(wy[s][t]);
#pragma unroll
        for (int k = 0; k < kFuseLines; ++k) tsy[k] = fh_df_fma(w, fh_df_from_pair(d[t][k]), tsy[k]);
      }
  };
#pragma unroll
  for (int k = 0; k < kFuseLines; ++k) f[k] = ylive(k) ? __ldcg(a.Cd + yid(k)) : make_float2(0.f, 0.f);
  {
    float2 r[kFuseLines], d[kSub - 1][kFuseLines];
    x_load(a.s0, r, d);
    x_sum(a.s0, r, d);
  }

  for (int s = a.s0; s < a.s0 + a.ns; ++s) {
    const int j = a.j8 + s;
    TG_STAMP(0);
    // ---- x half step (fr_d_t_g_2d.cpp:2577-2590): field and newest layer
    {
      const fh_df kst = fh_df_from_pair(cx[s][0]), S2 = fh_df_from_pair(cx[s][1]), st = fh_df_from_pair(cx[s][2]);
      const float2 *lat = s >= 1 ? tiny + (long long)(s - 1) * g.P : nullptr;
      const fh_df wl_ = s >= 1 ? fh_df_from_pair(wx[s][s - 1]) : fh_df{0.f, 0.f};
      float2 c[kFuseLines], d[kFuseLines];
#pragma unroll
      for (int k = 0; k < kFuseLines; ++k) {
        c[k] = xlive(k) ? __ldcg(a.Cd + xid(k)) : make_float2(0.f, 0.f);
        d[k] = (lat && xlive(k)) ? __ldcg(lat + xid(k)) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int k = 0; k < kFuseLines; ++k)
        if (xlive(k)) {
          const fh_df ts = lat ? fh_df_fma(wl_, fh_df_from_pair(d[k]), tsx[k]) : tsx[k];
          fh_df om = fh_df_fma(kst, fh_df_from_pair(c[k]), S2);
          om = fh_df_fma(st, ts, om);
          xch[k * kFuseSL + tg_fslot(xi)] = fh_df_pair(fh_df_neg(fh_df_mul(fh_df_from_pair(g_x[k * kFuseNL + xi - 1]), om)));
        }
    }
    y_prefetch(s);  // after the x loads: the copies run under the x solve
    __syncthreads();
    TG_STAMP(1);
    if (xl_ok(grp))
      tg_group_solve(Nx, fa_x + grp * kFuseSL, al_x + grp * kFuseSL, xch + grp * kFuseSL, ub_sm[grp], fh_df{0.f, 0.f},
                     fh_df_from_pair(cx[s][3]), scan_sm[grp], &uN_sm[grp], 1 + grp, gt, w4);
    __syncthreads();
    TG_STAMP(2);
#pragma unroll
    for (int k = 0; k < kFuseLines; ++k)
      if (xlive(k)) a.Chd[xid(k)] = xch[k * kFuseSL + tg_fslot(xi)];
    if (tid < 3 * kFuseLines) {  // nodes 0, Nx, Nx + 1 of the four lines: Ch and C
      const int l = tid / 3, k = tid % 3;
      if (xl_ok(l)) {
        const float2 v = ub_sm[l][k == 0 ? 0 : 1];
        const long long id = (long long)(line0 + l) * g.ld + (k == 0 ? 0 : Nx - 1 + k);
        a.Chd[id] = v;
        a.Cd[id] = v;
      }
    }
    tg_grid_arrive(a.bar);
    TG_STAMP(7);
    {  // the y history part overlaps the barrier (its layers are complete)
      float2 r[kFuseLines], d[kSub - 1][kFuseLines];
      y_load(s, r, d);
      y_sum(s, r, d);
    }
    TG_STAMP(8);
    if (!tg_grid_wait(a.bar, ++nb * nblk, a.err)) return;
    TG_STAMP(3);
    // ---- y half step (fr_d_t_g_2d.cpp:2591-2606): the half-step field
    {
      const fh_df kst = fh_df_from_pair(cy[s][0]), kyh = fh_df_from_pair(cy[s][1]), S2 = fh_df_from_pair(cy[s][2]),
                  st = fh_df_from_pair(cy[s][3]);
      float2 c[kFuseLines];
#pragma unroll
      for (int k = 0; k < kFuseLines; ++k) c[k] = ylive(k) ? __ldcg(a.Chd + yid(k)) : make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < kFuseLines; ++k)
        if (ylive(k)) {
          const fh_df cc = fh_df_from_pair(c[k]);
          // old[size-2] - old[size-1] (fr_d_t_g_2d.cpp:3478-3481)
          const fh_df tt = fh_df_fma(kyh, fh_df_sub(fh_df_from_pair(f[k]), cc), tsy[k]);
          fh_df om = fh_df_fma(kst, cc, S2);
          om = fh_df_fma(st, tt, om);
          xch[yc * kFuseSL + tg_fslot(yq(k))] =
              fh_df_pair(fh_df_neg(fh_df_mul(fh_df_from_pair(g_y[yc * kFuseNL + yq(k) - 1]), om)));
        }
    }
    __syncthreads();
    TG_STAMP(4);
    if (yl_ok(grp))
      tg_group_solve(Ny, fa_y + grp * kFuseSL, al_y + grp * kFuseSL, xch + grp * kFuseSL, ub_sm[grp], fh_df{1.f, 0.f},
                     fh_df{0.f, 0.f}, scan_sm[grp], &uN_sm[grp], 1 + grp, gt, w4);
    __syncthreads();
    TG_STAMP(5);
    {
      float2 *Dj = a.D + (long long)j * g.P;
      const int c = s - a.s0;  // this launch's layer index (cached below kYCache)
#pragma unroll
      for (int k = 0; k < kFuseLines; ++k)
        if (ylive(k)) {
          const float2 u = xch[yc * kFuseSL + tg_fslot(yq(k))];
          const float2 dn = fh_df_pair(fh_df_sub(fh_df_from_pair(u), fh_df_from_pair(f[k])));
          a.Cd[yid(k)] = u;
          Dj[yid(k)] = dn;
          f[k] = u;  // the old field of the next step
          if (c < kYCache) ys(ycache + c * kFuseLines * kFuseThreads, k) = dn;
        }
      if (tid < 3 * kFuseLines) {  // rows 0, Ny, Ny + 1 of the four columns: C only
        const int l = tid / 3, k = tid % 3;
        if (yl_ok(l)) {
          const long long id = (long long)(line0 + l) + (long long)(k == 0 ? 0 : Ny - 1 + k) * g.ld;
          a.Cd[id] = ub_sm[l][k == 0 ? 0 : 1];
        }
      }
    }
    if (s + 1 < a.s0 + a.ns) {
      tg_grid_arrive(a.bar);
      TG_STAMP(9);
      {  // the x history part of the next step overlaps the barrier (layers up to j - 1 are complete)
        float2 r[kFuseLines], d[kSub - 1][kFuseLines];
        x_load(s + 1, r, d);
        x_sum(s + 1, r, d);
      }
      TG_STAMP(10);
      if (!tg_grid_wait(a.bar, ++nb * nblk, a.err)) return;
    }
    TG_STAMP(6);
  }
}

__global__ void k_to_pairs(const double *__restrict__ x, float2 *__restrict__ y, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = fh_df_pair(fh_df_from_double(x[i]));
}
__global__ void k_from_pairs(const float2 *__restrict__ y, double *__restrict__ x, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = fh_df_to_double(fh_df_from_pair(y[i]));
}

// ------------------------------------------------------------------ host

static constexpr int kWeightTableMaxSteps = 4096;  // 2 x 4096^2 doubles = 268 MB

// One line per thread, serial FP64 recurrences: few threads per CTA spread the
// lines over many SMs (each chain is paced by FP64 latency).
static constexpr int kFactorThreads = 8;

static int tg_factor(fh_tg_solver *s, const double *cwj) {
  fh_ctx *ctx = s->ctx;
  const fh_tg_dev &g = s->dv;
  int rc;
  const size_t lsm = sizeof(double) * kFactorLineArrays * (size_t)std::max(g.sN, g.M);
  if (lsm <= 48 * 1024) {
    // one warp per line
    k_tg_factor_line<<<(unsigned)(g.M - 1), 32, lsm, ctx->stream>>>(g, 0, s->V2.as<double>(), cwj,
                                                                   s->alx.as<double>(), s->gx.as<double>(),
                                                                   s->fax.as<double>(), s->pfx.as<double>(),
                                                                   s->pbx.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor_line(x)"))) return rc;
    k_tg_factor_line<<<(unsigned)(g.sN - 1), 32, lsm, ctx->stream>>>(g, 1, s->V2.as<double>(), cwj,
                                                                    s->aly.as<double>(), s->gy.as<double>(),
                                                                    s->fay.as<double>(), s->pfy.as<double>(),
                                                                    s->pby.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor_line(y)"))) return rc;
  } else {
    // longer lines: the same passes as separate launches over global memory
    const unsigned cgrid = (unsigned)fh_ceil_div(g.P, 256);
    k_tg_factor_coef<<<cgrid, 256, 0, ctx->stream>>>(g, 0, s->V2.as<double>(), s->pfx.as<double>(),
                                                     s->pbx.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor_coef(x)"))) return rc;
    k_tg_factor_coef<<<cgrid, 256, 0, ctx->stream>>>(g, 1, s->V2.as<double>(), s->pfy.as<double>(),
                                                     s->pby.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor_coef(y)"))) return rc;
    k_tg_factor<<<(unsigned)fh_ceil_div(g.M, kFactorThreads), kFactorThreads, 0, ctx->stream>>>(
        g, 0, cwj, s->alx.as<double>(), s->gx.as<double>(), s->fax.as<double>(), s->pfx.as<double>(),
        s->pbx.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor(x)"))) return rc;
    k_tg_factor<<<(unsigned)fh_ceil_div(g.sN, kFactorThreads), kFactorThreads, 0, ctx->stream>>>(
        g, 1, cwj, s->aly.as<double>(), s->gy.as<double>(), s->fay.as<double>(), s->pfy.as<double>(),
        s->pby.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor(y)"))) return rc;
    k_tg_factor_ratio<<<cgrid, 256, 0, ctx->stream>>>(g, 0, s->alx.as<double>(), s->gx.as<double>(),
                                                      s->fax.as<double>(), s->pfx.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor_ratio(x)"))) return rc;
    k_tg_factor_ratio<<<cgrid, 256, 0, ctx->stream>>>(g, 1, s->aly.as<double>(), s->gy.as<double>(),
                                                      s->fay.as<double>(), s->pfy.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor_ratio(y)"))) return rc;
    k_tg_factor_prefix<<<(unsigned)fh_ceil_div(g.M, kFactorThreads), kFactorThreads, 0, ctx->stream>>>(
        g, 0, s->alx.as<double>(), s->fax.as<double>(), s->pfx.as<double>(), s->pbx.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor_prefix(x)"))) return rc;
    k_tg_factor_prefix<<<(unsigned)fh_ceil_div(g.sN, kFactorThreads), kFactorThreads, 0, ctx->stream>>>(
        g, 1, s->aly.as<double>(), s->fay.as<double>(), s->pfy.as<double>(), s->pby.as<double>());
    if ((rc = fh_after_launch(ctx, "k_tg_factor_prefix(y)"))) return rc;
  }
  if (s->dfsweep) {
    const fh_dbuf *src[10] = {&s->fax, &s->gx, &s->alx, &s->pfx, &s->pbx, &s->fay, &s->gy, &s->aly, &s->pfy, &s->pby};
    fh_dbuf *dst[10] = {&s->fax2, &s->gx2, &s->alx2, &s->pfx2, &s->pbx2,
                        &s->fay2, &s->gy2, &s->aly2, &s->pfy2, &s->pby2};
    for (int q = 0; q < 10; ++q) {
      k_to_pairs<<<(unsigned)fh_ceil_div(g.P, 256), 256, 0, ctx->stream>>>(src[q]->as<double>(), dst[q]->as<float2>(),
                                                                          g.P);
      if ((rc = fh_after_launch(ctx, "k_to_pairs"))) return rc;
    }
  }
  return FH_OK;
}

// Step j of the double-float sweeps (blocked mode); the block-start work,
// the weights and the factorization of step j are already enqueued.
//   per-solve weight table: mid rows at each sub-block start (k_tg_mid_tc),
//     the sweeps add the sub-block's own layers [j8, j);
//   per-step weight row (more steps than the table holds): one near sum over
//     the block's layers [j0, j) per step, far row folded in.
// Mid rows of sub-block jb over all the block's layers [j0, jb) on the tensor
// cores (k_tg_mid_tc), on top of base (far rows of step jb, or none).
static int tg_mid_tc(fh_tg_solver *s, cudaStream_t st, int jb, int j0, const float2 *base, long long ldbase,
                     float2 *out) {
  const fh_tg_dev &g = s->dv;
  const int K = jb - j0, KS = (K + 15) / 16, sb = jb / kSub;
  if (K < 1 || KS > 4) return fh_set_error(s->ctx, FH_EINVAL, "tensor-core mid rows: %d layers", K);
  const int nr = min(kSub, s->max_steps - jb);
  const float2 *D = reinterpret_cast<const float2 *>(s->D.as<double>()) + (long long)j0 * g.P;
  const uint8_t *ws = s->mws.as<uint8_t>() + (size_t)sb * kMtWBytes;
  const int8_t *we = s->mwe.as<int8_t>() + (size_t)sb * kMtRows;
  const unsigned grid = (unsigned)fh_ceil_div(g.P, 128);
  int *err = s->derr.as<int>();
  switch (KS) {
    case 1: k_tg_mid_tc<1><<<grid, 256, kMtSmem, st>>>(D, g.P, K, ws, we, nr, base, ldbase, out, g.P, err); break;
    case 2: k_tg_mid_tc<2><<<grid, 256, kMtSmem, st>>>(D, g.P, K, ws, we, nr, base, ldbase, out, g.P, err); break;
    case 3: k_tg_mid_tc<3><<<grid, 256, kMtSmem, st>>>(D, g.P, K, ws, we, nr, base, ldbase, out, g.P, err); break;
    default: k_tg_mid_tc<4><<<grid, 256, kMtSmem, st>>>(D, g.P, K, ws, we, nr, base, ldbase, out, g.P, err); break;
  }
  return fh_after_launch(s->ctx, "k_tg_mid_tc");
}

static int tg_step_df(fh_tg_solver *s, const double *Wj, const double *cwj, int max_n, int *done) {
  fh_ctx *ctx = s->ctx;
  const fh_tg_dev &g = s->dv;
  const int j = s->tstep;
  const int ldw = s->max_steps;
  const int j0 = s->blk ? s->j0 : 0;
  const float2 *D2 = reinterpret_cast<const float2 *>(s->D.as<double>());
  float2 *part = s->part.as<float2>();
  const float2 *farj = (s->blk && j0 > 0) ? s->far.as<float2>() + 2LL * (j - j0) * s->ldfar : nullptr;
  const float2 *rbx = farj, *rby = farj ? farj + s->ldfar : nullptr;
  const float2 *tiny = nullptr;
  const double *wtx = nullptr, *wty = nullptr;
  int nt = 0, rc;
  if (s->wtab) {
    const int j8 = (j / kSub) * kSub;  // >= j0: blocks are whole sub-blocks
    if (j8 > j0) {
      if (j == j8) {
        fh_prof_mark(ctx, FH_PROF_HISTORY, false);
        rc = tg_mid_tc(s, ctx->stream, j8, j0, farj, s->ldfar, part);
        fh_prof_mark(ctx, FH_PROF_HISTORY, true);
        if (rc) return rc;
      }
      rbx = part + 2LL * (j - j8) * g.P;
      rby = rbx + g.P;
    }
    if (s->fused) {
      // steps j .. j + ns - 1 of this sub-block in one cooperative launch
      const int ns = min(max_n, kSub - (j - j8));
      tg_fuse_args fa;
      fa.g = g;
      fa.Cd = s->Cd.as<float2>();
      fa.Chd = s->Chd.as<float2>();
      fa.D = reinterpret_cast<float2 *>(s->D.as<double>());
      fa.fax = s->fax2.as<float2>();
      fa.gx = s->gx2.as<float2>();
      fa.alx = s->alx2.as<float2>();
      fa.fay = s->fay2.as<float2>();
      fa.gy = s->gy2.as<float2>();
      fa.aly = s->aly2.as<float2>();
      fa.W = s->W.as<double>();
      fa.cwall = s->cw.as<double>();
      fa.ldw = ldw;
      fa.j8 = j8;
      fa.s0 = j - j8;
      fa.ns = ns;
      fa.bar = s->bar.as<unsigned>();
      fa.err = s->derr.as<int>();
      if (j8 > j0) {  // mid rows of the sub-block
        fa.rb0 = part;
        fa.rb_step = 2LL * g.P;
        fa.rb_xy = g.P;
      } else if (s->blk && j0 > 0) {  // far rows of the block
        fa.rb0 = s->far.as<float2>() + 2LL * (j8 - j0) * s->ldfar;
        fa.rb_step = 2LL * s->ldfar;
        fa.rb_xy = s->ldfar;
      } else {
        fa.rb0 = nullptr;
        fa.rb_step = fa.rb_xy = 0;
      }
      FH_CUDA_TRY(ctx, cudaMemsetAsync(s->bar.p, 0, sizeof(unsigned), ctx->stream));
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)s->fuse_blocks);
      cfg.blockDim = dim3(kFuseThreads);
      cfg.dynamicSmemBytes = kFuseSmem;
      cfg.stream = ctx->stream;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      fh_prof_mark(ctx, FH_PROF_SWEEP, false);
      const cudaError_t e = cudaLaunchKernelEx(&cfg, k_tg_sweeps_fused, fa);
      fh_prof_mark(ctx, FH_PROF_SWEEP, true);
      if (e != cudaSuccess) return fh_set_error(ctx, FH_ECUDA, "k_tg_sweeps_fused: %s", cudaGetErrorString(e));
      if ((rc = fh_after_launch(ctx, "k_tg_sweeps_fused"))) return rc;
      s->tstep += ns;
      *done = ns;
      return FH_OK;
    }
    nt = j - j8;
    tiny = D2 + (long long)j8 * g.P;
    wtx = Wj + j8;
    wty = Wj + ldw + j8;
  } else if (j - j0 >= 1) {
    // one split: the block holds at most 63 near layers
    const int K = j - j0, kchunk = (int)fh_ceil_div(K, 4) * 4;
    if ((rc = fh_launch_hist_sum_df_partials(ctx, 2, K, g.P, Wj + j0, ldw, D2 + (long long)j0 * g.P, g.P, 1, kchunk,
                                             reinterpret_cast<double *>(part), g.P, farj, s->ldfar, 1)))
      return rc;
    rbx = part;
    rby = part + g.P;
  }
  fh_prof_mark(ctx, FH_PROF_SWEEP, false);
  const size_t smx = sizeof(float2) * kXLines * 5 * (size_t)tg_line_stride(g.sN);
  k_tg_xsweep_df<<<(unsigned)fh_ceil_div(g.M - 1, kXLines), kXThreads, smx, ctx->stream>>>(
      g, s->Cd.as<float2>(), s->Chd.as<float2>(), rbx, tiny, nt, wtx, s->fax2.as<float2>(), s->gx2.as<float2>(),
      s->alx2.as<float2>(), s->pfx2.as<float2>(), s->pbx2.as<float2>(), cwj);
  if ((rc = fh_after_launch(ctx, "k_tg_xsweep_df"))) return rc;
  const size_t smy = sizeof(float2) * 4 * 6 * (size_t)tg_line_stride(g.M);
  k_tg_ysweep_df<<<(unsigned)fh_ceil_div(g.sN - 1, 4), kYThreads, smy, ctx->stream>>>(
      g, s->Cd.as<float2>(), s->Chd.as<float2>(), reinterpret_cast<float2 *>(s->D.as<double>()) + (long long)j * g.P,
      rby, tiny, nt, wty, s->fay2.as<float2>(), s->gy2.as<float2>(), s->aly2.as<float2>(), s->pfy2.as<float2>(),
      s->pby2.as<float2>(), cwj);
  fh_prof_mark(ctx, FH_PROF_SWEEP, true);
  if ((rc = fh_after_launch(ctx, "k_tg_ysweep_df"))) return rc;
  s->tstep++;
  *done = 1;
  return FH_OK;
}

// Enqueues the next step (or, for the fused sweeps, up to max_n steps of the
// current sub-block); *done receives the number of steps enqueued.
static int tg_one_step(fh_tg_solver *s, int max_n, int *done) {
  *done = 1;
  fh_ctx *ctx = s->ctx;
  const fh_tg_dev &g = s->dv;
  const int j = s->tstep;
  const int ldw = s->max_steps;
  int rc;
  const bool blocked = s->blk != nullptr;
  if (s->dfsweep && j == 0) {
    k_to_pairs<<<(unsigned)fh_ceil_div(g.P, 256), 256, 0, ctx->stream>>>(s->C.as<double>(), s->Cd.as<float2>(), g.P);
    if ((rc = fh_after_launch(ctx, "k_to_pairs"))) return rc;
  }
  if (blocked && j > 0 && j % kTgBlock == 0) {
    // new block: planes for layers [j-64, j), weight planes for steps j..j+63,
    // far rows S_far[2r + {0,1}] = sum_{k<j} w_{j+r}(k) D[k] on the tensor cores
    fh_prof_mark(ctx, FH_PROF_WEIGHTS, false);
    if ((rc = fh_blk_convert(ctx, *s->blk, s->D.as<double>(), g.P, j - kTgBlock, s->df ? 1 : 0))) return rc;
    if ((rc = fh_blk_tg_weights(ctx, *s->blk, j, g.Da, g.tau, g.alpha, g.beta, g.hcut,
                                s->wtab ? s->W.as<double>() : nullptr,
                                s->max_steps, s->max_steps)))
      return rc;
    fh_prof_mark(ctx, FH_PROF_WEIGHTS, true);
    // restricted summing with psi = t: the layers older than j - rs_lag have
    // zero weight for every step of the block; their chunk groups are skipped
    const int gbeg = s->rs_lag >= 0 && j > s->rs_lag ? (j - s->rs_lag) / (2 * 64) : 0;
    if ((rc = fh_blk_gemm(ctx, *s->blk, j, s->far.as<float2>(), s->ldfar, gbeg))) return rc;
    s->j0 = j;
  }
  // history layers summed in FP64 this step: the current block in blocked
  // mode; with restricted summing and psi = t, the layers within the cut lag
  int kstart = blocked ? s->j0 : 0;
  if (!blocked && s->rs_lag >= 0 && j > s->rs_lag) kstart = j - s->rs_lag;
  if (s->one_layer()) kstart = j;  // series expansions: no layer sums
  const int knear = j - kstart;
  const double *Wj;
  if (s->wtab) {
    if (j == 0) {
      fh_prof_mark(ctx, FH_PROF_WEIGHTS, false);
      dim3 gw((unsigned)fh_ceil_div(s->max_steps, kWallThreads), (unsigned)s->max_steps);
      k_tg_weights_all<<<gw, kWallThreads, 0, ctx->stream>>>(g, s->max_steps, s->W.as<double>(), ldw,
                                                            s->cw.as<double>());
      if ((rc = fh_after_launch(ctx, "k_tg_weights_all"))) return rc;
      if (s->mid_tc) {
        k_tg_mid_wslice<<<(unsigned)fh_ceil_div(s->max_steps, kSub), 128, 0, ctx->stream>>>(
            s->W.as<double>(), ldw, s->max_steps, s->mws.as<uint8_t>(), s->mwe.as<int8_t>());
        if ((rc = fh_after_launch(ctx, "k_tg_mid_wslice"))) return rc;
      }
      fh_prof_mark(ctx, FH_PROF_WEIGHTS, true);
    }
    Wj = s->W.as<double>() + (long long)j * 2 * ldw;
  } else {
    fh_prof_mark(ctx, FH_PROF_WEIGHTS, false);
    k_tg_weights<<<(unsigned)fh_ceil_div(knear > 0 ? knear : 1, 128), 128, 0, ctx->stream>>>(
        g, j, kstart, s->W.as<double>(), ldw, s->cw.as<double>());
    fh_prof_mark(ctx, FH_PROF_WEIGHTS, true);
    if ((rc = fh_after_launch(ctx, "k_tg_weights"))) return rc;
    Wj = s->W.as<double>();
  }
  const double *cwj = s->wtab ? s->cw.as<double>() + 4LL * j : s->cw.as<double>();
  if (!s->factor_fixed || j == 0)
    if ((rc = tg_factor(s, cwj))) return rc;
  if (s->dfsweep) return tg_step_df(s, Wj, cwj, max_n, done);
  // far-history rows of this step ((hi, lo) pairs, x row 2r, y row 2r+1)
  const float2 *far = nullptr;
  if (blocked && s->j0 > 0) far = s->far.as<float2>() + 2LL * (j - s->j0) * s->ldfar;
  int splits = 0, kchunk = 0;
  if (s->ser_J && j >= 1) {
    fh_prof_mark(ctx, FH_PROF_HISTORY, false);
    k_tg_series<<<(unsigned)fh_ceil_div(g.P, 256), 256, 0, ctx->stream>>>(
        s->D.as<double>(), s->df ? 1 : 0, s->H.as<double>(), s->ser_J, g.P,
        s->ser_tab.as<double>() + 3LL * s->ser_J * j, g.Da, s->part.as<double>());
    fh_prof_mark(ctx, FH_PROF_HISTORY, true);
    if ((rc = fh_after_launch(ctx, "k_tg_series"))) return rc;
    splits = 1;
  }
  if (s->two && j >= 1) {
    fh_prof_mark(ctx, FH_PROF_HISTORY, false);
    const double a = s->p.alpha;
    rc = fh_ta_step(ctx, s->two, j, s->D.as<double>(), s->df ? 1 : 0, g.P, g.Da * (pow(g.tau, 1.0 - a) / (1.0 - a)),
                    s->part.as<double>(), ctx->stream);
    fh_prof_mark(ctx, FH_PROF_HISTORY, true);
    if (rc) return rc;
    splits = 1;
  }
  if (knear >= 1) {
    fh_hist_plan(g.P, knear, s->max_splits, &splits, &kchunk);
    if (s->df)
      rc = fh_launch_hist_sum_df_partials(ctx, 2, knear, g.P, Wj + kstart, ldw,
                                          reinterpret_cast<const float2 *>(s->D.as<double>()) + (long long)kstart * g.P,
                                          g.P, splits, kchunk, s->part.as<double>(), g.P, far, s->ldfar, 0);
    else
      rc = fh_launch_hist_sum_partials(ctx, 2, knear, g.P, Wj + kstart, ldw,
                                       s->D.as<double>() + (long long)kstart * g.P, g.P, splits, kchunk,
                                       s->part.as<double>(), g.P);
    if (rc) return rc;
  }
  // the near kernel has folded the far rows in; otherwise the sweeps add them
  const float2 *farx = nullptr, *fary = nullptr;
  if (far && !(knear >= 1 && s->df)) {
    farx = far;
    fary = far + s->ldfar;
  }
  fh_prof_mark(ctx, FH_PROF_SWEEP, false);
  auto n1 = [&](int half) {
    const long long nn = (long long)(g.sN + 1) * (g.M + 1);
    k_tg_n1<<<(unsigned)fh_ceil_div(nn, 256), 256, 0, ctx->stream>>>(g, half, s->C.as<double>(), s->Ch.as<double>(),
                                                                    s->mass_c1, s->mass_tsb, s->Nn.as<double>(),
                                                                    s->dN.as<double>());
    return fh_after_launch(ctx, "k_tg_n1");
  };
  const double *dNp = s->massN ? s->dN.as<double>() : nullptr;
  if (s->massN && (rc = n1(0))) return rc;
  const size_t smx = sizeof(double) * kXLines * 5 * (size_t)tg_line_stride(g.sN);
  k_tg_xsweep<<<(unsigned)fh_ceil_div(g.M - 1, kXLines), kXThreads, smx, ctx->stream>>>(
      g, s->C.as<double>(), s->Ch.as<double>(), s->part.as<double>(), g.P, splits, s->fax.as<double>(),
      s->gx.as<double>(), s->alx.as<double>(), s->pfx.as<double>(), s->pbx.as<double>(), cwj, farx, dNp);
  if ((rc = fh_after_launch(ctx, "k_tg_xsweep"))) return rc;
  if (s->massN && (rc = n1(1))) return rc;
  const size_t smy = sizeof(double) * 4 * 6 * (size_t)tg_line_stride(g.M);
  k_tg_ysweep<<<(unsigned)fh_ceil_div(g.sN - 1, 4), kYThreads, smy, ctx->stream>>>(
      g, s->C.as<double>(), s->Ch.as<double>(), s->D.as<double>() + (s->one_layer() ? 0LL : (long long)j * g.P),
      s->part.as<double>(), g.P,
      splits, s->fay.as<double>(), s->gy.as<double>(), s->aly.as<double>(), s->pfy.as<double>(),
      s->pby.as<double>(), cwj, fary, s->df ? 1 : 0, dNp);
  fh_prof_mark(ctx, FH_PROF_SWEEP, true);
  if ((rc = fh_after_launch(ctx, "k_tg_ysweep"))) return rc;
  s->tstep++;
  return FH_OK;
}

// Double-float sweeps keep the field as pairs; the FP64 field C (returned by
// fh_tg_field / fh_tg_get_c_host) is refreshed at the end of every step call.
static int tg_publish(fh_tg_solver *s) {
  if (!s->dfsweep || s->tstep == 0) return FH_OK;
  fh_ctx *ctx = s->ctx;
  k_from_pairs<<<(unsigned)fh_ceil_div(s->dv.P, 256), 256, 0, ctx->stream>>>(s->Cd.as<float2>(), s->C.as<double>(),
                                                                            s->dv.P);
  return fh_after_launch(ctx, "k_from_pairs");
}

// The sweeps' dynamic shared memory grows with the line length.  The limit is
// a per-function attribute of the device, shared by every solver in the
// process, so it only ever grows (a smaller solver created later must not
// lower it below what an earlier, larger one launches with).
static int tg_set_smem_attrs(fh_ctx *ctx, int sN, int M) {
  static std::mutex mu;
  static int cur_x[64], cur_y[64];
  const int smx = (int)(sizeof(double) * kXLines * 5 * (size_t)tg_line_stride(sN));
  const int smy = (int)(sizeof(double) * 4 * 6 * (size_t)tg_line_stride(M));
  FH_REQUIRE(ctx, smx <= 200 * 1024 && smy <= 200 * 1024, FH_EINVAL,
             "fh_tg_create: grid too large for the sweeps (sN <= 1170, M <= 970)");
  FH_REQUIRE(ctx, ctx->device >= 0 && ctx->device < 64, FH_EINVAL, "fh_tg_create: device index");
  std::lock_guard<std::mutex> lk(mu);
  if (smx > cur_x[ctx->device]) {
    FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_tg_xsweep, cudaFuncAttributeMaxDynamicSharedMemorySize, smx));
    FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_tg_xsweep_df, cudaFuncAttributeMaxDynamicSharedMemorySize, smx));
    cur_x[ctx->device] = smx;
  }
  // the fused sweeps hold both directions' tables; larger grids use the per-step kernels
  if (sN <= kFuseMaxN && M <= kFuseMaxN) {
    static int cur_f[64];
    const int smf = (int)kFuseSmem;
    if (smf > cur_f[ctx->device] && smf <= 220 * 1024) {
      FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_tg_sweeps_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, smf));
      cur_f[ctx->device] = smf;
    }
  }
  if (smy > cur_y[ctx->device]) {
    FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_tg_ysweep, cudaFuncAttributeMaxDynamicSharedMemorySize, smy));
    FH_CUDA_TRY(ctx, cudaFuncSetAttribute(k_tg_ysweep_df, cudaFuncAttributeMaxDynamicSharedMemorySize, smy));
    cur_y[ctx->device] = smy;
  }
  return FH_OK;
}

extern "C" {

int fh_tg_create(fh_ctx *ctx, const fh_tg_params *p, int max_steps, int mode, fh_tg_solver **out) {
  FH_REQUIRE(ctx, ctx && p && out, FH_EINVAL, "fh_tg_create: null argument");
  *out = nullptr;
  FH_REQUIRE(ctx, p->sN >= 2 && p->M >= 2 && p->sN <= 4096 && p->M <= 4096, FH_EINVAL,
             "fh_tg_create: need 2 <= sN, M <= 4096");
  FH_REQUIRE(ctx, p->alpha > 0.0 && p->alpha < 1.0 && p->beta > 0.0 && p->tau > 0.0, FH_EINVAL,
             "fh_tg_create: need 0 < alpha < 1, beta > 0, tau > 0");
  FH_REQUIRE(ctx, p->dL > 0.0 && p->dLx > 0.0 && p->sigma > 0.0, FH_EINVAL, "fh_tg_create: bad geometry");
  FH_REQUIRE(ctx, max_steps >= 1, FH_EINVAL, "fh_tg_create: max_steps >= 1");
  FH_REQUIRE(ctx, mode == FH_TG_FP64 || mode == FH_TG_BLOCKED || mode == FH_TG_DF64, FH_EINVAL,
             "fh_tg_create: unknown mode %d", mode);
  {
    const int rc0 = tg_set_smem_attrs(ctx, p->sN, p->M);
    if (rc0) return rc0;
  }
  fh_tg_solver *s = new fh_tg_solver();
  s->ctx = ctx;
  s->p = *p;
  s->mode = mode;
  s->df = (mode != FH_TG_FP64);
  s->max_steps = max_steps;
  fh_tg_dev &g = s->dv;
  g.sN = p->sN;
  g.M = p->M;
  g.ld = p->sN + 2;
  g.P = (long long)(p->sN + 2) * (p->M + 2);
  if (g.P & 1) g.P += 1;  // even pitch for 16-byte history loads
  g.tau = p->tau;
  g.alpha = p->alpha;
  g.beta = p->beta;
  g.Da = 1.0 / tgamma(1.0 - p->alpha);  // TG_solver ctor (fr_d_t_g_2d.cpp:2391-2394)
  g.st = p->sigma / p->tau;
  g.d = p->d;
  g.C1 = p->C1;
  g.S = p->S;
  g.dL = p->dL;
  g.dLx = p->dLx;
  s->factor_fixed = (p->beta == 1.0);
  s->wtab = max_steps <= kWeightTableMaxSteps;
  const size_t fld = sizeof(double) * (size_t)g.P;
  int rc;
  if ((rc = fh_alloc(ctx, s->C, fld)) || (rc = fh_alloc(ctx, s->Ch, fld)) || (rc = fh_alloc(ctx, s->V2, fld)) ||
      (rc = fh_alloc(ctx, s->alx, fld)) || (rc = fh_alloc(ctx, s->gx, fld)) || (rc = fh_alloc(ctx, s->fax, fld)) ||
      (rc = fh_alloc(ctx, s->pfx, fld)) || (rc = fh_alloc(ctx, s->pbx, fld)) || (rc = fh_alloc(ctx, s->aly, fld)) ||
      (rc = fh_alloc(ctx, s->gy, fld)) || (rc = fh_alloc(ctx, s->fay, fld)) || (rc = fh_alloc(ctx, s->pfy, fld)) ||
      (rc = fh_alloc(ctx, s->pby, fld)) ||
      (rc = fh_alloc(ctx, s->D, fld * (size_t)max_steps)) ||
      (rc = fh_alloc(ctx, s->W, sizeof(double) * 2 * (size_t)max_steps *
                                    (max_steps <= kWeightTableMaxSteps ? (size_t)max_steps : 1))) ||
      (rc = fh_alloc(ctx, s->cw, sizeof(double) * 4 * (max_steps <= kWeightTableMaxSteps ? (size_t)max_steps : 1))) ||
      (rc = fh_alloc(ctx, s->part, fld * 2 * (size_t)s->max_splits, false))) {
    delete s;
    return rc;
  }
  s->dfsweep = (mode == FH_TG_BLOCKED);
  if (s->dfsweep) {
    const size_t fp = sizeof(float2) * (size_t)g.P;
    fh_dbuf *arr[12] = {&s->Cd, &s->Chd, &s->fax2, &s->gx2, &s->alx2, &s->pfx2,
                        &s->pbx2, &s->fay2, &s->gy2, &s->aly2, &s->pfy2, &s->pby2};
    for (auto *b : arr)
      if ((rc = fh_alloc(ctx, *b, fp))) {
        delete s;
        return rc;
      }
    // fused sub-block sweeps: fixed factorization, per-solve weight table, both
    // directions' tables in shared memory, one resident CTA per four lines
    const int nblk = std::max((g.M - 1) / kFuseLines + 1, (g.sN - 1) / kFuseLines + 1);  // lines 4b .. 4b + 3
    int nsm = 0, per_sm = 0;
    const size_t smf = kFuseSmem;
    if (s->factor_fixed && s->wtab && g.sN <= kFuseMaxN && g.M <= kFuseMaxN && smf <= 220 * 1024 &&
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tg_sweeps_fused, kFuseThreads, smf) == cudaSuccess &&
        nblk <= nsm * per_sm) {
      if ((rc = fh_alloc(ctx, s->bar, sizeof(unsigned))) || (rc = fh_alloc(ctx, s->derr, sizeof(int)))) {
        delete s;
        return rc;
      }
      s->fused = true;
      s->fuse_blocks = nblk;
    }
    cudaGetLastError();
  }
  if (s->dfsweep && s->wtab) {
    // mid rows on the tensor cores: every sub-block's weight slices, error flag
    const size_t nsub = (size_t)fh_ceil_div(max_steps, kSub);
    if ((rc = fh_alloc(ctx, s->mws, (size_t)kMtWBytes * nsub)) ||
        (rc = fh_alloc(ctx, s->mwe, (size_t)kMtRows * nsub)) ||
        (!s->derr.p && (rc = fh_alloc(ctx, s->derr, sizeof(int))))) {
      delete s;
      return rc;
    }
    cudaError_t e = cudaFuncSetAttribute(k_tg_mid_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMtSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_tg_mid_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMtSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_tg_mid_tc<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMtSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_tg_mid_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMtSmem);
    if (e != cudaSuccess) {
      delete s;
      return fh_set_error(ctx, FH_ECUDA, "fh_tg_create: mid-row kernel: %s", cudaGetErrorString(e));
    }
    s->mid_tc = true;
  }
  if (mode == FH_TG_BLOCKED && max_steps > kTgBlock) {
    s->blk = fh_blk_new();
    const int kcap = (int)fh_ceil_div(max_steps, kTgBlock) * kTgBlock;
    if ((rc = fh_blk_init(ctx, *s->blk, g.P, kcap))) {
      delete s;
      return rc;
    }
    s->ldfar = fh_blk_ppad(*s->blk);
    if ((rc = fh_alloc(ctx, s->far, sizeof(float2) * 2 * kTgBlock * (size_t)s->ldfar, false))) {
      delete s;
      return rc;
    }
  }
  *out = s;
  return FH_OK;
}

int fh_tg_destroy(fh_tg_solver *s) {
  if (!s) return FH_OK;
  if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
  delete s;
  return FH_OK;
}

// Closed-form psi = t weight of the lag-d layer pair (interval [j-d, j-d+1])
// at time j + ja, ja = 0.5 (x sums) or 1 (y sums), without Da tau^(1-a)/(1-a).
static double tg_lag_weight(double d, double ja, double a) {
  return pow(d + ja, 1.0 - a) - pow(d + ja - 1.0, 1.0 - a);
}

int fh_tg_set_restricted(fh_tg_solver *s, double dt_eps) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_restricted: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, dt_eps >= 0.0 && dt_eps < 1e300, FH_EINVAL, "fh_tg_set_restricted: dt_eps = %g", dt_eps);
  FH_REQUIRE(ctx, s->tstep == 0, FH_EINVAL, "fh_tg_set_restricted: only before the first step of a solve");
  s->dv.hcut = dt_eps;
  s->rs_lag = -1;
  if (dt_eps > 0.0 && s->p.beta == 1.0) {
    // first lag whose x and y weights are both below dt_eps (1 - 1e-9) (the
    // device weights there are certainly cut: they differ from these by ulps);
    // all longer lags have smaller weights, so the sums may start at j - rs_lag
    const double a = s->p.alpha, f = s->dv.Da * pow(s->p.tau, 1.0 - a) / (1.0 - a);
    const double cut = dt_eps * (1.0 - 1e-9);
    for (int d = 1; d <= s->max_steps; ++d)
      if (f * tg_lag_weight(d, 0.5, a) < cut && f * tg_lag_weight(d, 1.0, a) < cut) {
        s->rs_lag = d;
        break;
      }
  }
  s->graph.reset();
  return FH_OK;
}

int fh_tg_set_series(fh_tg_solver *s, int nterms) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_series: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, nterms >= 0 && nterms <= kSerMaxTerms, FH_EINVAL, "fh_tg_set_series: nterms = %d (0..%d)", nterms,
             kSerMaxTerms);
  FH_REQUIRE(ctx, s->tstep == 0, FH_EINVAL, "fh_tg_set_series: only before the first step of a solve");
  FH_REQUIRE(ctx, nterms == 0 || (s->p.beta == 1.0 && s->mode != FH_TG_BLOCKED), FH_EINVAL,
             "fh_tg_set_series: psi = t and the FP64 or DF64 mode only");
  FH_REQUIRE(ctx, nterms == 0 || !s->two, FH_EINVAL, "fh_tg_set_series: the two-series approximation is enabled");
  const fh_tg_dev &g = s->dv;
  int rc;
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  // new buffers first: on failure the solver keeps its previous configuration
  fh_dbuf nD, nH, ntab;
  // the history store: every layer pair, or only the newest for the series
  if ((rc = fh_alloc(ctx, nD, sizeof(double) * (size_t)g.P * (nterms ? 1 : (size_t)s->max_steps)))) return rc;
  auto adopt = [](fh_dbuf &dst, fh_dbuf &src) {
    std::swap(dst.p, src.p);
    std::swap(dst.bytes, src.bytes);
  };
  s->graph.reset();
  if (nterms == 0) {
    adopt(s->D, nD);
    s->H.release();
    s->ser_tab.release();
    s->ser_J = 0;
    return FH_OK;
  }
  // coefficient rows of every step j >= 1 (fr_d_t_g_2d.cpp _kb_row2 2965-3040
  // for psi = t, where the inner integral is exact after one term, and
  // _kb_row2_fixed_coefs 3041-3057), in the reference's arithmetic
  const int J = nterms;
  std::vector<double> tab((size_t)s->max_steps * 3 * J, 0.0);
  const double tau = s->p.tau, a = s->p.alpha;
  for (int j = 1; j < s->max_steps; ++j) {
    double *c = tab.data() + (size_t)j * 3 * J, *ex = c + J, *ey = c + 2 * J;
    const double t0 = tau * (double)(j - 1), t1 = tau * (double)j;
    double v6 = t0 / t1, mult = t1;
    for (int n = 0; n < J; ++n) {
      double v3;
      if (n == 0) {
        v3 = (t1 - t0) / t1;
      } else {
        v6 *= t0 / t1;
        v3 = 0.0 + 1.0 * ((1.0 / (n + 1.0)) * (1 - v6));
      }
      c[n] = mult * v3;
      mult *= t1;
    }
    for (int m = 0; m < 2; ++m) {
      double *e = m ? ey : ex;
      const double gtj = tau * ((double)j + (m ? 1.0 : 0.5));
      double v1 = pow(gtj, -a), i = 0.0;
      for (int n = 0; n < J; ++n) {
        e[n] = v1;
        i += 1.0;
        v1 *= -(-a - i + 1.0) / (i * gtj);
        if (!std::isfinite(v1)) break;  // the remaining coefficients stay 0
      }
    }
  }
  if ((rc = fh_alloc(ctx, nH, sizeof(double) * (size_t)J * (size_t)g.P)) ||
      (rc = fh_alloc(ctx, ntab, sizeof(double) * tab.size(), false)))
    return rc;
  FH_CUDA_TRY(ctx, cudaMemcpy(ntab.p, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
  adopt(s->D, nD);
  adopt(s->H, nH);
  adopt(s->ser_tab, ntab);
  s->ser_J = J;
  return FH_OK;
}

int fh_tg_set_two_series(fh_tg_solver *s, int enable) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_two_series: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, s->tstep == 0, FH_EINVAL, "fh_tg_set_two_series: only before the first step of a solve");
  FH_REQUIRE(ctx, !enable || (s->p.beta == 1.0 && s->mode != FH_TG_BLOCKED), FH_EINVAL,
             "fh_tg_set_two_series: psi = t and the FP64 or DF64 mode only");
  FH_REQUIRE(ctx, !enable || !s->ser_J, FH_EINVAL, "fh_tg_set_two_series: the series expansion is enabled");
  FH_REQUIRE(ctx, s->p.alpha > 0.0 && s->p.alpha < 1.0, FH_EINVAL, "fh_tg_set_two_series: alpha = %g",
             s->p.alpha);
  const fh_tg_dev &g = s->dv;
  int rc;
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  // new buffers first: on failure the solver keeps its previous configuration
  fh_dbuf nD;
  if ((rc = fh_alloc(ctx, nD, sizeof(double) * (size_t)g.P * (enable ? 1 : (size_t)s->max_steps)))) return rc;
  fh_ta *t = nullptr;
  if (enable && (rc = fh_ta_create(ctx, s->p.alpha, s->max_steps, g.P, &t))) return rc;
  std::swap(s->D.p, nD.p);
  std::swap(s->D.bytes, nD.bytes);
  if (s->two) fh_ta_delete(s->two);
  s->two = t;
  s->graph.reset();
  return FH_OK;
}

int fh_tg_set_mass_exchange(fh_tg_solver *s, int enable, double massN_a, double massN_b) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_mass_exchange: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, s->tstep == 0, FH_EINVAL, "fh_tg_set_mass_exchange: only before the first step of a solve");
  FH_REQUIRE(ctx, !enable || s->mode != FH_TG_BLOCKED, FH_EINVAL,
             "fh_tg_set_mass_exchange: the FP64 or DF64 mode only");
  FH_REQUIRE(ctx, !enable || (std::isfinite(massN_a) && std::isfinite(massN_b) &&
                              2.0 + s->p.tau * massN_a * massN_b != 0.0),
             FH_EINVAL, "fh_tg_set_mass_exchange: a = %g, b = %g", massN_a, massN_b);
  int rc;
  if (enable && !s->Nn.p) {
    if ((rc = fh_alloc(ctx, s->Nn, sizeof(double) * (size_t)s->dv.P)) ||
        (rc = fh_alloc(ctx, s->dN, sizeof(double) * (size_t)s->dv.P)))
      return rc;
  }
  if (!enable) {
    s->Nn.release();
    s->dN.release();
  }
  s->massN = enable != 0;
  // the reference's operand order: 1/(2 + (tau a) b) and (tau sigma) b
  s->mass_c1 = 1.0 / (2.0 + s->p.tau * massN_a * massN_b);
  s->mass_tsb = s->p.tau * s->p.sigma * massN_b;
  s->graph.reset();
  return FH_OK;
}

int fh_tg_set_diffusion(fh_tg_solver *s, int fixed_d, double lambda, double ka0, double k) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_diffusion: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, s->tstep == 0, FH_EINVAL, "fh_tg_set_diffusion: only before the first step of a solve");
  FH_REQUIRE(ctx, fixed_d || (std::isfinite(lambda) && std::isfinite(ka0) && std::isfinite(k) && k != 0.0),
             FH_EINVAL, "fh_tg_set_diffusion: lambda = %g, ka0 = %g, k = %g", lambda, ka0, k);
  s->dv.fixed_d = fixed_d ? 1 : 0;
  s->dv.lam = lambda;
  s->dv.ka0 = ka0;
  s->dv.kk = fixed_d ? 1.0 : k;
  s->graph.reset();  // the factor tables are rebuilt at the first step of a solve
  return FH_OK;
}

// Zero series accumulators at the start of a solve.
static int tg_series_reset(fh_tg_solver *s) {
  if (!s->ser_J) return FH_OK;
  FH_CUDA_TRY(s->ctx, cudaMemsetAsync(s->H.p, 0, s->H.bytes, s->ctx->stream));
  return FH_OK;
}

int fh_tg_set_state(fh_tg_solver *s, const double *V2, const double *C) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_state: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, V2 && C, FH_EINVAL, "fh_tg_set_state: null pointer");
  const size_t n = sizeof(double) * (size_t)(s->p.sN + 2) * (s->p.M + 2);
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->V2.p, V2, n, cudaMemcpyDeviceToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->C.p, C, n, cudaMemcpyDeviceToDevice, ctx->stream));
  if (s->derr.p) FH_CUDA_TRY(ctx, cudaMemsetAsync(s->derr.p, 0, sizeof(int), ctx->stream));
  if (s->massN) FH_CUDA_TRY(ctx, cudaMemsetAsync(s->Nn.p, 0, s->Nn.bytes, ctx->stream));  // N starts at 0
  if (int rc = tg_series_reset(s)) return rc;
  s->tstep = 0;
  s->j0 = 0;
  s->have_state = true;
  return FH_OK;
}

int fh_tg_set_state_host(fh_tg_solver *s, const double *V2_host, const double *C_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_set_state_host: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, V2_host && C_host, FH_EINVAL, "fh_tg_set_state_host: null pointer");
  const size_t n = sizeof(double) * (size_t)(s->p.sN + 2) * (s->p.M + 2);
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->V2.p, V2_host, n, cudaMemcpyHostToDevice, ctx->stream));
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(s->C.p, C_host, n, cudaMemcpyHostToDevice, ctx->stream));
  if (s->derr.p) FH_CUDA_TRY(ctx, cudaMemsetAsync(s->derr.p, 0, sizeof(int), ctx->stream));
  if (s->massN) FH_CUDA_TRY(ctx, cudaMemsetAsync(s->Nn.p, 0, s->Nn.bytes, ctx->stream));  // N starts at 0
  if (int rc = tg_series_reset(s)) return rc;
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  s->tstep = 0;
  s->j0 = 0;
  s->have_state = true;
  return FH_OK;
}

int fh_tg_step(fh_tg_solver *s, int nsteps) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_step: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, s->have_state, FH_EINVAL, "fh_tg_step: state not set");
  FH_REQUIRE(ctx, nsteps >= 0, FH_EINVAL, "fh_tg_step: nsteps < 0");
  FH_REQUIRE(ctx, s->tstep + nsteps <= s->max_steps, FH_ENOMEM, "fh_tg_step: history full (%d + %d > %d)", s->tstep,
             nsteps, s->max_steps);
  if (ctx->graphs && s->tstep == 0 && nsteps > 1) {
    int rc = fh_graph_run(ctx, s->graph, nsteps, [&]() {
      for (int n = 0, d = 1; n < nsteps; n += d) {
        int r = tg_one_step(s, nsteps - n, &d);
        if (r) return r;
      }
      return tg_publish(s);
    });
    if (rc) return rc;
    s->tstep = nsteps;
    s->j0 = (s->blk && nsteps > kTgBlock) ? ((nsteps - 1) / kTgBlock) * kTgBlock : 0;
    return FH_OK;
  }
  for (int n = 0, d = 1; n < nsteps; n += d) {
    int rc = tg_one_step(s, nsteps - n, &d);
    if (rc) return rc;
  }
  return tg_publish(s);
}

int fh_tg_get_n_host(fh_tg_solver *s, double *N_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_get_n_host: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, N_host, FH_EINVAL, "fh_tg_get_n_host: null pointer");
  FH_REQUIRE(ctx, s->massN, FH_EINVAL, "fh_tg_get_n_host: the mass exchange is off");
  const size_t n = sizeof(double) * (size_t)(s->p.sN + 2) * (s->p.M + 2);
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(N_host, s->Nn.p, n, cudaMemcpyDeviceToHost, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FH_OK;
}

int fh_tg_get_c_host(fh_tg_solver *s, double *C_host) {
  FH_REQUIRE(nullptr, s, FH_EINVAL, "fh_tg_get_c_host: null solver");
  fh_ctx *ctx = s->ctx;
  FH_REQUIRE(ctx, C_host, FH_EINVAL, "fh_tg_get_c_host: null pointer");
  const size_t n = sizeof(double) * (size_t)(s->p.sN + 2) * (s->p.M + 2);
  FH_CUDA_TRY(ctx, cudaMemcpyAsync(C_host, s->C.p, n, cudaMemcpyDeviceToHost, ctx->stream));
  FH_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (s->derr.p) {
    int h = 0;
    FH_CUDA_TRY(ctx, cudaMemcpy(&h, s->derr.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) return fh_set_error(ctx, FH_ETIMEOUT, "a bounded device wait expired (fused sweeps or mid rows)");
  }
  return FH_OK;
}

long long fh_tg_device_bytes(const fh_tg_solver *s) {
  if (!s) return -1;
  const fh_dbuf *bufs[] = {&s->C,    &s->Ch,   &s->V2,   &s->D,    &s->W,    &s->cw,   &s->part, &s->alx,
                           &s->gx,   &s->fax,  &s->pfx,  &s->pbx,  &s->aly,  &s->gy,   &s->fay,  &s->pfy,
                           &s->pby,  &s->far,  &s->Cd,   &s->Chd,  &s->fax2, &s->gx2,  &s->alx2, &s->pfx2,
                           &s->pbx2, &s->fay2, &s->gy2,  &s->aly2, &s->pfy2, &s->pby2, &s->bar,  &s->derr,
                           &s->H,    &s->ser_tab, &s->Nn,   &s->dN,   &s->mws,  &s->mwe};
  size_t n = 0;
  for (const fh_dbuf *d : bufs) n += d->bytes;
  if (s->blk) n += fh_blk_bytes(*s->blk);
  if (s->two) n += fh_ta_bytes(s->two);
  return (long long)n;
}

const double *fh_tg_field(const fh_tg_solver *s) { return s ? s->C.as<double>() : nullptr; }

int fh_tg_tstep(const fh_tg_solver *s) { return s ? s->tstep : -1; }

}  // extern "C"
