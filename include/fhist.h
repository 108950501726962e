/*
 * fhist.h -- C ABI of libfhist, the GB300 (sm_103a) implementation of the
 * fractional-derivative history path of sevaboh/theses_code:
 *   per time step, the weighted sum over all stored time layers (L1
 *   Caputo-Gerasimov, psi-Caputo or Atangana-Baleanu weights), then the
 *   implicit tridiagonal solve of every grid line (ADI x/y sweeps in 2D).
 *
 * Conventions
 *  - Plain C types only; every array argument is a DEVICE pointer unless the
 *    parameter name ends in _host.  Sizes are element counts.
 *  - Every call returns an int status (FH_OK on success) and never aborts;
 *    fh_last_error() gives a one-line reason.  Work is enqueued on the
 *    context's stream; host-buffer calls synchronise that stream.
 *  - Calls on one context are not thread-safe; use one context per thread.
 *  - Destroy solver objects before the context they were created on.
 *  - Each entry point names the reference interface it replaces (file:line in
 *    the reference repository).
 */
#ifndef FHIST_H
#define FHIST_H

#ifdef __cplusplus
extern "C" {
#endif

#define FH_OK 0
#define FH_EINVAL 1      /* bad argument                                  */
#define FH_ENOMEM 2      /* device allocation failed / history full      */
#define FH_ECUDA 3       /* CUDA runtime error                            */
#define FH_ENONFINITE 4  /* non-finite value in a result                  */
#define FH_ETIMEOUT 5    /* a bounded device wait ran out                 */
#define FH_ERANGE 6      /* argument outside the evaluated range          */
#define FH_ENOTSUP 7     /* combination not supported                     */

typedef struct fh_ctx fh_ctx;

/* ------------------------------------------------------------- context */
/* Replaces the reference offload wrapper (OpenCL_program / OpenCL_commandqueue,
 * opencl_cuda_base.cpp:353-455, 212-318; CUDA backend 467-752). */
int fh_version(void);
int fh_ctx_create(int device, fh_ctx **out);
int fh_ctx_destroy(fh_ctx *ctx);
const char *fh_last_error(const fh_ctx *ctx);
int fh_ctx_sync(fh_ctx *ctx);
/* A multi-step call that starts from the initial state (fh_*_step right after
 * setting the state) is recorded once as a CUDA graph and replayed by later
 * identical calls (on by default).  With kernel profiling on, the profiling
 * marks are recorded into the graph and each replay synchronises the stream. */
int fh_ctx_set_graphs(fh_ctx *ctx, int enable);
/* Non-blocking: 1 if all work enqueued on the context finished, 0 if not, < 0 on error. */
int fh_ctx_query(fh_ctx *ctx);
int fh_ctx_set_stream(fh_ctx *ctx, void *cuda_stream);
void *fh_ctx_get_stream(fh_ctx *ctx);
/* Number of kernels this context has launched so far. */
long long fh_ctx_launch_count(const fh_ctx *ctx);

/* Live kernel timing with CUDA events recorded on the context stream around
 * each launch of a kernel class (off by default; enabling clears the totals).
 * FH_PROF_HISTORY: history-sum kernels (FP64 / double-float, CUDA cores);
 * FH_PROF_SWEEP: line-sweep kernels; FH_PROF_WEIGHTS: weight kernels and, in
 * blocked mode, the per-block slicing of weights and history layers;
 * FH_PROF_GEMM: the tensor-core far-history contraction.  _read synchronises
 * the stream. */
#define FH_PROF_HISTORY 0
#define FH_PROF_SWEEP 1
#define FH_PROF_WEIGHTS 2
#define FH_PROF_GEMM 3
#define FH_PROF_KINDS 4
int fh_ctx_profile(fh_ctx *ctx, int enable);
int fh_ctx_profile_read(fh_ctx *ctx, int kind, double *total_ms, long long *launches);

/* ------------------------------------------------------------- weights */
/* w[k] = scale * int_{(x0+k)tau}^{(x0+k+len)tau} (psi(X tau) - psi(s))^(-alpha) ds,
 * k = 0..K-1, psi(t) = t^beta.  Replaces H_solver::kb/calc_int/_kb_row/_kb_row2
 * (mt_psi_caputo.cpp:435-747), TG_solver_::kb (fr_d_t_g_2d.cpp:3059-3239) and the
 * OpenCL calc_kb kernels (fr_d_t_g_2d.cpp:1492-1547).  beta == 1 uses the
 * reference's closed form; other beta the converged integral. */
int fh_weights_psi(fh_ctx *ctx, int K, double x0, double len, double X, double tau,
                   double alpha, double beta, double scale, double *w);

/* L1 Caputo-Gerasimov coefficients of H_solver::Om1 (mt_minimal.cpp:926-934):
 * w[t] = (os-t)^(1-alpha) - (os-t-1)^(1-alpha), t = 0..os-2. */
int fh_weights_l1(fh_ctx *ctx, int os, double alpha, double *w);

/* Atangana-Baleanu lag weights of MF_intF_simple (MF_int_series.cpp:614-718,
 * MF_int_choice 523-530): w[lag] = int_{(lag-1)tau}^{lag tau} E_alpha(-alpha/(1-alpha) u^alpha) du
 * for lag = 1..n, and w[0] = w[1].  FH_ERANGE if the series would cancel badly. */
int fh_weights_ab(fh_ctx *ctx, int n, double tau, double alpha, double *w);

/* out[i] = E_{a,b}(z[i]) (mittag_leffler, mittag-lefler.cpp:239-293). */
int fh_mittag_leffler(fh_ctx *ctx, int n, double a, double b, const double *z, double *out);

/* ------------------------------------------------------------- history */
/* S[m*ldS + p] = sum_{k<K} W[m*ldw + k] * D[k*ldd + p], m < M (M = 1 or 2), p < P.
 * D holds layer differences (layer k+1 minus layer k), point index contiguous.
 * Replaces the history loops of H_solver::Om1 (mt_psi_caputo.cpp:1315-1342),
 * TG_solver_::Om1 (fr_d_t_g_2d.cpp:3340-3490), H_solver::time_summing
 * (irrigation_fractional.cpp:4099-4177) and the GPU Sum kernels
 * (irrigation_fractional.cpp:1224-1495).  P and ldd must be even, D 16-byte aligned.
 * Asynchronous on the context stream; its split partials live in a workspace
 * the context keeps, which a call grows (allocating, after synchronising the
 * stream) only when it needs more than earlier calls did, so repeated calls of
 * one size neither allocate nor synchronise. */
int fh_history_sum(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw,
                   const double *D, long long ldd, double *S, long long ldS);

/* Reference Sum-kernel form on stored layers (fr_ocl_call_sum,
 * irrigation_fractional.cpp:1828-1896): S[p] = sum_{t<K} w[t]*(H[(t+1)ldh+p] - H[t ldh+p]). */
/* Series accumulators of the irrigation model (sum_alg 2, time_summing
 * irrigation_fractional.cpp:4150-4164; the reference's CUDA/OpenCL Sum kernels
 * 1224-1561 with sum_alg 2): per point p, for n < J,
 *   H[n*ldh + p] += c[n] * Dn[p]                      (Htmp update)
 * then S[p] = (sum_n e[n] * H[n*ldh + p]) / tau     (_kb_row2_fixed_coefs / tau[tstep])
 * in the reference's operation order.  The caller supplies the step's
 * coefficients (host arrays of J values): c[n] = g(T)^(n+1) row2_precalc[n]
 * (zero beyond the precomputed row), e[n] the running factor of
 * _kb_row2_fixed_coefs (e[0] = g(T_{j+1})^-alpha, e[n] = e[n-1] * -(-alpha - n
 * + 1) / (n g(T_{j+1}))), tau = tau[tstep]; Dn = the newest layer difference.
 * J <= FH_SERIES_MAX_TERMS.  H is the caller's J x ldh accumulator array. */
#define FH_SERIES_MAX_TERMS 256
int fh_series_sum(fh_ctx *ctx, int J, long long P, const double *c_host, const double *e_host, double tau,
                  const double *Dn, double *H, long long ldh, double *S);
int fh_history_sum_layers(fh_ctx *ctx, int K, long long P, const double *w, const double *H,
                          long long ldh, double *S);

/* Blocked contraction on the tensor cores: S[m*ldS + p] = sum_{k<K} W[m*ldw + k] D[k*ldd + p]
 * for m < 128.  Every 64-layer chunk of W rows and D points gets a power-of-two
 * scale and is cut into four integer bf16 slices; the ten slice products up to
 * level 3 are summed exactly in the FP32 tensor-core accumulators and combined
 * in double-float, FP64 result.  K must be a positive multiple of 64.  Error
 * ~2^-32 of the chunk maxima of |W||D|.  This is the far-history GEMM of the
 * blocked form of fr_d_t_g_2d.cpp:3340-3384 (one weight row per future half
 * step); it allocates its own plane storage. */
int fh_history_contract_bf16(fh_ctx *ctx, int K, long long P, const double *W, int ldw,
                               const double *D, long long ldd, double *S, long long ldS);

/* Allocation-free variant of fh_history_sum: same arguments, and the same
 * sums within FP64 rounding (when M*P > FH_NOALLOC_SCRATCH_DOUBLES/16 the fixed
 * array holds fewer split partials than fh_history_sum plans, so the layers are
 * grouped into fewer, longer splits and the partials are added in another
 * order).  No counterpart in the reference.  For callers that cannot call
 * cudaMalloc when they need the sum: applications that hand all device memory
 * to their own pool or admit work against a fixed memory budget, and step
 * loops where a cudaMalloc/cudaFree pair would synchronise the device.  The
 * split-K partial sums go to a fixed array of FH_NOALLOC_SCRATCH_DOUBLES
 * doubles (16 MiB) that every GPU loading the library reserves until the
 * process exits; the call never allocates.  Limit: M*P <=
 * FH_NOALLOC_SCRATCH_DOUBLES, else FH_ERANGE; K has no limit (a split of any
 * length stages its weights in pieces).  The first call on a device looks up
 * the array's device address (and loads the library's device code there):
 * make that first call before any stream capture.  All calls on a device share
 * the array and it keeps the last call's partials; calls whose GPU work
 * overlaps (other streams or contexts on the same device) race on it and must
 * be serialised by the caller. */
#define FH_NOALLOC_SCRATCH_DOUBLES 2097152LL
int fh_history_sum_noalloc(fh_ctx *ctx, int M, int K, long long P, const double *W, int ldw,
                           const double *D, long long ldd, double *S, long long ldS);

/* --------------------------------------------------------- tridiagonal */
/* nsys systems A_i u_{i-1} - R_i u_i + B_i u_{i+1} = Om_i, i = 1..N-1, with
 * u_0 = al1[s] u_1 + bt1[s] and u_N = u_right[s] (right_mode 0) or
 * u_N = Bt_N/(1-Al_N) (right_mode 1); u_{N+1} = u_N.  System s uses entries
 * [s*lds, s*lds + N] of A, R, B, Om and [s*ldu, s*ldu + N+1] of u.
 * Replaces H_solver::al1/bt1/U1 (mt_minimal.cpp:829-858, 942-1031) and
 * TG_solver::U1 (fr_d_t_g_2d.cpp:2523-2551).  Asynchronous on the context
 * stream, with Al in the context's workspace (as fh_history_sum). */
int fh_tridiag_batched(fh_ctx *ctx, int nsys, int N, const double *A, const double *R,
                       const double *B, const double *Om, long long lds, const double *al1,
                       const double *bt1, int right_mode, const double *u_right, double *u,
                       long long ldu);

/* Parallel cyclic reduction with the semantics of pcr_solver (nvidia_pcr.cpp:424-458):
 * a_i x_{i-1} + b_i x_i + c_i x_{i+1} = d_i for nsys systems of n unknowns stored
 * back to back (a_0 and c_{n-1} ignored).  n <= 2048. */
int fh_pcr_solver(fh_ctx *ctx, const double *a, const double *b, const double *c, const double *d,
                  double *x, int n, int nsys);

/* ------------------------------------------------ 1D H_solver, batched */
#define FH_W_L1 0   /* mt_minimal.cpp H_solver: L1 weights, Da = tau^-a/Gamma(2-a)        */
#define FH_W_PSI 1  /* mt_psi_caputo.cpp H_solver: psi-Caputo weights, Da = 1/(tau Gamma(2-a)) */
#define FH_K_CONST 0
#define FH_K_EXP 1

typedef struct {
  int N;            /* intervals; nodes 0..N plus ghost N+1             */
  double L;         /* domain length, dL = L/N                          */
  double tau;       /* time step                                        */
  double alpha;     /* time-derivative order, 0 < alpha < 1             */
  int weights;      /* FH_W_L1 or FH_W_PSI                              */
  double beta;      /* psi(t) = t^beta (FH_W_PSI)                       */
  int kmodel;       /* FH_K_CONST: K = kc ; FH_K_EXP: K = kc exp(kgam u) */
  double kc, kgam;
  double cinv;      /* constant 1/(dw/dh) factor                        */
  int gravity;      /* add (K_i - K_{i-1})/dL to the right part         */
  double al_left, bt_left; /* u_0 = al_left u_1 + bt_left               */
  double u_right;   /* Dirichlet value at node N                        */
} fh_h_params;

typedef struct fh_h_batch fh_h_batch;

/* A batch of independent H_solver instances (mt_psi_caputo.cpp:369-1507 /
 * mt_minimal.cpp:276-1048 with gamma = 1) advanced in lock step, one history
 * ring per batch.  max_steps bounds the stored history. */
int fh_h_batch_create(fh_ctx *ctx, int ninst, const fh_h_params *params_host, int max_steps,
                      fh_h_batch **out);
int fh_h_batch_destroy(fh_h_batch *b);
/* Total number of doubles of the concatenated state (sum of N_i + 2). */
long long fh_h_batch_state_size(const fh_h_batch *b);
/* Device bytes the batch holds (history, tables, work buffers); -1 for null.
 * No reference counterpart (serving admission). */
long long fh_h_batch_device_bytes(const fh_h_batch *b);
/* Concatenated per-instance U arrays (N_i + 2 each, instance order); resets tstep to 1. */
int fh_h_batch_set_u_host(fh_h_batch *b, const double *U_host);
int fh_h_batch_set_u(fh_h_batch *b, const double *U);
/* Continuous batching: instance i starts a new solve (parameters p, initial
 * state U0_host of p->N + 2 values) between two steps of the batch, while
 * the other instances go on.  Its steps count from 1 again, its history
 * starts empty (the earlier occupant's history slots are never read), and
 * its result after n further batch steps equals a fresh solve of n steps
 * within rounding (the history sums split at the batch's slot boundaries).
 * p->N may not exceed the node count the instance was created with (rounded
 * up to even); the occupant runs until the batch's max_steps is reached.
 * FP64 and DF64 history modes, no space-fractional instances in the batch.
 * Whole-batch state setters put every instance back on the batch clock.
 * No reference counterpart (the reference runs one solve per object). */
int fh_h_batch_restart(fh_h_batch *b, int i, const fh_h_params *p, const double *U0_host);
/* Small batches (at most 32 instances of at most 2046 interior nodes, FP64
 * history, no space-fractional instances) run all the steps of one
 * fh_h_batch_step call in one launch: a cluster of eight CTAs per instance
 * shares the history sum (distributed shared memory) and one of them solves
 * the line, step after step, with cluster barriers between.  On by default;
 * enable = 0 steps such batches kernel by kernel like larger ones (the same
 * sums within FP64 rounding: the history splits differ).  No reference
 * counterpart. */
int fh_h_batch_set_persistent(fh_h_batch *b, int enable);
int fh_h_batch_get_u_host(fh_h_batch *b, double *U_host);
/* U of instances [first, first+count) only (concatenated), synchronising the stream. */
int fh_h_batch_get_u_range_host(fh_h_batch *b, int first, int count, double *U_host);
/* H_solver::calc_step repeated nsteps times (tstep starts at 1). */
int fh_h_batch_step(fh_h_batch *b, int nsteps);
/* Space-fractional Caputo derivative in z, H_solver with gamma < 1 (the
 * calc_v term of Om1, mt_minimal.cpp:228-271,879-905 and
 * mt_psi_caputo.cpp:749-777,1293-1313, with Dg and the kb(gamma, i-1, i, i)
 * factor of A_, B, R, mt_psi_caputo.cpp:1164-1181, mt_minimal.cpp:744-749):
 * gamma_host[i] in (0, 1] per instance, 1 = classical second derivative (the
 * default).  Instances with gamma < 1 need N <= 2048.  Only before the first
 * step.  The nonlocal sum costs O(N^2) FP64 FMAs per instance and step, as in
 * the reference. */
int fh_h_batch_set_space_order(fh_h_batch *b, const double *gamma_host);
int fh_h_batch_tstep(const fh_h_batch *b);
/* History storage, before the first step: FH_H_FP64 (default), FH_H_DF64
 * ((hi, lo) FP32 pairs summed in double-float on the FP32 pipe, 2^-48
 * relative storage precision; solution within 1e-12 of the FP64 path on the
 * parity cases) or FH_H_BLOCKED: per block of 64 steps, the history slots
 * older than the block are contracted once for all 64 steps on the tensor
 * cores (exact bf16 slices with per-point and per-row power-of-two scales,
 * tcgen05, one 128-point tile of one instance against that instance's 64
 * weight rows), the block's own slots are summed per step in double-float
 * from a 128-layer ring; line solves and weights stay FP64; the history costs
 * 8 bytes per value (slice planes) and the full FP64 history is not kept.
 * Bound 1e-9 relative against the FP64 oracle.  No counterpart in the
 * reference. */
#define FH_H_FP64 0
#define FH_H_DF64 1
#define FH_H_BLOCKED 2
int fh_h_batch_set_mode(fh_h_batch *b, int mode);
/* Launch-shape autotuner for the batch history sum: times the candidate tile
 * CTAs (128/256/512 threads) x K-split caps (1/8/64) on the batch's buffers
 * and keeps the fastest; *best_ms (optional) receives its time per launch.
 * Not during a stream capture.  No counterpart in the reference. */
int fh_h_batch_autotune(fh_h_batch *b, float *best_ms);
int fh_h_batch_launch_shape(const fh_h_batch *b, int *tile_threads, int *split_cap);

/* ------------------------------------------------------ 2D TG_solver ADI */
typedef struct {
  int sN, M;        /* i = 0..sN, j = 0..M, array (sN+2)x(M+2), idx = i + j*(sN+2) */
  double tau, alpha, beta;
  double sigma, d, C1, S;
  double dL, dLx;   /* steps of the x sweep (along i) and y sweep (along j) */
} fh_tg_params;

#define FH_TG_FP64 0      /* FP64 history, FP64 FMA sums (bit-faithful arithmetic)        */
#define FH_TG_BLOCKED 1   /* far history on the tensor cores (exact bf16 slices), near in DF64 */
#define FH_TG_DF64 2      /* history as (hi, lo) FP32 pairs, double-float sums on the FP32 pipe */

typedef struct fh_tg_solver fh_tg_solver;

/* TG_solver_<func,1,kform> with dt_alg 0 (fr_d_t_g_2d.cpp:2037-4052): fixed
 * diffusion coefficient d, psi(t) = t^beta, full history. */
int fh_tg_create(fh_ctx *ctx, const fh_tg_params *p, int max_steps, int mode, fh_tg_solver **out);
int fh_tg_destroy(fh_tg_solver *s);
/* V2 = |v|^2 per node and the initial field, (sN+2)*(M+2) each. */
int fh_tg_set_state_host(fh_tg_solver *s, const double *V2_host, const double *C_host);
/* Device-pointer variant (inputs already resident in HBM). */
int fh_tg_set_state(fh_tg_solver *s, const double *V2, const double *C);
/* Restricted summing, TG_solver_ with dt_alg 2 (replaces the Om1 loop
 * fr_d_t_g_2d.cpp:3356-3380 and the kb precalculation 3101-3232 with dt_alg
 * 2): every history sum runs from the newest layer pair back and stops at the
 * first weight below dt_eps (weights include Da).  dt_eps = 0 restores the
 * full history (dt_alg 0).  Only before the first step of a solve (after
 * fh_tg_create or fh_tg_set_state).  With psi = t the sums read only the
 * layers within the lag where the weights fall below dt_eps; the history
 * store keeps every layer. */
int fh_tg_set_restricted(fh_tg_solver *s, double dt_eps);
/* Series expansion of the history sums, TG_solver_ with dt_alg 3 and
 * dt_eps = nterms (replaces the Om1 series branch fr_d_t_g_2d.cpp:3384-3429
 * with _kb_row2 2965-3040 and _kb_row2_fixed_coefs 3041-3057): per node
 * nterms accumulators of the binomial series of (t_n - s)^(-alpha) replace
 * the stored layers (memory nterms + 1 layers instead of max_steps).
 * psi = t, FH_TG_FP64 or FH_TG_DF64 only; nterms = 0 restores the full
 * history; 1..256.  Only before the first step of a solve. */
int fh_tg_set_series(fh_tg_solver *s, int nterms);
/* Two-series approximation of the history sums, TG_solver_ with dt_alg 4
 * (replaces the Om1 branch fr_d_t_g_2d.cpp:3438-3469 with calc_va and the
 * ia / ibk approximations 246-745): per node long (powers of t) and short
 * (Taylor) series whose coefficients absorb each new layer difference, each
 * within approx_eps = 1e-7 of its share of the sum.  The approximation
 * bookkeeping does not depend on the field and is planned on the host for
 * every step up to max_steps when enabled; the device keeps the coefficients
 * per node (tens of approximations of up to 20 terms per direction) and the
 * newest layer only.  psi = t, FH_TG_FP64 or FH_TG_DF64, no series expansion
 * at the same time; enable = 0 restores the full history.  Only before the
 * first step of a solve. */
int fh_tg_set_two_series(fh_tg_solver *s, int enable);
/* Mass exchange with a non-soluble phase, TG_solver with massN != 0
 * (TG_solver::N1 fr_d_t_g_2d.cpp:2503-2521 before each half step, the right
 * parts' (1/tau)(N - prevN) 3330-3332): per node
 * N' = (2 N + tau sigma b C) / (2 + tau a b) with a = massN_a, b = massN_b (the
 * reference's globals, 0.1 by default); N starts at 0 with every
 * fh_tg_set_state.  FH_TG_FP64 or FH_TG_DF64; enable = 0 turns it off.  Only
 * before the first step of a solve. */
int fh_tg_set_mass_exchange(fh_tg_solver *s, int enable, double massN_a, double massN_b);
/* Diffusion coefficient: fixed_d = 1 keeps the constant d of fh_tg_params
 * (TG_solver_<func,1,kform>); fixed_d = 0 uses D = lambda |v| (ka0 / k) per
 * node (TG_solver_<func,0,0>::D, fr_d_t_g_2d.cpp:2787-2800, the reference's
 * lambda = l, ka0 = ka[0], k = its averaged filtration coefficient) in the
 * coefficients A_, B (3242-3257).  Any mode.  Only before the first step of a
 * solve. */
int fh_tg_set_diffusion(fh_tg_solver *s, int fixed_d, double lambda, double ka0, double k);
/* The host bookkeeping of fh_tg_set_two_series for inspection (no device
 * work, no reference counterpart): per step j = 1 .. max_steps - 1 and
 * direction d (0: x sums, 1: y sums) spans[4 (2 j + d) + 0..2] = {first item,
 * first update item, end}; an item is 4 ints {kind | terms << 8, slot,
 * source slot, coefficient offset}, kind 0 evaluate (basis values at the
 * offset), 1 copy the source slot, 2 / 3 add to a long / short slot and 4 / 5
 * initialise one with the newest layer's coefficients ak[k] (F g[k]) (ak at
 * the offset, g after them; long slots keep c[0] = 0).  nslots[2]: slots per
 * point and direction; dterm[2]: the newest layer's weight.  Call with null
 * items / coef / spans to obtain *n_items and *n_coef, then with buffers of
 * those sizes (spans: 8 (max_steps + 1) ints). */
int fh_tg_two_series_plan(double alpha, int max_steps, int *nslots, double *dterm, int *n_items, int *items,
                          int *n_coef, double *coef, int *spans);
/* TG_solver::calc_step repeated nsteps times. */
int fh_tg_step(fh_tg_solver *s, int nsteps);
int fh_tg_get_c_host(fh_tg_solver *s, double *C_host);
/* The non-soluble phase N ((sN+2)*(M+2) values, the reference's b_N) with the
 * mass exchange on; synchronises the stream. */
int fh_tg_get_n_host(fh_tg_solver *s, double *N_host);
/* Device pointer to the current field ((sN+2)*(M+2) doubles, owned by the solver). */
/* Device bytes the solver holds (history, tables, work buffers); -1 for
 * null.  No reference counterpart (serving admission). */
long long fh_tg_device_bytes(const fh_tg_solver *s);
const double *fh_tg_field(const fh_tg_solver *s);
int fh_tg_tstep(const fh_tg_solver *s);

/* ----------------------------------------- 1D Atangana-Baleanu solver */
typedef struct fh_ab_solver fh_ab_solver;

/* solve_and_check (MF_int_series.cpp:875-958) with MF_intF_simple history:
 * m intervals on [0,1], A C_{j-1} + Bd C_j + Cc C_{j+1} = Rp_j, Dirichlet ends. */
int fh_ab_create(fh_ctx *ctx, int m, int max_steps, double tau, double alpha, fh_ab_solver **out);
int fh_ab_destroy(fh_ab_solver *s);
/* Source rows src_host[r*(m+1) + j]; step i uses row min(i-1, nrows-1).
 * Boundary values bl_host/br_host likewise per row. */
int fh_ab_set_source_host(fh_ab_solver *s, int nrows, const double *src_host, const double *bl_host,
                          const double *br_host);
int fh_ab_set_c_host(fh_ab_solver *s, const double *C_host);
int fh_ab_set_c(fh_ab_solver *s, const double *C);
/* Override the current-step coefficient Ii (default: the lag-1 weight). */
int fh_ab_set_current_coef(fh_ab_solver *s, double Ii);
/* Replace the history weights of lags 1..n (w_host[l-1] = weight of lag l,
 * before the first step) by a caller's table: the I_cache of MF_intF_simple
 * (MF_int_series.cpp:614-718), whose entries MF_int_choice (523-530) takes
 * from the integral-representation quadrature MF_intFv (469-521) once
 * (a/(1-a)) (lag tau)^a >= 1, where that quadrature is a few percent from
 * the converged series the library evaluates by default. */
int fh_ab_set_lag_weights_host(fh_ab_solver *s, int n, const double *w_host);
/* History mode, before the first step: FH_AB_FP64 (default, FP64 sums) or
 * FH_AB_BLOCKED (entries older than the current 128-step block contracted on
 * the tensor cores with exact bf16 slices, the rest in FP64; ~2x the history
 * memory).  No counterpart in the reference. */
#define FH_AB_FP64 0
#define FH_AB_BLOCKED 1
int fh_ab_set_mode(fh_ab_solver *s, int mode);
int fh_ab_step(fh_ab_solver *s, int nsteps);
int fh_ab_get_c_host(fh_ab_solver *s, double *C_host);

#ifdef __cplusplus
}
#endif
#endif /* FHIST_H */
