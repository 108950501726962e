/*
 * fh_oracle.h -- CPU oracle for the fractional-history hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (sevaboh/theses_code) used as the checker for the CUDA library.
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may
 * load it; the product path (libfhist) never links or calls it.
 *
 * Every function names the reference file:line it restates.  All arithmetic
 * is IEEE double unless stated otherwise; sums follow the reference's loop
 * order so that the oracle reproduces the reference to rounding.
 */
#ifndef FH_ORACLE_H
#define FH_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- weights */

/* int_{x0*tau}^{x1*tau} (psi(X*tau) - psi(s))^(-alpha) ds, psi(t) = t^beta.
 * beta == 1 follows H_solver::_kb_row (mt_psi_caputo.cpp:497-515) term for
 * term (the series stops after one term because (psi^-1)'' = 0).  beta != 1
 * evaluates the converged value of the same integral through the regularised
 * incomplete-beta form (series in y and 1-y, no truncation tolerance). */
double fho_psi_int(double x0, double x1, double X, double tau, double alpha, double beta);

/* L1 Caputo-Gerasimov coefficient b_k = (k+1)^(1-a) - k^(1-a)
 * (mt_minimal.cpp:930, in the reference's own form). */
double fho_l1_b(int k, double alpha);

/* Mittag-Leffler E_{a,b}(z) by its power series in long double
 * (mittag-lefler.cpp:239-293 restricted to the series branch). */
double fho_mittag_leffler(double a, double b, double z);

/* Atangana-Baleanu lag weight I(lag) = int_{(lag-1)tau}^{lag tau} E_a(-a/(1-a) u^a) du
 * (MF_int_series.cpp:523-530 MF_int_choice / 436-455 MF_int), evaluated as the
 * term-wise integrated ML series in long double.  Returns NaN when the series
 * would lose more than 6 digits to cancellation. */
double fho_ab_int(int lag, double tau, double alpha);

/* ------------------------------------------------------------ primitives */

/* S[p] = sum_{t=0}^{K-1} w[t] * (H[(t+1)*ld + p] - H[t*ld + p]),  p < P,
 * summed in ascending t like H_solver::Om1 (mt_psi_caputo.cpp:1315-1342). */
void fho_history_sum_layers(const double *H, int K, int ld, int P, const double *w, double *S);

/* Thomas sweep in the reference sign convention  A_i u_{i-1} - R_i u_i + B_i u_{i+1} = Om_i,
 * i = 1..N-1, u_0 = al1*u_1 + bt1 (H_solver::al1/bt1, mt_minimal.cpp:829-858,942-980).
 * right_mode 0: u_N = u_right (Dirichlet, H_solver::U1 bottom_cond 1, mt_minimal.cpp:1000-1006);
 * right_mode 1: u_N = Bt[N]/(1-Al[N]) (TG_solver::U1, fr_d_t_g_2d.cpp:2533).
 * Back substitution u_i = Al[i+1] u_{i+1} + Bt[i+1] for i = N-1..0, then u_{N+1} = u_N.
 * Arrays A,R,B,Om are indexed 0..N (entries 1..N-1 used); u has N+2 entries. */
void fho_thomas(int N, const double *A, const double *R, const double *B, const double *Om,
                double al1, double bt1, int right_mode, double u_right, double *u);

/* ------------------------------------------------------- 1D H_solver path */

enum { FHO_W_L1 = 0, FHO_W_PSI = 1 };
enum { FHO_K_CONST = 0, FHO_K_EXP = 1 };

typedef struct {
  int N;          /* intervals; nodes 0..N plus ghost N+1                        */
  double L;       /* domain length, dL = L/N                                      */
  double tau;     /* time step                                                    */
  double alpha;   /* time-derivative order                                        */
  int weights;    /* FHO_W_L1 (mt_minimal H_solver) or FHO_W_PSI (mt_psi_caputo)   */
  double beta;    /* psi(t) = t^beta for FHO_W_PSI                                */
  int kmodel;     /* FHO_K_CONST: K=kc ; FHO_K_EXP: K = kc*exp(kgam*u)            */
  double kc, kgam;
  double cinv;    /* constant 1/(dw/dh) multiplier                                */
  int gravity;    /* add (K(i)-K(i-1))/dL to the right part                       */
  double al_left, bt_left; /* u_0 = al_left*u_1 + bt_left                         */
  double u_right; /* Dirichlet value at node N                                    */
  double gamma;   /* space-derivative order (1: classical second derivative)      */
  double pert;    /* 0 for the reference's arithmetic; e > 0 multiplies every K_i and
                   * every history weight by 1 +- e (signs from a fixed hash of the
                   * node or slot and the step): the run measures how far rounding-
                   * level differences (another libm's exp or pow) move the solution */
} fho_h_params;

/* Runs `steps` calls of H_solver::calc_step (tstep starting at 1) on U (N+2 values,
 * updated in place).  hist must hold (steps)*(N+2) doubles; layer t is the
 * solution saved after step t+1, as the reference's oldH vector.
 * Returns 0 on success. */
int fho_h_solve(const fho_h_params *p, double *U, int steps, double *hist);

/* --------------------------------------------------- 2D TG_solver ADI path */

typedef struct {
  int sN, M;          /* grid: i = 0..sN, j = 0..M, array (sN+2) x (M+2), idx = i + j*(sN+2) */
  double tau, alpha, beta;
  double sigma;       /* porosity sigma                                     */
  double d;           /* fixed diffusion coefficient (fixed_d = 1)          */
  double C1;          /* x-sweep Dirichlet value at i = 0                   */
  double S;           /* constant source _S                                 */
  double dL, dLx;     /* steps in i (x-sweep) and j (y-sweep)               */
  int dt_alg;         /* 0 full history, 2 restricted summing, 3 series,
                         4 two-series approximation (psi = t)               */
  double dt_eps;      /* dt_alg 2: the sums stop at the first |weight| < eps;
                         dt_alg 3 (psi = t): number of series terms          */
  int massN;          /* mass exchange with a non-soluble phase (N1 stage)   */
  double massN_a, massN_b;
  int fixed_d;        /* 1: D = d; 0: D = lambda |v| ka0 / kk per node
                         (TG_solver_<func,0,0>, fr_d_t_g_2d.cpp:2787-2800)   */
  double lambda, ka0, kk;
} fho_tg_params;

/* Runs `steps` TG_solver::calc_step calls (fr_d_t_g_2d.cpp:2552-2718) with
 * dt_alg 0 or 2 (restricted summing: each history sum runs from the newest
 * layer pair back and stops at the first weight below dt_eps,
 * fr_d_t_g_2d.cpp:3356-3380) or 3 (series expansion, psi = t, dt_eps terms,
 * fr_d_t_g_2d.cpp:3384-3429) or 4 (two-series approximation, psi = t,
 * fr_d_t_g_2d.cpp:246-745 and 3438-3469), int_alg 1, massN 0, testing 0.
 * Returns 2 for dt_alg 3 or 4 with psi != t or dt_alg 3 with dt_eps < 1.  C is updated in place; V2 is |v|^2
 * per node.  work must hold (steps+1) full layers (the full-step layers; the
 * reference's half-step layers are never read by the dt_alg 0 sums except the
 * newest, which is C itself during the y sweep).  Returns 0 on success. */
int fho_tg_solve(const fho_tg_params *p, const double *V2, double *C, int steps, double *work);

/* dt_alg 4 bookkeeping alone: the numbers of long (ia) and short (ibk)
 * approximations per point after each of `steps` layers (offsets a, b). */
int fho_tg_two_series_counts(double alpha, int steps, double a, double b, int *nia, int *nibk);

/* dt_alg 4 sums alone for given layer differences F[r][p] (r = 0..nsteps,
 * F[0] unused): Vx[j][p], Vy[j][p] (j = 1..nsteps) = calc_va of block j - 1
 * with the x (1.5, 0.5) and y (2, 1) offsets, before the factor
 * Da tau^(1-alpha) / (1-alpha). */
int fho_two_series_sums(double alpha, int nsteps, int P, const double *F, double *Vx, double *Vy);

/* ------------------------------------------- 1D Atangana-Baleanu solve path */

/* solve_and_check (MF_int_series.cpp:875-958) with simple=1, quad=0:
 *   A C_{j-1} + Bd C_j + Cc C_{j+1} = Rp_j on m intervals, Dirichlet ends.
 * src(j, i) values are given as src[(i-1)*(m+1)+j] for steps i = 1..n;
 * left/right boundary values per step in bl[i-1], br[i-1].
 * w[lag] (lag = 1..n) are the lag weights I(lag); w[0] is the current-step
 * coefficient Ii = MF_int_choice(tau,tau,0) (mathematically I(1)); C (m+1) is updated in place.
 * If err != NULL, *err receives sum over steps of sum_j (C_j - exact)^2 / ((m+1) n)
 * with exact[(i-1)*(m+1)+j] (pass NULL exact to skip). */
int fho_ab_solve(int m, int n, double tau, double alpha, const double *w, const double *src,
                 const double *bl, const double *br, double *C, const double *exact, double *err);

#ifdef __cplusplus
}
#endif
#endif
