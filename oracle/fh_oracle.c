/*
 * fh_oracle.c -- CPU oracle (test infrastructure only; see fh_oracle.h).
 *
 * Plain C99 restatement of the reference solvers' hot path.  Nothing in the
 * CUDA product path links this file.  Loops follow the reference's order so
 * that results reproduce the reference to rounding; weights for psi != t and
 * the Atangana-Baleanu kernel are evaluated to convergence in long double.
 */
#include "fh_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ weights */

/* psi = t^beta interval weights (beta != 1), long double:
 *   int_{x0 tau}^{x1 tau} (T^beta - s^beta)^(-alpha) ds = T^(1-alpha beta)/beta [B(y1) - B(y0)],
 *   T = X tau, y = (x/X)^beta, B(y) = B(y; a, b) the lower incomplete beta, a = 1/beta, b = 1-alpha.
 * The difference of the two incomplete-beta values is evaluated directly, from
 * divided differences of its series, so that no leading digits cancel late in
 * a solve:
 *   lower side: B(y) = r P(y), r = x/X, P(y) = sum_j (1-b)_j y^j / (j! (a+j));
 *               B(y1) - B(y0) = (r1 - r0) P(y0) + r1 (y1 - y0) P[y0, y1]
 *   upper side: B(1) - B(y) = U(c) = c^b Q(c), c = 1 - y, Q(c) = sum_j (1-a)_j c^j / (j! (b+j));
 *               U(c0) - U(c1) = (c0^b - c1^b) Q(c1) + c0^b (c0 - c1) Q[c1, c0]
 * (P[u, v] = (P(v) - P(u)) / (v - u)).  This is the converged value of the
 * integral that H_solver::calc_int / _kb_row (mt_psi_caputo.cpp:497-564,
 * 720-741) sums as a series to global_eps. */

/* S = sum_j c_j z0^j, D = sum_j c_j h_{j-1}(z0, z1) with c_j = (p)_j / (j! (q+j)),
 * h_{j-1} = sum_{i<j} z0^i z1^(j-1-i) (so that D = the divided difference). */
static void ib_series_dd(long double p, long double q, long double z0, long double z1, long double *S,
                         long double *D) {
  long double s = 0.0L, d = 0.0L, c = 1.0L, pw = 1.0L, h = 0.0L;
  for (int j = 0; j < 4000; ++j) {
    const long double cj = c / (q + (long double)j);
    const long double ts = cj * pw, td = cj * h;
    s += ts;
    d += td;
    if (j > 2 && fabsl(ts) <= 1e-24L * fabsl(s) && fabsl(td) <= 1e-24L * fabsl(d)) break;
    h = z1 * h + pw;
    pw *= z0;
    c *= ((long double)j + p) / (long double)(j + 1);
    if (c == 0.0L) break;
  }
  *S = s;
  *D = d;
}

static long double ib_series(long double p, long double q, long double z) {
  long double S, D;
  ib_series_dd(p, q, z, z, &S, &D);
  return S;
}

double fho_psi_int(double x0, double x1, double X, double tau, double alpha, double beta) {
  if (beta == 1.0) {
    /* H_solver::_kb_row, branch g(t1) <= gtj (mt_psi_caputo.cpp:506-515): one term,
     * since inv_g_der(.,n>=2,.) == 0 for psi = t. */
    double t0 = tau * x0, t1 = tau * x1, gtj = tau * X;
    double v = gtj / gtj; /* inv_g_der(gtj,1,inv_g_der(gtj,0,1)) = der/t with der = t */
    v *= pow(gtj, 1 - alpha);
    double v3 = pow(fabs(1.0 - t1 / gtj), 1 - alpha);
    double v4 = pow(fabs(1.0 - t0 / gtj), 1 - alpha);
    double v2 = -(v3 - v4) / (1 - alpha);
    double sum = 0.0;
    sum += v2 * v;
    return sum;
  }
  const long double a = 1.0L / (long double)beta, b = 1.0L - (long double)alpha, be = (long double)beta;
  const long double Xl = X, r0 = (long double)x0 / Xl, r1 = (long double)x1 / Xl;
  const int zero0 = !(x0 > 0.0), top = !(x1 < X);
  /* beta log(x/X) and beta log(x1/x0); y1 - y0 without cancellation */
  const long double t1 = top ? 0.0L : be * log1pl(((long double)x1 - Xl) / Xl);
  const long double t0 = zero0 ? 0.0L : be * log1pl(((long double)x0 - Xl) / Xl);
  const long double td = zero0 ? 0.0L : be * log1pl(((long double)x1 - (long double)x0) / (long double)x0);
  const long double y1 = top ? 1.0L : expl(t1), y0 = zero0 ? 0.0L : expl(t0);
  const long double dy = zero0 ? y1 : y0 * expm1l(td);
  long double diff;
  if (y1 <= 0.55L) {
    long double S, D;
    ib_series_dd(1.0L - b, a, y0, y1, &S, &D);
    const long double dr = ((long double)x1 - (long double)x0) / Xl; /* not r1 - r0 */
    diff = zero0 ? r1 * ib_series(1.0L - b, a, y1) : dr * S + r1 * dy * D;
  } else if (y0 >= 0.45L) {
    const long double c1 = top ? 0.0L : -expm1l(t1), c0 = c1 + dy;
    if (c1 <= 0.0L) {
      diff = powl(c0, b) * ib_series(1.0L - a, b, c0);
    } else {
      long double S, D;
      ib_series_dd(1.0L - a, b, c1, c0, &S, &D);
      const long double c1b = powl(c1, b), dcb = c1b * expm1l(b * log1pl(dy / c1));
      diff = dcb * S + (c1b + dcb) * dy * D;
    }
  } else {
    /* the interval spans both sides (X of a few steps) */
    const long double btot = expl(lgammal(a) + lgammal(b) - lgammal(a + b));
    const long double c1 = top ? 0.0L : -expm1l(t1);
    const long double up = c1 <= 0.0L ? 0.0L : powl(c1, b) * ib_series(1.0L - a, b, c1);
    const long double lo = zero0 ? 0.0L : r0 * ib_series(1.0L - b, a, y0);
    diff = (btot - up) - lo;
  }
  long double T = Xl * (long double)tau;
  long double pre = powl(T, 1.0L - (long double)alpha * (long double)beta) / (long double)beta;
  return (double)(pre * diff);
}

double fho_l1_b(int k, double alpha) {
  /* mt_minimal.cpp:930: kv = pow(os-t, 1-alpha) - pow(os-t-1, 1-alpha) with k = os-t-1 */
  return pow((double)(k + 1), 1.0 - alpha) - pow((double)k, 1.0 - alpha);
}

double fho_mittag_leffler(double a, double b, double z) {
  long double s = 0.0L, mx = 0.0L;
  long double lz = logl(fabsl((long double)z));
  for (int k = 0; k < 5000; ++k) {
    long double p = (long double)a * k + (long double)b;
    long double t;
    if (z == 0.0) {
      t = (k == 0) ? 1.0L / tgammal(p) : 0.0L;
    } else {
      t = expl((long double)k * lz - lgammal(p));
      if (z < 0.0 && (k & 1)) t = -t;
      /* 1/Gamma(p) changes sign for p < 0 only; p > 0 here for a, b > 0 */
    }
    s += t;
    if (fabsl(t) > mx) mx = fabsl(t);
    if (k > 4 && fabsl(t) <= 1e-24L * fabsl(s) && fabsl(t) < mx) break;
  }
  if (s != 0.0L && mx / fabsl(s) > 1e6L) return NAN;
  return (double)s;
}

double fho_ab_int(int lag, double tau, double alpha) {
  /* I(lag) = sum_k (-lam)^k / Gamma(a k + 2) * (x1^(a k + 1) - x0^(a k + 1)),
   * lam = a/(1-a), x1 = lag*tau, x0 = (lag-1)*tau: the ML series of
   * MF_int (MF_int_series.cpp:436-455) integrated term by term. */
  long double a = alpha, lam = a / (1.0L - a);
  long double x1 = (long double)lag * (long double)tau;
  long double lx1 = logl(x1), llam = logl(lam);
  long double lr = (lag >= 2) ? log1pl(-1.0L / (long double)lag) : 0.0L;
  long double s = 0.0L, mx = 0.0L;
  for (int k = 0; k < 5000; ++k) {
    long double p = a * k + 1.0L;
    long double frac = (lag >= 2) ? -expm1l(p * lr) : 1.0L; /* 1 - (x0/x1)^p */
    long double mag = expl((long double)k * llam + p * lx1 - lgammal(p + 1.0L));
    long double t = mag * frac;
    if (k & 1) t = -t;
    s += t;
    if (fabsl(t) > mx) mx = fabsl(t);
    if (k > 4 && fabsl(t) <= 1e-24L * fabsl(s) && fabsl(t) < mx) break;
  }
  if (s == 0.0L || mx / fabsl(s) > 1e6L) return NAN;
  return (double)s;
}

/* --------------------------------------------------------------- primitives */

void fho_history_sum_layers(const double *H, int K, int ld, int P, const double *w, double *S) {
  for (int p = 0; p < P; ++p) {
    double ts = 0.0;
    for (int t = 0; t < K; ++t) ts += w[t] * (H[(size_t)(t + 1) * ld + p] - H[(size_t)t * ld + p]);
    S[p] = ts;
  }
}

void fho_thomas(int N, const double *A, const double *R, const double *B, const double *Om,
                double al1, double bt1, int right_mode, double u_right, double *u) {
  double *Al = (double *)malloc(sizeof(double) * (size_t)(N + 2));
  double *Bt = (double *)malloc(sizeof(double) * (size_t)(N + 2));
  Al[1] = al1;
  Bt[1] = bt1;
  for (int i = 1; i < N; ++i) Al[i + 1] = B[i] / (R[i] - A[i] * Al[i]);
  for (int i = 1; i < N; ++i) {
    if (Al[i + 1] == 0.0 && B[i] == 0.0)
      Bt[i + 1] = (A[i] * Bt[i] - Om[i]) / (R[i] - A[i] * Al[i]);
    else
      Bt[i + 1] = (Al[i + 1] / B[i]) * (A[i] * Bt[i] - Om[i]);
  }
  u[N] = right_mode == 0 ? u_right : Bt[N] / (1.0 - Al[N]);
  for (int i = N - 1; i >= 0; --i) u[i] = Al[i + 1] * u[i + 1] + Bt[i + 1];
  u[N + 1] = u[N];
  free(Al);
  free(Bt);
}

/* ------------------------------------------------------- 1D H_solver path */

/* The space-fractional part of H_solver::Om1 (gamma < 1): V_i = calc_v of the
 * first differences F_j = U_{j+1} - U_j, j = 0..i-1 (mt_minimal.cpp:228-271,
 * mt_psi_caputo.cpp:749-777 with with_zero = 1): mt_minimal weighs F_j by
 * (i-j+1)^A - (i-j)^A, mt_psi_caputo by A kb_space[i][j-1] (j >= 1) or
 * A kb_space[i+1][0] (j = 0), kb_space[a][t0] = calc_int(gamma, t0, t0+1, a,
 * dL, 0) (1461-1472; psi = x in space), A = 1 - gamma.  V_0 = 0. */
static void h_space_v(const fho_h_params *p, int N, double dL, const double *U, double *F, double *V) {
  const double A = 1.0 - p->gamma;
  for (int i = 1; i < N; ++i) F[i] = U[i + 1] - U[i];
  F[0] = U[1] - U[0];
  V[0] = 0.0;
  for (int i = 1; i < N; ++i) {
    double v = 0.0;
    for (int j = 0; j <= i - 1; ++j) {
      double kv;
      if (p->weights == FHO_W_L1)
        kv = pow((double)i - (double)j + 1, A) - pow((double)i - (double)j, A);
      else if (j != 0)
        kv = A * fho_psi_int(j - 1, j, i, dL, p->gamma, 1.0);
      else
        kv = A * fho_psi_int(0, 1, i + 1, dL, p->gamma, 1.0);
      v += kv * F[j];
    }
    V[i] = v;
  }
}

/* +1 or -1 from a hash of (i, t): the sign pattern of fho_h_params.pert. */
static double pert_sign(unsigned i, unsigned t) {
  unsigned long long h = (i + 1ULL) * 0x9E3779B97F4A7C15ULL ^ (t + 1ULL) * 0xC2B2AE3D27D4EB4FULL;
  h ^= h >> 29;
  h *= 0xBF58476D1CE4E5B9ULL;
  h ^= h >> 32;
  return (h & 1ULL) ? 1.0 : -1.0;
}

int fho_h_solve(const fho_h_params *p, double *U, int steps, double *hist) {
  if (!(p->gamma > 0.0 && p->gamma <= 1.0)) return 2; /* gamma in (0, 1] */
  const int N = p->N, ld = N + 2;
  const double dL = p->L / N;
  const int frac = p->gamma != 1.0;
  /* reset_D: mt_minimal.cpp:744-749 Dg = dL^(-1-gamma)/Gamma(2-gamma);
   * mt_psi_caputo.cpp:1176-1181 Dg = dL^-2/Gamma(2-gamma) with the factor
   * kb(gamma, i-1, i, i) (1-gamma) in A_, B, R (1164-1175) */
  const double Dg = !frac ? pow(dL, -2.0)
                          : (p->weights == FHO_W_L1 ? pow(dL, -1.0 - p->gamma) : pow(dL, -2.0)) / tgamma(2.0 - p->gamma);
  const double a = p->alpha;
  /* reset_D: mt_minimal.cpp:744-749 (tau^-a) / mt_psi_caputo.cpp:1176-1181 (tau^-1) */
  const double Da = (p->weights == FHO_W_L1) ? pow(p->tau, -a) / tgamma(2.0 - a)
                                             : pow(p->tau, -1.0) / tgamma(2.0 - a);
  double *K = (double *)malloc(sizeof(double) * ld);
  double *Ac = (double *)malloc(sizeof(double) * ld);
  double *Bc = (double *)malloc(sizeof(double) * ld);
  double *Rc = (double *)malloc(sizeof(double) * ld);
  double *Om = (double *)malloc(sizeof(double) * ld);
  double *w = (double *)malloc(sizeof(double) * (size_t)(steps + 2));
  double *F = (double *)malloc(sizeof(double) * ld), *V = (double *)malloc(sizeof(double) * ld);
  if (!K || !Ac || !Bc || !Rc || !Om || !w || !F || !V) return 1;
  int nsaved = 0;
  for (int tstep = 1; tstep <= steps; ++tstep) {
    const int os = nsaved;
    double wc;
    if (p->weights == FHO_W_L1) {
      wc = 1.0;
      for (int t = 0; t < os - 1; ++t)
        w[t] = pow((double)(os - t), 1.0 - a) - pow((double)(os - t - 1), 1.0 - a);
    } else {
      /* kb_time[aa] = calc_int(alpha, aa, aa+1, tstep+1, tau, 1)  (mt_psi_caputo.cpp:1481-1489) */
      wc = fho_psi_int(tstep, tstep + 1, tstep + 1, p->tau, a, p->beta) * (1 - a);
      for (int t = 0; t < os - 1; ++t) w[t] = fho_psi_int(t, t + 1, tstep + 1, p->tau, a, p->beta) * (1 - a);
    }
    for (int i = 0; i <= N; ++i) K[i] = (p->kmodel == FHO_K_CONST) ? p->kc : p->kc * exp(p->kgam * U[i]);
    if (p->pert != 0.0) {
      for (int i = 0; i <= N; ++i) K[i] *= 1.0 + p->pert * pert_sign((unsigned)i, (unsigned)tstep);
      for (int t = 0; t < os - 1; ++t) w[t] *= 1.0 + p->pert * pert_sign((unsigned)t + 100000u, (unsigned)tstep);
    }
    if (frac) h_space_v(p, N, dL, U, F, V);
    for (int i = 1; i < N; ++i) {
      const double kbf = (frac && p->weights == FHO_W_PSI) ? fho_psi_int(i - 1, i, i, dL, p->gamma, 1.0) : 1.0;
      const double g1 = frac ? 1.0 - p->gamma : 1.0;
      Ac[i] = Dg * K[i - 1] * p->cinv;
      Bc[i] = Dg * K[i + 1] * p->cinv;
      Rc[i] = p->cinv * (K[i + 1] + K[i - 1]) * Dg;
      if (frac && p->weights == FHO_W_PSI) {
        Ac[i] = Ac[i] * kbf * g1;
        Bc[i] = Bc[i] * kbf * g1;
        Rc[i] = Rc[i] * kbf * g1;
      }
      Rc[i] += Da * wc;
      Om[i] = -Da * wc * U[i];
      if (frac) Om[i] = -Dg * p->cinv * (K[i] * V[i] - K[i - 1] * V[i - 1]) - Da * wc * U[i];
      if (p->gravity) Om[i] += (K[i] - K[i - 1]) / dL; /* (KK(p)-KK(p-1))/dL, mt_minimal.cpp:904 */
      double ts = 0.0;
      if (os >= 2) {
        /* The reference walks `double **oldp = &old[0][1]` with prev = oldp[0][id]
         * (mt_minimal.cpp:913-917, mt_psi_caputo.cpp:1321-1326): term t reads
         * cur = layer[t+1] against the previous read, i.e. w[t]*(layer[t+1]-layer[t])
         * for t >= 1, while the t = 0 term is layer[1]-layer[1] = 0.  The oldest
         * difference layer[1]-layer[0] therefore never enters the sum. */
        const double *oldp = hist + (size_t)1 * ld;
        double prev = oldp[i];
        for (int t = 0; t < os - 1; ++t, oldp += ld) {
          double cur = oldp[i];
          ts += w[t] * (cur - prev);
          prev = cur;
        }
      }
      Om[i] += Da * ts;
    }
    fho_thomas(N, Ac, Rc, Bc, Om, p->al_left, p->bt_left, 0, p->u_right, U);
    memcpy(hist + (size_t)os * ld, U, sizeof(double) * ld);
    nsaved++;
  }
  free(K); free(Ac); free(Bc); free(Rc); free(Om); free(w); free(F); free(V);
  return 0;
}

/* --------------------------------------------------- 2D TG_solver ADI path */

/* One x line (dir 0, line jj) or y line (dir 1, line ii) of TG_solver::calc_step. */
/* D of TG_solver_::D (fr_d_t_g_2d.cpp:2787-2800): d, or with fixed_d = 0 and
 * kform 0 lambda |v| (ka[0] / k) at the node. */
static double tg_D(const fho_tg_params *p, const double *V2, size_t id) {
  if (p->fixed_d) return p->d;
  const double v = sqrt(V2[id]);
  const double k_ = p->ka0 / p->kk;
  return p->lambda * v * k_;
}

static void tg_line(const fho_tg_params *p, const double *V2, double *C, const double *work, int j, int dir, int line,
                    double kcur, double kyh, const double *wk, const double *hs, const double *Nn, const double *Np,
                    double *A, double *B, double *R, double *Om, double *u) {
  const int sN = p->sN, M = p->M, ld = sN + 2;
  const size_t P = (size_t)(sN + 2) * (M + 2);
  const double st = p->sigma / p->tau;
  const int N = dir == 0 ? sN : M;
  const double dl = dir == 0 ? p->dL : p->dLx;
  const size_t step = dir == 0 ? 1 : (size_t)ld;  /* neighbour along the line */
  for (int i = 1; i < N; ++i) {
    const size_t id = dir == 0 ? (size_t)i + (size_t)line * ld : (size_t)line + (size_t)i * ld;
    /* A_ and B (3242-3257): D(i-1) + D(i) and D(i+1) + D(i) */
    const double Dm = tg_D(p, V2, id - step), Dc = tg_D(p, V2, id), Dp = tg_D(p, V2, id + step);
    if (dir == 0) {
      A[i] = (V2[id] / dl) * ((0.5 * (Dm + Dc) / dl) + 0.5);
      B[i] = (V2[id] / dl) * ((0.5 * (Dp + Dc) / dl) - 0.5);
    } else {
      A[i] = (V2[id] / (dl * dl)) * 0.5 * (Dm + Dc);
      B[i] = (V2[id] / (dl * dl)) * 0.5 * (Dp + Dc);
    }
    R[i] = st * (kcur + 0.0) + A[i] + B[i];
    Om[i] = -st * (kcur + 0.0) * C[id];
    Om[i] += p->S * 0.5;
    if (Nn) Om[i] += (1.0 / p->tau) * (Nn[id] - Np[id]); /* mass exchange (3330-3332) */
    double ts = 0.0;
    if (hs) /* dt_alg 3: the series value of this step */
      ts = hs[id];
    else if (2 * j + 1 + dir >= 3)
      for (int k = j - 1; k >= 0; --k) {
        if (p->dt_alg == 2 && fabs(wk[k]) < p->dt_eps) break; /* restricted summing (3364-3380) */
        ts += wk[k] * (work[(size_t)(k + 1) * P + id] - work[(size_t)k * P + id]);
      }
    /* y half-step term with the reference's operand order old[size-2]-old[size-1] (3479-3481) */
    if (dir == 1) ts += (kyh + 0.0) * (work[(size_t)j * P + id] - C[id]);
    Om[i] += st * ts;
  }
  for (int i = 0; i <= N + 1; ++i)
    u[i] = C[dir == 0 ? (size_t)i + (size_t)line * ld : (size_t)line + (size_t)i * ld];
  fho_thomas(N, A, R, B, Om, dir == 0 ? 0.0 : 1.0, dir == 0 ? p->C1 : 0.0, 1, 0.0, u);
  for (int i = 0; i <= N + 1; ++i)
    C[dir == 0 ? (size_t)i + (size_t)line * ld : (size_t)line + (size_t)i * ld] = u[i];
}

/* dt_alg 3, psi = t (fr_d_t_g_2d.cpp:3384-3429 with _kb_row2 2965-3040 and
 * _kb_row2_fixed_coefs 3041-3057, dt_eps = J terms): per point the series
 * accumulators H[n] = sum_t int_{t tau}^{(t+1) tau} s^n ds (C^{t+1} - C^t)
 * gain the newest layer pair each step (the x and y sums of the reference
 * keep two equal copies), and the history sum at time gtj is
 * Da sum_n (alpha)_n / n! gtj^(-alpha-n) H[n], cut at the first non-finite
 * coefficient. */
static void tg_series_add(const fho_tg_params *p, int J, int j, size_t P, const double *dnew, const double *dold,
                          double *H) {
  const double t0 = p->tau * (double)(j - 1), t1 = p->tau * (double)j; /* interval j-1 */
  double v6 = t0 / t1, mult = t1;
  for (int n = 0; n < J; ++n) {
    double v3;
    if (n == 0) {
      v3 = (t1 - t0) / t1;
    } else {
      v6 *= t0 / t1;
      v3 = 0.0 + 1.0 * ((1.0 / (n + 1.0)) * (1 - v6)); /* inv_g_der(t1, 1, t1) = 1 for psi = t */
    }
    const double c = mult * v3;
    for (size_t id = 0; id < P; ++id) H[(size_t)n * P + id] += c * (dnew[id] - dold[id]);
    mult *= t1;
  }
}

static void tg_series_eval(const fho_tg_params *p, int J, double gtj, size_t P, const double *H, double Da,
                           double *out) {
  const double a = p->alpha;
  for (size_t id = 0; id < P; ++id) out[id] = 0.0;
  double v1 = pow(gtj, -a), i = 0.0;
  for (int n = 0; n < J; ++n) {
    for (size_t id = 0; id < P; ++id) out[id] += v1 * H[(size_t)n * P + id];
    i += 1.0;
    v1 *= -(-a - i + 1.0) / (i * gtj);
    if (!isfinite(v1)) break;
  }
  for (size_t id = 0; id < P; ++id) out[id] = Da * out[id];
}

/* dt_alg 4, psi = t: two-series approximation of the history sums
 * (fr_d_t_g_2d.cpp:246-745, used by TG_solver_::Om1 3438-3469).  Per point
 * the sum S(x) = sum_r g(x, r) F[r], g(x, r) = (x - r + a)^A - (x - r + b)^A,
 * A = 1 - alpha, F[r] = C^r - C^(r-1) (the full-step differences H42), is
 * carried by
 *   "ia" approximations   sum_k c_k x^(A-k)       valid for x >= min
 *     (binomial series of g in 1/x; fr_d_t_g_2d.cpp:265-333), and
 *   "ibk" approximations  sum_k c_k (x - b)^k     valid for min <= x <= max
 *     (Taylor series of g around b; 351-471),
 * whose coefficients are linear in F.  calc_va (477-745) evaluates the sum at
 * x = block + 1 from the approximations plus the newest term directly, then
 * folds F[block + 1] into them, creating, splitting and retiring
 * approximations so that each stays within approx_eps = 1e-7 of its share.
 * The ranges depend on A, a, b and the block only, not on F.  Integer time
 * grid (Ts = NULL), one layer per block (bs = 1), as the solver calls it. */
#define TA_AK 10
#define TA_MAXAK 20
static const double ta_approx_eps = 1e-7, ta_eps = 1e-9;

typedef struct {
  double min;
  int nterms;
  double c[TA_MAXAK];
} ta_ia;
typedef struct {
  double min, max, b;
  int nterms, old;
  double c[TA_MAXAK];
} ta_ibk;
typedef struct {
  ta_ia *ia;
  ta_ibk *ibk;
  int nia, cia, nibk, cibk;
} ta_set;

/* prod_{i=1}^{n-1} (A - i + 1) / i in the reference's order */
static double ta_ak(double A, int n) {
  double ak = 1;
  for (int i = 1; i < n; i++) ak *= (A - i + 1) / i;
  return ak;
}

/* ia_mini (fr_d_t_g_2d.cpp:255-266) */
static double ta_ia_mini(double A, double r, int nterms, double a, double b) {
  const double ak = ta_ak(A, nterms);
  return pow(fabs(ak * (pow(a - r, (double)nterms) - pow(b - r, (double)nterms)) / ta_approx_eps),
             1.0 / (nterms - A));
}

/* ibk_i2 (fr_d_t_g_2d.cpp:337-371), Ts = NULL, step = -1 */
static double ta_ibk_i2(double A, double r, double b, int nterms, double a, double c) {
  const double ak = ta_ak(A, nterms);
  if (fabs(b - r) < 1e-10) return pow(fabs(ta_approx_eps / ak), 1.0 / nterms);
  const double p1 = pow((a + b - r), A) / pow((a + b - r), nterms);
  const double p2 = pow((c + b - r), A) / pow((c + b - r), nterms);
  return pow(fabs(ta_approx_eps / (ak * (p1 - p2))), 1.0 / nterms);
}

/* ia_approximation(A, rmin, rmax, F, NULL, cmin, nt, a, b) (285-314) */
static ta_ia ta_ia_make(double A, double rmin, double rmax, const double *F, double cmin, int nt, double a,
                        double b) {
  ta_ia q;
  double ak = 1;
  q.c[0] = 0;
  for (int i = 1; i < nt; i++) {
    ak *= (A - i + 1) / i;
    double krk = 0.0;
    for (int j = (int)rmin; j < rmax; j++) krk += F[j] * (pow(a - (double)j, (double)i) - pow(b - (double)j, (double)i));
    q.c[i] = ak * krk;
  }
  for (int i = nt; i < TA_MAXAK; i++) q.c[i] = 0.0;
  q.min = cmin != -1 ? cmin : ceil(ta_ia_mini(A, rmax, nt, a, b));
  if (!isfinite(q.min)) q.min = rmax;
  q.nterms = nt;
  return q;
}

static double ta_ia_calc(const ta_ia *q, double A, double x) {
  double ret = 0.0;
  for (int i = 0; i < q->nterms; i++) ret += q->c[i] * pow(x, A - (double)i);
  return ret;
}

/* ibk_approximation(A, rmin, rmax, F, NULL, b, i2, nt, a, _b) (401-436) */
static ta_ibk ta_ibk_make(double A, double rmin, double rmax, const double *F, double b, double i2, int nt,
                          double a, double _b) {
  ta_ibk q;
  double ak = 1;
  q.b = b;
  for (int i = 0; i < nt; i++) {
    if (i != 0) ak *= (A - i + 1) / i;
    double krk = 0.0;
    for (int j = (int)rmin; j < rmax; j++)
      krk += F[j] * (pow(a + b - (double)j, A - (double)i) - pow(_b + b - (double)j, A - (double)i));
    q.c[i] = ak * krk;
  }
  for (int i = nt; i < TA_MAXAK; i++) q.c[i] = 0.0;
  q.min = i2 != -1 ? i2 : b - floor(ta_ibk_i2(A, rmax, b, nt, a, _b));
  q.max = b;
  q.nterms = nt;
  q.old = 0;
  return q;
}

static double ta_ibk_calc(const ta_ibk *q, double x) {
  double ret = 0.0, xbk = 1;
  for (int i = 0; i < q->nterms; i++) {
    ret += q->c[i] * xbk;
    xbk *= (x - q->b);
  }
  return ret;
}

static void ta_push_ibk(ta_set *S, ta_ibk q) {
  if (S->nibk == S->cibk) {
    S->cibk = S->cibk ? 2 * S->cibk : 16;
    S->ibk = (ta_ibk *)realloc(S->ibk, sizeof(ta_ibk) * (size_t)S->cibk);
  }
  S->ibk[S->nibk++] = q;
}
static void ta_push_ia(ta_set *S, ta_ia q) {
  if (S->nia == S->cia) {
    S->cia = S->cia ? 2 * S->cia : 4;
    S->ia = (ta_ia *)realloc(S->ia, sizeof(ta_ia) * (size_t)S->cia);
  }
  S->ia[S->nia++] = q;
}
static void ta_erase_ibk(ta_set *S, int j) {
  memmove(S->ibk + j, S->ibk + j + 1, sizeof(ta_ibk) * (size_t)(S->nibk - j - 1));
  S->nibk--;
}

/* A series of short approximations of the current layer covering [rr, upto]:
 * centres b found by the fixed point b = rr + i2(r, b) + 1 (the loops of
 * steps 2, 3 and 5 of calc_va); r2 is the r argument of ibk_i2. */
static double ta_series(ta_set *S, double A, int block, const double *F, double rr, double r2, double upto,
                        int cap, double a, double _b, int cmp_ceil) {
  double bb0 = rr, bb = rr;
  do {
    bb = rr + 1;
    do {
      bb0 = bb;
      bb = rr + ta_ibk_i2(A, r2, bb, TA_AK, a, _b) + 1;
    } while ((bb - bb0) > ta_eps);
    if (!isfinite(bb)) {
      bb = bb0;
      if (!isfinite(bb)) bb = rr;
    }
    ta_ibk q = ta_ibk_make(A, block + 1, block + 2, F, floor(bb), rr, TA_AK, a, _b);
    rr = floor(bb) + 1;
    if (cap && floor(bb) > upto) q.max = upto;
    ta_push_ibk(S, q);
  } while (floor(bb) < (cmp_ceil ? ceil(upto) : upto));
  return rr;
}

/* calc_va(A, 1, block, F, &V, NULL, ias, ibks, a, _b) (fr_d_t_g_2d.cpp:477-745) */
static double ta_calc_va(ta_set *S, double A, int block, const double *F, double a, double _b) {
  const double rmax = (double)(block + 2);
  const int rmaxidx = block + 2;
  double V = 0.0;
  if (A == 0.0) return V;
  {
    const int i = block + 1;
    const double ii = i;
    for (int j = 0; j < S->nia; j++)
      if (ii >= S->ia[j].min) V += ta_ia_calc(&S->ia[j], A, ii);
    for (int j = 0; j < S->nibk; j++)
      if ((ii >= S->ibk[j].min) && (ii <= S->ibk[j].max)) V += ta_ibk_calc(&S->ibk[j], ii);
    double v = 0.0;
    for (int j = block + 1; j <= i; j++) v += (pow((double)i - (double)j + a, A) - pow((double)i - (double)j + _b, A)) * F[j];
    V += v;
  }
  /* 1) retire short approximations that end before rmax */
  for (int j = 0; j < S->nibk; j++)
    if (S->ibk[j].max < rmax) {
      ta_erase_ibk(S, j);
      j--;
    }
  /* 2) fold the layer into the short approximations ahead of it; split those
   * the new layer's series cannot cover with MAXAK terms */
  int ss = S->nibk;
  for (int j = 0; j < ss; j++)
    if (S->ibk[j].min >= rmax && S->ibk[j].old == 0) {
      int spl = 0;
      ta_ibk i2;
      ta_ibk bibk = ta_ibk_make(A, block + 1, block + 2, F, S->ibk[j].b, -1.0, TA_AK, a, _b);
      if (bibk.min > S->ibk[j].min) {
        int t;
        for (t = TA_AK; t < TA_MAXAK; t++)
          if ((S->ibk[j].b - ta_ibk_i2(A, rmaxidx, S->ibk[j].b, t, a, _b)) < S->ibk[j].min) break;
        if (t == TA_MAXAK)
          spl = 1;
        else
          bibk = ta_ibk_make(A, block + 1, block + 2, F, S->ibk[j].b, -1.0, t, a, _b);
        if (spl) i2 = S->ibk[j];
      }
      for (int i = 0; i < bibk.nterms; i++) S->ibk[j].c[i] += bibk.c[i];
      if (S->ibk[j].nterms < bibk.nterms) S->ibk[j].nterms = bibk.nterms;
      if (spl && bibk.min > S->ibk[j].min) {
        i2.max = ceil(bibk.min);
        S->ibk[j].min = i2.max + 1;
        i2.old = 1;
        if (S->ibk[j].min > S->ibk[j].max) {
          i2.max = S->ibk[j].max;
          ta_erase_ibk(S, j);
          j--;
          ss--;
        }
        ta_push_ibk(S, i2);
        ta_series(S, A, block, F, i2.min, i2.min, i2.max, 1, a, _b, 0);
      }
    }
  /* 3) new short approximations of this layer for the range of the newest
   * approximation that straddles rmax */
  double bm1 = -1;
  for (int j = 0; j < S->nibk; j++)
    if (S->ibk[j].max >= rmax && S->ibk[j].min < rmax && S->ibk[j].max > bm1 && S->ibk[j].old == 0) {
      bm1 = S->ibk[j].max;
      S->ibk[j].old = 1;
    }
  if (bm1 != -1) {
    for (int j = 0; j < S->nibk; j++)
      if (S->ibk[j].max < bm1) S->ibk[j].old = 1;
    ta_series(S, A, block, F, rmax, rmaxidx, bm1, 1, a, _b, 0);
  }
  /* 4) the long approximation of this layer joins the newest one when it is
   * valid from an earlier point */
  ta_ia bia = ta_ia_make(A, block + 1, block + 2, F, -1, TA_AK, a, _b);
  if (S->nia && bia.min < S->ia[S->nia - 1].min) {
    ta_ia *last = &S->ia[S->nia - 1];
    for (int i = 0; i < bia.nterms; i++) last->c[i] += bia.c[i];
    if (last->nterms < bia.nterms) last->nterms = bia.nterms;
    return V;
  }
  /* 5) otherwise short approximations bridge to its minimum and it is added */
  bm1 = rmax;
  for (int j = 0; j < S->nibk; j++)
    if ((S->ibk[j].max + 1) > bm1) bm1 = S->ibk[j].max + 1;
  bia.min = ta_series(S, A, block, F, bm1, rmaxidx, bia.min, 0, a, _b, 1);
  ta_push_ia(S, bia);
  return V;
}

static void ta_free(ta_set *S) {
  free(S->ia);
  free(S->ibk);
  memset(S, 0, sizeof(*S));
}

int fho_two_series_sums(double alpha, int nsteps, int P, const double *F, double *Vx, double *Vy) {
  for (int p = 0; p < P; ++p) {
    ta_set sx, sy;
    memset(&sx, 0, sizeof(sx));
    memset(&sy, 0, sizeof(sy));
    double *Fi = (double *)malloc(sizeof(double) * (size_t)(nsteps + 1));
    if (!Fi) return 1;
    for (int r = 0; r <= nsteps; ++r) Fi[r] = F[(size_t)r * P + p];
    for (int j = 1; j <= nsteps; ++j) {
      Vx[(size_t)j * P + p] = ta_calc_va(&sx, 1.0 - alpha, j - 1, Fi, 1.5, 0.5);
      Vy[(size_t)j * P + p] = ta_calc_va(&sy, 1.0 - alpha, j - 1, Fi, 2.0, 1.0);
    }
    free(Fi);
    ta_free(&sx);
    ta_free(&sy);
  }
  return 0;
}

int fho_tg_two_series_counts(double alpha, int steps, double a, double b, int *nia, int *nibk) {
  ta_set S;
  memset(&S, 0, sizeof(S));
  double *F = (double *)calloc((size_t)steps + 2, sizeof(double));
  if (!F) return 1;
  for (int r = 0; r < steps + 2; ++r) F[r] = 1.0;
  for (int blk = 0; blk < steps; ++blk) {
    ta_calc_va(&S, 1.0 - alpha, blk, F, a, b);
    nia[blk] = S.nia;
    nibk[blk] = S.nibk;
  }
  ta_free(&S);
  free(F);
  return 0;
}

int fho_tg_solve(const fho_tg_params *p, const double *V2, double *C, int steps, double *work) {
  const int sN = p->sN, M = p->M;
  const size_t P = (size_t)(sN + 2) * (M + 2);
  const int nmax = (sN > M ? sN : M) + 2;
  const double a = p->alpha;
  const double Da = 1.0 / tgamma(1.0 - a); /* TG_solver ctor, fr_d_t_g_2d.cpp:2391-2394 */
  double *wx = (double *)malloc(sizeof(double) * (size_t)(steps + 1));
  double *wy = (double *)malloc(sizeof(double) * (size_t)(steps + 1));
  if (!wx || !wy) return 1;
  const int J = p->dt_alg == 3 ? (int)p->dt_eps : 0;
  if (p->dt_alg == 3 && (J < 1 || p->beta != 1.0)) return 2;
  if (p->dt_alg == 4 && p->beta != 1.0) return 2;
  /* mass exchange: N starts at 0 (TG_solver::initial) */
  double *Nn = p->massN ? (double *)calloc(P, sizeof(double)) : NULL;
  double *Np = p->massN ? (double *)calloc(P, sizeof(double)) : NULL;
  if (p->massN && (!Nn || !Np)) return 1;
  /* dt_alg 4: per point the approximations of the x and y sums (Happ1 with
   * offsets (1.5, 0.5), Happ2 with (2, 1); fr_d_t_g_2d.cpp:3444-3462) */
  ta_set *tax = NULL, *tay = NULL;
  double *F4 = NULL;
  if (p->dt_alg == 4) {
    tax = (ta_set *)calloc(P, sizeof(ta_set));
    tay = (ta_set *)calloc(P, sizeof(ta_set));
    F4 = (double *)calloc((size_t)(steps + 2) * P, sizeof(double));
    if (!tax || !tay || !F4) return 1;
  }
  double *H = J ? (double *)calloc((size_t)J * P, sizeof(double)) : NULL;
  const int hs_on = J || p->dt_alg == 4;
  double *hx = hs_on ? (double *)malloc(sizeof(double) * P) : NULL, *hy = hs_on ? (double *)malloc(sizeof(double) * P) : NULL;
  if (hs_on && (!hx || !hy)) return 1;
  if (J && !H) return 1;
  memcpy(work, C, sizeof(double) * P); /* full-step layer 0 (TG_solver::initial) */
#define KB(s, ja, sa, l) (Da * fho_psi_int((double)(s) + (sa), (double)(s) + (sa) + (l), (double)j + (ja), p->tau, a, p->beta))
  for (int j = 0; j < steps; ++j) {
    /* weights of TG_solver_::kb (fr_d_t_g_2d.cpp:3059-3239), dt_alg 0 */
    const double kx = KB(j, 0.5, 0.0, 0.5), ky = KB(j, 1.0, 0.5, 0.5), kyh = KB(j, 1.0, 0.0, 0.5);
    for (int k = 0; k < j; ++k) { wx[k] = KB(k, 0.5, 0.0, 1.0); wy[k] = KB(k, 1.0, 0.0, 1.0); }
    const double *hsx = NULL, *hsy = NULL;
    if (J && j >= 1) {
      tg_series_add(p, J, j, P, work + (size_t)j * P, work + (size_t)(j - 1) * P, H);
      tg_series_eval(p, J, p->tau * ((double)j + 0.5), P, H, Da, hx);
      tg_series_eval(p, J, p->tau * ((double)j + 1.0), P, H, Da, hy);
      hsx = hx;
      hsy = hy;
    }
    if (p->dt_alg == 4 && j >= 1) {
      /* F4[id][r] = C^r - C^(r-1) for the newest r = j; both sums at x = j */
      const double A = 1.0 - a, sc = Da * (pow(p->tau, 1.0 - a) / (1.0 - a));
#pragma omp parallel for schedule(static)
      for (size_t id = 0; id < P; ++id) {
        double *Fi = F4 + id * (size_t)(steps + 2);
        Fi[j] = work[(size_t)j * P + id] - work[(size_t)(j - 1) * P + id];
        hx[id] = ta_calc_va(&tax[id], A, j - 1, Fi, 1.5, 0.5) * sc;
        hy[id] = ta_calc_va(&tay[id], A, j - 1, Fi, 2.0, 1.0) * sc;
      }
      hsx = hx;
      hsy = hy;
    }
    /* x half-step: lines jj = 1..M-1 (fr_d_t_g_2d.cpp:2577-2590); y half-step: lines
     * ii = 1..sN-1 (2634-2648).  Lines are independent, so they run in parallel. */
    for (int dir = 0; dir < 2; ++dir) {
      const int nlines = dir == 0 ? M : sN;
      if (Nn) /* N1 before each half step (2503-2521): nodes i <= sN, j <= M */
        for (int jj = 0; jj <= M; ++jj)
          for (int ii = 0; ii <= sN; ++ii) {
            const size_t id = (size_t)ii + (size_t)jj * (sN + 2);
            Np[id] = Nn[id];
            Nn[id] = (1.0 / (2.0 + p->tau * p->massN_a * p->massN_b)) *
                     (2 * Np[id] + p->tau * p->sigma * p->massN_b * C[id]);
          }
#pragma omp parallel
      {
        double *A = (double *)malloc(sizeof(double) * nmax), *B = (double *)malloc(sizeof(double) * nmax);
        double *R = (double *)malloc(sizeof(double) * nmax), *Om = (double *)malloc(sizeof(double) * nmax);
        double *u = (double *)malloc(sizeof(double) * nmax);
#pragma omp for schedule(static)
        for (int line = 1; line < nlines; ++line)
          tg_line(p, V2, C, work, j, dir, line, dir == 0 ? kx : ky, kyh, dir == 0 ? wx : wy, dir == 0 ? hsx : hsy,
                  Nn, Np, A, B, R, Om, u);
        free(A); free(B); free(R); free(Om); free(u);
      }
    }
    memcpy(work + (size_t)(j + 1) * P, C, sizeof(double) * P);
  }
#undef KB
  free(wx); free(wy); free(H); free(hx); free(hy);
  if (tax)
    for (size_t id = 0; id < P; ++id) {
      ta_free(&tax[id]);
      ta_free(&tay[id]);
    }
  free(tax); free(tay); free(F4); free(Nn); free(Np);
  return 0;
}

/* ------------------------------------------- 1D Atangana-Baleanu solve path */

int fho_ab_solve(int m, int n, double tau, double alpha, const double *w, const double *src,
                 const double *bl, const double *br, double *C, const double *exact, double *err) {
  const double h = 1.0 / m, a = alpha;
  const double A = -(1.0 / (h * h)) - (1.0 / (2.0 * h));
  const double Cc = -(1.0 / (h * h)) + (1.0 / (2.0 * h));
  const double Ii = w[0]; /* current-step coefficient (the reference's Ii, equal to I(1)) */
  const double Bd = (Ii / (1.0 - a)) + (2.0 / (h * h));
  double *prevC = (double *)calloc((size_t)(m + 1), sizeof(double));
  double *Rp = (double *)calloc((size_t)(m + 1), sizeof(double));
  double *al = (double *)calloc((size_t)(m + 1), sizeof(double));
  double *bt = (double *)calloc((size_t)(m + 1), sizeof(double));
  double *dts = (double *)calloc((size_t)(m + 1) * (size_t)(n + 1), sizeof(double));
  if (!prevC || !Rp || !al || !bt || !dts) return 1;
  double e = 0.0;
  for (int i = 1; i <= n; ++i) {
    for (int j = 0; j <= m; ++j) {
      Rp[j] = (Ii / (1.0 - a)) * C[j] + src[(size_t)(i - 1) * (m + 1) + j];
      if (i >= 2) {
        double prev_dtC = (C[j] - prevC[j]) / tau;
        dts[(size_t)j * (n + 1) + (i - 2)] = prev_dtC;
        double ret = 0.0;
        for (int tt = 0; tt < i - 1; ++tt) ret += dts[(size_t)j * (n + 1) + tt] * w[i - tt];
        Rp[j] -= ret / (1.0 - a);
      }
    }
    for (int j = 0; j <= m; ++j) prevC[j] = C[j];
    al[0] = 0;
    bt[0] = bl[i - 1];
    for (int j = 1; j <= m; ++j) {
      al[j] = Cc / (Bd - A * al[j - 1]);
      bt[j] = (Rp[j] - A * bt[j - 1]) / (Bd - A * al[j - 1]);
    }
    C[m] = br[i - 1];
    for (int j = m - 1; j >= 0; --j) C[j] = bt[j] - al[j] * C[j + 1];
    if (exact)
      for (int j = 0; j <= m; ++j) {
        double d = fabs(C[j] - exact[(size_t)(i - 1) * (m + 1) + j]);
        e += d * d;
      }
  }
  if (err) *err = e / ((m + 1.0) * n);
  free(prevC); free(Rp); free(al); free(bt); free(dts);
  return 0;
}
