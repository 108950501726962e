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
static void tg_line(const fho_tg_params *p, const double *V2, double *C, const double *work, int j, int dir, int line,
                    double kcur, double kyh, const double *wk, const double *hs, double *A, double *B, double *R,
                    double *Om, double *u) {
  const int sN = p->sN, M = p->M, ld = sN + 2;
  const size_t P = (size_t)(sN + 2) * (M + 2);
  const double st = p->sigma / p->tau;
  const int N = dir == 0 ? sN : M;
  const double dl = dir == 0 ? p->dL : p->dLx;
  for (int i = 1; i < N; ++i) {
    const size_t id = dir == 0 ? (size_t)i + (size_t)line * ld : (size_t)line + (size_t)i * ld;
    if (dir == 0) {
      A[i] = (V2[id] / dl) * ((0.5 * (p->d + p->d) / dl) + 0.5);
      B[i] = (V2[id] / dl) * ((0.5 * (p->d + p->d) / dl) - 0.5);
    } else {
      A[i] = (V2[id] / (dl * dl)) * 0.5 * (p->d + p->d);
      B[i] = (V2[id] / (dl * dl)) * 0.5 * (p->d + p->d);
    }
    R[i] = st * (kcur + 0.0) + A[i] + B[i];
    Om[i] = -st * (kcur + 0.0) * C[id];
    Om[i] += p->S * 0.5;
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
  double *H = J ? (double *)calloc((size_t)J * P, sizeof(double)) : NULL;
  double *hx = J ? (double *)malloc(sizeof(double) * P) : NULL, *hy = J ? (double *)malloc(sizeof(double) * P) : NULL;
  if (J && (!H || !hx || !hy)) return 1;
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
    /* x half-step: lines jj = 1..M-1 (fr_d_t_g_2d.cpp:2577-2590); y half-step: lines
     * ii = 1..sN-1 (2634-2648).  Lines are independent, so they run in parallel. */
    for (int dir = 0; dir < 2; ++dir) {
      const int nlines = dir == 0 ? M : sN;
#pragma omp parallel
      {
        double *A = (double *)malloc(sizeof(double) * nmax), *B = (double *)malloc(sizeof(double) * nmax);
        double *R = (double *)malloc(sizeof(double) * nmax), *Om = (double *)malloc(sizeof(double) * nmax);
        double *u = (double *)malloc(sizeof(double) * nmax);
#pragma omp for schedule(static)
        for (int line = 1; line < nlines; ++line)
          tg_line(p, V2, C, work, j, dir, line, dir == 0 ? kx : ky, kyh, dir == 0 ? wx : wy, dir == 0 ? hsx : hsy,
                  A, B, R, Om, u);
        free(A); free(B); free(R); free(Om); free(u);
      }
    }
    memcpy(work + (size_t)(j + 1) * P, C, sizeof(double) * P);
  }
#undef KB
  free(wx); free(wy); free(H); free(hx); free(hy);
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
