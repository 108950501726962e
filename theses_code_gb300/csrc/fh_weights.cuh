// fh_weights.cuh -- device evaluation of the history weights (FP64).
//
// psi-Caputo weights for psi(t) = t^beta (beta != 1):
//   w = int_{x0 tau}^{x1 tau} (psi(X tau) - psi(s))^(-alpha) ds
//     = T^(1 - alpha beta) / beta * [B(y1; a, b) - B(y0; a, b)],
//   T = X tau, y = (x/X)^beta, a = 1/beta, b = 1 - alpha, B the lower
//   incomplete beta function.
// Late in a solve the two incomplete-beta values agree in their leading
// log10(X) digits, so their difference is never formed: it is evaluated
// directly from divided differences of the series (every term of the result
// has the sign of the result, or at worst half its size with the opposite
// sign), which keeps each weight within a few ulps for any step number.
//   lower side (y <= ~1/2):  B(y; a, b) = r P(y),  r = x/X = y^a,
//     P(y) = sum_j Lc_j y^j,  Lc_j = (1-b)_j / (j! (a+j));
//     B(y1) - B(y0) = (r1 - r0) P(y0) + r1 (y1 - y0) P[y0, y1]
//   upper side (c = 1 - y <= ~1/2):  B(1) - B(y) = U(c) = c^b Q(c),
//     Q(c) = sum_j Uc_j c^j,  Uc_j = (1-a)_j / (j! (b+j));
//     U(c0) - U(c1) = (c0^b - c1^b) Q(c1) + c0^b (c0 - c1) Q[c1, c0]
// with P[u, v] = (P(v) - P(u)) / (v - u) the divided difference, y1 - y0 from
// expm1 of beta log(x1/x0), and c0^b - c1^b from expm1 of b log1p.
#pragma once
#include "fh_common.cuh"

// Terms of the tabulated series (kIbTerms coefficients per side); arguments up
// to 0.55 leave a tail below 2^-64 of the sum.
constexpr int kIbTerms = 80;
// Branch limits of an interval [y0, y1]: lower series when y1 <= kIbLowMax,
// upper series when y0 >= kIbUpMin (c0 <= 0.55); an interval spanning both
// (only for X of a few steps, where the cancellation is a few digits at most)
// is the complete beta function minus both tails.
constexpr double kIbLowMax = 0.55, kIbUpMin = 0.45;

// Series value S = p(z0) and divided difference D = p[z0, z1] of
// p(z) = sum_j coef(j) z^j for j < n, by Horner with the divided-difference
// recurrence D_j = D_{j+1} z1 + S_{j+1}(z0).
template <class Coef>
__device__ __forceinline__ void fh_series_dd(const Coef &coef, int n, double z0, double z1, double &S, double &D) {
  double s = coef(n - 1), d = 0.0;
#pragma unroll 4
  for (int j = n - 2; j >= 0; --j) {
    d = fma(d, z1, s);
    s = fma(s, z0, coef(j));
  }
  S = s;
  D = d;
}

template <class Coef>
__device__ __forceinline__ double fh_series(const Coef &coef, int n, double z) {
  double s = coef(n - 1);
#pragma unroll 4
  for (int j = n - 2; j >= 0; --j) s = fma(s, z, coef(j));
  return s;
}

// Terms for a tail below 2^-61 of the sum at argument z <= 0.55: both
// coefficient sequences are bounded by their first term (|(1-a)_j / j!| <= 1
// for 0 < a <= 2), so the tail after n terms is at most z^n / (1 - z) of the
// sum.  FP32 log2 with two terms of margin.
__device__ __forceinline__ int fh_ib_nterms(double z) {
  if (!(z > 0.0)) return 1;
  const int n = (int)(62.0f / -__log2f((float)z)) + 2;
  return n < kIbTerms ? n : kIbTerms;
}

// Lc[j] = (1-b)_j / (j! (a+j)), Uc[j] = (1-a)_j / (j! (b+j)), j < kIbTerms.
__device__ __forceinline__ void fh_ib_tables(double a, double b, double *Lc, double *Uc) {
  double c = 1.0, d = 1.0;
  for (int j = 0; j < kIbTerms; ++j) {
    Lc[j] = c / (a + (double)j);
    Uc[j] = d / (b + (double)j);
    c *= ((double)(j + 1) - b) / (double)(j + 1);
    d *= ((double)(j + 1) - a) / (double)(j + 1);
  }
}

// expm1 of a double-double argument (h + l), |l| <= ulp(h).
__device__ __forceinline__ double fh_expm1_dd(double h, double l) {
  const double e = expm1(h);
  return fma(e + 1.0, l, e);
}

// Geometry of one interval [x0, x1] (0 <= x0 < x1 <= X) on the psi grid, with
// the logs that fix it: l0 = log(x0/X), l1 = log(x1/X), ld = log(x1/x0), each
// as a double-double (head, tail); l0 and ld are unused when x0 = 0.
struct fh_ib_slot {
  double r0, r1;   // x/X
  double dr;       // (x1 - x0)/X, rounded once (not r1 - r0)
  double l0h, l0l, l1h, l1l, ldh, ldl;
  bool zero0;      // x0 == 0
  bool top;        // x1 == X
};

// B(y1) - B(y0) for one interval from the coefficient sources lc(j), uc(j)
// (b = 1 - alpha; rlo = kIbLowMax^(1/beta), the largest x1/X of the lower
// branch; btot() = B(a, b), needed by the spanning branch only).
template <class LC, class UC, class BT>
__device__ __forceinline__ double fh_ib_diff(const fh_ib_slot &q, double beta, double b, double rlo, const BT &btot,
                                             const LC &lc, const UC &uc) {
  if (q.r1 <= rlo) {  // y1 <= kIbLowMax: lower series
    if (q.zero0) {
      const double e1 = exp(beta * q.l1h);
      const double y1 = fma(e1, beta * q.l1l, e1);
      return q.r1 * fh_series(lc, fh_ib_nterms(y1), y1);
    }
    const double e0 = exp(beta * q.l0h);
    const double y0 = fma(e0, beta * q.l0l, e0);
    const double dy = y0 * fh_expm1_dd(beta * q.ldh, beta * q.ldl);  // y1 - y0
    double S, D;
    fh_series_dd(lc, fh_ib_nterms(y0 + dy), y0, y0 + dy, S, D);
    return q.dr * S + q.r1 * dy * D;
  }
  // c = 1 - y = -expm1(beta log(x/X)); y1 - y0 = -y1 expm1(-beta log(x1/x0))
  const double c1 = q.top ? 0.0 : -fh_expm1_dd(beta * q.l1h, beta * q.l1l);
  const double y1 = 1.0 - c1;
  double y0 = 0.0, dy = y1;
  if (!q.zero0) {
    dy = -y1 * fh_expm1_dd(-beta * q.ldh, -beta * q.ldl);
    y0 = y1 - dy;
  }
  if (y0 >= kIbUpMin) {  // c0 <= 1 - kIbUpMin: upper series
    const double c0 = c1 + dy;
    if (c1 <= 0.0) return exp(b * log(c0)) * fh_series(uc, fh_ib_nterms(c0), c0);
    double S, D;
    fh_series_dd(uc, fh_ib_nterms(c0), c1, c0, S, D);
    const double c1b = exp(b * log(c1));
    const double dcb = c1b * expm1(b * log1p(dy / c1));  // c0^b - c1^b
    return dcb * S + (c1b + dcb) * dy * D;
  }
  // spans both sides (X of a few steps): B(a, b) - U(c1) - B(y0)
  const double up = c1 <= 0.0 ? 0.0 : exp(b * log(c1)) * fh_series(uc, kIbTerms, c1);
  const double lo = q.zero0 ? 0.0 : q.r0 * fh_series(lc, kIbTerms, y0);
  return (btot() - up) - lo;
}

// Coefficients read from a table.
struct fh_ib_coef_tab {
  const double *__restrict__ t;
  __device__ __forceinline__ double operator()(int j) const { return t[j]; }
};

// int_{x0 tau}^{x1 tau} (X tau - s)^(-alpha) ds (psi = t): the closed form in
// the operation order of H_solver::_kb_row (mt_psi_caputo.cpp:506-515;
// TG_solver_::_kb_row fr_d_t_g_2d.cpp:2960-2985).
__device__ __forceinline__ double fh_psi_int_t(double x0, double x1, double X, double tau, double alpha) {
  const double t0 = tau * x0, t1 = tau * x1, gtj = tau * X;
  double v = gtj / gtj;
  v *= pow(gtj, 1 - alpha);
  const double v3 = pow(fabs(1.0 - t1 / gtj), 1 - alpha);
  const double v4 = pow(fabs(1.0 - t0 / gtj), 1 - alpha);
  const double v2 = -(v3 - v4) / (1 - alpha);
  double sum = 0.0;
  sum += v2 * v;
  return sum;
}

// int_{x0 tau}^{x1 tau} (psi(X tau) - psi(s))^(-alpha) ds with psi(t) = t^beta.
// beta == 1: fh_psi_int_t.
// beta != 1: the divided-difference form above; the coefficients are built in
// a local table once per call (this form serves per-solve and per-block weight
// tables; the batched per-step weights read per-instance tables instead).
// beta != 1 with the coefficient tables of fh_ib_tables(1/beta, 1 - alpha),
// rlo = pow(kIbLowMax, 1/beta) and btot = B(1/beta, 1 - alpha) supplied by the
// caller (computed once for many slots).
__device__ __forceinline__ double fh_psi_int_pre(double x0, double x1, double X, double tau, double alpha,
                                                 double beta, const double *Lc, const double *Uc, double rlo,
                                                 double btot) {
  const double b = 1.0 - alpha;
  fh_ib_slot q;
  q.zero0 = !(x0 > 0.0);
  q.top = !(x1 < X);
  q.r0 = x0 / X;
  q.r1 = x1 / X;
  q.dr = (x1 - x0) / X;
  auto lrat = [](double x, double X) { return 2.0 * x <= X ? log(x / X) : log1p((x - X) / X); };
  q.l1h = q.top ? 0.0 : lrat(x1, X);
  q.l1l = 0.0;
  q.l0h = q.zero0 ? 0.0 : lrat(x0, X);
  q.l0l = 0.0;
  q.ldh = q.zero0 ? 0.0 : log1p((x1 - x0) / x0);
  q.ldl = 0.0;
  const fh_ib_coef_tab lc{Lc}, uc{Uc};
  const double diff = fh_ib_diff(q, beta, b, rlo, [&] { return btot; }, lc, uc);
  const double T = X * tau;
  return pow(T, 1.0 - alpha * beta) / beta * diff;
}

__device__ __forceinline__ double fh_psi_int(double x0, double x1, double X, double tau, double alpha,
                                             double beta) {
  if (beta == 1.0) return fh_psi_int_t(x0, x1, X, tau, alpha);
  const double a = 1.0 / beta, b = 1.0 - alpha;
  fh_ib_slot q;
  q.zero0 = !(x0 > 0.0);
  q.top = !(x1 < X);
  q.r0 = x0 / X;
  q.r1 = x1 / X;
  q.dr = (x1 - x0) / X;
  // log(x/X): log of the rounded ratio for x <= X/2, else log1p((x - X)/X)
  // (x - X is exact on the half-step grid), both within an ulp of the value
  auto lrat = [](double x, double X) { return 2.0 * x <= X ? log(x / X) : log1p((x - X) / X); };
  q.l1h = q.top ? 0.0 : lrat(x1, X);
  q.l1l = 0.0;
  q.l0h = q.zero0 ? 0.0 : lrat(x0, X);
  q.l0l = 0.0;
  q.ldh = q.zero0 ? 0.0 : log1p((x1 - x0) / x0);
  q.ldl = 0.0;
  double Lc[kIbTerms], Uc[kIbTerms];
  fh_ib_tables(a, b, Lc, Uc);
  const fh_ib_coef_tab lc{Lc}, uc{Uc};
  const double diff = fh_ib_diff(q, beta, b, pow(kIbLowMax, a),
                                 [&] { return exp(lgamma(a) + lgamma(b) - lgamma(a + b)); }, lc, uc);
  const double T = X * tau;
  return pow(T, 1.0 - alpha * beta) / beta * diff;
}
