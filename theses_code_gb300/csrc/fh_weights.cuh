// fh_weights.cuh -- device evaluation of the history weights (FP64).
#pragma once
#include "fh_common.cuh"

// Lower incomplete beta B(y; a, b) = y^a sum_j (1-b)_j y^j / (j! (a+j)), y <= 1/2.
__device__ __forceinline__ double fh_ib_lower(double y, double a, double b) {
  if (y <= 0.0) return 0.0;
  double s = 0.0, c = 1.0, yj = 1.0;
  for (int j = 0; j < 400; ++j) {
    const double t = c * yj / (a + (double)j);
    s += t;
    if (fabs(t) <= 1e-17 * fabs(s)) break;
    c *= ((double)(j + 1) - b) / (double)(j + 1);
    yj *= y;
    if (c == 0.0) break;
  }
  return pow(y, a) * s;
}

// Upper tail B(1;a,b) - B(y;a,b) in c = 1-y: c^b sum_j (1-a)_j c^j / (j! (b+j)), c <= 1/2.
__device__ __forceinline__ double fh_ib_upper(double c, double a, double b) {
  if (c <= 0.0) return 0.0;
  double s = 0.0, d = 1.0, cj = 1.0;
  for (int j = 0; j < 400; ++j) {
    const double t = d * cj / (b + (double)j);
    s += t;
    if (fabs(t) <= 1e-17 * fabs(s)) break;
    d *= ((double)(j + 1) - a) / (double)(j + 1);
    cj *= c;
    if (d == 0.0) break;
  }
  return pow(c, b) * s;
}

// int_{x0 tau}^{x1 tau} (psi(X tau) - psi(s))^(-alpha) ds with psi(t) = t^beta.
// beta == 1: the closed form in the operation order of H_solver::_kb_row
// (mt_psi_caputo.cpp:506-515; TG_solver_::_kb_row fr_d_t_g_2d.cpp:2960-2985).
// beta != 1: T^(1-alpha beta)/beta * [B(y1; 1/beta, 1-alpha) - B(y0; 1/beta, 1-alpha)],
// y = (s/T)^beta, evaluated on the side (y or 1-y) where its series converges.
__device__ __forceinline__ double fh_psi_int(double x0, double x1, double X, double tau, double alpha,
                                             double beta) {
  if (beta == 1.0) {
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
  const double a = 1.0 / beta, b = 1.0 - alpha;
  const double y0 = pow(x0 / X, beta), y1 = pow(x1 / X, beta);
  const double c0 = (x0 >= X) ? 0.0 : -expm1(beta * log1p((x0 - X) / X));
  const double c1 = (x1 >= X) ? 0.0 : -expm1(beta * log1p((x1 - X) / X));
  double diff;
  if (y1 <= 0.5) {
    diff = fh_ib_lower(y1, a, b) - fh_ib_lower(y0, a, b);
  } else if (y0 > 0.5) {
    diff = fh_ib_upper(c0, a, b) - fh_ib_upper(c1, a, b);
  } else {
    const double btot = exp(lgamma(a) + lgamma(b) - lgamma(a + b));
    diff = (btot - fh_ib_upper(c1, a, b)) - fh_ib_lower(y0, a, b);
  }
  const double T = X * tau;
  return pow(T, 1.0 - alpha * beta) / beta * diff;
}

// ---- tabulated series for many weights of one (alpha, beta) pair
// Both incomplete-beta series above have coefficients that depend only on
// (a, b) = (1/beta, 1-alpha); with them tabulated, a series is one Horner
// polynomial of kIbTerms FMAs (their arguments stay <= 1/2, so 64 terms reach
// 2^-64 of the leading term) instead of a loop with two divisions per term.
constexpr int kIbTerms = 64;

// Lc[j] = (1-b)_j / (j! (a+j)), Uc[j] = (1-a)_j / (j! (b+j)).
__device__ __forceinline__ void fh_ib_tables(double a, double b, double *Lc, double *Uc) {
  double c = 1.0, d = 1.0;
  for (int j = 0; j < kIbTerms; ++j) {
    Lc[j] = c / (a + (double)j);
    Uc[j] = d / (b + (double)j);
    c *= ((double)(j + 1) - b) / (double)(j + 1);
    d *= ((double)(j + 1) - a) / (double)(j + 1);
  }
}

// Terms of a tabulated series at argument y in (0, 1/2] for a tail below
// 2^-61 of its sum: both coefficient sequences are bounded by their first
// term (|(1-a)_j / j!| <= 1 for 0 < a <= 2), so the tail after n terms is at
// most 2 y^n of the sum.  FP32 log2 with two terms of margin.
__device__ __forceinline__ int fh_ib_nterms(double y) {
  const int n = (int)(62.0f / -__log2f((float)y)) + 2;
  return n < kIbTerms ? n : kIbTerms;
}

// Horner over the first n coefficients.
__device__ __forceinline__ double fh_horner_n(const double *__restrict__ c, double y, int n) {
  double s = c[n - 1];
#pragma unroll 4
  for (int j = n - 2; j >= 0; --j) s = fma(s, y, c[j]);
  return s;
}

__device__ __forceinline__ double fh_horner(const double *__restrict__ c, double y) {
  double s = c[kIbTerms - 1];
#pragma unroll 8
  for (int j = kIbTerms - 2; j >= 0; --j) s = fma(s, y, c[j]);
  return s;
}

// fh_psi_int for beta != 1 from the tables: B(y; a, b) = y^a Lc(y) with
// y^a = x/X exactly (a = 1/beta, y = (x/X)^beta), upper tail c^b Uc(c).
__device__ __forceinline__ double fh_psi_int_tab(double x0, double x1, double X, double tau, double alpha,
                                                 double beta, const double *__restrict__ Lc,
                                                 const double *__restrict__ Uc) {
  const double a = 1.0 / beta, b = 1.0 - alpha;
  const double r0 = x0 / X, r1 = x1 / X;
  const double y0 = pow(r0, beta), y1 = pow(r1, beta);
  auto lower = [&](double y, double r) { return y <= 0.0 ? 0.0 : r * fh_horner(Lc, y); };
  auto upper = [&](double x) {
    if (x >= X) return 0.0;
    const double c = -expm1(beta * log1p((x - X) / X));
    return c <= 0.0 ? 0.0 : pow(c, b) * fh_horner(Uc, c);
  };
  double diff;
  if (y1 <= 0.5) {
    diff = lower(y1, r1) - lower(y0, r0);
  } else if (y0 > 0.5) {
    diff = upper(x0) - upper(x1);
  } else {
    const double btot = exp(lgamma(a) + lgamma(b) - lgamma(a + b));
    diff = (btot - upper(x1)) - lower(y0, r0);
  }
  const double T = X * tau;
  return pow(T, 1.0 - alpha * beta) / beta * diff;
}

