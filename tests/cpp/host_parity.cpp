// Parity driver for the C++ host classes (include/fhist.hpp) against the CPU
// oracle, written the way the reference drives its solvers: construct, fill
// the public state, set_state(), loop calc_step(), read the state back.
// Prints one line per case ("<case> <rel max-norm err> <bound>") and exits
// non-zero if any case misses its bound.  Test infrastructure: links the
// oracle library as the checker.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "fh_oracle.h"
#include "fhist.hpp"

// relative max-norm difference; infinite when either side holds a non-finite value
static double relmax(const std::vector<double> &a, const std::vector<double> &b, size_t off = 0, size_t n = 0) {
  if (n == 0) n = b.size();
  double num = 0.0, den = 0.0;
  for (size_t i = 0; i < n; ++i) {
    if (!std::isfinite(a[off + i]) || !std::isfinite(b[i])) return INFINITY;
    num = std::fmax(num, std::fabs(a[off + i] - b[i]));
    den = std::fmax(den, std::fabs(b[i]));
  }
  return den > 0.0 ? num / den : num;
}

static int report(const char *name, double err, double bound) {
  std::printf("%s %.3e %.0e\n", name, err, bound);
  return err <= bound ? 0 : 1;
}

// The oracle's parameters of a TG case: fixed diffusion coefficient unless
// set otherwise, full history.
static fho_tg_params oracle_tg(const fh_tg_params &p) {
  fho_tg_params q{};
  q.sN = p.sN;
  q.M = p.M;
  q.tau = p.tau;
  q.alpha = p.alpha;
  q.beta = p.beta;
  q.sigma = p.sigma;
  q.d = p.d;
  q.C1 = p.C1;
  q.S = p.S;
  q.dL = p.dL;
  q.dLx = p.dLx;
  q.fixed_d = 1;
  return q;
}

// TG_solver::solve-style loop (fr_d_t_g_2d.cpp:4328-4465) on a small grid.
// variant 1: mass exchange and the velocity-dependent coefficient together;
// variant 2: the two-series approximation (dt_alg 4).
static int tg_case(fhist::Context &ctx, int mode, int steps, double bound, const char *name, int variant = 0) {
  const int sN = 40, M = 33;
  fh_tg_params p = {sN, M, variant == 2 ? 1e-3 : 5e-4, variant == 2 ? 0.6 : 0.7, 1.0, 0.2, 0.1, 0.2, 0.01,
                    1.0 / sN, 1.0 / M};
  fhist::TG_solver s(ctx, p, steps, mode);
  fho_tg_params q = oracle_tg(p);
  const double lam = 5.0, ka0 = 1.005e-3, kk = 2.0 * std::sqrt(5.0) / (M_PI * 2.5);
  if (variant == 1) {
    s.set_mass_exchange(true, 0.4, 1.5);
    s.set_diffusion(false, lam, ka0, kk);
    q.massN = 1;
    q.massN_a = 0.4;
    q.massN_b = 1.5;
    q.fixed_d = 0;
    q.lambda = lam;
    q.ka0 = ka0;
    q.kk = kk;
  } else if (variant == 2) {
    s.set_two_series(true);
    q.dt_alg = 4;
    q.dt_eps = 1e-8;
  }
  const int ld = sN + 2;
  for (int j = 0; j < M + 2; ++j)
    for (int i = 0; i < sN + 2; ++i) {
      const double x = double(i) / sN, y = double(j) / M;
      s.V2[i + j * ld] = 0.3 + 0.7 * std::pow(std::sin(3.0 * x + 1.0) * std::cos(2.0 * y), 2);
      s.b_C[i + j * ld] = std::exp(-((x - 0.45) * (x - 0.45) + (y - 0.55) * (y - 0.55)) / 0.02);
    }
  std::vector<double> C0 = s.b_C;
  s.set_state();
  for (int t = 0; t < steps; ++t) s.calc_step();
  s.get();
  std::vector<double> ref = C0, work(size_t(steps + 1) * ref.size());
  if (fho_tg_solve(&q, s.V2.data(), ref.data(), steps, work.data())) return 1;
  if (variant == 1) {
    // the non-soluble phase took up mass
    s.get_n();
    double nmax = 0.0;
    for (double v : s.b_N) nmax = std::isfinite(v) ? std::fmax(nmax, std::fabs(v)) : INFINITY;
    if (!(nmax > 0.0 && std::isfinite(nmax))) return report(name, INFINITY, bound);
  }
  if (s.device_bytes() <= 0) return report(name, INFINITY, bound);
  return report(name, relmax(s.b_C, ref), bound);
}

static int h_case(fhist::Context &ctx, int weights, double beta, const char *name) {
  const int N = 120, steps = 60;
  fh_h_params p = {N, 1.0, 1e-3, 0.8, weights, beta, FH_K_CONST, 1.0, 0.0, 1.0, 0, 0.0, 0.0, 0.0};
  fhist::H_solver s(ctx, p, steps + 1);
  for (int i = 0; i <= N + 1; ++i) s.U[size_t(i)] = i < N ? std::sin(M_PI * i / N) : 0.0;
  std::vector<double> ref = s.U;
  s.set_state();
  for (int t = 0; t < steps; ++t) s.calc_step();
  s.get();
  fho_h_params q = {N, 1.0, 1e-3, 0.8, weights, beta, FHO_K_CONST, 1.0, 0.0, 1.0, 0, 0.0, 0.0, 0.0, 1.0};
  std::vector<double> hist(size_t(steps) * (N + 2));
  if (fho_h_solve(&q, ref.data(), steps, hist.data())) return 1;
  return report(name, relmax(s.U, ref), 1e-12);
}

// Continuous batching through the host class: instance 1 of a two-instance
// batch restarts with a smaller node count after 20 steps; after 30 more
// both instances match their own solves.
static int h_restart_case(fhist::Context &ctx) {
  const int N0 = 120, N1 = 100, steps = 50, first = 20;
  fh_h_params p0 = {N0, 1.0, 1e-3, 0.8, FH_W_L1, 1.0, FH_K_CONST, 1.0, 0.0, 1.0, 0, 0.0, 0.0, 0.0};
  fh_h_params p1 = p0, p1b = p0;
  p1b.N = N1;
  p1b.alpha = 0.6;
  fhist::H_solver_batch b(ctx, {p0, p1}, steps + 1);
  std::vector<double> u0(size_t(N0) + 2, 0.0), u1b(size_t(N1) + 2, 0.0);
  for (int i = 0; i < N0; ++i) u0[size_t(i)] = std::sin(M_PI * i / N0);
  for (int i = 0; i < N1; ++i) u1b[size_t(i)] = std::sin(2.0 * M_PI * i / N1) * 0.5;
  std::copy(u0.begin(), u0.end(), b.U_of(0));
  std::copy(u0.begin(), u0.end(), b.U_of(1));
  b.set_state();
  b.calc_steps(first);
  b.restart(1, p1b, u1b);
  b.calc_steps(steps - first);
  b.get();
  fho_h_params q0 = {N0, 1.0, 1e-3, 0.8, FH_W_L1, 1.0, FHO_K_CONST, 1.0, 0.0, 1.0, 0, 0.0, 0.0, 0.0, 1.0};
  fho_h_params q1 = q0;
  q1.N = N1;
  q1.alpha = 0.6;
  std::vector<double> r0 = u0, r1 = u1b;
  std::vector<double> h0(size_t(steps) * (N0 + 2)), h1(size_t(steps) * (N1 + 2));
  if (fho_h_solve(&q0, r0.data(), steps, h0.data()) || fho_h_solve(&q1, r1.data(), steps - first, h1.data())) return 1;
  const double e0 = relmax(b.U, r0, 0, r0.size()), e1 = relmax(b.U, r1, size_t(N0) + 2, r1.size());
  if (b.device_bytes() <= 0) return report("h_batch_restart", INFINITY, 1e-12);
  return report("h_batch_restart", std::fmax(e0, e1), 1e-12);
}

static int ab_case(fhist::Context &ctx) {
  const int m = 256, n = 120;
  const double tau = 1e-3, alpha = 0.6;
  fhist::AB_solver s(ctx, m, n, tau, alpha);
  std::vector<double> src(size_t(m) + 1), bl(1, 0.0), br(1, 0.0);
  for (int j = 0; j <= m; ++j) src[size_t(j)] = std::sin(M_PI * j / m) + 0.3 * std::sin(3 * M_PI * j / m);
  s.set_source(1, src.data(), bl.data(), br.data());
  s.set_state();
  for (int t = 0; t < n; ++t) s.calc_step();
  s.get();
  // oracle: per-step source rows, lag weights from the oracle's own series
  std::vector<double> w(size_t(n) + 1), srcs(size_t(n) * (m + 1)), bls(size_t(n), 0.0), brs(size_t(n), 0.0);
  for (int lag = 1; lag <= n; ++lag) w[size_t(lag)] = fho_ab_int(lag, tau, alpha);
  w[0] = w[1];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= m; ++j) srcs[size_t(i) * (m + 1) + j] = src[size_t(j)];
  std::vector<double> ref(size_t(m) + 1, 0.0);
  if (fho_ab_solve(m, n, tau, alpha, w.data(), srcs.data(), bls.data(), brs.data(), ref.data(), nullptr, nullptr))
    return 1;
  return report("ab_solver", relmax(s.C, ref), 1e-12);
}

int main() {
  int bad = 0;
  try {
    fhist::Context ctx(0);
    bad += tg_case(ctx, FH_TG_FP64, 30, 1e-12, "tg_solver_fp64");
    bad += tg_case(ctx, FH_TG_DF64, 30, 1e-12, "tg_solver_df64");
    bad += tg_case(ctx, FH_TG_BLOCKED, 150, 1e-9, "tg_solver_blocked");
    bad += tg_case(ctx, FH_TG_FP64, 60, 1e-12, "tg_solver_massN_variable_d", 1);
    bad += tg_case(ctx, FH_TG_FP64, 200, 1e-12, "tg_solver_two_series", 2);
    bad += h_case(ctx, FH_W_L1, 1.0, "h_solver_l1");
    bad += h_case(ctx, FH_W_PSI, 1.3, "h_solver_psi");
    bad += h_restart_case(ctx);
    bad += ab_case(ctx);
  } catch (const fhist::Error &e) {
    std::printf("error %d: %s\n", e.code, e.what());
    return 2;
  }
  return bad ? 1 : 0;
}
