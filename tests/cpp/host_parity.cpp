// Parity driver for the C++ host classes (include/fhist.hpp) against the CPU
// oracle, written the way the reference drives its solvers: construct, fill
// the public state, set_state(), loop calc_step(), read the state back.
// Prints one line per case ("<case> <rel max-norm err> <bound>") and exits
// non-zero if any case misses its bound.  Test infrastructure: links the
// oracle library as the checker.
#include <cmath>
#include <cstdio>
#include <vector>

#include "fh_oracle.h"
#include "fhist.hpp"

static double relmax(const std::vector<double> &a, const std::vector<double> &b) {
  double num = 0.0, den = 0.0;
  for (size_t i = 0; i < a.size(); ++i) {
    num = std::fmax(num, std::fabs(a[i] - b[i]));
    den = std::fmax(den, std::fabs(b[i]));
  }
  return den > 0.0 ? num / den : num;
}

static int report(const char *name, double err, double bound) {
  std::printf("%s %.3e %.0e\n", name, err, bound);
  return err <= bound ? 0 : 1;
}

// TG_solver::solve-style loop (fr_d_t_g_2d.cpp:4328-4465) on a small grid.
static int tg_case(fhist::Context &ctx, int mode, int steps, double bound, const char *name) {
  const int sN = 40, M = 33;
  fh_tg_params p = {sN, M, 5e-4, 0.7, 1.0, 0.2, 0.1, 0.2, 0.01, 1.0 / sN, 1.0 / M};
  fhist::TG_solver s(ctx, p, steps, mode);
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
  fho_tg_params q = {sN, M, p.tau, p.alpha, p.beta, p.sigma, p.d, p.C1, p.S, p.dL, p.dLx};
  std::vector<double> ref = C0, work(size_t(steps + 1) * ref.size());
  if (fho_tg_solve(&q, s.V2.data(), ref.data(), steps, work.data())) return 1;
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
    bad += h_case(ctx, FH_W_L1, 1.0, "h_solver_l1");
    bad += h_case(ctx, FH_W_PSI, 1.3, "h_solver_psi");
    bad += ab_case(ctx);
  } catch (const fhist::Error &e) {
    std::printf("error %d: %s\n", e.code, e.what());
    return 2;
  }
  return bad ? 1 : 0;
}
