// Harness around the reference Atangana-Baleanu routines (MF_int_series.cpp):
// mittag_leffler, MF_int_choice lag weights and solve_and_check.
// Test infrastructure only.
//
// argv: ml a b z eps          -> "ml value"
//       abw alpha tau n       -> "abw lag value" for lag = 1..n (weights of MF_intF_simple at step n)
//       ii alpha tau          -> "ii value" (current-step coefficient of solve_and_check)
//       solve alpha T n m     -> "err value" (F_func 0, simple 1)
//       field alpha T n m     -> "err value" and "c j value" for the field of the
//                                last step, j = 0..m
//       ablag alpha tau n     -> "ablag L value", L = 1..n: the lag weights that
//                                MF_intF_simple caches when solve_and_check runs
//                                (lag L first needed at step L with tt = 0)
//
// solve_and_check keeps its field in a local vector; the only place the field
// leaves the function is its error loop, d = fabs(C[j] - CC(h j, i tau)).  The
// reference TU is therefore compiled with fabs routed through a recorder that
// keeps the last m+1 arguments: after the call they are C[j] - CC of the last
// step, and C[j] = that + CC (the subtraction is exact: C[j] and CC agree to
// far better than a factor 2).  <cmath> is included first, so the macro only
// reaches the reference's own code.
#include <cmath>
#include <vector>
static std::vector<double> g_fabs_ring;
static size_t g_fabs_pos = 0;
static inline double harness_fabs(double x) {
  if (!g_fabs_ring.empty()) {
    g_fabs_ring[g_fabs_pos] = x;
    g_fabs_pos = (g_fabs_pos + 1) % g_fabs_ring.size();
  }
  return std::fabs(x);
}
#define fabs(x) harness_fabs(x)
#define main reference_main
#include "MF_int_series.cpp"
#undef main
#undef fabs
#include <cstdio>
#include <cstdlib>
#include <cstring>

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  F_notimes = 1;
  no_prints = 1;
  if (!strcmp(argv[1], "ml") && argc >= 6) {
    printf("ml %.17g\n", mittag_leffler(atof(argv[2]), atof(argv[3]), atof(argv[4]), atof(argv[5])));
  } else if (!strcmp(argv[1], "abw") && argc >= 5) {
    double a = atof(argv[2]), tau = atof(argv[3]);
    int n = atoi(argv[4]);
    for (int tt = 0; tt < n; ++tt)
      printf("abw %d %.17g\n", n - tt, MF_int_choice(n * tau, tt * tau + tau, tt * tau, a, a, 1000, 1000));
  } else if (!strcmp(argv[1], "ii") && argc >= 4) {
    double a = atof(argv[2]), tau = atof(argv[3]);
    printf("ii %.17g\n", MF_int_choice(tau, tau, 0, a, a, 1000, 1000, 1e-10));
  } else if (!strcmp(argv[1], "solve") && argc >= 6) {
    F_func = 0;
    F_nosimple = 0;
    double e = solve_and_check(atof(argv[2]), atof(argv[3]), atoi(argv[4]), atoi(argv[5]), 1);
    printf("err %.17g\n", e);
  } else if (!strcmp(argv[1], "ablag") && argc >= 5) {
    double a = atof(argv[2]), tau = atof(argv[3]);
    int n = atoi(argv[4]);
    for (int L = 1; L <= n; ++L) {
      const int tt = 0;
      printf("ablag %d %.17g\n", L, MF_int_choice(L * tau, tt * tau + tau, tt * tau, a, a, 1000, 1000));
    }
  } else if (!strcmp(argv[1], "field") && argc >= 6) {
    F_func = 0;
    F_nosimple = 0;
    const double a = atof(argv[2]), T = atof(argv[3]);
    const int n = atoi(argv[4]), m = atoi(argv[5]);
    g_fabs_ring.assign((size_t)m + 1, 0.0);
    g_fabs_pos = 0;
    const double e = solve_and_check(a, T, n, m, 1);
    printf("err %.17g\n", e);
    const double h = 1.0 / m, tau = T / n;
    for (int j = 0; j <= m; ++j) {
      const double d = g_fabs_ring[(g_fabs_pos + (size_t)j) % g_fabs_ring.size()];
      printf("c %d %.17g\n", j, d + CC(h * j, n * tau));
    }
  } else {
    return 2;
  }
  return 0;
}
