// Harness around the reference Atangana-Baleanu routines (MF_int_series.cpp):
// mittag_leffler, MF_int_choice lag weights and solve_and_check.
// Test infrastructure only.
//
// argv: ml a b z eps          -> "ml value"
//       abw alpha tau n       -> "abw lag value" for lag = 1..n (weights of MF_intF_simple at step n)
//       ii alpha tau          -> "ii value" (current-step coefficient of solve_and_check)
//       solve alpha T n m     -> "err value" (F_func 0, simple 1)
#define main reference_main
#include "MF_int_series.cpp"
#undef main
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
  } else {
    return 2;
  }
  return 0;
}
