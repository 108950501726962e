// Harness around H_solver::calc_int (mt_psi_caputo.cpp:720-741): prints the
// psi-Caputo time weights kb(alpha, t0, t0+1, a) for psi(t) = t^beta computed
// by the reference's own series (_kb_row / _kb_row2) at a given tolerance.
// Test infrastructure only (see harness_h_solver.cpp).
//
// argv: alpha beta tau eps a0 a1   -> for a in [a0,a1]: all t0 < a... prints
//       "w a t0 value" lines.
#define main reference_main
#include "mt_psi_caputo.cpp"
#undef main
#include <cstdio>
#include <cstdlib>

int main(int argc, char **argv) {
  if (argc < 7) return 2;
  omp_init_lock(&lock);
  double alpha_ = atof(argv[1]), beta_ = atof(argv[2]), tau_ = atof(argv[3]);
  global_eps = global_eps2 = atof(argv[4]);
  integr_max_niter = 100000000;
  int a0 = atoi(argv[5]), a1 = atoi(argv[6]);
  func_in_kernel = (beta_ == 1.0) ? 0 : 3;
  func_power = beta_;
  BS = 2; NB = 1; sN = N = 2; sNB = 1;
  F = new double[N + 2];
  BVK = new double[BS];
  H_solver s(0, 2, 1, 1, tau_, alpha_, 1.0, NULL, 0, 1.0, 0.5, -20.0);
  for (int a = a0; a <= a1; ++a)
    for (int t0 = 0; t0 < a; ++t0)
      printf("w %d %d %.17g\n", a, t0, s.calc_int(alpha_, t0, t0 + 1, a, tau_, 1));
  return 0;
}
