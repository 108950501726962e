// Harness around the reference 1D H_solver (mt_minimal.cpp / mt_psi_caputo.cpp).
// Test infrastructure only: compiled from the read-only reference sources by
// oracle/ref/Makefile into oracle/_ref/; used to produce golden fixtures.
//
// The solver is driven in its linear configuration: gamma = 1 (classical
// second derivative in z, calc_v returns zero), cv_form 2 with -U >= 10 so that
// inv_dw_dh = 20, k_form 0 (KK = k), rp_form 0, no irrigation, bottom_cond 1
// (Dirichlet Hbottom), flags 4 (day/night coefficient 1).
//
// argv: BS NB L tau alpha k steps Hbottom [func_in_kernel func_power_t eps [gamma]]
// (gamma < 1: the space-fractional Caputo derivative in z, calc_v non-zero)
// stdin: N+1 initial values U[0..N]
// stdout: "uc <value>" then "u <N+2 values>" after the last step.
#ifndef REF_TU
#error "REF_TU must name the reference translation unit"
#endif
#define main reference_main
#include REF_TU
#undef main
#include <cstdio>
#include <cstdlib>

int main(int argc, char **argv) {
  if (argc < 9) { fprintf(stderr, "usage\n"); return 2; }
  BS = atoi(argv[1]);
  NB = atoi(argv[2]);
  double Lz = atof(argv[3]), tau_ = atof(argv[4]), alpha_ = atof(argv[5]), kk = atof(argv[6]);
  int steps = atoi(argv[7]);
  double hb = atof(argv[8]);
#ifdef PSI_CAPUTO
  omp_init_lock(&lock);
  if (argc >= 12) {
    func_in_kernel = atoi(argv[9]);
    func_power_t = atof(argv[10]);
    global_eps = global_eps2 = atof(argv[11]);
    integr_max_niter = 100000000;
  }
#endif
  sN = N = BS * NB;
  sNB = NB;
  F = new double[N + 2];
  BVK = new double[BS];
  flags = 4;
  const double gam = argc >= 13 ? atof(argv[12]) : 1.0;
  H_solver s(0, 2, 1, 1, tau_, alpha_, gam, NULL, 0, Lz, 0.5, hb);
  s.k = kk;
  for (int i = 0; i <= N; ++i)
    if (scanf("%lf", &s.U[i]) != 1) return 3;
  printf("uc %.17g\n", s.Uc());
  for (int t = 0; t < steps; ++t) s.calc_step();
  printf("u");
  for (int i = 0; i <= N + 1; ++i) printf(" %.17g", s.U[i]);
  printf("\n");
  return 0;
}
