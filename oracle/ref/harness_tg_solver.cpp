// Harness around the reference 2D ADI solver TG_solver_<0,1,0>
// (fr_d_t_g_2d.cpp:2037-4052): psi(t) = t (Caputo-Gerasimov), fixed diffusion
// coefficient, dt_alg 0 (full history) or 2 (restricted summing with dt_eps),
// int_alg 1 (_kb_row weights, exact for psi = t), no mass exchange.  V2 (|v|^2)
// and the initial field are injected after construction.  Test infrastructure
// only.
//
// argv: sN M tau alpha d C1 S steps [dt_alg dt_eps [massN massN_a massN_b [fixed_d]]]
// (massN != 0: the mass-exchange stage N1 with the globals massN_a, massN_b;
// fixed_d 0: TG_solver_<0,0,0>, D = lambda |v| ka[0] / k with the
// constructor's lambda 5 and k = 2 sqrt(5) / (2.5 pi); "dcoef lambda ka0 k"
// is printed)
// stdin: (sN+2)*(M+2) values of V2 then (sN+2)*(M+2) initial values
// stdout: "geom dL dLx sigma" then "c <values>" after the last step.
#define main reference_main
#include "fr_d_t_g_2d.cpp"
#undef main
#include <cstdio>
#include <cstdlib>
#include <cstring>

template <class S>
static int run(S &s, int steps) {
  const int P = (sN + 2) * (_M + 2);
  for (int i = 0; i < P; ++i)
    if (scanf("%lf", &s.V2[i]) != 1) return 3;
  for (int i = 0; i < P; ++i)
    if (scanf("%lf", &s.b_C[i]) != 1) return 3;
  memcpy(s.oldC[0], s.b_C, sizeof(double) * P);
  if (massN)
    for (int i = 0; i < P; ++i) s.b_N[i] = s.b_prevN[i] = 0.0;
  printf("geom %.17g %.17g %.17g\n", s.sdL, s.dLx, s.sigma);
  printf("dcoef %.17g %.17g %.17g\n", s.lambda, s.ka[0], s.k);
  for (int t = 0; t < steps; ++t) s.calc_step();
  printf("c");
  for (int i = 0; i < P; ++i) printf(" %.17g", s.b_C[i]);
  printf("\n");
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 9) return 2;
  sN = atoi(argv[1]);
  _M = atoi(argv[2]);
  double tau_ = atof(argv[3]), alpha_ = atof(argv[4]), d_ = atof(argv[5]);
  double c1 = atof(argv[6]), s_ = atof(argv[7]);
  int steps = atoi(argv[8]);
  int_alg = 1;
  dt_alg = argc >= 11 ? atoi(argv[9]) : 0;
  if (argc >= 11) dt_eps = atof(argv[10]);
  massN = argc >= 14 ? atoi(argv[11]) : 0;
  if (argc >= 14) {
    massN_a = atof(argv[12]);
    massN_b = atof(argv[13]);
  }
  const int fixed = argc >= 15 ? atoi(argv[14]) : 1;
  testing = 0;
  use_ocl = 0;
  debug_level = 0;
  if (fixed) {
    TG_solver_<0, 1, 0> s(tau_, alpha_, 0, 0, d_, -1, 5, 1.0, -1, -1, NULL, 0, -1, 0, c1, s_);
    return run(s, steps);
  }
  TG_solver_<0, 0, 0> s(tau_, alpha_, 0, 0, d_, -1, 5, 1.0, -1, -1, NULL, 0, -1, 0, c1, s_);
  return run(s, steps);
}
