// The drop-in binding of the 2D ADI path, compiled against the reference class
// itself: TG_solver_fhist derives from the reference's TG_solver_<0,1,0>
// (fr_d_t_g_2d.cpp:2773-4052) and replaces its calc_step (2552-2718) by one
// libfhist step, keeping the field on the device until the driver reads it
// back.  The members it hands to the library (sN, _M, tau, alpha, func_power,
// sigma, d_value, C1, _S, sdL, dLx, V2, b_C, tstep) are the reference's own.
//
// Test infrastructure: built from the read-only reference sources by the
// Makefile in this directory (outputs in oracle/_ref/) and linked with
// libfhist.so, which shows that the binding compiles and links against the
// reference's class.  Running it needs a GPU; without one the library's error
// path is taken (exit code 4, message from fh_last_error).
//
// argv: sN M tau alpha d C1 S steps
// stdin: (sN+2)*(M+2) values of V2 then (sN+2)*(M+2) initial values
// stdout: "c <values>" after the last step.
#define main reference_main
#include "fr_d_t_g_2d.cpp"
#undef main
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "fhist.h"

class TG_solver_fhist : public TG_solver_<0, 1, 0> {
 public:
  using TG_solver_<0, 1, 0>::TG_solver_;
  fh_ctx *fh = nullptr;
  fh_tg_solver *fs = nullptr;
  int use_fhist = 0;

  ~TG_solver_fhist() {
    fh_tg_destroy(fs);
    fh_ctx_destroy(fh);
  }
  // after the constructor (and the caller) filled V2 and b_C
  int fhist_init(int max_steps, int mode) {
    if (fh_ctx_create(0, &fh) != FH_OK) return report();
    fh_tg_params p = {sN, _M, tau, alpha, func_power, sigma, d_value, C1, _S, sdL, dLx};
    if (fh_tg_create(fh, &p, max_steps, mode, &fs) != FH_OK) return report();
    if (fh_tg_set_state_host(fs, V2, b_C) != FH_OK) return report();
    use_fhist = 1;
    return FH_OK;
  }
  // TG_solver::calc_step with the library path taken first (the reference's
  // own path is the base class's, unchanged)
  int calc_step() {
    if (use_fhist) {
      if (fh_tg_step(fs, 1) != FH_OK) return report();
      tstep++;
      return FH_OK;
    }
    TG_solver_<0, 1, 0>::calc_step();
    return FH_OK;
  }
  // before testing_check / output: the field back into b_C
  int fhist_get() { return fh_tg_get_c_host(fs, b_C) == FH_OK ? FH_OK : report(); }

 private:
  int report() {
    fprintf(stderr, "libfhist: %s\n", fh_last_error(fh));
    return FH_ECUDA;
  }
};

int main(int argc, char **argv) {
  if (argc < 9) return 2;
  sN = atoi(argv[1]);
  _M = atoi(argv[2]);
  const double tau_ = atof(argv[3]), alpha_ = atof(argv[4]), d_ = atof(argv[5]);
  const double c1 = atof(argv[6]), s_ = atof(argv[7]);
  const int steps = atoi(argv[8]);
  int_alg = 1;
  dt_alg = 0;
  massN = 0;
  testing = 0;
  use_ocl = 0;
  debug_level = 0;
  TG_solver_fhist s(tau_, alpha_, 0, 0, d_, -1, 5, 1.0, -1, -1, NULL, 0, -1, 0, c1, s_);
  const int P = (sN + 2) * (_M + 2);
  for (int i = 0; i < P; ++i)
    if (scanf("%lf", &s.V2[i]) != 1) return 3;
  for (int i = 0; i < P; ++i)
    if (scanf("%lf", &s.b_C[i]) != 1) return 3;
  memcpy(s.oldC[0], s.b_C, sizeof(double) * P);
  if (s.fhist_init(steps, FH_TG_FP64) != FH_OK) return 4;
  for (int t = 0; t < steps; ++t)
    if (s.calc_step() != FH_OK) return 4;
  if (s.fhist_get() != FH_OK) return 4;
  printf("c");
  for (int i = 0; i < P; ++i) printf(" %.17g", s.b_C[i]);
  printf("\n");
  return 0;
}
