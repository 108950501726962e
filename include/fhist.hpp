// fhist.hpp -- C++ host classes over the libfhist C ABI, shaped like the
// reference solver classes so that a time loop written against them reads like
// the reference's own drivers (TG_solver::solve, fr_d_t_g_2d.cpp:4328-4465;
// H_solver users in mt_psi_caputo.cpp:1750-1954; solve_and_check,
// MF_int_series.cpp:875-958):
//
//   fhist::TG_solver        TG_solver_<func,1,kform> with dt_alg 0 (fr_d_t_g_2d.cpp:2037-4052)
//   fhist::H_solver         one H_solver instance (mt_psi_caputo.cpp:369-1507,
//                           mt_minimal.cpp:276-1048 with gamma = 1)
//   fhist::H_solver_batch   many H_solver instances advanced in lock step
//   fhist::AB_solver        the solve_and_check time loop (MF_int_series.cpp:875-958)
//
// The public members carry the reference's names (b_C, V2, tstep, tau, alpha,
// U ...).  The host arrays are mirrors: the state lives on the GPU, calc_step()
// advances it there, get() copies it back into the mirror (the reference reads
// b_C / U after calc_step; call get() before such a read) and set_state()
// uploads the mirror.  Errors throw fhist::Error with the library's message.
// Header-only; link with -lfhist.
#pragma once

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "fhist.h"

namespace fhist {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string &msg) : std::runtime_error(msg), code(code) {}
  int code;
};

// One CUDA stream on one device (the reference's OpenCL_program +
// OpenCL_commandqueue pair, opencl_cuda_base.cpp:212-455).
class Context {
 public:
  explicit Context(int device = 0) {
    const int rc = fh_ctx_create(device, &h_);
    if (rc != FH_OK) throw Error(rc, fh_last_error(nullptr));
  }
  ~Context() {
    if (h_) fh_ctx_destroy(h_);
  }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  fh_ctx *get() const { return h_; }
  void check(int rc) const {
    if (rc != FH_OK) throw Error(rc, fh_last_error(h_));
  }
  void sync() const { check(fh_ctx_sync(h_)); }
  void set_graphs(bool on) const { check(fh_ctx_set_graphs(h_, on ? 1 : 0)); }

 private:
  fh_ctx *h_ = nullptr;
};

// 2D ADI solver with the full fractional history.  mode: FH_TG_FP64 (plain,
// FP64 sums), FH_TG_DF64 (double-float history) or FH_TG_BLOCKED (tensor-core
// far history).
class TG_solver {
 public:
  int sN, _M;                 // i = 0..sN, j = 0..M
  double tau, alpha, func_power, sigma, d_value, C1, _S, sdL, dLx;
  int tstep = 0;              // completed full steps
  std::vector<double> b_C;    // field, idx = i + j*(sN+2)
  std::vector<double> V2;     // |v|^2 per node
  std::vector<double> b_N;    // non-soluble phase (mass exchange on), filled by get_n()

  TG_solver(Context &ctx, const fh_tg_params &p, int max_steps, int mode = FH_TG_FP64)
      : sN(p.sN), _M(p.M), tau(p.tau), alpha(p.alpha), func_power(p.beta), sigma(p.sigma), d_value(p.d),
        C1(p.C1), _S(p.S), sdL(p.dL), dLx(p.dLx), b_C(size_t(p.sN + 2) * (p.M + 2), 0.0),
        V2(size_t(p.sN + 2) * (p.M + 2), 0.0), b_N(size_t(p.sN + 2) * (p.M + 2), 0.0), ctx_(ctx) {
    ctx_.check(fh_tg_create(ctx_.get(), &p, max_steps, mode, &s_));
  }
  ~TG_solver() {
    if (s_) fh_tg_destroy(s_);
  }
  TG_solver(const TG_solver &) = delete;
  TG_solver &operator=(const TG_solver &) = delete;

  // uploads b_C and V2 and restarts the time loop
  void set_state() {
    ctx_.check(fh_tg_set_state_host(s_, V2.data(), b_C.data()));
    tstep = 0;
  }
  // dt_alg 2 with dt_eps (restricted summing), or dt_alg 0 with dt_eps = 0;
  // before the first step of a solve
  void set_restricted(double dt_eps) { ctx_.check(fh_tg_set_restricted(s_, dt_eps)); }
  // dt_alg 3 with dt_eps = nterms (series expansion, psi = t), 0 = full history
  void set_series(int nterms) { ctx_.check(fh_tg_set_series(s_, nterms)); }
  // dt_alg 4 (two-series approximation, psi = t), before the first step
  void set_two_series(bool enable = true) { ctx_.check(fh_tg_set_two_series(s_, enable ? 1 : 0)); }
  // massN: mass exchange with the non-soluble phase (the globals massN_a, massN_b)
  void set_mass_exchange(bool enable, double massN_a, double massN_b) {
    ctx_.check(fh_tg_set_mass_exchange(s_, enable ? 1 : 0, massN_a, massN_b));
  }
  // TG_solver_<func, fixed_d, 0>: fixed_d false gives D = lambda |v| (ka0 / k) per node
  void set_diffusion(bool fixed_d, double lambda, double ka0, double k) {
    ctx_.check(fh_tg_set_diffusion(s_, fixed_d ? 1 : 0, lambda, ka0, k));
  }
  // TG_solver::calc_step (fr_d_t_g_2d.cpp:2552): x half step, y half step
  void calc_step() { calc_steps(1); }
  void calc_steps(int n) {
    ctx_.check(fh_tg_step(s_, n));
    tstep = fh_tg_tstep(s_);
  }
  // device field -> b_C
  void get() { ctx_.check(fh_tg_get_c_host(s_, b_C.data())); }
  // device N -> b_N (mass exchange on)
  void get_n() { ctx_.check(fh_tg_get_n_host(s_, b_N.data())); }
  const double *device_field() const { return fh_tg_field(s_); }
  long long device_bytes() const { return fh_tg_device_bytes(s_); }

 private:
  Context &ctx_;
  fh_tg_solver *s_ = nullptr;
};

// Many H_solver instances in lock step; U holds the concatenated N_i + 2 node
// values of every instance.
class H_solver_batch {
 public:
  std::vector<fh_h_params> params;
  std::vector<double> U;
  int tstep = 1;  // the reference starts its time loop at tstep 1

  H_solver_batch(Context &ctx, std::vector<fh_h_params> ps, int max_steps)
      : params(std::move(ps)), ctx_(ctx) {
    ctx_.check(fh_h_batch_create(ctx_.get(), int(params.size()), params.data(), max_steps, &b_));
    U.assign(size_t(fh_h_batch_state_size(b_)), 0.0);
    size_t o = 0;
    for (const auto &p : params) {
      offset_.push_back(o);
      o += size_t(p.N) + 2;
    }
  }
  ~H_solver_batch() {
    if (b_) fh_h_batch_destroy(b_);
  }
  H_solver_batch(const H_solver_batch &) = delete;
  H_solver_batch &operator=(const H_solver_batch &) = delete;

  double *U_of(int inst) { return U.data() + offset_[size_t(inst)]; }
  void set_state() {
    ctx_.check(fh_h_batch_set_u_host(b_, U.data()));
    tstep = 1;
  }
  // H_solver::calc_step on every instance
  void calc_step() { calc_steps(1); }
  void calc_steps(int n) {
    ctx_.check(fh_h_batch_step(b_, n));
    tstep = fh_h_batch_tstep(b_);
  }
  // space-derivative order per instance (gamma < 1: fractional in z), before the first step
  void set_space_order(const std::vector<double> &gamma) { ctx_.check(fh_h_batch_set_space_order(b_, gamma.data())); }
  // FH_H_FP64, FH_H_DF64 or FH_H_BLOCKED, before the first step
  void set_mode(int mode) { ctx_.check(fh_h_batch_set_mode(b_, mode)); }
  // small FP64 batches: all steps of a call in one launch (default on)
  void set_persistent(bool enable) { ctx_.check(fh_h_batch_set_persistent(b_, enable ? 1 : 0)); }
  // instance i starts a new solve (continuous batching) from U0 (p.N + 2 values,
  // p.N at most the instance's node count at creation); the others go on.
  // U is laid out again for the new node count and refreshed from the device.
  void restart(int i, const fh_h_params &p, const std::vector<double> &U0) {
    ctx_.check(fh_h_batch_restart(b_, i, &p, U0.data()));
    params[size_t(i)] = p;
    size_t o = 0;
    for (size_t q = 0; q < params.size(); ++q) {
      offset_[q] = o;
      o += size_t(params[q].N) + 2;
    }
    U.assign(size_t(fh_h_batch_state_size(b_)), 0.0);
    get();
  }
  void get() { ctx_.check(fh_h_batch_get_u_host(b_, U.data())); }
  long long device_bytes() const { return fh_h_batch_device_bytes(b_); }

 private:
  Context &ctx_;
  fh_h_batch *b_ = nullptr;
  std::vector<size_t> offset_;
};

// A single H_solver: public U (N + 2 nodes), tau, alpha, tstep as in the reference.
class H_solver {
 public:
  int N;
  double L, dL, tau, alpha;
  int &tstep;
  std::vector<double> &U;

  H_solver(Context &ctx, const fh_h_params &p, int max_steps)
      : N(p.N), L(p.L), dL(p.L / p.N), tau(p.tau), alpha(p.alpha), tstep(batch_.tstep), U(batch_.U),
        batch_(ctx, std::vector<fh_h_params>{p}, max_steps) {}
  void set_state() { batch_.set_state(); }
  void calc_step() { batch_.calc_step(); }
  void calc_steps(int n) { batch_.calc_steps(n); }
  void get() { batch_.get(); }

 private:
  H_solver_batch batch_;
};

// The Atangana-Baleanu time loop of solve_and_check: C (m + 1 nodes).
class AB_solver {
 public:
  int m;
  double tau, alpha;
  int step = 0;
  std::vector<double> C;

  AB_solver(Context &ctx, int m_, int max_steps, double tau_, double alpha_, int mode = FH_AB_FP64)
      : m(m_), tau(tau_), alpha(alpha_), C(size_t(m_) + 1, 0.0), ctx_(ctx) {
    ctx_.check(fh_ab_create(ctx_.get(), m, max_steps, tau, alpha, &s_));
    if (mode != FH_AB_FP64) ctx_.check(fh_ab_set_mode(s_, mode));
  }
  ~AB_solver() {
    if (s_) fh_ab_destroy(s_);
  }
  AB_solver(const AB_solver &) = delete;
  AB_solver &operator=(const AB_solver &) = delete;

  // source rows src[r*(m+1) + j] and boundary values per row
  void set_source(int nrows, const double *src, const double *bl, const double *br) {
    ctx_.check(fh_ab_set_source_host(s_, nrows, src, bl, br));
  }
  void set_current_coef(double Ii) { ctx_.check(fh_ab_set_current_coef(s_, Ii)); }
  // the reference's lag-weight cache (MF_intF_simple I_cache), lags 1..n
  void set_lag_weights(const std::vector<double> &w) {
    ctx_.check(fh_ab_set_lag_weights_host(s_, (int)w.size(), w.data()));
  }
  void set_state() {
    ctx_.check(fh_ab_set_c_host(s_, C.data()));
    step = 0;
  }
  void calc_step() { calc_steps(1); }
  void calc_steps(int n) {
    ctx_.check(fh_ab_step(s_, n));
    step += n;
  }
  void get() { ctx_.check(fh_ab_get_c_host(s_, C.data())); }

 private:
  Context &ctx_;
  fh_ab_solver *s_ = nullptr;
};

}  // namespace fhist
