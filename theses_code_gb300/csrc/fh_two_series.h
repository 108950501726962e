// fh_two_series.h -- two-series approximation of the 2D history sums
// (dt_alg 4): host bookkeeping tables and the per-step kernel launch.
#pragma once
#include <cuda_runtime.h>

#include "fh_internal.h"

struct fh_ta;

// Plans every step 1 .. max_steps - 1 of a solve at alpha (psi = t) and
// allocates the per-point coefficient slots of both directions for P points.
int fh_ta_create(fh_ctx *ctx, double alpha, int max_steps, long long P, fh_ta **out);
void fh_ta_delete(fh_ta *t);
// Device bytes held (tables and coefficient slots).
size_t fh_ta_bytes(const fh_ta *t);
// Step j >= 1: the x and y sums at x = j into part[0][p], part[1][p] (times
// sc = Da tau^(1-alpha) / (1-alpha)), then the newest layer Dn = C^j - C^(j-1)
// (FP64, or (hi, lo) pairs when df) folded into the approximations.
int fh_ta_step(fh_ctx *ctx, const fh_ta *t, int j, const double *Dn, int df, long long P, double sc, double *part,
               cudaStream_t st);
