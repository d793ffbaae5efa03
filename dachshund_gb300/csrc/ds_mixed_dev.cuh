// Device helpers of the mixed-precision solver's scalar recurrence, shared by
// the per-kernel iteration (mixed.cu) and the persistent one (persist.cu).
#pragma once

#include "ds_f32.h"

namespace ds {

// Reliable-update decision after iteration `it` (st->rnorm, st->rmax set):
// the recurrence residual fell by delta since the last update, reached
// tol |b|, hit the iteration cap, or stagnated (did not halve in STALL_ITERS
// iterations, which FP32 rounding can cause far from x or near tol; the
// update then restarts the recurrence with beta = 0).
constexpr int STALL_ITERS = 30;
__device__ __forceinline__ bool update_due(MixedState* st, int it) {
  if (st->rnorm < 0.5 * st->rbest) {
    st->rbest = st->rnorm;
    st->it_best = it;
  }
  const bool stall = it - st->it_best >= STALL_ITERS;
  if (stall) st->stalled = 1;
  return st->rnorm < st->delta * st->rmax || st->rnorm <= st->tol_norm_b ||
         it >= st->max_iter || stall;
}

// Recurrence restart after an FP64 update that did not end the solve.
__device__ __forceinline__ void restart_after_update(MixedState* st, double rt, double rz) {
  st->beta = st->stalled ? 0.0 : rz / st->rz_old;
  st->rmax = rt;
  st->rbest = rt;
  st->it_best = st->iter;
  st->stalled = 0;
}

}  // namespace ds
