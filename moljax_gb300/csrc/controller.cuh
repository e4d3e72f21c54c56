// The accept/reject and PI step-size update of one adaptive attempt, shared by
// the single-solve controller kernel (csrc/imex.cu) and the batched controller
// (csrc/imex_batch.cu).  One thread applies it to one DevState.
#pragma once

#include "spectral.cuh"

namespace mjx {

// NaN-propagating min/max (jnp.minimum/maximum semantics).
__device__ __forceinline__ double jmax(double a, double b) { return (a != a || b != b) ? (a + b) : (a > b ? a : b); }
__device__ __forceinline__ double jmin(double a, double b) { return (a != a || b != b) ? (a + b) : (a < b ? a : b); }
__device__ __forceinline__ double jclip(double x, double lo, double hi) { return jmin(jmax(x, lo), hi); }

// tot: sum over every degree of freedom of (err / (atol + rtol |y_new|))^2; bad: any
// non-finite value.  Applies moljax/core/stepping.py:1246-1359 (scaled_error_norm,
// propose_dt_imex, the accept and reject branches, the loop stop and final status) to
// st and returns whether the run continues.  hist_t / hist_dt may be null.
__device__ __forceinline__ bool ctl_update(DevState* st, double tot, int bad, double n_dof,
                                           const mjx_pid_params& P, double* hist_t, double* hist_dt) {
  const double order = (double)st->order;
  const double dtc = st->dtc;
  // stepping.py:1246-1247
  const double e = jmax(sqrt(tot / n_dof), 1e-10);
  const int finite = !bad;
  const bool accept = (e <= 1.0) && finite;
  // dt_policy.py:544-610 (propose_dt_imex)
  double dt_a, pe_new;
  if (e <= 1.0) {  // pid_controller_dt (178-227)
    const double kI = P.kI / order, kP = P.kP / order;
    const double es = jmax(e, 1e-10), pes = jmax(st->prev_err, 1e-10);
    double fac = pow(1.0 / es, kI) * pow(pes / es, kP);
    fac = jclip(fac * P.safety, P.min_factor, P.max_factor);
    dt_a = jclip(dtc * fac, P.dt_min, P.dt_max);
    pe_new = e;
  } else {  // handle_rejected_step (230-268)
    const double kI = P.kI / order;
    double fac = P.safety * pow(1.0 / jmax(e, 1.0), kI);
    fac = jclip(fac, P.min_factor, 1.0);
    dt_a = jclip(dtc * fac, P.dt_min, P.dt_max);
    pe_new = st->prev_err;
  }
  const double dt_new = jclip(jmin(dt_a, st->dt_cfl), P.dt_min, P.dt_max);
  st->err_last = e;
  st->save_slot = -1;
  if (accept) {  // stepping.py:1271-1309
    if (st->n_acc % st->save_every == 0) {
      if (hist_t) hist_t[st->write_idx] = st->t + dtc;
      if (hist_dt) hist_dt[st->write_idx - 1] = dtc;
      st->save_slot = st->write_idx;
      st->write_idx += 1;
    }
    st->t = st->t + dtc;
    st->cur = 1 - st->cur;
    st->dt = dt_new;
    st->prev_err = pe_new;
    st->dt_last_accepted = dtc;
    st->n_acc += 1;
  } else {  // stepping.py:1311-1334
    const double dtr = jmax(dt_new * 0.5, P.dt_min);
    st->dt = dtr;
    if (dtr <= P.dt_min * 1.1) st->status = MJX_STATUS_DT_TOO_SMALL_CODE;
    st->n_rej += 1;
  }
  if (!finite) { st->status = MJX_STATUS_NON_FINITE_CODE; st->finite = 0; }
  st->attempts += 1;
  const bool running = st->status == MJX_STATUS_RUNNING_CODE && st->t < st->t_end &&
                       st->write_idx < st->max_saves && st->attempts < st->max_attempts;
  if (running) {
    st->dtc = jmin(st->dt, st->t_end - st->t);
  } else {
    st->done = 1;
    if (st->t >= st->t_end) st->status = MJX_STATUS_SUCCESS_CODE;             // 1351-1359
    else if (st->write_idx >= st->max_saves) st->status = MJX_STATUS_MAX_STEPS_CODE;
    else if (st->status == MJX_STATUS_RUNNING_CODE) st->status = MJX_STATUS_MAX_STEPS_CODE;
  }
  return running;
}

}  // namespace mjx
