// Device side of a driven run: the end of a loop iteration of the
// reference's Simulation (melvin/Simulation.py:99-100,134-135,
// melvin/Ticker.py:1-35) and the CFL check of Integrator.set_dt
// (melvin/Integrator.py:35-44), done by one thread on the device-resident
// mgb_run_state so that no host synchronisation is needed.
#include <climits>

#include "internal.h"

namespace mgb {

struct TickArgs {
  double final_time, cfl_cutoff, dx, dz, pause_time;
  long long upto;    // iterations [.., upto) have been launched
  long long horizon;
  int flags, cfl_cadence, tracker_cadence, capacity;
  double* tracker_t;
  double* tracker_ke;
  double* tracker_flux;  // or null
};

// Python's builtin min(a, b) as the reference calls it: `b` when b < a,
// else `a` (so a NaN first argument survives, a NaN second one does not).
__device__ __forceinline__ double py_min(double a, double b) { return b < a ? b : a; }

__global__ void k_run_tick(mgb_run_state* st, TickArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  st->dt_changed = 0;  // the coefficient refresh of the previous tick has run
  if (st->status != MGB_RUN_RUNNING) return;
  // Simulation.end_loop of every iteration that ran since the last tick:
  // loop_counter += 1; t += dt (dt is constant between ticks).
  const long long loop_before = st->loop;
  while (st->loop < a.upto && st->loop < st->stop_loop) {
    st->loop += 1;
    st->t += st->dt;
  }
  const bool ended = st->loop > loop_before;  // an end_loop ran in this tick
  const bool ran = st->loop == a.upto && a.upto > 0;
  // tickers after the last iteration, in the order the examples register
  // them (config_cfl before config_scalar_trackers)
  if (ran && (a.flags & MGB_RUN_CFL) && st->cfl_counter < st->loop) {
    const double cfl_dt = py_min(a.dx / st->diag[1], a.dz / st->diag[2]);
    if (st->dt > cfl_dt || cfl_dt != cfl_dt) {
      // set_dt raises before the ticker counts the firing
      st->status = MGB_RUN_CFL_BREACH;
      st->stop_loop = st->loop;
      return;
    }
    while (st->dt > a.cfl_cutoff * cfl_dt) {
      st->dt = st->dt * 0.9;
      st->dt_changed = 1;
    }
    st->cfl_counter += a.cfl_cadence;
    st->cfl_fired += 1;
  }
  if (ran && (a.flags & MGB_RUN_TRACK) && st->tracker_counter < st->loop) {
    if (st->ntracked < a.capacity) {
      a.tracker_t[st->ntracked] = st->t;
      a.tracker_ke[st->ntracked] = st->diag[0];
      if (a.tracker_flux) a.tracker_flux[st->ntracked] = st->diag[3];
      st->ntracked += 1;
    } else {
      st->dropped += 1;
    }
    st->tracker_counter += a.tracker_cadence;
    st->tracker_fired += 1;
  }
  // Simulation.is_running for the coming iterations: iteration j runs while
  // its start time t_j < final_time (t_{j+1} = t_j + dt) and the end_loop
  // that produced t_j did not pass the pause time (a time-based ticker of
  // the caller fires there).  The start time of the current iteration is
  // tested against the pause time only when its end_loop ran here: after a
  // pause the caller has fired its tickers.  The caller ticks again within
  // `horizon` iterations, so the search stops there.
  double tt = st->t;
  long long j = st->loop;
  const long long lim = j + a.horizon;
  bool stop = tt >= a.final_time || (ended && tt > a.pause_time);
  while (!stop && j < lim) {
    tt += st->dt;
    ++j;
    stop = tt >= a.final_time || tt > a.pause_time;
  }
  st->stop_loop = stop ? j : LLONG_MAX;
  if (st->loop >= st->stop_loop) st->status = st->t >= a.final_time ? MGB_RUN_FINISHED : MGB_RUN_PAUSED;
}

int run_tick(const mgb_plan* p, mgb_run_state* st, const mgb_run_config* cfg, long long upto, int flags,
             cudaStream_t s) {
  TickArgs a;
  a.final_time = cfg->final_time;
  a.cfl_cutoff = cfg->cfl_cutoff;
  a.dx = p->g.dx;
  a.dz = p->g.dz;
  a.pause_time = cfg->pause_time;
  a.upto = upto;
  a.horizon = cfg->horizon;
  a.flags = flags;
  a.cfl_cadence = cfg->cfl_cadence;
  a.tracker_cadence = cfg->tracker_cadence;
  a.capacity = cfg->capacity;
  a.tracker_t = cfg->tracker_t;
  a.tracker_ke = cfg->tracker_ke;
  a.tracker_flux = cfg->tracker_flux;
  k_run_tick<<<1, 32, 0, s>>>(st, a);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

}  // namespace mgb
