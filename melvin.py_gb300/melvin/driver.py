"""The Simulation loop driven on the GPU.

The reference runs its loop on the host (examples/*.py):

    while simulation.is_running():          # t < final_time
        ... loop body ...                   # here: Stepper.step
        simulation.end_loop()               # loop_counter += 1; t += dt; tickers

and the loop-counted tickers of ``end_loop`` (melvin/Ticker.py:1-35) call
``Integrator.set_dt`` every ``cfl_cadence`` loops (a host reduction of the
velocity and a possible ``Exception("CFL condition breached")``,
melvin/Integrator.py:35-44) and the scalar trackers every
``tracker_cadence`` loops (melvin/Simulation.py:86-97): in the examples the
kinetic energy (melvin/utility.py:42-59) and the Nusselt number
(examples/double_diffusive_convection.py:20-23).  Each of those reads
the device, so the reference synchronises at every check.

:class:`DeviceRun` keeps t, dt, the loop counter, the ticker counters and the
stop point in device memory (``mgb_run_state``).  Every iteration is one
``mgb_run_step``: the fused step with dt read from the device, whose kernels
return at once for iterations past the stop point, followed when a ticker
fires by a one-thread tick kernel (end_loop, the CFL shrink or breach, a
kinetic-energy sample).  Loop-counted tickers fire on iterations known in
advance, so the host queues iterations without waiting and reads the state
once per chunk.  The results are those of the host loop: the same dt
sequence, the same final time and loop count, the same tracker samples, the
same state (tested against the Simulation's own loop).

Time-based tickers (dumps, saves) stay on the host: the device pauses the
run after the end_loop whose t passes the next of their times, the host
fires them and the run resumes.  When a dump falls on the same iteration as
a CFL check that shrinks dt, the dump records the new dt (the host loop
records the old one when the dump ticker was registered first).  Other
loop-counted host tickers (the wall-clock estimate) fire at those pauses and
at the end of a run.
"""

from __future__ import annotations

import ctypes as C
import functools
import os

import numpy as np
import torch

from . import _native as N


class DeviceRun:
    """Run `simulation`'s loop with the fused `stepper` as its body.

    cfl             CFL check every ``cfl_cadence`` loops (default: when
                    ``simulation.config_cfl`` was called)
    horizon         iterations between ticks at most (the stop point is
                    searched that far ahead)
    capacity        kinetic-energy samples held on the device per segment

    Scalar trackers are sampled on the device from the step's own
    start-of-step velocity and fields: the kinetic energy
    (``calc_kinetic_energy``, or a tracker file named "kinetic_energy") and
    the Nusselt number 1 - mean(tmp * uz) (``calc_nusselt_number`` of one of
    the stepper's fields, bound with functools.partial as the examples do).
    Other tracker functions need host arrays and raise ValueError.
    """

    def __init__(self, simulation, stepper, cfl=None, horizon=64, capacity=1 << 16):
        self.sim, self.stepper = simulation, stepper
        self.plan = stepper.plan
        self.device = stepper.device
        self.cfl = hasattr(simulation, "_cfl_ticker") if cfl is None else bool(cfl)
        if self.cfl and not hasattr(simulation, "_cfl_ticker"):
            raise ValueError("cfl=True needs simulation.config_cfl(ux, uz) first (as the reference)")
        self.kinds, flux = [], None
        trackers = getattr(simulation, "_trackers", [])
        fns = getattr(simulation, "_tracker_fns", [None] * len(trackers))
        for tr, fn in zip(trackers, fns):
            kind, var = self._classify(tr, fn)
            if kind == "nusselt":
                if flux is not None and var is not flux:
                    raise ValueError("Nusselt trackers of different fields cannot share the device flux")
                flux = var
            self.kinds.append(kind)
        self.track = bool(self.kinds)
        stepper.set_flux_field(flux)
        self.flux = flux is not None
        self.horizon = int(horizon)
        self.capacity = int(capacity) if self.track else 0
        self._state = torch.zeros(C.sizeof(N.MgbRunState), dtype=torch.uint8, device=self.device)
        self._host = torch.zeros(C.sizeof(N.MgbRunState), dtype=torch.uint8).pin_memory()
        self._trk = torch.zeros((3, max(self.capacity, 1)), dtype=torch.float64, device=self.device)
        self.last_state = None

    @staticmethod
    def _classify(tracker, fn):
        """("ke", None) or ("nusselt", tmp Variable) for a tracker function."""
        if isinstance(fn, functools.partial):
            name = getattr(fn.func, "__name__", "")
            if name == "calc_kinetic_energy":
                return "ke", None
            if name == "calc_nusselt_number" and fn.args:
                return "nusselt", fn.args[0]
        stem = os.path.splitext(os.path.basename(tracker._filename))[0]
        if stem == "kinetic_energy":
            return "ke", None
        raise ValueError(f"tracker {tracker._filename!r}: only the kinetic energy and the Nusselt number "
                         "(calc_nusselt_number bound to a stepped field) run on the device")

    # -- state transfer -------------------------------------------------

    def _upload(self, st):
        self._host.copy_(torch.frombuffer(bytearray(bytes(st)), dtype=torch.uint8))
        self._state.copy_(self._host, non_blocking=True)

    def read_state(self) -> N.MgbRunState:
        """The device run state (synchronises with the stream)."""
        self._host.copy_(self._state)
        return N.MgbRunState.from_buffer_copy(self._host.numpy().tobytes())

    # -- the loop ---------------------------------------------------------

    def _host_tickers(self):
        sim = self.sim
        dev = {id(getattr(sim, "_cfl_ticker", None)) if self.cfl else None,
               id(getattr(sim, "_tracker_ticker", None)) if self.track else None}
        return [t for t in sim._tickers if id(t) not in dev]

    def run(self, max_steps=None, chunk=256):
        """Run until t reaches final_time, the CFL check fails (raises
        ``Exception("CFL condition breached")``, as the reference does) or
        `max_steps` iterations have run.  Synchronises once per `chunk`
        iterations and at every pause.  Returns the iterations that ran."""
        total = 0
        while max_steps is None or total < max_steps:
            ran, status = self._segment(None if max_steps is None else max_steps - total, chunk)
            total += ran
            host = self._host_tickers()
            if status == N.RUN_PAUSED or (status == N.RUN_FINISHED and ran):
                for t in host:  # end_loop of the last iteration that ran
                    t.tick(self.sim._t, self.sim._loop_counter)
            if status == N.RUN_CFL_BREACH:
                raise Exception("CFL condition breached")
            if status != N.RUN_PAUSED:
                break
        return total

    def _segment(self, budget, chunk):
        sim, st_ = self.sim, self.stepper
        p, integ = sim._params, sim._integrator
        order = p.integrator_order
        cfl_t = getattr(sim, "_cfl_ticker", None) if self.cfl else None
        trk_t = getattr(sim, "_tracker_ticker", None) if self.track else None
        timed = [t._counter for t in self._host_tickers() if not t._by_counter]

        s0 = N.MgbRunState()
        s0.t, s0.dt, s0.loop = float(sim._t), float(integ._dt), int(sim._loop_counter)
        s0.stop_loop = 1 << 62
        s0.cfl_counter = int(cfl_t._counter) if cfl_t else 0
        s0.tracker_counter = int(trk_t._counter) if trk_t else 0
        s0.status = N.RUN_RUNNING
        self._upload(s0)
        cfg = N.MgbRunConfig()
        cfg.final_time = float(p.final_time)
        cfg.cfl_cutoff = float(p.cfl_cutoff)
        cfg.cfl_cadence = int(p.cfl_cadence) if cfl_t else 0
        cfg.tracker_cadence = int(p.tracker_cadence) if trk_t else 0
        cfg.capacity = self.capacity
        cfg.horizon = self.horizon
        cfg.pause_time = float(min(timed)) if timed else float("inf")
        cfg.tracker_t = self._trk[0].data_ptr()
        cfg.tracker_ke = self._trk[1].data_ptr()
        cfg.tracker_flux = self._trk[2].data_ptr() if self.flux else None

        st_.prepare(s0.dt)
        self.plan.last_prepared = st_
        lib, h = self.plan.lib, self.plan.handle
        stream = N.stream_handle(self.device)
        state_p = C.c_void_p(self._state.data_ptr())
        N.check(lib.mgb_run_begin(h, state_p, C.byref(cfg), stream))

        loop0 = s0.loop
        curr0 = st_.fields[0].dvar._curr_idx
        for i, f in enumerate(st_.fields):
            if f.dvar._curr_idx != curr0:
                raise ValueError("all histories of a fused step must share curr_idx")
            st_._q[i] = f.var._sdata.data_ptr()
            st_._h[i] = f.dvar._data.data_ptr()
        hc, ht = s0.cfl_counter, s0.tracker_counter
        since, k = 0, 0
        status = self.read_state().status
        while status == N.RUN_RUNNING and (budget is None or k < budget):
            n = chunk if budget is None else min(chunk, budget - k)
            for i in range(n):
                L = loop0 + k + i
                flags = 0
                if cfg.cfl_cadence and hc < L + 1:
                    flags |= N.RUN_CFL
                    hc += cfg.cfl_cadence
                if cfg.tracker_cadence and ht < L + 1:
                    flags |= N.RUN_TRACK
                    ht += cfg.tracker_cadence
                since += 1
                if i == n - 1 or since >= self.horizon:
                    flags |= N.RUN_TICK
                if flags:
                    since = 0
                N.check(lib.mgb_run_step(h, C.byref(st_.eq), st_._q, st_._h, (curr0 + k + i) % order, L, flags,
                                         N.ptr(st_.work), state_p, C.byref(cfg), stream))
            k += n
            status = self.read_state().status
        return self._pull(s0, curr0, order, cfl_t, trk_t)

    def _pull(self, s0, curr0, order, cfl_t, trk_t):
        """Copy the device run state back into the Simulation."""
        sim, integ = self.sim, self.sim._integrator
        s = self.read_state()
        ran = int(s.loop - s0.loop)
        sim._t = float(s.t)
        sim._loop_counter = int(s.loop)
        integ._dt = float(s.dt)
        for f in self.stepper.fields:
            f.dvar._curr_idx = (curr0 + ran) % order
        if cfl_t is not None:
            cfl_t._counter = int(s.cfl_counter)
            cfl_t.times_fired += int(s.cfl_fired)
        if trk_t is not None:
            trk_t._counter = int(s.tracker_counter)
            trk_t.times_fired += int(s.tracker_fired)
            n = int(s.ntracked)
            if n:
                tv = self._trk[:, :n].cpu().numpy()
                for tracker, kind in zip(sim._trackers, self.kinds):
                    vals = tv[1] if kind == "ke" else 1.0 - tv[2]
                    for t, v in zip(tv[0], vals):
                        tracker.append(float(t), np.float64(v))
            if s.dropped:
                raise RuntimeError(f"{s.dropped} kinetic-energy samples did not fit the device buffer "
                                   f"(capacity {self.capacity})")
        self.last_state = s
        return ran, int(s.status)
