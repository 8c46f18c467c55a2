"""Fused timestep: the whole user loop body in one native call.

The reference advances a simulation with a hand-written loop whose body
calls one API verb per term (e.g. examples/taylor_green_vortex.py:87-93,
examples/rayleigh_benard_convection.py:97-142).  A :class:`Stepper` takes
the same equations as data -- for every advected field its diffusion
coefficient, its linear terms and its boundary rule -- and evaluates the
loop body with ``mgb_step``: three kernels for a fully spectral grid, four
(five for the predictor-corrector) for Fourier-x / Dirichlet-z.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _native as N

OPS = {"value": 0, "ddx": 1, "ddz": 2}
INTEGRATORS = {"semi-implicit": N.INT_SEMI_IMPLICIT, "explicit": N.INT_EXPLICIT, "pece": N.INT_PECE}


class Term:
    """``rhs += coef * op(src)``; ``src`` is an advected Variable or "psi"."""

    def __init__(self, src, op="value", coef=1.0):
        if op not in OPS:
            raise ValueError(f"op must be one of {sorted(OPS)}")
        self.src, self.op, self.coef = src, op, float(coef)


class FieldEquation:
    """d(var)/dt = -u.grad(var) + sum(terms) + kappa * lap(var), history in
    `dvar`, boundary rule `bc` (MGB_BC_* flags) applied after the update."""

    def __init__(self, var, dvar, kappa=0.0, terms=(), bc=0):
        self.var, self.dvar, self.kappa, self.terms, self.bc = var, dvar, float(kappa), list(terms), int(bc)


class Stepper:
    def __init__(self, simulation, fields, integrator=None, order=None, alpha=None):
        p = simulation._params
        if not 1 <= len(fields) <= 3:
            raise ValueError("a fused step advances 1 to 3 fields (field 0 is the vorticity)")
        self.sim = simulation
        self.fields = list(fields)
        self.plan = N.plan_for(p)
        self.device = self.plan.device
        integ = integrator or p.integrator
        if integ not in INTEGRATORS:
            raise ValueError(f"integrator {integ!r}")
        eq = N.MgbEquation()
        eq.nfields = len(fields)
        eq.integrator = INTEGRATORS[integ]
        eq.order = int(order or p.integrator_order)
        eq.alpha = float(p.alpha if alpha is None else alpha)
        index = {id(f.var): i for i, f in enumerate(self.fields)}
        for i, f in enumerate(self.fields):
            fe = eq.f[i]
            fe.kappa = f.kappa
            fe.bc = f.bc
            if len(f.terms) > 4:
                raise ValueError("at most 4 linear terms per field")
            fe.nterms = len(f.terms)
            for k, t in enumerate(f.terms):
                if isinstance(t.src, str):
                    if t.src != "psi":
                        raise ValueError(f"term source {t.src!r}")
                    src = -1
                else:
                    if id(t.src) not in index:
                        raise ValueError("a term's source must be one of the advected fields or 'psi'")
                    src = index[id(t.src)]
                fe.terms[k] = N.MgbTerm(src, OPS[t.op], t.coef)
        self.eq = eq
        self.work = self.plan.step_work(len(fields))
        self.diag = torch.zeros(4, dtype=torch.float64, device=self.device)
        self._q = (C.c_void_p * 3)()
        self._h = (C.c_void_p * 3)()
        self._prepared_dt = None

    def set_flux_field(self, var):
        """Make the step's diagnostics carry a fourth value, the convective
        flux mean(uz * q) of the advected field `var` at the start of the
        step (None: three values)."""
        if var is None:
            self.eq.diag_flux = 0
            self.diag[3:].zero_()  # nothing writes it from here on
            return
        for i, f in enumerate(self.fields):
            if f.var is var:
                self.eq.diag_flux = i + 1
                return
        raise ValueError("the flux field must be one of the stepper's advected fields")

    def prepare(self, dt):
        """(Re)compute the per-mode update coefficients for `dt`."""
        self.plan.call("mgb_step_prepare", C.byref(self.eq), float(dt), N.ptr(self.work),
                       N.stream_handle(self.device))
        self._prepared_dt = float(dt)

    def _ensure(self, dt):
        if self._prepared_dt != float(dt) or self.plan.last_prepared is not self:
            self.prepare(dt)
            self.plan.last_prepared = self

    def step(self, dt=None, diagnostics=False):
        """Advance every field by one step; returns the device tensor
        (kinetic energy, max ux, max uz, convective flux) of the start-of-step
        velocity when `diagnostics` is set (the flux only after
        set_flux_field, else 0)."""
        dt = self.sim._integrator._dt if dt is None else dt
        self._ensure(dt)
        curr = self.fields[0].dvar._curr_idx
        for i, f in enumerate(self.fields):
            if f.dvar._curr_idx != curr:
                raise ValueError("all histories of a fused step must share curr_idx")
            self._q[i] = f.var._sdata.data_ptr()
            self._h[i] = f.dvar._data.data_ptr()
        self.plan.call(
            "mgb_step", C.byref(self.eq), self._q, self._h, curr, float(dt), N.ptr(self.work),
            N.ptr(self.diag) if diagnostics else None, N.stream_handle(self.device),
        )
        for f in self.fields:
            f.dvar.advance()
        return self.diag if diagnostics else None

    def autotune(self, dt=None, **kw):
        """Time the fused step's tile variants on this stepper and keep the
        fastest (:func:`melvin.autotune.tune`); the fields are left as they
        were."""
        from .autotune import tune

        return tune(self, dt=dt, **kw)

    def kernel_count(self):
        n = C.c_int32()
        N.check(self.plan.lib.mgb_step_kernel_count(self.plan.handle, C.byref(self.eq), C.byref(n)))
        return n.value

    def step_events(self, events, dt=None):
        """`step` that also records ``events[0]`` before the first kernel and
        ``events[k]`` after kernel k (torch.cuda.Event objects, already
        recorded once so that they exist)."""
        dt = self.sim._integrator._dt if dt is None else dt
        self._ensure(dt)
        curr = self.fields[0].dvar._curr_idx
        for i, f in enumerate(self.fields):
            self._q[i] = f.var._sdata.data_ptr()
            self._h[i] = f.dvar._data.data_ptr()
        ev = (C.c_void_p * len(events))(*[e.cuda_event for e in events])
        N.check(self.plan.lib.mgb_step_events(
            self.plan.handle, C.byref(self.eq), self._q, self._h, curr, float(dt), N.ptr(self.work), None,
            N.stream_handle(self.device), ev, len(events)))
        for f in self.fields:
            f.dvar.advance()

    def step_host(self, states, histories, dt=None):
        """One step of fields whose state and history live in host memory.

        ``states[i]`` and ``histories[i]`` are pinned CPU tensors shaped like
        field i's state and history (the device tensors are the staging
        copies).  On the current stream the states go up, the step runs and
        the states come back.  On a second stream the history slots the
        update reads go up, overlapping the transforms (the update, kernel 2,
        waits for them through mgb_step_waits), and after the states the slot
        the step wrote comes back, overlapping what the current stream runs
        next.  The slot the step overwrites whole is not uploaded.  Fully
        spectral plans.  Returns the bytes copied up and down.  The host
        tensors hold the result once the event ``host_done`` has completed; a
        later call orders its copies after it."""
        if self.plan.grid.fdm_z:
            raise NotImplementedError("step_host: fully spectral plans only")
        dt = self.sim._integrator._dt if dt is None else dt
        self._ensure(dt)
        main = torch.cuda.current_stream(self.device)
        if getattr(self, "_copy_stream", None) is None:
            self._copy_stream = torch.cuda.Stream(device=self.device)
            self._hist_ready = torch.cuda.Event()
            self._states_down = torch.cuda.Event()
            self.host_done = torch.cuda.Event(enable_timing=True)
        cs = self._copy_stream
        curr = self.fields[0].dvar._curr_idx
        order = self.fields[0].dvar._data.shape[0]
        read = [s for s in range(order) if s != curr]
        up = down = 0
        cs.wait_stream(main)  # after the current stream's earlier work (the step before read these slots)
        with torch.cuda.stream(cs):
            for f, h in zip(self.fields, histories):
                for s in read:
                    f.dvar._data[s].copy_(h[s], non_blocking=True)
                    up += h[s].numel() * h.element_size()
            self._hist_ready.record(cs)
        for i, (f, h) in enumerate(zip(self.fields, states)):
            if f.dvar._curr_idx != curr:
                raise ValueError("all histories of a fused step must share curr_idx")
            f.var._sdata.copy_(h, non_blocking=True)
            up += h.numel() * h.element_size()
            self._q[i] = f.var._sdata.data_ptr()
            self._h[i] = f.dvar._data.data_ptr()
        waits = (C.c_void_p * 3)(None, None, self._hist_ready.cuda_event)
        N.check(self.plan.lib.mgb_step_waits(
            self.plan.handle, C.byref(self.eq), self._q, self._h, curr, float(dt), N.ptr(self.work), None,
            N.stream_handle(self.device), waits, 3))
        for f, hs in zip(self.fields, states):
            hs.copy_(f.var._sdata, non_blocking=True)
            down += hs.numel() * hs.element_size()
        # the written history slot goes down on the second stream once the
        # states are down (two downloads at once share one direction's
        # bandwidth), so it overlaps whatever the current stream runs next
        self._states_down.record(main)
        cs.wait_event(self._states_down)
        with torch.cuda.stream(cs):
            for f, hh in zip(self.fields, histories):
                hh[curr].copy_(f.dvar._data[curr], non_blocking=True)
                down += hh[curr].numel() * hh.element_size()
            self.host_done.record(cs)
        for f in self.fields:
            f.dvar.advance()
        return up, down
