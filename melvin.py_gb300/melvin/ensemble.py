"""Ensembles: many independent simulations of one grid advanced together.

Each member is a complete simulation (its own spectral state and
derivative history); every kernel of a step covers all members at once
(``mgb_batch_step``), and :meth:`Ensemble.graph` captures several steps
into one CUDA graph so an ensemble advances ``nsteps`` steps per graph
launch.  Members live in slots of pooled tensors, so members that start or
finish at different times can share a batch (see :mod:`melvin.serving`).
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from .stepper import INTEGRATORS, OPS


class FieldSpec:
    """One advected field: diffusion coefficient, linear terms
    ``(src, op, coef)`` with src a field index or -1 for psi, and a boundary
    rule (MGB_BC_* flags)."""

    def __init__(self, kappa, terms=(), bc=0):
        self.kappa, self.terms, self.bc = float(kappa), list(terms), int(bc)


class Ensemble:
    def __init__(self, params, fields, nslots, integrator=None, order=None, alpha=None, term_coef=None):
        self.params = params
        self.plan = N.plan_for(params)
        self.device = self.plan.device
        self.F = len(fields)
        if not 1 <= self.F <= 3:
            raise ValueError("1 to 3 advected fields")
        self.nslots = int(nslots)
        rows, cols = self.plan.spectral_shape
        order = int(order or params.integrator_order)
        self.order = order
        integ = integrator or params.integrator
        eq = N.MgbEquation()
        eq.nfields = self.F
        eq.integrator = INTEGRATORS[integ]
        eq.order = order
        eq.alpha = float(params.alpha if alpha is None else alpha)
        for i, fs in enumerate(fields):
            fe = eq.f[i]
            fe.kappa = fs.kappa
            fe.bc = fs.bc
            fe.nterms = len(fs.terms)
            for k, (src, op, coef) in enumerate(fs.terms):
                fe.terms[k] = N.MgbTerm(int(src), OPS[op] if isinstance(op, str) else int(op), float(coef))
        self.eq = eq
        self.q = torch.zeros((self.nslots, self.F, rows, cols), dtype=torch.complex128, device=self.device)
        self.hist = torch.zeros((self.nslots, self.F, order, rows, cols), dtype=torch.complex128, device=self.device)
        self.curr = 0
        self.term_coef = None
        if term_coef is not None:
            self.term_coef = torch.as_tensor(term_coef, dtype=torch.float64, device=self.device).reshape(
                self.nslots, 3, 4).contiguous()
        b = C.c_size_t()
        N.check(self.plan.lib.mgb_batch_workspace_bytes(self.plan.handle, self.F, self.nslots, C.byref(b)))
        self.work = torch.empty(b.value, dtype=torch.uint8, device=self.device)
        self.diag = torch.zeros((self.nslots, 3), dtype=torch.float64, device=self.device)
        self._prepared = None
        self._stepped = False

    # ---- state -----------------------------------------------------------
    def load_physical(self, slot, arrays):
        """Load physical fields (one (nx, nz) array per field) into a slot
        and clear its history."""
        from .SpectralTransformer import SpectralTransformer

        st = SpectralTransformer(self.params)
        for f, arr in enumerate(arrays):
            st.to_spectral(arr, out=self.q[slot, f])
        self.hist[slot].zero_()

    def reset_history(self, slots=None):
        if slots is None:
            self.hist.zero_()
        else:
            self.hist[slots] = 0

    # ---- stepping ----------------------------------------------------------
    def prepare(self, dt):
        """(Re)compute the update coefficients for `dt` when they are not the
        ones the plan last prepared for this ensemble's workspace."""
        if self._prepared != float(dt) or self.plan.last_prepared is not self:
            self.plan.call("mgb_step_prepare", C.byref(self.eq), float(dt), N.ptr(self.work),
                           N.stream_handle(self.device))
            self._prepared = float(dt)
            self.plan.last_prepared = self

    def _batch(self, members):
        bt = N.MgbBatch()
        if members is None:
            bt.count = self.nslots
            bt.members = None
        else:
            bt.count = int(members.numel())
            bt.members = members.data_ptr()
        bt.q = self.q.data_ptr()
        bt.hist = self.hist.data_ptr()
        bt.term_coef = None if self.term_coef is None else self.term_coef.data_ptr()
        return bt

    def step(self, dt, members=None, diagnostics=False):
        """Advance the listed slots (an int32 device tensor; all slots when
        None) by one step.  Every member shares ``curr``: members joining a
        running batch start with a zero history, as a fresh simulation does."""
        self.prepare(dt)
        bt = self._batch(members)
        self.plan.call("mgb_batch_step", C.byref(self.eq), C.byref(bt), self.curr, float(dt), N.ptr(self.work),
                       N.ptr(self.diag) if diagnostics else None, N.stream_handle(self.device))
        self.curr = (self.curr + 1) % self.order
        self._stepped = True
        return self.diag if diagnostics else None

    def autotune(self, dt, members=None, **kw):
        """Time the fused step's tile variants on this ensemble (the listed
        members) and keep the fastest (:func:`melvin.autotune.tune`); the
        states are left as they were.  Tune before capturing a graph."""
        from .autotune import tune

        return tune(self, dt=dt, members=members, **kw)

    def graph(self, dt, nsteps, members=None):
        """Capture ``nsteps`` steps (a multiple of the integrator order, so
        the history slot pattern repeats) into a CUDA graph; returns a
        callable that replays them.  The member list, dt and the equation
        are fixed at capture."""
        if nsteps % self.order:
            raise ValueError(f"nsteps must be a multiple of the integrator order {self.order}")
        if not self._stepped:
            raise RuntimeError("advance the ensemble once with step() before capturing: the first launch of "
                               "each kernel sets attributes that cannot be set inside a capture")
        self.prepare(dt)
        curr0 = self.curr
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        bt = self._batch(members)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for k in range(nsteps):
                    N.check(self.plan.lib.mgb_batch_step(
                        self.plan.handle, C.byref(self.eq), C.byref(bt), (curr0 + k) % self.order, float(dt),
                        N.ptr(self.work), None, C.c_void_p(s.cuda_stream)))
        torch.cuda.current_stream(self.device).wait_stream(s)

        def replay():
            g.replay()
            self.curr = curr0  # nsteps is a multiple of the order

        replay.graph = g
        return replay

    def chunk_graph(self, dt, nsteps, members, stream):
        """Capture ``nsteps`` steps of ``members`` (a device int32 tensor whose
        contents may change between replays; its address and length are
        fixed at capture) from the current history slot into a CUDA graph on
        ``stream``, without the device-wide synchronisation of
        :meth:`graph`, so that other streams keep running.  Returns a callable
        that replays the steps on the current stream and advances ``curr``;
        it must be called with ``curr`` where it was at capture.  The capture
        itself runs nothing."""
        if not self._stepped:
            raise RuntimeError("advance the ensemble once with step() before capturing")
        self.prepare(dt)
        curr0, end = self.curr, (self.curr + nsteps) % self.order
        g = torch.cuda.CUDAGraph()
        bt = self._batch(members)
        with torch.cuda.stream(stream):
            g.capture_begin(capture_error_mode="thread_local")
            try:
                for k in range(nsteps):
                    N.check(self.plan.lib.mgb_batch_step(
                        self.plan.handle, C.byref(self.eq), C.byref(bt), (curr0 + k) % self.order, float(dt),
                        N.ptr(self.work), None, C.c_void_p(stream.cuda_stream)))
            finally:
                g.capture_end()

        def replay():
            if self.curr != curr0:
                raise RuntimeError(f"chunk graph captured at history slot {curr0}, ensemble at {self.curr}")
            g.replay()
            self.curr = end

        replay.graph = g
        return replay


class EnsembleGroup:
    """Ensembles of different grid sizes (or precisions) advanced together.

    :meth:`graph` captures every ensemble's batched steps into ONE CUDA
    graph; each ensemble's launch sequence is an independent branch of the
    graph (forked from and joined back into the capture stream), so the
    small grids' kernels fill the GPU beside the large ones' and one replay
    advances every member of every size.  Each ensemble needs its own plan
    (one ensemble per grid and precision), because a plan's prepared
    update coefficients belong to one workspace."""

    def __init__(self, ensembles):
        self.ensembles = list(ensembles)
        plans = [id(e.plan) for e in self.ensembles]
        if len(set(plans)) != len(plans):
            raise ValueError("an EnsembleGroup holds one ensemble per grid and precision")
        devs = {str(e.device) for e in self.ensembles}
        if len(devs) != 1:
            raise ValueError("all ensembles of a group must be on one device")
        self.device = self.ensembles[0].device

    def _dts(self, dt):
        return [float(d) for d in (dt if isinstance(dt, (list, tuple)) else [dt] * len(self.ensembles))]

    def step(self, dt, members=None):
        """One step of every ensemble (launched one ensemble after the other
        on the current stream); `dt` and `members` may be per-ensemble lists."""
        mems = members if isinstance(members, (list, tuple)) else [members] * len(self.ensembles)
        for e, d, m in zip(self.ensembles, self._dts(dt), mems):
            e.step(d, m)

    def graph(self, dt, nsteps, members=None):
        """Capture `nsteps` steps of every ensemble (a multiple of every
        ensemble's integrator order) into one graph; returns a callable that
        replays it.  dt, member lists and equations are fixed at capture."""
        dts = self._dts(dt)
        mems = members if isinstance(members, (list, tuple)) else [members] * len(self.ensembles)
        for e, d in zip(self.ensembles, dts):
            if nsteps % e.order:
                raise ValueError(f"nsteps must be a multiple of every integrator order ({e.order})")
            if not e._stepped:
                raise RuntimeError("advance every ensemble once with step() before capturing")
            e.prepare(d)
        currs = [e.curr for e in self.ensembles]
        dev = self.device
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream(device=dev)
        branches = [torch.cuda.Stream(device=dev) for _ in self.ensembles]
        cap.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(cap):
            with torch.cuda.graph(g, stream=cap):
                for e, d, m, br, c0 in zip(self.ensembles, dts, mems, branches, currs):
                    br.wait_stream(cap)  # fork
                    bt = e._batch(m)
                    for k in range(nsteps):
                        N.check(e.plan.lib.mgb_batch_step(
                            e.plan.handle, C.byref(e.eq), C.byref(bt), (c0 + k) % e.order, d, N.ptr(e.work), None,
                            C.c_void_p(br.cuda_stream)))
                for br in branches:
                    cap.wait_stream(br)  # join
        torch.cuda.current_stream(dev).wait_stream(cap)

        def replay():
            g.replay()
            for e, c0 in zip(self.ensembles, currs):
                e.curr = c0  # nsteps is a multiple of every order

        replay.graph = g
        return replay
