"""Time integration (melvin/Integrator.py) on the GPU.

Predictor AB2/AB4 (:5-18), corrector AM2/AM4 (:20-33), the CFL timestep
control ``set_dt`` (:35-44), ``_explicit`` (:53-56) and
``_semi_implicit_spectral`` (:58-63, bound only for fully spectral grids,
:78-81).  Each update is one fused kernel over the spectral state.
"""

import numpy as np
import torch

from . import _native as N
from ._arrays import as_device


class Integrator:
    def __init__(self, params, xp=None):
        self._params = params
        self._xp = xp
        self._dt = params.initial_dt
        self._dx = params.dx
        self._dz = params.dz
        self._cfl_cutoff = params.cfl_cutoff
        self._plan = N.plan_for(params)
        self._device = self._plan.device
        self._order = params.integrator_order
        if self._order in (2, 4):
            self.predictor = self._adams_bashforth
            self.corrector = self._adams_moulton
        if params.integrator == "semi-implicit":
            if params.is_fully_spectral():
                self.integrate = self._semi_implicit_spectral
                self._alpha = params.alpha
        elif params.integrator == "explicit":
            self.integrate = self._explicit
        self._diag = None

    def _adams(self, dvar, corrector):
        out = torch.empty(self._plan.spectral_shape, dtype=torch.complex128, device=self._device)
        self._plan.call("mgb_adams", int(corrector), N.ptr(dvar._data), self._order, dvar._curr_idx,
                        float(self._dt), N.ptr(out), N.stream_handle(self._device))
        return out

    def _adams_bashforth(self, dvar):
        return self._adams(dvar, 0)

    def _adams_moulton(self, dvar):
        return self._adams(dvar, 1)

    def diagnostics(self, ux, uz):
        """Device (kinetic energy, max ux, max uz) of physical velocities."""
        pl = self._plan
        if self._diag is None:
            self._diag = torch.empty(3, dtype=torch.float64, device=self._device)
        a = as_device(ux.getp() if hasattr(ux, "getp") else ux, torch.float64, self._device, pl.physical_shape)
        b = as_device(uz.getp() if hasattr(uz, "getp") else uz, torch.float64, self._device, pl.physical_shape)
        pl.call("mgb_diagnostics", N.ptr(a), N.ptr(b), N.ptr(self._diag), N.ptr(pl.work()),
                N.stream_handle(self._device))
        return self._diag

    def set_dt(self, ux, uz):
        """Sets dt from the CFL limit ``min(dx/max(ux), dz/max(uz))``."""
        d = self.diagnostics(ux, uz).cpu().numpy()
        with np.errstate(divide="ignore", invalid="ignore"):
            cfl_dt = min(np.float64(self._dx) / d[1], np.float64(self._dz) / d[2])
        if self._dt > cfl_dt or np.isnan(cfl_dt):
            raise Exception("CFL condition breached")
        while self._dt > self._cfl_cutoff * cfl_dt:
            self._dt = self._dt * 0.9

    def override_dt(self, dt):
        self._dt = dt

    def get_dt(self):
        return self._dt

    def _explicit(self, var, dvar, diffusion_term):
        pl = self._plan
        d = as_device(diffusion_term, torch.complex128, self._device, pl.spectral_shape)
        pl.call("mgb_integrate_explicit", N.ptr(var._sdata), N.ptr(dvar._data), self._order, dvar._curr_idx,
                float(self._dt), N.ptr(d), N.stream_handle(self._device))
        dvar.advance()

    def _semi_implicit_spectral(self, var, dvar, lin_op):
        pl = self._plan
        if isinstance(lin_op, torch.Tensor) and lin_op.is_complex():
            if torch.any(lin_op.imag != 0):
                raise NotImplementedError("complex linear operators are not supported by the GPU path")
            lin_op = lin_op.real
        L = as_device(lin_op, torch.float64, self._device, pl.spectral_shape)
        pl.call("mgb_integrate_semi_implicit", N.ptr(var._sdata), N.ptr(dvar._data), self._order,
                dvar._curr_idx, float(self._dt), float(self._alpha), N.ptr(L), N.stream_handle(self._device))
        dvar.advance()
