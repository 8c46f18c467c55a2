"""Spatial derivatives (melvin/SpatialDifferentiator.py) on the GPU.

``pddx``/``pddz``: central finite differences of order 2 or 4 on physical
arrays, periodic along spectral axes, Dirichlet (outer points left 0) along
an FDM axis.  ``sddx``/``sddz``/``sd2dx2``/``sd2dz2``: spectral factors for
complex-exponential bases; on an FDM z axis ``sddz``/``sd2dz2`` apply the z
stencils to the spectral array (:36-43).  ``calc_lap``: the Laplacian symbol.
"""

import torch

from . import _native as N
from ._arrays import as_device, finish, native_target
from .BasisFunctions import BasisFunctions, gen_diff2_factors, gen_diff_factors


class SpatialDifferentiator:
    def __init__(self, params, xp=None, array_factory=None):
        self._params = params
        self._xp = xp
        self._plan = N.plan_for(params)
        self._device = self._plan.device
        if params.discretisation[0] == "fdm":
            raise NotImplementedError("Finite difference not implemented in x direction")
        self._fdm_z = params.discretisation[1] == "fdm"
        self._diffx_factors = gen_diff_factors(params.lx)
        self._diffz_factors = gen_diff_factors(params.lz)
        self._diff2x_factors = gen_diff2_factors(params.lx)
        self._diff2z_factors = gen_diff2_factors(params.lz)
        self._array_factory = array_factory

    # -- physical finite differences -------------------------------------
    def _phys(self, name, var, out):
        pl = self._plan
        src = as_device(var, torch.float64, self._device, pl.physical_shape)
        dst, out = native_target(out, torch.float64, pl.physical_shape, self._device)
        if dst.data_ptr() == src.data_ptr():
            dst = torch.empty_like(src)
        pl.call(name, N.ptr(src), N.ptr(dst), N.stream_handle(self._device))
        return finish(dst, out)

    def pddx(self, var, out=None):
        return self._phys("mgb_pddx", var, out)

    def pddz(self, var, out=None):
        if self._fdm_z and tuple(getattr(var, "shape", ())) == tuple(self._plan.spectral_shape):
            return self._spec(N.DDZ, var, out)
        return self._phys("mgb_pddz", var, out)

    def pd2dz2(self, var, out=None):
        return self._spec(N.D2DZ2, var, out)

    # -- spectral verbs --------------------------------------------------
    def _spec(self, kind, var, out=None):
        pl = self._plan
        src = as_device(var, torch.complex128, self._device, pl.spectral_shape)
        dst, out = native_target(out, torch.complex128, pl.spectral_shape, self._device)
        if dst.data_ptr() == src.data_ptr():
            dst = torch.empty_like(src)
        pl.call("mgb_spectral_derivative", kind, N.ptr(src), N.ptr(dst), N.stream_handle(self._device))
        return finish(dst, out)

    def _check_basis(self, basis_fn, axis):
        if basis_fn is BasisFunctions.COMPLEX_EXP:
            return True
        if basis_fn is BasisFunctions.FDM:
            return False
        raise NotImplementedError(f"{basis_fn!r} derivatives along {axis} are not built for the GPU path")

    def sddx(self, var, basis_fn=BasisFunctions.COMPLEX_EXP):
        if not self._check_basis(basis_fn, "x"):
            return torch.zeros(self._plan.spectral_shape, dtype=torch.complex128, device=self._device)
        return self._spec(N.DDX, var)

    def sddz(self, var, basis_fn=BasisFunctions.COMPLEX_EXP):
        if self._fdm_z:
            return self._spec(N.DDZ, var)
        if not self._check_basis(basis_fn, "z"):
            return torch.zeros(self._plan.spectral_shape, dtype=torch.complex128, device=self._device)
        return self._spec(N.DDZ, var)

    def sd2dx2(self, var, basis_fn=BasisFunctions.COMPLEX_EXP):
        if not self._check_basis(basis_fn, "x"):
            return torch.zeros(self._plan.spectral_shape, dtype=torch.complex128, device=self._device)
        return self._spec(N.D2DX2, var)

    def sd2dz2(self, var, basis_fn=BasisFunctions.COMPLEX_EXP):
        if self._fdm_z:
            return self._spec(N.D2DZ2, var)
        if not self._check_basis(basis_fn, "z"):
            return torch.zeros(self._plan.spectral_shape, dtype=torch.complex128, device=self._device)
        return self._spec(N.D2DZ2, var)

    def snabla2(self, var):
        return self._spec(N.NABLA2, var)

    def calc_lap(self, basis_fns=(BasisFunctions.COMPLEX_EXP, BasisFunctions.COMPLEX_EXP)):
        """Real Laplacian symbol (melvin/SpatialDifferentiator.py:70-74)."""
        for ax, b in zip("xz", basis_fns):
            if b not in (BasisFunctions.COMPLEX_EXP, BasisFunctions.FDM):
                raise NotImplementedError(f"{b!r} along {ax} is not built for the GPU path")
        lap = torch.empty(self._plan.spectral_shape, dtype=torch.float64, device=self._device)
        self._plan.call("mgb_laplacian", N.ptr(lap), N.stream_handle(self._device))
        return lap
