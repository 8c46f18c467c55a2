"""Spatial derivatives (melvin/SpatialDifferentiator.py) on the GPU.

``pddx``/``pddz``: central finite differences of order 2 or 4 on physical
arrays, periodic along spectral axes, Dirichlet (outer points left 0) along
an FDM axis.  ``sddx``/``sddz``/``sd2dx2``/``sd2dz2``: spectral factors of
the axis basis (complex exponential i*2*pi*n/L, cosine -pi*n/L, sine
pi*n/L, melvin/BasisFunctions.py:26-59); on an FDM z axis ``sddz``/``sd2dz2``
apply the z stencils to the spectral array (:36-43).  ``calc_lap``: the
Laplacian symbol of the bases.
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

    def _spec_basis(self, kind, bx, bz, var, out=None):
        pl = self._plan
        src = as_device(var, torch.complex128, self._device, pl.spectral_shape)
        dst, out = native_target(out, torch.complex128, pl.spectral_shape, self._device)
        pl.call("mgb_spectral_derivative_basis", kind, int(bx), int(bz), N.ptr(src), N.ptr(dst),
                N.stream_handle(self._device))
        return finish(dst, out)

    def _kind_of(self, basis_fn, axis):
        """'exp', 'zero' (FDM axis: factor 0, melvin/BasisFunctions.py:26-36) or 'mirror'."""
        if basis_fn is BasisFunctions.COMPLEX_EXP:
            return "exp"
        if basis_fn is BasisFunctions.FDM:
            return "zero"
        if basis_fn in (BasisFunctions.COSINE, BasisFunctions.SINE):
            return "mirror"
        raise NotImplementedError(f"{basis_fn!r} derivatives along {axis}")

    def _zeros(self):
        return torch.zeros(self._plan.spectral_shape, dtype=torch.complex128, device=self._device)

    def sddx(self, var, basis_fn=BasisFunctions.COMPLEX_EXP):
        k = self._kind_of(basis_fn, "x")
        if k == "zero":
            return self._zeros()
        return self._spec(N.DDX, var) if k == "exp" else self._spec_basis(N.DDX, basis_fn, 0, var)

    def sddz(self, var, basis_fn=BasisFunctions.COMPLEX_EXP):
        if self._fdm_z:
            return self._spec(N.DDZ, var)
        k = self._kind_of(basis_fn, "z")
        if k == "zero":
            return self._zeros()
        return self._spec(N.DDZ, var) if k == "exp" else self._spec_basis(N.DDZ, 0, basis_fn, var)

    def sd2dx2(self, var, basis_fn=BasisFunctions.COMPLEX_EXP):
        k = self._kind_of(basis_fn, "x")
        if k == "zero":
            return self._zeros()
        return self._spec(N.D2DX2, var) if k == "exp" else self._spec_basis(N.D2DX2, basis_fn, 0, var)

    def sd2dz2(self, var, basis_fn=BasisFunctions.COMPLEX_EXP):
        if self._fdm_z:
            return self._spec(N.D2DZ2, var)
        k = self._kind_of(basis_fn, "z")
        if k == "zero":
            return self._zeros()
        return self._spec(N.D2DZ2, var) if k == "exp" else self._spec_basis(N.D2DZ2, 0, basis_fn, var)

    def snabla2(self, var, basis_fns=(BasisFunctions.COMPLEX_EXP, BasisFunctions.COMPLEX_EXP)):
        bx, bz = basis_fns
        if bx in (BasisFunctions.COSINE, BasisFunctions.SINE) or bz in (BasisFunctions.COSINE, BasisFunctions.SINE):
            return self._spec_basis(N.NABLA2, int(bx), int(bz), var)
        return self._spec(N.NABLA2, var)

    def calc_lap(self, basis_fns=(BasisFunctions.COMPLEX_EXP, BasisFunctions.COMPLEX_EXP)):
        """Real Laplacian symbol of the bases (melvin/SpatialDifferentiator.py:70-74)."""
        bx, bz = (basis_fns if basis_fns is not None else (BasisFunctions.COMPLEX_EXP, BasisFunctions.COMPLEX_EXP))
        for ax, b in (("x", bx), ("z", bz)):
            if b not in (BasisFunctions.COMPLEX_EXP, BasisFunctions.FDM, BasisFunctions.COSINE, BasisFunctions.SINE):
                raise NotImplementedError(f"{b!r} along {ax}")
        lap = torch.empty(self._plan.spectral_shape, dtype=torch.float64, device=self._device)
        mirror = [int(b) if b in (BasisFunctions.COSINE, BasisFunctions.SINE) else 0 for b in (bx, bz)]
        if any(mirror):
            self._plan.call("mgb_laplacian_basis", mirror[0], mirror[1], N.ptr(lap), N.stream_handle(self._device))
        else:
            self._plan.call("mgb_laplacian", N.ptr(lap), N.stream_handle(self._device))
        return lap
