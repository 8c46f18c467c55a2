"""Physical <-> spectral transforms (melvin/SpectralTransformer.py) on the GPU.

Fully spectral grids use the 2D path (:90-199): 2/3 truncation to
``(2nn+1, nm)``, ``*nx*nz`` before the inverse and ``/(nx*nz)`` after the
forward transform.  Fourier-x / FDM-z grids use the x-only path (:33-88).  Cosine and sine
bases (:108-146, :169-196) use mirrored transforms of 2(n-1) points; any
transform length in [16, 4096] runs (powers of two as block FFTs, others as
Bluestein convolutions).  Unlike the reference, to_physical does not double
the zeroth cosine mode of its input in place.
"""

import torch

from . import _native as N
from ._arrays import as_device, finish, native_target
from .BasisFunctions import BasisFunctions

_EXP = BasisFunctions.COMPLEX_EXP
_FDM = BasisFunctions.FDM
_COS = BasisFunctions.COSINE
_SIN = BasisFunctions.SINE


class SpectralTransformer:
    def __init__(self, params, xp=None, array_factory=None):
        self._p = params
        self._xp = xp
        self._array_factory = array_factory
        self._plan = N.plan_for(params)
        self._device = self._plan.device

    def _basis(self, basis_functions):
        """None for the default basis of the grid, else (bx, bz) of a
        cosine / sine combination."""
        b = list(basis_functions)
        if self._p.discretisation[1] == "fdm":
            if b in ([_EXP, _EXP], [_EXP, _FDM]):
                return None
            raise NotImplementedError(f"basis functions {b} on a Dirichlet z grid (expected [COMPLEX_EXP, FDM])")
        if any(x not in (_EXP, _COS, _SIN) for x in b):
            raise NotImplementedError(f"basis functions {b} on a fully spectral grid")
        if b == [_EXP, _EXP]:
            return None
        return int(b[0]), int(b[1])

    def to_physical(self, in_arr, out=None, basis_functions=(_EXP, _EXP)):
        basis = self._basis(basis_functions)
        pl = self._plan
        src = as_device(in_arr, torch.complex128, self._device, pl.spectral_shape)
        dst, out = native_target(out, torch.float64, pl.physical_shape, self._device)
        if basis is None:
            pl.call("mgb_to_physical", N.ptr(src), N.ptr(dst), N.ptr(pl.work()), N.stream_handle(self._device))
        else:
            pl.call("mgb_to_physical_basis", basis[0], basis[1], N.ptr(src), N.ptr(dst), N.ptr(pl.work()),
                    N.stream_handle(self._device))
        return finish(dst, out)

    def to_spectral(self, in_arr, out=None, basis_functions=(_EXP, _EXP)):
        basis = self._basis(basis_functions)
        pl = self._plan
        src = as_device(in_arr, torch.float64, self._device, pl.physical_shape)
        dst, out = native_target(out, torch.complex128, pl.spectral_shape, self._device)
        if basis is None:
            pl.call("mgb_to_spectral", N.ptr(src), N.ptr(dst), N.ptr(pl.work()), N.stream_handle(self._device))
        else:
            pl.call("mgb_to_spectral_basis", basis[0], basis[1], N.ptr(src), N.ptr(dst), N.ptr(pl.work()),
                    N.stream_handle(self._device))
        return finish(dst, out)
