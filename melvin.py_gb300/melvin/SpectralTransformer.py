"""Physical <-> spectral transforms (melvin/SpectralTransformer.py) on the GPU.

Fully spectral grids use the 2D path (:90-199): 2/3 truncation to
``(2nn+1, nm)``, ``*nx*nz`` before the inverse and ``/(nx*nz)`` after the
forward transform.  Fourier-x / FDM-z grids use the x-only path (:33-88).
Cosine and sine bases are not built for the GPU.
"""

import torch

from . import _native as N
from ._arrays import as_device, finish, native_target
from .BasisFunctions import BasisFunctions

_EXP = BasisFunctions.COMPLEX_EXP
_FDM = BasisFunctions.FDM


class SpectralTransformer:
    def __init__(self, params, xp=None, array_factory=None):
        self._p = params
        self._xp = xp
        self._array_factory = array_factory
        self._plan = N.plan_for(params)
        self._device = self._plan.device

    def _check_basis(self, basis_functions):
        b = list(basis_functions)
        want = [_EXP, _FDM] if self._p.discretisation[1] == "fdm" else [_EXP, _EXP]
        if b != want:
            raise NotImplementedError(
                f"basis functions {b} are not built for the GPU path (expected {want})"
            )

    def to_physical(self, in_arr, out=None, basis_functions=(_EXP, _EXP)):
        if self._p.discretisation[1] == "fdm" and list(basis_functions) == [_EXP, _EXP]:
            basis_functions = (_EXP, _FDM)
        self._check_basis(basis_functions)
        pl = self._plan
        src = as_device(in_arr, torch.complex128, self._device, pl.spectral_shape)
        dst, out = native_target(out, torch.float64, pl.physical_shape, self._device)
        pl.call("mgb_to_physical", N.ptr(src), N.ptr(dst), N.ptr(pl.work()), N.stream_handle(self._device))
        return finish(dst, out)

    def to_spectral(self, in_arr, out=None, basis_functions=(_EXP, _EXP)):
        if self._p.discretisation[1] == "fdm" and list(basis_functions) == [_EXP, _EXP]:
            basis_functions = (_EXP, _FDM)
        self._check_basis(basis_functions)
        pl = self._plan
        src = as_device(in_arr, torch.float64, self._device, pl.physical_shape)
        dst, out = native_target(out, torch.complex128, pl.spectral_shape, self._device)
        pl.call("mgb_to_spectral", N.ptr(src), N.ptr(dst), N.ptr(pl.work()), N.stream_handle(self._device))
        return finish(dst, out)
