"""Streamfunction inversion (melvin/LaplacianSolver.py) on the GPU.

Fully spectral: ``rhs / lap`` with ``lap[0, 0] := 1`` (:58-68).  Fourier-x /
FDM-z: per x-mode Dirichlet tridiagonal systems (:21-56, 70-79) solved by a
batched Thomas kernel with factors precomputed in the plan.
"""

import numpy as np
import scipy.sparse
import torch

from . import _native as N
from ._arrays import as_device, finish, native_target
from .BasisFunctions import BasisFunctions


class LaplacianSolver:
    def __init__(self, params, xp=None, basis_fns=None, spatial_diff=None, array_factory=None):
        self._params = params
        self._xp = xp
        self._plan = N.plan_for(params)
        self._device = self._plan.device
        self._array_factory = array_factory
        self._laps = None
        self._mirror = None
        if basis_fns is not None and params.is_fully_spectral():
            m = [int(b) if b in (BasisFunctions.COSINE, BasisFunctions.SINE) else 0 for b in basis_fns]
            self._mirror = tuple(m) if any(m) else None
        if params.is_fully_spectral() and spatial_diff is not None:
            self.lap = spatial_diff.calc_lap(basis_fns)

    @property
    def laps(self):
        """Host (scipy CSR) copies of the per-mode Dirichlet matrices, for
        inspection and tests; the device solve never uses them."""
        if self._laps is None:
            p = self._params
            kx = 2 * np.pi / p.lx
            inv = 1.0 / p.dz ** 2
            mats = []
            for n in range(p.nn):
                diag = np.full(p.nz, -((n * kx) ** 2 + 2.0 * inv), dtype=np.complex128)
                lo = np.full(p.nz - 1, inv, dtype=np.complex128)
                up = lo.copy()
                diag[0] = diag[-1] = 1.0
                up[0] = 0.0
                lo[-1] = 0.0
                mats.append(scipy.sparse.diags([lo, diag, up], [-1, 0, 1], format="csr"))
            self._laps = mats
        return self._laps

    def solve(self, rhs, out=None):
        pl = self._plan
        src = as_device(rhs, torch.complex128, self._device, pl.spectral_shape)
        dst, out = native_target(out, torch.complex128, pl.spectral_shape, self._device)
        if dst.data_ptr() == src.data_ptr() and self._params.discretisation[1] == "fdm":
            dst = torch.empty_like(src)
        if self._mirror is None:
            pl.call("mgb_poisson_solve", N.ptr(src), N.ptr(dst), N.stream_handle(self._device))
        else:  # the Laplacian of the cosine / sine bases (melvin/LaplacianSolver.py:58-68)
            pl.call("mgb_poisson_solve_basis", self._mirror[0], self._mirror[1], N.ptr(src), N.ptr(dst),
                    N.stream_handle(self._device))
        return finish(dst, out)
