"""Helpers of melvin/utility.py, on the GPU where they touch field data."""

import numpy as np
import scipy.sparse
import scipy.sparse.linalg
import torch
from numpy.random import default_rng

from . import _native as N
from .BasisFunctions import BasisFunctions


def sech(x):
    return 1.0 / np.cosh(x)


def load_scipy_sparse(xp=None):
    return scipy.sparse


def load_scipy_sparse_linalg(xp=None):
    return scipy.sparse.linalg


def init_var_with_noise(var, epsilon, seed=0):
    """Uniform noise ``epsilon*(2*U[0,1)-1)`` from ``default_rng(seed)``,
    loaded as physical data (melvin/utility.py:31-39)."""
    rng = default_rng(seed)
    shape = tuple(var.getp().shape)
    data_p = np.zeros(shape)
    data_p += epsilon * (2 * rng.random(shape) - 1.0)
    var.load(data_p, is_physical=True)


def calc_kinetic_energy(ux, uz, xp=None, params=None):
    """``0.5*sum(ux^2+uz^2)/(nx*nz)`` (melvin/utility.py:42-59) as a
    deterministic device reduction; returns a Python float."""
    pl = N.plan_for(params if params is not None else ux._params)
    dev = pl.device
    out = torch.empty(3, dtype=torch.float64, device=dev)
    pl.call("mgb_diagnostics", N.ptr(ux.getp()), N.ptr(uz.getp()), N.ptr(out), N.ptr(pl.work()),
            N.stream_handle(dev))
    return float(out[0].item())


def calc_nusselt_number(tmp, uz, xp=None, params=None):
    """``1 - mean(tmp * uz)`` over the physical fields, the tracker of
    examples/double_diffusive_convection.py:20-23 (after Stellmach et al.
    2011); returns a Python float."""
    return float(1.0 - torch.mean(tmp.getp() * uz.getp()).item())


def calc_velocity_from_vorticity(vorticity, streamfunction, ux, uz, laplacian_solver=None):
    """psi = solve(-w); ux = -d/dz psi, uz = d/dx psi (melvin/utility.py:62-79).

    Fully spectral: writes psi, ux, uz spectral data and ux, uz physical data
    (two kernels).  FDM z: writes psi spectral and physical data, uz spectral
    data and ux, uz physical data; ux spectral data is left untouched, as in
    the reference.
    """
    p = vorticity._params
    pl = N.plan_for(p)
    dev = pl.device
    fdm = streamfunction._basis_functions[1] is BasisFunctions.FDM
    pl.call(
        "mgb_velocity_from_vorticity",
        N.ptr(vorticity._sdata),
        N.ptr(streamfunction._sdata),
        None if fdm else N.ptr(ux._sdata),
        N.ptr(uz._sdata),
        N.ptr(streamfunction._pdata) if fdm else None,
        N.ptr(ux._pdata),
        N.ptr(uz._pdata),
        N.ptr(pl.work()),
        N.stream_handle(dev),
    )
