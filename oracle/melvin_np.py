"""NumPy restatement of Melvin.py's numerics (test infrastructure only).

Each function states the reference behaviour it follows, with the reference
file:line it restates.  The FFTs are ``numpy.fft`` (pocketfft) and the
Dirichlet Poisson factorisation is ``scipy.sparse.linalg.factorized``
(SuperLU): the reference's own third-party calls at
``melvin/SpectralTransformer.py:58,85,132,191`` and
``melvin/LaplacianSolver.py:53-55``, at the versions installed here.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse
import scipy.sparse.linalg


# ---------------------------------------------------------------------------
# Derived grid parameters -- melvin/Parameters.py:63-92
# ---------------------------------------------------------------------------


@dataclass
class Grid:
    """The derived-shape rules of ``Parameters.set_derived_params``.

    melvin/Parameters.py:63-92: ``nn=(nx-1)//3`` for a spectral x axis,
    ``nm=(nz-1)//3`` for a spectral z axis, spectral shape ``(2nn+1, nm)``
    when fully spectral and ``(nn, nz)`` for Fourier-x/FDM-z, ``dx=lx/nx``,
    ``dz=lz/nz`` (also for the Dirichlet axis).
    """

    nx: int
    nz: int
    lx: float
    lz: float
    fdm_z: bool = False
    order: int = 2  # spatial_derivative_order
    nn: int = field(init=False)
    nm: int = field(init=False)

    def __post_init__(self):
        self.nn = (self.nx - 1) // 3
        self.nm = None if self.fdm_z else (self.nz - 1) // 3
        self.dx = self.lx / self.nx
        self.dz = self.lz / self.nz

    @property
    def spectral_shape(self):
        if self.fdm_z:
            return (self.nn, self.nz)
        return (2 * self.nn + 1, self.nm)

    @property
    def physical_shape(self):
        return (self.nx, self.nz)


def mode_numbers(g: Grid):
    """Integer mode-number meshgrids ``(n, m)`` (melvin/ArrayFactory.py:8-26).

    Fully spectral: ``n = 0..nn, -nn..-1`` and ``m = 0..nm-1``;
    Fourier-x/FDM-z: ``n = 0..nn-1`` and ``m = 0..nz-1``.
    """
    if g.fdm_z:
        n = np.arange(g.nn)
        m = np.arange(g.nz)
    else:
        n = np.concatenate((np.arange(g.nn + 1), np.arange(-g.nn, 0)))
        m = np.arange(g.nm)
    return np.meshgrid(n, m, indexing="ij")


# ---------------------------------------------------------------------------
# Transforms -- melvin/SpectralTransformer.py
# ---------------------------------------------------------------------------


def to_physical(g: Grid, s: np.ndarray) -> np.ndarray:
    """Spectral -> physical.

    Fully spectral (melvin/SpectralTransformer.py:90-150 with _scale_2d 21-24):
    the ``(2nn+1, nm)`` block is placed in a zero ``(nx, nz//2+1)`` array --
    rows ``0..nn`` at the top, rows ``-nn..-1`` at the bottom, columns
    ``0..nm-1`` -- multiplied by ``nx*nz`` and passed to ``irfft2``.

    Fourier-x/FDM-z (melvin/SpectralTransformer.py:33-61 with _scale_1d
    26-31): rows ``0..nn-1`` go into a zero ``(nx//2+1, nz)`` array,
    multiplied by ``nx``, ``irfft`` along x (axis 0).
    """
    if g.fdm_z:
        pad = np.zeros((g.nx // 2 + 1, g.nz), dtype=np.complex128)
        pad[: g.nn] = s[: g.nn]
        return np.fft.irfft(pad * g.nx, n=g.nx, axis=0)
    nn, nm = g.nn, g.nm
    pad = np.zeros((g.nx, g.nz // 2 + 1), dtype=np.complex128)
    pad[: nn + 1, :nm] = s[: nn + 1, :nm]
    pad[-nn:, :nm] = s[-nn:, :nm]
    pad *= g.nx * g.nz
    return np.fft.irfft2(pad, s=(g.nx, g.nz))


def to_spectral(g: Grid, p: np.ndarray) -> np.ndarray:
    """Physical -> spectral, the inverse of :func:`to_physical`.

    Fully spectral (melvin/SpectralTransformer.py:152-199): ``rfft2`` divided
    by ``nx*nz``, keeping rows ``0..nn`` and ``-nn..-1`` and columns
    ``0..nm-1``.  Fourier-x/FDM-z (melvin/SpectralTransformer.py:63-88):
    ``rfft`` along x divided by ``nx``, keeping rows ``0..nn-1``.
    """
    if g.fdm_z:
        f = np.fft.rfft(p, axis=0) / g.nx
        return np.ascontiguousarray(f[: g.nn])
    nn, nm = g.nn, g.nm
    f = np.fft.rfft2(p) / (g.nx * g.nz)
    out = np.empty((2 * nn + 1, nm), dtype=np.complex128)
    out[: nn + 1] = f[: nn + 1, :nm]
    out[-nn:] = f[-nn:, :nm]
    return out


# Cosine / sine bases -- melvin/SpectralTransformer.py:90-199 with
# BasisFunctions.COSINE (1) and SINE (2) on a fully spectral grid.  A cosine
# or sine axis of n points is the mirrored periodic signal of 2(n-1) points
# (even extension for cosine, odd for sine); x_factor / z_factor are n, n-1
# or -1j*(n-1); the zeroth cosine mode is doubled before the inverse and
# halved after the forward transform.  (The reference doubles it in its
# input array in place; this restatement works on a copy.)
EXP, COS, SIN = 0, 1, 2


def _axis_factor(basis, n):
    if basis == COS:
        return n - 1
    if basis == SIN:
        return -1j * (n - 1)
    return n


def _axis_len(basis, n):
    return 2 * (n - 1) if basis in (COS, SIN) else n


def to_physical_basis(g: Grid, s: np.ndarray, bx: int, bz: int) -> np.ndarray:
    nn, nm = g.nn, g.nm
    s = np.array(s, dtype=np.complex128, copy=True)
    if bx == COS:
        s[0] *= 2
    if bz == COS:
        s[:, 0] *= 2
    lx = _axis_len(bx, g.nx)
    hz = 2 * (g.nz - 1) // 2 + 1 if bz in (COS, SIN) else g.nz // 2 + 1
    pad = np.zeros((lx, hz), dtype=np.complex128)
    pad[: nn + 1, :nm] = s[: nn + 1, :nm]
    pad[-nn:, :nm] = s[-nn:, :nm]
    pad *= _axis_factor(bx, g.nx) * _axis_factor(bz, g.nz)
    out = np.fft.irfft2(pad)
    if bx in (COS, SIN):
        out = out[: g.nx]
    if bz in (COS, SIN):
        out = out[:, : g.nz]
    return out


def to_spectral_basis(g: Grid, p: np.ndarray, bx: int, bz: int) -> np.ndarray:
    nn, nm = g.nn, g.nm
    a = np.asarray(p, dtype=np.float64)
    if bx == COS:
        a = np.concatenate((a[:-1], a[:0:-1]))
    elif bx == SIN:
        a = np.concatenate((a[:-1], -a[:0:-1]))
    if bz == COS:
        a = np.concatenate((a[:, :-1], a[:, :0:-1]), axis=1)
    elif bz == SIN:
        a = np.concatenate((a[:, :-1], -a[:, :0:-1]), axis=1)
    f = np.fft.rfft2(a) / (_axis_factor(bx, g.nx) * _axis_factor(bz, g.nz))
    if bx == COS:
        f[0] /= 2
    if bz == COS:
        f[:, 0] /= 2
    out = np.empty((2 * nn + 1, nm), dtype=np.complex128)
    out[: nn + 1] = f[: nn + 1, :nm]
    out[-nn:] = f[-nn:, :nm]
    return out


def _basis_dfac(basis, length):
    # calc_diff_wavelength / L (melvin/BasisFunctions.py:26-36,44-52)
    return {EXP: 1j * 2 * np.pi, SIN: np.pi, COS: -np.pi}[basis] / length


def _basis_d2fac(basis, length):
    # -|wavelength|^2 / L^2 (melvin/BasisFunctions.py:39-42,55-59)
    return -np.abs({EXP: 1j * 2 * np.pi, SIN: np.pi, COS: -np.pi}[basis]) ** 2 / length ** 2


def sddx_basis(g: Grid, s, bx):
    n, _ = mode_numbers(g)
    return _basis_dfac(bx, g.lx) * n * s


def sddz_basis(g: Grid, s, bz):
    _, m = mode_numbers(g)
    return _basis_dfac(bz, g.lz) * m * s


def sd2dx2_basis(g: Grid, s, bx):
    n, _ = mode_numbers(g)
    return _basis_d2fac(bx, g.lx) * n ** 2 * s


def sd2dz2_basis(g: Grid, s, bz):
    _, m = mode_numbers(g)
    return _basis_d2fac(bz, g.lz) * m ** 2 * s


def laplacian_symbol_basis(g: Grid, bx, bz):
    n, m = mode_numbers(g)
    return _basis_d2fac(bx, g.lx) * n ** 2 + _basis_d2fac(bz, g.lz) * m ** 2


def poisson_basis(g: Grid, rhs, bx, bz):
    """_solve_fully_spectral with the Laplacian of the bases, (0, 0) divided
    by 1 (melvin/LaplacianSolver.py:58-68)."""
    lap = laplacian_symbol_basis(g, bx, bz).astype(np.complex128)
    lap[0, 0] = 1.0
    return rhs / lap


# ---------------------------------------------------------------------------
# Finite-difference stencils -- melvin/SpatialDifferentiator.py:76-185
# ---------------------------------------------------------------------------


def _central_diff(v: np.ndarray, h: float, axis: int, order: int, periodic: bool):
    """First derivative by a central stencil along ``axis``.

    Order 2: ``(v[i+1]-v[i-1])/(2h)`` (melvin/SpatialDifferentiator.py:76-104).
    Order 4: ``(-v[i+2]/4 + 2v[i+1] - 2v[i-1] + v[i-2]/4)/(3h)``
    (melvin/SpatialDifferentiator.py:130-185).  A periodic axis wraps; a
    Dirichlet axis leaves the outer 1 (order 2) or 2 (order 4) points at 0.
    """
    vv = np.moveaxis(v, axis, 0)
    out = np.zeros_like(vv)
    if order == 2:
        if periodic:
            out[:] = (np.roll(vv, -1, 0) - np.roll(vv, 1, 0)) / (2 * h)
        else:
            out[1:-1] = (vv[2:] - vv[:-2]) / (2 * h)
    elif order == 4:
        if periodic:
            out[:] = (
                -0.25 * np.roll(vv, -2, 0)
                + 2 * np.roll(vv, -1, 0)
                - 2 * np.roll(vv, 1, 0)
                + 0.25 * np.roll(vv, 2, 0)
            ) / (3 * h)
        else:
            out[2:-2] = (
                -0.25 * vv[4:] + 2 * vv[3:-1] - 2 * vv[1:-3] + 0.25 * vv[:-4]
            ) / (3 * h)
    else:
        raise NotImplementedError(f"spatial_derivative_order={order}")
    return np.moveaxis(out, 0, axis)


def pddx(g: Grid, v: np.ndarray) -> np.ndarray:
    """Physical d/dx; x is always periodic on this path."""
    return _central_diff(v, g.dx, 0, g.order, periodic=True)


def pddz(g: Grid, v: np.ndarray) -> np.ndarray:
    """Physical d/dz; periodic when z is spectral, Dirichlet when FDM."""
    return _central_diff(v, g.dz, 1, g.order, periodic=not g.fdm_z)


def pd2dz2(g: Grid, v: np.ndarray) -> np.ndarray:
    """FD second derivative along z applied to a (complex) spectral array.

    melvin/SpatialDifferentiator.py:106-128: interior only, order 2
    ``(v[j+1]-2v[j]+v[j-1])/dz^2`` on ``1..nz-2``; order 4
    ``(-v[j+2]/12 + 4v[j+1]/3 - 5v[j]/2 + 4v[j-1]/3 - v[j-2]/12)/dz^2`` on
    ``2..nz-3``; the boundary columns stay 0.
    """
    out = np.zeros_like(v)
    dz2 = g.dz ** 2
    if g.order == 2:
        out[:, 1:-1] = (v[:, 2:] - 2 * v[:, 1:-1] + v[:, :-2]) / dz2
    elif g.order == 4:
        out[:, 2:-2] = (
            -1.0 / 12 * v[:, 4:]
            + 4.0 / 3 * v[:, 3:-1]
            - 5.0 / 2 * v[:, 2:-2]
            + 4.0 / 3 * v[:, 1:-3]
            - 1.0 / 12 * v[:, :-4]
        ) / dz2
    else:
        raise NotImplementedError(f"spatial_derivative_order={g.order}")
    return out


# ---------------------------------------------------------------------------
# Spectral derivative verbs -- melvin/SpatialDifferentiator.py:50-74,
# factors from melvin/BasisFunctions.py:26-59 (complex-exponential basis)
# ---------------------------------------------------------------------------


def _dfac(length):
    # calc_diff_wavelength(COMPLEX_EXP) / L  (melvin/BasisFunctions.py:26-36)
    return 1j * 2 * np.pi / length


def _d2fac(length):
    # -|2*pi*i|^2 / L^2  (melvin/BasisFunctions.py:39-42,55-59)
    return -np.abs(1j * 2 * np.pi) ** 2 / length ** 2


def sddx(g: Grid, s):
    n, _ = mode_numbers(g)
    return _dfac(g.lx) * n * s


def sddz(g: Grid, s):
    """Spectral d/dz; for FDM-z the reference binds ``pddz`` instead
    (melvin/SpatialDifferentiator.py:36-40)."""
    if g.fdm_z:
        return pddz(g, s)
    _, m = mode_numbers(g)
    return _dfac(g.lz) * m * s


def sd2dx2(g: Grid, s):
    n, _ = mode_numbers(g)
    return _d2fac(g.lx) * n ** 2 * s


def sd2dz2(g: Grid, s):
    if g.fdm_z:
        return pd2dz2(g, s)
    _, m = mode_numbers(g)
    return _d2fac(g.lz) * m ** 2 * s


def snabla2(g: Grid, s):
    """``Variable.snabla2`` = sd2dx2 + sd2dz2 (melvin/Variable.py:111-113)."""
    return sd2dx2(g, s) + sd2dz2(g, s)


def laplacian_symbol(g: Grid):
    """``calc_lap`` (melvin/SpatialDifferentiator.py:70-74): real array
    ``d2x*n^2 + d2z*m^2``; entry (0, 0) is 0.  On an FDM z axis the z factor
    is that of the FDM basis, ``-|0|^2/lz^2`` (melvin/BasisFunctions.py:26-42),
    so only the x term remains."""
    n, m = mode_numbers(g)
    d2z = -np.abs(0) ** 2 / g.lz ** 2 if g.fdm_z else _d2fac(g.lz)
    return _d2fac(g.lx) * n ** 2 + d2z * m ** 2


# ---------------------------------------------------------------------------
# Streamfunction inversion -- melvin/LaplacianSolver.py
# ---------------------------------------------------------------------------


class PoissonSolver:
    """Solve ``lap(psi) = rhs`` for psi.

    Fully spectral (melvin/LaplacianSolver.py:58-68): ``rhs / lap`` with the
    (0, 0) entry of ``lap`` replaced by 1.

    Fourier-x/FDM-z (melvin/LaplacianSolver.py:21-56, 70-79): for each x-mode
    ``n < nn`` a complex tridiagonal matrix with off-diagonals ``1/dz^2`` and
    diagonal ``-((n*2*pi/lx)^2 + 2/dz^2)``, whose first and last rows are the
    identity (so psi equals rhs there), LU-factorised by SuperLU.  The
    second-order operator is used whatever the spatial derivative order.
    """

    def __init__(self, g: Grid):
        self.g = g
        if not g.fdm_z:
            lap = laplacian_symbol(g)
            lap[0, 0] = 1.0
            self._lap = lap
            return
        kx = 2 * np.pi / g.lx
        inv_dz2 = 1.0 / g.dz ** 2
        self.mats = []
        self._solvers = []
        for n in range(g.nn):
            diag = np.full(g.nz, -((n * kx) ** 2 + 2.0 * inv_dz2))
            off = np.full(g.nz - 1, inv_dz2)
            diag[0] = diag[-1] = 1.0
            upper = off.copy()
            lower = off.copy()
            upper[0] = 0.0  # row 0 -> identity
            lower[-1] = 0.0  # row nz-1 -> identity
            a = scipy.sparse.diags(
                [lower, diag, upper], [-1, 0, 1], shape=(g.nz, g.nz),
                dtype=np.complex128, format="csc",
            )
            self.mats.append(a)
            self._solvers.append(scipy.sparse.linalg.factorized(a))

    def solve(self, rhs):
        if not self.g.fdm_z:
            return rhs / self._lap
        out = np.empty_like(rhs)
        for n in range(self.g.nn):
            out[n] = self._solvers[n](rhs[n])
        return out


# ---------------------------------------------------------------------------
# Nonlinear term and velocity -- melvin/Variable.py:119-128,
# melvin/utility.py:62-79
# ---------------------------------------------------------------------------


def vec_dot_nabla(g: Grid, q_s, ux_p, uz_p):
    """``Variable.vec_dot_nabla`` (melvin/Variable.py:119-128): physical q,
    then ``pddx(ux*q) + pddz(uz*q)`` and one forward transform.

    Returns ``(spectral result, physical q)``.
    """
    q_p = to_physical(g, q_s)
    j = pddx(g, ux_p * q_p) + pddz(g, uz_p * q_p)
    return to_spectral(g, j), q_p


def velocity_from_vorticity(g: Grid, solver: PoissonSolver, w_s):
    """``calc_velocity_from_vorticity`` (melvin/utility.py:62-79).

    ``psi = solve(-w)``.  ``uz = d/dx psi`` is always the spectral x
    derivative (x is a complex-exponential axis), then to physical.  Fully
    spectral: ``ux = -d/dz psi`` spectrally, then to physical.  FDM-z: psi to
    physical and ``ux = -pddz(psi)`` by the Dirichlet stencil; ux's spectral
    array stays untouched (zero).

    Returns a dict with psi_s, ux_s, uz_s, ux_p, uz_p (and psi_p for FDM-z).
    """
    psi_s = solver.solve(-w_s)
    out = {"psi_s": psi_s}
    if g.fdm_z:
        psi_p = to_physical(g, psi_s)
        out["psi_p"] = psi_p
        out["ux_p"] = -pddz(g, psi_p)
        out["ux_s"] = np.zeros_like(psi_s)
        out["uz_s"] = sddx(g, psi_s)
        out["uz_p"] = to_physical(g, out["uz_s"])
    else:
        ux_s = -sddz(g, psi_s)
        uz_s = sddx(g, psi_s)
        out["ux_s"] = ux_s
        out["uz_s"] = uz_s
        out["ux_p"] = to_physical(g, ux_s)
        out["uz_p"] = to_physical(g, uz_s)
    return out


# ---------------------------------------------------------------------------
# Time derivative history and integrators -- melvin/TimeDerivative.py,
# melvin/Integrator.py
# ---------------------------------------------------------------------------


class History:
    """Ring buffer of ``order`` spectral slots (melvin/TimeDerivative.py:9-39).

    Starts at zeros with ``curr = 0``; ``get(i)`` reads slot ``curr + i``
    with Python negative-index wrap; ``advance`` rotates ``curr``.
    """

    def __init__(self, order, shape):
        self.order = order
        self.data = np.zeros((order,) + tuple(shape), dtype=np.complex128)
        self.curr = 0

    def set(self, value):
        self.data[self.curr] = value

    def add(self, value):
        self.data[self.curr] += value

    def get(self, i=0):
        return self.data[self.curr + i]

    def advance(self):
        self.curr = (self.curr + 1) % self.order


def adams_bashforth(h: History, dt):
    """AB2 ``dt/2 (3f0 - f-1)`` / AB4 ``dt/24 (55f0 - 59f-1 + 37f-2 - 9f-3)``
    (melvin/Integrator.py:5-18)."""
    if h.order == 2:
        return dt / 2 * (3 * h.get() - h.get(-1))
    if h.order == 4:
        return dt / 24 * (55 * h.get() - 59 * h.get(-1) + 37 * h.get(-2) - 9 * h.get(-3))
    raise NotImplementedError(f"integrator_order={h.order}")


def adams_moulton(h: History, dt):
    """AM2 ``dt/2 (f0 + f-1)`` / AM4 ``dt/24 (9f0 + 19f-1 - 5f-2 + f-3)``
    (melvin/Integrator.py:20-33)."""
    if h.order == 2:
        return dt / 2 * (h.get() + h.get(-1))
    if h.order == 4:
        return dt / 24 * (9 * h.get() + 19 * h.get(-1) - 5 * h.get(-2) + h.get(-3))
    raise NotImplementedError(f"integrator_order={h.order}")


def semi_implicit_update(q, h: History, lin_op, dt, alpha):
    """``_semi_implicit_spectral`` (melvin/Integrator.py:58-63): in place
    ``q = ((1+(1-a)dt L) q + AB(h)) / (1 - a dt L)``, then advance."""
    rhs = (1 + (1 - alpha) * dt * lin_op) * q + adams_bashforth(h, dt)
    q[:] = rhs / (1 - alpha * dt * lin_op)
    h.advance()


def explicit_update(q, h: History, diffusion, dt):
    """``_explicit`` (melvin/Integrator.py:53-56): ``f0 += D``, ``q += AB(h)``,
    advance."""
    h.add(diffusion)
    q += adams_bashforth(h, dt)
    h.advance()


# ---------------------------------------------------------------------------
# Diagnostics -- melvin/utility.py:42-59, melvin/Integrator.py:35-44
# ---------------------------------------------------------------------------


def kinetic_energy(g: Grid, ux_p, uz_p):
    """``0.5 * sum(ux^2 + uz^2) / (nx*nz)`` (melvin/utility.py:42-59)."""
    return 0.5 * np.sum(uz_p ** 2 + ux_p ** 2) / (g.nx * g.nz)


def cfl_dt(g: Grid, ux_p, uz_p, dt, cutoff):
    """``Integrator.set_dt`` (melvin/Integrator.py:35-44).

    ``cfl = min(dx/max(ux), dz/max(uz))`` with the signed maximum; raises on
    ``dt > cfl`` or NaN; otherwise shrinks dt by 0.9 until
    ``dt <= cutoff*cfl``.  Returns the new dt.
    """
    c = min(g.dx / np.max(ux_p), g.dz / np.max(uz_p))
    if dt > c or math.isnan(c):
        raise RuntimeError("CFL condition breached")
    while dt > cutoff * c:
        dt = dt * 0.9
    return dt
