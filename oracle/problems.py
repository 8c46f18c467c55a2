"""Loop bodies and seeded initial conditions of the benchmark problems
(test infrastructure only).

A problem is a list of advected fields (field 0 = vorticity), each with a
diffusion coefficient, linear terms and a boundary rule, advanced the way
the reference's example loops do:

* fully spectral: examples/taylor_green_vortex.py:85-95,
  examples/kelvin_helmholtz_instability.py:115-131 (ink update enabled),
  examples/double_diffusive_convection.py:100-126;
* Fourier-x / Dirichlet-z: examples/rayleigh_benard_convection.py:95-145.

All right-hand sides are evaluated at the start-of-step states, as the
examples do.  ``pece`` (AB predictor, re-evaluation, AM corrector) is
defined here from the reference's own formulae (melvin/Integrator.py:5-33);
the reference defines the corrector but never calls it.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import melvin_np as M

BC_ZERO_M0 = 1
BC_DIRICHLET_W = 2
BC_DIRICHLET_T = 4


@dataclass
class FieldSpec:
    kappa: float
    terms: list = field(default_factory=list)  # (src index or -1 for psi, 'value'|'ddx'|'ddz', coef)
    bc: int = 0


def apply_bc(g: M.Grid, q, bc):
    """Boundary rules of the examples, on spectral data in place.

    ZERO_M0: ``q[:, 0] = 0`` (examples/double_diffusive_convection.py:122-124).
    DIRICHLET_W / DIRICHLET_T: examples/rayleigh_benard_convection.py:112-142
    with ``e`` = 1 (order 2) or 2 (order 4) edge points.
    """
    e = g.order // 2
    if bc & BC_ZERO_M0:
        q[:, 0] = 0.0
    if bc & BC_DIRICHLET_W:
        q[1:, :e] = 0.0
        q[1:, -e:] = 0.0
        q[0, :] = 0.0
    if bc & BC_DIRICHLET_T:
        q[0, :e] = 1.0
        q[0, -e:] = 0.0
        q[1:, :e] = 0.0
        q[1:, -e:] = 0.0


class Problem:
    """A set of advected fields with histories, stepped like the examples."""

    def __init__(self, g: M.Grid, specs, states, dt, integrator="semi-implicit", order=2, alpha=0.51):
        self.g = g
        self.specs = list(specs)
        self.q = [np.array(s, dtype=np.complex128) for s in states]
        self.h = [M.History(order, g.spectral_shape) for _ in self.specs]
        self.dt = dt
        self.integrator = integrator
        self.order = order
        self.alpha = alpha
        self.solver = M.PoissonSolver(g)
        self.lap = M.laplacian_symbol(g)
        self.last_velocity = None

    def _rhs(self, states):
        """Right-hand sides (without diffusion) at `states` plus the velocity."""
        g = self.g
        vel = M.velocity_from_vorticity(g, self.solver, states[0])
        out = []
        for i, spec in enumerate(self.specs):
            r = -M.vec_dot_nabla(g, states[i], vel["ux_p"], vel["uz_p"])[0]
            for src, op, coef in spec.terms:
                s = vel["psi_s"] if src < 0 else states[src]
                if op == "ddx":
                    s = M.sddx(g, s)
                elif op == "ddz":
                    s = M.sddz(g, s)
                r = r + coef * s
            out.append(r)
        return out, vel

    def step(self):
        g, dt = self.g, self.dt
        if self.integrator == "semi-implicit":
            rhs, vel = self._rhs(self.q)
            for i, spec in enumerate(self.specs):
                self.h[i].set(rhs[i])
                M.semi_implicit_update(self.q[i], self.h[i], spec.kappa * self.lap, dt, self.alpha)
                apply_bc(g, self.q[i], spec.bc)
        elif self.integrator == "explicit":
            rhs, vel = self._rhs(self.q)
            for i, spec in enumerate(self.specs):
                self.h[i].set(rhs[i])
                M.explicit_update(self.q[i], self.h[i], spec.kappa * M.snabla2(g, self.q[i]), dt)
            for i, spec in enumerate(self.specs):
                apply_bc(g, self.q[i], spec.bc)
        elif self.integrator == "pece":
            q0 = [q.copy() for q in self.q]
            rhs, vel = self._rhs(self.q)
            pred = []
            for i, spec in enumerate(self.specs):
                self.h[i].set(rhs[i] + spec.kappa * M.snabla2(g, self.q[i]))
                p = self.q[i] + M.adams_bashforth(self.h[i], dt)
                apply_bc(g, p, spec.bc)
                pred.append(p)
                self.h[i].advance()
            rhs2, _ = self._rhs(pred)
            for i, spec in enumerate(self.specs):
                self.h[i].set(rhs2[i] + spec.kappa * M.snabla2(g, pred[i]))
                self.q[i] = q0[i] + M.adams_moulton(self.h[i], dt)
                apply_bc(g, self.q[i], spec.bc)
        else:
            raise ValueError(self.integrator)
        self.last_velocity = vel
        return vel


# ---------------------------------------------------------------------------
# Problem definitions (equations) -- mirror melvin.equations
# ---------------------------------------------------------------------------


def vorticity_specs(nu):
    return [FieldSpec(nu)]


def kh_specs(nu, kappa):
    return [FieldSpec(nu), FieldSpec(kappa)]


def ddc_spectral_specs(Pr, R0, tau):
    return [
        FieldSpec(Pr, [(2, "ddx", Pr), (1, "ddx", -Pr)]),
        FieldSpec(1.0, [(-1, "ddx", -1.0)], BC_ZERO_M0),
        FieldSpec(tau, [(-1, "ddx", -1.0 / R0)], BC_ZERO_M0),
    ]


def rbc_specs(Pr, Ra):
    return [FieldSpec(Pr, [(1, "ddx", -Pr * Ra)], BC_DIRICHLET_W), FieldSpec(1.0, [], BC_DIRICHLET_T)]


def ddc_dirichlet_specs(Pr, Ra_T, R_rho, Le):
    return [
        FieldSpec(Pr, [(1, "ddx", -Pr * Ra_T), (2, "ddx", Pr * Ra_T / R_rho)], BC_DIRICHLET_W),
        FieldSpec(1.0, [], BC_DIRICHLET_T),
        FieldSpec(1.0 / Le, [], BC_DIRICHLET_T),
    ]


# ---------------------------------------------------------------------------
# Seeded initial conditions (physical fields)
# ---------------------------------------------------------------------------


def coords(g: M.Grid):
    x = np.linspace(0, g.lx, g.nx, endpoint=False)
    z = np.linspace(0, g.lz, g.nz, endpoint=False)
    return np.meshgrid(x, z, indexing="ij")


def taylor_green_ic(g: M.Grid, eps=1e-3, seed=0):
    """``w = 2 sin x sin z + eps*(2*U-1)`` on [0, 2pi]^2."""
    X, Z = coords(g)
    rng = np.random.default_rng(seed)
    return 2 * np.sin(X) * np.sin(Z) + eps * (2 * rng.random((g.nx, g.nz)) - 1)


def turbulence_ic(g: M.Grid, k0=10.0, seed=0):
    """Vorticity with energy spectrum ``E(k) ~ k^4 exp(-(k/k0)^2)`` and
    uniform random phases, scaled to unit RMS velocity ``sqrt(<ux^2+uz^2>)``
    (velocity from the exact spectral inversion)."""
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(g.nx, d=g.lx / (2 * np.pi * g.nx))
    kz = np.fft.rfftfreq(g.nz, d=g.lz / (2 * np.pi * g.nz))
    KX, KZ = np.meshgrid(kx, kz, indexing="ij")
    k = np.sqrt(KX ** 2 + KZ ** 2)
    E = k ** 4 * np.exp(-((k / k0) ** 2))
    amp = np.sqrt(np.where(k > 0, k * E / np.pi, 0.0))
    phase = rng.uniform(0, 2 * np.pi, size=amp.shape)
    what = amp * np.exp(1j * phase)
    w = np.fft.irfft2(what, s=(g.nx, g.nz))
    wh = np.fft.rfft2(w)
    k2 = np.where(k > 0, k ** 2, 1.0)
    psih = wh / k2
    ux = np.fft.irfft2(-1j * KZ * psih, s=(g.nx, g.nz))
    uz = np.fft.irfft2(1j * KX * psih, s=(g.nx, g.nz))
    rms = np.sqrt(np.mean(ux ** 2 + uz ** 2))
    return w / rms


def kh_ic(g: M.Grid, delta, seed=0, eps=1e-3):
    """Double shear layer ``u(z) = tanh((z-pi)/d) - tanh((z-pi/2)/d)``:
    vorticity ``w = du/dz`` (with ux = -d/dz psi, uz = d/dx psi and
    lap psi = -w, melvin/utility.py:62-79, w = d ux/dz - d uz/dx) plus
    ``eps * sum_{k=1..4} sin(k x + phi_k)`` with seeded phases; passive scalar
    ``c = -u(z)/2`` (1 inside the layer pair, 0 outside)."""
    X, Z = coords(g)
    rng = np.random.default_rng(seed)
    d = delta
    dudz = (1 / np.cosh((Z - np.pi) / d)) ** 2 / d - (1 / np.cosh((Z - np.pi / 2) / d)) ** 2 / d
    u = np.tanh((Z - np.pi) / d) - np.tanh((Z - np.pi / 2) / d)
    phases = rng.uniform(0, 2 * np.pi, size=4)
    pert = sum(np.sin(k * X + phases[k - 1]) for k in range(1, 5))
    return dudz + eps * pert, -0.5 * u


def conductive_ic(g: M.Grid, eps=1e-3, seed=0):
    """``1 - z + eps*(2*U-1)`` on z = linspace(0, lz, nz, endpoint=False)
    (examples/rayleigh_benard_convection.py:22-29 profile)."""
    _, Z = coords(g)
    rng = np.random.default_rng(seed)
    return 1 - Z + eps * (2 * rng.random((g.nx, g.nz)) - 1)
