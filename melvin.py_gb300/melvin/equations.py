"""The loop bodies of the reference examples as fused-step equations.

Each builder returns a :class:`~melvin.stepper.Stepper`.  Citations are to
the example whose loop body the equation restates.
"""

from . import _native as N
from .stepper import FieldEquation, Stepper, Term


def vorticity(sim, w, dw, nu, **kw):
    """Taylor-Green / decaying turbulence: ``dw = -u.grad w``,
    ``lin_op = nu*lap`` (examples/taylor_green_vortex.py:87-93)."""
    return Stepper(sim, [FieldEquation(w, dw, kappa=nu)], **kw)


def kelvin_helmholtz(sim, w, dw, c, dc, nu, kappa, **kw):
    """Vorticity plus a passive scalar ("ink") advected by the same flow,
    each with its own diffusivity (examples/kelvin_helmholtz_instability.py:115-129
    with the ink update enabled)."""
    return Stepper(sim, [FieldEquation(w, dw, kappa=nu), FieldEquation(c, dc, kappa=kappa)], **kw)


def double_diffusive_spectral(sim, w, dw, tmp, dtmp, xi, dxi, Pr, R0, tau, **kw):
    """Fully spectral double-diffusive convection with background gradients
    (examples/double_diffusive_convection.py:100-124)."""
    return Stepper(sim, [
        FieldEquation(w, dw, kappa=Pr, terms=[Term(xi, "ddx", Pr), Term(tmp, "ddx", -Pr)]),
        FieldEquation(tmp, dtmp, kappa=1.0, terms=[Term("psi", "ddx", -1.0)], bc=N.BC_ZERO_M0),
        FieldEquation(xi, dxi, kappa=tau, terms=[Term("psi", "ddx", -1.0 / R0)], bc=N.BC_ZERO_M0),
    ], **kw)


def rayleigh_benard(sim, w, dw, tmp, dtmp, Pr, Ra, **kw):
    """Rayleigh-Benard convection, Fourier x / Dirichlet z, explicit
    diffusion ``Pr*snabla2(w)`` and ``snabla2(tmp)``, buoyancy
    ``-Pr*Ra*d/dx tmp`` and the boundary rules
    (examples/rayleigh_benard_convection.py:97-142)."""
    return Stepper(sim, [
        FieldEquation(w, dw, kappa=Pr, terms=[Term(tmp, "ddx", -Pr * Ra)], bc=N.BC_DIRICHLET_W),
        FieldEquation(tmp, dtmp, kappa=1.0, bc=N.BC_DIRICHLET_T),
    ], **kw)


def double_diffusive_dirichlet(sim, w, dw, T, dT, S, dS, Pr, Ra_T, R_rho, Le, **kw):
    """Double-diffusive convection on the Rayleigh-Benard discretisation:
    temperature T and salinity S with full linear profiles and the RBC
    boundary rules, buoyancy ``-Pr*Ra_T*(dT/dx - dS/dx / R_rho)``, salinity
    diffusivity ``1/Le``.  Composed from
    examples/double_diffusive_convection.py:106-120 (terms, ``tau = 1/Le``,
    ``R0 = R_rho``) and examples/rayleigh_benard_convection.py:97-142
    (discretisation, buoyancy scaling, boundary rules)."""
    return Stepper(sim, [
        FieldEquation(w, dw, kappa=Pr, terms=[Term(T, "ddx", -Pr * Ra_T), Term(S, "ddx", Pr * Ra_T / R_rho)],
                      bc=N.BC_DIRICHLET_W),
        FieldEquation(T, dT, kappa=1.0, bc=N.BC_DIRICHLET_T),
        FieldEquation(S, dS, kappa=1.0 / Le, bc=N.BC_DIRICHLET_T),
    ], **kw)
