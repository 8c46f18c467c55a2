"""Generate golden vectors by running the reference Melvin.py (NumPy backend).

Run in a container that has the reference checked out (default location
``/root/reference``, or pass it as the first argument):

    python tests/golden/make_golden.py [/path/to/Melvin.py]

It writes ``tests/golden/reference_golden.npz``: seeded inputs and the
reference's outputs for every verb of the hot path at small sizes, plus
short trajectories of the example loop bodies (Taylor-Green, Kelvin-Helmholtz
with ink, fully spectral double-diffusive convection, Rayleigh-Benard and
double-diffusive convection on the Fourier-x/Dirichlet-z grid, and a
predictor-corrector composed from the reference's own AB4/AM4 formulae).
The reference package is imported unmodified; nothing here is shipped.
"""

import io
import os
import sys
from contextlib import redirect_stdout

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
sys.path.insert(0, REF)

from melvin import BasisFunctions, Parameters, Simulation  # noqa: E402
from melvin.utility import calc_kinetic_energy, calc_velocity_from_vorticity  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.npz")
EXP = BasisFunctions.COMPLEX_EXP
FDM = BasisFunctions.FDM
G = {}


def params(nx, nz, lx, lz, fdm=False, order=2, iorder=2, integrator="semi-implicit", dt=1e-3):
    d = {
        "nx": nx, "nz": nz, "lx": lx, "lz": lz, "final_time": 1.0, "initial_dt": dt,
        "spatial_derivative_order": order, "integrator_order": iorder, "integrator": integrator,
        "discretisation": ["spectral", "fdm" if fdm else "spectral"],
    }
    return Parameters(d)


def rand_spec(rng, shape, hermitian_m0=False):
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    return a


def verbs(tag, p, rng):
    """Unit outputs of every verb on seeded inputs."""
    with redirect_stdout(io.StringIO()):
        sim = Simulation(p, np)
    fdm = p.discretisation[1] == "fdm"
    bf = [EXP, FDM] if fdm else [EXP, EXP]
    st, sd = sim._spectral_trans, sim._spatial_diff
    s = rand_spec(rng, p.spectral_shape)
    phys = rng.standard_normal((p.nx, p.nz))
    ux = rng.standard_normal((p.nx, p.nz))
    uz = rng.standard_normal((p.nx, p.nz))
    G[f"{tag}/in_spec"] = s
    G[f"{tag}/in_phys"] = phys
    G[f"{tag}/in_ux"] = ux
    G[f"{tag}/in_uz"] = uz
    G[f"{tag}/to_physical"] = st.to_physical(s.copy(), basis_functions=bf)
    G[f"{tag}/to_spectral"] = st.to_spectral(phys.copy(), basis_functions=bf)
    G[f"{tag}/pddx"] = sd.pddx(phys.copy())
    G[f"{tag}/pddz"] = sd.pddz(phys.copy())
    q = sim.make_variable("q", bf)
    q.sets(s.copy())
    G[f"{tag}/sddx"] = q.sddx()
    G[f"{tag}/sd2dx2"] = q.sd2dx2()
    G[f"{tag}/snabla2"] = q.snabla2()
    G[f"{tag}/lap"] = q.lap()
    if not fdm:
        G[f"{tag}/sddz"] = q.sddz()
        G[f"{tag}/sd2dz2"] = q.sd2dz2()
    else:
        G[f"{tag}/pd2dz2"] = sd.pd2dz2(s.copy())
    G[f"{tag}/vec_dot_nabla"] = q.vec_dot_nabla(ux, uz)
    G[f"{tag}/vec_dot_nabla_phys"] = q.getp().copy()
    with redirect_stdout(io.StringIO()):
        sim.init_laplacian_solver(bf)
    solver = sim.get_laplacian_solver()
    G[f"{tag}/poisson"] = solver.solve(s.copy())
    w = sim.make_variable("w", bf)
    psi = sim.make_variable("psi", bf)
    vx = sim.make_variable("ux", bf)
    vz = sim.make_variable("uz", bf)
    w.sets(s.copy())
    calc_velocity_from_vorticity(w, psi, vx, vz, solver)
    G[f"{tag}/vel_psi"] = psi.gets().copy()
    G[f"{tag}/vel_ux_p"] = vx.getp().copy()
    G[f"{tag}/vel_uz_p"] = vz.getp().copy()
    if not fdm:
        G[f"{tag}/vel_ux_s"] = vx.gets().copy()
        G[f"{tag}/vel_uz_s"] = vz.gets().copy()
    else:
        G[f"{tag}/vel_psi_p"] = psi.getp().copy()
    G[f"{tag}/ke"] = np.float64(calc_kinetic_energy(vx, vz, np, p))
    # integrators on a random history
    dv = sim.make_derivative("dq")
    for k in range(p.integrator_order):
        dv.advance()
        dv[:] = rand_spec(rng, p.spectral_shape)
    dv.set_curr_idx(1)
    G[f"{tag}/hist"] = dv.get_all().copy()
    G[f"{tag}/ab"] = sim._integrator.predictor(dv)
    G[f"{tag}/am"] = sim._integrator.corrector(dv)


def basis_verbs(tag, p, bf, rng):
    """The reference's cosine / sine basis transforms and spectral verbs
    (melvin/SpectralTransformer.py:90-199, melvin/SpatialDifferentiator.py:50-74,
    melvin/LaplacianSolver.py:58-68) on seeded inputs.  to_physical doubles
    the zeroth cosine mode of its input in place, so it gets a copy."""
    with redirect_stdout(io.StringIO()):
        sim = Simulation(p, np)
    st = sim._spectral_trans
    s = rand_spec(rng, p.spectral_shape)
    phys = rng.standard_normal((p.nx, p.nz))
    G[f"{tag}/in_spec"] = s
    G[f"{tag}/in_phys"] = phys
    G[f"{tag}/basis"] = np.array([int(bf[0]), int(bf[1])])
    G[f"{tag}/to_physical"] = st.to_physical(s.copy(), basis_functions=bf)
    G[f"{tag}/to_spectral"] = st.to_spectral(phys.copy(), basis_functions=bf)
    q = sim.make_variable("q", bf)
    q.sets(s.copy())
    for verb in ("sddx", "sddz", "sd2dx2", "sd2dz2", "snabla2", "lap"):
        G[f"{tag}/{verb}"] = getattr(q, verb)()
    with redirect_stdout(io.StringIO()):
        sim.init_laplacian_solver(bf)
    G[f"{tag}/poisson"] = sim.get_laplacian_solver().solve(s.copy())


def trajectory(tag, p, fields, init, nsteps, body):
    """Run `nsteps` of `body` with the reference objects; store states."""
    with redirect_stdout(io.StringIO()):
        sim = Simulation(p, np)
    fdm = p.discretisation[1] == "fdm"
    bf = [EXP, FDM] if fdm else [EXP, EXP]
    V = {name: sim.make_variable(name, bf) for name in fields + ["psi", "ux", "uz"]}
    D = {name: sim.make_derivative("d" + name) for name in fields}
    with redirect_stdout(io.StringIO()):
        sim.init_laplacian_solver(bf)
    for name, arr in init.items():
        V[name].load(arr, is_physical=True)
        G[f"{tag}/init_{name}"] = arr
    for name in fields:
        G[f"{tag}/s0_{name}"] = V[name].gets().copy()
    ke = []
    for n in range(nsteps):
        body(sim, p, V, D)
        ke.append(calc_kinetic_energy(V["ux"], V["uz"], np, p))
        for name in fields:
            G[f"{tag}/s{n + 1}_{name}"] = V[name].gets().copy()
    G[f"{tag}/ke"] = np.array(ke)
    G[f"{tag}/nsteps"] = np.int64(nsteps)


def tg_body(nu):
    def body(sim, p, V, D):
        w = V["w"]
        calc_velocity_from_vorticity(w, V["psi"], V["ux"], V["uz"], sim.get_laplacian_solver())
        lin_op = nu * w.lap()
        D["w"][:] = -w.vec_dot_nabla(V["ux"].getp(), V["uz"].getp())
        sim._integrator.integrate(w, D["w"], lin_op)
    return body


def kh_body(nu, kappa):
    def body(sim, p, V, D):
        w, c = V["w"], V["c"]
        calc_velocity_from_vorticity(w, V["psi"], V["ux"], V["uz"], sim.get_laplacian_solver())
        lin_op = nu * w.lap()
        D["w"][:] = -w.vec_dot_nabla(V["ux"].getp(), V["uz"].getp())
        sim._integrator.integrate(w, D["w"], lin_op)
        lin_op = kappa * c.lap()
        D["c"][:] = -c.vec_dot_nabla(V["ux"].getp(), V["uz"].getp())
        sim._integrator.integrate(c, D["c"], lin_op)
    return body


def ddc_spectral_body(Pr, R0, tau):
    def body(sim, p, V, D):
        w, tmp, xi, uz = V["w"], V["tmp"], V["xi"], V["uz"]
        calc_velocity_from_vorticity(w, V["psi"], V["ux"], uz, sim.get_laplacian_solver())
        lin_op = Pr * w.lap()
        D["w"][:] = -w.vec_dot_nabla(V["ux"].getp(), uz.getp()) + Pr * xi.sddx() - Pr * tmp.sddx()
        sim._integrator.integrate(w, D["w"], lin_op)
        lin_op = tmp.lap()
        D["tmp"][:] = -tmp.vec_dot_nabla(V["ux"].getp(), uz.getp()) - uz[:]
        sim._integrator.integrate(tmp, D["tmp"], lin_op)
        lin_op = tau * xi.lap()
        D["xi"][:] = -xi.vec_dot_nabla(V["ux"].getp(), uz.getp()) - uz[:] / R0
        sim._integrator.integrate(xi, D["xi"], lin_op)
        tmp[:, 0] = 0.0
        xi[:, 0] = 0.0
    return body


def bcs(p, w, scalars):
    e = p.spatial_derivative_order // 2
    w[1:, :e] = 0.0
    w[1:, -e:] = 0.0
    for t in scalars:
        t[0, :e] = 1.0
        t[0, -e:] = 0.0
        t[1:, :e] = 0.0
        t[1:, -e:] = 0.0
    w[0, :] = 0.0


def dirichlet_rhs(V, D, p, terms):
    """dq[:] = -q.vec_dot_nabla + linear terms (no diffusion)."""
    ux, uz = V["ux"].getp(), V["uz"].getp()
    for name, lin in terms.items():
        q = V[name]
        D[name][:] = -q.vec_dot_nabla(ux, uz) + sum(c * V[s].sddx() for s, c in lin)


def dirichlet_body(kappas, terms, pece=False):
    names = list(kappas)

    def explicit(sim, p, V, D):
        calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], sim.get_laplacian_solver())
        diff = {n: kappas[n] * V[n].snabla2() for n in names}
        dirichlet_rhs(V, D, p, terms)
        for n in names:
            sim._integrator.integrate(V[n], D[n], diff[n])
        bcs(p, V["w"], [V[n] for n in names[1:]])

    def pece_body(sim, p, V, D):
        integ = sim._integrator
        old = {n: V[n].gets().copy() for n in names}
        calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], sim.get_laplacian_solver())
        diff = {n: kappas[n] * V[n].snabla2() for n in names}
        dirichlet_rhs(V, D, p, terms)
        for n in names:
            D[n][:] += diff[n]
            V[n][:] = old[n] + integ.predictor(D[n])
        bcs(p, V["w"], [V[n] for n in names[1:]])
        for n in names:
            D[n].advance()
        ux_keep, uz_keep = V["ux"].getp().copy(), V["uz"].getp().copy()
        calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], sim.get_laplacian_solver())
        diff = {n: kappas[n] * V[n].snabla2() for n in names}
        dirichlet_rhs(V, D, p, terms)
        for n in names:
            D[n][:] += diff[n]
            V[n][:] = old[n] + integ.corrector(D[n])
        bcs(p, V["w"], [V[n] for n in names[1:]])
        # report the start-of-step velocity, as the other bodies do
        V["ux"].setp(ux_keep)
        V["uz"].setp(uz_keep)

    return pece_body if pece else explicit


# dt / CFL-limit ratios tried on every velocity set: no shrink, no shrink,
# four shrinks, seven shrinks, breach (cfl_cutoff = 0.5; every ratio is at
# least 1% away from a shrink-count boundary 0.5 / 0.9^k)
CFL_RATIOS = (0.01, 0.3, 0.7, 0.95, 1.2)


def set_dt_outcomes(sim, ux, uz, dts):
    """Integrator.set_dt (melvin/Integrator.py:35-44) from each dt in `dts`:
    the dt it leaves, or NaN where it raises "CFL condition breached"."""
    out = []
    for dt in dts:
        sim._integrator.override_dt(float(dt))
        try:
            with np.errstate(all="ignore"):
                sim._integrator.set_dt(ux, uz)
            out.append(sim._integrator.get_dt())
        except Exception as e:  # the reference raises a bare Exception
            assert str(e) == "CFL condition breached", e
            out.append(np.nan)
    return np.array(out, dtype=np.float64)


def cfl_limit(p, vx, vz):
    with np.errstate(all="ignore"):
        return min(p.dx / np.max(vx), p.dz / np.max(vz))


def cfl_cases(rng):
    """set_dt on seeded velocity sets: plain random; a signed maximum far
    below the absolute one; all-negative ux; ux = 0; a NaN in ux (caught:
    Python's min keeps a NaN first argument); a NaN in uz (missed: min drops
    a NaN second argument).  dts are CFL_RATIOS times the set's own limit
    (the random set's limit where that is not a positive number)."""
    for tag, p in (("cfl_fs32", params(32, 32, 2 * np.pi, 2 * np.pi)),
                   ("cfl_fd32x17", params(32, 17, 2.0, 1.0, fdm=True, integrator="explicit"))):
        with redirect_stdout(io.StringIO()):
            sim = Simulation(p, np)
        bf = [EXP, FDM] if p.discretisation[1] == "fdm" else [EXP, EXP]
        ux, uz = sim.make_variable("ux", bf), sim.make_variable("uz", bf)
        a = rng.standard_normal((p.nx, p.nz))
        b = rng.standard_normal((p.nx, p.nz))
        nan_a, nan_b = a.copy(), b.copy()
        nan_a[3, 5] = np.nan
        nan_b[7, 2] = np.nan
        sets = {
            "random": (a, b),
            "signed": (0.25 - 4.0 * np.abs(a), 0.05 * b),
            "negative": (-0.1 - np.abs(a), b),
            "zero_x": (np.zeros_like(a), b),
            "nan_ux": (nan_a, b),
            "nan_uz": (a, nan_b),
        }
        c0 = cfl_limit(p, a, b)
        names = []
        for name, (vx, vz) in sets.items():
            c = cfl_limit(p, vx, vz)
            dts = (c if c > 0 and np.isfinite(c) else c0) * np.array(CFL_RATIOS)
            ux.setp(vx.copy())
            uz.setp(vz.copy())
            G[f"{tag}/{name}/ux"] = vx
            G[f"{tag}/{name}/uz"] = vz
            G[f"{tag}/{name}/max"] = np.array([np.max(vx), np.max(vz)])
            G[f"{tag}/{name}/dts"] = dts
            G[f"{tag}/{name}/dt_out"] = set_dt_outcomes(sim, ux, uz, dts)
            names.append(name)
        G[f"{tag}/sets"] = np.array(names)


def cfl_e2e_cases():
    """set_dt on the velocity the reference derives from a vorticity field
    (calc_velocity_from_vorticity, melvin/utility.py:62-79), as the CFL
    ticker sees it after the first loop iteration.  Fully spectral: a
    narrow jet ux ~ -3 sech^2((z-pi)/0.3) (so max(ux) ~ 0.29 while
    max|ux| ~ 2.7) plus a Taylor-Green cell; Dirichlet z: a convection roll
    plus a jet-like vorticity."""
    two_pi = 2 * np.pi
    p = params(32, 32, two_pi, two_pi, dt=1e-3)
    x = np.linspace(0, p.lx, p.nx, endpoint=False)
    z = np.linspace(0, p.lz, p.nz, endpoint=False)
    X, Z = np.meshgrid(x, z, indexing="ij")
    d = 0.3
    # u = -3 sech^2((z-pi)/d): w = du/dz = 6 sech^2 tanh / d (lap psi = -w, ux = -d psi/dz)
    s2 = (1 / np.cosh((Z - np.pi) / d)) ** 2
    w_fs = 6.0 * s2 * np.tanh((Z - np.pi) / d) / d + 0.4 * np.sin(X) * np.sin(Z)
    pf = params(32, 17, 2.0, 1.0, fdm=True, integrator="explicit", dt=1e-5)
    x = np.linspace(0, pf.lx, pf.nx, endpoint=False)
    z = np.linspace(0, pf.lz, pf.nz, endpoint=False)
    X, Z = np.meshgrid(x, z, indexing="ij")
    w_fd = 50.0 * np.sin(np.pi * X) * np.sin(np.pi * Z) + 20.0 * np.sin(2 * np.pi * Z)
    for tag, p, w0 in (("cfl_e2e_fs32", p, w_fs), ("cfl_e2e_fd32x17", pf, w_fd)):
        with redirect_stdout(io.StringIO()):
            sim = Simulation(p, np)
        bf = [EXP, FDM] if p.discretisation[1] == "fdm" else [EXP, EXP]
        V = {n: sim.make_variable(n, bf) for n in ("w", "psi", "ux", "uz")}
        with redirect_stdout(io.StringIO()):
            sim.init_laplacian_solver(bf)
        V["w"].load(w0, is_physical=True)
        calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], sim.get_laplacian_solver())
        vx, vz = V["ux"].getp().copy(), V["uz"].getp().copy()
        dts = cfl_limit(p, vx, vz) * np.array(CFL_RATIOS)
        G[f"{tag}/init_w"] = w0
        G[f"{tag}/ux"] = vx
        G[f"{tag}/uz"] = vz
        G[f"{tag}/max"] = np.array([np.max(vx), np.max(vz)])
        G[f"{tag}/dts"] = dts
        G[f"{tag}/dt_out"] = set_dt_outcomes(sim, V["ux"], V["uz"], dts)


def load_resample_case(rng):
    """Variable.load of a spectral array from a finer fully spectral grid
    (melvin/Variable.py:67-85,142-151).  The reference resamples into a real
    array, so only a real-valued input keeps its values; it is used here
    where it works: a 64x64 spectrum (43 x 21) loaded on a 32x32 grid
    (21 x 10)."""
    with redirect_stdout(io.StringIO()):
        sim = Simulation(params(32, 32, 2 * np.pi, 2 * np.pi), np)
    v = sim.make_variable("v", [EXP, EXP])
    fine = rng.standard_normal(params(64, 64, 2 * np.pi, 2 * np.pi).spectral_shape)
    v.load(fine, is_physical=False)
    G["load_resample/in_spec"] = fine
    G["load_resample/out_spec"] = v.gets().copy()


def main():
    rng = np.random.default_rng(12345)
    two_pi = 2 * np.pi
    # ---- verbs ----
    verbs("fs32_o2", params(32, 32, two_pi, two_pi, order=2), rng)
    verbs("fs32x64_o4", params(32, 64, 1.0, 2.0, order=4, iorder=4), rng)
    verbs("fd32x17_o2", params(32, 17, 2.0, 1.0, fdm=True, order=2, integrator="explicit"), rng)
    verbs("fd64x21_o4", params(64, 21, 2.0, 1.0, fdm=True, order=4, iorder=4, integrator="explicit"), rng)

    # ---- trajectories ----
    def coords(p):
        x = np.linspace(0, p.lx, p.nx, endpoint=False)
        z = np.linspace(0, p.lz, p.nz, endpoint=False)
        return np.meshgrid(x, z, indexing="ij")

    p = params(32, 32, two_pi, two_pi, order=2, iorder=2, dt=1e-2)
    X, Z = coords(p)
    w0 = 2 * np.sin(X) * np.sin(Z) + 1e-3 * (2 * np.random.default_rng(0).random((32, 32)) - 1)
    trajectory("tg32_o2_ab2", p, ["w"], {"w": w0}, 8, tg_body(1e-2))

    p = params(32, 32, two_pi, two_pi, order=4, iorder=4, dt=1e-2)
    trajectory("tg32_o4_ab4", p, ["w"], {"w": w0}, 8, tg_body(1e-2))

    p = params(64, 32, two_pi, two_pi, order=2, iorder=2, dt=5e-3)
    X, Z = coords(p)
    d = 0.3
    u = np.tanh((Z - np.pi) / d) - np.tanh((Z - np.pi / 2) / d)
    wk = (1 / np.cosh((Z - np.pi) / d)) ** 2 / d - (1 / np.cosh((Z - np.pi / 2) / d)) ** 2 / d
    wk = wk + 1e-3 * np.sin(X)
    trajectory("kh64x32", p, ["w", "c"], {"w": wk, "c": -0.5 * u}, 8, kh_body(1e-3, 2e-3))

    p = params(32, 32, 4.0, 2.0, order=2, iorder=2, dt=1e-3)
    r = np.random.default_rng(7)
    init = {n: 1e-1 * (2 * r.random((32, 32)) - 1) for n in ["w", "tmp", "xi"]}
    trajectory("ddcs32", p, ["w", "tmp", "xi"], init, 6, ddc_spectral_body(7.0, 1.1, 1.0 / 3.0))

    p = params(32, 17, 2.0, 1.0, fdm=True, order=4, iorder=4, integrator="explicit", dt=1e-5)
    X, Z = coords(p)
    t0 = 1 - Z + 1e-3 * (2 * np.random.default_rng(0).random((32, 17)) - 1)
    rbc_terms = {"w": [("tmp", -1.0 * 1e5)], "tmp": []}
    trajectory("rbc32x17_o4_ab4", p, ["w", "tmp"], {"w": np.zeros((32, 17)), "tmp": t0}, 8,
               dirichlet_body({"w": 1.0, "tmp": 1.0}, rbc_terms))

    p = params(32, 17, 2.0, 1.0, fdm=True, order=2, iorder=2, integrator="explicit", dt=1e-5)
    trajectory("rbc32x17_o2_ab2", p, ["w", "tmp"], {"w": np.zeros((32, 17)), "tmp": t0}, 8,
               dirichlet_body({"w": 1.0, "tmp": 1.0}, rbc_terms))

    p = params(32, 17, 2.0, 1.0, fdm=True, order=4, iorder=4, integrator="explicit", dt=1e-5)
    trajectory("rbc32x17_pece4", p, ["w", "tmp"], {"w": np.zeros((32, 17)), "tmp": t0}, 8,
               dirichlet_body({"w": 1.0, "tmp": 1.0}, rbc_terms, pece=True))

    p = params(32, 17, 2.0, 1.0, fdm=True, order=2, iorder=2, integrator="explicit", dt=2e-6)
    Pr, RaT, Rr, Le = 7.0, 1e5, 2.0, 10.0
    s0 = 1 - Z + 1e-3 * (2 * np.random.default_rng(1).random((32, 17)) - 1)
    ddc_terms = {"w": [("T", -Pr * RaT), ("S", Pr * RaT / Rr)], "T": [], "S": []}
    trajectory("ddcd32x17", p, ["w", "T", "S"], {"w": np.zeros((32, 17)), "T": t0, "S": s0}, 8,
               dirichlet_body({"w": Pr, "T": 1.0, "S": 1.0 / Le}, ddc_terms))

    # ---- cosine / sine bases (n = 2^k + 1 on a mirrored axis) ----
    rb = np.random.default_rng(2024)
    COS, SIN = BasisFunctions.COSINE, BasisFunctions.SINE
    for (nx, nz, bf) in [(65, 64, [COS, EXP]), (65, 64, [SIN, EXP]), (64, 65, [EXP, COS]), (64, 65, [EXP, SIN]),
                         (65, 65, [COS, COS]), (65, 65, [SIN, SIN]), (65, 65, [SIN, COS]), (33, 65, [COS, SIN])]:
        tag = f"basis{nx}x{nz}_{int(bf[0])}{int(bf[1])}"
        basis_verbs(tag, params(nx, nz, 1.0, 2.0), bf, rb)

    # ---- transform lengths that are not powers of two (2(n-1) or n) ----
    rg = np.random.default_rng(2025)
    for (nx, nz, bf) in [(40, 48, [COS, EXP]), (48, 40, [EXP, SIN]), (33, 45, [SIN, COS]), (24, 36, [EXP, EXP]),
                         (130, 100, [COS, COS])]:
        tag = f"basis{nx}x{nz}_{int(bf[0])}{int(bf[1])}"
        basis_verbs(tag, params(nx, nz, 1.0, 2.0), bf, rg)

    # ---- Integrator.set_dt ----
    cfl_cases(np.random.default_rng(31))
    cfl_e2e_cases()

    # ---- host I/O ----
    load_resample_case(np.random.default_rng(41))

    np.savez_compressed(OUT, **G)
    print(f"wrote {OUT}: {len(G)} arrays, {os.path.getsize(OUT) / 1024:.1f} KiB")


if __name__ == "__main__":
    main()
