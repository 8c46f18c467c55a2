"""The CPU oracle against the reference's own outputs (golden vectors made
by tests/golden/make_golden.py) and against the known-answer tests of the
reference test suite (test/SpectralTransformer_test.py,
test/Variable_test.py, test/LaplacianSolver_test.py), restated."""

import numpy as np
import pytest

import oracle as O
from oracle import problems as P
from cases import TRAJ_CASES, VERB_CASES, grid_of
from conftest import rel_l2

# The oracle calls the same NumPy/SciPy routines in the same order as the
# reference, so its outputs agree to rounding (bit-exact for most verbs).
TOL = 1e-13


def oracle_verbs(g, d, tag):
    s, ph, ux, uz = (d[f"{tag}/in_{k}"] for k in ("spec", "phys", "ux", "uz"))
    out = {
        "to_physical": O.to_physical(g, s),
        "to_spectral": O.to_spectral(g, ph),
        "pddx": O.pddx(g, ph),
        "pddz": O.pddz(g, ph),
        "sddx": O.sddx(g, s),
        "sd2dx2": O.sd2dx2(g, s),
        "snabla2": O.snabla2(g, s),
        "lap": O.laplacian_symbol(g),
    }
    if g.fdm_z:
        out["pd2dz2"] = O.pd2dz2(g, s)
    else:
        out["sddz"] = O.sddz(g, s)
        out["sd2dz2"] = O.sd2dz2(g, s)
    v, qp = O.vec_dot_nabla(g, s, ux, uz)
    out["vec_dot_nabla"], out["vec_dot_nabla_phys"] = v, qp
    solver = O.PoissonSolver(g)
    out["poisson"] = solver.solve(s)
    vel = O.velocity_from_vorticity(g, solver, s)
    out["vel_psi"], out["vel_ux_p"], out["vel_uz_p"] = vel["psi_s"], vel["ux_p"], vel["uz_p"]
    if g.fdm_z:
        out["vel_psi_p"] = vel["psi_p"]
    else:
        out["vel_ux_s"], out["vel_uz_s"] = vel["ux_s"], vel["uz_s"]
    out["ke"] = O.kinetic_energy(g, vel["ux_p"], vel["uz_p"])
    h = O.History(d[f"{tag}/hist"].shape[0], g.spectral_shape)
    h.data[:] = d[f"{tag}/hist"]
    h.curr = 1
    out["ab"] = O.adams_bashforth(h, 1e-3)
    out["am"] = O.adams_moulton(h, 1e-3)
    return out


@pytest.mark.parametrize("tag", list(VERB_CASES))
def test_oracle_verbs_match_reference(golden, tag):
    g = grid_of(tag)
    for name, val in oracle_verbs(g, golden, tag).items():
        assert rel_l2(val, golden[f"{tag}/{name}"]) < TOL, name


@pytest.mark.parametrize("tag", list(TRAJ_CASES))
def test_oracle_trajectories_match_reference(golden, tag):
    g, specs, names, integ, order, dt = TRAJ_CASES[tag]
    pr = P.Problem(g, specs, [golden[f"{tag}/s0_{n}"] for n in names], dt, integ, order)
    kes = []
    for s in range(int(golden[f"{tag}/nsteps"])):
        vel = pr.step()
        kes.append(O.kinetic_energy(g, vel["ux_p"], vel["uz_p"]))
        for i, n in enumerate(names):
            assert rel_l2(pr.q[i], golden[f"{tag}/s{s + 1}_{n}"]) < TOL, (s, n)
    assert rel_l2(np.array(kes), golden[f"{tag}/ke"]) < TOL


# ---- known answers of the reference test suite ------------------------------


def _kat_grid(fdm=False):
    # test/conftest.py:12-34: 256 x 256, lx = lz = 1
    return O.Grid(256, 256, 1.0, 1.0, fdm, 2)


def test_kat_transform_periodic():
    # test/SpectralTransformer_test.py:27-61
    g = _kat_grid()
    x = np.linspace(0, 1.0, g.nx, endpoint=False)
    X, Z = np.meshgrid(x, x, indexing="ij")
    phys = np.cos(2 * np.pi * X) + 2.0 * np.sin(2 * 2 * np.pi * Z)
    s = O.to_spectral(g, phys)
    want = np.zeros(g.spectral_shape, dtype=complex)
    want[1, 0] = 0.5
    want[-1, 0] = 0.5
    want[0, 2] = 2.0j / -2.0
    np.testing.assert_array_almost_equal(s, want)
    np.testing.assert_array_almost_equal(O.to_physical(g, s), phys)


def test_kat_transform_fdm_z():
    # test/SpectralTransformer_test.py:313-348
    g = _kat_grid(fdm=True)
    x = np.linspace(0, 1.0, g.nx, endpoint=False)
    z = np.linspace(0, 1.0, g.nz)
    X, _ = np.meshgrid(x, z, indexing="ij")
    phys = 3.0 + np.cos(2 * np.pi * X) + 2.0 * np.cos(2 * 2 * np.pi * X)
    s = O.to_spectral(g, phys)
    want = np.zeros(g.spectral_shape, dtype=complex)
    want[0, :] = 3.0
    want[1, :] = 0.5
    want[2, :] = 1.0
    np.testing.assert_array_almost_equal(s, want)
    np.testing.assert_array_almost_equal(O.to_physical(g, s), phys)


def test_kat_fd_derivatives():
    # test/Variable_test.py:16-46
    g = _kat_grid()
    x = np.linspace(0, 1.0, g.nx, endpoint=False)
    X, Z = np.meshgrid(x, x, indexing="ij")
    v = np.cos(2 * np.pi * X) * np.cos(2 * np.pi * Z)
    assert O.pddx(g, v)[:, 0] == pytest.approx(-2 * np.pi * np.sin(2 * np.pi * x), rel=1e-3)
    assert O.pddz(g, v)[0, :] == pytest.approx(-2 * np.pi * np.sin(2 * np.pi * x), rel=1e-3)


def test_kat_fdm_nabla2():
    # test/Variable_test.py:49-73
    g = _kat_grid(fdm=True)
    z = np.linspace(0, 1.0, g.nz, endpoint=False)
    s = np.zeros(g.spectral_shape, dtype=complex)
    s[1] = 0.5 * z ** 2
    got = O.snabla2(g, s)
    want = np.zeros_like(got)
    want[1] = -((2 * np.pi) ** 2) * s[1] + 1
    np.testing.assert_array_almost_equal(got[1, 1:-1], want[1, 1:-1])


def test_kat_spectral_nabla2():
    # test/Variable_test.py:76-100
    g = _kat_grid()
    got = O.snabla2(g, np.ones(g.spectral_shape, dtype=complex))
    n, m = O.mode_numbers(g)
    np.testing.assert_array_almost_equal(got, -((2 * np.pi * n) ** 2) - (2 * np.pi * m) ** 2)


def test_kat_fdm_laplacian_roundtrip():
    # test/LaplacianSolver_test.py:37-59 (with the x-mode term included)
    g = _kat_grid(fdm=True)
    solver = O.PoissonSolver(g)
    truth = np.ones(g.spectral_shape, dtype=complex)
    rhs = np.stack([solver.mats[n] @ truth[n] for n in range(g.nn)])
    np.testing.assert_array_almost_equal(solver.solve(rhs), truth)


def test_pece_is_pinned_to_reference_formulae(golden):
    # AB4 predictor / AM4 corrector composed from melvin/Integrator.py:8-33
    h = O.History(4, (3, 2))
    rng = np.random.default_rng(0)
    h.data[:] = rng.standard_normal(h.data.shape)
    h.curr = 2
    f0, f1, f2, f3 = h.get(), h.get(-1), h.get(-2), h.get(-3)
    np.testing.assert_allclose(O.adams_bashforth(h, 0.1), 0.1 / 24 * (55 * f0 - 59 * f1 + 37 * f2 - 9 * f3))
    np.testing.assert_allclose(O.adams_moulton(h, 0.1), 0.1 / 24 * (9 * f0 + 19 * f1 - 5 * f2 + f3))


def test_kh_initial_condition_sign():
    # w = d ux/dz - d uz/dx with lap psi = -w, ux = -dpsi/dz: a shear flow
    # u(z) needs w = du/dz.
    g = O.Grid(64, 256, 2 * np.pi, 2 * np.pi)
    w, c = P.kh_ic(g, 0.2, eps=0.0)
    vel = O.velocity_from_vorticity(g, O.PoissonSolver(g), O.to_spectral(g, w))
    _, Z = P.coords(g)
    u = np.tanh((Z - np.pi) / 0.2) - np.tanh((Z - np.pi / 2) / 0.2)
    assert rel_l2(vel["ux_p"], u - u.mean()) < 1e-2
    np.testing.assert_allclose(c, -0.5 * u)


# ---- cosine / sine bases -------------------------------------------------

from cases import BASIS_TAGS, basis_grid  # noqa: E402


@pytest.mark.parametrize("tag", BASIS_TAGS)
def test_oracle_basis_verbs_match_reference(golden, tag):
    from oracle import melvin_np as M

    g = basis_grid(tag)
    bx, bz = (int(v) for v in golden[f"{tag}/basis"])
    s, p = golden[f"{tag}/in_spec"], golden[f"{tag}/in_phys"]
    got = {
        "to_physical": M.to_physical_basis(g, s, bx, bz),
        "to_spectral": M.to_spectral_basis(g, p, bx, bz),
        "sddx": M.sddx_basis(g, s, bx),
        "sddz": M.sddz_basis(g, s, bz),
        "sd2dx2": M.sd2dx2_basis(g, s, bx),
        "sd2dz2": M.sd2dz2_basis(g, s, bz),
        "snabla2": M.sd2dx2_basis(g, s, bx) + M.sd2dz2_basis(g, s, bz),
        "lap": M.laplacian_symbol_basis(g, bx, bz),
        "poisson": M.poisson_basis(g, s, bx, bz),
    }
    for k, v in got.items():
        np.testing.assert_array_equal(v, golden[f"{tag}/{k}"], err_msg=k)


def _kat_mgrid(nx=65, nz=65):
    return O.Grid(nx, nz, 1.0, 1.0)


def test_kat_transform_cosine_x_periodic_z():
    """test/SpectralTransformer_test.py:64-97 restated at nx = 65 (2^6 + 1), nz = 64."""
    from oracle import melvin_np as M

    g = _kat_mgrid(65, 64)
    X, Z = np.meshgrid(np.linspace(0, 1.0, g.nx), np.linspace(0, 1.0, g.nz, endpoint=False), indexing="ij")
    phys = np.cos(np.pi * X) + 2.0 * np.cos(2 * np.pi * X)
    spec = M.to_spectral_basis(g, phys, M.COS, M.EXP)
    want = np.zeros(g.spectral_shape, complex)
    want[1, 0], want[2, 0], want[-1, 0], want[-2, 0] = 1.0, 2.0, 1.0, 2.0
    np.testing.assert_array_almost_equal(spec, want)
    np.testing.assert_array_almost_equal(M.to_physical_basis(g, spec, M.COS, M.EXP), phys)


def test_kat_transform_periodic_x_cosine_z():
    """test/SpectralTransformer_test.py:100-125 restated at nx = 64, nz = 65."""
    from oracle import melvin_np as M

    g = _kat_mgrid(64, 65)
    X, Z = np.meshgrid(np.linspace(0, 1.0, g.nx, endpoint=False), np.linspace(0, 1.0, g.nz), indexing="ij")
    phys = np.cos(np.pi * Z) + 2.0 * np.cos(2 * np.pi * Z)
    spec = M.to_spectral_basis(g, phys, M.EXP, M.COS)
    want = np.zeros(g.spectral_shape, complex)
    want[0, 1], want[0, 2] = 1.0, 2.0
    np.testing.assert_array_almost_equal(spec, want)
    np.testing.assert_array_almost_equal(M.to_physical_basis(g, spec, M.EXP, M.COS), phys)


def test_kat_transform_cosine_both():
    """test/SpectralTransformer_test.py:128-170 restated at 65 x 65."""
    from oracle import melvin_np as M

    g = _kat_mgrid()
    X, Z = np.meshgrid(np.linspace(0, 1.0, g.nx), np.linspace(0, 1.0, g.nz), indexing="ij")
    phys = (np.cos(np.pi * Z) + 2.0 * np.cos(2 * np.pi * Z) + np.cos(np.pi * X)
            + 2.0 * np.cos(2 * np.pi * X) * np.cos(1 * np.pi * Z))
    spec = M.to_spectral_basis(g, phys, M.COS, M.COS)
    want = np.zeros(g.spectral_shape, complex)
    want[0, 1], want[0, 2] = 1.0, 2.0
    want[1, 0], want[2, 1], want[-1, 0], want[-2, 1] = 1.0, 2.0, 1.0, 2.0
    np.testing.assert_array_almost_equal(spec, want)
    np.testing.assert_array_almost_equal(M.to_physical_basis(g, spec, M.COS, M.COS), phys)


def test_kat_transform_sine_both():
    """test/SpectralTransformer_test.py:173-205 restated at 65 x 65."""
    from oracle import melvin_np as M

    g = _kat_mgrid()
    X, Z = np.meshgrid(np.linspace(0, 1.0, g.nx), np.linspace(0, 1.0, g.nz), indexing="ij")
    phys = np.sin(np.pi * Z) * np.sin(np.pi * X) + 2.0 * np.sin(2 * np.pi * Z) * np.sin(3 * np.pi * X)
    spec = M.to_spectral_basis(g, phys, M.SIN, M.SIN)
    want = np.zeros(g.spectral_shape, complex)
    want[1, 1], want[-1, 1], want[3, 2], want[-3, 2] = 1.0, -1.0, 2.0, -2.0
    np.testing.assert_array_almost_equal(spec, want)
    np.testing.assert_array_almost_equal(M.to_physical_basis(g, spec, M.SIN, M.SIN), phys)


def _oracle_set_dt(g, ux, uz, dt):
    """The oracle's set_dt, NaN where it raises the CFL breach."""
    from cases import CFL_CUTOFF

    try:
        with np.errstate(all="ignore"):
            return O.cfl_dt(g, ux, uz, dt, CFL_CUTOFF)
    except RuntimeError:
        return np.nan


@pytest.mark.parametrize("tag", ["cfl_fs32", "cfl_fd32x17"])
def test_oracle_set_dt_matches_reference(golden, tag):
    """Integrator.set_dt (melvin/Integrator.py:35-44) on every velocity set:
    the dt left behind is bit-equal, breaches (signed maximum <= 0, a NaN in
    ux) agree, and a NaN in uz alone is missed as the reference misses it."""
    from cases import CFL_GRIDS

    g = CFL_GRIDS[tag]
    for s in golden[f"{tag}/sets"]:
        ux, uz = golden[f"{tag}/{s}/ux"], golden[f"{tag}/{s}/uz"]
        got = [_oracle_set_dt(g, ux, uz, dt) for dt in golden[f"{tag}/{s}/dts"]]
        np.testing.assert_array_equal(got, golden[f"{tag}/{s}/dt_out"], err_msg=str(s))
    assert np.isnan(golden[f"{tag}/nan_ux/dt_out"]).all()
    assert not np.isnan(golden[f"{tag}/nan_uz/dt_out"][:4]).any()
    assert np.isnan(golden[f"{tag}/negative/dt_out"]).all()


@pytest.mark.parametrize("tag", ["cfl_e2e_fs32", "cfl_e2e_fd32x17"])
def test_oracle_velocity_set_dt_matches_reference(golden, tag):
    """set_dt on the velocity derived from a vorticity field: the oracle's
    velocity equals the reference's and the dt outcomes are identical."""
    from cases import CFL_E2E_GRIDS

    g = CFL_E2E_GRIDS[tag]
    vel = O.velocity_from_vorticity(g, O.PoissonSolver(g), O.to_spectral(g, golden[f"{tag}/init_w"]))
    assert rel_l2(vel["ux_p"], golden[f"{tag}/ux"]) < TOL
    assert rel_l2(vel["uz_p"], golden[f"{tag}/uz"]) < TOL
    got = [_oracle_set_dt(g, vel["ux_p"], vel["uz_p"], dt) for dt in golden[f"{tag}/dts"]]
    np.testing.assert_array_equal(got, golden[f"{tag}/dt_out"])
