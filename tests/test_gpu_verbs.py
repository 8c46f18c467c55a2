"""Parity of every per-verb GPU kernel with the reference outputs (golden
vectors) and with the oracle at larger sizes.  FP64 throughout: the
tolerance is 1e-12 relative L2 (differences come only from the FFT
algorithm and the order of floating-point operations)."""

import numpy as np
import pytest
import torch

import oracle as O
from cases import VERB_CASES, grid_of, params_dict
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def make_sim(g, integrator, order, precision="double"):
    import melvin

    p = melvin.Parameters(params_dict(g, integrator, order, precision=precision))
    return melvin.Simulation(p, torch), p


def basis(g):
    from melvin import BasisFunctions as B

    return [B.COMPLEX_EXP, B.FDM if g.fdm_z else B.COMPLEX_EXP]


def host(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


@pytest.mark.parametrize("tag", list(VERB_CASES))
def test_verbs_match_reference(cuda, golden, tag):
    from melvin.utility import calc_kinetic_energy, calc_velocity_from_vorticity

    nx, nz, lx, lz, fdm, order, iorder, integ = VERB_CASES[tag]
    g = grid_of(tag)
    sim, p = make_sim(g, integ, iorder)
    bf = basis(g)
    st, sd = sim._spectral_trans, sim._spatial_diff
    s, ph, ux, uz = (golden[f"{tag}/in_{k}"] for k in ("spec", "phys", "ux", "uz"))
    got = {
        "to_physical": st.to_physical(s, basis_functions=bf),
        "to_spectral": st.to_spectral(ph, basis_functions=bf),
        "pddx": sd.pddx(ph),
        "pddz": sd.pddz(ph),
    }
    q = sim.make_variable("q", bf)
    q.sets(s)
    got["sddx"] = q.sddx()
    got["sd2dx2"] = q.sd2dx2()
    got["snabla2"] = q.snabla2()
    got["lap"] = q.lap()
    if fdm:
        got["pd2dz2"] = sd.pd2dz2(s)
    else:
        got["sddz"] = q.sddz()
        got["sd2dz2"] = q.sd2dz2()
    got["vec_dot_nabla"] = q.vec_dot_nabla(torch.as_tensor(ux, device=cuda), torch.as_tensor(uz, device=cuda))
    got["vec_dot_nabla_phys"] = q.getp()
    sim.init_laplacian_solver(bf)
    solver = sim.get_laplacian_solver()
    got["poisson"] = solver.solve(s)
    w, psi, vx, vz = (sim.make_variable(n, bf) for n in ("w", "psi", "ux", "uz"))
    w.sets(s)
    calc_velocity_from_vorticity(w, psi, vx, vz, solver)
    got["vel_psi"], got["vel_ux_p"], got["vel_uz_p"] = psi.gets(), vx.getp(), vz.getp()
    if fdm:
        got["vel_psi_p"] = psi.getp()
    else:
        got["vel_ux_s"], got["vel_uz_s"] = vx.gets(), vz.gets()
    got["ke"] = calc_kinetic_energy(vx, vz, torch, p)
    dv = sim.make_derivative("dq")
    dv._data.copy_(torch.as_tensor(golden[f"{tag}/hist"], device=cuda))
    dv.set_curr_idx(1)
    got["ab"] = sim._integrator.predictor(dv)
    got["am"] = sim._integrator.corrector(dv)
    torch.cuda.synchronize()
    bad = {k: rel_l2(host(v), golden[f"{tag}/{k}"]) for k, v in got.items()}
    assert all(e < TOL for e in bad.values()), {k: f"{e:.2e}" for k, e in bad.items() if e >= TOL}


@pytest.mark.parametrize(
    "nx,nz,fdm,order",
    [(256, 256, False, 2), (128, 512, False, 4), (2048, 64, False, 2), (128, 65, True, 4), (1024, 33, True, 2),
     (16, 16, False, 2), (4096, 16, False, 4)],
)
def test_transforms_and_jacobian_vs_oracle(cuda, nx, nz, fdm, order):
    """Random inputs at sizes beyond the golden set, including the smallest
    and largest transform lengths built."""
    g = O.Grid(nx, nz, 2.0, 1.5, fdm, order)
    sim, p = make_sim(g, "explicit" if fdm else "semi-implicit", 2)
    bf = basis(g)
    rng = np.random.default_rng(nx + nz)
    s = rng.standard_normal(g.spectral_shape) + 1j * rng.standard_normal(g.spectral_shape)
    ph, ux, uz = (rng.standard_normal((nx, nz)) for _ in range(3))
    st = sim._spectral_trans
    assert rel_l2(host(st.to_physical(s, basis_functions=bf)), O.to_physical(g, s)) < TOL
    assert rel_l2(host(st.to_spectral(ph, basis_functions=bf)), O.to_spectral(g, ph)) < TOL
    q = sim.make_variable("q", bf)
    q.sets(s)
    v = q.vec_dot_nabla(torch.as_tensor(ux, device=cuda), torch.as_tensor(uz, device=cuda))
    want, want_p = O.vec_dot_nabla(g, s, ux, uz)
    assert rel_l2(host(v), want) < TOL
    assert rel_l2(host(q.getp()), want_p) < TOL


def test_round_trip_property_2048(cuda):
    """to_spectral(to_physical(s)) == s for a dealiased spectrum, at 2048^2
    (size-independent property)."""
    g = O.Grid(2048, 2048, 2 * np.pi, 2 * np.pi)
    sim, p = make_sim(g, "semi-implicit", 2)
    rng = np.random.default_rng(1)
    s = torch.as_tensor(O.to_spectral(g, rng.standard_normal((2048, 2048))), device=cuda)
    st = sim._spectral_trans
    back = st.to_spectral(st.to_physical(s))
    assert rel_l2(host(back), host(s)) < TOL


def test_sizes_that_are_not_powers_of_two(cuda):
    """A fully spectral 96 x 64 grid transforms like the oracle (the 96-point
    axis as a Bluestein convolution) at 1e-12; the fused kernels refuse it
    loudly, and so do an FDM-z grid with nx = 96 and an axis above 4096."""
    import melvin
    from melvin import BasisFunctions as B
    from melvin._native import MelvinUnsupported

    g = O.Grid(96, 64, 1.0, 1.0)
    p = melvin.Parameters({"nx": 96, "nz": 64, "lx": 1.0, "lz": 1.0, "final_time": 1.0})
    sim = melvin.Simulation(p, torch)
    rng = np.random.default_rng(96)
    phys = rng.standard_normal((96, 64))
    spec = sim._spectral_trans.to_spectral(torch.as_tensor(phys, device=cuda)).cpu().numpy()
    assert rel_l2(spec, O.to_spectral(g, phys)) < TOL
    back = sim._spectral_trans.to_physical(torch.as_tensor(spec, device=cuda)).cpu().numpy()
    assert rel_l2(back, O.to_physical(g, spec)) < TOL
    q = sim.make_variable("q", [B.COMPLEX_EXP, B.COMPLEX_EXP])
    q.sets(spec)
    with pytest.raises(MelvinUnsupported):
        q.vec_dot_nabla(phys, phys)
    for d in ({"nx": 96, "nz": 33, "discretisation": ["spectral", "fdm"]}, {"nx": 4100, "nz": 64}):
        d.update(lx=1.0, lz=1.0, final_time=1.0)
        with pytest.raises(MelvinUnsupported):
            melvin.Simulation(melvin.Parameters(d), torch)


@pytest.mark.parametrize("nx,nz", [(64, 18), (64, 19), (64, 35), (64, 66), (64, 130), (64, 258), (32, 513),
                                   (32, 530), (16, 1100), (2048, 1800)])
def test_dirichlet_poisson_vs_oracle(cuda, nx, nz):
    """LaplacianSolver.solve on Fourier-x / Dirichlet-z grids against the
    oracle's sparse LU solve (melvin/LaplacianSolver.py:21-56, 70-79): every
    number of lanes per mode of the segmented sweep (1 to 32), last rounds
    of every fill, and the largest grid.

    The x-mode 0 matrix has condition number kappa ~ 4 lz^2 / (pi^2 dz^2)
    (1.3e6 at nz = 1800), so two exact-arithmetic-equivalent eliminations of a
    white-noise right-hand side differ by ~kappa * eps in the forward error
    (the oracle's LU and a sequential Thomas sweep do).  The bars are the
    backward error, normwise per mode, below 1e-14 (both solvers give ~2e-16),
    and the forward error within 20 kappa eps of the oracle."""
    g = O.Grid(nx, nz, 2.0, 1.0, True, 2)
    sim, p = make_sim(g, "explicit", 2)
    bf = basis(g)
    rng = np.random.default_rng(nz)
    s = rng.standard_normal(g.spectral_shape) + 1j * rng.standard_normal(g.spectral_shape)
    sim.init_laplacian_solver(bf)
    got = host(sim.get_laplacian_solver().solve(torch.as_tensor(s, device=cuda)))
    lu = O.PoissonSolver(g)
    want = lu.solve(s)
    kappa = 4 * (g.lz / g.dz) ** 2 / np.pi ** 2
    assert rel_l2(got, want) < 20 * kappa * np.finfo(float).eps
    for n in range(g.nn):
        a = lu.mats[n]
        back = np.abs(a @ got[n] - s[n]).max() / (abs(a).sum(axis=1).max() * np.abs(got[n]).max() + np.abs(s[n]).max())
        assert back < 1e-14, (n, back)
    # the identity end rows pass the right-hand side through unchanged
    assert np.array_equal(got[:, 0], s[:, 0]) and np.array_equal(got[:, -1], s[:, -1])
