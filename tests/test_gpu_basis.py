"""Cosine and sine bases on the GPU against the reference (golden vectors
from running melvin/SpectralTransformer.py, SpatialDifferentiator.py and
LaplacianSolver.py with COSINE / SINE bases): transforms, spectral
derivative verbs, Laplacian and Poisson solve at 1e-12 relative L2, on
power-of-two transform lengths and on others (Bluestein: 78, 88, 24, 36,
258, 198 points); the reference's analytic transform tests at their own
256 x 256 grid (510-point mirrored transforms); errors for what stays
unsupported."""

import numpy as np
import pytest
import torch

from cases import BASIS_TAGS, basis_grid
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def make(g, bf, lx=1.0, lz=2.0):
    import melvin

    p = melvin.Parameters({"nx": g.nx, "nz": g.nz, "lx": lx, "lz": lz, "final_time": 1.0, "device": "cuda:0"})
    return p, melvin.Simulation(p, torch)


@pytest.mark.parametrize("tag", BASIS_TAGS)
def test_basis_verbs_match_reference(cuda, golden, tag):
    from melvin import BasisFunctions as B

    g = basis_grid(tag)
    bx, bz = (int(v) for v in golden[f"{tag}/basis"])
    bf = [B(bx), B(bz)]
    p, sim = make(g, bf)
    s = golden[f"{tag}/in_spec"]
    st = sim._spectral_trans
    src = torch.as_tensor(s, device=cuda)
    keep = src.clone()
    phys = st.to_physical(src, basis_functions=bf)
    assert rel_l2(phys.cpu().numpy(), golden[f"{tag}/to_physical"]) < TOL
    assert torch.equal(src, keep)  # the input is left as it was
    spec = st.to_spectral(torch.as_tensor(golden[f"{tag}/in_phys"], device=cuda), basis_functions=bf)
    assert rel_l2(spec.cpu().numpy(), golden[f"{tag}/to_spectral"]) < TOL
    q = sim.make_variable("q", bf)
    q.sets(s)
    for verb in ("sddx", "sddz", "sd2dx2", "sd2dz2", "snabla2", "lap"):
        got = getattr(q, verb)()
        assert rel_l2(got.cpu().numpy(), golden[f"{tag}/{verb}"]) < TOL, verb
    sim.init_laplacian_solver(bf)
    got = sim.get_laplacian_solver().solve(torch.as_tensor(s, device=cuda))
    assert rel_l2(got.cpu().numpy(), golden[f"{tag}/poisson"]) < TOL


def test_basis_round_trip_at_2049(cuda):
    """A 2049 x 2048 cosine-x grid (4096-point mirrored transform): physical ->
    spectral -> physical reproduces a field built from kept modes."""
    import oracle as O
    from melvin import BasisFunctions as B

    g = O.Grid(2049, 2048, 1.0, 2.0)
    bf = [B.COSINE, B.COMPLEX_EXP]
    p, sim = make(g, bf)
    st = sim._spectral_trans
    rng = np.random.default_rng(3)
    s = np.zeros(g.spectral_shape, complex)
    s[:40, :40] = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
    s[-39:, :40] = s[1:40, :40][::-1]            # cosine: mirrored rows carry the same coefficient
    s[:, 0] = s[:, 0].real                        # real zeroth z mode of a real field
    phys = st.to_physical(torch.as_tensor(s, device=cuda), basis_functions=bf)
    back = st.to_spectral(phys, basis_functions=bf)
    assert rel_l2(back.cpu().numpy(), s) < 1e-12


# The reference's analytic basis tests (test/SpectralTransformer_test.py:64-310)
# on their own fixture grid, 256 x 256 with lx = lz = 1 (test/conftest.py:
# 12-30): physical fields of a few exact modes, the exact spectra.  A cosine
# or sine axis of 256 points is a 510-point mirrored transform (Bluestein).
# Tolerance: 1e-12 absolute on the spectra (the reference's own check is
# 6 decimals) and on the physical round trip.
def _kat_fields(X, Z):
    return {
        "cos_x_periodic_z": (np.cos(np.pi * X) + 2.0 * np.cos(2 * np.pi * X),
                             {(1, 0): 1.0, (2, 0): 2.0, (-1, 0): 1.0, (-2, 0): 2.0}),
        "periodic_x_cos_z": (np.cos(np.pi * Z) + 2.0 * np.cos(2 * np.pi * Z), {(0, 1): 1.0, (0, 2): 2.0}),
        "cos_both": (np.cos(np.pi * Z) + 2.0 * np.cos(2 * np.pi * Z) + np.cos(np.pi * X)
                     + 2.0 * np.cos(2 * np.pi * X) * np.cos(1 * np.pi * Z),
                     {(0, 1): 1.0, (0, 2): 2.0, (1, 0): 1.0, (2, 1): 2.0, (-1, 0): 1.0, (-2, 1): 2.0}),
        "sin_both": (np.sin(np.pi * Z) * np.sin(np.pi * X) + 2.0 * np.sin(2 * np.pi * Z) * np.sin(3 * np.pi * X),
                     {(1, 1): 1.0, (-1, 1): -1.0, (3, 2): 2.0, (-3, 2): -2.0}),
        "sin_x_periodic_z": (np.sin(np.pi * X) + 2.0 * np.sin(2 * np.pi * X),
                             {(1, 0): 1.0, (-1, 0): -1.0, (2, 0): 2.0, (-2, 0): -2.0}),
        "sin_x_cos_z": (np.sin(np.pi * X) + 2.0 * np.sin(2 * np.pi * X),
                        {(1, 0): 1.0, (-1, 0): -1.0, (2, 0): 2.0, (-2, 0): -2.0}),
        "cos_x_sin_z": (np.cos(np.pi * X) * np.sin(np.pi * Z) + 2.0 * np.cos(3 * np.pi * X) * np.sin(2 * np.pi * Z)
                        + 3.0 * np.sin(2 * np.pi * Z),
                        {(1, 1): 1.0, (-1, 1): 1.0, (0, 2): 3.0, (3, 2): 2.0, (-3, 2): 2.0}),
    }


KAT_BASES = {"cos_x_periodic_z": (1, 0), "periodic_x_cos_z": (0, 1), "cos_both": (1, 1), "sin_both": (2, 2),
             "sin_x_periodic_z": (2, 0), "sin_x_cos_z": (2, 1), "cos_x_sin_z": (1, 2)}


@pytest.mark.parametrize("kat", list(KAT_BASES))
def test_reference_basis_kats_at_256(cuda, kat):
    import oracle as O
    from melvin import BasisFunctions as B

    bx, bz = KAT_BASES[kat]
    g = O.Grid(256, 256, 1.0, 1.0)
    bf = [B(bx), B(bz)]
    p, sim = make(g, bf, 1.0, 1.0)
    x = np.linspace(0, 1.0, 256, endpoint=bx != 0)
    z = np.linspace(0, 1.0, 256, endpoint=bz != 0)
    X, Z = np.meshgrid(x, z, indexing="ij")
    phys, modes = _kat_fields(X, Z)[kat]
    want = np.zeros(p.spectral_shape, complex)
    for (r, m), v in modes.items():
        want[r, m] = v
    st = sim._spectral_trans
    spec = st.to_spectral(torch.as_tensor(phys, device=cuda), basis_functions=bf).cpu().numpy()
    np.testing.assert_allclose(spec, want, rtol=0, atol=1e-12)
    back = st.to_physical(torch.as_tensor(spec, device=cuda), basis_functions=bf).cpu().numpy()
    np.testing.assert_allclose(back, phys, rtol=0, atol=1e-12)


def test_unsupported_sizes_raise(cuda):
    import melvin
    import oracle as O
    from melvin import BasisFunctions as B

    # a cosine axis of 2050 points is a 4098-point transform, above the 4096 limit
    g = O.Grid(2050, 64, 1.0, 1.0)
    p, sim = make(g, [B.COSINE, B.COMPLEX_EXP])
    with pytest.raises(NotImplementedError):
        sim._spectral_trans.to_physical(torch.zeros(p.spectral_shape, dtype=torch.complex128, device=cuda),
                                        basis_functions=[B.COSINE, B.COMPLEX_EXP])
    # a plan with an axis that is not a power of two has the transforms, not the fused kernels
    g = O.Grid(24, 36, 1.0, 1.0)
    p, sim = make(g, [B.COMPLEX_EXP, B.COMPLEX_EXP])
    q = sim.make_variable("q", [B.COMPLEX_EXP, B.COMPLEX_EXP])
    q.sets(np.ones(p.spectral_shape, complex))
    with pytest.raises(NotImplementedError):
        q.vec_dot_nabla(np.zeros((24, 36)), np.zeros((24, 36)))
    # an axis above 4096 points has no plan
    with pytest.raises(NotImplementedError):
        melvin._native.plan_for(melvin.Parameters({"nx": 4100, "nz": 64, "lx": 1.0, "lz": 1.0, "final_time": 1.0,
                                                   "device": "cuda:0"}))
