"""Cosine and sine bases on the GPU against the reference (golden vectors
from running melvin/SpectralTransformer.py, SpatialDifferentiator.py and
LaplacianSolver.py with COSINE / SINE bases): transforms, spectral
derivative verbs, Laplacian and Poisson solve at 1e-12 relative L2; the
reference's analytic transform tests; errors for unsupported sizes."""

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


def test_unsupported_basis_lengths_raise(cuda):
    import oracle as O
    from melvin import BasisFunctions as B

    g = O.Grid(256, 256, 1.0, 1.0)  # the reference's own test size: a 510-point mirrored transform
    p, sim = make(g, [B.COSINE, B.COMPLEX_EXP])
    with pytest.raises(NotImplementedError):
        sim._spectral_trans.to_physical(torch.zeros(p.spectral_shape, dtype=torch.complex128, device=cuda),
                                        basis_functions=[B.COSINE, B.COMPLEX_EXP])
    g = O.Grid(65, 64, 1.0, 1.0)  # a mirrored-only axis: complex-exponential transforms are refused
    p, sim = make(g, [B.COMPLEX_EXP, B.COMPLEX_EXP])
    with pytest.raises(NotImplementedError):
        sim._spectral_trans.to_physical(torch.zeros(p.spectral_shape, dtype=torch.complex128, device=cuda))
