"""mgb_vec_dot_nabla_noalloc: the nonlinear term for callers that cannot
allocate device memory (its scratch lives in a fixed array inside the
library).  Its results must equal those of mgb_vec_dot_nabla, which uses a
caller workspace, on two calls in a row -- the second call reuses the
shared array the first one left behind.  Same FP64 tolerance as the other
parity tests (1e-12 relative L2; the two paths run the same kernels, so
they agree exactly in practice)."""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-12


def rel(a, b):
    return (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item()


@pytest.mark.parametrize("nx,nz,fdm,order", [(256, 256, False, 2), (512, 512, False, 4), (256, 129, True, 4)])
def test_noalloc_matches_workspace_entry_point(cuda, nx, nz, fdm, order):
    from melvin import _native as N

    lib = N.load_library()
    plan = N.Plan(nx, nz, 2.0, 1.0, fdm, order, N.PREC_DOUBLE, cuda)
    rows, cols = plan.spectral_shape
    stream = N.stream_handle(cuda)
    rng = np.random.default_rng(nx + nz)
    for call in range(2):
        q = torch.as_tensor(rng.standard_normal((rows, cols)) + 1j * rng.standard_normal((rows, cols)), device=cuda)
        ux = torch.as_tensor(rng.standard_normal((nx, nz)), device=cuda)
        uz = torch.as_tensor(rng.standard_normal((nx, nz)), device=cuda)
        out_ref = torch.empty((rows, cols), dtype=torch.complex128, device=cuda)
        out_new = torch.full((rows, cols), float("nan"), dtype=torch.complex128, device=cuda)
        qp_ref = torch.empty((nx, nz), dtype=torch.float64, device=cuda)
        qp_new = torch.full((nx, nz), float("nan"), dtype=torch.float64, device=cuda)
        N.check(lib.mgb_vec_dot_nabla(plan.handle, N.ptr(q), N.ptr(qp_ref), N.ptr(ux), N.ptr(uz), N.ptr(out_ref),
                                      N.ptr(plan.work()), stream))
        N.check(lib.mgb_vec_dot_nabla_noalloc(plan.handle, N.ptr(q), N.ptr(qp_new), N.ptr(ux), N.ptr(uz),
                                              N.ptr(out_new), stream))
        torch.cuda.synchronize()
        assert rel(out_new, out_ref) < TOL, call
        assert rel(qp_new, qp_ref) < TOL, call


@pytest.mark.parametrize("nx,nz,fdm", [(1024, 1024, False), (2048, 2048, False), (1024, 513, True)])
def test_noalloc_rejects_grids_beyond_its_scratch(cuda, nx, nz, fdm):
    """Just past the 4 MiB scratch: 1024^2 fully spectral needs two
    1024 x 341 complex128 intermediates (11 MB); 1024x513 with a Dirichlet z
    axis needs one 1024 x 513 double field (4.2 MB).  The call returns
    MGB_ERR_UNSUPPORTED with a message and launches nothing."""
    from melvin import _native as N

    lib = N.load_library()
    plan = N.Plan(nx, nz, 1.0, 1.0, fdm, 2, N.PREC_DOUBLE, cuda)
    rows, cols = plan.spectral_shape
    q = torch.zeros((rows, cols), dtype=torch.complex128, device=cuda)
    p = torch.zeros((nx, nz), dtype=torch.float64, device=cuda)
    st = lib.mgb_vec_dot_nabla_noalloc(plan.handle, N.ptr(q), N.ptr(p), N.ptr(p), N.ptr(p), N.ptr(q),
                                       N.stream_handle(cuda))
    assert st == N.MGB_ERR_UNSUPPORTED
    assert b"scratch" in lib.mgb_last_error()
