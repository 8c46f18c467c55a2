"""mgb_fp64_fma_probe, the kernel behind the FP64-ALU roofline that the
benchmark reports: it reports the flops of the launch it made (an FMA
counts two), writes nothing to its sink, and rejects bad sizes."""

import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


def test_fp64_fma_probe(cuda):
    from melvin import _native as N

    lib = N.load_library()
    sink = torch.zeros(8, dtype=torch.float64, device=cuda)
    flops = C.c_double()
    N.check(lib.mgb_fp64_fma_probe(N.ptr(sink), 8, 1024, C.byref(flops), N.stream_handle(cuda)))
    torch.cuda.synchronize()
    assert flops.value == 2 * 8 * 1024 * 256 * 8  # 2 flops x 8 chains x iters x threads x blocks
    assert torch.count_nonzero(sink).item() == 0
    assert lib.mgb_fp64_fma_probe(N.ptr(sink), 0, 1024, C.byref(flops), N.stream_handle(cuda)) == N.MGB_ERR_INVALID
