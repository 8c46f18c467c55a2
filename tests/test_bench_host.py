"""The benchmark's roofline arithmetic on the CPU: the algorithmic bytes per
launch of the three fused-step kernels (S = (2nn+1) nm spectral elements,
Pk = nx nm intermediate elements, 16-byte state, 16- or 8-byte
intermediates) and the fractions computed from event times."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_kernel_model_bytes_at_2048():
    n = 2048
    nn = nm = (n - 1) // 3
    S, Pk = (2 * nn + 1) * nm, n * nm
    fp64 = bench.kernel_model(n, split=False)
    assert fp64["xinv"]["bytes"] == 16 * S + 3 * 16 * Pk
    assert fp64["zstep"]["bytes"] == 5 * 16 * Pk
    assert fp64["xfwd"]["bytes"] == 2 * 16 * Pk + 4 * 16 * S
    assert sum(k["bytes"] for k in fp64.values()) == 297_952_160  # 5 ws S + 10 wi Pk
    split = bench.kernel_model(n, split=True)
    assert split["zstep"]["bytes"] == 5 * 8 * Pk
    assert sum(k["bytes"] for k in split.values()) == 5 * 16 * S + 10 * 8 * Pk


def test_roofline_picks_the_longest_kernel_and_step_fraction():
    model = bench.kernel_model(2048, split=False)
    names = ["xinv", "zstep", "xfwd"]
    kernel_ms = [[0.25, 0.26], [0.67, 0.67], [0.13, 0.14]]
    roof, k = bench.roofline(model, kernel_ms, names, 6685.1, "measured", {}, "fp64", 1.06)
    assert k == 1 and roof["kernel"] == "zstep"
    assert roof["achieved"] == pytest.approx(model["zstep"]["bytes"] / 0.67e-3 / 1e9, abs=0.1)
    assert roof["frac"] == pytest.approx(roof["achieved"] / 6685.1, abs=1e-4)
    assert roof["step_achieved"] == pytest.approx(297_952_160 / 1.06e-3 / 1e9, abs=0.1)
    assert roof["step_frac"] == pytest.approx(roof["step_achieved"] / 6685.1, abs=1e-4)
    assert roof["traffic"] is None


def test_aggregate_throughput_counts_every_rank():
    # N GPUs, each stepping its own n x n simulation K times in `secs`
    assert bench.aggregate_throughput(2048 * 2048, 20, 4, 0.5) == pytest.approx(4 * 2048 * 2048 * 20 / 0.5 / 1e6)
