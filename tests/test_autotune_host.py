"""Host logic of the tile autotuner (no GPU): the coordinate-descent search
and the variant listing, on synthetic timings and a stand-in plan."""

import itertools

import pytest

pytest.importorskip("torch")

from melvin import autotune  # noqa: E402


def table_measure(costs, log):
    def measure(tiles):
        log.append(tiles)
        return costs[tiles]
    return measure


def test_search_finds_separable_optimum():
    # additive per-family costs: coordinate descent reaches the global optimum in one sweep
    per = [{0: 3.0, 1: 2.0, 2: 4.0}, {0: 5.0, 1: 1.0}, {0: 2.0, 3: 1.5}]
    costs = {t: sum(per[f][v] for f, v in enumerate(t)) for t in itertools.product(*[list(p) for p in per])}
    log = []
    best, ms, ms0, trials = autotune.search(table_measure(costs, log), [list(p) for p in per], (0, 0, 0))
    assert best == (1, 1, 3)
    assert ms == pytest.approx(4.5) and ms0 == pytest.approx(10.0)
    assert trials[0] == ((0, 0, 0), 10.0)
    assert len(log) <= 1 + 2 * (2 + 1 + 1)  # at most two sweeps


def test_search_keeps_default_within_min_gain():
    costs = {(0, 0, 0): 1.0, (1, 0, 0): 0.99, (0, 1, 0): 1.2, (0, 0, 1): 1.01}
    best, ms, ms0, _ = autotune.search(table_measure(costs, []), [[0, 1], [0, 1], [0, 1]], (0, 0, 0),
                                       min_gain=0.02)
    assert best == (0, 0, 0) and ms == ms0 == 1.0


def test_search_starts_from_current_selection():
    costs = {t: 1.0 + 0.1 * sum(t) for t in itertools.product([0, 1], [0, 1], [0, 1])}
    best, _, ms0, trials = autotune.search(table_measure(costs, []), [[0, 1]] * 3, (1, 1, 1))
    assert trials[0][0] == (1, 1, 1) and ms0 == pytest.approx(1.3)
    assert best == (0, 0, 0)


class FakePlan:
    """tile_info of a plan whose variants 0 and 2 coincide, 3 does not fit,
    and 4 has variant 0's shape and radix but the register-resident kind
    (in the z family only)."""

    def tile_info(self, family, nfields, v):
        shape = {0: 4, 1: 2, 2: 4, 3: 8, 4: 4}[v]
        kind = 1 if v == 4 else 0
        return (v != 3 and (v != 4 or family == 1), shape, 8, 1024 * shape, kind)


def test_variants_deduplicate_and_skip_unavailable():
    ch = autotune.variants(FakePlan(), 1)
    assert ch == [[0, 1], [0, 1, 4], [0, 1]]
    d = autotune.describe(FakePlan(), 2)
    assert set(d) == {"xinv", "zstep", "xfwd"}
    assert d["zstep"][3] == (3, False, 8, 8, 8192, 0)
    assert d["zstep"][4] == (4, True, 4, 8, 4096, 1)


def test_tune_rejects_other_objects():
    with pytest.raises(TypeError):
        autotune.tune(object())
