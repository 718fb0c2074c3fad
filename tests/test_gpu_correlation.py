"""Pair correlations on the GPU (rp_correlation_*, rampack_gb300.correlation) against the
reference's own observables (tests/golden/correlation.npz) and the oracle restatement
(tests/test_correlation_oracle.py pins it to the reference):

* bin counts and PairDensityCorrelation values bit for bit; PairAveragedCorrelation values
  (FP64 sums in another order than the reference's serial loop) to 1e-12 relative;
* the cell-grid enumeration against every pair examined (RP_CORR_ALL_PAIRS) and the FP32
  pre-filter against FP64 alone (RP_CORR_FP64_ONLY) at the benchmarked sizes;
* the 64,000-spherocylinder workload against the oracle's counts at full size."""
import numpy as np
import pytest

import pyoracle as po
import systems
from correlation_cases import CORRELATIONS, POLY_AXES
from test_correlation_oracle import GOLD, case_desc

pytestmark = pytest.mark.gpu

AVG_RTOL = 1e-12


def observable(case, flags=0):
    from rampack_gb300 import correlation as K
    name, en, lax, mil, fn, ax, focal, max_r, nb = case
    kind = systems.ALL[name]()[0]
    enum = [K.RadialEnumerator(focal), K.LinearEnumerator("xyz"[lax], focal),
            K.LayerwiseRadialEnumerator(mil, focal)][en]
    if fn == 0:
        return K.PairDensityCorrelation(enum, max_r, nb, print_count=True, flags=flags)
    axis = ("primary", "secondary", "auxiliary")[ax]
    prim, sec = POLY_AXES if kind == po.POLYSPHERE else (None, None)
    f = [None, K.S110Correlation, K.S220Correlation, K.S221Correlation, K.AxesAngle][fn](axis, prim, sec)
    return K.PairAveragedCorrelation(enum, f, max_r, nb, print_count=True, flags=flags)


def assert_same(fn, got, want):
    x, y, c = got
    wx, wy, wc = want
    assert np.array_equal(x, wx)
    assert np.array_equal(c, wc), f"{np.count_nonzero(c != wc)} bins differ"
    if fn == 0:
        assert np.array_equal(y, wy, equal_nan=True)
    else:
        assert np.allclose(y, wy, rtol=AVG_RTOL, atol=1e-12, equal_nan=True)


def two_snapshots(obs, cfg):
    from rampack_gb300.packing import GpuPacking
    with GpuPacking(*cfg) as g:
        obs.add_snapshot(g)
        g.upload(*systems.compressed(cfg, 0.97)[2:5])
        obs.add_snapshot(g)
    return obs.values()


@pytest.mark.parametrize("i", range(len(CORRELATIONS)))
def test_correlation_matches_the_reference(engine, i):
    z = np.load(GOLD)
    case = CORRELATIONS[i]
    cfg = systems.ALL[case[0]]()
    with observable(case) as obs:
        got = two_snapshots(obs, cfg)
        assert obs.info()["snapshots"] == 2
    assert_same(case[4], got, (z[f"c{i}_x"], z[f"c{i}_y"], z[f"c{i}_count"]))


@pytest.mark.parametrize("i", range(len(CORRELATIONS)))
def test_grid_and_filter_change_nothing(engine, i):
    # the same observable with every pair examined, and with every pair decided in FP64
    from rampack_gb300 import _lib
    case = CORRELATIONS[i]
    cfg = systems.ALL[case[0]]()
    base = two_snapshots(observable(case), cfg)
    for flags in (_lib.CORR_ALL_PAIRS, _lib.CORR_FP64_ONLY, _lib.CORR_ALL_PAIRS | _lib.CORR_FP64_ONLY):
        assert_same(case[4], two_snapshots(observable(case, flags), cfg), base)


@pytest.mark.parametrize("name", ["hs_small", "sc_l2", "poly_banana", "sc_l2_dense"])
@pytest.mark.parametrize("en", [0, 1, 2])
def test_counts_match_the_oracle(oracle, engine, name, en):
    # more enumerators and reaches than the fixtures: one snapshot's raw counts against the
    # oracle's (the compressed state overlaps, which the observables do not care about)
    from rampack_gb300.packing import GpuPacking
    cfg = systems.compressed(systems.ALL[name](), 0.95)
    for max_r, nb in ((2.5, 7), (6.0, 120)):
        case = (name, en, 2, (1, 0, 1), 0, 0, "o", max_r, nb)
        _, d = case_desc(case)
        with observable(case) as obs, GpuPacking(*cfg) as g:
            obs.add_snapshot(g)
            counts, _ = obs.last_snapshot()
        assert np.array_equal(counts, po.pair_counts(d, *cfg[2:5])), (max_r, nb)


def test_observable_lifecycle(engine):
    from rampack_gb300 import correlation as K
    from rampack_gb300.packing import GpuPacking
    cfg = systems.sc_l2()
    obs = K.PairDensityCorrelation(K.RadialEnumerator(), 4.0, 8, print_count=True)
    with GpuPacking(*cfg) as g:
        obs.add_snapshot(g)
        first = obs.values()
        obs.add_snapshot(g)
        x, y, c = obs.values()
        assert np.array_equal(y, first[1]) and np.array_equal(c, 2 * first[2])
        obs.clear()
        assert obs.info()["snapshots"] == 0 and not obs.values()[1].any()
        obs.add_snapshot(g)
        assert np.array_equal(obs.values()[1], first[1])
        lines = obs.print().splitlines()
        assert len(lines) == 8 and lines[0].split()[0] == "0.25"
    with GpuPacking(*systems.hs_small()) as g:
        with pytest.raises(Exception):
            obs.add_snapshot(g)   # another shape
    obs.close()


@pytest.mark.parametrize("workload,max_r,nb", [("sc_64000", 5.0, 100), ("banana_1e5", 4.0, 80)])
def test_full_size_counts_match_the_oracle(oracle, engine, workload, max_r, nb):
    from rampack_gb300 import workloads as W
    from rampack_gb300.packing import GpuPacking
    cfg = {"sc_64000": W.config_sc_64000, "banana_1e5": W.config_banana_1e5}[workload]()
    if workload == "banana_1e5":   # the oracle's all-pairs loop at 10^5 takes minutes: a 30,000 slice
        kind, prm, pos, rot, box = cfg
        cfg = (kind, prm, pos[:30000], rot[:30000], box)
    case = ("sc_l2", 0, 0, (0, 0, 1), 0, 0, "o", max_r, nb)
    _, d = case_desc(case)
    with observable(case) as obs, GpuPacking(*cfg) as g:
        obs.add_snapshot(g)
        counts, _ = obs.last_snapshot()
    want = po.pair_counts(d, *cfg[2:5])
    assert np.array_equal(counts, want)


@pytest.mark.parametrize("focal,fn,en", [("o", 0, 0), ("beg", 1, 0), ("o", 0, 2), ("end", 2, 2)])
def test_full_size_grid_and_binning_equal_exhaustive(engine, focal, fn, en):
    # 10^6 spherocylinders after a few sweeps: the cell grid finds every pair within reach
    # exactly once (the all-pairs enumeration examines 5 x 10^11 pairs on the GPU), and the
    # FP32 binning with its FP64 guard band bins every pair as FP64 alone; g(r) tends to 1
    from rampack_gb300 import _lib
    from rampack_gb300 import workloads as W
    from rampack_gb300.packing import GpuPacking
    cfg = W.config_sc_1e6()
    case = ("sc_l2", en, 0, (0, 0, 10), fn, 0, focal, 8.0, 200)
    with GpuPacking(*cfg) as g:
        for c in range(3):
            g.sweep(0.2, 0.2, seed=11, counter=c, stats=False)
        res = []
        for flags in (0, _lib.CORR_ALL_PAIRS, _lib.CORR_FP64_ONLY):
            with observable(case, flags) as obs:
                obs.add_snapshot(g)
                res.append(obs.values())
                if flags == 0:
                    fp64 = obs.info()["pairs_tested"]
    for r in res[1:]:
        assert np.array_equal(res[0][2], r[2])
        if fn == 0:
            assert np.array_equal(res[0][1], r[1])
        else:
            assert np.allclose(res[0][1], r[1], rtol=AVG_RTOL, atol=1e-12, equal_nan=True)
    assert res[0][2].sum() > 0 and fp64 < res[0][2].sum() / 10
    if fn == 0 and en == 0:
        assert abs(res[0][1][-20:].mean() - 1.0) < 0.1
