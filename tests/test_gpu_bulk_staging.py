"""Bulk staging (rp_set_bulk_staging): each cell's 3x3x3 neighbourhood copied into shared
memory by cp.async.bulk, one copy per neighbour cell and array, completing on an mbarrier.

The staged records and their shift into the home cell's frame are the per-lane path's, so
sweeps must leave bit-identical states, statistics and logs with either staging, and a logged
sweep with bulk staging must replay on the CPU oracle move by move (plain scans, overlap
counting, rototranslations, and the overflow rerun of neighbourhoods above the staging
capacity)."""
import numpy as np
import pytest

import pyoracle as po
import systems

pytestmark = pytest.mark.gpu

CASES = ["hs_small", "hs_dense", "sc_l2", "sc_l2_dense", "sc_l5", "poly_banana", "poly_dense", "hs_tiny", "sc_tiny",
         "psc_bent", "psc_tiny"]


def steps(cfg):
    return (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)


def run(cfg, bulk, sweeps=4, log=False, counting=False, flags=None):
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = cfg
    t, r = steps(cfg)
    out = []
    with GpuPacking(kind, prm, pos, rot, box) as g:
        g.set_bulk_staging(bulk)
        if counting:
            g.set_counting(True)
        for c in range(sweeps):
            st = g.sweep(t, r, seed=4242, counter=c, log=log, **(flags or {}))
            out.append((st["moves"], st["accepted"], st["rejected_overlap"], st["rejected_domain"]))
            if log:
                out.append(g.sweep_log())
        if counting:
            out.append(g.cached_overlaps())
        return g.state(), out


def same(a, b):
    (p1, r1, _), s1 = a
    (p2, r2, _), s2 = b
    assert np.array_equal(p1, p2) and np.array_equal(r1, r2)
    assert len(s1) == len(s2)
    for x, y in zip(s1, s2):
        if isinstance(x, tuple) and len(x) == 2 and isinstance(x[0], np.ndarray):
            assert x[0].tobytes() == y[0].tobytes() and np.array_equal(x[1], y[1])
        else:
            assert x == y


@pytest.mark.parametrize("name", CASES)
def test_bulk_staging_leaves_the_same_state(engine, name):
    cfg = systems.ALL[name]()
    same(run(cfg, False, log=True), run(cfg, True, log=True))


@pytest.mark.parametrize("name", CASES)
def test_bulk_staged_sweeps_replay_on_oracle(oracle, engine, name):
    from rampack_gb300.packing import GpuPacking
    cfg = systems.ALL[name]()
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    t, r = steps(cfg)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        g.set_bulk_staging(True)
        for cycle in range(3):
            st = g.sweep(t, r, seed=515, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            assert st["moves"] == len(moves)
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want), np.count_nonzero(codes != want)
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
    cpu.close()


@pytest.mark.parametrize("name", ["sc_l2_dense", "poly_dense", "hs_dense"])
def test_bulk_staging_in_overlap_counting(engine, name):
    cfg = list(systems.ALL[name]())
    cfg[2] = cfg[2] * 0.93          # compressed: overlaps to count
    cfg[4] = np.asarray(cfg[4]) * 0.93
    same(run(tuple(cfg), False, counting=True, log=True), run(tuple(cfg), True, counting=True, log=True))


@pytest.mark.parametrize("name", ["sc_l2", "poly_banana"])
def test_bulk_staging_with_rototranslations(engine, name):
    cfg = systems.ALL[name]()
    flags = {"rototranslation": True}
    same(run(cfg, False, log=True, flags=flags), run(cfg, True, log=True, flags=flags))


def test_bulk_staging_at_full_size(engine):
    """The bench's 10^6 spherocylinders: three sweeps with bulk staging end in the state of
    three with per-lane staging."""
    from rampack_gb300 import workloads as W
    cfg = W.config_sc_1e6()
    same(run(cfg, False, sweeps=3), run(cfg, True, sweeps=3))
