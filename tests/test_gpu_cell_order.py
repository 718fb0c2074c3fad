"""The order in which a sweep's warps take a checkerboard phase's cells (rp_set_cell_order):
by occupancy, largest first (the default), or in cell-index order.  Cells of one phase are
never neighbours, so both orders must leave bit-identical states, statistics and logs (the
parity tests replay the default order on the oracle)."""
import numpy as np
import pytest

import systems

pytestmark = pytest.mark.gpu

CASES = ["hs_small", "hs_dense", "sc_l2", "sc_l2_dense", "sc_l5", "poly_banana", "psc_bent", "hs_tiny", "sc_tiny"]


def run(cfg, order, sweeps=4, counting=False):
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = cfg
    t, r = (0.1, 0.0) if kind == 0 else (0.2, 0.2)
    out = []
    with GpuPacking(kind, prm, pos, rot, box) as g:
        g.set_cell_order(order)
        if counting:
            g.set_counting(True)
        for c in range(sweeps):
            st = g.sweep(t, r, seed=99, counter=c, log=True)
            moves, codes = g.sweep_log()
            out.append((st["moves"], st["accepted"], st["rejected_overlap"], st["rejected_domain"],
                        moves.tobytes(), codes.tobytes()))
            # a box move between sweeps rebuilds or remaps the grid (a new order)
            nb = np.asarray(g.state()[2]).reshape(9) * 1.001
            out.append(g.try_scaling(nb))
        if counting:
            out.append(g.cached_overlaps())
        return g.state(), out


@pytest.mark.parametrize("name", CASES)
def test_cell_order_leaves_the_same_state(engine, name):
    cfg = systems.ALL[name]()
    (p1, r1, _), s1 = run(cfg, False)
    (p2, r2, _), s2 = run(cfg, True)
    assert s1 == s2
    assert np.array_equal(p1, p2) and np.array_equal(r1, r2)


def test_cell_order_in_overlap_counting(engine):
    cfg = list(systems.ALL["sc_l2_dense"]())
    cfg[2] = cfg[2] * 0.95
    cfg[4] = np.asarray(cfg[4]) * 0.95
    (p1, r1, _), s1 = run(tuple(cfg), False, counting=True)
    (p2, r2, _), s2 = run(tuple(cfg), True, counting=True)
    assert s1 == s2
    assert np.array_equal(p1, p2) and np.array_equal(r1, r2)


def run_soft(cfg, order, kind, eps, sigma, hard, sweeps=3):
    from rampack_gb300.packing import GpuPacking
    t, r = (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)
    out = []
    with GpuPacking(*cfg) as g:
        g.set_cell_order(order)
        g.set_soft(kind, eps, sigma, hard)
        g.set_temperature(1.0)
        for c in range(sweeps):
            st = g.sweep(t, r, seed=31, counter=c, log=True)
            moves, codes = g.sweep_log()
            out.append((st["moves"], st["accepted"], moves.tobytes(), codes.tobytes()))
        return g.state(), out


@pytest.mark.parametrize("name,kind,eps,sigma,hard", [("hs_small", 1, 1.0, 1.0, False), ("sc_l2", 2, 1.0, 1.2, True)])
def test_cell_order_in_soft_sweeps(engine, name, kind, eps, sigma, hard):
    """The FP64 sweep of soft parts takes the same occupancy order."""
    cfg = systems.ALL[name]()
    (p1, r1, _), s1 = run_soft(cfg, False, kind, eps, sigma, hard)
    (p2, r2, _), s2 = run_soft(cfg, True, kind, eps, sigma, hard)
    assert s1 == s2
    assert np.array_equal(p1, p2) and np.array_equal(r1, r2)


def test_cell_order_in_convex_sweeps(engine):
    """And the FP64 sweep of generic convex bodies."""
    from rampack_gb300 import _lib
    from rampack_gb300.packing import GpuPacking
    from convex_bodies import BODIES, CIRCUMSPHERE, lattice
    pos, rot, box = lattice(6, 2.02 * CIRCUMSPHERE["cuboid"])
    res = []
    for order in (False, True):
        with GpuPacking(_lib.SHAPE_CONVEX, BODIES["cuboid"], pos, rot, box) as g:
            g.set_cell_order(order)
            logs = []
            for c in range(3):
                g.sweep(0.3, 0.3, seed=8, counter=c, log=True)
                moves, codes = g.sweep_log()
                logs.append((moves.tobytes(), codes.tobytes()))
            res.append((g.state(), logs))
    (s1, l1), (s2, l2) = res
    assert l1 == l2
    assert all(np.array_equal(a, b) for a, b in zip(s1, s2))
