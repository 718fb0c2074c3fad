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
