"""Box moves that keep the old cell grid (k_remap) against the oracle.

After a box rescale every particle keeps its relative coordinates up to rounding; when the new
box has the old grid's divisions and origin, the engine copies the old cells and recomputes
only the FP32 cell-local positions instead of rebuilding the grid.  The grid must be the one a
rebuild would build: the overlap decisions of box moves (early-exit recount, and the full
counts of overlap counting mode) equal the oracle's Packing::tryScaling, accepted states keep
sweeping identically to the oracle's replay, and a rounding-induced cell change falls back to
the rebuild (counted by rp_get_grid_counters, Packing::getNeighbourGridRebuilds).
"""
import numpy as np
import pytest

import pyoracle as po
import systems
from test_gpu_parity import cpu_packing, gpu_packing, steps

pytestmark = pytest.mark.gpu

CASES = ["hs_small", "sc_l2", "sc_l5", "poly_banana", "psc_bent"]


def scaled(box, f, shear=0.0):
    b = np.asarray(box, dtype=np.float64).reshape(3, 3) * f
    b[0, 1] += shear * b[1, 1]
    return b.reshape(9)


@pytest.mark.parametrize("name", CASES)
def test_box_moves_on_the_kept_grid_decide_as_the_oracle(oracle, engine, name):
    cfg = systems.ALL[name]()
    cpu, g = cpu_packing(cfg), gpu_packing(cfg)
    t, r = steps(cfg)
    with g:
        before = g.grid_counters()
        remapped = 0
        for cycle in range(6):
            g.sweep(t, r, seed=77, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
            _, _, b = g.state()
            for f, shear in ((1.0 - 1e-4, 0.0), (1.0 + 1e-4, 1e-5), (0.9999, -2e-5)):
                nb = scaled(b, f, shear)
                c0 = g.grid_counters()
                dg, dc = g.try_scaling(nb), cpu.try_scaling(nb)
                assert dg == dc, (cycle, f, dg, dc)
                c1 = g.grid_counters()
                remapped += c1["remaps"] - c0["remaps"]
                if dg == 0 and cycle % 2 == 0:
                    b = nb  # accepted: sweep on from the rescaled state
                    break
                g.revert_scaling()
                cpu.revert_scaling()
        gp, gr, gb = g.state()
        cp, cr, cb = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr) and np.array_equal(gb, cb)
        after = g.grid_counters()
        assert remapped > 0 and after["remaps"] - before["remaps"] == remapped
    cpu.close()


@pytest.mark.parametrize("name,factor", [("hs_dense", 0.97), ("sc_l2_dense", 0.97), ("poly_dense", 0.98)])
def test_counting_box_moves_on_the_kept_grid(oracle, engine, name, factor):
    """Overlap counting: the full recount on the kept grid equals the oracle's count."""
    cfg = systems.compressed(systems.ALL[name](), factor)
    cpu, g = cpu_packing(cfg), gpu_packing(cfg)
    cpu.set_counting(True)
    with g:
        g.set_counting(True)
        assert g.cached_overlaps() == cpu.cached_overlaps() > 0
        _, _, b = g.state()
        remaps0 = g.grid_counters()["remaps"]
        for f in (1.0 - 3e-5, 1.0 + 3e-5, 1.0 - 1e-4):
            nb = scaled(b, f)
            dg, dc = g.try_scaling(nb), cpu.try_scaling(nb)
            assert dg == dc
            assert g.cached_overlaps() == cpu.cached_overlaps()
            g.revert_scaling()
            cpu.revert_scaling()
            assert g.cached_overlaps() == cpu.cached_overlaps()
        assert g.grid_counters()["remaps"] > remaps0
    cpu.close()


def test_changed_divisions_rebuild(oracle, engine):
    """A box move that changes the number of cells rebuilds the grid."""
    cfg = systems.ALL["hs_small"]()
    cpu, g = cpu_packing(cfg), gpu_packing(cfg)
    with g:
        g.sweep(0.1, 0.0, seed=5, counter=0)
        _, _, b = g.state()
        dims0 = g.grid()[0]["dims"]
        c0 = g.grid_counters()
        nb = scaled(b, 1.25)  # an expansion: more cells of the same minimum size
        g.try_scaling(nb)
        assert g.grid()[0]["dims"] != dims0
        c1 = g.grid_counters()
        assert c1["rebuilds"] == c0["rebuilds"] + 1 and c1["remaps"] == c0["remaps"]
    cpu.close()
