"""Overlap counting mode (Packing::toggleOverlapCounting, core/Packing.cpp:304-323,
:1049-1060) on the GPU against the CPU oracle, on compressed systems that hold overlaps:
cached counts, per-move outcome codes (3 = dE -inf, 1 = +inf, 0 = 0) of move lists and of
logged sweeps, final FP64 states, and counting box moves with revert."""
import numpy as np
import pytest

import pyoracle as po
import systems
from test_gpu_parity import draw_cell_moves, gpu_packing, steps

pytestmark = pytest.mark.gpu

CASES = [("hs_dense", 0.97), ("sc_l2_dense", 0.97), ("sc_l2", 0.94), ("hs_tiny", 0.95), ("poly_banana", 0.97),
         ("poly_dense", 0.98), ("psc_bent", 0.95), ("psc_tiny", 0.95)]


def setup(name, factor):
    cfg = systems.compressed(systems.ALL[name](), factor)
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    cpu.set_counting(True)
    g = gpu_packing(cfg)
    g.set_counting(True)
    return cfg, cpu, g


@pytest.mark.parametrize("name,factor", CASES)
def test_counting_move_lists(oracle, engine, name, factor):
    cfg, cpu, g = setup(name, factor)
    with g:
        assert g.cached_overlaps() == cpu.cached_overlaps() > 0
        t, r = steps(cfg)
        for rnd in range(2):
            moves, bounds = draw_cell_moves(cpu, g, 100 + rnd, t, r, (0.13 * rnd, 0.29, 0.71 * rnd))
            codes = g.run_moves(moves)
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
            assert np.any((codes & 3) == 3)  # some moves relieve overlaps
            assert g.cached_overlaps() == cpu.cached_overlaps()
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
        assert g.count_total_overlaps(False) == g.cached_overlaps()


@pytest.mark.parametrize("name,factor", CASES)
@pytest.mark.parametrize("fp64_only", [False, True])
def test_counting_sweeps_replay(oracle, engine, name, factor, fp64_only):
    cfg, cpu, g = setup(name, factor)
    t, r = steps(cfg)
    with g:
        for cycle in range(2):
            g.sweep(t, r, seed=77, counter=cycle, log=True, fp64_only=fp64_only)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
            assert g.cached_overlaps() == cpu.cached_overlaps()
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)


@pytest.mark.parametrize("name,factor", CASES[:3] + [("poly_banana", 0.97), ("psc_bent", 0.95)])
def test_counting_box_moves(oracle, engine, name, factor):
    cfg, cpu, g = setup(name, factor)
    rng = np.random.default_rng(3)
    with g:
        for k in range(8):
            _, _, box = cpu.state()
            nb = box.reshape(3, 3) * (1 + rng.uniform(-0.01, 0.01)) + rng.uniform(-0.003, 0.003, (3, 3))
            want = cpu.try_scaling(nb.reshape(9))
            got = g.try_scaling(nb.reshape(9))
            assert got == want
            assert g.cached_overlaps() == cpu.cached_overlaps()
            if k % 2 == 0:
                cpu.revert_scaling()
                g.revert_scaling()
                assert g.cached_overlaps() == cpu.cached_overlaps()
        gp, gr, gb = g.state()
        cp, cr, cb = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gb, cb)
