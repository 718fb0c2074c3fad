"""Hard walls on the GPU (rp_set_walls) against the oracle with the same walls (pinned to the
reference by tests/test_walls.py): recounts, move lists, logged sweeps, overlap counting,
box moves and orientation renormalisation."""
import os

import numpy as np
import pytest

import pyoracle as po
import systems
from test_gpu_parity import draw_cell_moves, gpu_packing, steps

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "walls.npz")
CASES = [("hs_small", 1), ("sc_l2", 5), ("poly_banana", 2), ("sc_l2_dense", 7), ("hs_tiny", 3), ("sc_tiny", 6),
         ("poly_dense", 4), ("psc_bent", 3)]
# (index in tests/golden/walls.npz, system, wall mask)
GOLDEN = [(0, "hs_small", 1), (1, "sc_l2", 5), (2, "poly_banana", 2), (3, "sc_l2_dense", 7), (4, "psc_bent", 3)]


def pair(name, mask, counting=False):
    cfg = systems.ALL[name]()
    cpu = po.CpuPacking("oracle", *cfg, threads=1)
    cpu.set_walls(mask)
    g = gpu_packing(cfg)
    g.set_walls(mask)
    if counting:
        cpu.set_counting(True)
        g.set_counting(True)
    return cfg, cpu, g


def test_wall_counts_match_the_reference(engine):
    z = np.load(GOLD)
    for i, name, mask in GOLDEN:
        cfg = systems.ALL[name]()
        with gpu_packing(cfg) as g:
            g.set_walls(mask)
            assert [g.count_total_overlaps(False), g.count_total_overlaps(True) > 0] == \
                [int(z[f"w{i}_counts"][0]), int(z[f"w{i}_counts"][1]) > 0]


@pytest.mark.parametrize("name,mask", CASES)
def test_wall_move_lists_and_sweeps(oracle, engine, name, mask):
    cfg, cpu, g = pair(name, mask)
    t, r = steps(cfg)
    with g:
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False)
        moves, bounds = draw_cell_moves(cpu, g, 9, t, r, (0.31, 0.17, 0.83))
        assert np.array_equal(g.run_moves(moves), cpu.replay(moves, bounds)[0])
        for cycle in range(2):
            g.sweep(t, r, seed=606, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            assert np.array_equal(codes, cpu.replay(moves, bounds)[0]), cycle
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False)
        # box moves: a compression and an expansion with walls
        for f in (0.995, 1.003):
            _, _, box = cpu.state()
            nb = (box.reshape(3, 3) * f).reshape(9)
            assert g.try_scaling(nb) == cpu.try_scaling(nb)
        gp, _, gb = g.state()
        cp, _, cb = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gb, cb)


@pytest.mark.parametrize("name,mask", [("hs_small", 1), ("sc_l2", 5), ("sc_l2_dense", 7), ("poly_banana", 2),
                                       ("psc_bent", 3)])
def test_wall_overlap_counting(oracle, engine, name, mask):
    cfg, cpu, g = pair(name, mask, counting=True)
    t, r = steps(cfg)
    with g:
        assert g.cached_overlaps() == cpu.cached_overlaps() > 0
        for cycle in range(2):
            g.sweep(t, r, seed=707, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            assert np.array_equal(codes, cpu.replay(moves, bounds)[0])
            assert g.cached_overlaps() == cpu.cached_overlaps()
        assert g.count_total_overlaps(False) == g.cached_overlaps()


@pytest.mark.parametrize("name,mask", [("sc_l2", 7), ("poly_banana", 2)])
def test_wall_renormalisation(oracle, engine, name, mask):
    cfg = systems.ALL[name]()
    kind, prm, pos, rot, box = cfg
    noisy = rot + np.random.default_rng(3).normal(scale=1e-7, size=rot.shape)
    cpu = po.CpuPacking("oracle", kind, prm, pos, noisy, box, threads=1)
    cpu.set_walls(mask)
    with gpu_packing((kind, prm, pos, noisy, box)) as g:
        g.set_walls(mask)
        rejected = cpu.renormalize_orientations(False)
        assert rejected > 0  # fixes of particles touching a wall are refused
        assert g.renormalize_orientations(False) == rejected
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gr, cr)
