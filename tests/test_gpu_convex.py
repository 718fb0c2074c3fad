"""Generic convex bodies (GenericXenoCollideTraits, rp_create_convex) on the GPU.

The device evaluates the XCBodyBuilder geometry's support function and XenoCollide's portal
refinement in FP64 in the reference's operation order: its pair decisions must equal the
reference's own (tests/golden/convex.npz, written by the reference's classes), and packings
must count overlaps, sweep, take single and box moves exactly as the oracle (pinned to the
reference in tests/test_convex_oracle.py): identical outcome codes, counts and final FP64
states.
"""
import os

import numpy as np
import pytest

import pyoracle as po
from convex_bodies import BODIES, CIRCUMSPHERE, lattice

pytestmark = pytest.mark.gpu

PACKED = ["cuboid", "cone", "capsule_wrap", "rotated_sum", "ellipsoid", "football", "saucer"]


def packing(name, factor=1.0, n_side=6):
    from rampack_gb300 import _lib
    from rampack_gb300.packing import GpuPacking
    pos, rot, box = lattice(n_side, 2.02 * CIRCUMSPHERE[name])
    pos, box = pos * factor, np.asarray(box) * factor
    cpu = po.CpuPacking("oracle", po.CONVEX, BODIES[name], pos, rot, box, threads=1)
    g = GpuPacking(_lib.SHAPE_CONVEX, BODIES[name], pos, rot, box)
    return cpu, g


def same_state(g, cpu):
    gp, gr, gb = g.state()
    cp, cr, cb = cpu.state()
    return np.array_equal(gp, cp) and np.array_equal(gr, cr) and np.array_equal(gb, cb)


def test_pair_decisions_match_the_reference_fixture(engine):
    from rampack_gb300 import _lib
    from rampack_gb300.packing import GpuPacking
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "convex.npz"))
    pos, rot, box = lattice(2, 10.0)
    for name in z["names"]:
        with GpuPacking(_lib.SHAPE_CONVEX, BODIES[str(name)], pos, rot, box) as g:
            got = g.convex_pair_overlaps(np.zeros_like(z[f"{name}_p2"]), z[f"{name}_r1"], z[f"{name}_p2"],
                                         z[f"{name}_r2"])
        assert np.array_equal(got, z[f"{name}_overlap"]), (name, np.count_nonzero(got != z[f"{name}_overlap"]))


@pytest.mark.parametrize("name", PACKED)
def test_counts_and_logged_sweeps_replay_on_the_oracle(oracle, engine, name):
    cpu, g = packing(name)
    with g:
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False) == 0
        for cycle in range(3):
            st = g.sweep(0.4, 0.4, seed=21, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want), np.count_nonzero(codes != want)
            assert 0 < st["accepted"] < st["moves"]
        assert same_state(g, cpu)
        # box moves on the swept state: the oracle's tryScaling decisions
        _, _, b = g.state()
        for f in (0.97, 0.995, 1.01):
            nb = np.asarray(b).reshape(9) * f
            assert g.try_scaling(nb) == cpu.try_scaling(nb), f
            g.revert_scaling()
            cpu.revert_scaling()
    cpu.close()


@pytest.mark.parametrize("name", ["cuboid", "cone", "rotated_sum"])
def test_overlap_counting(oracle, engine, name):
    """A compressed lattice holding overlaps: cached counts, logged counting sweeps and a
    counting box move equal the oracle's."""
    cpu, g = packing(name, factor=0.75)
    cpu.set_counting(True)
    with g:
        g.set_counting(True)
        assert g.cached_overlaps() == cpu.cached_overlaps() > 0
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False)
        relieved = 0
        for cycle in range(3):
            g.sweep(0.3, 0.3, seed=5, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
            relieved += np.count_nonzero((codes & 3) == 3)
            assert g.cached_overlaps() == cpu.cached_overlaps()
        assert relieved > 0  # some moves reduced the overlap count (dE = -inf)
        assert same_state(g, cpu)
        _, _, b = g.state()
        nb = np.asarray(b).reshape(9) * 1.02
        assert g.try_scaling(nb) == cpu.try_scaling(nb)
        assert g.cached_overlaps() == cpu.cached_overlaps()
    cpu.close()


@pytest.mark.parametrize("name", ["capsule_wrap", "rotated_sum"])
def test_single_moves_of_the_serial_path(oracle, engine, name):
    cpu, g = packing(name, n_side=4)
    with g:
        rng = cpu.rng(17)
        moves = cpu.draw_moves(rng, 0.6, 0.6, np.arange(cpu.n), cpu.n, 2 * cpu.n, domain=-1)
        cpu.rng_free(rng)
        codes = np.zeros(len(moves), dtype=np.uint8)
        for i, m in enumerate(moves):
            de = g.try_move(int(m["particle"]), int(m["type"]), m["translation"], m["rotation"])
            code = 0 if not np.isinf(de) else 1
            if m["uniform"] <= np.exp(-de):
                g.accept_move()
                code |= 0x80
            codes[i] = code
        want, _ = cpu.replay(moves, None)
        assert np.array_equal(codes, want), np.count_nonzero(codes != want)
        assert 0 < np.count_nonzero(codes & 0x80) < len(codes)
        assert same_state(g, cpu)
    cpu.close()


@pytest.mark.parametrize("name,factor", [("cuboid", 1.0), ("cuboid", 0.8), ("cone", 0.8)])
@pytest.mark.parametrize("allow", [False, True])
def test_orientation_fixes(oracle, engine, name, factor, allow):
    """Packing::renormalizeOrientations: rejected counts and FP64 states as the oracle's."""
    from rampack_gb300 import _lib
    from rampack_gb300.packing import GpuPacking
    pos, rot, box = lattice(5, 2.02 * CIRCUMSPHERE[name])
    pos, box = pos * factor, np.asarray(box) * factor
    rot = rot + np.random.default_rng(2).normal(0.0, 1e-7, rot.shape)
    cpu = po.CpuPacking("oracle", po.CONVEX, BODIES[name], pos, rot, box)
    with GpuPacking(_lib.SHAPE_CONVEX, BODIES[name], pos, rot, box) as g:
        assert g.renormalize_orientations(allow) == cpu.renormalize_orientations(allow)
        assert same_state(g, cpu)
    cpu.close()


@pytest.mark.parametrize("name,mask", [("cuboid", 7), ("cone", 5), ("rotated_sum", 2)])
def test_walls(oracle, engine, name, mask):
    """Hard walls (XenoCollideTraits::overlapWithWall): a lattice pushed against the near walls,
    some bodies through them; counts, logged sweeps in counting mode and a box move, then plain
    sweeps, a single-move stream and orientation fixes, all as the oracle's (pinned to the
    reference with walls in tests/test_convex_oracle.py)."""
    from rampack_gb300 import _lib
    from rampack_gb300.packing import GpuPacking
    spacing = 2.02 * CIRCUMSPHERE[name]
    pos, rot, box = lattice(5, spacing)
    pos = pos - 0.3 * spacing
    cpu = po.CpuPacking("oracle", po.CONVEX, BODIES[name], pos, rot, box, threads=1)
    cpu.set_walls(mask)
    cpu.set_counting(True)
    with GpuPacking(_lib.SHAPE_CONVEX, BODIES[name], pos, rot, box) as g:
        g.set_walls(mask)
        g.set_counting(True)
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False) > 0
        assert g.count_total_overlaps(True) == cpu.count_overlaps(True) == 1
        assert g.cached_overlaps() == cpu.cached_overlaps()
        for cycle in range(2):
            g.sweep(0.3, 0.3, seed=13, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want), np.count_nonzero(codes != want)
            assert g.cached_overlaps() == cpu.cached_overlaps()
        nb = np.asarray(g.state()[2]).reshape(9) * 0.99
        assert g.try_scaling(nb) == cpu.try_scaling(nb)
        assert g.cached_overlaps() == cpu.cached_overlaps()
        assert same_state(g, cpu)
    cpu.close()
    # plain mode: sweeps and a single-move stream from the same start, then orientation fixes
    cpu = po.CpuPacking("oracle", po.CONVEX, BODIES[name], pos, rot, box, threads=1)
    cpu.set_walls(mask)
    with GpuPacking(_lib.SHAPE_CONVEX, BODIES[name], pos, rot, box) as g:
        g.set_walls(mask)
        for cycle in range(2):
            st = g.sweep(0.4, 0.4, seed=3, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want), np.count_nonzero(codes != want)
            assert 0 < st["accepted"] < st["moves"]
        rng = cpu.rng(5)
        moves = cpu.draw_moves(rng, 0.5, 0.5, np.arange(cpu.n), cpu.n, cpu.n, domain=-1)
        cpu.rng_free(rng)
        codes = np.zeros(len(moves), dtype=np.uint8)
        for i, m in enumerate(moves):
            de = g.try_move(int(m["particle"]), int(m["type"]), m["translation"], m["rotation"])
            code = 0 if not np.isinf(de) else 1
            if m["uniform"] <= np.exp(-de):
                g.accept_move()
                code |= 0x80
            codes[i] = code
        want, _ = cpu.replay(moves, None)
        assert np.array_equal(codes, want), np.count_nonzero(codes != want)
        assert same_state(g, cpu)
        p, r, b = g.state()
        r = r + np.random.default_rng(4).normal(0.0, 1e-7, r.shape)
    cpu.close()
    cpu = po.CpuPacking("oracle", po.CONVEX, BODIES[name], p, r, b)
    cpu.set_walls(mask)
    with GpuPacking(_lib.SHAPE_CONVEX, BODIES[name], p, r, b) as g:
        g.set_walls(mask)
        assert g.renormalize_orientations(False) == cpu.renormalize_orientations(False)
        assert same_state(g, cpu)
    cpu.close()


def test_unsupported_operations_are_refused(engine):
    from rampack_gb300._lib import EngineError
    cpu, g = packing("cuboid", n_side=3)
    with g:
        with pytest.raises(EngineError):
            g.set_soft(2, 1.0, 1.0)
    cpu.close()
    from rampack_gb300 import _lib
    from rampack_gb300.packing import GpuPacking
    pos, rot, box = lattice(2, 10.0)
    with pytest.raises(EngineError, match="convex body"):
        GpuPacking(_lib.SHAPE_CONVEX, "sphere 1; sphere 1", pos, rot, box)
