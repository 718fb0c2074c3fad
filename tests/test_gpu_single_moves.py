"""Unrestricted single moves (rp_try_move / rp_accept_move) against the oracle.

The reference's serial path (Simulation::performMovesWithoutDomainDivision,
core/Simulation.cpp:365-390) tries one move at a time with no ActiveDomain
(Packing::tryTranslation / tryRotation / tryMove with std::nullopt, core/Packing.cpp:84-164)
and accepts it after the Metropolis test (core/Simulation.cpp:483).  Streams of such moves are
drawn with the reference's sampler algorithms (restated in the oracle) over all particles,
run through the engine's per-move entry points one move at a time, and replayed on the oracle
with no ActiveDomain: every energy class, every accept/reject and the final FP64 state must be
identical.  Also covered: overlap counting (energies -inf / 0 / +inf and the cached count),
device sweeps and box moves after single moves (the cell grid is rebuilt from the moved
state), more moved particles than the engine keeps out of its grid, and the errors of
accepting with no tried move pending.
"""
import numpy as np
import pytest

import pyoracle as po
import systems
from rampack_gb300 import _lib
from rampack_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = ["hs_small", "hs_dense", "sc_l2", "sc_l2_dense", "sc_l5", "poly_banana", "poly_dense", "hs_tiny", "sc_tiny",
         "psc_bent", "psc_tiny"]


def steps(cfg):
    return (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)


def serial_moves(cpu, seed, trans, rot, rounds=1):
    """Moves of the serial path: per move a move type, the sampler's draws, a particle out of
    all N and the Metropolis uniform (the reference samplers' algorithm, no domain)."""
    rng = cpu.rng(seed)
    ntypes = (trans > 0) + (rot > 0)
    idx = np.arange(cpu.n)
    mv = np.concatenate([cpu.draw_moves(rng, trans, rot, idx, cpu.n, ntypes * cpu.n, domain=-1)
                         for _ in range(rounds)])
    cpu.rng_free(rng)
    return mv


def run_single(g, moves, temperature=1.0):
    """The moves one at a time through rp_try_move / rp_accept_move; the outcome codes."""
    codes = np.zeros(len(moves), dtype=np.uint8)
    for i, m in enumerate(moves):
        de = g.try_move(int(m["particle"]), int(m["type"]), m["translation"], m["rotation"])
        code = 0 if de == 0 else (1 if de > 0 else 3)
        if m["uniform"] <= np.exp(-de / temperature):
            g.accept_move()
            code |= _lib.CODE_ACCEPTED
        codes[i] = code
    return codes


def assert_same_state(g, cpu):
    gp, gr, gb = g.state()
    cp, cr, cb = cpu.state()
    assert np.array_equal(gp, cp) and np.array_equal(gr, cr) and np.array_equal(gb, cb)


@pytest.mark.parametrize("name", CASES)
def test_serial_stream_parity(oracle, engine, name):
    from rampack_gb300.packing import GpuPacking
    cfg = systems.ALL[name]()
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    t, r = steps(cfg)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        moves = serial_moves(cpu, 31, t, r)
        got = run_single(g, moves)
        want, _ = cpu.replay(moves, None)
        assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} of {len(got)} codes differ"
        acc = np.count_nonzero(got & _lib.CODE_ACCEPTED)
        assert 0 < acc < len(got)
        assert_same_state(g, cpu)
        # a logged device sweep after the single moves starts from the moved state
        g.sweep(t, r, seed=5, counter=0, log=True)
        lm, lc = g.sweep_log()
        _, _, bounds = g.grid()
        want, _ = cpu.replay(lm, bounds)
        assert np.array_equal(lc, want)
        assert_same_state(g, cpu)
        # and single moves after the sweep
        moves = serial_moves(cpu, 32, t, r)
        got = run_single(g, moves)
        want, _ = cpu.replay(moves, None)
        assert np.array_equal(got, want)
        assert_same_state(g, cpu)


@pytest.mark.parametrize("name", ["hs_dense", "sc_l2_dense", "poly_dense", "psc_bent"])
def test_serial_stream_with_overlaps_in_counting_mode(oracle, engine, name):
    from rampack_gb300.packing import GpuPacking
    cfg = systems.compressed(systems.ALL[name](), 0.97)
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    cpu.set_counting(True)
    t, r = steps(cfg)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        g.set_counting(True)
        assert g.cached_overlaps() == cpu.cached_overlaps() > 0
        moves = serial_moves(cpu, 77, t, r)
        got = run_single(g, moves)
        want, _ = cpu.replay(moves, None)
        assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} codes differ"
        assert np.count_nonzero((got & 3) == 3) > 0  # some moves removed overlaps
        assert g.cached_overlaps() == cpu.cached_overlaps()
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False)
        assert_same_state(g, cpu)


def test_box_move_after_single_moves(oracle, engine):
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = systems.ALL["sc_l2"]()
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        moves = serial_moves(cpu, 3, 0.2, 0.2)
        got = run_single(g, moves)
        want, _ = cpu.replay(moves, None)
        assert np.array_equal(got, want)
        _, _, b = g.state()
        for f in (1.001, 0.999, 0.98):
            nb = np.asarray(b, dtype=np.float64).reshape(9) * f
            assert g.try_scaling(nb) == cpu.try_scaling(nb)
            g.revert_scaling()
            cpu.revert_scaling()
        assert_same_state(g, cpu)
        # single moves after the reverted box moves
        moves = serial_moves(cpu, 4, 0.2, 0.2)
        got = run_single(g, moves)
        want, _ = cpu.replay(moves, None)
        assert np.array_equal(got, want)
        assert_same_state(g, cpu)


def test_more_moved_particles_than_the_grid_keeps_aside(oracle, engine):
    """8000 spherocylinders: the serial stream moves more than 4096 distinct particles, so
    the engine rebuilds its grid in the middle of the stream; decisions stay the oracle's."""
    from rampack_gb300.packing import GpuPacking
    cfg = systems.thermalise(W.spherocylinders((20, 20, 20), 0.30, 2.0, 0.5, aspect=(1, 1, 3)), 3,
                             translation_step=0.2, rotation_step=0.2)
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        moves = serial_moves(cpu, 11, 0.2, 0.2)
        got = run_single(g, moves)
        want, _ = cpu.replay(moves, None)
        assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} codes differ"
        moved = np.unique(moves["particle"][(got & _lib.CODE_ACCEPTED) != 0])
        assert len(moved) > 4096
        assert_same_state(g, cpu)


def test_accept_needs_a_tried_move(engine):
    from rampack_gb300.packing import GpuPacking
    from rampack_gb300._lib import EngineError
    kind, prm, pos, rot, box = systems.ALL["hs_small"]()
    with GpuPacking(kind, prm, pos, rot, box) as g:
        with pytest.raises(EngineError):
            g.accept_move()
        g.try_move(0, 0, (0.01, 0.0, 0.0))
        g.accept_move()
        with pytest.raises(EngineError):  # accepted once
            g.accept_move()
        g.try_move(1, 0, (0.01, 0.0, 0.0))
        g.sweep(0.1, 0.0, seed=1, counter=0)
        with pytest.raises(EngineError):  # the sweep changed the packing
            g.accept_move()
        with pytest.raises(EngineError):
            g.try_move(len(pos), 0, (0.0, 0.0, 0.0))


@pytest.mark.parametrize("name", ["hs_small", "sc_l2", "poly_banana", "psc_bent"])
def test_single_moves_with_an_active_domain(oracle, engine, name):
    """Moves drawn per cell of the engine's grid, each tried with its cell as ActiveDomain
    (Packing::tryTranslation(..., ActiveDomain)): energies and accepts as the oracle's."""
    from rampack_gb300.packing import GpuPacking
    from test_gpu_parity import draw_cell_moves
    cfg = systems.ALL[name]()
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    t, r = steps(cfg)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        moves, bounds = draw_cell_moves(cpu, g, 17, t, r, (0.31, 0.52, 0.73))
        got = np.zeros(len(moves), dtype=np.uint8)
        for i, m in enumerate(moves):
            de = g.try_move(int(m["particle"]), int(m["type"]), m["translation"], m["rotation"],
                            domain=bounds[int(m["domain"])])
            code = 0 if de == 0 else 1
            if m["uniform"] <= np.exp(-de):
                g.accept_move()
                code |= _lib.CODE_ACCEPTED
            got[i] = code
        want, _ = cpu.replay(moves, bounds)
        want = np.where((want & 3) == 2, (want & ~np.uint8(3)) | 1, want).astype(np.uint8)  # outside: +inf as well
        assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} codes differ"
        assert_same_state(g, cpu)
