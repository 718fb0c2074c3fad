"""GPU parity against the CPU oracle (the reference's algorithm restated; pinned to the
reference's own outputs by tests/test_oracle_vs_reference.py and the golden fixtures).

Every decision is compared bit-exactly: overlap counts, per-move outcome codes
(accept/reject and the reason), the final FP64 positions and orientations, and box-move
outcomes.  Move streams are drawn by the reference's sampler algorithms (restated in
the oracle) or logged by the GPU's own device-driven sweep and replayed serially."""
import numpy as np
import pytest

import pyoracle as po
import systems
from rampack_gb300 import _lib

pytestmark = pytest.mark.gpu

CASES = ["hs_small", "hs_dense", "sc_l2", "sc_l2_dense", "sc_l5", "poly_banana", "poly_dense", "hs_tiny", "sc_tiny",
         "psc_bent", "psc_tiny"]


def gpu_packing(cfg):
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = cfg
    return GpuPacking(kind, prm, pos, rot, box)


def cpu_packing(cfg):
    kind, prm, pos, rot, box = cfg
    return po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)


def steps(cfg):
    return (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("factor", [1.0, 0.97, 0.9])
def test_count_overlaps(oracle, engine, name, factor):
    cfg = systems.ALL[name]()
    if factor != 1.0:
        cfg = systems.compressed(cfg, factor)
    cpu = cpu_packing(cfg)
    expect = cpu.count_overlaps(False)
    expect_early = cpu.count_overlaps(True)
    with gpu_packing(cfg) as g:
        for shift in [(0, 0, 0), (0.37, 0.81, 0.05)]:
            g.set_grid(shift)
            assert g.count_total_overlaps(False) == expect
            assert g.count_total_overlaps(True) == expect_early
    if factor == 1.0:
        assert expect == 0


def draw_cell_moves(cpu, g, seed, trans, rot, shift):
    """Moves for every active cell, phase by phase, drawn with the reference samplers'
    algorithm from each cell's particle list (DD domain = cell)."""
    from rampack_gb300.packing import cell_phase
    info = g.set_grid(shift)
    _, cells, bounds = g.grid()
    dims = info["dims"]
    rng = cpu.rng(seed)
    chunks = []
    phase = [cell_phase(dims, c) for c in range(info["num_cells"])]
    for ph in sorted(set(phase)):
        for cell in range(info["num_cells"]):
            if phase[cell] != ph:
                continue
            idx = np.nonzero(cells == cell)[0]
            if len(idx) == 0:
                continue
            ntypes = (trans > 0) + (rot > 0)
            chunks.append(cpu.draw_moves(rng, trans, rot, idx, len(idx), ntypes * len(idx), domain=cell))
    cpu.rng_free(rng)
    return np.concatenate(chunks), bounds


@pytest.mark.parametrize("name", CASES)
def test_move_list_parity(oracle, engine, name):
    cfg = systems.ALL[name]()
    cpu = cpu_packing(cfg)
    t, r = steps(cfg)
    with gpu_packing(cfg) as g:
        for rnd, shift in enumerate([(0.0, 0.0, 0.0), (0.61, 0.13, 0.77), (0.29, 0.93, 0.41)]):
            moves, bounds = draw_cell_moves(cpu, g, 100 + rnd, t, r, shift)
            got = g.run_moves(moves)
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(got, want), f"round {rnd}: {np.count_nonzero(got != want)} codes differ"
            gp, gr, gb = g.state()
            cp, cr, cb = cpu.state()
            assert np.array_equal(gp, cp) and np.array_equal(gr, cr) and np.array_equal(gb, cb)
        acc = np.count_nonzero(got & _lib.CODE_ACCEPTED)
        assert 0 < acc < len(got)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("fp64_only", [False, True])
def test_sweep_log_replays_on_oracle(oracle, engine, name, fp64_only):
    cfg = systems.ALL[name]()
    cpu = cpu_packing(cfg)
    t, r = steps(cfg)
    with gpu_packing(cfg) as g:
        for cycle in range(3):
            st = g.sweep(t, r, seed=2024, counter=cycle, log=True, fp64_only=fp64_only)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            assert st["moves"] == len(moves) == (1 + (r > 0)) * g.n
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want), f"cycle {cycle}: {np.count_nonzero(codes != want)} codes differ"
            gp, gr, _ = g.state()
            cp, cr, _ = cpu.state()
            assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
            assert g.count_total_overlaps(True) == 0


@pytest.mark.parametrize("name", ["sc_l2", "sc_l2_dense", "sc_l5", "poly_banana", "poly_dense", "hs_dense",
                                  "sc_tiny", "hs_tiny", "psc_bent"])
def test_rototranslation_sweeps_replay_on_oracle(oracle, engine, name):
    # RototranslationSampler moves (translation and rotation in one move, ActiveDomain
    # checked): every logged move of type 2 replays on the oracle's tryMove
    cfg = systems.ALL[name]()
    cpu = cpu_packing(cfg)
    t, r = (0.1 if cfg[0] == 0 else 0.2), 0.3
    if "dense" in name:
        t, r = 0.03, 0.03  # both parts at once: smaller steps keep some moves accepted
    with gpu_packing(cfg) as g:
        for cycle in range(3):
            st = g.sweep(t, r, seed=77, counter=cycle, log=True, rototranslation=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            assert st["moves"] == len(moves) == g.n and np.all(moves["type"] == 2)
            assert st["rotations"] == g.n and st["translations"] == 0
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want), f"cycle {cycle}: {np.count_nonzero(codes != want)} codes differ"
            acc = np.count_nonzero(codes & _lib.CODE_ACCEPTED)
            assert acc == st["accepted"] and 0 < acc < g.n
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
        assert g.count_total_overlaps(True) == 0
        with pytest.raises(Exception):
            g.sweep(t, 0.0, seed=1, counter=9, rototranslation=True)  # both steps are needed


@pytest.mark.parametrize("name", ["sc_l2", "sc_l2_dense", "sc_tiny"])
def test_flip_moves(oracle, engine, name):
    # FlipSampler moves (drawn per cell by the oracle's restatement of the reference's
    # sampler, pinned by tests/test_oracle_golden.py) through the move-list entry
    from rampack_gb300.packing import cell_phase
    cfg = systems.ALL[name]()
    cpu = cpu_packing(cfg)
    with gpu_packing(cfg) as g:
        for rnd, shift in enumerate([(0.0, 0.0, 0.0), (0.37, 0.71, 0.05)]):
            info = g.set_grid(shift)
            _, cells, bounds = g.grid()
            phase = [cell_phase(info["dims"], c) for c in range(info["num_cells"])]
            rng = cpu.rng(55 + rnd)
            chunks = []
            for ph in sorted(set(phase)):
                for cell in range(info["num_cells"]):
                    idx = np.nonzero(cells == cell)[0]
                    if phase[cell] == ph and len(idx):
                        chunks.append(cpu.draw_flips(rng, idx, len(idx), flip_axis=(0.0, 1.0, 0.0), domain=cell))
            cpu.rng_free(rng)
            moves = np.concatenate(chunks)
            codes = g.run_moves(moves)
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
            assert np.count_nonzero(codes & _lib.CODE_ACCEPTED) > 0
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)


@pytest.mark.parametrize("name", ["hs_small", "hs_dense", "hs_tiny"])
def test_sphere_sweeps_with_rotations_replay_on_oracle(oracle, engine, name):
    # the Simulation's samplers rotate spheres too (an orientation change that never overlaps)
    cfg = systems.ALL[name]()
    cpu = cpu_packing(cfg)
    with gpu_packing(cfg) as g:
        for cycle in range(2):
            st = g.sweep(0.1, 0.3, seed=31, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            assert st["moves"] == len(moves) == 2 * g.n and st["rotations"] > 0
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
            assert st["accepted"] - st["accepted_translations"] == st["rotations"]  # every rotation accepted
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)


@pytest.mark.parametrize("name", CASES)
def test_staging_filter_keeps_every_decision(oracle, engine, name):
    # candidates left out by the staging filter can never overlap a mover in its cell:
    # forced on, the logged sweeps replay on the oracle and end in the state of the
    # unfiltered sweeps
    cfg = systems.ALL[name]()
    t, r = steps(cfg)
    states = []
    for mode in (2, 0):
        cpu = cpu_packing(cfg)
        with gpu_packing(cfg) as g:
            g.set_staging_filter(mode)
            for cycle in range(3):
                g.sweep(t, r, seed=91, counter=cycle, log=True)
                moves, codes = g.sweep_log()
                _, _, bounds = g.grid()
                want, _ = cpu.replay(moves, bounds)
                assert np.array_equal(codes, want), (mode, cycle)
            states.append(g.state())
    assert np.array_equal(states[0][0], states[1][0]) and np.array_equal(states[0][1], states[1][1])


@pytest.mark.parametrize("name", ["sc_l2_dense", "poly_dense"])
def test_fp32_filter_matches_fp64_only(engine, name):
    cfg = systems.ALL[name]()
    t, r = steps(cfg)
    states = []
    for fp64_only in (False, True):
        with gpu_packing(cfg) as g:
            for cycle in range(4):
                g.sweep(t, r, seed=7, counter=cycle, fp64_only=fp64_only)
            states.append(g.state())
    assert np.array_equal(states[0][0], states[1][0]) and np.array_equal(states[0][1], states[1][1])


@pytest.mark.parametrize("name", CASES)
def test_box_moves(oracle, engine, name):
    cfg = systems.ALL[name]()
    cpu = cpu_packing(cfg)
    rng = np.random.default_rng(5)
    with gpu_packing(cfg) as g:
        for k in range(12):
            _, _, box = cpu.state()
            b = box.reshape(3, 3)
            if k % 3 == 0:
                nb = b * (1 + rng.uniform(-0.02, 0.02))
            elif k % 3 == 1:
                nb = b + rng.uniform(-0.05, 0.05, size=(3, 3))
            else:
                nb = b * 0.9
            nb = nb.reshape(9)
            want = cpu.try_scaling(nb)
            got = g.try_scaling(nb)
            assert got == want
            if want > 0:
                cpu.revert_scaling()
                g.revert_scaling()
            gp, gr, gb = g.state()
            cp, cr, cb = cpu.state()
            assert np.array_equal(gp, cp) and np.array_equal(gb, cb)


@pytest.mark.parametrize("shear", [0.0, 0.04])
def test_tiny_box_without_reference_grid(oracle, engine, shear):
    """Boxes where the reference keeps no neighbour grid measure sphere distances with the
    periodic boundary conditions' formula; in a sheared box that is not the geometric
    distance, so every pair is decided in FP64 (and the decisions still match)."""
    kind, prm, pos, rot, box = systems.hs_tiny()
    b = box.reshape(3, 3).copy()
    b[0, 1] = shear * b[1, 1]
    b[1, 2] = -shear * b[2, 2]
    rel = pos @ np.linalg.inv(box.reshape(3, 3)).T
    cfg = (kind, prm, np.ascontiguousarray(rel @ b.T), rot, b.reshape(9))
    cpu = cpu_packing(cfg)
    with gpu_packing(cfg) as g:
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False)
        for cycle in range(4):
            g.sweep(0.1, 0.0, seed=31, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
        gp, _, _ = g.state()
        cp, _, _ = cpu.state()
        assert np.array_equal(gp, cp)
