"""Two cells per warp (rp_set_cells_per_warp(h, 2)) against a warp per cell and the oracle.

With two cells per warp each half-warp sweeps its own cell and reads the spherocylinder axes
from the FP32 mirror instead of staging them; the proposal stream of a move depends only on
its cell and index, so the sweeps must leave bit-identical states, statistics and logs, and
a logged sweep must replay on the CPU oracle move by move."""
import numpy as np
import pytest

import pyoracle as po
import systems

pytestmark = pytest.mark.gpu

CASES = ["hs_small", "hs_dense", "sc_l2", "sc_l2_dense", "sc_l5", "hs_tiny", "sc_tiny"]
# neighbourhoods too large for a half-warp's staging capacity keep a warp per cell
WARP_PER_CELL = {"sc_l5"}


def steps(cfg):
    return (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)


def run(cfg, cells, sweeps=4, fp64_only=False, log=False, expect=None):
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = cfg
    t, r = steps(cfg)
    out = []
    with GpuPacking(kind, prm, pos, rot, box) as g:
        g.set_cells_per_warp(cells)
        for c in range(sweeps):
            st = g.sweep(t, r, seed=77, counter=c, log=log, fp64_only=fp64_only)
            assert g.cells_per_warp() == (cells if expect is None else expect)  # the path expected ran
            out.append((st["moves"], st["accepted"], st["rejected_overlap"], st["rejected_domain"]))
            if log:
                out.append(g.sweep_log())
        return g.state(), out


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("fp64_only", [False, True])
def test_two_cells_per_warp_leave_the_same_state(engine, name, fp64_only):
    cfg = systems.ALL[name]()
    (p1, r1, b1), s1 = run(cfg, 1, fp64_only=fp64_only)
    (p2, r2, b2), s2 = run(cfg, 2, fp64_only=fp64_only, expect=1 if name in WARP_PER_CELL else 2)
    assert s1 == s2
    assert np.array_equal(p1, p2) and np.array_equal(r1, r2)


@pytest.mark.parametrize("name", CASES)
def test_two_cells_per_warp_log_replays_on_oracle(oracle, engine, name):
    from rampack_gb300.packing import GpuPacking
    cfg = systems.ALL[name]()
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    t, r = steps(cfg)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        g.set_cells_per_warp(2)
        for cycle in range(3):
            g.sweep(t, r, seed=909, counter=cycle, log=True)
            assert g.cells_per_warp() == (1 if name in WARP_PER_CELL else 2)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want), np.count_nonzero(codes != want)
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)


def test_two_cells_per_warp_at_full_size(engine):
    """The bench's 10^6 spherocylinders: three sweeps with two cells per warp end in the state
    of three sweeps with a warp per cell."""
    from rampack_gb300 import workloads as W
    cfg = W.config_sc_1e6()
    (p1, r1, _), s1 = run(cfg, 1, sweeps=3)
    (p2, r2, _), s2 = run(cfg, 2, sweeps=3)
    assert s1 == s2
    assert np.array_equal(p1, p2) and np.array_equal(r1, r2)
