"""The GPU engine against golden fixtures produced by the reference's own code
(tests/golden/make_golden.py): overlap counts, per-move outcome codes, final FP64 state
and box-move outcomes must match bit for bit; plus the reference's Packing unit-test
known answers (test/unit_tests/core/PackingTest.cpp:86-166) run on the GPU."""
import math
import os

import numpy as np
import pytest

from rampack_gb300 import _lib

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("name", ["hs", "sc_l2", "sc_l5"])
def test_golden_system(engine, name):
    from rampack_gb300.packing import GpuPacking
    g = load(f"system_{name}.npz")
    kind, prm = int(g["kind"]), g["params"]
    with GpuPacking(kind, prm, g["comp_pos"], g["rot"], g["comp_box"]) as comp:
        assert comp.count_total_overlaps(False) == int(g["comp_count"])
        assert comp.count_total_overlaps(True) == int(g["comp_count_early"])
    with GpuPacking(kind, prm, g["pos"], g["rot"], g["box"]) as pk:
        assert pk.count_total_overlaps(False) == int(g["count"])
        assert pk.count_total_overlaps(True) == int(g["count_early"])
        moff, coff = 0, 0
        for shift, nm, nc in zip(g["shifts"], g["chunk_moves"], g["chunk_cells"]):
            info = pk.set_grid(shift)
            _, _, bounds = pk.grid()
            assert info["num_cells"] == nc
            assert np.array_equal(bounds, g["bounds"][coff:coff + nc])
            mv = g["moves"][moff:moff + nm].copy()
            mv["domain"] -= coff
            codes = pk.run_moves(mv)
            assert np.array_equal(codes, g["codes"][moff:moff + nm])
            moff += nm
            coff += nc
        p, r, b = pk.state()
        assert np.array_equal(p, g["move_pos"]) and np.array_equal(r, g["move_rot"]) and np.array_equal(b, g["move_box"])
        for nb, dE in zip(g["scale_boxes"], g["scale_dE"]):
            got = pk.try_scaling(nb)
            assert got == dE
            if got > 0:
                pk.revert_scaling()
        p, r, b = pk.state()
        assert np.array_equal(p, g["final_pos"]) and np.array_equal(r, g["final_rot"])
        assert np.array_equal(b, g["final_box"])


def hs_three():
    pos = np.array([[0.5, 0.5, 0.5], [4.5, 0.5, 0.5], [2.5, 2.5, 4.0]])
    rot = np.tile(np.eye(3).reshape(9), (3, 1))
    return _lib.SHAPE_SPHERE, np.array([0.25]), pos, rot, np.diag([5.0, 5, 5]).reshape(9)


@pytest.mark.parametrize("factor,expect", [(1.1, 0.0), (0.51, 0.0), (0.49, math.inf)])
def test_known_answer_scaling(engine, factor, expect):
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = hs_three()
    with GpuPacking(kind, prm, pos, rot, box) as pk:
        assert pk.try_scaling(box * factor) == expect
        p, _, _ = pk.state()
        assert p == pytest.approx(pos * factor, abs=1e-9)
        if expect > 0:
            pk.revert_scaling()
            p, _, b = pk.state()
            assert np.array_equal(p, pos) and np.array_equal(b, box)


@pytest.mark.parametrize("dy", [2.45, 2.55, 0.01])
def test_known_answer_translation_with_active_domain(engine, oracle, dy):
    """PackingTest.cpp:150-166's translations of particle 2, made inside particle 2's grid
    cell as ActiveDomain: the GPU and the oracle replay agree on the outcome code."""
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = hs_three()
    with GpuPacking(kind, prm, pos, rot, box) as pk:
        info = pk.set_grid((0.0, 0.0, 0.0))
        _, cells, bounds = pk.grid()
        assert info["dims"] == (8, 8, 8)  # floor(5 / (0.5 (1 + 1e-9))) = 9, odd above 3: one cell fewer
        mv = np.zeros(1, dtype=_lib.MOVE_DTYPE)
        mv["particle"], mv["type"], mv["domain"], mv["uniform"] = 2, 0, int(cells[2]), 0.5
        mv["translation"][0] = [dy, dy, dy] if dy < 0.1 else [2, dy, -3.5]
        codes = pk.run_moves(mv)
        cpu = oracle.CpuPacking("oracle", kind, prm, pos, rot, box)
        want, _ = cpu.replay(mv, bounds)
        assert np.array_equal(codes, want)
        assert (codes[0] & 3) == (0 if dy < 0.1 else 2)
