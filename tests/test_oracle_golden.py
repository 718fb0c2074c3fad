"""The oracle against golden fixtures produced by the reference's own code
(tests/golden/make_golden.py): every value must match bit for bit."""
import ast
import os

import numpy as np
import pytest

import pyoracle as po

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def test_pair_overlaps(oracle):
    g = load("pairs.npz")
    bad = 0
    for i in range(len(g["overlap"])):
        kind = int(g["kind"][i])
        prm = np.array([g["params"][i][1]]) if kind == po.SPHERE else g["params"][i]
        ov = po.pair_overlap("oracle", kind, prm, g["p1"][i], g["r1"][i], g["p2"][i], g["r2"][i],
                             translation=g["translation"][i])
        bad += int(ov) != int(g["overlap"][i])
    assert bad == 0


def test_box_geometry_and_rotations(oracle):
    g = load("geometry.npz")
    for b, inv, h, v in zip(g["boxes"], g["inv"], g["heights"], g["volume"]):
        i2, h2, v2 = po.box_info("oracle", b)
        assert np.array_equal(i2, inv) and np.array_equal(h2, h) and v2 == v
    for a, ang, r in zip(g["axes"], g["angles"], g["rotations"]):
        assert np.array_equal(po.rotation("oracle", a, ang), r)


def test_proposal_stream(oracle):
    g = load("proposals.npz")
    from rampack_gb300 import workloads as W
    kind, prm, pos, rot, box = W.spherocylinders((6, 6, 6), 0.3, 2.0, 0.5, aspect=(1, 1, 3))
    pk = po.CpuPacking("oracle", kind, prm, pos, rot, box)
    r = pk.rng(int(g["seed"]))
    mv = pk.draw_moves(r, float(g["trans"]), float(g["rot"]), g["idx"], int(g["per_type"]), len(g["moves"]),
                       domain=5)
    pk.rng_free(r)
    assert mv.tobytes() == g["moves"].tobytes()


def test_flip_stream(oracle):
    # FlipSampler (core/move_samplers/FlipSampler.cpp:18-41) for spherocylinders: the body
    # flip axis is the primary axis z crossed with x, i.e. y (ShapeGeometry::findFlipAxis)
    g = load("flips.npz")
    import systems
    kind, prm, pos, _, box = systems.sc_l2()
    pk = po.CpuPacking("oracle", kind, prm, pos, g["rot"], box)
    r = pk.rng(int(g["seed"]))
    mv = pk.draw_flips(r, g["idx"], len(g["moves"]), flip_axis=(0.0, 1.0, 0.0))
    pk.rng_free(r)
    assert mv.tobytes() == g["moves"].tobytes()
    assert np.all(mv["type"] == 1)


@pytest.mark.parametrize("name", ["hs", "sc_l2", "sc_l5"])
def test_system(oracle, name):
    g = load(f"system_{name}.npz")
    kind, prm = int(g["kind"]), g["params"]
    pk = po.CpuPacking("oracle", kind, prm, g["pos"], g["rot"], g["box"])
    assert pk.count_overlaps(False) == int(g["count"])
    assert pk.count_overlaps(True) == int(g["count_early"])
    comp = po.CpuPacking("oracle", kind, prm, g["comp_pos"], g["rot"], g["comp_box"])
    assert comp.count_overlaps(False) == int(g["comp_count"])
    assert comp.count_overlaps(True) == int(g["comp_count_early"])
    codes, _ = pk.replay(g["moves"], g["bounds"])
    assert np.array_equal(codes, g["codes"])
    p, r, b = pk.state()
    assert np.array_equal(p, g["move_pos"]) and np.array_equal(r, g["move_rot"]) and np.array_equal(b, g["move_box"])
    for nb, dE in zip(g["scale_boxes"], g["scale_dE"]):
        got = pk.try_scaling(nb)
        assert got == dE
        if got > 0:
            pk.revert_scaling()
    p, r, b = pk.state()
    assert np.array_equal(p, g["final_pos"]) and np.array_equal(r, g["final_rot"]) and np.array_equal(b, g["final_box"])


@pytest.mark.parametrize("name", ["hs1000", "sc_dd"])
def test_cycle_loop(oracle, name):
    g = load(f"sim_{name}.npz")
    kw = ast.literal_eval(str(g["params_json"]))
    pk = po.CpuPacking("oracle", int(g["kind"]), g["params"], g["pos"], g["rot"], g["box"],
                       threads=kw.get("threads", 1))
    st = po.run_cycles(pk, int(g["cycles"]), **kw)
    assert list(st.moves) == list(g["moves"]) and list(st.accepted) == list(g["accepted"])
    p, r, b = pk.state()
    assert np.array_equal(p, g["final_pos"]) and np.array_equal(r, g["final_rot"]) and np.array_equal(b, g["final_box"])
