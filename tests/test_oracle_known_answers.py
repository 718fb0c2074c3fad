"""Known-answer cases of the reference's own unit tests, restated against the oracle
(test/unit_tests/core/shapes/SpherocylinderTraitsTest.cpp:14-123,
SphereTraitsTest.cpp:24-44, PeriodicBoundaryConditionsTest.cpp:9-70,
TriclinicBoxTest.cpp:11-65, PackingTest.cpp:86-166)."""
import math

import numpy as np
import pytest

import pyoracle as po


def rot_euler_y(angle):
    return np.array([math.cos(angle), 0, math.sin(angle), 0, 1, 0, -math.sin(angle), 0, math.cos(angle)])


def m(a):
    return np.asarray(a, dtype=np.float64).reshape(3, 3)


# SpherocylinderTraitsTest.cpp: SpherocylinderTraits(3, 2), shapes rotated by
# rotation(0, pi/2, 0) then the listed matrix, translated by the listed vector * 0.95 (overlap)
# or * 1.05 (no overlap).
SC_CASES = {
    "sphere-sphere": (
        [0.92669949443125, -0.3009522885099318, 0.2250683608628711, 0.3235062902233933, 0.943614995716347,
         -0.07024542721869537, -0.191237358292679, 0.1379074323590797, 0.971807497858173],
        [0.1017126282787795, -0.2093565370521866, 0.972535028491077, 0.5191108031629524, 0.845122866944617,
         0.127637431056981, -0.848633322046771, 0.4918711011645504, 0.1946389081120092],
        [1, 2, 3], [-3.5, 2.9, -0.5]),
    "sphere-cylinder": (
        [0.936848795202308, -0.03157560239884583, 0.34830635403497, -0.03157560239884583, 0.984212198800577,
         0.174153177017485, -0.34830635403497, -0.174153177017485, 0.921060994002885],
        [0.07918504528890558, 0.3698006820181268, -0.925730621823391, -0.2008438095940726, 0.915521563787973,
         0.348542723904781, 0.976417683550607, 0.1583278933673811, 0.1467677942585273],
        [1, 2, 3], [-0.5, 4, -2]),
    "cylinder-cylinder": (
        [0.921060994002885, 0.1446263415347036, 0.361565853836759, -0.1446263415347036, 0.989111861241777,
         -0.02722034689555686, -0.361565853836759, -0.02722034689555686, 0.931949132761108],
        [0.4161880560663263, 0.5570946854720225, -0.7186327388914037, -0.902545539870646, 0.1570999152673587,
         -0.4009129145869377, -0.1104493116652922, 0.815453939865286, 0.5681864320017205],
        [1, 2, 3], [-0.5, 1.7, -0.8]),
}


@pytest.mark.parametrize("case", list(SC_CASES))
@pytest.mark.parametrize("scale,expect", [(0.95, True), (1.05, False)])
def test_spherocylinder_known_answers(oracle, case, scale, expect):
    ra, rb, ta, tb = SC_CASES[case]
    corr = m(rot_euler_y(math.pi / 2))
    r1 = (m(ra) @ corr).reshape(9)
    r2 = (m(rb) @ corr).reshape(9)
    p1 = np.array(ta, dtype=float) * scale
    p2 = np.array(tb, dtype=float) * scale
    prm = np.array([3.0, 2.0])
    for which in ("oracle",) + (("reference",) if po.reference_available() else ()):
        assert po.pair_overlap(which, po.SPHEROCYLINDER, prm, p1, r1, p2, r2) == expect
        assert po.pair_overlap(which, po.SPHEROCYLINDER, prm, p2, r2, p1, r1) == expect


@pytest.mark.parametrize("z1,expect", [(96.6, True), (96.4, False)])
def test_spherocylinder_through_pbc(oracle, z1, expect):
    # SpherocylinderTraits(3, 2) aligned with z in a periodic box of side 100
    box = np.diag([100.0, 100.0, 100.0]).reshape(9)
    eye = np.eye(3).reshape(9)
    prm = np.array([3.0, 2.0])
    assert po.pair_overlap("oracle", po.SPHEROCYLINDER, prm, [50, 50, z1], eye, [50, 50, 3.5], eye, box=box) == expect


@pytest.mark.parametrize("y1,expect", [(19.1, True), (18.9, False)])
def test_sphere_through_pbc(oracle, y1, expect):
    # SphereTraits(2.5) in a periodic box of side 20: a 3-4-5 triangle through the y boundary
    box = np.diag([20.0, 20.0, 20.0]).reshape(9)
    eye = np.eye(3).reshape(9)
    assert po.pair_overlap("oracle", po.SPHERE, [2.5], [1, y1, 10], eye, [5, 2, 10], eye, box=box) == expect
    assert po.pair_overlap("oracle", po.SPHERE, [2.5], [5, 2, 10], eye, [1, y1, 10], eye, box=box) == expect


def test_triclinic_box(oracle):
    # TriclinicBoxTest.cpp: sides {16, 8, 0}, {4, 16, 0}, {0, 0, 10}
    box = np.array([16, 4, 0, 8, 16, 0, 0, 0, 10], dtype=float)
    inv, h, v = po.box_info("oracle", box)
    assert v == pytest.approx(2240)
    assert h == pytest.approx([56 / math.sqrt(17), 28 / math.sqrt(5), 10])
    assert m(inv) @ np.array([9, 8, 5.0]) == pytest.approx([0.5, 0.25, 0.5])


def hs_three():
    # PackingTest.cpp:86-96: hard spheres r=0.25 at three positions in a 5x5x5 box
    pos = np.array([[0.5, 0.5, 0.5], [4.5, 0.5, 0.5], [2.5, 2.5, 4.0]])
    rot = np.tile(np.eye(3).reshape(9), (3, 1))
    return po.SPHERE, np.array([0.25]), pos, rot, np.diag([5.0, 5, 5]).reshape(9)


@pytest.mark.parametrize("factor,expect", [(1.1, 0.0), (0.51, 0.0), (0.49, math.inf)])
def test_packing_scaling_known_answers(oracle, factor, expect):
    kind, prm, pos, rot, box = hs_three()
    pk = po.CpuPacking("oracle", kind, prm, pos, rot, box)
    assert pk.try_scaling(box * factor) == expect
    p, _, _ = pk.state()
    assert p == pytest.approx(pos * factor, abs=1e-9)
    if expect > 0:
        pk.revert_scaling()
        p, _, b = pk.state()
        assert np.array_equal(p, pos) and np.array_equal(b, box)


@pytest.mark.parametrize("dy,expect", [(2.45, 0), (2.55, 1)])
def test_packing_translation_known_answers(oracle, dy, expect):
    # PackingTest.cpp:150-166: particle 2 translated by {2, dy, -3.5} touches particle 1 through y
    kind, prm, pos, rot, box = hs_three()
    pk = po.CpuPacking("oracle", kind, prm, pos, rot, box)
    mv = np.zeros(1, dtype=po.MOVE_DTYPE)
    mv["particle"], mv["type"], mv["domain"], mv["uniform"] = 2, 0, -1, 0.5
    mv["translation"][0] = [2, dy, -3.5]
    mv["rotation"][0] = np.eye(3).reshape(9)
    codes, _ = pk.replay(mv)
    assert (codes[0] & 3) == expect
    p, _, _ = pk.state()
    want = pos.copy()
    if not expect:
        want[2] = [4.5, 4.95, 0.5]
    assert p == pytest.approx(want, abs=1e-9)
