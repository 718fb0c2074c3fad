"""Generic convex bodies (GenericXenoCollideTraits) in the oracle, pinned to the reference.

The oracle restates XCBodyBuilder, the XenoCollide geometries and the portal refinement
(oracle/rpo_xc.hpp); the reference's own classes are compiled in place (oracle/_ref).  For
bodies covering every primitive and operation, random pairs around contact (between the
insphere and circumsphere distances, random orientations) must get identical decisions, and
packings of them must count overlaps, replay move streams and run the cycle loop identically.
Skipped where the reference library is not built (the GPU machine); tests/golden/convex.npz
carries the same pin there.
"""
import numpy as np
import pytest

import pyoracle as po

from convex_bodies import BODIES, lattice, random_pairs


@pytest.mark.parametrize("name", sorted(BODIES))
def test_pair_decisions_match_the_reference(oracle, name):
    if not po.reference_available():
        pytest.skip("reference library not built here")
    script = BODIES[name]
    p1, r1, p2, r2 = random_pairs(np.random.default_rng(11), 7500)
    hits = 0
    for k in range(len(p1)):
        a = po.convex_overlap("oracle", script, p1[k], r1[k], p2[k], r2[k])
        b = po.convex_overlap("reference", script, p1[k], r1[k], p2[k], r2[k])
        assert a == b, (name, k, p2[k], r1[k], r2[k])
        hits += a
    assert 0 < hits < len(p1), (name, hits)


def test_invalid_scripts_fail_in_both(oracle):
    if not po.reference_available():
        pytest.skip("reference library not built here")
    for bad in ("sphere -1", "cuboid 1 2", "sum", "sphere 1; sphere 1", "blob 1", ""):
        with pytest.raises(ValueError):
            po.convex_overlap("oracle", bad, np.zeros(3), np.eye(3), np.ones(3), np.eye(3))
        with pytest.raises(ValueError):
            po.convex_overlap("reference", bad, np.zeros(3), np.eye(3), np.ones(3), np.eye(3))


# lattice spacings just above twice the circumsphere radius: no overlaps at the start (the cycle
# loop requires none), contacts after a few moves
PACKINGS = {"cuboid": 3.76, "cone": 2.02, "capsule_wrap": 2.22, "rotated_sum": 2.76}


@pytest.mark.parametrize("name", sorted(PACKINGS))
def test_packings_match_the_reference(oracle, name):
    """Counts, a replayed serial move stream and an NpT cycle-loop run: identical codes, counts
    and final states."""
    if not po.reference_available():
        pytest.skip("reference library not built here")
    script = BODIES[name]
    pos, rot, box = lattice(6, PACKINGS[name])
    out = {}
    for which in ("oracle", "reference"):
        pk = po.CpuPacking(which, po.CONVEX, script, pos, rot, box, threads=1)
        c0 = pk.count_overlaps(False)
        rng = po.CpuPacking("oracle", po.CONVEX, script, pos, rot, box, threads=1)
        g = rng.rng(3)
        moves = rng.draw_moves(g, 0.3, 0.3, np.arange(rng.n), rng.n, 2 * rng.n, domain=-1)
        rng.rng_free(g)
        rng.close()
        codes, _ = pk.replay(moves, None)
        c1 = pk.count_overlaps(False)
        st = po.run_cycles(pk, 20, translation_step=0.2, rotation_step=0.2, box_kind=1, box_step=0.01,
                           pressure=2.0, temperature=1.0, seed=9)
        p, r, b = pk.state()
        out[which] = (c0, codes, c1, (st.moves[0], st.accepted[0], st.moves[1], st.accepted[1], st.scalings,
                                      st.scalings_accepted), p, r, b)
        pk.close()
    a, b = out["oracle"], out["reference"]
    assert a[0] == b[0] and a[2] == b[2]
    assert np.array_equal(a[1], b[1])
    assert 0 < np.count_nonzero(a[1] & 0x80) < len(a[1])
    assert a[3] == b[3]
    for x, y in zip(a[4:], b[4:]):
        assert np.array_equal(x, y)


def test_oracle_matches_the_golden_fixture(oracle):
    """The restatement against the reference's decisions recorded in tests/golden/convex.npz
    (runs where the reference is absent too)."""
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "convex.npz"))
    for name in z["names"]:
        script = BODIES[str(name)]
        r1, p2, r2, want = z[f"{name}_r1"], z[f"{name}_p2"], z[f"{name}_r2"], z[f"{name}_overlap"]
        got = [po.convex_overlap("oracle", script, np.zeros(3), r1[k], p2[k], r2[k]) for k in range(len(p2))]
        assert np.array_equal(np.array(got), want), name


def test_engine_builder_refuses_as_the_reference(oracle, engine):
    """The engine's host builder (rp_create_convex) refuses invalid scripts before touching a
    device, with the reference XCBodyBuilder's own messages."""
    if not po.reference_available():
        pytest.skip("reference library not built here")
    import ctypes as C
    lib = engine.load()
    for bad in ("sphere -1", "cuboid 1 2", "sum", "wrap 3", "sphere 1; sphere 1", "blob 1", "", "diff",
                "football 1 1", "saucer 1 3", "dup 2", "sphere 1; pop; pop", "segment 0", "ellipse 1 -2"):
        with pytest.raises(ValueError) as ref:
            po.convex_overlap("reference", bad, np.zeros(3), np.eye(3), np.ones(3), np.eye(3))
        h = C.c_void_p()
        rc = lib.rp_create_convex(bad.encode(), 10, 0, C.byref(h))
        assert rc == -1, (bad, rc)  # RP_ERR_ARG
        msg = lib.rp_last_error(None).decode()
        assert msg == "convex body: " + str(ref.value), (bad, msg, str(ref.value))


@pytest.mark.parametrize("name,factor", [("cuboid", 1.0), ("cuboid", 0.8), ("cone", 0.8)])
@pytest.mark.parametrize("allow", [False, True])
def test_orientation_fixes_match_the_reference(oracle, name, factor, allow):
    """Packing::renormalizeOrientations on convex bodies with orientations 1e-7 off orthonormal
    (compressed lattices hold overlaps, so some fixes are rejected)."""
    if not po.reference_available():
        pytest.skip("reference library not built here")
    from convex_bodies import CIRCUMSPHERE
    pos, rot, box = lattice(5, 2.02 * CIRCUMSPHERE[name])
    pos, box = pos * factor, np.asarray(box) * factor
    rot = rot + np.random.default_rng(2).normal(0.0, 1e-7, rot.shape)
    a = po.CpuPacking("oracle", po.CONVEX, BODIES[name], pos, rot, box)
    b = po.CpuPacking("reference", po.CONVEX, BODIES[name], pos, rot, box)
    assert a.renormalize_orientations(allow) == b.renormalize_orientations(allow)
    sa, sb = a.state(), b.state()
    assert np.array_equal(sa[0], sb[0]) and np.array_equal(sa[1], sb[1])


@pytest.mark.parametrize("name,mask", [("cuboid", 7), ("cone", 5), ("rotated_sum", 2)])
def test_walls_match_the_reference(oracle, name, mask):
    """Hard walls (XenoCollideTraits::overlapWithWall, core/shapes/XenoCollideTraits.h:170-186):
    a lattice pushed against the near walls (some bodies through them), its counts, a replayed
    move stream, the same stream in overlap-counting mode and a box move; then an NpT cycle-loop
    run from a lattice clear of the walls.  Identical codes, counts and FP64 states."""
    if not po.reference_available():
        pytest.skip("reference library not built here")
    from convex_bodies import CIRCUMSPHERE
    spacing = 2.02 * CIRCUMSPHERE[name]
    pos0, rot, box = lattice(5, spacing)
    pos = pos0 - 0.3 * spacing
    g = po.CpuPacking("oracle", po.CONVEX, BODIES[name], pos, rot, box, threads=1)
    r = g.rng(7)
    moves = g.draw_moves(r, 0.4, 0.4, np.arange(g.n), g.n, 3 * g.n, domain=-1)
    g.rng_free(r)
    g.close()
    out = {}
    for which in ("oracle", "reference"):
        pk = po.CpuPacking(which, po.CONVEX, BODIES[name], pos, rot, box, threads=1)
        pk.set_walls(mask)
        counts = (pk.count_overlaps(False), pk.count_overlaps(True))
        codes, _ = pk.replay(moves, None)
        st = pk.state()
        nb = np.asarray(box).reshape(9) * 0.99
        de = pk.try_scaling(nb)
        pk.close()
        c = po.CpuPacking(which, po.CONVEX, BODIES[name], pos, rot, box, threads=1)
        c.set_walls(mask)
        c.set_counting(True)
        c0 = c.cached_overlaps()
        ccodes, deltas = c.replay(moves, None)
        cfin = c.cached_overlaps()
        c.close()
        s = po.CpuPacking(which, po.CONVEX, BODIES[name], pos0, rot, box, threads=1)
        s.set_walls(mask)
        run = po.run_cycles(s, 15, translation_step=0.3, rotation_step=0.3, box_kind=1, box_step=0.01,
                            pressure=2.0, temperature=1.0, seed=4)
        out[which] = (counts, codes, st, de, c0, ccodes, deltas, cfin,
                      (run.moves[0], run.accepted[0], run.scalings, run.scalings_accepted), s.state())
        s.close()
    a, b = out["oracle"], out["reference"]
    assert a[0] == b[0] and a[0][0] > 0, (a[0], b[0])   # the shifted lattice meets the walls
    assert np.array_equal(a[1], b[1])
    for x, y in zip(a[2], b[2]):
        assert np.array_equal(x, y)
    assert a[3] == b[3]
    assert a[4] == b[4] and a[7] == b[7] and a[4] != a[7]
    assert np.array_equal(a[5], b[5]) and np.array_equal(a[6], b[6])
    assert a[8] == b[8]
    for x, y in zip(a[9], b[9]):
        assert np.array_equal(x, y)
