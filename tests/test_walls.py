"""Hard walls (Packing::toggleWalls) in the oracle, against the reference's own outcomes
(tests/golden/walls.npz, make_golden.py walls): overlap counts, a replayed move list, a box
move, and the same moves in overlap-counting mode, bit for bit."""
import hashlib
import os

import numpy as np
import pytest

import pyoracle as po
import systems

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "walls.npz")
WALLS = [("hs_small", 1), ("sc_l2", 5), ("poly_banana", 2), ("sc_l2_dense", 7), ("psc_bent", 3)]


def digest(pos, rot):
    h = hashlib.sha256(np.ascontiguousarray(pos, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(rot, dtype=np.float64).tobytes())
    return np.frombuffer(h.digest(), dtype=np.uint8)


@pytest.mark.parametrize("i", range(len(WALLS)))
def test_oracle_walls_match_the_reference(oracle, i):
    z = np.load(GOLD)
    name, mask = WALLS[i]
    cfg = systems.ALL[name]()
    pk = po.CpuPacking("oracle", *cfg)
    pk.set_walls(mask)
    assert [pk.count_overlaps(False), pk.count_overlaps(True)] == list(z[f"w{i}_counts"])
    codes, _ = pk.replay(z[f"w{i}_moves"])
    assert np.array_equal(codes, z[f"w{i}_codes"])
    p, r, b = pk.state()
    assert np.array_equal(digest(p, r), z[f"w{i}_state"])
    nb = (b.reshape(3, 3) * 0.995).reshape(9)
    assert pk.try_scaling(nb) == float(z[f"w{i}_box_dE"])
    assert np.array_equal(digest(*pk.state()[:2]), z[f"w{i}_box_state"])
    if f"w{i}_count_codes" in z:
        c = po.CpuPacking("oracle", *cfg)
        c.set_walls(mask)
        c.set_counting(True)
        codes, deltas = c.replay(z[f"w{i}_moves"])
        assert np.array_equal(codes, z[f"w{i}_count_codes"]) and np.array_equal(deltas, z[f"w{i}_count_deltas"])
        assert c.cached_overlaps() == int(z[f"w{i}_count_final"])
