"""The nematic-order restatement (oracle/observables.py) pinned to the reference's own
NematicOrder (core/observables/NematicOrder.cpp:9-56).

tests/golden/nematic.npz holds five orientation sets of spherocylinders (aligned along z,
isotropic, near-aligned, nematic along a tilted director, a thermalised packing) with the Q
tensor and P2 that the reference's NematicOrder computed for them
(tests/golden/make_golden.py nematic).  The restatement must reproduce them to 1e-14; where
the reference library is built here, it is also compared live on fresh orientation sets.
"""
import os

import numpy as np
import pytest

from oracle import observables as obs

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture():
    return np.load(os.path.join(HERE, "golden", "nematic.npz"))


def test_restatement_matches_reference_fixture():
    z = fixture()
    assert len(z["names"]) == 5
    for name in z["names"]:
        q, p2 = obs.nematic_order(z[f"{name}_rot"])
        np.testing.assert_allclose(q, z[f"{name}_q"], rtol=0, atol=1e-14, err_msg=str(name))
        assert abs(p2 - float(z[f"{name}_p2"][0])) <= 1e-14, name


def test_restatement_matches_reference_live(oracle):
    import pyoracle as po
    if not po.reference_available():
        pytest.skip("reference library not built (no reference checkout)")
    rng = np.random.default_rng(99)
    for n, spread in [(64, 3.2), (777, 0.5), (2000, 0.05)]:
        rot = []
        for _ in range(n):
            ax = rng.normal(size=3)
            ax /= np.linalg.norm(ax)
            rot.append(po.rotation("reference", ax, float(rng.uniform(-spread, spread))))
        rot = np.array(rot)
        pk = po.CpuPacking("reference", po.SPHEROCYLINDER, np.array([2.0, 0.5]), np.zeros((n, 3)), rot,
                           np.eye(3).reshape(9) * 50.0)
        qr, p2r = pk.nematic_order()
        pk.close()
        q, p2 = obs.nematic_order(rot)
        np.testing.assert_allclose(q, qr, rtol=0, atol=1e-14)
        assert abs(p2 - p2r) <= 1e-14
