"""Box-move proposals of the engine's cycle loop (rp_box_proposals, the scalers of
rampack_gb300/csrc/rp_sim.cu) against the reference's own TriclinicBoxScaler family and
std::mt19937 draws (tests/golden/box_proposals.npz, make_golden.py box): bit for bit."""
import os

import numpy as np
import pytest

from rampack_gb300 import _lib
from rampack_gb300 import simulation as S

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "box_proposals.npz")


def scalers():
    z = np.load(GOLD)
    i = 0
    while f"s{i}_spec" in z:
        yield i, z
        i += 1


@pytest.mark.parametrize("i", range(9))
def test_box_proposals_match_the_reference(engine, i):
    z = np.load(GOLD)
    kind, tog, ind, g0, g1, g2, ng = [int(v) for v in z[f"s{i}_spec"]]
    d = _lib.BoxScalerDesc(kind=kind, scale_together=tog, num_groups=ng, independent=ind, step=float(z[f"s{i}_step"]))
    for k, g in enumerate((g0, g1, g2)):
        d.groups[k] = g
    boxes, u = S.box_proposals(d, 1234 + i, z["box"], len(z[f"s{i}_uniforms"]))
    assert np.array_equal(boxes.view(np.uint64), z[f"s{i}_boxes"].view(np.uint64))
    assert np.array_equal(u, z[f"s{i}_uniforms"])


def test_scaler_builders(engine):
    d = S.log_volume(0.01, ("xy", "z"), independent=True)
    assert d.kind == _lib.SCALER_LOG and d.num_groups == 2 and list(d.groups)[:2] == [3, 4] and d.independent == 1
    assert S.delta_triclinic(0.005).scale_together == 1
    with pytest.raises(Exception):
        S.box_proposals(_lib.BoxScalerDesc(kind=2, num_groups=0, step=0.1), 1, np.eye(3).reshape(9), 3)


def test_quantity_matches_the_reference_formula():
    # Quantity::calculateFromSamples (utils/Quantity.cpp:45-61), sums in std::accumulate order
    x = [0.1, 0.7, 0.2, 1e-3, 3.3]
    m, e = S.quantity(x)
    acc = 0.0
    for v in x:
        acc += v
    mean = acc / len(x)
    sq = 0.0
    for v in x:
        sq += (mean - v) ** 2
    assert m == mean and e == np.sqrt(sq / len(x) / (len(x) - 1))
    assert S.quantity([]) == (0.0, 0.0) and S.quantity([5.0]) == (5.0, 0.0)


def test_observable_formulas(oracle):
    # N / V and the shapes' volumes as the reference computes them: V from its box, the
    # volumes from SphereTraits / SpherocylinderTraits (checked against the reference's own
    # box volume through the oracle library's reference build when it is present)
    import math
    from rampack_gb300 import _lib
    box = np.array([10.0, 0.3, -0.2, 0.1, 11.0, 0.05, -0.0, -0.4, 12.5])
    m = box.reshape(3, 3)
    assert math.isclose(S.box_volume(box), abs(np.linalg.det(m)), rel_tol=1e-14)
    assert S.shape_volume(_lib.SHAPE_SPHERE, [0.5]) == 4. / 3 * math.pi * math.pow(0.5, 3)
    assert S.shape_volume(_lib.SHAPE_SPHEROCYLINDER, [2.0, 0.5]) == math.pi * 0.5 * 0.5 * 2.0 + 4. / 3 * math.pi * 0.125
    if oracle.reference_available():
        _, _, v = oracle.box_info("reference", box)
        assert S.box_volume(box) == v
