"""The pair-correlation oracle (oracle/rpo_correlation.hpp) pinned to the reference:

* the known answers of the reference's own unit tests
  (test/unit_tests/core/observables/correlation/*Test.cpp), restated here with the mocked
  enumerators and functions replaced by direct consumePair calls;
* the golden fixtures made by the reference's own PairDensityCorrelation /
  PairAveragedCorrelation (tests/golden/correlation.npz), bit for bit;

and the host side of rampack_gb300.correlation (named points, signature names, output
formatting, descriptor checks of rp_correlation_create) without a GPU."""
import ctypes as C
import math
import os

import numpy as np
import pytest

import pyoracle as po
import systems
from correlation_cases import CORRELATIONS, NAMED_POINTS, POLY_AXES

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "correlation.npz")


def printed(x, y, count=None):
    from rampack_gb300.correlation import _cpp_format
    return "".join(f"{_cpp_format(a)} {_cpp_format(b)}" + ("" if count is None else f" {int(c)}") + "\n"
                   for a, b, c in zip(x, y, count if count is not None else x))


def test_pair_density_correlation_known_answer(oracle):
    # PairDensityCorrelationTest.cpp:19-66: bins [0, 2), [2, 4], four shapes, two snapshots
    c = po.OracleCorrelation(po.pair_desc(function=0, max_r=4.0, num_bins=2))
    for i, j, d in [(0, 0, 1.5), (0, 1, 2.5), (0, 2, 3.5), (1, 2, 5.5)]:
        c.consume(i, j, (d, 0, 0))
    c.renormalize([2.0 / e / 4 for e in (1, 2)])
    c.next_snapshot()
    for i, j, d in [(0, 1, 1.5), (1, 2, 2.3)]:
        c.consume(i, j, (d, 0, 0))
    c.renormalize([2.0 / e / 4 for e in (0.5, 0.25)])
    c.next_snapshot()
    x, y, _ = c.values()
    assert printed(x, y) == "1 0.5\n3 1.25\n"
    assert list(c.dividers()) == [0, 2, 4]


def test_pair_averaged_correlation_known_answer(oracle):
    # PairAveragedCorrelationTest.cpp:15-69: values 1, 2 | 3, 4 averaged per bin
    c = po.OracleCorrelation(po.pair_desc(function=1, max_r=4.0, num_bins=2))
    for i, j, d, v in [(0, 0, 1.5, 1), (0, 2, 1.8, 2), (1, 2, 5.5, 99)]:
        c.consume(i, j, (d, 0, 0), v)
    c.next_snapshot()
    for i, j, d, v in [(0, 1, 1.5, 3), (1, 2, 2.5, 4)]:
        c.consume(i, j, (d, 0, 0), v)
    c.next_snapshot()
    x, y, cnt = c.values()
    assert printed(x, y) == "1 2\n3 4\n"
    assert list(cnt) == [3, 1]


def pairs_map(desc, pos, box):
    rot = np.tile(np.eye(3).reshape(9), (len(pos), 1))
    ij, d = po.enumerate_pairs(desc, np.asarray(pos, dtype=np.float64), rot, np.asarray(box).reshape(9))
    out = {}
    for (i, j), v in zip(ij, d):
        assert (int(i), int(j)) not in out
        out[(int(i), int(j))] = v
    return out


def test_radial_enumerator_known_answer(oracle):
    # RadialEnumeratorTest.cpp:15-59
    box = np.diag([10.0, 10.0, 10.0])
    pos = [(1, 1, 1), (1, 3, 1), (9, 9, 9)]
    m = pairs_map(po.pair_desc(enumerator=0), pos, box)
    assert len(m) == 6
    for k in ((0, 0), (1, 1), (2, 2)):
        assert np.array_equal(m[k], [0, 0, 0])
    for k, v in {(0, 1): (0, 2, 0), (0, 2): (-2, -2, -2), (1, 2): (-2, -4, -2)}.items():
        assert np.allclose(m[k], v, atol=1e-12, rtol=0)
    rho = 3 / 1000.0
    got = po.expected_in_shells(po.pair_desc(enumerator=0), 3, box, [1, 2, 3])
    assert np.allclose(got, [4 / 3 * math.pi * 7 * rho, 4 / 3 * math.pi * 19 * rho])


def test_linear_enumerator_known_answer(oracle):
    # LinearEnumeratorTest.cpp:15-65: a sheared box, axis y
    box = np.array([[5.0, 5.0, 0.0], [0.0, 5.0, 0.0], [0.0, 0.0, 10.0]])
    pos = [(1.5, 0.5, 5), (3.5, 1.5, 5), (4.5, 1.5, 5), (6.5, 3.5, 5)]
    d = po.pair_desc(enumerator=1, linear_axis=1)
    m = pairs_map(d, pos, box)
    want = {(0, 0): (0, 0, 0), (0, 1): (0, 1, 0), (0, 2): (0, 1, 0), (0, 3): (0, -2, 0), (1, 1): (0, 0, 0),
            (1, 2): (0, 0, 0), (1, 3): (0, 2, 0), (2, 2): (0, 0, 0), (2, 3): (0, 2, 0), (3, 3): (0, 0, 0)}
    assert set(m) == set(want)
    for k, v in want.items():
        assert np.array_equal(m[k], v), k
    assert np.allclose(po.expected_in_shells(d, 4, box, [0.5, 1, 1.5]), [0.4, 0.4])


def test_layerwise_radial_enumerator_known_answer(oracle):
    # LayerwiseRadialEnumeratorTest.cpp:15-71: two skew layers joined through the boundary
    box = np.array([[12.0, 4.0, 0.0], [0.0, 8.0, 0.0], [0.0, 0.0, 10.0]])
    pos = [(2, 1, 5), (5, 1, 5), (6, 4, 5), (13, 4, 5), (4, 6, 5)]
    d = po.pair_desc(enumerator=2, miller=(1, -2, 0))
    m = pairs_map(d, pos, box)
    assert len(m) == 9
    t = np.array([7.0, 2.0]) / math.hypot(7, 2)
    t3 = np.array([t[0], t[1], 0.0])
    for k in ((0, 0), (1, 1), (2, 2), (3, 3), (4, 4)):
        assert np.array_equal(m[k], [0, 0, 0])
    for k, v in {(0, 1): (3, 0), (2, 3): (-5, 0), (2, 4): (-2, 2), (3, 4): (3, 2)}.items():
        assert np.allclose(m[k], np.dot(t, v) * t3, atol=1e-12, rtol=0), k
    area = 2 * (2 * math.sqrt(53)) * 10
    assert np.allclose(po.expected_in_shells(d, 5, box, [1, 2, 3]),
                       [5 * math.pi * 3 / area, 5 * math.pi * 5 / area])


def case_desc(case):
    from rampack_gb300.correlation import _normalized, named_point
    name, en, lax, mil, fn, ax, focal, max_r, nb = case
    cfg = systems.ALL[name]()
    kind, prm = cfg[0], cfg[1]
    prim, sec = ((0.0, 0.0, 1.0), (1.0, 0.0, 0.0))
    if kind == po.POLYSPHERE:
        prim, sec = _normalized(POLY_AXES[0]), _normalized(POLY_AXES[1])
    d = po.pair_desc(enumerator=en, linear_axis=lax, miller=mil, function=fn, axis=ax, num_bins=nb, max_r=max_r,
                     focal=named_point(kind, prm, focal), primary=prim, secondary=sec)
    return cfg, d


@pytest.mark.parametrize("i", range(len(CORRELATIONS)))
def test_oracle_matches_reference_fixture(oracle, i):
    z = np.load(GOLD)
    cfg, d = case_desc(CORRELATIONS[i])
    c = po.OracleCorrelation(d)
    c.add_snapshot(*cfg[2:5])
    c.add_snapshot(*systems.compressed(cfg, 0.97)[2:5])
    x, y, cnt = c.values()
    assert np.array_equal(x, z[f"c{i}_x"])
    assert np.array_equal(cnt, z[f"c{i}_count"])
    assert np.array_equal(y, z[f"c{i}_y"], equal_nan=True)


def test_named_points_match_the_reference():
    from rampack_gb300.correlation import named_point
    z = np.load(GOLD)
    for i, (name, point) in enumerate(NAMED_POINTS):
        cfg = systems.ALL[name]()
        assert np.array_equal(named_point(cfg[0], cfg[1], point), z[f"p{i}"]), (name, point)
    with pytest.raises(Exception):
        named_point(1, np.array([2.0, 0.5]), "s0")


def test_signature_names_and_output_format(engine):
    from rampack_gb300 import correlation as K
    assert K.PairDensityCorrelation(K.RadialEnumerator(), 4, 2).signature_name == "rho_r"
    assert K.PairDensityCorrelation(K.LinearEnumerator("y"), 4, 2).signature_name == "rho_y"
    assert K.PairDensityCorrelation(K.LayerwiseRadialEnumerator((1, 0, 0)), 4, 2).signature_name == "rho_lr"
    for f, name in ((K.S110Correlation(), "S110"), (K.S220Correlation(), "S220"), (K.S221Correlation(), "S221"),
                    (K.AxesAngle(), "theta")):
        assert K.PairAveragedCorrelation(K.RadialEnumerator(), f, 4, 2).signature_name == name + "_r"
    # std::ostream defaults: 6 significant digits, %g style
    assert [K._cpp_format(v) for v in (1.0, 0.5, 1.25, 1234567.0, 1e-7, 2.0 / 3)] == \
        ["1", "0.5", "1.25", "1.23457e+06", "1e-07", "0.666667"]
    # an observable without snapshots prints the empty histogram: bin middles and zeros
    obs = K.PairDensityCorrelation(K.RadialEnumerator(), 4.0, 2, print_count=True)
    assert obs.print() == "1 0 0\n3 0 0\n"
    with pytest.raises(Exception):
        K.LayerwiseRadialEnumerator((0, 0, 0))


def test_descriptor_checks_without_a_gpu(engine):
    # rp_correlation_create validates the description on the host, as the reference's
    # constructors do (Expects), and allocates nothing on a device
    from rampack_gb300 import _lib
    lib = _lib.load()

    def create(**kw):
        d = _lib.PairDesc()
        d.num_bins, d.max_r = 10, 2.0
        d.miller = (C.c_int32 * 3)(0, 0, 1)
        for k, v in kw.items():
            setattr(d, k, v)
        h = C.c_void_p()
        rc = lib.rp_correlation_create(C.byref(d), C.byref(h))
        if rc == 0:
            snaps, tested = C.c_int64(), C.c_int64()
            assert lib.rp_correlation_info(h, C.byref(snaps), C.byref(tested)) == 0 and snaps.value == 0
            x, y, c = np.zeros(10), np.zeros(10), np.zeros(10, dtype=np.uint64)
            assert lib.rp_correlation_values(h, _lib.dptr(x), _lib.dptr(y), c.ctypes.data_as(C.POINTER(C.c_uint64))) == 0
            assert np.allclose(x, 0.1 + 0.2 * np.arange(10)) and not y.any()
            assert lib.rp_correlation_destroy(h) == 0
        return rc

    assert create() == 0
    assert create(enumerator=2) == 0
    assert create(num_bins=0) == -1
    assert create(num_bins=_lib.CORR_MAX_BINS + 1) == -1
    assert create(max_r=0.0) == -1
    assert create(max_r=float("nan")) == -1
    assert create(enumerator=3) == -1
    assert create(function=5) == -1
    assert create(linear_axis=3) == -1
    assert create(enumerator=2, miller=(C.c_int32 * 3)(0, 0, 0)) == -1
