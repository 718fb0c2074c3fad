"""Orientation renormalisation (Packing::renormalizeOrientations, core/Packing.cpp:1178-1240):
the oracle against the reference compiled here (CPU), and the engine against the oracle
(GPU): rejected counts and FP64 states bit-exact, followed by a logged sweep that must
replay identically (it depends on the polysphere centres the pass recomputes)."""
import numpy as np
import pytest

import pyoracle as po
import systems


def perturbed(cfg, noise, seed=3, factor=1.0):
    kind, prm, pos, rot, box = systems.compressed(cfg, factor) if factor != 1.0 else cfg
    rng = np.random.default_rng(seed)
    rot = rot + rng.normal(0.0, noise, rot.shape)
    return kind, prm, pos, np.ascontiguousarray(rot), box


# (system, orientation noise, box factor): orientations off orthonormal by up to 1e-7 (the
# engine takes rotations to within 1e-6); compressed systems hold overlaps, so some fixes
# are rejected and the serial remainder of the pass runs
CASES = [("sc_l2_dense", 1e-9, 1.0), ("sc_l2_dense", 1e-7, 0.99), ("sc_l5", 1e-7, 0.995), ("hs_dense", 1e-7, 0.98),
         ("poly_dense", 1e-9, 1.0), ("poly_dense", 1e-7, 0.995), ("poly_banana", 1e-7, 0.99),
         ("psc_bent", 1e-7, 0.995), ("psc_bent", 1e-9, 1.0)]


@pytest.mark.parametrize("name,noise,factor", CASES)
@pytest.mark.parametrize("allow", [False, True])
def test_oracle_matches_reference(oracle, name, noise, factor, allow):
    if not po.reference_available():
        pytest.skip("reference library not built here")
    cfg = perturbed(systems.ALL[name](), noise, factor=factor)
    kind, prm, pos, rot, box = cfg
    a = po.CpuPacking("oracle", kind, prm, pos, rot, box)
    b = po.CpuPacking("reference", kind, prm, pos, rot, box)
    assert a.renormalize_orientations(allow) == b.renormalize_orientations(allow)
    sa, sb = a.state(), b.state()
    assert np.array_equal(sa[0], sb[0]) and np.array_equal(sa[1], sb[1])
    assert a.count_overlaps(False) == b.count_overlaps(False)


@pytest.mark.gpu
@pytest.mark.parametrize("name,noise,factor", CASES)
@pytest.mark.parametrize("allow", [False, True])
def test_engine_matches_oracle(oracle, engine, name, noise, factor, allow):
    from rampack_gb300.packing import GpuPacking
    cfg = perturbed(systems.ALL[name](), noise, factor=factor)
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        want = cpu.renormalize_orientations(allow)
        assert g.renormalize_orientations(allow) == want
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
        # the moves after the pass depend on the recomputed polysphere centres
        t, r = (0.1, 0.0) if kind == 0 else (0.2, 0.2)
        g.sweep(t, r, seed=77, counter=0, log=True)
        moves, codes = g.sweep_log()
        _, _, bounds = g.grid()
        got, _ = cpu.replay(moves, bounds)
        assert np.array_equal(codes, got)
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)


@pytest.mark.gpu
def test_upload_refuses_non_rotations(engine):
    from rampack_gb300.packing import GpuPacking
    from rampack_gb300._lib import EngineError
    kind, prm, pos, rot, box = systems.sc_l2()
    bad = rot.copy()
    bad[5] *= 1.01  # one axis 1 % too long
    with pytest.raises(EngineError):
        GpuPacking(kind, prm, pos, bad, box)
