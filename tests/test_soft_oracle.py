"""The oracle's soft interactions pinned to the reference's own classes.

rampack joins a soft central interaction to a hard shape through CompoundShapeTraits /
CompoundInteraction (core/interactions/CompoundInteraction.cpp:9-49; casino's overlap
relaxation with a helper shape, frontend/modes/CasinoMode.cpp:288-289), or uses it alone
(SphereTraits(r, centralInteraction)).  The oracle restates the energy sums of
Packing::calculateParticleEnergy and getTotalEnergy (core/Packing.cpp:649-764) and the soft
branches of tryTranslation / tryScaling and Simulation::tryScaling.  Move streams replay on
the oracle and on the reference compiled here with identical outcome codes, identical move
energies (bit for bit: both sum in the neighbour grid's order) and identical final states;
total energies and cycle-loop runs with box moves agree bit for bit (one thread).
"""
import numpy as np
import pytest

import pyoracle as po
import systems

WCA, SIC = 1, 2

CASES = {
    # name: (system, compression, soft kind, epsilon, sigma, with the hard part, counting)
    "hs_core_sic": ("hs_dense", 1.0, SIC, 1.0, 1.3, True, False),
    "hs_wca_alone": ("hs_small", 1.0, WCA, 1.0, 1.0, False, False),
    "sc_wca": ("sc_l2", 1.0, WCA, 1.0, 1.2, True, False),
    "banana_sic": ("poly_banana", 1.0, SIC, 2.0, 1.1, True, False),
    "hs_relax_sic": ("hs_dense", 0.95, SIC, 1.0, 1.05, True, True),
    "banana_relax": ("poly_dense", 0.97, SIC, 0.5, 1.05, True, True),
}


def packings(name):
    sysname, factor, kind, eps, sigma, hard, counting = CASES[name]
    cfg = systems.ALL[sysname]()
    if factor != 1.0:
        cfg = systems.compressed(cfg, factor)
    out = []
    for which in ("oracle", "reference"):
        pk = po.CpuPacking(which, *cfg, threads=1)
        pk.set_soft(kind, eps, sigma, hard)
        if counting:
            pk.set_counting(True)
        out.append(pk)
    return cfg, out


@pytest.fixture(scope="module", autouse=True)
def need_reference(oracle):
    if not po.reference_available():
        pytest.skip("reference library not built (no reference checkout)")


@pytest.mark.parametrize("name", sorted(CASES))
def test_serial_moves_match_the_reference(name):
    cfg, (cpu, ref) = packings(name)
    assert cpu.total_energy() == ref.total_energy()
    t, r = (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)
    rng = cpu.rng(5)
    ntypes = (t > 0) + (r > 0)
    moves = cpu.draw_moves(rng, t, r, np.arange(cpu.n), cpu.n, ntypes * cpu.n, domain=-1)
    cpu.rng_free(rng)
    c1, d1, e1 = cpu.replay(moves, None, energies=True)
    c2, d2, e2 = ref.replay(moves, None, energies=True)
    assert np.array_equal(c1, c2) and np.array_equal(d1, d2)
    assert np.array_equal(e1, e2)
    finite = np.isfinite(e1)
    assert np.count_nonzero(finite & (e1 != 0)) > 0  # soft energy changes were evaluated
    p1, r1, b1 = cpu.state()
    p2, r2, b2 = ref.state()
    assert np.array_equal(p1, p2) and np.array_equal(r1, r2)
    assert cpu.total_energy() == ref.total_energy()
    # box moves: the total energy change (and the overlap answer)
    for f in (1.002, 0.998):
        nb = np.asarray(b1).reshape(9) * f
        assert cpu.try_scaling(nb) == ref.try_scaling(nb)
        cpu.revert_scaling()
        ref.revert_scaling()


@pytest.mark.parametrize("name", ["hs_core_sic", "sc_wca", "banana_sic"])
def test_cycle_loop_matches_the_reference(name):
    cfg, (cpu, ref) = packings(name)
    t, r = (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)
    kw = dict(translation_step=t, rotation_step=r, box_kind=2, box_step=0.002, pressure=2.0, temperature=1.0,
              seed=21)
    s1 = po.run_cycles(cpu, 6, **kw)
    s2 = po.run_cycles(ref, 6, **kw)
    p1, r1, b1 = cpu.state()
    p2, r2, b2 = ref.state()
    assert np.array_equal(p1, p2) and np.array_equal(r1, r2) and np.array_equal(b1, b2)
    assert s1.scalings_accepted == s2.scalings_accepted
