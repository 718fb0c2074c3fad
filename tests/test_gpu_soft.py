"""Soft interactions on the GPU (rp_set_soft) against the oracle.

A central potential on the interaction centres joined to the hard shape (CompoundInteraction,
core/interactions/CompoundInteraction.cpp:9-49), or alone, with the oracle pinned to the
reference's own classes (tests/test_soft_oracle.py).  The engine sums the pair energies in
another order than the reference's neighbour-grid walk, so energies agree to a relative
1e-12 of the sum of their magnitudes; every Metropolis decision and the final FP64 state must
be identical:

* single moves of the serial path (rp_try_move / rp_accept_move): energy classes, energies
  and accepts against the oracle's replay;
* device sweeps (every move in FP64, one warp per cell): a logged sweep replays move by move on
  the oracle with the logged uniforms;
* box moves: the change of the total energy (Packing::getTotalEnergy) and the overlap answer;
* overlap relaxation (counting mode with a soft helper), as casino runs it.
"""
import numpy as np
import pytest

import pyoracle as po
import systems
from rampack_gb300 import _lib

pytestmark = pytest.mark.gpu

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
RTOL = 1e-12


def make(name):
    from rampack_gb300.packing import GpuPacking
    sysname, factor, kind, eps, sigma, hard, counting = CASES[name]
    cfg = systems.ALL[sysname]()
    if factor != 1.0:
        cfg = systems.compressed(cfg, factor)
    cpu = po.CpuPacking("oracle", *cfg, threads=1)
    cpu.set_soft(kind, eps, sigma, hard)
    g = GpuPacking(*cfg)
    g.set_soft(kind, eps, sigma, hard)
    if counting:
        cpu.set_counting(True)
        g.set_counting(True)
    return cfg, cpu, g


def close(a, b, scale):
    return abs(a - b) <= RTOL * max(1.0, scale)


def same_state(g, cpu):
    gp, gr, gb = g.state()
    cp, cr, cb = cpu.state()
    return np.array_equal(gp, cp) and np.array_equal(gr, cr) and np.array_equal(gb, cb)


@pytest.mark.parametrize("name", sorted(CASES))
def test_soft_single_moves(oracle, engine, name):
    cfg, cpu, g = make(name)
    with g:
        e0 = cpu.total_energy()
        assert close(g.total_energy(), e0, abs(e0))
        t, r = (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)
        rng = cpu.rng(9)
        ntypes = (t > 0) + (r > 0)
        moves = cpu.draw_moves(rng, t, r, np.arange(cpu.n), cpu.n, ntypes * cpu.n, domain=-1)
        cpu.rng_free(rng)
        codes = np.zeros(len(moves), dtype=np.uint8)
        energies = np.zeros(len(moves))
        for i, m in enumerate(moves):
            de = g.try_move(int(m["particle"]), int(m["type"]), m["translation"], m["rotation"])
            energies[i] = de
            code = 0 if not np.isinf(de) else (1 if de > 0 else 3)
            if m["uniform"] <= np.exp(-de):
                g.accept_move()
                code |= _lib.CODE_ACCEPTED
            codes[i] = code
        want, _, wde = cpu.replay(moves, None, energies=True)
        assert np.array_equal(codes, want), np.count_nonzero(codes != want)
        fin = np.isfinite(wde)
        assert np.array_equal(np.isfinite(energies), fin)
        assert np.array_equal(energies[~fin], wde[~fin])
        assert np.all(np.abs(energies[fin] - wde[fin]) <= RTOL * np.maximum(1.0, np.abs(wde[fin]) * 100))
        assert np.count_nonzero(wde[fin] != 0) > 0
        assert same_state(g, cpu)
        e1 = cpu.total_energy()
        assert close(g.total_energy(), e1, abs(e1))
        if CASES[name][6]:
            assert g.cached_overlaps() == cpu.cached_overlaps()
        # box moves: the total energy change
        _, _, b = cpu.state()
        for f in (1.002, 0.998):
            nb = np.asarray(b).reshape(9) * f
            dg, dc = g.try_scaling(nb), cpu.try_scaling(nb)
            assert (dg == dc) if np.isinf(dc) else close(dg, dc, abs(e1)), (f, dg, dc)
            g.revert_scaling()
            cpu.revert_scaling()


@pytest.mark.parametrize("name", sorted(CASES))
def test_soft_sweep_log_replays_on_oracle(oracle, engine, name):
    cfg, cpu, g = make(name)
    t, r = (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)
    with g:
        g.set_temperature(1.0)
        for cycle in range(3):
            st = g.sweep(t, r, seed=515, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds, temperature=1.0)
            assert np.array_equal(codes, want), np.count_nonzero(codes != want)
            assert 0 < st["accepted"] < st["moves"]
        assert same_state(g, cpu)
        if CASES[name][6]:
            assert g.cached_overlaps() == cpu.cached_overlaps()
        # an unchanged soft part again removes nothing; removing it restores the hard path
        g.set_soft(_lib.SOFT_NONE)
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False) or CASES[name][5] is False


def test_lennard_jones_is_refused(engine):
    from rampack_gb300.packing import GpuPacking
    from rampack_gb300._lib import EngineError
    cfg = systems.ALL["hs_small"]()
    with GpuPacking(*cfg) as g:
        with pytest.raises(EngineError):
            g.set_soft(_lib.SOFT_LENNARD_JONES, 1.0, 1.0)
