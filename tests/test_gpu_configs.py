"""The benchmark's small hard-sphere configuration run as stated, on the GPU, against the oracle.

Hard spheres of diameter 1, N = 1000 started on a 10x10x10 simple-cubic lattice in a cubic
box at packing fraction 0.30, NpT at T = 1 and p* = 10, translation moves of step 0.1
(uniform in a cube) and isotropic volume moves with ln V uniform in +-0.01 (the reference's
AnisotropicVolumeScaler over a LogScalingFactorSampler on X & Y & Z, 0.01 / 3 per side),
10^4 cycles with fixed steps:

* the engine's native cycle loop (Simulation over a GpuPacking: device sweeps, reference
  box scaler with std::mt19937 draws, host Metropolis pre-check) and the oracle's cycle loop
  (the reference's Simulation restated, mt19937 proposals), six independent runs each, give
  mean number densities that agree within 3 combined standard errors of the run means;
* a logged device sweep of the equilibrated GPU state replays move by move on the oracle
  with identical outcome codes and final FP64 state, and a box move on it decides as the
  oracle's tryScaling.

The runs are seeded, so the outcome is deterministic.
"""
import math

import numpy as np
import pytest

import pyoracle as po
from oracle import observables as obs
from rampack_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PRESSURE, TRANSLATION, BOX_STEP = 10.0, 0.1, 0.01 / 3
SKIP, CYCLES, EVERY = 2000, 8000, 10  # 10^4 cycles; the density sampled every 10 after 2000
RUNS = 6                               # independent runs per implementation


def gpu_run(seed=1234):
    from rampack_gb300.packing import GpuPacking
    from rampack_gb300.simulation import Simulation, box_volume, log_volume
    kind, prm, pos, rot, box = W.config_hs_1000()
    rho = []
    g = GpuPacking(kind, prm, pos, rot, box)
    sim = Simulation(g, TRANSLATION, 0.0, seed=seed, scaler=log_volume(BOX_STEP))
    sim.set_conditions(1.0, PRESSURE)
    sim.run(SKIP)
    for _ in range(CYCLES // EVERY):
        st = sim.run(EVERY)
        rho.append(g.n / box_volume(st["box"]))
    st = sim.stats()
    sim.close()
    return g, rho, st


def oracle_run(seed):
    kind, prm, pos, rot, box = W.config_hs_1000()
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    kw = dict(translation_step=TRANSLATION, box_kind=2, box_step=BOX_STEP, pressure=PRESSURE, temperature=1.0)
    po.run_cycles(cpu, SKIP, seed=seed, **kw)
    rho = []
    for k in range(CYCLES // EVERY):
        po.run_cycles(cpu, EVERY, seed=seed * 100003 + k, **kw)
        p, _, b = cpu.state()
        rho.append(obs.number_density(len(p), b))
    cpu.close()
    return rho


def test_config_hs_1000_density_matches_the_oracle(oracle, engine):
    """The mean density of each run over its last 8000 cycles, for six independent runs of
    each implementation: the two ensembles of run means agree within 3 combined standard
    errors.  (With ln V steps of 0.01 the gas compresses slowly from phi = 0.30 under p* = 10:
    about 2 % of the box moves are accepted, so the runs are compared as wholes.)"""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(RUNS) as ex:  # the oracle's C calls release the GIL
        cpu_runs = list(ex.map(oracle_run, [7 + r for r in range(RUNS)]))
    gpu_means = []
    for r in range(RUNS):
        g, rho, st = gpu_run(1234 + r)
        try:
            assert st["cycles"] == SKIP + CYCLES
            assert st["box_moves"] == SKIP + CYCLES
            assert 0.002 < st["accepted_box_moves"] / st["box_moves"] < 0.5
            assert g.count_total_overlaps(False) == 0
        finally:
            g.close()
        gpu_means.append(float(np.mean(rho)))
    cpu_means = [float(np.mean(rho)) for rho in cpu_runs]
    mg, eg = obs.sem(gpu_means)
    mc, ec = obs.sem(cpu_means)
    rho0 = 1000 / np.linalg.det(np.asarray(W.config_hs_1000()[4]).reshape(3, 3))
    assert mg > rho0 and mc > rho0  # the pressure compresses the gas
    assert abs(mg - mc) <= 3 * math.hypot(eg, ec), (mg, eg, mc, ec, gpu_means, cpu_means)


def test_config_hs_1000_logged_sweep_replays_on_the_oracle(oracle, engine):
    g, _, st = gpu_run()
    try:
        p0, r0, b0 = g.state()
        cpu = po.CpuPacking("oracle", W.SPHERE, np.array([0.5]), p0, r0, b0)
        for cycle in range(3):
            g.sweep(TRANSLATION, 0.0, seed=4321, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want), np.count_nonzero(codes != want)
        gp, grot, gb = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(grot, cr)
        # a compressing box move on the swept state: the engine's decision is the oracle's
        for f in (0.999, 0.99):
            nb = np.asarray(gb, dtype=np.float64).reshape(9) * f
            de_g = g.try_scaling(nb)
            de_c = cpu.try_scaling(nb)
            assert de_g == de_c, (f, de_g, de_c)
            g.revert_scaling()
            cpu.revert_scaling()
    finally:
        g.close()


def test_config_bent_chains_learned_ordering(oracle, engine):
    """The learned-ordering configuration's bent chains as stated: N = 10^5 chains of 5 spheres
    (diameter 1, bond 0.6, 30 degrees between bonds) at packing fraction 0.45; the ranking
    network (13 features, 64 x 64 hidden, BF16 weights, FP32 accumulation) trained on the
    device on 10^7 pair outcomes the sweep itself logged; an ordered sweep leaves the state
    bit-identical to the plain sweep's, and its log replays on the oracle move by move."""
    from rampack_gb300 import _lib
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = W.config_banana_1e5()
    assert len(pos) == 100_000
    with GpuPacking(kind, prm, pos, rot, box) as g:
        for c in range(4):  # off the lattice
            g.sweep(0.2, 0.2, seed=1, counter=c, stats=False)
        start = g.state()
        g.pair_log_enable(10_000_000, 1)
        sweeps = 0
        while g.pair_log_count() < 10_000_000:
            g.sweep(0.2, 0.2, seed=2, counter=sweeps, stats=False)
            sweeps += 1
            assert sweeps <= 40
        feats, labels = g.pair_log()
        assert len(feats) == 10_000_000 and 0 < labels.mean() < 1
        _, l0 = g.mlp_gradient(feats[:200_000], labels[:200_000])
        g.mlp_train(epochs=2, batch=1024, lr=2e-3, seed=1)
        _, l1 = g.mlp_gradient(feats[:200_000], labels[:200_000])
        assert l1 < 0.8 * l0, (l0, l1)
        g.pair_log_enable(0)
        results = {}
        for mode in (_lib.ORDER_OFF, _lib.ORDER_MLP):
            g.upload(*start)
            g.set_ordering(mode, every=4)
            pairs = 0
            for c in range(3):
                st = g.sweep(0.2, 0.2, seed=3, counter=c)
                pairs += st["pair_tests"]
            results[mode] = (g.state(), pairs)
        (p0, r0, _), pairs0 = results[_lib.ORDER_OFF]
        (p1, r1, _), pairs1 = results[_lib.ORDER_MLP]
        assert np.array_equal(p0, p1) and np.array_equal(r0, r1)
        assert pairs1 < pairs0
        # an ordered, logged sweep replays on the oracle
        g.upload(*start)
        cpu = po.CpuPacking("oracle", kind, prm, *start, threads=8)
        g.set_ordering(_lib.ORDER_MLP, every=1)
        g.sweep(0.2, 0.2, seed=7, counter=0, log=True)
        moves, codes = g.sweep_log()
        _, _, bounds = g.grid()
        want, _ = cpu.replay(moves, bounds)
        assert np.array_equal(codes, want), np.count_nonzero(codes != want)
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
