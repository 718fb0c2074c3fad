"""Ensemble parity of the device-driven sweep (Philox proposals, per-sweep rotation table).

Replay tests prove every logged decision; these check that the proposal distribution is
the reference's, through equilibrium averages:

* hard spheres r=0.5, N=50, V0=200, T=1, p=1 with delta-volume box moves: the mean number
  density must match the value the reference's own validation test expects, 0.398574
  (test/validation_tests/SimulationTest.cpp:91-111, Carnahan-Starling), within 3 sigma and
  with a relative error under 3 %, sampled as that test samples (100 samples, one every
  100 cycles after 5000 cycles);
* spherocylinders l=3 r=0.5 (N=108) under delta-volume box moves: number density and
  nematic order P2 of the GPU run agree with a run of the CPU oracle (the reference's
  algorithm, mt19937 proposals) within 3 combined sigma of block averages.

The runs are seeded, so the outcome is deterministic.
"""
import math

import numpy as np
import pytest

import pyoracle as po
from oracle import observables as obs
from rampack_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def gpu_npt(g, cycles, sample_every, skip, trans, rot, pressure, propose, seed, sample):
    rng = np.random.default_rng(seed)
    box = np.array(g.state()[2])
    out = []
    for c in range(skip + cycles):
        g.sweep(trans, rot, seed=seed, counter=c, stats=False)
        nb = propose(box, rng)
        v0, v1 = abs(np.linalg.det(box.reshape(3, 3))), abs(np.linalg.det(nb.reshape(3, 3)))
        expo = g.n * math.log(v1 / v0) - pressure * (v1 - v0)
        if rng.uniform() <= math.exp(min(expo, 700.0)):
            if g.try_scaling(nb) > 0:
                g.revert_scaling()
            else:
                box = nb
        if c >= skip and (c - skip) % sample_every == sample_every - 1:
            out.append(sample(g, box))
    return out


def delta_volume(step):
    # DeltaVolumeScaler (core/volume_scalers/DeltaVolumeScaler.cpp:10-19) through
    # TriclinicAdapter: every side times cbrt((V + dV) / V), dV uniform in +-step
    def propose(box, rng):
        v = abs(np.linalg.det(box.reshape(3, 3)))
        dv = (2 * rng.uniform() - 1) * step
        return box * np.cbrt((dv + v) / v)
    return propose


def log_isotropic(step):
    # AnisotropicVolumeScaler over LogScalingFactorSampler, all sides together
    def propose(box, rng):
        return box * math.exp(rng.uniform(-step, step))
    return propose


def test_hard_sphere_density_matches_the_reference_expectation(engine):
    from rampack_gb300.packing import GpuPacking
    side = 200.0 ** (1 / 3)
    pos = W.lattice((4, 4, 4), (side / 4, side / 4, side / 4))[:50]
    rot = W.aligned_rotations(50)
    with GpuPacking(W.SPHERE, np.array([0.5]), pos, rot, W.diag_box(side, side, side)) as g:
        rho = gpu_npt(g, 10000, 100, 5000, 0.4, 0.0, 1.0, delta_volume(1.0), 1234,
                      lambda g, box: obs.number_density(g.n, box))
    mean, err = obs.sem(rho)
    expected = 0.398574
    assert abs(mean - expected) <= 3 * err, (mean, err)
    assert err / mean < 0.03


def blocked(samples, block=10):
    """Means of consecutive blocks of samples (decorrelates slow volume fluctuations)."""
    x = np.asarray(samples, dtype=np.float64)
    n = len(x) // block
    return x[:n * block].reshape(n, block).mean(1)


def test_spherocylinder_ensemble_matches_the_oracle(oracle, engine):
    # the reference's spherocylinder validation system (l=3, r=0.5, T=1, p=0.5, translation
    # 0.5 + rotation 1, delta-volume box moves), with 108 instead of 50 particles so that the
    # box stays more than two interaction ranges high
    from rampack_gb300.packing import GpuPacking
    kind, prm = W.SPHEROCYLINDER, np.array([3.0, 0.5])
    pos = W.lattice((6, 6, 3), (2.0, 2.0, 4.2))
    rot = W.aligned_rotations(len(pos))
    box = W.diag_box(12.0, 12.0, 12.6)
    pressure, trans, rot_step, box_step = 0.5, 0.5, 1.0, 3.0
    skip, samples, every = 5000, 100, 100

    def heights_volume(b):
        m = b.reshape(3, 3)
        s = [m[:, k] for k in range(3)]
        v = abs(np.dot(np.cross(s[0], s[1]), s[2]))
        return np.prod([v / np.linalg.norm(np.cross(s[(k + 1) % 3], s[(k + 2) % 3])) for k in range(3)])

    def delta_volume_heights(box, rng):
        # DeltaVolumeScaler: the "volume" is the product of the box heights
        v = heights_volume(box)
        dv = (2 * rng.uniform() - 1) * box_step
        return box * np.cbrt((dv + v) / v)

    with GpuPacking(kind, prm, pos, rot, box) as g:
        gs = gpu_npt(g, samples * every, every, skip, trans, rot_step, pressure, delta_volume_heights, 99,
                     lambda g, box: (obs.number_density(g.n, box), g.nematic_order()[1]))

    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    kw = dict(translation_step=trans, rotation_step=rot_step, box_kind=3, box_step=box_step, pressure=pressure,
              temperature=1.0)
    po.run_cycles(cpu, skip, seed=7, **kw)
    cs = []
    for k in range(samples):
        po.run_cycles(cpu, every, seed=1000 + k, **kw)
        p, r, b = cpu.state()
        cs.append((obs.number_density(len(p), b), obs.nematic_order(r)[1]))

    for q, name in ((0, "density"), (1, "P2")):
        mg, eg = obs.sem(blocked([s[q] for s in gs]))
        mc, ec = obs.sem(blocked([s[q] for s in cs]))
        assert abs(mg - mc) <= 3 * math.hypot(eg, ec), (name, mg, eg, mc, ec)


@pytest.mark.parametrize("name", ["sc_l2", "poly_banana"])
def test_nematic_order_matches_the_restatement(engine, name):
    import systems
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = systems.ALL[name]()
    with GpuPacking(kind, prm, pos, rot, box) as g:
        q, p2 = g.nematic_order()
    qr, p2r = obs.nematic_order(rot)
    np.testing.assert_allclose(q, qr, rtol=0, atol=1e-12)
    assert abs(p2 - p2r) <= 1e-12


def test_nematic_order_matches_the_reference_fixture(engine):
    """rp_nematic_order on the orientation sets whose Q tensor and P2 the reference's own
    NematicOrder computed (tests/golden/nematic.npz), to 1e-12."""
    import os
    from rampack_gb300.packing import GpuPacking
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nematic.npz"))
    for name in z["names"]:
        rot = z[f"{name}_rot"]
        n = len(rot)
        # particles on a loose simple-cubic lattice, so that the packing is valid
        k = int(np.ceil(n ** (1 / 3)))
        idx = np.arange(n)
        pos = np.stack([idx % k, (idx // k) % k, idx // (k * k)], axis=1) * 4.0 + 2.0
        box = np.eye(3) * (4.0 * k)
        with GpuPacking(po.SPHEROCYLINDER, (2.0, 0.5), pos, rot, box) as g:
            q, p2 = g.nematic_order()
        np.testing.assert_allclose(q, z[f"{name}_q"], rtol=0, atol=1e-12, err_msg=str(name))
        assert abs(p2 - float(z[f"{name}_p2"][0])) <= 1e-12, name
