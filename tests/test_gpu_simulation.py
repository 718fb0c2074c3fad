"""The cycle loop (rp_sim_*, rampack_gb300.simulation): its step-size adaptation replays the
reference's rule cycle by cycle (oracle/adaptation.py), its NpT runs reproduce the
reference's own validation expectations (test/validation_tests/SimulationTest.cpp:49-100:
hard-sphere gases, thermalisation with step adaptation then 100 samples), and it records
trajectories and keeps overlap counts consistent."""
import math

import numpy as np
import pytest

import systems
from adaptation import Adaptation

pytestmark = pytest.mark.gpu


def heights(box):
    m = np.asarray(box).reshape(3, 3)
    s = [m[:, k] for k in range(3)]
    v = abs(np.dot(np.cross(s[0], s[1]), s[2]))
    return [v / np.linalg.norm(np.cross(s[(k + 1) % 3], s[(k + 2) % 3])) for k in range(3)]


@pytest.mark.parametrize("name,steps,scaler", [
    ("sc_l2", (1.5, 2.5), ("delta_triclinic", 0.05)),     # too large: steps shrink
    ("hs_small", (0.01, 0.01), ("log_volume", 1e-4)),      # too small: steps grow
    ("hs_tiny", (9.0, 0.5), ("delta_volume", 20.0)),       # translation above its implicit maximum
])
def test_step_adaptation_replays_the_reference_rule(engine, name, steps, scaler):
    from rampack_gb300 import simulation as S
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = systems.ALL[name]()
    with GpuPacking(kind, prm, pos, rot, box) as g:
        sc = getattr(S, scaler[0])(scaler[1])
        with S.Simulation(g, steps[0], steps[1], 99, sc) as sim:
            sim.set_conditions(1.0, 2.0)
            ref = Adaptation(g.n, steps[0], steps[1], scaler[1])
            last = sim.stats()
            changed = 0
            for c in range(400):
                box_before = last["box"]
                st = sim.run(1, adjust_steps=True)
                ref.ct.add(st["translations"] - last["translations"],
                           st["accepted_translations"] - last["accepted_translations"])
                ref.cr.add(st["rotations"] - last["rotations"], st["accepted_rotations"] - last["accepted_rotations"])
                ref.cb.add(st["box_moves"] - last["box_moves"], st["accepted_box_moves"] - last["accepted_box_moves"])
                before = (ref.t, ref.r, ref.b)
                ref.evaluate(min(heights(box_before)) / 2)
                changed += before != (ref.t, ref.r, ref.b)
                assert (st["translation_step"], st["rotation_step"], st["box_step"]) == (ref.t, ref.r, ref.b), c
                last = st
            assert changed >= 3
            assert st["cycles"] == 400 and st["box_moves"] == 400


def test_rototranslation_adaptation_replays_the_reference_rule(engine):
    # one RototranslationSampler: both steps shrink together, and grow with the translation's
    # factor (its rotation step follows the translation's increase)
    from rampack_gb300 import simulation as S
    from rampack_gb300.packing import GpuPacking
    for name, steps in (("sc_l2", (1.2, 1.5)), ("hs_small", (0.02, 0.05))):
        kind, prm, pos, rot, box = systems.ALL[name]()
        with GpuPacking(kind, prm, pos, rot, box) as g, \
                S.Simulation(g, steps[0], steps[1], 17, rototranslation=True) as sim:
            ref = Adaptation(g.n, steps[0], steps[1], 0.0, rototranslation=True)
            last = sim.stats()
            changed = 0
            for c in range(350):
                box_before = last["box"]
                st = sim.run(1, adjust_steps=True)
                assert st["translations"] == 0
                ref.cr.add(st["rotations"] - last["rotations"], st["accepted_rotations"] - last["accepted_rotations"])
                before = (ref.t, ref.r)
                ref.evaluate(min(heights(box_before)) / 2)
                changed += before != (ref.t, ref.r)
                assert (st["translation_step"], st["rotation_step"]) == (ref.t, ref.r), (name, c)
                last = st
            assert changed >= 2


def test_step_adaptation_stops_at_the_rotation_cap(engine):
    # spheres accept every rotation: the rotation step grows to pi and stays there
    from rampack_gb300 import simulation as S
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = systems.hs_small()
    with GpuPacking(kind, prm, pos, rot, box) as g, S.Simulation(g, 0.05, 3.0, 5) as sim:
        st = sim.run(300, adjust_steps=True)
    assert st["rotation_step"] == math.pi and st["box_moves"] == 0


def hs_gas(n, volume, radius):
    from rampack_gb300 import workloads as W
    side = volume ** (1 / 3)
    pos = W.lattice((4, 4, 4), (side / 4, side / 4, side / 4))[:n]
    return W.SPHERE, np.array([radius]), pos, W.aligned_rotations(n), W.diag_box(side, side, side)


@pytest.mark.parametrize("temperature,volume,radius,expected", [
    (10.0, 5000.0, 0.05, 0.0999791),   # dilute gas from too small steps (SimulationTest.cpp:49-75)
    (1.0, 200.0, 0.5, 0.398574),       # degenerate gas (SimulationTest.cpp:77-100)
])
def test_hard_sphere_gas_matches_the_reference_validation(engine, temperature, volume, radius, expected):
    from rampack_gb300 import simulation as S
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = hs_gas(50, volume, radius)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        with S.Simulation(g, 1.0, 0.1, 1234, S.delta_volume(1.0)) as sim:
            (avg, samples) = sim.integrate(temperature, 1.0, 5000, 10000, 100)
    mean, err = avg["number_density"]
    assert len(samples["number_density"]) == 100
    assert abs(mean - expected) <= 3 * err, (mean, err, expected)
    assert err / mean < 0.03


def test_rototranslation_ensemble_matches_separate_samplers(engine):
    # the same NpT state (spherocylinders l=3 r=0.5 at p=0.5, delta-volume box moves) sampled
    # with one RototranslationSampler and with translation + rotation samplers: number
    # density and nematic order agree within 3 combined sigma of block averages
    from rampack_gb300 import simulation as S
    from rampack_gb300 import workloads as W
    from rampack_gb300.packing import GpuPacking
    kind, prm = W.SPHEROCYLINDER, np.array([3.0, 0.5])
    pos = W.lattice((6, 6, 3), (2.0, 2.0, 4.2))
    out = []
    for rt, seed in ((True, 1234), (False, 4321)):
        with GpuPacking(kind, prm, pos, W.aligned_rotations(len(pos)), W.diag_box(12.0, 12.0, 12.6)) as g:
            with S.Simulation(g, 0.5, 1.0, seed, S.delta_volume(10.0), rototranslation=rt) as sim:
                _, samples = sim.integrate(1.0, 0.5, 5000, 20000, 100, observables=("number_density",
                                                                                     "nematic_order"))
        out.append(samples)

    def blocked(x, block=10):
        x = np.asarray(x)
        n = len(x) // block
        b = x[:n * block].reshape(n, block).mean(1)
        return b.mean(), b.std(ddof=1) / np.sqrt(n)

    for q in ("number_density", "nematic_order"):
        (m1, e1), (m2, e2) = blocked(out[0][q]), blocked(out[1][q])
        assert abs(m1 - m2) <= 3 * math.hypot(e1, e2), (q, m1, e1, m2, e2)


def test_integrate_records_a_trajectory(engine, tmp_path):
    from rampack_gb300 import simulation as S
    from rampack_gb300.packing import GpuPacking
    from rampack_gb300.snapshots import RamtrjRecorder, ramtrj_info, read_ramtrj
    kind, prm, pos, rot, box = systems.sc_l2()
    f = tmp_path / "t.ramtrj"
    with GpuPacking(kind, prm, pos, rot, box) as g, S.Simulation(g, 0.2, 0.2, 3, S.delta_triclinic(0.005)) as sim:
        with RamtrjRecorder(f, g.n, 10) as rec:
            avg, _ = sim.integrate(1.0, 1.5, 20, 50, 10, observables=("number_density", "nematic_order"),
                                   snapshot_every=10, recorder=rec)
        p, r, b = g.state()
    assert ramtrj_info(f)["snapshots"] == 5
    p2, r2, b2 = read_ramtrj(f, 4)
    assert np.array_equal(p2, p) and np.array_equal(b2, b)
    assert 0 < avg["nematic_order"][0] <= 1


def test_counting_mode_box_moves(engine):
    # overlap counting: box moves take the energy change first (Simulation::tryScaling's
    # counting branch); the cached count stays the recount
    from rampack_gb300 import simulation as S
    from rampack_gb300.packing import GpuPacking
    cfg = systems.compressed(systems.sc_l2(), 0.97)
    with GpuPacking(*cfg) as g:
        g.set_counting(True)
        before = g.cached_overlaps()
        with S.Simulation(g, 0.1, 0.1, 8, S.delta_triclinic(0.01)) as sim:
            sim.set_conditions(1.0, 1.0)
            st = sim.run(60)
        assert st["box_moves"] == 60
        assert g.cached_overlaps() == g.count_total_overlaps(False)
        assert g.cached_overlaps() < before


def test_store_and_continue(engine, tmp_path):
    # a run stored mid-way (RAMSNAP with "cycles" and "step.<sampler>.<step>" entries, as the
    # reference's FileSnapshotWriter writes them) continues in a fresh packing exactly as the
    # uninterrupted run: same state, steps and cycle count
    from rampack_gb300 import simulation as S
    from rampack_gb300.packing import GpuPacking
    from rampack_gb300.snapshots import read_ramsnap
    kind, prm, pos, rot, box = systems.sc_l2()
    f = tmp_path / "mid.ramsnap"
    with GpuPacking(kind, prm, pos, rot, box) as g, S.Simulation(g, 0.3, 0.3, 21, S.delta_triclinic(0.01)) as sim:
        sim.set_conditions(1.0, 1.5)
        sim.run(250, adjust_steps=True)
        aux = sim.store(f)
        sim.run(20, adjust_steps=True)
        end = g.state()
        end_stats = sim.stats()
    assert aux["cycles"] == "250" and set(aux) == {"cycles", "step.translation.translation",
                                                  "step.rotation.rotation", "step.scaling.scaling"}
    assert read_ramsnap(f)[3] == aux
    with GpuPacking(kind, prm, pos, rot, box) as g, S.Simulation(g, 0.3, 0.3, 21, S.delta_triclinic(0.01)) as sim:
        sim.set_conditions(1.0, 1.5)
        sim.restore(f)
        assert sim.stats()["translation_step"] == float(aux["step.translation.translation"])
        # the box moves' generator starts afresh in a continued run (the reference reseeds it too),
        # so the continued run is compared without box moves
    with GpuPacking(kind, prm, pos, rot, box) as g1, GpuPacking(kind, prm, pos, rot, box) as g2:
        s1 = S.Simulation(g1, 0.3, 0.3, 21)
        s1.run(30)
        s1.store(f)
        s1.run(10)
        s2 = S.Simulation(g2, 0.3, 0.3, 21)
        s2.restore(f)
        s2.run(10)
        assert s2.stats()["cycles"] == 40
        a, b = g1.state(), g2.state()
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
        s1.close()
        s2.close()
