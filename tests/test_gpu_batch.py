"""Batched replicas (rp_batch_*): every replica's logged sweeps replay on the CPU oracle
with identical outcome codes and final FP64 states, box moves match the oracle's
tryScaling per replica, and other launch shapes (cell factor, warps per block) keep the
decisions exact."""
import numpy as np
import pytest

import pyoracle as po
import systems

pytestmark = pytest.mark.gpu

def sc2(counts, phi):
    from rampack_gb300 import workloads as W
    return systems.thermalise(W.spherocylinders(counts, phi, 2.0, 0.5, aspect=(1, 1, 3)), 5, translation_step=0.2,
                              rotation_step=0.2)


# replicas of one shape each (spherocylinders l=2 r=0.5; spheres r=0.5), of different sizes
SETS = {
    "spherocylinders": [systems.sc_l2, systems.sc_l2_dense, lambda: sc2((6, 6, 3), 0.3), lambda: sc2((8, 8, 4), 0.4)],
    "spheres": [systems.hs_small, systems.hs_dense, systems.hs_tiny],
}


def make_batch(builders, tuning=None):
    from rampack_gb300.packing import BatchPacking
    cfgs = [f() for f in builders]
    kind, prm = cfgs[0][0], cfgs[0][1]
    b = BatchPacking(kind, prm, [c[2:] for c in cfgs])
    if tuning:
        b.set_tuning(*tuning)
    cpus = [po.CpuPacking("oracle", c[0], c[1], c[2], c[3], c[4], threads=1) for c in cfgs]
    return b, cpus


@pytest.mark.parametrize("which", sorted(SETS))
@pytest.mark.parametrize("tuning", [None, (1.25, 2), (1.1, 8), "filter"])
def test_batch_sweeps_replay_on_oracle(oracle, engine, which, tuning):
    b, cpus = make_batch(SETS[which], None if tuning == "filter" else tuning)
    if tuning == "filter":
        b.set_staging_filter(2)
    t, r = (0.1, 0.0) if which == "spheres" else (0.2, 0.2)
    with b:
        for cycle in range(2):
            st = b.sweep(t, r, seed=2024, counter=cycle, log=True)
            for k, cpu in enumerate(cpus):
                moves, codes = b.sweep_log(k)
                assert st[k]["moves"] == len(moves) == (1 + (r > 0)) * b.sizes[k]
                _, _, bounds = b.grid(k)
                want, _ = cpu.replay(moves, bounds)
                assert np.array_equal(codes, want), f"replica {k} cycle {cycle}"
        for k, cpu in enumerate(cpus):
            gp, gr, gb = b.state(k)
            cp, cr, cb = cpu.state()
            assert np.array_equal(gp, cp) and np.array_equal(gr, cr) and np.array_equal(gb, cb)
            assert b.count_total_overlaps(k, True) == 0


@pytest.mark.parametrize("which", sorted(SETS))
def test_batch_box_moves(oracle, engine, which):
    b, cpus = make_batch(SETS[which])
    rng = np.random.default_rng(9)
    with b:
        for step in range(6):
            boxes, propose = [], []
            for k, cpu in enumerate(cpus):
                _, _, box = cpu.state()
                m = box.reshape(3, 3)
                f = [0.985, 1.01, 0.995, 1.0][(k + step) % 4]
                boxes.append((m * f + rng.uniform(-0.002, 0.002, (3, 3))).reshape(9))
                propose.append((k + step) % 3 != 2)
            dE = b.try_scaling(np.array(boxes), np.array(propose, dtype=np.uint8))
            revert = np.zeros(b.R, dtype=np.uint8)
            for k, cpu in enumerate(cpus):
                if not propose[k]:
                    assert dE[k] == 0
                    continue
                want = cpu.try_scaling(boxes[k])
                assert dE[k] == want, (k, step, dE[k], want)
                if want > 0:
                    cpu.revert_scaling()
                    revert[k] = 1
            b.revert_scaling(revert)
            b.sweep(0.1 if which == "spheres" else 0.2, 0.0 if which == "spheres" else 0.2, seed=5, counter=step,
                    log=True)
            for k, cpu in enumerate(cpus):
                moves, codes = b.sweep_log(k)
                _, _, bounds = b.grid(k)
                want, _ = cpu.replay(moves, bounds)
                assert np.array_equal(codes, want)
        for k, cpu in enumerate(cpus):
            gp, gr, gb = b.state(k)
            cp, cr, cb = cpu.state()
            assert np.array_equal(gp, cp) and np.array_equal(gr, cr) and np.array_equal(gb, cb)


def test_batch_replica_seeds(engine):
    from rampack_gb300 import packing
    assert packing.replica_seed(7, 0) == 7
    assert packing.replica_seed(7, 2) == (7 + 2 * 0x9E3779B97F4A7C15) % (1 << 64)


def test_batch_upload_all_and_states(oracle, engine):
    # every replica's state through one batched upload (rp_batch_upload_states) after some
    # oracle cycles, read back at once (rp_batch_download_states), then sweeps replayed
    from rampack_gb300.packing import BatchPacking, EngineError
    cfgs = [f() for f in SETS["spherocylinders"]]
    kind, prm = cfgs[0][0], cfgs[0][1]
    cpus = [po.CpuPacking("oracle", c[0], c[1], c[2], c[3], c[4], threads=1) for c in cfgs]
    for k, cpu in enumerate(cpus):
        po.run_cycles(cpu, 2, seed=40 + k, translation_step=0.2, rotation_step=0.2, box_kind=1, box_step=0.003,
                      pressure=2.0, temperature=1.0)
    st = [cpu.state() for cpu in cpus]
    pos = np.concatenate([s[0] for s in st])
    rot = np.concatenate([s[1] for s in st])
    boxes = np.stack([s[2] for s in st])
    with BatchPacking(kind, prm, [c[2:] for c in cfgs]) as b:
        b.upload_all(pos, rot, boxes)
        gp, gr, gb = b.states()
        assert np.array_equal(gp, pos) and np.array_equal(gr, rot) and np.array_equal(gb, boxes)
        for k in range(b.R):
            assert b.count_total_overlaps(k) == 0
        for cycle in range(2):
            b.sweep(0.2, 0.2, seed=17, counter=cycle, log=True)
            for k, cpu in enumerate(cpus):
                moves, codes = b.sweep_log(k)
                _, _, bounds = b.grid(k)
                want, _ = cpu.replay(moves, bounds)
                assert np.array_equal(codes, want)
        gp, gr, gb = b.states()
        off = 0
        for k, cpu in enumerate(cpus):
            cp, cr, cb = cpu.state()
            n = len(cp)
            assert np.array_equal(gp[off:off + n], cp) and np.array_equal(gr[off:off + n], cr)
            assert np.array_equal(gb[k], cb)
            off += n
        # a particle outside its box is refused (the rebuild clamps its cell and sets a status)
        bad = pos.copy()
        bad[sum(b.sizes[:2]) + 3] += boxes[2].reshape(3, 3)[:, 0] * 1.5
        with pytest.raises(EngineError, match="outside"):
            b.upload_all(bad, rot, boxes)
        b.upload_all(pos, rot, boxes)
        assert b.count_total_overlaps(1) == 0


def test_batch_rototranslation_sweeps_replay_on_oracle(oracle, engine):
    b, cpus = make_batch(SETS["spherocylinders"])
    with b:
        for cycle in range(2):
            st = b.sweep(0.2, 0.3, seed=404, counter=cycle, log=True, rototranslation=True)
            for k, cpu in enumerate(cpus):
                moves, codes = b.sweep_log(k)
                assert st[k]["moves"] == len(moves) == b.sizes[k] and np.all(moves["type"] == 2)
                _, _, bounds = b.grid(k)
                want, _ = cpu.replay(moves, bounds)
                assert np.array_equal(codes, want)
        for k, cpu in enumerate(cpus):
            gp, gr, gb = b.state(k)
            cp, cr, cb = cpu.state()
            assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
