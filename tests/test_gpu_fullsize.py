"""Parity at the benchmarked sizes: the bench workloads (10^6 spherocylinders, 10^5 bent
chains, 64,000 long spherocylinders) swept on the GPU with every move logged, the logs
replayed move by move on the CPU oracle (same outcome codes, same final FP64 state), a
box move compared with the oracle's tryScaling, and the FP32-filtered sweep compared with
the all-FP64 one (identical states)."""
import numpy as np
import pytest

import pyoracle as po

pytestmark = pytest.mark.gpu

WORKLOADS = ["sc_1e6", "banana_1e5", "sc_64000", "bent_rods_1e5"]


def config(name):
    from rampack_gb300 import workloads as W
    return {"sc_1e6": W.config_sc_1e6, "banana_1e5": W.config_banana_1e5, "sc_64000": W.config_sc_64000,
            "bent_rods_1e5": W.config_bent_rods_1e5}[name]()


@pytest.mark.parametrize("name", WORKLOADS)
def test_full_size_sweep_replays_on_oracle(oracle, engine, name):
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = config(name)
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    with GpuPacking(kind, prm, pos, rot, box) as g:
        st = g.sweep(0.2, 0.2, seed=2026, counter=0, log=True)
        moves, codes = g.sweep_log()
        _, _, bounds = g.grid()
        assert st["moves"] == len(moves) == 2 * len(pos)
        want, _ = cpu.replay(moves, bounds)
        assert np.array_equal(codes, want), f"{np.count_nonzero(codes != want)} of {len(codes)} codes differ"
        gp, gr, gb = g.state()
        cp, cr, cb = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr) and np.array_equal(gb, cb)
        # a box move on the swept state: the recount decides as the oracle's tryScaling
        nb = (box.reshape(3, 3) * 0.999 + np.eye(3) * 0.001).reshape(9)
        assert g.try_scaling(nb) == cpu.try_scaling(nb)
        gp, _, gb = g.state()
        cp, _, cb = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gb, cb)
        assert g.count_total_overlaps(False) == cpu.count_overlaps(False)


def test_full_size_fp32_filter_equals_fp64(engine):
    # the FP32 filter with its FP64 guard band decides exactly as FP64 alone, at 10^6
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = config("sc_1e6")
    states = []
    for fp64_only in (False, True):
        with GpuPacking(kind, prm, pos, rot, box) as g:
            for c in range(3):
                g.sweep(0.2, 0.2, seed=5, counter=c, stats=False, fp64_only=fp64_only)
            states.append(g.state())
            assert g.count_total_overlaps(True) == 0
    assert all(np.array_equal(a, b) for a, b in zip(states[0], states[1]))


def test_replicas_64_sweeps_replay_on_oracle(oracle, engine):
    # the 64-replica workload (408,345 particles in two batches): one logged batched sweep,
    # every replica replayed on its own oracle packing
    from rampack_gb300 import workloads as W
    from rampack_gb300.packing import BatchPacking
    reps = W.config_replicas_64(1234)
    for kind in (W.SPHERE, W.SPHEROCYLINDER):
        idx = [i for i, r in enumerate(reps) if r[0] == kind]
        prm = reps[idx[0]][1]
        t, r = (0.2, 0.0) if kind == W.SPHERE else (0.2, 0.2)
        with BatchPacking(kind, prm, [reps[i][2:5] for i in idx]) as b:
            b.sweep(t, r, seed=77, counter=3, log=True)
            for k, i in enumerate(idx):
                cpu = po.CpuPacking("oracle", kind, prm, *reps[i][2:5], threads=1)
                moves, codes = b.sweep_log(k)
                _, _, bounds = b.grid(k)
                want, _ = cpu.replay(moves, bounds)
                assert np.array_equal(codes, want), (kind, k)
                gp, gr, _ = b.state(k)
                cp, cr, _ = cpu.state()
                assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
