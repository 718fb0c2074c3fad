"""Snapshot and trajectory files written from device state: Packing::store of a GPU
packing equals the oracle's RAMSNAP of its downloaded state byte for byte, restore puts the
same state back, and a RAMTRJ recorded asynchronously while the packing keeps sweeping holds
exactly the states at the recorded cycles."""
import numpy as np
import pytest

import snapshots as S
import systems
from test_gpu_parity import gpu_packing, steps

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["sc_l2", "hs_small", "poly_banana"])
def test_store_restore(engine, tmp_path, name):
    cfg = systems.ALL[name]()
    t, r = steps(cfg)
    with gpu_packing(cfg) as g:
        for c in range(3):
            g.sweep(t, r, seed=11, counter=c, stats=False)
        pos, rot, box = g.state()
        aux = {"cycles": "3", "note": "from the device"}
        f = tmp_path / "s.ramsnap"
        g.store(f, aux)
        assert f.read_bytes() == S.ramsnap_bytes(pos, rot, box, aux)
        g.sweep(t, r, seed=11, counter=3, stats=False)
        assert g.restore(f) == aux
        p2, r2, b2 = g.state()
        assert np.array_equal(p2, pos) and np.array_equal(r2, rot) and np.array_equal(b2, box)
        assert g.count_total_overlaps(False) == 0


@pytest.mark.parametrize("name", ["sc_l2", "poly_banana"])
def test_trajectory_recorded_while_sweeping(engine, tmp_path, name):
    from rampack_gb300.snapshots import RamtrjRecorder, read_ramtrj
    cfg = systems.ALL[name]()
    t, r = steps(cfg)
    f = tmp_path / "t.ramtrj"
    states = []
    with gpu_packing(cfg) as g:
        with RamtrjRecorder(f, g.n, 2) as rec:
            for c in range(1, 9):
                g.sweep(t, r, seed=5, counter=c, stats=False)
                if c % 2 == 0:
                    states.append(g.state())   # the state the record below must capture
                    rec.record(g, c)           # returns at once; the next sweeps run meanwhile
    data = f.read_bytes()
    assert data == S.ramtrj_bytes(states, 2)
    for k, (p, rt, b) in enumerate(states):
        p2, r2, b2 = read_ramtrj(f, k)
        assert np.array_equal(p2, p) and np.array_equal(b2, b)
        np.testing.assert_allclose(r2, rt, rtol=0, atol=1e-14)  # through the Euler angles


def test_store_large(engine, tmp_path):
    # N = 100,000 bent chains after sweeps: the file reads back bit for bit, and a sample of
    # its lines equals the oracle's formatting
    from rampack_gb300 import workloads as W
    from rampack_gb300.packing import GpuPacking
    from rampack_gb300.snapshots import read_ramsnap
    kind, prm, pos, rot, box = W.config_banana_1e5()
    with GpuPacking(kind, prm, pos, rot, box) as g:
        g.sweep(0.2, 0.2, seed=3, counter=0, stats=False)
        p, r, b = g.state()
        f = tmp_path / "big.ramsnap"
        g.store(f, {"n": str(g.n)})
    p2, r2, b2, aux = read_ramsnap(f)
    assert np.array_equal(p2, p) and np.array_equal(r2, r) and np.array_equal(b2, b) and aux == {"n": "100000"}
    lines = f.read_bytes().split(b"\n")
    sel = np.arange(0, len(p), 997)
    want = S.ramsnap_bytes(p[sel], r[sel], b).split(b"\n")[3:-1]
    assert [lines[4 + i] for i in sel] == want
