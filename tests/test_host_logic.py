"""Host-side logic that needs no GPU: workloads, the benchmark's helpers and the
multi-rank reduction (two gloo ranks on CPU)."""
import math
import os
import socket

import numpy as np
import pytest

from rampack_gb300 import workloads as W


def test_workload_packing_fraction():
    kind, prm, pos, rot, box = W.config_sc_1e6()
    assert len(pos) == 1_000_000 and kind == W.SPHEROCYLINDER
    vol = abs(np.linalg.det(box.reshape(3, 3)))
    assert len(pos) * W.spherocylinder_volume(2.0, 0.5) / vol == pytest.approx(0.50)
    kind, prm, pos, rot, box = W.config_hs_1000()
    assert len(pos) == 1000 and box[0] == pytest.approx((1000 * math.pi / 6 / 0.30) ** (1 / 3))
    rel = pos @ np.linalg.inv(box.reshape(3, 3)).T
    assert rel.min() > 0 and rel.max() < 1


def test_cpu_domains():
    import bench
    assert bench.cpu_domains(8) == (2, 2, 2)
    assert bench.cpu_domains(16) == (2, 2, 4)
    assert bench.cpu_domains(1) == (1, 1, 1)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    v = bench.reduce_max(10.0 * (rank + 1), dist)
    dist.barrier()
    out.put((rank, v))
    dist.destroy_process_group()


def test_reduce_max_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert sorted(res) == [(0, 20.0), (1, 20.0)]


def test_banana_centres_match_the_reference(oracle):
    # the workload builder restates PolysphereBananaTraits::generateGeometry; pinned
    # against the reference's own generator where the reference is built
    import math
    import pyoracle as po
    from rampack_gb300 import workloads as W
    if not po.reference_available():
        pytest.skip("reference library not built here")
    for arc_r, arc_a, n in [(0.6 / (2 * math.sin(math.radians(15))), math.radians(120), 5), (2.0, math.radians(200), 7),
                            (1.0, math.radians(60), 2)]:
        mine = W.banana_centres(arc_r, arc_a, n)
        ref = po.banana_centres(arc_r, arc_a, n, 0.5)
        assert np.array_equal(mine, ref[:, :3])
