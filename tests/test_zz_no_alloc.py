"""The allocation-free overlap count, rp_count_overlaps_static, against rp_count_overlaps.

rp_count_overlaps_static serves callers that may not allocate device memory (a framework
that pools all of it, or a pipeline where cudaMalloc would synchronise the device): it
reads positions and orientations from the caller's device buffers and works out of one
fixed scratch array inside the library.  The caller's buffers here come from torch.  Two
calls in a row must give the same counts as the allocating entry point (exact integers).
This file is collected last so that it also runs after every other test in one process.
"""
import ctypes as C

import numpy as np
import pytest

import systems
from rampack_gb300 import _lib

pytestmark = pytest.mark.gpu


def static_count(lib, cfg, early: bool, stream=None) -> int:
    import torch
    kind, prm, pos, rot, box = cfg
    desc = _lib.ShapeDesc()
    desc.kind = kind
    if kind == _lib.SHAPE_SPHERE:
        desc.radius = float(prm[0])
    else:
        desc.length, desc.radius = float(prm[0]), float(prm[1])
    d_pos = torch.from_numpy(np.ascontiguousarray(pos, dtype=np.float64)).cuda()
    d_rot = torch.from_numpy(np.ascontiguousarray(rot, dtype=np.float64).reshape(-1, 9)).cuda()
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    torch.cuda.synchronize()
    out = C.c_int64(-1)
    rc = lib.rp_count_overlaps_static(C.byref(desc), len(pos), C.c_void_p(d_pos.data_ptr()),
                                      C.c_void_p(d_rot.data_ptr()), _lib.dptr(b), 1 if early else 0,
                                      C.c_void_p(stream), C.byref(out))
    assert rc == 0, f"rp_count_overlaps_static returned {rc}"
    return int(out.value)


@pytest.mark.parametrize("name,factor", [("sc_l2", 1.0), ("sc_l2", 0.97), ("hs_dense", 0.97), ("sc_l5", 0.9)])
def test_static_count_matches_allocating_entry_point(engine, name, factor):
    from rampack_gb300.packing import GpuPacking
    lib = _lib.load()
    cfg = systems.ALL[name]()
    if factor != 1.0:
        cfg = systems.compressed(cfg, factor)
    kind, prm, pos, rot, box = cfg
    with GpuPacking(kind, prm, pos, rot, box) as g:
        want_full = g.count_total_overlaps(False)
        want_early = g.count_total_overlaps(True)
    for _ in range(2):  # two calls in a row share (and must clear) the scratch array
        assert static_count(lib, cfg, False) == want_full
        assert static_count(lib, cfg, True) == want_early


def test_static_count_rejects_oversize(engine):
    import torch
    lib = _lib.load()
    desc = _lib.ShapeDesc()
    desc.kind = _lib.SHAPE_SPHERE
    desc.radius = 0.5
    b = np.eye(3).reshape(9) * 100.0
    d_pos = torch.zeros(3, dtype=torch.float64, device="cuda")
    d_rot = torch.zeros(9, dtype=torch.float64, device="cuda")
    out = C.c_int64()
    # n above the limit is refused before any device memory is touched
    rc = lib.rp_count_overlaps_static(C.byref(desc), 65537, C.c_void_p(d_pos.data_ptr()),
                                      C.c_void_p(d_rot.data_ptr()), _lib.dptr(b), 0, None, C.byref(out))
    assert rc == -7  # RP_ERR_CAPACITY


def test_static_count_dilute_packing_gets_larger_cells(engine):
    """1000 spheres in a box of side 60: range-sized cells would number 216,000, above the
    scratch's 65,536; the count enlarges its cells and still equals the allocating count."""
    from rampack_gb300.packing import GpuPacking
    lib = _lib.load()
    rng = np.random.default_rng(1234)
    box = np.eye(3) * 60.0
    pos = rng.uniform(0.0, 60.0, size=(1000, 3))
    rot = np.tile(np.eye(3).reshape(9), (1000, 1))
    cfg = (_lib.SHAPE_SPHERE, (0.5,), pos, rot, box)
    with GpuPacking(*cfg) as g:
        want = g.count_total_overlaps(False)
    assert want > 0  # the random gas has overlapping pairs
    for _ in range(2):
        assert static_count(lib, cfg, False) == want
        assert static_count(lib, cfg, True) == 1


def test_static_count_refuses_host_pointers(engine):
    """Positions in host memory are refused with RP_ERR_ARG before any kernel runs."""
    import torch
    lib = _lib.load()
    desc = _lib.ShapeDesc()
    desc.kind = _lib.SHAPE_SPHERE
    desc.radius = 0.5
    b = np.eye(3).reshape(9) * 10.0
    h_pos = np.zeros((8, 3))
    d_rot = torch.zeros(8 * 9, dtype=torch.float64, device="cuda")
    out = C.c_int64(-1)
    rc = lib.rp_count_overlaps_static(C.byref(desc), 8, C.c_void_p(h_pos.ctypes.data), C.c_void_p(d_rot.data_ptr()),
                                      _lib.dptr(b), 0, None, C.byref(out))
    assert rc == -1  # RP_ERR_ARG
    assert out.value == -1
    # the library still works after the refusal
    cfg = systems.ALL["hs_dense"]()
    assert static_count(lib, cfg, False) >= 0
