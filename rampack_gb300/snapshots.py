"""Snapshot (RAMSNAP) and trajectory (RAMTRJ) files of packings, through the C ABI.

The Python face of ``rp_ramsnap_*`` / ``rp_ramtrj_*`` (rampack_gb300/csrc/rp_io.cu), which
write and read the reference's formats byte for byte: ``Packing::store`` /
``Packing::restore`` (core/Packing.cpp:956-964, core/io/RamsnapWriter.cpp,
core/io/RamsnapReader.cpp) and ``RamtrjRecorder`` / ``RamtrjPlayer`` (core/io/Ramtrj*.cpp).
Errors raise ``EngineError`` with the reference's message (e.g. ``Broken RAMSNAP file:
dimensions``), as the reference raises ``RamsnapException`` / ``RamtrjException``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import EngineError, dptr


def _check(lib, rc: int):
    if rc != 0:
        msg = lib.rp_io_last_error()
        raise EngineError(rc, msg.decode() if msg else "")


def _aux_arrays(aux):
    items = list((aux or {}).items())
    keys = (C.c_char_p * max(1, len(items)))(*[str(k).encode() for k, _ in items])
    values = (C.c_char_p * max(1, len(items)))(*[str(v).encode() for _, v in items])
    return len(items), keys, values


def _path(path) -> bytes:
    return os.fsencode(path)


def write_ramsnap(path, pos, rot, box, aux=None) -> None:
    """RAMSNAP of a state held on the host (``pos`` [n, 3], ``rot`` [n, 9] row-major,
    ``box`` [9] row-major with the sides as columns); ``aux`` maps keys (no whitespace)
    to values."""
    lib = _lib.load()
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    rot = np.ascontiguousarray(rot, dtype=np.float64).reshape(-1, 9)
    box = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    if len(pos) != len(rot):
        raise ValueError("pos and rot differ in length")
    n, keys, values = _aux_arrays(aux)
    _check(lib, lib.rp_ramsnap_write_host(_path(path), len(pos), dptr(pos), dptr(rot), dptr(box), n, keys, values))


def read_ramsnap(path):
    """(pos [n, 3], rot [n, 9], box [9], aux dict) of a RAMSNAP file."""
    lib = _lib.load()
    snap = C.c_void_p()
    _check(lib, lib.rp_ramsnap_load(_path(path), C.byref(snap)))
    try:
        n, naux = C.c_int64(), C.c_int32()
        _check(lib, lib.rp_ramsnap_info(snap, C.byref(n), C.byref(naux)))
        pos, rot, box = np.zeros((n.value, 3)), np.zeros((n.value, 9)), np.zeros(9)
        _check(lib, lib.rp_ramsnap_get(snap, dptr(pos), dptr(rot), dptr(box)))
        aux = {}
        for i in range(naux.value):
            k, v = C.c_char_p(), C.c_char_p()
            _check(lib, lib.rp_ramsnap_aux(snap, i, C.byref(k), C.byref(v)))
            aux[k.value.decode()] = v.value.decode()
    finally:
        lib.rp_ramsnap_free(snap)
    return pos, rot, box, aux


class RamtrjRecorder:
    """A RAMTRJ trajectory being recorded (``RamtrjRecorder``): ``record(packing, cycle)``
    takes a ``GpuPacking``'s state in order with its moves and returns while the download,
    conversion and write go on; ``record_host`` takes host arrays."""

    def __init__(self, path, num_particles: int, cycle_step: int, append: bool = False):
        self.lib = _lib.load()
        self.h = C.c_void_p()
        _check(self.lib, self.lib.rp_ramtrj_open(_path(path), int(num_particles), int(cycle_step),
                                                 1 if append else 0, C.byref(self.h)))

    def record(self, packing, cycle: int) -> None:
        _check(self.lib, self.lib.rp_ramtrj_record(self.h, packing.h, int(cycle)))

    def record_host(self, pos, rot, box, cycle: int) -> None:
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        rot = np.ascontiguousarray(rot, dtype=np.float64).reshape(-1, 9)
        box = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        _check(self.lib, self.lib.rp_ramtrj_record_host(self.h, dptr(pos), dptr(rot), dptr(box), int(cycle)))

    def flush(self) -> None:
        _check(self.lib, self.lib.rp_ramtrj_flush(self.h))

    def snapshots(self) -> int:
        c = C.c_int64()
        _check(self.lib, self.lib.rp_ramtrj_snapshots(self.h, C.byref(c)))
        return int(c.value)

    def close(self) -> None:
        if getattr(self, "h", None):
            h, self.h = self.h, None
            _check(self.lib, self.lib.rp_ramtrj_close(h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ramtrj_info(path) -> dict:
    """Header of a well-formed RAMTRJ file."""
    lib = _lib.load()
    n, s, c, v = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
    _check(lib, lib.rp_ramtrj_info(_path(path), C.byref(n), C.byref(s), C.byref(c), C.byref(v)))
    return {"num_particles": n.value, "snapshots": s.value, "cycle_step": c.value,
            "version": (v.value >> 8, v.value & 0xff)}


def read_ramtrj(path, snapshot: int):
    """(pos, rot, box) of snapshot ``snapshot`` (from 0) of a RAMTRJ file, orientations
    rebuilt from the stored Euler angles."""
    lib = _lib.load()
    n = ramtrj_info(path)["num_particles"]
    pos, rot, box = np.zeros((n, 3)), np.zeros((n, 9)), np.zeros(9)
    _check(lib, lib.rp_ramtrj_read(_path(path), int(snapshot), dptr(pos), dptr(rot), dptr(box)))
    return pos, rot, box
