"""Python mirror of the reference's Packing interface (core/Packing.h:32-466) over the C ABI.

``GpuPacking`` holds one packing of spheres or spherocylinders in GPU memory.  Its
methods keep the reference's names and meaning where one exists:

* ``count_total_overlaps(early_exit)``  — Packing::countTotalOverlaps (core/Packing.cpp:519-559)
* ``try_scaling(box)`` / ``revert_scaling()`` — Packing::tryScaling / revertScaling
  (core/Packing.cpp:172-208, :363-371); ``try_scaling`` returns +inf on overlap, else 0
* ``run_moves(moves)`` — a list of Packing::tryTranslation / tryRotation / tryMove calls,
  each followed by the Metropolis test and acceptMove (core/Simulation.cpp:466-490)
* ``sweep(...)`` — one device-driven pass of domain-decomposed moves
  (core/Simulation.cpp:396-445)

Errors raise ``EngineError`` with the C status, as the reference raises
PreconditionException / ValidationException.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import (MOVE_DTYPE, EngineError, GridInfo, ShapeDesc, SweepParams, SweepStats, dptr, fptr)


def ring_colour(n: int, c: int) -> int:
    """Checkerboard colour of cell coordinate c on a ring of n cells (the engine's rule:
    one colour for n = 1, alternating for even n, c mod 3 for odd n with the last cell of a
    ring with n mod 3 = 1 taking colour 1)."""
    if n == 1:
        return 0
    if n % 2 == 0:
        return c & 1
    if n % 3 == 1 and c == n - 1:
        return 1
    return c % 3


def cell_phase(dims, cell: int) -> int:
    """The sweep phase of a cell: colours coded p0 + 3 p1 + 9 p2."""
    cx, cy, cz = cell % dims[0], (cell // dims[0]) % dims[1], cell // (dims[0] * dims[1])
    return ring_colour(dims[0], cx) + 3 * ring_colour(dims[1], cy) + 9 * ring_colour(dims[2], cz)


class GpuPacking:
    def __init__(self, kind: int, params, pos, rot, box, device: int = 0):
        self.lib = _lib.load()
        script = params if kind == _lib.SHAPE_CONVEX else None
        params = np.zeros(0) if script is not None else np.asarray(params, dtype=np.float64).reshape(-1)
        desc = ShapeDesc()
        desc.kind = kind
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.n = pos.shape[0]
        self.kind = kind
        self.params = params
        h = C.c_void_p()
        if kind == _lib.SHAPE_CONVEX:
            # a generic convex body: the XCBodyBuilder script
            self.script = str(script)
            rc = self.lib.rp_create_convex(self.script.encode(), self.n, device, C.byref(h))
            if rc != 0:
                raise EngineError(rc, "rp_create_convex failed: " + self.lib.rp_last_error(None).decode())
        elif kind == _lib.SHAPE_POLYSPHERE:
            # params as the oracle's: [k, (x, y, z, r) per centre]
            k = int(params[0])
            data = params[1:1 + 4 * k].reshape(k, 4)
            centres = np.ascontiguousarray(data[:, :3])
            radii = np.ascontiguousarray(data[:, 3])
            rc = self.lib.rp_create_polysphere(k, dptr(centres), dptr(radii), self.n, device, C.byref(h))
            if rc != 0:
                raise EngineError(rc, "rp_create_polysphere failed")
        elif kind == _lib.SHAPE_POLYSPHEROCYLINDER:
            # params as the oracle's: [k, (x, y, z, hx, hy, hz, r) per spherocylinder]
            k = int(params[0])
            data = params[1:1 + 7 * k].reshape(k, 7)
            centres = np.ascontiguousarray(data[:, :3])
            half_axes = np.ascontiguousarray(data[:, 3:6])
            radii = np.ascontiguousarray(data[:, 6])
            rc = self.lib.rp_create_polyspherocylinder(k, dptr(centres), dptr(half_axes), dptr(radii), self.n, device,
                                                       C.byref(h))
            if rc != 0:
                raise EngineError(rc, "rp_create_polyspherocylinder failed")
        else:
            if kind == _lib.SHAPE_SPHERE:
                desc.radius = float(params[0])
            elif kind == _lib.SHAPE_SPHEROCYLINDER:
                desc.length, desc.radius = float(params[0]), float(params[1])
            else:
                raise EngineError(-5, f"shape kind {kind} is not handled by the GPU engine")
            rc = self.lib.rp_create(C.byref(desc), self.n, device, C.byref(h))
            if rc != 0:
                raise EngineError(rc, "rp_create failed")
        self.h = h
        self.upload(pos, rot, box)

    # ---- plumbing ----
    def _check(self, rc: int):
        if rc != 0:
            msg = self.lib.rp_last_error(self.h)
            raise EngineError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.rp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- state ----
    def upload(self, pos, rot, box):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        rot = np.ascontiguousarray(rot, dtype=np.float64).reshape(-1, 9)
        box = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        if pos.shape[0] != self.n or rot.shape[0] != self.n:
            raise EngineError(-1, "state size mismatch")
        self._check(self.lib.rp_upload_state(self.h, dptr(pos), dptr(rot), dptr(box)))

    def state(self, out=None):
        """(positions N x 3, orientations N x 9, box 9).  With out = (pos, rot, box), downloads
        into those C-contiguous float64 arrays (pinned host memory makes it a direct DMA)."""
        if out is None:
            out = (np.zeros((self.n, 3)), np.zeros((self.n, 9)), np.zeros(9))
        pos, rot, box = out
        for a, shape in ((pos, (self.n, 3)), (rot, (self.n, 9)), (box, (9,))):
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size != int(np.prod(shape)):
                raise EngineError(-1, "state buffers must be C-contiguous float64 of the packing's size")
        self._check(self.lib.rp_download_state(self.h, dptr(pos), dptr(rot), dptr(box)))
        return pos, rot, box

    def store(self, path, aux=None) -> None:
        """Packing::store (core/Packing.cpp:956-959): a RAMSNAP file of the device state."""
        from .snapshots import _aux_arrays, _check, _path
        n, keys, values = _aux_arrays(aux)
        _check(self.lib, self.lib.rp_ramsnap_write(self.h, _path(path), n, keys, values))

    def restore(self, path) -> dict:
        """Packing::restore (core/Packing.cpp:961-964): loads a RAMSNAP file of this
        packing's size onto the device; returns its aux entries."""
        from .snapshots import read_ramsnap
        pos, rot, box, aux = read_ramsnap(path)
        self.upload(pos, rot, box)
        return aux

    # ---- overlaps ----
    def count_total_overlaps(self, early_exit: bool = False) -> int:
        out = C.c_int64()
        self._check(self.lib.rp_count_overlaps(self.h, 1 if early_exit else 0, C.byref(out)))
        return int(out.value)

    # ---- grid and moves ----
    @staticmethod
    def _info(info: GridInfo) -> dict:
        return {"dims": tuple(info.dims), "max_occupancy": info.max_occupancy, "shift": tuple(info.shift),
                "cell_height": tuple(info.cell_height), "num_cells": int(info.num_cells)}

    def set_grid(self, shift=(0.0, 0.0, 0.0)) -> dict:
        """Rebuilds the checkerboard grid with a relative origin shift; returns its layout."""
        s = np.ascontiguousarray(shift, dtype=np.float64)
        info = GridInfo()
        self._check(self.lib.rp_set_grid(self.h, dptr(s), C.byref(info)))
        return self._info(info)

    def grid(self):
        """(layout, cell of every particle, ActiveDomain bounds lo[3] hi[3] of every cell)."""
        info = GridInfo()
        self._check(self.lib.rp_get_grid(self.h, C.byref(info), None, None))
        cells = np.zeros(self.n, dtype=np.int32)
        bounds = np.zeros((int(info.num_cells), 6))
        self._check(self.lib.rp_get_grid(self.h, None, cells.ctypes.data_as(C.POINTER(C.c_int32)), dptr(bounds)))
        return self._info(info), cells, bounds

    def run_moves(self, moves: np.ndarray) -> np.ndarray:
        moves = np.ascontiguousarray(moves, dtype=MOVE_DTYPE)
        codes = np.zeros(len(moves), dtype=np.uint8)
        self._check(self.lib.rp_run_moves(self.h, moves.ctypes.data_as(C.c_void_p), len(moves),
                                          codes.ctypes.data_as(C.c_void_p)))
        return codes

    def try_move(self, particle: int, type_: int, translation=(0.0, 0.0, 0.0), rotation=None, domain=None) -> float:
        """Packing::tryTranslation / tryRotation / tryMove (rp_try_move), with no ActiveDomain or
        with `domain` = its relative bounds (lo[3], hi[3]): the move's energy (0 or +inf; -inf,
        0 or +inf in overlap counting); the tried state waits for accept_move."""
        m = np.zeros(1, dtype=MOVE_DTYPE)
        m["particle"] = particle
        m["type"] = type_
        m["domain"] = -1
        m["translation"] = np.asarray(translation, dtype=np.float64).reshape(3)
        m["rotation"] = np.eye(3).reshape(9) if rotation is None else np.asarray(rotation, dtype=np.float64).reshape(9)
        de = C.c_double()
        dom = None if domain is None else np.ascontiguousarray(domain, dtype=np.float64).reshape(6)
        self._check(self.lib.rp_try_move(self.h, m.ctypes.data_as(C.c_void_p), None if dom is None else dptr(dom),
                                         C.byref(de)))
        return de.value

    def accept_move(self):
        """Packing::acceptTranslation / acceptRotation / acceptMove (rp_accept_move)."""
        self._check(self.lib.rp_accept_move(self.h))

    def sweep(self, translation_step: float, rotation_step: float, seed: int, counter: int,
              log: bool = False, fp64_only: bool = False, stats: bool = True, rototranslation: bool = False):
        """One device sweep: 2N moves (translations and rotations), or N rototranslations."""
        p = SweepParams()
        p.translation_step = translation_step
        p.rotation_step = rotation_step
        p.seed = seed
        p.counter = counter
        p.flags = ((_lib.SWEEP_LOG if log else 0) | (_lib.SWEEP_FP64_ONLY if fp64_only else 0) |
                   (_lib.SWEEP_ROTOTRANSLATION if rototranslation else 0))
        st = SweepStats()
        self._check(self.lib.rp_sweep(self.h, C.byref(p), C.byref(st) if stats else None))
        return st.as_dict() if stats else None

    def set_walls(self, mask: int):
        """Packing::toggleWalls: bit i puts hard walls across box side i (rp_set_walls)."""
        self._check(self.lib.rp_set_walls(self.h, int(mask)))

    def set_soft(self, kind: int, epsilon: float = 0.0, sigma: float = 1.0, hard: bool = True):
        """A soft central interaction on the interaction centres joined to the hard shape, or
        alone (rp_set_soft): _lib.SOFT_REPULSIVE_LJ or _lib.SOFT_SQUARE_INVERSE_CORE."""
        self._check(self.lib.rp_set_soft(self.h, int(kind), float(epsilon), float(sigma), 1 if hard else 0))

    def set_temperature(self, temperature: float):
        self._check(self.lib.rp_set_temperature(self.h, float(temperature)))

    def total_energy(self) -> float:
        """Packing::getTotalEnergy (rp_total_energy)."""
        e = C.c_double()
        self._check(self.lib.rp_total_energy(self.h, C.byref(e)))
        return float(e.value)

    def set_bulk_staging(self, on: bool):
        """Stage sweep neighbourhoods with bulk asynchronous copies (1) or per-lane loads (0)
        (rp_set_bulk_staging)."""
        self._check(self.lib.rp_set_bulk_staging(self.h, 1 if on else 0))

    def set_cell_order(self, on: bool):
        """Sweep each phase's cells by occupancy, largest first (1), or in index order (0)
        (rp_set_cell_order)."""
        self._check(self.lib.rp_set_cell_order(self.h, 1 if on else 0))

    def set_cells_per_warp(self, cells: int):
        """1: a warp sweeps one cell; 2: each half-warp sweeps its own (rp_set_cells_per_warp)."""
        self._check(self.lib.rp_set_cells_per_warp(self.h, int(cells)))

    def cells_per_warp(self) -> int:
        """Cells per warp the last sweep used (rp_get_cells_per_warp)."""
        v = C.c_int32()
        self._check(self.lib.rp_get_cells_per_warp(self.h, C.byref(v)))
        return int(v.value)

    def set_staging_filter(self, mode: int = 1):
        """0 off, 1 where it pays (default), 2 wherever valid (rp_set_staging_filter)."""
        self._check(self.lib.rp_set_staging_filter(self.h, int(mode)))

    def sweep_log(self):
        cnt = C.c_int64()
        self._check(self.lib.rp_sweep_log(self.h, None, None, 0, C.byref(cnt)))
        moves = np.zeros(cnt.value, dtype=MOVE_DTYPE)
        codes = np.zeros(cnt.value, dtype=np.uint8)
        self._check(self.lib.rp_sweep_log(self.h, moves.ctypes.data_as(C.c_void_p),
                                          codes.ctypes.data_as(C.c_void_p), cnt.value, C.byref(cnt)))
        return moves, codes

    def stats(self) -> dict:
        st = SweepStats()
        self._check(self.lib.rp_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    def convex_pair_overlaps(self, pos1, rot1, pos2, rot2) -> np.ndarray:
        """XenoCollideTraits::overlapBetween of the handle's convex body on independent pairs
        (no periodic image), decided on the device."""
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (pos1, rot1, pos2, rot2)]
        n = a[0].reshape(-1, 3).shape[0]
        out = np.zeros(n, dtype=np.uint8)
        self._check(self.lib.rp_convex_pair_overlaps(self.h, n, dptr(a[0]), dptr(a[1]), dptr(a[2]), dptr(a[3]),
                                                     out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out.astype(bool)

    def grid_counters(self) -> dict:
        """Full cell-grid rebuilds (Packing::getNeighbourGridRebuilds) and box moves that kept
        the old cells (remaps) since creation."""
        rb, rm = C.c_uint64(), C.c_uint64()
        self._check(self.lib.rp_get_grid_counters(self.h, C.byref(rb), C.byref(rm)))
        return {"rebuilds": rb.value, "remaps": rm.value}

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.rp_get_stream(self.h, C.byref(s)))
        return int(s.value or 0)

    def set_timing(self, on: bool = True):
        self._check(self.lib.rp_set_timing(self.h, 1 if on else 0))

    def timing(self) -> dict:
        ng = len(_lib.KERNEL_GROUPS)
        ms = (C.c_double * ng)()
        groups = (C.c_uint64 * ng)()
        self._check(self.lib.rp_get_timing(self.h, ms, groups))
        return {name: (float(ms[k]), int(groups[k])) for k, name in enumerate(_lib.KERNEL_GROUPS)}

    # ---- learned ordering of the overlap tests ----
    def mlp_init(self, seed: int = 0):
        self._check(self.lib.rp_mlp_init(self.h, seed))

    def mlp_params(self) -> np.ndarray:
        w = np.zeros(_lib.MLP_NPARAM, dtype=np.float32)
        self._check(self.lib.rp_mlp_get_params(self.h, fptr(w)))
        return w

    def set_mlp_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32).reshape(_lib.MLP_NPARAM)
        self._check(self.lib.rp_mlp_set_params(self.h, fptr(w)))

    def mlp_predict(self, feats) -> np.ndarray:
        f = np.ascontiguousarray(feats, dtype=np.float32).reshape(-1, _lib.MLP_FEATURES)
        out = np.zeros(len(f), dtype=np.float32)
        self._check(self.lib.rp_mlp_predict(self.h, fptr(f), len(f), fptr(out)))
        return out

    def mlp_gradient(self, feats, labels):
        f = np.ascontiguousarray(feats, dtype=np.float32).reshape(-1, _lib.MLP_FEATURES)
        lab = np.ascontiguousarray(labels, dtype=np.uint8).reshape(len(f))
        g = np.zeros(_lib.MLP_NPARAM, dtype=np.float32)
        loss = C.c_float()
        self._check(self.lib.rp_mlp_gradient(self.h, fptr(f), lab.ctypes.data_as(C.c_void_p), len(f), fptr(g),
                                             C.byref(loss)))
        return g, float(loss.value)

    def pair_log_enable(self, capacity: int, every: int = 1):
        self._check(self.lib.rp_pair_log_enable(self.h, capacity, every))

    def pair_log(self, capacity: int | None = None):
        cnt = C.c_int64()
        self._check(self.lib.rp_pair_log_read(self.h, None, None, 0, C.byref(cnt)))
        k = cnt.value if capacity is None else min(cnt.value, capacity)
        f = np.zeros((k, _lib.MLP_FEATURES), dtype=np.float32)
        lab = np.zeros(k, dtype=np.uint8)
        self._check(self.lib.rp_pair_log_read(self.h, fptr(f), lab.ctypes.data_as(C.c_void_p), k, C.byref(cnt)))
        return f, lab

    def pair_log_count(self) -> int:
        """Pair outcomes held by the log (at most its capacity)."""
        cnt = C.c_int64()
        self._check(self.lib.rp_pair_log_read(self.h, None, None, 0, C.byref(cnt)))
        return int(cnt.value)

    def pair_log_clear(self):
        self._check(self.lib.rp_pair_log_clear(self.h))

    def mlp_train(self, epochs: int, batch: int, lr: float, seed: int = 0) -> float:
        loss = C.c_float()
        self._check(self.lib.rp_mlp_train(self.h, epochs, batch, lr, seed, C.byref(loss)))
        return float(loss.value)

    def set_ordering(self, mode: int, every: int = 1):
        self._check(self.lib.rp_set_ordering(self.h, mode, every))

    # ---- overlap counting ----
    def set_counting(self, on: bool = True):
        """Packing::toggleOverlapCounting."""
        self._check(self.lib.rp_set_counting(self.h, 1 if on else 0))

    def cached_overlaps(self) -> int:
        """Packing::getCachedNumberOfOverlaps."""
        c = C.c_int64()
        self._check(self.lib.rp_cached_overlaps(self.h, C.byref(c)))
        return int(c.value)

    # ---- observables ----
    def nematic_order(self):
        """(Q tensor 3x3, P2) of the current state (NematicOrder::calculate)."""
        q = np.zeros(9)
        p2 = C.c_double()
        self._check(self.lib.rp_nematic_order(self.h, dptr(q), C.byref(p2)))
        return q.reshape(3, 3), float(p2.value)

    # ---- orientation renormalisation ----
    def renormalize_orientations(self, allow_overlaps: bool = False) -> int:
        """Packing::renormalizeOrientations: the number of particles whose fix was rejected."""
        r = C.c_int64()
        self._check(self.lib.rp_renormalize_orientations(self.h, 1 if allow_overlaps else 0, C.byref(r)))
        return int(r.value)

    # ---- box moves ----
    def try_scaling(self, box) -> float:
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        dE = C.c_double()
        self._check(self.lib.rp_try_scaling(self.h, dptr(b), C.byref(dE)))
        return float(dE.value)

    def revert_scaling(self):
        self._check(self.lib.rp_revert_scaling(self.h))


INF = math.inf


class BatchPacking:
    """Many independent packings of one shape kind advanced together (rp_batch_*).

    ``systems`` is a list of (pos, rot, box); every replica shares the shape ``kind`` and
    ``params`` (sphere radius, or spherocylinder length and radius)."""

    def __init__(self, kind: int, params, systems, device: int = 0):
        self.lib = _lib.load()
        params = np.asarray(params, dtype=np.float64).reshape(-1)
        desc = ShapeDesc()
        desc.kind = kind
        if kind == _lib.SHAPE_SPHERE:
            desc.radius = float(params[0])
        elif kind == _lib.SHAPE_SPHEROCYLINDER:
            desc.length, desc.radius = float(params[0]), float(params[1])
        else:
            raise EngineError(-5, f"shape kind {kind} is not batched")
        self.kind, self.params = kind, params
        self.sizes = [len(np.asarray(p).reshape(-1, 3)) for p, _, _ in systems]
        self.R = len(systems)
        n = (C.c_int64 * self.R)(*self.sizes)
        h = C.c_void_p()
        rc = self.lib.rp_batch_create(C.byref(desc), self.R, n, device, C.byref(h))
        if rc != 0:
            raise EngineError(rc, "rp_batch_create failed")
        self.h = h
        for r, (pos, rot, box) in enumerate(systems):
            self.upload(r, pos, rot, box)

    def _check(self, rc: int):
        if rc != 0:
            msg = self.lib.rp_batch_last_error(self.h)
            raise EngineError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.rp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload(self, r: int, pos, rot, box):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        rot = np.ascontiguousarray(rot, dtype=np.float64).reshape(-1, 9)
        box = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        self._check(self.lib.rp_batch_upload_state(self.h, r, dptr(pos), dptr(rot), dptr(box)))

    def state(self, r: int):
        n = self.sizes[r]
        pos, rot, box = np.zeros((n, 3)), np.zeros((n, 9)), np.zeros(9)
        self._check(self.lib.rp_batch_download_state(self.h, r, dptr(pos), dptr(rot), dptr(box)))
        return pos, rot, box

    def count_total_overlaps(self, r: int, early_exit: bool = False) -> int:
        c = C.c_int64()
        self._check(self.lib.rp_batch_count_overlaps(self.h, r, 1 if early_exit else 0, C.byref(c)))
        return int(c.value)

    def grid(self, r: int):
        info = GridInfo()
        self._check(self.lib.rp_batch_get_grid(self.h, r, C.byref(info), None, None))
        cells = np.zeros(self.sizes[r], dtype=np.int32)
        bounds = np.zeros((int(info.num_cells), 6))
        self._check(self.lib.rp_batch_get_grid(self.h, r, None, cells.ctypes.data_as(C.POINTER(C.c_int32)),
                                               dptr(bounds)))
        return GpuPacking._info(info), cells, bounds

    def sweep(self, translation_step: float, rotation_step: float, seed: int, counter: int, log: bool = False,
              stats: bool = True, fp64_only: bool = False, rototranslation: bool = False):
        p = SweepParams()
        p.translation_step, p.rotation_step, p.seed, p.counter = translation_step, rotation_step, seed, counter
        p.flags = ((_lib.SWEEP_LOG if log else 0) | (_lib.SWEEP_FP64_ONLY if fp64_only else 0) |
                   (_lib.SWEEP_ROTOTRANSLATION if rototranslation else 0))
        st = (SweepStats * self.R)() if stats else None
        self._check(self.lib.rp_batch_sweep(self.h, C.byref(p), st))
        return [s.as_dict() for s in st] if stats else None

    def sweep_log(self, r: int):
        cnt = C.c_int64()
        self._check(self.lib.rp_batch_sweep_log(self.h, r, None, None, 0, C.byref(cnt)))
        moves = np.zeros(cnt.value, dtype=MOVE_DTYPE)
        codes = np.zeros(cnt.value, dtype=np.uint8)
        self._check(self.lib.rp_batch_sweep_log(self.h, r, moves.ctypes.data_as(C.c_void_p),
                                                codes.ctypes.data_as(C.c_void_p), cnt.value, C.byref(cnt)))
        return moves, codes

    def try_scaling(self, boxes, propose) -> np.ndarray:
        b = np.ascontiguousarray(boxes, dtype=np.float64).reshape(self.R, 9)
        m = np.ascontiguousarray(propose, dtype=np.uint8).reshape(self.R)
        dE = np.zeros(self.R)
        self._check(self.lib.rp_batch_try_scaling(self.h, dptr(b), m.ctypes.data_as(C.c_void_p), dptr(dE)))
        return dE

    def revert_scaling(self, mask):
        m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(self.R)
        self._check(self.lib.rp_batch_revert_scaling(self.h, m.ctypes.data_as(C.c_void_p)))

    def set_tuning(self, cell_factor: float = 1.0, warps_per_block: int = 4):
        self._check(self.lib.rp_batch_set_tuning(self.h, cell_factor, warps_per_block))

    def set_walls(self, mask: int):
        """rp_set_walls for every replica."""
        self._check(self.lib.rp_batch_set_walls(self.h, int(mask)))

    def set_staging_filter(self, mode: int = 1):
        """rp_set_staging_filter for every replica."""
        self._check(self.lib.rp_batch_set_staging_filter(self.h, int(mode)))

    def upload_all(self, pos, rot, boxes):
        """Every replica's state at once (rp_batch_upload_states): pos [sum n, 3] and
        rot [sum n, 9] with the replicas' particles in replica order, boxes [R, 9]."""
        total = sum(self.sizes)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(total, 3)
        rot = np.ascontiguousarray(rot, dtype=np.float64).reshape(total, 9)
        boxes = np.ascontiguousarray(boxes, dtype=np.float64).reshape(self.R, 9)
        self._check(self.lib.rp_batch_upload_states(self.h, dptr(pos), dptr(rot), dptr(boxes)))

    def states(self, out=None):
        """Every replica's state at once (rp_batch_download_states), into ``out`` =
        (pos, rot, boxes) when given (e.g. pinned buffers)."""
        total = sum(self.sizes)
        if out is None:
            out = (np.zeros((total, 3)), np.zeros((total, 9)), np.zeros((self.R, 9)))
        pos, rot, boxes = out
        for a, shape in ((pos, (total, 3)), (rot, (total, 9)), (boxes, (self.R, 9))):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != shape[0] * shape[1]:
                raise ValueError("out arrays must be C-contiguous float64 of the batch's sizes")
        self._check(self.lib.rp_batch_download_states(self.h, dptr(pos), dptr(rot), dptr(boxes)))
        return pos.reshape(total, 3), rot.reshape(total, 9), boxes.reshape(self.R, 9)

    def set_timing(self, on: bool = True):
        self._check(self.lib.rp_batch_set_timing(self.h, 1 if on else 0))

    def timing(self):
        """({group: (ms, groups)}, kernel launches of the batch and its replicas)."""
        ng = len(_lib.KERNEL_GROUPS)
        ms = (C.c_double * ng)()
        groups = (C.c_uint64 * ng)()
        launches = C.c_uint64()
        self._check(self.lib.rp_batch_get_timing(self.h, ms, groups, C.byref(launches)))
        return {name: (float(ms[k]), int(groups[k])) for k, name in enumerate(_lib.KERNEL_GROUPS)}, int(launches.value)


def replica_seed(seed: int, r: int) -> int:
    """The sweep seed replica r of a batch uses (rp_batch_sweep)."""
    return (seed + _lib.BATCH_SEED_STRIDE * r) % (1 << 64)
