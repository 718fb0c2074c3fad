"""ORACLE — test infrastructure only.

ctypes wrapper over the two CPU implementations of the move-and-overlap path:

* ``liboracle.so`` — this project's C++ restatement (oracle/rpo_*.hpp), portable;
* ``_ref/librpref.so`` — the reference's own sources compiled in place by
  ``make -C oracle ref`` (only where the reference checkout is present).

Both export the same entry points (``rpo_*`` / ``ref_*``), so one Python class
drives either.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "librpref.so")
# the reference checkout (read-only): RAMPACK_REFERENCE_DIR, else the default mount point
REFERENCE_DIR = os.environ.get("RAMPACK_REFERENCE_DIR", "/root/reference")

SPHERE, SPHEROCYLINDER, POLYSPHERE = 0, 1, 2
# generic convex bodies (GenericXenoCollideTraits): `params` is the XCBodyBuilder script
CONVEX = 4

MOVE_DTYPE = np.dtype([
    ("particle", "<i4"), ("type", "<i4"), ("domain", "<i4"), ("reserved", "<i4"),
    ("translation", "<f8", (3,)), ("rotation", "<f8", (9,)), ("uniform", "<f8"),
])
assert MOVE_DTYPE.itemsize == 120


class SimParams(C.Structure):
    _fields_ = [("temperature", C.c_double), ("pressure", C.c_double),
                ("translation_step", C.c_double), ("rotation_step", C.c_double),
                ("box_kind", C.c_int32), ("adjust_steps", C.c_int32), ("box_step", C.c_double),
                ("domains", C.c_int64 * 3), ("seed", C.c_uint64), ("threads", C.c_int64)]


class SimStats(C.Structure):
    _fields_ = [("moves", C.c_int64 * 2), ("accepted", C.c_int64 * 2),
                ("scalings", C.c_int64), ("scalings_accepted", C.c_int64), ("cycles", C.c_int64),
                ("domains", C.c_int64 * 3),
                ("move_us", C.c_double), ("scaling_us", C.c_double), ("total_us", C.c_double),
                ("steps", C.c_double * 2), ("box_step", C.c_double)]


def build(reference: bool = False) -> None:
    """Compiles liboracle.so (and the reference library when asked and possible)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if reference and os.path.isdir(os.path.join(REFERENCE_DIR, "src")):
        subprocess.run(["make", "-s", "-j", str(os.cpu_count() or 4), "-C", HERE, "ref", f"REF={REFERENCE_DIR}"],
                       check=True)


def reference_available() -> bool:
    return os.path.exists(REF_SO)


_LIBS: dict = {}

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)


def _lib(which: str):
    if which in _LIBS:
        return _LIBS[which]
    path, pre = (ORACLE_SO, "rpo_") if which == "oracle" else (REF_SO, "ref_")
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = C.CDLL(path)
    sig = {
        "create": (_P, [C.c_int, _D, C.c_int, C.c_int64, _D, _D, _D, C.c_int]),
        "destroy": (None, [_P]),
        "count_overlaps": (C.c_int64, [_P, C.c_int]),
        "set_counting": (None, [_P, C.c_int]),
        "cached_overlaps": (C.c_int64, [_P]),
        "replay": (C.c_int, [_P, _P, C.c_int64, _D, C.c_double, _P, _P]),
        "try_scaling": (C.c_double, [_P, _D]),
        "revert_scaling": (None, [_P]),
        "renormalize": (C.c_int64, [_P, C.c_int]),
        "get_state": (None, [_P, _D, _D, _D]),
        "ng_divisions": (C.c_int, [_P, _I64]),
        "pair_overlap": (C.c_int, [C.c_int, _D, C.c_int, _D, _D, C.c_int, _D, _D, C.c_int, C.c_int, _D, _D]),
        "box_info": (None, [_D, _D, _D, _D]),
        "rotation": (None, [_D, C.c_double, _D]),
        "rng_create": (_P, [C.c_uint64]),
        "rng_destroy": (None, [_P]),
        "set_soft": (C.c_int, [_P, C.c_int, C.c_double, C.c_double, C.c_int]),
        "total_energy": (C.c_double, [_P]),
        "replay_energies": (C.c_int, [_P, _P, C.c_int64, _D, C.c_double, _P, _P, _D]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, pre + name)
        f.restype, f.argtypes = res, args
    if which == "oracle":
        lib.rpo_draw_moves.restype = C.c_int
        lib.rpo_draw_moves.argtypes = [_P, C.c_double, C.c_double, _D, _I64, C.c_int64, C.c_int64, C.c_int64,
                                       C.c_int32, _P]
        lib.rpo_sim_create.restype = _P
        lib.rpo_sim_create.argtypes = [_P, C.POINTER(SimParams)]
        lib.rpo_sim_run.restype = C.c_int
        lib.rpo_sim_run.argtypes = [_P, C.c_int64, C.POINTER(SimStats)]
        lib.rpo_sim_destroy.argtypes = [_P]
        lib.rpo_segment_distance2.restype = C.c_double
        lib.rpo_segment_distance2.argtypes = [_D, _D, _D, _D]
    else:
        lib.ref_draw_moves.restype = C.c_int
        lib.ref_draw_moves.argtypes = [_P, _P, C.c_double, C.c_double, _I64, C.c_int64, C.c_int64, C.c_int64,
                                       C.c_int32, _P]
        lib.ref_sim_run.restype = C.c_int
        lib.ref_sim_run.argtypes = [_P, C.POINTER(SimParams), C.c_int64, C.POINTER(SimStats)]
        lib.ref_banana_centres.restype = C.c_int
        lib.ref_banana_centres.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double, _D]
        lib.ref_nematic_order.restype = C.c_int
        lib.ref_nematic_order.argtypes = [_P, _D]
    _LIBS[which] = (lib, pre)
    return _LIBS[which]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def shape_params(kind: int, **kw) -> np.ndarray:
    if kind == SPHERE:
        return np.array([kw["radius"]], dtype=np.float64)
    if kind == SPHEROCYLINDER:
        return np.array([kw["length"], kw["radius"]], dtype=np.float64)
    centres = np.asarray(kw["centres"], dtype=np.float64).reshape(-1, 3)
    radii = np.asarray(kw["radii"], dtype=np.float64).reshape(-1)
    out = [float(len(radii))]
    for c, r in zip(centres, radii):
        out += [c[0], c[1], c[2], r]
    return np.array(out, dtype=np.float64)


class CpuPacking:
    """A Packing on the CPU: ``which`` = "oracle" (restatement) or "reference"."""

    def __init__(self, which: str, kind: int, params: np.ndarray, pos: np.ndarray, rot: np.ndarray,
                 box: np.ndarray, threads: int = 1):
        self.lib, self.pre = _lib("oracle" if which == "oracle" else "reference")
        self.which = which
        self.kind = kind
        self.params = params if kind == CONVEX else np.ascontiguousarray(params, dtype=np.float64)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        rot = np.ascontiguousarray(rot, dtype=np.float64).reshape(-1, 9)
        box = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        self.n = pos.shape[0]
        if kind == CONVEX:
            f = self._f("create_convex")
            f.restype, f.argtypes = _P, [C.c_char_p, C.c_int64, _D, _D, _D, C.c_int]
            self.script = params
            self.h = f(params.encode(), self.n, _dp(pos), _dp(rot), _dp(box), threads)
        else:
            self.h = self._f("create")(kind, _dp(self.params), len(self.params), self.n, _dp(pos), _dp(rot),
                                       _dp(box), threads)
        if not self.h:
            raise ValueError("packing construction failed")

    def _f(self, name):
        return getattr(self.lib, self.pre + name)

    def close(self):
        if self.h:
            self._f("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nematic_order(self):
        """(Q tensor 3x3, P2) from the reference's own NematicOrder (reference library only)."""
        if self.which != "reference":
            raise ValueError("nematic_order: the reference's NematicOrder is in the reference library only")
        out = np.zeros(7)
        if self.lib.ref_nematic_order(self.h, _dp(out)) != 0:
            raise RuntimeError("NematicOrder::calculate failed")
        q = np.array([[out[1], out[2], out[3]], [out[2], out[4], out[5]], [out[3], out[5], out[6]]])
        return q, float(out[0])

    def count_overlaps(self, early_exit: bool = False) -> int:
        return int(self._f("count_overlaps")(self.h, 1 if early_exit else 0))

    def set_walls(self, mask: int) -> None:
        """Packing::toggleWalls: bit i puts hard walls across box side i."""
        f = self._f("set_walls")
        f.restype, f.argtypes = None, [_P, C.c_int]
        f(self.h, int(mask))

    def set_counting(self, on: bool) -> None:
        self._f("set_counting")(self.h, 1 if on else 0)

    def cached_overlaps(self) -> int:
        return int(self._f("cached_overlaps")(self.h))

    def replay(self, moves: np.ndarray, domains: np.ndarray | None = None, temperature: float = 1.0,
               energies: bool = False):
        """Codes and overlap-count deltas of the moves replayed in order; with `energies` also
        each move's energy (0, +-inf or the soft energy change)."""
        moves = np.ascontiguousarray(moves, dtype=MOVE_DTYPE)
        codes = np.zeros(len(moves), dtype=np.uint8)
        deltas = np.zeros(len(moves), dtype=np.int32)
        de = np.zeros(len(moves), dtype=np.float64)
        dom = None if domains is None else np.ascontiguousarray(domains, dtype=np.float64)
        rc = self._f("replay_energies")(self.h, moves.ctypes.data_as(C.c_void_p), len(moves),
                                        None if dom is None else _dp(dom), temperature,
                                        codes.ctypes.data_as(C.c_void_p), deltas.ctypes.data_as(C.c_void_p), _dp(de))
        if rc != 0:
            raise RuntimeError("replay failed")
        return (codes, deltas, de) if energies else (codes, deltas)

    def set_soft(self, kind: int, epsilon: float, sigma: float, hard: bool = True) -> None:
        """A soft central interaction on the shape's interaction centres: kind 1
        RepulsiveLennardJones, 2 SquareInverseCore, joined to the hard shape (or alone)."""
        if self._f("set_soft")(self.h, int(kind), float(epsilon), float(sigma), 1 if hard else 0) != 0:
            raise ValueError("soft interaction refused")

    def total_energy(self) -> float:
        """Packing::getTotalEnergy."""
        return float(self._f("total_energy")(self.h))

    def try_scaling(self, box: np.ndarray) -> float:
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        return float(self._f("try_scaling")(self.h, _dp(b)))

    def revert_scaling(self) -> None:
        self._f("revert_scaling")(self.h)

    def renormalize_orientations(self, allow_overlaps: bool = False) -> int:
        """Packing::renormalizeOrientations: the number of particles whose fix was rejected."""
        return int(self._f("renormalize")(self.h, 1 if allow_overlaps else 0))

    def state(self):
        pos = np.zeros((self.n, 3))
        rot = np.zeros((self.n, 9))
        box = np.zeros(9)
        self._f("get_state")(self.h, _dp(pos), _dp(rot), _dp(box))
        return pos, rot, box

    def ng_divisions(self):
        d = np.zeros(3, dtype=np.int64)
        ok = self._f("ng_divisions")(self.h, d.ctypes.data_as(_I64))
        return tuple(int(x) for x in d) if ok else None

    def draw_moves(self, rng, trans_step: float, rot_step: float, idxs, per_type: int, n: int,
                   domain: int = -1) -> np.ndarray:
        idxs = np.ascontiguousarray(idxs, dtype=np.int64)
        out = np.zeros(n, dtype=MOVE_DTYPE)
        if self.which == "oracle":
            _, _, box = self.state()
            rc = self.lib.rpo_draw_moves(rng, trans_step, rot_step, _dp(box), idxs.ctypes.data_as(_I64), len(idxs),
                                         per_type, n, domain, out.ctypes.data_as(C.c_void_p))
        else:
            rc = self.lib.ref_draw_moves(rng, self.h, trans_step, rot_step, idxs.ctypes.data_as(_I64), len(idxs),
                                         per_type, n, domain, out.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise RuntimeError("draw_moves failed")
        return out

    def draw_flips(self, rng, idxs, n: int, flip_axis=None, origin=(0.0, 0.0, 0.0), domain: int = -1) -> np.ndarray:
        """FlipSampler moves: the oracle's restatement (flip_axis and origin in the body frame)
        or the reference's own sampler set up for this packing's shape."""
        from rampack_gb300._lib import MOVE_DTYPE
        idxs = np.ascontiguousarray(idxs, dtype=np.int64)
        out = np.zeros(n, dtype=MOVE_DTYPE)
        if self.which == "oracle":
            _, rot, _ = self.state()
            rot = np.ascontiguousarray(rot)
            fa = np.ascontiguousarray(flip_axis, dtype=np.float64)
            go = np.ascontiguousarray(origin, dtype=np.float64)
            self.lib.rpo_draw_flips.restype = C.c_int
            self.lib.rpo_draw_flips.argtypes = [_P, _D, _D, _D, _I64, C.c_int64, C.c_int64, C.c_int32, _P]
            rc = self.lib.rpo_draw_flips(rng, _dp(rot), _dp(fa), _dp(go), idxs.ctypes.data_as(_I64), len(idxs), n,
                                         domain, out.ctypes.data_as(_P))
        else:
            self.lib.ref_draw_flips.restype = C.c_int
            self.lib.ref_draw_flips.argtypes = [_P, _P, _I64, C.c_int64, C.c_int64, C.c_int32, _P]
            rc = self.lib.ref_draw_flips(rng, self.h, idxs.ctypes.data_as(_I64), len(idxs), n, domain,
                                         out.ctypes.data_as(_P))
        if rc != 0:
            raise ValueError("flip draw failed")
        return out

    def rng(self, seed: int):
        return self._f("rng_create")(seed)

    def rng_free(self, r) -> None:
        self._f("rng_destroy")(r)


def sim_params(**kw) -> SimParams:
    p = SimParams()
    p.temperature = kw.get("temperature", 1.0)
    p.pressure = kw.get("pressure", 1.0)
    p.translation_step = kw.get("translation_step", 0.0)
    p.rotation_step = kw.get("rotation_step", 0.0)
    p.box_kind = kw.get("box_kind", 0)
    p.adjust_steps = 1 if kw.get("adjust_steps", False) else 0
    p.box_step = kw.get("box_step", 0.0)
    d = kw.get("domains", (1, 1, 1))
    for i in range(3):
        p.domains[i] = d[i]
    p.seed = kw.get("seed", 1234)
    p.threads = kw.get("threads", 1)
    return p


def run_cycles(pk: CpuPacking, cycles: int, **kw) -> SimStats:
    """Runs the cycle loop (Simulation::integrate) on a CpuPacking."""
    st = SimStats()
    p = sim_params(**kw)
    if pk.which == "oracle":
        s = pk.lib.rpo_sim_create(pk.h, C.byref(p))
        if not s:
            raise ValueError("bad simulation parameters")
        try:
            if pk.lib.rpo_sim_run(s, cycles, C.byref(st)) != 0:
                raise RuntimeError("cycle loop failed")
        finally:
            pk.lib.rpo_sim_destroy(s)
    else:
        if pk.lib.ref_sim_run(pk.h, C.byref(p), cycles, C.byref(st)) != 0:
            raise RuntimeError("reference integrate failed")
    return st


def pair_overlap(which: str, kind: int, params, p1, r1, p2, r2, c1: int = 0, c2: int = 0,
                 box=None, translation=None) -> bool:
    lib, pre = _lib("oracle" if which == "oracle" else "reference")
    prm = np.ascontiguousarray(params, dtype=np.float64)
    a = [np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (p1, r1, p2, r2)]
    bc_kind, b, t = 0, None, None
    if box is not None:
        bc_kind, b = 1, np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    elif translation is not None:
        bc_kind, t = 2, np.ascontiguousarray(translation, dtype=np.float64).reshape(3)
    r = getattr(lib, pre + "pair_overlap")(kind, _dp(prm), len(prm), _dp(a[0]), _dp(a[1]), c1, _dp(a[2]), _dp(a[3]),
                                           c2, bc_kind, None if b is None else _dp(b), None if t is None else _dp(t))
    if r < 0:
        raise ValueError("bad shape")
    return bool(r)


def convex_overlap(which: str, script: str, p1, r1, p2, r2) -> bool:
    """XenoCollideTraits::overlapBetween of two placed convex bodies (no periodic image)."""
    lib, pre = _lib("oracle" if which == "oracle" else "reference")
    a = [np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (p1, r1, p2, r2)]
    if which == "oracle":
        f = lib.rpo_convex_overlap
        f.restype, f.argtypes = C.c_int, [C.c_char_p, _D, _D, _D, _D]
        r = f(script.encode(), *[_dp(x) for x in a])
        if r < 0:
            raise ValueError("invalid convex body script")
    else:
        f = lib.ref_convex_overlap
        f.restype, f.argtypes = C.c_int, [C.c_char_p, _D, _D, _D, _D, C.c_char_p, C.c_int]
        err = _errbuf()
        r = f(script.encode(), *[_dp(x) for x in a], err, 512)
        if r < 0:
            raise ValueError(err.value.decode())
    return bool(r)


def rotation(which: str, axis, angle: float) -> np.ndarray:
    lib, pre = _lib("oracle" if which == "oracle" else "reference")
    ax = np.ascontiguousarray(axis, dtype=np.float64)
    out = np.zeros(9)
    getattr(lib, pre + "rotation")(_dp(ax), angle, _dp(out))
    return out


def box_info(which: str, box):
    lib, pre = _lib("oracle" if which == "oracle" else "reference")
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    inv, h, v = np.zeros(9), np.zeros(3), np.zeros(1)
    getattr(lib, pre + "box_info")(_dp(b), _dp(inv), _dp(h), _dp(v))
    return inv, h, float(v[0])


def banana_centres(arc_radius: float, arc_angle: float, n: int, sphere_radius: float) -> np.ndarray:
    """Body-frame centres of a bent polysphere, from the reference's own generator."""
    lib, _ = _lib("reference")
    out = np.zeros(4 * n)
    k = lib.ref_banana_centres(arc_radius, arc_angle, n, sphere_radius, _dp(out))
    return out[:4 * k].reshape(k, 4)


# ---- the reference's own snapshot and trajectory writers / readers (fixture generation) ----

def _errbuf():
    return C.create_string_buffer(512)


def ref_ramsnap_write(path: str, kind: int, params, pos, rot, box, aux=None) -> None:
    """Packing::store of a reference packing built from the state."""
    lib, _ = _lib("reference")
    pk = CpuPacking("reference", kind, params, pos, rot, box, threads=1)
    items = list((aux or {}).items())
    keys = (C.c_char_p * max(1, len(items)))(*[k.encode() for k, _ in items])
    vals = (C.c_char_p * max(1, len(items)))(*[v.encode() for _, v in items])
    err = _errbuf()
    lib.ref_ramsnap_write.restype = C.c_int
    lib.ref_ramsnap_write.argtypes = [_P, C.c_char_p, C.c_int, _P, _P, C.c_char_p, C.c_int]
    rc = lib.ref_ramsnap_write(pk.h, path.encode(), len(items), C.cast(keys, _P), C.cast(vals, _P), err, 512)
    pk.close()
    if rc != 0:
        raise ValueError(err.value.decode())


def ref_ramsnap_read(path: str, kind: int, params, cap: int = 1 << 20):
    """Packing::restore: (pos, rot, box, aux) or ValueError with the reference's message."""
    lib, _ = _lib("reference")
    prm = np.ascontiguousarray(params, dtype=np.float64)
    pos, rot, box = np.zeros((cap, 3)), np.zeros((cap, 9)), np.zeros(9)
    aux, err = C.create_string_buffer(1 << 16), _errbuf()
    lib.ref_ramsnap_read.restype = C.c_int64
    lib.ref_ramsnap_read.argtypes = [C.c_char_p, C.c_int, _D, C.c_int, _D, _D, _D, C.c_int64, C.c_char_p, C.c_int,
                                     C.c_char_p, C.c_int]
    n = lib.ref_ramsnap_read(path.encode(), kind, _dp(prm), len(prm), _dp(pos), _dp(rot), _dp(box), cap, aux,
                             1 << 16, err, 512)
    if n < 0:
        raise ValueError(err.value.decode())
    entries = {}
    for ln in aux.value.decode().split("\n"):
        if ln:
            k, v = ln.split("\t", 1)
            entries[k] = v
    return pos[:n].copy(), rot[:n].copy(), box, entries


def ref_ramtrj_write(path: str, kind: int, params, states, cycle_step: int) -> None:
    """RamtrjRecorder over `states` = [(pos, rot, box), ...]."""
    lib, _ = _lib("reference")
    prm = np.ascontiguousarray(params, dtype=np.float64)
    pos = np.ascontiguousarray(np.concatenate([np.asarray(s[0]).reshape(-1, 3) for s in states]))
    rot = np.ascontiguousarray(np.concatenate([np.asarray(s[1]).reshape(-1, 9) for s in states]))
    boxes = np.ascontiguousarray(np.stack([np.asarray(s[2]).reshape(9) for s in states]))
    n = len(np.asarray(states[0][0]).reshape(-1, 3))
    err = _errbuf()
    lib.ref_ramtrj_write.restype = C.c_int
    lib.ref_ramtrj_write.argtypes = [C.c_char_p, C.c_int, _D, C.c_int, C.c_int64, C.c_int64, C.c_int64, _D, _D, _D,
                                     C.c_char_p, C.c_int]
    rc = lib.ref_ramtrj_write(path.encode(), kind, _dp(prm), len(prm), n, len(states), cycle_step, _dp(pos),
                              _dp(rot), _dp(boxes), err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())


def ref_ramtrj_read(path: str, kind: int, params, index: int, n: int):
    """RamtrjPlayer::jumpToSnapshot: (pos, rot, box) of snapshot `index` (from 0)."""
    lib, _ = _lib("reference")
    prm = np.ascontiguousarray(params, dtype=np.float64)
    pos, rot, box = np.zeros((n, 3)), np.zeros((n, 9)), np.zeros(9)
    err = _errbuf()
    lib.ref_ramtrj_read.restype = C.c_int
    lib.ref_ramtrj_read.argtypes = [C.c_char_p, C.c_int, _D, C.c_int, C.c_int64, _D, _D, _D, C.c_char_p, C.c_int]
    rc = lib.ref_ramtrj_read(path.encode(), kind, _dp(prm), len(prm), index, _dp(pos), _dp(rot), _dp(box), err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    return pos, rot, box


def ref_box_proposals(kind: int, together: int, groups, independent: int, step: float, seed: int, box, count: int):
    """The reference's box scalers (TriclinicDeltaScaler, TriclinicAdapter over
    AnisotropicVolumeScaler / DeltaVolumeScaler) drawing `count` proposals from one box with
    std::mt19937(seed), each followed by Simulation's unit-interval draw."""
    lib, _ = _lib("reference")
    lib.ref_box_proposals.restype = C.c_int
    lib.ref_box_proposals.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_double, C.c_uint64,
                                      _D, C.c_int64, _D, _D]
    g = (C.c_int * 3)(*(list(groups) + [0, 0, 0])[:3])
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    boxes, u = np.zeros((count, 9)), np.zeros(count)
    if lib.ref_box_proposals(kind, together, len(groups), g, independent, step, seed, _dp(b), count, _dp(boxes),
                             _dp(u)) != 0:
        raise ValueError("bad scaler")
    return boxes, u


# ---- pair correlations (core/observables/correlation/*) --------------------------------

class PairDesc(C.Structure):
    """Same layout as rpo_pair_desc (oracle/rpo_capi.cpp) and rp_pair_desc."""
    _fields_ = [("enumerator", C.c_int32), ("linear_axis", C.c_int32), ("miller", C.c_int32 * 3),
                ("function", C.c_int32), ("axis", C.c_int32), ("num_bins", C.c_int32), ("flags", C.c_int32),
                ("reserved", C.c_int32), ("max_r", C.c_double),
                ("focal", C.c_double * 3), ("primary", C.c_double * 3), ("secondary", C.c_double * 3)]


def pair_desc(enumerator: int = 0, linear_axis: int = 0, miller=(0, 0, 1), function: int = 0, axis: int = 0,
              num_bins: int = 10, max_r: float = 1.0, focal=(0.0, 0.0, 0.0), primary=(0.0, 0.0, 1.0),
              secondary=(1.0, 0.0, 0.0)) -> PairDesc:
    return PairDesc(enumerator, linear_axis, (C.c_int32 * 3)(*miller), function, axis, num_bins, 0, 0, max_r,
                    (C.c_double * 3)(*focal), (C.c_double * 3)(*primary), (C.c_double * 3)(*secondary))


def _corr_lib():
    lib, _ = _lib("oracle")
    if not getattr(lib, "_corr_bound", False):
        PD = C.POINTER(PairDesc)
        sig = {"rpo_corr_create": (_P, [PD]), "rpo_corr_destroy": (None, [_P]),
               "rpo_corr_add_snapshot": (C.c_int, [_P, C.c_int64, _D, _D, _D]),
               "rpo_corr_consume": (None, [_P, C.c_int64, C.c_int64, _D, C.c_double]),
               "rpo_corr_renormalize": (None, [_P, _D]), "rpo_corr_next_snapshot": (None, [_P]),
               "rpo_corr_dividers": (None, [_P, _D]),
               "rpo_corr_dump": (None, [_P, _D, _D, C.POINTER(C.c_uint64)]),
               "rpo_enumerate_pairs": (C.c_int64, [PD, C.c_int64, _D, _D, _D, C.c_int64, _I64, _D]),
               "rpo_expected_in_shells": (C.c_int, [PD, C.c_int64, _D, _D, C.c_int, _D]),
               "rpo_axis_function": (C.c_double, [C.c_int, _D, _D, _D]),
               "rpo_pair_counts": (None, [PD, C.c_int64, _D, _D, _D, C.c_int, C.POINTER(C.c_uint64)])}
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        lib._corr_bound = True
    return lib


def _state(pos, rot, box):
    p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    r = np.ascontiguousarray(rot, dtype=np.float64).reshape(-1, 9)
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    return p, r, b


class OracleCorrelation:
    """PairDensityCorrelation (function 0) or PairAveragedCorrelation (functions 1-4:
    S110, S220, S221, AxesAngle) restated single-threaded in oracle/rpo_correlation.hpp."""

    def __init__(self, desc: PairDesc):
        self.lib = _corr_lib()
        self.desc = desc
        self.h = self.lib.rpo_corr_create(C.byref(desc))
        if not self.h:
            raise ValueError("bad correlation description")

    def add_snapshot(self, pos, rot, box) -> None:
        p, r, b = _state(pos, rot, box)
        if self.lib.rpo_corr_add_snapshot(self.h, len(p), _dp(p), _dp(r), _dp(b)) != 0:
            raise ValueError("snapshot failed")

    def consume(self, i: int, j: int, d, value: float = 0.0) -> None:
        v = np.ascontiguousarray(d, dtype=np.float64)
        self.lib.rpo_corr_consume(self.h, i, j, _dp(v), value)

    def renormalize(self, factors) -> None:
        f = np.ascontiguousarray(factors, dtype=np.float64)
        self.lib.rpo_corr_renormalize(self.h, _dp(f))

    def next_snapshot(self) -> None:
        self.lib.rpo_corr_next_snapshot(self.h)

    def dividers(self) -> np.ndarray:
        out = np.zeros(self.desc.num_bins + 1)
        self.lib.rpo_corr_dividers(self.h, _dp(out))
        return out

    def values(self):
        nb = self.desc.num_bins
        x, y, c = np.zeros(nb), np.zeros(nb), np.zeros(nb, dtype=np.uint64)
        self.lib.rpo_corr_dump(self.h, _dp(x), _dp(y), c.ctypes.data_as(C.POINTER(C.c_uint64)))
        return x, y, c

    def close(self) -> None:
        if self.h:
            self.lib.rpo_corr_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def enumerate_pairs(desc: PairDesc, pos, rot, box):
    """Every (i, j, separation) an enumerator hands its consumer, in its order."""
    lib = _corr_lib()
    p, r, b = _state(pos, rot, box)
    n = len(p)
    cap = n * (n + 1) // 2
    ij, d = np.zeros((max(cap, 1), 2), dtype=np.int64), np.zeros((max(cap, 1), 3))
    k = lib.rpo_enumerate_pairs(C.byref(desc), n, _dp(p), _dp(r), _dp(b), cap,
                                ij.ctypes.data_as(_I64), _dp(d))
    return ij[:k], d[:k]


def pair_counts(desc: PairDesc, pos, rot, box, threads: int = 0) -> np.ndarray:
    """One snapshot's bin counts (the density correlation's pairs i < j, the averaged ones'
    i <= j), the rows shared among threads (0: all cores)."""
    lib = _corr_lib()
    p, r, b = _state(pos, rot, box)
    out = np.zeros(desc.num_bins, dtype=np.uint64)
    lib.rpo_pair_counts(C.byref(desc), len(p), _dp(p), _dp(r), _dp(b), threads or (os.cpu_count() or 1),
                        out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return out


def expected_in_shells(desc: PairDesc, n: int, box, bounds) -> np.ndarray:
    lib = _corr_lib()
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    bd = np.ascontiguousarray(bounds, dtype=np.float64)
    out = np.zeros(max(len(bd) - 1, 0))
    lib.rpo_expected_in_shells(C.byref(desc), n, _dp(b), _dp(bd), len(bd), _dp(out))
    return out


def axis_function(f: int, a1, a2, d) -> float:
    lib = _corr_lib()
    v = [np.ascontiguousarray(x, dtype=np.float64) for x in (a1, a2, d)]
    return lib.rpo_axis_function(f, *[_dp(x) for x in v])


def ref_named_point(kind: int, params, name: str) -> np.ndarray:
    """ShapeGeometry::getNamedPoint of the reference's own traits."""
    lib, _ = _lib("reference")
    lib.ref_named_point.restype = C.c_int
    lib.ref_named_point.argtypes = [C.c_int, _D, C.c_int, C.c_char_p, _D]
    prm = np.ascontiguousarray(params, dtype=np.float64)
    out = np.zeros(3)
    if lib.ref_named_point(kind, _dp(prm), len(prm), name.encode(), _dp(out)) != 0:
        raise KeyError(name)
    return out


def ref_pair_correlation(kind: int, params, states, desc: PairDesc, focal_name: str = "o",
                         primary=None, secondary=None):
    """The reference's own PairDensityCorrelation / PairAveragedCorrelation over its
    enumerators: one addSnapshot per (pos, rot, box) state, then print(), parsed at full
    precision.  Polysphere axes come from `primary` / `secondary` (body frame)."""
    lib, _ = _lib("reference")
    lib.ref_pair_correlation.restype = C.c_int
    lib.ref_pair_correlation.argtypes = [C.c_int, _D, C.c_int, _D, _D, C.c_int64, C.c_int, _D, _D, _D, C.c_int,
                                         C.c_int, C.POINTER(C.c_int), C.c_char_p, C.c_int, C.c_int, C.c_double,
                                         C.c_int, _D, _D, C.POINTER(C.c_uint64)]
    prm = np.ascontiguousarray(params, dtype=np.float64)
    n = len(np.asarray(states[0][0]).reshape(-1, 3))
    pos = np.ascontiguousarray(np.concatenate([np.asarray(s[0]).reshape(-1) for s in states]), dtype=np.float64)
    rot = np.ascontiguousarray(np.concatenate([np.asarray(s[1]).reshape(-1) for s in states]), dtype=np.float64)
    box = np.ascontiguousarray(np.concatenate([np.asarray(s[2]).reshape(-1) for s in states]), dtype=np.float64)
    a1 = None if primary is None else _dp(np.ascontiguousarray(primary, dtype=np.float64))
    a2 = None if secondary is None else _dp(np.ascontiguousarray(secondary, dtype=np.float64))
    nb = desc.num_bins
    x, y, c = np.zeros(nb), np.zeros(nb), np.zeros(nb, dtype=np.uint64)
    mil = (C.c_int * 3)(*desc.miller)
    got = lib.ref_pair_correlation(kind, _dp(prm), len(prm), a1, a2, n, len(states), _dp(pos), _dp(rot), _dp(box),
                                   desc.enumerator, desc.linear_axis, mil, focal_name.encode(), desc.function,
                                   desc.axis, desc.max_r, nb, _dp(x), _dp(y), c.ctypes.data_as(C.POINTER(C.c_uint64)))
    if got != nb:
        raise ValueError(f"reference correlation failed ({got})")
    return x, y, c
