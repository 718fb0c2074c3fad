"""ctypes binding of the C ABI declared in include/rampack_gb300.h.

The shared library is built in-tree (``rampack_gb300/build.py``).  There is no
fallback: when the library is missing or cannot be loaded, importing the engine
raises, so no CPU path can stand in for the GPU one.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librampack_gb300.so")

RP_OK = 0
ERRORS = {
    -1: "RP_ERR_ARG", -2: "RP_ERR_CUDA", -3: "RP_ERR_STATE", -4: "RP_ERR_OVERLAP",
    -5: "RP_ERR_UNSUPPORTED", -6: "RP_ERR_DEVICE", -7: "RP_ERR_CAPACITY", -8: "RP_ERR_FORMAT", -9: "RP_ERR_IO",
}
SHAPE_SPHERE, SHAPE_SPHEROCYLINDER, SHAPE_POLYSPHERE = 0, 1, 2
# creation kind of polyspherocylinders (the handle then runs as a multi-centre body)
SHAPE_POLYSPHEROCYLINDER = 3
SHAPE_CONVEX = 4      # generic convex body (rp_create_convex): params is the XCBodyBuilder script
MAX_CENTRES = 8
MOVE_TRANSLATION, MOVE_ROTATION, MOVE_ROTOTRANSLATION = 0, 1, 2
CODE_ACCEPTED = 0x80
SWEEP_LOG, SWEEP_FP64_ONLY, SWEEP_ROTOTRANSLATION = 1, 2, 4

MOVE_DTYPE = np.dtype([
    ("particle", "<i4"), ("type", "<i4"), ("domain", "<i4"), ("reserved", "<i4"),
    ("translation", "<f8", (3,)), ("rotation", "<f8", (9,)), ("uniform", "<f8"),
])
assert MOVE_DTYPE.itemsize == 120


class ShapeDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("radius", C.c_double), ("length", C.c_double)]


class GridInfo(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("max_occupancy", C.c_int32), ("shift", C.c_double * 3),
                ("cell_height", C.c_double * 3), ("num_cells", C.c_int64)]


class SweepParams(C.Structure):
    _fields_ = [("translation_step", C.c_double), ("rotation_step", C.c_double), ("seed", C.c_uint64),
                ("counter", C.c_uint64), ("flags", C.c_int32), ("reserved", C.c_int32)]


class SweepStats(C.Structure):
    _fields_ = [("moves", C.c_uint64), ("accepted", C.c_uint64), ("rejected_overlap", C.c_uint64),
                ("rejected_domain", C.c_uint64), ("pair_tests", C.c_uint64), ("fp64_pairs", C.c_uint64),
                ("translations", C.c_uint64), ("rotations", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("accepted_translations", C.c_uint64)]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


class BoxScalerDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("scale_together", C.c_int32), ("num_groups", C.c_int32),
                ("groups", C.c_int32 * 3), ("independent", C.c_int32), ("reserved", C.c_int32), ("step", C.c_double)]


class SimParams(C.Structure):
    _fields_ = [("temperature", C.c_double), ("pressure", C.c_double), ("translation_step", C.c_double),
                ("rotation_step", C.c_double), ("scaler", BoxScalerDesc), ("seed", C.c_uint64),
                ("rototranslation", C.c_int32), ("reserved", C.c_int32)]


class PairDesc(C.Structure):
    """rp_pair_desc: one pair-correlation observable."""
    _fields_ = [("enumerator", C.c_int32), ("linear_axis", C.c_int32), ("miller", C.c_int32 * 3),
                ("function", C.c_int32), ("axis", C.c_int32), ("num_bins", C.c_int32), ("flags", C.c_int32),
                ("reserved", C.c_int32), ("max_r", C.c_double),
                ("focal", C.c_double * 3), ("primary", C.c_double * 3), ("secondary", C.c_double * 3)]


PAIRS_RADIAL, PAIRS_LINEAR, PAIRS_LAYERWISE = 0, 1, 2
CORR_DENSITY, CORR_S110, CORR_S220, CORR_S221, CORR_AXES_ANGLE = 0, 1, 2, 3, 4
AXIS_PRIMARY, AXIS_SECONDARY, AXIS_AUXILIARY = 0, 1, 2
CORR_MAX_BINS = 65536
CORR_ALL_PAIRS, CORR_FP64_ONLY = 1, 2


class SimStats(C.Structure):
    _fields_ = [("cycles", C.c_uint64), ("translations", C.c_uint64), ("accepted_translations", C.c_uint64),
                ("rotations", C.c_uint64), ("accepted_rotations", C.c_uint64), ("box_moves", C.c_uint64),
                ("accepted_box_moves", C.c_uint64), ("translation_step", C.c_double), ("rotation_step", C.c_double),
                ("box_step", C.c_double), ("box", C.c_double * 9), ("move_ms", C.c_double),
                ("scaling_ms", C.c_double)]

    def as_dict(self) -> dict:
        out = {name: getattr(self, name) for name, _ in self._fields_}
        out["box"] = np.array(list(self.box))
        return out


SCALER_NONE, SCALER_DELTA_TRICLINIC, SCALER_LOG, SCALER_LINEAR, SCALER_DELTA_VOLUME = 0, 1, 2, 3, 4

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)

# name -> (restype, argtypes); every function declared in include/rampack_gb300.h
SIGNATURES = {
    "rp_create": (C.c_int, [C.POINTER(ShapeDesc), C.c_int64, C.c_int, C.POINTER(C.c_void_p)]),
    "rp_create_polysphere": (C.c_int, [C.c_int32, _D, _D, C.c_int64, C.c_int, C.POINTER(C.c_void_p)]),
    "rp_create_polyspherocylinder": (C.c_int, [C.c_int32, _D, _D, _D, C.c_int64, C.c_int, C.POINTER(C.c_void_p)]),
    "rp_create_convex": (C.c_int, [C.c_char_p, C.c_int64, C.c_int, C.POINTER(C.c_void_p)]),
    "rp_convex_pair_overlaps": (C.c_int, [_P, C.c_int64, _D, _D, _D, _D, C.POINTER(C.c_uint8)]),
    "rp_destroy": (C.c_int, [_P]),
    "rp_last_error": (C.c_char_p, [_P]),
    "rp_upload_state": (C.c_int, [_P, _D, _D, _D]),
    "rp_download_state": (C.c_int, [_P, _D, _D, _D]),
    "rp_count_overlaps": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int64)]),
    "rp_set_grid": (C.c_int, [_P, _D, C.POINTER(GridInfo)]),
    "rp_get_grid": (C.c_int, [_P, C.POINTER(GridInfo), C.POINTER(C.c_int32), _D]),
    "rp_run_moves": (C.c_int, [_P, _P, C.c_int64, _P]),
    "rp_try_move": (C.c_int, [_P, _P, _D, _D]),
    "rp_set_cells_per_warp": (C.c_int, [_P, C.c_int32]),
    "rp_set_bulk_staging": (C.c_int, [_P, C.c_int32]),
    "rp_set_cell_order": (C.c_int, [_P, C.c_int32]),
    "rp_set_soft": (C.c_int, [_P, C.c_int32, C.c_double, C.c_double, C.c_int32]),
    "rp_set_temperature": (C.c_int, [_P, C.c_double]),
    "rp_total_energy": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "rp_get_cells_per_warp": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "rp_accept_move": (C.c_int, [_P]),
    "rp_sweep": (C.c_int, [_P, C.POINTER(SweepParams), C.POINTER(SweepStats)]),
    "rp_sweep_log": (C.c_int, [_P, _P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "rp_try_scaling": (C.c_int, [_P, _D, _D]),
    "rp_revert_scaling": (C.c_int, [_P]),
    "rp_get_stats": (C.c_int, [_P, C.POINTER(SweepStats)]),
    "rp_get_grid_counters": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "rp_get_stream": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "rp_set_timing": (C.c_int, [_P, C.c_int]),
    "rp_get_timing": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "rp_count_overlaps_static": (C.c_int, [C.POINTER(ShapeDesc), C.c_int64, _P, _P, _D, C.c_int, _P,
                                           C.POINTER(C.c_int64)]),
    "rp_mlp_init": (C.c_int, [_P, C.c_uint64]),
    "rp_mlp_set_params": (C.c_int, [_P, _F]),
    "rp_mlp_get_params": (C.c_int, [_P, _F]),
    "rp_mlp_predict": (C.c_int, [_P, _F, C.c_int64, _F]),
    "rp_mlp_gradient": (C.c_int, [_P, _F, _P, C.c_int64, _F, _F]),
    "rp_pair_log_enable": (C.c_int, [_P, C.c_int64, C.c_int32]),
    "rp_pair_log_read": (C.c_int, [_P, _F, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "rp_pair_log_clear": (C.c_int, [_P]),
    "rp_mlp_train": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_float, C.c_uint64, _F]),
    "rp_set_ordering": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "rp_renormalize_orientations": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int64)]),
    "rp_nematic_order": (C.c_int, [_P, _D, _D]),
    "rp_set_counting": (C.c_int, [_P, C.c_int]),
    "rp_cached_overlaps": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "rp_batch_create": (C.c_int, [C.POINTER(ShapeDesc), C.c_int32, C.POINTER(C.c_int64), C.c_int,
                                  C.POINTER(C.c_void_p)]),
    "rp_batch_destroy": (C.c_int, [_P]),
    "rp_batch_last_error": (C.c_char_p, [_P]),
    "rp_batch_upload_state": (C.c_int, [_P, C.c_int32, _D, _D, _D]),
    "rp_batch_download_state": (C.c_int, [_P, C.c_int32, _D, _D, _D]),
    "rp_batch_count_overlaps": (C.c_int, [_P, C.c_int32, C.c_int, C.POINTER(C.c_int64)]),
    "rp_batch_get_grid": (C.c_int, [_P, C.c_int32, C.POINTER(GridInfo), C.POINTER(C.c_int32), _D]),
    "rp_batch_sweep_log": (C.c_int, [_P, C.c_int32, _P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "rp_batch_sweep": (C.c_int, [_P, C.POINTER(SweepParams), C.POINTER(SweepStats)]),
    "rp_batch_try_scaling": (C.c_int, [_P, _D, _P, _D]),
    "rp_batch_revert_scaling": (C.c_int, [_P, _P]),
    "rp_batch_set_tuning": (C.c_int, [_P, C.c_double, C.c_int32]),
    "rp_batch_upload_states": (C.c_int, [_P, _D, _D, _D]),
    "rp_batch_download_states": (C.c_int, [_P, _D, _D, _D]),
    "rp_batch_set_timing": (C.c_int, [_P, C.c_int]),
    "rp_batch_get_timing": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "rp_set_staging_filter": (C.c_int, [_P, C.c_int32]),
    "rp_set_walls": (C.c_int, [_P, C.c_int32]),
    "rp_batch_set_walls": (C.c_int, [_P, C.c_int32]),
    "rp_batch_set_staging_filter": (C.c_int, [_P, C.c_int32]),
    "rp_sim_create": (C.c_int, [_P, C.POINTER(SimParams), C.POINTER(C.c_void_p)]),
    "rp_sim_run": (C.c_int, [_P, C.c_int64, C.c_int, C.POINTER(SimStats)]),
    "rp_sim_get_stats": (C.c_int, [_P, C.POINTER(SimStats)]),
    "rp_sim_set_steps": (C.c_int, [_P, C.c_double, C.c_double, C.c_double]),
    "rp_sim_set_conditions": (C.c_int, [_P, C.c_double, C.c_double]),
    "rp_sim_set_cycles": (C.c_int, [_P, C.c_uint64]),
    "rp_sim_last_error": (C.c_char_p, [_P]),
    "rp_sim_destroy": (C.c_int, [_P]),
    "rp_box_proposals": (C.c_int, [C.POINTER(BoxScalerDesc), C.c_uint64, _D, C.c_int64, _D, _D]),
    "rp_io_last_error": (C.c_char_p, []),
    "rp_ramsnap_write": (C.c_int, [_P, C.c_char_p, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p)]),
    "rp_ramsnap_write_host": (C.c_int, [C.c_char_p, C.c_int64, _D, _D, _D, C.c_int32, C.POINTER(C.c_char_p),
                                        C.POINTER(C.c_char_p)]),
    "rp_ramsnap_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "rp_ramsnap_info": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "rp_ramsnap_get": (C.c_int, [_P, _D, _D, _D]),
    "rp_ramsnap_aux": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p)]),
    "rp_ramsnap_free": (C.c_int, [_P]),
    "rp_ramtrj_open": (C.c_int, [C.c_char_p, C.c_int64, C.c_int64, C.c_int, C.POINTER(C.c_void_p)]),
    "rp_ramtrj_record": (C.c_int, [_P, _P, C.c_int64]),
    "rp_ramtrj_record_host": (C.c_int, [_P, _D, _D, _D, C.c_int64]),
    "rp_ramtrj_flush": (C.c_int, [_P]),
    "rp_ramtrj_snapshots": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "rp_ramtrj_close": (C.c_int, [_P]),
    "rp_ramtrj_info": (C.c_int, [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int32)]),
    "rp_ramtrj_read": (C.c_int, [C.c_char_p, C.c_int64, _D, _D, _D]),
    "rp_correlation_create": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "rp_correlation_add_snapshot": (C.c_int, [_P, _P]),
    "rp_correlation_values": (C.c_int, [_P, _D, _D, C.POINTER(C.c_uint64)]),
    "rp_correlation_last_snapshot": (C.c_int, [_P, C.POINTER(C.c_uint64), _D]),
    "rp_correlation_info": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "rp_correlation_clear": (C.c_int, [_P]),
    "rp_correlation_last_error": (C.c_char_p, [_P]),
    "rp_correlation_destroy": (C.c_int, [_P]),
}
KERNEL_GROUPS = ["sweep", "rebuild", "count", "rescale", "overflow", "order", "mlp", "fix", "single"]
MLP_NPARAM = 5313
MLP_FEATURES = 16
ORDER_OFF, ORDER_MLP, ORDER_DISTANCE = 0, 1, 2
SOFT_NONE, SOFT_REPULSIVE_LJ, SOFT_SQUARE_INVERSE_CORE, SOFT_LENNARD_JONES = 0, 1, 2, 3
BATCH_SEED_STRIDE = 0x9E3779B97F4A7C15

_LIB = None


def load(path: str | None = None):
    """Loads the engine library (once) and declares every entry point."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"rampack_gb300: CUDA library not built ({p}); run rampack_gb300/build.py")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    _LIB = lib
    return lib


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_F)
