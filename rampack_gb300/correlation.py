"""Pair correlations of a packing, built on the GPU through the C ABI.

The Python face of ``rp_correlation_*`` (rampack_gb300/csrc/rp_correlation.cu), mirroring
the reference's observables of core/observables/correlation and correlation_functions:

* enumerators: ``RadialEnumerator`` (RadialEnumerator.h:15-40), ``LinearEnumerator``
  (LinearEnumerator.h:16-60) and ``LayerwiseRadialEnumerator``
  (LayerwiseRadialEnumerator.h:19-50), each measuring from a named point of the shape;
* correlation functions ``S110Correlation``, ``S220Correlation``, ``S221Correlation`` and
  ``AxesAngle`` over the primary, secondary or auxiliary axis;
* observables ``PairDensityCorrelation`` (PairDensityCorrelation.h:22-80) and
  ``PairAveragedCorrelation`` (PairAveragedCorrelation.h:21-75) with ``add_snapshot``,
  ``print``, ``clear`` and the reference's signature names.

Bin counts are the reference's exactly; the density correlation's values too (they are
counts times the reference's normalisation).  The averaged correlations' values are sums
in another order than the reference's serial loop, equal to rounding.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import EngineError, PairDesc, dptr

_AXES = {"primary": _lib.AXIS_PRIMARY, "secondary": _lib.AXIS_SECONDARY, "auxiliary": _lib.AXIS_AUXILIARY}


def _normalized(v) -> tuple:
    """Vector::normalized (geometry/Vector.h:225-228): v / |v|, a divisor of 1 skipped."""
    x, y, z = (float(a) for a in v)
    n = math.sqrt(((0.0 + x * x) + y * y) + z * z)
    return (x, y, z) if n == 1.0 else (x / n, y / n, z / n)


def named_point(kind: int, params, name: str) -> tuple:
    """ShapeGeometry::getNamedPoint (core/ShapeGeometry.cpp:16-24) of this engine's shapes, in
    the body frame: "o" the geometric origin ({0, 0, 0} for all three), "cm" of spheres and
    spherocylinders (SphereTraits.cpp:19, SpherocylinderTraits.cpp:18), the spherocylinder
    cap centres "beg" / "end" ({0, 0, -+l/2}, SpherocylinderTraits.cpp:19-26) and the
    polysphere centres "s<i>" (PolysphereTraits.cpp:185-188)."""
    params = np.asarray(params, dtype=np.float64).reshape(-1)
    if name == "o":
        return (0.0, 0.0, 0.0)
    if kind in (_lib.SHAPE_SPHERE, _lib.SHAPE_SPHEROCYLINDER) and name == "cm":
        return (0.0, 0.0, 0.0)
    if kind == _lib.SHAPE_SPHEROCYLINDER and name in ("beg", "end"):
        s = 0.5 * (-1.0 if name == "beg" else 1.0) * float(params[0])
        if s == 1.0:
            return (0.0, 0.0, 1.0)
        return (0.0 + 0.0 * s, 0.0 + 0.0 * s, 0.0 + 1.0 * s)
    if kind == _lib.SHAPE_POLYSPHERE and name.startswith("s") and name[1:].isdigit():
        i, k = int(name[1:]), int(params[0])
        if i < k:
            return tuple(float(x) for x in params[1 + 4 * i:4 + 4 * i])
    if kind == _lib.SHAPE_POLYSPHEROCYLINDER and name[:1] in ("o", "b", "e") and name[1:].isdigit():
        # "o<i>", "b<i>", "e<i>": centre, centre - half axis, centre + half axis of
        # spherocylinder i (PolyspherocylinderTraits.cpp:42-47)
        i, k = int(name[1:]), int(params[0])
        if i < k:
            d = [float(x) for x in params[1 + 7 * i:8 + 7 * i]]
            c, h = d[:3], d[3:6]
            if name[0] == "o":
                return tuple(c)
            return tuple(c[a] - h[a] for a in range(3)) if name[0] == "b" else tuple(c[a] + h[a] for a in range(3))
    raise EngineError(-1, f"ShapeGeometry::getNamedPoint : unknown point name '{name}'")


class _Enumerator:
    def __init__(self, focal_point="o"):
        self.focal_point = focal_point

    def _fill(self, d: PairDesc, kind: int, params) -> None:
        fp = self.focal_point
        d.focal = (C.c_double * 3)(*(named_point(kind, params, fp) if isinstance(fp, str) else fp))


class RadialEnumerator(_Enumerator):
    """Distances between the focal points (RadialEnumerator.cpp:9-29)."""
    signature_name = "r"

    def _fill(self, d, kind, params):
        super()._fill(d, kind, params)
        d.enumerator = _lib.PAIRS_RADIAL


class LinearEnumerator(_Enumerator):
    """Separations projected on the normal of the box faces across side x, y or z
    (LinearEnumerator.cpp:37-67)."""

    def __init__(self, axis: str, focal_point="o"):
        super().__init__(focal_point)
        if axis not in ("x", "y", "z"):
            raise EngineError(-1, f"unknown axis {axis!r}")
        self.axis = axis
        self.signature_name = axis

    def _fill(self, d, kind, params):
        super()._fill(d, kind, params)
        d.enumerator = _lib.PAIRS_LINEAR
        d.linear_axis = "xyz".index(self.axis)


class LayerwiseRadialEnumerator(_Enumerator):
    """In-layer distances of pairs in the same layer of the Miller-index planes
    (LayerwiseRadialEnumerator.cpp:18-46)."""
    signature_name = "lr"

    def __init__(self, miller_indices, focal_point="o"):
        super().__init__(focal_point)
        m = tuple(int(x) for x in miller_indices)
        if len(m) != 3 or not any(m):
            raise EngineError(-1, "Miller indices must have a nonzero entry")
        self.miller = m

    def _fill(self, d, kind, params):
        super()._fill(d, kind, params)
        d.enumerator = _lib.PAIRS_LAYERWISE
        d.miller = (C.c_int32 * 3)(*self.miller)


class _AxisCorrelation:
    code = 0
    signature_name = ""

    def __init__(self, axis: str = "primary", primary=None, secondary=None):
        """``axis`` is ShapeGeometry::Axis; ``primary`` / ``secondary`` give the body-frame
        axes of polyspheres (PolysphereGeometry, normalised as its constructor does);
        spherocylinders have the primary axis {0, 0, 1} (SpherocylinderTraits.cpp:52-54)."""
        if axis not in _AXES:
            raise EngineError(-1, f"unknown axis {axis!r}")
        self.axis = axis
        self.primary, self.secondary = primary, secondary

    def _fill(self, d: PairDesc, kind: int) -> None:
        d.function = self.code
        d.axis = _AXES[self.axis]
        prim, sec = self.primary, self.secondary
        if kind == _lib.SHAPE_SPHEROCYLINDER:
            prim = (0.0, 0.0, 1.0) if prim is None else prim
            if self.axis != "primary" and sec is None:
                raise EngineError(-5, "ShapeGeometry::getSecondaryAxis : unsupported")
        elif kind == _lib.SHAPE_SPHERE:
            raise EngineError(-5, "ShapeGeometry::getPrimaryAxis : unsupported")
        else:
            if prim is None:
                raise EngineError(-5, "PolysphereGeometry::getPrimaryAxis: primary axis not defined")
            if self.axis != "primary" and sec is None:
                raise EngineError(-5, "PolysphereGeometry::getSecondaryAxis: secondary axis not defined")
            prim = _normalized(prim)
            sec = None if sec is None else _normalized(sec)
        d.primary = (C.c_double * 3)(*prim)
        if sec is not None:
            d.secondary = (C.c_double * 3)(*sec)


class S110Correlation(_AxisCorrelation):
    """a1 . a2 (S110Correlation.h)."""
    code, signature_name = _lib.CORR_S110, "S110"


class S220Correlation(_AxisCorrelation):
    """3/2 ((a1 . a2)^2 - 1/3) (S220Correlation.h)."""
    code, signature_name = _lib.CORR_S220, "S220"


class S221Correlation(_AxisCorrelation):
    """((a1 ^ a2) . r/|r|) (a1 . a2) (S221Correlation.h)."""
    code, signature_name = _lib.CORR_S221, "S221"


class AxesAngle(_AxisCorrelation):
    """The angle between the axes in degrees, 180 acos|a1 . a2| / pi (AxesAngle.h)."""
    code, signature_name = _lib.CORR_AXES_ANGLE, "theta"


def _cpp_format(v: float) -> str:
    """std::ostream's default formatting of a double (%g, 6 significant digits)."""
    if math.isnan(v):
        return "-nan" if math.copysign(1.0, v) < 0 else "nan"
    return f"{v:g}"


class _PairObservable:
    def __init__(self, enumerator, function, max_r: float, num_bins: int, print_count: bool, flags: int):
        self.lib = _lib.load()
        self.enumerator, self.function = enumerator, function
        self.max_r, self.num_bins, self.print_count = float(max_r), int(num_bins), print_count
        self.flags = int(flags)
        self.h = None
        self._shape = None

    def _create(self, packing) -> None:
        shape = (packing.kind, tuple(np.asarray(packing.params, dtype=np.float64).reshape(-1)))
        if self.h is not None:
            if shape != self._shape:
                raise EngineError(-1, "snapshots of another shape")
            return
        d = PairDesc()
        d.num_bins, d.max_r, d.flags = self.num_bins, self.max_r, self.flags
        d.primary = (C.c_double * 3)(0.0, 0.0, 1.0)
        d.secondary = (C.c_double * 3)(1.0, 0.0, 0.0)
        self.enumerator._fill(d, packing.kind, packing.params)
        if self.function is not None:
            self.function._fill(d, packing.kind)
        h = C.c_void_p()
        rc = self.lib.rp_correlation_create(C.byref(d), C.byref(h))
        if rc != 0:
            raise EngineError(rc, "rp_correlation_create: invalid description")
        self.h, self._shape, self.desc = h, shape, d

    def _check(self, rc: int) -> None:
        if rc != 0:
            msg = self.lib.rp_correlation_last_error(self.h)
            raise EngineError(rc, msg.decode() if msg else "")

    def add_snapshot(self, packing, temperature: float = 1.0, pressure: float = 1.0) -> None:
        """BulkObservable::addSnapshot on the packing's current state (GPU)."""
        self._create(packing)
        self._check(self.lib.rp_correlation_add_snapshot(self.h, packing.h))

    def values(self):
        """HistogramBuilder::dumpValues: bin middles, values and accumulated counts."""
        nb = self.num_bins
        x, y, c = np.zeros(nb), np.zeros(nb), np.zeros(nb, dtype=np.uint64)
        if self.h is None:
            step = self.max_r / nb
            return np.array([0.0 + (b + 0.5) * step for b in range(nb)]), y, c
        self._check(self.lib.rp_correlation_values(self.h, dptr(x), dptr(y), c.ctypes.data_as(C.POINTER(C.c_uint64))))
        return x, y, c

    def last_snapshot(self):
        """The last snapshot's raw bins: pair counts and value sums."""
        nb = self.num_bins
        c, s = np.zeros(nb, dtype=np.uint64), np.zeros(nb)
        self._check(self.lib.rp_correlation_last_snapshot(self.h, c.ctypes.data_as(C.POINTER(C.c_uint64)), dptr(s)))
        return c, s

    def info(self) -> dict:
        snaps, tested = C.c_int64(), C.c_int64()
        if self.h is None:
            return {"snapshots": 0, "pairs_tested": 0}
        self._check(self.lib.rp_correlation_info(self.h, C.byref(snaps), C.byref(tested)))
        return {"snapshots": snaps.value, "pairs_tested": tested.value}

    def print(self) -> str:
        """print(): "distance value [count]" per bin, as the reference's stream output."""
        x, y, c = self.values()
        lines = []
        for xi, yi, ci in zip(x, y, c):
            s = f"{_cpp_format(xi)} {_cpp_format(yi)}"
            if self.print_count:
                s += f" {int(ci)}"
            lines.append(s + "\n")
        return "".join(lines)

    def clear(self) -> None:
        if self.h is not None:
            self._check(self.lib.rp_correlation_clear(self.h))

    def close(self) -> None:
        if self.h is not None:
            self.lib.rp_correlation_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PairDensityCorrelation(_PairObservable):
    """Pair density correlation g(r): bin counts over the expected counts of a homogeneous
    packing, averaged over snapshots (PairDensityCorrelation.cpp:4-37)."""

    def __init__(self, enumerator, max_r: float, num_bins: int, print_count: bool = False, *, flags: int = 0):
        """``flags``: ``CORR_ALL_PAIRS`` / ``CORR_FP64_ONLY`` of rampack_gb300._lib (results unchanged)."""
        super().__init__(enumerator, None, max_r, num_bins, print_count, flags)

    @property
    def signature_name(self) -> str:
        return "rho_" + self.enumerator.signature_name


class PairAveragedCorrelation(_PairObservable):
    """A correlation function averaged over all pairs in each distance bin
    (PairAveragedCorrelation.cpp:4-31)."""

    def __init__(self, enumerator, function, max_r: float, num_bins: int, print_count: bool = False, *,
                 flags: int = 0):
        super().__init__(enumerator, function, max_r, num_bins, print_count, flags)

    @property
    def signature_name(self) -> str:
        return self.function.signature_name + "_" + self.enumerator.signature_name
