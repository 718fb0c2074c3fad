"""The Monte Carlo driver around a GpuPacking: the reference's Simulation for hard bodies.

``Simulation.integrate`` follows ``Simulation::integrate`` (core/Simulation.cpp:93-200):
a thermalisation phase whose step sizes adapt (``Simulation::evaluateCounters``), then an
averaging phase sampling observables every ``averaging_every`` cycles, the averages with the
standard error of ``Quantity::calculateFromSamples`` (utils/Quantity.cpp:45-61); snapshots go
to an optional ``RamtrjRecorder``.  Each cycle is one device sweep plus one box move whose
proposal comes from the reference's box scalers with a std::mt19937 (``rp_sim_*``, native
loop in rampack_gb300/csrc/rp_sim.cu).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import BoxScalerDesc, EngineError, SimParams, SimStats, dptr

AXES = {"x": 1, "y": 2, "z": 4}


def _groups(spec) -> list[int]:
    out = []
    for g in spec:
        m = 0
        for a in g:
            m |= AXES[a]
        out.append(m)
    return out


def delta_triclinic(step: float, scale_together: bool = True) -> BoxScalerDesc:
    """TriclinicDeltaScaler(step, scaleTogether)."""
    return BoxScalerDesc(kind=_lib.SCALER_DELTA_TRICLINIC, scale_together=1 if scale_together else 0, step=step)


def _volume(kind: int, step: float, groups, independent: bool) -> BoxScalerDesc:
    g = _groups(groups)
    if not 1 <= len(g) <= 3:
        raise ValueError("one to three scaling directions")
    d = BoxScalerDesc(kind=kind, num_groups=len(g), independent=1 if independent else 0, step=step)
    for i, m in enumerate(g):
        d.groups[i] = m
    return d


def log_volume(step: float, groups=("xyz",), independent: bool = False) -> BoxScalerDesc:
    """TriclinicAdapter(AnisotropicVolumeScaler(LogScalingFactorSampler, directions)); each
    group ("xyz", "xy", "z", ...) is one direction scaled by one factor (X & Y & Z ...), groups
    joined by |."""
    return _volume(_lib.SCALER_LOG, step, groups, independent)


def linear_volume(step: float, groups=("xyz",), independent: bool = False) -> BoxScalerDesc:
    """As log_volume with LinearScalingFactorSampler."""
    return _volume(_lib.SCALER_LINEAR, step, groups, independent)


def delta_volume(step: float) -> BoxScalerDesc:
    """TriclinicAdapter(DeltaVolumeScaler)."""
    return BoxScalerDesc(kind=_lib.SCALER_DELTA_VOLUME, step=step)


def box_proposals(scaler: BoxScalerDesc, seed: int, box, count: int):
    """(boxes [count, 9], uniforms [count]): the proposals and Metropolis draws
    Simulation::tryScaling takes from std::mt19937(seed), every one from ``box``."""
    lib = _lib.load()
    b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
    boxes, u = np.zeros((count, 9)), np.zeros(count)
    rc = lib.rp_box_proposals(C.byref(scaler), seed, dptr(b), count, dptr(boxes), dptr(u))
    if rc != 0:
        raise EngineError(rc, "rp_box_proposals: invalid scaler")
    return boxes, u


def quantity(samples) -> tuple[float, float]:
    """Quantity::calculateFromSamples: the mean and its standard error."""
    x = [float(v) for v in samples]
    if not x:
        return 0.0, 0.0
    if len(x) == 1:
        return x[0], 0.0
    # std::accumulate order (plain left-to-right sums; Python's sum() compensates)
    total = 0.0
    for v in x:
        total += v
    mean = total / len(x)
    err = 0.0
    for v in x:
        err += (mean - v) ** 2
    return mean, math.sqrt(err / len(x) / (len(x) - 1))


def box_volume(box) -> float:
    """TriclinicBox::getVolume (core/TriclinicBox.cpp:35-38): |(s0 ^ s1) * s2| of the box
    sides (the matrix columns), in the reference's operation order."""
    b = [float(x) for x in np.asarray(box).reshape(9)]
    s0, s1, s2 = (b[0], b[3], b[6]), (b[1], b[4], b[7]), (b[2], b[5], b[8])
    c = (s0[1] * s1[2] - s0[2] * s1[1], s0[2] * s1[0] - s0[0] * s1[2], s0[0] * s1[1] - s0[1] * s1[0])
    d = 0.0
    for k in range(3):
        d += c[k] * s2[k]
    return abs(d)


def shape_volume(kind: int, params) -> float:
    """SphereTraits::getVolume / SpherocylinderTraits::getVolume
    (core/shapes/SphereTraits.cpp:31-33, SpherocylinderTraits.cpp:48-50)."""
    p = np.asarray(params, dtype=np.float64).reshape(-1)
    if kind == _lib.SHAPE_SPHERE:
        return 4. / 3 * math.pi * math.pow(float(p[0]), 3)
    if kind == _lib.SHAPE_SPHEROCYLINDER:
        r, length = float(p[1]), float(p[0])
        return math.pi * r * r * length + 4. / 3 * math.pi * math.pow(r, 3)
    if kind == _lib.SHAPE_POLYSPHEROCYLINDER:
        # PolyspherocylinderGeometry::calculateVolume (PolyspherocylinderTraits.cpp:12-20) for
        # non-overlapping spherocylinders: the sum of SpherocylinderData::getVolume (:86-91)
        volume = 0.0
        for i in range(int(p[0])):
            d = p[1 + 7 * i:8 + 7 * i]
            r = float(d[6])
            half = math.sqrt(((0.0 + d[3] * d[3]) + d[4] * d[4]) + d[5] * d[5])
            r2 = r * r
            volume = volume + (4 * math.pi / 3 * (r2 * r) + math.pi * r2 * (2 * half))
        return volume
    raise ValueError("the volume of this shape kind is not restated")


def number_density(packing, stats) -> float:
    """NumberDensity (core/observables/NumberDensity.h): N / V (Packing::getNumberDensity)."""
    return packing.n / box_volume(stats["box"])


def packing_fraction(packing, stats) -> float:
    """PackingFraction (core/observables/PackingFraction.h): number density x shape volume."""
    return number_density(packing, stats) * shape_volume(packing.kind, packing.params)


def nematic_order(packing, stats) -> float:
    return packing.nematic_order()[1]


OBSERVABLES = {"number_density": number_density, "packing_fraction": packing_fraction,
               "nematic_order": nematic_order}


class Simulation:
    """Simulation(packing, translationStep, rotationStep, seed, boxScaler) for hard bodies."""

    def __init__(self, packing, translation_step: float, rotation_step: float, seed: int,
                 scaler: BoxScalerDesc | None = None, rototranslation: bool = False):
        """TranslationSampler + RotationSampler (a step of 0 disables one), or with
        ``rototranslation`` one RototranslationSampler(translation_step, rotation_step)."""
        self.lib = _lib.load()
        self.packing = packing
        self.translation_step, self.rotation_step = translation_step, rotation_step
        self.rototranslation = rototranslation
        self.has_scaler = scaler is not None and scaler.kind != _lib.SCALER_NONE
        p = SimParams(temperature=1.0, pressure=0.0, translation_step=translation_step, rotation_step=rotation_step,
                      seed=seed, rototranslation=1 if rototranslation else 0)
        if scaler is not None:
            p.scaler = scaler
        self.h = C.c_void_p()
        rc = self.lib.rp_sim_create(packing.h, C.byref(p), C.byref(self.h))
        if rc != 0:
            raise EngineError(rc, "rp_sim_create failed (a packing with a state and valid parameters are needed)")

    def _check(self, rc: int):
        if rc != 0:
            msg = self.lib.rp_sim_last_error(self.h)
            raise EngineError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.rp_sim_destroy(self.h)
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

    def set_conditions(self, temperature: float, pressure: float):
        self._check(self.lib.rp_sim_set_conditions(self.h, temperature, pressure))

    def set_steps(self, translation_step: float, rotation_step: float, box_step: float = 0.0):
        self._check(self.lib.rp_sim_set_steps(self.h, translation_step, rotation_step, box_step))

    def run(self, cycles: int, adjust_steps: bool = False) -> dict:
        """`cycles` cycles of Simulation::performCycle; the running totals and current steps."""
        st = SimStats()
        self._check(self.lib.rp_sim_run(self.h, int(cycles), 1 if adjust_steps else 0, C.byref(st)))
        return st.as_dict()

    def stats(self) -> dict:
        st = SimStats()
        self._check(self.lib.rp_sim_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    # ---- continuation (the reference's --continue through RAMSNAP aux entries) ----
    def aux_info(self) -> dict:
        """FileSnapshotWriter::prepareAuxInfo (frontend/FileSnapshotWriter.cpp:46-61):
        "cycles" and "step.<sampler>.<step>" entries, step sizes at max_digits10."""
        st = self.stats()
        aux = {"cycles": str(int(st["cycles"]))}
        if self.rototranslation:
            aux["step.rototranslation.translation"] = "%.17g" % st["translation_step"]
            aux["step.rototranslation.rotation"] = "%.17g" % st["rotation_step"]
        else:
            if self.translation_step > 0:
                aux["step.translation.translation"] = "%.17g" % st["translation_step"]
            if self.rotation_step > 0:
                aux["step.rotation.rotation"] = "%.17g" % st["rotation_step"]
        if self.has_scaler:
            aux["step.scaling.scaling"] = "%.17g" % st["box_step"]
        return aux

    def store(self, path) -> dict:
        """The packing as RAMSNAP with the aux entries a continued run needs."""
        aux = self.aux_info()
        self.packing.store(path, aux)
        return aux

    def restore(self, path) -> dict:
        """PackingLoader's continuation (frontend/PackingLoader.cpp:177-223): the state, the
        cycle count and the step sizes of a RAMSNAP file this packing's size."""
        aux = self.packing.restore(path)
        if "cycles" not in aux:
            raise EngineError(-8, "No 'cycles' key in RAMSNAP metadata")
        st = self.stats()
        t = float(aux.get("step.rototranslation.translation" if self.rototranslation else "step.translation.translation",
                          st["translation_step"]))
        r = float(aux.get("step.rototranslation.rotation" if self.rototranslation else "step.rotation.rotation",
                          st["rotation_step"]))
        b = float(aux.get("step.scaling.scaling", st["box_step"]))
        self.set_steps(t, r, b)
        self._check(self.lib.rp_sim_set_cycles(self.h, int(aux["cycles"])))
        return aux

    def integrate(self, temperature: float, pressure: float, thermalisation_cycles: int, averaging_cycles: int,
                  averaging_every: int, observables=("number_density",), snapshot_every: int = 0, recorder=None):
        """Simulation::integrate: thermalisation with step adaptation, then averaging;
        returns {observable: (mean, standard error)} and the samples."""
        self.set_conditions(temperature, pressure)
        done = 0
        while done < thermalisation_cycles:
            k = min(1000, thermalisation_cycles - done)
            self.run(k, adjust_steps=True)
            done += k
        samples = {name: [] for name in observables}
        for c in range(1, averaging_cycles + 1):
            st = self.run(1)
            if c % averaging_every == 0:
                for name in observables:
                    samples[name].append(OBSERVABLES[name](self.packing, st))
            if recorder is not None and snapshot_every and c % snapshot_every == 0:
                recorder.record(self.packing, c // snapshot_every * snapshot_every)
        return {name: quantity(v) for name, v in samples.items()}, samples
