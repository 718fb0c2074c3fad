"""Seeded test systems: lattices from rampack_gb300.workloads, thermalised by the CPU
oracle's cycle loop (the reference's Simulation restated), optionally compressed so
that overlaps appear."""
from __future__ import annotations

import functools

import numpy as np

import pyoracle as po
from rampack_gb300 import workloads as W


def thermalise(cfg, cycles: int, seed: int = 1234, **kw):
    kind, prm, pos, rot, box = cfg
    pk = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=kw.pop("threads", 1))
    if cycles:
        po.run_cycles(pk, cycles, seed=seed, **kw)
    p, r, b = pk.state()
    pk.close()
    return kind, prm, p, r, b


@functools.lru_cache(maxsize=None)
def hs_small():
    """Hard spheres d=1, N=512 at phi=0.30, 30 NpT cycles (p*=10)."""
    return thermalise(W.hard_spheres(8, 0.30), 30, translation_step=0.1, box_kind=2, box_step=0.01 / 3,
                      pressure=10.0)


@functools.lru_cache(maxsize=None)
def hs_dense():
    """Hard spheres d=1, N=1000 at phi=0.45, 30 NVT cycles."""
    return thermalise(W.hard_spheres(10, 0.45), 30, translation_step=0.1)


@functools.lru_cache(maxsize=None)
def sc_l2():
    """Spherocylinders l=2 r=0.5, N=1000, phi=0.35, triclinic after 20 NpT cycles."""
    return thermalise(W.spherocylinders((10, 10, 10), 0.35, 2.0, 0.5, aspect=(1, 1, 3)), 20,
                      translation_step=0.2, rotation_step=0.2, box_kind=1, box_step=0.005, pressure=1.5)


@functools.lru_cache(maxsize=None)
def sc_l2_dense():
    """Spherocylinders l=2 r=0.5, N=1728, phi=0.50, 15 NVT cycles (dense, many rejections)."""
    return thermalise(W.spherocylinders((12, 12, 12), 0.50, 2.0, 0.5, aspect=(1, 1, 3)), 15,
                      translation_step=0.2, rotation_step=0.2)


@functools.lru_cache(maxsize=None)
def sc_l5():
    """Spherocylinders l=5 r=0.5, N=2000 (10x10x20), phi=0.35, 10 NpT cycles."""
    return thermalise(W.spherocylinders((10, 10, 20), 0.35, 5.0, 0.5, aspect=(1, 1, 6)), 10,
                      translation_step=0.2, rotation_step=0.2, box_kind=1, box_step=0.005, pressure=1.5)


BANANA = dict(arc_radius=0.6 / (2 * np.sin(np.radians(15))), arc_angle=np.radians(120), n_spheres=5)


@functools.lru_cache(maxsize=None)
def poly_banana():
    """Bent 5-sphere chains (r=0.5, arc 120 degrees), N=400, phi=0.35, triclinic after 10 NpT cycles."""
    return thermalise(W.bananas((8, 10, 5), 0.35, **BANANA), 10, translation_step=0.2, rotation_step=0.2,
                      box_kind=1, box_step=0.005, pressure=1.5)


@functools.lru_cache(maxsize=None)
def poly_dense():
    """Bent 5-sphere chains, N=480, phi=0.45, 10 NVT cycles (dense, many rejections)."""
    return thermalise(W.bananas((8, 10, 6), 0.45, **BANANA), 10, translation_step=0.2, rotation_step=0.2)


@functools.lru_cache(maxsize=None)
def hs_tiny():
    """Hard spheres d=1, N=27 in a 3.9^3 box: the reference keeps no neighbour grid here."""
    return thermalise((W.SPHERE, np.array([0.5]), W.lattice((3, 3, 3), (1.3, 1.3, 1.3)), W.aligned_rotations(27),
                       W.diag_box(3.9, 3.9, 3.9)), 20, translation_step=0.1)


@functools.lru_cache(maxsize=None)
def sc_tiny():
    """Spherocylinders l=3 r=0.5, N=50 in a 10^3 box (no neighbour grid in the reference), 20 NVT cycles."""
    return thermalise((W.SPHEROCYLINDER, np.array([3.0, 0.5]), W.lattice((5, 5, 2), (2.0, 2.0, 5.0)),
                       W.aligned_rotations(50), W.diag_box(10.0, 10.0, 10.0)), 20,
                      translation_step=0.5, rotation_step=0.5)


@functools.lru_cache(maxsize=None)
def psc_bent():
    """Bent rods of two spherocylinders (r = 0.25, 60 degree kink), N = 432, 12 NpT cycles."""
    return thermalise(W.bent_rods((6, 8, 9)), 12, translation_step=0.15, rotation_step=0.15, box_kind=1,
                      box_step=0.005, pressure=2.0)


@functools.lru_cache(maxsize=None)
def psc_tiny():
    """Bent rods, N = 24 in a small box (no neighbour grid in the reference), 10 NVT cycles."""
    return thermalise(W.bent_rods((2, 4, 3), spacing=(2.0, 1.0, 1.3)), 10, translation_step=0.2,
                      rotation_step=0.2)


def compressed(cfg, factor: float):
    """The same configuration with box and positions scaled by `factor` (overlaps for factor < 1)."""
    kind, prm, pos, rot, box = cfg
    b = np.array(box, dtype=np.float64).reshape(3, 3)
    rel = np.clip(pos @ np.linalg.inv(b).T, 1e-9, 1 - 1e-9)
    nb = b * factor
    p = rel @ nb.T
    return kind, prm, np.ascontiguousarray(p), rot, nb.reshape(9)


ALL = {"hs_small": hs_small, "hs_dense": hs_dense, "sc_l2": sc_l2, "sc_l2_dense": sc_l2_dense, "sc_l5": sc_l5,
       "poly_banana": poly_banana, "poly_dense": poly_dense, "hs_tiny": hs_tiny, "sc_tiny": sc_tiny,
       "psc_bent": psc_bent, "psc_tiny": psc_tiny}
