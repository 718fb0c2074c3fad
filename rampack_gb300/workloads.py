"""Synthetic initial configurations for the benchmark systems.

Each builder returns ``(kind, params, pos[N,3], rot[N,9], box[9])`` in the layout
the C-ABI takes: FP64 positions, row-major FP64 rotation matrices (the particle
axis is column 2, as ``SpherocylinderTraits::getPrimaryAxis``,
core/shapes/SpherocylinderTraits.cpp:52-54), and the row-major box matrix whose
columns are the box sides (core/TriclinicBox.h).  Lattices are orthorhombic with
particles at cell centres, like the reference's ``OrthorhombicArrangingModel``
(core/lattice/OrthorhombicArrangingModel.h:55-62); all particles start aligned
with the identity orientation.
"""
from __future__ import annotations

import math

import numpy as np

SPHERE, SPHEROCYLINDER, POLYSPHERE = 0, 1, 2


def sphere_volume(r: float) -> float:
    return 4.0 / 3.0 * math.pi * r ** 3


def spherocylinder_volume(length: float, r: float) -> float:
    return math.pi * r * r * length + 4.0 / 3.0 * math.pi * r ** 3


def lattice(counts, cell) -> np.ndarray:
    """Cell-centred orthorhombic lattice: counts (nx, ny, nz), cell (ax, ay, az)."""
    nx, ny, nz = counts
    ax, ay, az = cell
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    pos = np.stack([(i.ravel() + 0.5) * ax, (j.ravel() + 0.5) * ay, (k.ravel() + 0.5) * az], axis=1)
    return np.ascontiguousarray(pos, dtype=np.float64)


def aligned_rotations(n: int) -> np.ndarray:
    return np.tile(np.eye(3).reshape(9), (n, 1)).astype(np.float64)


def diag_box(lx: float, ly: float, lz: float) -> np.ndarray:
    return np.array([lx, 0, 0, 0, ly, 0, 0, 0, lz], dtype=np.float64)


def hard_spheres(n_side: int, phi: float, radius: float = 0.5):
    """Hard spheres on an n_side^3 simple-cubic lattice in a cubic box at packing fraction phi."""
    n = n_side ** 3
    side = (n * sphere_volume(radius) / phi) ** (1.0 / 3.0)
    a = side / n_side
    pos = lattice((n_side, n_side, n_side), (a, a, a))
    return SPHERE, np.array([radius]), pos, aligned_rotations(n), diag_box(side, side, side)


def spherocylinders(counts, phi: float, length: float, radius: float = 0.5, aspect=(1.0, 1.0, None)):
    """Aligned spherocylinders (axis along z) on an orthorhombic lattice at packing fraction phi.

    ``aspect`` is the lattice cell aspect ratio; None for z picks (length + 2r)/(2r), the
    ratio of the particle's extents.
    """
    nx, ny, nz = counts
    n = nx * ny * nz
    az_ratio = aspect[2] if aspect[2] is not None else (length + 2 * radius) / (2 * radius)
    ratios = np.array([aspect[0], aspect[1], az_ratio], dtype=np.float64)
    vol = n * spherocylinder_volume(length, radius) / phi
    a = (vol / (n * ratios.prod())) ** (1.0 / 3.0)
    cell = a * ratios
    if cell[2] < length + 2 * radius or min(cell[0], cell[1]) < 2 * radius:
        raise ValueError("packing fraction too high for an aligned lattice")
    pos = lattice(counts, cell)
    box = diag_box(cell[0] * nx, cell[1] * ny, cell[2] * nz)
    return SPHEROCYLINDER, np.array([length, radius]), pos, aligned_rotations(n), box


# The benchmark systems (sizes as quoted for the reference's hot path).
def config_hs_1000():
    """Hard spheres d=1, N=1000 on a 10^3 simple-cubic lattice at phi=0.30."""
    return hard_spheres(10, 0.30)


def config_sc_64000():
    """Spherocylinders l=5 r=0.5, N=64000 (40^3), aligned, cell aspect 1:1:6, phi=0.35."""
    return spherocylinders((40, 40, 40), 0.35, 5.0, 0.5, aspect=(1.0, 1.0, 6.0))


def config_sc_1e6():
    """Spherocylinders l=2 r=0.5, N=1,000,000 (100^3), aligned, cell aspect 1:1:3, phi=0.50."""
    return spherocylinders((100, 100, 100), 0.50, 2.0, 0.5, aspect=(1.0, 1.0, 3.0))
