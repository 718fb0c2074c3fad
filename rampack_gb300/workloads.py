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
POLYSPHEROCYLINDER = 3


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


def banana_centres(arc_radius: float, arc_angle: float, n: int) -> np.ndarray:
    """Body-frame sphere centres of a bent chain, PolysphereBananaTraits::generateGeometry
    (core/shapes/PolysphereBananaTraits.cpp:46-82): n points on an arc of radius
    arc_radius spanning arc_angle in the xz plane, the point at -(arc_radius, 0, 0)
    rotated about y by -arc_angle/2 + i arc_angle/(n-1); for arc_angle < pi the chain is
    shifted along x so that its first sphere sits at x = 0."""
    if not (arc_radius > 0 and 0 < arc_angle < 2 * math.pi and n >= 2):
        raise ValueError("bad banana geometry")
    step = arc_angle / (n - 1)
    angle = -arc_angle / 2
    pts = []
    for _ in range(n):
        # Matrix<3,3>::rotation(0, angle, 0) applied to (-R, 0, 0)
        c, s = math.cos(angle), math.sin(angle)
        pts.append([c * -arc_radius, 0.0, -s * -arc_radius])
        angle += step
    pts = np.array(pts, dtype=np.float64)
    if arc_angle < math.pi:
        pts[:, 0] += -pts[0, 0]
    return pts


def banana_volume(centres: np.ndarray, radius: float, arc_angle: float) -> float:
    """PolysphereBananaTraits::calculateVolume (core/shapes/PolysphereBananaTraits.cpp:95-117):
    n spheres minus n-1 lenses of neighbouring spheres (plus the first-last lens past pi)."""
    n = len(centres)

    def lens(d):
        return math.pi * (4 * radius + d) * (2 * radius - d) ** 2 / 12 if d < 2 * radius else 0.0

    v = n * sphere_volume(radius) - (n - 1) * lens(float(np.linalg.norm(centres[0] - centres[1])))
    if arc_angle > math.pi and n > 2:
        v -= lens(float(np.linalg.norm(centres[0] - centres[-1])))
    return v


def polysphere_params(centres: np.ndarray, radii) -> np.ndarray:
    """Shape parameters of a polysphere: [k, (x, y, z, r) per centre]."""
    radii = np.broadcast_to(np.asarray(radii, dtype=np.float64), (len(centres),))
    out = [float(len(centres))]
    for c, r in zip(centres, radii):
        out += [float(c[0]), float(c[1]), float(c[2]), float(r)]
    return np.array(out, dtype=np.float64)


def bananas(counts, phi: float, arc_radius: float, arc_angle: float, n_spheres: int, radius: float = 0.5):
    """Aligned bent chains on an orthorhombic lattice whose cell is the chain's bounding
    box (spheres included) scaled uniformly to packing fraction phi."""
    centres = banana_centres(arc_radius, arc_angle, n_spheres)
    lo, hi = centres.min(0) - radius, centres.max(0) + radius
    ext = hi - lo
    v = banana_volume(centres, radius, arc_angle)
    s = (v / (phi * ext.prod())) ** (1.0 / 3.0)
    if s < 1.0:
        raise ValueError("packing fraction too high for an aligned lattice")
    cell = ext * s
    nx, ny, nz = counts
    n = nx * ny * nz
    pos = lattice(counts, cell) - (lo + hi) / 2  # bounding boxes centred in the lattice cells
    box = diag_box(cell[0] * nx, cell[1] * ny, cell[2] * nz)
    pos = np.mod(pos, np.array([cell[0] * nx, cell[1] * ny, cell[2] * nz]))
    return POLYSPHERE, polysphere_params(centres, radius), np.ascontiguousarray(pos), aligned_rotations(n), box


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


def config_banana_1e5():
    """Bent 5-sphere chains (sphere radius 0.5, 30 degrees between successive bonds of
    length 0.6: arc angle 120 degrees, arc radius 0.6 / (2 sin 15 degrees)),
    N = 100,000 (50 x 80 x 25), aligned, phi = 0.45."""
    return bananas((50, 80, 25), 0.45, 0.6 / (2 * math.sin(math.radians(15))), math.radians(120), 5)


def config_bent_rods_1e5():
    """Bent rods of two spherocylinders (radius 0.25, half axes (0.3, 0, +-0.15) at x = -+0.35:
    a 60 degree kink), N = 100,000 (25 x 40 x 100), aligned on a lattice of cells
    2.0 x 0.62 x 0.95 (packing fraction about 0.33)."""
    return bent_rods((25, 40, 100))


def replica_lattice(kind: int, n: int, phi: float, length: float = 3.0, radius: float = 0.5):
    """N particles (spheres, or spherocylinders aligned along z) on the first N sites of an
    orthorhombic lattice whose cell aspect follows the particle's extents, in a box of
    packing fraction phi."""
    if kind == SPHERE:
        v, aspect = sphere_volume(radius), np.array([1.0, 1.0, 1.0])
    else:
        v, aspect = spherocylinder_volume(length, radius), np.array([1.0, 1.0, (length + 2 * radius) / (2 * radius)])
    m = max(1, int(math.ceil((n * aspect[2]) ** (1.0 / 3.0))))  # a near-cubic box
    q = int(math.ceil(n / (m * m)))
    a = (n * v / phi / (aspect[2] * m * m * q)) ** (1.0 / 3.0)
    cell = a * aspect
    if kind == SPHERE and a < 2 * radius or kind == SPHEROCYLINDER and (a < 2 * radius or cell[2] < length + 2 * radius):
        raise ValueError("packing fraction too high for the lattice")
    pos = lattice((m, m, q), cell)[:n]
    prm = np.array([radius]) if kind == SPHERE else np.array([length, radius])
    return kind, prm, np.ascontiguousarray(pos), aligned_rotations(n), diag_box(cell[0] * m, cell[1] * m, cell[2] * q)


def config_replicas_64(seed: int = 1234):
    """64 replicas: 32 hard-sphere (r=0.5) and 32 spherocylinder (l=3, r=0.5) systems with
    N_i = round(exp(U(ln 500, ln 20000))) (numpy generator seeded with `seed`), pressures
    log-spaced on [1, 20], started on lattices at phi=0.30.  Returns a list of
    (kind, params, pos, rot, box, pressure)."""
    rng = np.random.default_rng(seed)
    sizes = np.round(np.exp(rng.uniform(math.log(500), math.log(20000), 64))).astype(int)
    pressures = np.exp(np.linspace(math.log(1.0), math.log(20.0), 64))
    out = []
    for i in range(64):
        kind = SPHERE if i < 32 else SPHEROCYLINDER
        out.append(replica_lattice(kind, int(sizes[i]), 0.30) + (float(pressures[i]),))
    return out


# A bent rod of two spherocylinders meeting at a 60 degree kink (PolyspherocylinderTraits
# data: centre, half axis, radius per spherocylinder).
BENT_ROD = ((-0.35, 0.0, 0.0, 0.3, 0.0, 0.15, 0.25), (0.35, 0.0, 0.0, 0.3, 0.0, -0.15, 0.25))


def polyspherocylinder_params(data) -> np.ndarray:
    """{k, (x, y, z, hx, hy, hz, r) per spherocylinder}."""
    return np.array([float(len(data))] + [float(v) for d in data for v in d])


def bent_rods(counts, spacing=(2.0, 0.62, 0.95)):
    """Aligned bent rods on an orthorhombic lattice (contact-free at the given spacing)."""
    pos = lattice(counts, spacing)
    box = diag_box(counts[0] * spacing[0], counts[1] * spacing[1], counts[2] * spacing[2])
    return POLYSPHEROCYLINDER, polyspherocylinder_params(BENT_ROD), pos, aligned_rotations(len(pos)), box



# A generic convex body (GenericXenoCollideTraits): a 1 x 1 x 2 cuboid rounded by a sphere of
# radius 0.1 (the Minkowski sum), as an XCBodyBuilder script.
CONVEX = 4
ROUNDED_BOX = "cuboid 1 1 2; sphere 0.1; sum"


def config_convex(n_side=64, spacing=(1.5, 1.5, 2.5)):
    """n_side^3 rounded boxes, aligned, on an orthorhombic lattice (contact-free: the bodies span
    1.2 x 1.2 x 2.2), packing fraction about 0.55."""
    counts = (n_side, n_side, n_side)
    pos = lattice(counts, spacing)
    box = diag_box(counts[0] * spacing[0], counts[1] * spacing[1], counts[2] * spacing[2])
    return CONVEX, ROUNDED_BOX, pos, aligned_rotations(len(pos)), box
