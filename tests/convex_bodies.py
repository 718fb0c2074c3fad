"""Generic convex bodies of the tests: XCBodyBuilder scripts covering every primitive and
operation (geometry/xenocollide/XCBodyBuilder.cpp:194-294), and random rotations."""
import numpy as np

BODIES = {
    "cuboid": "cuboid 1 2 3",
    "spherocylinder_sum": "segment 2; sphere 0.5; sum",
    "cylinder": "disk 1; segment 0.4; sum",
    "ellipsoid": "ellipsoid 1 0.6 0.3",
    "football": "football 3 0.8",
    "saucer": "saucer 1 0.5",
    "rounded_rectangle": "rectangle 1 2; sphere 0.2; sum",
    "cone": "ellipse 1 0.5; point 0 0 0.7; wrap",
    "capsule_wrap": "sphere 0.5; move 0 0 0.6; sphere 0.5; move 0 0 -0.6; wrap",
    "rotated_sum": "cuboid 1 1 1; rot 30 20 10; sphere 0.3; move 0.2 0 0; sum",
    # the vertices placed by move (XCPoint's own radii are 0 whatever its position, so a hull
    # of points given by position alone has circumsphere radius 0 in the reference)
    "tetrahedron": "point 0 0 0; point 0 0 0; move 1 0 0; point 0 0 0; move 0 1 0; point 0 0 0; move 0 0 1; wrap 4",
    "difference": "cuboid 1 1 1; sphere 0.4; move 0.1 0 0; diff",
    "sphere": "sphere 0.5",
}

# circumsphere radius of each body's geometry (the builder's radii), for lattice spacings
CIRCUMSPHERE = {"cuboid": 1.8708, "cone": 1.0, "capsule_wrap": 1.1, "rotated_sum": 1.3661,
                "ellipsoid": 1.0, "football": 1.5, "saucer": 1.0}


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]).reshape(9)


def random_pairs(rng, n, scales=(0.3, 0.8, 1.3, 2.0, 3.5)):
    """n pairs: the first body at the origin, the second in a random direction at one of the
    scaled distances (x 0.7-1.3), both randomly rotated."""
    p2, r1, r2 = [], [], []
    for k in range(n):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        r1.append(random_rotation(rng))
        r2.append(random_rotation(rng))
        p2.append(d * scales[k % len(scales)] * rng.uniform(0.7, 1.3))
    return np.zeros((n, 3)), np.array(r1), np.array(p2), np.array(r2)


def lattice(n_side, spacing, seed=5):
    """n_side^3 bodies on a simple cubic lattice, randomly rotated, in a cubic box."""
    pos = np.array([[(i + 0.5) * spacing, (j + 0.5) * spacing, (k + 0.5) * spacing]
                    for i in range(n_side) for j in range(n_side) for k in range(n_side)])
    rng = np.random.default_rng(seed)
    rot = np.array([random_rotation(rng) for _ in range(len(pos))])
    box = np.eye(3).reshape(9) * n_side * spacing
    return pos, rot, box
