"""CPU restatement of the observables the ensemble tests average (test infrastructure only).

* ``nematic_order``: NematicOrder::calculate and calculateEigenvalues
  (core/observables/NematicOrder.cpp:9-56): Q = 1/2 (3 <u u^T> - I) summed over the
  particles' primary axes in index order, P2 = the eigenvalue of largest magnitude from
  the Cardano formula (arXiv:1306.6291).
* ``number_density``: N / V (core/observables/NumberDensity.cpp).
* ``sem``: mean and standard error of samples taken far enough apart to be independent.
"""
from __future__ import annotations

import math

import numpy as np


def primary_axes(rot: np.ndarray) -> np.ndarray:
    """Column 2 of each row-major orientation: the primary axis of spherocylinders
    (SpherocylinderTraits.cpp:52-54) and of the bent chains (axis {0, 0, 1} in the body frame)."""
    r = np.asarray(rot, dtype=np.float64).reshape(-1, 9)
    return np.ascontiguousarray(r[:, [2, 5, 8]])


def eigenvalues(q: np.ndarray):
    a11, a12, a13, a22, a23, a33 = q[0, 0], q[0, 1], q[0, 2], q[1, 1], q[1, 2], q[2, 2]
    b = a11 + a22 + a33
    c = a11 * a22 + a11 * a33 + a22 * a33 - a12 * a12 - a13 * a13 - a23 * a23
    d = a11 * a23 * a23 + a22 * a13 * a13 + a33 * a12 * a12 - a11 * a22 * a33 - 2 * a12 * a13 * a23
    p = b * b - 3 * c
    if p <= 0:
        return [b / 3] * 3
    sp = math.sqrt(p)
    qq = 2 * b * b * b - 9 * b * c - 27 * d
    ratio = qq / 2 / (sp * sp * sp)
    if abs(ratio) > 1:
        ratio = -1.0 if ratio < 0 else 1.0
    delta = math.acos(ratio)
    return [1. / 3 * (b + 2 * sp * math.cos(delta / 3)), 1. / 3 * (b + 2 * sp * math.cos((delta + 2 * math.pi) / 3)),
            1. / 3 * (b + 2 * sp * math.cos((delta - 2 * math.pi) / 3))]


def nematic_order(rot: np.ndarray):
    """(Q tensor 3x3, P2) of the orientations."""
    u = primary_axes(rot)
    s = np.zeros((3, 3))
    for ax in u:  # index order, as the reference sums
        for i in range(3):
            for j in range(3):
                s[i, j] += ax[i] * ax[j]
    s /= float(len(u))
    q = 0.5 * (3. * s - np.eye(3))
    ev = eigenvalues(q)
    return q, max(ev, key=abs)


def number_density(n: int, box) -> float:
    return n / abs(np.linalg.det(np.asarray(box, dtype=np.float64).reshape(3, 3)))


def sem(samples):
    x = np.asarray(samples, dtype=np.float64)
    return float(x.mean()), float(x.std(ddof=1) / math.sqrt(len(x)))
