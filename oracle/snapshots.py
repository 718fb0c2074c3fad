"""ORACLE (test infrastructure only): the reference's snapshot and trajectory formats
restated in Python, the checker of the engine's writers and readers.

* RAMSNAP (core/io/RamsnapWriter.cpp:8-48): the number of aux entries, "key value" lines in
  key order (a std::map), the 9 box entries row by row, the number of shapes, then per shape
  "x y z" + 8 spaces + the 9 orientation entries; every number as ``operator<<`` prints it at
  precision max_digits10 in defaultfloat, i.e. C's "%.17g" (Python's %-formatting gives the
  same correctly rounded digits).
* RAMSNAP reading (core/io/RamsnapReader.cpp:16-96), for files with whitespace-separated
  numbers: aux entries are "key" then the rest of the line after whitespace; the box line
  holds 3 (a cuboid's sides) or 9 numbers.
* RAMTRJ (core/io/RamtrjIO.cpp:16-101): header "RAMTRJ\\n", minor and major version bytes
  (1, 1), then numParticles, numSnapshots, cycleStep as 8-byte little-endian integers; per
  snapshot the box (9 doubles) and per particle the position and the first Euler-angle
  solution (geometry/EulerAngles.cpp:12-46, C library asin/cos/atan2 — Python's math module
  calls the same functions); read back through Matrix::rotation(ax, ay, az)
  (geometry/Matrix.tpp:411-434).

Pinned against fixtures written by the reference itself (tests/golden/io_*.{ramsnap,ramtrj}).
"""
from __future__ import annotations

import math
import struct

import numpy as np


def fmt(x: float) -> str:
    return "%.17g" % float(x)


def ramsnap_bytes(pos, rot, box, aux=None) -> bytes:
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    rot = np.asarray(rot, dtype=np.float64).reshape(-1, 9)
    box = np.asarray(box, dtype=np.float64).reshape(9)
    aux = dict(aux or {})
    out = [f"{len(aux)}\n"]
    for k in sorted(aux, key=lambda s: s.encode()):
        out.append(f"{k} {aux[k]}\n")
    out.append(" ".join(fmt(v) for v in box) + "\n")
    out.append(f"{len(pos)}\n")
    for p, o in zip(pos, rot):
        out.append(" ".join(fmt(v) for v in p) + "        " + " ".join(fmt(v) for v in o) + "\n")
    return "".join(out).encode()


def parse_ramsnap(data: bytes):
    """(pos, rot, box, aux) of a RAMSNAP text; raises ValueError with the reference's message."""
    text = data.decode()
    p = 0
    ws = " \n\t\r\v\f"

    def skip():
        nonlocal p
        while p < len(text) and text[p] in ws:
            p += 1

    def word():
        nonlocal p
        skip()
        q = p
        while q < len(text) and text[q] not in ws:
            q += 1
        w, p = text[p:q], q
        return w

    def line():
        nonlocal p
        q = text.find("\n", p)
        q = len(text) if q < 0 else q
        s, p = text[p:q], min(len(text), q + 1)
        return s

    w = word()
    if not w.isdigit():
        raise ValueError("Broken RAMSNAP file: aux info size")
    aux = {}
    for i in range(int(w)):
        k = word()
        skip()
        if not k or p >= len(text):
            raise ValueError(f"Broken RAMSNAP file: aux info entry {i}")
        aux[k] = line()
    toks = line().split()
    try:
        vals = [float(t) for t in toks]
    except ValueError:
        raise ValueError("Broken RAMSNAP file: dimensions") from None
    if len(vals) == 3:
        box = np.diag(vals).reshape(9)
    elif len(vals) >= 9:
        box = np.array(vals[:9])
    else:
        raise ValueError("Broken RAMSNAP file: dimensions")
    m = box.reshape(3, 3)
    if abs(np.dot(np.cross(m[:, 0], m[:, 1]), m[:, 2])) == 0:
        raise ValueError("Broken RAMSNAP file: zero box volume")
    w = word()
    if not w.isdigit():
        raise ValueError("Broken RAMSNAP file: size")
    n = int(w)
    rest = text[p:].split()
    if len(rest) < 12 * n:
        raise ValueError(f"Broken RAMSNAP file: shape {len(rest) // 12}/{n}")
    arr = np.array([float(t) for t in rest[:12 * n]], dtype=np.float64).reshape(n, 12)
    return arr[:, :3].copy(), arr[:, 3:].copy(), box, aux


def euler_first(o) -> tuple[float, float, float]:
    """EulerAngles(matrix).first; raises ValueError when the matrix is not a rotation."""
    o = [float(x) for x in np.asarray(o).reshape(9)]
    eps = 1e-12
    for i in range(3):
        for j in range(3):
            s = 0.0
            for k in range(3):
                s += o[3 * i + k] * o[3 * j + k]
            if not abs(s - (1.0 if i == j else 0.0)) < eps:
                raise ValueError("not a rotation matrix")
    R11, R12, R13, R21, R31, R32, R33 = o[0], o[1], o[2], o[3], o[6], o[7], o[8]
    if R31 > -1 + eps or R31 < 1 - eps:
        theta = -math.asin(R31)
        c1 = math.cos(theta)
        return math.atan2(R32 / c1, R33 / c1), theta, math.atan2(R21 / c1, R11 / c1)
    if R31 < 0:
        return math.atan2(R12, R13), math.pi / 2, 0.0
    return math.atan2(-R12, -R13), -math.pi / 2, 0.0


def euler_matrix(a) -> np.ndarray:
    sx, sy, sz = math.sin(a[0]), math.sin(a[1]), math.sin(a[2])
    cx, cy, cz = math.cos(a[0]), math.cos(a[1]), math.cos(a[2])
    return np.array([cy * cz, sx * sy * cz - cx * sz, cx * sy * cz + sx * sz,
                     cy * sz, sx * sy * sz + cx * cz, cx * sy * sz - sx * cz,
                     -sy, sx * cy, cx * cy])


def ramtrj_bytes(states, cycle_step: int) -> bytes:
    """A whole RAMTRJ file of `states` = [(pos, rot, box), ...]."""
    n = len(np.asarray(states[0][0]).reshape(-1, 3))
    out = [b"RAMTRJ\n", bytes([1, 1]), struct.pack("<QQQ", n, len(states), cycle_step)]
    for pos, rot, box in states:
        pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        rot = np.asarray(rot, dtype=np.float64).reshape(-1, 9)
        rec = np.zeros((n, 6))
        rec[:, :3] = pos
        for i in range(n):
            rec[i, 3:] = euler_first(rot[i])
        out.append(np.asarray(box, dtype="<f8").reshape(9).tobytes())
        out.append(rec.astype("<f8").tobytes())
    return b"".join(out)


def parse_ramtrj(data: bytes):
    """(header dict, [(pos, rot, box), ...]) of a RAMTRJ file."""
    if data[:7] != b"RAMTRJ\n":
        raise ValueError("RAMTRJ read error: magic")
    minor, major = data[7], data[8]
    n, count, step = struct.unpack("<QQQ", data[9:33])
    size = 9 * 8 + n * 48
    if len(data) != 33 + count * size:
        raise ValueError("RAMTRJ read error: broken snapshot structure")
    out = []
    for s in range(count):
        b = np.frombuffer(data, dtype="<f8", count=9 + 6 * n, offset=33 + s * size)
        rec = b[9:].reshape(n, 6)
        rot = np.array([euler_matrix(r[3:]) for r in rec])
        out.append((rec[:, :3].copy(), rot, b[:9].copy()))
    return {"num_particles": n, "snapshots": count, "cycle_step": step, "version": (major, minor)}, out
