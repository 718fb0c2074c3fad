// ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load or call anything under oracle/; the
// product path (rampack_gb300/) never does.
//
// FP64 geometry restated from the reference in the reference's own operation
// order, so that results are bit-identical to the reference built with
// -ffp-contract=off.  Every function names the reference file:line it follows.
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <limits>

namespace rpo {

using V3 = std::array<double, 3>;
using M3 = std::array<double, 9>;  // row-major, element (i, j) at [3*i + j]

// geometry/Matrix.tpp:78-92 (operator+/-) — element-wise.
inline V3 add(const V3 &a, const V3 &b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
inline V3 sub(const V3 &a, const V3 &b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }

// geometry/Vector.tpp:53-59 — dot product accumulated from zero, i = 0, 1, 2.
inline double dot(const V3 &a, const V3 &b) {
    double p = 0;
    for (int i = 0; i < 3; i++) p += a[i] * b[i];
    return p;
}
inline double norm2(const V3 &a) { return dot(a, a); }  // Vector.h:207 norm2 = v*v

// geometry/Matrix.tpp:162-172 (operator*=(scalar)): scalar 0 fills zeros, scalar 1
// is a no-op, anything else multiplies element-wise.
inline V3 vscale(const V3 &a, double x) {
    if (x == 0) return {0.0, 0.0, 0.0};
    if (x == 1) return a;
    return {a[0] * x, a[1] * x, a[2] * x};
}
inline M3 mscale(const M3 &a, double x) {
    M3 r{};
    if (x == 0) return r;
    if (x == 1) return a;
    for (int i = 0; i < 9; i++) r[i] = a[i] * x;
    return r;
}
// geometry/Matrix.tpp:178-185 (operator/=): divisor 1 is a no-op.
inline V3 vdiv(const V3 &a, double x) {
    if (x == 1) return a;
    return {a[0] / x, a[1] / x, a[2] / x};
}

// geometry/Matrix.tpp:104-113 — i-j-k product accumulated from zero.  A Vector is a
// 3x1 Matrix, so matrix·vector uses the same loop (Vector.tpp:65-69).
inline V3 mv(const M3 &m, const V3 &v) {
    V3 r{};
    for (int i = 0; i < 3; i++) {
        double s = 0;
        for (int k = 0; k < 3; k++) s += m[3 * i + k] * v[k];
        r[i] = s;
    }
    return r;
}
inline M3 mm(const M3 &a, const M3 &b) {
    M3 r{};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += a[3 * i + k] * b[3 * k + j];
            r[3 * i + j] = s;
        }
    return r;
}
inline M3 madd(const M3 &a, const M3 &b) {
    M3 r{};
    for (int i = 0; i < 9; i++) r[i] = a[i] + b[i];
    return r;
}
inline M3 msub(const M3 &a, const M3 &b) {
    M3 r{};
    for (int i = 0; i < 9; i++) r[i] = a[i] - b[i];
    return r;
}
inline M3 transpose(const M3 &a) {
    return {a[0], a[3], a[6], a[1], a[4], a[7], a[2], a[5], a[8]};
}
inline M3 identity() { return {1, 0, 0, 0, 1, 0, 0, 0, 1}; }

// geometry/Vector.tpp:105-112 — cross product.
inline V3 cross(const V3 &a, const V3 &b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
inline V3 column(const M3 &m, int c) { return {m[c], m[3 + c], m[6 + c]}; }

// geometry/Matrix.tpp:355-359 — 3x3 determinant, six triple products left to right.
inline double det3(const M3 &a) {
    return a[0] * a[4] * a[8] + a[1] * a[5] * a[6] + a[2] * a[3] * a[7]
           - a[2] * a[4] * a[6] - a[1] * a[3] * a[8] - a[0] * a[5] * a[7];
}
// geometry/Matrix.tpp:296-327 + :338-342 — minor = det of the 2x2 submatrix without row/col.
inline double minor3(const M3 &a, int row, int col) {
    double m[4];
    int k = 0;
    for (int i = 0; i < 3; i++) {
        if (i == row) continue;
        for (int j = 0; j < 3; j++) {
            if (j == col) continue;
            m[k++] = a[3 * i + j];
        }
    }
    return m[0] * m[3] - m[1] * m[2];
}
// geometry/Matrix.tpp:261-271 — adjugate / determinant.
inline M3 inverse3(const M3 &a) {
    double d = det3(a);
    M3 r{};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            r[3 * i + j] = ((i + j) % 2 == 0) ? (minor3(a, j, i) / d) : (-minor3(a, j, i) / d);
    return r;
}

// geometry/Matrix.tpp:440-450 — Rodrigues: I + K sin(a) + ((1 - cos a) K) K.
inline M3 rotation_axis_angle(const V3 &axis, double angle) {
    double s = std::sin(angle);
    double c = std::cos(angle);
    M3 K = {0, -axis[2], axis[1], axis[2], 0, -axis[0], -axis[1], axis[0], 0};
    M3 first = madd(identity(), mscale(K, s));
    M3 second = mm(mscale(K, 1 - c), K);
    return madd(first, second);
}
// geometry/Matrix.tpp:408-436 — rotation from three Euler angles.
inline M3 rotation_euler(double ax, double ay, double az) {
    double sx = std::sin(ax), sy = std::sin(ay), sz = std::sin(az);
    double cx = std::cos(ax), cy = std::cos(ay), cz = std::cos(az);
    return {cy * cz, sx * sy * cz - cx * sz, cx * sy * cz + sx * sz,
            cy * sz, sx * sy * sz + cx * cz, cx * sy * sz - sx * cz,
            -sy, sx * cy, cx * cy};
}

// core/TriclinicBox.h:61-70, TriclinicBox.cpp:16-51.
struct Box {
    M3 dim{};
    M3 inv{};
    Box() = default;
    explicit Box(const M3 &d) : dim{d}, inv{inverse3(d)} {}
    V3 rel_to_abs(const V3 &v) const { return mv(dim, v); }
    V3 abs_to_rel(const V3 &v) const { return mv(inv, v); }
    std::array<V3, 3> sides() const {
        return {rel_to_abs({1, 0, 0}), rel_to_abs({0, 1, 0}), rel_to_abs({0, 0, 1})};
    }
    double volume() const {
        auto s = sides();
        return std::abs(dot(cross(s[0], s[1]), s[2]));
    }
    V3 heights() const {
        auto s = sides();
        double vol = volume();
        return {vol / std::sqrt(norm2(cross(s[1], s[2]))), vol / std::sqrt(norm2(cross(s[2], s[0]))),
                vol / std::sqrt(norm2(cross(s[0], s[1])))};
    }
    bool operator==(const Box &o) const { return dim == o.dim; }
};

// core/PeriodicBoundaryConditions.cpp:11-22.
inline V3 pbc_correction(const Box &box, const V3 &pos) {
    V3 rel = box.abs_to_rel(pos);
    V3 corr{};
    for (int i = 0; i < 3; i++) {
        while (rel[i] + corr[i] < 0) corr[i] += 1;
        while (rel[i] + corr[i] >= 1) corr[i] -= 1;
    }
    return box.rel_to_abs(corr);
}
// core/PeriodicBoundaryConditions.cpp:24-36.
inline V3 pbc_translation(const Box &box, const V3 &p1, const V3 &p2) {
    V3 r1 = box.abs_to_rel(p1), r2 = box.abs_to_rel(p2);
    V3 t{};
    for (int i = 0; i < 3; i++) {
        while (r2[i] + t[i] - r1[i] > 0.5) t[i] -= 1;
        while (r2[i] + t[i] - r1[i] < -0.5) t[i] += 1;
    }
    return box.rel_to_abs(t);
}
// core/PeriodicBoundaryConditions.cpp:38-50.
inline double pbc_distance2(const Box &box, const V3 &p1, const V3 &p2) {
    V3 r1 = box.abs_to_rel(p1), r2 = box.abs_to_rel(p2);
    V3 d{};
    for (int i = 0; i < 3; i++) {
        double x = std::abs(r2[i] - r1[i]);
        while (x > 0.5) x -= 1;
        d[i] = x;
    }
    return norm2(box.rel_to_abs(d));
}

// A boundary-condition view used by the overlap tests: either the full periodic
// box (no neighbour grid) or a fixed cell translation (core/Packing.cpp:22-43,
// HardcodedTranslation), or free space (core/FreeBoundaryConditions.h).
struct BC {
    enum Kind { FIXED, PERIODIC, FREE } kind = FREE;
    V3 t{};
    const Box *box = nullptr;
    static BC fixed(const V3 &t) { BC b; b.kind = FIXED; b.t = t; return b; }
    static BC periodic(const Box &bx) { BC b; b.kind = PERIODIC; b.box = &bx; return b; }
    V3 translation(const V3 &p1, const V3 &p2) const {
        if (kind == FIXED) return t;
        if (kind == PERIODIC) return pbc_translation(*box, p1, p2);
        return {0, 0, 0};
    }
    double distance2(const V3 &p1, const V3 &p2) const {
        if (kind == FIXED) return norm2(sub(add(p2, t), p1));
        if (kind == PERIODIC) return pbc_distance2(*box, p1, p2);
        return norm2(sub(p2, p1));
    }
};

// geometry/SegmentDistanceCalculator.h:22-85 (Sunday's closest-points algorithm),
// restated with the same branch structure and operation order.
inline double segment_distance2(const V3 &s11, const V3 &s12, const V3 &s21, const V3 &s22) {
    const double EPS = 0.0000000001;
    V3 u = sub(s12, s11), v = sub(s22, s21), w = sub(s11, s21);
    double a = dot(u, u), b = dot(u, v), c = dot(v, v), d = dot(u, w), e = dot(v, w);
    double D = a * c - b * b;
    double sc, sN, sD = D;
    double tc, tN, tD = D;
    if (D < EPS) {
        sN = 0.0;
        sD = 1.0;
        tN = e;
        tD = c;
    } else {
        sN = (b * e - c * d);
        tN = (a * e - b * d);
        if (sN < 0.0) {
            sN = 0.0;
            tN = e;
            tD = c;
        } else if (sN > sD) {
            sN = sD;
            tN = e + b;
            tD = c;
        }
    }
    if (tN < 0.0) {
        tN = 0.0;
        if (-d < 0.0) sN = 0.0;
        else if (-d > a) sN = sD;
        else { sN = -d; sD = a; }
    } else if (tN > tD) {
        tN = tD;
        if ((-d + b) < 0.0) sN = 0;
        else if ((-d + b) > a) sN = sD;
        else { sN = (-d + b); sD = a; }
    }
    sc = (std::abs(sN) < EPS ? 0.0 : sN / sD);
    tc = (std::abs(tN) < EPS ? 0.0 : tN / tD);
    V3 dP = sub(add(w, vscale(u, sc)), vscale(v, tc));
    return norm2(dP);
}

}  // namespace rpo
