// FP64 geometry of the hard-particle path, shared by host and device code.
//
// Every expression follows the reference's operation order (cited per function) and
// is evaluated without fused multiply-add: on the device through __dmul_rn/__dadd_rn
// (which the compiler never contracts), on the host under -ffp-contract=off.  The
// results are therefore bit-identical to the reference's FP64 arithmetic.
#pragma once

#include <cstdint>
#include <cmath>

#ifdef __CUDACC__
#define RP_HD __host__ __device__ __forceinline__
#else
#define RP_HD inline
#endif

namespace rp {

#if defined(__CUDA_ARCH__)
RP_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
RP_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
RP_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
RP_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
#else
RP_HD double dmul(double a, double b) { return a * b; }
RP_HD double dadd(double a, double b) { return a + b; }
RP_HD double dsub(double a, double b) { return a - b; }
RP_HD double ddiv(double a, double b) { return a / b; }
#endif

struct d3 {
    double x, y, z;
};

RP_HD d3 add3(d3 a, d3 b) { return {dadd(a.x, b.x), dadd(a.y, b.y), dadd(a.z, b.z)}; }
RP_HD d3 sub3(d3 a, d3 b) { return {dsub(a.x, b.x), dsub(a.y, b.y), dsub(a.z, b.z)}; }

// geometry/Vector.tpp:53-59: ((0 + a0 b0) + a1 b1) + a2 b2
RP_HD double dot3(d3 a, d3 b) {
    double p = 0.0;
    p = dadd(p, dmul(a.x, b.x));
    p = dadd(p, dmul(a.y, b.y));
    p = dadd(p, dmul(a.z, b.z));
    return p;
}
RP_HD double norm2(d3 a) { return dot3(a, a); }

// geometry/Matrix.tpp:162-172: multiplication by a scalar; 0 fills zeros, 1 is a no-op.
RP_HD d3 scale3(d3 a, double s) {
    if (s == 0.0) return {0.0, 0.0, 0.0};
    if (s == 1.0) return a;
    return {dmul(a.x, s), dmul(a.y, s), dmul(a.z, s)};
}

// Row i of a row-major 3x3 matrix times v (Matrix.tpp:104-113, accumulated from zero).
RP_HD double mrow(const double *m, int i, d3 v) {
    double s = 0.0;
    s = dadd(s, dmul(m[3 * i + 0], v.x));
    s = dadd(s, dmul(m[3 * i + 1], v.y));
    s = dadd(s, dmul(m[3 * i + 2], v.z));
    return s;
}
RP_HD d3 mv3(const double *m, d3 v) { return {mrow(m, 0, v), mrow(m, 1, v), mrow(m, 2, v)}; }

// Element (i, j) of a·b for row-major 3x3 matrices (Matrix.tpp:104-113).
RP_HD double mm_elem(const double *a, const double *b, int i, int j) {
    double s = 0.0;
    s = dadd(s, dmul(a[3 * i + 0], b[0 * 3 + j]));
    s = dadd(s, dmul(a[3 * i + 1], b[1 * 3 + j]));
    s = dadd(s, dmul(a[3 * i + 2], b[2 * 3 + j]));
    return s;
}

// Matrix.tpp:355-359 (left-to-right triple products)
RP_HD double det3(const double *a) {
    double r = dmul(dmul(a[0], a[4]), a[8]);
    r = dadd(r, dmul(dmul(a[1], a[5]), a[6]));
    r = dadd(r, dmul(dmul(a[2], a[3]), a[7]));
    r = dsub(r, dmul(dmul(a[2], a[4]), a[6]));
    r = dsub(r, dmul(dmul(a[1], a[3]), a[8]));
    r = dsub(r, dmul(dmul(a[0], a[5]), a[7]));
    return r;
}
// Matrix.tpp:296-327 — 2x2 minor without (row, col), as m0 m3 - m1 m2.
RP_HD double minor3(const double *a, int row, int col) {
    double m[4];
    int k = 0;
    for (int i = 0; i < 3; i++) {
        if (i == row) continue;
        for (int j = 0; j < 3; j++) {
            if (j == col) continue;
            m[k++] = a[3 * i + j];
        }
    }
    return dsub(dmul(m[0], m[3]), dmul(m[1], m[2]));
}
// Matrix.tpp:261-271 — adjugate over determinant.
RP_HD void inverse3(const double *a, double *out) {
    double d = det3(a);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double mnr = minor3(a, j, i);
            out[3 * i + j] = ((i + j) % 2 == 0) ? ddiv(mnr, d) : ddiv(-mnr, d);
        }
}

RP_HD d3 cross3(d3 a, d3 b) {
    return {dsub(dmul(a.y, b.z), dmul(a.z, b.y)), dsub(dmul(a.z, b.x), dmul(a.x, b.z)),
            dsub(dmul(a.x, b.y), dmul(a.y, b.x))};
}

// core/PeriodicBoundaryConditions.cpp:11-22 — correction that wraps a position into
// [0, 1) relative coordinates.  `rel` receives the relative position before wrapping.
RP_HD d3 pbc_correction(const double *box, const double *inv, d3 pos, bool *wrapped) {
    d3 rel = mv3(inv, pos);
    double c[3] = {0.0, 0.0, 0.0};
    double r[3] = {rel.x, rel.y, rel.z};
    bool any = false;
    for (int i = 0; i < 3; i++) {
        while (dadd(r[i], c[i]) < 0.0) { c[i] = dadd(c[i], 1.0); any = true; }
        while (dadd(r[i], c[i]) >= 1.0) { c[i] = dsub(c[i], 1.0); any = true; }
    }
    if (wrapped) *wrapped = any;
    return mv3(box, d3{c[0], c[1], c[2]});
}

// core/PeriodicBoundaryConditions.cpp:24-36 — nearest-image translation in relative units.
RP_HD d3 pbc_translation(const double *box, const double *inv, d3 p1, d3 p2) {
    d3 r1 = mv3(inv, p1), r2 = mv3(inv, p2);
    double a[3] = {r1.x, r1.y, r1.z}, b[3] = {r2.x, r2.y, r2.z}, t[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 3; i++) {
        while (dsub(dadd(b[i], t[i]), a[i]) > 0.5) t[i] = dsub(t[i], 1.0);
        while (dsub(dadd(b[i], t[i]), a[i]) < -0.5) t[i] = dadd(t[i], 1.0);
    }
    return mv3(box, d3{t[0], t[1], t[2]});
}

// core/PeriodicBoundaryConditions.cpp:38-50 — the distance^2 the reference uses for sphere
// centres when it keeps no neighbour grid: per relative coordinate |r2 - r1| folded down
// by whole boxes into (-1/2, 1/2], back to absolute coordinates, squared norm.
RP_HD double pbc_distance2(const double *box, const double *inv, d3 p1, d3 p2) {
    d3 r1 = mv3(inv, p1), r2 = mv3(inv, p2);
    double a[3] = {r1.x, r1.y, r1.z}, b[3] = {r2.x, r2.y, r2.z}, d[3];
    for (int i = 0; i < 3; i++) {
        double c = fabs(dsub(b[i], a[i]));
        while (c > 0.5) c = dsub(c, 1.0);
        d[i] = c;
    }
    return norm2(mv3(box, d3{d[0], d[1], d[2]}));
}

// core/ActiveDomain.cpp:8-21 — strict bounds in relative coordinates; end <= beg wraps.
RP_HD bool inside_domain(const double *inv, d3 pos, const double *lo, const double *hi) {
    d3 rel = mv3(inv, pos);
    double r[3] = {rel.x, rel.y, rel.z};
    for (int i = 0; i < 3; i++) {
        if (hi[i] > lo[i]) {
            if (r[i] <= lo[i] || r[i] >= hi[i]) return false;
        } else {
            if (r[i] <= lo[i] && r[i] >= hi[i]) return false;
        }
    }
    return true;
}

// geometry/SegmentDistanceCalculator.h:22-85 — Sunday's closest points of two segments.
RP_HD double segment_distance2(d3 s11, d3 s12, d3 s21, d3 s22) {
    const double EPS = 0.0000000001;
    d3 u = sub3(s12, s11), v = sub3(s22, s21), w = sub3(s11, s21);
    double a = dot3(u, u), b = dot3(u, v), c = dot3(v, v), d = dot3(u, w), e = dot3(v, w);
    double D = dsub(dmul(a, c), dmul(b, b));
    double sc, sN, sD = D;
    double tc, tN, tD = D;
    if (D < EPS) {
        sN = 0.0;
        sD = 1.0;
        tN = e;
        tD = c;
    } else {
        sN = dsub(dmul(b, e), dmul(c, d));
        tN = dsub(dmul(a, e), dmul(b, d));
        if (sN < 0.0) {
            sN = 0.0;
            tN = e;
            tD = c;
        } else if (sN > sD) {
            sN = sD;
            tN = dadd(e, b);
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
        if (dadd(-d, b) < 0.0) sN = 0.0;
        else if (dadd(-d, b) > a) sN = sD;
        else { sN = dadd(-d, b); sD = a; }
    }
    sc = (fabs(sN) < EPS ? 0.0 : ddiv(sN, sD));
    tc = (fabs(tN) < EPS ? 0.0 : ddiv(tN, tD));
    d3 dP = sub3(add3(w, scale3(u, sc)), scale3(v, tc));
    return norm2(dP);
}

// Shape parameters of the exact FP64 pair test.  Thresholds are computed on the host
// exactly as the reference computes them (std::pow(2r, 2), 4*r*r, std::pow(2r + l, 2)).
struct ExactShape {
    int kind;            // 0 sphere, 1 spherocylinder
    double sphere_thr;   // sphere: std::pow(2 * radius, 2)
    double cap_half;     // spherocylinder: 0.5 * length (the cap offset factor 0.5 * (+-1) * length)
    double neg_cap_half; // 0.5 * (-1) * length
    double core_thr;     // spherocylinder: 4 * radius * radius
    double far_thr;      // spherocylinder: std::pow(2 * radius + length, 2)
};

// Exact pair test with a fixed translation t added to particle 2 (the neighbour-grid
// path of core/Packing.cpp:379-397 with HardcodedTranslation, Packing.cpp:22-43).
//   spheres:         SphereTraits.cpp:56-65   -> (p2 + t - p1).norm2() < (2r)^2
//   spherocylinders: SpherocylinderTraits.cpp:28-46
// a1, a2: column 2 of each orientation (the spherocylinder axis).
RP_HD bool exact_overlap(const ExactShape &s, d3 p1, d3 a1, d3 p2, d3 a2, d3 t) {
    d3 p2bc = add3(p2, t);
    double d2 = norm2(sub3(p2bc, p1));
    if (s.kind == 0) return d2 < s.sphere_thr;
    if (d2 < s.core_thr) return true;
    if (d2 >= s.far_thr) return false;
    d3 c11 = add3(p1, scale3(a1, s.neg_cap_half));
    d3 c12 = add3(p1, scale3(a1, s.cap_half));
    d3 c21 = add3(p2bc, scale3(a2, s.neg_cap_half));
    d3 c22 = add3(p2bc, scale3(a2, s.cap_half));
    return segment_distance2(c11, c12, c21, c22) < s.core_thr;
}

// Packing::fixRotationMatrix (core/Packing.cpp:1214-1219): three Newton-Schulz steps
// R <- 1.5 R - 0.5 R R^T R as the reference's Matrix operators evaluate them: the scalar
// products element-wise, then (0.5 R) R^T, then that times R (i-j-k sums from zero), then
// the element-wise difference.
RP_HD void fix_rotation(double *r) {
    for (int it = 0; it < 3; it++) {
        double a[9], h[9], t[9], p[9], q[9];
        for (int k = 0; k < 9; k++) {
            a[k] = dmul(r[k], 1.5);
            h[k] = dmul(r[k], 0.5);
        }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) t[3 * i + j] = r[3 * j + i];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) p[3 * i + j] = mm_elem(h, t, i, j);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) q[3 * i + j] = mm_elem(p, r, i, j);
        for (int k = 0; k < 9; k++) r[k] = dsub(a[k], q[k]);
    }
}

// --------------------------------------------------------------------------------
// Philox-4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11,
// "Parallel random numbers: as easy as 1, 2, 3"): ten rounds of two 32x32->64
// multiplications with a Weyl-sequence key schedule.
// --------------------------------------------------------------------------------
struct u4 {
    uint32_t a, b, c, d;
};

RP_HD uint32_t mulhi32(uint32_t x, uint32_t y) {
#if defined(__CUDA_ARCH__)
    return __umulhi(x, y);
#else
    return static_cast<uint32_t>((static_cast<uint64_t>(x) * y) >> 32);
#endif
}

RP_HD u4 philox(u4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = mulhi32(M0, ctr.a), lo0 = M0 * ctr.a;
        uint32_t hi1 = mulhi32(M1, ctr.c), lo1 = M1 * ctr.c;
        ctr = u4{hi1 ^ ctr.b ^ k0, lo1, hi0 ^ ctr.d ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

// Wall overlaps of one body (Packing::countParticleWallOverlaps, core/Packing.cpp:1086-1139,
// with SphereTraits.cpp:67-75, SpherocylinderTraits.cpp:56-73, PolysphereTraits.cpp:129-136):
// per walled axis the nearer wall, if within `half` of the position; `axis` is the
// spherocylinder axis, `cen` the polysphere's rotated centres (ncen of them), `hax` the
// polyspherocylinder's rotated half axes (orientation * body half axis).  Returns the
// number of overlaps, or 1 at the first with early exit.
RP_HD int wall_overlap_count(int walls, const double (*wall_vec)[3], const double *wall_far, double half, int kind,
                             const double *radius, double half_len, d3 pos, d3 axis, const double *cen, int ncen,
                             bool early, const double *hax = nullptr) {
    int cnt = 0;
    for (int i = 0; i < 3; i++) {
        if (!((walls >> i) & 1)) continue;
        const d3 w{wall_vec[i][0], wall_vec[i][1], wall_vec[i][2]};
        const d3 far{wall_far[0], wall_far[1], wall_far[2]};
        d3 o{0.0, 0.0, 0.0}, ww = w;
        if (dot3(pos, w) < half) {
        } else if (dot3(sub3(far, pos), w) < half) {
            o = far;
            ww = d3{-w.x, -w.y, -w.z};
        } else {
            continue;
        }
        if (kind == 0) {
            if (dot3(ww, sub3(pos, o)) < radius[0]) cnt++;
        } else if (kind == 1) {
            const d3 h{dmul(axis.x, half_len), dmul(axis.y, half_len), dmul(axis.z, half_len)};
            if (dot3(ww, sub3(add3(pos, h), o)) < radius[0] || dot3(ww, sub3(sub3(pos, h), o)) < radius[0]) cnt++;
        } else {
            for (int k = 0; k < ncen; k++) {
                const d3 cp = add3(pos, d3{cen[3 * k], cen[3 * k + 1], cen[3 * k + 2]});
                bool hit;
                if (hax) {   // PolyspherocylinderTraits.cpp:149-166: either cap of the segment
                    const d3 h{hax[3 * k], hax[3 * k + 1], hax[3 * k + 2]};
                    hit = dot3(ww, sub3(sub3(cp, h), o)) < radius[k] || dot3(ww, sub3(add3(cp, h), o)) < radius[k];
                } else {
                    hit = dot3(ww, sub3(cp, o)) < radius[k];
                }
                if (hit) {
                    cnt++;
                    if (early) return 1;
                }
            }
        }
        if (early && cnt) return 1;
    }
    return cnt;
}

// Uniform float in [0, 1) from the top 24 bits; uniform float in [-1, 1).
RP_HD float u01f(uint32_t x) { return static_cast<float>(x >> 8) * (1.0f / 16777216.0f); }
RP_HD float pm1f(uint32_t x) { return static_cast<float>(x >> 8) * (1.0f / 8388608.0f) - 1.0f; }

}  // namespace rp
