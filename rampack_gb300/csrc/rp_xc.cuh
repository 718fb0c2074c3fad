// Generic convex shapes (GenericXenoCollideTraits, core/shapes/GenericXenoCollideTraits.h):
// a body given by an XCBodyBuilder script (geometry/xenocollide/XCBodyBuilder.cpp), its support
// function, and the overlap test of core/shapes/XenoCollideTraits.h:147-168 by Minkowski portal
// refinement (Snethen's XenoCollide, geometry/xenocollide/XenoCollide.h:74-168).
//
// The builder runs on the host and flattens the geometry into an array of nodes (primitives and
// the Minkowski sum / difference / convex hull operations of geometry/xenocollide/
// XCOperations.cpp); the support function walks that array with an explicit stack, on the host
// and on the device.  Every FP64 expression follows the reference's operation order
// (geometry/Vector.tpp, geometry/Matrix.tpp: dot and matrix products accumulated from zero,
// scalar products with Matrix::operator*='s 0 / 1 cases, divisions skipped for 1) without
// contraction, so support points, portals and decisions are the reference's bit for bit.
#pragma once

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "rp_geom.cuh"

// The support functions and the refinement loops are called from many places of the move
// kernels; kept out of line on the device so that the kernels' code stays small enough for the
// instruction cache (inlined, they made instruction fetch the dominant stall).
#ifdef __CUDACC__
#define RP_XC_FN static __host__ __device__ __noinline__
#else
#define RP_XC_FN static inline
#endif

namespace rp {

enum XcType : int32_t {
    XC_POINT = 0, XC_SEGMENT, XC_RECTANGLE, XC_CUBOID, XC_DISK, XC_SPHERE, XC_ELLIPSE, XC_ELLIPSOID, XC_FOOTBALL,
    XC_SAUCER, XC_SUM, XC_DIFF, XC_MAX
};
constexpr int XC_MAX_NODES = 48;    // nodes of one body (a duplicated shape is shared)
constexpr int XC_MAX_ENTRIES = 8;   // entries of one sum or convex hull
constexpr int XC_MAX_DEPTH = 12;    // nesting of operations
constexpr int XC_MPR_LIMIT = 4096;  // portal iterations before a pair is reported as numerically stuck

// One geometry: a primitive with its constructor's parameters, or an operation over entries,
// each entry a node placed at a position and orientation in this node's frame.
struct XcNode {
    int32_t type;
    int32_t nent;
    int32_t ent[XC_MAX_ENTRIES];
    double epos[XC_MAX_ENTRIES][3];
    double erot[XC_MAX_ENTRIES][9];
    double p[3];         // point: position; segment, disk, sphere: (half length | radius);
                         // rectangle, cuboid: half sides; ellipse, ellipsoid: semi-axes;
                         // football: (half length, radius); saucer: (radius, half thickness)
    double circ, insph;  // circumsphere and insphere radii about the node's origin
    double centre[3];    // AbstractXCGeometry::getCenter
};

// FP32 copy of a node for the device's filter (xc_overlap_filtered).
struct XcNodeF {
    int32_t type;
    int32_t nent;
    int32_t ent[XC_MAX_ENTRIES];
    float epos[XC_MAX_ENTRIES][3];
    float erot[XC_MAX_ENTRIES][9];
    float p[3];
};

struct XcShape {
    XcNode node[XC_MAX_NODES];
    XcNodeF fnode[XC_MAX_NODES];
    float fcentre[3];
    int32_t nnodes;
    int32_t root;
    int32_t flat;        // the root is a primitive, or an operation whose entries are all primitives
    double circ, insph;  // the root's radii
    double centre[3];    // the root's centre
};

// ---- vector helpers in the reference's operation order ------------------------------------

RP_HD d3 neg3(d3 a) { return {-a.x, -a.y, -a.z}; }
// Vector / scalar (Matrix.tpp:182-189): each entry divided unless the scalar is 1.
RP_HD d3 div3(d3 a, double s) {
    if (s == 1.0) return a;
    return {ddiv(a.x, s), ddiv(a.y, s), ddiv(a.z, s)};
}
RP_HD double norm3(d3 a) { return sqrt(norm2(a)); }
RP_HD d3 normalized3(d3 a) { return div3(a, norm3(a)); }
RP_HD d3 cmul3(d3 a, d3 b) { return {dmul(a.x, b.x), dmul(a.y, b.y), dmul(a.z, b.z)}; }
// rot^T * n (transpose, then the product accumulated from zero)
RP_HD d3 mtv3(const double *m, d3 v) {
    double r[3];
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        s = dadd(s, dmul(m[0 * 3 + i], v.x));
        s = dadd(s, dmul(m[1 * 3 + i], v.y));
        s = dadd(s, dmul(m[2 * 3 + i], v.z));
        r[i] = s;
    }
    return {r[0], r[1], r[2]};
}
// XCUtils.h:34-37
RP_HD bool xc_zero(d3 v) {
    const double z = 9.094947e-13;
    return fabs(v.x) < z && fabs(v.y) < z && fabs(v.z) < z;
}
RP_HD d3 ld3(const double *p) { return {p[0], p[1], p[2]}; }

// Support point of a primitive in its own frame (geometry/xenocollide/XCPrimitives.cpp:30-163,
// XCPrimitives.h:44, :145).
RP_XC_FN d3 xc_primitive_support(const XcNode &g, d3 n) {
    switch (g.type) {
        case XC_POINT:
            return ld3(g.p);
        case XC_SEGMENT:
            return {0.0, 0.0, n.z < 0 ? -g.p[0] : g.p[0]};
        case XC_RECTANGLE: {
            d3 r = ld3(g.p);
            if (n.x < 0) r.x = -r.x;
            if (n.y < 0) r.y = -r.y;
            return r;
        }
        case XC_CUBOID: {
            d3 r = ld3(g.p);
            if (n.x < 0) r.x = -r.x;
            if (n.y < 0) r.y = -r.y;
            if (n.z < 0) r.z = -r.z;
            return r;
        }
        case XC_DISK: {
            const d3 n2{n.x, n.y, 0.0};
            if (xc_zero(n2)) return {0.0, 0.0, 0.0};
            return scale3(normalized3(n2), g.p[0]);
        }
        case XC_SPHERE:
            return scale3(normalized3(n), g.p[0]);
        case XC_ELLIPSE: {
            const d3 n2 = cmul3(ld3(g.p), n);
            if (xc_zero(n2)) return {0.0, 0.0, 0.0};
            return cmul3(normalized3(n2), ld3(g.p));
        }
        case XC_ELLIPSOID:
            return cmul3(normalized3(cmul3(n, ld3(g.p))), ld3(g.p));
        case XC_FOOTBALL: {
            const double r1 = g.p[1], h = g.p[0];
            const double r2 = dmul(0.5, dadd(ddiv(dmul(h, h), r1), r1));  // radius of curvature
            const d3 n3 = normalized3(n);
            if (dmul(n3.z, r2) < -h) return {0.0, 0.0, -h};
            if (dmul(n3.z, r2) > h) return {0.0, 0.0, h};
            const d3 n2 = normalized3(d3{n.x, n.y, 0.0});
            return add3(scale3(neg3(n2), dsub(r2, r1)), scale3(n3, r2));
        }
        case XC_SAUCER: {
            const double t = g.p[1], h = g.p[0];
            const double r2 = dmul(0.5, dadd(ddiv(dmul(h, h), t), t));
            const d3 n3 = normalized3(n);
            d3 n4{n.x, n.y, 0.0};
            if (!xc_zero(n4)) {
                n4 = normalized3(n4);
                const double threshold = dadd(dmul(n3.x, n3.x), dmul(n3.y, n3.y));
                if (dmul(dmul(threshold, r2), r2) > dmul(h, h)) return scale3(n4, h);
            }
            d3 n2{0.0, 0.0, 1.0};
            if (n.z < 0) n2 = neg3(n2);
            return add3(scale3(neg3(n2), dsub(r2, t)), scale3(n3, r2));
        }
        default:
            return {0.0, 0.0, 0.0};
    }
}

// The support point of a flat body (a primitive, or one operation over primitives) without a
// stack: the same arithmetic as xc_support, entry by entry in registers.
RP_XC_FN d3 xc_support_flat(const XcShape &s, d3 n) {
    const XcNode &g = s.node[s.root];
    if (g.type < XC_SUM) return xc_primitive_support(g, n);
    d3 acc{0.0, 0.0, 0.0};
    double best = 0.0;
    #pragma unroll 1
    for (int i = 0; i < g.nent; i++) {
        const d3 dir = (g.type == XC_DIFF && i == 1) ? neg3(n) : n;
        const d3 r = xc_primitive_support(s.node[g.ent[i]], mtv3(g.erot[i], dir));
        const d3 w = add3(mv3(g.erot[i], r), ld3(g.epos[i]));
        if (g.type == XC_SUM) {
            acc = add3(acc, w);
        } else if (g.type == XC_MAX) {
            const double proj = dot3(w, n);
            if (i == 0 || proj > best) {
                acc = w;
                best = proj;
            }
        } else {
            acc = i == 0 ? w : sub3(acc, w);
        }
    }
    return acc;
}

// AbstractXCGeometry::getSupportPoint of node `root`: sums (XCOperations.cpp:38-43), differences
// (:82-86) and convex hulls (:102-118) evaluated depth first with an explicit stack.  Returns
// false if the nesting is deeper than the stack (the builder refuses such bodies).
RP_XC_FN bool xc_support(const XcShape &s, int root, d3 n, d3 &out) {
    struct Frame {
        int node, i;
        d3 n, acc;
        double best;
    };
    Frame st[XC_MAX_DEPTH];
    int top = 0;
    st[0] = Frame{root, 0, n, {0.0, 0.0, 0.0}, 0.0};
    d3 r{0.0, 0.0, 0.0};
    bool have_r = false;
    for (;;) {
        Frame &f = st[top];
        const XcNode &g = s.node[f.node];
        if (have_r) {
            // child f.i returned r in its own frame: place it in this node's frame
            const d3 w = add3(mv3(g.erot[f.i], r), ld3(g.epos[f.i]));
            if (g.type == XC_SUM) {
                f.acc = add3(f.acc, w);
            } else if (g.type == XC_MAX) {
                const double proj = dot3(w, f.n);
                if (f.i == 0 || proj > f.best) {
                    f.acc = w;
                    f.best = proj;
                }
            } else {  // XC_DIFF: p1 - p2
                f.acc = f.i == 0 ? w : sub3(f.acc, w);
            }
            f.i++;
            have_r = false;
        }
        if (g.type < XC_SUM) {
            r = xc_primitive_support(g, f.n);
        } else if (f.i < g.nent) {
            if (top + 1 >= XC_MAX_DEPTH) return false;
            const d3 dir = (g.type == XC_DIFF && f.i == 1) ? neg3(f.n) : f.n;
            st[top + 1] = Frame{g.ent[f.i], 0, mtv3(g.erot[f.i], dir), {0.0, 0.0, 0.0}, 0.0};
            top++;
            continue;
        } else {
            r = f.acc;
        }
        if (top == 0) {
            out = r;
            return true;
        }
        top--;
        have_r = true;
    }
}

// XenoCollide.h:58-66: the support point of a placed body.
RP_XC_FN bool xc_transform_support(const XcShape &s, const double *rot, d3 pos, d3 n, d3 &out) {
    d3 local;
    if (s.flat) local = xc_support_flat(s, mtv3(rot, n));
    else if (!xc_support(s, s.root, mtv3(rot, n), local)) return false;
    out = add3(mv3(rot, local), pos);
    return true;
}

// The support point of the Minkowski difference body2 - body1 in direction n.
RP_HD bool xc_diff_support(const XcShape &s, const double *rot1, d3 pos1, const double *rot2, d3 pos2, d3 n, d3 &v) {
    d3 a, b;
    if (!xc_transform_support(s, rot2, pos2, n, a)) return false;
    if (!xc_transform_support(s, rot1, pos1, neg3(n), b)) return false;
    v = sub3(a, b);
    return true;
}

// XenoCollide::Intersect (XenoCollide.h:74-168) for two copies of the body; `stuck` is set when
// the portal iterations exceed XC_MPR_LIMIT or the geometry is too deep (the pair is then
// reported as overlapping).
RP_XC_FN bool xc_intersect(const XcShape &s, const double *rot1, d3 pos1, const double *rot2, d3 pos2, double tol,
                        bool &stuck) {
    const d3 c = ld3(s.centre);
    const d3 v0 = sub3(add3(mv3(rot2, c), pos2), add3(mv3(rot1, c), pos1));
    if (xc_zero(v0)) return true;
    d3 n = neg3(v0);
    d3 v1, v2, v3, v4;
    if (!xc_diff_support(s, rot1, pos1, rot2, pos2, n, v1)) return stuck = true;
    if (dot3(v1, n) <= 0) return false;
    n = cross3(v1, v0);
    if (xc_zero(n)) return true;
    if (!xc_diff_support(s, rot1, pos1, rot2, pos2, n, v2)) return stuck = true;
    if (dot3(v2, n) <= 0) return false;
    n = cross3(sub3(v1, v0), sub3(v2, v0));
    if (dot3(n, v0) > 0) {
        const d3 tmp = v1;
        v1 = v2;
        v2 = tmp;
        n = neg3(n);
    }
    for (int it = 0; it < XC_MPR_LIMIT; it++) {
        // phase one: a portal that the origin ray passes through
        if (!xc_diff_support(s, rot1, pos1, rot2, pos2, n, v3)) return stuck = true;
        if (dot3(v3, n) <= 0) return false;
        if (dot3(cross3(v1, v3), v0) < 0) {
            v2 = v3;
            n = cross3(sub3(v1, v0), sub3(v3, v0));
            continue;
        }
        if (dot3(cross3(v3, v2), v0) < 0) {
            v1 = v3;
            n = cross3(sub3(v3, v0), sub3(v2, v0));
            continue;
        }
        // phase two: refine the portal
        for (int jt = 0; jt < XC_MPR_LIMIT; jt++) {
            n = cross3(sub3(v2, v1), sub3(v3, v1));
            if (dot3(n, v1) >= 0) return true;
            if (!xc_diff_support(s, rot1, pos1, rot2, pos2, n, v4)) return stuck = true;
            n = normalized3(n);
            if (-dot3(v4, n) >= 0 || dot3(sub3(v4, v3), n) <= tol) return false;
            const d3 cr = cross3(v4, v0);
            if (dot3(v1, cr) > 0) {
                if (dot3(v2, cr) > 0) v1 = v4;
                else v3 = v4;
            } else {
                if (dot3(v3, cr) > 0) v2 = v4;
                else v1 = v4;
            }
        }
        return stuck = true;
    }
    return stuck = true;
}

// XenoCollideTraits::overlapBetween (core/shapes/XenoCollideTraits.h:147-168) with the second
// body already at its image (pos2bc = pos2 + translation).
RP_HD bool xc_overlap(const XcShape &s, d3 pos1, const double *rot1, d3 pos2bc, const double *rot2, bool &stuck) {
    const double rc = dadd(s.circ, s.circ);
    const double ri = dadd(s.insph, s.insph);
    const double d2 = norm2(sub3(pos2bc, pos1));
    if (d2 > dmul(rc, rc)) return false;
    if (d2 < dmul(ri, ri)) return true;
    return xc_intersect(s, rot1, pos1, rot2, pos2bc, 1.0e-12, stuck);
}

// ---- FP32 portal refinement with FP64 certificates (device) -----------------------------------
//
// The exact test above is the reference's decision, but each portal iteration is hundreds of FP64
// instructions.  The filter runs the same portal refinement in FP32 and turns its outcome into a
// certificate checked in FP64 on the real bodies:
//  * a miss ends with a direction n along which the Minkowski difference's support point has a
//    non-positive projection (or the portal's tolerance exit): if the FP64 support point along n
//    projects below -margin, the bodies are separated by at least margin along n;
//  * a hit ends with a tetrahedron (the centre difference v0 and three support points, each kept
//    with the direction that produced it) containing the origin: the three support points
//    recomputed in FP64 span, with v0, a tetrahedron inside the Minkowski difference (a convex
//    set); if the origin lies inside it farther than margin from every face, the bodies overlap
//    by at least margin.
// A body separated or overlapping by margin = 1e-7 (|p2 - p1| + 2 circumsphere radius) + 1e-9 is
// decided the same way by the reference's FP64 refinement (whose rounding is near 1e-15 relative,
// whose tolerance is 1e-12 and whose colinearity shortcut acts below 1e-12), so a certified answer
// is the reference's; everything else — near-touching pairs, degenerate portals, the refinement's
// special cases — runs the exact test.

struct f3v {
    float x, y, z;
};
RP_HD f3v fadd(f3v a, f3v b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
RP_HD f3v fsub(f3v a, f3v b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
RP_HD f3v fneg(f3v a) { return {-a.x, -a.y, -a.z}; }
RP_HD f3v fscale(f3v a, float s) { return {a.x * s, a.y * s, a.z * s}; }
RP_HD float fdot(f3v a, f3v b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
RP_HD f3v fcross(f3v a, f3v b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
RP_HD f3v fnormalized(f3v a) { return fscale(a, 1.0f / sqrtf(fdot(a, a))); }
RP_HD f3v fmv(const float *m, f3v v) {
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z};
}
RP_HD f3v fmtv(const float *m, f3v v) {
    return {m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
            m[2] * v.x + m[5] * v.y + m[8] * v.z};
}
RP_HD bool fzero(f3v v) {
    const float z = 1e-20f;
    return fabsf(v.x) < z && fabsf(v.y) < z && fabsf(v.z) < z;
}

RP_XC_FN f3v xcf_primitive(const XcNodeF &g, f3v n) {
    const f3v p{g.p[0], g.p[1], g.p[2]};
    switch (g.type) {
        case XC_POINT: return p;
        case XC_SEGMENT: return {0.f, 0.f, n.z < 0 ? -p.x : p.x};
        case XC_RECTANGLE: return {n.x < 0 ? -p.x : p.x, n.y < 0 ? -p.y : p.y, 0.f};
        case XC_CUBOID: return {n.x < 0 ? -p.x : p.x, n.y < 0 ? -p.y : p.y, n.z < 0 ? -p.z : p.z};
        case XC_DISK: {
            const f3v n2{n.x, n.y, 0.f};
            if (fzero(n2)) return {0.f, 0.f, 0.f};
            return fscale(fnormalized(n2), p.x);
        }
        case XC_SPHERE: return fscale(fnormalized(n), p.x);
        case XC_ELLIPSE: {
            const f3v n2{p.x * n.x, p.y * n.y, 0.f};
            if (fzero(n2)) return {0.f, 0.f, 0.f};
            const f3v u = fnormalized(n2);
            return {u.x * p.x, u.y * p.y, 0.f};
        }
        case XC_ELLIPSOID: {
            const f3v u = fnormalized(f3v{n.x * p.x, n.y * p.y, n.z * p.z});
            return {u.x * p.x, u.y * p.y, u.z * p.z};
        }
        case XC_FOOTBALL: {
            const float r1 = p.y, h = p.x, r2 = 0.5f * (h * h / r1 + r1);
            const f3v n3 = fnormalized(n);
            if (n3.z * r2 < -h) return {0.f, 0.f, -h};
            if (n3.z * r2 > h) return {0.f, 0.f, h};
            const f3v n2 = fnormalized(f3v{n.x, n.y, 0.f});
            return fadd(fscale(n2, -(r2 - r1)), fscale(n3, r2));
        }
        case XC_SAUCER: {
            const float t = p.y, h = p.x, r2 = 0.5f * (h * h / t + t);
            const f3v n3 = fnormalized(n);
            const f3v n4{n.x, n.y, 0.f};
            if (!fzero(n4) && (n3.x * n3.x + n3.y * n3.y) * r2 * r2 > h * h) return fscale(fnormalized(n4), h);
            const f3v n2{0.f, 0.f, n.z < 0 ? -1.f : 1.f};
            return fadd(fscale(n2, -(r2 - t)), fscale(n3, r2));
        }
        default: return {0.f, 0.f, 0.f};
    }
}

// FP32 support point of the body (depth-first with an explicit stack, as xc_support).
RP_XC_FN bool xcf_support(const XcShape &s, f3v n, f3v &out) {
    struct Frame {
        int node, i;
        f3v n, acc;
        float best;
    };
    Frame st[XC_MAX_DEPTH];
    int top = 0;
    st[0] = Frame{s.root, 0, n, {0.f, 0.f, 0.f}, 0.f};
    f3v r{0.f, 0.f, 0.f};
    bool have_r = false;
    for (;;) {
        Frame &f = st[top];
        const XcNodeF &g = s.fnode[f.node];
        if (have_r) {
            const f3v w = fadd(fmv(g.erot[f.i], r), f3v{g.epos[f.i][0], g.epos[f.i][1], g.epos[f.i][2]});
            if (g.type == XC_SUM) {
                f.acc = fadd(f.acc, w);
            } else if (g.type == XC_MAX) {
                const float proj = fdot(w, f.n);
                if (f.i == 0 || proj > f.best) {
                    f.acc = w;
                    f.best = proj;
                }
            } else {
                f.acc = f.i == 0 ? w : fsub(f.acc, w);
            }
            f.i++;
            have_r = false;
        }
        if (g.type < XC_SUM) {
            r = xcf_primitive(g, f.n);
        } else if (f.i < g.nent) {
            if (top + 1 >= XC_MAX_DEPTH) return false;
            const f3v dir = (g.type == XC_DIFF && f.i == 1) ? fneg(f.n) : f.n;
            st[top + 1] = Frame{g.ent[f.i], 0, fmtv(g.erot[f.i], dir), {0.f, 0.f, 0.f}, 0.f};
            top++;
            continue;
        } else {
            r = f.acc;
        }
        if (top == 0) {
            out = r;
            return true;
        }
        top--;
        have_r = true;
    }
}

// FP32 support point of a flat body (a primitive, or one operation over primitives) without a
// stack, entry by entry as xcf_support.
RP_XC_FN f3v xcf_support_flat(const XcShape &s, f3v n) {
    const XcNodeF &g = s.fnode[s.root];
    if (g.type < XC_SUM) return xcf_primitive(g, n);
    f3v acc{0.f, 0.f, 0.f};
    float best = 0.f;
    #pragma unroll 1
    for (int i = 0; i < g.nent; i++) {
        const f3v dir = (g.type == XC_DIFF && i == 1) ? fneg(n) : n;
        const f3v r = xcf_primitive(s.fnode[g.ent[i]], fmtv(g.erot[i], dir));
        const f3v w = fadd(fmv(g.erot[i], r), f3v{g.epos[i][0], g.epos[i][1], g.epos[i][2]});
        if (g.type == XC_SUM) {
            acc = fadd(acc, w);
        } else if (g.type == XC_MAX) {
            const float proj = fdot(w, n);
            if (i == 0 || proj > best) {
                acc = w;
                best = proj;
            }
        } else {
            acc = i == 0 ? w : fsub(acc, w);
        }
    }
    return acc;
}

// Support point of body2 - body1 along n (FP32); body 1 at the origin.
RP_HD bool xcf_diff(const XcShape &s, const float *r1, const float *r2, f3v p2, f3v n, f3v &v) {
    f3v a, b;
    if (s.flat) {
        a = xcf_support_flat(s, fmtv(r2, n));
        b = xcf_support_flat(s, fmtv(r1, fneg(n)));
    } else {
        if (!xcf_support(s, fmtv(r2, n), a)) return false;
        if (!xcf_support(s, fmtv(r1, fneg(n)), b)) return false;
    }
    v = fsub(fadd(fmv(r2, a), p2), fmv(r1, b));
    return true;
}

// The FP32 refinement: 0 miss (separating direction in n; *h the FP32 support projection along
// the unit n, or +inf after the tolerance exit), 1 hit (portal directions d[0..2] of v1, v2,
// v3), -1 undecided.
RP_XC_FN int xcf_refine(const XcShape &s, const float *r1, const float *r2, f3v p2, f3v &n, f3v *d, float *h) {
    *h = INFINITY;
    const f3v c{s.fcentre[0], s.fcentre[1], s.fcentre[2]};
    const f3v v0 = fsub(fadd(fmv(r2, c), p2), fmv(r1, c));
    if (fzero(v0)) return -1;
    f3v v1, v2, v3, v4;
    n = fneg(v0);
    if (!xcf_diff(s, r1, r2, p2, n, v1)) return -1;
    d[0] = n;
    if (fdot(v1, n) <= 0) {
        *h = fdot(v1, n) / sqrtf(fdot(n, n));
        return 0;
    }
    n = fcross(v1, v0);
    if (fzero(n)) return -1;
    if (!xcf_diff(s, r1, r2, p2, n, v2)) return -1;
    d[1] = n;
    if (fdot(v2, n) <= 0) {
        *h = fdot(v2, n) / sqrtf(fdot(n, n));
        return 0;
    }
    n = fcross(fsub(v1, v0), fsub(v2, v0));
    if (fdot(n, v0) > 0) {
        const f3v t = v1;
        v1 = v2;
        v2 = t;
        const f3v td = d[0];
        d[0] = d[1];
        d[1] = td;
        n = fneg(n);
    }
    #pragma unroll 1
    for (int it = 0; it < 64; it++) {
        if (!xcf_diff(s, r1, r2, p2, n, v3)) return -1;
        const f3v d3 = n;
        if (fdot(v3, n) <= 0) {
            *h = fdot(v3, n) / sqrtf(fdot(n, n));
            return 0;
        }
        if (fdot(fcross(v1, v3), v0) < 0) {
            v2 = v3;
            d[1] = d3;
            n = fcross(fsub(v1, v0), fsub(v3, v0));
            continue;
        }
        if (fdot(fcross(v3, v2), v0) < 0) {
            v1 = v3;
            d[0] = d3;
            n = fcross(fsub(v3, v0), fsub(v2, v0));
            continue;
        }
        d[2] = d3;
        #pragma unroll 1
        for (int jt = 0; jt < 64; jt++) {
            n = fcross(fsub(v2, v1), fsub(v3, v1));
            if (fdot(n, v1) >= 0) return 1;
            if (!xcf_diff(s, r1, r2, p2, n, v4)) return -1;
            const f3v d4 = n;
            n = fnormalized(n);
            if (fdot(v4, n) <= 0) {
                *h = fdot(v4, n);  // n is a unit vector here
                return 0;
            }
            if (fdot(fsub(v4, v3), n) <= 1e-6f * (fabsf(fdot(v4, n)) + 1e-30f)) return 0;  // thin: origin beyond
            const f3v cr = fcross(v4, v0);
            if (fdot(v1, cr) > 0) {
                if (fdot(v2, cr) > 0) {
                    v1 = v4;
                    d[0] = d4;
                } else {
                    v3 = v4;
                    d[2] = d4;
                }
            } else {
                if (fdot(v3, cr) > 0) {
                    v2 = v4;
                    d[1] = d4;
                } else {
                    v1 = v4;
                    d[0] = d4;
                }
            }
        }
        return -1;
    }
    return -1;
}

// Signed distance-like value of the origin from the plane of face (a, b, c), positive on the side
// of vertex e: (m . (0 - a)) * sign(m . (e - a)) / |m|, m = (b - a) x (c - a).
RP_HD double face_clearance(d3 a, d3 b, d3 c, d3 e) {
    const d3 m = cross3(sub3(b, a), sub3(c, a));
    const double se = dot3(m, sub3(e, a));
    const double so = -dot3(m, a);
    const double mm = sqrt(norm2(m));
    if (!(mm > 0) || se == 0) return -1.0;
    return (se > 0 ? so : -so) / mm;
}

// FP64 support points for the certificates of flat bodies: the same geometry in plain double
// arithmetic (contracted, one division per normalisation) — its rounding, near 1e-15 relative,
// stays far below the certificates' margin, which is all a certificate needs.
RP_XC_FN d3 xc_primitive_cert(const XcNode &g, d3 n) {
    const d3 p{g.p[0], g.p[1], g.p[2]};
    switch (g.type) {
        case XC_POINT: return p;
        case XC_SEGMENT: return {0.0, 0.0, n.z < 0 ? -p.x : p.x};
        case XC_RECTANGLE: return {n.x < 0 ? -p.x : p.x, n.y < 0 ? -p.y : p.y, 0.0};
        case XC_CUBOID: return {n.x < 0 ? -p.x : p.x, n.y < 0 ? -p.y : p.y, n.z < 0 ? -p.z : p.z};
        case XC_DISK: {
            const double l2 = n.x * n.x + n.y * n.y;
            if (!(l2 > 0)) return {0.0, 0.0, 0.0};
            const double k = p.x / sqrt(l2);
            return {n.x * k, n.y * k, 0.0};
        }
        case XC_SPHERE: {
            const double k = p.x / sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
            return {n.x * k, n.y * k, n.z * k};
        }
        case XC_ELLIPSE: {
            const double ux = p.x * n.x, uy = p.y * n.y, l2 = ux * ux + uy * uy;
            if (!(l2 > 0)) return {0.0, 0.0, 0.0};
            const double k = 1.0 / sqrt(l2);
            return {ux * k * p.x, uy * k * p.y, 0.0};
        }
        case XC_ELLIPSOID: {
            const double ux = p.x * n.x, uy = p.y * n.y, uz = p.z * n.z;
            const double k = 1.0 / sqrt(ux * ux + uy * uy + uz * uz);
            return {ux * k * p.x, uy * k * p.y, uz * k * p.z};
        }
        default: {
            // football, saucer: the exact evaluation (a few instructions more)
            return xc_primitive_support(g, n);
        }
    }
}

// Support point of body2 - body1 along n for the certificates (flat bodies; others take the
// exact evaluation).
RP_XC_FN bool xc_diff_support_cert(const XcShape &s, const double *rot1, d3 pos1, const double *rot2, d3 pos2, d3 n,
                                   d3 &v) {
    if (!s.flat) return xc_diff_support(s, rot1, pos1, rot2, pos2, n, v);
    const XcNode &g = s.node[s.root];
    d3 side[2];
    #pragma unroll 1
    for (int b = 0; b < 2; b++) {
        const double *rot = b == 0 ? rot2 : rot1;
        const d3 dir = b == 0 ? n : d3{-n.x, -n.y, -n.z};
        const d3 ln{rot[0] * dir.x + rot[3] * dir.y + rot[6] * dir.z, rot[1] * dir.x + rot[4] * dir.y + rot[7] * dir.z,
                    rot[2] * dir.x + rot[5] * dir.y + rot[8] * dir.z};
        d3 acc{0.0, 0.0, 0.0};
        if (g.type < XC_SUM) {
            acc = xc_primitive_cert(g, ln);
        } else {
            double best = 0.0;
            #pragma unroll 1
            for (int i = 0; i < g.nent; i++) {
                const double *er = g.erot[i];
                const d3 d = (g.type == XC_DIFF && i == 1) ? d3{-ln.x, -ln.y, -ln.z} : ln;
                const d3 cd{er[0] * d.x + er[3] * d.y + er[6] * d.z, er[1] * d.x + er[4] * d.y + er[7] * d.z,
                            er[2] * d.x + er[5] * d.y + er[8] * d.z};
                const d3 r = xc_primitive_cert(s.node[g.ent[i]], cd);
                const d3 w{er[0] * r.x + er[1] * r.y + er[2] * r.z + g.epos[i][0],
                           er[3] * r.x + er[4] * r.y + er[5] * r.z + g.epos[i][1],
                           er[6] * r.x + er[7] * r.y + er[8] * r.z + g.epos[i][2]};
                if (g.type == XC_SUM) {
                    acc = {acc.x + w.x, acc.y + w.y, acc.z + w.z};
                } else if (g.type == XC_MAX) {
                    const double pr = w.x * ln.x + w.y * ln.y + w.z * ln.z;
                    if (i == 0 || pr > best) {
                        acc = w;
                        best = pr;
                    }
                } else {
                    acc = i == 0 ? w : d3{acc.x - w.x, acc.y - w.y, acc.z - w.z};
                }
            }
        }
        side[b] = {rot[0] * acc.x + rot[1] * acc.y + rot[2] * acc.z, rot[3] * acc.x + rot[4] * acc.y + rot[5] * acc.z,
                   rot[6] * acc.x + rot[7] * acc.y + rot[8] * acc.z};
    }
    v = {side[0].x + pos2.x - side[1].x - pos1.x, side[0].y + pos2.y - side[1].y - pos1.y,
         side[0].z + pos2.z - side[1].z - pos1.z};
    return true;
}

// The FP32 filter of a pair within the circumspheres and beyond the inspheres: 0 certified
// separated, 1 certified overlapping, -1 undecided (the exact refinement decides).
RP_XC_FN int xc_filter(const XcShape &s, d3 pos1, const double *rot1, d3 pos2bc, const double *rot2) {
    const d3 dp = sub3(pos2bc, pos1);
    float r1f[9], r2f[9];
    for (int k = 0; k < 9; k++) {
        r1f[k] = static_cast<float>(rot1[k]);
        r2f[k] = static_cast<float>(rot2[k]);
    }
    f3v n, dirs[3];
    float h32;
    const int hint = xcf_refine(s, r1f, r2f, f3v{(float)dp.x, (float)dp.y, (float)dp.z}, n, dirs, &h32);
    const double scale = sqrt(norm2(dp)) + dadd(s.circ, s.circ);
    // a miss certified in FP32 alone: the support projection of the Minkowski difference is a
    // sum, or a maximum, of the parts' projections, each computed to a few FP32 roundings of
    // terms no larger than the scale, so an FP32 projection below -1e-4 scale is negative
    if (hint == 0 && h32 < static_cast<float>(-(1e-4 * scale + 1e-6))) return 0;
    const double margin = 1e-7 * scale + 1e-9;
    if (hint == 0) {
        const d3 nd{n.x, n.y, n.z};
        const double nn = sqrt(norm2(nd));
        d3 v;
        if (nn > 0 && xc_diff_support_cert(s, rot1, pos1, rot2, pos2bc, nd, v) && dot3(v, nd) < -margin * nn)
            return 0;
    } else if (hint == 1) {
        const d3 c = ld3(s.centre);
        const d3 v0 = sub3(add3(mv3(rot2, c), pos2bc), add3(mv3(rot1, c), pos1));
        d3 w[3];
        bool ok = true;
        #pragma unroll 1
        for (int k = 0; k < 3 && ok; k++)
            ok = xc_diff_support_cert(s, rot1, pos1, rot2, pos2bc, d3{dirs[k].x, dirs[k].y, dirs[k].z}, w[k]);
        if (ok && face_clearance(w[0], w[1], w[2], v0) > margin && face_clearance(v0, w[1], w[2], w[0]) > margin &&
            face_clearance(v0, w[0], w[2], w[1]) > margin && face_clearance(v0, w[0], w[1], w[2]) > margin)
            return 1;
    }
    return -1;
}

// XenoCollideTraits::overlapBetween with the FP32 filter and its FP64 certificates; the exact
// refinement decides whatever they leave open.
RP_HD bool xc_overlap_filtered(const XcShape &s, d3 pos1, const double *rot1, d3 pos2bc, const double *rot2,
                               bool &stuck) {
    const double rc = dadd(s.circ, s.circ);
    const double ri = dadd(s.insph, s.insph);
    const double d2 = norm2(sub3(pos2bc, pos1));
    if (d2 > dmul(rc, rc)) return false;
    if (d2 < dmul(ri, ri)) return true;
    const int f = xc_filter(s, pos1, rot1, pos2bc, rot2);
    if (f >= 0) return f == 1;
    return xc_intersect(s, rot1, pos1, rot2, pos2bc, 1.0e-12, stuck);
}

// XenoCollideTraits::overlapWithWall (core/shapes/XenoCollideTraits.h:170-186): the wall normal w
// taken into the body frame, the body's support point against it, and the wall plane through o.
RP_XC_FN bool xc_wall_overlap(const XcShape &s, d3 pos, const double *rot, d3 o, d3 w) {
    const d3 nv = mtv3(rot, w);
    d3 sp;
    if (s.flat) sp = xc_support_flat(s, neg3(nv));
    else if (!xc_support(s, s.root, neg3(nv), sp)) return true;
    const d3 origin = mtv3(rot, sub3(o, pos));
    const double dist_support = dot3(neg3(sp), nv);
    const double dist_wall = dot3(neg3(origin), nv);
    return !(dist_wall > dist_support);
}

// Packing::countParticleWallOverlaps (core/Packing.cpp:1086-1139) for a convex body: per walled
// axis the nearer wall (through the origin, or through the far corner with the normal reversed)
// when the position lies within half the total range of it.
RP_HD int xc_wall_count(const XcShape &s, int walls, const double (*wall_vec)[3], const double *wall_far, double half,
                        d3 pos, const double *rot, bool early) {
    int cnt = 0;
    for (int i = 0; i < 3; i++) {
        if (!((walls >> i) & 1)) continue;
        const d3 w{wall_vec[i][0], wall_vec[i][1], wall_vec[i][2]};
        const d3 far{wall_far[0], wall_far[1], wall_far[2]};
        bool hit;
        if (dot3(pos, w) < half) hit = xc_wall_overlap(s, pos, rot, d3{0.0, 0.0, 0.0}, w);
        else if (dot3(sub3(far, pos), w) < half) hit = xc_wall_overlap(s, pos, rot, far, neg3(w));
        else continue;
        if (hit) {
            cnt++;
            if (early) return 1;
        }
    }
    return cnt;
}

// ---- the builder (host) ---------------------------------------------------------------------

// XCBodyBuilder (geometry/xenocollide/XCBodyBuilder.cpp:37-294) over the flattened node array:
// processes a script of commands, one per line or separated by ';'.  On success the shape holds
// the body (the last shape on the stack; its own move and rot are not part of the body, as
// releaseCollideGeometry returns the bare geometry) and `error` is empty.
bool xc_build(const std::string &script, XcShape &out, std::string &error);

}  // namespace rp
