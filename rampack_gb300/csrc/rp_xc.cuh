// Generic convex shapes (GenericXenoCollideTraits, core/shapes/GenericXenoCollideTraits.h):
// a body given by an XCBodyBuilder script (geometry/xenocollide/XCBodyBuilder.cpp), its support
// function, and the overlap test of core/shapes/XenoCollideTraits.h:118-140 by Minkowski portal
// refinement (Snethen's XenoCollide, geometry/xenocollide/XenoCollide.h:62-170).
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

struct XcShape {
    XcNode node[XC_MAX_NODES];
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
// XCUtils.h:31-34
RP_HD bool xc_zero(d3 v) {
    const double z = 9.094947e-13;
    return fabs(v.x) < z && fabs(v.y) < z && fabs(v.z) < z;
}
RP_HD d3 ld3(const double *p) { return {p[0], p[1], p[2]}; }

// Support point of a primitive in its own frame (geometry/xenocollide/XCPrimitives.cpp:36-163,
// XCPrimitives.h:44, :145).
RP_HD d3 xc_primitive_support(const XcNode &g, d3 n) {
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
RP_HD d3 xc_support_flat(const XcShape &s, d3 n) {
    const XcNode &g = s.node[s.root];
    if (g.type < XC_SUM) return xc_primitive_support(g, n);
    d3 acc{0.0, 0.0, 0.0};
    double best = 0.0;
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
RP_HD bool xc_support(const XcShape &s, int root, d3 n, d3 &out) {
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

// XenoCollide.h:55-61: the support point of a placed body.
RP_HD bool xc_transform_support(const XcShape &s, const double *rot, d3 pos, d3 n, d3 &out) {
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

// XenoCollide::Intersect (XenoCollide.h:67-169) for two copies of the body; `stuck` is set when
// the portal iterations exceed XC_MPR_LIMIT or the geometry is too deep (the pair is then
// reported as overlapping).
RP_HD bool xc_intersect(const XcShape &s, const double *rot1, d3 pos1, const double *rot2, d3 pos2, double tol,
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

// XenoCollideTraits::overlapBetween (core/shapes/XenoCollideTraits.h:118-140) with the second
// body already at its image (pos2bc = pos2 + translation).
RP_HD bool xc_overlap(const XcShape &s, d3 pos1, const double *rot1, d3 pos2bc, const double *rot2, bool &stuck) {
    const double rc = dadd(s.circ, s.circ);
    const double ri = dadd(s.insph, s.insph);
    const double d2 = norm2(sub3(pos2bc, pos1));
    if (d2 > dmul(rc, rc)) return false;
    if (d2 < dmul(ri, ri)) return true;
    return xc_intersect(s, rot1, pos1, rot2, pos2bc, 1.0e-12, stuck);
}

// ---- the builder (host) ---------------------------------------------------------------------

// XCBodyBuilder (geometry/xenocollide/XCBodyBuilder.cpp:37-294) over the flattened node array:
// processes a script of commands, one per line or separated by ';'.  On success the shape holds
// the body (the last shape on the stack; its own move and rot are not part of the body, as
// releaseCollideGeometry returns the bare geometry) and `error` is empty.
bool xc_build(const std::string &script, XcShape &out, std::string &error);

}  // namespace rp
