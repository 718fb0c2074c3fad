// ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load or call anything under oracle/; the
// product path (rampack_gb300/) never does.
//
// Generic convex bodies restated from the reference: the XenoCollide geometries
// (geometry/xenocollide/XCPrimitives.cpp, XCOperations.cpp), XCBodyBuilder's commands
// (geometry/xenocollide/XCBodyBuilder.cpp:37-294), Snethen's portal refinement as adapted in
// geometry/xenocollide/XenoCollide.h:74-168 and the pair test of
// core/shapes/XenoCollideTraits.h:147-168 — as polymorphic objects, the reference's own
// structure, in its operation order (compiled with -ffp-contract=off).
#pragma once

#include <algorithm>
#include <cmath>
#include <list>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "rpo_geometry.hpp"

namespace rpo {

// geometry/xenocollide/XCUtils.h:31-39
inline bool xc_is_zero(const V3 &v) {
    constexpr double ZERO = 9.094947e-13;
    return std::abs(v[0]) < ZERO && std::abs(v[1]) < ZERO && std::abs(v[2]) < ZERO;
}
inline V3 xc_comp_mul(const V3 &a, const V3 &b) { return {a[0] * b[0], a[1] * b[1], a[2] * b[2]}; }
inline V3 xc_neg(const V3 &a) { return {-a[0], -a[1], -a[2]}; }
inline V3 xc_normalized(const V3 &a) { return vdiv(a, std::sqrt(norm2(a))); }

// AbstractXCGeometry (geometry/xenocollide/AbstractXCGeometry.h:39-47)
struct XcGeom {
    virtual ~XcGeom() = default;
    virtual V3 support(const V3 &n) const = 0;
    virtual V3 centre() const { return {0, 0, 0}; }
    virtual double circ() const = 0;
    virtual double insph() const = 0;
};
using XcPtr = std::shared_ptr<XcGeom>;

struct XcPoint : XcGeom {   // XCPrimitives.h:34-48
    V3 pos;
    explicit XcPoint(const V3 &p) : pos(p) {}
    V3 support(const V3 &) const override { return pos; }
    V3 centre() const override { return pos; }
    double circ() const override { return 0; }
    double insph() const override { return 0; }
};
struct XcSegment : XcGeom {   // XCPrimitives.cpp:30-41
    double h;
    explicit XcSegment(double hl) : h(hl) {}
    V3 support(const V3 &n) const override {
        V3 v{0, 0, 0};
        v[2] = n[2] < 0 ? -h : h;
        return v;
    }
    double circ() const override { return h; }
    double insph() const override { return 0; }
};
struct XcRectangle : XcGeom {   // XCPrimitives.cpp:43-54
    V3 half;
    double c;
    XcRectangle(double hx, double hy) : half{hx, hy, 0}, c(std::sqrt(norm2(half))) {}
    V3 support(const V3 &n) const override {
        V3 r = half;
        if (n[0] < 0) r[0] = -r[0];
        if (n[1] < 0) r[1] = -r[1];
        return r;
    }
    double circ() const override { return c; }
    double insph() const override { return 0; }
};
struct XcCuboid : XcGeom {   // XCPrimitives.cpp:56-69
    V3 half;
    double c, i;
    explicit XcCuboid(const V3 &h) : half(h), c(std::sqrt(norm2(h))), i(*std::min_element(h.begin(), h.end())) {}
    V3 support(const V3 &n) const override {
        V3 r = half;
        for (int k = 0; k < 3; k++)
            if (n[k] < 0) r[k] = -r[k];
        return r;
    }
    double circ() const override { return c; }
    double insph() const override { return i; }
};
struct XcDisk : XcGeom {   // XCPrimitives.cpp:71-81
    double r;
    explicit XcDisk(double rr) : r(rr) {}
    V3 support(const V3 &n) const override {
        V3 n2 = n;
        n2[2] = 0;
        if (xc_is_zero(n2)) return {0, 0, 0};
        return vscale(xc_normalized(n2), r);
    }
    double circ() const override { return r; }
    double insph() const override { return 0; }
};
struct XcSphere : XcGeom {   // XCPrimitives.h:135-148
    double r;
    explicit XcSphere(double rr) : r(rr) {}
    V3 support(const V3 &n) const override { return vscale(xc_normalized(n), r); }
    double circ() const override { return r; }
    double insph() const override { return r; }
};
struct XcEllipse : XcGeom {   // XCPrimitives.cpp:87-100
    V3 axes;
    double c;
    XcEllipse(double a, double b) : axes{a, b, 0}, c(*std::max_element(axes.begin(), axes.end())) {}
    V3 support(const V3 &n) const override {
        V3 n2 = xc_comp_mul(axes, n);
        if (xc_is_zero(n2)) return {0, 0, 0};
        return xc_comp_mul(xc_normalized(n2), axes);
    }
    double circ() const override { return c; }
    double insph() const override { return 0; }
};
struct XcEllipsoid : XcGeom {   // XCPrimitives.cpp:102-113
    V3 axes;
    double c, i;
    explicit XcEllipsoid(const V3 &a)
        : axes(a), c(*std::max_element(a.begin(), a.end())), i(*std::min_element(a.begin(), a.end())) {}
    V3 support(const V3 &n) const override { return xc_comp_mul(xc_normalized(xc_comp_mul(n, axes)), axes); }
    double circ() const override { return c; }
    double insph() const override { return i; }
};
struct XcFootball : XcGeom {   // XCPrimitives.cpp:115-135
    double h, r1;
    XcFootball(double hl, double r) : h(hl), r1(r) {}
    V3 support(const V3 &n) const override {
        double r2 = 0.5f * (h * h / r1 + r1);
        V3 n3 = xc_normalized(n);
        if (n3[2] * r2 < -h) return {0, 0, -h};
        if (n3[2] * r2 > h) return {0, 0, h};
        V3 n2 = xc_normalized(V3{n[0], n[1], 0});
        return add(vscale(xc_neg(n2), r2 - r1), vscale(n3, r2));
    }
    double circ() const override { return h; }
    double insph() const override { return r1; }
};
struct XcSaucer : XcGeom {   // XCPrimitives.cpp:137-163
    double h, t;
    XcSaucer(double radius, double half_thickness) : h(radius), t(half_thickness) {}
    V3 support(const V3 &n) const override {
        double r2 = 0.5f * (h * h / t + t);
        V3 n3 = xc_normalized(n);
        V3 n4{n[0], n[1], 0};
        if (!xc_is_zero(n4)) {
            n4 = xc_normalized(n4);
            double threshold = n3[0] * n3[0] + n3[1] * n3[1];
            if (threshold * r2 * r2 > h * h) return vscale(n4, h);
        }
        V3 n2{0, 0, 1};
        if (n[2] < 0) n2 = xc_neg(n2);
        return add(vscale(xc_neg(n2), r2 - t), vscale(n3, r2));
    }
    double circ() const override { return h; }
    double insph() const override { return t; }
};

struct XcEntry {
    XcPtr g;
    V3 pos;
    M3 rot;
};
inline V3 xc_entry_support(const XcEntry &e, const V3 &n) {
    return add(mv(e.rot, e.g->support(mv(transpose(e.rot), n))), e.pos);
}
inline V3 xc_entry_centre(const XcEntry &e) { return add(mv(e.rot, e.g->centre()), e.pos); }

struct XcSum : XcGeom {   // XCOperations.cpp:31-70
    std::vector<XcEntry> entries;
    double c = 0, i = 0;
    void add_entry(const XcEntry &e) {
        entries.push_back(e);
        V3 cs{0, 0, 0};
        double csum = 0, isum = 0;
        for (auto &x : entries) {
            cs = add(cs, x.pos);
            csum += x.g->circ();
            isum += x.g->insph();
        }
        double d = std::sqrt(norm2(cs));
        c = d + csum;
        i = std::max(0., isum - d);
    }
    V3 support(const V3 &n) const override {
        V3 p{0, 0, 0};
        for (auto &e : entries) p = add(p, xc_entry_support(e, n));
        return p;
    }
    V3 centre() const override {
        V3 p{0, 0, 0};
        for (auto &e : entries) p = add(p, xc_entry_centre(e));
        return p;
    }
    double circ() const override { return c; }
    double insph() const override { return i; }
};
struct XcDiff : XcGeom {   // XCOperations.cpp:72-97
    XcEntry a, b;
    double c, i;
    XcDiff(const XcEntry &e1, const XcEntry &e2) : a(e1), b(e2) {
        double d = std::sqrt(norm2(sub(a.pos, b.pos)));
        c = d + a.g->circ() + b.g->circ();
        i = std::max(0., a.g->insph() + b.g->insph() - d);
    }
    V3 support(const V3 &n) const override {
        V3 p1 = add(mv(a.rot, a.g->support(mv(transpose(a.rot), n))), a.pos);
        V3 p2 = add(mv(b.rot, b.g->support(mv(transpose(b.rot), xc_neg(n)))), b.pos);
        return sub(p1, p2);
    }
    V3 centre() const override { return sub(xc_entry_centre(a), xc_entry_centre(b)); }
    double circ() const override { return c; }
    double insph() const override { return i; }
};
struct XcMax : XcGeom {   // XCOperations.cpp:97-185
    std::vector<XcEntry> entries;
    double c = 0, i = 0;
    void add_entry(const XcEntry &e) {
        entries.push_back(e);
        c = std::sqrt(norm2(entries.front().pos)) + entries.front().g->circ();
        for (auto &x : entries) c = std::max(c, std::sqrt(norm2(x.pos)) + x.g->circ());
        if (entries.size() == 1)
            i = std::max(0.0, entries.front().g->insph() - std::sqrt(norm2(entries.front().pos)));
        else if (entries.size() == 2)
            i = insphere2();
        else
            i = 0;
    }
    double insphere2() const {
        const XcEntry &e1 = entries[0], &e2 = entries[1];
        double i1 = e1.g->insph(), i2 = e2.g->insph();
        V3 diff = sub(e2.pos, e1.pos);
        double dn = std::sqrt(norm2(diff));
        V3 nd = vdiv(diff, dn);
        if (dn / std::max(i1, i2) < 1e-14) return std::min(i1, i2);
        double t = -dot(e1.pos, nd) / dn;
        if (t < 0) return 0;
        if (t > 1) return 0;
        double pr = dot(e1.pos, nd);
        double off = std::sqrt(std::max(0.0, norm2(e1.pos) - pr * pr));
        double r = (1 - t) * i1 + t * i2;
        return std::max(0.0, r - off);
    }
    V3 support(const V3 &n) const override {
        V3 v = xc_entry_support(entries.front(), n);
        double best = dot(v, n);
        for (std::size_t k = 1; k < entries.size(); k++) {
            V3 v1 = xc_entry_support(entries[k], n);
            double pr = dot(v1, n);
            if (pr > best) {
                v = v1;
                best = pr;
            }
        }
        return v;
    }
    V3 centre() const override {
        V3 p{0, 0, 0};
        for (auto &e : entries) p = add(p, xc_entry_centre(e));
        return vdiv(p, static_cast<double>(entries.size()));
    }
    double circ() const override { return c; }
    double insph() const override { return i; }
};

// XCBodyBuilder: commands one per line or separated by ';'; throws std::invalid_argument.
inline XcPtr xc_build_script(const std::string &script) {
    struct Item {
        XcPtr g;
        M3 rot;
        V3 pos;
    };
    std::list<Item> st;
    auto need = [](bool ok, const char *msg) {
        if (!ok) throw std::invalid_argument(msg);
    };
    auto push = [&](XcPtr g) { st.push_back(Item{std::move(g), identity(), V3{0, 0, 0}}); };
    auto pop_entry = [&]() {
        Item it = st.back();
        st.pop_back();
        return XcEntry{it.g, it.pos, it.rot};
    };
    std::vector<std::string> cmds;
    {
        std::string cur;
        for (char ch : script + "\n") {
            if (ch == '\n' || ch == ';') {
                cmds.push_back(cur);
                cur.clear();
            } else {
                cur += ch;
            }
        }
    }
    for (const std::string &raw : cmds) {
        std::istringstream in(raw);
        std::string name;
        if (!(in >> name)) continue;
        double a, b, c;
        if (name == "cuboid") {
            in >> a >> b >> c;
            need(bool(in) && a > 0 && b > 0 && c > 0, "cuboid");
            push(std::make_shared<XcCuboid>(V3{a / 2, b / 2, c / 2}));
        } else if (name == "disk") {
            in >> a;
            need(bool(in) && a > 0, "disk");
            push(std::make_shared<XcDisk>(a));
        } else if (name == "ellipse") {
            in >> a >> b;
            need(bool(in) && a > 0 && b > 0, "ellipse");
            push(std::make_shared<XcEllipse>(a, b));
        } else if (name == "ellipsoid") {
            in >> a >> b >> c;
            need(bool(in) && a > 0 && b > 0 && c > 0, "ellipsoid");
            push(std::make_shared<XcEllipsoid>(V3{a, b, c}));
        } else if (name == "football") {
            in >> a >> b;
            need(bool(in) && a > 0 && b > 0 && a >= 2 * b, "football");
            push(std::make_shared<XcFootball>(a / 2, b));
        } else if (name == "point") {
            in >> a >> b >> c;
            need(bool(in), "point");
            push(std::make_shared<XcPoint>(V3{a, b, c}));
        } else if (name == "rectangle") {
            in >> a >> b;
            need(bool(in) && a > 0 && b > 0, "rectangle");
            push(std::make_shared<XcRectangle>(a / 2, b / 2));
        } else if (name == "saucer") {
            in >> a >> b;
            need(bool(in) && a > 0 && b > 0 && b <= 2 * a, "saucer");
            push(std::make_shared<XcSaucer>(a, b / 2));
        } else if (name == "segment") {
            in >> a;
            need(bool(in) && a > 0, "segment");
            push(std::make_shared<XcSegment>(a / 2));
        } else if (name == "sphere") {
            in >> a;
            need(bool(in) && a > 0, "sphere");
            push(std::make_shared<XcSphere>(a));
        } else if (name == "move") {
            in >> a >> b >> c;
            need(bool(in) && !st.empty(), "move");
            st.back().pos = add(st.back().pos, V3{a, b, c});
        } else if (name == "rot") {
            in >> a >> b >> c;
            need(bool(in) && !st.empty(), "rot");
            st.back().rot = mm(rotation_euler(a * M_PI / 180, b * M_PI / 180, c * M_PI / 180), st.back().rot);
        } else if (name == "sum" || name == "wrap") {
            std::size_t k = 2;
            in >> std::ws;
            if (in.peek() != std::char_traits<char>::eof()) {
                in >> k;
                need(bool(in), "sum/wrap count");
            }
            need(k >= 2 && st.size() >= k, "sum/wrap");
            if (name == "sum") {
                auto s = std::make_shared<XcSum>();
                for (std::size_t q = 0; q < k; q++) s->add_entry(pop_entry());
                push(s);
            } else {
                auto m = std::make_shared<XcMax>();
                for (std::size_t q = 0; q < k; q++) m->add_entry(pop_entry());
                push(m);
            }
        } else if (name == "diff") {
            need(st.size() >= 2, "diff");
            XcEntry e2 = pop_entry();
            XcEntry e1 = pop_entry();
            push(std::make_shared<XcDiff>(e1, e2));
        } else if (name == "dup") {
            std::size_t k;
            in >> k;
            need(bool(in) && k > 0 && k <= st.size(), "dup");
            auto it = st.end();
            std::advance(it, -static_cast<long>(k));
            for (std::size_t q = 0; q < k; q++) st.push_back(*it++);
        } else if (name == "pop") {
            need(!st.empty(), "pop");
            st.pop_back();
        } else if (name == "swap") {
            need(st.size() >= 2, "swap");
            auto i1 = std::prev(st.end());
            auto i2 = std::prev(i1);
            std::swap(*i1, *i2);
        } else {
            throw std::invalid_argument("unknown command " + name);
        }
    }
    need(st.size() == 1, "the script must leave one shape");
    return st.back().g;
}

// XenoCollide::Intersect (geometry/xenocollide/XenoCollide.h:58-168)
inline V3 xc_tsv(const XcGeom &g, const M3 &rot, const V3 &pos, const V3 &n) {
    return add(mv(rot, g.support(mv(transpose(rot), n))), pos);
}
inline bool xc_intersect(const XcGeom &g1, const M3 &r1, const V3 &p1, const XcGeom &g2, const M3 &r2, const V3 &p2,
                         double tol) {
    V3 v0 = sub(add(mv(r2, g2.centre()), p2), add(mv(r1, g1.centre()), p1));
    if (xc_is_zero(v0)) return true;
    V3 n = xc_neg(v0);
    V3 v1 = sub(xc_tsv(g2, r2, p2, n), xc_tsv(g1, r1, p1, xc_neg(n)));
    if (dot(v1, n) <= 0) return false;
    n = cross(v1, v0);
    if (xc_is_zero(n)) return true;
    V3 v2 = sub(xc_tsv(g2, r2, p2, n), xc_tsv(g1, r1, p1, xc_neg(n)));
    if (dot(v2, n) <= 0) return false;
    n = cross(sub(v1, v0), sub(v2, v0));
    if (dot(n, v0) > 0) {
        std::swap(v1, v2);
        n = xc_neg(n);
    }
    while (true) {
        V3 v3 = sub(xc_tsv(g2, r2, p2, n), xc_tsv(g1, r1, p1, xc_neg(n)));
        if (dot(v3, n) <= 0) return false;
        if (dot(cross(v1, v3), v0) < 0) {
            v2 = v3;
            n = cross(sub(v1, v0), sub(v3, v0));
            continue;
        }
        if (dot(cross(v3, v2), v0) < 0) {
            v1 = v3;
            n = cross(sub(v3, v0), sub(v2, v0));
            continue;
        }
        while (true) {
            n = cross(sub(v2, v1), sub(v3, v1));
            if (dot(n, v1) >= 0) return true;
            V3 v4 = sub(xc_tsv(g2, r2, p2, n), xc_tsv(g1, r1, p1, xc_neg(n)));
            n = xc_normalized(n);
            if (-dot(v4, n) >= 0 || dot(sub(v4, v3), n) <= tol) return false;
            V3 cr = cross(v4, v0);
            if (dot(v1, cr) > 0) {
                if (dot(v2, cr) > 0) v1 = v4;
                else v3 = v4;
            } else {
                if (dot(v3, cr) > 0) v2 = v4;
                else v1 = v4;
            }
        }
    }
}

// XenoCollideTraits::overlapBetween (core/shapes/XenoCollideTraits.h:147-168), the second body
// at p2bc = pos2 + translation.
inline bool xc_overlap(const XcGeom &g, const V3 &p1, const M3 &o1, const V3 &p2bc, const M3 &o2) {
    double rc = g.circ() + g.circ();
    double ri = g.insph() + g.insph();
    double d2 = norm2(sub(p2bc, p1));
    if (d2 > rc * rc) return false;
    if (d2 < ri * ri) return true;
    return xc_intersect(g, o1, p1, g, o2, p2bc, 1.0e-12);
}

}  // namespace rpo
