// XCBodyBuilder (geometry/xenocollide/XCBodyBuilder.cpp) over the flattened node array of
// rp_xc.cuh: the commands of XCBodyBuilder::processCommand (:181-294), the primitives'
// constructors (geometry/xenocollide/XCPrimitives.cpp:30-163) and the operations' radii and
// centres (geometry/xenocollide/XCOperations.cpp:30-185), host only.
#include <algorithm>
#include <cmath>
#include <sstream>

#include "rp_xc.cuh"

namespace rp {

namespace {

struct BuilderShape {   // XCBodyBuilder::XCShape
    int node;
    double rot[9];
    double pos[3];
};

// Matrix<3,3>::rotation(ax, ay, az) (geometry/Matrix.tpp:411-434)
void euler_rotation(double ax, double ay, double az, double *m) {
    const double sx = std::sin(ax), sy = std::sin(ay), sz = std::sin(az);
    const double cx = std::cos(ax), cy = std::cos(ay), cz = std::cos(az);
    m[0] = cy * cz;
    m[1] = sx * sy * cz - cx * sz;
    m[2] = cx * sy * cz + sx * sz;
    m[3] = cy * sz;
    m[4] = sx * sy * sz + cx * cz;
    m[5] = cx * sy * sz - sx * cz;
    m[6] = -sy;
    m[7] = sx * cy;
    m[8] = cx * cy;
}

struct Builder {
    XcShape &out;
    std::string &error;
    std::vector<BuilderShape> stack;

    bool fail(const std::string &msg) {
        error = msg;
        return false;
    }

    int new_node(int type) {
        if (out.nnodes >= XC_MAX_NODES) return -1;
        XcNode &g = out.node[out.nnodes];
        g = XcNode{};
        g.type = type;
        return out.nnodes++;
    }

    bool push_primitive(int type, double a, double b, double c, double circ, double insph) {
        const int id = new_node(type);
        if (id < 0) return fail("the body has more than " + std::to_string(XC_MAX_NODES) + " geometries");
        XcNode &g = out.node[id];
        g.p[0] = a;
        g.p[1] = b;
        g.p[2] = c;
        g.circ = circ;
        g.insph = insph;
        if (type == XC_POINT) {  // XCPoint::getCenter is its position (XCPrimitives.h:45)
            g.centre[0] = a;
            g.centre[1] = b;
            g.centre[2] = c;
        }
        BuilderShape s{id, {1, 0, 0, 0, 1, 0, 0, 0, 1}, {0, 0, 0}};
        stack.push_back(s);
        return true;
    }

    // rot * centre(child) + pos, each entry's centre in this node's frame
    d3 placed_centre(const XcNode &g, int i) const {
        return add3(mv3(g.erot[i], ld3(out.node[g.ent[i]].centre)), ld3(g.epos[i]));
    }

    // XCSum / XCMax: `count` shapes popped from the stack in turn become the entries
    // (XCBodyBuilder.cpp:158-170, :180-192)
    bool combine(int type, std::size_t count) {
        if (count > static_cast<std::size_t>(XC_MAX_ENTRIES))
            return fail("more than " + std::to_string(XC_MAX_ENTRIES) + " components in one sum or wrap");
        const int id = new_node(type);
        if (id < 0) return fail("the body has more than " + std::to_string(XC_MAX_NODES) + " geometries");
        XcNode &g = out.node[id];
        g.nent = static_cast<int>(count);
        for (std::size_t i = 0; i < count; i++) {
            const BuilderShape s = stack.back();
            stack.pop_back();
            g.ent[i] = s.node;
            for (int k = 0; k < 3; k++) g.epos[i][k] = s.pos[k];
            for (int k = 0; k < 9; k++) g.erot[i][k] = s.rot[k];
        }
        if (type == XC_SUM) {
            // XCSum::recalculateGeometry (XCOperations.cpp:57-70) and getCenter (:45-50)
            d3 centre_sum{0.0, 0.0, 0.0}, centre{0.0, 0.0, 0.0};
            double circ_sum = 0.0, insph_sum = 0.0;
            for (int i = 0; i < g.nent; i++) {
                centre_sum = add3(centre_sum, ld3(g.epos[i]));
                circ_sum += out.node[g.ent[i]].circ;
                insph_sum += out.node[g.ent[i]].insph;
                centre = add3(centre, placed_centre(g, i));
            }
            const double disp = norm3(centre_sum);
            g.circ = disp + circ_sum;
            g.insph = std::max(0., insph_sum - disp);
            g.centre[0] = centre.x, g.centre[1] = centre.y, g.centre[2] = centre.z;
        } else {
            // XCMax::recalculateGeometry (XCOperations.cpp:143-152), getCenter (:122-127)
            g.circ = norm3(ld3(g.epos[0])) + out.node[g.ent[0]].circ;
            d3 centre{0.0, 0.0, 0.0};
            for (int i = 0; i < g.nent; i++) {
                const double r = norm3(ld3(g.epos[i])) + out.node[g.ent[i]].circ;
                g.circ = std::max(g.circ, r);
                centre = add3(centre, placed_centre(g, i));
            }
            centre = div3(centre, static_cast<double>(g.nent));
            g.centre[0] = centre.x, g.centre[1] = centre.y, g.centre[2] = centre.z;
            g.insph = g.nent == 2 ? hull_insphere2(g) : 0.0;  // >= 3 entries: 0 (:133-135)
        }
        stack.push_back(BuilderShape{id, {1, 0, 0, 0, 1, 0, 0, 0, 1}, {0, 0, 0}});
        return true;
    }

    // XCMax::calculateInsphereRadius2 (XCOperations.cpp:159-185)
    double hull_insphere2(const XcNode &g) const {
        const double ins1 = out.node[g.ent[0]].insph, ins2 = out.node[g.ent[1]].insph;
        const d3 p1 = ld3(g.epos[0]), p2 = ld3(g.epos[1]);
        const d3 diff = sub3(p2, p1);
        const double diff_norm = norm3(diff);
        const d3 normal = div3(diff, diff_norm);
        if (diff_norm / std::max(ins1, ins2) < 1e-14) return std::min(ins1, ins2);
        const double t = -dot3(p1, normal) / diff_norm;
        if (t < 0) return 0;
        if (t > 1) return 0;
        const double proj = dot3(p1, normal);
        const double offset = std::sqrt(std::max(0.0, norm2(p1) - proj * proj));
        const double r = (1 - t) * ins1 + t * ins2;
        return std::max(0.0, r - offset);
    }

    // XCDiff (XCOperations.cpp:72-97)
    bool diff() {
        if (stack.size() < 2) return fail("Shape stack contains < 2 shapes; cannot compute Minkowski difference");
        const BuilderShape s2 = stack.back();
        stack.pop_back();
        const BuilderShape s1 = stack.back();
        stack.pop_back();
        const int id = new_node(XC_DIFF);
        if (id < 0) return fail("the body has more than " + std::to_string(XC_MAX_NODES) + " geometries");
        XcNode &g = out.node[id];
        g.nent = 2;
        const BuilderShape *s[2] = {&s1, &s2};
        for (int i = 0; i < 2; i++) {
            g.ent[i] = s[i]->node;
            for (int k = 0; k < 3; k++) g.epos[i][k] = s[i]->pos[k];
            for (int k = 0; k < 9; k++) g.erot[i][k] = s[i]->rot[k];
        }
        const XcNode &a = out.node[g.ent[0]], &b = out.node[g.ent[1]];
        const double disp = norm3(sub3(ld3(g.epos[0]), ld3(g.epos[1])));
        g.circ = disp + a.circ + b.circ;
        g.insph = std::max(0., a.insph + b.insph - disp);
        const d3 c = sub3(placed_centre(g, 0), placed_centre(g, 1));
        g.centre[0] = c.x, g.centre[1] = c.y, g.centre[2] = c.z;
        stack.push_back(BuilderShape{id, {1, 0, 0, 0, 1, 0, 0, 0, 1}, {0, 0, 0}});
        return true;
    }

    static bool anything_left(std::istringstream &in) {
        in >> std::ws;
        return in.peek() != std::char_traits<char>::eof();
    }

    // XCBodyBuilder::processCommand (XCBodyBuilder.cpp:194-294)
    bool command(const std::string &cmd) {
        std::istringstream in(cmd);
        std::string name;
        in >> name;
        double a = 0, b = 0, c = 0;
        if (name == "cuboid") {
            in >> a >> b >> c;
            if (!in) return fail("Malformed command arguments. Usage: cuboid [side x] [side y] [side z]");
            if (!(a > 0 && b > 0 && c > 0)) return fail("All cuboid side lengths should be positive");
            const d3 h{a / 2, b / 2, c / 2};
            return push_primitive(XC_CUBOID, h.x, h.y, h.z, norm3(h), std::min({h.x, h.y, h.z}));
        } else if (name == "diff") {
            return diff();
        } else if (name == "disk") {
            in >> a;
            if (!in) return fail("Malformed command arguments. Usage: disk [radius]");
            if (!(a > 0)) return fail("Disk radius should be positive");
            return push_primitive(XC_DISK, a, 0, 0, a, 0);
        } else if (name == "dup") {
            std::size_t k = 0;
            in >> k;
            if (!in) return fail("Malformed command arguments. Usage: dup [number of shapes]");
            if (k == 0) return fail("Number of shapes to duplicate should be positive");
            if (k > stack.size()) return fail("Number of shapes to duplicate is greater than total number of shapes");
            const std::size_t from = stack.size() - k;
            for (std::size_t i = 0; i < k; i++) stack.push_back(stack[from + i]);
            return true;
        } else if (name == "ellipse") {
            in >> a >> b;
            if (!in) return fail("Malformed command arguments. Usage: ellipse [semi-axis x] [semi-axis y]");
            if (!(a > 0 && b > 0)) return fail("Ellipse semiaxes' lengths should be positive");
            return push_primitive(XC_ELLIPSE, a, b, 0, std::max({a, b, 0.0}), 0);
        } else if (name == "ellipsoid") {
            in >> a >> b >> c;
            if (!in)
                return fail("Malformed command arguments. Usage: ellipsoid [semi-axis x] [semi-axis y] [semi-axis z]");
            if (!(a > 0 && b > 0 && c > 0)) return fail("Ellipsoid semiaxes' lengths should be positive");
            return push_primitive(XC_ELLIPSOID, a, b, c, std::max({a, b, c}), std::min({a, b, c}));
        } else if (name == "football") {
            in >> a >> b;
            if (!in) return fail("Malformed command arguments. Usage: football [length] [radius]");
            if (!(a > 0 && b > 0)) return fail("Length and radius of a football should be positive");
            if (!(a >= 2 * b)) return fail("Length of football should not be not smaller than its diameter");
            return push_primitive(XC_FOOTBALL, a / 2, b, 0, a / 2, b);
        } else if (name == "move") {
            in >> a >> b >> c;
            if (!in) return fail("Malformed command arguments. Usage: move [delta x] [delta y] [delta z]");
            if (stack.empty()) return fail("Shape stack is empty; cannot move");
            BuilderShape &s = stack.back();
            s.pos[0] = s.pos[0] + a;
            s.pos[1] = s.pos[1] + b;
            s.pos[2] = s.pos[2] + c;
            return true;
        } else if (name == "point") {
            in >> a >> b >> c;
            if (!in) return fail("Malformed command arguments. Usage: point [x] [y] [z]");
            return push_primitive(XC_POINT, a, b, c, 0, 0);
        } else if (name == "pop") {
            if (stack.empty()) return fail("Shape stack is empty; cannot pop last element");
            stack.pop_back();
            return true;
        } else if (name == "rectangle") {
            in >> a >> b;
            if (!in) return fail("Malformed command arguments. Usage: rectangle [side x] [side y]");
            if (!(a > 0 && b > 0)) return fail("Rectangle side lengths should be positive");
            const d3 h{a / 2, b / 2, 0.0};
            return push_primitive(XC_RECTANGLE, h.x, h.y, 0, norm3(h), 0);
        } else if (name == "rot") {
            in >> a >> b >> c;
            if (!in) return fail("Malformed command arguments. Usage: rot [angle x] [angle y] [angle z]");
            if (stack.empty()) return fail("Shape stack is empty; cannot rotate");
            double r[9], o[9];
            euler_rotation(a * M_PI / 180, b * M_PI / 180, c * M_PI / 180, r);
            double *cur = stack.back().rot;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) o[3 * i + j] = mm_elem(r, cur, i, j);
            for (int k = 0; k < 9; k++) cur[k] = o[k];
            return true;
        } else if (name == "saucer") {
            in >> a >> b;
            if (!in) return fail("Malformed command arguments. Usage: saucer [radius] [thickness]");
            if (!(a > 0 && b > 0)) return fail("Saucer radius and thickness should be positive");
            if (!(b <= 2 * a)) return fail("Saucer thickness cannot be larger than its diameter");
            return push_primitive(XC_SAUCER, a, b / 2, 0, a, b / 2);
        } else if (name == "segment") {
            in >> a;
            if (!in) return fail("Malformed command arguments. Usage: segment [length]");
            if (!(a > 0)) return fail("Segment length should be positive");
            return push_primitive(XC_SEGMENT, a / 2, 0, 0, a / 2, 0);
        } else if (name == "sphere") {
            in >> a;
            if (!in) return fail("Malformed command arguments. Usage: sphere [radius]");
            if (!(a > 0)) return fail("Sphere radius should be positive");
            return push_primitive(XC_SPHERE, a, 0, 0, a, a);
        } else if (name == "sum" || name == "wrap") {
            std::size_t k = 2;
            if (anything_left(in)) {
                in >> k;
                if (!in) return fail("Malformed command arguments. Usage: " + name + " ([number of shapes])");
            }
            if (k < 2)
                return fail(name == "sum" ? "Minkowski sum requires at least 2 components"
                                          : "Convex hull sum requires at least 2 components");
            if (stack.size() < k)
                return fail(name == "sum" ? "Shape stack contains too few shapes; cannot compute Minkowski sum"
                                          : "Shape stack contains too few shapes; cannot compute convex hull");
            return combine(name == "sum" ? XC_SUM : XC_MAX, k);
        } else if (name == "swap") {
            if (stack.size() < 2) return fail("Shape stack contains < 2 shapes; cannot swap them");
            std::swap(stack[stack.size() - 1], stack[stack.size() - 2]);
            return true;
        }
        return fail("Unknown XCBodyBuilder command: " + name);
    }

    int depth(int node) const {
        const XcNode &g = out.node[node];
        if (g.type < XC_SUM) return 1;
        int d = 0;
        for (int i = 0; i < g.nent; i++) d = std::max(d, depth(g.ent[i]));
        return d + 1;
    }
};

std::string trim(const std::string &s) {
    const auto b = s.find_first_not_of(" \t\r\n");
    if (b == std::string::npos) return "";
    const auto e = s.find_last_not_of(" \t\r\n");
    return s.substr(b, e - b + 1);
}

}  // namespace

bool xc_build(const std::string &script, XcShape &out, std::string &error) {
    out = XcShape{};
    error.clear();
    Builder b{out, error, {}};
    std::string cmd;
    for (std::size_t i = 0; i <= script.size(); i++) {
        if (i == script.size() || script[i] == '\n' || script[i] == ';') {
            const std::string c = trim(cmd);
            cmd.clear();
            if (c.empty()) continue;
            if (!b.command(c)) return false;
        } else {
            cmd += script[i];
        }
    }
    // XCBodyBuilder::releaseCollideGeometry (XCBodyBuilder.cpp:37-48): the bare geometry
    if (b.stack.empty()) return b.fail("XCBodyBuilder: shape stack is empty");
    if (b.stack.size() > 1)
        return b.fail("XCBodyBuilder: shape stack contains more than 1 shape; did you forget to use sum, diff or wrap?");
    out.root = b.stack.back().node;
    if (b.depth(out.root) > XC_MAX_DEPTH - 1)
        return b.fail("the body nests more than " + std::to_string(XC_MAX_DEPTH - 1) + " geometries");
    // the FP32 copy of every node for the device's filter
    for (int i = 0; i < out.nnodes; i++) {
        const XcNode &g = out.node[i];
        XcNodeF &f = out.fnode[i];
        f.type = g.type;
        f.nent = g.nent;
        for (int e = 0; e < XC_MAX_ENTRIES; e++) {
            f.ent[e] = g.ent[e];
            for (int k = 0; k < 3; k++) f.epos[e][k] = static_cast<float>(g.epos[e][k]);
            for (int k = 0; k < 9; k++) f.erot[e][k] = static_cast<float>(g.erot[e][k]);
        }
        for (int k = 0; k < 3; k++) f.p[k] = static_cast<float>(g.p[k]);
    }
    const XcNode &r = out.node[out.root];
    for (int k = 0; k < 3; k++) out.fcentre[k] = static_cast<float>(r.centre[k]);
    out.flat = 1;
    if (r.type >= XC_SUM)
        for (int i = 0; i < r.nent; i++) out.flat = out.flat && out.node[r.ent[i]].type < XC_SUM;
    out.circ = r.circ;
    out.insph = r.insph;
    for (int k = 0; k < 3; k++) out.centre[k] = r.centre[k];
    return true;
}

}  // namespace rp
