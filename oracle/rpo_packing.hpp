// ORACLE — test infrastructure only (see rpo_geometry.hpp).
//
// CPU restatement of the reference's move-and-overlap path: hard interactions
// (core/shapes/*Traits.cpp), the linked-list NeighbourGrid with reflected halo
// cells (core/NeighbourGrid.cpp), and Packing's try/accept/revert and overlap
// counting (core/Packing.cpp).  Thread-slot temporaries follow the reference
// (one temp slot per OpenMP thread at the end of the shape vector).
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <numeric>
#include <optional>
#include <stdexcept>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#define RPO_TID static_cast<std::size_t>(omp_get_thread_num())
#define RPO_MAXTHREADS static_cast<std::size_t>(omp_get_max_threads())
#else
#define RPO_TID std::size_t(0)
#define RPO_MAXTHREADS std::size_t(1)
#endif

#include "rpo_geometry.hpp"
#include "rpo_xc.hpp"

namespace rpo {

struct Shape {
    V3 pos{};
    M3 rot = identity();
    // core/Shape.cpp:9-12
    void translate(const V3 &t, const Box &box) {
        pos = add(pos, t);
        pos = add(pos, pbc_correction(box, pos));
    }
    // core/Shape.cpp:14-16
    void rotate(const M3 &r) { rot = mm(r, rot); }
};

enum ShapeKind { SPHERE = 0, SPHEROCYLINDER = 1, POLYSPHERE = 2, CONVEX = 4 };

// The hard interactions of the BASELINE shapes.
struct Interaction {
    int kind = SPHERE;
    double radius = 0.5;   // sphere / spherocylinder radius
    double length = 0;     // spherocylinder cylinder length
    std::vector<V3> centres;      // polysphere body-frame sphere centres
    std::vector<double> radii;    // polysphere sphere radii
    // polyspherocylinders (PolyspherocylinderTraits): each centre is a spherocylinder with
    // this body-frame half axis (SpherocylinderData::halfAxis); empty for polyspheres
    std::vector<V3> half_axes;
    // generic convex bodies (GenericXenoCollideTraits): the XCBodyBuilder geometry
    std::shared_ptr<XcGeom> xc;

    // Soft part: a CentralInteraction helper installed on the same interaction centres and
    // joined to the hard shape by CompoundInteraction (core/interactions/CompoundInteraction.cpp:9-49):
    // 0 none, 1 RepulsiveLennardJonesInteraction (RepulsiveLennardJonesInteraction.cpp:9-22),
    // 2 SquareInverseCoreInteraction (SquareInverseCoreInteraction.cpp:8-15); `hard` false
    // leaves the soft part alone (SphereTraits(r, centralInteraction), no hard core)
    int soft = 0;
    double soft_eps = 0, soft_sigma = 0;
    double soft_cut = 0;   // RepulsiveLennardJones: sigma * std::pow(2., 1./6)
    bool hard = true;

    void set_soft(int kind, double eps, double sigma, bool with_hard) {
        soft = kind;
        soft_eps = eps;
        soft_sigma = sigma;
        soft_cut = sigma * std::pow(2., 1. / 6);
        hard = with_hard;
    }
    // CentralInteraction::getRangeRadius of the potential (RepulsiveLennardJonesInteraction.h:26,
    // SquareInverseCoreInteraction.h:22)
    double soft_range() const { return soft == 1 ? soft_cut : (soft == 2 ? soft_sigma : 0.0); }
    // calculateEnergyForDistance2
    double energy_for_distance2(double d2) const {
        if (soft == 1) {
            if (d2 >= soft_cut * soft_cut) return 0;
            double x2 = soft_sigma * soft_sigma / d2;
            double x6 = x2 * x2 * x2;
            double x12 = x6 * x6;
            return 4 * soft_eps * (x12 - x6) + soft_eps;
        }
        if (soft == 2) return soft_eps * std::max(0.0, std::pow(soft_sigma, 2) / d2 - 1);
        return 0;
    }
    // CentralInteraction::calculateEnergyBetween (core/interactions/CentralInteraction.h:55-63)
    double energy(const V3 &p1, const V3 &p2, const BC &bc) const { return energy_for_distance2(bc.distance2(p1, p2)); }

    bool segments() const { return !half_axes.empty(); }
    // SpherocylinderData::circumsphereRadius = radius + |halfAxis|
    // (PolyspherocylinderTraits.cpp:78-84)
    double circumsphere(std::size_t i) const { return radii[i] + std::sqrt(norm2(half_axes[i])); }

    // CompoundInteraction: the larger of the hard and the soft range (CompoundInteraction.cpp:33-35)
    double range() const {
        if (!soft) return hard_range();
        return hard ? std::max(hard_range(), soft_range()) : soft_range();
    }
    // SphereTraits.h:34, SpherocylinderTraits.h:81, PolysphereTraits.cpp:115-121
    double hard_range() const {
        if (kind == SPHERE) return 2 * radius;
        if (kind == SPHEROCYLINDER) return 2 * radius + length;
        if (kind == CONVEX) return 2 * xc->circ();   // XenoCollideTraits.h:188-202
        if (segments()) {   // PolyspherocylinderTraits.cpp:140-147
            double m = circumsphere(0);
            for (std::size_t i = 1; i < radii.size(); i++)
                if (m < circumsphere(i)) m = circumsphere(i);
            return 2 * m;
        }
        return 2 * *std::max_element(radii.begin(), radii.end());
    }
    // Interaction.cpp:55-70 (both parts share the interaction centres, so the compound's
    // larger total range is the larger range plus the centres' extent)
    double total_range() const {
        double r = range();
        if (kind != POLYSPHERE) return r;
        double m2 = 0;
        for (auto &c : centres) m2 = std::max(m2, norm2(c));
        return 2 * std::sqrt(m2) + r;
    }
    std::size_t num_centres() const { return kind == POLYSPHERE ? centres.size() : 0; }

    // overlapWithWall: SphereTraits.cpp:67-75, SpherocylinderTraits.cpp:56-73 (either cap
    // closer to the wall plane than the radius), PolysphereTraits.cpp:129-136 (centre idx)
    bool overlap_with_wall(const V3 &pos, const M3 &rot, std::size_t idx, const V3 &origin, const V3 &wall) const {
        if (!hard) return false;   // a soft part has no wall part (CentralInteraction.h:48)
        if (kind == SPHERE) return dot(wall, sub(pos, origin)) < radius;
        if (kind == CONVEX) {   // XenoCollideTraits.h:170-186, in the body frame
            const V3 nv = mv(transpose(rot), wall);
            const V3 sp = xc->support(xc_neg(nv));
            const V3 o = mv(transpose(rot), sub(origin, pos));
            return !(dot(xc_neg(o), nv) > dot(xc_neg(sp), nv));
        }
        if (kind == POLYSPHERE && segments()) {   // PolyspherocylinderTraits.cpp:149-166
            V3 half = mv(rot, half_axes[idx]);
            if (dot(wall, sub(sub(pos, half), origin)) < radii[idx]) return true;
            if (dot(wall, sub(add(pos, half), origin)) < radii[idx]) return true;
            return false;
        }
        if (kind == POLYSPHERE) return dot(wall, sub(pos, origin)) < radii[idx];
        V3 half = vscale(column(rot, 2), length / 2);
        if (dot(wall, sub(add(pos, half), origin)) < radius) return true;
        if (dot(wall, sub(sub(pos, half), origin)) < radius) return true;
        return false;
    }
    // CompoundInteraction::isConvex (CompoundInteraction.cpp:25-30): the hard part's, none without
    bool convex() const { return hard && kind != POLYSPHERE; }

    // SpherocylinderTraits.cpp:23-25
    V3 cap(int sign, const V3 &pos, const M3 &rot) const {
        return add(pos, vscale(column(rot, 2), 0.5 * sign * length));
    }

    bool overlap(const V3 &p1, const M3 &o1, std::size_t i1, const V3 &p2, const M3 &o2, std::size_t i2,
                 const BC &bc) const {
        if (!hard) return false;   // no hard part: nothing overlaps
        if (kind == SPHERE) {
            // SphereTraits.cpp:56-65
            return bc.distance2(p1, p2) < std::pow(2 * radius, 2);
        } else if (kind == CONVEX) {
            // XenoCollideTraits.h:147-168
            return xc_overlap(*xc, p1, o1, add(p2, bc.translation(p1, p2)), o2);
        } else if (kind == SPHEROCYLINDER) {
            // SpherocylinderTraits.cpp:28-46
            V3 p2bc = add(p2, bc.translation(p1, p2));
            double d2 = norm2(sub(p2bc, p1));
            if (d2 < 4 * radius * radius) return true;
            else if (d2 >= std::pow(2 * radius + length, 2)) return false;
            return segment_distance2(cap(-1, p1, o1), cap(1, p1, o1), cap(-1, p2bc, o2), cap(1, p2bc, o2))
                   < 4 * radius * radius;
        } else if (segments()) {
            // PolyspherocylinderTraits.cpp:102-124
            V3 p2bc = add(p2, bc.translation(p1, p2));
            double d2 = norm2(sub(p2bc, p1));
            double in = radii[i1] + radii[i2];
            double in2 = in * in;
            if (d2 < in2) return true;
            double circ = circumsphere(i1) + circumsphere(i2);
            if (d2 >= circ * circ) return false;
            V3 h1 = mv(o1, half_axes[i1]), h2 = mv(o2, half_axes[i2]);
            return segment_distance2(add(p1, h1), sub(p1, h1), add(p2bc, h2), sub(p2bc, h2)) < in2;
        } else {
            // PolysphereTraits.cpp:97-106
            double r = radii[i1] + radii[i2];
            return bc.distance2(p1, p2) < r * r;
        }
    }
};

// ---------------------------------------------------------------------------------------
// NeighbourGrid restated from core/NeighbourGrid.cpp.  Cells carry a one-cell reflected
// halo on every face; a halo cell aliases a real cell plus one of 27 box translations.
// ---------------------------------------------------------------------------------------
class NeighbourGrid {
public:
    static constexpr std::size_t END = std::numeric_limits<std::size_t>::max();

    Box box;
    std::array<std::size_t, 3> div{};   // including the two halo layers
    V3 rel_cell{};
    std::vector<std::size_t> heads, succ, reflected, trans_idx;
    std::array<V3, 27> translations{};
    std::size_t num_cells = 0;
    std::vector<std::size_t> offsets, positive_offsets;

    NeighbourGrid(const Box &b, double cell, std::size_t n_ids) {
        setup_sizes(b, cell);
        heads.assign(num_cells, END);
        trans_idx.resize(num_cells);
        reflected.resize(num_cells);
        succ.assign(n_ids, END);
        for (std::size_t i = 0; i < num_cells; i++) reflected_data(i, reflected[i], trans_idx[i]);
        fill_offsets();
    }

    // NeighbourGrid.cpp:178-201
    void setup_sizes(const Box &b, double cell) {
        V3 h = b.heights();
        std::array<std::size_t, 3> d{};
        for (int i = 0; i < 3; i++) {
            d[i] = static_cast<std::size_t>(std::floor(h[i] / cell)) + 2;
            if (d[i] < 3) throw std::runtime_error("Neighbour grid cell too big");
        }
        box = b;
        div = d;
        for (int i = 0; i < 3; i++) rel_cell[i] = 1 / static_cast<double>(div[i] - 2);
        // NeighbourGrid.cpp:203-217
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++) {
                    V3 rel{static_cast<double>(i) - 1, static_cast<double>(j) - 1., static_cast<double>(k) - 1.};
                    translations[i * 9 + j * 3 + k] = box.rel_to_abs(rel);
                }
        num_cells = div[0] * div[1] * div[2];
    }

    // NeighbourGrid.cpp:13-34
    std::size_t position_to_cell(const V3 &p) const {
        std::size_t r = 0;
        V3 rel = box.abs_to_rel(p);
        for (int i = 2; i >= 0; i--) {
            const double EPS = std::numeric_limits<double>::epsilon() * 10;
            double x = rel[i];
            if (x < 0) {
                if (!(x > -EPS)) throw std::runtime_error("position outside the box");
                x = 0;
            } else if (x >= 1) {
                if (!(x < 1 + EPS)) throw std::runtime_error("position outside the box");
                x = 1 - EPS;
            }
            std::size_t c = static_cast<int>(x / rel_cell[i]) + 1;
            r = div[i] * r + c;
        }
        return r;
    }
    std::array<std::size_t, 3> cell_coords(std::size_t n) const {
        std::array<std::size_t, 3> c{};
        for (int i = 0; i < 3; i++) { c[i] = n % div[i]; n /= div[i]; }
        return c;
    }
    std::size_t coords_to_cell(const std::array<std::size_t, 3> &c) const {
        std::size_t r = 0;
        for (int i = 2; i >= 0; i--) r = div[i] * r + c[i];
        return r;
    }
    std::size_t real_coords_to_cell(const std::array<std::size_t, 3> &c) const {
        std::size_t r = 0;
        for (int i = 2; i >= 0; i--) r = div[i] * r + c[i] + 1;
        return r;
    }
    // NeighbourGrid.cpp:80-100
    void reflected_data(std::size_t cell, std::size_t &real, std::size_t &tidx) const {
        auto c = cell_coords(cell);
        std::array<std::size_t, 3> tc{1, 1, 1};
        bool refl = false;
        for (int i = 0; i < 3; i++) {
            if (c[i] == 0) { c[i] = div[i] - 2; tc[i] = 0; refl = true; }
            else if (c[i] == div[i] - 1) { c[i] = 1; tc[i] = 2; refl = true; }
        }
        if (!refl) { real = cell; tidx = 13; return; }
        real = coords_to_cell(c);
        tidx = tc[0] * 9 + tc[1] * 3 + tc[2];
    }
    // NeighbourGrid.cpp:113-143 — offsets of the 27 (and 13 "positive") neighbours,
    // measured around a middle cell, sorted and de-duplicated.
    void fill_offsets() {
        offsets.clear();
        positive_offsets.clear();
        std::array<std::size_t, 3> mid{div[0] / 2, div[1] / 2, div[2] / 2};
        std::size_t mid_no = coords_to_cell(mid);
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) {
                    std::array<std::size_t, 3> c{mid[0] + i - 1, mid[1] + j - 1, mid[2] + k - 1};
                    std::size_t no = coords_to_cell(c);
                    offsets.push_back(no - mid_no);
                    if (9 * i + 3 * j + k > 13) positive_offsets.push_back(no - mid_no);
                }
        std::sort(offsets.begin(), offsets.end());
        offsets.erase(std::unique(offsets.begin(), offsets.end()), offsets.end());
        std::sort(positive_offsets.begin(), positive_offsets.end());
        positive_offsets.erase(std::unique(positive_offsets.begin(), positive_offsets.end()),
                               positive_offsets.end());
    }
    void add(std::size_t id, std::size_t cell) {
        succ[id] = heads[cell];
        heads[cell] = id;
    }
    void add_at(std::size_t id, const V3 &p) { add(id, position_to_cell(p)); }
    // NeighbourGrid.cpp:238-258
    void remove(std::size_t id, const V3 &p) {
        std::size_t i = position_to_cell(p);
        std::size_t h = heads[i];
        if (h == id) {
            heads[i] = succ[id];
            succ[id] = END;
        } else {
            while (h != END) {
                if (succ[h] == id) {
                    succ[h] = succ[id];
                    succ[id] = END;
                    break;
                }
                h = succ[h];
            }
        }
    }
    void clear() {
        std::fill(heads.begin(), heads.end(), END);
        std::fill(succ.begin(), succ.end(), END);
    }
    // NeighbourGrid.cpp:312-340
    bool resize(const Box &b, double cell) {
        auto old_div = div;
        std::size_t old_cells = num_cells;
        setup_sizes(b, cell);
        if (div == old_div) {
            clear();
            return false;
        }
        if (old_cells < num_cells) {
            heads.resize(num_cells);
            trans_idx.resize(num_cells);
            reflected.resize(num_cells);
        }
        for (std::size_t i = 0; i < num_cells; i++) reflected_data(i, reflected[i], trans_idx[i]);
        fill_offsets();
        clear();
        return true;
    }
    std::array<std::size_t, 3> real_divisions() const { return {div[0] - 2, div[1] - 2, div[2] - 2}; }

    // Iterates (first id in the neighbour cell, translation) over the cell's neighbourhood,
    // as NeighboursViewIterator::operator* does (NeighbourGrid.h:192-198).
    template <typename F>
    void for_each_neighbour_cell(std::size_t cell_no, bool positive, F &&f) const {
        const auto &offs = positive ? positive_offsets : offsets;
        for (std::size_t off : offs) {
            std::size_t nb = cell_no + off;
            f(heads[reflected[nb]], translations[trans_idx[nb]]);
        }
    }
};

// ---------------------------------------------------------------------------------------
// Packing restated from core/Packing.cpp (hard interactions only: the soft energy terms
// are identically zero for every BASELINE shape).
// ---------------------------------------------------------------------------------------
class Packing {
public:
    static constexpr double INF = std::numeric_limits<double>::infinity();

    std::vector<Shape> shapes;           // size() real shapes + move_threads temp slots
    std::vector<V3> centres;             // body-frame-rotated centres (polysphere)
    std::vector<V3> abs_centres;         // absolute, PBC-corrected centres
    Box box;
    std::optional<NeighbourGrid> ng, temp_ng;
    double range = 0;
    std::size_t num_centres = 0;
    std::size_t move_threads = 1, scaling_threads = 1;
    bool counting = false;
    std::array<bool, 3> has_wall{};      // Packing::toggleWalls (core/Packing.cpp:1075-1084)
    bool has_any_walls = false;
    std::size_t num_overlaps = 0;
    std::vector<std::size_t> last_altered;
    std::vector<int> last_delta;
    std::size_t last_scaling_overlaps = 0;
    Box last_box;
    std::vector<Shape> last_shapes;
    std::size_t ng_rebuilds = 0, ng_resizes = 0;

    Packing(const Box &b, std::vector<Shape> s, const Interaction &inter, std::size_t mthreads, std::size_t sthreads)
        : move_threads{mthreads == 0 ? RPO_MAXTHREADS : mthreads},
          scaling_threads{sthreads == 0 ? RPO_MAXTHREADS : sthreads} {
        reset(std::move(s), b, inter);
    }

    std::size_t size() const { return shapes.size() - move_threads; }

    // Packing.cpp:67-82
    void reset(std::vector<Shape> s, const Box &b, const Interaction &inter) {
        if (s.empty()) throw std::invalid_argument("empty packing");
        if (b.volume() == 0) throw std::invalid_argument("zero box volume");
        for (auto &sh : s)
            for (double x : b.abs_to_rel(sh.pos))
                if (x < 0 || x >= 1) throw std::invalid_argument("shape outside the box");
        shapes = std::move(s);
        box = b;
        range = inter.range();
        shapes.resize(shapes.size() + move_threads);
        last_altered.assign(move_threads, 0);
        last_delta.assign(move_threads, 0);
        setup_for_interaction(inter);
    }

    // Packing.cpp:931-950
    void setup_for_interaction(const Interaction &inter) {
        range = inter.range();
        num_centres = inter.num_centres();
        centres.clear();
        abs_centres.clear();
        if (num_centres > 0) {
            centres.reserve(shapes.size() * num_centres);
            abs_centres.resize(shapes.size() * num_centres);
            for (auto &sh : shapes)
                for (auto &c : inter.centres) centres.push_back(mv(sh.rot, c));
            recalc_abs_centres();
        }
        rebuild_ng();
        if (counting) num_overlaps = count_total_overlaps(inter, false);
    }

    void recalc_abs_centres() {
        std::size_t n = size();
        #pragma omp parallel for num_threads(scaling_threads)
        for (std::size_t i = 0; i < n; i++) recalc_abs_centres(i);
    }
    // Packing.cpp:1041-1047
    void recalc_abs_centres(std::size_t i) {
        for (std::size_t c = 0; c < num_centres; c++) {
            std::size_t ci = i * num_centres + c;
            V3 p = add(shapes[i].pos, centres[ci]);
            abs_centres[ci] = add(p, pbc_correction(box, p));
        }
    }

    // Packing.cpp:858-899
    void rebuild_ng() {
        double cell = range;
        double min_cell = std::cbrt(std::abs(box.volume()) / size()) / 5;
        if (range < min_cell) cell = min_cell;
        V3 h = box.heights();
        if (cell * 4 > *std::max_element(h.begin(), h.end())) { ng.reset(); return; }
        const double CELL_EPS = 1 + 1e-12;
        if (cell * CELL_EPS > *std::min_element(h.begin(), h.end())) { ng.reset(); return; }
        std::size_t ids = num_centres == 0 ? size() : num_centres * size();
        if (!ng.has_value()) ng.emplace(box, cell, ids);
        else ng_resizes += ng->resize(box, cell);
        add_all_to_ng();
        ng_rebuilds++;
    }
    // Packing.cpp:901-929 — parallel cell numbers, serial head insertion.
    void add_all_to_ng() {
        std::size_t n = size();
        if (num_centres == 0) {
            std::vector<std::size_t> cells(n);
            #pragma omp parallel for num_threads(scaling_threads)
            for (std::size_t i = 0; i < n; i++) cells[i] = ng->position_to_cell(shapes[i].pos);
            for (std::size_t i = 0; i < n; i++) ng->add(i, cells[i]);
        } else {
            std::vector<std::size_t> cells(n * num_centres);
            #pragma omp parallel for num_threads(scaling_threads)
            for (std::size_t i = 0; i < n; i++)
                for (std::size_t c = 0; c < num_centres; c++)
                    cells[i * num_centres + c] = ng->position_to_cell(abs_centres[i * num_centres + c]);
            for (std::size_t i = 0; i < n * num_centres; i++) ng->add(i, cells[i]);
        }
    }

    // ----- single-particle overlap counting: Packing.cpp:373-429, :619-647, :587-616 -----
    std::size_t count_particle_overlaps(std::size_t orig, std::size_t temp, const Interaction &inter,
                                        bool early) const {
        std::size_t cnt = 0;
        if (ng.has_value()) {
            if (num_centres == 0) {
                const V3 &pos = shapes[temp].pos;
                std::size_t cell_no = ng->position_to_cell(pos);
                const auto &offs = ng->offsets;
                for (std::size_t off : offs) {
                    std::size_t nb = cell_no + off;
                    BC bc = BC::fixed(ng->translations[ng->trans_idx[nb]]);
                    for (std::size_t j = ng->heads[ng->reflected[nb]]; j != NeighbourGrid::END; j = ng->succ[j]) {
                        if (orig == j) continue;
                        if (inter.overlap(shapes[temp].pos, shapes[temp].rot, 0, shapes[j].pos, shapes[j].rot, 0,
                                          bc)) {
                            if (early) return 1;
                            cnt++;
                        }
                    }
                }
            } else {
                for (std::size_t c1 = 0; c1 < num_centres; c1++) {
                    std::size_t co = centre_overlaps_ng(orig, temp, c1, inter, early);
                    if (early && co > 0) return co;
                    cnt += co;
                }
            }
        } else {
            for (std::size_t j = 0; j < size(); j++) {
                if (orig == j) continue;
                std::size_t po = pair_overlaps_no_ng(temp, j, inter, early);
                if (early && po) return po;
                cnt += po;
            }
        }
        std::size_t wall = 0;
        if (has_any_walls) wall = count_particle_wall_overlaps(temp, inter, early);
        return cnt + wall;
    }

    // Packing::countParticleWallOverlaps (core/Packing.cpp:1086-1139): the wall pair of each
    // walled axis spans the other two box sides; a particle meets the nearer one (through the
    // origin, or through the far corner) when its position lies within half the total
    // interaction range of it
    std::size_t count_particle_wall_overlaps(std::size_t idx, const Interaction &inter, bool early) const {
        std::size_t cnt = 0;
        const auto s = box.sides();
        const V3 origin{0, 0, 0};
        const V3 further = add(add(add(origin, s[0]), s[1]), s[2]);
        const double half = inter.total_range() / 2;
        for (std::size_t i = 0; i < 3; i++) {
            if (!has_wall[i]) continue;
            const V3 c = cross(s[(i + 1) % 3], s[(i + 2) % 3]);
            const V3 wall = vdiv(c, std::sqrt(norm2(c)));
            const V3 &pos = shapes[idx].pos;
            const M3 &rot = shapes[idx].rot;
            V3 o, w;
            if (dot(pos, wall) < half) {
                o = origin;
                w = wall;
            } else if (dot(sub(further, pos), wall) < half) {
                o = further;
                w = {-wall[0], -wall[1], -wall[2]};
            } else {
                continue;
            }
            if (num_centres == 0) {
                if (inter.overlap_with_wall(pos, rot, 0, o, w)) {
                    if (early) return 1;
                    cnt++;
                }
            } else {
                for (std::size_t k = 0; k < num_centres; k++) {
                    const V3 cp = add(pos, centres[idx * num_centres + k]);
                    if (inter.overlap_with_wall(cp, rot, k, o, w)) {
                        if (early) return 1;
                        cnt++;
                    }
                }
            }
        }
        return cnt;
    }

    // ----- soft energies: Packing.cpp:649-687 (calculateParticleEnergy), :711-764 -----
    double particle_energy(std::size_t orig, std::size_t temp, const Interaction &inter) const {
        if (!inter.soft) return 0;
        double energy = 0;
        if (ng.has_value()) {
            if (num_centres == 0) {
                const V3 &pos = shapes[temp].pos;
                std::size_t cell_no = ng->position_to_cell(pos);
                for (std::size_t off : ng->offsets) {
                    std::size_t nb = cell_no + off;
                    BC bc = BC::fixed(ng->translations[ng->trans_idx[nb]]);
                    for (std::size_t j = ng->heads[ng->reflected[nb]]; j != NeighbourGrid::END; j = ng->succ[j]) {
                        if (orig == j) continue;
                        energy += inter.energy(pos, shapes[j].pos, bc);
                    }
                }
            } else {
                for (std::size_t c1 = 0; c1 < num_centres; c1++) energy += centre_energy_ng(orig, temp, c1, inter);
            }
        } else {
            for (std::size_t j = 0; j < size(); j++) {
                if (orig == j) continue;
                energy += pair_energy_no_ng(temp, j, inter);
            }
        }
        return energy;
    }

    // Packing::calculateInteractionCentreEnergyWithNG (core/Packing.cpp:740-764)
    double centre_energy_ng(std::size_t orig, std::size_t temp, std::size_t c1, const Interaction &inter) const {
        double energy = 0;
        V3 p1 = abs_centres[temp * num_centres + c1];
        std::size_t cell_no = ng->position_to_cell(p1);
        for (std::size_t off : ng->offsets) {
            std::size_t nb = cell_no + off;
            BC bc = BC::fixed(ng->translations[ng->trans_idx[nb]]);
            for (std::size_t ci2 = ng->heads[ng->reflected[nb]]; ci2 != NeighbourGrid::END; ci2 = ng->succ[ci2]) {
                std::size_t j = ci2 / num_centres;
                if (j == orig) continue;
                energy += inter.energy(p1, abs_centres[ci2], bc);
            }
        }
        return energy;
    }

    // Packing::calculateEnergyBetweenParticlesWithoutNG (core/Packing.cpp:711-738)
    double pair_energy_no_ng(std::size_t temp, std::size_t other, const Interaction &inter) const {
        BC bc = BC::periodic(box);
        if (num_centres == 0) return 0.0 + inter.energy(shapes[temp].pos, shapes[other].pos, bc);
        double energy = 0;
        for (std::size_t c1 = 0; c1 < num_centres; c1++)
            for (std::size_t c2 = 0; c2 < num_centres; c2++)
                energy += inter.energy(abs_centres[temp * num_centres + c1], abs_centres[other * num_centres + c2], bc);
        return energy;
    }

    // Packing::getTotalEnergyNGCellHelper (core/Packing.cpp:766-836)
    double total_energy_cell_helper(const std::array<std::size_t, 3> &coord, const Interaction &inter) const {
        double energy = 0;
        std::size_t cell_no = ng->real_coords_to_cell(coord);
        BC zero = BC::fixed({});
        for (std::size_t a = ng->heads[cell_no]; a != NeighbourGrid::END; a = ng->succ[a]) {
            std::size_t pa = num_centres == 0 ? a : a / num_centres;
            const V3 &p1 = num_centres == 0 ? shapes[pa].pos : abs_centres[a];
            for (std::size_t b = ng->succ[a]; b != NeighbourGrid::END; b = ng->succ[b]) {
                std::size_t pb = num_centres == 0 ? b : b / num_centres;
                if (num_centres != 0 && pa == pb) continue;
                energy += inter.energy(p1, num_centres == 0 ? shapes[pb].pos : abs_centres[b], zero);
            }
            for (std::size_t off : ng->positive_offsets) {
                std::size_t nb = cell_no + off;
                BC bc = BC::fixed(ng->translations[ng->trans_idx[nb]]);
                for (std::size_t b = ng->heads[ng->reflected[nb]]; b != NeighbourGrid::END; b = ng->succ[b]) {
                    std::size_t pb = num_centres == 0 ? b : b / num_centres;
                    if (num_centres != 0 && pa == pb) continue;
                    energy += inter.energy(p1, num_centres == 0 ? shapes[pb].pos : abs_centres[b], bc);
                }
            }
        }
        return energy;
    }

    // Packing::getTotalEnergy (core/Packing.cpp:689-709): cells in parallel with an OpenMP sum
    // (one thread reproduces the reference's serial order)
    double total_energy(const Interaction &inter) const {
        if (!inter.soft) return 0;
        double energy = 0;
        if (ng.has_value()) {
            auto d = ng->real_divisions();
            #pragma omp parallel for collapse(3) reduction(+ : energy) num_threads(scaling_threads)
            for (std::size_t i = 0; i < d[0]; i++)
                for (std::size_t j = 0; j < d[1]; j++)
                    for (std::size_t k = 0; k < d[2]; k++) energy += total_energy_cell_helper({i, j, k}, inter);
        } else {
            for (std::size_t i = 0; i < size(); i++)
                for (std::size_t j = i + 1; j < size(); j++) energy += pair_energy_no_ng(i, j, inter);
        }
        return energy;
    }

    // Packing::countWallOverlaps (core/Packing.cpp:561-580)
    std::size_t count_wall_overlaps(const Interaction &inter, bool early) const {
        if (!has_any_walls) return 0;
        std::size_t cnt = 0;
        for (std::size_t i = 0; i < size(); i++) {
            std::size_t c = count_particle_wall_overlaps(i, inter, early);
            if (early && c > 0) return c;
            cnt += c;
        }
        return cnt;
    }

    std::size_t centre_overlaps_ng(std::size_t orig, std::size_t temp, std::size_t c1, const Interaction &inter,
                                   bool early) const {
        std::size_t cnt = 0;
        std::size_t ci1 = temp * num_centres + c1;
        V3 p1 = abs_centres[ci1];
        const M3 &o1 = shapes[temp].rot;
        std::size_t cell_no = ng->position_to_cell(p1);
        for (std::size_t off : ng->offsets) {
            std::size_t nb = cell_no + off;
            BC bc = BC::fixed(ng->translations[ng->trans_idx[nb]]);
            for (std::size_t ci2 = ng->heads[ng->reflected[nb]]; ci2 != NeighbourGrid::END; ci2 = ng->succ[ci2]) {
                std::size_t j = ci2 / num_centres;
                if (j == orig) continue;
                std::size_t c2 = ci2 % num_centres;
                if (inter.overlap(p1, o1, c1, abs_centres[ci2], shapes[j].rot, c2, bc)) {
                    if (early) return 1;
                    cnt++;
                }
            }
        }
        return cnt;
    }

    std::size_t pair_overlaps_no_ng(std::size_t temp, std::size_t other, const Interaction &inter,
                                    bool early) const {
        std::size_t cnt = 0;
        BC bc = BC::periodic(box);
        if (num_centres == 0) {
            if (inter.overlap(shapes[temp].pos, shapes[temp].rot, 0, shapes[other].pos, shapes[other].rot, 0, bc)) {
                if (early) return 1;
                cnt++;
            }
        } else {
            for (std::size_t c1 = 0; c1 < num_centres; c1++) {
                const V3 &p1 = abs_centres[temp * num_centres + c1];
                for (std::size_t c2 = 0; c2 < num_centres; c2++) {
                    const V3 &p2 = abs_centres[other * num_centres + c2];
                    if (inter.overlap(p1, shapes[temp].rot, c1, p2, shapes[other].rot, c2, bc)) {
                        if (early) return 1;
                        cnt++;
                    }
                }
            }
        }
        return cnt;
    }

    // ----- all-pairs counting: Packing.cpp:431-559 -----
    std::size_t count_cell_helper(const std::array<std::size_t, 3> &coord, const Interaction &inter,
                                  bool early) const {
        std::size_t cnt = 0;
        std::size_t cell_no = ng->real_coords_to_cell(coord);
        BC zero = BC::fixed({});
        for (std::size_t a = ng->heads[cell_no]; a != NeighbourGrid::END; a = ng->succ[a]) {
            std::size_t pa = num_centres == 0 ? a : a / num_centres;
            std::size_t ca = num_centres == 0 ? 0 : a % num_centres;
            const V3 &p1 = num_centres == 0 ? shapes[pa].pos : abs_centres[a];
            const M3 &o1 = shapes[pa].rot;
            for (std::size_t b = ng->succ[a]; b != NeighbourGrid::END; b = ng->succ[b]) {
                std::size_t pb = num_centres == 0 ? b : b / num_centres;
                if (num_centres != 0 && pa == pb) continue;
                std::size_t cb = num_centres == 0 ? 0 : b % num_centres;
                const V3 &p2 = num_centres == 0 ? shapes[pb].pos : abs_centres[b];
                if (inter.overlap(p1, o1, ca, p2, shapes[pb].rot, cb, zero)) {
                    if (early) return 1;
                    cnt++;
                }
            }
            for (std::size_t off : ng->positive_offsets) {
                std::size_t nb = cell_no + off;
                BC bc = BC::fixed(ng->translations[ng->trans_idx[nb]]);
                for (std::size_t b = ng->heads[ng->reflected[nb]]; b != NeighbourGrid::END; b = ng->succ[b]) {
                    std::size_t pb = num_centres == 0 ? b : b / num_centres;
                    if (num_centres != 0 && pa == pb) continue;
                    std::size_t cb = num_centres == 0 ? 0 : b % num_centres;
                    const V3 &p2 = num_centres == 0 ? shapes[pb].pos : abs_centres[b];
                    if (inter.overlap(p1, o1, ca, p2, shapes[pb].rot, cb, bc)) {
                        if (early) return 1;
                        cnt++;
                    }
                }
            }
        }
        return cnt;
    }

    std::size_t count_total_overlaps(const Interaction &inter, bool early) const {
        std::size_t cnt = 0;
        if (ng.has_value()) {
            std::atomic<bool> found = false;
            auto d = ng->real_divisions();
            #pragma omp parallel for collapse(3) reduction(+ : cnt) num_threads(scaling_threads)
            for (std::size_t i = 0; i < d[0]; i++)
                for (std::size_t j = 0; j < d[1]; j++)
                    for (std::size_t k = 0; k < d[2]; k++) {
                        if (early && found.load(std::memory_order_relaxed)) continue;
                        std::size_t c = count_cell_helper({i, j, k}, inter, early);
                        if (early && c > 0) found.store(true, std::memory_order_relaxed);
                        cnt += c;
                    }
            if (early && cnt) return 1;
        } else {
            for (std::size_t i = 0; i < size(); i++)
                for (std::size_t j = i + 1; j < size(); j++) {
                    std::size_t po = pair_overlaps_no_ng(i, j, inter, early);
                    if (early && po > 0) return po;
                    cnt += po;
                }
        }
        return cnt + count_wall_overlaps(inter, early);
    }

    // ----- moves: Packing.cpp:84-164, :304-323 -----
    double move_overlap_energy(std::size_t idx, std::size_t temp, const Interaction &inter) {
        if (!inter.hard) return 0;   // no hard part (core/Packing.cpp:307)
        if (counting) {
            std::size_t before = count_particle_overlaps(idx, idx, inter, false);
            std::size_t after = count_particle_overlaps(idx, temp, inter, false);
            int &delta = last_delta[RPO_TID];
            delta = static_cast<int>(after) - static_cast<int>(before);
            if (delta < 0) return -INF;
            if (delta > 0) return INF;
        } else if (count_particle_overlaps(idx, temp, inter, true) > 0) {
            return INF;
        }
        return 0;
    }

    void prepare_temp_centres(std::size_t idx) {
        std::size_t from = idx * num_centres, to = (size() + RPO_TID) * num_centres;
        for (std::size_t c = 0; c < num_centres; c++) centres[to + c] = centres[from + c];
    }
    void rotate_temp_centres(const M3 &r) {
        std::size_t o = (size() + RPO_TID) * num_centres;
        for (std::size_t c = 0; c < num_centres; c++) centres[o + c] = mv(r, centres[o + c]);
    }

    // ActiveDomain::isInside (core/ActiveDomain.cpp:8-21): strict bounds in relative
    // coordinates; end <= beg denotes an interval wrapping through 0.
    static bool inside(const Box &box, const double *lo, const double *hi, const V3 &pos) {
        V3 rel = box.abs_to_rel(pos);
        for (int i = 0; i < 3; i++) {
            if (hi[i] > lo[i]) {
                if (rel[i] <= lo[i] || rel[i] >= hi[i]) return false;
            } else {
                if (rel[i] <= lo[i] && rel[i] >= hi[i]) return false;
            }
        }
        return true;
    }

    // type 0 translation, 1 rotation, 2 translation + rotation (tryTranslation,
    // tryRotation, tryMove).  bounds == nullptr means no ActiveDomain.  Returns the
    // energy; `outside` reports the ActiveDomain rejection.
    double try_move(int type, std::size_t idx, const V3 &t, const M3 &r, const Interaction &inter,
                    const double *lo, const double *hi, bool *outside = nullptr) {
        if (idx >= size()) throw std::out_of_range("particle index");
        std::size_t temp = size() + RPO_TID;
        last_altered[RPO_TID] = idx;
        shapes[temp] = shapes[idx];
        if (outside) *outside = false;
        if (type == 0 || type == 2) {
            shapes[temp].translate(t, box);
            if (lo && !inside(box, lo, hi, shapes[temp].pos)) {
                if (outside) *outside = true;
                return INF;
            }
        }
        if (type == 1 || type == 2) shapes[temp].rotate(r);
        if (num_centres != 0) {
            prepare_temp_centres(idx);
            if (type != 0) rotate_temp_centres(r);
            recalc_abs_centres(temp);
        }
        double overlap_energy = move_overlap_energy(idx, temp, inter);
        if (overlap_energy != 0 || !inter.soft) return overlap_energy;
        // soft part: the particle's energy after the move minus before (core/Packing.cpp:103-108)
        double initial = particle_energy(idx, idx, inter);
        double final_ = particle_energy(idx, temp, inter);
        return final_ - initial;
    }

    // Packing.cpp:234-302 (acceptTranslation / acceptRotation / acceptMove share this
    // effect for hard bodies: the temp slot replaces the particle and the grid follows).
    void accept(int type) {
        std::size_t idx = last_altered[RPO_TID];
        std::size_t temp = size() + RPO_TID;
        bool regrid = ng.has_value() && (num_centres != 0 || type != 1);
        if (regrid) {
            if (num_centres == 0) ng->remove(idx, shapes[idx].pos);
            else
                for (std::size_t c = 0; c < num_centres; c++)
                    ng->remove(idx * num_centres + c, abs_centres[idx * num_centres + c]);
        }
        if (type == 0) shapes[idx].pos = shapes[temp].pos;
        else if (type == 1) shapes[idx].rot = shapes[temp].rot;
        else shapes[idx] = shapes[temp];
        if (num_centres != 0) {
            std::size_t from = temp * num_centres, to = idx * num_centres;
            for (std::size_t c = 0; c < num_centres; c++) {
                centres[to + c] = centres[from + c];
                abs_centres[to + c] = abs_centres[from + c];
            }
        }
        if (regrid) {
            if (num_centres == 0) ng->add_at(idx, shapes[idx].pos);
            else
                for (std::size_t c = 0; c < num_centres; c++)
                    ng->add_at(idx * num_centres + c, abs_centres[idx * num_centres + c]);
        }
        if (counting) {
            #pragma omp critical
            num_overlaps += last_delta[RPO_TID];
        }
    }

    // ----- box moves: Packing.cpp:166-208, :363-371, :1155-1176 -----
    static bool box_upscaled(const Box &ob, const Box &nb) {
        auto os = ob.sides(), ns = nb.sides();
        const double EPS = 100 * std::numeric_limits<double>::epsilon();
        for (int i = 0; i < 3; i++) {
            double d = dot(os[i], ns[i]);
            double n2o = norm2(os[i]), n2n = norm2(ns[i]);
            if (std::abs(d * d / n2o / n2n - 1) > EPS) return false;
            if (d * d / n2o / n2o < 1 + EPS) return false;
        }
        return true;
    }

    double try_scaling(const Box &nb, const Interaction &inter) {
        last_box = box;
        last_shapes = shapes;
        double initial_energy = total_energy(inter);   // core/Packing.cpp:178
        last_scaling_overlaps = num_overlaps;
        box = nb;
        std::size_t n = size();
        for (std::size_t i = 0; i < n; i++)
            shapes[i].pos = box.rel_to_abs(last_box.abs_to_rel(shapes[i].pos));
        std::swap(ng, temp_ng);
        if (num_centres != 0) recalc_abs_centres();
        rebuild_ng();
        if (inter.hard) {   // core/Packing.cpp:191-203
            if (counting) {
                num_overlaps = count_total_overlaps(inter, false);
                int delta = static_cast<int>(num_overlaps) - static_cast<int>(last_scaling_overlaps);
                if (delta < 0) return -INF;
                if (delta > 0) return INF;
            } else {
                bool cannot = inter.convex() && box_upscaled(last_box, box);
                if (!cannot && count_total_overlaps(inter, true) > 0) return INF;
            }
        }
        double final_energy = total_energy(inter);
        return final_energy - initial_energy;
    }

    void revert_scaling() {
        shapes = last_shapes;
        box = last_box;
        std::swap(ng, temp_ng);
        if (num_centres != 0) recalc_abs_centres();
        num_overlaps = last_scaling_overlaps;
    }

    void set_counting(bool on, const Interaction &inter) {
        counting = on;
        if (counting) num_overlaps = count_total_overlaps(inter, false);
    }

    // Packing.cpp:1214-1219 — three Newton–Schulz steps R <- 1.5 R - 0.5 R R^T R.
    static void fix_rotation(M3 &r) {
        for (int i = 0; i < 3; i++) r = msub(mscale(r, 1.5), mm(mm(mscale(r, 0.5), transpose(r)), r));
    }

    // Packing.cpp:1178-1212 (renormalizeOrientations) with tryOrientationFix
    // (:1221-1240).  With allow_overlaps the reference copies the shapes before fixing them
    // and resets the packing with that copy, so orientations stay as they were and only the
    // rotated centres are recomputed from the body frame.  Otherwise every particle, in index
    // order, tries its fixed orientation (centres rotated afresh from the body frame) as a
    // rotation move on thread slot 0 and keeps it when the move energy is not positive.
    std::size_t renormalize_orientations(const Interaction &inter, bool allow_overlaps) {
        if (allow_overlaps) {
            std::vector<Shape> copy(shapes.begin(), shapes.begin() + static_cast<std::ptrdiff_t>(size()));
            reset(std::move(copy), box, inter);
            return 0;
        }
        std::size_t rejected = 0;
        std::size_t temp = size();
        for (std::size_t i = 0; i < size(); i++) {
            last_altered[0] = i;
            shapes[temp].pos = shapes[i].pos;
            M3 r = shapes[i].rot;
            fix_rotation(r);
            shapes[temp].rot = r;
            if (num_centres > 0) {
                for (std::size_t c = 0; c < num_centres; c++) centres[temp * num_centres + c] = mv(r, inter.centres[c]);
                recalc_abs_centres(temp);
            }
            if (move_overlap_energy(i, temp, inter) > 0) rejected++;
            else accept(1);
        }
        return rejected;
    }
};

}  // namespace rpo
