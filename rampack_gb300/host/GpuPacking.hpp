// GpuPacking: the reference's Packing interface (core/Packing.h:32-466) over the C ABI of
// rampack_gb300 (include/rampack_gb300.h), for a C++ caller such as rampack's Simulation.
//
// Header-only; link against librampack_gb300.so.  Method names, argument meaning, the
// energy encoding (0 or +inf; -inf only in overlap counting) and the error behaviour follow
// Packing.  BasicGpuPacking is a template over the caller's types, so that the reference can
// pass its own objects unchanged:
//  * Vector: a position or translation with operator[] (Vector<3>, or std::array<double, 3>);
//  * Matrix: an orientation, rotation or box with operator()(i, j) (Matrix<3, 3>) or a
//    row-major std::array<double, 9>;
//  * Domain: an ActiveDomain with getBoundsForCoordinate(i).beg / .end
//    (core/ActiveDomain.h:19-53), passed as std::optional like Packing::tryTranslation's;
//  * Raise: how a failing call reports, Raise::raise(message, function, line) (the reference
//    side throws its PreconditionException; the default throws std::runtime_error).
// GpuPacking is the instantiation over std::array types.
//  * tryTranslation / tryRotation / tryMove evaluate one move on the device and keep the
//    tried state there; acceptTranslation / acceptRotation / acceptMove commit it
//    (rp_try_move / rp_accept_move, no grid rebuild per move);
//  * performMoves is the batched entry that replaces Simulation::performMovesWithDomainDivision
//    (core/Simulation.cpp:396-445): one device sweep of 2N moves.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <map>
#include <optional>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/rampack_gb300.h"

namespace rampack_gb300 {

using Vec3 = std::array<double, 3>;
using Mat3 = std::array<double, 9>;  // row-major Matrix<3, 3>

namespace detail {
// element (i, j) of a Matrix<3, 3>-like object or of a row-major array of 9
template <class M>
double mat_at(const M &m, int i, int j) {
    if constexpr (std::is_invocable_v<const M &, std::size_t, std::size_t>)
        return static_cast<double>(m(static_cast<std::size_t>(i), static_cast<std::size_t>(j)));
    else
        return static_cast<double>(m[static_cast<std::size_t>(3 * i + j)]);
}
template <class V>
double vec_at(const V &v, int i) {
    return static_cast<double>(v[static_cast<std::size_t>(i)]);
}
}  // namespace detail

// ActiveDomain stand-in with the reference's accessor (relative bounds per coordinate).
struct DomainBounds {
    struct RegionBounds {
        double beg{}, end{};
    };
    std::array<RegionBounds, 3> bounds{};
    const RegionBounds &getBoundsForCoordinate(std::size_t i) const { return bounds[i]; }
};

// The default error report: std::runtime_error with the library's message.
struct ThrowRuntimeError {
    [[noreturn]] static void raise(const std::string &what, const char *, int) { throw std::runtime_error(what); }
};

// A particle's state as the engine stores it: position and row-major orientation.
struct Shape {
    Vec3 position{};
    Mat3 orientation{1, 0, 0, 0, 1, 0, 0, 0, 1};
};

// One sphere or spherocylinder of a multi-centre body: PolysphereTraits::SphereData
// (position, radius) or PolyspherocylinderTraits::SpherocylinderData (position, half axis,
// radius), in the body frame.
struct Centre {
    Vec3 position{};
    double radius = 0;
    Vec3 half_axis{};
};

template <class Vector = Vec3, class Matrix = Mat3, class Domain = DomainBounds, class Raise = ThrowRuntimeError>
class BasicGpuPacking {
public:
    using Vec3 = rampack_gb300::Vec3;
    using Mat3 = rampack_gb300::Mat3;
    using Shape = rampack_gb300::Shape;
    using Centre = rampack_gb300::Centre;
    static constexpr double INF = std::numeric_limits<double>::infinity();

    // Packing(box, shapes, bc, interaction, moveThreads, scalingThreads) for hard spheres
    // (length < 0) or spherocylinders of the given length.
    BasicGpuPacking(const Mat3 &box, const std::vector<Shape> &shapes, double radius, double length = -1,
                    int device = 0) {
        rp_shape_desc d{};
        d.kind = length < 0 ? RP_SHAPE_SPHERE : RP_SHAPE_SPHEROCYLINDER;
        d.radius = radius;
        d.length = length < 0 ? 0 : length;
        check(rp_create(&d, static_cast<int64_t>(shapes.size()), device, &h_), "rp_create");
        n_ = shapes.size();
        reset(shapes, box);
    }
    // Packing(box, shapes, bc, interaction, ...) for polyspheres (PolysphereTraits) or, with
    // `spherocylinders`, polyspherocylinders (PolyspherocylinderTraits).
    BasicGpuPacking(const Mat3 &box, const std::vector<Shape> &shapes, const std::vector<Centre> &centres,
                    bool spherocylinders, int device = 0) {
        std::vector<double> pos, half, radii;
        for (const auto &c : centres) {
            pos.insert(pos.end(), c.position.begin(), c.position.end());
            half.insert(half.end(), c.half_axis.begin(), c.half_axis.end());
            radii.push_back(c.radius);
        }
        const auto k = static_cast<int32_t>(centres.size());
        const auto n = static_cast<int64_t>(shapes.size());
        if (spherocylinders)
            check(rp_create_polyspherocylinder(k, pos.data(), half.data(), radii.data(), n, device, &h_),
                  "rp_create_polyspherocylinder");
        else
            check(rp_create_polysphere(k, pos.data(), radii.data(), n, device, &h_), "rp_create_polysphere");
        n_ = shapes.size();
        reset(shapes, box);
    }
    BasicGpuPacking(const BasicGpuPacking &) = delete;
    BasicGpuPacking &operator=(const BasicGpuPacking &) = delete;
    ~BasicGpuPacking() {
        if (h_) rp_destroy(h_);
    }

    // Packing::reset (core/Packing.cpp:67-82)
    void reset(const std::vector<Shape> &shapes, const Mat3 &box) {
        std::vector<double> pos(3 * shapes.size()), rot(9 * shapes.size());
        for (std::size_t i = 0; i < shapes.size(); i++) {
            for (int k = 0; k < 3; k++) pos[3 * i + k] = shapes[i].position[k];
            for (int k = 0; k < 9; k++) rot[9 * i + k] = shapes[i].orientation[k];
        }
        check(rp_upload_state(h_, pos.data(), rot.data(), box.data()), "rp_upload_state");
        box_ = box;
    }

    std::size_t size() const { return n_; }
    const Mat3 &getBox() const { return box_; }

    std::vector<Shape> getShapes() const {
        std::vector<double> pos(3 * n_), rot(9 * n_);
        Mat3 box{};
        check(rp_download_state(h_, pos.data(), rot.data(), box.data()), "rp_download_state");
        std::vector<Shape> out(n_);
        for (std::size_t i = 0; i < n_; i++) {
            for (int k = 0; k < 3; k++) out[i].position[k] = pos[3 * i + k];
            for (int k = 0; k < 9; k++) out[i].orientation[k] = rot[9 * i + k];
        }
        return out;
    }

    // Packing::tryTranslation / tryRotation / tryMove (core/Packing.cpp:84-164); with no
    // domain (std::nullopt) the reference's serial path, with one the move must keep the
    // particle inside it
    double tryTranslation(std::size_t idx, const Vector &t, const std::optional<Domain> &domain = std::nullopt) {
        return tryAny(RP_MOVE_TRANSLATION, idx, &t, nullptr, domain);
    }
    double tryRotation(std::size_t idx, const Matrix &r) {
        return tryAny(RP_MOVE_ROTATION, idx, nullptr, &r, std::nullopt);
    }
    double tryMove(std::size_t idx, const Vector &t, const Matrix &r, const std::optional<Domain> &domain = std::nullopt) {
        return tryAny(RP_MOVE_ROTOTRANSLATION, idx, &t, &r, domain);
    }

    // Packing::acceptTranslation / acceptRotation / acceptMove (core/Packing.cpp:234-302)
    void acceptTranslation() { check(rp_accept_move(h_), "rp_accept_move", __LINE__); }
    void acceptRotation() { check(rp_accept_move(h_), "rp_accept_move", __LINE__); }
    void acceptMove() { check(rp_accept_move(h_), "rp_accept_move", __LINE__); }

    // Packing::countTotalOverlaps (core/Packing.cpp:519-559)
    std::size_t countTotalOverlaps(bool earlyExit = false) const {
        int64_t c = 0;
        check(rp_count_overlaps(h_, earlyExit ? 1 : 0, &c), "rp_count_overlaps");
        return static_cast<std::size_t>(c);
    }

    // Packing::tryScaling / revertScaling (core/Packing.cpp:172-208, :363-371)
    double tryScaling(const Mat3 &newBox) {
        double dE = 0;
        check(rp_try_scaling(h_, newBox.data(), &dE), "rp_try_scaling");
        prev_box_ = box_;
        box_ = newBox;
        return dE;
    }
    void revertScaling() {
        check(rp_revert_scaling(h_), "rp_revert_scaling");
        box_ = prev_box_;
    }

    // Packing::renormalizeOrientations (core/Packing.cpp:1178-1212): the number of
    // particles whose Newton-Schulz-fixed orientation was rejected.
    std::size_t renormalizeOrientations(bool allowOverlaps) {
        int64_t rejected = 0;
        check(rp_renormalize_orientations(h_, allowOverlaps ? 1 : 0, &rejected), "rp_renormalize_orientations");
        return static_cast<std::size_t>(rejected);
    }

    // Packing::store / Packing::restore (core/Packing.cpp:956-964) with a file path: the
    // RAMSNAP file of the device state, byte for byte the reference's RamsnapWriter output;
    // restore loads a file of this packing's size and returns its aux entries.
    void store(const std::string &path, const std::map<std::string, std::string> &auxInfo = {}) const {
        std::vector<const char *> keys, values;
        for (auto &kv : auxInfo) {
            keys.push_back(kv.first.c_str());
            values.push_back(kv.second.c_str());
        }
        checkIo(rp_ramsnap_write(h_, path.c_str(), static_cast<int32_t>(keys.size()), keys.data(), values.data()),
                "rp_ramsnap_write");
    }
    std::map<std::string, std::string> restore(const std::string &path) {
        void *snap = nullptr;
        checkIo(rp_ramsnap_load(path.c_str(), &snap), "rp_ramsnap_load");
        int64_t n = 0;
        int32_t naux = 0;
        rp_ramsnap_info(snap, &n, &naux);
        if (static_cast<std::size_t>(n) != n_) {
            rp_ramsnap_free(snap);
            Raise::raise("restore: the file holds " + std::to_string(n) + " shapes, the packing " + std::to_string(n_),
                         "restore", __LINE__);
        }
        std::vector<double> pos(3 * n_), rot(9 * n_);
        Mat3 box{};
        rp_ramsnap_get(snap, pos.data(), rot.data(), box.data());
        std::map<std::string, std::string> aux;
        for (int32_t i = 0; i < naux; i++) {
            const char *k = nullptr, *v = nullptr;
            rp_ramsnap_aux(snap, i, &k, &v);
            aux[k] = v;
        }
        rp_ramsnap_free(snap);
        check(rp_upload_state(h_, pos.data(), rot.data(), box.data()), "rp_upload_state");
        box_ = box;
        return aux;
    }

    // Packing::toggleOverlapCounting / getCachedNumberOfOverlaps (core/Packing.cpp:1049-1060)
    void toggleOverlapCounting(bool countOverlaps) {
        check(rp_set_counting(h_, countOverlaps ? 1 : 0), "rp_set_counting");
    }
    std::size_t getCachedNumberOfOverlaps() const {
        int64_t c = 0;
        check(rp_cached_overlaps(h_, &c), "rp_cached_overlaps");
        return static_cast<std::size_t>(c);
    }

    // Packing::toggleWalls (core/Packing.cpp:1075-1084)
    void toggleWalls(const std::array<bool, 3> &axisWalls) {
        const int32_t mask = (axisWalls[0] ? 1 : 0) | (axisWalls[1] ? 2 : 0) | (axisWalls[2] ? 4 : 0);
        check(rp_set_walls(h_, mask), "rp_set_walls");
    }

    // The handle, for rp_* calls this class does not wrap (e.g. rp_ramtrj_record).
    void *handle() const { return h_; }

    // The batched move entry: one device sweep (2N moves for translation + rotation, N for one
    // of them or, with `rototranslation`, N moves of both at once).
    rp_sweep_stats performMoves(double translationStep, double rotationStep, uint64_t seed, uint64_t cycle,
                                bool rototranslation = false) {
        rp_sweep_params p{};
        p.translation_step = translationStep;
        p.rotation_step = rotationStep;
        p.seed = seed;
        p.counter = cycle;
        p.flags = rototranslation ? RP_SWEEP_ROTOTRANSLATION : 0;
        rp_sweep_stats st{};
        check(rp_sweep(h_, &p, &st), "rp_sweep");
        return st;
    }

private:
    void *h_ = nullptr;
    std::size_t n_ = 0;
    Mat3 box_{}, prev_box_{};

    void check(int rc, const char *what, int line = 0) const {
        if (rc != RP_OK) Raise::raise(std::string(what) + ": " + rp_last_error(h_), what, line);
    }
    static void checkIo(int rc, const char *what) {
        if (rc != RP_OK) Raise::raise(std::string(what) + ": " + rp_io_last_error(), what, 0);
    }

    double tryAny(int type, std::size_t idx, const Vector *t, const Matrix *r, const std::optional<Domain> &domain) {
        if (idx >= n_) Raise::raise("particle index out of range", "tryMove", __LINE__);
        rp_move m{};
        m.particle = static_cast<int32_t>(idx);
        m.type = type;
        m.domain = -1;
        for (int k = 0; k < 3; k++) m.translation[k] = t ? detail::vec_at(*t, k) : 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) m.rotation[3 * i + j] = r ? detail::mat_at(*r, i, j) : (i == j ? 1.0 : 0.0);
        double bounds[6];
        if (domain)
            for (int k = 0; k < 3; k++) {
                bounds[k] = domain->getBoundsForCoordinate(static_cast<std::size_t>(k)).beg;
                bounds[3 + k] = domain->getBoundsForCoordinate(static_cast<std::size_t>(k)).end;
            }
        double dE = 0;
        check(rp_try_move(h_, &m, domain ? bounds : nullptr, &dE), "rp_try_move", __LINE__);
        return dE;
    }
};

using GpuPacking = BasicGpuPacking<>;

// RamtrjRecorder (core/io/RamtrjRecorder.cpp): a RAMTRJ trajectory; recordSnapshot takes a
// GpuPacking's state in order with its moves and returns while the file is written.
class RamtrjRecorder {
public:
    RamtrjRecorder(const std::string &path, std::size_t numParticles, std::size_t cycleStep, bool append = false) {
        if (rp_ramtrj_open(path.c_str(), static_cast<int64_t>(numParticles), static_cast<int64_t>(cycleStep),
                           append ? 1 : 0, &r_) != RP_OK)
            throw std::runtime_error(std::string("rp_ramtrj_open: ") + rp_io_last_error());
    }
    RamtrjRecorder(const RamtrjRecorder &) = delete;
    RamtrjRecorder &operator=(const RamtrjRecorder &) = delete;
    ~RamtrjRecorder() {
        if (r_) rp_ramtrj_close(r_);
    }
    template <class Packing>
    void recordSnapshot(const Packing &packing, std::size_t cycle) {
        if (rp_ramtrj_record(r_, packing.handle(), static_cast<int64_t>(cycle)) != RP_OK)
            throw std::runtime_error(std::string("rp_ramtrj_record: ") + rp_io_last_error());
    }
    void close() {
        void *r = r_;
        r_ = nullptr;
        if (r && rp_ramtrj_close(r) != RP_OK) throw std::runtime_error(std::string("rp_ramtrj_close: ") + rp_io_last_error());
    }

private:
    void *r_ = nullptr;
};

}  // namespace rampack_gb300
