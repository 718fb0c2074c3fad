// GpuPacking: the reference's Packing interface (core/Packing.h:32-466) over the C ABI of
// rampack_gb300 (include/rampack_gb300.h), for a C++ caller such as rampack's Simulation.
//
// Header-only; link against librampack_gb300.so.  Method names, argument meaning, the
// energy encoding (0 or +inf; -inf only in overlap counting) and the error behaviour (a
// failing call throws std::runtime_error, which rampack's callers treat like its own
// PreconditionException) follow Packing.  Differences, stated where they apply:
//  * every single move runs with the particle's current grid cell as its ActiveDomain
//    (the engine has no unrestricted single-move path);
//  * acceptTranslation/acceptRotation/acceptMove re-run the last tried move with a
//    Metropolis uniform of 0 (always accepted), which commits the same temp state the
//    reference's acceptMove commits (core/Packing.cpp:278-302);
//  * performMoves is the batched entry that replaces Simulation::performMovesWithDomainDivision
//    (core/Simulation.cpp:396-445): one device sweep of 2N moves.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/rampack_gb300.h"

namespace rampack_gb300 {

using Vec3 = std::array<double, 3>;
using Mat3 = std::array<double, 9>;  // row-major Matrix<3, 3>

class GpuPacking {
public:
    using Vec3 = rampack_gb300::Vec3;
    using Mat3 = rampack_gb300::Mat3;
    struct Shape {
        Vec3 position{};
        Mat3 orientation{1, 0, 0, 0, 1, 0, 0, 0, 1};
    };

    // Packing(box, shapes, bc, interaction, moveThreads, scalingThreads) for hard spheres
    // (length < 0) or spherocylinders of the given length.
    GpuPacking(const Mat3 &box, const std::vector<Shape> &shapes, double radius, double length = -1, int device = 0) {
        rp_shape_desc d{};
        d.kind = length < 0 ? RP_SHAPE_SPHERE : RP_SHAPE_SPHEROCYLINDER;
        d.radius = radius;
        d.length = length < 0 ? 0 : length;
        check(rp_create(&d, static_cast<int64_t>(shapes.size()), device, &h_), "rp_create");
        n_ = shapes.size();
        reset(shapes, box);
    }
    GpuPacking(const GpuPacking &) = delete;
    GpuPacking &operator=(const GpuPacking &) = delete;
    ~GpuPacking() {
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
        last_ = {};
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

    // Packing::tryTranslation / tryRotation / tryMove (core/Packing.cpp:84-164)
    double tryTranslation(std::size_t idx, const Vec3 &t) { return tryAny(RP_MOVE_TRANSLATION, idx, t, identity()); }
    double tryRotation(std::size_t idx, const Mat3 &r) { return tryAny(RP_MOVE_ROTATION, idx, Vec3{}, r); }
    double tryMove(std::size_t idx, const Vec3 &t, const Mat3 &r) { return tryAny(RP_MOVE_ROTOTRANSLATION, idx, t, r); }

    // Packing::acceptTranslation / acceptRotation / acceptMove (core/Packing.cpp:234-302)
    void acceptTranslation() { commit(); }
    void acceptRotation() { commit(); }
    void acceptMove() { commit(); }

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

    // The batched move entry: one device sweep (2N moves for translation + rotation).
    rp_sweep_stats performMoves(double translationStep, double rotationStep, uint64_t seed, uint64_t cycle) {
        rp_sweep_params p{};
        p.translation_step = translationStep;
        p.rotation_step = rotationStep;
        p.seed = seed;
        p.counter = cycle;
        rp_sweep_stats st{};
        check(rp_sweep(h_, &p, &st), "rp_sweep");
        return st;
    }

private:
    void *h_ = nullptr;
    std::size_t n_ = 0;
    Mat3 box_{}, prev_box_{};
    rp_move last_{};

    static Mat3 identity() { return Mat3{1, 0, 0, 0, 1, 0, 0, 0, 1}; }

    void check(int rc, const char *what) const {
        if (rc != RP_OK) throw std::runtime_error(std::string(what) + ": " + rp_last_error(h_));
    }

    int cellOf(std::size_t idx) const {
        std::vector<int32_t> cells(n_);
        check(rp_get_grid(h_, nullptr, cells.data(), nullptr), "rp_get_grid");
        return cells[idx];
    }

    double tryAny(int type, std::size_t idx, const Vec3 &t, const Mat3 &r) {
        if (idx >= n_) throw std::runtime_error("particle index out of range");
        rp_move m{};
        m.particle = static_cast<int32_t>(idx);
        m.type = type;
        m.domain = cellOf(idx);
        for (int k = 0; k < 3; k++) m.translation[k] = t[k];
        for (int k = 0; k < 9; k++) m.rotation[k] = r[k];
        m.uniform = 2.0;  // > 1: evaluated, never accepted
        uint8_t code = 0;
        check(rp_run_moves(h_, &m, 1, &code), "rp_run_moves");
        last_ = m;
        switch (code & 3) {
            case 0: return 0.0;
            case 3: return -std::numeric_limits<double>::infinity();
            default: return std::numeric_limits<double>::infinity();
        }
    }

    void commit() {
        rp_move m = last_;
        m.uniform = 0.0;  // u <= exp(-dE/T) holds for every dE: the temp state is committed
        uint8_t code = 0;
        check(rp_run_moves(h_, &m, 1, &code), "rp_run_moves");
    }
};

}  // namespace rampack_gb300
