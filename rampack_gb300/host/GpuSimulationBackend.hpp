// GpuSimulationBackend: the device backend that `rampack casino` selects with `gpu = True` in the
// PYON `rampack(...)` dataclass (casino_gpu.patch: src/frontend/matchers/RampackMatcher.cpp:367-396,
// src/frontend/modes/CasinoMode.cpp:171).
//
// It implements the SimulationBackend interface that the patch adds to the reference
// (src/core/SimulationBackend.h) and is compiled inside the reference's own build: it includes the
// reference's headers and talks to the device through BasicGpuPacking over the C ABI.  The
// reference's Simulation keeps its samplers, box scaler, generators, the Metropolis test of box
// moves (core/Simulation.cpp:493-531), counters and step-size adaptation (:533-607); this class
//  * runs each cycle's particle moves as one device sweep (Simulation::performMoves,
//    core/Simulation.cpp:365-390): the sweep's proposals use the samplers' current step sizes and
//    a Philox stream keyed by the casino seed and numbered by the cycle, so the moves are the
//    device's own draws, not the samplers' std::mt19937 draws;
//  * tries and reverts box moves on the device (Packing::tryScaling / revertScaling);
//  * fixes orientations on the device (Packing::renormalizeOrientations);
//  * writes its state into the reference's Packing before every snapshot, averaging point, inline
//    info and at the end of a run (Packing::reset, then a recount when overlaps are counted).
// Supported: spheres, spherocylinders, polyspheres (incl. bananas) and polyspherocylinders with hard
// interactions and walls; translation, rotation, translation + rotation, or rototranslation move
// samplers; overlap relaxation without a helper shape.  Anything else raises ValidationException.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "core/SimulationBackend.h"
#include "core/shapes/PolysphereTraits.h"
#include "core/shapes/PolyspherocylinderTraits.h"
#include "core/shapes/SphereTraits.h"
#include "core/shapes/SpherocylinderTraits.h"
#include "utils/Exceptions.h"

#include "GpuPacking.hpp"

namespace rampack_gb300 {

// A failing device call surfaces as the reference's ValidationException (casino prints it and exits).
struct RaiseValidation {
    [[noreturn]] static void raise(const std::string &what, const char *, int) {
        throw ValidationException("GPU backend: " + what);
    }
};

class GpuSimulationBackend : public SimulationBackend {
public:
    using Device = BasicGpuPacking<Vec3, Mat3, DomainBounds, RaiseValidation>;

    GpuSimulationBackend(std::size_t seed, const std::array<bool, 3> &walls, int device = 0)
            : seed_{static_cast<uint64_t>(seed)}, walls_{walls}, device_{device}
    { }

    void attach(const Packing &packing, const ShapeTraits &shapeTraits, bool countOverlaps) override {
        const Interaction &interaction = shapeTraits.getInteraction();
        if (interaction.hasSoftPart())
            fail("soft interactions (and overlap relaxation with a helper shape) run on the CPU only");
        std::vector<Shape> shapes(packing.size());
        for (std::size_t i = 0; i < packing.size(); i++) {
            const auto &s = packing[i];
            for (int k = 0; k < 3; k++) shapes[i].position[k] = s.getPosition()[k];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) shapes[i].orientation[3 * a + b] = s.getOrientation()(a, b);
        }
        box_ = packing.getBox();
        const Mat3 box = toMat(box_);
        dev_.reset();
        if (auto sphere = dynamic_cast<const SphereTraits *>(&shapeTraits)) {
            dev_ = std::make_unique<Device>(box, shapes, sphere->getRadius(), -1.0, device_);
        } else if (auto sc = dynamic_cast<const SpherocylinderTraits *>(&shapeTraits)) {
            dev_ = std::make_unique<Device>(box, shapes, sc->getRadius(), sc->getLength(), device_);
        } else if (auto psc = dynamic_cast<const PolyspherocylinderTraits *>(&shapeTraits)) {
            std::vector<Centre> centres;
            for (const auto &d : psc->getSpherocylinderData())
                centres.push_back(Centre{toVec(d.position), d.radius, toVec(d.halfAxis)});
            dev_ = std::make_unique<Device>(box, shapes, centres, true, device_);
        } else if (auto ps = dynamic_cast<const PolysphereTraits *>(&shapeTraits)) {
            std::vector<Centre> centres;
            for (const auto &d : ps->getSphereData())
                centres.push_back(Centre{toVec(d.position), d.radius, Vec3{}});
            dev_ = std::make_unique<Device>(box, shapes, centres, false, device_);
        } else {
            fail("the shape is not one of sphere, spherocylinder, polysphere (incl. bananas) or polyspherocylinder");
        }
        if (walls_[0] || walls_[1] || walls_[2]) dev_->toggleWalls(walls_);
        dev_->toggleOverlapCounting(countOverlaps);
    }

    std::vector<MoveCount> performMoves(const std::vector<std::shared_ptr<MoveSampler>> &moveSamplers,
                                        double temperature, std::size_t cycle) override {
        (void)temperature;  // hard interactions: dE is 0 or infinite
        requireAttached();
        // the samplers' kinds and current steps (MoveSampler::getName / getStepSizes)
        double tstep = 0, rstep = 0;
        int translation = -1, rotation = -1, rototranslation = -1;
        for (std::size_t i = 0; i < moveSamplers.size(); i++) {
            const std::string name = moveSamplers[i]->getName();
            const auto steps = moveSamplers[i]->getStepSizes();
            if (name == "translation" && translation < 0) {
                translation = static_cast<int>(i);
                tstep = steps.at(0).second;
            } else if (name == "rotation" && rotation < 0) {
                rotation = static_cast<int>(i);
                rstep = steps.at(0).second;
            } else if (name == "rototranslation" && rototranslation < 0) {
                rototranslation = static_cast<int>(i);
                for (const auto &st : steps) {
                    if (st.first == "translation") tstep = st.second;
                    if (st.first == "rotation") rstep = st.second;
                }
            } else {
                fail("move type '" + name + "' (or this combination of move types) is not supported");
            }
        }
        if (rototranslation >= 0 && (translation >= 0 || rotation >= 0))
            fail("rototranslation moves together with translation or rotation moves are not supported");
        std::vector<MoveCount> counts(moveSamplers.size());
        const rp_sweep_stats st = dev_->performMoves(translation >= 0 || rototranslation >= 0 ? tstep : 0.0,
                                                     rotation >= 0 || rototranslation >= 0 ? rstep : 0.0, seed_,
                                                     static_cast<uint64_t>(cycle), rototranslation >= 0);
        if (rototranslation >= 0) {
            counts[rototranslation] = MoveCount{st.moves, st.accepted};
        } else {
            if (translation >= 0) counts[translation] = MoveCount{st.translations, st.accepted_translations};
            if (rotation >= 0) counts[rotation] = MoveCount{st.rotations, st.accepted - st.accepted_translations};
        }
        return counts;
    }

    [[nodiscard]] const TriclinicBox &getBox() const override { return box_; }

    double tryScaling(const TriclinicBox &newBox) override {
        requireAttached();
        const double dE = dev_->tryScaling(toMat(newBox));
        prevBox_ = box_;
        box_ = newBox;
        return dE;
    }

    void revertScaling() override {
        requireAttached();
        dev_->revertScaling();
        box_ = prevBox_;
    }

    [[nodiscard]] std::size_t getCachedNumberOfOverlaps() const override {
        requireAttached();
        return dev_->getCachedNumberOfOverlaps();
    }

    std::size_t renormalizeOrientations(bool allowOverlaps) override {
        requireAttached();
        return dev_->renormalizeOrientations(allowOverlaps);
    }

    void store(Packing &packing, const Interaction &interaction, bool countOverlaps) const override {
        requireAttached();
        const auto shapes = dev_->getShapes();
        std::vector<::Shape> out;
        out.reserve(shapes.size());
        for (const auto &s : shapes) {
            Matrix<3, 3> o;
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) o(a, b) = s.orientation[3 * a + b];
            out.emplace_back(Vector<3>{s.position[0], s.position[1], s.position[2]}, o);
        }
        packing.reset(std::move(out), box_, interaction);
        if (countOverlaps) packing.toggleOverlapCounting(true, interaction);
    }

private:
    uint64_t seed_;
    std::array<bool, 3> walls_;
    int device_;
    std::unique_ptr<Device> dev_;
    TriclinicBox box_, prevBox_;

    [[noreturn]] static void fail(const std::string &what) { RaiseValidation::raise(what, "", 0); }

    void requireAttached() const {
        if (!dev_) fail("no packing attached (Simulation::integrate or relaxOverlaps attaches one)");
    }

    static Mat3 toMat(const TriclinicBox &box) {
        const auto &m = box.getDimensions();
        Mat3 out{};
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) out[3 * a + b] = m(a, b);
        return out;
    }

    static Vec3 toVec(const Vector<3> &v) { return Vec3{v[0], v[1], v[2]}; }
};

}  // namespace rampack_gb300
