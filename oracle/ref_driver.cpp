// ORACLE — test infrastructure only (see rpo_geometry.hpp).
//
// C entry points over the reference's OWN classes (Packing, SpherocylinderTraits,
// Simulation, ...), compiled from the reference sources in place by oracle/Makefile
// into oracle/_ref/librpref.so.  Used only in the build container, to pin the
// restatement in oracle/rpo_*.hpp and to generate the golden fixtures under
// tests/golden/.  Mirrors the rpo_* entry points of rpo_capi.cpp one for one.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <map>
#include <memory>
#include <random>
#include <sstream>

#include "core/ActiveDomain.h"
#include "core/Packing.h"
#include "core/PeriodicBoundaryConditions.h"
#include "core/FreeBoundaryConditions.h"
#include "core/Simulation.h"
#include "core/ObservablesCollector.h"
#include "core/observables/NematicOrder.h"
#include "core/interactions/RepulsiveLennardJonesInteraction.h"
#include "core/interactions/SquareInverseCoreInteraction.h"
#include "core/shapes/CompoundShapeTraits.h"
#include "core/observables/correlation/LayerwiseRadialEnumerator.h"
#include "core/observables/correlation/LinearEnumerator.h"
#include "core/observables/correlation/PairAveragedCorrelation.h"
#include "core/observables/correlation/PairDensityCorrelation.h"
#include "core/observables/correlation/RadialEnumerator.h"
#include "core/observables/correlation_functions/AxesAngle.h"
#include "core/observables/correlation_functions/S110Correlation.h"
#include "core/observables/correlation_functions/S220Correlation.h"
#include "core/observables/correlation_functions/S221Correlation.h"
#include "core/io/RamtrjPlayer.h"
#include "core/io/RamtrjRecorder.h"
#include "core/move_samplers/FlipSampler.h"
#include "core/move_samplers/RotationSampler.h"
#include "core/move_samplers/TranslationSampler.h"
#include "core/shapes/PolysphereTraits.h"
#include "core/shapes/PolysphereBananaTraits.h"
#include "core/shapes/PolyspherocylinderTraits.h"
#include "core/shapes/SphereTraits.h"
#include "core/shapes/SpherocylinderTraits.h"
#include "core/shapes/GenericXenoCollideTraits.h"
#include "geometry/xenocollide/XCBodyBuilder.h"
#include "core/volume_scalers/AnisotropicVolumeScaler.h"
#include "core/volume_scalers/DeltaVolumeScaler.h"
#include "core/volume_scalers/LinearScalingFactorSampler.h"
#include "core/volume_scalers/LogScalingFactorSampler.h"
#include "core/volume_scalers/TriclinicAdapter.h"
#include "core/volume_scalers/TriclinicDeltaScaler.h"
#include "utils/Logger.h"

namespace {

std::shared_ptr<ShapeTraits> make_traits(int kind, const double *prm, int np) {
    if (kind == 0 && np >= 1) return std::make_shared<SphereTraits>(prm[0]);
    if (kind == 1 && np >= 2) return std::make_shared<SpherocylinderTraits>(prm[0], prm[1]);
    if (kind == 2 && np >= 1) {
        int k = static_cast<int>(prm[0]);
        std::vector<PolysphereTraits::SphereData> data;
        for (int i = 0; i < k; i++)
            data.emplace_back(Vector<3>{prm[1 + 4 * i], prm[2 + 4 * i], prm[3 + 4 * i]}, prm[4 + 4 * i]);
        PolysphereTraits::PolysphereGeometry geom(std::move(data), std::nullopt, std::nullopt, {0, 0, 0}, 1.0);
        return std::make_shared<PolysphereTraits>(std::move(geom));
    }
    if (kind == 3 && np >= 1) {
        int k = static_cast<int>(prm[0]);
        std::vector<PolyspherocylinderTraits::SpherocylinderData> data;
        for (int i = 0; i < k; i++) {
            const double *d = prm + 1 + 7 * i;
            data.emplace_back(Vector<3>{d[0], d[1], d[2]}, Vector<3>{d[3], d[4], d[5]}, d[6]);
        }
        PolyspherocylinderTraits::PolyspherocylinderGeometry geom(std::move(data), std::nullopt, std::nullopt,
                                                                  {0, 0, 0}, 1.0);
        return std::make_shared<PolyspherocylinderTraits>(std::move(geom));
    }
    return nullptr;
}

Matrix<3, 3> load_m(const double *p) {
    Matrix<3, 3> m;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) m(i, j) = p[3 * i + j];
    return m;
}
void store_m(const Matrix<3, 3> &m, double *p) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) p[3 * i + j] = m(i, j);
}

// A fixed-translation boundary condition, with the semantics of the reference's
// Packing-internal HardcodedTranslation (core/Packing.cpp:22-43): the neighbour-grid path
// of the pair tests.
class FixedTranslationBC : public BoundaryConditions {
    Vector<3> t;

public:
    explicit FixedTranslationBC(const Vector<3> &t_) : t{t_} {}
    void setBox(const TriclinicBox &) override {}
    [[nodiscard]] Vector<3> getCorrection(const Vector<3> &) const override {
        throw std::runtime_error("FixedTranslationBC::getCorrection");
    }
    [[nodiscard]] Vector<3> getTranslation(const Vector<3> &, const Vector<3> &) const override { return t; }
    [[nodiscard]] double getDistance2(const Vector<3> &p1, const Vector<3> &p2) const override {
        return (p2 + this->t - p1).norm2();
    }
};

struct Handle {
    std::shared_ptr<ShapeTraits> traits;
    std::unique_ptr<Packing> pk;
    int threads = 1;
    bool counting = false;
    int kind = 0;
    std::vector<double> prm;
};

}  // namespace

extern "C" {

struct ref_move {
    int32_t particle;
    int32_t type;
    int32_t domain;
    int32_t reserved;
    double translation[3];
    double rotation[9];
    double uniform;
};

void *ref_create(int kind, const double *prm, int np, int64_t n, const double *pos, const double *rot,
                 const double *box9, int threads) {
    auto h = std::make_unique<Handle>();
    h->traits = make_traits(kind, prm, np);
    if (!h->traits) return nullptr;
    h->threads = threads;
    h->kind = kind;
    h->prm.assign(prm, prm + np);
    std::vector<Shape> shapes;
    for (int64_t i = 0; i < n; i++)
        shapes.emplace_back(Vector<3>{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}, load_m(rot + 9 * i));
    try {
        h->pk = std::make_unique<Packing>(TriclinicBox(load_m(box9)), std::move(shapes),
                                          std::make_unique<PeriodicBoundaryConditions>(),
                                          h->traits->getInteraction(), threads, threads);
    } catch (const std::exception &) {
        return nullptr;
    }
    return h.release();
}

// GenericXenoCollideTraits from an XCBodyBuilder script (commands one per line or separated by
// ';', each through XCBodyBuilder::processCommand), as the frontend's generic_convex shape
// builds it (frontend/matchers/ShapeMatcher.cpp:411-441; volume 1, no axes).
static std::shared_ptr<ShapeTraits> make_convex_traits(const char *script) {
    XCBodyBuilder builder;
    std::string cur;
    std::string text = std::string(script) + "\n";
    for (char ch : text) {
        if (ch == '\n' || ch == ';') {
            if (cur.find_first_not_of(" \t\r") != std::string::npos) builder.processCommand(cur);
            cur.clear();
        } else {
            cur += ch;
        }
    }
    auto geometry = builder.releaseCollideGeometry();
    return std::make_shared<GenericXenoCollideTraits>(geometry, std::nullopt, std::nullopt, Vector<3>{0, 0, 0}, 1.0,
                                                      ShapeGeometry::NamedPoints{});
}

void *ref_create_convex(const char *script, int64_t n, const double *pos, const double *rot, const double *box9,
                        int threads) {
    auto h = std::make_unique<Handle>();
    try {
        h->traits = make_convex_traits(script);
    } catch (const std::exception &) {
        return nullptr;
    }
    h->threads = threads;
    h->kind = 4;
    std::vector<Shape> shapes;
    for (int64_t i = 0; i < n; i++)
        shapes.emplace_back(Vector<3>{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}, load_m(rot + 9 * i));
    try {
        h->pk = std::make_unique<Packing>(TriclinicBox(load_m(box9)), std::move(shapes),
                                          std::make_unique<PeriodicBoundaryConditions>(),
                                          h->traits->getInteraction(), threads, threads);
    } catch (const std::exception &) {
        return nullptr;
    }
    return h.release();
}

// The reference's own pair test of two placed bodies (XenoCollideTraits::overlapBetween with
// free boundary conditions: the second body at pos2 exactly); -1 with the builder's message in
// err for an invalid script.
int ref_convex_overlap(const char *script, const double *pos1, const double *rot1, const double *pos2,
                       const double *rot2, char *err, int errlen) {
    try {
        auto traits = make_convex_traits(script);
        FreeBoundaryConditions fbc;
        return traits->getInteraction().overlapBetween(Vector<3>{pos1[0], pos1[1], pos1[2]}, load_m(rot1), 0,
                                                       Vector<3>{pos2[0], pos2[1], pos2[2]}, load_m(rot2), 0, fbc)
                   ? 1
                   : 0;
    } catch (const std::exception &e) {
        if (err && errlen > 0) std::snprintf(err, static_cast<std::size_t>(errlen), "%s", e.what());
        return -1;
    }
}

void ref_destroy(void *hp) { delete static_cast<Handle *>(hp); }

// The shape joined with a soft helper on its interaction centres, as casino's overlap
// relaxation joins a helper shape (frontend/modes/CasinoMode.cpp:288-289): CompoundShapeTraits
// of the shape and SphereTraits / PolysphereTraits carrying a RepulsiveLennardJones (kind 1) or
// SquareInverseCore (kind 2) interaction; hard = 0 uses the soft traits alone.  The packing is
// set up for the new interaction (Packing::setupForInteraction).
int ref_set_soft(void *hp, int kind, double eps, double sigma, int hard) {
    auto *h = static_cast<Handle *>(hp);
    try {
        std::shared_ptr<CentralInteraction> ci;
        if (kind == 1) ci = std::make_shared<RepulsiveLennardJonesInteraction>(eps, sigma);
        else if (kind == 2) ci = std::make_shared<SquareInverseCoreInteraction>(eps, sigma);
        else return -1;
        std::shared_ptr<ShapeTraits> soft;
        if (h->kind == 0 || h->kind == 1) {
            soft = std::make_shared<SphereTraits>(h->kind == 0 ? h->prm[0] : h->prm[1], ci);
        } else if (h->kind == 2) {
            int k = static_cast<int>(h->prm[0]);
            std::vector<PolysphereTraits::SphereData> data;
            for (int i = 0; i < k; i++)
                data.emplace_back(Vector<3>{h->prm[1 + 4 * i], h->prm[2 + 4 * i], h->prm[3 + 4 * i]}, h->prm[4 + 4 * i]);
            PolysphereTraits::PolysphereGeometry geom(std::move(data), std::nullopt, std::nullopt, {0, 0, 0}, 1.0);
            soft = std::make_shared<PolysphereTraits>(std::move(geom), ci);
        } else {
            return -1;
        }
        if (hard) {
            h->traits = std::make_shared<CompoundShapeTraits>(h->traits, soft);
        } else {
            if (h->kind == 1) return -1;
            h->traits = soft;
        }
        h->pk->setupForInteraction(h->traits->getInteraction());
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

double ref_total_energy(void *hp) {
    auto *h = static_cast<Handle *>(hp);
    return h->pk->getTotalEnergy(h->traits->getInteraction());
}

// NematicOrder::calculate (core/observables/NematicOrder.cpp:9-28) of the handle's packing
// with the Q tensor dumped: out7 = P2, Q_11, Q_12, Q_13, Q_22, Q_23, Q_33.
int ref_nematic_order(void *hp, double *out7) {
    auto *h = static_cast<Handle *>(hp);
    try {
        NematicOrder no(true);
        no.calculate(*h->pk, 1.0, 1.0, *h->traits);
        std::vector<double> v = no.getIntervalValues();
        if (v.size() != 7) return -1;
        for (int i = 0; i < 7; i++) out7[i] = v[i];
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

int64_t ref_count_overlaps(void *hp, int early) {
    auto *h = static_cast<Handle *>(hp);
    return static_cast<int64_t>(h->pk->countTotalOverlaps(h->traits->getInteraction(), early != 0));
}

void ref_set_walls(void *hp, int mask) {
    auto *h = static_cast<Handle *>(hp);
    h->pk->toggleWalls({(mask & 1) != 0, (mask & 2) != 0, (mask & 4) != 0});
}

void ref_set_counting(void *hp, int on) {
    auto *h = static_cast<Handle *>(hp);
    h->pk->toggleOverlapCounting(on != 0, h->traits->getInteraction());
    h->counting = on != 0;
}

int64_t ref_cached_overlaps(void *hp) {
    return static_cast<int64_t>(static_cast<Handle *>(hp)->pk->getCachedNumberOfOverlaps());
}

int ref_replay_energies(void *hp, const ref_move *mv, int64_t n, const double *domains, double temperature,
                        uint8_t *out_code, int32_t *out_delta, double *out_energy);

int ref_replay(void *hp, const ref_move *mv, int64_t n, const double *domains, double temperature,
               uint8_t *out_code, int32_t *out_delta) {
    return ref_replay_energies(hp, mv, n, domains, temperature, out_code, out_delta, nullptr);
}

int ref_replay_energies(void *hp, const ref_move *mv, int64_t n, const double *domains, double temperature,
                        uint8_t *out_code, int32_t *out_delta, double *out_energy) {
    auto *h = static_cast<Handle *>(hp);
    Packing &pk = *h->pk;
    const Interaction &inter = h->traits->getInteraction();
    try {
        for (int64_t i = 0; i < n; i++) {
            const ref_move &m = mv[i];
            Vector<3> t{m.translation[0], m.translation[1], m.translation[2]};
            Matrix<3, 3> r = load_m(m.rotation);
            std::optional<ActiveDomain> ad;
            if (m.domain >= 0 && domains) {
                const double *d = domains + 6 * m.domain;
                std::array<ActiveDomain::RegionBounds, 3> b{};
                for (int k = 0; k < 3; k++) b[k] = {d[k], d[3 + k]};
                ad.emplace(pk.getBox(), b);
            }
            std::size_t before = h->counting ? pk.getCachedNumberOfOverlaps() : 0;
            double dE = 0;
            bool outside = false;
            if (m.type == 0) {
                dE = pk.tryTranslation(m.particle, t, inter, ad);
                if (ad.has_value() && dE == std::numeric_limits<double>::infinity()) {
                    // distinguish the ActiveDomain rejection from an overlap
                    Shape s = pk[m.particle];
                    PeriodicBoundaryConditions pbc(pk.getBox());
                    s.translate(t, pbc);
                    outside = !ad->isInside(s.getPosition());
                }
            } else if (m.type == 1) {
                dE = pk.tryRotation(m.particle, r, inter);
            } else {
                dE = pk.tryMove(m.particle, t, r, inter, ad);
            }
            uint8_t code = 0;
            if (outside) code = 2;
            else if (dE == std::numeric_limits<double>::infinity()) code = 1;
            else if (dE == -std::numeric_limits<double>::infinity()) code = 3;
            bool acc = m.uniform <= std::exp(-dE / temperature);
            if (acc) {
                pk.acceptMove();
                code |= 0x80;
            }
            out_code[i] = code;
            if (out_energy) out_energy[i] = dE;
            if (out_delta)
                out_delta[i] = h->counting
                                   ? (acc ? static_cast<int32_t>(pk.getCachedNumberOfOverlaps() - before) : 0)
                                   : 0;
        }
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

double ref_try_scaling(void *hp, const double *box9) {
    auto *h = static_cast<Handle *>(hp);
    return h->pk->tryScaling(TriclinicBox(load_m(box9)), h->traits->getInteraction());
}

void ref_revert_scaling(void *hp) { static_cast<Handle *>(hp)->pk->revertScaling(); }

int64_t ref_renormalize(void *hp, int allow_overlaps) {
    auto *h = static_cast<Handle *>(hp);
    return static_cast<int64_t>(h->pk->renormalizeOrientations(h->traits->getInteraction(), allow_overlaps != 0));
}

void ref_get_state(void *hp, double *pos, double *rot, double *box9) {
    auto *h = static_cast<Handle *>(hp);
    for (std::size_t i = 0; i < h->pk->size(); i++) {
        const Shape &s = (*h->pk)[i];
        for (int k = 0; k < 3; k++)
            if (pos) pos[3 * i + k] = s.getPosition()[k];
        if (rot) store_m(s.getOrientation(), rot + 9 * i);
    }
    if (box9) store_m(h->pk->getBox().getDimensions(), box9);
}

int ref_ng_divisions(void *hp, int64_t *div3) {
    auto *h = static_cast<Handle *>(hp);
    if (h->pk->getNeighbourGridMemoryUsage() == 0) return 0;
    auto d = h->pk->getNeighbourGridCellDivisions();
    for (int i = 0; i < 3; i++) div3[i] = static_cast<int64_t>(d[i]);
    return 1;
}

int ref_pair_overlap(int kind, const double *prm, int np, const double *p1, const double *r1, int c1,
                     const double *p2, const double *r2, int c2, int bc_kind, const double *box9,
                     const double *t3) {
    auto traits = make_traits(kind, prm, np);
    if (!traits) return -1;
    const Interaction &in = traits->getInteraction();
    Vector<3> v1{p1[0], p1[1], p1[2]}, v2{p2[0], p2[1], p2[2]};
    if (bc_kind == 1) {
        PeriodicBoundaryConditions pbc(TriclinicBox(load_m(box9)));
        return in.overlapBetween(v1, load_m(r1), c1, v2, load_m(r2), c2, pbc) ? 1 : 0;
    }
    if (bc_kind == 2) {
        FixedTranslationBC fixed(Vector<3>{t3[0], t3[1], t3[2]});
        return in.overlapBetween(v1, load_m(r1), c1, v2, load_m(r2), c2, fixed) ? 1 : 0;
    }
    FreeBoundaryConditions fbc;
    return in.overlapBetween(v1, load_m(r1), c1, v2, load_m(r2), c2, fbc) ? 1 : 0;
}

void ref_rotation(const double *axis3, double angle, double *out9) {
    store_m(Matrix<3, 3>::rotation(Vector<3>{axis3[0], axis3[1], axis3[2]}, angle), out9);
}

void ref_box_info(const double *box9, double *inv9, double *heights3, double *volume) {
    TriclinicBox b(load_m(box9));
    Matrix<3, 3> inv = b.getDimensions().inverse();
    if (inv9) store_m(inv, inv9);
    auto h = b.getHeights();
    if (heights3)
        for (int i = 0; i < 3; i++) heights3[i] = h[i];
    if (volume) *volume = b.getVolume();
}

// Body-frame sphere centres and radii of a bent polysphere (PolysphereBananaTraits).
int ref_banana_centres(double arc_radius, double arc_angle, int n, double sphere_radius, double *out4) {
    PolysphereBananaTraits traits(arc_radius, arc_angle, static_cast<std::size_t>(n), sphere_radius);
    const auto &data = traits.getSphereData();
    for (std::size_t i = 0; i < data.size(); i++) {
        for (int k = 0; k < 3; k++) out4[4 * i + k] = data[i].position[k];
        out4[4 * i + 3] = data[i].radius;
    }
    return static_cast<int>(data.size());
}

struct ref_rng {
    std::mt19937 mt;
};
void *ref_rng_create(uint64_t seed) { return new ref_rng{std::mt19937(static_cast<unsigned long>(seed))}; }
void ref_rng_destroy(void *r) { delete static_cast<ref_rng *>(r); }

// Draws moves with the reference's own samplers (TranslationSampler, RotationSampler)
// in Simulation::tryMove's order: move-type int, sampler draws, Metropolis uniform.
int ref_draw_moves(void *rp, void *hp, double trans_step, double rot_step, const int64_t *idxs, int64_t nidx,
                   int64_t per_type, int64_t n, int32_t domain, ref_move *out) {
    auto &mt = static_cast<ref_rng *>(rp)->mt;
    auto *h = static_cast<Handle *>(hp);
    std::vector<std::unique_ptr<MoveSampler>> samplers;
    if (trans_step > 0) samplers.push_back(std::make_unique<TranslationSampler>(trans_step));
    if (rot_step > 0) samplers.push_back(std::make_unique<RotationSampler>(rot_step));
    std::vector<std::size_t> list(idxs, idxs + nidx);
    std::uniform_real_distribution<double> unit;
    std::size_t total = static_cast<std::size_t>(per_type) * samplers.size();
    for (int64_t i = 0; i < n; i++) {
        std::uniform_int_distribution<std::size_t> md(0, total - 1);
        std::size_t sampled = md(mt);
        std::size_t k = sampled / static_cast<std::size_t>(per_type);
        auto data = samplers[k]->sampleMove(*h->pk, list, mt);
        ref_move &m = out[i];
        std::memset(&m, 0, sizeof(m));
        m.particle = static_cast<int32_t>(data.particleIdx);
        m.type = data.moveType == MoveSampler::MoveType::TRANSLATION ? 0 : 1;
        m.domain = domain;
        for (int q = 0; q < 3; q++) m.translation[q] = data.translation[q];
        store_m(data.rotation, m.rotation);
        m.uniform = unit(mt);
    }
    return 0;
}

// FlipSampler (core/move_samplers/FlipSampler.cpp) set up for the handle's shape, drawing
// `n` moves from the particle list
int ref_draw_flips(void *rp, void *hp, const int64_t *idxs, int64_t nidx, int64_t n, int32_t domain, ref_move *out) {
    auto &mt = static_cast<ref_rng *>(rp)->mt;
    auto *h = static_cast<Handle *>(hp);
    try {
        FlipSampler fs(1);
        fs.setupForShapeTraits(*h->traits);
        std::vector<std::size_t> list(idxs, idxs + nidx);
        std::uniform_real_distribution<double> unit;
        for (int64_t i = 0; i < n; i++) {
            auto data = fs.sampleMove(*h->pk, list, mt);
            ref_move &m = out[i];
            std::memset(&m, 0, sizeof(m));
            m.particle = static_cast<int32_t>(data.particleIdx);
            m.type = data.moveType == MoveSampler::MoveType::TRANSLATION ? 0
                     : data.moveType == MoveSampler::MoveType::ROTATION ? 1 : 2;
            m.domain = domain;
            for (int q = 0; q < 3; q++) m.translation[q] = data.translation[q];
            store_m(data.rotation, m.rotation);
            m.uniform = unit(mt);
        }
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

struct ref_sim_params {
    double temperature, pressure, translation_step, rotation_step;
    int32_t box_kind, adjust_steps;
    double box_step;
    int64_t domains[3];
    uint64_t seed;
    int64_t threads;
};

struct ref_sim_stats {
    int64_t moves[2], accepted[2];
    int64_t scalings, scalings_accepted, cycles;
    int64_t domains[3];
    double move_us, scaling_us, total_us;
    double steps[2];
    double box_step;
};

// Runs Simulation::integrate (thermalisation when adjust_steps, else averaging) for
// `cycles` cycles on the handle's packing; the packing is moved into the Simulation and
// its final state copied back.
int ref_sim_run(void *hp, const ref_sim_params *p, int64_t cycles, ref_sim_stats *out) {
    auto *h = static_cast<Handle *>(hp);
    try {
        std::vector<std::unique_ptr<MoveSampler>> samplers;
        if (p->translation_step > 0) samplers.push_back(std::make_unique<TranslationSampler>(p->translation_step));
        if (p->rotation_step > 0) samplers.push_back(std::make_unique<RotationSampler>(p->rotation_step));
        std::unique_ptr<TriclinicBoxScaler> scaler;
        if (p->box_kind == 1) {
            scaler = std::make_unique<TriclinicDeltaScaler>(p->box_step, true);
        } else if (p->box_kind == 2) {
            auto vs = std::make_unique<AnisotropicVolumeScaler>(std::make_unique<LogScalingFactorSampler>(),
                                                                AnisotropicVolumeScaler::X & AnisotropicVolumeScaler::Y
                                                                    & AnisotropicVolumeScaler::Z);
            scaler = std::make_unique<TriclinicAdapter>(std::move(vs), p->box_step);
        } else if (p->box_kind == 3) {
            scaler = std::make_unique<TriclinicAdapter>(std::make_unique<DeltaVolumeScaler>(), p->box_step);
        }
        std::array<std::size_t, 3> dd{static_cast<std::size_t>(p->domains[0]), static_cast<std::size_t>(p->domains[1]),
                                      static_cast<std::size_t>(p->domains[2])};
        Simulation sim(std::move(h->pk), std::move(samplers), static_cast<unsigned long>(p->seed), std::move(scaler),
                       dd, false);
        Simulation::Environment env;
        env.setTemperature(p->temperature);
        env.setPressure(p->pressure);
        if (p->box_kind == 0) env.disableBoxScaling();
        Simulation::IntegrationParameters ip;
        if (p->adjust_steps) ip.thermalisationCycles = static_cast<std::size_t>(cycles);
        else ip.averagingCycles = static_cast<std::size_t>(cycles);
        ip.averagingEvery = static_cast<std::size_t>(cycles);
        ip.snapshotEvery = static_cast<std::size_t>(cycles);
        ip.inlineInfoEvery = static_cast<std::size_t>(cycles);
        auto collector = std::make_shared<ObservablesCollector>();
        std::ostringstream sink;
        Logger logger(sink);
        sim.integrate(env, ip, *h->traits, collector, {}, logger);
        if (out) {
            std::memset(out, 0, sizeof(*out));
            auto stats = sim.getMovesStatistics();
            int slot = 0;
            for (const auto &st : stats) {
                if (st.groupName == "scaling") {
                    out->scalings = static_cast<int64_t>(st.totalMoves);
                    out->scalings_accepted = static_cast<int64_t>(st.acceptedMoves);
                    if (!st.stepSizeDatas.empty()) out->box_step = st.stepSizeDatas.front().stepSize;
                    continue;
                }
                int k = st.groupName == "rotation" ? 1 : (st.groupName == "translation" ? 0 : slot);
                slot++;
                if (k > 1) continue;
                out->moves[k] = static_cast<int64_t>(st.totalMoves);
                out->accepted[k] = static_cast<int64_t>(st.acceptedMoves);
                if (!st.stepSizeDatas.empty()) out->steps[k] = st.stepSizeDatas.front().stepSize;
            }
            out->cycles = static_cast<int64_t>(sim.getPerformedCycles());
            out->move_us = sim.getMoveMicroseconds();
            out->scaling_us = sim.getScalingMicroseconds();
            out->total_us = sim.getTotalMicroseconds();
        }
        // take the packing back
        const Packing &fin = sim.getPacking();
        std::vector<Shape> shapes(fin.begin(), fin.end());
        h->pk = std::make_unique<Packing>(fin.getBox(), std::move(shapes),
                                          std::make_unique<PeriodicBoundaryConditions>(),
                                          h->traits->getInteraction(), h->threads, h->threads);
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

// ---- snapshot and trajectory files through the reference's own readers and writers ----

// Packing::store (core/Packing.cpp:956-959): RAMSNAP of the handle's packing; 0, or -1 with
// the exception text in err
int ref_ramsnap_write(void *hp, const char *path, int naux, const char *const *keys, const char *const *values,
                      char *err, int errcap) {
    auto *h = static_cast<Handle *>(hp);
    std::map<std::string, std::string> aux;
    for (int i = 0; i < naux; i++) aux[keys[i]] = values[i];
    try {
        std::ofstream out(path);
        h->pk->store(out, aux);
        return out ? 0 : -1;
    } catch (const std::exception &e) {
        std::snprintf(err, errcap, "%s", e.what());
        return -1;
    }
}

// Packing::restore (core/Packing.cpp:961-964) into an empty packing of a shape kind: the
// number of shapes (at most cap are returned), or -1 with the exception text in err; aux
// entries as "key\tvalue\n" lines in auxbuf
int64_t ref_ramsnap_read(const char *path, int kind, const double *prm, int np, double *pos, double *rot,
                         double *box9, int64_t cap, char *auxbuf, int auxcap, char *err, int errcap) {
    auto traits = make_traits(kind, prm, np);
    if (!traits) return -1;
    try {
        Packing pk(std::make_unique<PeriodicBoundaryConditions>(), 1, 1);
        std::ifstream in(path);
        auto aux = pk.restore(in, traits->getInteraction());
        std::string a;
        for (auto &kv : aux) a += kv.first + "\t" + kv.second + "\n";
        std::snprintf(auxbuf, auxcap, "%s", a.c_str());
        for (std::size_t i = 0; i < pk.size() && static_cast<int64_t>(i) < cap; i++) {
            for (int k = 0; k < 3; k++) pos[3 * i + k] = pk[i].getPosition()[k];
            store_m(pk[i].getOrientation(), rot + 9 * i);
        }
        store_m(pk.getBox().getDimensions(), box9);
        return static_cast<int64_t>(pk.size());
    } catch (const std::exception &e) {
        std::snprintf(err, errcap, "%s", e.what());
        return -1;
    }
}

// RamtrjRecorder (core/io/RamtrjRecorder.cpp): a new trajectory of `snapshots` states
// (pos [snapshots][n][3], rot [snapshots][n][9], boxes [snapshots][9]) of a shape kind
int ref_ramtrj_write(const char *path, int kind, const double *prm, int np, int64_t n, int64_t snapshots,
                     int64_t cycle_step, const double *pos, const double *rot, const double *boxes, char *err,
                     int errcap) {
    auto traits = make_traits(kind, prm, np);
    if (!traits) return -1;
    try {
        auto stream = std::make_unique<std::fstream>(path, std::ios::in | std::ios::out | std::ios::binary |
                                                           std::ios::trunc);
        RamtrjRecorder rec(std::move(stream), static_cast<std::size_t>(n), static_cast<std::size_t>(cycle_step),
                           false);
        for (int64_t s = 0; s < snapshots; s++) {
            std::vector<Shape> shapes;
            for (int64_t i = 0; i < n; i++) {
                const double *p = pos + 3 * (s * n + i);
                shapes.emplace_back(Vector<3>{p[0], p[1], p[2]}, load_m(rot + 9 * (s * n + i)));
            }
            Packing pk(TriclinicBox(load_m(boxes + 9 * s)), std::move(shapes),
                       std::make_unique<PeriodicBoundaryConditions>(), traits->getInteraction(), 1, 1);
            rec.recordSnapshot(pk, static_cast<std::size_t>((s + 1) * cycle_step));
        }
        rec.close();
        return 0;
    } catch (const std::exception &e) {
        std::snprintf(err, errcap, "%s", e.what());
        return -1;
    }
}

// RamtrjPlayer::jumpToSnapshot (core/io/RamtrjPlayer.cpp:71-86): snapshot `index` (from 0)
int ref_ramtrj_read(const char *path, int kind, const double *prm, int np, int64_t index, double *pos, double *rot,
                    double *box9, char *err, int errcap) {
    auto traits = make_traits(kind, prm, np);
    if (!traits) return -1;
    try {
        auto in = std::make_unique<std::ifstream>(path, std::ios::in | std::ios::binary);
        RamtrjPlayer player(std::move(in));
        Packing pk(std::make_unique<PeriodicBoundaryConditions>(), 1, 1);
        // an empty packing of the right size for the player to reset
        std::ifstream probe(path, std::ios::binary);
        char magic[7];
        unsigned char ver[2];
        std::size_t hdr[3];
        probe.read(magic, 7);
        probe.read(reinterpret_cast<char *>(ver), 2);
        probe.read(reinterpret_cast<char *>(hdr), sizeof(hdr));
        std::vector<Shape> shapes(hdr[0]);
        pk.reset(std::move(shapes), TriclinicBox(1.0), traits->getInteraction());
        player.jumpToSnapshot(pk, traits->getInteraction(), static_cast<std::size_t>((index + 1) * hdr[2]));
        for (std::size_t i = 0; i < pk.size(); i++) {
            for (int k = 0; k < 3; k++) pos[3 * i + k] = pk[i].getPosition()[k];
            store_m(pk[i].getOrientation(), rot + 9 * i);
        }
        store_m(pk.getBox().getDimensions(), box9);
        return 0;
    } catch (const std::exception &e) {
        std::snprintf(err, errcap, "%s", e.what());
        return -1;
    }
}

// TriclinicBoxScaler::updateBox then Simulation's unit-interval draw, `count` times from the
// same box with one std::mt19937(seed): the box-move proposal stream of the reference.
// kind 1 TriclinicDeltaScaler, 2 log / 3 linear AnisotropicVolumeScaler through
// TriclinicAdapter (groups: axis masks combined with & inside, | between), 4 DeltaVolumeScaler.
int ref_box_proposals(int kind, int together, int ngroups, const int *groups, int independent, double step,
                      uint64_t seed, const double *box9, int64_t count, double *boxes, double *uniforms) {
    std::unique_ptr<TriclinicBoxScaler> sc;
    if (kind == 1) {
        sc = std::make_unique<TriclinicDeltaScaler>(step, together != 0);
    } else if (kind == 4) {
        sc = std::make_unique<TriclinicAdapter>(std::make_unique<DeltaVolumeScaler>(), step);
    } else if (kind == 2 || kind == 3) {
        using SD = AnisotropicVolumeScaler::ScalingDirection;
        SD dir;
        for (int g = 0; g < ngroups; g++) {
            SD one;
            bool first = true;
            const SD axes[3] = {AnisotropicVolumeScaler::X, AnisotropicVolumeScaler::Y, AnisotropicVolumeScaler::Z};
            for (int a = 0; a < 3; a++)
                if (groups[g] & (1 << a)) {
                    one = first ? axes[a] : (one & axes[a]);
                    first = false;
                }
            dir = g == 0 ? one : (dir | one);
        }
        std::unique_ptr<ScalingFactorSampler> fs;
        if (kind == 2) fs = std::make_unique<LogScalingFactorSampler>();
        else fs = std::make_unique<LinearScalingFactorSampler>();
        sc = std::make_unique<TriclinicAdapter>(
            std::make_unique<AnisotropicVolumeScaler>(std::move(fs), dir, independent != 0), step);
    } else {
        return -1;
    }
    std::mt19937 mt(seed);
    std::uniform_real_distribution<double> unit;
    TriclinicBox box(load_m(box9));
    for (int64_t k = 0; k < count; k++) {
        TriclinicBox nb = sc->updateBox(box, mt);
        store_m(nb.getDimensions(), boxes + 9 * k);
        uniforms[k] = unit(mt);
    }
    return 0;
}

// ---- pair correlations: the reference's own PairDensityCorrelation /
// PairAveragedCorrelation over its RadialEnumerator, LinearEnumerator and
// LayerwiseRadialEnumerator, one snapshot per packing state, printed at full precision

std::shared_ptr<ShapeTraits> make_traits_axes(int kind, const double *prm, int np, const double *primary,
                                              const double *secondary) {
    if (kind != 2) return make_traits(kind, prm, np);
    int k = static_cast<int>(prm[0]);
    std::vector<PolysphereTraits::SphereData> data;
    for (int i = 0; i < k; i++)
        data.emplace_back(Vector<3>{prm[1 + 4 * i], prm[2 + 4 * i], prm[3 + 4 * i]}, prm[4 + 4 * i]);
    std::optional<Vector<3>> a1, a2;
    if (primary) a1 = Vector<3>{primary[0], primary[1], primary[2]};
    if (secondary) a2 = Vector<3>{secondary[0], secondary[1], secondary[2]};
    PolysphereTraits::PolysphereGeometry geom(std::move(data), a1, a2, {0, 0, 0}, 1.0);
    return std::make_shared<PolysphereTraits>(std::move(geom));
}

int ref_named_point(int kind, const double *prm, int np, const char *name, double *out3) {
    auto traits = make_traits(kind, prm, np);
    try {
        auto v = traits->getGeometry().getNamedPoint(name);
        for (int i = 0; i < 3; i++) out3[i] = v[i];
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

int ref_pair_correlation(int kind, const double *prm, int np, const double *primary, const double *secondary,
                         int64_t n, int nsnap, const double *pos, const double *rot, const double *box9,
                         int enumerator, int linear_axis, const int *miller, const char *focal, int function,
                         int axis, double max_r, int num_bins, double *x, double *y, uint64_t *count) {
    auto traits = make_traits_axes(kind, prm, np, primary, secondary);
    if (!traits) return -1;
    std::shared_ptr<PairEnumerator> en;
    if (enumerator == 0)
        en = std::make_shared<RadialEnumerator>(focal);
    else if (enumerator == 1)
        en = std::make_shared<LinearEnumerator>(static_cast<LinearEnumerator::Axis>(linear_axis), focal);
    else
        en = std::make_shared<LayerwiseRadialEnumerator>(std::array<int, 3>{miller[0], miller[1], miller[2]},
                                                         focal);
    auto ax = static_cast<ShapeGeometry::Axis>(axis);
    std::unique_ptr<BulkObservable> obs;
    std::shared_ptr<CorrelationFunction> fn;
    if (function == 1) fn = std::make_shared<S110Correlation>(ax);
    if (function == 2) fn = std::make_shared<S220Correlation>(ax);
    if (function == 3) fn = std::make_shared<S221Correlation>(ax);
    if (function == 4) fn = std::make_shared<AxesAngle>(ax);
    if (function == 0)
        obs = std::make_unique<PairDensityCorrelation>(en, max_r, num_bins, true);
    else
        obs = std::make_unique<PairAveragedCorrelation>(en, fn, max_r, num_bins, true);
    try {
        for (int s = 0; s < nsnap; s++) {
            std::vector<Shape> shapes;
            const double *p = pos + 3 * n * s, *r = rot + 9 * n * s;
            for (int64_t i = 0; i < n; i++)
                shapes.emplace_back(Vector<3>{p[3 * i], p[3 * i + 1], p[3 * i + 2]}, load_m(r + 9 * i));
            Packing pk(TriclinicBox(load_m(box9 + 9 * s)), std::move(shapes),
                       std::make_unique<PeriodicBoundaryConditions>(), traits->getInteraction(), 1, 1);
            obs->addSnapshot(pk, 1, 1, *traits);
        }
    } catch (const std::exception &e) {
        std::fprintf(stderr, "ref_pair_correlation: %s\n", e.what());
        return -2;
    }
    std::ostringstream out;
    out << std::setprecision(17);
    obs->print(out);
    std::istringstream in(out.str());
    std::string line;
    int b = 0;
    while (std::getline(in, line) && b < num_bins) {
        std::istringstream ls(line);
        std::string xs, ys;
        ls >> xs >> ys >> count[b];
        x[b] = std::stod(xs);
        y[b] = (ys.find("nan") != std::string::npos) ? std::nan("") : std::stod(ys);
        b++;
    }
    return b;
}

}  // extern "C"
