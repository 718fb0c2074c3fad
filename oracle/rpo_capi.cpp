// ORACLE — test infrastructure only (see rpo_geometry.hpp).
//
// C entry points over the CPU restatement, loaded with ctypes by the tests and by
// bench.py's CPU-baseline leg.  Shape kinds: 0 sphere {r}, 1 spherocylinder {l, r},
// 2 polysphere {k, x0, y0, z0, r0, ..., x(k-1), y(k-1), z(k-1), r(k-1)}.
#include <cstdint>
#include <cstring>
#include <memory>

#include "rpo_correlation.hpp"
#include "rpo_sim.hpp"

using namespace rpo;

namespace {

struct Handle {
    Interaction inter;
    std::unique_ptr<Packing> pk;
};

bool make_interaction(int kind, const double *prm, int np, Interaction &out) {
    out.kind = kind;
    if (kind == SPHERE) {
        if (np < 1) return false;
        out.radius = prm[0];
    } else if (kind == SPHEROCYLINDER) {
        if (np < 2) return false;
        out.length = prm[0];
        out.radius = prm[1];
    } else if (kind == POLYSPHERE) {
        if (np < 1) return false;
        int k = static_cast<int>(prm[0]);
        if (k < 1 || np < 1 + 4 * k) return false;
        for (int i = 0; i < k; i++) {
            out.centres.push_back({prm[1 + 4 * i], prm[2 + 4 * i], prm[3 + 4 * i]});
            out.radii.push_back(prm[4 + 4 * i]);
        }
    } else if (kind == 3) {
        // polyspherocylinder {k, (x, y, z, hx, hy, hz, r) per spherocylinder}: a multi-centre
        // body like the polysphere, each centre with a half axis
        if (np < 1) return false;
        int k = static_cast<int>(prm[0]);
        if (k < 1 || np < 1 + 7 * k) return false;
        out.kind = POLYSPHERE;
        for (int i = 0; i < k; i++) {
            const double *d = prm + 1 + 7 * i;
            out.centres.push_back({d[0], d[1], d[2]});
            out.half_axes.push_back({d[3], d[4], d[5]});
            out.radii.push_back(d[6]);
        }
    } else {
        return false;
    }
    return true;
}

M3 load_m3(const double *p) {
    M3 m{};
    std::memcpy(m.data(), p, sizeof(double) * 9);
    return m;
}

}  // namespace

extern "C" {

// Same layout as rp_move in include/rampack_gb300.h (120 bytes).
struct rpo_move {
    int32_t particle;
    int32_t type;
    int32_t domain;
    int32_t reserved;
    double translation[3];
    double rotation[9];
    double uniform;
};

int rpo_move_size() { return static_cast<int>(sizeof(rpo_move)); }

void *rpo_create(int kind, const double *prm, int np, int64_t n, const double *pos, const double *rot,
                 const double *box9, int threads) {
    auto h = std::make_unique<Handle>();
    if (!make_interaction(kind, prm, np, h->inter)) return nullptr;
    std::vector<Shape> shapes(static_cast<std::size_t>(n));
    for (int64_t i = 0; i < n; i++) {
        shapes[i].pos = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        shapes[i].rot = load_m3(rot + 9 * i);
    }
    try {
        h->pk = std::make_unique<Packing>(Box(load_m3(box9)), std::move(shapes), h->inter,
                                          static_cast<std::size_t>(threads), static_cast<std::size_t>(threads));
    } catch (const std::exception &) {
        return nullptr;
    }
    return h.release();
}

// A generic convex body (GenericXenoCollideTraits) from an XCBodyBuilder script: commands one
// per line or separated by ';'; null for an invalid script.
void *rpo_create_convex(const char *script, int64_t n, const double *pos, const double *rot, const double *box9,
                        int threads) {
    auto h = std::make_unique<Handle>();
    h->inter.kind = CONVEX;
    try {
        h->inter.xc = xc_build_script(script);
    } catch (const std::exception &) {
        return nullptr;
    }
    std::vector<Shape> shapes(static_cast<std::size_t>(n));
    for (int64_t i = 0; i < n; i++) {
        shapes[i].pos = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        shapes[i].rot = load_m3(rot + 9 * i);
    }
    try {
        h->pk = std::make_unique<Packing>(Box(load_m3(box9)), std::move(shapes), h->inter,
                                          static_cast<std::size_t>(threads), static_cast<std::size_t>(threads));
    } catch (const std::exception &) {
        return nullptr;
    }
    return h.release();
}

// The pair test alone: XenoCollideTraits::overlapBetween of two placed bodies (the second at
// pos2 exactly, no periodic image); -1 for an invalid script.
int rpo_convex_overlap(const char *script, const double *pos1, const double *rot1, const double *pos2,
                       const double *rot2) {
    XcPtr g;
    try {
        g = xc_build_script(script);
    } catch (const std::exception &) {
        return -1;
    }
    return xc_overlap(*g, {pos1[0], pos1[1], pos1[2]}, load_m3(rot1), {pos2[0], pos2[1], pos2[2]}, load_m3(rot2)) ? 1
                                                                                                                : 0;
}

void rpo_destroy(void *hp) { delete static_cast<Handle *>(hp); }

// A soft part joined to the shape's hard interaction (CompoundInteraction with a central
// helper on the same interaction centres): kind 1 RepulsiveLennardJones, 2 SquareInverseCore;
// hard = 0 keeps the soft part alone (spheres and polyspheres).  The packing is set up
// again for the compound's range (Packing::setupForInteraction).
int rpo_set_soft(void *hp, int kind, double eps, double sigma, int hard) {
    auto *h = static_cast<Handle *>(hp);
    if (kind < 1 || kind > 2 || !(sigma > 0) || (kind == 1 && !(eps > 0)) || (kind == 2 && eps == 0)) return -1;
    if (!hard && (h->inter.kind == SPHEROCYLINDER || h->inter.segments())) return -1;
    h->inter.set_soft(kind, eps, sigma, hard != 0);
    try {
        h->pk->setup_for_interaction(h->inter);
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

// Packing::getTotalEnergy (core/Packing.cpp:689-709)
double rpo_total_energy(void *hp) {
    auto *h = static_cast<Handle *>(hp);
    return h->pk->total_energy(h->inter);
}

int64_t rpo_size(void *hp) { return static_cast<int64_t>(static_cast<Handle *>(hp)->pk->size()); }

int64_t rpo_count_overlaps(void *hp, int early) {
    auto *h = static_cast<Handle *>(hp);
    return static_cast<int64_t>(h->pk->count_total_overlaps(h->inter, early != 0));
}

// Packing::toggleWalls (core/Packing.cpp:1081-1084): bit i walls the planes spanned by the
// box sides other than side i
void rpo_set_walls(void *hp, int mask) {
    auto *h = static_cast<Handle *>(hp);
    for (int i = 0; i < 3; i++) h->pk->has_wall[i] = ((mask >> i) & 1) != 0;
    h->pk->has_any_walls = (mask & 7) != 0;
}

void rpo_set_counting(void *hp, int on) {
    auto *h = static_cast<Handle *>(hp);
    h->pk->set_counting(on != 0, h->inter);
}

int64_t rpo_cached_overlaps(void *hp) { return static_cast<int64_t>(static_cast<Handle *>(hp)->pk->num_overlaps); }

// Replays proposals in order through tryTranslation/tryRotation/tryMove + Metropolis +
// acceptMove (core/Simulation.cpp:466-490).  domains: 6 doubles per record (lo[3], hi[3]),
// indexed by rpo_move::domain; domain < 0 means no ActiveDomain.  out_code per move:
// low two bits 0 = dE 0, 1 = overlap (+inf), 2 = outside the active domain (+inf),
// 3 = -inf (fewer overlaps, counting mode); bit 7 = accepted.  out_delta (optional)
// receives the overlap-count delta in counting mode.
int rpo_replay_energies(void *hp, const rpo_move *mv_, int64_t n, const double *domains, double temperature,
                        uint8_t *out_code, int32_t *out_delta, double *out_energy);

int rpo_replay(void *hp, const rpo_move *mv_, int64_t n, const double *domains, double temperature,
               uint8_t *out_code, int32_t *out_delta) {
    return rpo_replay_energies(hp, mv_, n, domains, temperature, out_code, out_delta, nullptr);
}

// As rpo_replay, also writing each move's energy (0, +-inf, or the soft energy change).
int rpo_replay_energies(void *hp, const rpo_move *mv_, int64_t n, const double *domains, double temperature,
                        uint8_t *out_code, int32_t *out_delta, double *out_energy) {
    auto *h = static_cast<Handle *>(hp);
    Packing &pk = *h->pk;
    try {
        for (int64_t i = 0; i < n; i++) {
            const rpo_move &m = mv_[i];
            V3 t{m.translation[0], m.translation[1], m.translation[2]};
            M3 r = load_m3(m.rotation);
            const double *lo = nullptr, *hi = nullptr;
            if (m.domain >= 0 && domains) {
                lo = domains + 6 * m.domain;
                hi = lo + 3;
            }
            bool outside = false;
            pk.last_delta[0] = 0;
            double dE = pk.try_move(m.type, static_cast<std::size_t>(m.particle), t, r, h->inter, lo, hi, &outside);
            uint8_t code = 0;
            if (outside) code = 2;
            else if (dE == Packing::INF) code = 1;
            else if (dE == -Packing::INF) code = 3;
            bool acc = m.uniform <= std::exp(-dE / temperature);
            if (acc) {
                pk.accept(2);
                code |= 0x80;
            }
            out_code[i] = code;
            if (out_energy) out_energy[i] = dE;
            if (out_delta) out_delta[i] = (pk.counting && acc) ? pk.last_delta[0] : 0;
        }
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

double rpo_try_scaling(void *hp, const double *box9) {
    auto *h = static_cast<Handle *>(hp);
    return h->pk->try_scaling(Box(load_m3(box9)), h->inter);
}

void rpo_revert_scaling(void *hp) { static_cast<Handle *>(hp)->pk->revert_scaling(); }

int64_t rpo_renormalize(void *hp, int allow_overlaps) {
    auto *h = static_cast<Handle *>(hp);
    return static_cast<int64_t>(h->pk->renormalize_orientations(h->inter, allow_overlaps != 0));
}

void rpo_get_state(void *hp, double *pos, double *rot, double *box9) {
    auto *h = static_cast<Handle *>(hp);
    std::size_t n = h->pk->size();
    for (std::size_t i = 0; i < n; i++) {
        const Shape &s = h->pk->shapes[i];
        if (pos) std::memcpy(pos + 3 * i, s.pos.data(), 3 * sizeof(double));
        if (rot) std::memcpy(rot + 9 * i, s.rot.data(), 9 * sizeof(double));
    }
    if (box9) std::memcpy(box9, h->pk->box.dim.data(), 9 * sizeof(double));
}

// Real (non-halo) neighbour-grid divisions; returns 0 when the packing has no grid.
int rpo_ng_divisions(void *hp, int64_t *div3) {
    auto *h = static_cast<Handle *>(hp);
    if (!h->pk->ng.has_value()) return 0;
    auto d = h->pk->ng->real_divisions();
    for (int i = 0; i < 3; i++) div3[i] = static_cast<int64_t>(d[i]);
    return 1;
}

// One pair test.  bc_kind 0 free, 1 periodic in box9, 2 fixed translation t3.
int rpo_pair_overlap(int kind, const double *prm, int np, const double *p1, const double *r1, int c1,
                     const double *p2, const double *r2, int c2, int bc_kind, const double *box9,
                     const double *t3) {
    Interaction in;
    if (!make_interaction(kind, prm, np, in)) return -1;
    Box bx;
    BC bc;
    if (bc_kind == 1) {
        bx = Box(load_m3(box9));
        bc = BC::periodic(bx);
    } else if (bc_kind == 2) {
        bc = BC::fixed({t3[0], t3[1], t3[2]});
    }
    return in.overlap({p1[0], p1[1], p1[2]}, load_m3(r1), c1, {p2[0], p2[1], p2[2]}, load_m3(r2), c2, bc) ? 1 : 0;
}

// Geometry helpers exposed for golden checks.
void rpo_box_info(const double *box9, double *inv9, double *heights3, double *volume) {
    Box b(load_m3(box9));
    if (inv9) std::memcpy(inv9, b.inv.data(), 9 * sizeof(double));
    V3 h = b.heights();
    if (heights3) std::memcpy(heights3, h.data(), 3 * sizeof(double));
    if (volume) *volume = b.volume();
}

void rpo_rotation(const double *axis3, double angle, double *out9) {
    M3 r = rotation_axis_angle({axis3[0], axis3[1], axis3[2]}, angle);
    std::memcpy(out9, r.data(), 9 * sizeof(double));
}

void rpo_rotation_euler(double ax, double ay, double az, double *out9) {
    M3 r = rotation_euler(ax, ay, az);
    std::memcpy(out9, r.data(), 9 * sizeof(double));
}

double rpo_segment_distance2(const double *a, const double *b, const double *c, const double *d) {
    return segment_distance2({a[0], a[1], a[2]}, {b[0], b[1], b[2]}, {c[0], c[1], c[2]}, {d[0], d[1], d[2]});
}

// ---- proposal streams drawn exactly as the reference's samplers draw them ----
struct rpo_rng {
    std::mt19937 mt;
};

void *rpo_rng_create(uint64_t seed) { return new rpo_rng{std::mt19937(static_cast<unsigned long>(seed))}; }
void rpo_rng_destroy(void *r) { delete static_cast<rpo_rng *>(r); }

// Draws n moves over the particle list idxs, as one DD domain of Simulation::tryMove
// does (Simulation.cpp:454-483): move type from uniform_int over the per-type
// accumulations (per_type moves each), the sampler's draws, then the Metropolis
// uniform.  Samplers: translation (if trans_step > 0) then rotation (if rot_step > 0).
int rpo_draw_moves(void *rp, double trans_step, double rot_step, const double *box9, const int64_t *idxs,
                   int64_t nidx, int64_t per_type, int64_t n, int32_t domain, rpo_move *out) {
    auto &mt = static_cast<rpo_rng *>(rp)->mt;
    if (nidx <= 0 || per_type <= 0) return -1;
    std::vector<int> kinds;
    if (trans_step > 0) kinds.push_back(0);
    if (rot_step > 0) kinds.push_back(1);
    if (kinds.empty()) return -1;
    Box box(load_m3(box9));
    V3 h = box.heights();
    double max_t = std::min({h[0], h[1], h[2]}) / 2;
    std::uniform_real_distribution<double> unit;
    std::size_t total = static_cast<std::size_t>(per_type) * kinds.size();
    for (int64_t i = 0; i < n; i++) {
        std::uniform_int_distribution<std::size_t> md(0, total - 1);
        std::size_t sampled = md(mt);
        std::size_t k = sampled / static_cast<std::size_t>(per_type);
        rpo_move &m = out[i];
        std::memset(&m, 0, sizeof(m));
        M3 r{};  // MoveData's default-constructed (zero) matrix for translations (core/MoveSampler.h:40-49)
        V3 t{};
        if (kinds[k] == 0) {
            double a = std::min(max_t, trans_step);
            std::uniform_real_distribution<double> d(-a, a);
            t = {d(mt), d(mt), d(mt)};
            m.type = 0;
        } else {
            std::uniform_real_distribution<double> ang(-rot_step, rot_step);
            std::uniform_real_distribution<double> pm(-1, 1);
            V3 axis;
            do {
                axis = {pm(mt), pm(mt), pm(mt)};
            } while (norm2(axis) > 1);
            double angle = ang(mt);
            r = rotation_axis_angle(vdiv(axis, std::sqrt(norm2(axis))), angle);
            m.type = 1;
        }
        std::uniform_int_distribution<std::size_t> pd(0, static_cast<std::size_t>(nidx) - 1);
        m.particle = static_cast<int32_t>(idxs[pd(mt)]);
        m.domain = domain;
        std::memcpy(m.translation, t.data(), sizeof(m.translation));
        std::memcpy(m.rotation, r.data(), sizeof(m.rotation));
        m.uniform = unit(mt);
    }
    return 0;
}

// FlipSampler::sampleMove (core/move_samplers/FlipSampler.cpp:18-41): a particle from the
// list, then a rotation by pi about its flip axis (the body-frame flip axis turned by its
// orientation and normalised); with a geometric origin away from zero the move is a
// rototranslation that keeps the origin in place.  `rot` holds every particle's orientation.
int rpo_draw_flips(void *rp, const double *rot, const double *flip_axis, const double *origin, const int64_t *idxs,
                   int64_t nidx, int64_t n, int32_t domain, rpo_move *out) {
    auto &mt = static_cast<rpo_rng *>(rp)->mt;
    if (nidx <= 0) return -1;
    const V3 fa{flip_axis[0], flip_axis[1], flip_axis[2]}, go{origin[0], origin[1], origin[2]};
    constexpr double EPS = 1e-14;
    const bool origin_zero = norm2(go) < EPS * EPS;
    std::uniform_real_distribution<double> unit;
    for (int64_t i = 0; i < n; i++) {
        std::uniform_int_distribution<std::size_t> pd(0, static_cast<std::size_t>(nidx) - 1);
        const int64_t pid = idxs[pd(mt)];
        const M3 o = load_m3(rot + 9 * pid);
        const V3 a = mv(o, fa);
        const M3 r = rotation_axis_angle(vdiv(a, std::sqrt(norm2(a))), M_PI);
        rpo_move &m = out[i];
        std::memset(&m, 0, sizeof(m));
        V3 t{};
        if (origin_zero) {
            m.type = 1;
        } else {
            m.type = 2;
            const V3 g = mv(o, go);
            const V3 rg = mv(r, g);
            t = {-rg[0] + g[0], -rg[1] + g[1], -rg[2] + g[2]};
        }
        m.particle = static_cast<int32_t>(pid);
        m.domain = domain;
        std::memcpy(m.translation, t.data(), sizeof(m.translation));
        std::memcpy(m.rotation, r.data(), sizeof(m.rotation));
        m.uniform = unit(mt);
    }
    return 0;
}

// ---- the cycle loop (CPU baseline and ensemble checks) ----
struct rpo_sim_params {
    double temperature, pressure, translation_step, rotation_step;
    int32_t box_kind, adjust_steps;
    double box_step;
    int64_t domains[3];
    uint64_t seed;
    int64_t threads;
};

struct rpo_sim_stats {
    int64_t moves[2], accepted[2];
    int64_t scalings, scalings_accepted, cycles;
    int64_t domains[3];
    double move_us, scaling_us, total_us;
    double steps[2];
    double box_step;
};

struct SimHandle {
    Handle *h;
    std::unique_ptr<Simulation> sim;
};

void *rpo_sim_create(void *hp, const rpo_sim_params *p) {
    auto *h = static_cast<Handle *>(hp);
    SimParams sp;
    sp.temperature = p->temperature;
    sp.pressure = p->pressure;
    sp.translation_step = p->translation_step;
    sp.rotation_step = p->rotation_step;
    sp.box_kind = p->box_kind;
    sp.box_step = p->box_step;
    for (int i = 0; i < 3; i++) sp.domains[i] = static_cast<std::size_t>(p->domains[i]);
    sp.seed = static_cast<unsigned long>(p->seed);
    sp.threads = static_cast<std::size_t>(p->threads);
    sp.adjust_steps = p->adjust_steps != 0;
    if (sp.domains[0] * sp.domains[1] * sp.domains[2] > h->pk->move_threads) return nullptr;
    auto *s = new SimHandle{h, std::make_unique<Simulation>(*h->pk, h->inter, sp)};
    return s;
}

void rpo_sim_destroy(void *sp) { delete static_cast<SimHandle *>(sp); }

int rpo_sim_run(void *sp, int64_t cycles, rpo_sim_stats *out) {
    auto *s = static_cast<SimHandle *>(sp);
    auto &sim = *s->sim;
    try {
        auto t0 = std::chrono::high_resolution_clock::now();
        for (int64_t c = 0; c < cycles; c++) sim.cycle();
        auto t1 = std::chrono::high_resolution_clock::now();
        sim.total_us += std::chrono::duration<double, std::micro>(t1 - t0).count();
    } catch (const std::exception &) {
        return -1;
    }
    if (out) {
        std::memset(out, 0, sizeof(*out));
        for (std::size_t i = 0; i < sim.samplers.size() && i < 2; i++) {
            out->moves[sim.samplers[i]] = static_cast<int64_t>(sim.counters[i].moves);
            out->accepted[sim.samplers[i]] = static_cast<int64_t>(sim.counters[i].accepted);
            out->steps[sim.samplers[i]] = sim.steps[i];
        }
        out->scalings = static_cast<int64_t>(sim.scaling.moves);
        out->scalings_accepted = static_cast<int64_t>(sim.scaling.accepted);
        out->cycles = static_cast<int64_t>(sim.cycles);
        for (int i = 0; i < 3; i++) out->domains[i] = static_cast<int64_t>(sim.p.domains[i]);
        out->move_us = sim.move_us;
        out->scaling_us = sim.scaling_us;
        out->total_us = sim.total_us;
        out->box_step = sim.p.box_step;
    }
    return 0;
}

// ---- pair correlations (core/observables/correlation/*) ----------------------------

// Same layout as rp_pair_desc in include/rampack_gb300.h.
struct rpo_pair_desc {
    int32_t enumerator;
    int32_t linear_axis;
    int32_t miller[3];
    int32_t function;
    int32_t axis;
    int32_t num_bins;
    int32_t flags;
    int32_t reserved;
    double max_r;
    double focal[3];
    double primary[3];
    double secondary[3];
};

static CorrSpec load_spec(const rpo_pair_desc *d) {
    CorrSpec s;
    s.enumerator = d->enumerator;
    s.linear_axis = d->linear_axis;
    for (int i = 0; i < 3; i++) {
        s.miller[i] = d->miller[i];
        s.focal[i] = d->focal[i];
        s.primary[i] = d->primary[i];
        s.secondary[i] = d->secondary[i];
    }
    s.function = d->function;
    s.axis = d->axis;
    s.num_bins = d->num_bins;
    s.max_r = d->max_r;
    return s;
}

static void load_state(int64_t n, const double *pos, const double *rot, std::vector<V3> &p, std::vector<M3> &r) {
    p.resize(n);
    r.resize(n);
    for (int64_t i = 0; i < n; i++) {
        p[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        r[i] = load_m3(rot + 9 * i);
    }
}

void *rpo_corr_create(const rpo_pair_desc *d) {
    if (!d || d->num_bins < 1 || !(d->max_r > 0)) return nullptr;
    return new Correlation(load_spec(d));
}
void rpo_corr_destroy(void *c) { delete static_cast<Correlation *>(c); }

int rpo_corr_add_snapshot(void *c, int64_t n, const double *pos, const double *rot, const double *box9) {
    std::vector<V3> p;
    std::vector<M3> r;
    load_state(n, pos, rot, p, r);
    try {
        static_cast<Correlation *>(c)->add_snapshot(p, r, Box(load_m3(box9)));
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}

// one consumePair with the correlation function's value given (the mocked enumerators and
// functions of the reference's unit tests), then renormalizeBins / nextSnapshot
void rpo_corr_consume(void *c, int64_t i, int64_t j, const double *d3, double value) {
    static_cast<Correlation *>(c)->consume(i, j, {d3[0], d3[1], d3[2]}, value);
}
void rpo_corr_renormalize(void *c, const double *factors) {
    auto *k = static_cast<Correlation *>(c);
    k->hist.renormalize(std::vector<double>(factors, factors + k->hist.bins));
}
void rpo_corr_next_snapshot(void *c) { static_cast<Correlation *>(c)->hist.next_snapshot(); }
void rpo_corr_dividers(void *c, double *out) {
    auto v = static_cast<Correlation *>(c)->hist.dividers();
    std::memcpy(out, v.data(), sizeof(double) * v.size());
}
void rpo_corr_dump(void *c, double *x, double *y, uint64_t *count) {
    auto *k = static_cast<Correlation *>(c);
    k->hist.dump(!k->density(), x, y, count);
}

// the pairs an enumerator produces (i, j, separation) for n focal points at the given
// positions (orientations apply the focal point); returns the number of pairs, writing at
// most `cap` of them
int64_t rpo_enumerate_pairs(const rpo_pair_desc *d, int64_t n, const double *pos, const double *rot,
                            const double *box9, int64_t cap, int64_t *ij, double *diff) {
    std::vector<V3> p;
    std::vector<M3> r;
    load_state(n, pos, rot, p, r);
    CorrSpec s = load_spec(d);
    int64_t k = 0;
    enumerate_pairs(s, Box(load_m3(box9)), focal_points(p, r, s.focal), [&](std::size_t i, std::size_t j, const V3 &v) {
        if (k < cap) {
            ij[2 * k] = static_cast<int64_t>(i);
            ij[2 * k + 1] = static_cast<int64_t>(j);
            for (int a = 0; a < 3; a++) diff[3 * k + a] = v[a];
        }
        k++;
    });
    return k;
}

// one snapshot's bin counts, rows shared among `threads` threads
void rpo_pair_counts(const rpo_pair_desc *d, int64_t n, const double *pos, const double *rot, const double *box9,
                     int threads, uint64_t *out) {
    std::vector<V3> p;
    std::vector<M3> r;
    load_state(n, pos, rot, p, r);
    CorrSpec s = load_spec(d);
    auto c = pair_counts(s, Box(load_m3(box9)), focal_points(p, r, s.focal), threads);
    std::memcpy(out, c.data(), sizeof(uint64_t) * c.size());
}

int rpo_expected_in_shells(const rpo_pair_desc *d, int64_t n, const double *box9, const double *bounds, int nb,
                           double *out) {
    auto v = expected_in_shells(load_spec(d), Box(load_m3(box9)), n, std::vector<double>(bounds, bounds + nb));
    std::memcpy(out, v.data(), sizeof(double) * v.size());
    return static_cast<int>(v.size());
}

double rpo_axis_function(int f, const double *a1, const double *a2, const double *d) {
    return axis_function(f, {a1[0], a1[1], a1[2]}, {a2[0], a2[1], a2[2]}, {d[0], d[1], d[2]});
}

}  // extern "C"
