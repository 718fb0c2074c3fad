// The Monte Carlo cycle loop around one packing on the GPU: Simulation::performCycle for
// hard bodies (core/Simulation.cpp:325-363) with the particle moves as one device sweep,
// box moves proposed by the reference's TriclinicBoxScaler family from a std::mt19937 and
// pre-checked on the host (Simulation::tryScaling, core/Simulation.cpp:493-531), and the
// thermalisation's step-size adaptation (Simulation::evaluateCounters,
// core/Simulation.cpp:533-607; TranslationSampler.cpp:48-59, RotationSampler.cpp:36-49,
// TriclinicBoxScaler.cpp:9-18).
//
// The box scalers restate core/volume_scalers/*.cpp draw for draw (libstdc++'s mt19937 and
// distributions, the same on every host this builds for), so one seed gives the reference's
// box proposals; rp_box_proposals exposes that sequence alone.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <string>

#include "rampack_gb300.h"
#include "rp_geom.cuh"

namespace rp {
bool handle_box(void *handle, double *box9);
bool handle_soft(void *handle);
bool handle_counting(void *handle);
int64_t handle_size(void *handle);
}  // namespace rp

namespace {

using rp::d3;

constexpr double PI = 3.14159265358979323846;  // M_PI

// TriclinicBox::getSides (core/TriclinicBox.cpp:27-33): the columns, each entry as
// dimensions · e_j accumulates it (0 + x turns -0 into +0)
void sides_of(const double *box, d3 s[3]) {
    for (int j = 0; j < 3; j++) s[j] = d3{box[j] + 0.0, box[3 + j] + 0.0, box[6 + j] + 0.0};
}

// TriclinicBox::getHeights (core/TriclinicBox.cpp:40-51)
void heights_of(const double *box, double h[3]) {
    d3 s[3];
    sides_of(box, s);
    const double vol = std::fabs(rp::dot3(rp::cross3(s[0], s[1]), s[2]));
    h[0] = vol / std::sqrt(rp::norm2(rp::cross3(s[1], s[2])));
    h[1] = vol / std::sqrt(rp::norm2(rp::cross3(s[2], s[0])));
    h[2] = vol / std::sqrt(rp::norm2(rp::cross3(s[0], s[1])));
}

double volume_of(const double *box) {
    d3 s[3];
    sides_of(box, s);
    return std::fabs(rp::dot3(rp::cross3(s[0], s[1]), s[2]));
}

bool valid_scaler(const rp_box_scaler_desc &d) {
    if (d.kind == RP_SCALER_NONE) return true;
    if (!(d.step > 0)) return false;
    if (d.kind == RP_SCALER_DELTA_TRICLINIC || d.kind == RP_SCALER_DELTA_VOLUME) return true;
    if (d.kind != RP_SCALER_LOG && d.kind != RP_SCALER_LINEAR) return false;
    if (d.num_groups < 1 || d.num_groups > 3) return false;
    for (int g = 0; g < d.num_groups; g++)
        if (d.groups[g] < 1 || d.groups[g] > 7) return false;
    return true;
}

// TriclinicBoxScaler::updateBox of the configured scaler, `step` its current step size.
void propose_box(const rp_box_scaler_desc &d, double step, const double *box, std::mt19937 &mt, double *out) {
    if (d.kind == RP_SCALER_DELTA_TRICLINIC) {
        // TriclinicDeltaScaler::updateBox (core/volume_scalers/TriclinicDeltaScaler.cpp:7-25)
        std::memcpy(out, box, 9 * sizeof(double));
        std::uniform_real_distribution<double> dist(-step, step);
        if (d.scale_together) {
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) out[3 * i + j] += dist(mt);
        } else {
            std::uniform_int_distribution<std::size_t> side_dist(0, 2);
            const std::size_t side = side_dist(mt);
            for (int i = 0; i < 3; i++) out[3 * i + side] += dist(mt);
        }
        return;
    }
    // TriclinicAdapter::updateBox (core/volume_scalers/TriclinicAdapter.h:27-33): the sides
    // times factors the VolumeScaler samples from the box heights
    double h[3];
    heights_of(box, h);
    double f[3] = {1, 1, 1};
    if (d.kind == RP_SCALER_DELTA_VOLUME) {
        // DeltaVolumeScaler::sampleScalingFactors (core/volume_scalers/DeltaVolumeScaler.cpp:10-19)
        std::uniform_real_distribution<double> unit(0, 1);
        const double dv = (2 * unit(mt) - 1) * step;
        const double cur = ((1. * h[0]) * h[1]) * h[2];
        const double fac = std::cbrt((dv + cur) / cur);
        f[0] = f[1] = f[2] = fac;
    } else {
        // AnisotropicVolumeScaler::sampleScalingFactors (AnisotropicVolumeScaler.cpp:12-30) over
        // LogScalingFactorSampler (LogScalingFactorSampler.cpp:8-19) or
        // LinearScalingFactorSampler (LinearScalingFactorSampler.cpp:9-24)
        auto sample = [&](int mask, double out3[3]) {
            std::uniform_real_distribution<double> dist(-step, step);
            const double x = dist(mt);
            for (int i = 0; i < 3; i++) out3[i] = 1;
            for (int i = 0; i < 3; i++) {
                if (!(mask & (1 << i))) continue;
                out3[i] = d.kind == RP_SCALER_LOG ? std::exp(x) : (h[i] + x) / h[i];
            }
        };
        if (d.independent && d.num_groups > 1) {
            std::uniform_int_distribution<std::size_t> pick(0, static_cast<std::size_t>(d.num_groups - 1));
            sample(d.groups[pick(mt)], f);
        } else {
            for (int g = 0; g < d.num_groups; g++) {
                double single[3];
                sample(d.groups[g], single);
                for (int i = 0; i < 3; i++) f[i] = f[i] * single[i];
            }
        }
    }
    d3 s[3];
    sides_of(box, s);
    for (int j = 0; j < 3; j++) {
        const d3 v{s[j].x * f[j], s[j].y * f[j], s[j].z * f[j]};
        out[j] = v.x;
        out[3 + j] = v.y;
        out[6 + j] = v.z;
    }
}

// Simulation::Counter (core/Simulation.cpp:609-640): totals and the moves since the last
// evaluation of the step sizes
struct Counter {
    uint64_t moves = 0, accepted = 0, since = 0, since_accepted = 0;
    void add(uint64_t m, uint64_t a) {
        moves += m;
        accepted += a;
        since += m;
        since_accepted += a;
    }
    double rate() const { return since == 0 ? 0.0 : static_cast<double>(since_accepted) / static_cast<double>(since); }
    void reset() { since = since_accepted = 0; }
};

struct Sim {
    void *h = nullptr;
    rp_sim_params p{};
    std::mt19937 mt;
    std::uniform_real_distribution<double> unit{0, 1};
    double tstep = 0, rstep = 0, bstep = 0, max_trans = 0;
    Counter trans, rot, box;
    uint64_t cycles = 0;
    uint64_t last_moves[3]{};  // device counters at the last read: translations, rotations, accepted translations
    uint64_t last_accepted = 0;
    double move_ms = 0, scaling_ms = 0;
    int64_t n = 0;
    std::string err;

    int fail(int code, const std::string &msg) {
        err = msg;
        return code;
    }
};

int sim_fail(Sim *s, int code, const char *what, void *handle) {
    return s->fail(code, std::string(what) + ": " + rp_last_error(handle));
}

// Simulation::tryScaling (core/Simulation.cpp:493-531): 1 accepted, 0 rejected, < 0 error
int try_scaling(Sim *s) {
    double oldb[9], newb[9];
    if (!rp::handle_box(s->h, oldb)) return s->fail(RP_ERR_STATE, "no state uploaded");
    propose_box(s->p.scaler, s->bstep, oldb, s->mt, newb);
    const double oldV = std::fabs(volume_of(oldb)), newV = std::fabs(volume_of(newb));
    if (newV == 0) return s->fail(RP_ERR_ARG, "a box proposal has zero volume");
    const double dV = newV - oldV, factor = newV / oldV;
    const double N = static_cast<double>(s->n);
    const double T = s->p.temperature, P = s->p.pressure;
    double dE = 0;
    if (rp::handle_counting(s->h) || rp::handle_soft(s->h)) {
        // overlaps counted or a soft part: the energy change is needed before the Metropolis test
        if (rp_try_scaling(s->h, newb, &dE) != RP_OK) return sim_fail(s, RP_ERR_DEVICE, "rp_try_scaling", s->h);
        const double ex = N * std::log(factor) - dE / T - P * dV / T;
        if (s->unit(s->mt) <= std::exp(ex)) return 1;
        if (rp_revert_scaling(s->h) != RP_OK) return sim_fail(s, RP_ERR_DEVICE, "rp_revert_scaling", s->h);
        return 0;
    }
    const double ex = N * std::log(factor) - P * dV / T;
    if (s->unit(s->mt) > std::exp(ex)) return 0;
    if (rp_try_scaling(s->h, newb, &dE) != RP_OK) return sim_fail(s, RP_ERR_DEVICE, "rp_try_scaling", s->h);
    if (dE > 0) {
        if (rp_revert_scaling(s->h) != RP_OK) return sim_fail(s, RP_ERR_DEVICE, "rp_revert_scaling", s->h);
        return 0;
    }
    return 1;
}

// Simulation::evaluateMoleculeMoveCounter / evaluateScalingMoveCounter
// (core/Simulation.cpp:533-607): a sampler is evaluated once 100·N of its moves were made
// since its last evaluation (N requested moves per cycle), the box scaler after 100 moves
void evaluate_counters(Sim *s) {
    const uint64_t requested = static_cast<uint64_t>(s->n);  // getNumOfRequestedMoves(N) = N
    if (s->p.rototranslation) {
        // RototranslationSampler::increaseStepSize / decreaseStepSize
        // (core/move_samplers/RototranslationSampler.cpp:50-61, :87-93)
        if (s->rot.since >= 100 * requested) {
            const double rate = s->rot.rate();
            s->rot.reset();
            if (rate > 0.2) {
                const double old = s->tstep;
                if (!(s->max_trans > 0 && s->tstep >= s->max_trans)) s->tstep *= 1.1;
                s->rstep *= s->tstep / old;
            } else if (rate < 0.1) {
                s->tstep /= 1.1;
                s->rstep /= 1.1;
            }
        }
    } else {
        if (s->p.translation_step > 0 && s->trans.since >= 100 * requested) {
            const double rate = s->trans.rate();
            s->trans.reset();
            if (rate > 0.2) {
                // TranslationSampler::increaseStepSize: refused at the implicit maximum
                if (!(s->max_trans > 0 && s->tstep >= s->max_trans)) s->tstep *= 1.1;
            } else if (rate < 0.1) {
                s->tstep /= 1.1;
            }
        }
        if (s->p.rotation_step > 0 && s->rot.since >= 100 * requested) {
            const double rate = s->rot.rate();
            s->rot.reset();
            if (rate > 0.2) {
                s->rstep *= 1.1;
                if (s->rstep > PI) s->rstep = PI;
            } else if (rate < 0.1) {
                s->rstep /= 1.1;
            }
        }
    }
    if (s->p.scaler.kind != RP_SCALER_NONE && s->box.since >= 100) {
        const double rate = s->box.rate();
        s->box.reset();
        if (rate > 0.2) s->bstep *= 1.1;
        else if (rate < 0.1) s->bstep /= 1.1;
    }
}

// the device's per-type counters since the last read
int read_moves(Sim *s) {
    rp_sweep_stats st{};
    if (rp_get_stats(s->h, &st) != RP_OK) return sim_fail(s, RP_ERR_DEVICE, "rp_get_stats", s->h);
    const uint64_t dt = st.translations - s->last_moves[0], dr = st.rotations - s->last_moves[1];
    const uint64_t dat = st.accepted_translations - s->last_moves[2];
    const uint64_t da = st.accepted - s->last_accepted;
    s->trans.add(dt, dat);
    s->rot.add(dr, da - dat);
    s->last_moves[0] = st.translations;
    s->last_moves[1] = st.rotations;
    s->last_moves[2] = st.accepted_translations;
    s->last_accepted = st.accepted;
    return RP_OK;
}

void fill_stats(const Sim *s, rp_sim_stats *o) {
    std::memset(o, 0, sizeof(*o));
    o->cycles = s->cycles;
    o->translations = s->trans.moves;
    o->accepted_translations = s->trans.accepted;
    o->rotations = s->rot.moves;
    o->accepted_rotations = s->rot.accepted;
    o->box_moves = s->box.moves;
    o->accepted_box_moves = s->box.accepted;
    o->translation_step = s->tstep;
    o->rotation_step = s->rstep;
    o->box_step = s->bstep;
    rp::handle_box(s->h, o->box);
    o->move_ms = s->move_ms;
    o->scaling_ms = s->scaling_ms;
}

}  // namespace

extern "C" {

int rp_box_proposals(const rp_box_scaler_desc *d, uint64_t seed, const double *box9, int64_t count, double *boxes,
                     double *uniforms) {
    if (!d || !box9 || count < 0 || (count > 0 && !boxes) || !valid_scaler(*d) || d->kind == RP_SCALER_NONE)
        return RP_ERR_ARG;
    std::mt19937 mt(static_cast<std::mt19937::result_type>(seed));
    std::uniform_real_distribution<double> unit(0, 1);
    for (int64_t k = 0; k < count; k++) {
        propose_box(*d, d->step, box9, mt, boxes + 9 * k);
        const double u = unit(mt);
        if (uniforms) uniforms[k] = u;
    }
    return RP_OK;
}

int rp_sim_create(void *handle, const rp_sim_params *p, void **sim) {
    if (!handle || !p || !sim) return RP_ERR_ARG;
    *sim = nullptr;
    double box[9];
    if (!rp::handle_box(handle, box)) return RP_ERR_STATE;
    if (!(p->temperature > 0) || !valid_scaler(p->scaler) || p->translation_step < 0 || p->rotation_step < 0 ||
        (p->translation_step == 0 && p->rotation_step == 0) ||
        (p->rototranslation && !(p->translation_step > 0 && p->rotation_step > 0)))
        return RP_ERR_ARG;
    Sim *s = new (std::nothrow) Sim();
    if (!s) return RP_ERR_ARG;
    s->h = handle;
    s->p = *p;
    s->mt.seed(static_cast<std::mt19937::result_type>(p->seed));
    s->tstep = p->translation_step;
    s->rstep = p->rotation_step;
    s->bstep = p->scaler.step;
    s->n = rp::handle_size(handle);
    rp_sweep_stats st{};
    if (rp_get_stats(handle, &st) != RP_OK) {
        delete s;
        return RP_ERR_DEVICE;
    }
    s->last_moves[0] = st.translations;
    s->last_moves[1] = st.rotations;
    s->last_moves[2] = st.accepted_translations;
    s->last_accepted = st.accepted;
    rp_set_temperature(handle, p->temperature);
    *sim = s;
    return RP_OK;
}

int rp_sim_run(void *sim, int64_t cycles, int adjust_steps, rp_sim_stats *stats) {
    Sim *s = static_cast<Sim *>(sim);
    if (!s || cycles < 0) return RP_ERR_ARG;
    for (int64_t c = 0; c < cycles; c++) {
        auto t0 = std::chrono::steady_clock::now();
        // TranslationSampler's implicit maximum: half the smallest box height
        double box[9], h[3];
        rp::handle_box(s->h, box);
        heights_of(box, h);
        s->max_trans = std::min(h[0], std::min(h[1], h[2])) / 2;
        rp_sweep_params sp{};
        sp.translation_step = s->tstep;
        sp.rotation_step = s->rstep;
        if (s->p.rototranslation) {
            // RototranslationSampler::sampleMove draws angles within min(step, pi)
            sp.rotation_step = std::min(s->rstep, PI);
            sp.flags |= RP_SWEEP_ROTOTRANSLATION;
        }
        sp.seed = s->p.seed;
        sp.counter = s->cycles;
        if (rp_sweep(s->h, &sp, nullptr) != RP_OK) return sim_fail(s, RP_ERR_DEVICE, "rp_sweep", s->h);
        auto t1 = std::chrono::steady_clock::now();
        s->move_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        if (s->p.scaler.kind != RP_SCALER_NONE) {
            const int ok = try_scaling(s);
            if (ok < 0) return ok;
            s->box.add(1, ok ? 1 : 0);
            s->scaling_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
        }
        if (adjust_steps) {
            int rc = read_moves(s);
            if (rc) return rc;
            evaluate_counters(s);
        }
        s->cycles++;
    }
    int rc = read_moves(s);
    if (rc) return rc;
    if (stats) fill_stats(s, stats);
    return RP_OK;
}

int rp_sim_get_stats(void *sim, rp_sim_stats *stats) {
    Sim *s = static_cast<Sim *>(sim);
    if (!s || !stats) return RP_ERR_ARG;
    int rc = read_moves(s);
    if (rc) return rc;
    fill_stats(s, stats);
    return RP_OK;
}

int rp_sim_set_steps(void *sim, double translation_step, double rotation_step, double box_step) {
    Sim *s = static_cast<Sim *>(sim);
    if (!s || translation_step < 0 || rotation_step < 0 || box_step < 0) return RP_ERR_ARG;
    if ((translation_step > 0) != (s->p.translation_step > 0) || (rotation_step > 0) != (s->p.rotation_step > 0))
        return RP_ERR_ARG;
    s->tstep = translation_step;
    s->rstep = rotation_step;
    if (s->p.scaler.kind != RP_SCALER_NONE && box_step > 0) s->bstep = box_step;
    return RP_OK;
}

int rp_sim_set_cycles(void *sim, uint64_t cycles) {
    Sim *s = static_cast<Sim *>(sim);
    if (!s) return RP_ERR_ARG;
    s->cycles = cycles;
    return RP_OK;
}

int rp_sim_set_conditions(void *sim, double temperature, double pressure) {
    Sim *s = static_cast<Sim *>(sim);
    if (!s || !(temperature > 0)) return RP_ERR_ARG;
    s->p.temperature = temperature;
    s->p.pressure = pressure;
    return rp_set_temperature(s->h, temperature);  // the sweeps' Metropolis test of soft energies
}

const char *rp_sim_last_error(void *sim) {
    Sim *s = static_cast<Sim *>(sim);
    return s ? s->err.c_str() : "null simulation";
}

int rp_sim_destroy(void *sim) {
    delete static_cast<Sim *>(sim);
    return RP_OK;
}

}  // extern "C"
