// ORACLE — test infrastructure only (see rpo_geometry.hpp).
//
// Restatement of the reference's Monte Carlo driver for hard bodies: move samplers
// (core/move_samplers/TranslationSampler.cpp, RotationSampler.cpp), box scalers
// (core/volume_scalers/TriclinicDeltaScaler.cpp, TriclinicAdapter.h +
// AnisotropicVolumeScaler.cpp + LogScalingFactorSampler.cpp), spatial domain
// decomposition (core/DomainDecomposition.cpp, ActiveDomain.cpp) and the cycle loop
// (core/Simulation.cpp:325-607).  Used as the timed CPU baseline ("port") when the
// reference itself cannot be built, and to check ensemble averages.
#pragma once

#include <chrono>
#include <random>

#include "rpo_packing.hpp"

namespace rpo {

struct TooNarrowDomain {
    std::size_t coord;
};

// core/DomainDecomposition.cpp:36-117
class DomainDecomposition {
public:
    std::array<std::size_t, 3> dd{};
    std::array<std::vector<std::array<double, 2>>, 3> bounds;  // {beg, end} per domain
    std::vector<std::vector<std::size_t>> particles;

    static double fit(double x) { return x < 0 ? x + 1 : (x >= 1 ? x - 1 : x); }

    DomainDecomposition(const Packing &pk, const Interaction &inter, const std::array<std::size_t, 3> &dd_,
                        const std::array<std::size_t, 3> &ngdiv, const V3 &origin)
        : dd{dd_} {
        const Box &box = pk.box;
        double range = inter.range(), total = inter.total_range();
        V3 h = box.heights();
        V3 orel = box.abs_to_rel(origin);
        for (int c = 0; c < 3; c++) {
            if (dd[c] < 2) continue;
            double cell = h[c] / ngdiv[c];
            double whole = 1. / dd[c];
            double ghost = (total - range + cell) / h[c];
            double cellrel = 1. / ngdiv[c];
            if (whole - ghost <= cellrel) throw TooNarrowDomain{static_cast<std::size_t>(c)};
            bounds[c].assign(dd[c], {0, 0});
            double prev_end = -std::numeric_limits<double>::infinity();
            for (std::size_t d = 0; d < dd[c]; d++) {
                double theo = orel[c] + d * whole;
                double mid = (std::round(theo * ngdiv[c] - 0.5) + 0.5) / ngdiv[c];
                std::size_t prev = (d + dd[c] - 1) % dd[c];
                double &gbeg = bounds[c][prev][1];
                double &gend = bounds[c][d][0];
                gbeg = mid - ghost / 2;
                gend = mid + ghost / 2;
                if (!(gbeg > prev_end)) throw std::runtime_error("malformed domain");
                prev_end = gend;
                gbeg = fit(gbeg);
                gend = fit(gend);
            }
        }
        std::size_t nd = dd[0] * dd[1] * dd[2];
        particles.assign(nd, {});
        std::size_t n = pk.size();
        std::vector<std::size_t> dom(n);
        const std::size_t GHOST = std::numeric_limits<std::size_t>::max();
        #pragma omp parallel for num_threads(nd)
        for (std::size_t i = 0; i < n; i++) {
            V3 r = box.abs_to_rel(pk.shapes[i].pos);
            std::array<std::size_t, 3> co{};
            for (int k = 0; k < 3; k++) {
                int c = std::floor((r[k] - orel[k]) * dd[k]);
                co[k] = (c + dd[k]) % dd[k];
            }
            dom[i] = in_region(r, co) ? idx(co) : GHOST;
        }
        for (std::size_t i = 0; i < n; i++)
            if (dom[i] != GHOST) particles[dom[i]].push_back(i);
    }
    std::size_t idx(const std::array<std::size_t, 3> &c) const {
        std::size_t r = 0;
        for (int i = 0; i < 3; i++) r = dd[i] * r + c[i];
        return r;
    }
    bool in_region(const V3 &v, const std::array<std::size_t, 3> &c) const {
        for (int i = 0; i < 3; i++) {
            if (dd[i] < 2) continue;
            double b = bounds[i][c[i]][0], e = bounds[i][c[i]][1];
            if (b < e) {
                if (v[i] <= b || v[i] >= e) return false;
            } else {
                if (v[i] <= b && v[i] >= e) return false;
            }
        }
        return true;
    }
    // DomainDecomposition.cpp:163-177
    void active_bounds(const std::array<std::size_t, 3> &c, double *lo, double *hi) const {
        for (int i = 0; i < 3; i++) {
            if (dd[i] < 2) {
                lo[i] = -std::numeric_limits<double>::infinity();
                hi[i] = std::numeric_limits<double>::infinity();
            } else {
                lo[i] = bounds[i][c[i]][0];
                hi[i] = bounds[i][c[i]][1];
            }
        }
    }
};

struct Counter {
    std::size_t moves = 0, accepted = 0, since = 0, acc_since = 0;
    void inc(bool a) { moves++; since++; if (a) { accepted++; acc_since++; } }
    double current_rate() const { return static_cast<double>(acc_since) / static_cast<double>(since); }
    void reset_current() { since = 0; acc_since = 0; }
    Counter &operator+=(const Counter &o) {
        moves += o.moves; accepted += o.accepted; since += o.since; acc_since += o.acc_since;
        return *this;
    }
};

// A proposed particle move, as MoveSampler::MoveData (core/MoveSampler.h:40-49).
struct Move {
    int type = 0;
    std::size_t idx = 0;
    V3 t{};
    M3 r = identity();
};

struct SimParams {
    double temperature = 1, pressure = 1;
    double translation_step = 0;   // 0 disables the translation sampler
    double rotation_step = 0;      // 0 disables the rotation sampler
    int box_kind = 0;              // 0 none, 1 delta_triclinic(scale together), 2 isotropic log, 3 delta volume
    double box_step = 0;
    std::array<std::size_t, 3> domains{1, 1, 1};
    unsigned long seed = 1234;
    std::size_t threads = 1;
    bool adjust_steps = false;     // thermalisation-phase step-size adaptation
};

class Simulation {
public:
    Packing &pk;
    const Interaction &inter;
    SimParams p;
    std::vector<std::mt19937> mts;
    std::vector<int> samplers;        // 0 translation, 1 rotation
    std::vector<double> steps;
    std::vector<double> max_trans;    // TranslationSampler implicit max step
    std::vector<Counter> counters;
    Counter scaling;
    double move_us = 0, scaling_us = 0, total_us = 0;
    std::size_t cycles = 0;
    std::uniform_real_distribution<double> unit;

    Simulation(Packing &pk_, const Interaction &in, const SimParams &p_) : pk{pk_}, inter{in}, p{p_} {
        std::size_t nd = p.domains[0] * p.domains[1] * p.domains[2];
        for (std::size_t i = 0; i < nd; i++) mts.emplace_back(p.seed + i);
        if (p.translation_step > 0) { samplers.push_back(0); steps.push_back(p.translation_step); }
        if (p.rotation_step > 0) { samplers.push_back(1); steps.push_back(p.rotation_step); }
        max_trans.assign(samplers.size(), 0);
        counters.assign(samplers.size(), {});
    }

    std::vector<std::size_t> accumulations(std::size_t n) const {
        std::vector<std::size_t> acc;
        std::size_t a = 0;
        for (std::size_t i = 0; i < samplers.size(); i++) { a += n; acc.push_back(a); }
        return acc;
    }

    // TranslationSampler.cpp:20-37, RotationSampler.cpp:13-34
    Move sample(std::size_t s, const std::vector<std::size_t> &idxs, std::mt19937 &mt) {
        using URD = std::uniform_real_distribution<double>;
        Move m;
        if (samplers[s] == 0) {
            m.type = 0;
            V3 h = pk.box.heights();
            max_trans[s] = std::min({h[0], h[1], h[2]}) / 2;
            double a = std::min(max_trans[s], steps[s]);
            URD d(-a, a);
            m.t = {d(mt), d(mt), d(mt)};
        } else {
            m.type = 1;
            URD ang(-steps[s], steps[s]);
            URD pm(-1, 1);
            V3 axis;
            do {
                axis = {pm(mt), pm(mt), pm(mt)};
            } while (norm2(axis) > 1);
            double angle = ang(mt);
            m.r = rotation_axis_angle(vdiv(axis, std::sqrt(norm2(axis))), angle);
        }
        std::uniform_int_distribution<std::size_t> pd(0, idxs.size() - 1);
        m.idx = idxs[pd(mt)];
        return m;
    }

    // Simulation.cpp:447-491 (move types: translation -> tryTranslation, rotation ->
    // tryRotation; acceptance always via acceptMove).
    bool try_move(const std::vector<std::size_t> &idxs, std::vector<Counter> &cnt,
                  const std::vector<std::size_t> &acc, const double *lo, const double *hi) {
        auto &mt = mts[RPO_TID];
        std::uniform_int_distribution<std::size_t> md(0, acc.back() - 1);
        std::size_t sampled = md(mt);
        std::size_t type = 0;
        for (auto a : acc) {
            if (sampled < a) break;
            type++;
        }
        Move m = sample(type, idxs, mt);
        double dE = pk.try_move(m.type, m.idx, m.t, m.r, inter, m.type == 0 ? lo : nullptr, hi);
        if (unit(mt) <= std::exp(-dE / p.temperature)) {
            pk.accept(2);
            cnt[type].inc(true);
            return true;
        }
        cnt[type].inc(false);
        return false;
    }

    std::vector<std::size_t> all_idx() const {
        std::vector<std::size_t> v(pk.size());
        std::iota(v.begin(), v.end(), 0);
        return v;
    }

    // Simulation.cpp:365-445
    void perform_moves() {
        std::size_t nd = p.domains[0] * p.domains[1] * p.domains[2];
        while (true) {
            try {
                if (nd == 1) {
                    auto acc = accumulations(pk.size());
                    auto idxs = all_idx();
                    for (std::size_t i = 0; i < acc.back(); i++) try_move(idxs, counters, acc, nullptr, nullptr);
                } else {
                    moves_dd();
                }
                break;
            } catch (const TooNarrowDomain &ex) {
                p.domains[ex.coord]--;
                nd = p.domains[0] * p.domains[1] * p.domains[2];
            }
        }
    }

    void moves_dd() {
        auto &mt = mts[0];
        V3 origin{unit(mt), unit(mt), unit(mt)};
        origin = pk.box.rel_to_abs(origin);
        if (!pk.ng.has_value()) throw std::runtime_error("domain decomposition needs a neighbour grid");
        DomainDecomposition dd(pk, inter, p.domains, pk.ng->real_divisions(), origin);
        std::size_t nd = p.domains[0] * p.domains[1] * p.domains[2];
        std::vector<std::vector<Counter>> tcnt(nd, std::vector<Counter>(counters.size()));
        #pragma omp parallel for collapse(3) num_threads(pk.move_threads)
        for (std::size_t i = 0; i < p.domains[0]; i++)
            for (std::size_t j = 0; j < p.domains[1]; j++)
                for (std::size_t k = 0; k < p.domains[2]; k++) {
                    std::array<std::size_t, 3> c{i, j, k};
                    const auto &idxs = dd.particles[dd.idx(c)];
                    double lo[3], hi[3];
                    dd.active_bounds(c, lo, hi);
                    if (idxs.empty()) continue;
                    auto acc = accumulations(pk.size() / nd);
                    for (std::size_t x = 0; x < acc.back(); x++) try_move(idxs, tcnt[RPO_TID % nd], acc, lo, hi);
                }
        for (auto &tc : tcnt)
            for (std::size_t s = 0; s < counters.size(); s++) counters[s] += tc[s];
    }

    // TriclinicDeltaScaler.cpp:7-25 (scale together) and TriclinicAdapter.h:27-33 with an
    // isotropic AnisotropicVolumeScaler over LogScalingFactorSampler.
    Box propose_box(std::mt19937 &mt) {
        const Box &ob = pk.box;
        if (p.box_kind == 1) {
            M3 d = ob.dim;
            std::uniform_real_distribution<double> sd(-p.box_step, p.box_step);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) d[3 * i + j] += sd(mt);
            return Box(d);
        }
        if (p.box_kind == 3) {
            // DeltaVolumeScaler.cpp:10-19 through TriclinicAdapter.h:27-33: dV uniform in
            // +-step, every side times cbrt((dV + V) / V) with V the product of the heights
            std::uniform_real_distribution<double> u01(0, 1);
            double dv = (2 * u01(mt) - 1) * p.box_step;
            V3 h = ob.heights();
            double cur = 1.;
            for (int i = 0; i < 3; i++) cur *= h[i];
            double f3 = std::cbrt((dv + cur) / cur);
            auto s3 = ob.sides();
            for (int i = 0; i < 3; i++) s3[i] = vscale(s3[i], f3);
            M3 d3m{};
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) d3m[3 * i + j] = s3[j][i];
            return Box(d3m);
        }
        std::uniform_real_distribution<double> ld(-p.box_step, p.box_step);
        double f = std::exp(ld(mt));
        V3 factors{1, 1, 1};
        V3 single{f, f, f};
        for (int i = 0; i < 3; i++) factors[i] = factors[i] * single[i];
        auto s = ob.sides();
        for (int i = 0; i < 3; i++) s[i] = vscale(s[i], factors[i]);
        M3 d{};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) d[3 * i + j] = s[j][i];
        return Box(d);
    }

    // Simulation.cpp:493-531
    bool try_scaling() {
        auto &mt = mts.front();
        Box nb = propose_box(mt);
        double oldV = std::abs(pk.box.volume()), newV = std::abs(nb.volume());
        double dV = newV - oldV, factor = newV / oldV;
        double N = static_cast<double>(pk.size());
        if (inter.soft || pk.counting) {
            // a nontrivial energy change (soft part, or counted overlaps): scaling tried first
            double dE = pk.try_scaling(nb, inter);
            double exponent = N * std::log(factor) - dE / p.temperature - p.pressure * dV / p.temperature;
            if (unit(mt) <= std::exp(exponent)) return true;
            pk.revert_scaling();
            return false;
        }
        double expo = N * std::log(factor) - p.pressure * dV / p.temperature;
        if (unit(mt) > std::exp(expo)) return false;
        if (pk.try_scaling(nb, inter) > 0) {
            pk.revert_scaling();
            return false;
        }
        return true;
    }

    void evaluate_counters() {
        for (std::size_t i = 0; i < samplers.size(); i++) {
            auto &c = counters[i];
            if (c.since < 100 * pk.size()) continue;
            double rate = c.current_rate();
            c.reset_current();
            if (rate > 0.2) {
                if (samplers[i] == 0) {
                    if (!(max_trans[i] > 0 && steps[i] >= max_trans[i])) steps[i] *= 1.1;
                } else {
                    steps[i] *= 1.1;
                    if (steps[i] > M_PI) steps[i] = M_PI;
                }
            } else if (rate < 0.1) {
                steps[i] /= 1.1;
            }
        }
        if (p.box_kind != 0 && scaling.since >= 100) {
            double rate = scaling.current_rate();
            scaling.reset_current();
            if (rate > 0.2) p.box_step *= 1.1;
            else if (rate < 0.1) p.box_step /= 1.1;
        }
    }

    // Simulation.cpp:325-363
    void cycle() {
        auto t0 = std::chrono::high_resolution_clock::now();
        perform_moves();
        auto t1 = std::chrono::high_resolution_clock::now();
        move_us += std::chrono::duration<double, std::micro>(t1 - t0).count();
        if (p.box_kind != 0) {
            bool ok = try_scaling();
            scaling.inc(ok);
            auto t2 = std::chrono::high_resolution_clock::now();
            scaling_us += std::chrono::duration<double, std::micro>(t2 - t1).count();
        }
        if (p.adjust_steps) evaluate_counters();
        cycles++;
    }
};

}  // namespace rpo
