// ORACLE — test infrastructure only (see rpo_geometry.hpp).
//
// Pair correlations restated from core/observables/correlation/* and
// core/observables/HistogramBuilder.{h,tpp} / Histogram.tpp, single-threaded (the
// reference's PairConsumer default of one thread), so that the enumeration order and
// therefore every FP64 sum are the reference's own.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <vector>

#include "rpo_geometry.hpp"

namespace rpo {

enum { PAIRS_RADIAL = 0, PAIRS_LINEAR = 1, PAIRS_LAYERWISE = 2 };
enum { CORR_DENSITY = 0, CORR_S110 = 1, CORR_S220 = 2, CORR_S221 = 3, CORR_AXES_ANGLE = 4 };
enum { AXIS_PRIMARY = 0, AXIS_SECONDARY = 1, AXIS_AUXILIARY = 2 };

struct CorrSpec {
    int enumerator = PAIRS_RADIAL;
    int linear_axis = 0;       // LinearEnumerator::Axis X, Y, Z
    int miller[3] = {0, 0, 1};
    int function = CORR_DENSITY;
    int axis = AXIS_PRIMARY;   // ShapeGeometry::Axis of the axis correlations
    int num_bins = 1;
    double max_r = 1;
    V3 focal{};                // the named point in the body frame (ShapeGeometry::getNamedPoint)
    V3 primary{0, 0, 1};       // body-frame primary and secondary axes
    V3 secondary{1, 0, 0};
};

// geometry/Vector.h:225-228: v / |v| (Matrix.tpp:178-185 skips a divisor of exactly 1).
inline V3 normalized(const V3 &v) { return vdiv(v, std::sqrt(norm2(v))); }

// Packing::dumpNamedPoints (core/Packing.cpp:1144-1153): position + orientation * point.
inline std::vector<V3> focal_points(const std::vector<V3> &pos, const std::vector<M3> &rot, const V3 &point) {
    std::vector<V3> out(pos.size());
    for (std::size_t i = 0; i < pos.size(); i++) out[i] = add(pos[i], mv(rot[i], point));
    return out;
}

// The axis a correlation function reads (core/observables/correlation_functions/
// AxisCorrelation.cpp:9-27): orientation * body axis; the auxiliary axis is
// (primary ^ secondary).normalized() (core/ShapeGeometry.h:79-81).
inline V3 shape_axis(const CorrSpec &s, const M3 &rot) {
    if (s.axis == AXIS_PRIMARY) return mv(rot, s.primary);
    if (s.axis == AXIS_SECONDARY) return mv(rot, s.secondary);
    return normalized(cross(mv(rot, s.primary), mv(rot, s.secondary)));
}

// correlation_functions/S110Correlation.h, S220Correlation.h, S221Correlation.h, AxesAngle.h.
inline double axis_function(int f, const V3 &a1, const V3 &a2, const V3 &d) {
    switch (f) {
        case CORR_S110: return dot(a1, a2);
        case CORR_S220: return 1.5 * (std::pow(dot(a1, a2), 2) - 1. / 3);
        case CORR_S221: return dot(cross(a1, a2), normalized(d)) * dot(a1, a2);
        case CORR_AXES_ANGLE: return 180 * std::acos(std::abs(dot(a1, a2))) / M_PI;
    }
    throw std::runtime_error("unknown correlation function");
}

// LayerwiseRadialEnumerator::calculateK (LayerwiseRadialEnumerator.cpp:12-16):
// 2 pi (B^-1)^T h.
inline V3 layer_k(const Box &box, const int *miller) {
    V3 h{static_cast<double>(miller[0]), static_cast<double>(miller[1]), static_cast<double>(miller[2])};
    return vscale(mv(transpose(box.inv), h), 2 * M_PI);
}

// LayerwiseRadialEnumerator::calculateTauAngle (LayerwiseRadialEnumerator.cpp:48-57):
// arg of the sum of exp(i k.r) over the focal points in index order.
inline double layer_tau(const V3 &k, const std::vector<V3> &pts) {
    using namespace std::complex_literals;
    std::complex<double> tau{0};
    for (const auto &p : pts) tau = tau + std::exp(1i * dot(k, p));
    return std::arg(tau);
}

// The per-snapshot constants of the enumerators: the linear one's face normal
// (LinearEnumerator.cpp:45-56), the layerwise one's k, k/|k| and tau.
struct PairFrame {
    V3 dir{}, k{}, kn{};
    double tau = 0;
    PairFrame(const CorrSpec &s, const Box &box, const std::vector<V3> &pts) {
        if (s.enumerator == PAIRS_LINEAR) {
            auto sd = box.sides();
            const int a = s.linear_axis;
            dir = normalized(cross(sd[(a + 1) % 3], sd[(a + 2) % 3]));
        } else if (s.enumerator == PAIRS_LAYERWISE) {
            k = layer_k(box, s.miller);
            kn = normalized(k);
            tau = layer_tau(k, pts);
        }
    }
};

// The body of the three enumerators' pair loops (RadialEnumerator.cpp:19-25,
// LinearEnumerator.cpp:58-64, LayerwiseRadialEnumerator.cpp:31-43): the second point
// moved by the periodic translation, the separation projected as each enumerator does;
// false when the layerwise enumerator skips the pair.
inline bool pair_separation(const CorrSpec &s, const PairFrame &f, const Box &box, const V3 &p1, const V3 &q,
                            V3 &d) {
    V3 p2 = add(q, pbc_translation(box, p1, q));
    if (s.enumerator == PAIRS_LAYERWISE) {
        double l1 = std::round((dot(p1, f.k) - f.tau) / (2 * M_PI));
        double l2 = std::round((dot(p2, f.k) - f.tau) / (2 * M_PI));
        if (l1 != l2) return false;
    }
    d = sub(p2, p1);
    if (s.enumerator == PAIRS_LINEAR)
        d = vscale(f.dir, dot(d, f.dir));
    else if (s.enumerator == PAIRS_LAYERWISE)
        d = sub(d, vscale(f.kn, dot(d, f.kn)));
    return true;
}

// The enumerators' loops over every pair i <= j in index order.
inline void enumerate_pairs(const CorrSpec &s, const Box &box, const std::vector<V3> &pts,
                            const std::function<void(std::size_t, std::size_t, const V3 &)> &consume) {
    PairFrame f(s, box, pts);
    V3 d;
    for (std::size_t i = 0; i < pts.size(); i++)
        for (std::size_t j = i; j < pts.size(); j++)
            if (pair_separation(s, f, box, pts[i], pts[j], d)) consume(i, j, d);
}

// The bin counts of one snapshot (pairs i < j for the density correlation, i <= j for the
// averaged ones) with the rows shared among threads: counts do not depend on the order.
inline std::vector<uint64_t> pair_counts(const CorrSpec &s, const Box &box, const std::vector<V3> &pts,
                                         int threads) {
    PairFrame f(s, box, pts);
    const double step = s.max_r / static_cast<double>(s.num_bins);
    const std::size_t first = s.function == CORR_DENSITY ? 1 : 0;
    const int64_t n = static_cast<int64_t>(pts.size());
    std::vector<uint64_t> total(s.num_bins);
#pragma omp parallel num_threads(threads)
    {
        std::vector<uint64_t> mine(s.num_bins);
        V3 d;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; i++)
            for (std::size_t j = i + first; j < pts.size(); j++) {
                if (!pair_separation(s, f, box, pts[i], pts[j], d)) continue;
                double dist = std::sqrt(norm2(d));
                if (dist > s.max_r) continue;
                auto idx = static_cast<std::size_t>(std::floor(dist / step));
                if (idx >= static_cast<std::size_t>(s.num_bins)) idx = s.num_bins - 1;
                mine[idx]++;
            }
#pragma omp critical
        for (int b = 0; b < s.num_bins; b++) total[b] += mine[b];
    }
    return total;
}

// getExpectedNumOfMoleculesInShells of the three enumerators (RadialEnumerator.cpp:31-48,
// LinearEnumerator.cpp:18-35, LayerwiseRadialEnumerator.cpp:70-92).
inline std::vector<double> expected_in_shells(const CorrSpec &s, const Box &box, std::size_t n,
                                              const std::vector<double> &bounds) {
    const double rho = static_cast<double>(n) / box.volume();   // Packing::getNumberDensity
    std::vector<double> out;
    if (s.enumerator == PAIRS_LINEAR) {
        double volume = box.volume();
        double height = box.heights()[s.linear_axis];
        double area = volume / height;
        for (std::size_t i = 0; i + 1 < bounds.size(); i++) out.push_back((bounds[i + 1] - bounds[i]) * area * rho);
        return out;
    }
    std::vector<double> m;
    if (s.enumerator == PAIRS_RADIAL) {
        for (double r : bounds) m.push_back(4. / 3 * M_PI * r * r * r * rho);
    } else {
        V3 k = layer_k(box, s.miller);
        double layer = 2 * M_PI / std::sqrt(norm2(k));
        double area_density = rho * layer;
        for (double r : bounds) m.push_back(M_PI * r * r * area_density);
    }
    for (std::size_t i = 0; i + 1 < m.size(); i++) out.push_back(m[i + 1] - m[i]);
    return out;
}

// HistogramBuilder<1> (HistogramBuilder.tpp) with one thread, and the bin arithmetic of
// Histogram.tpp: step (max - min) / bins, index floor((x - min) / step) clamped to the
// last bin, dividers min (n - i)/n + max i/n, bin middles min + (i + 0.5) step.
struct Histogram1 {
    double min = 0, max = 1, step = 1;
    int bins = 1;
    std::vector<double> value, cur_value;
    std::vector<uint64_t> count, cur_count;
    int64_t snapshots = 0;

    Histogram1(double mn, double mx, int nb)
            : min{mn}, max{mx}, step{(mx - mn) / static_cast<double>(nb)}, bins{nb}, value(nb), cur_value(nb),
              count(nb), cur_count(nb) {}
    void add(double x, double v) {
        auto idx = static_cast<std::size_t>(std::floor((x - min) / step));
        if (idx >= static_cast<std::size_t>(bins)) idx = bins - 1;
        cur_value[idx] += v;
        cur_count[idx]++;
    }
    std::vector<double> dividers() const {
        std::vector<double> r(bins + 1);
        double nd = static_cast<double>(bins);
        for (int i = 0; i <= bins; i++) {
            double id = static_cast<double>(i);
            r[i] = min * ((nd - id) / nd) + max * (id / nd);
        }
        return r;
    }
    void renormalize(const std::vector<double> &f) {
        for (int i = 0; i < bins; i++) cur_value[i] *= f[i];
    }
    void next_snapshot() {
        for (int i = 0; i < bins; i++) {
            value[i] += cur_value[i];
            count[i] += cur_count[i];
            cur_value[i] = 0;
            cur_count[i] = 0;
        }
        snapshots++;
    }
    // dumpValues: SUM divides the values by the number of snapshots, AVERAGE each value by
    // its bin's count; counts are kept.  No snapshots: the initial (zero) histogram.
    void dump(bool average, double *x, double *y, uint64_t *c) const {
        for (int i = 0; i < bins; i++) {
            x[i] = min + (static_cast<double>(i) + 0.5) * step;
            if (snapshots == 0) {
                y[i] = 0;
                c[i] = 0;
                continue;
            }
            y[i] = average ? value[i] / static_cast<double>(count[i]) : value[i] / static_cast<double>(snapshots);
            c[i] = count[i];
        }
    }
};

// PairDensityCorrelation (function CORR_DENSITY, PairDensityCorrelation.cpp:4-37) or
// PairAveragedCorrelation with an axis function (PairAveragedCorrelation.cpp:4-31).
struct Correlation {
    CorrSpec spec;
    Histogram1 hist;

    explicit Correlation(const CorrSpec &s) : spec{s}, hist(0, s.max_r, s.num_bins) {}

    bool density() const { return spec.function == CORR_DENSITY; }

    // consumePair with the correlation function's value already evaluated
    void consume(std::size_t i, std::size_t j, const V3 &d, double value) {
        if (density() && i == j) return;
        double dist = std::sqrt(norm2(d));
        if (dist > hist.max) return;
        hist.add(dist, density() ? 1 : value);
    }

    void add_snapshot(const std::vector<V3> &pos, const std::vector<M3> &rot, const Box &box) {
        auto pts = focal_points(pos, rot, spec.focal);
        std::vector<V3> axes;
        if (!density())
            for (const auto &r : rot) axes.push_back(shape_axis(spec, r));
        enumerate_pairs(spec, box, pts, [&](std::size_t i, std::size_t j, const V3 &d) {
            consume(i, j, d, density() ? 0 : axis_function(spec.function, axes[i], axes[j], d));
        });
        if (density()) {
            auto f = expected_in_shells(spec, box, pos.size(), hist.dividers());
            for (auto &x : f) x = 2. / x / static_cast<double>(pos.size());
            hist.renormalize(f);
        }
        hist.next_snapshot();
    }
};

}  // namespace rpo
