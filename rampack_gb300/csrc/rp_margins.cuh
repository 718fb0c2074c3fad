// FP32 filter margins of sphere and spherocylinder pair tests (host code).
//
// One definition for every entry point that decides pairs in FP32 over a cell grid: the
// handle's sweeps, recounts and box moves (dev_state in rp_api.cu) and the allocation-free
// count (rp_static.cu).  A pair is decided in FP32 only when its FP32 value clears a margin
// that bounds the FP32 error; otherwise it is re-decided in FP64 with the reference's
// arithmetic (SphereTraits.cpp:56-65, SpherocylinderTraits.cpp:28-46).
#pragma once

#include <algorithm>
#include <cmath>

#include "rp_internal.cuh"

namespace rp {

// Thresholds for a sphere (kind RP_SHAPE_SPHERE, radius r) or spherocylinder (radius r,
// cylinder length l) whose FP32 coordinates are cell-local: lrow is the largest row norm of
// the cell matrix (box / dims), box the row-major box.  Polysphere thresholds depend on the
// centres and are formed by the caller.
inline FilterConsts hard_filter_consts(int kind, double r, double l, double lrow, const double *box) {
    const double u32 = std::ldexp(1.0, -24);
    // Per-component bound of the FP32 separation error, in units of u32 times the largest
    // cell-local coordinate L: candidate coordinates (rebuild 4, mirror updates
    // MIRROR_ROUNDINGS, offset 3, staging 2), the difference (3) and the mover (4 + its
    // mirror updates + the translation 1) sum to 25; 32 covers them.  A freshly rebuilt
    // grid (a recount with no sweep since) has fewer roundings and is covered too.
    const double e_sep = 32.0 * u32 * (lrow + 1.0);
    // FP32 axes: the FP64 axis rounded (1), a rotated mover's FP32 product (<= 6)
    const double e_axis = 8.0 * u32;
    const double safety = 2.0;
    FilterConsts fc{};
    // bound on |d2_32 - d2| at a threshold thr = d^2: 2 d |delta| + |delta|^2 with
    // |delta| <= sqrt(3) e_sep, plus the FP32 evaluation of the squared norm (3 roundings)
    auto margin = [&](double thr) {
        double d = std::sqrt(thr);
        return safety * (2.0 * d * std::sqrt(3.0) * e_sep + 3.0 * e_sep * e_sep + 4.0 * u32 * thr);
    };
    if (kind == RP_SHAPE_SPHERE) {
        double thr = std::pow(2 * r, 2);
        fc.sphere_lo = static_cast<float>(thr - margin(thr));
        fc.sphere_hi = static_cast<float>(thr + margin(thr));
    } else if (kind == RP_SHAPE_SPHEROCYLINDER) {
        double core = 4 * r * r, far = std::pow(2 * r + l, 2);
        fc.core_lo = static_cast<float>(core - margin(core));
        fc.core_hi = static_cast<float>(core + margin(core));
        fc.far_lo = static_cast<float>(far - margin(far));
        fc.far_hi = static_cast<float>(far + margin(far));
        fc.core_thr = static_cast<float>(core);
        // Segment certificate.  Input errors move each cap by at most dend, which changes
        // the segment distance d by at most 2 dend; near the threshold (d ~ 2r; farther away
        // the decision has a margin larger than any of these terms) that is
        // 2 (2r)(2 dend) + (2 dend)^2 in d^2.  FP32 evaluation of dP = w + s u - t v
        // (|w| <= 2r + 2l, |u| = |v| = l) errs by at most 4 u32 sqrt(3) (|w| + 2 l) per
        // vector, giving 2 (1.1 * 2r) ddp + ddp^2 in f; the gap G adds 4 u32 (2r) l.
        double dend = std::sqrt(3.0) * (e_sep + l * e_axis);
        double ddp = 4.0 * u32 * std::sqrt(3.0) * (2 * r + 4 * l);
        double eval = 2.0 * 1.1 * (2 * r) * ddp + ddp * ddp + 4.0 * u32 * (2 * r) * l;
        // FP64 evaluates the distance at its own closest-point parameters, with its own
        // inputs; rounding in sN = b e - c d and D = a c - b^2 (|b|, |c| <= l^2,
        // |d|, |e| <= l (2r + 2l)) moves the parameters by at most noise / D, which raises
        // its distance^2 above the minimum by at most g64 = 2 (2r) l sqrt(2) noise / D.
        // Pairs whose (cancellation-free) D is below d_min are re-decided in FP64; g64 at
        // d_min joins the certificate's margin.
        double pmax = 0;
        for (int i = 0; i < 3; i++)
            pmax = std::max(pmax, std::fabs(box[3 * i]) + std::fabs(box[3 * i + 1]) + std::fabs(box[3 * i + 2]));
        const double u64 = std::ldexp(1.0, -52);
        const double noise = 8.0 * u64 * 2.0 * l * l * l * (2 * r + 2 * l);
        const double g64 = 2e-6;
        fc.d_min = static_cast<float>(std::max(4.0 * (2 * r) * l * std::sqrt(2.0) * noise / g64 * 10.0,
                                               1e-9 * l * l * l * l));
        fc.seg_err = static_cast<float>(safety * (2.0 * (2 * r) * 2.0 * dend + 4.0 * dend * dend + eval) + g64);
        // Parallel branch (SegmentDistanceCalculator.h:35-39, taken when FP64's D < 1e-10):
        // FP64's D = l^4 sin^2(theta) up to ~4 ulp(l^4), so sin(theta) < theta_lim keeps it
        // there; FP32 axes add up to ~4 * 2^-24 to the angle.  The branch evaluates the
        // distance from the s = 0 end, at most 2 (2r) l sin(theta) above the minimum.
        const double d_noise = 16.0 * l * l * l * u64 * (pmax + l);  // FP64 rounding in its D
        const double theta_lim = std::sqrt(std::max(0.0, 0.8e-10 - d_noise)) / (l * l) - 8.0 * u32;
        if (l > 0 && theta_lim > 0) {
            fc.d_par = static_cast<float>(l * l * l * l * theta_lim * theta_lim * 0.5);
            fc.par_err = static_cast<float>(4.0 * (2 * r + 1e-3) * l * (theta_lim + 8.0 * u32) + 1e-6);
        } else {
            fc.d_par = 0.0f;
            fc.par_err = 0.0f;
        }
        fc.len = static_cast<float>(l);
        fc.half_len = static_cast<float>(0.5 * l);
    }
    fc.cell_margin = 1e-5f;
    return fc;
}

}  // namespace rp
