// Orientation renormalisation (Packing::renormalizeOrientations, core/Packing.cpp:1178-1212,
// with tryOrientationFix, :1221-1240): every particle, in index order, tries its
// Newton-Schulz-fixed orientation as a rotation move and keeps it when the fixed body
// overlaps nothing.
//
// The serial order matters only through neighbours: particle i sees neighbours j < i in
// their final state and j > i as they were.  The device first computes every fixed state,
// then tests all particles at once assuming every earlier neighbour accepted its fix.  If
// none is rejected that assumption held for every particle and the outcome is the serial
// one.  Otherwise the fixes before the first rejected index stand (they saw exactly the
// serial states) and one warp finishes the rest in index order.  The tests are the
// reference's FP64 arithmetic throughout (no FP32 filter: the pass is rare).
#include <cuda_runtime.h>

#include "rp_internal.cuh"

namespace rp {

namespace {

__device__ __forceinline__ d3 ld3(const double *p) { return d3{p[0], p[1], p[2]}; }

// Fixed orientation, rotated centres (afresh from the body frame, as tryOrientationFix
// does) and absolute centres of every particle.
__global__ void k_fix_prepare(DevState s, const double *cbody, double *rotfix, double *cenfix, double *absfix) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    double r[9];
    for (int k = 0; k < 9; k++) r[k] = s.rot64[9 * i + k];
    fix_rotation(r);
    for (int k = 0; k < 9; k++) rotfix[9 * i + k] = r[k];
    if (s.ncen > 0) {
        d3 p = ld3(s.pos64 + 3 * i);
        for (int b = 0; b < s.ncen; b++) {
            d3 c = mv3(r, ld3(cbody + 3 * b));
            d3 q = add3(p, c);
            d3 a = add3(q, pbc_correction(s.box, s.inv, q, nullptr));
            const size_t ci = 3 * ((size_t)i * s.ncen + b);
            cenfix[ci] = c.x;
            cenfix[ci + 1] = c.y;
            cenfix[ci + 2] = c.z;
            absfix[ci] = a.x;
            absfix[ci + 1] = a.y;
            absfix[ci + 2] = a.z;
        }
    }
}

// Rotated centres afresh from the body frame (Packing::setupForInteraction after a reset,
// core/Packing.cpp:940-944).
__global__ void k_fresh_centres(DevState s, const double *cbody) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= s.n * s.ncen) return;
    const int64_t i = t / s.ncen;
    const int b = (int)(t % s.ncen);
    d3 c = mv3(s.rot64 + 9 * i, ld3(cbody + 3 * b));
    s.cen64[3 * t] = c.x;
    s.cen64[3 * t + 1] = c.y;
    s.cen64[3 * t + 2] = c.z;
}

struct Version {
    const double *rot, *abs;  // orientations [n][9], absolute centres [n][ncen][3]
};

// Does particle i, at its position with orientation ri (absolute centres ai), overlap
// particle j in state v?  The image is the nearest one (core/PeriodicBoundaryConditions.cpp:24-36),
// the only one within range for the boxes the neighbour grid accepts.
__device__ __forceinline__ bool overlaps_pair(const DevState &s, d3 pi, const double *ri, const double *ai, int64_t j,
                                              const Version &v) {
    d3 pj = ld3(s.pos64 + 3 * j);
    if (s.kind == 3) {
        // generic convex bodies: XenoCollideTraits::overlapBetween (core/shapes/XenoCollideTraits.h:147-168)
        bool stuck = false;
        const bool ov = xc_overlap_filtered(*s.xc, pi, ri, add3(pj, pbc_translation(s.box, s.inv, pi, pj)),
                                            v.rot + 9 * j, stuck);
        if (stuck) atomicOr(s.status, ST_PORTAL_STUCK);
        return ov;
    }
    if (s.ncen == 0 && s.kind == 0 && s.pbc_fold) return pbc_distance2(s.box, s.inv, pi, pj) < s.ex.sphere_thr;
    if (s.ncen == 0) {
        d3 t = pbc_translation(s.box, s.inv, pi, pj);
        const double *rj = v.rot + 9 * j;
        return exact_overlap(s.ex, pi, d3{ri[2], ri[5], ri[8]}, pj, d3{rj[2], rj[5], rj[8]}, t);
    }
    for (int a = 0; a < s.ncen; a++) {
        d3 pa = ld3(ai + 3 * a);
        d3 ha{0.0, 0.0, 0.0};
        if (s.segs) ha = mv3(ri, d3{s.chax[a][0], s.chax[a][1], s.chax[a][2]});
        for (int b = 0; b < s.ncen; b++) {
            d3 pb = ld3(v.abs + 3 * ((size_t)j * s.ncen + b));
            if (s.segs) {
                // PolyspherocylinderTraits::overlapBetween (PolyspherocylinderTraits.cpp:102-124)
                d3 q = add3(pb, pbc_translation(s.box, s.inv, pa, pb));
                double d2 = norm2(sub3(q, pa));
                const double in2 = s.cthr64[a * MAX_CEN + b];
                if (d2 < in2) return true;
                if (d2 >= s.circ64[a * MAX_CEN + b]) continue;
                d3 hb = mv3(v.rot + 9 * j, d3{s.chax[b][0], s.chax[b][1], s.chax[b][2]});
                if (segment_distance2(add3(pa, ha), sub3(pa, ha), add3(q, hb), sub3(q, hb)) < in2) return true;
                continue;
            }
            if (s.pbc_fold) {
                if (pbc_distance2(s.box, s.inv, pa, pb) < s.cthr64[a * MAX_CEN + b]) return true;
                continue;
            }
            d3 t = pbc_translation(s.box, s.inv, pa, pb);
            if (norm2(sub3(add3(pb, t), pa)) < s.cthr64[a * MAX_CEN + b]) return true;
        }
    }
    return false;
}

// The fixed particle against the hard walls (its position unchanged, its orientation and
// rotated centres fixed).
__device__ __forceinline__ bool overlaps_walls(const DevState &s, d3 pi, const double *ri, const double *ci) {
    if (!s.walls) return false;
    if (s.kind == 3)   // generic convex bodies: XenoCollideTraits::overlapWithWall
        return xc_wall_count(*s.xc, s.walls, s.wall_vec, s.wall_far, s.wall_half, pi, ri, true) != 0;
    double hx[3 * MAX_CEN];
    if (s.segs)
        for (int a = 0; a < s.ncen; a++) {
            d3 h = mv3(ri, d3{s.chax[a][0], s.chax[a][1], s.chax[a][2]});
            hx[3 * a] = h.x, hx[3 * a + 1] = h.y, hx[3 * a + 2] = h.z;
        }
    return wall_overlap_count(s.walls, s.wall_vec, s.wall_far, s.wall_half, s.ncen ? 2 : s.kind, s.wall_radius,
                              s.wall_half_len, pi, d3{ri[2], ri[5], ri[8]}, ci, s.ncen, true,
                              s.segs ? hx : nullptr) != 0;
}

// The candidates of particle i: the particles of its cell and the 26 around it.
template <typename F>
__device__ __forceinline__ bool any_candidate(const GridDev &g, int64_t i, F &&f) {
    const int cell = g.pid_cell[i];
    const int cx = cell % g.dims[0], cy = (cell / g.dims[0]) % g.dims[1], cz = cell / (g.dims[0] * g.dims[1]);
    for (int o = 0; o < 27; o++) {
        int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = o / 9 - 1;
        auto wrap = [](int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); };
        int nb = wrap(cx + ox, g.dims[0]) + g.dims[0] * (wrap(cy + oy, g.dims[1]) + g.dims[1] * wrap(cz + oz, g.dims[2]));
        for (int k = g.start[nb]; k < g.start[nb + 1]; k++)
            if (f((int64_t)g.slot_pid[k])) return true;
    }
    return false;
}

// All particles at once, every earlier neighbour assumed fixed.  rejected[i] = 1 if the
// fixed particle overlaps; first = the smallest rejected index.
__global__ void k_fix_check(DevState s, GridDev g, const double *rotfix, const double *cenfix, const double *absfix,
                            uint8_t *rejected, unsigned long long *first) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const d3 pi = ld3(s.pos64 + 3 * i);
    const double *ri = rotfix + 9 * i;
    const double *ai = s.ncen ? absfix + 3 * (size_t)i * s.ncen : nullptr;
    const Version fixed{rotfix, absfix}, current{s.rot64, s.abs64};
    bool ov = any_candidate(g, i, [&](int64_t j) {
        if (j == i) return false;
        return overlaps_pair(s, pi, ri, ai, j, j < i ? fixed : current);
    });
    if (!ov) ov = overlaps_walls(s, pi, ri, s.ncen ? cenfix + 3 * (size_t)i * s.ncen : nullptr);
    rejected[i] = ov ? 1 : 0;
    if (ov) atomicMin(first, (unsigned long long)i);
}

// Copies the fixed state of particles [from, to) into the live state.
__global__ void k_fix_commit(DevState s, const double *rotfix, const double *cenfix, const double *absfix,
                             int64_t from, int64_t to) {
    int64_t i = from + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= to) return;
    for (int k = 0; k < 9; k++) s.rot64[9 * i + k] = rotfix[9 * i + k];
    for (int e = 0; e < 3 * s.ncen; e++) {
        s.cen64[3 * (size_t)i * s.ncen + e] = cenfix[3 * (size_t)i * s.ncen + e];
        s.abs64[3 * (size_t)i * s.ncen + e] = absfix[3 * (size_t)i * s.ncen + e];
    }
}

// The serial remainder: one warp takes the particles from `from` on in index order; lanes
// split the candidates, the live state holds every decision already made.
__global__ void k_fix_serial(DevState s, GridDev g, const double *rotfix, const double *cenfix, const double *absfix,
                             int64_t from, unsigned long long *nrej) {
    const int lane = threadIdx.x & 31;
    const Version current{s.rot64, s.abs64};
    unsigned long long rej = 0;
    for (int64_t i = from; i < s.n; i++) {
        const d3 pi = ld3(s.pos64 + 3 * i);
        const double *ri = rotfix + 9 * i;
        const double *ai = s.ncen ? absfix + 3 * (size_t)i * s.ncen : nullptr;
        const int cell = g.pid_cell[i];
        const int cx = cell % g.dims[0], cy = (cell / g.dims[0]) % g.dims[1], cz = cell / (g.dims[0] * g.dims[1]);
        bool ov = false;
        for (int o = 0; o < 27 && !ov; o++) {
            int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = o / 9 - 1;
            auto wrap = [](int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); };
            int nb = wrap(cx + ox, g.dims[0]) +
                     g.dims[0] * (wrap(cy + oy, g.dims[1]) + g.dims[1] * wrap(cz + oz, g.dims[2]));
            const int b = g.start[nb], e = g.start[nb + 1];
            for (int kb = b; kb < e; kb += 32) {
                const int k = kb + lane;
                bool hit = false;
                if (k < e) {
                    const int64_t j = g.slot_pid[k];
                    if (j != i) hit = overlaps_pair(s, pi, ri, ai, j, current);
                }
                if (__ballot_sync(0xffffffffu, hit)) {
                    ov = true;
                    break;
                }
            }
        }
        if (!ov) {
            int w = 0;
            if (lane == 0) w = overlaps_walls(s, pi, ri, s.ncen ? cenfix + 3 * (size_t)i * s.ncen : nullptr) ? 1 : 0;
            ov = __shfl_sync(0xffffffffu, w, 0) != 0;
        }
        if (ov) {
            rej++;
        } else if (lane < 9) {
            s.rot64[9 * i + lane] = ri[lane];
        }
        if (!ov)
            for (int e = lane; e < 3 * s.ncen; e += 32) {
                s.cen64[3 * (size_t)i * s.ncen + e] = cenfix[3 * (size_t)i * s.ncen + e];
                s.abs64[3 * (size_t)i * s.ncen + e] = absfix[3 * (size_t)i * s.ncen + e];
            }
        __syncwarp();
        __threadfence_block();
    }
    if (lane == 0) *nrej = rej;
}

}  // namespace

cudaError_t launch_fix_prepare(const DevState &s, const double *cbody, double *rotfix, double *cenfix, double *absfix,
                               cudaStream_t st) {
    k_fix_prepare<<<(unsigned)((s.n + 127) / 128), 128, 0, st>>>(s, cbody, rotfix, cenfix, absfix);
    return cudaGetLastError();
}

cudaError_t launch_fresh_centres(const DevState &s, const double *cbody, cudaStream_t st) {
    int64_t t = s.n * s.ncen;
    if (t == 0) return cudaSuccess;
    k_fresh_centres<<<(unsigned)((t + 255) / 256), 256, 0, st>>>(s, cbody);
    return cudaGetLastError();
}

cudaError_t launch_fix_check(const DevState &s, const GridDev &g, const double *rotfix, const double *cenfix, const double *absfix,
                             uint8_t *rejected, unsigned long long *first, cudaStream_t st) {
    k_fix_check<<<(unsigned)((s.n + 127) / 128), 128, 0, st>>>(s, g, rotfix, cenfix, absfix, rejected, first);
    return cudaGetLastError();
}

cudaError_t launch_fix_commit(const DevState &s, const double *rotfix, const double *cenfix, const double *absfix,
                              int64_t from, int64_t to, cudaStream_t st) {
    if (to <= from) return cudaSuccess;
    k_fix_commit<<<(unsigned)((to - from + 255) / 256), 256, 0, st>>>(s, rotfix, cenfix, absfix, from, to);
    return cudaGetLastError();
}

cudaError_t launch_fix_serial(const DevState &s, const GridDev &g, const double *rotfix, const double *cenfix,
                              const double *absfix, int64_t from, unsigned long long *nrej, cudaStream_t st) {
    k_fix_serial<<<1, 32, 0, st>>>(s, g, rotfix, cenfix, absfix, from, nrej);
    return cudaGetLastError();
}

}  // namespace rp
