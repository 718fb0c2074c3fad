// Moves decided entirely in FP64, one warp each:
//
//  * single moves: Packing::tryTranslation / tryRotation / tryMove with or without an
//    ActiveDomain (core/Packing.cpp:84-164) and Packing::accept* (:234-302), the reference's
//    serial path (Simulation::performMovesWithoutDomainDivision, core/Simulation.cpp:365-390):
//    one launch tests one move, one launch commits it (rp_try_move / rp_accept_move);
//  * sweeps of packings with a soft part (a central potential joined to the hard shape by
//    CompoundInteraction, core/interactions/CompoundInteraction.cpp:9-49): one warp per active
//    cell of a checkerboard phase, every move's hard test and energy change in FP64;
//  * the total soft energy (Packing::getTotalEnergy, core/Packing.cpp:689-764) for box moves.
//
// A move's exact FP64 state is computed as the reference computes its temp shape
// (Shape::translate with the periodic correction, Shape::rotate, the rotated and absolute
// interaction centres), and every candidate within reach of it is decided in FP64 with the
// reference's pair test at every periodic image within reach: that is the set of
// (candidate, translation) pairs the reference's neighbour grid visits that can overlap, so
// the any-overlap answer and, in overlap counting, the counts are the reference's.  The soft
// potentials vanish beyond their range, so the energies sum over the same pairs (in another
// order than the reference's neighbour-grid walk).  Candidates come from the handle's cell
// grid (cells at least one interaction range high); particles moved by single moves since the
// grid was built are skipped in their old cells and tested from a short list instead.
#include <cuda_runtime.h>
#include <math_constants.h>

#include "rp_sweep.cuh"

namespace rp {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int SOFT_WARPS = 4;   // warps per block of the soft sweep
constexpr int XC_QUEUE = 256;   // convex bodies: near (candidate, image) pairs queued per warp

// One mover in shared memory: [0] the tried state, [1] the current one.
struct Mover {
    double pos[2][3], rot[2][9];
    double abs[2][3 * MAX_CEN];         // absolute interaction centres of both states
    double hax[2][3 * MAX_CEN];         // polyspherocylinders: orientation * half axis
    double cen[3 * MAX_CEN];            // the tried state's rotated centres
    int cells[2][27];                   // distinct grid cells around each state's position
    int ncells[2];
    int cstart[2][28];                  // prefix of those cells' occupancies
    int outside;                        // the tried position lies outside the ActiveDomain
    mutable int xq[XC_QUEUE];           // convex bodies: candidate * 28 + image of the near pairs
};

// Grid cell coordinate d of fractional coordinate r: the rebuild's own arithmetic (assign_one).
__device__ __forceinline__ int cell_coord(const GridDev &g, int d, double r) {
    double u = r - g.shift[d];
    if (u < 0.0) u += 1.0;
    int cd = static_cast<int>(u * g.dims[d]);
    if (cd >= g.dims[d]) cd = g.dims[d] - 1;
    if (cd < 0) cd = 0;
    return cd;
}

// The distinct cells among the 27 around cell coordinates c (a grid dimension of one or two
// cells names the same cell several times; its particles are listed once and tested at every
// image within reach instead).
__device__ int neighbour_cells(const GridDev &g, const int c[3], int *out) {
    int k = 0;
    const bool distinct = g.dims[0] >= 3 && g.dims[1] >= 3 && g.dims[2] >= 3;
    for (int oz = -1; oz <= 1; oz++)
        for (int oy = -1; oy <= 1; oy++)
            for (int ox = -1; ox <= 1; ox++) {
                int nb = wrap_cell(c[0] + ox, g.dims[0]) +
                         g.dims[0] * (wrap_cell(c[1] + oy, g.dims[1]) + g.dims[1] * wrap_cell(c[2] + oz, g.dims[2]));
                bool seen = false;
                if (!distinct)
                    for (int q = 0; q < k; q++) seen = seen || out[q] == nb;
                if (!seen) out[k++] = nb;
            }
    return k;
}

// CentralInteraction::calculateEnergyForDistance2 of the soft part, in the reference's
// operation order: RepulsiveLennardJonesInteraction.cpp:9-17, SquareInverseCoreInteraction.cpp:13-15.
// (cut^2, sigma^2 and 4 eps are the host's products of the same operands, identical roundings).
__device__ double soft_energy(const DevState &s, double d2) {
    if (s.soft == 1) {
        if (d2 >= s.soft_cut2) return 0.0;
        const double x2 = ddiv(s.soft_sigma2, d2);
        const double x6 = dmul(dmul(x2, x2), x2);
        const double x12 = dmul(x6, x6);
        return dadd(dmul(s.soft_4eps, dsub(x12, x6)), s.soft_eps);
    }
    if (s.soft == 2) {
        const double v = dsub(ddiv(s.soft_sigma2, d2), 1.0);
        return dmul(s.soft_eps, 0.0 < v ? v : 0.0);  // std::max(0.0, v)
    }
    return 0.0;
}

// Pair test of a sphere, spherocylinder or generic convex mover (position p, axis a,
// orientation rot) against particle j at translation t (null: no grid in the reference, the
// periodic boundary conditions' nearest image), SphereTraits.cpp:56-65 /
// SpherocylinderTraits.cpp:28-46 / XenoCollideTraits.h:147-168 (the mover is the first body,
// as in Packing::countParticleOverlaps).
template <int KIND>
__device__ bool body_overlap(const DevState &s, d3 p, d3 a, const double *rot, int j, const d3 *t) {
    const d3 pj = load_d3(s.pos64 + 3 * (size_t)j);
    const double *rj = s.rot64 + 9 * (size_t)j;
    if constexpr (KIND == 3) {
        const d3 q = add3(pj, t ? *t : pbc_translation(s.box, s.inv, p, pj));
        bool stuck = false;
        const bool ov = xc_overlap_filtered(*s.xc, p, rot, q, rj, stuck);
        if (stuck) atomicOr(s.status, ST_PORTAL_STUCK);
        return ov;
    } else {
        const d3 aj{rj[2], rj[5], rj[8]};
        if (t) return exact_overlap(s.ex, p, a, pj, aj, *t);
        if (KIND == 0) return pbc_distance2(s.box, s.inv, p, pj) < s.ex.sphere_thr;
        return exact_overlap(s.ex, p, a, pj, aj, pbc_translation(s.box, s.inv, p, pj));
    }
}

// Centre a of a multi-centre mover (absolute centre pa, half axis ha) against centre b of body
// j at translation t (null: the nearest image): PolysphereTraits::HardInteraction
// (core/shapes/PolysphereTraits.cpp:97-106, the cell's translation as core/Packing.cpp:40-42)
// or PolyspherocylinderTraits::overlapBetween (core/shapes/PolyspherocylinderTraits.cpp:102-124).
__device__ bool centre_overlap(const DevState &s, d3 pa, d3 ha, int a, int j, int b, const d3 *t) {
    const d3 pb = load_d3(s.abs64 + 3 * ((size_t)j * s.ncen + b));
    const double in2 = s.cthr64[a * MAX_CEN + b];
    if (s.segs) {
        const d3 tt = t ? *t : pbc_translation(s.box, s.inv, pa, pb);
        const d3 q = add3(pb, tt);
        const double d2 = norm2(sub3(q, pa));
        if (d2 < in2) return true;
        if (d2 >= s.circ64[a * MAX_CEN + b]) return false;
        const d3 hj = mv3(s.rot64 + 9 * (size_t)j, d3{s.chax[b][0], s.chax[b][1], s.chax[b][2]});
        return segment_distance2(add3(pa, ha), sub3(pa, ha), add3(q, hj), sub3(q, hj)) < in2;
    }
    if (t) return norm2(sub3(add3(pb, *t), pa)) < in2;
    return pbc_distance2(s.box, s.inv, pa, pb) < in2;
}

// FP32 separation q - p of two FP64 points (one FP64 subtraction per coordinate, shared by
// the images tested next).
__device__ __forceinline__ float3 separation32(const double *q, const double *p) {
    return make_float3(static_cast<float>(q[0] - p[0]), static_cast<float>(q[1] - p[1]),
                       static_cast<float>(q[2] - p[2]));
}

// The FP32 separation at image m against the pre-filter reach.
__device__ __forceinline__ bool within_reach(const SingleArgs &A, float3 sep, int mx, int my, int mz) {
    const float3 t32 = mat32(A.box32, (float)mx, (float)my, (float)mz);
    const float ex = sep.x + t32.x, ey = sep.y + t32.y, ez = sep.z + t32.z;
    return ex * ex + ey * ey + ez * ez <= A.reach2;
}

__device__ __forceinline__ d3 image_translation(const DevState &s, int mx, int my, int mz) {
    return load_d3(s.trans + 3 * (((mx + 2) * 5 + (my + 2)) * 5 + (mz + 2)));
}

// The periodic images m in {-1, 0, 1}^3 of a pair within the pre-filter reach, given its FP32
// separation q - p, in the order of the 27-image loop; f(mx, my, mz) returns true to stop.
// Where the reach is below 0.45 of every box height (one_image), an image within reach has
// every fractional separation component below 0.45 in magnitude and any other image is a
// whole box height away in some direction, so the only candidate is the image whose
// fractional separation rounds to zero (FP32 rounding is ~1e-6 against the 0.05 margin): it
// alone goes through the same pre-filter test, and the images passed are the 27-image loop's.
template <typename F>
__device__ __forceinline__ void for_each_image(const SingleArgs &A, float3 sep, F &&f) {
    if (A.one_image) {
        const float *iv = A.s.inv32;
        const int mx = -__float2int_rn(iv[0] * sep.x + iv[1] * sep.y + iv[2] * sep.z);
        const int my = -__float2int_rn(iv[3] * sep.x + iv[4] * sep.y + iv[5] * sep.z);
        const int mz = -__float2int_rn(iv[6] * sep.x + iv[7] * sep.y + iv[8] * sep.z);
        if (mx < -1 || mx > 1 || my < -1 || my > 1 || mz < -1 || mz > 1) return;
        if (within_reach(A, sep, mx, my, mz)) f(mx, my, mz);
        return;
    }
    for (int mx = -1; mx <= 1; mx++)
        for (int my = -1; my <= 1; my++)
            for (int mz = -1; mz <= 1; mz++)
                if (within_reach(A, sep, mx, my, mz) && f(mx, my, mz)) return;
}

// Overlapping pairs of a mover state (position p, axis a; multi-centre: absolute centres abs,
// half axes hax) with body j over every periodic image within reach (each absolute centre is
// wrapped into the box on its own, so images are enumerated per centre pair); at most 1 with
// `early`.
template <int KIND>
__device__ int candidate_overlaps(const SingleArgs &A, const double *p, d3 a, const double *rot, const double *abs,
                                  const double *hax, int j, bool early) {
    const DevState &s = A.s;
    int cnt = 0;
    if constexpr (KIND != 2) {
        const d3 pp{p[0], p[1], p[2]};
        if (s.pbc_fold) return body_overlap<KIND>(s, pp, a, rot, j, nullptr) ? 1 : 0;
        const float3 sep = separation32(s.pos64 + 3 * (size_t)j, p);
        for_each_image(A, sep, [&](int mx, int my, int mz) {
            const d3 t = image_translation(s, mx, my, mz);
            if (!body_overlap<KIND>(s, pp, a, rot, j, &t)) return false;
            cnt++;
            return early;
        });
        return cnt;
    } else {
        for (int ca = 0; ca < s.ncen; ca++) {
            const d3 pa{abs[3 * ca], abs[3 * ca + 1], abs[3 * ca + 2]};
            const d3 ha = hax ? d3{hax[3 * ca], hax[3 * ca + 1], hax[3 * ca + 2]} : d3{0.0, 0.0, 0.0};
            for (int b = 0; b < s.ncen; b++) {
                if (s.pbc_fold) {
                    if (centre_overlap(s, pa, ha, ca, j, b, nullptr)) {
                        if (early) return 1;
                        cnt++;
                    }
                    continue;
                }
                const float3 sep = separation32(s.abs64 + 3 * ((size_t)j * s.ncen + b), abs + 3 * ca);
                for_each_image(A, sep, [&](int mx, int my, int mz) {
                    const d3 t = image_translation(s, mx, my, mz);
                    if (!centre_overlap(s, pa, ha, ca, j, b, &t)) return false;
                    cnt++;
                    return early;
                });
                if (early && cnt) return 1;
            }
        }
        return cnt;
    }
}

// Soft energy of a mover state with body j: every centre pair at every image within reach
// (CentralInteraction::calculateEnergyBetween with the cell's translation, or the periodic
// boundary conditions' distance where the reference keeps no grid).
template <int KIND>
__device__ double candidate_energy(const SingleArgs &A, const double *p, const double *abs, int j) {
    const DevState &s = A.s;
    double e = 0.0;
    const int K = KIND == 2 ? s.ncen : 1;
    for (int ca = 0; ca < K; ca++) {
        const double *pa = KIND == 2 ? abs + 3 * ca : p;
        const d3 pa3{pa[0], pa[1], pa[2]};
        for (int b = 0; b < K; b++) {
            const double *pb = KIND == 2 ? s.abs64 + 3 * ((size_t)j * s.ncen + b) : s.pos64 + 3 * (size_t)j;
            const d3 pb3{pb[0], pb[1], pb[2]};
            if (s.pbc_fold) {
                e = dadd(e, soft_energy(s, pbc_distance2(s.box, s.inv, pa3, pb3)));
                continue;
            }
            // q - p in FP64: the pre-filter's separation, and the zero image's difference ((q + 0) - p
            // is q - p up to the sign of a zero, which the squared norm drops)
            const d3 dd = sub3(pb3, pa3);
            const float3 sep = make_float3(static_cast<float>(dd.x), static_cast<float>(dd.y), static_cast<float>(dd.z));
            for_each_image(A, sep, [&](int mx, int my, int mz) {
                const double d2 = (mx | my | mz) ? norm2(sub3(add3(pb3, image_translation(s, mx, my, mz)), pa3))
                                                 : norm2(dd);
                e = dadd(e, soft_energy(s, d2));
                return false;
            });
        }
    }
    return e;
}

// The candidate behind index k of mover state `which`: particles of its neighbour cells in
// grid order, then the particles moved since the grid was built; -1 for one to skip.
__device__ __forceinline__ int candidate_at(const SingleArgs &A, const Mover &mv, int which, int k, int in_cells) {
    if (k < in_cells) {
        // the last cell whose prefix is at most k (empty cells share their successor's prefix)
        int c = 0, hi = mv.ncells[which] - 1;
        while (c < hi) {
            const int mid = (c + hi + 1) >> 1;
            if (mv.cstart[which][mid] <= k) c = mid;
            else hi = mid - 1;
        }
        const int cell = mv.cells[which][c];
        const int j = A.g.slot_pid[A.g.start[cell] + (k - mv.cstart[which][c])];
        return (A.disp_flag && A.disp_flag[j]) ? -1 : j;  // moved since: tested from the list
    }
    return A.disp_list[k - in_cells];
}

// Generic convex bodies: the radii tests of XenoCollideTraits::overlapBetween
// (core/shapes/XenoCollideTraits.h:155-163) decide most (candidate, image) pairs at once; the
// pairs between insphere and circumsphere distance are queued and their refinements run packed
// 32 to a warp pass, so the lanes of a pass all refine (instead of a few lanes per candidate
// round).  Same pairs and decisions as the per-candidate loop; the count, or 0 / 1 with `early`.
__device__ int warp_overlaps_convex(const SingleArgs &A, const Mover &mv, int which, bool early, int pid) {
    const DevState &s = A.s;
    const int lane = threadIdx.x & 31;
    const int in_cells = mv.cstart[which][mv.ncells[which]];
    const int total = in_cells + A.ndisp;
    const double *rot = mv.rot[which];
    const d3 p{mv.pos[which][0], mv.pos[which][1], mv.pos[which][2]};
    const double rc = dadd(s.xc->circ, s.xc->circ), ri = dadd(s.xc->insph, s.xc->insph);
    const double rc2 = dmul(rc, rc), ri2 = dmul(ri, ri);
    int cnt = 0, nq = 0;
    // refine the queued pairs, 32 to a pass; true on an overlap with `early`
    auto drain = [&]() -> bool {
        for (int b = 0; b < nq; b += 32) {
            int c = 0;
            if (b + lane < nq) {
                const int e = mv.xq[b + lane];
                const int j = e / 28, m = e % 28;
                const d3 pj = load_d3(s.pos64 + 3 * (size_t)j);
                const d3 t = m == 27 ? pbc_translation(s.box, s.inv, p, pj)
                                     : image_translation(s, m / 9 - 1, (m / 3) % 3 - 1, m % 3 - 1);
                bool stuck = false;
                const int f = xc_filter(*s.xc, p, rot, add3(pj, t), s.rot64 + 9 * (size_t)j);
                c = f >= 0 ? f : (xc_intersect(*s.xc, rot, p, s.rot64 + 9 * (size_t)j, add3(pj, t), 1.0e-12, stuck) ? 1 : 0);
                if (stuck) atomicOr(s.status, ST_PORTAL_STUCK);
            }
            if (early && __any_sync(FULL, c != 0)) return true;
            cnt += c;
        }
        __syncwarp();  // every lane has read its entries before the queue is refilled
        nq = 0;
        return false;
    };
    for (int base = 0; base < total; base += 32) {
        const int k = base + lane;
        int certain = 0;
        int near_e[4];
        int nnear = 0;
        if (k < total) {
            const int j = candidate_at(A, mv, which, k, in_cells);
            if (j >= 0 && j != pid) {
                const double *pjp = s.pos64 + 3 * (size_t)j;
                const d3 pj = load_d3(pjp);
                if (s.pbc_fold) {
                    const d3 q = add3(pj, pbc_translation(s.box, s.inv, p, pj));
                    const double d2 = norm2(sub3(q, p));
                    if (d2 < ri2) certain++;
                    else if (!(d2 > rc2)) near_e[nnear++] = j * 28 + 27;
                } else {
                    const float3 sep = separation32(pjp, mv.pos[which]);
                    for_each_image(A, sep, [&](int mx, int my, int mz) {
                        const int m = (mx + 1) * 9 + (my + 1) * 3 + (mz + 1);
                        const double d2 = norm2(sub3(add3(pj, image_translation(s, mx, my, mz)), p));
                        if (d2 > rc2) return false;
                        if (d2 < ri2) {
                            certain++;
                        } else if (nnear < 4) {
                            near_e[nnear++] = j * 28 + m;
                        } else {
                            bool stuck = false;  // a fifth near image of one candidate: decided here
                            const d3 t = image_translation(s, mx, my, mz);
                            const int f = xc_filter(*s.xc, p, rot, add3(pj, t), s.rot64 + 9 * (size_t)j);
                            certain += f >= 0 ? f
                                              : (xc_intersect(*s.xc, rot, p, s.rot64 + 9 * (size_t)j, add3(pj, t),
                                                              1.0e-12, stuck) ? 1 : 0);
                            if (stuck) atomicOr(s.status, ST_PORTAL_STUCK);
                        }
                        return false;
                    });
                }
            }
        }
        if (early && __any_sync(FULL, certain != 0)) return 1;
        cnt += certain;
        // queue this round's near pairs (at most 4 per lane)
        if (nq + 4 * 32 > XC_QUEUE && drain()) return 1;
        for (int r = 0; r < 4; r++) {
            const bool has = r < nnear;
            const unsigned bal = __ballot_sync(FULL, has);
            if (!bal) break;
            if (has) mv.xq[nq + __popc(bal & ((1u << lane) - 1))] = near_e[r];
            nq += __popc(bal);
        }
        __syncwarp();
    }
    if (drain()) return 1;
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(FULL, cnt, d);
    if (s.walls && !(early && cnt)) {
        // hard walls after the pairs (core/Packing.cpp:424-428)
        int w = 0;
        if (lane == 0) w = xc_wall_count(*s.xc, s.walls, s.wall_vec, s.wall_far, s.wall_half, p, rot, early);
        cnt += __shfl_sync(FULL, w, 0);
    }
    return early ? (cnt > 0 ? 1 : 0) : cnt;
}

// Overlaps of mover state `which` with every candidate, then the walls (the count, or 0 / 1
// with `early`: Packing::countParticleOverlaps, core/Packing.cpp:373-429); the whole warp.
template <int KIND>
__device__ int warp_overlaps(const SingleArgs &A, const Mover &mv, int which, bool early, int pid) {
    if constexpr (KIND == 3) return warp_overlaps_convex(A, mv, which, early, pid);
    const DevState &s = A.s;
    const int lane = threadIdx.x & 31;
    const int in_cells = mv.cstart[which][mv.ncells[which]];
    const int total = in_cells + A.ndisp;
    const d3 a{mv.rot[which][2], mv.rot[which][5], mv.rot[which][8]};
    const double *hax = (KIND == 2 && s.segs) ? mv.hax[which] : nullptr;
    int cnt = 0;
    for (int base = 0; base < total; base += 32) {
        const int k = base + lane;
        int c = 0;
        if (k < total) {
            const int j = candidate_at(A, mv, which, k, in_cells);
            // the self-skip compares particle indices (core/Packing.cpp:633-635)
            if (j >= 0 && j != pid)
                c = candidate_overlaps<KIND>(A, mv.pos[which], a, mv.rot[which], mv.abs[which], hax, j, early);
        }
        if (early && __any_sync(FULL, c != 0)) return 1;
        cnt += c;
    }
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(FULL, cnt, d);
    if (s.walls) {
        // hard walls after the pairs (core/Packing.cpp:424-428)
        int w = 0;
        if (lane == 0) {
            const d3 p{mv.pos[which][0], mv.pos[which][1], mv.pos[which][2]};
            const double *cen = KIND == 2 ? (which == 0 ? mv.cen : s.cen64 + 3 * (size_t)pid * s.ncen) : nullptr;
            w = wall_overlap_count(s.walls, s.wall_vec, s.wall_far, s.wall_half, KIND, s.wall_radius, s.wall_half_len,
                                   p, a, cen, KIND == 2 ? s.ncen : 0, early, hax);
        }
        cnt += __shfl_sync(FULL, w, 0);
    }
    return early ? (cnt > 0 ? 1 : 0) : cnt;
}

// Soft energy of mover state `which` with every candidate (Packing::calculateParticleEnergy,
// core/Packing.cpp:649-687); the whole warp, a fixed reduction order.
template <int KIND>
__device__ double warp_energy(const SingleArgs &A, const Mover &mv, int which, int pid) {
    const int lane = threadIdx.x & 31;
    const int in_cells = mv.cstart[which][mv.ncells[which]];
    const int total = in_cells + A.ndisp;
    double e = 0.0;
    for (int k = lane; k < total; k += 32) {
        const int j = candidate_at(A, mv, which, k, in_cells);
        if (j >= 0 && j != pid) e = dadd(e, candidate_energy<KIND>(A, mv.pos[which], mv.abs[which], j));
    }
    for (int d = 16; d > 0; d >>= 1) e = dadd(e, __shfl_xor_sync(FULL, e, d));
    return e;
}

// The whole warp: the current state and the temp shape of move m of particle pid
// (core/Packing.cpp:86-93, 113-116, 137-146), the ActiveDomain test of a translation (lo null:
// none; bounded[d] 0: dimension d unbounded), and the neighbour cells of the temp state and,
// with `both`, of the current one.  Each coordinate's arithmetic is the serial restatement's
// (Shape::translate with pbc_correction, mv3, cell_coord, mm_elem), spread over lanes: lane i < 3
// computes coordinate i of the temp position and its domain test, lane 3w + i coordinate i of
// state w's cell, lane e < 9 element e of the rotated orientation, lane q < 27 neighbour q;
// the values meet through shuffles.
template <int KIND>
__device__ void build_mover(const SingleArgs &A, Mover &mv, const rp_move &m, int pid, bool both,
                            const double *lo, const double *hi, const int *bounded) {
    const DevState &s = A.s;
    const GridDev &g = A.g;
    const int lane = threadIdx.x & 31;
    const int i = lane % 3;
    const double *p0p = s.pos64 + 3 * (size_t)pid;
    const double *o0 = s.rot64 + 9 * (size_t)pid;
    const bool trans = m.type != RP_MOVE_ROTATION;
    const d3 p0 = load_d3(p0p);
    const double p0i = p0p[i];
    // Shape::translate (core/Shape.cpp:9-12): q = p0 + t on lanes 0-2 (p0 for a rotation)
    const double qi = trans ? dadd(p0i, m.translation[i]) : p0i;
    const d3 q{__shfl_sync(FULL, qi, 0), __shfl_sync(FULL, qi, 1), __shfl_sync(FULL, qi, 2)};
    // fractional coordinate i of q (lanes 0-2) and of the current position (lanes 3-5)
    double ri = mrow(s.inv, i, lane < 3 ? q : p0);
    double p1i = qi;
    if (trans) {
        // PeriodicBoundaryConditions::getCorrection (pbc_correction) row i: the wrap count c
        // from q's fractional coordinate, then q + box * c
        double c = 0.0;
        if (lane < 3) {
            while (dadd(ri, c) < 0.0) c = dadd(c, 1.0);
            while (dadd(ri, c) >= 1.0) c = dsub(c, 1.0);
        }
        if (__any_sync(FULL, c != 0.0)) {
            const d3 cv{__shfl_sync(FULL, c, 0), __shfl_sync(FULL, c, 1), __shfl_sync(FULL, c, 2)};
            p1i = dadd(qi, mrow(s.box, i, cv));
        } else {
            p1i = dadd(qi, s.box_zero[i]);  // box * (0, 0, 0), the same products and sums
        }
        // the temp position's fractional coordinate is q's unless the correction changed q
        const bool changed = lane < 3 && __double_as_longlong(p1i) != __double_as_longlong(qi);
        if (__any_sync(FULL, changed)) {
            const d3 p1v{__shfl_sync(FULL, p1i, 0), __shfl_sync(FULL, p1i, 1), __shfl_sync(FULL, p1i, 2)};
            ri = mrow(s.inv, i, lane < 3 ? p1v : p0);
        }
    }
    const d3 p1{__shfl_sync(FULL, p1i, 0), __shfl_sync(FULL, p1i, 1), __shfl_sync(FULL, p1i, 2)};
    // the ActiveDomain of a translation or rototranslation, tested before any overlap
    // (core/Packing.cpp:94-96, :141-143; ActiveDomain::isInside, core/ActiveDomain.cpp:8-21)
    bool out = false;
    if (lo && trans && lane < 3 && !(bounded && !bounded[i])) {
        if (hi[i] > lo[i]) out = ri <= lo[i] || ri >= hi[i];
        else out = ri <= lo[i] && ri >= hi[i];
    }
    const int outside = __any_sync(FULL, out) ? 1 : 0;
    if (lane < 3) {
        mv.pos[0][lane] = p1i;
        mv.pos[1][lane] = p0i;
    }
    if (lane < 9) {  // Shape::rotate: R * O (core/Shape.cpp:14-16)
        const double o0e = o0[lane];
        mv.rot[0][lane] = m.type != RP_MOVE_TRANSLATION ? mm_elem(m.rotation, o0, lane / 3, lane % 3) : o0e;
        mv.rot[1][lane] = o0e;
    }
    if (lane == 0) mv.outside = outside;
    const int cdi = cell_coord(g, i, ri);
    const bool distinct = g.dims[0] >= 3 && g.dims[1] >= 3 && g.dims[2] >= 3;
    for (int w = 0; w < (both ? 2 : 1); w++) {
        // the distinct cells among the 27 around state w's cell, in neighbour_cells' order, and
        // the prefix of their occupancies
        const int c0 = __shfl_sync(FULL, cdi, 3 * w), c1 = __shfl_sync(FULL, cdi, 3 * w + 1),
                  c2 = __shfl_sync(FULL, cdi, 3 * w + 2);
        int nb = -1;
        if (lane < 27)
            nb = wrap_cell(c0 + lane % 3 - 1, g.dims[0]) +
                 g.dims[0] * (wrap_cell(c1 + (lane / 3) % 3 - 1, g.dims[1]) +
                              g.dims[1] * wrap_cell(c2 + lane / 9 - 1, g.dims[2]));
        bool keep = lane < 27;
        if (!distinct)  // a dimension of one or two cells: keep the first of equal cells
            for (int q = 0; q < 27; q++) {
                const int o = __shfl_sync(FULL, nb, q);
                if (q < lane && o == nb) keep = false;
            }
        const unsigned bal = __ballot_sync(FULL, keep);
        const int at = __popc(bal & ((1u << lane) - 1));
        const int occ = keep ? g.start[nb + 1] - g.start[nb] : 0;
        int incl = occ;
        for (int d = 1; d < 32; d <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, d);
            if (lane >= d) incl += v;
        }
        if (keep) {
            mv.cells[w][at] = nb;
            mv.cstart[w][at] = incl - occ;
        }
        if (lane == 31) {
            mv.ncells[w] = __popc(bal);
            mv.cstart[w][__popc(bal)] = incl;
        }
    }
    __syncwarp();
    if (KIND == 2 && lane == 0) {
        const double *o1 = mv.rot[0];
        for (int a = 0; a < s.ncen; a++) {
            // the temp centres, rotated by R (core/Packing.cpp:357-361), and the absolute
            // centres: position + centre with the periodic correction (:1041-1047)
            d3 c = load_d3(s.cen64 + 3 * ((size_t)pid * s.ncen + a));
            if (m.type != RP_MOVE_TRANSLATION) c = mv3(m.rotation, c);
            const d3 q = add3(p1, c);
            const d3 ab = add3(q, pbc_correction(s.box, s.inv, q, nullptr));
            mv.cen[3 * a] = c.x, mv.cen[3 * a + 1] = c.y, mv.cen[3 * a + 2] = c.z;
            mv.abs[0][3 * a] = ab.x, mv.abs[0][3 * a + 1] = ab.y, mv.abs[0][3 * a + 2] = ab.z;
            for (int d = 0; d < 3; d++) mv.abs[1][3 * a + d] = s.abs64[3 * ((size_t)pid * s.ncen + a) + d];
            if (s.segs) {
                // orientation * half axis (PolyspherocylinderTraits.cpp:118-119)
                const d3 hb{s.chax[a][0], s.chax[a][1], s.chax[a][2]};
                const d3 h1 = mv3(o1, hb), h0 = mv3(o0, hb);
                mv.hax[0][3 * a] = h1.x, mv.hax[0][3 * a + 1] = h1.y, mv.hax[0][3 * a + 2] = h1.z;
                mv.hax[1][3 * a] = h0.x, mv.hax[1][3 * a + 1] = h0.y, mv.hax[1][3 * a + 2] = h0.z;
            }
        }
    }
    __syncwarp();
}

// The move's energy (the whole warp, after build_mover): the ActiveDomain, then the hard part
// (any overlap, or in overlap counting the sign of the change of the mover's count:
// core/Packing.cpp:304-323), then the soft part's energy change (core/Packing.cpp:103-108).
template <int KIND>
__device__ double move_energy(const SingleArgs &A, const Mover &mv, int pid, int &delta) {
    const DevState &s = A.s;
    delta = 0;
    if (mv.outside) return CUDART_INF;
    if (!s.soft_only) {
        if (s.counting) {
            const int after = warp_overlaps<KIND>(A, mv, 0, false, pid);
            const int before = warp_overlaps<KIND>(A, mv, 1, false, pid);
            delta = after - before;
            if (delta < 0) return -CUDART_INF;
            if (delta > 0) return CUDART_INF;
        } else if (warp_overlaps<KIND>(A, mv, 0, true, pid)) {
            return CUDART_INF;
        }
    }
    if (!s.soft) return 0.0;
    const double initial = warp_energy<KIND>(A, mv, 1, pid);
    const double final_ = warp_energy<KIND>(A, mv, 0, pid);
    return dsub(final_, initial);
}

template <int KIND>
__global__ void __launch_bounds__(32) k_try_single(SingleArgs A) {
    __shared__ Mover mv;
    const int pid = A.m.particle;
    build_mover<KIND>(A, mv, A.m, pid, A.s.counting || A.s.soft, A.has_domain ? A.dom_lo : nullptr,
                      A.has_domain ? A.dom_hi : nullptr, nullptr);
    int delta = 0;
    const double dE = move_energy<KIND>(A, mv, pid, delta);
    if (threadIdx.x == 0) {
        SingleTry *o = A.out;
        for (int d = 0; d < 3; d++) o->pos[d] = mv.pos[0][d];
        for (int e = 0; e < 9; e++) o->rot[e] = mv.rot[0][e];
        if (KIND == 2)
            for (int q = 0; q < 3 * A.s.ncen; q++) {
                o->cen[q] = mv.cen[q];
                o->abs[q] = mv.abs[0][q];
            }
        o->dE = dE;
        o->outside = mv.outside;
        o->particle = pid;
        o->type = A.m.type;
        o->delta = delta;
        o->valid = 1;
    }
}

// Packing::acceptTranslation / acceptRotation / acceptMove (core/Packing.cpp:234-302): the temp
// state replaces the particle (rotated and absolute centres included), the cached overlap count
// takes the move's delta, and the particle joins the list of those moved since the grid was
// built (slot < 0: it is there already).
__global__ void k_commit_single(DevState s, SingleTry *t, uint8_t *disp_flag, int32_t *disp_list, int slot) {
    if (threadIdx.x != 0 || !t->valid) return;
    const int pid = t->particle;
    if (t->type != RP_MOVE_ROTATION)
        for (int d = 0; d < 3; d++) s.pos64[3 * (size_t)pid + d] = t->pos[d];
    if (t->type != RP_MOVE_TRANSLATION)
        for (int e = 0; e < 9; e++) s.rot64[9 * (size_t)pid + e] = t->rot[e];
    for (int q = 0; q < 3 * s.ncen; q++) {
        s.cen64[3 * (size_t)pid * s.ncen + q] = t->cen[q];
        s.abs64[3 * (size_t)pid * s.ncen + q] = t->abs[q];
    }
    if (s.counting) atomicAdd(s.overlaps, (unsigned long long)(long long)t->delta);
    if (slot >= 0) {
        disp_flag[pid] = 1;
        disp_list[slot] = pid;
    }
    t->valid = 0;
}

// ---- soft sweeps ----------------------------------------------------------------------

// Metropolis acceptance u <= exp(-dE / T) (core/Simulation.cpp:483) for the sweep's own
// uniforms (multiples of 2^-53 in [0, 1)) and T > 0, without the FP64 exponential where the
// answer is certain: dE <= 0 accepts (exp >= 1 > u); an exponent below -80 accepts only u = 0
// (exp < 2e-35 below the smallest positive u); otherwise CUDA's FP32 expf decides wherever u
// lies more than 1e-4 (relative) away from it, far beyond the FP32 errors of the exponent
// (< 5e-6 relative at |x| <= 80), of expf (a few ulp) and of u; the band in between, and a NaN,
// take the FP64 exponential.  The decision is that of the FP64 test in every case.
__device__ __forceinline__ bool metropolis(double u, double dE, double T) {
    if (dE <= 0.0) return true;
    const double x = T == 1.0 ? -dE : -dE / T;   // a division by one is exact
    if (x < -80.0) return u == 0.0;
    const float ef = expf(static_cast<float>(x)), uf = static_cast<float>(u);
    if (uf <= ef * (1.0f - 1e-4f)) return true;
    if (uf >= ef * (1.0f + 1e-4f)) return false;
    return u <= exp(x);
}

// The Metropolis uniform of move mi of a cell: 53 bits of a Philox draw apart from the
// proposal's words.
__device__ double soft_uniform(const SoftSweepArgs &A, int cell, int mi) {
    const u4 q = philox(u4{(uint32_t)mi, (uint32_t)cell, (uint32_t)A.counter, (uint32_t)(A.counter >> 32) ^ 0x2545f491u},
                        (uint32_t)A.seed ^ 0x9e3779b9u, (uint32_t)(A.seed >> 32));
    // (a >> 5) * 2^26 + (b >> 6) is an integer below 2^53: formed exactly as one, then scaled
    const uint64_t k = (static_cast<uint64_t>(q.a >> 5) << 26) | static_cast<uint64_t>(q.b >> 6);
    return static_cast<double>(k) * (1.0 / 9007199254740992.0);
}

template <int KIND>
__global__ void __launch_bounds__(SOFT_WARPS * 32, 4) k_soft_sweep(SoftSweepArgs A) {
    __shared__ Mover movers[SOFT_WARPS];
    __shared__ rp_move moves[SOFT_WARPS];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Mover &mv = movers[wib];
    rp_move &m = moves[wib];
    const SingleArgs &C = A.c;
    const DevState &S = C.s;
    const GridDev &G = C.g;
    const int ntypes = sweep_move_types(A.types);
    unsigned n_moves = 0, n_acc = 0, n_ov = 0, n_dom = 0, n_tr = 0, n_rot = 0, n_acc_tr = 0;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.next_item, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= A.num_active) break;
        int c[3];
        if (A.work) {  // the phase's cells by occupancy, largest first
            const int w = A.work[item];
            c[0] = w % G.dims[0];
            c[1] = (w / G.dims[0]) % G.dims[1];
            c[2] = w / (G.dims[0] * G.dims[1]);
        } else {
            int w = item;
            const int a0 = w % A.active[0];
            w /= A.active[0];
            const int a1 = w % A.active[1];
            const int a2 = w / A.active[1];
            const int cc[3] = {a0, a1, a2};
            for (int d = 0; d < 3; d++) c[d] = ring_cell(G.dims[d], A.phase[d], cc[d]);
        }
        const int cell = c[0] + G.dims[0] * (c[1] + G.dims[1] * c[2]);
        const int gbase = G.start[cell];
        const int occ = G.start[cell + 1] - gbase;
        // the cell's ActiveDomain bounds (a dimension of one cell is unbounded)
        double lo[3], hi[3];
        int bounded[3];
        for (int d = 0; d < 3; d++) {
            lo[d] = G.bounds[G.boundsoff[d] + 2 * c[d]];
            hi[d] = G.bounds[G.boundsoff[d] + 2 * c[d] + 1];
            bounded[d] = G.dims[d] > 1;
        }
        const int nmoves = ntypes * occ;
        u4 rnd = u4{0u, 0u, 0u, 0u};
        for (int mi = 0; mi < nmoves; mi++) {
            if ((mi & 31) == 0)
                rnd = philox(u4{(uint32_t)(mi + lane), (uint32_t)cell, (uint32_t)A.counter, (uint32_t)(A.counter >> 32)},
                             (uint32_t)A.seed, (uint32_t)(A.seed >> 32));
            const int src = mi & 31;
            const u4 r = u4{__shfl_sync(FULL, rnd.a, src), __shfl_sync(FULL, rnd.b, src), __shfl_sync(FULL, rnd.c, src),
                            __shfl_sync(FULL, rnd.d, src)};
            const int type = ntypes == 2 ? ((r.a >> 31) ? 1 : 0) : ((A.types & 1) ? 0 : 1);
            const int slot = (int)(((uint64_t)(r.a & 0x7fffffffu) * (uint32_t)occ) >> 31);
            const int pid = G.slot_pid[gbase + slot];
            const double uni = soft_uniform(A, cell, mi);
            if (lane == 0) {
                // the proposal: a translation uniform in the cube of the step (an FP32 value, exact
                // as FP64), or a rotation of this sweep's table or its transpose
                m.particle = pid;
                m.type = type;
                m.domain = cell;
                m.reserved = 0;
                m.uniform = uni;
                for (int q = 0; q < 9; q++) m.rotation[q] = (q % 4 == 0) ? 1.0 : 0.0;
                for (int d = 0; d < 3; d++) m.translation[d] = 0.0;
                if (type == 0) {
                    m.translation[0] = (double)(pm1f(r.b) * A.tstep);
                    m.translation[1] = (double)(pm1f(r.c) * A.tstep);
                    m.translation[2] = (double)(pm1f(r.d) * A.tstep);
                } else {
                    const uint32_t idx = r.b & A.rtab_mask;
                    const bool inv = (r.c & 1u) != 0;
                    const double *R = A.rtab64 + 9 * (size_t)idx;
                    for (int q = 0; q < 9; q++) m.rotation[q] = inv ? R[3 * (q % 3) + q / 3] : R[q];
                }
            }
            __syncwarp();
            build_mover<KIND>(C, mv, m, pid, true, lo, hi, bounded);
            int delta = 0;
            const double dE = move_energy<KIND>(C, mv, pid, delta);
            // Metropolis (core/Simulation.cpp:483): u <= exp(-dE / T)
            const bool acc = metropolis(uni, dE, C.temperature);
            const uint8_t code = mv.outside ? 2 : (dE == CUDART_INF ? 1 : (dE == -CUDART_INF ? 3 : 0));
            if (acc && lane == 0) {
                // Packing::acceptMove (core/Packing.cpp:278-302)
                if (type != RP_MOVE_ROTATION)
                    for (int d = 0; d < 3; d++) S.pos64[3 * (size_t)pid + d] = mv.pos[0][d];
                if (type != RP_MOVE_TRANSLATION)
                    for (int e = 0; e < 9; e++) S.rot64[9 * (size_t)pid + e] = mv.rot[0][e];
                for (int q = 0; q < 3 * S.ncen; q++) {
                    S.cen64[3 * (size_t)pid * S.ncen + q] = mv.cen[q];
                    S.abs64[3 * (size_t)pid * S.ncen + q] = mv.abs[0][q];
                }
                if (S.counting) atomicAdd(S.overlaps, (unsigned long long)(long long)delta);
            }
            if (lane == 0 && A.log) {
                A.log[(size_t)ntypes * (size_t)gbase + mi] = m;
                A.log_codes[(size_t)ntypes * (size_t)gbase + mi] = code | (acc ? RP_CODE_ACCEPTED : 0);
            }
            __syncwarp();
            n_moves++;
            n_acc += acc ? 1 : 0;
            n_ov += (code == 1) ? 1 : 0;
            n_dom += (code == 2) ? 1 : 0;
            n_tr += type == 0 ? 1 : 0;
            n_rot += type != 0 ? 1 : 0;
            n_acc_tr += (type == 0 && acc) ? 1 : 0;
        }
    }
    if (lane == 0 && n_moves) {
        unsigned long long *Cn = S.counters;
        atomicAdd(Cn + 0, (unsigned long long)n_moves);
        atomicAdd(Cn + 1, (unsigned long long)n_acc);
        atomicAdd(Cn + 2, (unsigned long long)n_ov);
        atomicAdd(Cn + 3, (unsigned long long)n_dom);
        atomicAdd(Cn + 6, (unsigned long long)n_tr);
        atomicAdd(Cn + 7, (unsigned long long)n_rot);
        atomicAdd(Cn + 8, (unsigned long long)n_acc_tr);
    }
}

// ---- total soft energy ----------------------------------------------------------------

// Per particle i: its pairs with every j > i at every image within reach (each unordered pair
// once, as Packing::getTotalEnergy sums them); the grid current for every particle.
template <int KIND>
__global__ void k_pair_energies(SingleArgs A, double *out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= A.s.n) return;
    const DevState &s = A.s;
    const GridDev &g = A.g;
    const double *p = s.pos64 + 3 * i;
    const double *abs = KIND == 2 ? s.abs64 + 3 * i * s.ncen : nullptr;
    const int own = g.pid_cell[i];
    const int c[3] = {own % g.dims[0], (own / g.dims[0]) % g.dims[1], own / (g.dims[0] * g.dims[1])};
    int cells[27];
    const int nc = neighbour_cells(g, c, cells);
    double e = 0.0;
    for (int q = 0; q < nc; q++) {
        const int cell = cells[q];
        for (int k = g.start[cell]; k < g.start[cell + 1]; k++) {
            const int j = g.slot_pid[k];
            if (j > i) e = dadd(e, candidate_energy<KIND>(A, p, abs, j));
        }
    }
    out[i] = e;
}

// Packing::countTotalOverlaps for generic convex bodies (core/Packing.cpp:519-559), every pair
// decided in FP64: per particle i its pairs with every j > i at every image within reach (the
// lower index as the first body), with the early-exit flag polled per candidate cell.
template <int KIND>
__global__ void k_count_fp64(SingleArgs A, int early, unsigned long long *out, int *flag) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= A.s.n) return;
    const DevState &s = A.s;
    const GridDev &g = A.g;
    const double *p = s.pos64 + 3 * i;
    const double *rot = s.rot64 + 9 * i;
    const d3 a{rot[2], rot[5], rot[8]};
    const int own = g.pid_cell[i];
    const int c[3] = {own % g.dims[0], (own / g.dims[0]) % g.dims[1], own / (g.dims[0] * g.dims[1])};
    int cells[27];
    const int nc = neighbour_cells(g, c, cells);
    unsigned long long cnt = 0;
    for (int q = 0; q < nc; q++) {
        if (early && *(volatile int *)flag) break;
        const int cell = cells[q];
        for (int k = g.start[cell]; k < g.start[cell + 1]; k++) {
            const int j = g.slot_pid[k];
            if (j <= i) continue;
            const int o = candidate_overlaps<KIND>(A, p, a, rot, nullptr, nullptr, j, early != 0);
            if (o) {
                cnt += (unsigned long long)o;
                if (early) {
                    atomicExch(flag, 1);
                    break;
                }
            }
        }
    }
    // Packing::countTotalOverlaps adds every particle's wall overlaps (core/Packing.cpp:558)
    if (KIND == 3 && s.walls && !(early && (cnt || *(volatile int *)flag))) {
        const int w = xc_wall_count(*s.xc, s.walls, s.wall_vec, s.wall_far, s.wall_half, load_d3(p), rot, early != 0);
        if (w && early) atomicExch(flag, 1);
        cnt += (unsigned long long)w;
    }
    if (cnt) atomicAdd(out, cnt);
}

// XenoCollideTraits::overlapBetween of n independent pairs of placed convex bodies (the second
// body at its given position, no periodic image), one thread each.
__global__ void k_convex_pairs(const XcShape *xc, int64_t n, const double *p1, const double *r1, const double *p2,
                               const double *r2, uint8_t *out, uint32_t *status) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool stuck = false;
    const bool ov = xc_overlap_filtered(*xc, load_d3(p1 + 3 * i), r1 + 9 * i, load_d3(p2 + 3 * i), r2 + 9 * i, stuck);
    if (stuck) atomicOr(status, ST_PORTAL_STUCK);
    out[i] = ov ? 1 : 0;
}

// Sum of n values in one block in a fixed order (deterministic): each thread its stride,
// then a tree.
__global__ void k_sum_fixed(const double *v, int64_t n, double *out) {
    __shared__ double part[1024];
    double e = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) e = dadd(e, v[i]);
    part[threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] = dadd(part[threadIdx.x], part[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = part[0];
}

}  // namespace

cudaError_t launch_try_single(const SingleArgs &a, cudaStream_t st) {
    if (a.s.kind == 0) k_try_single<0><<<1, 32, 0, st>>>(a);
    else if (a.s.kind == 1) k_try_single<1><<<1, 32, 0, st>>>(a);
    else if (a.s.kind == 2) k_try_single<2><<<1, 32, 0, st>>>(a);
    else k_try_single<3><<<1, 32, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_commit_single(const DevState &s, SingleTry *t, uint8_t *disp_flag, int32_t *disp_list, int slot,
                                 cudaStream_t st) {
    k_commit_single<<<1, 32, 0, st>>>(s, t, disp_flag, disp_list, slot);
    return cudaGetLastError();
}

// One phase of a soft sweep: `nwarps` persistent warps over the phase's active cells.
cudaError_t launch_soft_sweep(const SoftSweepArgs &a, int nwarps, cudaStream_t st) {
    if (nwarps <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((nwarps + SOFT_WARPS - 1) / SOFT_WARPS);
    if (a.c.s.kind == 0) k_soft_sweep<0><<<blocks, SOFT_WARPS * 32, 0, st>>>(a);
    else if (a.c.s.kind == 1) k_soft_sweep<1><<<blocks, SOFT_WARPS * 32, 0, st>>>(a);
    else if (a.c.s.kind == 2) k_soft_sweep<2><<<blocks, SOFT_WARPS * 32, 0, st>>>(a);
    else k_soft_sweep<3><<<blocks, SOFT_WARPS * 32, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_convex_pairs(const XcShape *xc, int64_t n, const double *p1, const double *r1, const double *p2,
                                const double *r2, uint8_t *out, uint32_t *status, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_convex_pairs<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(xc, n, p1, r1, p2, r2, out, status);
    return cudaGetLastError();
}

// Packing::countTotalOverlaps of generic convex bodies, every pair in FP64.
cudaError_t launch_count_fp64(const SingleArgs &a, int early, unsigned long long *out, int *flag, cudaStream_t st) {
    const unsigned nb = (unsigned)((a.s.n + 127) / 128);
    k_count_fp64<3><<<nb, 128, 0, st>>>(a, early, out, flag);
    return cudaGetLastError();
}

// Packing::getTotalEnergy into *out (device): per-particle pair sums into scratch[n], then a
// fixed-order sum.
cudaError_t launch_total_energy(const SingleArgs &a, double *scratch, double *out, cudaStream_t st) {
    const unsigned nb = (unsigned)((a.s.n + 127) / 128);
    if (a.s.kind == 0) k_pair_energies<0><<<nb, 128, 0, st>>>(a, scratch);
    else if (a.s.kind == 1) k_pair_energies<1><<<nb, 128, 0, st>>>(a, scratch);
    else k_pair_energies<2><<<nb, 128, 0, st>>>(a, scratch);
    k_sum_fixed<<<1, 1024, 0, st>>>(scratch, a.s.n, out);
    return cudaGetLastError();
}

}  // namespace rp
