// Unrestricted single moves: Packing::tryTranslation / tryRotation / tryMove with no
// ActiveDomain (std::nullopt, core/Packing.cpp:84-164) and Packing::accept* (:234-302), the
// reference's serial path (Simulation::performMovesWithoutDomainDivision,
// core/Simulation.cpp:365-390).  The per-move entry of the C ABI (rp_try_move /
// rp_accept_move): one launch tests one move, one launch commits it.
//
// A tried move's exact FP64 state is computed as the reference computes its temp shape
// (Shape::translate with the periodic correction, Shape::rotate, the rotated and absolute
// interaction centres), and every candidate within reach of it is decided in FP64 with the
// reference's pair test at every periodic image within reach: that is the set of
// (candidate, translation) pairs the reference's neighbour grid visits that can overlap, so
// the any-overlap answer and, in overlap counting, the counts are the reference's.
// Candidates come from the handle's cell grid (cells at least one interaction range high);
// particles moved by single moves since the grid was built are skipped in their old cells
// and tested from a short list instead, so a commit never rebuilds the grid.
#include <cuda_runtime.h>
#include <math_constants.h>

#include "rp_sweep.cuh"

namespace rp {

namespace {

constexpr int SINGLE_THREADS = 128;

struct SingleShared {
    double pos[2][3], rot[2][9];        // [0] the tried state, [1] the current one
    double abs[2][3 * MAX_CEN];         // absolute interaction centres of both states
    double hax[2][3 * MAX_CEN];         // polyspherocylinders: orientation * half axis
    double cen[3 * MAX_CEN];            // the tried state's rotated centres
    int cells[2][27];                   // distinct grid cells around each state's position
    int ncells[2];
    int cstart[2][28];                  // prefix of those cells' occupancies, then the list
    int hit;
    int count[2];
    int outside;                        // the tried position lies outside the ActiveDomain
};

// Grid cell of an FP64 position: the rebuild's own arithmetic (assign_one).
__device__ int cell_of(const DevState &s, const GridDev &g, d3 p, int c[3]) {
    d3 r = mv3(s.inv, p);
    double rr[3] = {r.x, r.y, r.z};
    for (int d = 0; d < 3; d++) {
        double u = rr[d] - g.shift[d];
        if (u < 0.0) u += 1.0;
        int cd = static_cast<int>(u * g.dims[d]);
        if (cd >= g.dims[d]) cd = g.dims[d] - 1;
        if (cd < 0) cd = 0;
        c[d] = cd;
    }
    return c[0] + g.dims[0] * (c[1] + g.dims[1] * c[2]);
}

// The distinct cells among the 27 around cell coordinates c (a grid dimension of one or two
// cells names the same cell several times; its particles are listed once and tested at every
// image within reach instead).
__device__ int neighbour_cells(const GridDev &g, const int c[3], int *out) {
    int k = 0;
    for (int oz = -1; oz <= 1; oz++)
        for (int oy = -1; oy <= 1; oy++)
            for (int ox = -1; ox <= 1; ox++) {
                int nb = wrap_cell(c[0] + ox, g.dims[0]) +
                         g.dims[0] * (wrap_cell(c[1] + oy, g.dims[1]) + g.dims[1] * wrap_cell(c[2] + oz, g.dims[2]));
                bool seen = false;
                for (int q = 0; q < k; q++) seen = seen || out[q] == nb;
                if (!seen) out[k++] = nb;
            }
    return k;
}

// Pair test of a sphere or spherocylinder mover state `which` against particle j at
// translation t (null: no grid in the reference, the periodic boundary conditions' nearest
// image), SphereTraits.cpp:56-65 / SpherocylinderTraits.cpp:28-46.
template <int KIND>
__device__ bool body_overlap(const DevState &s, const SingleShared &sh, int which, int j, const d3 *t) {
    const d3 p{sh.pos[which][0], sh.pos[which][1], sh.pos[which][2]};
    const d3 a{sh.rot[which][2], sh.rot[which][5], sh.rot[which][8]};
    const d3 pj = load_d3(s.pos64 + 3 * (size_t)j);
    const double *rj = s.rot64 + 9 * (size_t)j;
    const d3 aj{rj[2], rj[5], rj[8]};
    if (t) return exact_overlap(s.ex, p, a, pj, aj, *t);
    if (KIND == 0) return pbc_distance2(s.box, s.inv, p, pj) < s.ex.sphere_thr;
    return exact_overlap(s.ex, p, a, pj, aj, pbc_translation(s.box, s.inv, p, pj));
}

// Centre a of a multi-centre mover state `which` against centre b of body j at translation t
// (null: the nearest image): PolysphereTraits::HardInteraction (core/shapes/PolysphereTraits.cpp:97-106,
// the cell's translation as core/Packing.cpp:40-42) or PolyspherocylinderTraits::overlapBetween
// (core/shapes/PolyspherocylinderTraits.cpp:102-124).
__device__ bool centre_overlap(const DevState &s, const SingleShared &sh, int which, int a, int j, int b, const d3 *t) {
    const d3 pa{sh.abs[which][3 * a], sh.abs[which][3 * a + 1], sh.abs[which][3 * a + 2]};
    const d3 pb = load_d3(s.abs64 + 3 * ((size_t)j * s.ncen + b));
    const double in2 = s.cthr64[a * MAX_CEN + b];
    if (s.segs) {
        const d3 tt = t ? *t : pbc_translation(s.box, s.inv, pa, pb);
        const d3 q = add3(pb, tt);
        const double d2 = norm2(sub3(q, pa));
        if (d2 < in2) return true;
        if (d2 >= s.circ64[a * MAX_CEN + b]) return false;
        const d3 ha{sh.hax[which][3 * a], sh.hax[which][3 * a + 1], sh.hax[which][3 * a + 2]};
        const d3 hj = mv3(s.rot64 + 9 * (size_t)j, d3{s.chax[b][0], s.chax[b][1], s.chax[b][2]});
        return segment_distance2(add3(pa, ha), sub3(pa, ha), add3(q, hj), sub3(q, hj)) < in2;
    }
    if (t) return norm2(sub3(add3(pb, *t), pa)) < in2;
    return pbc_distance2(s.box, s.inv, pa, pb) < in2;
}

// FP32 separation q - p (FP64 points) at image m, against the pre-filter reach.
__device__ __forceinline__ bool within_reach(const SingleArgs &A, const double *q, const double *p, int mx, int my,
                                             int mz) {
    const float3 t32 = mat32(A.box32, (float)mx, (float)my, (float)mz);
    const float ex = static_cast<float>(q[0] - p[0]) + t32.x;
    const float ey = static_cast<float>(q[1] - p[1]) + t32.y;
    const float ez = static_cast<float>(q[2] - p[2]) + t32.z;
    return ex * ex + ey * ey + ez * ez <= A.reach2;
}

// Overlapping pairs of the mover state `which` with body j over every periodic image within
// reach (each absolute centre is wrapped into the box on its own, so the images of a body
// pair are enumerated per centre pair); at most 1 with `early`.
template <int KIND>
__device__ int candidate_overlaps(const SingleArgs &A, const SingleShared &sh, int which, int j, bool early) {
    const DevState &s = A.s;
    int cnt = 0;
    if constexpr (KIND != 2) {
        if (s.pbc_fold) return body_overlap<KIND>(s, sh, which, j, nullptr) ? 1 : 0;
        const double *pj = s.pos64 + 3 * (size_t)j;
        for (int mx = -1; mx <= 1; mx++)
            for (int my = -1; my <= 1; my++)
                for (int mz = -1; mz <= 1; mz++) {
                    if (!within_reach(A, pj, sh.pos[which], mx, my, mz)) continue;
                    const d3 t = load_d3(s.trans + 3 * (((mx + 2) * 5 + (my + 2)) * 5 + (mz + 2)));
                    if (body_overlap<KIND>(s, sh, which, j, &t)) {
                        if (early) return 1;
                        cnt++;
                    }
                }
        return cnt;
    } else {
    for (int a = 0; a < s.ncen; a++)
        for (int b = 0; b < s.ncen; b++) {
            if (s.pbc_fold) {
                if (centre_overlap(s, sh, which, a, j, b, nullptr)) {
                    if (early) return 1;
                    cnt++;
                }
                continue;
            }
            const double *pb = s.abs64 + 3 * ((size_t)j * s.ncen + b);
            for (int mx = -1; mx <= 1; mx++)
                for (int my = -1; my <= 1; my++)
                    for (int mz = -1; mz <= 1; mz++) {
                        if (!within_reach(A, pb, sh.abs[which] + 3 * a, mx, my, mz)) continue;
                        const d3 t = load_d3(s.trans + 3 * (((mx + 2) * 5 + (my + 2)) * 5 + (mz + 2)));
                        if (centre_overlap(s, sh, which, a, j, b, &t)) {
                            if (early) return 1;
                            cnt++;
                        }
                    }
        }
    return cnt;
    }
}

// Overlaps of mover state `which` with every candidate (pairs, then walls): the count, or
// 0 / 1 with `early` (Packing::countParticleOverlaps, core/Packing.cpp:373-429).
template <int KIND>
__device__ int state_overlaps(const SingleArgs &A, SingleShared &sh, int which, bool early) {
    const DevState &s = A.s;
    const GridDev &g = A.g;
    const int pid = A.m.particle;
    const int in_cells = sh.cstart[which][sh.ncells[which]];
    const int total = in_cells + A.ndisp;
    int cnt = 0;
    for (int k = threadIdx.x; k < total; k += blockDim.x) {
        if (early && *(volatile int *)&sh.hit) break;
        int j;
        if (k < in_cells) {
            int c = 0;
            while (sh.cstart[which][c + 1] <= k) c++;
            const int cell = sh.cells[which][c];
            j = g.slot_pid[g.start[cell] + (k - sh.cstart[which][c])];
            if (A.disp_flag[j]) continue;  // moved since the grid was built: tested from the list
        } else {
            j = A.disp_list[k - in_cells];
        }
        if (j == pid) continue;  // the self-skip compares particle indices (core/Packing.cpp:633-635)
        const int c = candidate_overlaps<KIND>(A, sh, which, j, early);
        if (c) {
            cnt += c;
            if (early) sh.hit = 1;
        }
    }
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, d);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&sh.count[which], cnt);
    __syncthreads();
    int out = sh.count[which];
    if (early) out = out > 0 ? 1 : 0;
    if (s.walls && !(early && out)) {
        // hard walls after the pairs (core/Packing.cpp:424-428)
        const d3 p{sh.pos[which][0], sh.pos[which][1], sh.pos[which][2]};
        const d3 a{sh.rot[which][2], sh.rot[which][5], sh.rot[which][8]};
        const double *cen = KIND == 2 ? (which == 0 ? sh.cen : s.cen64 + 3 * (size_t)pid * s.ncen) : nullptr;
        out += wall_overlap_count(s.walls, s.wall_vec, s.wall_far, s.wall_half, KIND, s.wall_radius, s.wall_half_len,
                                  p, a, cen, KIND == 2 ? s.ncen : 0, early, KIND == 2 && s.segs ? sh.hax[which] : nullptr);
        if (early) out = out > 0 ? 1 : 0;
    }
    return out;
}

template <int KIND>
__global__ void __launch_bounds__(SINGLE_THREADS) k_try_single(SingleArgs A) {
    __shared__ SingleShared sh;
    const DevState &s = A.s;
    const rp_move &m = A.m;
    const int pid = m.particle;
    const bool counting = s.counting != 0;
    if (threadIdx.x == 0) {
        // the current state and the temp shape (core/Packing.cpp:86-93, 113-116, 137-146)
        const d3 p0 = load_d3(s.pos64 + 3 * (size_t)pid);
        const double *o0 = s.rot64 + 9 * (size_t)pid;
        d3 p1 = p0;
        if (m.type != RP_MOVE_ROTATION) {
            // Shape::translate (core/Shape.cpp:9-12) with PeriodicBoundaryConditions::getCorrection
            const d3 q = add3(p0, d3{m.translation[0], m.translation[1], m.translation[2]});
            p1 = add3(q, pbc_correction(s.box, s.inv, q, nullptr));
        }
        double o1[9];
        for (int e = 0; e < 9; e++) o1[e] = o0[e];
        if (m.type != RP_MOVE_TRANSLATION)  // Shape::rotate: R * O (core/Shape.cpp:14-16)
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) o1[3 * i + j] = mm_elem(m.rotation, o0, i, j);
        sh.pos[0][0] = p1.x, sh.pos[0][1] = p1.y, sh.pos[0][2] = p1.z;
        sh.pos[1][0] = p0.x, sh.pos[1][1] = p0.y, sh.pos[1][2] = p0.z;
        for (int e = 0; e < 9; e++) {
            sh.rot[0][e] = o1[e];
            sh.rot[1][e] = o0[e];
        }
        if (KIND == 2) {
            for (int a = 0; a < s.ncen; a++) {
                // the temp centres, rotated by R (core/Packing.cpp:357-361), and the absolute
                // centres: position + centre with the periodic correction (:1041-1047)
                d3 c = load_d3(s.cen64 + 3 * ((size_t)pid * s.ncen + a));
                if (m.type != RP_MOVE_TRANSLATION) c = mv3(m.rotation, c);
                const d3 q = add3(p1, c);
                const d3 ab = add3(q, pbc_correction(s.box, s.inv, q, nullptr));
                sh.cen[3 * a] = c.x, sh.cen[3 * a + 1] = c.y, sh.cen[3 * a + 2] = c.z;
                sh.abs[0][3 * a] = ab.x, sh.abs[0][3 * a + 1] = ab.y, sh.abs[0][3 * a + 2] = ab.z;
                for (int d = 0; d < 3; d++) sh.abs[1][3 * a + d] = s.abs64[3 * ((size_t)pid * s.ncen + a) + d];
                if (s.segs) {
                    // orientation * half axis (PolyspherocylinderTraits.cpp:118-119)
                    const d3 hb{s.chax[a][0], s.chax[a][1], s.chax[a][2]};
                    const d3 h1 = mv3(o1, hb), h0 = mv3(o0, hb);
                    sh.hax[0][3 * a] = h1.x, sh.hax[0][3 * a + 1] = h1.y, sh.hax[0][3 * a + 2] = h1.z;
                    sh.hax[1][3 * a] = h0.x, sh.hax[1][3 * a + 1] = h0.y, sh.hax[1][3 * a + 2] = h0.z;
                }
            }
        }
        // the ActiveDomain of a translation or rototranslation, tested before any overlap
        // (core/Packing.cpp:94-96, :141-143; ActiveDomain::isInside, core/ActiveDomain.cpp:8-21)
        sh.outside = A.has_domain && m.type != RP_MOVE_ROTATION && !inside_domain(s.inv, p1, A.dom_lo, A.dom_hi);
        for (int w = 0; w < (counting ? 2 : 1); w++) {
            int c[3];
            cell_of(s, A.g, d3{sh.pos[w][0], sh.pos[w][1], sh.pos[w][2]}, c);
            sh.ncells[w] = neighbour_cells(A.g, c, sh.cells[w]);
            int acc = 0;
            for (int q = 0; q < sh.ncells[w]; q++) {
                sh.cstart[w][q] = acc;
                acc += A.g.start[sh.cells[w][q] + 1] - A.g.start[sh.cells[w][q]];
            }
            sh.cstart[w][sh.ncells[w]] = acc;
        }
        sh.hit = 0;
        sh.count[0] = sh.count[1] = 0;
    }
    __syncthreads();
    double dE;
    int delta = 0;
    if (sh.outside) {
        dE = CUDART_INF;
    } else if (counting) {
        // Packing::calculateMoveOverlapEnergy in counting mode (core/Packing.cpp:307-317)
        const int after = state_overlaps<KIND>(A, sh, 0, false);
        const int before = state_overlaps<KIND>(A, sh, 1, false);
        delta = after - before;
        dE = delta < 0 ? -CUDART_INF : (delta > 0 ? CUDART_INF : 0.0);
    } else {
        dE = state_overlaps<KIND>(A, sh, 0, true) ? CUDART_INF : 0.0;
    }
    if (threadIdx.x == 0) {
        SingleTry *o = A.out;
        for (int d = 0; d < 3; d++) o->pos[d] = sh.pos[0][d];
        for (int e = 0; e < 9; e++) o->rot[e] = sh.rot[0][e];
        if (KIND == 2)
            for (int q = 0; q < 3 * s.ncen; q++) {
                o->cen[q] = sh.cen[q];
                o->abs[q] = sh.abs[0][q];
            }
        o->dE = dE;
        o->outside = sh.outside;
        o->particle = pid;
        o->type = m.type;
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

}  // namespace

cudaError_t launch_try_single(const SingleArgs &a, cudaStream_t st) {
    if (a.s.kind == 0) k_try_single<0><<<1, SINGLE_THREADS, 0, st>>>(a);
    else if (a.s.kind == 1) k_try_single<1><<<1, SINGLE_THREADS, 0, st>>>(a);
    else k_try_single<2><<<1, SINGLE_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_commit_single(const DevState &s, SingleTry *t, uint8_t *disp_flag, int32_t *disp_list, int slot,
                                 cudaStream_t st) {
    k_commit_single<<<1, 32, 0, st>>>(s, t, disp_flag, disp_list, slot);
    return cudaGetLastError();
}

}  // namespace rp
