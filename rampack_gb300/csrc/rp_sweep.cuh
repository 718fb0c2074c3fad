// Device building blocks of the move-and-overlap path shared by the single-system
// kernels (rp_kernels.cu) and the batched-replica kernels (rp_batch.cu): the FP32 filter
// stages, the exact FP64 pair tests, and the per-cell move sweep of one warp.
#pragma once

#include <cuda_runtime.h>

#include "rp_bulk.cuh"
#include "rp_internal.cuh"

namespace rp {

__device__ __forceinline__ int wrap_cell(int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); }

// Neighbour enumeration: lane 0 is the cell itself, lanes 1..26 the other offsets.
__device__ __forceinline__ void lane_offset(int lane, int &ox, int &oy, int &oz) {
    int t = lane == 0 ? 13 : (lane <= 13 ? lane - 1 : lane);
    ox = t % 3 - 1;
    oy = (t / 3) % 3 - 1;
    oz = t / 9 - 1;
}

__device__ __forceinline__ float3 mat32(const float *m, float x, float y, float z) {
    return make_float3(fmaf(m[0], x, fmaf(m[1], y, m[2] * z)), fmaf(m[3], x, fmaf(m[4], y, m[5] * z)),
                       fmaf(m[6], x, fmaf(m[7], y, m[8] * z)));
}

__device__ __forceinline__ float dot3f(float3 a, float3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }

// A group of GW consecutive lanes that sweeps one cell: the whole warp (GW = 32) or either
// half of it (GW = 16, two cells per warp).  Its votes and shuffles name the group's own lanes
// (lane = 0..GW-1); ballots return group-relative bits, so a group's code reads the same for
// both widths.  With GW = 16 the two halves of a warp run their cells independently.
template <int GW>
struct Grp {
    static_assert(GW == 32 || GW == 16, "a group is a warp or half a warp");
    unsigned mask;  // the group's lanes in the warp
    int base;       // its first lane
    int lane;       // this thread's lane in the group
    __device__ __forceinline__ Grp() {
        const int wl = threadIdx.x & 31;
        base = GW == 32 ? 0 : (wl & 16);
        lane = wl - base;
        mask = GW == 32 ? 0xffffffffu : (0xffffu << base);
    }
    __device__ __forceinline__ unsigned ballot(bool p) const {
        const unsigned b = __ballot_sync(mask, p);
        return GW == 32 ? b : ((b & mask) >> base);
    }
    template <class T>
    __device__ __forceinline__ T shfl(T v, int src) const { return __shfl_sync(mask, v, base + src); }
    template <class T>
    __device__ __forceinline__ T shfl_up(T v, int d) const { return __shfl_up_sync(mask, v, d, GW); }
    template <class T>
    __device__ __forceinline__ T shfl_xor(T v, int d) const { return __shfl_xor_sync(mask, v, d, GW); }
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
};

// ---------------------------------------------------------------------------------
// FP32 classification of one pair.  0: no overlap, 1: overlap, 2: undecided in FP32
// (re-decided in FP64).  d = p_j - p_i (candidate minus mover), a_i/a_j unit axes.
// ---------------------------------------------------------------------------------
// Centre-distance stage: 0 no overlap, 1 overlap, 2 undecided (FP64), 3 needs the
// segment stage (spherocylinders).
template <int KIND>
__device__ __forceinline__ int d2_stage(const FilterConsts &fc, float d2) {
    if (KIND == 0) {
        if (d2 < fc.sphere_lo) return 1;
        if (d2 > fc.sphere_hi) return 0;
        return 2;
    } else if (KIND == 2) {
        // polyspheres: bodies farther apart than twice the largest centre reach cannot
        // touch; closer ones go to the sphere-pair stage
        return d2 > fc.far_hi ? 0 : 3;
    } else {
        if (d2 > fc.far_hi) return 0;
        if (d2 < fc.core_lo) return 1;
        if (d2 < fc.core_hi || d2 > fc.far_lo) return 2;
        return 3;
    }
}

// Segment stage of a spherocylinder pair: the closest points of the two axes (same
// branch structure as the FP64 reference), then a convexity certificate: for any feasible
// (s, t), f* >= f(s, t) - G with G the Frank-Wolfe gap of the box-constrained quadratic.
// 0 no overlap, 1 overlap, 2 undecided (FP64).  d = p_j - p_i, ai/aj unit axes.
__device__ __forceinline__ int seg_stage(const FilterConsts &fc, float3 d, float3 ai, float3 aj) {
    const float l = fc.len, h = fc.half_len;
    float3 u = make_float3(l * ai.x, l * ai.y, l * ai.z);
    float3 v = make_float3(l * aj.x, l * aj.y, l * aj.z);
    float3 w = make_float3(-d.x - h * (ai.x - aj.x), -d.y - h * (ai.y - aj.y), -d.z - h * (ai.z - aj.z));
    float a = dot3f(u, u), b = dot3f(u, v), c = dot3f(v, v), dd = dot3f(u, w), e = dot3f(v, w);
    // D = |u|^2 |v|^2 - (u.v)^2 = |u x v|^2, evaluated without cancellation: nearly parallel
    // axes (D below d_min) are left to FP64, whose own parameter error grows like 1/D
    float3 cr = make_float3(fmaf(u.y, v.z, -u.z * v.y), fmaf(u.z, v.x, -u.x * v.z), fmaf(u.x, v.y, -u.y * v.x));
    float D = dot3f(cr, cr);
    // axes parallel to within d_par: the FP64 reference certainly takes its parallel branch
    // (D < 1e-10: closest points from the s = 0 end), whose distance exceeds the true
    // minimum by at most par_err; in between the two thresholds FP64 decides
    const bool par = D < fc.d_par;
    if (!par && D < fc.d_min) return 2;
    float sN, tN, sD, tD;
    if (par) {
        sN = 0.f; sD = 1.f; tN = e; tD = c;
    } else {
        sN = fmaf(b, e, -c * dd);
        tN = fmaf(a, e, -b * dd);
        sD = D;
        tD = D;
        if (sN < 0.f) {
            sN = 0.f; tN = e; tD = c;
        } else if (sN > sD) {
            sN = sD; tN = e + b; tD = c;
        }
    }
    if (tN < 0.f) {
        tN = 0.f;
        if (-dd < 0.f) sN = 0.f;
        else if (-dd > a) sN = sD;
        else { sN = -dd; sD = a; }
    } else if (tN > tD) {
        tN = tD;
        if (b - dd < 0.f) sN = 0.f;
        else if (b - dd > a) sN = sD;
        else { sN = b - dd; sD = a; }
    }
    float sc = fminf(fmaxf(__fdividef(sN, sD), 0.f), 1.f);
    float tc = fminf(fmaxf(__fdividef(tN, tD), 0.f), 1.f);
    float3 dP = make_float3(fmaf(sc, u.x, fmaf(-tc, v.x, w.x)), fmaf(sc, u.y, fmaf(-tc, v.y, w.y)),
                            fmaf(sc, u.z, fmaf(-tc, v.z, w.z)));
    float f = dot3f(dP, dP);
    float gs = dot3f(dP, u), gt = -dot3f(dP, v);
    float G = 2.f * (gs * sc - fminf(gs, 0.f) + gt * tc - fminf(gt, 0.f));
    const float err = par ? fc.seg_err + fc.par_err : fc.seg_err;
    if (f + err < fc.core_thr) return 1;
    if (f - G - err >= fc.core_thr) return 0;
    return 2;
}

// FP32 classification of one pair: 0 no overlap, 1 overlap, 2 undecided in FP32.
template <int KIND>
__device__ __forceinline__ int classify(const FilterConsts &fc, float3 d, float3 ai, float3 aj) {
    int cls = d2_stage<KIND>(fc, dot3f(d, d));
    if (KIND == 1 && cls == 3) cls = seg_stage(fc, d, ai, aj);
    return cls;
}

// FP32 classification of one candidate body against the mover's moved FP32 centres (the
// centre-pair stage of multi-centre bodies): dq = candidate body - mover body position,
// cj its FP32 centres, wx the mover's, thr the centre-pair thresholds (lo block, then hi
// block).  1 a certain overlap, 2 undecided (FP64), 0 none.
__device__ __forceinline__ int poly_body_class(int K, const float4 *wx, const float *thr, float3 dq, const float4 *cj) {
    int cls = 0;
    for (int j = 0; j < K && cls != 1; j++) {
        const float4 c = cj[j];
        const float3 bj = make_float3(dq.x + c.x, dq.y + c.y, dq.z + c.z);
        for (int a = 0; a < K; a++) {
            const float4 m = wx[a];
            const float3 d = make_float3(bj.x - m.x, bj.y - m.y, bj.z - m.z);
            const float d2 = dot3f(d, d);
            if (d2 < thr[a * MAX_CEN + j]) {
                cls = 1;
                break;
            }
            if (d2 <= thr[MAX_CEN * MAX_CEN + a * MAX_CEN + j]) cls = 2;
        }
    }
    return cls;
}

// Image of candidate j relative to mover i, recovered from the FP32 separation dsep
// (candidate minus mover, in the right image) and the FP64 positions: the integer box
// translation m with p_j + box·m - p_i ≈ dsep.  Returns the index into the translation table.
__device__ __forceinline__ int image_index(const DevState &s, float3 dsep, d3 pi, d3 pj) {
    float3 raw = make_float3(static_cast<float>(pj.x - pi.x), static_cast<float>(pj.y - pi.y),
                             static_cast<float>(pj.z - pi.z));
    float3 rel = mat32(s.inv32, dsep.x - raw.x, dsep.y - raw.y, dsep.z - raw.z);
    int mx = __float2int_rn(rel.x), my = __float2int_rn(rel.y), mz = __float2int_rn(rel.z);
    mx = max(-2, min(2, mx));
    my = max(-2, min(2, my));
    mz = max(-2, min(2, mz));
    return ((mx + 2) * 5 + (my + 2)) * 5 + (mz + 2);
}

__device__ __forceinline__ d3 load_d3(const double *p) { return d3{p[0], p[1], p[2]}; }

// Exact FP64 test of mover (pi, ai) against particle pid_j seen at FP32 separation dsep.
// With no neighbour grid (s.pbc_fold) the reference tests each pair once, at its nearest
// image; a box of two cells across stages a candidate once per image, so only the staged
// copy that is the nearest image (relative separation within 1/2 in every dimension) is
// tested.  The other copy lies at least half a box height away, beyond the interaction
// range of the boxes this engine accepts.
__device__ __forceinline__ bool nearest_copy(const DevState &s, float3 dsep) {
    const float3 r = mat32(s.inv32, dsep.x, dsep.y, dsep.z);
    const float h = 0.5f + 1e-5f;
    return fabsf(r.x) <= h && fabsf(r.y) <= h && fabsf(r.z) <= h;
}

__device__ __forceinline__ bool exact_pair(const DevState &s, d3 pi, d3 ai, int pid_j, float3 dsep) {
    d3 pj = load_d3(s.pos64 + 3 * (size_t)pid_j);
    const double *rj = s.rot64 + 9 * (size_t)pid_j;
    d3 aj = d3{rj[2], rj[5], rj[8]};
    if (s.kind == 0 && s.pbc_fold) return nearest_copy(s, dsep) && pbc_distance2(s.box, s.inv, pi, pj) < s.ex.sphere_thr;
    int m = image_index(s, dsep, pi, pj);
    d3 t = load_d3(s.trans + 3 * m);
    return exact_overlap(s.ex, pi, ai, pj, aj, t);
}


// Exact FP64 test of centre a of a body, at absolute position pa, against centre j of
// body pid_j seen at FP32 separation dsep (candidate minus mover): the reference's
// (pos2 + t - pos1).norm2() < (r_a + r_j)^2 (core/Packing.cpp:40-42,
// core/shapes/PolysphereTraits.cpp:97-106) with t the box translation of that image.
// Polyspherocylinders (s.segs): PolyspherocylinderTraits::overlapBetween
// (core/shapes/PolyspherocylinderTraits.cpp:102-124) with the image's translation (the
// periodic boundary conditions' own when the reference keeps no grid): inspheres,
// circumspheres, then the distance of the segments centre -+ orientation * half axis; `ha`
// is the half axis of centre a of the first body (orientation already applied).
__device__ __forceinline__ bool exact_centre_pair(const DevState &s, d3 pa, int a, int pid_j, int j, float3 dsep,
                                                  d3 ha = d3{0.0, 0.0, 0.0}) {
    d3 pb = load_d3(s.abs64 + 3 * ((size_t)pid_j * s.ncen + j));
    if (s.pbc_fold && !nearest_copy(s, dsep)) return false;
    if (s.segs) {
        d3 t = s.pbc_fold ? pbc_translation(s.box, s.inv, pa, pb) : load_d3(s.trans + 3 * image_index(s, dsep, pa, pb));
        d3 q = add3(pb, t);
        double d2 = norm2(sub3(q, pa));
        const double in2 = s.cthr64[a * MAX_CEN + j];
        if (d2 < in2) return true;
        if (d2 >= s.circ64[a * MAX_CEN + j]) return false;
        d3 hj = mv3(s.rot64 + 9 * (size_t)pid_j, d3{s.chax[j][0], s.chax[j][1], s.chax[j][2]});
        return segment_distance2(add3(pa, ha), sub3(pa, ha), add3(q, hj), sub3(q, hj)) < in2;
    }
    if (s.pbc_fold) return pbc_distance2(s.box, s.inv, pa, pb) < s.cthr64[a * MAX_CEN + j];
    int m = image_index(s, dsep, pa, pb);
    d3 t = load_d3(s.trans + 3 * m);
    d3 d = sub3(add3(pb, t), pa);
    return norm2(d) < s.cthr64[a * MAX_CEN + j];
}

// ---------------------------------------------------------------------------------
// Checkerboard sweep: one warp per active cell.
//
// Per move, all lanes draw (or read) the same proposal; the FP32 pass tests the staged
// neighbourhood 32 candidates at a time with a ballot for the early exit.  Pass 1 decides
// on the centre distance alone and compacts the spherocylinder pairs that need the
// segment test into a shared-memory queue, so that pass 2 runs the segment test on full
// warps.  Pairs the FP32 filter cannot decide go to a second queue; only a move that
// survives the FP32 filter builds its exact FP64 state (one box row per lane, one matrix
// entry per lane), re-decides the queued pairs in FP64 and, when accepted, writes back.
// ---------------------------------------------------------------------------------
struct WarpStats {
    unsigned moves, accepted, rej_overlap, rej_domain, pairs, fp64, trans, rots, acc_trans;
    // bulk staging (whole warps): the group's barrier (null: per-lane loads), the parity of
    // its next phase, and whether a copy timed out (the group then stops)
    uint64_t *bar;
    unsigned bphase;
    int abort;
};

// Polls of a staging barrier before its copies count as lost (~0.1 s).
constexpr int STAGE_WAIT_LIMIT = 1 << 21;

// MODE 0: plain sweep; 1: learned-ordering pre-test and pair log; 2: overlap counting
// (Packing::toggleOverlapCounting, core/Packing.cpp:304-323: the move's energy is the sign of
// the change of the mover's overlap count).
template <int KIND, bool LIST, int MODE, int GW = 32>
__device__ __forceinline__ void sweep_cell(const SweepArgs &A, const int item, const int cell_direct, const int cap,
                                           int32_t *ovf, int32_t *ovf_count, float4 *cpos, float4 *cax,
                                           uint16_t *qseg, uint16_t *qun, uint8_t *nacc, uint16_t *pstage,
                                           uint32_t *cslot, float4 *wx, WarpStats &ws) {
    constexpr bool LEARN = MODE == 1;
    constexpr bool COUNT = MODE == 2;
    constexpr bool RT = MODE == 3;  // every move a rototranslation (the plain scan otherwise)
    const Grp<GW> grp;
    const int lane = grp.lane;
    // two cells per warp (GW = 16): spherocylinder axes are read from the L2-resident FP32
    // mirror through each candidate's mirror slot instead of being staged, which halves the
    // shared memory per cell
    constexpr bool AXM = GW == 16 && KIND == 1;
    const unsigned lt = (1u << lane) - 1u;
    const DevState &S = A.s;
    const GridDev &G = A.g;

    // ---- which cell ----
    int cell, c[3];
    if (cell_direct >= 0) {
        cell = cell_direct;
    } else if (A.work) {
        cell = A.work[item];
    } else if (LIST) {
        cell = A.list_cells[item];
    } else {
        int w = item;
        int a0 = w % A.active[0];
        w /= A.active[0];
        int a1 = w % A.active[1];
        int a2 = w / A.active[1];
        int cc[3] = {a0, a1, a2};
        for (int d = 0; d < 3; d++) c[d] = ring_cell(G.dims[d], A.phase[d], cc[d]);
        cell = c[0] + G.dims[0] * (c[1] + G.dims[1] * c[2]);
    }
    c[0] = cell % G.dims[0];
    c[1] = (cell / G.dims[0]) % G.dims[1];
    c[2] = cell / (G.dims[0] * G.dims[1]);

    // ---- stage the 3x3x3 neighbourhood (own cell first): neighbour cell lane + GW r ----
    constexpr int NR = 32 / GW;  // neighbour cells per lane (27 cells over the group's lanes)
    int cnt[NR], st[NR], kcnt[NR], pre[NR];
    float3 off[NR];
    // with the staging filter, a neighbour cell's particles farther than the interaction
    // range from the home cell (whose movers stay inside it: the cell is their ActiveDomain)
    // are left out; the own cell (neighbour 0) is always staged whole
    const bool filt = G.stage_filter && !LEARN;
    auto keep = [&](const float4 &p, const float3 &o) {
        const float3 f = mat32(G.cellinv, p.x + o.x, p.y + o.y, p.z + o.z);
        const float e0 = fmaxf(fmaxf(-f.x, f.x - 1.f), 0.f) * G.stage_h[0];
        const float e1 = fmaxf(fmaxf(-f.y, f.y - 1.f), 0.f) * G.stage_h[1];
        const float e2 = fmaxf(fmaxf(-f.z, f.z - 1.f), 0.f) * G.stage_h[2];
        return fmaxf(e0, fmaxf(e1, e2)) <= G.stage_thr;
    };
    int total = 0;
#pragma unroll
    for (int r = 0; r < NR; r++) {
        const int nbl = lane + GW * r;
        cnt[r] = 0;
        st[r] = 0;
        off[r] = make_float3(0.f, 0.f, 0.f);
        if (nbl < 27) {
            int ox, oy, oz;
            lane_offset(nbl, ox, oy, oz);
            int nb = wrap_cell(c[0] + ox, G.dims[0]) +
                     G.dims[0] * (wrap_cell(c[1] + oy, G.dims[1]) + G.dims[1] * wrap_cell(c[2] + oz, G.dims[2]));
            st[r] = G.start[nb];
            cnt[r] = G.start[nb + 1] - st[r];
            off[r] = mat32(G.cellmat, (float)ox, (float)oy, (float)oz);
        }
        kcnt[r] = cnt[r];
        if (filt && nbl > 0 && nbl < 27) {
            kcnt[r] = 0;
            for (int k = 0; k < cnt[r]; k++) kcnt[r] += keep(G.mpos[st[r] + k], off[r]) ? 1 : 0;
        }
        int incl = kcnt[r];
        for (int d = 1; d < GW; d <<= 1) {
            int y = grp.shfl_up(incl, d);
            if (lane >= d) incl += y;
        }
        pre[r] = total + incl - kcnt[r];
        total += grp.shfl(incl, GW - 1);
    }
    const int occ = grp.shfl(cnt[0], 0);
    const int gbase = grp.shfl(st[0], 0);
    if (total > cap) {
        if (lane == 0) {
            if (ovf) {
                int k = atomicAdd(ovf_count, 1);
                ovf[k] = cell;
            } else {
                atomicOr(S.status, ST_CAPACITY);
            }
        }
        return;
    }
    const bool bulk = GW == 32 && !filt && ws.bar != nullptr;
    if (bulk) {
        // bulk staging: one copy per neighbour cell and array (a cell is a contiguous run of
        // the slot-ordered mirror; float4 records, so addresses and sizes are multiples of
        // 16 bytes), all in flight at once on the group's barrier; then each lane shifts its
        // cell's staged positions into the home cell's frame, as the per-lane copy does
        constexpr bool WITH_AX = KIND == 1 && !AXM;
        fence_proxy_async_smem();  // this lane's reads and writes of the buffers come first
        grp.sync();
        if (lane == 0) mbar_arrive_expect_tx(ws.bar, (uint32_t)total * (WITH_AX ? 32u : 16u));
        grp.sync();
        if (lane < 27 && cnt[0] > 0) {
            bulk_g2s(cpos + pre[0], G.mpos + st[0], (uint32_t)cnt[0] * 16u, ws.bar);
            if (WITH_AX) bulk_g2s(cax + pre[0], G.maxis + st[0], (uint32_t)cnt[0] * 16u, ws.bar);
        }
        if (KIND == 2 || AXM)
            for (int k = 0; k < cnt[0]; k++) cslot[pre[0] + k] = (uint32_t)(st[0] + k);
        const bool landed = mbar_wait(ws.bar, ws.bphase, STAGE_WAIT_LIMIT);
        if (grp.ballot(!landed)) {
            // lost copies: flag, give those in flight a last bounded wait, stop the group
            if (lane == 0) atomicOr(S.status, ST_STAGE_TIMEOUT);
            mbar_wait(ws.bar, ws.bphase, STAGE_WAIT_LIMIT);
            ws.abort = 1;
            return;
        }
        ws.bphase ^= 1u;
        if (lane < 27)
            for (int k = 0; k < cnt[0]; k++) {
                float4 &p = cpos[pre[0] + k];
                p.x += off[0].x;
                p.y += off[0].y;
                p.z += off[0].z;
            }
    }
#pragma unroll
    for (int r = 0; r < NR && !bulk; r++) {
        const int nbl = lane + GW * r;
        if (!filt) {
            // every neighbour staged: positions known from the prefix sum (loads pipeline freely)
            const int base = pre[r];
            for (int k = 0; k < cnt[r]; k++) {
                float4 p = G.mpos[st[r] + k];
                p.x += off[r].x;
                p.y += off[r].y;
                p.z += off[r].z;
                cpos[base + k] = p;
                if (KIND == 1 && !AXM) cax[base + k] = G.maxis[st[r] + k];
                if (KIND == 2 || AXM) cslot[base + k] = (uint32_t)(st[r] + k);  // its centres stay in the L2-resident mirror
            }
        } else {
            int j = pre[r];
            for (int k = 0; k < cnt[r]; k++) {
                float4 p = G.mpos[st[r] + k];
                if (nbl > 0 && !keep(p, off[r])) continue;
                p.x += off[r].x;
                p.y += off[r].y;
                p.z += off[r].z;
                cpos[j] = p;
                if (KIND == 1 && !AXM) cax[j] = G.maxis[st[r] + k];
                if (KIND == 2 || AXM) cslot[j] = (uint32_t)(st[r] + k);
                j++;
            }
        }
    }
    // polyspheres: the warp's scratch holds the mover's FP32 centres (wx[0..K)), the
    // centre-pair thresholds (lo, hi) and the mover's exact new centres and absolute centres
    float *wthr = reinterpret_cast<float *>(wx + MAX_CEN);
    double *wabs = reinterpret_cast<double *>(wx + MAX_CEN + MAX_CEN * MAX_CEN / 2);
    double *wcen = wabs + 3 * MAX_CEN;
    double *whax = wcen + 3 * MAX_CEN;   // polyspherocylinders: the mover's rotated half axes
    if (KIND == 2)
        for (int t = lane; t < 2 * MAX_CEN * MAX_CEN; t += GW) wthr[t] = G.cthr[t];
    const bool self_images = (G.dims[0] == 1) || (G.dims[1] == 1) || (G.dims[2] == 1);
    // per own-cell particle: FP32 roundings accumulated in its mirror position this sweep
    for (int k = lane; k < occ; k += GW) nacc[k] = 0;
    if (LEARN && A.partners) {
        // the ranked partners of the cell's particles, as indices into the staged
        // neighbourhood (a partner out of reach of this cell's neighbourhood gets none)
        static_assert(!LEARN || GW == 32, "the partner pre-test stages with whole warps");
        const int base_nb = pre[0];
        for (int eb = 0; eb < occ * MLP_PARTNERS; eb += GW) {
            const int e = eb + lane;
            int sj = -1;
            if (e < occ * MLP_PARTNERS) {
                const int pk = __float_as_int(cpos[e / MLP_PARTNERS].w);
                const int pj = A.partners[MLP_PARTNERS * (size_t)pk + e % MLP_PARTNERS];
                if (pj >= 0) sj = G.pid_slot[pj];
            }
            int idx = 0xffff;
            for (int nb = 0; nb < 27; nb++) {
                const int s0 = grp.shfl(st[0], nb), c0 = grp.shfl(cnt[0], nb),
                          b0 = grp.shfl(base_nb, nb);
                if (idx == 0xffff && sj >= s0 && sj < s0 + c0) idx = b0 + sj - s0;
            }
            if (e < occ * MLP_PARTNERS) pstage[e] = (uint16_t)idx;
        }
    }
    grp.sync();

    // this lane's dimension (lanes 0-2): ActiveDomain bounds and cell coordinate
    const int ld = lane < 3 ? lane : 0;
    const int c_ld = ld == 0 ? c[0] : (ld == 1 ? c[1] : c[2]);
    const int dims_ld = ld == 0 ? G.dims[0] : (ld == 1 ? G.dims[1] : G.dims[2]);
    const int boff_ld = ld == 0 ? G.boundsoff[0] : (ld == 1 ? G.boundsoff[1] : G.boundsoff[2]);
    const double shift_ld = ld == 0 ? G.shift[0] : (ld == 1 ? G.shift[1] : G.shift[2]);
    const double lo_d = G.bounds[boff_ld + 2 * c_ld];
    const double hi_d = G.bounds[boff_ld + 2 * c_ld + 1];
    // this lane's matrix entry (lanes 0-8)
    const int ei = lane < 9 ? lane / 3 : 0, ej = lane < 9 ? lane % 3 : 0;

    int nmoves, mbeg = 0;
    if (LIST) {
        int li = A.work ? -1 : item;
        if (A.work) {
            for (int q = 0; q < A.num_list; q++)
                if (A.list_cells[q] == cell) li = q;
        }
        mbeg = A.list_begin[li];
        nmoves = A.list_begin[li + 1] - mbeg;
    } else {
        nmoves = sweep_move_types(A.types) * occ;
    }
    const int ntypes = sweep_move_types(A.types);

    u4 rnd_lane = u4{0u, 0u, 0u, 0u};  // Philox output of move (batch base + lane)
    for (int mi = 0; mi < nmoves; mi++) {
        if (!LIST && (mi & (GW - 1)) == 0) {
            // draw the next GW moves' random words at once, one move per lane (the words
            // of a move depend only on its index and cell, whatever the group width)
            rnd_lane = philox(u4{(uint32_t)(mi + lane), (uint32_t)cell, (uint32_t)A.counter,
                                 (uint32_t)(A.counter >> 32)},
                              (uint32_t)A.seed, (uint32_t)(A.seed >> 32));
        }
        // ---- the proposal (FP32 view; FP64 inputs kept for the exact path) ----
        int type, slot = -1, out_index = -1;
        double uni = 0.5;
        double t64_lane = 0.0;      // translation component of this lane's dimension
        float3 t32 = make_float3(0.f, 0.f, 0.f);
        float R32[9];
        uint32_t rot_idx = 0;       // drawn rotation: table entry and transpose flag
        bool rot_inv = false;
        const rp_move *mrec = nullptr;
        if (LIST) {
            out_index = A.move_out[mbeg + mi];
            mrec = A.moves + out_index;
            type = mrec->type;
            int want = mrec->particle;
            for (int kb = 0; kb < occ; kb += GW) {
                int k = kb + lane;
                bool hit = k < occ && __float_as_int(cpos[k].w) == want;
                unsigned bal = grp.ballot(hit);
                if (bal) {
                    slot = kb + __ffs(bal) - 1;
                    break;
                }
            }
            if (slot < 0) {
                if (lane == 0) {
                    atomicOr(S.status, ST_PARTICLE_NOT_IN_CELL);
                    if (A.codes) A.codes[out_index] = 0xff;
                }
                continue;
            }
            t32 = make_float3((float)mrec->translation[0], (float)mrec->translation[1], (float)mrec->translation[2]);
            t64_lane = mrec->translation[ld];
            uni = mrec->uniform;
            for (int q = 0; q < 9; q++) R32[q] = (float)mrec->rotation[q];
        } else {
            const int src = mi & (GW - 1);
            u4 r = u4{grp.shfl(rnd_lane.a, src), grp.shfl(rnd_lane.b, src),
                      grp.shfl(rnd_lane.c, src), grp.shfl(rnd_lane.d, src)};
            const bool rt = RT || (COUNT && A.types == SWEEP_ROTOTRANSLATION);
            if (rt) type = 2;
            else if (ntypes == 2) type = (r.a >> 31) ? 1 : 0;
            else type = (A.types & 1) ? 0 : 1;
            slot = (int)(((uint64_t)(r.a & 0x7fffffffu) * (uint32_t)occ) >> 31);
            if (type == 0 || rt) {
                // pm1f takes the top 24 bits of a word: a rototranslation's rotation takes
                // the low bytes
                t32 = make_float3(pm1f(r.b) * A.tstep, pm1f(r.c) * A.tstep, pm1f(r.d) * A.tstep);
                t64_lane = ld == 0 ? (double)t32.x : (ld == 1 ? (double)t32.y : (double)t32.z);
            }
            if (type != 0) {
                // a rotation of this sweep's table, or its transpose (the inverse)
                if (rt) {
                    rot_idx = ((r.b & 0xffu) | ((r.c & 0xffu) << 8)) & A.rtab_mask;
                    rot_inv = (r.d & 1u) != 0;
                } else {
                    rot_idx = r.b & A.rtab_mask;
                    rot_inv = (r.c & 1u) != 0;
                }
                if (KIND >= 1) {
                    const float4 *R4 = reinterpret_cast<const float4 *>(A.rtab32) + 3 * (size_t)rot_idx;
                    float4 x0 = R4[0], x1 = R4[1], x2 = R4[2];
                    float R[9] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w, x2.x};
                    for (int q = 0; q < 9; q++) R32[q] = rot_inv ? R[3 * (q % 3) + q / 3] : R[q];
                }
            }
        }
        const float4 pcur = cpos[slot];
        const int pid = __float_as_int(pcur.w);
        // the mover's FP64 state, loaded now and first used after the FP32 filter:
        // lanes 0-2 hold the position, lanes 0-8 the orientation entries
        const double pos_own = S.pos64[3 * (size_t)pid + ld];
        const double rot_own = S.rot64[9 * (size_t)pid + (lane < 9 ? lane : 0)];
        float3 ai = make_float3(0.f, 0.f, 1.f);
        if (KIND == 1) {
            float4 a = AXM ? G.maxis[(size_t)gbase + slot] : cax[slot];
            ai = make_float3(a.x, a.y, a.z);
        }
        float3 pn = make_float3(pcur.x, pcur.y, pcur.z);
        float3 an = ai;
        if (type != 1) pn = make_float3(pcur.x + t32.x, pcur.y + t32.y, pcur.z + t32.z);
        if (type != 0 && KIND == 1) an = mat32(R32, ai.x, ai.y, ai.z);
        if (KIND == 2) {
            // the mover's FP32 centres after the move (rotated by the FP32 rotation)
            if (lane < S.ncen) {
                const float4 c = G.mcen[((size_t)gbase + slot) * S.ncen + lane];
                float3 cn = make_float3(c.x, c.y, c.z);
                if (type != 0) cn = mat32(R32, cn.x, cn.y, cn.z);
                wx[lane] = make_float4(cn.x, cn.y, cn.z, 0.f);
            }
            grp.sync();
        }

        // ---- FP32 ActiveDomain test (translations): 0 inside, 1 outside, 2 undecided;
        //      and whether the PBC correction may move the particle through the box ----
        int dom = 0;
        float3 fnew = make_float3(0.f, 0.f, 0.f);
        if (type != 1) {
            fnew = mat32(G.cellinv, pn.x, pn.y, pn.z);
            float fm[3] = {fnew.x, fnew.y, fnew.z};
            const float mg = S.fc.cell_margin;
            for (int d = 0; d < 3; d++) {
                if (G.dims[d] > 1) {
                    if (fm[d] < -mg || fm[d] > 1.f + mg) dom = 1;
                    else if (dom == 0 && (fm[d] < mg || fm[d] > 1.f - mg)) dom = 2;
                }
            }
        }

        // ---- learned ordering: pre-test the mover's best-ranked partners ----
        // (the staged candidate and the FP32 arithmetic of the full scan, so a certain
        // overlap here is one the scan would find)
        bool overlap = false;
        if (LEARN && A.partners && dom != 1 && !A.fp64_only) {
            int cls = 0;
            bool tested = false;
            if (lane < MLP_PARTNERS) {
                const int k = pstage[MLP_PARTNERS * slot + lane];
                if (k != 0xffff) {
                    const float4 q = cpos[k];
                    if (__float_as_int(q.w) != pid) {
                        const float3 dq = make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z);
                        if (KIND == 2) {
                            // the partner body's centre pairs against the mover's moved centres
                            if (d2_stage<2>(S.fc, dot3f(dq, dq)) == 3)
                                cls = poly_body_class(S.ncen, wx, wthr, dq, G.mcen + (size_t)cslot[k] * S.ncen);
                        } else {
                            float3 aj = make_float3(0.f, 0.f, 1.f);
                            if (KIND == 1) {
                                const float4 a = cax[k];
                                aj = make_float3(a.x, a.y, a.z);
                            }
                            cls = classify<KIND>(S.fc, dq, an, aj);
                        }
                        tested = true;
                    }
                }
            }
            const unsigned nt = __popc(grp.ballot(tested));
            if (lane == 0) ws.pairs += nt;
            if (grp.ballot(cls == 1)) overlap = true;
        }

        // ---- FP32 pass 1: centre distances, SWEEP_P1 candidates per lane per round (independent
        //      tests in flight), queued in candidate order ----
        int nseg = 0, nun = 0;
        if (!COUNT && dom != 1 && !overlap) {
            for (int base = 0; base < total; base += SWEEP_P1 * GW) {
                int cl[SWEEP_P1];
#pragma unroll
                for (int u = 0; u < SWEEP_P1; u++) {
                    const int k = base + u * GW + lane;
                    cl[u] = 0;
                    if (k < total) {
                        const float4 q = cpos[k];
                        if (__float_as_int(q.w) != pid) {
                            const float dx = q.x - pn.x, dy = q.y - pn.y, dz = q.z - pn.z;
                            cl[u] = A.fp64_only ? 2 : d2_stage<KIND>(S.fc, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                        }
                    }
                }
                if (lane == 0) ws.pairs += (unsigned)min(SWEEP_P1 * GW, total - base);
                bool hit = false;
#pragma unroll
                for (int u = 0; u < SWEEP_P1; u++) hit = hit || cl[u] == 1;
                if (grp.ballot(hit)) {
                    overlap = true;
                    break;
                }
#pragma unroll
                for (int u = 0; u < SWEEP_P1; u++) {
                    const int k = base + u * GW + lane;
                    if (KIND >= 1) {
                        const unsigned bs = grp.ballot(cl[u] == 3);
                        if (cl[u] == 3) qseg[nseg + __popc(bs & lt)] = (uint16_t)k;
                        nseg += __popc(bs);
                    }
                    const unsigned bu = grp.ballot(cl[u] == 2);
                    if (cl[u] == 2) qun[nun + __popc(bu & lt)] = (uint16_t)k;
                    nun += __popc(bu);
                }
            }
        }
        grp.sync();
        // ---- FP32 pass 2 (polyspheres): every centre pair of a near body, one body per lane ----
        if (!COUNT && KIND == 2 && !overlap) {
            const int K = S.ncen;
            for (int base = 0; base < nseg; base += GW) {
                const int i = base + lane;
                int cls = 0, k = 0;
                if (i < nseg) {
                    k = qseg[i];
                    const float4 q = cpos[k];
                    cls = poly_body_class(K, wx, wthr, make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z),
                                          G.mcen + (size_t)cslot[k] * K);
                }
                if (LEARN && A.pair_every > 0 && ((mi + cell) % A.pair_every) == 0) {
                    // training data of the ranking network: the body pair as it was before
                    // the move (whole orientations: the bodies are bent), labelled with the
                    // certain outcome after it
                    const bool rec = i < nseg && cls != 2;
                    const unsigned bal = grp.ballot(rec);
                    unsigned long long base_idx = 0;
                    if (lane == 0 && bal) base_idx = atomicAdd(A.pair_count, (unsigned long long)__popc(bal));
                    base_idx = grp.shfl(base_idx, 0);
                    const unsigned long long idx = base_idx + __popc(bal & lt);
                    float ri[9];
                    for (int e = 0; e < 9; e++) ri[e] = (float)grp.shfl(rot_own, e);
                    if (rec && idx < A.pair_cap) {
                        const float4 q = cpos[k];
                        const double *oj = S.rot64 + 9 * (size_t)__float_as_int(q.w);
                        float rj[9];
                        for (int e = 0; e < 9; e++) rj[e] = (float)oj[e];
                        float f[MLP_IN];
                        mlp_features_body(make_float3(q.x - pcur.x, q.y - pcur.y, q.z - pcur.z), ri, rj, A.inv_range,
                                          f);
                        float4 *dst = reinterpret_cast<float4 *>(A.pair_feats + idx * MLP_IN);
                        dst[0] = make_float4(f[0], f[1], f[2], f[3]);
                        dst[1] = make_float4(f[4], f[5], f[6], f[7]);
                        dst[2] = make_float4(f[8], f[9], f[10], f[11]);
                        dst[3] = make_float4(f[12], f[13], f[14], f[15]);
                        A.pair_labels[idx] = cls == 1 ? 1 : 0;
                    }
                }
                if (grp.ballot(cls == 1)) {
                    overlap = true;
                    break;
                }
                unsigned b2 = grp.ballot(cls == 2);
                if (cls == 2) qun[nun + __popc(b2 & lt)] = (uint16_t)k;
                nun += __popc(b2);
            }
            grp.sync();
        }
        // ---- FP32 pass 2 (spherocylinders): segment distances on full warps, two per lane per
        //      round (the queued order; the learned-ordering log keeps one per lane) ----
        if (!COUNT && KIND == 1 && !overlap && !LEARN) {
            for (int base = 0; base < nseg; base += 2 * GW) {
                int cls[2] = {0, 0}, kk[2] = {0, 0};
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const int i = base + u * GW + lane;
                    if (i < nseg) {
                        kk[u] = qseg[i];
                        const float4 q = cpos[kk[u]];
                        const float4 a = AXM ? G.maxis[cslot[kk[u]]] : cax[kk[u]];
                        cls[u] = seg_stage(S.fc, make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z), an,
                                           make_float3(a.x, a.y, a.z));
                    }
                }
                if (grp.ballot(cls[0] == 1 || cls[1] == 1)) {
                    overlap = true;
                    break;
                }
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const unsigned b2 = grp.ballot(cls[u] == 2);
                    if (cls[u] == 2) qun[nun + __popc(b2 & lt)] = (uint16_t)kk[u];
                    nun += __popc(b2);
                }
            }
            grp.sync();
        }
        if (!COUNT && KIND == 1 && !overlap && LEARN) {
            for (int base = 0; base < nseg; base += GW) {
                int i = base + lane;
                int cls = 0, k = 0;
                if (i < nseg) {
                    k = qseg[i];
                    float4 q = cpos[k];
                    float4 a = AXM ? G.maxis[cslot[k]] : cax[k];
                    cls = seg_stage(S.fc, make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z), an,
                                    make_float3(a.x, a.y, a.z));
                }
                if (LEARN && A.pair_every > 0 && ((mi + cell) % A.pair_every) == 0) {
                    // training data of the ranking network: the pair as it was before the
                    // move, labelled with the certain outcome after it
                    const bool rec = i < nseg && cls != 2;
                    const unsigned bal = grp.ballot(rec);
                    unsigned long long base_idx = 0;
                    if (lane == 0 && bal) base_idx = atomicAdd(A.pair_count, (unsigned long long)__popc(bal));
                    base_idx = grp.shfl(base_idx, 0);
                    const unsigned long long idx = base_idx + __popc(bal & lt);
                    if (rec && idx < A.pair_cap) {
                        float4 q = cpos[k];
                        float4 a = AXM ? G.maxis[cslot[k]] : cax[k];
                        float f[MLP_IN];
                        mlp_features(make_float3(q.x - pcur.x, q.y - pcur.y, q.z - pcur.z), ai,
                                     make_float3(a.x, a.y, a.z), A.inv_range, f);
                        float4 *dst = reinterpret_cast<float4 *>(A.pair_feats + idx * MLP_IN);
                        dst[0] = make_float4(f[0], f[1], f[2], f[3]);
                        dst[1] = make_float4(f[4], f[5], f[6], f[7]);
                        dst[2] = make_float4(f[8], f[9], f[10], f[11]);
                        dst[3] = make_float4(f[12], f[13], f[14], f[15]);
                        A.pair_labels[idx] = cls == 1 ? 1 : 0;
                    }
                }
                if (grp.ballot(cls == 1)) {
                    overlap = true;
                    break;
                }
                unsigned b2 = grp.ballot(cls == 2);
                if (cls == 2) qun[nun + __popc(b2 & lt)] = (uint16_t)k;
                nun += __popc(b2);
            }
            grp.sync();
        }

        uint8_t code = dom == 1 ? 2 : (overlap ? 1 : 0);
        // ---- FP64: the exact proposal of a surviving move (or of an accepted u == 0 move) ----
        // (an overlap found near the cell wall still needs the exact ActiveDomain test: the
        // reference rejects a move that leaves the domain before it tests any overlap)
        const bool need64 = (code == 0) || (uni <= 0.0) || (dom == 2);
        const bool needR = type != 0 && (need64 || A.log != nullptr);
        double rel_own = 0.0, pnew_own = 0.0, onew_own = 0.0, rrow[3] = {0.0, 0.0, 0.0};
        bool exact_rel = false;     // rel_own holds the exact FP64 relative coordinate
        d3 pnew{0, 0, 0}, anew{0, 0, 0};
        if (needR) {
            // row ei of the move's rotation (lanes 0-8 hold rows 0..2 three times over)
            if (LIST) {
                rrow[0] = mrec->rotation[3 * ei];
                rrow[1] = mrec->rotation[3 * ei + 1];
                rrow[2] = mrec->rotation[3 * ei + 2];
            } else {
                const double *R = A.rtab64 + 9 * (size_t)rot_idx;
                rrow[0] = rot_inv ? R[ei] : R[3 * ei];
                rrow[1] = rot_inv ? R[3 + ei] : R[3 * ei + 1];
                rrow[2] = rot_inv ? R[6 + ei] : R[3 * ei + 2];
            }
        }
        if (need64) {
            if (type != 1) {
                // May the PBC correction move the particle through the box?  FP32 relative
                // coordinates of the stored (wrapped) position and of the translated one in
                // the same image: s + (c + f) / n, minus the stored position's wrap k.
                bool maywrap = false;
                {
                    float3 f0 = mat32(G.cellinv, pcur.x, pcur.y, pcur.z);
                    float fm[3] = {fnew.x, fnew.y, fnew.z}, fo[3] = {f0.x, f0.y, f0.z};
                    const float mg = S.fc.cell_margin;
                    for (int d = 0; d < 3; d++) {
                        float rold = G.fshift[d] + ((float)c[d] + fo[d]) * G.finv_dims[d];
                        float rnew = G.fshift[d] + ((float)c[d] + fm[d]) * G.finv_dims[d];
                        float k = rold >= 1.f ? 1.f : 0.f;
                        if (fabsf(rold - 1.f) < mg) maywrap = true;
                        rnew -= k;
                        if (rnew < mg || rnew > 1.f - mg) maywrap = true;
                    }
                }
                // Shape::translate with the PBC correction (core/Shape.cpp:9-12,
                // core/PeriodicBoundaryConditions.cpp:11-22), one box row per lane
                if (!LIST) t64_lane = (double)(ld == 0 ? t32.x : (ld == 1 ? t32.y : t32.z));
                double p1 = dadd(pos_own, t64_lane);
                if (!maywrap) {
                    // FP32 shows every relative coordinate clear of 0 and 1: no correction,
                    // which is box · 0 = +0 exactly
                    pnew_own = dadd(p1, 0.0);
                    if (dom == 2) {
                        d3 P1{grp.shfl(p1, 0), grp.shfl(p1, 1), grp.shfl(p1, 2)};
                        rel_own = mrow(S.inv, ld, P1);
                        exact_rel = true;
                    }
                } else {
                    d3 P1{grp.shfl(p1, 0), grp.shfl(p1, 1), grp.shfl(p1, 2)};
                    double rel = mrow(S.inv, ld, P1);
                    double cr = 0.0;
                    while (dadd(rel, cr) < 0.0) cr = dadd(cr, 1.0);
                    while (dadd(rel, cr) >= 1.0) cr = dsub(cr, 1.0);
                    if (grp.ballot(lane < 3 && cr != 0.0) == 0u) {
                        pnew_own = dadd(p1, 0.0);
                        rel_own = rel;
                    } else {
                        d3 C{grp.shfl(cr, 0), grp.shfl(cr, 1), grp.shfl(cr, 2)};
                        pnew_own = dadd(p1, mrow(S.box, ld, C));
                        d3 PN{grp.shfl(pnew_own, 0), grp.shfl(pnew_own, 1),
                              grp.shfl(pnew_own, 2)};
                        rel_own = mrow(S.inv, ld, PN);
                    }
                    exact_rel = true;
                }
                pnew = d3{grp.shfl(pnew_own, 0), grp.shfl(pnew_own, 1), grp.shfl(pnew_own, 2)};
                if (dom == 2) {
                    // ActiveDomain::isInside (core/ActiveDomain.cpp:8-21) on the exact position
                    bool out = false;
                    if (lane < 3 && dims_ld > 1) {
                        if (hi_d > lo_d) out = rel_own <= lo_d || rel_own >= hi_d;
                        else out = rel_own <= lo_d && rel_own >= hi_d;
                    }
                    if (grp.ballot(out)) code = 2;
                }
            } else {
                pnew = d3{grp.shfl(pos_own, 0), grp.shfl(pos_own, 1), grp.shfl(pos_own, 2)};
            }
            if (type != 0) {
                // Shape::rotate: R · O (core/Shape.cpp:14-16, Matrix.tpp:104-113), entry (ei, ej) per lane
                double oe = rot_own;
                double o0 = grp.shfl(oe, ej), o1 = grp.shfl(oe, 3 + ej),
                       o2 = grp.shfl(oe, 6 + ej);
                double s = 0.0;
                s = dadd(s, dmul(rrow[0], o0));
                s = dadd(s, dmul(rrow[1], o1));
                s = dadd(s, dmul(rrow[2], o2));
                onew_own = s;
                anew = d3{grp.shfl(s, 2), grp.shfl(s, 5), grp.shfl(s, 8)};
            } else {
                anew = d3{grp.shfl(rot_own, 2), grp.shfl(rot_own, 5), grp.shfl(rot_own, 8)};
            }
            if (KIND == 2) {
                // the mover's centres: rotated by R (Packing::rotateTempInteractionCentres,
                // core/Packing.cpp:357-361), then position + centre wrapped into the box
                // (core/Packing.cpp:1041-1047); one centre per lane
                double R[9];
                for (int d = 0; d < 3; d++) {
                    R[3 * d] = grp.shfl(rrow[0], 3 * d);
                    R[3 * d + 1] = grp.shfl(rrow[1], 3 * d);
                    R[3 * d + 2] = grp.shfl(rrow[2], 3 * d);
                }
                if (lane < S.ncen) {
                    d3 c = load_d3(S.cen64 + 3 * ((size_t)pid * S.ncen + lane));
                    if (type != 0) c = mv3(R, c);
                    d3 q = add3(pnew, c);
                    d3 a = add3(q, pbc_correction(S.box, S.inv, q, nullptr));
                    wcen[3 * lane] = c.x;
                    wcen[3 * lane + 1] = c.y;
                    wcen[3 * lane + 2] = c.z;
                    wabs[3 * lane] = a.x;
                    wabs[3 * lane + 1] = a.y;
                    wabs[3 * lane + 2] = a.z;
                }
                if (S.segs) {
                    // orientation * half axis with the mover's new orientation
                    // (PolyspherocylinderTraits.cpp:118-119)
                    const double oe = type != 0 ? onew_own : rot_own;
                    double O[9];
                    for (int e = 0; e < 9; e++) O[e] = grp.shfl(oe, e);
                    if (lane < S.ncen) {
                        d3 h = mv3(O, d3{S.chax[lane][0], S.chax[lane][1], S.chax[lane][2]});
                        whax[3 * lane] = h.x;
                        whax[3 * lane + 1] = h.y;
                        whax[3 * lane + 2] = h.z;
                    }
                }
                grp.sync();
            }
            // the guard band: queued pairs re-decided in FP64
            if (KIND == 2 && code == 0 && nun > 0) {
                // every centre pair of the queued bodies, one pair per lane: with K^2 <= 16,
                // 32 / K^2 bodies per pass (the FP64 segment tests of polyspherocylinders
                // keep the lanes busy), else one body per pass
                const int K = S.ncen;
                const int KK = K * K;
                const int per = KK <= GW / 2 ? GW / KK : 1;
                bool ov = false;
                for (int q0 = 0; q0 < nun && !ov; q0 += per) {
                    const int qi = q0 + (per > 1 ? lane / KK : 0);
                    const int k = qun[qi < nun ? qi : q0];
                    const float4 q = cpos[k];
                    const float3 dq = make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z);
                    const float4 *cj = G.mcen + (size_t)cslot[k] * K;
                    for (int tb = 0; tb < (per > 1 ? 1 : KK); tb += GW) {
                        const int t = per > 1 ? lane % KK : tb + lane;
                        bool hit = false;
                        if (t < KK && qi < nun && (per == 1 || lane < per * KK)) {
                            const int a = t / K, j = t % K;
                            const float4 m = wx[a];
                            const float4 c = cj[j];
                            const float3 d = make_float3((dq.x + c.x) - m.x, (dq.y + c.y) - m.y, (dq.z + c.z) - m.z);
                            hit = exact_centre_pair(S, d3{wabs[3 * a], wabs[3 * a + 1], wabs[3 * a + 2]}, a,
                                                    __float_as_int(q.w), j, d,
                                                    d3{whax[3 * a], whax[3 * a + 1], whax[3 * a + 2]});
                        }
                        if (grp.ballot(hit)) {
                            ov = true;
                            break;
                        }
                    }
                }
                ws.fp64 += nun;
                if (ov) code = 1;
            }
            if (KIND != 2 && code == 0 && nun > 0) {
                bool ov = false;
                for (int qb = 0; qb < nun; qb += GW) {
                    int qi = qb + lane;
                    bool hit = false;
                    if (qi < nun) {
                        int k = qun[qi];
                        float4 q = cpos[k];
                        hit = exact_pair(S, pnew, anew, __float_as_int(q.w),
                                         make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z));
                    }
                    if (grp.ballot(hit)) {
                        ov = true;
                        break;
                    }
                }
                ws.fp64 += nun;
                if (ov) code = 1;
            }
            // hard walls: the mover at its exact new state (Packing::countParticleOverlaps adds
            // the wall overlaps after the pairs, core/Packing.cpp:424-428)
            if (!COUNT && S.walls && code == 0) {
                int wov = 0;
                if (lane == 0)
                    wov = wall_overlap_count(S.walls, S.wall_vec, S.wall_far, S.wall_half, KIND, S.wall_radius,
                                             S.wall_half_len, pnew, anew, KIND == 2 ? wcen : nullptr,
                                             KIND == 2 ? S.ncen : 0, true, KIND == 2 && S.segs ? whax : nullptr);
                if (grp.shfl(wov, 0)) code = 1;
            }
        }

        // ---- overlap counting: the mover's overlaps before and after the move, every
        //      candidate classified (no early exit), undecided pairs in FP64 ----
        int cdelta = 0;
        if (COUNT && code == 0) {
            const d3 pc64{grp.shfl(pos_own, 0), grp.shfl(pos_own, 1), grp.shfl(pos_own, 2)};
            const d3 ac64{grp.shfl(rot_own, 2), grp.shfl(rot_own, 5), grp.shfl(rot_own, 8)};
            int before = 0, after = 0;
            if (KIND == 2) {
                // multi-centre bodies: every centre pair of every candidate body, the mover's
                // current centres (FP32 mirror, FP64 absolute centres) and its new ones
                const int K = S.ncen;
                const float4 *mcur = G.mcen + ((size_t)gbase + slot) * K;
                const bool exact = A.fp64_only || S.pbc_fold == 2;
                for (int k = lane; k < total; k += GW) {
                    const float4 q = cpos[k];
                    const int pj = __float_as_int(q.w);
                    if (pj == pid) continue;
                    const float3 db = make_float3(q.x - pcur.x, q.y - pcur.y, q.z - pcur.z);
                    const float3 da = make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z);
                    const float4 *cj = G.mcen + (size_t)cslot[k] * K;
                    for (int j = 0; j < K; j++) {
                        const float4 c = cj[j];
                        for (int a = 0; a < K; a++) {
                            const float lo = wthr[a * MAX_CEN + j], hi = wthr[MAX_CEN * MAX_CEN + a * MAX_CEN + j];
                            const float4 m0 = mcur[a];
                            const float3 d0 = make_float3((db.x + c.x) - m0.x, (db.y + c.y) - m0.y, (db.z + c.z) - m0.z);
                            const float q0 = dot3f(d0, d0);
                            int cb = exact ? 2 : (q0 < lo ? 1 : (q0 <= hi ? 2 : 0));
                            if (cb == 2) {
                                d3 h0{0.0, 0.0, 0.0};
                                if (S.segs)
                                    h0 = mv3(S.rot64 + 9 * (size_t)pid, d3{S.chax[a][0], S.chax[a][1], S.chax[a][2]});
                                cb = exact_centre_pair(S, load_d3(S.abs64 + 3 * ((size_t)pid * K + a)), a, pj, j, d0,
                                                       h0) ? 1 : 0;
                            }
                            const float4 m1 = wx[a];
                            const float3 d1 = make_float3((da.x + c.x) - m1.x, (da.y + c.y) - m1.y, (da.z + c.z) - m1.z);
                            const float q1 = dot3f(d1, d1);
                            int ca = exact ? 2 : (q1 < lo ? 1 : (q1 <= hi ? 2 : 0));
                            if (ca == 2)
                                ca = exact_centre_pair(S, d3{wabs[3 * a], wabs[3 * a + 1], wabs[3 * a + 2]}, a, pj, j, d1,
                                                       d3{whax[3 * a], whax[3 * a + 1], whax[3 * a + 2]}) ? 1 : 0;
                            before += cb;
                            after += ca;
                        }
                    }
                }
                if (S.walls && lane == 0) {
                    double hcur[3 * MAX_CEN];
                    if (S.segs)
                        for (int a = 0; a < K; a++) {
                            d3 h = mv3(S.rot64 + 9 * (size_t)pid, d3{S.chax[a][0], S.chax[a][1], S.chax[a][2]});
                            hcur[3 * a] = h.x, hcur[3 * a + 1] = h.y, hcur[3 * a + 2] = h.z;
                        }
                    before += wall_overlap_count(S.walls, S.wall_vec, S.wall_far, S.wall_half, 2, S.wall_radius, 0.0,
                                                 pc64, ac64, S.cen64 + 3 * (size_t)pid * K, K, false,
                                                 S.segs ? hcur : nullptr);
                    after += wall_overlap_count(S.walls, S.wall_vec, S.wall_far, S.wall_half, 2, S.wall_radius, 0.0,
                                                pnew, anew, wcen, K, false, S.segs ? whax : nullptr);
                }
            }
            for (int k = lane; k < (KIND == 2 ? 0 : total); k += GW) {
                const float4 q = cpos[k];
                const int pj = __float_as_int(q.w);
                if (pj == pid) continue;
                float3 aj = make_float3(0.f, 0.f, 1.f);
                if (KIND == 1) {
                    const float4 a = AXM ? G.maxis[cslot[k]] : cax[k];
                    aj = make_float3(a.x, a.y, a.z);
                }
                const float3 db = make_float3(q.x - pcur.x, q.y - pcur.y, q.z - pcur.z);
                int cb = A.fp64_only ? 2 : classify<KIND>(S.fc, db, ai, aj);
                if (cb == 2) cb = exact_pair(S, pc64, ac64, pj, db) ? 1 : 0;
                const float3 da = make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z);
                int ca = A.fp64_only ? 2 : classify<KIND>(S.fc, da, an, aj);
                if (ca == 2) ca = exact_pair(S, pnew, anew, pj, da) ? 1 : 0;
                before += cb == 1 ? 1 : 0;
                after += ca == 1 ? 1 : 0;
            }
            if (KIND != 2 && S.walls && lane == 0) {
                before += wall_overlap_count(S.walls, S.wall_vec, S.wall_far, S.wall_half, KIND, S.wall_radius,
                                             S.wall_half_len, pc64, ac64, nullptr, 0, false);
                after += wall_overlap_count(S.walls, S.wall_vec, S.wall_far, S.wall_half, KIND, S.wall_radius,
                                            S.wall_half_len, pnew, anew, nullptr, 0, false);
            }
            for (int d = GW / 2; d > 0; d >>= 1) {
                before += grp.shfl_xor(before, d);
                after += grp.shfl_xor(after, d);
            }
            if (lane == 0) ws.pairs += (unsigned)(2 * (total - 1));
            cdelta = after - before;
            code = cdelta < 0 ? 3 : (cdelta > 0 ? 1 : 0);
        }

        // ---- Metropolis (core/Simulation.cpp:483): u <= exp(-dE/T), dE in {-inf, 0, +inf} ----
        const bool acc = code == 3 ? true : ((code == 0) ? (uni <= 1.0) : (uni <= 0.0));
        if (acc) {
            const size_t gslot = (size_t)gbase + slot;
            // Packing::acceptMove adds the move's overlap delta in counting mode (core/Packing.cpp:298-300)
            if (COUNT && lane == 0) atomicAdd(S.overlaps, (unsigned long long)(long long)cdelta);
            float4 np = pcur;
            float4 na = (KIND == 1 && !AXM) ? cax[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
            grp.sync();
            if (type != 1) {
                if (lane < 3) S.pos64[3 * (size_t)pid + lane] = pnew_own;
            }
            const int na_cnt = nacc[slot];
            if (type != 1 && !exact_rel && na_cnt < MIRROR_ROUNDINGS) {
                // the FP32 proposal becomes the mirror position: one more FP32 rounding
                // (t32 is the exact FP32 value of the FP64 translation), bounded per sweep
                np = make_float4(pn.x, pn.y, pn.z, pcur.w);
                if (lane == 0) nacc[slot] = (uint8_t)(na_cnt + 1);
            } else if (type != 1) {
                if (!exact_rel) rel_own = mrow(S.inv, ld, pnew);
                if (lane == 0) nacc[slot] = 0;
                // new cell-local FP32 position from the FP64 relative coordinates
                double u = rel_own - shift_ld;
                if (u < 0.0) u += 1.0;
                double fd = u * dims_ld - c_ld;
                if (fd < -0.5) fd += dims_ld;
                if (fd > dims_ld - 0.5) fd -= dims_ld;
                float f = (float)fd;
                float f0 = grp.shfl(f, 0), f1 = grp.shfl(f, 1), f2 = grp.shfl(f, 2);
                float3 loc = mat32(G.cellmat, f0, f1, f2);
                np = make_float4(loc.x, loc.y, loc.z, pcur.w);
            }
            if (type != 0) {
                if (lane < 9) S.rot64[9 * (size_t)pid + lane] = onew_own;
                const float of = (float)onew_own;
                na = make_float4(grp.shfl(of, 2), grp.shfl(of, 5), grp.shfl(of, 8), 0.f);
            }
            if (lane == 0) {
                cpos[slot] = np;
                G.mpos[gslot] = np;
                if (KIND == 1 && type != 0) {
                    if (!AXM) cax[slot] = na;
                    G.maxis[gslot] = na;
                }
            }
            if (KIND == 2 && lane < S.ncen) {
                // Packing::acceptTempInteractionCentres (core/Packing.cpp:339-348)
                const size_t ci = (size_t)pid * S.ncen + lane;
                for (int d = 0; d < 3; d++) S.abs64[3 * ci + d] = wabs[3 * lane + d];
                if (type != 0) {
                    for (int d = 0; d < 3; d++) S.cen64[3 * ci + d] = wcen[3 * lane + d];
                    const float4 c32 = make_float4((float)wcen[3 * lane], (float)wcen[3 * lane + 1],
                                                   (float)wcen[3 * lane + 2], 0.f);
                    G.mcen[gslot * S.ncen + lane] = c32;
                }
            }
            if (self_images) {
                // the own cell is staged several times (periodic images): refresh every copy
                grp.sync();
                for (int k = lane + occ; k < total; k += GW) {
                    float4 q = cpos[k];
                    if (__float_as_int(q.w) == pid) {
                        cpos[k] = make_float4(np.x + (q.x - pcur.x), np.y + (q.y - pcur.y), np.z + (q.z - pcur.z), q.w);
                        if (KIND == 1 && type != 0 && !AXM) cax[k] = na;
                    }
                }
            }
            grp.sync();
        }

        const uint8_t full_code = code | (acc ? RP_CODE_ACCEPTED : 0);
        if (LIST) {
            if (lane == 0 && A.codes) A.codes[out_index] = full_code;
        } else if (A.log) {
            rp_move *rec = A.log + (size_t)ntypes * (size_t)gbase + mi;
            if (lane < 3) rec->translation[lane] = t64_lane;
            const double rj = ej == 0 ? rrow[0] : (ej == 1 ? rrow[1] : rrow[2]);
            if (lane < 9) rec->rotation[lane] = type != 0 ? rj : (lane % 4 == 0 ? 1.0 : 0.0);
            if (lane == 0) {
                rec->particle = pid;
                rec->type = type;
                rec->domain = cell;
                rec->reserved = 0;
                rec->uniform = uni;
                A.log_codes[(size_t)ntypes * (size_t)gbase + mi] = full_code;
            }
        }
        ws.moves++;
        if (acc) ws.accepted++;
        if (code == 1) ws.rej_overlap++;
        if (code == 2) ws.rej_domain++;
        if (type == 0) ws.trans++;
        else ws.rots++;
        if (type == 0 && acc) ws.acc_trans++;
    }
}

// ---------------------------------------------------------------------------------
// Per-particle and per-cell bodies of the cell-list rebuild and of the recount (the
// single-system kernels in rp_kernels.cu and the batched ones in rp_batch.cu call them)
// ---------------------------------------------------------------------------------
// The checks of an uploaded state for one particle: core/Packing.cpp:1069-1075
// (areShapesWithinBox: relative coordinates in [0, 1)), and orientations that are rotations
// (the engine's cell sizes and FP32 margins take a unit axis for spherocylinders and an
// orthonormal matrix for polyspheres).
__device__ __forceinline__ void validate_one(const DevState &s, int64_t i, const double rr[3]) {
    if (!(rr[0] >= 0.0 && rr[0] < 1.0 && rr[1] >= 0.0 && rr[1] < 1.0 && rr[2] >= 0.0 && rr[2] < 1.0))
        atomicOr(s.status, ST_OUTSIDE);
    const double *o = s.rot64 + 9 * i;
    bool bad = false;
    for (int a = 0; a < 3; a++)
        for (int b = a; b < 3; b++) {
            if (s.kind == 1 && (a != 2 || b != 2)) continue;
            if (s.kind == 0) continue;
            double g2 = o[a] * o[b] + o[3 + a] * o[3 + b] + o[6 + a] * o[6 + b];
            if (!(fabs(g2 - (a == b ? 1.0 : 0.0)) < 1e-6)) bad = true;
        }
    if (bad) atomicOr(s.status, ST_NOT_ROTATION);
}

__device__ __forceinline__ void validate_particle(const DevState &s, int64_t i) {
    const d3 r = mv3(s.inv, load_d3(s.pos64 + 3 * i));
    const double rr[3] = {r.x, r.y, r.z};
    validate_one(s, i, rr);
}

// Particle i's cell and FP32 cell-local position: relative coordinates box^-1 r in FP64, the
// cell of each shifted coordinate and the in-cell fraction mapped through the FP32 cell matrix.
__device__ __forceinline__ int locate_one(const DevState &s, const GridDev &g, int64_t i, float3 &loc) {
    d3 p = load_d3(s.pos64 + 3 * i);
    d3 r = mv3(s.inv, p);
    double rr[3] = {r.x, r.y, r.z};
    if (s.strict_box) {
        validate_one(s, i, rr);
    } else if (!(fabs(rr[0] - 0.5) < 0.5 + 1e-9 && fabs(rr[1] - 0.5) < 0.5 + 1e-9 && fabs(rr[2] - 0.5) < 0.5 + 1e-9)) {
        atomicOr(s.status, ST_NUMERIC);  // rescaled positions drift at most a few ulp outside
    }
    int c[3];
    float f[3];
    for (int d = 0; d < 3; d++) {
        double u = rr[d] - g.shift[d];
        if (u < 0.0) u += 1.0;
        double un = u * g.dims[d];
        int cd = static_cast<int>(un);
        if (cd >= g.dims[d]) cd = g.dims[d] - 1;
        if (cd < 0) cd = 0;
        c[d] = cd;
        f[d] = static_cast<float>(un - cd);
    }
    loc = mat32(g.cellmat, f[0], f[1], f[2]);
    return c[0] + g.dims[0] * (c[1] + g.dims[1] * c[2]);
}

__device__ __forceinline__ void assign_one(const DevState &s, const GridDev &g, int64_t i) {
    float3 loc;
    const int cell = locate_one(s, g, i, loc);
    g.plocal[i] = make_float4(loc.x, loc.y, loc.z, 0.f);
    g.pid_cell[i] = cell;
    g.rank[i] = atomicAdd(g.count + cell, 1);
}

__device__ __forceinline__ void scatter_one(const GridDev &g, int64_t i) {
    g.slot_pid[g.start[g.pid_cell[i]] + g.rank[i]] = static_cast<int32_t>(i);
}

// Sorts a cell's particles by index (a deterministic order independent of the atomic
// arrival order) and writes the FP32 mirror in cell order.
__device__ __forceinline__ void finish_one(const DevState &s, const GridDev &g, int cell) {
    int b = g.start[cell], e = g.start[cell + 1];
    for (int k = b + 1; k < e; k++) {
        int v = g.slot_pid[k];
        int j = k - 1;
        while (j >= b && g.slot_pid[j] > v) {
            g.slot_pid[j + 1] = g.slot_pid[j];
            j--;
        }
        g.slot_pid[j + 1] = v;
    }
    for (int k = b; k < e; k++) {
        int pid = g.slot_pid[k];
        g.pid_slot[pid] = k;
        float4 l = g.plocal[pid];
        g.mpos[k] = make_float4(l.x, l.y, l.z, __int_as_float(pid));
        const double *r = s.rot64 + 9 * (size_t)pid;
        g.maxis[k] = make_float4(static_cast<float>(r[2]), static_cast<float>(r[5]), static_cast<float>(r[8]), 0.f);
        for (int b = 0; b < s.ncen; b++) {
            const double *c = s.cen64 + 3 * ((size_t)pid * s.ncen + b);
            g.mcen[(size_t)k * s.ncen + b] =
                make_float4(static_cast<float>(c[0]), static_cast<float>(c[1]), static_cast<float>(c[2]), 0.f);
        }
    }
}

template <int KIND>
__device__ __forceinline__ void count_one(const DevState &s, const GridDev &g, int64_t slot, int early,
                                          unsigned long long *out, int *flag) {
    float4 pi4 = g.mpos[slot];
    int pid = __float_as_int(pi4.w);
    int cell = g.pid_cell[pid];
    int cx = cell % g.dims[0], cy = (cell / g.dims[0]) % g.dims[1], cz = cell / (g.dims[0] * g.dims[1]);
    float3 ai = make_float3(0.f, 0.f, 0.f);
    if (KIND == 1) {
        float4 a = g.maxis[slot];
        ai = make_float3(a.x, a.y, a.z);
    }
    unsigned long long cnt = 0;
    bool have64 = false;
    d3 pi64{0, 0, 0}, ai64{0, 0, 0};
    for (int o = 0; o < 27; o++) {
        if (early && *(volatile int *)flag) break;
        int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = o / 9 - 1;
        int nb = wrap_cell(cx + ox, g.dims[0]) +
                 g.dims[0] * (wrap_cell(cy + oy, g.dims[1]) + g.dims[1] * wrap_cell(cz + oz, g.dims[2]));
        float3 off = mat32(g.cellmat, (float)ox, (float)oy, (float)oz);
        int b = g.start[nb], e = g.start[nb + 1];
        for (int k = b; k < e; k++) {
            float4 q = g.mpos[k];
            int pj = __float_as_int(q.w);
            if (pj <= pid) continue;
            float3 dsep = make_float3((q.x + off.x) - pi4.x, (q.y + off.y) - pi4.y, (q.z + off.z) - pi4.z);
            float3 aj = make_float3(0.f, 0.f, 0.f);
            if (KIND == 1) {
                float4 a = g.maxis[k];
                aj = make_float3(a.x, a.y, a.z);
            }
            int cls = (KIND != 1 && s.pbc_fold == 2) ? 2 : classify<KIND>(s.fc, dsep, ai, aj);
            bool ov = cls == 1;
            if (cls == 2) {
                if (!have64) {
                    pi64 = load_d3(s.pos64 + 3 * (size_t)pid);
                    const double *r = s.rot64 + 9 * (size_t)pid;
                    ai64 = d3{r[2], r[5], r[8]};
                    have64 = true;
                }
                atomicAdd(s.counters + 5, 1ull);
                ov = exact_pair(s, pi64, ai64, pj, dsep);
            }
            if (ov) {
                cnt++;
                if (early) {
                    atomicExch(flag, 1);
                    break;
                }
            }
        }
    }
    // Packing::countTotalOverlaps adds every particle's wall overlaps (core/Packing.cpp:558-580)
    if (s.walls && !(early && *(volatile int *)flag)) {
        const double *r = s.rot64 + 9 * (size_t)pid;
        const int w = wall_overlap_count(s.walls, s.wall_vec, s.wall_far, s.wall_half, KIND, s.wall_radius,
                                         s.wall_half_len, load_d3(s.pos64 + 3 * (size_t)pid), d3{r[2], r[5], r[8]},
                                         nullptr, 0, early != 0);
        if (w && early) atomicExch(flag, 1);
        cnt += (unsigned long long)w;
    }
    if (cnt) atomicAdd(out, cnt);
}

__device__ __forceinline__ void count_poly_one(const DevState &s, const GridDev &g, int64_t slot, int early,
                                               unsigned long long *out, int *flag) {
    const int K = s.ncen;
    float4 pi4 = g.mpos[slot];
    int pid = __float_as_int(pi4.w);
    int cell = g.pid_cell[pid];
    int cx = cell % g.dims[0], cy = (cell / g.dims[0]) % g.dims[1], cz = cell / (g.dims[0] * g.dims[1]);
    unsigned long long cnt = 0;
    double hx[3 * MAX_CEN];   // polyspherocylinders: orientation * half axis of each centre
    if (s.segs)
        for (int a = 0; a < K; a++) {
            d3 h = mv3(s.rot64 + 9 * (size_t)pid, d3{s.chax[a][0], s.chax[a][1], s.chax[a][2]});
            hx[3 * a] = h.x, hx[3 * a + 1] = h.y, hx[3 * a + 2] = h.z;
        }
    for (int o = 0; o < 27; o++) {
        if (early && *(volatile int *)flag) break;
        int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = o / 9 - 1;
        int nb = wrap_cell(cx + ox, g.dims[0]) +
                 g.dims[0] * (wrap_cell(cy + oy, g.dims[1]) + g.dims[1] * wrap_cell(cz + oz, g.dims[2]));
        float3 off = mat32(g.cellmat, (float)ox, (float)oy, (float)oz);
        int b = g.start[nb], e = g.start[nb + 1];
        for (int k = b; k < e; k++) {
            float4 q = g.mpos[k];
            int pj = __float_as_int(q.w);
            if (pj <= pid) continue;
            float3 dq = make_float3((q.x + off.x) - pi4.x, (q.y + off.y) - pi4.y, (q.z + off.z) - pi4.z);
            if (dot3f(dq, dq) > s.fc.far_hi) continue;
            for (int j = 0; j < K; j++) {
                float4 cj = g.mcen[(size_t)k * K + j];
                float3 bj = make_float3(dq.x + cj.x, dq.y + cj.y, dq.z + cj.z);
                for (int a = 0; a < K; a++) {
                    float4 ca = g.mcen[(size_t)slot * K + a];
                    float3 d = make_float3(bj.x - ca.x, bj.y - ca.y, bj.z - ca.z);
                    float d2 = dot3f(d, d);
                    const bool exact = s.pbc_fold == 2;
                    bool ov = !exact && d2 < g.cthr[a * MAX_CEN + j];
                    if (!ov && (exact || d2 <= g.cthr[MAX_CEN * MAX_CEN + a * MAX_CEN + j])) {
                        atomicAdd(s.counters + 5, 1ull);
                        if (s.cq_buf) {
                            const int qi = atomicAdd(s.cq_count, 1);
                            if (qi < s.cq_cap) {
                                s.cq_buf[qi] = DeferredPair{pid, pj, a * MAX_CEN + j, 0, make_float4(d.x, d.y, d.z, 0.f)};
                                continue;
                            }
                        }
                        ov = exact_centre_pair(s, load_d3(s.abs64 + 3 * ((size_t)pid * K + a)), a, pj, j, d,
                                               s.segs ? d3{hx[3 * a], hx[3 * a + 1], hx[3 * a + 2]} : d3{0, 0, 0});
                    }
                    if (ov) {
                        cnt++;
                        if (early) {
                            atomicExch(flag, 1);
                            atomicAdd(out, cnt);
                            return;
                        }
                    }
                }
            }
        }
    }
    if (s.walls && !(early && *(volatile int *)flag)) {
        const int w = wall_overlap_count(s.walls, s.wall_vec, s.wall_far, s.wall_half, 2, s.wall_radius, 0.0,
                                         load_d3(s.pos64 + 3 * (size_t)pid), d3{0, 0, 0},
                                         s.cen64 + 3 * (size_t)pid * K, K, early != 0, s.segs ? hx : nullptr);
        if (w && early) atomicExch(flag, 1);
        cnt += (unsigned long long)w;
    }
    if (cnt) atomicAdd(out, cnt);
}

}  // namespace rp
