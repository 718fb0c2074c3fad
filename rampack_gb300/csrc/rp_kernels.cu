// Device kernels of the move-and-overlap path (sm_103a):
//   * counting-sort cell-list rebuild with an FP32 cell-local mirror in cell order,
//   * checkerboard move sweep: one warp per active cell, the cell's 3x3x3
//     neighbourhood staged in shared memory, warp-ballot early exit, FP32 filter with
//     FP64 re-decision in a guard band,
//   * all-pairs overlap recount with an early-exit flag,
//   * FP64 box rescale.
#include <cuda_runtime.h>

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

// ---------------------------------------------------------------------------------
// FP32 classification of one pair.  0: no overlap, 1: overlap, 2: undecided in FP32
// (re-decided in FP64).  d = p_j - p_i (candidate minus mover), a_i/a_j unit axes.
// ---------------------------------------------------------------------------------
template <int KIND>
__device__ __forceinline__ int classify(const FilterConsts &fc, float3 d, float3 ai, float3 aj) {
    float d2 = dot3f(d, d);
    if (KIND == 0) {
        if (d2 < fc.sphere_lo) return 1;
        if (d2 > fc.sphere_hi) return 0;
        return 2;
    } else {
        if (d2 > fc.far_hi) return 0;
        if (d2 < fc.core_lo) return 1;
        if (d2 < fc.core_hi || d2 > fc.far_lo) return 2;
        // Segment-segment distance of the two cylinder axes (same branch structure as
        // the FP64 reference), then a convexity certificate: for any feasible (s, t),
        // f* >= f(s, t) - G with G the Frank-Wolfe gap of the box-constrained problem.
        const float l = fc.len, h = fc.half_len;
        float3 u = make_float3(l * ai.x, l * ai.y, l * ai.z);
        float3 v = make_float3(l * aj.x, l * aj.y, l * aj.z);
        float3 w = make_float3(-d.x - h * (ai.x - aj.x), -d.y - h * (ai.y - aj.y), -d.z - h * (ai.z - aj.z));
        float a = dot3f(u, u), b = dot3f(u, v), c = dot3f(v, v), dd = dot3f(u, w), e = dot3f(v, w);
        float D = fmaf(a, c, -b * b);
        if (D < fc.d_min) return 2;
        float sN = fmaf(b, e, -c * dd), tN = fmaf(a, e, -b * dd), sD = D, tD = D;
        if (sN < 0.f) {
            sN = 0.f; tN = e; tD = c;
        } else if (sN > sD) {
            sN = sD; tN = e + b; tD = c;
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
        if (f + fc.seg_err < fc.core_thr) return 1;
        if (f - G - fc.seg_err >= fc.core_thr) return 0;
        return 2;
    }
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
__device__ __forceinline__ bool exact_pair(const DevState &s, d3 pi, d3 ai, int pid_j, float3 dsep) {
    d3 pj = load_d3(s.pos64 + 3 * (size_t)pid_j);
    const double *rj = s.rot64 + 9 * (size_t)pid_j;
    d3 aj = d3{rj[2], rj[5], rj[8]};
    int m = image_index(s, dsep, pi, pj);
    d3 t = load_d3(s.trans + 3 * m);
    return exact_overlap(s.ex, pi, ai, pj, aj, t);
}

// ---------------------------------------------------------------------------------
// Cell-list rebuild
// ---------------------------------------------------------------------------------
__global__ void k_assign(DevState s, GridDev g) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    d3 p = load_d3(s.pos64 + 3 * i);
    d3 r = mv3(s.inv, p);
    double rr[3] = {r.x, r.y, r.z};
    // core/Packing.cpp:1069-1075 (areShapesWithinBox): relative coordinates in [0, 1)
    if (s.strict_box) {
        if (!(rr[0] >= 0.0 && rr[0] < 1.0 && rr[1] >= 0.0 && rr[1] < 1.0 && rr[2] >= 0.0 && rr[2] < 1.0))
            atomicOr(s.status, ST_OUTSIDE);
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
    int cell = c[0] + g.dims[0] * (c[1] + g.dims[1] * c[2]);
    float3 loc = mat32(g.cellmat, f[0], f[1], f[2]);
    g.plocal[i] = make_float4(loc.x, loc.y, loc.z, 0.f);
    g.pid_cell[i] = cell;
    g.rank[i] = atomicAdd(g.count + cell, 1);
}

// Two-level exclusive scan of the cell counts (4096 cells per block).
__global__ void k_scan_blocks(const int32_t *count, int32_t *start, int32_t *block_sums, int ncell,
                              int32_t *max_occ) {
    __shared__ int32_t warp_tot[32];
    int base = blockIdx.x * 4096 + threadIdx.x * 4;
    int v[4];
    int local_max = 0;
    for (int k = 0; k < 4; k++) {
        v[k] = (base + k < ncell) ? count[base + k] : 0;
        local_max = max(local_max, v[k]);
    }
    int tsum = v[0] + v[1] + v[2] + v[3];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = tsum;
    for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    for (int d = 16; d > 0; d >>= 1) local_max = max(local_max, __shfl_xor_sync(0xffffffffu, local_max, d));
    if (lane == 31) warp_tot[wid] = incl;
    if (lane == 0) atomicMax(max_occ, local_max);
    __syncthreads();
    if (wid == 0) {
        int wv = warp_tot[lane];
        int wi = wv;
        for (int d = 1; d < 32; d <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += y;
        }
        warp_tot[lane] = wi - wv;
        if (lane == 31) block_sums[blockIdx.x] = wi;
    }
    __syncthreads();
    int run = warp_tot[wid] + incl - tsum;
    for (int k = 0; k < 4; k++) {
        if (base + k < ncell) start[base + k] = run;
        run += v[k];
    }
}

__global__ void k_scan_sums(int32_t *block_sums, int nblocks, int32_t *start, int ncell) {
    // single block: sequential prefix over the (few) block sums
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int run = 0;
        for (int b = 0; b < nblocks; b++) {
            int v = block_sums[b];
            block_sums[b] = run;
            run += v;
        }
        start[ncell] = run;
    }
}

__global__ void k_scan_add(int32_t *start, const int32_t *block_sums, int ncell) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncell) start[i] += block_sums[i / 4096];
}

__global__ void k_scatter(DevState s, GridDev g) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    g.slot_pid[g.start[g.pid_cell[i]] + g.rank[i]] = static_cast<int32_t>(i);
}

// Sorts each cell's particles by index (a deterministic order independent of the
// atomic arrival order) and writes the FP32 mirror in cell order.
__global__ void k_cell_finish(DevState s, GridDev g) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= g.ncell) return;
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
    }
}

// ---------------------------------------------------------------------------------
// Box rescale: positions keep their relative coordinates (core/Packing.cpp:183-184:
// newBox.relativeToAbsolute(oldBox.absoluteToRelative(pos))).
// ---------------------------------------------------------------------------------
struct Mat9 {
    double m[9];
};

__global__ void k_rescale(const double *src, double *dst, int64_t n, Mat9 old_inv, Mat9 new_box) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    d3 p = load_d3(src + 3 * i);
    d3 r = mv3(old_inv.m, p);
    d3 q = mv3(new_box.m, r);
    dst[3 * i] = q.x;
    dst[3 * i + 1] = q.y;
    dst[3 * i + 2] = q.z;
}

// ---------------------------------------------------------------------------------
// All-pairs recount: one thread per particle (slot order); each unordered pair and
// periodic image is visited once (candidate index greater than own index).
// ---------------------------------------------------------------------------------
template <int KIND>
__global__ void k_count(DevState s, GridDev g, int early, unsigned long long *out, int *flag) {
    int64_t slot = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (slot >= s.n) return;
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
            int cls = classify<KIND>(s.fc, dsep, ai, aj);
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
    if (cnt) atomicAdd(out, cnt);
}

template __global__ void k_count<0>(DevState, GridDev, int, unsigned long long *, int *);
template __global__ void k_count<1>(DevState, GridDev, int, unsigned long long *, int *);

// ---------------------------------------------------------------------------------
// Checkerboard sweep: one warp per active cell.
// ---------------------------------------------------------------------------------
struct WarpStats {
    unsigned moves, accepted, rej_overlap, rej_domain, pairs, fp64, trans, rots;
};

template <int KIND, bool LIST>
__device__ __forceinline__ void sweep_cell(const SweepArgs &A, const int item, float4 *cpos, float4 *cax,
                                           uint16_t *queue, WarpStats &ws) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const DevState &S = A.s;
    const GridDev &G = A.g;

    // ---- which cell ----
    int cell, c[3];
    if (A.work) {
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
        for (int d = 0; d < 3; d++) c[d] = G.dims[d] == 1 ? 0 : 2 * cc[d] + A.phase[d];
        cell = c[0] + G.dims[0] * (c[1] + G.dims[1] * c[2]);
    }
    c[0] = cell % G.dims[0];
    c[1] = (cell / G.dims[0]) % G.dims[1];
    c[2] = cell / (G.dims[0] * G.dims[1]);

    // ---- stage the 3x3x3 neighbourhood (own cell first) ----
    int cnt = 0, st = 0;
    float3 off = make_float3(0.f, 0.f, 0.f);
    if (lane < 27) {
        int ox, oy, oz;
        lane_offset(lane, ox, oy, oz);
        int nb = wrap_cell(c[0] + ox, G.dims[0]) +
                 G.dims[0] * (wrap_cell(c[1] + oy, G.dims[1]) + G.dims[1] * wrap_cell(c[2] + oz, G.dims[2]));
        st = G.start[nb];
        cnt = G.start[nb + 1] - st;
        off = mat32(G.cellmat, (float)ox, (float)oy, (float)oz);
    }
    int incl = cnt;
    for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += y;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    const int occ = __shfl_sync(FULL, cnt, 0);
    const int gbase = __shfl_sync(FULL, st, 0);
    if (total > A.cap) {
        if (lane == 0) {
            if (A.overflow) {
                int k = atomicAdd(A.overflow_count, 1);
                A.overflow[k] = cell;
            } else {
                atomicOr(S.status, ST_CAPACITY);
            }
        }
        return;
    }
    {
        int base = incl - cnt;
        for (int k = 0; k < cnt; k++) {
            float4 p = G.mpos[st + k];
            p.x += off.x;
            p.y += off.y;
            p.z += off.z;
            cpos[base + k] = p;
            if (KIND == 1) cax[base + k] = G.maxis[st + k];
        }
    }
    // does the own cell appear more than once (a grid dimension of one cell)?
    const bool self_images = (G.dims[0] == 1) || (G.dims[1] == 1) || (G.dims[2] == 1);
    __syncwarp();

    // cell bounds (ActiveDomain) of this cell
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = G.bounds[G.boundsoff[d] + 2 * c[d]];
        hi[d] = G.bounds[G.boundsoff[d] + 2 * c[d] + 1];
    }

    int nmoves, mbeg = 0;
    if (LIST) {
        int li = A.work ? -1 : item;
        if (A.work) {
            // overflow rerun in list mode: find this cell's range
            for (int q = 0; q < A.num_list; q++)
                if (A.list_cells[q] == cell) li = q;
        }
        mbeg = A.list_begin[li];
        nmoves = A.list_begin[li + 1] - mbeg;
    } else {
        nmoves = ((A.types & 1) + ((A.types >> 1) & 1)) * occ;
    }
    const int ntypes = (A.types & 1) + ((A.types >> 1) & 1);

    for (int mi = 0; mi < nmoves; mi++) {
        // ---- the proposal ----
        int type, slot = -1;
        double t64[3] = {0.0, 0.0, 0.0}, R64[9];
        float R32[9];
        float3 t32 = make_float3(0.f, 0.f, 0.f);
        double uni = 0.5;
        int out_index = -1;
        if (LIST) {
            out_index = A.move_out[mbeg + mi];
            const rp_move &m = A.moves[out_index];
            type = m.type;
            int want = m.particle;
            for (int kb = 0; kb < occ; kb += 32) {
                int k = kb + lane;
                bool hit = k < occ && __float_as_int(cpos[k].w) == want;
                unsigned bal = __ballot_sync(FULL, hit);
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
            for (int q = 0; q < 3; q++) t64[q] = m.translation[q];
            for (int q = 0; q < 9; q++) R64[q] = m.rotation[q];
            uni = m.uniform;
            t32 = make_float3((float)t64[0], (float)t64[1], (float)t64[2]);
            for (int q = 0; q < 9; q++) R32[q] = (float)R64[q];
        } else {
            u4 r0 = philox(u4{(uint32_t)(2 * mi), (uint32_t)cell, (uint32_t)A.counter, (uint32_t)(A.counter >> 32)},
                           (uint32_t)A.seed, (uint32_t)(A.seed >> 32));
            u4 r1 = philox(u4{(uint32_t)(2 * mi + 1), (uint32_t)cell, (uint32_t)A.counter,
                              (uint32_t)(A.counter >> 32)},
                           (uint32_t)A.seed, (uint32_t)(A.seed >> 32));
            if (ntypes == 2) type = (r0.a >> 31) ? 1 : 0;
            else type = (A.types & 1) ? 0 : 1;
            slot = (int)__umulhi(r0.b, (uint32_t)occ);
            if (type == 0) {
                t32 = make_float3(pm1f(r0.c) * A.tstep, pm1f(r0.d) * A.tstep, pm1f(r1.a) * A.tstep);
                t64[0] = t32.x;
                t64[1] = t32.y;
                t64[2] = t32.z;
            } else {
                // Cayley map of v = tan(theta/2) * axis: an exactly orthogonal rotation in
                // FP64, angle theta uniform in [-step, step], axis uniform on the sphere.
                float z = pm1f(r1.b);
                float phi = 6.2831853f * u01f(r1.c);
                float sphi, cphi;
                sincosf(phi, &sphi, &cphi);
                float rs = sqrtf(fmaxf(0.f, 1.f - z * z));
                float th = pm1f(r1.d) * A.rstep;
                float tq = tanf(0.5f * th);
                float v[3] = {tq * rs * cphi, tq * rs * sphi, tq * z};
                float v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
                float k32 = 2.f / (1.f + v2);
                double vd[3] = {v[0], v[1], v[2]};
                double v2d = vd[0] * vd[0] + vd[1] * vd[1] + vd[2] * vd[2];
                double kd = 2.0 / (1.0 + v2d);
                float K[9] = {0.f, -v[2], v[1], v[2], 0.f, -v[0], -v[1], v[0], 0.f};
                double Kd[9] = {0.0, -vd[2], vd[1], vd[2], 0.0, -vd[0], -vd[1], vd[0], 0.0};
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        float e32 = K[3 * i + j] + v[i] * v[j] - (i == j ? v2 : 0.f);
                        R32[3 * i + j] = (i == j ? 1.f : 0.f) + k32 * e32;
                        double e64 = Kd[3 * i + j] + vd[i] * vd[j] - (i == j ? v2d : 0.0);
                        R64[3 * i + j] = (i == j ? 1.0 : 0.0) + kd * e64;
                    }
            }
        }
        if (type == 0) {
            for (int q = 0; q < 9; q++) {
                R32[q] = (q % 4 == 0) ? 1.f : 0.f;
                R64[q] = (q % 4 == 0) ? 1.0 : 0.0;
            }
        }
        const float4 pcur = cpos[slot];
        const int pid = __float_as_int(pcur.w);
        float3 ai = make_float3(0.f, 0.f, 1.f);
        if (KIND == 1) {
            float4 a = cax[slot];
            ai = make_float3(a.x, a.y, a.z);
        }
        float3 pn = make_float3(pcur.x, pcur.y, pcur.z);
        float3 an = ai;
        if (type == 0 || type == 2) pn = make_float3(pcur.x + t32.x, pcur.y + t32.y, pcur.z + t32.z);
        if ((type == 1 || type == 2) && KIND == 1) an = mat32(R32, ai.x, ai.y, ai.z);

        // ---- FP32 ActiveDomain test (translations) ----
        int dom = 0;  // 0 inside, 1 outside, 2 undecided
        if (type == 0 || type == 2) {
            float3 f = mat32(G.cellinv, pn.x, pn.y, pn.z);
            float fm[3] = {f.x, f.y, f.z};
            const float mg = S.fc.cell_margin;
            for (int d = 0; d < 3; d++) {
                if (G.dims[d] == 1) continue;
                if (fm[d] < -mg || fm[d] > 1.f + mg) dom = 1;
                else if (dom == 0 && (fm[d] < mg || fm[d] > 1.f - mg)) dom = 2;
            }
        }

        // ---- FP32 overlap filter over the staged neighbourhood ----
        bool overlap = false;
        int nq = 0;
        unsigned pairs = 0;
        if (dom != 1) {
            for (int base = 0; base < total; base += 32) {
                int k = base + lane;
                int cls = 0;
                if (k < total) {
                    float4 q = cpos[k];
                    if (__float_as_int(q.w) != pid) {
                        float3 dsep = make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z);
                        float3 aj = make_float3(0.f, 0.f, 1.f);
                        if (KIND == 1) {
                            float4 a = cax[k];
                            aj = make_float3(a.x, a.y, a.z);
                        }
                        cls = A.fp64_only ? 2 : classify<KIND>(S.fc, dsep, an, aj);
                        pairs++;
                    }
                }
                if (__ballot_sync(FULL, cls == 1)) {
                    overlap = true;
                    break;
                }
                unsigned un = __ballot_sync(FULL, cls == 2);
                if (un) {
                    if (cls == 2) queue[nq + __popc(un & ((1u << lane) - 1u))] = (uint16_t)k;
                    nq += __popc(un);
                }
            }
        }
        __syncwarp();

        // ---- FP64: exact proposal for moves that survived, and the guard band ----
        d3 p64 = load_d3(S.pos64 + 3 * (size_t)pid);
        d3 pnew = p64;
        double rel[3] = {0.0, 0.0, 0.0};
        bool exact_done = false;
        uint8_t code;
        if (dom == 1) {
            code = 2;
        } else if (overlap) {
            code = 1;
        } else {
            exact_done = true;
            if (type == 0 || type == 2) {
                // Shape::translate (core/Shape.cpp:9-12) with PBC correction
                d3 p1 = add3(p64, d3{t64[0], t64[1], t64[2]});
                bool wrapped = false;
                d3 corr = pbc_correction(S.box, S.inv, p1, &wrapped);
                pnew = add3(p1, corr);
                d3 r = mv3(S.inv, pnew);
                rel[0] = r.x;
                rel[1] = r.y;
                rel[2] = r.z;
                if (!inside_domain(S.inv, pnew, lo, hi)) code = 2;
                else code = 0;
            } else {
                code = 0;
            }
            if (code == 0 && nq > 0) {
                // orientation after the move: R · O (core/Shape.cpp:14-16), column 2
                const double *ro = S.rot64 + 9 * (size_t)pid;
                d3 anew;
                if (type == 1 || type == 2) {
                    double o[9];
                    for (int q = 0; q < 9; q++) o[q] = ro[q];
                    anew = d3{mm_elem(R64, o, 0, 2), mm_elem(R64, o, 1, 2), mm_elem(R64, o, 2, 2)};
                } else {
                    anew = d3{ro[2], ro[5], ro[8]};
                }
                bool ov = false;
                for (int qb = 0; qb < nq; qb += 32) {
                    int qi = qb + lane;
                    bool hit = false;
                    if (qi < nq) {
                        int k = queue[qi];
                        float4 q = cpos[k];
                        float3 dsep = make_float3(q.x - pn.x, q.y - pn.y, q.z - pn.z);
                        hit = exact_pair(S, pnew, anew, __float_as_int(q.w), dsep);
                    }
                    if (__ballot_sync(FULL, hit)) {
                        ov = true;
                        break;
                    }
                }
                ws.fp64 += nq;
                if (ov) code = 1;
            }
        }
        ws.pairs += pairs;

        // ---- Metropolis (core/Simulation.cpp:483): u <= exp(-dE/T), dE in {0, +inf} ----
        bool acc = (code == 0) ? (uni <= 1.0) : (uni <= 0.0);
        if (acc) {
            if (!exact_done && (type == 0 || type == 2)) {
                // an accepted move with dE = +inf (u == 0 exactly): the reference still
                // commits the temp shape, so compute its translated position.
                d3 p1 = add3(p64, d3{t64[0], t64[1], t64[2]});
                d3 corr = pbc_correction(S.box, S.inv, p1, nullptr);
                pnew = add3(p1, corr);
                d3 r = mv3(S.inv, pnew);
                rel[0] = r.x;
                rel[1] = r.y;
                rel[2] = r.z;
            }
            const size_t gslot = (size_t)gbase + slot;
            float4 np = pcur;
            if (type == 0 || type == 2) {
                if (lane < 3) S.pos64[3 * (size_t)pid + lane] = lane == 0 ? pnew.x : (lane == 1 ? pnew.y : pnew.z);
                // new cell-local FP32 position from the FP64 relative coordinates
                float fr[3];
                for (int d = 0; d < 3; d++) {
                    double u = rel[d] - G.shift[d];
                    if (u < 0.0) u += 1.0;
                    double fd = u * G.dims[d] - c[d];
                    if (fd < -0.5) fd += G.dims[d];
                    if (fd > G.dims[d] - 0.5) fd -= G.dims[d];
                    fr[d] = (float)fd;
                }
                float3 loc = mat32(G.cellmat, fr[0], fr[1], fr[2]);
                np = make_float4(loc.x, loc.y, loc.z, pcur.w);
            }
            float4 na = make_float4(0.f, 0.f, 0.f, 0.f);
            if (type == 1 || type == 2) {
                double *ro = S.rot64 + 9 * (size_t)pid;
                double o[9];
                for (int q = 0; q < 9; q++) o[q] = ro[q];
                __syncwarp();
                double e = 0.0;
                if (lane < 9) e = mm_elem(R64, o, lane / 3, lane % 3);
                if (lane < 9) ro[lane] = e;
                double a0 = __shfl_sync(FULL, e, 2), a1 = __shfl_sync(FULL, e, 5), a2 = __shfl_sync(FULL, e, 8);
                na = make_float4((float)a0, (float)a1, (float)a2, 0.f);
            }
            __syncwarp();
            if (lane == 0) {
                cpos[slot] = np;
                G.mpos[gslot] = np;
                if (KIND == 1 && (type == 1 || type == 2)) {
                    cax[slot] = na;
                    G.maxis[gslot] = na;
                }
            }
            if (self_images) {
                // the own cell is staged several times (periodic images): refresh all copies
                __syncwarp();
                for (int k = lane + occ; k < total; k += 32) {
                    float4 q = cpos[k];
                    if (__float_as_int(q.w) == pid) {
                        float3 shift = make_float3(q.x - pcur.x, q.y - pcur.y, q.z - pcur.z);
                        cpos[k] = make_float4(np.x + shift.x, np.y + shift.y, np.z + shift.z, q.w);
                        if (KIND == 1 && (type == 1 || type == 2)) cax[k] = na;
                    }
                }
            }
            __syncwarp();
        }

        uint8_t full_code = code | (acc ? RP_CODE_ACCEPTED : 0);
        if (lane == 0) {
            if (LIST && A.codes) A.codes[out_index] = full_code;
            if (!LIST && A.log) {
                size_t li = (size_t)ntypes * (size_t)gbase + mi;
                rp_move rec;
                rec.particle = pid;
                rec.type = type;
                rec.domain = cell;
                rec.reserved = 0;
                for (int q = 0; q < 3; q++) rec.translation[q] = t64[q];
                for (int q = 0; q < 9; q++) rec.rotation[q] = R64[q];
                rec.uniform = uni;
                A.log[li] = rec;
                A.log_codes[li] = full_code;
            }
        }
        ws.moves++;
        if (acc) ws.accepted++;
        if (code == 1) ws.rej_overlap++;
        if (code == 2) ws.rej_domain++;
        if (type == 0) ws.trans++;
        else ws.rots++;
    }

}

template <int KIND, bool LIST>
__global__ void __launch_bounds__(SWEEP_WARPS * 32) k_sweep(const SweepArgs A) {
    extern __shared__ float4 smem[];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int warps_per_block = blockDim.x >> 5;
    const int warp = blockIdx.x * warps_per_block + wib;
    const int per_warp = A.cap * (KIND == 1 ? 2 : 1) + A.cap / 8;  // float4 units
    float4 *cpos = smem + (size_t)wib * per_warp;
    float4 *cax = cpos + A.cap;  // only for spherocylinders
    uint16_t *queue = reinterpret_cast<uint16_t *>(cpos + A.cap * (KIND == 1 ? 2 : 1));
    int nitems = A.work ? *A.work_count : (LIST ? A.num_list : A.num_active);
    WarpStats ws = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int item = warp; item < nitems; item += gridDim.x * warps_per_block) {
        sweep_cell<KIND, LIST>(A, item, cpos, cax, queue, ws);
        __syncwarp();
    }
    // ---- statistics ----
    unsigned pairs = ws.pairs;
    for (int d = 16; d > 0; d >>= 1) pairs += __shfl_xor_sync(FULL, pairs, d);
    if (lane == 0 && ws.moves) {
        unsigned long long *C = A.s.counters;
        atomicAdd(C + 0, (unsigned long long)ws.moves);
        atomicAdd(C + 1, (unsigned long long)ws.accepted);
        atomicAdd(C + 2, (unsigned long long)ws.rej_overlap);
        atomicAdd(C + 3, (unsigned long long)ws.rej_domain);
        atomicAdd(C + 4, (unsigned long long)pairs);
        atomicAdd(C + 5, (unsigned long long)ws.fp64);
        atomicAdd(C + 6, (unsigned long long)ws.trans);
        atomicAdd(C + 7, (unsigned long long)ws.rots);
    }
}

// ---------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------
cudaError_t launch_rebuild(const DevState &s, const GridDev &g, int32_t *block_sums, cudaStream_t st) {
    int64_t n = s.n;
    int tb = 256;
    unsigned nb = (unsigned)((n + tb - 1) / tb);
    cudaMemsetAsync(g.count, 0, sizeof(int32_t) * g.ncell, st);
    cudaMemsetAsync(g.max_occ, 0, sizeof(int32_t), st);
    k_assign<<<nb, tb, 0, st>>>(s, g);
    int nblocks = (g.ncell + 4095) / 4096;
    k_scan_blocks<<<nblocks, 1024, 0, st>>>(g.count, g.start, block_sums, g.ncell, g.max_occ);
    k_scan_sums<<<1, 32, 0, st>>>(block_sums, nblocks, g.start, g.ncell);
    k_scan_add<<<(g.ncell + 255) / 256, 256, 0, st>>>(g.start, block_sums, g.ncell);
    k_scatter<<<nb, tb, 0, st>>>(s, g);
    k_cell_finish<<<(g.ncell + 127) / 128, 128, 0, st>>>(s, g);
    return cudaGetLastError();
}

cudaError_t launch_rescale(const double *src, double *dst, int64_t n, const double *old_inv, const double *new_box,
                           cudaStream_t st) {
    Mat9 a, b;
    for (int i = 0; i < 9; i++) {
        a.m[i] = old_inv[i];
        b.m[i] = new_box[i];
    }
    k_rescale<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n, a, b);
    return cudaGetLastError();
}

cudaError_t launch_count(const DevState &s, const GridDev &g, int early, unsigned long long *out, int *flag,
                         cudaStream_t st) {
    unsigned nb = (unsigned)((s.n + 127) / 128);
    if (s.kind == 0) k_count<0><<<nb, 128, 0, st>>>(s, g, early, out, flag);
    else k_count<1><<<nb, 128, 0, st>>>(s, g, early, out, flag);
    return cudaGetLastError();
}

size_t sweep_smem_per_warp(int kind, int cap) {
    return (size_t)(cap * (kind == 1 ? 2 : 1) + cap / 8) * sizeof(float4);
}

cudaError_t launch_sweep(const SweepArgs &a, bool list, int nwarps, cudaStream_t st) {
    if (nwarps <= 0) return cudaSuccess;
    const int wpb = a.work ? 1 : SWEEP_WARPS;
    size_t smem = sweep_smem_per_warp(a.s.kind, a.cap) * wpb;
    unsigned blocks = (unsigned)((nwarps + wpb - 1) / wpb);
    cudaError_t e = cudaSuccess;
    if (a.s.kind == 0) {
        if (list) {
            e = cudaFuncSetAttribute(k_sweep<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_sweep<0, true><<<blocks, wpb * 32, smem, st>>>(a);
        } else {
            e = cudaFuncSetAttribute(k_sweep<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_sweep<0, false><<<blocks, wpb * 32, smem, st>>>(a);
        }
    } else {
        if (list) {
            e = cudaFuncSetAttribute(k_sweep<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_sweep<1, true><<<blocks, wpb * 32, smem, st>>>(a);
        } else {
            e = cudaFuncSetAttribute(k_sweep<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_sweep<1, false><<<blocks, wpb * 32, smem, st>>>(a);
        }
    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace rp
