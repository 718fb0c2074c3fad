// Device kernels of the move-and-overlap path (sm_103a):
//   * counting-sort cell-list rebuild with an FP32 cell-local mirror in cell order,
//   * checkerboard move sweep: one warp per active cell, the cell's 3x3x3
//     neighbourhood staged in shared memory, warp-ballot early exit, FP32 filter with
//     FP64 re-decision in a guard band,
//   * all-pairs overlap recount with an early-exit flag,
//   * FP64 box rescale.
#include <cuda_runtime.h>

#include "rp_sweep.cuh"

namespace rp {

// ---------------------------------------------------------------------------------
// Cell-list rebuild
// ---------------------------------------------------------------------------------
__global__ void k_assign(DevState s, GridDev g) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < s.n) assign_one(s, g, i);
}

// An uploaded state's checks alone (the cell grid is built when first needed).
__global__ void k_validate(DevState s) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < s.n) validate_particle(s, i);
}

// Two-level exclusive scan of the cell counts (4096 cells per block).
// Occupancy-order key of a cell: its checkerboard phase, then its occupancy bin (largest
// first).  Persistent sweep warps take a phase's cells in this order, so the phase ends on
// short cells; any order of one phase's cells gives the same results (they are never
// neighbours).
__device__ __forceinline__ int order_key(const int dims[3], int c, int occ) {
    return cell_phase(dims, c) * ORDER_BINS + ORDER_BINS - 1 - min(occ, ORDER_BINS - 1);
}

// Block prefix sums of the cell counts (4096 cells per block); with order_cnt, also the
// counts of the cells per order key (block-local in shared memory, one global add per key).
__global__ void k_scan_blocks(const int32_t *count, int32_t *start, int32_t *block_sums, int ncell,
                              int32_t *max_occ, int3 dims, int32_t *order_cnt) {
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t okeys[27 * ORDER_BINS];
    if (order_cnt)
        for (int i = threadIdx.x; i < 27 * ORDER_BINS; i += blockDim.x) okeys[i] = 0;
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
    if (order_cnt) {
        const int d[3] = {dims.x, dims.y, dims.z};
        for (int k = 0; k < 4; k++)
            if (base + k < ncell) atomicAdd(&okeys[order_key(d, base + k, v[k])], 1);
        __syncthreads();
        for (int i = threadIdx.x; i < 27 * ORDER_BINS; i += blockDim.x)
            if (okeys[i]) atomicAdd(order_cnt + i, okeys[i]);
    }
}

// One block: sequential prefix over the (few) block sums; with order_cnt (1024 threads), the
// exclusive scan of the order keys' counts into order_off, the counts reset to zero.
__global__ void k_scan_sums(int32_t *block_sums, int nblocks, int32_t *start, int ncell, int32_t *order_cnt,
                            int32_t *order_off) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int run = 0;
        for (int b = 0; b < nblocks; b++) {
            int v = block_sums[b];
            block_sums[b] = run;
            run += v;
        }
        start[ncell] = run;
    }
    if (!order_cnt) return;
    static_assert(27 * ORDER_BINS <= 1024, "one thread per order key");
    __shared__ int32_t warp_sum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int v = t < 27 * ORDER_BINS ? order_cnt[t] : 0;
    int incl = v;
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
        int x = warp_sum[lane];
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        warp_sum[lane] = x;  // inclusive over warps
    }
    __syncthreads();
    if (t < 27 * ORDER_BINS) {
        order_off[t] = (w > 0 ? warp_sum[w - 1] : 0) + incl - v;
        order_cnt[t] = 0;
    }
}

// Block offsets added to the cell starts; with order, each cell placed in its key's range
// (ranks block-local in shared memory, one global reservation per key and block).
__global__ void __launch_bounds__(256) k_scan_add(int32_t *start, const int32_t *block_sums, int ncell,
                                                   const int32_t *count, int3 dims, int32_t *order_off,
                                                   int32_t *order) {
    __shared__ int32_t okeys[27 * ORDER_BINS], obase[27 * ORDER_BINS];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncell) start[i] += block_sums[i / 4096];
    if (!order) return;
    for (int k = threadIdx.x; k < 27 * ORDER_BINS; k += blockDim.x) okeys[k] = 0;
    __syncthreads();
    const int d[3] = {dims.x, dims.y, dims.z};
    const int key = i < ncell ? order_key(d, i, count[i]) : -1;
    const int rank = key >= 0 ? atomicAdd(&okeys[key], 1) : 0;
    __syncthreads();
    for (int k = threadIdx.x; k < 27 * ORDER_BINS; k += blockDim.x)
        if (okeys[k]) obase[k] = atomicAdd(order_off + k, okeys[k]);
    __syncthreads();
    if (key >= 0) order[obase[key] + rank] = i;
}

__global__ void k_scatter(DevState s, GridDev g) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < s.n) scatter_one(g, i);
}

// Sorts each cell's particles by index (a deterministic order independent of the
// atomic arrival order) and writes the FP32 mirror in cell order.
__global__ void k_cell_finish(DevState s, GridDev g) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell < g.ncell) finish_one(s, g, cell);
}

// The grid of a rescaled box whose cells are the old grid's cells (same divisions and origin):
// after a box rescale every particle keeps its relative coordinates up to rounding, so it
// normally stays in its cell.  The cell lists, the FP32 axes and centres (unchanged by a
// rescale) are copied from the old grid in its slot order (particle indices ascending in every
// cell, as a rebuild leaves them) and the FP32 cell-local positions are recomputed from the
// rescaled FP64 positions with the rebuild's arithmetic, so the result is the grid a full
// rebuild would build.  A particle whose cell changed raises *moved: the caller then rebuilds.
// One pass, bound like k_assign by the FP64 relative coordinates.
__global__ void k_remap(DevState s, GridDev g, GridDev old, int *moved) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k <= g.ncell) g.start[k] = old.start[k];
    if (k == 0) *g.max_occ = *old.max_occ;
    if (k >= s.n) return;
    const int pid = old.slot_pid[k];
    float3 loc;
    const int cell = locate_one(s, g, pid, loc);
    if (cell != old.pid_cell[pid]) *moved = 1;
    g.slot_pid[k] = pid;
    g.pid_slot[pid] = static_cast<int32_t>(k);
    g.pid_cell[pid] = cell;
    g.mpos[k] = make_float4(loc.x, loc.y, loc.z, __int_as_float(pid));
    g.maxis[k] = old.maxis[k];
    for (int b = 0; b < s.ncen; b++) g.mcen[k * s.ncen + b] = old.mcen[k * s.ncen + b];
}

// Absolute centres of every polysphere (Packing::recalculateAbsoluteInteractionCentres,
// core/Packing.cpp:1041-1047): position + rotated centre, then the PBC correction of
// that point (core/PeriodicBoundaryConditions.cpp:11-22).  One thread per centre.
__global__ void k_abs_centres(DevState s) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= s.n * s.ncen) return;
    const int64_t pid = t / s.ncen;
    d3 p = load_d3(s.pos64 + 3 * pid);
    d3 c = load_d3(s.cen64 + 3 * t);
    d3 q = add3(p, c);
    d3 a = add3(q, pbc_correction(s.box, s.inv, q, nullptr));
    s.abs64[3 * t] = a.x;
    s.abs64[3 * t + 1] = a.y;
    s.abs64[3 * t + 2] = a.z;
}

// ---------------------------------------------------------------------------------
// Rotation table of one sweep: random rotations R = I + k (K + v v^T - |v|^2 I),
// k = 2 / (1 + |v|^2), the Cayley map of v = tan(theta / 2) * axis with theta uniform in
// [-step, step] and the axis uniform on the sphere.  Each table entry is exactly the
// FP64 evaluation of that formula; moves draw an entry or its transpose (the inverse
// rotation) with equal probability, so the proposal distribution is symmetric.
// ---------------------------------------------------------------------------------
__global__ void k_rot_table(double *out64, float *out32, uint32_t count, uint64_t seed, uint64_t counter,
                            float step) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    u4 r = philox(u4{i, 0x726f74u, (uint32_t)counter, (uint32_t)(counter >> 32)}, (uint32_t)seed,
                  (uint32_t)(seed >> 32));
    float z = pm1f(r.a);
    float sphi, cphi;
    sincosf(6.2831853f * u01f(r.b), &sphi, &cphi);
    float rs = sqrtf(fmaxf(0.f, 1.f - z * z));
    float tq = tanf(0.5f * pm1f(r.c) * step);
    double v[3] = {tq * rs * cphi, tq * rs * sphi, tq * z};
    double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double kap = 2.0 / (1.0 + vv);
    double K[9] = {0.0, -v[2], v[1], v[2], 0.0, -v[0], -v[1], v[0], 0.0};
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            double e = (a == b ? 1.0 : 0.0) + kap * (K[3 * a + b] + v[a] * v[b] - (a == b ? vv : 0.0));
            out64[9 * (size_t)i + 3 * a + b] = e;
            out32[12 * (size_t)i + 3 * a + b] = (float)e;
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
    if (slot < s.n) count_one<KIND>(s, g, slot, early, out, flag);
}

template __global__ void k_count<0>(DevState, GridDev, int, unsigned long long *, int *);
template __global__ void k_count<1>(DevState, GridDev, int, unsigned long long *, int *);

// All-pairs recount of polyspheres: one thread per body; every unordered body pair and
// periodic image once, every pair of their centres (the count of overlapping centre pairs,
// as the reference's countTotalOverlaps counts them, core/Packing.cpp:468-512).
__global__ void k_count_poly(DevState s, GridDev g, int early, unsigned long long *out, int *flag) {
    int64_t slot = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (slot < s.n) count_poly_one(s, g, slot, early, out, flag);
}

// MODE 1 instantiates the learned-ordering pre-test and the pair-outcome log, MODE 2 the
// overlap counting, MODE 3 the plain scan of rototranslations (kept out of the plain
// kernel, whose registers and branches they would crowd)
template <int KIND, bool LIST, int MODE, int GW>
__global__ void __launch_bounds__(SWEEP_WARPS * 32, SWEEP_MIN_BLOCKS) k_sweep(const SweepArgs A) {
    extern __shared__ float4 smem[];
    const Grp<GW> grp;
    const int lane = grp.lane;
    const int gib = threadIdx.x / GW;                 // the lane group (one cell at a time) in the block
    const int groups_per_block = blockDim.x / GW;
    const int group = blockIdx.x * groups_per_block + gib;
    // per-group shared memory (float4 units): staged positions [cap], spherocylinder axes
    // [cap] (with two cells per warp their mirror slots [cap uint32] instead) or polysphere
    // mirror slots [cap uint32], two uint16 queues and a byte counter per slot [5 cap bytes],
    // partner slots [LEARN], polysphere scratch [SWEEP_POLY_SCRATCH]
    constexpr bool AXM = GW == 16 && KIND == 1;
    const int extra = KIND == 1 ? (AXM ? A.cap / 4 : A.cap) : (KIND == 2 ? A.cap / 4 : 0);
    constexpr bool LEARN = MODE == 1;
    const int per_group = A.cap + extra + A.cap / 4 + A.cap / 16 + (LEARN ? A.cap / 4 : 0) +
                          (KIND == 2 ? SWEEP_POLY_SCRATCH : 0);
    float4 *cpos = smem + (size_t)gib * per_group;
    float4 *cax = cpos + A.cap;                                  // spherocylinders
    uint32_t *cslot = reinterpret_cast<uint32_t *>(cpos + A.cap); // mirror slot of each candidate
    uint16_t *qseg = reinterpret_cast<uint16_t *>(cpos + A.cap + extra);
    uint16_t *qun = qseg + A.cap;
    uint8_t *nacc = reinterpret_cast<uint8_t *>(qun + A.cap);
    uint16_t *pstage = reinterpret_cast<uint16_t *>(nacc + A.cap);  // LEARN only: MLP_PARTNERS x cap
    // polyspheres: after the partner slots when the learned ordering is on
    float4 *wx = reinterpret_cast<float4 *>(nacc + A.cap) + (LEARN ? A.cap / 4 : 0);
    int nitems = A.work ? (A.work_count ? *A.work_count : A.num_work) : (LIST ? A.num_list : A.num_active);
    WarpStats ws{};
    __shared__ uint64_t stage_bar[SWEEP_WARPS];
    if (GW == 32 && A.bulk_stage) {
        // the group's staging barrier: one arrival (lane 0's expected bytes) per phase
        uint64_t *bar = stage_bar + gib;
        if (lane == 0) {
            mbar_init(bar, 1);
            fence_mbar_init();
            fence_proxy_async_smem();
        }
        grp.sync();
        ws.bar = bar;
    }
    // persistent launches (next_item set) take cells from a shared counter until none are
    // left; otherwise groups stride over the cells
    const int stride = gridDim.x * groups_per_block;
    int item = group;
    for (;;) {
        if (A.next_item) {
            int it = 0;
            if (lane == 0) it = atomicAdd(A.next_item, 1);
            item = grp.shfl(it, 0);
        }
        if (item >= nitems) break;
        sweep_cell<KIND, LIST, MODE, GW>(A, item, -1, A.cap, A.overflow, A.overflow_count, cpos, cax, qseg, qun, nacc,
                                          pstage, cslot, wx, ws);
        grp.sync();
        if (ws.abort) break;
        item += stride;
    }
    // ---- statistics ----
    unsigned pairs = ws.pairs;
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
        atomicAdd(C + 8, (unsigned long long)ws.acc_trans);
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
    const int3 dims = make_int3(g.dims[0], g.dims[1], g.dims[2]);
    const bool ord = g.order && g.order_cnt && g.order_off;
    k_scan_blocks<<<nblocks, 1024, 0, st>>>(g.count, g.start, block_sums, g.ncell, g.max_occ, dims,
                                             ord ? g.order_cnt : nullptr);
    k_scan_sums<<<1, ord ? 1024 : 32, 0, st>>>(block_sums, nblocks, g.start, g.ncell, ord ? g.order_cnt : nullptr,
                                                ord ? g.order_off : nullptr);
    k_scan_add<<<(g.ncell + 255) / 256, 256, 0, st>>>(g.start, block_sums, g.ncell, g.count, dims,
                                                      ord ? g.order_off : nullptr, ord ? g.order : nullptr);
    k_scatter<<<nb, tb, 0, st>>>(s, g);
    k_cell_finish<<<(g.ncell + 127) / 128, 128, 0, st>>>(s, g);
    return cudaGetLastError();
}

cudaError_t launch_remap(const DevState &s, const GridDev &g, const GridDev &old, int *moved, cudaStream_t st) {
    const int64_t threads = s.n > static_cast<int64_t>(g.ncell) + 1 ? s.n : static_cast<int64_t>(g.ncell) + 1;
    k_remap<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(s, g, old, moved);
    return cudaGetLastError();
}

// Exclusive scan of `ncell` counts into start[0..ncell] (start[ncell] = total); block_sums
// holds (ncell + 4095) / 4096 entries; max_occ receives the largest count.
cudaError_t launch_cell_scan(const int32_t *count, int32_t *start, int32_t *block_sums, int ncell,
                             int32_t *max_occ, cudaStream_t st) {
    int nblocks = (ncell + 4095) / 4096;
    k_scan_blocks<<<nblocks, 1024, 0, st>>>(count, start, block_sums, ncell, max_occ, make_int3(1, 1, 1), nullptr);
    k_scan_sums<<<1, 32, 0, st>>>(block_sums, nblocks, start, ncell, nullptr, nullptr);
    k_scan_add<<<(ncell + 255) / 256, 256, 0, st>>>(start, block_sums, ncell, nullptr, make_int3(1, 1, 1), nullptr,
                                                      nullptr);
    return cudaGetLastError();
}

cudaError_t launch_validate(const DevState &s, cudaStream_t st) {
    if (s.n == 0) return cudaSuccess;
    k_validate<<<(unsigned)((s.n + 255) / 256), 256, 0, st>>>(s);
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

// The recount's deferred centre pairs, one per thread: the exact FP64 test (with the
// polyspherocylinder segments' half axes), overlaps added to the count.
__global__ void k_count_deferred(DevState s, int early, unsigned long long *out, int *flag) {
    const int n = min(*s.cq_count, s.cq_cap);
    unsigned long long cnt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (early && *(volatile int *)flag) break;   // an overlap is already known
        const DeferredPair e = s.cq_buf[i];
        const int a = e.aj / MAX_CEN, j = e.aj % MAX_CEN;
        d3 ha{0.0, 0.0, 0.0};
        if (s.segs) ha = mv3(s.rot64 + 9 * (size_t)e.pid, d3{s.chax[a][0], s.chax[a][1], s.chax[a][2]});
        const d3 pa = load_d3(s.abs64 + 3 * ((size_t)e.pid * s.ncen + a));
        if (exact_centre_pair(s, pa, a, e.pj, j, make_float3(e.d.x, e.d.y, e.d.z), ha)) {
            cnt++;
            if (early) atomicExch(flag, 1);
        }
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(out, cnt);
}

cudaError_t launch_count(const DevState &s, const GridDev &g, int early, unsigned long long *out, int *flag,
                         cudaStream_t st) {
    unsigned nb = (unsigned)((s.n + 127) / 128);
    if (s.kind == 0) k_count<0><<<nb, 128, 0, st>>>(s, g, early, out, flag);
    else if (s.kind == 1) k_count<1><<<nb, 128, 0, st>>>(s, g, early, out, flag);
    else k_count_poly<<<nb, 128, 0, st>>>(s, g, early, out, flag);
    if (s.kind == 2 && s.cq_buf) {
        int sms = 152, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        k_count_deferred<<<sms * 8, 128, 0, st>>>(s, early, out, flag);
    }
    return cudaGetLastError();
}

cudaError_t launch_abs_centres(const DevState &s, cudaStream_t st) {
    int64_t t = s.n * s.ncen;
    if (t == 0) return cudaSuccess;
    k_abs_centres<<<(unsigned)((t + 255) / 256), 256, 0, st>>>(s);
    return cudaGetLastError();
}

size_t sweep_smem_per_warp(int kind, int cap, bool learn, int ncen) {
    const int extra = kind == 1 ? cap : (kind == 2 ? cap / 4 : 0);
    return (size_t)(cap + extra + cap / 4 + cap / 16 + (learn ? cap / 4 : 0) + (kind == 2 ? SWEEP_POLY_SCRATCH : 0)) *
           sizeof(float4);
}

// Shared memory of one cell's lane group when each warp sweeps two cells (spheres and
// spherocylinders, plain scans): the axes stay in the mirror, a slot index per candidate.
size_t sweep_smem_per_half(int kind, int cap) {
    const int extra = kind == 1 ? cap / 4 : 0;
    return (size_t)(cap + extra + cap / 4 + cap / 16) * sizeof(float4);
}

// Resident blocks per SM of the two-cells-per-warp sweep at staging capacity `cap`.
int sweep_half_blocks_per_sm(int kind, int cap) {
    const size_t smem = sweep_smem_per_half(kind, cap) * (SWEEP_WARPS * 2);
    int n = 0;
    cudaError_t e = kind == 0 ? cudaFuncSetAttribute(k_sweep<0, false, 0, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)smem)
                              : cudaFuncSetAttribute(k_sweep<1, false, 0, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)smem);
    if (e != cudaSuccess) return 0;
    e = kind == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep<0, false, 0, 16>, SWEEP_WARPS * 32, smem)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep<1, false, 0, 16>, SWEEP_WARPS * 32, smem);
    return e == cudaSuccess ? n : 0;
}

cudaError_t launch_rot_table(double *out64, float *out32, uint32_t count, uint64_t seed, uint64_t counter, float step,
                             cudaStream_t st) {
    k_rot_table<<<(count + 255) / 256, 256, 0, st>>>(out64, out32, count, seed, counter, step);
    return cudaGetLastError();
}

template <int KIND, bool LIST, int MODE, int GW = 32>
static cudaError_t launch_sweep_t(const SweepArgs &a, unsigned blocks, int threads, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_sweep<KIND, LIST, MODE, GW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    k_sweep<KIND, LIST, MODE, GW><<<blocks, threads, smem, st>>>(a);
    return cudaGetLastError();
}

// The plain scan of spheres or spherocylinders with two cells per warp: `ncells` lane groups
// of 16 (a.cap sized for sweep_smem_per_half).
cudaError_t launch_sweep_half(const SweepArgs &a, int ncells, cudaStream_t st) {
    if (ncells <= 0) return cudaSuccess;
    const int groups_per_block = SWEEP_WARPS * 2;
    const size_t smem = sweep_smem_per_half(a.s.kind, a.cap) * groups_per_block;
    const unsigned blocks = (unsigned)((ncells + groups_per_block - 1) / groups_per_block);
    const int th = SWEEP_WARPS * 32;
    return a.s.kind == 0 ? launch_sweep_t<0, false, 0, 16>(a, blocks, th, smem, st)
                         : launch_sweep_t<1, false, 0, 16>(a, blocks, th, smem, st);
}

cudaError_t launch_sweep(const SweepArgs &a, bool list, int nwarps, cudaStream_t st) {
    if (nwarps <= 0) return cudaSuccess;
    // the overflow rerun (large capacity, device-side count): one warp per block
    const int wpb = (a.work && a.work_count) ? 1 : SWEEP_WARPS;
    const bool count = a.s.counting != 0;
    // rototranslation sweeps have their own plain scan (no learned pre-test, no pair log)
    const bool rt = !list && !count && a.types == SWEEP_ROTOTRANSLATION;
    const bool learn = !list && !count && !rt && (a.partners != nullptr || a.pair_every > 0);
    size_t smem = sweep_smem_per_warp(a.s.kind, a.cap, learn, a.s.ncen) * wpb;
    unsigned blocks = (unsigned)((nwarps + wpb - 1) / wpb);
    const int th = wpb * 32;
    if (a.s.kind == 2) {
        if (count) return list ? launch_sweep_t<2, true, 2>(a, blocks, th, smem, st)
                               : launch_sweep_t<2, false, 2>(a, blocks, th, smem, st);
        if (list) return launch_sweep_t<2, true, 0>(a, blocks, th, smem, st);
        if (learn) return launch_sweep_t<2, false, 1>(a, blocks, th, smem, st);
        return rt ? launch_sweep_t<2, false, 3>(a, blocks, th, smem, st)
                  : launch_sweep_t<2, false, 0>(a, blocks, th, smem, st);
    }
    if (rt) return a.s.kind == 0 ? launch_sweep_t<0, false, 3>(a, blocks, th, smem, st)
                                 : launch_sweep_t<1, false, 3>(a, blocks, th, smem, st);
    if (a.s.kind == 0) {
        if (count) return list ? launch_sweep_t<0, true, 2>(a, blocks, th, smem, st)
                               : launch_sweep_t<0, false, 2>(a, blocks, th, smem, st);
        if (list) return launch_sweep_t<0, true, 0>(a, blocks, th, smem, st);
        return learn ? launch_sweep_t<0, false, 1>(a, blocks, th, smem, st)
                     : launch_sweep_t<0, false, 0>(a, blocks, th, smem, st);
    }
    if (count) return list ? launch_sweep_t<1, true, 2>(a, blocks, th, smem, st)
                           : launch_sweep_t<1, false, 2>(a, blocks, th, smem, st);
    if (list) return launch_sweep_t<1, true, 0>(a, blocks, th, smem, st);
    return learn ? launch_sweep_t<1, false, 1>(a, blocks, th, smem, st)
                 : launch_sweep_t<1, false, 0>(a, blocks, th, smem, st);
}

}  // namespace rp
