// Batched replicas: many independent packings of one shape kind advanced together.  Each
// launch covers every replica (particles, cells and checkerboard cells numbered
// consecutively across replicas, the replica of an index found by binary search in prefix
// offsets), so a whole batch costs the launches of one system: the cell-list rebuild, one
// persistent sweep launch and one overflow launch per phase, the box-move rescale and the
// recount.  Per replica the arithmetic is exactly the single-system path's (rp_sweep.cuh).
#include <cuda_runtime.h>

#include "rp_sweep.cuh"

namespace rp {

// SweepArgs in float4 units (each warp keeps a shared-memory copy of its replica's arguments)
constexpr int ARGS_F4 = (int)((sizeof(SweepArgs) + sizeof(float4) - 1) / sizeof(float4));
size_t batch_smem_per_warp(int kind, int cap);

namespace {

// Largest r with base[r] <= x (base ascending, base[0] = 0, base[R] = total).
__device__ __forceinline__ int find_rep(const int *base, int R, int x) {
    int lo = 0, hi = R - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_b_zero(const BatchRep *T, const int *cbase, int R) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cbase[R]) return;
    int r = find_rep(cbase, R, c);
    const GridDev &g = T[r].a.g;
    int local = c - cbase[r];
    g.count[local] = 0;
    if (local == 0) *g.max_occ = 0;
}

__global__ void k_b_assign(const BatchRep *T, const int *pbase, int R) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pbase[R]) return;
    int r = find_rep(pbase, R, i);
    assign_one(T[r].a.s, T[r].a.g, i - pbase[r]);
}

// One block per replica: exclusive scan of its cell counts into cell starts.
constexpr int SCAN_THREADS = 1024;
__global__ void __launch_bounds__(SCAN_THREADS) k_b_scan(const BatchRep *T) {
    __shared__ int warp_tot[32];
    const GridDev &g = T[blockIdx.x].a.g;
    const int n = g.ncell;
    const int per = (n + SCAN_THREADS - 1) / SCAN_THREADS;
    const int b = threadIdx.x * per, e = min(n, b + per);
    int sum = 0, mx = 0;
    for (int c = b; c < e; c++) {
        int v = g.count[c];
        sum += v;
        mx = max(mx, v);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = sum;
    for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    if (lane == 31) warp_tot[wid] = incl;
    if (lane == 0) atomicMax(g.max_occ, mx);
    __syncthreads();
    if (wid == 0) {
        int wv = warp_tot[lane], wi = wv;
        for (int d = 1; d < 32; d <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += y;
        }
        warp_tot[lane] = wi - wv;
        if (lane == 31) g.start[n] = wi;
    }
    __syncthreads();
    int run = warp_tot[wid] + incl - sum;
    for (int c = b; c < e; c++) {
        int v = g.count[c];
        g.start[c] = run;
        run += v;
    }
}

__global__ void k_b_scatter(const BatchRep *T, const int *pbase, int R) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pbase[R]) return;
    int r = find_rep(pbase, R, i);
    scatter_one(T[r].a.g, i - pbase[r]);
}

__global__ void k_b_finish(const BatchRep *T, const int *cbase, int R) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cbase[R]) return;
    int r = find_rep(cbase, R, c);
    finish_one(T[r].a.s, T[r].a.g, c - cbase[r]);
}

// Box move: newBox · (oldBox^-1 · r) for the particles of every rescaled replica, and the
// replica's new translation table (core/Packing.cpp:183-184, core/NeighbourGrid.cpp:203-217).
__global__ void k_b_rescale(const BatchRep *T, const int *pbase, int R) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pbase[R]) return;
    int r = find_rep(pbase, R, i);
    const BatchRep &B = T[r];
    if (!B.scale) return;
    const int64_t l = i - pbase[r];
    d3 p = d3{B.scale_src[3 * l], B.scale_src[3 * l + 1], B.scale_src[3 * l + 2]};
    d3 q = mv3(B.new_box, mv3(B.old_inv, p));
    B.scale_dst[3 * l] = q.x;
    B.scale_dst[3 * l + 1] = q.y;
    B.scale_dst[3 * l + 2] = q.z;
}

__global__ void k_b_trans(const BatchRep *T, int R) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= R * 125) return;
    const BatchRep &B = T[t / 125];
    if (!B.scale) return;
    int m = t % 125;
    d3 rel{static_cast<double>(m / 25) - 2, static_cast<double>((m / 5) % 5) - 2., static_cast<double>(m % 5) - 2.};
    d3 tr = mv3(B.new_box, rel);
    B.trans_dst[3 * m] = tr.x;
    B.trans_dst[3 * m + 1] = tr.y;
    B.trans_dst[3 * m + 2] = tr.z;
}

template <int KIND>
__global__ void k_b_count(const BatchRep *T, const int *pbase, int R, int early, unsigned long long *out, int *flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pbase[R]) return;
    int r = find_rep(pbase, R, i);
    count_one<KIND>(T[r].a.s, T[r].a.g, i - pbase[r], early, out + r, flags + r);
}

__device__ __forceinline__ void flush_stats(const SweepArgs &A, WarpStats &ws) {
    if ((threadIdx.x & 31) == 0 && ws.moves) {
        unsigned long long *C = A.s.counters;
        atomicAdd(C + 0, (unsigned long long)ws.moves);
        atomicAdd(C + 1, (unsigned long long)ws.accepted);
        atomicAdd(C + 2, (unsigned long long)ws.rej_overlap);
        atomicAdd(C + 3, (unsigned long long)ws.rej_domain);
        atomicAdd(C + 4, (unsigned long long)ws.pairs);
        atomicAdd(C + 5, (unsigned long long)ws.fp64);
        atomicAdd(C + 6, (unsigned long long)ws.trans);
        atomicAdd(C + 7, (unsigned long long)ws.rots);
        atomicAdd(C + 8, (unsigned long long)ws.acc_trans);
    }
    ws = WarpStats{};
}

// Phase k of every replica: persistent warps take checkerboard cells of the whole batch
// from one counter.  item_base holds the prefix offsets of this phase's cells per replica;
// every replica's staging capacity is `cap`.
template <int KIND, int WPB, int MODE>
__global__ void __launch_bounds__(WPB * 32, 16 / WPB)
    k_b_sweep(const BatchRep *T, const int *item_base, int R, int k, int *next_item, int cap) {
    extern __shared__ float4 smem[];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int per_warp = ARGS_F4 + cap * (KIND == 1 ? 2 : 1) + cap / 4 + cap / 16;
    SweepArgs *Aw = reinterpret_cast<SweepArgs *>(smem + (size_t)wib * per_warp);
    float4 *cpos = smem + (size_t)wib * per_warp + ARGS_F4;
    float4 *cax = cpos + cap;
    uint16_t *qseg = reinterpret_cast<uint16_t *>(cpos + cap * (KIND == 1 ? 2 : 1));
    uint16_t *qun = qseg + cap;
    uint8_t *nacc = reinterpret_cast<uint8_t *>(qun + cap);
    const int total = item_base[R];
    WarpStats ws{};
    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(next_item, 1);
        const int item = __shfl_sync(FULL, it, 0);
        if (item >= total) break;
        const int r = find_rep(item_base, R, item);
        const BatchRep &B = T[r];
        if (k >= B.nphases) continue;
        // the replica's arguments, copied into this warp's shared memory (read all through the cell)
        {
            const float4 *src = reinterpret_cast<const float4 *>(&B.a);
            float4 *dst = reinterpret_cast<float4 *>(Aw);
            for (int q = lane; q < ARGS_F4; q += 32) dst[q] = src[q];
            __syncwarp();
        }
        const SweepArgs &A = *Aw;
        const GridDev &G = A.g;
        const int local = item - item_base[r];
        const int ph = B.phases[k];
        int act[3], cc[3], c[3];
        for (int d = 0; d < 3; d++) act[d] = ring_count(G.dims[d], phase_digit(ph, d));
        cc[0] = local % act[0];
        cc[1] = (local / act[0]) % act[1];
        cc[2] = local / (act[0] * act[1]);
        for (int d = 0; d < 3; d++) c[d] = ring_cell(G.dims[d], phase_digit(ph, d), cc[d]);
        const int cell = c[0] + G.dims[0] * (c[1] + G.dims[1] * c[2]);
        sweep_cell<KIND, false, MODE>(A, local, cell, cap, A.overflow, A.overflow_count, cpos, cax, qseg, qun, nacc,
                                          nullptr, nullptr, nullptr, ws);
        __syncwarp();
        flush_stats(A, ws);
        __syncwarp();
    }
}

// The cells of phase k whose neighbourhood did not fit: one block (one warp, large shared
// memory) per replica, over that replica's overflow list; the list is emptied afterwards.
template <int KIND, int MODE>
__global__ void __launch_bounds__(32) k_b_overflow(const BatchRep *T, int k, int cap) {
    extern __shared__ float4 smem[];
    const SweepArgs &A = T[blockIdx.x].a;
    const int count = *A.overflow_count;
    if (count == 0) return;
    float4 *cpos = smem;
    float4 *cax = cpos + cap;
    uint16_t *qseg = reinterpret_cast<uint16_t *>(cpos + cap * (KIND == 1 ? 2 : 1));
    uint16_t *qun = qseg + cap;
    uint8_t *nacc = reinterpret_cast<uint8_t *>(qun + cap);
    WarpStats ws{};
    for (int q = 0; q < count; q++) {
        sweep_cell<KIND, false, MODE>(A, q, A.overflow[q], cap, nullptr, nullptr, cpos, cax, qseg, qun, nacc,
                                          nullptr, nullptr, nullptr, ws);
        __syncwarp();
    }
    flush_stats(A, ws);
    if (threadIdx.x == 0) *A.overflow_count = 0;
    (void)k;
}

template <int KIND, int WPB, int MODE>
cudaError_t launch_b_sweep_t(const BatchRep *T, const int *item_base, int R, int k, int *next_item, int cap,
                             int blocks, cudaStream_t st) {
    const size_t smem = (size_t)WPB * batch_smem_per_warp(KIND, cap);
    cudaError_t e =
        cudaFuncSetAttribute(k_b_sweep<KIND, WPB, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_b_sweep<KIND, WPB, MODE><<<blocks, WPB * 32, smem, st>>>(T, item_base, R, k, next_item, cap);
    return cudaGetLastError();
}

template <int KIND, int MODE>
cudaError_t launch_b_sweep_w(const BatchRep *T, const int *item_base, int R, int k, int *next_item, int cap, int wpb,
                             int blocks, cudaStream_t st) {
    if (wpb == 2) return launch_b_sweep_t<KIND, 2, MODE>(T, item_base, R, k, next_item, cap, blocks, st);
    if (wpb == 8) return launch_b_sweep_t<KIND, 8, MODE>(T, item_base, R, k, next_item, cap, blocks, st);
    return launch_b_sweep_t<KIND, 4, MODE>(T, item_base, R, k, next_item, cap, blocks, st);
}

template <int KIND, int MODE>
cudaError_t launch_b_overflow_t(const BatchRep *T, int R, int k, int cap, cudaStream_t st) {
    const size_t smem = batch_smem_per_warp(KIND, cap);
    cudaError_t e = cudaFuncSetAttribute(k_b_overflow<KIND, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_b_overflow<KIND, MODE><<<R, 32, smem, st>>>(T, k, cap);
    return cudaGetLastError();
}

}  // namespace

// All launchers take the device table T (R replicas) and the device prefix arrays
// item_base / pbase / cbase ([R + 1] each); totals are given for the grid sizes.
cudaError_t launch_b_rebuild(const BatchRep *T, const int *pbase, const int *cbase, int R, int total_particles,
                             int total_cells, cudaStream_t st) {
    const int tb = 256;
    k_b_zero<<<(total_cells + tb - 1) / tb, tb, 0, st>>>(T, cbase, R);
    k_b_assign<<<(total_particles + tb - 1) / tb, tb, 0, st>>>(T, pbase, R);
    k_b_scan<<<R, SCAN_THREADS, 0, st>>>(T);
    k_b_scatter<<<(total_particles + tb - 1) / tb, tb, 0, st>>>(T, pbase, R);
    k_b_finish<<<(total_cells + 127) / 128, 128, 0, st>>>(T, cbase, R);
    return cudaGetLastError();
}

cudaError_t launch_b_rescale(const BatchRep *T, const int *pbase, int R, int total_particles, cudaStream_t st) {
    k_b_rescale<<<(total_particles + 255) / 256, 256, 0, st>>>(T, pbase, R);
    k_b_trans<<<(R * 125 + 255) / 256, 256, 0, st>>>(T, R);
    return cudaGetLastError();
}

cudaError_t launch_b_count(const BatchRep *T, const int *pbase, int R, int total_particles, int kind, int early,
                           unsigned long long *out, int *flags, cudaStream_t st) {
    const unsigned nb = (unsigned)((total_particles + 127) / 128);
    if (kind == 0) k_b_count<0><<<nb, 128, 0, st>>>(T, pbase, R, early, out, flags);
    else k_b_count<1><<<nb, 128, 0, st>>>(T, pbase, R, early, out, flags);
    return cudaGetLastError();
}

size_t batch_smem_per_warp(int kind, int cap) {
    return (size_t)(ARGS_F4 + cap * (kind == 1 ? 2 : 1) + cap / 4 + cap / 16) * sizeof(float4);
}

cudaError_t launch_b_sweep(const BatchRep *T, const int *item_base, int R, int kind, int k, int *next_item, int cap,
                           int wpb, int blocks, bool rototranslation, cudaStream_t st) {
    if (kind == 0)
        return rototranslation ? launch_b_sweep_w<0, 3>(T, item_base, R, k, next_item, cap, wpb, blocks, st)
                               : launch_b_sweep_w<0, 0>(T, item_base, R, k, next_item, cap, wpb, blocks, st);
    return rototranslation ? launch_b_sweep_w<1, 3>(T, item_base, R, k, next_item, cap, wpb, blocks, st)
                           : launch_b_sweep_w<1, 0>(T, item_base, R, k, next_item, cap, wpb, blocks, st);
}

cudaError_t launch_b_overflow(const BatchRep *T, int R, int kind, int k, int cap, bool rototranslation,
                              cudaStream_t st) {
    if (kind == 0)
        return rototranslation ? launch_b_overflow_t<0, 3>(T, R, k, cap, st) : launch_b_overflow_t<0, 0>(T, R, k, cap, st);
    return rototranslation ? launch_b_overflow_t<1, 3>(T, R, k, cap, st) : launch_b_overflow_t<1, 0>(T, R, k, cap, st);
}

}  // namespace rp
