// Learned neighbour ordering (rp_mlp.cuh): training kernels (forward, backward, Adam) on
// logged pair outcomes, tensor-core inference (mma.sync m16n8k16, BF16 operands, FP32
// accumulation), and the per-sweep partner ranking the move sweep pre-tests.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "rp_internal.cuh"
#include "rp_mlp.cuh"

namespace rp {

__device__ __forceinline__ float bfr(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ---------------------------------------------------------------------------------
// Gradient of the mean binary cross-entropy over a batch, one block per slice of the
// batch, 64 pairs at a time with every activation in shared memory.  The forward pass
// rounds each layer's inputs and weights to BF16 (what the tensor cores see) and
// accumulates in FP32; the backward pass is FP32.
// ---------------------------------------------------------------------------------
constexpr int GB = 32;  // pairs per mini-tile (static shared memory stays under 48 KB)
constexpr int GT = 256; // threads per block

// Row r of the batch is pair (i0 + r) * mul + off (mod total) of the data set: a seeded
// shuffle when gcd(mul, total) = 1, the identity for mul = 1, off = 0.
struct BatchMap {
    int64_t i0, mul, off, total;
    __device__ __forceinline__ int64_t operator()(int64_t r) const {
        return (int64_t)(((unsigned long long)(i0 + r) * (unsigned long long)mul + (unsigned long long)off) %
                         (unsigned long long)total);
    }
};

__global__ void __launch_bounds__(GT) k_mlp_grad(const float *feats, const uint8_t *labels, int n, BatchMap map,
                                                  float inv_n, const float *w32, float *grad, float *loss_out) {
    __shared__ float W1[MLP_H * MLP_IN], W2[MLP_H * MLP_H], B1[MLP_H], B2[MLP_H], W3[MLP_H];
    __shared__ float X[GB * MLP_IN], H1[GB * MLP_H], H2[GB * MLP_H], DH[GB * MLP_H], DY[GB];
    const int tid = threadIdx.x;
    for (int i = tid; i < MLP_H * MLP_IN; i += GT) W1[i] = bfr(w32[MLP_W1 + i]);
    for (int i = tid; i < MLP_H * MLP_H; i += GT) W2[i] = bfr(w32[MLP_W2 + i]);
    if (tid < MLP_H) {
        B1[tid] = w32[MLP_B1 + tid];
        B2[tid] = w32[MLP_B2 + tid];
        W3[tid] = bfr(w32[MLP_W3 + tid]);
    }
    const float b3 = w32[MLP_B3];
    // per-thread gradient accumulators: W2 entries tid + 256 q, W1 entries tid + 256 q
    float gW2[16], gW1[4];
    for (int q = 0; q < 16; q++) gW2[q] = 0.f;
    for (int q = 0; q < 4; q++) gW1[q] = 0.f;
    float gB1 = 0.f, gB2 = 0.f, gW3 = 0.f, gB3 = 0.f, loss = 0.f;
    __syncthreads();
    for (int base = blockIdx.x * GB; base < n; base += gridDim.x * GB) {
        const int cnt = min(GB, n - base);
        for (int i = tid; i < GB * MLP_IN; i += GT) {
            int p = i / MLP_IN;
            X[i] = p < cnt ? bfr(feats[(size_t)map(base + p) * MLP_IN + (i % MLP_IN)]) : 0.f;
        }
        __syncthreads();
        // layer 1: H1 = relu(W1 x + b1), kept as the BF16 value layer 2 consumes
        for (int i = tid; i < GB * MLP_H; i += GT) {
            int p = i / MLP_H, o = i % MLP_H;
            float s = B1[o];
            for (int k = 0; k < MLP_IN; k++) s = fmaf(W1[o * MLP_IN + k], X[p * MLP_IN + k], s);
            H1[i] = s > 0.f ? bfr(s) : 0.f;
        }
        __syncthreads();
        for (int i = tid; i < GB * MLP_H; i += GT) {
            int p = i / MLP_H, o = i % MLP_H;
            float s = B2[o];
            for (int k = 0; k < MLP_H; k++) s = fmaf(W2[o * MLP_H + k], H1[p * MLP_H + k], s);
            H2[i] = s > 0.f ? s : 0.f;
        }
        __syncthreads();
        if (tid < GB) {
            float y = b3;
            for (int k = 0; k < MLP_H; k++) y = fmaf(W3[k], bfr(H2[tid * MLP_H + k]), y);
            float dy = 0.f;
            if (tid < cnt) {
                float lab = labels[map(base + tid)] ? 1.f : 0.f;
                float sg = 1.f / (1.f + __expf(-y));
                dy = (sg - lab) * inv_n;
                // numerically stable BCE with logits: max(y,0) - y*lab + log(1 + exp(-|y|))
                loss += (fmaxf(y, 0.f) - y * lab + log1pf(__expf(-fabsf(y)))) * inv_n;
            }
            DY[tid] = dy;
        }
        __syncthreads();
        // dW3, dB3 and dH2 = dy w3 [h2 > 0]
        if (tid < MLP_H) {
            float s = 0.f;
            for (int p = 0; p < GB; p++) s = fmaf(DY[p], bfr(H2[p * MLP_H + tid]), s);
            gW3 += s;
        }
        if (tid == 0)
            for (int p = 0; p < GB; p++) gB3 += DY[p];
        for (int i = tid; i < GB * MLP_H; i += GT) {
            int p = i / MLP_H, o = i % MLP_H;
            DH[i] = H2[i] > 0.f ? DY[p] * W3[o] : 0.f;
        }
        __syncthreads();
        // dW2 = sum_p dH2 h1^T, dB2 = sum_p dH2
        for (int q = 0; q < 16; q++) {
            int e = tid + GT * q, o = e / MLP_H, k = e % MLP_H;
            float s = 0.f;
            for (int p = 0; p < GB; p++) s = fmaf(DH[p * MLP_H + o], H1[p * MLP_H + k], s);
            gW2[q] += s;
        }
        if (tid < MLP_H) {
            float s = 0.f;
            for (int p = 0; p < GB; p++) s += DH[p * MLP_H + tid];
            gB2 += s;
        }
        __syncthreads();
        // dH1 = W2^T dH2 [h1 > 0], written over H2 (no longer needed)
        for (int i = tid; i < GB * MLP_H; i += GT) {
            int p = i / MLP_H, k = i % MLP_H;
            float s = 0.f;
            for (int o = 0; o < MLP_H; o++) s = fmaf(W2[o * MLP_H + k], DH[p * MLP_H + o], s);
            H2[i] = H1[i] > 0.f ? s : 0.f;
        }
        __syncthreads();
        for (int q = 0; q < 4; q++) {
            int e = tid + GT * q, o = e / MLP_IN, k = e % MLP_IN;
            float s = 0.f;
            for (int p = 0; p < GB; p++) s = fmaf(H2[p * MLP_H + o], X[p * MLP_IN + k], s);
            gW1[q] += s;
        }
        if (tid < MLP_H) {
            float s = 0.f;
            for (int p = 0; p < GB; p++) s += H2[p * MLP_H + tid];
            gB1 += s;
        }
        __syncthreads();
    }
    for (int q = 0; q < 16; q++) atomicAdd(grad + MLP_W2 + tid + GT * q, gW2[q]);
    for (int q = 0; q < 4; q++) atomicAdd(grad + MLP_W1 + tid + GT * q, gW1[q]);
    if (tid < MLP_H) {
        atomicAdd(grad + MLP_B1 + tid, gB1);
        atomicAdd(grad + MLP_B2 + tid, gB2);
        atomicAdd(grad + MLP_W3 + tid, gW3);
    }
    if (tid == 0) atomicAdd(grad + MLP_B3, gB3);
    if (tid < GB && loss != 0.f) atomicAdd(loss_out, loss);  // threads < GB accumulated losses
}

// Adam step on the FP32 master parameters; refreshes the BF16 copies.
__global__ void k_mlp_adam(float *w32, __nv_bfloat16 *w16, const float *grad, float *m, float *v, float lr,
                           float beta1, float beta2, float eps, float corr1, float corr2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_NPARAM) return;
    float g = grad[i];
    float mi = beta1 * m[i] + (1.f - beta1) * g;
    float vi = beta2 * v[i] + (1.f - beta2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float w = w32[i] - lr * (mi / corr1) / (sqrtf(vi / corr2) + eps);
    w32[i] = w;
    w16[i] = __float2bfloat16_rn(w);
}

__global__ void k_mlp_sync16(const float *w32, __nv_bfloat16 *w16) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < MLP_NPARAM) w16[i] = __float2bfloat16_rn(w32[i]);
}

// ---------------------------------------------------------------------------------
// Tensor-core inference of one tile of 16 pairs on one warp.  A fragments hold the tile's
// features, B fragments the BF16 weights; the layer-1 accumulators are re-packed in
// registers as the layer-2 A fragments (the m16n8 C layout of two adjacent n-tiles is the
// m16k16 A layout).  Returns the logits of rows g and g + 8 (g = lane / 4) in y0, y1.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// w16s: the BF16 parameters staged in shared memory (MLP_NPARAM values, W1/W2 rows
// contiguous); fa / fb: the 16 features of tile rows g and g + 8 of this lane.
__device__ __forceinline__ void mlp_tile(const __nv_bfloat16 *w16s, const float *w32, const float *fa,
                                         const float *fb, float &y0, float &y1) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a[4];
    a[0] = pack_bf16(fa[2 * t], fa[2 * t + 1]);
    a[1] = pack_bf16(fb[2 * t], fb[2 * t + 1]);
    a[2] = pack_bf16(fa[2 * t + 8], fa[2 * t + 9]);
    a[3] = pack_bf16(fb[2 * t + 8], fb[2 * t + 9]);
    (void)g;
    const uint32_t *W1u = reinterpret_cast<const uint32_t *>(w16s + MLP_W1);
    const uint32_t *W2u = reinterpret_cast<const uint32_t *>(w16s + MLP_W2);
    // layer 1: 8 n-tiles of 8 hidden units
    float h1[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int o = nt * 8 + g;
        float bias0 = w32[MLP_B1 + nt * 8 + 2 * t], bias1 = w32[MLP_B1 + nt * 8 + 2 * t + 1];
        h1[nt][0] = bias0;
        h1[nt][1] = bias1;
        h1[nt][2] = bias0;
        h1[nt][3] = bias1;
        mma_bf16(h1[nt], a, W1u[(o * MLP_IN + 2 * t) >> 1], W1u[(o * MLP_IN + 2 * t + 8) >> 1]);
#pragma unroll
        for (int q = 0; q < 4; q++) h1[nt][q] = fmaxf(h1[nt][q], 0.f);
    }
    // layer 2: 8 n-tiles x 4 k-tiles
    float h2[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        float bias0 = w32[MLP_B2 + nt * 8 + 2 * t], bias1 = w32[MLP_B2 + nt * 8 + 2 * t + 1];
        h2[nt][0] = bias0;
        h2[nt][1] = bias1;
        h2[nt][2] = bias0;
        h2[nt][3] = bias1;
    }
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        uint32_t a2[4];
        a2[0] = pack_bf16(h1[2 * kt][0], h1[2 * kt][1]);
        a2[1] = pack_bf16(h1[2 * kt][2], h1[2 * kt][3]);
        a2[2] = pack_bf16(h1[2 * kt + 1][0], h1[2 * kt + 1][1]);
        a2[3] = pack_bf16(h1[2 * kt + 1][2], h1[2 * kt + 1][3]);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int o = nt * 8 + g;
            mma_bf16(h2[nt], a2, W2u[(o * MLP_H + kt * 16 + 2 * t) >> 1], W2u[(o * MLP_H + kt * 16 + 2 * t + 8) >> 1]);
        }
    }
    // layer 3: row dot products, reduced over the four lanes of a row group
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        float w0 = __bfloat162float(w16s[MLP_W3 + nt * 8 + 2 * t]);
        float w1 = __bfloat162float(w16s[MLP_W3 + nt * 8 + 2 * t + 1]);
        s0 = fmaf(w0, bfr(fmaxf(h2[nt][0], 0.f)), fmaf(w1, bfr(fmaxf(h2[nt][1], 0.f)), s0));
        s1 = fmaf(w0, bfr(fmaxf(h2[nt][2], 0.f)), fmaf(w1, bfr(fmaxf(h2[nt][3], 0.f)), s1));
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    y0 = s0 + w32[MLP_B3];
    y1 = s1 + w32[MLP_B3];
}

__global__ void k_mlp_predict(const float *feats, int n, const float *w32, const __nv_bfloat16 *w16, float *out) {
    __shared__ __align__(16) __nv_bfloat16 ws[MLP_NPARAM + 7];
    for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) ws[i] = w16[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int base = warp * 16;
    if (base >= n) return;
    const int g = lane >> 2;
    float fa[MLP_IN], fb[MLP_IN];
    for (int c = 0; c < MLP_IN; c++) {
        fa[c] = base + g < n ? feats[(size_t)(base + g) * MLP_IN + c] : 0.f;
        fb[c] = base + g + 8 < n ? feats[(size_t)(base + g + 8) * MLP_IN + c] : 0.f;
    }
    float y0, y1;
    mlp_tile(ws, w32, fa, fb, y0, y1);
    if ((lane & 3) == 0) {
        if (base + g < n) out[base + g] = y0;
        if (base + g + 8 < n) out[base + g + 8] = y1;
    }
}

// ---------------------------------------------------------------------------------
// Partner ranking: for every particle, its neighbours within the spherocylinder (or
// sphere) interaction range are scored — by the network (mode 1) or by their centre
// distance (mode 2, the untrained reference ordering) — and the best MLP_PARTNERS particle
// indices are stored for the sweep to pre-test.  One warp per cell.
// ---------------------------------------------------------------------------------
constexpr int SCORE_WARPS = 2;
constexpr int SCORE_CAP = 512;   // staged candidates per warp
constexpr int SCORE_LIST = 64;   // in-range candidates scored per particle

__global__ void __launch_bounds__(SCORE_WARPS * 32) k_score_partners(DevState S, GridDev G, const float *w32,
                                                                     const __nv_bfloat16 *w16, int mode,
                                                                     float inv_range, int32_t *partners) {
    __shared__ __align__(16) __nv_bfloat16 ws[MLP_NPARAM + 7];
    __shared__ float4 spos[SCORE_WARPS][SCORE_CAP];
    __shared__ float4 sax[SCORE_WARPS][SCORE_CAP];
    __shared__ uint16_t slist[SCORE_WARPS][SCORE_LIST];
    __shared__ float sscore[SCORE_WARPS][SCORE_LIST];
    const unsigned FULL = 0xffffffffu;
    for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) ws[i] = w16[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int warp = blockIdx.x * SCORE_WARPS + wib;
    if (warp >= G.ncell) return;
    const int cell = warp;
    int c[3] = {cell % G.dims[0], (cell / G.dims[0]) % G.dims[1], cell / (G.dims[0] * G.dims[1])};
    int cnt = 0, st = 0;
    float3 off = make_float3(0.f, 0.f, 0.f);
    if (lane < 27) {
        int t = lane == 0 ? 13 : (lane <= 13 ? lane - 1 : lane);
        int ox = t % 3 - 1, oy = (t / 3) % 3 - 1, oz = t / 9 - 1;
        auto wrap = [](int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); };
        int nb = wrap(c[0] + ox, G.dims[0]) + G.dims[0] * (wrap(c[1] + oy, G.dims[1]) + G.dims[1] * wrap(c[2] + oz, G.dims[2]));
        st = G.start[nb];
        cnt = G.start[nb + 1] - st;
        const float *m = G.cellmat;
        off = make_float3(m[0] * ox + m[1] * oy + m[2] * oz, m[3] * ox + m[4] * oy + m[5] * oz,
                          m[6] * ox + m[7] * oy + m[8] * oz);
    }
    int incl = cnt;
    for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(FULL, incl, d);
        if (lane >= d) incl += y;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    const int occ = __shfl_sync(FULL, cnt, 0);
    const int gbase = __shfl_sync(FULL, st, 0);
    if (total > SCORE_CAP) {
        for (int k = lane; k < occ; k += 32)
            for (int q = 0; q < MLP_PARTNERS; q++) partners[MLP_PARTNERS * (size_t)G.slot_pid[gbase + k] + q] = -1;
        return;
    }
    {
        int b = incl - cnt;
        for (int k = 0; k < cnt; k++) {
            float4 p = G.mpos[st + k];
            p.x += off.x;
            p.y += off.y;
            p.z += off.z;
            spos[wib][b + k] = p;
            sax[wib][b + k] = S.kind == 1 ? G.maxis[st + k] : make_float4(0.f, 0.f, 1.f, 0.f);
        }
    }
    __syncwarp();
    // in reach: spherocylinders and multi-centre bodies within their interaction range,
    // spheres within twice theirs
    const float thr = S.kind == 0 ? S.fc.sphere_hi * 4.0f : S.fc.far_hi;
    for (int i = 0; i < occ; i++) {
        const float4 pi = spos[wib][i];
        const int pid = __float_as_int(pi.w);
        const float4 ai4 = sax[wib][i];
        const float3 ai = make_float3(ai4.x, ai4.y, ai4.z);
        float ri[9];
        if (S.kind == 2)
            for (int e = 0; e < 9; e++) ri[e] = (float)S.rot64[9 * (size_t)pid + e];
        // in-range candidates
        int nl = 0;
        for (int b = 0; b < total; b += 32) {
            int k = b + lane;
            bool in = false;
            if (k < total) {
                float4 q = spos[wib][k];
                float dx = q.x - pi.x, dy = q.y - pi.y, dz = q.z - pi.z;
                in = __float_as_int(q.w) != pid && dx * dx + dy * dy + dz * dz < thr;
            }
            unsigned bal = __ballot_sync(FULL, in);
            int pos = nl + __popc(bal & ((1u << lane) - 1u));
            if (in && pos < SCORE_LIST) slist[wib][pos] = (uint16_t)k;
            nl += __popc(bal);
        }
        nl = min(nl, SCORE_LIST);
        __syncwarp();
        // scores (higher = pre-test first)
        if (mode == 1) {
            for (int tb = 0; tb < nl; tb += 16) {
                const int g = lane >> 2;
                float fa[MLP_IN], fb[MLP_IN];
                for (int h = 0; h < 2; h++) {
                    int li = tb + g + 8 * h;
                    float *f = h ? fb : fa;
                    if (li < nl) {
                        int k = slist[wib][li];
                        float4 q = spos[wib][k];
                        if (S.kind == 2) {
                            // bent bodies: features of the whole orientations
                            const double *oj = S.rot64 + 9 * (size_t)__float_as_int(q.w);
                            float rj[9];
                            for (int e = 0; e < 9; e++) rj[e] = (float)oj[e];
                            mlp_features_body(make_float3(q.x - pi.x, q.y - pi.y, q.z - pi.z), ri, rj, inv_range, f);
                        } else {
                            float4 aj = sax[wib][k];
                            mlp_features(make_float3(q.x - pi.x, q.y - pi.y, q.z - pi.z), ai,
                                         make_float3(aj.x, aj.y, aj.z), inv_range, f);
                        }
                    } else {
                        for (int c = 0; c < MLP_IN; c++) f[c] = 0.f;
                    }
                }
                float y0, y1;
                mlp_tile(ws, w32, fa, fb, y0, y1);
                if ((lane & 3) == 0) {
                    if (tb + g < nl) sscore[wib][tb + g] = y0;
                    if (tb + g + 8 < nl) sscore[wib][tb + g + 8] = y1;
                }
            }
        } else {
            for (int li = lane; li < nl; li += 32) {
                float4 q = spos[wib][slist[wib][li]];
                float dx = q.x - pi.x, dy = q.y - pi.y, dz = q.z - pi.z;
                sscore[wib][li] = -(dx * dx + dy * dy + dz * dz);
            }
        }
        __syncwarp();
        // best MLP_PARTNERS by score (warp arg-max, repeated)
        for (int q = 0; q < MLP_PARTNERS; q++) {
            float best = -3.0e38f;
            int bi = -1;
            for (int li = lane; li < nl; li += 32) {
                float sc = sscore[wib][li];
                if (sc > best) {
                    best = sc;
                    bi = li;
                }
            }
            for (int d = 16; d > 0; d >>= 1) {
                float ob = __shfl_xor_sync(FULL, best, d);
                int oi = __shfl_xor_sync(FULL, bi, d);
                if (ob > best || (ob == best && oi >= 0 && (bi < 0 || oi < bi))) {
                    best = ob;
                    bi = oi;
                }
            }
            int pj = -1;
            if (bi >= 0) pj = __float_as_int(spos[wib][slist[wib][bi]].w);
            if (lane == 0) partners[MLP_PARTNERS * (size_t)pid + q] = pj;
            __syncwarp();
            if (lane == 0 && bi >= 0) sscore[wib][bi] = -3.0e38f;
            __syncwarp();
        }
    }
}

cudaError_t launch_mlp_grad(const float *feats, const uint8_t *labels, int64_t total, int64_t i0, int n,
                            int64_t mul, int64_t off, const float *w32, float *grad, float *loss, int num_sms,
                            cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int blocks = min(4 * num_sms, (n + GB - 1) / GB);
    BatchMap map{i0, mul, off, total};
    k_mlp_grad<<<blocks, GT, 0, st>>>(feats, labels, n, map, 1.0f / n, w32, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float *w32, __nv_bfloat16 *w16, const float *grad, float *m, float *v, float lr,
                            int step, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(w32, w16, grad, m, v, lr, b1, b2, 1e-8f, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_mlp_sync16(const float *w32, __nv_bfloat16 *w16, cudaStream_t st) {
    k_mlp_sync16<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(w32, w16);
    return cudaGetLastError();
}

cudaError_t launch_mlp_predict(const float *feats, int n, const float *w32, const __nv_bfloat16 *w16, float *out,
                               cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int warps = (n + 15) / 16;
    k_mlp_predict<<<(warps + 3) / 4, 128, 0, st>>>(feats, n, w32, w16, out);
    return cudaGetLastError();
}

cudaError_t launch_score_partners(const DevState &s, const GridDev &g, const float *w32, const __nv_bfloat16 *w16,
                                  int mode, float inv_range, int32_t *partners, cudaStream_t st) {
    k_score_partners<<<(g.ncell + SCORE_WARPS - 1) / SCORE_WARPS, SCORE_WARPS * 32, 0, st>>>(s, g, w32, w16, mode,
                                                                                          inv_range, partners);
    return cudaGetLastError();
}

}  // namespace rp
