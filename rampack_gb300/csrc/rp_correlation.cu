// Pair correlations of the particles' focal points (core/observables/correlation/*):
// PairDensityCorrelation and PairAveragedCorrelation over the Radial, Linear and
// LayerwiseRadial enumerators, built on the GPU.
//
// The reference walks all N(N+1)/2 pairs on the CPU.  Here the focal points are binned
// into a cell grid whose cells are at least the enumerator's reach (max_r for the radial
// and the linear one — the latter only along its axis — and sqrt(max_r^2 + layer
// spacing^2) for the layerwise one), so every pair the reference keeps lies in
// neighbouring cells.  One thread per focal point walks the 3x3x3 neighbourhood (pairs
// taken once: later cell-sorted slots only), rejects far pairs with an FP32 test carrying
// a safety margin, and decides the rest in FP64 with the reference's own expressions (its
// periodic translation, projections, sqrt and bin index), so every bin count is the
// reference's exactly.  Bins are accumulated in shared memory per block and flushed with
// 64-bit atomics.  Value sums of the averaged correlations are FP64 sums in another order
// than the reference's serial loop (equal to rounding).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "rampack_gb300.h"
#include "rp_geom.cuh"

namespace rp {

struct PackingView {
    int device;
    cudaStream_t stream;
    int64_t n;
    const double *pos64;
    const double *rot64;
    double box[9], inv[9];
};
int packing_view(void *handle, PackingView *v, std::string &err);
cudaError_t launch_cell_scan(const int32_t *count, int32_t *start, int32_t *block_sums, int ncell,
                             int32_t *max_occ, cudaStream_t st);

namespace {

constexpr double PI = 3.14159265358979323846;
constexpr int CORR_THREADS = 256;
constexpr int SMEM_BINS = 4096;  // bins kept per block in shared memory (64 KB with the sums)

struct CorrGeom {
    double box[9], inv[9];
    float box32[9];
    int nc[3];
    int span[3];     // neighbour cells searched each way: 2 (cells of half the reach), 1, or 0 (one cell)
    int ncell;
    int nb;
    int lin_axis;
    int axis_mode;
    double focal[3], primary[3], secondary[3];
    double k[3], kn[3], tau, dir[3];
    double max_r, step;
    float thr2_32;   // FP32 rejection: squared distance above this is out of reach
    float lin_thr32; // FP32 rejection: |relative separation| along lin_axis above this
    float h32;       // the height across side lin_axis (linear enumerator)
    // FP32 binning: with t = d32 / step (FP32), the FP64 distance / step lies within
    // t -+ (bin_abs + bin_rel * t); in range for sure below in_lo, out of range above in_hi;
    // the bin is floor(t) when the interval stays inside it
    float inv_step32, bin_abs, bin_rel, in_lo, in_hi;
    // layerwise: Miller indices, tau / 2 pi and k / |k| in FP32; the layer value of a point
    // is r . h - tau / 2 pi in relative coordinates (p . k = 2 pi r . h), and bin_abs_lw the
    // absolute bin margin of the in-layer distance (its error grows with the full separation)
    float hm32[3], tau32, kn32[3], bin_abs_lw;
    float edge32;    // no FP32 rejection when a folded relative separation is this near 1/2
    int fp64_only;   // RP_CORR_FP64_ONLY: no FP32 pre-filter
};

struct SortedPoints {
    int32_t *idx;     // slot -> particle
    int32_t *cell;    // slot -> cell
    float4 *rel32;    // relative focal point (FP32 copy for the pre-filter)
    double *f64;      // [slot][3] focal point
    double *r64;      // [slot][3] relative focal point (inverse box x focal point)
    double *ax64;     // [slot][3] correlated axis (averaged correlations)
};

RP_HD double dsqrt(double x) {
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(x);
#else
    return std::sqrt(x);
#endif
}

// geometry/Vector.h:225-228 with Matrix.tpp:178-185: v / |v|, a divisor of 1 skipped.
RP_HD d3 normalized3(d3 v) {
    double n = dsqrt(norm2(v));
    if (n == 1.0) return v;
    return {ddiv(v.x, n), ddiv(v.y, n), ddiv(v.z, n)};
}

// Packing::dumpNamedPoints (core/Packing.cpp:1144-1153): position + orientation * point.
__device__ d3 focal_point(const CorrGeom &G, const double *pos64, const double *rot64, int64_t i) {
    const double *p = pos64 + 3 * i;
    d3 o = mv3(rot64 + 9 * i, d3{G.focal[0], G.focal[1], G.focal[2]});
    return add3(d3{p[0], p[1], p[2]}, o);
}

__device__ int cell_index(const CorrGeom &G, d3 rel) {
    const double r[3] = {rel.x, rel.y, rel.z};
    int c[3];
    for (int k = 0; k < 3; k++) {
        double w = r[k] - floor(r[k]);
        int v = static_cast<int>(w * G.nc[k]);
        c[k] = v < 0 ? 0 : (v >= G.nc[k] ? G.nc[k] - 1 : v);
    }
    return (c[2] * G.nc[1] + c[1]) * G.nc[0] + c[0];
}

__global__ void k_corr_cells(CorrGeom G, const double *pos64, const double *rot64, int64_t n, int32_t *cell_of,
                             int32_t *count, double *focal_out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    d3 f = focal_point(G, pos64, rot64, i);
    int c = cell_index(G, mv3(G.inv, f));
    cell_of[i] = c;
    atomicAdd(count + c, 1);
    if (focal_out) {
        focal_out[3 * i] = f.x;
        focal_out[3 * i + 1] = f.y;
        focal_out[3 * i + 2] = f.z;
    }
}

// AxisCorrelation::calculate (correlation_functions/AxisCorrelation.cpp:9-27) with the
// geometry's axes (orientation * body axis; auxiliary = (primary ^ secondary).normalized()).
__device__ d3 shape_axis(const CorrGeom &G, const double *rot) {
    d3 a1 = mv3(rot, d3{G.primary[0], G.primary[1], G.primary[2]});
    if (G.axis_mode == RP_AXIS_PRIMARY) return a1;
    d3 a2 = mv3(rot, d3{G.secondary[0], G.secondary[1], G.secondary[2]});
    if (G.axis_mode == RP_AXIS_SECONDARY) return a2;
    return normalized3(cross3(a1, a2));
}

__global__ void k_corr_scatter(CorrGeom G, const double *pos64, const double *rot64, int64_t n,
                               const int32_t *cell_of, const int32_t *start, int32_t *fill, SortedPoints S,
                               int want_axes) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cell_of[i];
    int slot = start[c] + atomicAdd(fill + c, 1);
    d3 f = focal_point(G, pos64, rot64, i);
    d3 r = mv3(G.inv, f);
    S.idx[slot] = static_cast<int32_t>(i);
    S.cell[slot] = c;
    S.rel32[slot] = make_float4(static_cast<float>(r.x), static_cast<float>(r.y), static_cast<float>(r.z), 0.f);
    double *fo = S.f64 + 3 * (int64_t)slot, *ro = S.r64 + 3 * (int64_t)slot;
    fo[0] = f.x, fo[1] = f.y, fo[2] = f.z;
    ro[0] = r.x, ro[1] = r.y, ro[2] = r.z;
    if (want_axes) {
        d3 a = shape_axis(G, rot64 + 9 * i);
        double *ao = S.ax64 + 3 * (int64_t)slot;
        ao[0] = a.x, ao[1] = a.y, ao[2] = a.z;
    }
}

// correlation_functions/S110Correlation.h, S220Correlation.h, S221Correlation.h,
// AxesAngle.h (std::pow(x, 2) is the correctly rounded x * x).
template <int F>
__device__ double axis_function(d3 a1, d3 a2, d3 d) {
    double c = dot3(a1, a2);
    if (F == RP_CORR_S110) return c;
    if (F == RP_CORR_S220) return dmul(1.5, dsub(dmul(c, c), 1. / 3));
    if (F == RP_CORR_S221) return dmul(dot3(cross3(a1, a2), normalized3(d)), c);
    return ddiv(dmul(180.0, acos(fabs(c))), PI);
}

__device__ __forceinline__ d3 load3(const double *p, int64_t slot) {
    const double *q = p + 3 * slot;
    return {q[0], q[1], q[2]};
}

// The FP64 decision for the pair of slots (lo, hi), lo holding the lower particle index
// (the reference's pair (i, j), i <= j, with the second point translated): the
// enumerator's separation (RadialEnumerator.cpp:19-25, LinearEnumerator.cpp:58-64,
// LayerwiseRadialEnumerator.cpp:31-43), then the consumer's distance cut and bin
// (PairDensityCorrelation.cpp:29-37, PairAveragedCorrelation.cpp:21-31, Histogram.tpp:61-69).
template <int E, int F>
__device__ void decide_pair(const CorrGeom &G, const SortedPoints &S, int64_t lo, int64_t hi,
                            unsigned long long *hc, double *hs) {
    d3 p1 = load3(S.f64, lo), p2 = load3(S.f64, hi);
    d3 r1 = load3(S.r64, lo), r2 = load3(S.r64, hi);
    // PeriodicBoundaryConditions::getTranslation (core/PeriodicBoundaryConditions.cpp:24-36)
    double a[3] = {r1.x, r1.y, r1.z}, b[3] = {r2.x, r2.y, r2.z}, t[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; k++) {
        while (dsub(dadd(b[k], t[k]), a[k]) > 0.5) t[k] = dsub(t[k], 1.0);
        while (dsub(dadd(b[k], t[k]), a[k]) < -0.5) t[k] = dadd(t[k], 1.0);
    }
    d3 q2 = add3(p2, mv3(G.box, d3{t[0], t[1], t[2]}));
    d3 k3{G.k[0], G.k[1], G.k[2]};
    if (E == RP_PAIRS_LAYERWISE) {
        double l1 = round(ddiv(dsub(dot3(p1, k3), G.tau), 2 * PI));
        double l2 = round(ddiv(dsub(dot3(q2, k3), G.tau), 2 * PI));
        if (l1 != l2) return;
    }
    d3 d = sub3(q2, p1);
    if (E == RP_PAIRS_LINEAR) {
        d3 dir{G.dir[0], G.dir[1], G.dir[2]};
        d = scale3(dir, dot3(d, dir));
    } else if (E == RP_PAIRS_LAYERWISE) {
        d3 kn{G.kn[0], G.kn[1], G.kn[2]};
        d = sub3(d, scale3(kn, dot3(d, kn)));
    }
    double dist = dsqrt(norm2(d));
    if (!(dist <= G.max_r)) return;   // PairDensityCorrelation.cpp:34-35 (distance > max: skipped)
    double q = floor(ddiv(dist, G.step));
    int bin = q >= static_cast<double>(G.nb) ? G.nb - 1 : static_cast<int>(q);
    atomicAdd(hc + bin, 1ull);
    if (F != RP_CORR_DENSITY) atomicAdd(hs + bin, axis_function<F>(load3(S.ax64, lo), load3(S.ax64, hi), d));
}

// One candidate pair (a, b), a's slot below b's: the FP32 pre-filter and binning.  Returns
// true when the pair needs the FP64 decision (the caller queues it).
template <int E, int F>
__device__ __forceinline__ bool examine_pair(const CorrGeom &G, const SortedPoints &S, int64_t a, int64_t b,
                                             float4 ra, unsigned long long *hc, double *hs) {
    const float4 rb = S.rel32[b];
    float f[3] = {rb.x - ra.x, rb.y - ra.y, rb.z - ra.z};
    const float e = 0.5f - G.edge32;
    bool edge = false;
    for (int k = 0; k < 3; k++) {
        f[k] -= rintf(f[k]);
        edge |= fabsf(f[k]) > e;
    }
    const bool fast = !edge && !G.fp64_only;
    float d32 = 0.f;
    if (fast) {
        if (E == RP_PAIRS_LINEAR) {
            const float fa = fabsf(f[0] * (G.lin_axis == 0) + f[1] * (G.lin_axis == 1) + f[2] * (G.lin_axis == 2));
            if (fa > G.lin_thr32) return false;
            d32 = fa * G.h32;
        } else {
            float d2 = 0.f;
            for (int i = 0; i < 3; i++) {
                float v = G.box32[3 * i] * f[0] + G.box32[3 * i + 1] * f[1] + G.box32[3 * i + 2] * f[2];
                d2 += v * v;
            }
            if (d2 > G.thr2_32) return false;
            d32 = d2 > 0.f ? d2 * rsqrtf(d2) : 0.f;   // within 2^-21 relative: inside the margin
        }
    }
    // layerwise: both layer values away from a rounding edge give the reference's layers
    // (different layers: dropped), then the in-layer FP32 distance is binned as below
    float babs = G.bin_abs;
    if (E == RP_PAIRS_LAYERWISE && fast && F != RP_CORR_S221) {
        const float va = ra.x * G.hm32[0] + ra.y * G.hm32[1] + ra.z * G.hm32[2] - G.tau32;
        const float vb = va + (f[0] * G.hm32[0] + f[1] * G.hm32[1] + f[2] * G.hm32[2]);
        const float la = rintf(va), lb = rintf(vb);
        if (fabsf(va - la) > 0.499f || fabsf(vb - lb) > 0.499f) return true;   // near a layer edge: FP64
        if (la != lb) return false;
        float s[3];
        for (int i = 0; i < 3; i++) s[i] = G.box32[3 * i] * f[0] + G.box32[3 * i + 1] * f[1] + G.box32[3 * i + 2] * f[2];
        const float dn = s[0] * G.kn32[0] + s[1] * G.kn32[1] + s[2] * G.kn32[2];
        float d2 = 0.f;
        for (int i = 0; i < 3; i++) {
            const float v = s[i] - dn * G.kn32[i];
            d2 += v * v;
        }
        d32 = d2 > 0.f ? d2 * rsqrtf(d2) : 0.f;
        babs = G.bin_abs_lw;
    }
    // FP32 binning: when the FP64 distance's whole error interval lies in one bin below max_r
    // (or beyond max_r), that bin is the reference's; pairs near a bin edge or max_r are
    // decided in FP64.  S221 (which reads the separation) always takes FP64.
    if (F != RP_CORR_S221 && fast) {
        const float t = d32 * G.inv_step32;
        const float m = babs + G.bin_rel * t;
        if (t - m > G.in_hi) return false;
        const float k = floorf(t), frac = t - k;   // exact
        if (t + m < G.in_lo && frac >= m && frac + m < 1.f) {
            const int bin = min(static_cast<int>(k), G.nb - 1);
            atomicAdd(hc + bin, 1ull);
            if (F != RP_CORR_DENSITY)
                atomicAdd(hs + bin, axis_function<F>(load3(S.ax64, a), load3(S.ax64, b), d3{0.0, 0.0, 0.0}));
            return false;
        }
    }
    return true;
}

// One warp per focal point a: the (up to 27) neighbour cells' slot ranges above a are laid
// end to end and the lanes walk them together, so every lane has the same trip count and
// the loads of consecutive slots coalesce.  Lane l < 27 holds neighbour cell l's first slot
// and the running total of the range lengths; each lane finds the cell of its candidate by
// advancing through that prefix with warp-uniform shuffles.  Pairs that need the FP64
// decision (and the averaged correlations' pairs (i, i)) are queued per warp in shared
// memory and decided 32 at a time, all lanes busy: FP64 issue is scarce on this part.
template <int E, int F>
__global__ void __launch_bounds__(CORR_THREADS, 2) k_corr_pairs(CorrGeom G, SortedPoints S, const int32_t *start,
                                                             int64_t n, int use_smem, unsigned long long *hist,
                                                             double *hsum, unsigned long long *tested) {
    extern __shared__ unsigned long long sh[];
    unsigned long long *hc = hist;
    double *hs = hsum;
    if (use_smem) {
        hc = sh;
        hs = reinterpret_cast<double *>(sh + G.nb);
        for (int b = threadIdx.x; b < G.nb; b += blockDim.x) {
            hc[b] = 0;
            if (F != RP_CORR_DENSITY) hs[b] = 0;
        }
        __syncthreads();
    }
    __shared__ int2 queue[CORR_THREADS / 32][64];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int2 *q = queue[threadIdx.x >> 5];
    int qn = 0;   // queued pairs of this warp (warp-uniform)
    // queue the lanes' pairs with `need` (slots ordered by particle index), and decide a full
    // batch of 32 when there is one
    auto enqueue = [&](bool need, int lo, int hi) {
        const unsigned bal = __ballot_sync(full, need);
        if (bal == 0) return;
        if (need) q[qn + __popc(bal & ((1u << lane) - 1))] = make_int2(lo, hi);
        qn += __popc(bal);
        __syncwarp();
        if (qn >= 32) {
            const int2 pr = q[qn - 32 + lane];
            __syncwarp();
            decide_pair<E, F>(G, S, pr.x, pr.y, hc, hs);
            qn -= 32;
        }
    };
    const int64_t warps = (int64_t)gridDim.x * (CORR_THREADS / 32);
    unsigned long long my_tested = 0;
    // neighbour offsets: -1..1 in a dimension of three or more cells, 0 otherwise
    const int wx = 2 * G.span[0] + 1, wy = 2 * G.span[1] + 1, wz = 2 * G.span[2] + 1;
    const int ncells = wx * wy * wz;   // at most 125
    for (int64_t a = blockIdx.x * (int64_t)(CORR_THREADS / 32) + (threadIdx.x >> 5); a < n; a += warps) {
        const int ia = S.idx[a];
        const int ca = S.cell[a];
        const float4 ra = S.rel32[a];
        if (F != RP_CORR_DENSITY) {  // the averaged correlations also take the pair (i, i)
            enqueue(lane == 0, static_cast<int>(a), static_cast<int>(a));
            my_tested += lane == 0;
        }
        const int cx = ca % G.nc[0], cy = (ca / G.nc[0]) % G.nc[1], cz = ca / (G.nc[0] * G.nc[1]);
        for (int chunk = 0; chunk < ncells; chunk += 32) {   // up to 32 neighbour cells at a time
            const int nbr = chunk + lane;
            int first = 0, len = 0;
            if (nbr < ncells) {
                const int ox = nbr % wx - G.span[0], oy = (nbr / wx) % wy - G.span[1], oz = nbr / (wx * wy) - G.span[2];
                const int x = (cx + ox + G.nc[0]) % G.nc[0], y = (cy + oy + G.nc[1]) % G.nc[1],
                          z = (cz + oz + G.nc[2]) % G.nc[2];
                const int c = (z * G.nc[1] + y) * G.nc[0] + x;
                int64_t b0 = start[c];
                const int64_t b1 = start[c + 1];
                if (b0 <= a) b0 = a + 1;
                first = static_cast<int>(b0);
                len = b1 > b0 ? static_cast<int>(b1 - b0) : 0;
            }
            int incl = len;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(full, incl, o);
                if (lane >= o) incl += y;
            }
            const int total = __shfl_sync(full, incl, 31);
            int cur = 0;
            for (int base = 0; base < total; base += 32) {
                const int k = base + lane;
                for (;;) {   // advance to the cell holding candidate k (at most 32 steps in all)
                    const int end = __shfl_sync(full, incl, cur);
                    const bool adv = k < total && k >= end;
                    if (!__any_sync(full, adv)) break;
                    if (adv) cur++;
                }
                const int cfirst = __shfl_sync(full, first, cur);
                const int cend = __shfl_sync(full, incl, cur);
                const int clen = __shfl_sync(full, len, cur);
                bool need = false;
                int lo = 0, hi = 0;
                if (k < total) {
                    const int b = cfirst + (k - (cend - clen));
                    need = examine_pair<E, F>(G, S, a, b, ra, hc, hs);
                    if (need) {
                        const bool a_first = ia < S.idx[b];
                        lo = a_first ? static_cast<int>(a) : b;
                        hi = a_first ? b : static_cast<int>(a);
                        my_tested++;
                    }
                }
                enqueue(need, lo, hi);
            }
        }
    }
    if (lane < qn) {   // the warp's last, partial batch
        const int2 pr = q[lane];
        decide_pair<E, F>(G, S, pr.x, pr.y, hc, hs);
    }
    for (int o = 16; o > 0; o >>= 1) my_tested += __shfl_xor_sync(full, my_tested, o);
    if (lane == 0 && my_tested) atomicAdd(tested, my_tested);
    if (use_smem) {
        __syncthreads();
        for (int b = threadIdx.x; b < G.nb; b += blockDim.x) {
            if (hc[b]) atomicAdd(hist + b, hc[b]);
            if (F != RP_CORR_DENSITY && hs[b] != 0.0) atomicAdd(hsum + b, hs[b]);
        }
    }
}

template <int E, int F>
cudaError_t launch_pairs_t(const CorrGeom &G, const SortedPoints &S, const int32_t *start, int64_t n, int grid,
                           int use_smem, size_t smem, unsigned long long *hist, double *hsum,
                           unsigned long long *tested, cudaStream_t st) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_corr_pairs<E, F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    k_corr_pairs<E, F><<<grid, CORR_THREADS, smem, st>>>(G, S, start, n, use_smem, hist, hsum, tested);
    return cudaGetLastError();
}

template <int E>
cudaError_t launch_pairs_e(int f, const CorrGeom &G, const SortedPoints &S, const int32_t *start, int64_t n,
                           int grid, int use_smem, size_t smem, unsigned long long *hist, double *hsum,
                           unsigned long long *tested, cudaStream_t st) {
    switch (f) {
        case RP_CORR_DENSITY:
            return launch_pairs_t<E, RP_CORR_DENSITY>(G, S, start, n, grid, use_smem, smem, hist, hsum, tested, st);
        case RP_CORR_S110:
            return launch_pairs_t<E, RP_CORR_S110>(G, S, start, n, grid, use_smem, smem, hist, hsum, tested, st);
        case RP_CORR_S220:
            return launch_pairs_t<E, RP_CORR_S220>(G, S, start, n, grid, use_smem, smem, hist, hsum, tested, st);
        case RP_CORR_S221:
            return launch_pairs_t<E, RP_CORR_S221>(G, S, start, n, grid, use_smem, smem, hist, hsum, tested, st);
        default:
            return launch_pairs_t<E, RP_CORR_AXES_ANGLE>(G, S, start, n, grid, use_smem, smem, hist, hsum, tested,
                                                         st);
    }
}

// ---- host side -----------------------------------------------------------------------

struct Corr {
    rp_pair_desc d{};
    std::string err;
    int device = -1;
    int64_t cap_n = 0;
    int64_t cap_cell = 0;
    int32_t *cell_of = nullptr, *count = nullptr, *start = nullptr, *fill = nullptr, *block_sums = nullptr,
            *max_occ = nullptr;
    SortedPoints S{};
    double *focal_out = nullptr;
    unsigned long long *hist = nullptr, *tested = nullptr;
    double *hsum = nullptr;
    // HistogramBuilder<1> state (HistogramBuilder.tpp): accumulated values and counts
    std::vector<double> value;
    std::vector<uint64_t> total;
    int64_t snapshots = 0;
    std::vector<uint64_t> last_count;
    std::vector<double> last_sum;
    int64_t last_tested = 0;

    int fail(int code, const std::string &m) {
        err = m;
        return code;
    }
    void free_points() {
        for (void *p : {(void *)cell_of, (void *)S.idx, (void *)S.cell, (void *)S.rel32, (void *)S.f64,
                        (void *)S.r64, (void *)S.ax64, (void *)focal_out})
            if (p) cudaFree(p);
        cell_of = nullptr;
        S = SortedPoints{};
        focal_out = nullptr;
        cap_n = 0;
    }
    void free_cells() {
        for (void *p : {(void *)count, (void *)start, (void *)fill, (void *)block_sums})
            if (p) cudaFree(p);
        count = start = fill = block_sums = nullptr;
        cap_cell = 0;
    }
    void free_all() {
        free_points();
        free_cells();
        for (void *p : {(void *)max_occ, (void *)hist, (void *)tested, (void *)hsum})
            if (p) cudaFree(p);
        max_occ = nullptr;
        hist = tested = nullptr;
        hsum = nullptr;
    }
};

bool is_density(const rp_pair_desc &d) { return d.function == RP_CORR_DENSITY; }

// TriclinicBox::getVolume / getHeights (core/TriclinicBox.cpp:35-51).
double box_volume(const double *box) {
    d3 s0 = mv3(box, {1, 0, 0}), s1 = mv3(box, {0, 1, 0}), s2 = mv3(box, {0, 0, 1});
    return std::abs(dot3(cross3(s0, s1), s2));
}
void box_heights(const double *box, double *h) {
    d3 s[3] = {mv3(box, {1, 0, 0}), mv3(box, {0, 1, 0}), mv3(box, {0, 0, 1})};
    double vol = box_volume(box);
    for (int k = 0; k < 3; k++) h[k] = vol / std::sqrt(norm2(cross3(s[(k + 1) % 3], s[(k + 2) % 3])));
}

// LayerwiseRadialEnumerator::calculateK (LayerwiseRadialEnumerator.cpp:12-16).
d3 layer_k(const double *inv, const int32_t *miller) {
    const double t[9] = {inv[0], inv[3], inv[6], inv[1], inv[4], inv[7], inv[2], inv[5], inv[8]};
    d3 v = mv3(t, d3{static_cast<double>(miller[0]), static_cast<double>(miller[1]),
                     static_cast<double>(miller[2])});
    return scale3(v, 2 * PI);
}

// getExpectedNumOfMoleculesInShells of the enumerators (RadialEnumerator.cpp:31-48,
// LinearEnumerator.cpp:18-35, LayerwiseRadialEnumerator.cpp:70-92) for the bin dividers
// (Histogram.tpp:141-151), turned into PairDensityCorrelation's factors
// 2 / expected / N (PairDensityCorrelation.cpp:4-14).
std::vector<double> density_factors(const rp_pair_desc &d, const double *box, const double *inv, int64_t n) {
    const int nb = d.num_bins;
    const double mn = 0.0, mx = d.max_r;
    std::vector<double> bounds(nb + 1);
    const double nbd = static_cast<double>(nb);
    for (int i = 0; i <= nb; i++) {
        double id = static_cast<double>(i);
        bounds[i] = mn * ((nbd - id) / nbd) + mx * (id / nbd);
    }
    const double rho = static_cast<double>(n) / box_volume(box);   // Packing::getNumberDensity
    std::vector<double> expected;
    if (d.enumerator == RP_PAIRS_LINEAR) {
        double h[3];
        box_heights(box, h);
        double area = box_volume(box) / h[d.linear_axis];
        for (int i = 0; i < nb; i++) expected.push_back((bounds[i + 1] - bounds[i]) * area * rho);
    } else {
        std::vector<double> m;
        if (d.enumerator == RP_PAIRS_RADIAL) {
            for (double r : bounds) m.push_back(4. / 3 * PI * r * r * r * rho);
        } else {
            d3 k = layer_k(inv, d.miller);
            double layer = 2 * PI / std::sqrt(norm2(k));
            double area_density = rho * layer;
            for (double r : bounds) m.push_back(PI * r * r * area_density);
        }
        for (int i = 0; i < nb; i++) expected.push_back(m[i + 1] - m[i]);
    }
    for (auto &x : expected) x = 2. / x / static_cast<double>(n);
    return expected;
}

#define CORR_CUDA(c, call)                                                                 \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return (c)->fail(RP_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

int ensure_buffers(Corr *c, const PackingView &v, int64_t ncell, bool axes) {
    if (c->device != v.device) {
        if (c->device >= 0) {
            cudaSetDevice(c->device);
            c->free_all();
        }
        CORR_CUDA(c, cudaSetDevice(v.device));
        c->device = v.device;
    }
    if (!c->hist) {
        const int nb = c->d.num_bins;
        CORR_CUDA(c, cudaMalloc(&c->hist, sizeof(unsigned long long) * nb));
        CORR_CUDA(c, cudaMalloc(&c->hsum, sizeof(double) * nb));
        CORR_CUDA(c, cudaMalloc(&c->tested, sizeof(unsigned long long)));
        CORR_CUDA(c, cudaMalloc(&c->max_occ, sizeof(int32_t)));
    }
    if (v.n > c->cap_n || (axes && !c->S.ax64)) {
        c->free_points();
        const int64_t m = std::max<int64_t>(v.n, 1);
        CORR_CUDA(c, cudaMalloc(&c->cell_of, sizeof(int32_t) * m));
        CORR_CUDA(c, cudaMalloc(&c->S.idx, sizeof(int32_t) * m));
        CORR_CUDA(c, cudaMalloc(&c->S.cell, sizeof(int32_t) * m));
        CORR_CUDA(c, cudaMalloc(&c->S.rel32, sizeof(float4) * m));
        CORR_CUDA(c, cudaMalloc(&c->S.f64, sizeof(double) * 3 * m));
        CORR_CUDA(c, cudaMalloc(&c->S.r64, sizeof(double) * 3 * m));
        CORR_CUDA(c, cudaMalloc(&c->focal_out, sizeof(double) * 3 * m));
        if (axes) CORR_CUDA(c, cudaMalloc(&c->S.ax64, sizeof(double) * 3 * m));
        c->cap_n = m;
    }
    if (ncell > c->cap_cell) {
        c->free_cells();
        CORR_CUDA(c, cudaMalloc(&c->count, sizeof(int32_t) * ncell));
        CORR_CUDA(c, cudaMalloc(&c->fill, sizeof(int32_t) * ncell));
        CORR_CUDA(c, cudaMalloc(&c->start, sizeof(int32_t) * (ncell + 1)));
        CORR_CUDA(c, cudaMalloc(&c->block_sums, sizeof(int32_t) * ((ncell + 4095) / 4096 + 1)));
        c->cap_cell = ncell;
    }
    return RP_OK;
}

int add_snapshot(Corr *c, void *handle) {
    PackingView v{};
    std::string e;
    int rc = packing_view(handle, &v, e);
    if (rc != RP_OK) return c->fail(rc, e);
    CORR_CUDA(c, cudaSetDevice(v.device));
    const rp_pair_desc &d = c->d;
    const bool axes = !is_density(d);
    if (v.n >= (int64_t(1) << 31)) return c->fail(RP_ERR_ARG, "too many particles for the correlation grid");

    CorrGeom G{};
    std::memcpy(G.box, v.box, sizeof(G.box));
    std::memcpy(G.inv, v.inv, sizeof(G.inv));
    for (int i = 0; i < 9; i++) G.box32[i] = static_cast<float>(v.box[i]);
    G.nb = d.num_bins;
    G.lin_axis = d.linear_axis;
    G.axis_mode = d.axis;
    for (int i = 0; i < 3; i++) {
        G.focal[i] = d.focal[i];
        G.primary[i] = d.primary[i];
        G.secondary[i] = d.secondary[i];
    }
    G.max_r = d.max_r;
    G.step = (d.max_r - 0.0) / static_cast<double>(d.num_bins);   // HistogramBuilder.tpp:91-92

    double h[3];
    box_heights(v.box, h);
    // the reach of a kept pair: the distance itself (radial), its projection on the axis
    // (linear) or the in-layer distance with at most one layer spacing across (layerwise)
    double reach = d.max_r;
    if (d.enumerator == RP_PAIRS_LAYERWISE) {
        d3 k = layer_k(v.inv, d.miller);
        d3 kn = normalized3(k);
        G.k[0] = k.x, G.k[1] = k.y, G.k[2] = k.z;
        G.kn[0] = kn.x, G.kn[1] = kn.y, G.kn[2] = kn.z;
        const double spacing = 2 * PI / std::sqrt(norm2(k));
        reach = std::sqrt(d.max_r * d.max_r + spacing * spacing);
    } else if (d.enumerator == RP_PAIRS_LINEAR) {
        // LinearEnumerator.cpp:45-56: the unit normal of the faces across side `axis`
        const int a = d.linear_axis;
        d3 s[3] = {mv3(v.box, {1, 0, 0}), mv3(v.box, {0, 1, 0}), mv3(v.box, {0, 0, 1})};
        d3 dir = normalized3(cross3(s[(a + 1) % 3], s[(a + 2) % 3]));
        G.dir[0] = dir.x, G.dir[1] = dir.y, G.dir[2] = dir.z;
    }
    // FP32 error bound.  A focal point's relative coordinates lie within R of the box
    // ([0, 1) plus the focal offset's reach); rounding them to FP32 moves a separation by at
    // most 2^-24 (2R + 1/2) per coordinate, and the FP32 product with the box and the norm
    // add at most a few 2^-24 of sum |B_ik| and of the distance: in all at most
    // 6e-8 (2R + 2.5) sum |B_ik| + 2e-7 d.  m_abs and m_rel take 2.5 and 5 times that, so an
    // FP32 distance d32 brackets the FP64 one in d32 -+ m with room for the FP64 rounding of
    // the bracket itself.
    double inv_row = 0, babs = 0;
    for (int i = 0; i < 3; i++) {
        inv_row = std::max(inv_row, std::sqrt(norm2(d3{v.inv[3 * i], v.inv[3 * i + 1], v.inv[3 * i + 2]})));
        for (int k = 0; k < 3; k++) babs += std::abs(v.box[3 * i + k]);
    }
    const double R = 1.0 + std::sqrt(norm2(d3{d.focal[0], d.focal[1], d.focal[2]})) * inv_row;
    const double m_abs = 1.5e-7 * (2 * R + 3) * babs, m_rel = 1e-6;
    // in bin units, with the FP32 roundings of t (1 / step and the product) and of t -+ m
    // (at most 2.4e-7 t in all) added to the relative part
    G.inv_step32 = static_cast<float>(1.0 / G.step);
    G.bin_abs = static_cast<float>(m_abs / G.step * (1 + 1e-6) + 2.5e-7);
    G.bin_rel = static_cast<float>(m_rel + 2.5e-6);   // also the rsqrt-based FP32 square root
    G.in_lo = static_cast<float>(d.num_bins * (1 - 1e-6));
    G.in_hi = static_cast<float>(d.num_bins * (1 + 1e-6));
    // layerwise: the in-layer distance is the separation minus its normal part, whose FP32
    // error adds a few 2^-24 of the whole separation (at most the reach): 2e-6 reach, with room
    G.bin_abs_lw = static_cast<float>((m_abs + 2e-6 * reach) / G.step * (1 + 1e-6) + 2.5e-7);
    for (int i = 0; i < 3; i++) {
        G.hm32[i] = static_cast<float>(d.miller[i]);
        G.kn32[i] = static_cast<float>(G.kn[i]);
    }
    const double thr = reach * (1 + m_rel) + m_abs;
    G.thr2_32 = static_cast<float>(thr * thr);
    G.lin_thr32 = static_cast<float>(thr / h[std::min(std::max(d.linear_axis, 0), 2)]);
    G.h32 = static_cast<float>(h[std::min(std::max(d.linear_axis, 0), 2)]);
    G.edge32 = 1e-4f;
    G.fp64_only = (d.flags & RP_CORR_FP64_ONLY) ? 1 : 0;

    // cells: in a dimension with room for five or more, half the reach across (searched two
    // cells each way: the 5x5x5 block holds 15.6 reach^3 against 27 for reach-wide cells),
    // else the reach across with three or more (one cell each way), else one cell.  A pair
    // within reach is then at most `span` cells apart in every dimension, and the offsets
    // -span..span name distinct cells.  Half-reach cells are used while they hold a few
    // points each on average.
    int64_t ncell = 1;
    const bool all_pairs = d.flags & RP_CORR_ALL_PAIRS;
    double half_cells = 1;
    for (int k = 0; k < 3; k++) {
        const bool restricted = d.enumerator != RP_PAIRS_LINEAR || k == d.linear_axis;
        half_cells *= restricted ? std::max(1.0, std::floor(2 * h[k] / (reach * (1 + 1e-5)))) : 1.0;
    }
    const bool halves = static_cast<double>(v.n) >= 4 * half_cells;
    for (int k = 0; k < 3; k++) {
        int m = 1, sp = 0;
        const bool restricted = d.enumerator != RP_PAIRS_LINEAR || k == d.linear_axis;
        if (restricted && !all_pairs) {
            const double q2 = std::floor(2 * h[k] / (reach * (1 + 1e-5)));
            const double q1 = std::floor(h[k] / (reach * (1 + 1e-5)));
            if (halves && q2 >= 5) {
                m = static_cast<int>(std::min(q2, 2048.0));
                sp = 2;
            } else if (q1 >= 3) {
                m = static_cast<int>(std::min(q1, 1024.0));
                sp = 1;
            }
        }
        G.nc[k] = m;
        G.span[k] = sp;
    }
    const int64_t max_cells = std::max<int64_t>(125, 2 * v.n);
    for (;;) {
        ncell = int64_t(G.nc[0]) * G.nc[1] * G.nc[2];
        if (ncell <= max_cells) break;
        // coarser cells keep every pair within reach `span` cells apart; too few of them for
        // distinct offsets: one cell in that dimension
        int k = (G.nc[0] >= G.nc[1] && G.nc[0] >= G.nc[2]) ? 0 : (G.nc[1] >= G.nc[2] ? 1 : 2);
        G.nc[k] = G.nc[k] * 3 / 4;
        if (G.nc[k] < 2 * G.span[k] + 1) {
            G.nc[k] = 1;
            G.span[k] = 0;
        }
    }
    G.ncell = static_cast<int>(ncell);

    rc = ensure_buffers(c, v, ncell, axes);
    if (rc != RP_OK) return rc;
    const int nb = d.num_bins;
    cudaStream_t st = v.stream;
    CORR_CUDA(c, cudaMemsetAsync(c->hist, 0, sizeof(unsigned long long) * nb, st));
    CORR_CUDA(c, cudaMemsetAsync(c->hsum, 0, sizeof(double) * nb, st));
    CORR_CUDA(c, cudaMemsetAsync(c->tested, 0, sizeof(unsigned long long), st));
    CORR_CUDA(c, cudaMemsetAsync(c->count, 0, sizeof(int32_t) * ncell, st));
    CORR_CUDA(c, cudaMemsetAsync(c->fill, 0, sizeof(int32_t) * ncell, st));
    CORR_CUDA(c, cudaMemsetAsync(c->max_occ, 0, sizeof(int32_t), st));
    const unsigned nblk = static_cast<unsigned>((v.n + CORR_THREADS - 1) / CORR_THREADS);
    const bool layers = d.enumerator == RP_PAIRS_LAYERWISE;
    if (v.n > 0) {
        k_corr_cells<<<nblk, CORR_THREADS, 0, st>>>(G, v.pos64, v.rot64, v.n, c->cell_of, c->count,
                                                    layers ? c->focal_out : nullptr);
        CORR_CUDA(c, cudaGetLastError());
    }
    if (layers) {
        // LayerwiseRadialEnumerator::calculateTauAngle (LayerwiseRadialEnumerator.cpp:48-57):
        // arg of the sum of exp(i k.r) over the focal points in index order, on the host
        std::vector<double> f(3 * v.n);
        if (v.n > 0)
            CORR_CUDA(c, cudaMemcpyAsync(f.data(), c->focal_out, sizeof(double) * 3 * v.n, cudaMemcpyDeviceToHost,
                                         st));
        CORR_CUDA(c, cudaStreamSynchronize(st));
        const d3 k{G.k[0], G.k[1], G.k[2]};
        std::complex<double> tau{0};
        const std::complex<double> im{0, 1};
        for (int64_t i = 0; i < v.n; i++) tau = tau + std::exp(im * dot3(k, d3{f[3 * i], f[3 * i + 1], f[3 * i + 2]}));
        G.tau = std::arg(tau);
        G.tau32 = static_cast<float>(G.tau / (2 * PI));
    }
    CORR_CUDA(c, launch_cell_scan(c->count, c->start, c->block_sums, G.ncell, c->max_occ, st));
    if (v.n > 0) {
        k_corr_scatter<<<nblk, CORR_THREADS, 0, st>>>(G, v.pos64, v.rot64, v.n, c->cell_of, c->start, c->fill, c->S,
                                                      axes ? 1 : 0);
        CORR_CUDA(c, cudaGetLastError());
        int dev_sms = 152;
        cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, v.device);
        const int64_t wblk = (v.n + CORR_THREADS / 32 - 1) / (CORR_THREADS / 32);   // one warp per point
        const int grid = static_cast<int>(std::min<int64_t>(wblk, int64_t(dev_sms) * 6));
        const int use_smem = nb <= SMEM_BINS ? 1 : 0;
        const size_t smem = use_smem ? size_t(nb) * (axes ? 16 : 8) : 0;
        cudaError_t le;
        if (d.enumerator == RP_PAIRS_RADIAL)
            le = launch_pairs_e<RP_PAIRS_RADIAL>(d.function, G, c->S, c->start, v.n, grid, use_smem, smem, c->hist,
                                                 c->hsum, c->tested, st);
        else if (d.enumerator == RP_PAIRS_LINEAR)
            le = launch_pairs_e<RP_PAIRS_LINEAR>(d.function, G, c->S, c->start, v.n, grid, use_smem, smem, c->hist,
                                                 c->hsum, c->tested, st);
        else
            le = launch_pairs_e<RP_PAIRS_LAYERWISE>(d.function, G, c->S, c->start, v.n, grid, use_smem, smem,
                                                    c->hist, c->hsum, c->tested, st);
        CORR_CUDA(c, le);
    }
    std::vector<unsigned long long> cnt(nb);
    std::vector<double> sums(nb);
    unsigned long long tested = 0;
    CORR_CUDA(c, cudaMemcpyAsync(cnt.data(), c->hist, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToHost, st));
    CORR_CUDA(c, cudaMemcpyAsync(sums.data(), c->hsum, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
    CORR_CUDA(c, cudaMemcpyAsync(&tested, c->tested, sizeof(tested), cudaMemcpyDeviceToHost, st));
    CORR_CUDA(c, cudaStreamSynchronize(st));

    // HistogramBuilder: add (value += 1 per pair for the density), renormalizeBins,
    // nextSnapshot (HistogramBuilder.tpp:12-28, Histogram.tpp:52-58)
    std::vector<double> snap(nb);
    if (is_density(d)) {
        auto f = density_factors(d, v.box, v.inv, v.n);
        for (int b = 0; b < nb; b++) snap[b] = static_cast<double>(cnt[b]) * f[b];
    } else {
        snap = sums;
    }
    for (int b = 0; b < nb; b++) {
        c->value[b] += snap[b];
        c->total[b] += cnt[b];
    }
    c->snapshots++;
    c->last_count.assign(cnt.begin(), cnt.end());
    c->last_sum = sums;
    c->last_tested = static_cast<int64_t>(tested);
    return RP_OK;
}

}  // namespace
}  // namespace rp

using rp::Corr;

extern "C" {

int rp_correlation_create(const rp_pair_desc *desc, void **corr) {
    if (!desc || !corr) return RP_ERR_ARG;
    *corr = nullptr;
    const rp_pair_desc &d = *desc;
    if (d.enumerator < RP_PAIRS_RADIAL || d.enumerator > RP_PAIRS_LAYERWISE) return RP_ERR_ARG;
    if (d.function < RP_CORR_DENSITY || d.function > RP_CORR_AXES_ANGLE) return RP_ERR_ARG;
    if (d.axis < RP_AXIS_PRIMARY || d.axis > RP_AXIS_AUXILIARY) return RP_ERR_ARG;
    if (d.linear_axis < 0 || d.linear_axis > 2) return RP_ERR_ARG;
    if (d.flags & ~(RP_CORR_ALL_PAIRS | RP_CORR_FP64_ONLY)) return RP_ERR_ARG;
    for (int i = 0; i < 3; i++)
        if (!std::isfinite(d.focal[i]) || !std::isfinite(d.primary[i]) || !std::isfinite(d.secondary[i]))
            return RP_ERR_ARG;
    if (d.num_bins < 1 || d.num_bins > RP_CORR_MAX_BINS || !(d.max_r > 0) || !std::isfinite(d.max_r))
        return RP_ERR_ARG;
    // LayerwiseRadialEnumerator's constructor: some Miller index nonzero
    if (d.enumerator == RP_PAIRS_LAYERWISE && d.miller[0] == 0 && d.miller[1] == 0 && d.miller[2] == 0)
        return RP_ERR_ARG;
    Corr *c = new (std::nothrow) Corr();
    if (!c) return RP_ERR_CAPACITY;
    c->d = d;
    c->value.assign(d.num_bins, 0.0);
    c->total.assign(d.num_bins, 0);
    *corr = c;
    return RP_OK;
}

int rp_correlation_add_snapshot(void *corr, void *handle) {
    Corr *c = static_cast<Corr *>(corr);
    if (!c) return RP_ERR_ARG;
    if (!handle) return c->fail(RP_ERR_ARG, "null handle");
    return rp::add_snapshot(c, handle);
}

int rp_correlation_values(void *corr, double *x, double *y, uint64_t *count) {
    Corr *c = static_cast<Corr *>(corr);
    if (!c || !x || !y || !count) return RP_ERR_ARG;
    const int nb = c->d.num_bins;
    const double step = (c->d.max_r - 0.0) / static_cast<double>(nb);
    for (int b = 0; b < nb; b++) {
        x[b] = 0.0 + (static_cast<double>(b) + 0.5) * step;   // Histogram.tpp:108-116
        if (c->snapshots == 0) {
            y[b] = 0.0;
            count[b] = 0;
            continue;
        }
        // HistogramBuilder.tpp:44-71: SUM (density) or AVERAGE (averaged correlations)
        y[b] = rp::is_density(c->d) ? c->value[b] / static_cast<double>(c->snapshots)
                                    : c->value[b] / static_cast<double>(c->total[b]);
        count[b] = c->total[b];
    }
    return RP_OK;
}

int rp_correlation_last_snapshot(void *corr, uint64_t *count, double *sums) {
    Corr *c = static_cast<Corr *>(corr);
    if (!c || !count || !sums) return RP_ERR_ARG;
    if (c->last_count.empty()) return c->fail(RP_ERR_STATE, "no snapshot taken");
    for (int b = 0; b < c->d.num_bins; b++) {
        count[b] = c->last_count[b];
        sums[b] = c->last_sum[b];
    }
    return RP_OK;
}

int rp_correlation_info(void *corr, int64_t *snapshots, int64_t *pairs_tested) {
    Corr *c = static_cast<Corr *>(corr);
    if (!c) return RP_ERR_ARG;
    if (snapshots) *snapshots = c->snapshots;
    if (pairs_tested) *pairs_tested = c->last_tested;
    return RP_OK;
}

int rp_correlation_clear(void *corr) {
    Corr *c = static_cast<Corr *>(corr);
    if (!c) return RP_ERR_ARG;
    std::fill(c->value.begin(), c->value.end(), 0.0);
    std::fill(c->total.begin(), c->total.end(), 0);
    c->snapshots = 0;
    return RP_OK;
}

const char *rp_correlation_last_error(void *corr) {
    Corr *c = static_cast<Corr *>(corr);
    return c ? c->err.c_str() : "null correlation";
}

int rp_correlation_destroy(void *corr) {
    Corr *c = static_cast<Corr *>(corr);
    if (!c) return RP_ERR_ARG;
    if (c->device >= 0) {
        cudaSetDevice(c->device);
        c->free_all();
    }
    delete c;
    return RP_OK;
}

}  // extern "C"
