// Allocation-free overlap count (rp_count_overlaps_static, include/rampack_gb300.h).
//
// Who needs it: callers that hold a packing in their own device memory and may not
// allocate more — a host framework that budgets or pools all device memory itself, or
// a stream-ordered pipeline in which a cudaMalloc/cudaFree would implicitly synchronise
// the device and stall the caller's other streams.  rp_create reserves per-handle
// buffers with cudaMalloc; this entry point instead works out of one fixed scratch
// array compiled into the library, and calls no allocating routine at all.
//
// The scratch is a file-scope __device__ array of RP_STATIC_SCRATCH_BYTES.  Every GPU
// that loads the library holds it until the process exits.  All calls share it and it
// keeps the previous call's contents, so the call clears what must start at zero
// (cell counts, occupancy maximum, result counter, early-exit flag, status word), and
// calls whose work overlaps on the GPU (other host threads, or several streams) race on
// it: callers must serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "rp_internal.cuh"
#include "rp_margins.cuh"

namespace rp {

cudaError_t launch_rebuild(const DevState &s, const GridDev &g, int32_t *block_sums, cudaStream_t st);
cudaError_t launch_count(const DevState &s, const GridDev &g, int early, unsigned long long *out, int *flag,
                         cudaStream_t st);

namespace {

constexpr int64_t SMAX_N = RP_STATIC_MAX_PARTICLES;
constexpr int64_t SMAX_CELLS = RP_STATIC_MAX_CELLS;

// Byte layout of the scratch array (every block 256-byte aligned).
constexpr size_t al(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t OFF_COUNT = 0;
constexpr size_t OFF_START = OFF_COUNT + al(sizeof(int32_t) * SMAX_CELLS);
constexpr size_t OFF_BSUMS = OFF_START + al(sizeof(int32_t) * (SMAX_CELLS + 1));
constexpr size_t OFF_MISC = OFF_BSUMS + al(sizeof(int32_t) * (SMAX_CELLS / 4096 + 1));
constexpr size_t OFF_TRANS = OFF_MISC + 256;  // max_occ, status, flag, result, counters
constexpr size_t OFF_SLOT = OFF_TRANS + al(sizeof(double) * 375);
constexpr size_t OFF_PSLOT = OFF_SLOT + al(sizeof(int32_t) * SMAX_N);
constexpr size_t OFF_PCELL = OFF_PSLOT + al(sizeof(int32_t) * SMAX_N);
constexpr size_t OFF_RANK = OFF_PCELL + al(sizeof(int32_t) * SMAX_N);
constexpr size_t OFF_MPOS = OFF_RANK + al(sizeof(int32_t) * SMAX_N);
constexpr size_t OFF_MAXIS = OFF_MPOS + al(sizeof(float4) * SMAX_N);
constexpr size_t OFF_PLOCAL = OFF_MAXIS + al(sizeof(float4) * SMAX_N);
constexpr size_t SCRATCH_END = OFF_PLOCAL + al(sizeof(float4) * SMAX_N);
static_assert(SCRATCH_END <= RP_STATIC_SCRATCH_BYTES, "scratch layout exceeds the declared size");

}  // namespace

static __device__ __align__(256) unsigned char g_static_scratch[RP_STATIC_SCRATCH_BYTES];

namespace {

// Device address of the scratch array, looked up once per device with that device current
// (in host code the array's name is only a host-side stand-in, not a device address).  The
// address belongs to the device's primary context: cudaDeviceReset destroys that context,
// and this entry point must not be called on that device after a reset.
std::mutex g_addr_mutex;
void *g_addr[64] = {};

int scratch_address(int device, void **out) {
    if (device < 0 || device >= 64) return RP_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[device]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return RP_ERR_CUDA;
        g_addr[device] = p;
    }
    *out = g_addr[device];
    return RP_OK;
}

}  // namespace
}  // namespace rp

using namespace rp;

extern "C" int rp_count_overlaps_static(const rp_shape_desc *shape, int64_t n, const double *d_pos,
                                        const double *d_rot, const double *box9, int early_exit, void *stream,
                                        int64_t *out_count) {
    if (!shape || !d_pos || !d_rot || !box9 || !out_count) return RP_ERR_ARG;
    if (n <= 0 || n > SMAX_N) return RP_ERR_CAPACITY;
    if (shape->kind != RP_SHAPE_SPHERE && shape->kind != RP_SHAPE_SPHEROCYLINDER) return RP_ERR_UNSUPPORTED;
    if (!(shape->radius > 0) || (shape->kind == RP_SHAPE_SPHEROCYLINDER && !(shape->length >= 0))) return RP_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return RP_ERR_CUDA;
    // The kernels read d_pos and d_rot directly: refuse, before any launch, pointers that
    // are not device (or managed) memory of the current device, e.g. a host array.
    for (const void *p : {static_cast<const void *>(d_pos), static_cast<const void *>(d_rot)}) {
        cudaPointerAttributes attr{};
        if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
            cudaGetLastError();  // clear the (non-sticky) error an unknown pointer leaves
            return RP_ERR_ARG;
        }
        if ((attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) || attr.device != device)
            return RP_ERR_ARG;
    }
    void *base_v = nullptr;
    int rc = scratch_address(device, &base_v);
    if (rc != RP_OK) return rc;
    unsigned char *base = static_cast<unsigned char *>(base_v);

    // ---- host set-up: box inverse, interaction range, grid, thresholds ----
    double inv[9];
    if (det3(box9) == 0) return RP_ERR_ARG;
    inverse3(box9, inv);
    const double r = shape->radius, l = shape->length;
    const double range = shape->kind == RP_SHAPE_SPHERE ? 2 * r : 2 * r + l;
    d3 s0{box9[0], box9[3], box9[6]}, s1{box9[1], box9[4], box9[7]}, s2{box9[2], box9[5], box9[8]};
    double vol = std::fabs(dot3(cross3(s0, s1), s2));
    double hgt[3] = {vol / std::sqrt(norm2(cross3(s1, s2))), vol / std::sqrt(norm2(cross3(s2, s0))),
                     vol / std::sqrt(norm2(cross3(s0, s1)))};
    {
        // the reference keeps no neighbour grid for small boxes (core/Packing.cpp:862-881)
        double ref_cell = std::max(range, std::cbrt(vol / static_cast<double>(n)) / 5);
        if (ref_cell * 4 > std::max({hgt[0], hgt[1], hgt[2]}) || ref_cell * (1 + 1e-12) > std::min({hgt[0], hgt[1], hgt[2]}))
            return RP_ERR_UNSUPPORTED;
    }
    GridDev g{};
    // Cells at least one interaction range high; a dilute packing whose range-sized cells
    // would exceed the scratch's cell table gets larger cells (still correct: every pair
    // within range lies in neighbouring cells), so only n itself is ever too large.
    double cell_min = range * (1.0 + 1e-9);
    for (int d = 0; d < 3; d++)
        if (!(hgt[d] >= cell_min)) return RP_ERR_UNSUPPORTED;
    for (;;) {
        int64_t ncell = 1;
        for (int d = 0; d < 3; d++) {
            double nd = std::floor(hgt[d] / cell_min);
            int nn = nd > SMAX_CELLS ? static_cast<int>(SMAX_CELLS) : static_cast<int>(nd);
            nn = nn >= 2 ? (nn & ~1) : 1;
            g.dims[d] = nn;
            g.shift[d] = 0.0;
            ncell *= nn;
        }
        if (ncell <= SMAX_CELLS) {
            g.ncell = static_cast<int>(ncell);
            break;
        }
        cell_min *= 1.125;
    }
    double cm[9], cminv[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) cm[3 * i + j] = box9[3 * i + j] / g.dims[j];
    inverse3(cm, cminv);
    double lrow = 0;
    for (int i = 0; i < 9; i++) {
        g.cellmat[i] = static_cast<float>(cm[i]);
        g.cellinv[i] = static_cast<float>(cminv[i]);
    }
    for (int i = 0; i < 3; i++)
        lrow = std::max(lrow, std::fabs(cm[3 * i]) + std::fabs(cm[3 * i + 1]) + std::fabs(cm[3 * i + 2]));
    g.count = reinterpret_cast<int32_t *>(base + OFF_COUNT);
    g.start = reinterpret_cast<int32_t *>(base + OFF_START);
    g.slot_pid = reinterpret_cast<int32_t *>(base + OFF_SLOT);
    g.pid_slot = reinterpret_cast<int32_t *>(base + OFF_PSLOT);
    g.pid_cell = reinterpret_cast<int32_t *>(base + OFF_PCELL);
    g.rank = reinterpret_cast<int32_t *>(base + OFF_RANK);
    g.mpos = reinterpret_cast<float4 *>(base + OFF_MPOS);
    g.maxis = reinterpret_cast<float4 *>(base + OFF_MAXIS);
    g.plocal = reinterpret_cast<float4 *>(base + OFF_PLOCAL);
    g.bounds = nullptr;
    int32_t *misc = reinterpret_cast<int32_t *>(base + OFF_MISC);
    g.max_occ = misc;
    uint32_t *status = reinterpret_cast<uint32_t *>(misc + 1);
    int *flag = misc + 2;
    unsigned long long *result = reinterpret_cast<unsigned long long *>(base + OFF_MISC + 16);
    unsigned long long *counters = reinterpret_cast<unsigned long long *>(base + OFF_MISC + 32);
    double *trans = reinterpret_cast<double *>(base + OFF_TRANS);

    DevState s{};
    s.n = n;
    s.kind = shape->kind;
    std::memcpy(s.box, box9, sizeof(s.box));
    std::memcpy(s.inv, inv, sizeof(s.inv));
    for (int i = 0; i < 9; i++) s.inv32[i] = static_cast<float>(inv[i]);
    s.pos64 = const_cast<double *>(d_pos);  // read only: rebuild and count never write positions
    s.rot64 = const_cast<double *>(d_rot);
    s.trans = trans;
    s.status = status;
    s.counters = counters;
    s.strict_box = 1;
    ExactShape ex{};
    ex.kind = shape->kind;
    if (shape->kind == RP_SHAPE_SPHERE) {
        ex.sphere_thr = std::pow(2 * r, 2);  // SphereTraits.cpp:64
    } else {
        ex.core_thr = 4 * r * r;                // SpherocylinderTraits.cpp:35
        ex.far_thr = std::pow(2 * r + l, 2);    // SpherocylinderTraits.cpp:37
        short beg = -1, end = 1;
        ex.neg_cap_half = 0.5 * beg * l;
        ex.cap_half = 0.5 * end * l;
    }
    s.ex = ex;
    // the same FP32 margins as the handle's recount (a fresh grid, no mirror updates)
    s.fc = hard_filter_consts(shape->kind, r, l, lrow, box9);
    double tt[375];
    for (int a = 0; a < 5; a++)
        for (int b = 0; b < 5; b++)
            for (int c = 0; c < 5; c++) {
                d3 t = mv3(box9, d3{static_cast<double>(a) - 2, static_cast<double>(b) - 2., static_cast<double>(c) - 2.});
                int idx = (a * 5 + b) * 5 + c;
                tt[3 * idx] = t.x;
                tt[3 * idx + 1] = t.y;
                tt[3 * idx + 2] = t.z;
            }

    // ---- device work: zero what must start at zero, rebuild the grid, count ----
    if (cudaMemcpyAsync(trans, tt, sizeof(tt), cudaMemcpyHostToDevice, st) != cudaSuccess) return RP_ERR_CUDA;
    if (cudaMemsetAsync(base + OFF_MISC, 0, 256, st) != cudaSuccess) return RP_ERR_CUDA;
    if (launch_rebuild(s, g, reinterpret_cast<int32_t *>(base + OFF_BSUMS), st) != cudaSuccess) return RP_ERR_CUDA;
    if (launch_count(s, g, early_exit ? 1 : 0, result, flag, st) != cudaSuccess) return RP_ERR_CUDA;
    unsigned long long cnt = 0;
    uint32_t stat = 0;
    if (cudaMemcpyAsync(&cnt, result, sizeof(cnt), cudaMemcpyDeviceToHost, st) != cudaSuccess) return RP_ERR_CUDA;
    if (cudaMemcpyAsync(&stat, status, sizeof(stat), cudaMemcpyDeviceToHost, st) != cudaSuccess) return RP_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return RP_ERR_CUDA;
    if (stat & ST_OUTSIDE) return RP_ERR_ARG;
    if (stat) return RP_ERR_DEVICE;
    *out_count = early_exit ? (cnt > 0 ? 1 : 0) : static_cast<int64_t>(cnt);
    return RP_OK;
}
