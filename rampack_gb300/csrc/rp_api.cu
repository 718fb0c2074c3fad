// C-ABI of the engine (include/rampack_gb300.h): handle lifetime, state transfer,
// cell-grid set-up, move lists, device-driven sweeps and box moves.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include "rp_internal.cuh"
#include "rp_margins.cuh"

namespace rp {

cudaError_t launch_rebuild(const DevState &s, const GridDev &g, int32_t *block_sums, cudaStream_t st);
cudaError_t launch_remap(const DevState &s, const GridDev &g, const GridDev &old, int *moved, cudaStream_t st);
cudaError_t launch_validate(const DevState &s, cudaStream_t st);
cudaError_t launch_rescale(const double *src, double *dst, int64_t n, const double *old_inv, const double *new_box,
                           cudaStream_t st);
cudaError_t launch_count(const DevState &s, const GridDev &g, int early, unsigned long long *out, int *flag,
                         cudaStream_t st);
cudaError_t launch_sweep(const SweepArgs &a, bool list, int nwarps, cudaStream_t st);
size_t sweep_smem_per_warp(int kind, int cap, bool learn = false, int ncen = 0);
cudaError_t launch_abs_centres(const DevState &s, cudaStream_t st);
cudaError_t launch_fix_prepare(const DevState &s, const double *cbody, double *rotfix, double *cenfix, double *absfix,
                               cudaStream_t st);
cudaError_t launch_fresh_centres(const DevState &s, const double *cbody, cudaStream_t st);
int axis_moment_blocks(int64_t n);
cudaError_t launch_b_rebuild(const BatchRep *T, const int *pbase, const int *cbase, int R, int total_particles,
                             int total_cells, cudaStream_t st);
cudaError_t launch_b_rescale(const BatchRep *T, const int *pbase, int R, int total_particles, cudaStream_t st);
cudaError_t launch_b_count(const BatchRep *T, const int *pbase, int R, int total_particles, int kind, int early,
                           unsigned long long *out, int *flags, cudaStream_t st);
size_t batch_smem_per_warp(int kind, int cap);
cudaError_t launch_b_sweep(const BatchRep *T, const int *item_base, int R, int kind, int k, int *next_item, int cap,
                           int wpb, int blocks, bool rototranslation, cudaStream_t st);
cudaError_t launch_b_overflow(const BatchRep *T, int R, int kind, int k, int cap, bool rototranslation,
                              cudaStream_t st);
cudaError_t launch_axis_moments(const double *rot64, int64_t n, double *partial, cudaStream_t st);
cudaError_t launch_fix_check(const DevState &s, const GridDev &g, const double *rotfix, const double *cenfix, const double *absfix,
                             uint8_t *rejected, unsigned long long *first, cudaStream_t st);
cudaError_t launch_fix_commit(const DevState &s, const double *rotfix, const double *cenfix, const double *absfix,
                              int64_t from, int64_t to, cudaStream_t st);
cudaError_t launch_fix_serial(const DevState &s, const GridDev &g, const double *rotfix, const double *cenfix,
                              const double *absfix, int64_t from, unsigned long long *nrej, cudaStream_t st);
cudaError_t launch_mlp_grad(const float *feats, const uint8_t *labels, int64_t total, int64_t i0, int n,
                            int64_t mul, int64_t off, const float *w32, float *grad, float *loss, int num_sms,
                            cudaStream_t st);
cudaError_t launch_mlp_adam(float *w32, __nv_bfloat16 *w16, const float *grad, float *m, float *v, float lr,
                            int step, cudaStream_t st);
cudaError_t launch_mlp_sync16(const float *w32, __nv_bfloat16 *w16, cudaStream_t st);
cudaError_t launch_mlp_predict(const float *feats, int n, const float *w32, const __nv_bfloat16 *w16, float *out,
                               cudaStream_t st);
cudaError_t launch_score_partners(const DevState &s, const GridDev &g, const float *w32, const __nv_bfloat16 *w16,
                                  int mode, float inv_range, int32_t *partners, cudaStream_t st);
cudaError_t launch_rot_table(double *out64, float *out32, uint32_t count, uint64_t seed, uint64_t counter, float step,
                             cudaStream_t st);
cudaError_t launch_sweep_half(const SweepArgs &a, int ncells, cudaStream_t st);
size_t sweep_smem_per_half(int kind, int cap);
int sweep_half_blocks_per_sm(int kind, int cap);
cudaError_t launch_try_single(const SingleArgs &a, cudaStream_t st);
cudaError_t launch_soft_sweep(const SoftSweepArgs &a, int nwarps, cudaStream_t st);
cudaError_t launch_count_fp64(const SingleArgs &a, int early, unsigned long long *out, int *flag, cudaStream_t st);
cudaError_t launch_convex_pairs(const XcShape *xc, int64_t n, const double *p1, const double *r1, const double *p2,
                                const double *r2, uint8_t *out, uint32_t *status, cudaStream_t st);
cudaError_t launch_total_energy(const SingleArgs &a, double *scratch, double *out, cudaStream_t st);
cudaError_t launch_commit_single(const DevState &s, SingleTry *t, uint8_t *disp_flag, int32_t *disp_list, int slot,
                                 cudaStream_t st);

namespace {

constexpr int OVF_WARPS = 152;          // overflow rerun: one warp per block, grid-stride over cells
constexpr size_t OVF_SMEM = 200 * 1024; // shared memory of one overflow warp

struct GridHost {
    GridDev d{};
    int64_t cells_alloc = 0;
    int64_t bounds_alloc = 0;
    int cap = 0;
    int cap_half = 0;         // staging capacity of a cell with two cells per warp (0: not offered)
    double cellmat64[9]{};
    std::vector<float> cthr;  // host copy of the FP32 centre-pair thresholds (polyspheres)
    std::vector<double> bounds_host;  // batch members: this grid's bounds, packed by the batch
    bool no_ng = false;       // the reference keeps no neighbour grid for this grid's box
};

// Per-group device timing: CUDA events around groups of launches, summed per group kind.
struct Timing {
    struct Mark {
        int kid;
        cudaEvent_t a, b;
    };
    bool on = false;
    std::vector<Mark> marks;
    std::vector<cudaEvent_t> pool;
    double ms[RP_NUM_KERNELS]{};
    uint64_t groups[RP_NUM_KERNELS]{};

    cudaEvent_t event() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    // the owner's stream has been synchronized
    void reset(bool enable) {
        for (auto &m : marks) {
            pool.push_back(m.a);
            pool.push_back(m.b);
        }
        marks.clear();
        for (int k = 0; k < RP_NUM_KERNELS; k++) {
            ms[k] = 0;
            groups[k] = 0;
        }
        on = enable;
    }
    // the owner's stream has been synchronized
    cudaError_t collect(double *out_ms, uint64_t *out_groups) {
        for (auto &m : marks) {
            float t = 0;
            cudaError_t e = cudaEventElapsedTime(&t, m.a, m.b);
            if (e != cudaSuccess) return e;
            ms[m.kid] += t;
            groups[m.kid] += 1;
            pool.push_back(m.a);
            pool.push_back(m.b);
        }
        marks.clear();
        for (int k = 0; k < RP_NUM_KERNELS; k++) {
            if (out_ms) out_ms[k] = ms[k];
            if (out_groups) out_groups[k] = groups[k];
        }
        return cudaSuccess;
    }
    void release() {
        for (auto &m : marks) {
            cudaEventDestroy(m.a);
            cudaEventDestroy(m.b);
        }
        marks.clear();
        for (auto e : pool) cudaEventDestroy(e);
        pool.clear();
    }
};

struct Handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    rp_shape_desc shape{};
    int64_t n = 0;
    double range = 0;
    bool has_state = false;
    double box[9]{}, inv[9]{};
    double saved_box[9]{}, saved_inv[9]{};
    bool can_revert = false;
    double *pos64[2] = {nullptr, nullptr};
    int pcur = 0;
    double *rot64 = nullptr;
    double *trans[2] = {nullptr, nullptr};
    GridHost grid[2];
    int gcur = 0;
    int32_t *block_sums = nullptr;
    int64_t block_sums_alloc = 0;
    uint32_t *status = nullptr;
    unsigned long long *counters = nullptr;
    double *rtab64 = nullptr;   // per-sweep rotation table
    float *rtab32 = nullptr;
    int32_t *item_counters = nullptr;  // work counters of persistent sweep launches
    int num_sms = 0;
    unsigned long long *count_out = nullptr;
    int *flag = nullptr;
    DeferredPair *cq_buf = nullptr;   // multi-centre recounts: deferred FP64 centre pairs
    int *cq_count = nullptr;
    static constexpr int CQ_CAP = 1 << 20;
    int32_t *overflow = nullptr;
    int32_t *overflow_count = nullptr;
    int64_t overflow_alloc = 0;
    ExactShape ex{};
    std::string err;
    // move lists
    rp_move *d_moves = nullptr;
    int64_t moves_alloc = 0;
    int32_t *d_list = nullptr;  // cells, begins, move_out packed
    int64_t list_alloc = 0;
    uint8_t *d_codes = nullptr;
    int64_t codes_alloc = 0;
    // sweep log
    rp_move *d_log = nullptr;
    uint8_t *d_log_codes = nullptr;
    int64_t log_alloc = 0;
    bool log_valid = false;
    int log_types = 0;
    std::vector<int32_t> log_start;
    int log_dims[3]{};
    std::vector<int> log_phases;
    // launch accounting and optional per-group device timing
    uint64_t launches = 0;
    Timing tm;
    bool strict_box = false;
    // polyspheres: body-frame centres and radii, the reference's centre range (its
    // neighbour-grid cell), rotated and absolute centres, exact pair thresholds
    int ncen = 0;
    double cbody[3 * MAX_CEN]{}, crad[MAX_CEN]{};
    int walls = 0;            // Packing::toggleWalls mask (bit i: walls across box side i)
    double total_range = 0;   // Interaction::getTotalRangeRadius (core/Interaction.cpp:55-70)
    double cthr_host[MAX_CEN * MAX_CEN]{};
    // polyspherocylinders: body-frame half axes and (c_a + c_b)^2 of the circumsphere radii
    int segs = 0;
    double chax[3 * MAX_CEN]{};
    double circ_host[MAX_CEN * MAX_CEN]{};
    double *circ64 = nullptr;
    double ref_range = 0;
    double *cen64 = nullptr;
    int stage_mode = 1;  // staging filter: 0 off, 1 where it pays (cells well above the range), 2 wherever valid
    int bulk_stage = 0;  // stage neighbourhoods with bulk asynchronous copies
    int cell_order = 1;  // plain sweeps take each phase's cells by occupancy, largest first
    bool grid_stale = false;  // an upload validated the state; the cell grid is built when first needed
    bool stale_unshifted = false;  // ... and it is built unshifted (not with the last grid's origin)
    uint64_t grid_rebuilds = 0;    // full cell-grid rebuilds (Packing::getNeighbourGridRebuilds)
    uint64_t grid_remaps = 0;      // box moves whose grid kept the old cells (k_remap)
    // consistent copy of the FP64 state for asynchronous snapshot downloads
    double *snap64 = nullptr;          // [n][3] positions then [n][9] orientations
    cudaEvent_t snap_free = nullptr;   // recorded when the last download out of snap64 ended
    double *abs64[2] = {nullptr, nullptr};
    double *cthr64 = nullptr;
    double *cbody_dev = nullptr;    // body-frame centres on the device
    XcShape *d_xc = nullptr;        // generic convex bodies: the geometry on the device
    // batched replicas: the batch owns the rotation table, counters, status word and the
    // device copy of the ActiveDomain bounds (setup_grid leaves the bounds in bounds_host)
    bool batch_member = false;
    // overlap counting (Packing::toggleOverlapCounting): the cached count lives on the device
    bool counting = false;
    unsigned long long *d_overlaps = nullptr;
    unsigned long long saved_overlaps = 0;  // count before the last box move (revertScaling)
    double cell_factor = 1.0;       // checkerboard cells at least cell_factor x the range
    // learned ordering: network parameters (FP32 master + BF16 copy), Adam moments, scratch
    float *mlp_w32 = nullptr, *mlp_grad = nullptr, *mlp_m = nullptr, *mlp_v = nullptr, *mlp_loss = nullptr;
    __nv_bfloat16 *mlp_w16 = nullptr;
    int mlp_step = 0;
    float *mlp_feats = nullptr;     // host-supplied pairs (predict / gradient)
    int64_t mlp_feats_alloc = 0;
    uint8_t *mlp_labels = nullptr;
    int64_t mlp_labels_alloc = 0;
    float *mlp_out = nullptr;
    int64_t mlp_out_alloc = 0;
    int32_t *partners = nullptr;    // [n][MLP_PARTNERS]
    bool partners_valid = false;
    int order_mode = RP_ORDER_OFF, order_every = 1, since_rank = 0;
    // pair-outcome log
    float *pair_feats = nullptr;
    uint8_t *pair_labels = nullptr;
    unsigned long long *pair_count = nullptr;
    int64_t pair_cap = 0;
    int pair_every = 0;
    // unrestricted single moves (rp_try_move / rp_accept_move): the tried state on the
    // device, and the particles moved by single moves since the cell grid was built (the
    // grid is then current for every other particle: grid_patched)
    SingleTry *d_try = nullptr;
    bool try_valid = false;
    int32_t try_particle = -1;
    int32_t *d_disp_list = nullptr;
    uint8_t *d_disp_flag = nullptr;
    std::vector<int32_t> disp_host;
    std::vector<uint8_t> disp_flag_host;
    bool grid_patched = false;
    static constexpr int DISP_CAP = 4096;  // moved particles before the grid is rebuilt
    // plain sweeps of spheres and spherocylinders: cells per warp (1, or 2: two lane groups
    // of 16 with the axes read from the mirror, twice the cells in flight per SM)
    int cells_per_warp = 1;
    int half_cap_cached = -1, half_blocks = 0;  // resident blocks per SM at that capacity
    int last_cells_per_warp = 0;                // what the last sweep's phases used
    // soft part (rp_set_soft): a central potential on the interaction centres joined to the
    // hard shape (CompoundInteraction), or alone; the shape's own ranges are kept to undo it
    int soft = 0;
    bool soft_only = false;
    double soft_eps = 0, soft_sigma = 0, soft_cut = 0;
    bool hard_ranges_saved = false;
    double hard_range = 0, hard_ref_range = 0, hard_total_range = 0;
    double temperature = 1.0;       // the Metropolis temperature of soft sweeps
    double *d_energy = nullptr;     // [n] per-particle pair energies, then their sum at [n]
};

// One group of kernel launches of a handle or a batch: counted, and bracketed by CUDA events
// on the owner's stream when its timing is on.
template <class Owner>
struct GroupOf {
    Owner *h;
    int kid;
    cudaEvent_t a = nullptr;
    GroupOf(Owner *h_, int kid_, int nkernels) : h{h_}, kid{kid_} {
        h->launches += static_cast<uint64_t>(nkernels);
        if (h->tm.on) {
            a = h->tm.event();
            cudaEventRecord(a, h->stream);
        }
    }
    ~GroupOf() {
        if (a) {
            cudaEvent_t b = h->tm.event();
            cudaEventRecord(b, h->stream);
            h->tm.marks.push_back({kid, a, b});
        }
    }
};
using Group = GroupOf<Handle>;

int fail(Handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    return code;
}

#define RP_CUDA(h, call)                                                                                  \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return fail((h), RP_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
cudaError_t ensure(T *&ptr, int64_t &alloc, int64_t need) {
    if (need <= alloc && ptr) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    alloc = 0;
    int64_t want = std::max<int64_t>(need, 1);
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&ptr), sizeof(T) * want);
    if (e == cudaSuccess) alloc = want;
    return e;
}

void heights_of(const double *box, double h[3]) {
    d3 s0{box[0], box[3], box[6]}, s1{box[1], box[4], box[7]}, s2{box[2], box[5], box[8]};
    // core/TriclinicBox.cpp:33-51 (volume = |(s0 x s1) . s2|, h_i = V / |s_j x s_k|)
    double vol = std::fabs(dot3(cross3(s0, s1), s2));
    h[0] = vol / std::sqrt(norm2(cross3(s1, s2)));
    h[1] = vol / std::sqrt(norm2(cross3(s2, s0)));
    h[2] = vol / std::sqrt(norm2(cross3(s0, s1)));
}

double volume_of(const double *box) {
    d3 s0{box[0], box[3], box[6]}, s1{box[1], box[4], box[7]}, s2{box[2], box[5], box[8]};
    return std::fabs(dot3(cross3(s0, s1), s2));
}

// core/Packing.cpp:1155-1176
bool box_upscaled(const double *ob, const double *nb) {
    const double EPS = 100 * std::numeric_limits<double>::epsilon();
    for (int i = 0; i < 3; i++) {
        d3 o{ob[i], ob[3 + i], ob[6 + i]}, n{nb[i], nb[3 + i], nb[6 + i]};
        double d = dot3(o, n), n2o = norm2(o), n2n = norm2(n);
        if (std::fabs(d * d / n2o / n2n - 1) > EPS) return false;
        if (d * d / n2o / n2o < 1 + EPS) return false;
    }
    return true;
}

// Box translations box·m, m in {-2..2}^3 (core/NeighbourGrid.cpp:203-217 for |m| <= 1).
void translation_table(const double *box, double *out) {
    for (int a = 0; a < 5; a++)
        for (int b = 0; b < 5; b++)
            for (int c = 0; c < 5; c++) {
                d3 rel{static_cast<double>(a) - 2, static_cast<double>(b) - 2., static_cast<double>(c) - 2.};
                d3 t = mv3(box, rel);
                int idx = (a * 5 + b) * 5 + c;
                out[3 * idx] = t.x;
                out[3 * idx + 1] = t.y;
                out[3 * idx + 2] = t.z;
            }
}

double cell_lrow(const GridHost &g) {
    double lrow = 0;
    for (int i = 0; i < 3; i++) {
        double r = 0;
        for (int j = 0; j < 3; j++) r += std::fabs(g.cellmat64[3 * i + j]);
        lrow = std::max(lrow, r);
    }
    return lrow;
}

// Margin of an FP32 polysphere distance^2 at threshold thr = d^2: the centre separation
// ((q - p) + c_j) - c_a carries the position error of the sphere filter (32 u32 (L + 1)
// per component, L the largest cell-local coordinate) plus the FP32 centres' error (the
// rounding of c, the FP32 rotation of the mover's centres: 8 u32 |c|) and the roundings of
// the two extra sums (2 u32 (2 L + 2 |c|)); 32 u32 (|c|max + L + 1) covers the latter.
double poly_margin(const Handle *h, const GridHost &g, double thr) {
    const double u32 = std::ldexp(1.0, -24);
    double cmax = 0;
    for (int b = 0; b < h->ncen; b++)
        cmax = std::max(cmax, std::sqrt(h->cbody[3 * b] * h->cbody[3 * b] + h->cbody[3 * b + 1] * h->cbody[3 * b + 1] +
                                        h->cbody[3 * b + 2] * h->cbody[3 * b + 2]));
    const double L = cell_lrow(g);
    const double e = 32.0 * u32 * (L + 1.0) + 32.0 * u32 * (cmax + L + 1.0);
    const double d = std::sqrt(thr);
    return 2.0 * (2.0 * d * std::sqrt(3.0) * e + 3.0 * e * e + 4.0 * u32 * thr);
}

DevState dev_state(Handle *h) {
    DevState s{};
    s.n = h->n;
    s.kind = h->shape.kind;
    s.xc = h->d_xc;
    std::memcpy(s.box, h->box, sizeof(s.box));
    std::memcpy(s.inv, h->inv, sizeof(s.inv));
    for (int i = 0; i < 3; i++) {
        double z = 0.0;
        for (int j = 0; j < 3; j++) z = z + h->box[3 * i + j] * 0.0;
        s.box_zero[i] = z;
    }
    for (int i = 0; i < 9; i++) s.inv32[i] = static_cast<float>(h->inv[i]);
    s.pos64 = h->pos64[h->pcur];
    s.rot64 = h->rot64;
    s.trans = h->trans[h->pcur];
    s.ex = h->ex;
    s.status = h->status;
    s.counters = h->counters;
    s.strict_box = h->strict_box ? 1 : 0;
    s.ncen = h->ncen;
    s.cen64 = h->cen64;
    s.abs64 = h->abs64[h->pcur];
    s.cthr64 = h->cthr64;
    s.segs = h->segs;
    for (int k = 0; k < MAX_CEN; k++)
        for (int d = 0; d < 3; d++) s.chax[k][d] = h->chax[3 * k + d];
    s.circ64 = h->circ64;
    if (h->grid[h->gcur].no_ng) {
        const bool sheared = h->box[1] != 0 || h->box[2] != 0 || h->box[3] != 0 || h->box[5] != 0 || h->box[6] != 0 ||
                             h->box[7] != 0;
        s.pbc_fold = sheared ? 2 : 1;
    } else {
        s.pbc_fold = 0;
    }
    s.counting = h->counting ? 1 : 0;
    s.overlaps = h->d_overlaps;
    s.walls = h->soft_only ? 0 : h->walls;   // a soft part alone has no wall part
    s.soft = h->soft;
    s.soft_only = h->soft_only ? 1 : 0;
    s.soft_eps = h->soft_eps;
    s.soft_sigma = h->soft_sigma;
    s.soft_cut = h->soft_cut;
    s.soft_cut2 = h->soft_cut * h->soft_cut;
    s.soft_sigma2 = h->soft_sigma * h->soft_sigma;
    s.soft_4eps = 4.0 * h->soft_eps;
    if (h->walls) {
        // Packing::countParticleWallOverlaps (core/Packing.cpp:1089-1101): the box sides
        // (TriclinicBox::getSides: box · e_i, accumulated from zero), the far corner as their
        // sum from the origin, each wall's unit normal (side i+1 ^ side i+2).normalized()
        d3 sd[3];
        for (int j = 0; j < 3; j++) sd[j] = d3{h->box[j] + 0.0, h->box[3 + j] + 0.0, h->box[6 + j] + 0.0};
        d3 far{0.0, 0.0, 0.0};
        for (int j = 0; j < 3; j++) far = add3(far, sd[j]);
        s.wall_far[0] = far.x;
        s.wall_far[1] = far.y;
        s.wall_far[2] = far.z;
        for (int i = 0; i < 3; i++) {
            const d3 c = cross3(sd[(i + 1) % 3], sd[(i + 2) % 3]);
            const double nrm = std::sqrt(norm2(c));
            s.wall_vec[i][0] = c.x / nrm;
            s.wall_vec[i][1] = c.y / nrm;
            s.wall_vec[i][2] = c.z / nrm;
        }
        s.wall_half = h->total_range / 2;
        s.wall_half_len = h->shape.kind == RP_SHAPE_SPHEROCYLINDER ? h->shape.length / 2 : 0.0;
        for (int k = 0; k < MAX_CEN; k++)
            s.wall_radius[k] = h->ncen > 0 ? h->crad[k] : h->shape.radius;
    }
    // ---- FP32 filter margins for the current grid ----
    const GridHost &g = h->grid[h->gcur];
    FilterConsts fc = hard_filter_consts(h->shape.kind, h->shape.radius, h->shape.length, cell_lrow(g), h->box);
    if (h->shape.kind == RP_SHAPE_POLYSPHERE) {
        // bodies whose centres are farther apart than twice the largest centre reach
        // (|c| + r) cannot touch; the centre-pair thresholds live in the grid (setup_grid)
        double far = h->range * h->range;
        fc.far_lo = static_cast<float>(far - poly_margin(h, g, far));
        fc.far_hi = static_cast<float>(far + poly_margin(h, g, far));
    }
    s.fc = fc;
    return s;
}

// Chooses the checkerboard grid for a box: cells at least one interaction range high
// in every direction, an even count per direction (or a single cell), so that cells of
// one colour never interact.
int setup_grid(Handle *h, GridHost &G, const double *box, const double *shift) {
    double hgt[3];
    heights_of(box, hgt);
    // at least one interaction range (bodies in two cells of one colour never interact),
    // and large enough that the grid has at most max(4096, 8 N) cells (a dilute system
    // would otherwise spread a few particles over millions of empty cells)
    const double max_cells = std::max(4096.0, 8.0 * static_cast<double>(h->n));
    const double cell_min =
        std::max(h->range * h->cell_factor, std::cbrt(volume_of(box) / max_cells)) * (1.0 + 1e-9);
    int dims[3];
    for (int d = 0; d < 3; d++) {
        if (!(hgt[d] >= h->range * (1.0 + 1e-9)))
            return fail(h, RP_ERR_UNSUPPORTED, "box height smaller than the interaction range");
        double nd = std::floor(hgt[d] / cell_min);
        if (nd > 1 << 20) return fail(h, RP_ERR_UNSUPPORTED, "too many cells");
        int n = static_cast<int>(nd);
        // three cells keep their size (three colours along this dimension: two would be half
        // as large again); larger odd counts drop one cell (two colours, cells at most a
        // quarter larger; measured faster than three colours, whose extra phases cost more)
        if (n < 1) n = 1;
        if (n > 3 && (n & 1)) n -= 1;
        dims[d] = n;
    }
    // The reference keeps no neighbour grid for small boxes (core/Packing.cpp:862-881) and
    // then tests every pair at its nearest periodic image, measuring sphere distances with
    // the periodic boundary conditions' formula.  That is the engine's decision too as long
    // as a pair has at most one image within range: every box height at least twice the
    // reference's interaction range.
    {
        double ref_cell = h->ref_range;
        double min_cell = std::cbrt(volume_of(box) / static_cast<double>(h->n)) / 5;
        if (h->ref_range < min_cell) ref_cell = min_cell;
        double mx = std::max({hgt[0], hgt[1], hgt[2]}), mn = std::min({hgt[0], hgt[1], hgt[2]});
        G.no_ng = ref_cell * 4 > mx || ref_cell * (1 + 1e-12) > mn;
        if (G.no_ng && !(mn >= 2 * h->ref_range * (1 + 1e-9)))
            return fail(h, RP_ERR_UNSUPPORTED,
                        "box too small: the reference keeps no neighbour grid and pairs have several images in range");
    }
    int64_t ncell = static_cast<int64_t>(dims[0]) * dims[1] * dims[2];
    if (ncell > (1ll << 30)) return fail(h, RP_ERR_UNSUPPORTED, "too many cells");
    GridDev &g = G.d;
    for (int d = 0; d < 3; d++) {
        g.dims[d] = dims[d];
        g.shift[d] = shift[d];
        g.fshift[d] = static_cast<float>(shift[d]);
        g.finv_dims[d] = 1.0f / static_cast<float>(dims[d]);
    }
    g.ncell = static_cast<int>(ncell);
    double inv_cm[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) G.cellmat64[3 * i + j] = box[3 * i + j] / dims[j];
    inverse3(G.cellmat64, inv_cm);
    for (int i = 0; i < 9; i++) {
        g.cellmat[i] = static_cast<float>(G.cellmat64[i]);
        g.cellinv[i] = static_cast<float>(inv_cm[i]);
    }
    // allocations
    if (ncell > G.cells_alloc) {
        cudaFree(g.count);
        cudaFree(g.start);
        cudaFree(g.order);
        g.count = g.start = g.order = nullptr;
        RP_CUDA(h, cudaMalloc(&g.count, sizeof(int32_t) * ncell));
        RP_CUDA(h, cudaMalloc(&g.start, sizeof(int32_t) * (ncell + 1)));
        RP_CUDA(h, cudaMalloc(&g.order, sizeof(int32_t) * ncell));
        G.cells_alloc = ncell;
    }
    if (!g.order_cnt) {
        RP_CUDA(h, cudaMalloc(&g.order_cnt, sizeof(int32_t) * 27 * ORDER_BINS));
        RP_CUDA(h, cudaMalloc(&g.order_off, sizeof(int32_t) * 27 * ORDER_BINS));
        RP_CUDA(h, cudaMemsetAsync(g.order_cnt, 0, sizeof(int32_t) * 27 * ORDER_BINS, h->stream));
    }
    if (!g.slot_pid) {
        int64_t n = h->n;
        RP_CUDA(h, cudaMalloc(&g.slot_pid, sizeof(int32_t) * n));
        RP_CUDA(h, cudaMalloc(&g.pid_slot, sizeof(int32_t) * n));
        RP_CUDA(h, cudaMalloc(&g.pid_cell, sizeof(int32_t) * n));
        RP_CUDA(h, cudaMalloc(&g.rank, sizeof(int32_t) * n));
        RP_CUDA(h, cudaMalloc(&g.mpos, sizeof(float4) * n));
        RP_CUDA(h, cudaMalloc(&g.maxis, sizeof(float4) * n));
        RP_CUDA(h, cudaMalloc(&g.plocal, sizeof(float4) * n));
        RP_CUDA(h, cudaMalloc(&g.max_occ, sizeof(int32_t)));
        if (h->ncen > 0) {
            RP_CUDA(h, cudaMalloc(&g.mcen, sizeof(float4) * n * h->ncen));
            RP_CUDA(h, cudaMalloc(&g.cthr, sizeof(float) * 2 * MAX_CEN * MAX_CEN));
        }
    }
    if (h->ncen > 0) {
        // FP32 centre-pair thresholds of this grid: (r_a + r_b)^2 - margin (overlap below) and
        // (r_a + r_b)^2 + margin (none above); for polyspherocylinders the upper one is the
        // circumspheres' (c_a + c_b)^2 + margin, between the two the segments decide in FP64
        std::vector<float> &t = G.cthr;
        t.assign(2 * MAX_CEN * MAX_CEN, 0.0f);
        for (int a = 0; a < h->ncen; a++)
            for (int b = 0; b < h->ncen; b++) {
                double thr = h->cthr_host[a * MAX_CEN + b];
                double hi = h->segs ? h->circ_host[a * MAX_CEN + b] : thr;
                t[a * MAX_CEN + b] = static_cast<float>(thr - poly_margin(h, G, thr));
                t[MAX_CEN * MAX_CEN + a * MAX_CEN + b] = static_cast<float>(hi + poly_margin(h, G, hi));
            }
        RP_CUDA(h, cudaMemcpyAsync(g.cthr, t.data(), sizeof(float) * t.size(), cudaMemcpyHostToDevice, h->stream));
    }
    // ActiveDomain bounds per cell and dimension
    int64_t nb = 2ll * (dims[0] + dims[1] + dims[2]);
    std::vector<double> bounds(nb);
    int off = 0;
    for (int d = 0; d < 3; d++) {
        g.boundsoff[d] = off;
        for (int c = 0; c < dims[d]; c++) {
            double lo, hi;
            if (dims[d] == 1) {
                lo = -std::numeric_limits<double>::infinity();
                hi = std::numeric_limits<double>::infinity();
            } else {
                lo = shift[d] + static_cast<double>(c) / dims[d];
                if (lo >= 1) lo -= 1;
                hi = shift[d] + static_cast<double>(c + 1) / dims[d];
                if (hi >= 1) hi -= 1;
            }
            bounds[off + 2 * c] = lo;
            bounds[off + 2 * c + 1] = hi;
        }
        off += 2 * dims[d];
    }
    if (h->batch_member) {
        G.bounds_host = bounds;  // the batch packs every replica's bounds into one copy
    } else {
        RP_CUDA(h, ensure(g.bounds, G.bounds_alloc, nb));
        RP_CUDA(h, cudaMemcpyAsync(g.bounds, bounds.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, h->stream));
    }
    // staging filter: with cells well above the interaction range a mover (which stays in
    // its cell, the ActiveDomain) cannot reach much of its neighbour cells; candidates beyond
    // the range from every face-slab of the home cell are not staged.  Off where a dimension
    // has a single cell (unbounded domain there) or where it would keep most candidates.
    double kept = 1.0;
    {
        double hb[3];
        heights_of(box, hb);
        const double thr = h->range * (1.0 + 1e-3) + 1e-3;
        g.stage_filter = 0;
        g.stage_thr = static_cast<float>(thr);
        for (int d = 0; d < 3; d++) {
            const double hc = hb[d] / dims[d];
            g.stage_h[d] = static_cast<float>(hc);
            kept *= std::min(1.0, (hc + 2.0 * thr) / (3.0 * hc));
        }
        // the learned ordering maps partners to unfiltered staging positions
        const bool allowed = h->stage_mode != 0 && h->order_mode == RP_ORDER_OFF && h->pair_cap == 0;
        if (dims[0] > 1 && dims[1] > 1 && dims[2] > 1 && allowed && (kept < 0.9 || h->stage_mode == 2))
            g.stage_filter = 1;
        if (!g.stage_filter) kept = 1.0;
    }
    // staged-candidate capacity per warp: mean neighbourhood plus six standard deviations
    double mean = 27.0 * kept * static_cast<double>(h->n) / static_cast<double>(ncell);
    int cap = static_cast<int>(mean + 6.0 * std::sqrt(mean) + 32.0);
    cap = (cap + 31) / 32 * 32;
    int maxcap = static_cast<int>(48 * 1024 / (sweep_smem_per_warp(h->shape.kind, 32, false, h->ncen) / 32));
    G.cap = std::min(cap, maxcap / 32 * 32);
    // two cells per warp: 32 lane groups per SM (4 blocks of 8) in 224 KB of shared memory
    // (capacities in multiples of 16); offered while that capacity holds the mean
    // neighbourhood plus four standard deviations (the rare larger neighbourhood reruns in the
    // overflow pass; larger neighbourhoods keep a warp per cell)
    G.cap_half = 0;
    if (h->shape.kind != RP_SHAPE_POLYSPHERE) {
        const int half_max = static_cast<int>(224 * 1024 / (SWEEP_WARPS * 2 * 4) /
                                              (sweep_smem_per_half(h->shape.kind, 16) / 16)) / 16 * 16;
        if (mean + 4.0 * std::sqrt(mean) + 16.0 <= half_max) G.cap_half = std::min(G.cap, half_max);
    }
    int64_t nblocks = (ncell + 4095) / 4096;
    RP_CUDA(h, ensure(h->block_sums, h->block_sums_alloc, nblocks));
    RP_CUDA(h, ensure(h->overflow, h->overflow_alloc, ncell));
    return RP_OK;
}

int rebuild(Handle *h, int gi, int pi) {
    int saved_g = h->gcur, saved_p = h->pcur;
    h->gcur = gi;
    h->pcur = pi;
    DevState s = dev_state(h);
    h->gcur = saved_g;
    h->pcur = saved_p;
    {
        Group grp(h, RP_KERNEL_REBUILD, 6);
        RP_CUDA(h, launch_rebuild(s, h->grid[gi].d, h->block_sums, h->stream));
    }
    h->grid_rebuilds++;
    // a grid built from the current positions lists every particle where it is
    if (!h->disp_host.empty()) {
        RP_CUDA(h, cudaMemsetAsync(h->d_disp_flag, 0, static_cast<size_t>(h->n), h->stream));
        for (int32_t p : h->disp_host) h->disp_flag_host[p] = 0;
        h->disp_host.clear();
    }
    h->grid_patched = false;
    return RP_OK;
}

// The grid of a rescaled state (rp_try_scaling; h->gcur / h->pcur already name grid `ng` and
// the rescaled positions): when its divisions and origin are the old grid's and the old grid
// lists every particle where it is, the old cells are kept and only the FP32 cell-local
// positions recomputed (k_remap, one pass, the grid a rebuild would build); a particle that
// changed cell through rounding falls back to the full rebuild.
int remap_or_rebuild(Handle *h, int old_g, int ng, int np) {
    const GridDev &o = h->grid[old_g].d, &g = h->grid[ng].d;
    bool same = !h->grid_patched && !h->grid_stale && h->disp_host.empty() && o.ncell == g.ncell && o.slot_pid;
    for (int d = 0; d < 3; d++) same = same && o.dims[d] == g.dims[d] && o.shift[d] == g.shift[d];
    if (same) {
        RP_CUDA(h, cudaMemsetAsync(h->flag, 0, sizeof(int), h->stream));
        {
            Group grp(h, RP_KERNEL_RESCALE, 1);
            RP_CUDA(h, launch_remap(dev_state(h), g, o, h->flag, h->stream));
        }
        int moved = 0;
        RP_CUDA(h, cudaMemcpyAsync(&moved, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
        if (!moved) {
            // the kept cells keep their occupancy order
            if (g.order && o.order)
                RP_CUDA(h, cudaMemcpyAsync(g.order, o.order, sizeof(int32_t) * g.ncell, cudaMemcpyDeviceToDevice,
                                           h->stream));
            h->grid_remaps++;
            return RP_OK;
        }
    }
    return rebuild(h, ng, np);
}

int check_status(Handle *h) {
    uint32_t st = 0;
    RP_CUDA(h, cudaMemcpyAsync(&st, h->status, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st) {
        RP_CUDA(h, cudaMemsetAsync(h->status, 0, sizeof(uint32_t), h->stream));
        char buf[256];
        std::snprintf(buf, sizeof(buf), "device status 0x%x%s%s%s%s", st,
                      (st & ST_PARTICLE_NOT_IN_CELL) ? " (a move's particle is not in its cell)" : "",
                      (st & ST_CAPACITY) ? " (a cell neighbourhood exceeds the staging capacity)" : "",
                      (st & ST_PORTAL_STUCK) ? " (a convex pair's portal refinement did not converge)" : "",
                      (st & ST_STAGE_TIMEOUT) ? " (a staging copy did not complete in time)" : "");
        if (st & ST_OUTSIDE) return fail(h, RP_ERR_ARG, "a particle lies outside the box");
        if (st & ST_NOT_ROTATION)
            return fail(h, RP_ERR_ARG, "an orientation is not a rotation matrix (|O^T O - I| >= 1e-6)");
        return fail(h, (st & ST_CAPACITY) ? RP_ERR_CAPACITY : RP_ERR_DEVICE, buf);
    }
    return RP_OK;
}

// The current cell grid, rebuilt if it is stale: unshifted after an upload, else with the
// origin of the grid it replaces (a soft sweep's log is read against that sweep's domains).
int ensure_grid(Handle *h) {
    if (!h->grid_stale) return RP_OK;
    double shift[3] = {0, 0, 0};
    if (!h->stale_unshifted)
        for (int d = 0; d < 3; d++) shift[d] = h->grid[h->gcur].d.shift[d];
    int rc = setup_grid(h, h->grid[h->gcur], h->box, shift);
    if (rc) return rc;
    rc = rebuild(h, h->gcur, h->pcur);
    if (rc) return rc;
    h->grid_stale = false;
    h->stale_unshifted = false;
    return RP_OK;
}

void phase_bits(const GridDev &g, int cell, int &ph) { ph = cell_phase(g.dims, cell); }

// Every phase of a grid (one colour per dimension), in a shuffled order.
void grid_phases(const GridDev &g, uint32_t x, std::vector<int> &phases) {
    phases.clear();
    for (int p2 = 0; p2 < ring_ncol(g.dims[2]); p2++)
        for (int p1 = 0; p1 < ring_ncol(g.dims[1]); p1++)
            for (int p0 = 0; p0 < ring_ncol(g.dims[0]); p0++) phases.push_back(p0 + 3 * p1 + 9 * p2);
    for (int k = static_cast<int>(phases.size()) - 1; k > 0; k--) {
        x = x * 1664525u + 1013904223u;
        int j = static_cast<int>((static_cast<uint64_t>(x) * (k + 1)) >> 32);
        std::swap(phases[k], phases[j]);
    }
}

// Cells of one phase.
int phase_cells(const GridDev &g, int ph, int act[3]) {
    for (int d = 0; d < 3; d++) act[d] = ring_count(g.dims[d], phase_digit(ph, d));
    return act[0] * act[1] * act[2];
}

SweepArgs base_args(Handle *h) {
    SweepArgs a{};
    a.s = dev_state(h);
    a.g = h->grid[h->gcur].d;
    a.cap = h->grid[h->gcur].cap;
    // sphere distances of a sheared box without the reference's grid are not geometric:
    // no FP32 certificate, every pair in FP64
    a.fp64_only = (a.s.pbc_fold == 2 && a.s.kind != 1) ? 1 : 0;
    a.bulk_stage = h->bulk_stage;
    a.overflow = h->overflow;
    a.overflow_count = h->overflow_count;
    return a;
}

// Where phase ph begins in the grid's occupancy order (phase-major): the cells of the phases
// before it (a colour digit beyond a dimension's colours names no cells).
static void order_starts(const GridDev &g, int start[27]) {
    int acc = 0;
    for (int ph = 0; ph < 27; ph++) {
        start[ph] = acc;
        int cnt = 1;
        for (int d = 0; d < 3; d++) {
            const int digit = phase_digit(ph, d);
            cnt *= digit < ring_ncol(g.dims[d]) ? ring_count(g.dims[d], digit) : 0;
        }
        acc += cnt;
    }
}

// Re-runs the cells of a phase whose neighbourhood did not fit the normal staging
// capacity, with one large-capacity warp per block (device-side work count).
int run_overflow(Handle *h, SweepArgs a, bool list) {
    int cap = static_cast<int>(OVF_SMEM / sweep_smem_per_warp(a.s.kind, 32, false, a.s.ncen) * 32);
    cap = cap / 32 * 32;
    a.cap = cap;
    a.work = h->overflow;
    a.work_count = h->overflow_count;
    a.partners = nullptr;  // the plain kernel: no partner pre-test, no pair log
    a.pair_every = 0;
    a.num_work = -1;
    a.overflow = nullptr;
    {
        Group grp(h, RP_KERNEL_OVERFLOW, 1);
        RP_CUDA(h, launch_sweep(a, list, OVF_WARPS, h->stream));
    }
    RP_CUDA(h, cudaMemsetAsync(h->overflow_count, 0, sizeof(int32_t), h->stream));
    return RP_OK;
}

// ---- learned ordering -----------------------------------------------------------
static_assert(MLP_NPARAM == RP_MLP_NPARAM && MLP_IN == RP_MLP_FEATURES, "network layout");


// He-uniform weights from a splitmix64 stream, zero biases.
void mlp_init_host(uint64_t seed, std::vector<float> &w) {
    w.assign(MLP_NPARAM, 0.f);
    uint64_t x = seed ^ 0x6a09e667f3bcc909ull;
    auto next = [&x]() {
        x += 0x9e3779b97f4a7c15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    const double a1 = std::sqrt(6.0 / MLP_FEATURES), a2 = std::sqrt(6.0 / MLP_H);
    for (int o = 0; o < MLP_H; o++)
        for (int k = 0; k < MLP_IN; k++) w[MLP_W1 + o * MLP_IN + k] = k < MLP_FEATURES ? static_cast<float>(a1 * next()) : 0.f;
    for (int i = 0; i < MLP_H * MLP_H; i++) w[MLP_W2 + i] = static_cast<float>(a2 * next());
    for (int i = 0; i < MLP_H; i++) w[MLP_W3 + i] = static_cast<float>(a2 * next());
}

int mlp_upload(Handle *h, const float *params) {
    RP_CUDA(h, cudaMemcpyAsync(h->mlp_w32, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, h->stream));
    RP_CUDA(h, cudaMemsetAsync(h->mlp_m, 0, sizeof(float) * MLP_NPARAM, h->stream));
    RP_CUDA(h, cudaMemsetAsync(h->mlp_v, 0, sizeof(float) * MLP_NPARAM, h->stream));
    RP_CUDA(h, launch_mlp_sync16(h->mlp_w32, h->mlp_w16, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    h->mlp_step = 0;
    h->partners_valid = false;
    return RP_OK;
}

// Allocates the network state on first use (seed-0 initialisation).
int mlp_ready(Handle *h) {
    if (h->mlp_w32) return RP_OK;
    RP_CUDA(h, cudaMalloc(&h->mlp_w32, sizeof(float) * MLP_NPARAM));
    RP_CUDA(h, cudaMalloc(&h->mlp_grad, sizeof(float) * MLP_NPARAM));
    RP_CUDA(h, cudaMalloc(&h->mlp_m, sizeof(float) * MLP_NPARAM));
    RP_CUDA(h, cudaMalloc(&h->mlp_v, sizeof(float) * MLP_NPARAM));
    RP_CUDA(h, cudaMalloc(&h->mlp_loss, sizeof(float)));
    RP_CUDA(h, cudaMalloc(&h->mlp_w16, sizeof(__nv_bfloat16) * (MLP_NPARAM + 7)));
    std::vector<float> w;
    mlp_init_host(0, w);
    return mlp_upload(h, w.data());
}

// Ranks every particle's in-range neighbours on the current grid (one launch).
int rank_partners(Handle *h) {
    int rc = mlp_ready(h);
    if (rc) return rc;
    if (!h->partners) RP_CUDA(h, cudaMalloc(&h->partners, sizeof(int32_t) * MLP_PARTNERS * h->n));
    {
        Group grp(h, RP_KERNEL_ORDER, 1);
        RP_CUDA(h, launch_score_partners(dev_state(h), h->grid[h->gcur].d, h->mlp_w32, h->mlp_w16, h->order_mode,
                                         static_cast<float>(1.0 / h->range), h->partners, h->stream));
    }
    h->partners_valid = true;
    h->since_rank = 0;
    return RP_OK;
}

// ---- batched replicas ----------------------------------------------------------------

struct Batch {
    int device = 0, kind = 0, R = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    std::vector<Handle *> rep;
    BatchRep *d_table = nullptr;                      // [R]
    int *d_bases = nullptr;                           // pbase, cbase, item_base of each phase: (2 + MAX_PHASES) x (R + 1)
    double *d_bounds = nullptr;                       // packed ActiveDomain bounds
    int64_t d_bounds_alloc = 0;
    // two pinned staging sets used alternately; a set is rewritten only after its copies ran
    struct Staging {
        BatchRep *table = nullptr;
        int *bases = nullptr;
        double *bounds = nullptr;
        int64_t bounds_alloc = 0;
        cudaEvent_t done = nullptr;
        bool pending = false;
    } stage[2];
    int cur = 0;
    double *rtab64 = nullptr;
    float *rtab32 = nullptr;
    int32_t *item_counters = nullptr;                 // [MAX_PHASES]
    unsigned long long *stats = nullptr;              // [R][NUM_COUNTERS]
    uint32_t *status = nullptr;                       // [R]
    unsigned long long *counts = nullptr, *h_counts = nullptr;  // [R]
    int *flags = nullptr, *h_flags = nullptr;         // [R]
    int wpb = 4;
    int smem_optin = 48 * 1024;                       // largest dynamic shared memory per block
    uint64_t launches = 0;
    Timing tm;
    std::string err;
};
using BGroup = GroupOf<Batch>;

int bfail(Batch *b, int code, const std::string &msg) {
    if (b) b->err = msg;
    return code;
}

#define RB_CUDA(b, call)                                                                                  \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return bfail((b), RP_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

// The grid origin and phase order of one replica's sweep, from the replica's Philox stream
// (the single-system sweep derives them the same way).
void sweep_origin(uint64_t seed, uint64_t counter, double shift[3], uint32_t &shuffle) {
    u4 r = philox(u4{0x5eedu, 0x9e37u, static_cast<uint32_t>(counter), static_cast<uint32_t>(counter >> 32)},
                  static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    shift[0] = (r.a >> 8) * (1.0 / 16777216.0);
    shift[1] = (r.b >> 8) * (1.0 / 16777216.0);
    shift[2] = (r.c >> 8) * (1.0 / 16777216.0);
    shuffle = r.d;
}

void phase_order(const GridDev &g, uint32_t x, std::vector<int> &phases) { grid_phases(g, x, phases); }

uint64_t replica_seed(uint64_t seed, int r) { return seed + RP_BATCH_SEED_STRIDE * static_cast<uint64_t>(r); }

// Packs every replica's current-grid bounds and fills the table entries and prefix
// arrays in the current pinned staging set (after its previous copies have run).
int batch_tables(Batch *b, int &total_items, int &total_p, int &total_c) {
    Batch::Staging &S = b->stage[b->cur];
    if (S.pending) RB_CUDA(b, cudaEventSynchronize(S.done));
    S.pending = false;
    int64_t nb = 0;
    for (Handle *h : b->rep) nb += static_cast<int64_t>(h->grid[h->gcur].bounds_host.size());
    if (nb > S.bounds_alloc) {
        cudaFreeHost(S.bounds);
        S.bounds = nullptr;
        S.bounds_alloc = 0;
        RB_CUDA(b, cudaMallocHost(&S.bounds, sizeof(double) * nb * 2));
        S.bounds_alloc = nb * 2;
    }
    if (nb > b->d_bounds_alloc) {
        RB_CUDA(b, cudaStreamSynchronize(b->stream));  // the old array may still be read
        cudaFree(b->d_bounds);
        b->d_bounds = nullptr;
        b->d_bounds_alloc = 0;
        RB_CUDA(b, cudaMalloc(&b->d_bounds, sizeof(double) * nb * 2));
        b->d_bounds_alloc = nb * 2;
    }
    int64_t off = 0;
    int *pb = S.bases, *cb = S.bases + (b->R + 1);
    pb[0] = cb[0] = 0;
    for (int r = 0; r < b->R; r++) {
        Handle *h = b->rep[r];
        GridHost &G = h->grid[h->gcur];
        std::memcpy(S.bounds + off, G.bounds_host.data(), sizeof(double) * G.bounds_host.size());
        G.d.bounds = b->d_bounds + off;
        off += static_cast<int64_t>(G.bounds_host.size());
        BatchRep &T = S.table[r];
        T = BatchRep{};
        T.a = base_args(h);
        pb[r + 1] = pb[r] + static_cast<int>(h->n);
        cb[r + 1] = cb[r] + G.d.ncell;
    }
    total_items = 0;
    total_p = pb[b->R];
    total_c = cb[b->R];
    return RP_OK;
}

// Copies the current staging set to the device and moves on to the other set.
int batch_copy(Batch *b) {
    Batch::Staging &S = b->stage[b->cur];
    int64_t nb = 0;
    for (Handle *h : b->rep) nb += static_cast<int64_t>(h->grid[h->gcur].bounds_host.size());
    RB_CUDA(b, cudaMemcpyAsync(b->d_bounds, S.bounds, sizeof(double) * nb, cudaMemcpyHostToDevice, b->stream));
    RB_CUDA(b, cudaMemcpyAsync(b->d_table, S.table, sizeof(BatchRep) * b->R, cudaMemcpyHostToDevice, b->stream));
    RB_CUDA(b, cudaMemcpyAsync(b->d_bases, S.bases, sizeof(int) * (2 + MAX_PHASES) * (b->R + 1), cudaMemcpyHostToDevice,
                               b->stream));
    RB_CUDA(b, cudaEventRecord(S.done, b->stream));
    S.pending = true;
    b->cur ^= 1;
    return RP_OK;
}

}  // namespace
}  // namespace rp

using namespace rp;

extern "C" {

// Device allocations and the stream of a new handle whose shape fields are set.
// why the last rp_create* on this thread failed, for rp_last_error(NULL)
static thread_local std::string g_create_error;

static int create_common(Handle *h, int64_t n, int device, void **handle) {
    h->device = device;
    h->n = n;
    g_create_error.clear();
    auto bail = [&](cudaError_t e) {
        h->err = cudaGetErrorString(e);
        g_create_error = std::string("creating the packing on device ") + std::to_string(device) + ": " + h->err;
        rp_destroy(h);
        return RP_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return bail(e);
    if ((e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return bail(e);
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
    for (int i = 0; i < 2; i++) {
        if ((e = cudaMalloc(&h->pos64[i], sizeof(double) * 3 * n)) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&h->trans[i], sizeof(double) * 3 * 125)) != cudaSuccess) return bail(e);
        if (h->ncen > 0 && (e = cudaMalloc(&h->abs64[i], sizeof(double) * 3 * n * h->ncen)) != cudaSuccess)
            return bail(e);
    }
    if (h->ncen > 0) {
        if ((e = cudaMalloc(&h->cen64, sizeof(double) * 3 * n * h->ncen)) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&h->cthr64, sizeof(double) * MAX_CEN * MAX_CEN)) != cudaSuccess) return bail(e);
        if ((e = cudaMemcpy(h->cthr64, h->cthr_host, sizeof(h->cthr_host), cudaMemcpyHostToDevice)) != cudaSuccess)
            return bail(e);
        if ((e = cudaMalloc(&h->circ64, sizeof(double) * MAX_CEN * MAX_CEN)) != cudaSuccess) return bail(e);
        if ((e = cudaMemcpy(h->circ64, h->circ_host, sizeof(h->circ_host), cudaMemcpyHostToDevice)) != cudaSuccess)
            return bail(e);
        if ((e = cudaMalloc(&h->cbody_dev, sizeof(h->cbody))) != cudaSuccess) return bail(e);
        if ((e = cudaMemcpy(h->cbody_dev, h->cbody, sizeof(h->cbody), cudaMemcpyHostToDevice)) != cudaSuccess)
            return bail(e);
    }
    if ((e = cudaMalloc(&h->rot64, sizeof(double) * 9 * n)) != cudaSuccess) return bail(e);
    if (!h->batch_member) {
        if ((e = cudaMalloc(&h->rtab64, sizeof(double) * 9 * ROT_TABLE)) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&h->rtab32, sizeof(float) * 12 * ROT_TABLE)) != cudaSuccess) return bail(e);
    }
    if ((e = cudaMalloc(&h->item_counters, sizeof(int32_t) * 64)) != cudaSuccess) return bail(e);
    if (!h->batch_member) {
        if ((e = cudaMalloc(&h->status, sizeof(uint32_t))) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&h->counters, sizeof(unsigned long long) * NUM_COUNTERS)) != cudaSuccess) return bail(e);
        cudaMemset(h->status, 0, sizeof(uint32_t));
        cudaMemset(h->counters, 0, sizeof(unsigned long long) * NUM_COUNTERS);
    }
    if ((e = cudaMalloc(&h->count_out, sizeof(unsigned long long))) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc(&h->flag, sizeof(int))) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc(&h->overflow_count, sizeof(int32_t))) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc(&h->d_overlaps, sizeof(unsigned long long))) != cudaSuccess) return bail(e);
    cudaMemset(h->d_overlaps, 0, sizeof(unsigned long long));
    cudaMemset(h->overflow_count, 0, sizeof(int32_t));
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return bail(e);
    *handle = h;
    return RP_OK;
}

int rp_create(const rp_shape_desc *shape, int64_t n, int device, void **handle) {
    if (!shape || !handle || n <= 0 || n > (1ll << 31) - 1) return RP_ERR_ARG;
    if (shape->kind != RP_SHAPE_SPHERE && shape->kind != RP_SHAPE_SPHEROCYLINDER) return RP_ERR_UNSUPPORTED;
    if (!(shape->radius > 0) || (shape->kind == RP_SHAPE_SPHEROCYLINDER && !(shape->length >= 0))) return RP_ERR_ARG;
    Handle *h = new (std::nothrow) Handle();
    if (!h) return RP_ERR_ARG;
    h->shape = *shape;
    double r = shape->radius, l = shape->length;
    ExactShape ex{};
    ex.kind = shape->kind;
    if (shape->kind == RP_SHAPE_SPHERE) {
        h->range = 2 * r;                      // SphereTraits.h:34
        ex.sphere_thr = std::pow(2 * r, 2);     // SphereTraits.cpp:64
    } else {
        h->range = 2 * r + l;                  // SpherocylinderTraits.h:81
        ex.core_thr = 4 * r * r;                // SpherocylinderTraits.cpp:35
        ex.far_thr = std::pow(2 * r + l, 2);    // SpherocylinderTraits.cpp:37
        short beg = -1, end = 1;                // SpherocylinderTraits.cpp:23-25
        ex.neg_cap_half = 0.5 * beg * l;
        ex.cap_half = 0.5 * end * l;
    }
    h->ref_range = h->range;
    h->total_range = h->range;  // no interaction centres
    h->ex = ex;
    return create_common(h, n, device, handle);
}

namespace {

// Polyspheres (PolysphereTraits) and polyspherocylinders (PolyspherocylinderTraits, half
// axes given): the multi-centre bodies of the engine.
int create_multi_centre(int32_t num_centres, const double *centres, const double *half_axes, const double *radii,
                        int64_t n, int device, void **handle) {
    if (!centres || !radii || !handle || n <= 0 || n > (1ll << 31) - 1) return RP_ERR_ARG;
    if (num_centres < 1 || num_centres > MAX_CEN) return RP_ERR_UNSUPPORTED;
    for (int b = 0; b < num_centres; b++) {
        if (!(radii[b] > 0)) return RP_ERR_ARG;
        for (int d = 0; d < 3; d++)
            if (!std::isfinite(centres[3 * b + d]) || (half_axes && !std::isfinite(half_axes[3 * b + d])))
                return RP_ERR_ARG;
    }
    Handle *h = new (std::nothrow) Handle();
    if (!h) return RP_ERR_ARG;
    h->shape.kind = RP_SHAPE_POLYSPHERE;
    h->ncen = num_centres;
    h->segs = half_axes ? 1 : 0;
    // a centre's reach: its sphere radius, or the spherocylinder's circumsphere radius
    // radius + |halfAxis| (PolyspherocylinderTraits.cpp:78-84)
    double outer[MAX_CEN]{};
    for (int b = 0; b < num_centres; b++) {
        outer[b] = radii[b];
        if (half_axes) {
            for (int d = 0; d < 3; d++) h->chax[3 * b + d] = half_axes[3 * b + d];
            const d3 ha{half_axes[3 * b], half_axes[3 * b + 1], half_axes[3 * b + 2]};
            outer[b] = radii[b] + std::sqrt(norm2(ha));
        }
    }
    double rmax = 0, omax = 0, reach = 0;
    for (int b = 0; b < num_centres; b++) {
        for (int d = 0; d < 3; d++) h->cbody[3 * b + d] = centres[3 * b + d];
        h->crad[b] = radii[b];
        rmax = std::max(rmax, radii[b]);
        omax = std::max(omax, outer[b]);
        double c = std::sqrt(centres[3 * b] * centres[3 * b] + centres[3 * b + 1] * centres[3 * b + 1] +
                             centres[3 * b + 2] * centres[3 * b + 2]);
        reach = std::max(reach, c + outer[b]);
    }
    for (int a = 0; a < num_centres; a++)
        for (int b = 0; b < num_centres; b++) {
            double r = radii[a] + radii[b];      // PolysphereTraits.cpp:104-105, PolyspherocylinderTraits.cpp:111-112
            h->cthr_host[a * MAX_CEN + b] = r * r;
            double c = outer[a] + outer[b];      // PolyspherocylinderTraits.cpp:115-116
            h->circ_host[a * MAX_CEN + b] = c * c;
        }
    h->shape.radius = rmax;
    // the reference's neighbour-grid cell: PolysphereTraits.cpp:115-120 (2 max r),
    // PolyspherocylinderTraits.cpp:140-147 (2 max circumsphere radius)
    h->ref_range = 2 * (half_axes ? omax : rmax);
    {
        // Interaction::getTotalRangeRadius: 2 sqrt(max |centre|^2) + range
        double m2 = 0;
        for (int b = 0; b < num_centres; b++) {
            const double r2 = centres[3 * b] * centres[3 * b] + centres[3 * b + 1] * centres[3 * b + 1] +
                              centres[3 * b + 2] * centres[3 * b + 2];
            if (r2 > m2) m2 = r2;
        }
        h->total_range = 2 * std::sqrt(m2) + h->ref_range;
    }
    // cells of the checkerboard: two bodies farther apart than twice the largest reach
    // |c| + r (or |c| + circumsphere radius) cannot touch (rotated centres keep |c| up to
    // FP64 rounding)
    h->range = 2 * reach * (1.0 + 1e-12);
    return create_common(h, n, device, handle);
}

}  // namespace

int rp_create_polysphere(int32_t num_centres, const double *centres, const double *radii, int64_t n, int device,
                         void **handle) {
    return create_multi_centre(num_centres, centres, nullptr, radii, n, device, handle);
}

int rp_create_polyspherocylinder(int32_t num_centres, const double *centres, const double *half_axes,
                                 const double *radii, int64_t n, int device, void **handle) {
    if (!half_axes) return RP_ERR_ARG;
    return create_multi_centre(num_centres, centres, half_axes, radii, n, device, handle);
}

// Generic convex bodies (GenericXenoCollideTraits): the XCBodyBuilder script's geometry on the
// device; the range is twice its circumsphere radius (XenoCollideTraits::getRangeRadius,
// core/shapes/XenoCollideTraits.h:188-202).
int rp_create_convex(const char *script, int64_t n, int device, void **handle) {
    // (the move kernels queue near pairs as particle * 28 + image in an int)
    if (!script || !handle || n <= 0 || n > ((1ll << 31) - 1) / 28) return RP_ERR_ARG;
    XcShape *xs = new (std::nothrow) XcShape();
    if (!xs) return RP_ERR_ARG;
    std::string err;
    if (!xc_build(script, *xs, err)) {
        g_create_error = "convex body: " + err;
        delete xs;
        return RP_ERR_ARG;
    }
    if (!(xs->circ > 0)) {
        g_create_error = "convex body: the body has no extent (circumsphere radius 0)";
        delete xs;
        return RP_ERR_ARG;
    }
    // the support function's explicit stack lives in each thread's local memory
    size_t stack = 0;
    if (cudaSetDevice(device) == cudaSuccess && cudaDeviceGetLimit(&stack, cudaLimitStackSize) == cudaSuccess &&
        stack < 4096)
        cudaDeviceSetLimit(cudaLimitStackSize, 4096);
    Handle *h = new (std::nothrow) Handle();
    if (!h) {
        delete xs;
        return RP_ERR_ARG;
    }
    h->shape.kind = RP_SHAPE_CONVEX;
    h->shape.radius = xs->circ;
    h->range = 2 * xs->circ;
    h->ref_range = h->range;
    h->total_range = h->range;
    int rc = create_common(h, n, device, handle);
    if (rc) {
        delete xs;
        return rc;
    }
    cudaError_t e = cudaMalloc(&h->d_xc, sizeof(XcShape));
    if (e == cudaSuccess) e = cudaMemcpy(h->d_xc, xs, sizeof(XcShape), cudaMemcpyHostToDevice);
    delete xs;
    if (e != cudaSuccess) {
        g_create_error = std::string("creating the packing on device ") + std::to_string(device) + ": " +
                         cudaGetErrorString(e);
        rp_destroy(h);
        *handle = nullptr;
        return RP_ERR_CUDA;
    }
    return RP_OK;
}

// The pair test of a convex handle's body on n pairs given in host arrays (parity checks of
// the device's support functions and portal refinement).
int rp_convex_pair_overlaps(void *handle, int64_t n, const double *pos1, const double *rot1, const double *pos2,
                            const double *rot2, uint8_t *out) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || n < 0 || (n > 0 && (!pos1 || !rot1 || !pos2 || !rot2 || !out))) return fail(h, RP_ERR_ARG, "bad argument");
    if (h->shape.kind != RP_SHAPE_CONVEX) return fail(h, RP_ERR_UNSUPPORTED, "not a convex-body handle");
    if (n == 0) return RP_OK;
    RP_CUDA(h, cudaSetDevice(h->device));
    const size_t nn = static_cast<size_t>(n);
    double *d = nullptr;
    uint8_t *o = nullptr;
    RP_CUDA(h, cudaMalloc(&d, sizeof(double) * 24 * nn));
    cudaError_t e = cudaMalloc(&o, nn);
    const size_t off[4] = {0, 3 * nn, 12 * nn, 15 * nn};
    const double *src[4] = {pos1, rot1, pos2, rot2};
    const size_t len[4] = {3 * nn, 9 * nn, 3 * nn, 9 * nn};
    for (int k = 0; k < 4 && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(d + off[k], src[k], sizeof(double) * len[k], cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = launch_convex_pairs(h->d_xc, n, d + off[0], d + off[1], d + off[2], d + off[3], o, h->status, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, o, nn, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    cudaFree(o);
    if (e != cudaSuccess) return fail(h, RP_ERR_CUDA, cudaGetErrorString(e));
    return check_status(h);
}

int rp_destroy(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->snap_free) {
        cudaEventSynchronize(h->snap_free);
        cudaEventDestroy(h->snap_free);
    }
    cudaFree(h->snap64);
    cudaFree(h->d_xc);
    for (int i = 0; i < 2; i++) {
        cudaFree(h->pos64[i]);
        cudaFree(h->trans[i]);
        GridDev &g = h->grid[i].d;
        cudaFree(g.count);
        cudaFree(g.start);
        cudaFree(g.order);
        cudaFree(g.order_cnt);
        cudaFree(g.order_off);
        cudaFree(g.slot_pid);
        cudaFree(g.pid_slot);
        cudaFree(g.pid_cell);
        cudaFree(g.rank);
        cudaFree(g.mpos);
        cudaFree(g.maxis);
        cudaFree(g.plocal);
        if (!h->batch_member) cudaFree(g.bounds);
        cudaFree(g.max_occ);
        cudaFree(g.mcen);
        cudaFree(g.cthr);
    }
    cudaFree(h->rot64);
    cudaFree(h->cen64);
    cudaFree(h->abs64[0]);
    cudaFree(h->abs64[1]);
    cudaFree(h->cthr64);
    cudaFree(h->circ64);
    cudaFree(h->cbody_dev);
    if (!h->batch_member) {
        cudaFree(h->rtab64);
        cudaFree(h->rtab32);
    }
    cudaFree(h->item_counters);
    cudaFree(h->block_sums);
    if (!h->batch_member) {
        cudaFree(h->status);
        cudaFree(h->counters);
    }
    cudaFree(h->count_out);
    cudaFree(h->cq_buf);
    cudaFree(h->cq_count);
    cudaFree(h->d_try);
    cudaFree(h->d_energy);
    cudaFree(h->d_disp_list);
    cudaFree(h->d_disp_flag);
    cudaFree(h->flag);
    cudaFree(h->overflow);
    cudaFree(h->overflow_count);
    cudaFree(h->d_overlaps);
    cudaFree(h->d_moves);
    cudaFree(h->d_list);
    cudaFree(h->d_codes);
    cudaFree(h->d_log);
    cudaFree(h->d_log_codes);
    for (void *p : {(void *)h->mlp_w32, (void *)h->mlp_grad, (void *)h->mlp_m, (void *)h->mlp_v,
                    (void *)h->mlp_loss, (void *)h->mlp_w16, (void *)h->mlp_feats, (void *)h->mlp_labels,
                    (void *)h->mlp_out, (void *)h->partners, (void *)h->pair_feats, (void *)h->pair_labels,
                    (void *)h->pair_count})
        cudaFree(p);
    h->tm.release();
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return RP_OK;
}

const char *rp_last_error(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (h) return h->err.c_str();
    return g_create_error.empty() ? "null handle" : g_create_error.c_str();
}

int rp_upload_state(void *handle, const double *pos, const double *rot, const double *box9) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !pos || !rot || !box9) return fail(h, RP_ERR_ARG, "null argument");
    RP_CUDA(h, cudaSetDevice(h->device));
    h->try_valid = false;
    double inv[9];
    if (det3(box9) == 0) return fail(h, RP_ERR_ARG, "box volume is zero");
    inverse3(box9, inv);
    std::memcpy(h->box, box9, sizeof(h->box));
    std::memcpy(h->inv, inv, sizeof(h->inv));
    h->pcur = 0;
    h->gcur = 0;
    h->partners_valid = false;
    RP_CUDA(h, cudaMemcpyAsync(h->pos64[0], pos, sizeof(double) * 3 * h->n, cudaMemcpyHostToDevice, h->stream));
    RP_CUDA(h, cudaMemcpyAsync(h->rot64, rot, sizeof(double) * 9 * h->n, cudaMemcpyHostToDevice, h->stream));
    if (h->ncen > 0) {
        // interactionCentres = orientation · centre (Packing::setupForInteraction,
        // core/Packing.cpp:940-944), on the device; absolute centres after the rebuild
        Group grp(h, RP_KERNEL_REBUILD, 1);
        RP_CUDA(h, launch_fresh_centres(dev_state(h), h->cbody_dev, h->stream));
    }
    double tt[375];
    translation_table(h->box, tt);
    RP_CUDA(h, cudaMemcpyAsync(h->trans[0], tt, sizeof(tt), cudaMemcpyHostToDevice, h->stream));
    h->has_state = false;
    int rc = RP_OK;
    if (h->batch_member) {
        // replicas: the grid at once (the batch reads the replicas' grids directly)
        double shift[3] = {0, 0, 0};
        rc = setup_grid(h, h->grid[0], h->box, shift);
        if (rc) return rc;
        h->strict_box = true;
        rc = rebuild(h, 0, 0);
        h->strict_box = false;
        if (rc) return rc;
    } else {
        // the checks alone; the next sweep builds its own grid, other calls build one first
        Group grp(h, RP_KERNEL_REBUILD, 1);
        RP_CUDA(h, launch_validate(dev_state(h), h->stream));
        h->grid_stale = true;
        h->stale_unshifted = true;
    }
    rc = check_status(h);  // every particle inside the box, orientations rotations
    if (rc) return rc;
    if (h->ncen > 0) {
        Group grp(h, RP_KERNEL_REBUILD, 1);
        RP_CUDA(h, launch_abs_centres(dev_state(h), h->stream));
    }
    h->has_state = true;
    h->can_revert = false;
    h->log_valid = false;
    return RP_OK;
}

int rp_download_state(void *handle, double *pos, double *rot, double *box9) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    RP_CUDA(h, cudaSetDevice(h->device));
    if (pos)
        RP_CUDA(h, cudaMemcpyAsync(pos, h->pos64[h->pcur], sizeof(double) * 3 * h->n, cudaMemcpyDeviceToHost,
                                   h->stream));
    if (rot)
        RP_CUDA(h, cudaMemcpyAsync(rot, h->rot64, sizeof(double) * 9 * h->n, cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    if (box9) std::memcpy(box9, h->box, sizeof(h->box));
    return RP_OK;
}

// FP32 pre-filter of a separation at one image: the interaction range (body range for
// multi-centre bodies) plus a margin far above the FP32 rounding of coordinates of the box's
// size; a single image per pair where that reach stays below 0.45 of every box height (the
// heights are the reciprocal norms of the inverse box's rows).
static void set_prefilter(SingleArgs &a, const Handle *h) {
    double pmax = 0, rowmax = 0;
    for (int i = 0; i < 3; i++) {
        pmax = std::max(pmax, std::fabs(h->box[3 * i]) + std::fabs(h->box[3 * i + 1]) + std::fabs(h->box[3 * i + 2]));
        const double *r = h->inv + 3 * i;
        rowmax = std::max(rowmax, std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]));
    }
    const double reach = h->range * (1.0 + 1e-3) + 1e-4 * (pmax + h->range);
    a.reach2 = static_cast<float>(reach * reach);
    for (int i = 0; i < 9; i++) a.box32[i] = static_cast<float>(h->box[i]);
    a.one_image = reach * rowmax <= 0.45 ? 1 : 0;
}

// The arguments of the FP64 kernels (single moves, soft and convex sweeps, FP64 recounts) for the
// current state: the FP32 pre-filter reach of a separation at one image is the interaction
// range (body range for multi-centre bodies) plus a margin far above the FP32 rounding of
// coordinates of the box's size.
SingleArgs single_args(Handle *h) {
    SingleArgs a{};
    a.s = dev_state(h);
    a.g = h->grid[h->gcur].d;
    set_prefilter(a, h);
    return a;
}

int rp_count_overlaps(void *handle, int early_exit, int64_t *out_count) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !out_count) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    RP_CUDA(h, cudaSetDevice(h->device));
    if (h->soft_only) {  // no hard part: nothing overlaps
        *out_count = 0;
        return RP_OK;
    }
    {
        int rg = ensure_grid(h);  // an upload defers the grid
        if (rg) return rg;
    }
    RP_CUDA(h, cudaMemsetAsync(h->count_out, 0, sizeof(unsigned long long), h->stream));
    RP_CUDA(h, cudaMemsetAsync(h->flag, 0, sizeof(int), h->stream));
    // polyspherocylinders: the FP64 segment tests of the recount go to a second, lane-dense
    // kernel (polyspheres' centre tests are cheap enough inline)
    const bool defer = h->ncen > 0 && h->segs;
    if (defer) {
        if (!h->cq_buf) {
            RP_CUDA(h, cudaMalloc(&h->cq_buf, sizeof(DeferredPair) * Handle::CQ_CAP));
            RP_CUDA(h, cudaMalloc(&h->cq_count, sizeof(int)));
        }
        RP_CUDA(h, cudaMemsetAsync(h->cq_count, 0, sizeof(int), h->stream));
    }
    DevState s = dev_state(h);
    if (defer) {
        s.cq_buf = h->cq_buf;
        s.cq_count = h->cq_count;
        s.cq_cap = Handle::CQ_CAP;
    }
    if (h->shape.kind == RP_SHAPE_CONVEX) {
        // generic convex bodies: every pair in FP64 over the images within reach
        SingleArgs a = single_args(h);
        Group grp(h, RP_KERNEL_COUNT, 1);
        RP_CUDA(h, launch_count_fp64(a, early_exit ? 1 : 0, h->count_out, h->flag, h->stream));
    } else {
        Group grp(h, RP_KERNEL_COUNT, defer ? 2 : 1);
        RP_CUDA(h, launch_count(s, h->grid[h->gcur].d, early_exit ? 1 : 0, h->count_out, h->flag, h->stream));
    }
    unsigned long long c = 0;
    RP_CUDA(h, cudaMemcpyAsync(&c, h->count_out, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    *out_count = early_exit ? (c > 0 ? 1 : 0) : static_cast<int64_t>(c);
    return check_status(h);
}

static int fill_info(Handle *h, rp_grid_info *info) {
    const GridDev &g = h->grid[h->gcur].d;
    int32_t mo = 0;
    RP_CUDA(h, cudaMemcpyAsync(&mo, g.max_occ, sizeof(mo), cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    double hgt[3];
    heights_of(h->box, hgt);
    for (int d = 0; d < 3; d++) {
        info->dims[d] = g.dims[d];
        info->shift[d] = g.shift[d];
        info->cell_height[d] = hgt[d] / g.dims[d];
    }
    info->max_occupancy = mo;
    info->num_cells = g.ncell;
    return RP_OK;
}

int rp_set_grid(void *handle, const double *shift3, rp_grid_info *info) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !shift3) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    for (int d = 0; d < 3; d++)
        if (!(shift3[d] >= 0 && shift3[d] < 1)) return fail(h, RP_ERR_ARG, "grid shift outside [0, 1)");
    RP_CUDA(h, cudaSetDevice(h->device));
    int rc = setup_grid(h, h->grid[h->gcur], h->box, shift3);
    if (rc) return rc;
    rc = rebuild(h, h->gcur, h->pcur);
    if (rc) return rc;
    h->grid_stale = false;
    h->stale_unshifted = false;
    h->can_revert = false;
    if (info) {
        rc = fill_info(h, info);
        if (rc) return rc;
    }
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    return RP_OK;
}

int rp_get_grid(void *handle, rp_grid_info *info, int32_t *cell_of_particle, double *bounds) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    RP_CUDA(h, cudaSetDevice(h->device));
    {
        int rg = ensure_grid(h);  // an upload defers the grid
        if (rg) return rg;
    }
    const GridDev &g = h->grid[h->gcur].d;
    if (info) {
        int rc = fill_info(h, info);
        if (rc) return rc;
    }
    if (cell_of_particle)
        RP_CUDA(h, cudaMemcpyAsync(cell_of_particle, g.pid_cell, sizeof(int32_t) * h->n, cudaMemcpyDeviceToHost,
                                   h->stream));
    if (bounds) {
        int64_t nb = 2ll * (g.dims[0] + g.dims[1] + g.dims[2]);
        std::vector<double> b(nb);
        RP_CUDA(h, cudaMemcpyAsync(b.data(), g.bounds, sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
        for (int64_t cell = 0; cell < g.ncell; cell++) {
            int c[3] = {static_cast<int>(cell % g.dims[0]), static_cast<int>((cell / g.dims[0]) % g.dims[1]),
                        static_cast<int>(cell / (static_cast<int64_t>(g.dims[0]) * g.dims[1]))};
            for (int d = 0; d < 3; d++) {
                bounds[6 * cell + d] = b[g.boundsoff[d] + 2 * c[d]];
                bounds[6 * cell + 3 + d] = b[g.boundsoff[d] + 2 * c[d] + 1];
            }
        }
    }
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    return RP_OK;
}

int rp_run_moves(void *handle, const rp_move *moves, int64_t n, uint8_t *out_codes) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || (!moves && n > 0)) return fail(h, RP_ERR_ARG, "null argument");
    if (h->soft || h->shape.kind == RP_SHAPE_CONVEX)
        return fail(h, RP_ERR_UNSUPPORTED, "move lists with a soft part or a convex body (use rp_try_move or rp_sweep)");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    if (n <= 0) return RP_OK;
    if (n > (1ll << 31) - 1) return fail(h, RP_ERR_ARG, "too many moves");
    RP_CUDA(h, cudaSetDevice(h->device));
    h->try_valid = false;
    {
        int rg = ensure_grid(h);  // an upload defers the grid
        if (rg) return rg;
    }
    const GridDev &g = h->grid[h->gcur].d;
    // validation and phase blocks (runs of equal checkerboard colour)
    std::vector<int> phase(n);
    for (int64_t i = 0; i < n; i++) {
        const rp_move &m = moves[i];
        if (m.domain < 0 || m.domain >= g.ncell) return fail(h, RP_ERR_ARG, "move names a cell outside the grid");
        if (m.particle < 0 || m.particle >= h->n) return fail(h, RP_ERR_ARG, "move names an unknown particle");
        if (m.type < 0 || m.type > 2) return fail(h, RP_ERR_ARG, "unknown move type");
        phase_bits(g, m.domain, phase[i]);
    }
    RP_CUDA(h, ensure(h->d_moves, h->moves_alloc, n));
    RP_CUDA(h, ensure(h->d_codes, h->codes_alloc, n));
    RP_CUDA(h, cudaMemcpyAsync(h->d_moves, moves, sizeof(rp_move) * n, cudaMemcpyHostToDevice, h->stream));
    // per block: cells, begin offsets, move order
    std::vector<int32_t> packed;
    struct Block {
        int64_t cells_off, begin_off, out_off;
        int ncells;
    };
    std::vector<Block> blocks;
    std::vector<int32_t> cell_count(g.ncell, 0), cell_pos(g.ncell, -1);
    int64_t i = 0;
    while (i < n) {
        int64_t j = i;
        while (j < n && phase[j] == phase[i]) j++;
        // stable grouping by cell, cells in order of first appearance
        std::vector<int32_t> cells;
        for (int64_t k = i; k < j; k++) {
            int c = moves[k].domain;
            if (cell_count[c]++ == 0) cells.push_back(c);
        }
        Block b{};
        b.ncells = static_cast<int>(cells.size());
        b.cells_off = static_cast<int64_t>(packed.size());
        packed.insert(packed.end(), cells.begin(), cells.end());
        b.begin_off = static_cast<int64_t>(packed.size());
        int32_t run = 0;
        for (int32_t c : cells) {
            packed.push_back(run);
            cell_pos[c] = run;
            run += cell_count[c];
        }
        packed.push_back(run);
        b.out_off = static_cast<int64_t>(packed.size());
        packed.resize(packed.size() + (j - i));
        for (int64_t k = i; k < j; k++) {
            int c = moves[k].domain;
            packed[b.out_off + cell_pos[c]++] = static_cast<int32_t>(k);
        }
        for (int32_t c : cells) {
            cell_count[c] = 0;
            cell_pos[c] = -1;
        }
        blocks.push_back(b);
        i = j;
    }
    RP_CUDA(h, ensure(h->d_list, h->list_alloc, static_cast<int64_t>(packed.size())));
    RP_CUDA(h, cudaMemcpyAsync(h->d_list, packed.data(), sizeof(int32_t) * packed.size(), cudaMemcpyHostToDevice,
                               h->stream));
    for (const Block &b : blocks) {
        SweepArgs a = base_args(h);
        a.moves = h->d_moves;
        a.list_cells = h->d_list + b.cells_off;
        a.list_begin = h->d_list + b.begin_off;
        a.move_out = h->d_list + b.out_off;
        a.num_list = b.ncells;
        a.codes = h->d_codes;
        a.types = 3;
        {
            Group grp(h, RP_KERNEL_SWEEP, 1);
            RP_CUDA(h, launch_sweep(a, true, b.ncells, h->stream));
        }
        int rc = run_overflow(h, a, true);
        if (rc) return rc;
    }
    if (out_codes)
        RP_CUDA(h, cudaMemcpyAsync(out_codes, h->d_codes, n, cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    h->can_revert = false;
    h->log_valid = false;
    return check_status(h);
}

int rp_sweep(void *handle, const rp_sweep_params *p, rp_sweep_stats *stats) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !p) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    int types = (p->translation_step > 0 ? 1 : 0) | (p->rotation_step > 0 ? 2 : 0);
    if (!types) return fail(h, RP_ERR_ARG, "no move type enabled");
    if (p->flags & RP_SWEEP_ROTOTRANSLATION) {
        if (types != 3) return fail(h, RP_ERR_ARG, "rototranslations need a translation and a rotation step");
        types = SWEEP_ROTOTRANSLATION;
    }
    RP_CUDA(h, cudaSetDevice(h->device));
    h->try_valid = false;
    // random grid origin and phase order from the Philox stream of this sweep
    u4 r = philox(u4{0x5eedu, 0x9e37u, static_cast<uint32_t>(p->counter), static_cast<uint32_t>(p->counter >> 32)},
                  static_cast<uint32_t>(p->seed), static_cast<uint32_t>(p->seed >> 32));
    double shift[3] = {(r.a >> 8) * (1.0 / 16777216.0), (r.b >> 8) * (1.0 / 16777216.0),
                       (r.c >> 8) * (1.0 / 16777216.0)};
    int rc = setup_grid(h, h->grid[h->gcur], h->box, shift);
    if (rc) return rc;
    rc = rebuild(h, h->gcur, h->pcur);
    if (rc) return rc;
    h->grid_stale = false;
    h->stale_unshifted = false;
    const GridDev &g = h->grid[h->gcur].d;
    // translation step limited to half the smallest box height (TranslationSampler.cpp:39-46)
    double hgt[3];
    heights_of(h->box, hgt);
    double tstep = std::min(p->translation_step, std::min({hgt[0], hgt[1], hgt[2]}) / 2);
    std::vector<int> phases;
    grid_phases(g, r.d, phases);
    int ntypes = sweep_move_types(types);
    bool log = (p->flags & RP_SWEEP_LOG) != 0;
    if (log) {
        int64_t before = h->log_alloc;
        RP_CUDA(h, ensure(h->d_log, h->log_alloc, ntypes * h->n));
        if (!h->d_log_codes || h->log_alloc != before) {
            cudaFree(h->d_log_codes);
            h->d_log_codes = nullptr;
            RP_CUDA(h, cudaMalloc(&h->d_log_codes, h->log_alloc));
        }
    }
    if (stats) RP_CUDA(h, cudaMemsetAsync(h->counters, 0, sizeof(unsigned long long) * NUM_COUNTERS, h->stream));
    RP_CUDA(h, cudaMemsetAsync(h->item_counters, 0, sizeof(int32_t) * 64, h->stream));
    if (types & (2 | SWEEP_ROTOTRANSLATION)) {
        Group grp(h, RP_KERNEL_SWEEP, 1);
        RP_CUDA(h, launch_rot_table(h->rtab64, h->rtab32, ROT_TABLE, p->seed, p->counter,
                                    static_cast<float>(p->rotation_step), h->stream));
    }
    if (h->order_mode != RP_ORDER_OFF && (!h->partners_valid || h->since_rank >= h->order_every)) {
        int rc2 = rank_partners(h);
        if (rc2) return rc2;
    }
    h->since_rank++;
    const bool fp64_sweep = h->soft || h->shape.kind == RP_SHAPE_CONVEX;
    if (fp64_sweep) {
        // a soft part or a generic convex body: every move decided in FP64 (hard part, then the
        // energy change with the Metropolis test at the handle's temperature), one warp per
        // active cell
        if (types == SWEEP_ROTOTRANSLATION)
            return fail(h, RP_ERR_UNSUPPORTED, "rototranslations with a soft part or a convex body");
        SoftSweepArgs sa{};
        sa.c.s = dev_state(h);
        sa.c.g = g;
        sa.c.temperature = h->temperature;
        set_prefilter(sa.c, h);
        sa.seed = p->seed;
        sa.counter = p->counter;
        sa.tstep = static_cast<float>(tstep);
        sa.types = types;
        sa.rtab64 = h->rtab64;
        sa.rtab_mask = ROT_TABLE - 1;
        if (log) {
            sa.log = h->d_log;
            sa.log_codes = h->d_log_codes;
        }
        int soft_phase = 0;
        int soft_start[27] = {0};
        const bool soft_ordered = h->cell_order && g.order;
        if (soft_ordered) order_starts(g, soft_start);
        for (int ph : phases) {
            int act[3];
            sa.num_active = phase_cells(g, ph, act);
            for (int d = 0; d < 3; d++) {
                sa.phase[d] = phase_digit(ph, d);
                sa.active[d] = act[d];
            }
            sa.work = soft_ordered ? g.order + soft_start[ph] : nullptr;
            sa.next_item = h->item_counters + soft_phase++;
            Group grp(h, RP_KERNEL_SWEEP, 1);
            RP_CUDA(h, launch_soft_sweep(sa, std::min(sa.num_active, h->num_sms * 16), h->stream));
        }
        // the FP32 mirror no longer follows the moved particles
        h->grid_stale = true;
        h->grid_patched = false;
    }
    int phase_no = 0;
    int order_start[27] = {0};
    const bool ordered = h->cell_order && !fp64_sweep && g.order;
    if (ordered) order_starts(g, order_start);
    for (int ph : (fp64_sweep ? std::vector<int>{} : phases)) {
        SweepArgs a = base_args(h);
        if (h->order_mode != RP_ORDER_OFF) a.partners = h->partners;
        if (h->pair_cap > 0) {
            a.pair_feats = h->pair_feats;
            a.pair_labels = h->pair_labels;
            a.pair_count = h->pair_count;
            a.pair_cap = static_cast<unsigned long long>(h->pair_cap);
            a.pair_every = h->pair_every;
        }
        a.inv_range = static_cast<float>(1.0 / h->range);
        a.next_item = h->item_counters + phase_no++;
        int act[3];
        a.num_active = phase_cells(g, ph, act);
        for (int d = 0; d < 3; d++) {
            a.phase[d] = phase_digit(ph, d);
            a.active[d] = act[d];
        }
        if (ordered) {
            a.work = g.order + order_start[ph];
            a.work_count = nullptr;
            a.num_work = a.num_active;
        }
        a.seed = p->seed;
        a.counter = p->counter;
        a.tstep = static_cast<float>(tstep);
        a.rstep = static_cast<float>(p->rotation_step);
        a.types = types;
        a.rtab64 = h->rtab64;
        a.rtab32 = h->rtab32;
        a.rtab_mask = ROT_TABLE - 1;
        if (p->flags & RP_SWEEP_FP64_ONLY) a.fp64_only = 1;
        if (log) {
            a.log = h->d_log;
            a.log_codes = h->d_log_codes;
        }
        // two cells per warp for the plain scans of spheres and spherocylinders
        const GridHost &gh = h->grid[h->gcur];
        const bool half = h->cells_per_warp == 2 && gh.cap_half > 0 && !h->counting && types != SWEEP_ROTOTRANSLATION &&
                          a.partners == nullptr && a.pair_every == 0;
        if (half && h->half_cap_cached != gh.cap_half) {
            h->half_blocks = sweep_half_blocks_per_sm(h->shape.kind, gh.cap_half);
            h->half_cap_cached = gh.cap_half;
        }
        {
            Group grp(h, RP_KERNEL_SWEEP, 1);
            h->last_cells_per_warp = (half && h->half_blocks > 0) ? 2 : 1;
            if (half && h->half_blocks > 0) {
                a.cap = gh.cap_half;
                const int resident = h->num_sms * h->half_blocks * SWEEP_WARPS * 2;
                RP_CUDA(h, launch_sweep_half(a, std::min(a.num_active, resident), h->stream));
                a.cap = gh.cap;
            } else {
                int resident = h->num_sms * SWEEP_WARPS * SWEEP_MIN_BLOCKS;
                RP_CUDA(h, launch_sweep(a, false, std::min(a.num_active, resident), h->stream));
            }
        }
        a.next_item = nullptr;
        rc = run_overflow(h, a, false);
        if (rc) return rc;
    }
    if (log) {
        h->log_valid = true;
        h->log_types = ntypes;
        h->log_phases = phases;
        for (int d = 0; d < 3; d++) h->log_dims[d] = g.dims[d];
        h->log_start.resize(g.ncell + 1);
        RP_CUDA(h, cudaMemcpyAsync(h->log_start.data(), g.start, sizeof(int32_t) * (g.ncell + 1),
                                   cudaMemcpyDeviceToHost, h->stream));
    }
    if (stats) {
        unsigned long long c[NUM_COUNTERS];
        RP_CUDA(h, cudaMemcpyAsync(c, h->counters, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
        stats->moves = c[0];
        stats->accepted = c[1];
        stats->rejected_overlap = c[2];
        stats->rejected_domain = c[3];
        stats->pair_tests = c[4];
        stats->fp64_pairs = c[5];
        stats->translations = c[6];
        stats->rotations = c[7];
        stats->accepted_translations = c[8];
        stats->kernel_launches = h->launches;
    }
    h->can_revert = false;
    if (stats || log) return check_status(h);
    return RP_OK;
}

int rp_sweep_log(void *handle, rp_move *moves, uint8_t *codes, int64_t capacity, int64_t *count) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !count) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->log_valid) return fail(h, RP_ERR_STATE, "no logged sweep");
    int64_t total = h->log_types * h->n;
    *count = total;
    if (!moves && !codes) return RP_OK;
    if (capacity < total) return fail(h, RP_ERR_ARG, "capacity too small");
    RP_CUDA(h, cudaSetDevice(h->device));
    std::vector<rp_move> raw(total);
    std::vector<uint8_t> rc(total);
    RP_CUDA(h, cudaMemcpyAsync(raw.data(), h->d_log, sizeof(rp_move) * total, cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaMemcpyAsync(rc.data(), h->d_log_codes, total, cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    const int *dims = h->log_dims;
    int64_t ncell = static_cast<int64_t>(dims[0]) * dims[1] * dims[2];
    int64_t o = 0;
    for (int ph : h->log_phases) {
        for (int64_t cell = 0; cell < ncell; cell++) {
            int cx = static_cast<int>(cell % dims[0]), cy = static_cast<int>((cell / dims[0]) % dims[1]),
                cz = static_cast<int>(cell / (static_cast<int64_t>(dims[0]) * dims[1]));
            int cp = ring_colour(dims[0], cx) + 3 * ring_colour(dims[1], cy) + 9 * ring_colour(dims[2], cz);
            if (cp != ph) continue;
            int64_t b = static_cast<int64_t>(h->log_types) * h->log_start[cell];
            int64_t e = static_cast<int64_t>(h->log_types) * h->log_start[cell + 1];
            for (int64_t k = b; k < e; k++) {
                if (moves) moves[o] = raw[k];
                if (codes) codes[o] = rc[k];
                o++;
            }
        }
    }
    return RP_OK;
}

// Packing::getTotalEnergy (core/Packing.cpp:689-764) of the current state on the device
// (each pair once, a fixed summation order); the grid is rebuilt first if out of date.
static int soft_total_energy(Handle *h, double *out) {
    *out = 0.0;
    if (!h->soft) return RP_OK;
    int rg = ensure_grid(h);
    if (rg) return rg;
    if (!h->d_energy) RP_CUDA(h, cudaMalloc(&h->d_energy, sizeof(double) * (h->n + 1)));
    SingleArgs a{};
    a.s = dev_state(h);
    a.g = h->grid[h->gcur].d;
    set_prefilter(a, h);
    {
        Group grp(h, RP_KERNEL_COUNT, 2);
        RP_CUDA(h, launch_total_energy(a, h->d_energy, h->d_energy + h->n, h->stream));
    }
    RP_CUDA(h, cudaMemcpyAsync(out, h->d_energy + h->n, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    return check_status(h);
}

int rp_total_energy(void *handle, double *energy) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !energy) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    RP_CUDA(h, cudaSetDevice(h->device));
    return soft_total_energy(h, energy);
}

int rp_try_scaling(void *handle, const double *new_box9, double *dE) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !new_box9 || !dE) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    if (det3(new_box9) == 0 || volume_of(new_box9) == 0) return fail(h, RP_ERR_ARG, "box volume is zero");
    RP_CUDA(h, cudaSetDevice(h->device));
    h->try_valid = false;
    {
        int rg = ensure_grid(h);  // an upload defers the grid
        if (rg) return rg;
    }
    // a soft part: the total energy before the rescale (core/Packing.cpp:178)
    double e0 = 0.0;
    if (h->soft) {
        int re = soft_total_energy(h, &e0);
        if (re) return re;
    }
    int np = 1 - h->pcur, ng = 1 - h->gcur;
    double new_inv[9];
    inverse3(new_box9, new_inv);
    {
        Group grp(h, RP_KERNEL_RESCALE, 1);
        RP_CUDA(h, launch_rescale(h->pos64[h->pcur], h->pos64[np], h->n, h->inv, new_box9, h->stream));
    }
    double tt[375];
    translation_table(new_box9, tt);
    RP_CUDA(h, cudaMemcpyAsync(h->trans[np], tt, sizeof(tt), cudaMemcpyHostToDevice, h->stream));
    // switch to the new state; the old one stays in the other buffers for revert
    std::memcpy(h->saved_box, h->box, sizeof(h->box));
    std::memcpy(h->saved_inv, h->inv, sizeof(h->inv));
    std::memcpy(h->box, new_box9, sizeof(h->box));
    std::memcpy(h->inv, new_inv, sizeof(h->inv));
    int old_p = h->pcur, old_g = h->gcur;
    h->pcur = np;
    h->gcur = ng;
    double shift[3] = {h->grid[old_g].d.shift[0], h->grid[old_g].d.shift[1], h->grid[old_g].d.shift[2]};
    int rc = setup_grid(h, h->grid[ng], h->box, shift);
    if (rc == RP_OK) rc = remap_or_rebuild(h, old_g, ng, np);
    if (rc == RP_OK && h->ncen > 0) {
        // Packing::tryScaling recalculates the absolute centres (core/Packing.cpp:186-187)
        Group grp(h, RP_KERNEL_RESCALE, 1);
        cudaError_t e = launch_abs_centres(dev_state(h), h->stream);
        if (e != cudaSuccess) rc = fail(h, RP_ERR_CUDA, cudaGetErrorString(e));
    }
    if (rc) {
        std::memcpy(h->box, h->saved_box, sizeof(h->box));
        std::memcpy(h->inv, h->saved_inv, sizeof(h->inv));
        h->pcur = old_p;
        h->gcur = old_g;
        return rc;
    }
    h->can_revert = true;
    h->log_valid = false;
    // the soft part's energy change, added where the hard part allows the move
    // (core/Packing.cpp:205-206)
    auto soft_change = [&](double *out) -> int {
        if (!h->soft || std::isinf(*out)) return RP_OK;
        double e1 = 0.0;
        int re = soft_total_energy(h, &e1);
        if (re) return re;
        *out = e1 - e0;
        return RP_OK;
    };
    if (h->soft_only) {
        *dE = 0;
        return soft_change(dE);
    }
    if (h->counting) {
        // counting mode: the full recount against the count before the move (core/Packing.cpp:189-196)
        RP_CUDA(h, cudaMemcpyAsync(&h->saved_overlaps, h->d_overlaps, sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, h->stream));
        int64_t cnt = 0;
        rc = rp_count_overlaps(h, 0, &cnt);
        if (rc) return rc;
        unsigned long long c = static_cast<unsigned long long>(cnt);
        RP_CUDA(h, cudaMemcpyAsync(h->d_overlaps, &c, sizeof(c), cudaMemcpyHostToDevice, h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
        const long long delta = cnt - static_cast<long long>(h->saved_overlaps);
        *dE = delta < 0 ? -std::numeric_limits<double>::infinity()
                        : (delta > 0 ? std::numeric_limits<double>::infinity() : 0.0);
        return soft_change(dE);
    }
    // A convex shape in a box that only grew cannot overlap (core/Packing.cpp:199-200);
    // polyspheres are not convex (PolysphereTraits.h:133).
    if (h->shape.kind != RP_SHAPE_POLYSPHERE && box_upscaled(h->saved_box, h->box)) {
        *dE = 0;
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
        return soft_change(dE);
    }
    int64_t cnt = 0;
    rc = rp_count_overlaps(h, 1, &cnt);
    if (rc) return rc;
    *dE = cnt > 0 ? std::numeric_limits<double>::infinity() : 0.0;
    return soft_change(dE);
}

int rp_revert_scaling(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    if (!h->can_revert) return fail(h, RP_ERR_STATE, "nothing to revert");
    h->try_valid = false;
    std::memcpy(h->box, h->saved_box, sizeof(h->box));
    std::memcpy(h->inv, h->saved_inv, sizeof(h->inv));
    h->pcur = 1 - h->pcur;
    h->gcur = 1 - h->gcur;
    h->can_revert = false;
    h->log_valid = false;
    if (h->counting) {
        RP_CUDA(h, cudaMemcpyAsync(h->d_overlaps, &h->saved_overlaps, sizeof(unsigned long long), cudaMemcpyHostToDevice,
                                   h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return RP_OK;
}

// Packing::tryTranslation / tryRotation / tryMove without an ActiveDomain (core/Packing.cpp:84-164).
int rp_try_move(void *handle, const rp_move *move, const double *domain6, double *dE) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !move || !dE) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    if (h->batch_member) return fail(h, RP_ERR_UNSUPPORTED, "single moves on a batch replica");
    if (move->type < RP_MOVE_TRANSLATION || move->type > RP_MOVE_ROTOTRANSLATION)
        return fail(h, RP_ERR_ARG, "unknown move type");
    if (move->particle < 0 || move->particle >= h->n) return fail(h, RP_ERR_ARG, "particle index out of range");
    RP_CUDA(h, cudaSetDevice(h->device));
    h->try_valid = false;
    if (!h->d_try) {
        RP_CUDA(h, cudaMalloc(&h->d_try, sizeof(SingleTry)));
        RP_CUDA(h, cudaMalloc(&h->d_disp_list, sizeof(int32_t) * Handle::DISP_CAP));
        RP_CUDA(h, cudaMalloc(&h->d_disp_flag, static_cast<size_t>(h->n)));
        RP_CUDA(h, cudaMemsetAsync(h->d_disp_flag, 0, static_cast<size_t>(h->n), h->stream));
        h->disp_flag_host.assign(static_cast<size_t>(h->n), 0);
        h->disp_host.clear();
    }
    // the grid serves single moves while only particles moved by single moves are out of
    // place (and few enough of them); otherwise it is rebuilt first
    if (h->grid_stale && !(h->grid_patched && static_cast<int>(h->disp_host.size()) < Handle::DISP_CAP)) {
        h->grid_patched = false;
        int rg = ensure_grid(h);
        if (rg) return rg;
    }
    SingleArgs a{};
    a.s = dev_state(h);
    a.g = h->grid[h->gcur].d;
    a.m = *move;
    a.out = h->d_try;
    a.disp_list = h->d_disp_list;
    a.disp_flag = h->d_disp_flag;
    a.ndisp = static_cast<int>(h->disp_host.size());
    set_prefilter(a, h);
    if (domain6) {
        a.has_domain = 1;
        for (int d = 0; d < 3; d++) {
            a.dom_lo[d] = domain6[d];
            a.dom_hi[d] = domain6[3 + d];
        }
    }
    {
        Group grp(h, RP_KERNEL_SINGLE, 1);
        RP_CUDA(h, launch_try_single(a, h->stream));
    }
    double e = 0;
    RP_CUDA(h, cudaMemcpyAsync(&e, &h->d_try->dE, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    int rc = check_status(h);  // synchronises
    if (rc) return rc;
    *dE = e;
    h->try_valid = true;
    h->try_particle = move->particle;
    return RP_OK;
}

// Packing::acceptTranslation / acceptRotation / acceptMove (core/Packing.cpp:234-302).
int rp_accept_move(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    if (!h->try_valid) return fail(h, RP_ERR_STATE, "no tried move to accept");
    RP_CUDA(h, cudaSetDevice(h->device));
    const int32_t pid = h->try_particle;
    int slot = -1;
    if (!h->disp_flag_host[pid]) {
        slot = static_cast<int>(h->disp_host.size());
        h->disp_host.push_back(pid);
        h->disp_flag_host[pid] = 1;
    }
    {
        Group grp(h, RP_KERNEL_SINGLE, 1);
        RP_CUDA(h, launch_commit_single(dev_state(h), h->d_try, h->d_disp_flag, h->d_disp_list, slot, h->stream));
    }
    h->try_valid = false;
    // the sweeps, recounts and box moves rebuild the grid (and the FP32 mirror) first
    h->grid_stale = true;
    h->grid_patched = true;
    h->log_valid = false;
    h->can_revert = false;
    return RP_OK;
}

int rp_get_stats(void *handle, rp_sweep_stats *stats) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !stats) return RP_ERR_ARG;
    RP_CUDA(h, cudaSetDevice(h->device));
    unsigned long long c[NUM_COUNTERS];
    RP_CUDA(h, cudaMemcpyAsync(c, h->counters, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    stats->moves = c[0];
    stats->accepted = c[1];
    stats->rejected_overlap = c[2];
    stats->rejected_domain = c[3];
    stats->pair_tests = c[4];
    stats->fp64_pairs = c[5];
    stats->translations = c[6];
    stats->rotations = c[7];
    stats->accepted_translations = c[8];
    stats->kernel_launches = h->launches;
    return RP_OK;
}

int rp_get_stream(void *handle, void **stream) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !stream) return RP_ERR_ARG;
    *stream = static_cast<void *>(h->stream);
    return RP_OK;
}

int rp_set_timing(void *handle, int on) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    RP_CUDA(h, cudaSetDevice(h->device));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    h->tm.reset(on != 0);
    return RP_OK;
}

int rp_get_timing(void *handle, double *ms, uint64_t *groups) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    RP_CUDA(h, cudaSetDevice(h->device));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    RP_CUDA(h, h->tm.collect(ms, groups));
    return RP_OK;
}

// ---- observables ----------------------------------------------------------------------

// NematicOrder::calculateEigenvalues (core/observables/NematicOrder.cpp:29-56), the Cardano
// formula of arXiv:1306.6291; a multiple of the identity has the triple eigenvalue b / 3.
static void q_eigenvalues(const double *q, double ev[3]) {
    double A11 = q[0], A12 = q[1], A13 = q[2], A22 = q[4], A23 = q[5], A33 = q[8];
    double b = A11 + A22 + A33;
    double c = A11 * A22 + A11 * A33 + A22 * A33 - A12 * A12 - A13 * A13 - A23 * A23;
    double d = A11 * A23 * A23 + A22 * A13 * A13 + A33 * A12 * A12 - A11 * A22 * A33 - 2 * A12 * A13 * A23;
    double p = b * b - 3 * c;
    if (!(p > 0)) {
        ev[0] = ev[1] = ev[2] = b / 3;
        return;
    }
    double sp = std::sqrt(p);
    double qq = 2 * b * b * b - 9 * b * c - 27 * d;
    double ratio = qq / 2 / (sp * sp * sp);
    if (std::abs(ratio) > 1) ratio = ratio < 0 ? -1 : 1;
    double delta = std::acos(ratio);
    ev[0] = 1. / 3 * (b + 2 * sp * std::cos(delta / 3));
    ev[1] = 1. / 3 * (b + 2 * sp * std::cos((delta + 2 * M_PI) / 3));
    ev[2] = 1. / 3 * (b + 2 * sp * std::cos((delta - 2 * M_PI) / 3));
}

int rp_nematic_order(void *handle, double *q9, double *p2) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !p2) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    if (h->shape.kind == RP_SHAPE_SPHERE) return fail(h, RP_ERR_UNSUPPORTED, "spheres have no primary axis");
    RP_CUDA(h, cudaSetDevice(h->device));
    const int nb = axis_moment_blocks(h->n);
    double *partial = nullptr;
    RP_CUDA(h, cudaMalloc(&partial, sizeof(double) * 6 * nb));
    std::vector<double> host(6 * nb);
    cudaError_t e = launch_axis_moments(h->rot64, h->n, partial, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host.data(), partial, sizeof(double) * 6 * nb, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(partial);
    RP_CUDA(h, e);
    h->launches += 1;
    double m[6] = {0, 0, 0, 0, 0, 0};
    for (int b = 0; b < nb; b++)
        for (int k = 0; k < 6; k++) m[k] += host[6 * b + k];
    const double S[9] = {m[0], m[1], m[2], m[1], m[3], m[4], m[2], m[4], m[5]};
    double q[9];
    const double n = static_cast<double>(h->n);
    for (int i = 0; i < 9; i++) {
        double s = S[i] / n;                               // QTensor /= size()
        double t = 3. * s - ((i % 4 == 0) ? 1.0 : 0.0);    // 3 Q - I
        q[i] = 0.5 * t;
    }
    double ev[3];
    q_eigenvalues(q, ev);
    double best = ev[0];
    for (int k = 1; k < 3; k++)
        if (std::abs(best) < std::abs(ev[k])) best = ev[k];
    *p2 = best;
    if (q9) std::memcpy(q9, q, sizeof(q));
    return RP_OK;
}

// ---- overlap counting ---------------------------------------------------------------------

int rp_set_counting(void *handle, int on) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    RP_CUDA(h, cudaSetDevice(h->device));
    h->try_valid = false;
    {
        int rg = ensure_grid(h);  // an upload defers the grid
        if (rg) return rg;
    }
    h->counting = on != 0;
    h->can_revert = false;
    if (h->counting) {
        // Packing::toggleOverlapCounting: the cached count starts from a full recount
        int64_t cnt = 0;
        int rc = rp_count_overlaps(h, 0, &cnt);
        if (rc) return rc;
        unsigned long long c = static_cast<unsigned long long>(cnt);
        RP_CUDA(h, cudaMemcpyAsync(h->d_overlaps, &c, sizeof(c), cudaMemcpyHostToDevice, h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return RP_OK;
}

int rp_cached_overlaps(void *handle, int64_t *count) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !count) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->counting) return fail(h, RP_ERR_STATE, "overlap counting is off");
    RP_CUDA(h, cudaSetDevice(h->device));
    unsigned long long c = 0;
    RP_CUDA(h, cudaMemcpyAsync(&c, h->d_overlaps, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    *count = static_cast<int64_t>(c);
    return RP_OK;
}

// ---- orientation renormalisation ----------------------------------------------------

int rp_renormalize_orientations(void *handle, int allow_overlaps, int64_t *rejected) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !rejected) return fail(h, RP_ERR_ARG, "null argument");
    if (!h->has_state) return fail(h, RP_ERR_STATE, "no state uploaded");
    if (h->soft) return fail(h, RP_ERR_UNSUPPORTED, "orientation fixes with a soft part");
    RP_CUDA(h, cudaSetDevice(h->device));
    h->try_valid = false;
    {
        int rg = ensure_grid(h);  // an upload defers the grid
        if (rg) return rg;
    }
    *rejected = 0;
    h->can_revert = false;
    h->log_valid = false;
    h->partners_valid = false;
    if (allow_overlaps) {
        if (h->ncen > 0) {
            Group grp(h, RP_KERNEL_FIX, 2);
            RP_CUDA(h, launch_fresh_centres(dev_state(h), h->cbody_dev, h->stream));
            RP_CUDA(h, launch_abs_centres(dev_state(h), h->stream));
        }
        int rc = rebuild(h, h->gcur, h->pcur);
        if (rc) return rc;
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
        return RP_OK;
    }
    const int64_t n = h->n, nc = std::max(1, h->ncen);
    double *rotfix = nullptr, *cenfix = nullptr, *absfix = nullptr;
    uint8_t *rej = nullptr;
    unsigned long long *words = nullptr;  // [0] first rejected index, [1] serial rejections
    struct Scratch {
        std::vector<void *> p;
        ~Scratch() {
            for (void *q : p) cudaFree(q);
        }
    } scratch;
    auto alloc = [&](void **q, size_t bytes) {
        cudaError_t e = cudaMalloc(q, bytes);
        if (e == cudaSuccess) scratch.p.push_back(*q);
        return e;
    };
    RP_CUDA(h, alloc(reinterpret_cast<void **>(&rotfix), sizeof(double) * 9 * n));
    RP_CUDA(h, alloc(reinterpret_cast<void **>(&cenfix), sizeof(double) * 3 * n * nc));
    RP_CUDA(h, alloc(reinterpret_cast<void **>(&absfix), sizeof(double) * 3 * n * nc));
    RP_CUDA(h, alloc(reinterpret_cast<void **>(&rej), n));
    RP_CUDA(h, alloc(reinterpret_cast<void **>(&words), 2 * sizeof(unsigned long long)));
    unsigned long long init[2] = {static_cast<unsigned long long>(n), 0};
    RP_CUDA(h, cudaMemcpyAsync(words, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    const DevState s = dev_state(h);
    const GridDev &g = h->grid[h->gcur].d;
    {
        Group grp(h, RP_KERNEL_FIX, 2);
        RP_CUDA(h, launch_fix_prepare(s, h->cbody_dev, rotfix, cenfix, absfix, h->stream));
        RP_CUDA(h, launch_fix_check(s, g, rotfix, cenfix, absfix, rej, words, h->stream));
    }
    unsigned long long first = 0;
    RP_CUDA(h, cudaMemcpyAsync(&first, words, sizeof(first), cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    const int64_t from = static_cast<int64_t>(first);
    {
        Group grp(h, RP_KERNEL_FIX, from < n ? 2 : 1);
        RP_CUDA(h, launch_fix_commit(s, rotfix, cenfix, absfix, 0, from, h->stream));
        if (from < n) RP_CUDA(h, launch_fix_serial(s, g, rotfix, cenfix, absfix, from, words + 1, h->stream));
    }
    if (from < n) {
        unsigned long long nr = 0;
        RP_CUDA(h, cudaMemcpyAsync(&nr, words + 1, sizeof(nr), cudaMemcpyDeviceToHost, h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
        *rejected = static_cast<int64_t>(nr);
    }
    int rc = rebuild(h, h->gcur, h->pcur);  // FP32 mirrors of the new orientations and centres
    if (rc) return rc;
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    return RP_OK;
}

// ---- learned ordering ---------------------------------------------------------------

int rp_mlp_init(void *handle, uint64_t seed) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    RP_CUDA(h, cudaSetDevice(h->device));
    int rc = mlp_ready(h);
    if (rc) return rc;
    std::vector<float> w;
    mlp_init_host(seed, w);
    return mlp_upload(h, w.data());
}

int rp_mlp_set_params(void *handle, const float *params) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !params) return fail(h, RP_ERR_ARG, "null argument");
    RP_CUDA(h, cudaSetDevice(h->device));
    int rc = mlp_ready(h);
    if (rc) return rc;
    return mlp_upload(h, params);
}

int rp_mlp_get_params(void *handle, float *params) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !params) return fail(h, RP_ERR_ARG, "null argument");
    RP_CUDA(h, cudaSetDevice(h->device));
    int rc = mlp_ready(h);
    if (rc) return rc;
    RP_CUDA(h, cudaMemcpyAsync(params, h->mlp_w32, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    return RP_OK;
}

int rp_mlp_predict(void *handle, const float *feats, int64_t n, float *logits) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || (n > 0 && (!feats || !logits)) || n < 0) return fail(h, RP_ERR_ARG, "bad argument");
    if (n > (int64_t{1} << 30)) return fail(h, RP_ERR_ARG, "too many pairs");
    if (n == 0) return RP_OK;
    RP_CUDA(h, cudaSetDevice(h->device));
    int rc = mlp_ready(h);
    if (rc) return rc;
    RP_CUDA(h, ensure(h->mlp_feats, h->mlp_feats_alloc, n * MLP_IN));
    RP_CUDA(h, ensure(h->mlp_out, h->mlp_out_alloc, n));
    RP_CUDA(h, cudaMemcpyAsync(h->mlp_feats, feats, sizeof(float) * MLP_IN * n, cudaMemcpyHostToDevice, h->stream));
    {
        Group grp(h, RP_KERNEL_MLP, 1);
        RP_CUDA(h, launch_mlp_predict(h->mlp_feats, static_cast<int>(n), h->mlp_w32, h->mlp_w16, h->mlp_out, h->stream));
    }
    RP_CUDA(h, cudaMemcpyAsync(logits, h->mlp_out, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    return RP_OK;
}

int rp_mlp_gradient(void *handle, const float *feats, const uint8_t *labels, int64_t n, float *grad, float *loss) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !feats || !labels || !grad || n <= 0) return fail(h, RP_ERR_ARG, "bad argument");
    if (n > (int64_t{1} << 30)) return fail(h, RP_ERR_ARG, "too many pairs");
    RP_CUDA(h, cudaSetDevice(h->device));
    int rc = mlp_ready(h);
    if (rc) return rc;
    RP_CUDA(h, ensure(h->mlp_feats, h->mlp_feats_alloc, n * MLP_IN));
    RP_CUDA(h, ensure(h->mlp_labels, h->mlp_labels_alloc, n));
    RP_CUDA(h, cudaMemcpyAsync(h->mlp_feats, feats, sizeof(float) * MLP_IN * n, cudaMemcpyHostToDevice, h->stream));
    RP_CUDA(h, cudaMemcpyAsync(h->mlp_labels, labels, n, cudaMemcpyHostToDevice, h->stream));
    RP_CUDA(h, cudaMemsetAsync(h->mlp_grad, 0, sizeof(float) * MLP_NPARAM, h->stream));
    RP_CUDA(h, cudaMemsetAsync(h->mlp_loss, 0, sizeof(float), h->stream));
    {
        Group grp(h, RP_KERNEL_MLP, 1);
        RP_CUDA(h, launch_mlp_grad(h->mlp_feats, h->mlp_labels, n, 0, static_cast<int>(n), 1, 0, h->mlp_w32,
                                   h->mlp_grad, h->mlp_loss, h->num_sms, h->stream));
    }
    RP_CUDA(h, cudaMemcpyAsync(grad, h->mlp_grad, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, h->stream));
    float l = 0;
    RP_CUDA(h, cudaMemcpyAsync(&l, h->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    if (loss) *loss = l;
    return RP_OK;
}

int rp_pair_log_enable(void *handle, int64_t capacity, int32_t every) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || capacity < 0 || (capacity > 0 && every <= 0)) return fail(h, RP_ERR_ARG, "bad argument");
    if (capacity > 0 && h->shape.kind == RP_SHAPE_CONVEX)
        return fail(h, RP_ERR_UNSUPPORTED, "the pair log of convex bodies");
    RP_CUDA(h, cudaSetDevice(h->device));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->pair_feats);
    cudaFree(h->pair_labels);
    h->pair_feats = nullptr;
    h->pair_labels = nullptr;
    h->pair_cap = 0;
    h->pair_every = 0;
    if (capacity == 0) return RP_OK;
    if (!h->pair_count) RP_CUDA(h, cudaMalloc(&h->pair_count, sizeof(unsigned long long)));
    RP_CUDA(h, cudaMalloc(&h->pair_feats, sizeof(float) * MLP_IN * capacity));
    RP_CUDA(h, cudaMalloc(&h->pair_labels, capacity));
    RP_CUDA(h, cudaMemsetAsync(h->pair_count, 0, sizeof(unsigned long long), h->stream));
    h->pair_cap = capacity;
    h->pair_every = every;
    return RP_OK;
}

static int pair_log_held(Handle *h, int64_t *held) {
    unsigned long long c = 0;
    if (h->pair_count) {
        RP_CUDA(h, cudaMemcpyAsync(&c, h->pair_count, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    *held = std::min<int64_t>(static_cast<int64_t>(c), h->pair_cap);
    return RP_OK;
}

int rp_pair_log_read(void *handle, float *feats, uint8_t *labels, int64_t capacity, int64_t *count) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !count || capacity < 0) return fail(h, RP_ERR_ARG, "bad argument");
    RP_CUDA(h, cudaSetDevice(h->device));
    int64_t held = 0;
    int rc = pair_log_held(h, &held);
    if (rc) return rc;
    *count = held;
    int64_t k = std::min(held, capacity);
    if (k > 0 && feats)
        RP_CUDA(h, cudaMemcpyAsync(feats, h->pair_feats, sizeof(float) * MLP_IN * k, cudaMemcpyDeviceToHost, h->stream));
    if (k > 0 && labels) RP_CUDA(h, cudaMemcpyAsync(labels, h->pair_labels, k, cudaMemcpyDeviceToHost, h->stream));
    RP_CUDA(h, cudaStreamSynchronize(h->stream));
    return RP_OK;
}

int rp_pair_log_clear(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    RP_CUDA(h, cudaSetDevice(h->device));
    if (h->pair_count) RP_CUDA(h, cudaMemsetAsync(h->pair_count, 0, sizeof(unsigned long long), h->stream));
    return RP_OK;
}

int rp_mlp_train(void *handle, int32_t epochs, int32_t batch, float lr, uint64_t seed, float *loss) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || epochs < 0 || batch <= 0 || !(lr > 0)) return fail(h, RP_ERR_ARG, "bad argument");
    RP_CUDA(h, cudaSetDevice(h->device));
    int rc = mlp_ready(h);
    if (rc) return rc;
    int64_t held = 0;
    rc = pair_log_held(h, &held);
    if (rc) return rc;
    if (held == 0) return fail(h, RP_ERR_STATE, "the pair log is empty");
    const int64_t nb = (held + batch - 1) / batch;
    float last = 0;
    for (int ep = 0; ep < epochs; ep++) {
        // a multiplier coprime with the log size and an offset: a seeded permutation
        uint64_t x = seed * 0x9e3779b97f4a7c15ull + static_cast<uint64_t>(ep) * 0xbf58476d1ce4e5b9ull + 1;
        x ^= x >> 29;
        int64_t mul = static_cast<int64_t>(x % static_cast<uint64_t>(held)) | 1;
        auto gcd = [](int64_t a, int64_t b) {
            while (b) {
                int64_t t = a % b;
                a = b;
                b = t;
            }
            return a;
        };
        while (gcd(mul, held) != 1) mul += 2;
        if (held == 1) mul = 1;
        const int64_t off = static_cast<int64_t>((x >> 17) % static_cast<uint64_t>(held));
        RP_CUDA(h, cudaMemsetAsync(h->mlp_loss, 0, sizeof(float), h->stream));
        Group grp(h, RP_KERNEL_MLP, static_cast<int>(2 * nb));
        for (int64_t b = 0; b < nb; b++) {
            const int64_t i0 = b * batch;
            const int cnt = static_cast<int>(std::min<int64_t>(batch, held - i0));
            RP_CUDA(h, cudaMemsetAsync(h->mlp_grad, 0, sizeof(float) * MLP_NPARAM, h->stream));
            RP_CUDA(h, launch_mlp_grad(h->pair_feats, h->pair_labels, held, i0, cnt, mul, off, h->mlp_w32,
                                       h->mlp_grad, h->mlp_loss, h->num_sms, h->stream));
            RP_CUDA(h, launch_mlp_adam(h->mlp_w32, h->mlp_w16, h->mlp_grad, h->mlp_m, h->mlp_v, lr, ++h->mlp_step,
                                       h->stream));
        }
        if (ep == epochs - 1) {
            RP_CUDA(h, cudaMemcpyAsync(&last, h->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, h->stream));
            RP_CUDA(h, cudaStreamSynchronize(h->stream));
        }
    }
    if (loss) *loss = static_cast<float>(last / static_cast<double>(nb));
    h->partners_valid = false;
    return RP_OK;
}

int rp_get_grid_counters(void *handle, uint64_t *rebuilds, uint64_t *remaps) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !rebuilds || !remaps) return fail(h, RP_ERR_ARG, "null argument");
    *rebuilds = h->grid_rebuilds;
    *remaps = h->grid_remaps;
    return RP_OK;
}

int rp_set_walls(void *handle, int32_t mask) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || mask < 0 || mask > 7) return fail(h, RP_ERR_ARG, "wall mask outside 0..7");
    h->walls = mask;
    h->try_valid = false;
    return RP_OK;
}

int rp_set_staging_filter(void *handle, int32_t mode) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || mode < 0 || mode > 2) return fail(h, RP_ERR_ARG, "bad argument");
    h->stage_mode = mode;
    return RP_OK;
}

int rp_set_cell_order(void *handle, int32_t on) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || (on != 0 && on != 1)) return fail(h, RP_ERR_ARG, "cell order must be 0 or 1");
    h->cell_order = on;
    return RP_OK;
}

int rp_set_bulk_staging(void *handle, int32_t on) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || (on != 0 && on != 1)) return fail(h, RP_ERR_ARG, "bulk staging must be 0 or 1");
    h->bulk_stage = on;
    return RP_OK;
}

int rp_set_cells_per_warp(void *handle, int32_t cells) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || (cells != 1 && cells != 2)) return fail(h, RP_ERR_ARG, "cells per warp must be 1 or 2");
    h->cells_per_warp = cells;
    return RP_OK;
}

// CompoundInteraction of the shape's hard interaction and a central potential on the same
// interaction centres (core/interactions/CompoundInteraction.cpp:9-49), as casino joins a
// helper shape for overlap relaxation (frontend/modes/CasinoMode.cpp:288-289); or the soft
// part alone (SphereTraits / PolysphereTraits with a CentralInteraction).
int rp_set_soft(void *handle, int32_t kind, double epsilon, double sigma, int32_t hard) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return RP_ERR_ARG;
    if (h->batch_member) return fail(h, RP_ERR_UNSUPPORTED, "soft parts on a batch replica");
    if (h->shape.kind == RP_SHAPE_CONVEX) return fail(h, RP_ERR_UNSUPPORTED, "soft parts of convex bodies");
    if (kind != RP_SOFT_NONE && kind != RP_SOFT_REPULSIVE_LJ && kind != RP_SOFT_SQUARE_INVERSE_CORE) {
        if (kind == RP_SOFT_LENNARD_JONES)
            return fail(h, RP_ERR_UNSUPPORTED,
                        "Lennard-Jones has no cut-off: the reference's energy then depends on its neighbour-grid cells");
        return fail(h, RP_ERR_ARG, "unknown soft interaction");
    }
    if (kind != RP_SOFT_NONE) {
        if (!(sigma > 0)) return fail(h, RP_ERR_ARG, "sigma must be positive");
        if (kind == RP_SOFT_REPULSIVE_LJ && !(epsilon > 0)) return fail(h, RP_ERR_ARG, "epsilon must be positive");
        if (kind == RP_SOFT_SQUARE_INVERSE_CORE && epsilon == 0) return fail(h, RP_ERR_ARG, "epsilon must be nonzero");
        if (!hard && (h->shape.kind == RP_SHAPE_SPHEROCYLINDER || h->segs))
            return fail(h, RP_ERR_UNSUPPORTED, "a soft part alone is built for spheres and polyspheres");
    }
    RP_CUDA(h, cudaSetDevice(h->device));
    if (!h->hard_ranges_saved) {
        h->hard_range = h->range;
        h->hard_ref_range = h->ref_range;
        h->hard_total_range = h->total_range;
        h->hard_ranges_saved = true;
    }
    h->soft = kind;
    h->soft_only = kind != RP_SOFT_NONE && !hard;
    h->soft_eps = epsilon;
    h->soft_sigma = sigma;
    h->soft_cut = sigma * std::pow(2., 1. / 6);  // RepulsiveLennardJonesInteraction.cpp:19-20
    h->range = h->hard_range;
    h->ref_range = h->hard_ref_range;
    h->total_range = h->hard_total_range;
    if (kind != RP_SOFT_NONE) {
        // the compound's range is the larger one (CompoundInteraction.cpp:33-35); the
        // checkerboard cells hold every body pair with a centre pair within it
        const double srange = kind == RP_SOFT_REPULSIVE_LJ ? h->soft_cut : sigma;
        double cmax = 0;
        for (int b = 0; b < h->ncen; b++)
            cmax = std::max(cmax, std::sqrt(h->cbody[3 * b] * h->cbody[3 * b] + h->cbody[3 * b + 1] * h->cbody[3 * b + 1] +
                                            h->cbody[3 * b + 2] * h->cbody[3 * b + 2]));
        const double body = (h->ncen > 0 ? 2 * cmax + srange : srange) * (1.0 + 1e-12);
        h->range = h->soft_only ? body : std::max(h->hard_range, body);
        h->ref_range = h->soft_only ? srange : std::max(h->hard_ref_range, srange);
        h->total_range = h->ncen > 0 ? 2 * cmax + h->ref_range : h->ref_range;
    }
    h->grid_stale = true;
    h->grid_patched = false;
    h->partners_valid = false;
    h->try_valid = false;
    h->log_valid = false;
    h->can_revert = false;
    if (h->counting && h->has_state) {
        // the cached count follows the new interaction (Packing::setupForInteraction)
        int64_t cnt = 0;
        int rc = rp_count_overlaps(h, 0, &cnt);
        if (rc) return rc;
        unsigned long long c = static_cast<unsigned long long>(cnt);
        RP_CUDA(h, cudaMemcpyAsync(h->d_overlaps, &c, sizeof(c), cudaMemcpyHostToDevice, h->stream));
        RP_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return RP_OK;
}

int rp_set_temperature(void *handle, double temperature) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !(temperature > 0)) return fail(h, RP_ERR_ARG, "temperature must be positive");
    h->temperature = temperature;
    return RP_OK;
}

int rp_get_cells_per_warp(void *handle, int32_t *last) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !last) return RP_ERR_ARG;
    *last = h->last_cells_per_warp;
    return RP_OK;
}

int rp_set_ordering(void *handle, int32_t mode, int32_t every) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || mode < RP_ORDER_OFF || mode > RP_ORDER_DISTANCE || every <= 0) return fail(h, RP_ERR_ARG, "bad argument");
    if (mode != RP_ORDER_OFF && h->shape.kind == RP_SHAPE_CONVEX)
        return fail(h, RP_ERR_UNSUPPORTED, "the learned ordering of convex bodies");
    h->order_mode = mode;
    h->order_every = every;
    h->partners_valid = false;
    return RP_OK;
}

// ---- batched replicas ---------------------------------------------------------------

int rp_batch_create(const rp_shape_desc *shape, int32_t replicas, const int64_t *n, int device, void **batch) {
    if (!shape || !n || !batch || replicas <= 0 || replicas > 4096) return RP_ERR_ARG;
    if (shape->kind != RP_SHAPE_SPHERE && shape->kind != RP_SHAPE_SPHEROCYLINDER) return RP_ERR_UNSUPPORTED;
    int64_t total = 0;
    for (int r = 0; r < replicas; r++) {
        if (n[r] <= 0) return RP_ERR_ARG;
        total += n[r];
    }
    if (total > (1ll << 31) - 1) return RP_ERR_ARG;
    Batch *b = new (std::nothrow) Batch();
    if (!b) return RP_ERR_ARG;
    b->device = device;
    b->kind = shape->kind;
    b->R = replicas;
    auto bail = [&](int rc) {
        rp_batch_destroy(b);
        return rc;
    };
    if (cudaSetDevice(device) != cudaSuccess) return bail(RP_ERR_CUDA);
    cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&b->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(RP_ERR_CUDA);
    const int R = replicas;
    bool ok = cudaMalloc(&b->d_table, sizeof(BatchRep) * R) == cudaSuccess &&
              cudaMalloc(&b->d_bases, sizeof(int) * (2 + MAX_PHASES) * (R + 1)) == cudaSuccess &&
              cudaMalloc(&b->rtab64, sizeof(double) * 9 * ROT_TABLE) == cudaSuccess &&
              cudaMalloc(&b->rtab32, sizeof(float) * 12 * ROT_TABLE) == cudaSuccess &&
              cudaMalloc(&b->item_counters, sizeof(int32_t) * MAX_PHASES) == cudaSuccess &&
              cudaMalloc(&b->stats, sizeof(unsigned long long) * NUM_COUNTERS * R) == cudaSuccess &&
              cudaMalloc(&b->status, sizeof(uint32_t) * R) == cudaSuccess &&
              cudaMalloc(&b->counts, sizeof(unsigned long long) * R) == cudaSuccess &&
              cudaMallocHost(&b->h_counts, sizeof(unsigned long long) * R) == cudaSuccess &&
              cudaMalloc(&b->flags, sizeof(int) * R) == cudaSuccess &&
              cudaMallocHost(&b->h_flags, sizeof(int) * R) == cudaSuccess;
    for (auto &S : b->stage)
        ok = ok && cudaMallocHost(&S.table, sizeof(BatchRep) * R) == cudaSuccess &&
             cudaMallocHost(&S.bases, sizeof(int) * (2 + MAX_PHASES) * (R + 1)) == cudaSuccess &&
             cudaEventCreateWithFlags(&S.done, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) return bail(RP_ERR_CUDA);
    cudaMemset(b->stats, 0, sizeof(unsigned long long) * NUM_COUNTERS * R);
    cudaMemset(b->status, 0, sizeof(uint32_t) * R);
    for (int r = 0; r < R; r++) {
        Handle *h = new (std::nothrow) Handle();
        if (!h) return bail(RP_ERR_ARG);
        h->batch_member = true;
        h->shape = *shape;
        double rad = shape->radius, l = shape->length;
        ExactShape ex{};
        ex.kind = shape->kind;
        if (shape->kind == RP_SHAPE_SPHERE) {
            h->range = 2 * rad;
            ex.sphere_thr = std::pow(2 * rad, 2);
        } else {
            h->range = 2 * rad + l;
            ex.core_thr = 4 * rad * rad;
            ex.far_thr = std::pow(2 * rad + l, 2);
            short beg = -1, end = 1;
            ex.neg_cap_half = 0.5 * beg * l;
            ex.cap_half = 0.5 * end * l;
        }
        h->ref_range = h->range;
        h->total_range = h->range;
        h->ex = ex;
        h->status = b->status + r;
        h->counters = b->stats + NUM_COUNTERS * r;
        h->rtab64 = b->rtab64;
        h->rtab32 = b->rtab32;
        void *hh = nullptr;
        int rc = create_common(h, n[r], device, &hh);
        if (rc) return bail(rc);
        b->rep.push_back(h);
    }
    *batch = b;
    return RP_OK;
}

int rp_batch_destroy(void *batch) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b) return RP_ERR_ARG;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (Handle *h : b->rep) rp_destroy(h);
    cudaFree(b->d_table);
    cudaFree(b->d_bases);
    cudaFree(b->d_bounds);
    cudaFree(b->rtab64);
    cudaFree(b->rtab32);
    cudaFree(b->item_counters);
    cudaFree(b->stats);
    cudaFree(b->status);
    cudaFree(b->counts);
    cudaFreeHost(b->h_counts);
    cudaFree(b->flags);
    cudaFreeHost(b->h_flags);
    for (auto &S : b->stage) {
        cudaFreeHost(S.table);
        cudaFreeHost(S.bases);
        cudaFreeHost(S.bounds);
        if (S.done) cudaEventDestroy(S.done);
    }
    b->tm.release();
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return RP_OK;
}

const char *rp_batch_last_error(void *batch) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b) return "null batch";
    if (!b->err.empty()) return b->err.c_str();
    for (Handle *h : b->rep)
        if (!h->err.empty()) return h->err.c_str();
    return "";
}

static Handle *batch_rep(Batch *b, int32_t r) {
    if (!b || r < 0 || r >= b->R) return nullptr;
    return b->rep[r];
}

int rp_batch_upload_state(void *batch, int32_t replica, const double *pos, const double *rot, const double *box9) {
    Batch *b = static_cast<Batch *>(batch);
    Handle *h = batch_rep(b, replica);
    if (!h) return bfail(b, RP_ERR_ARG, "bad replica");
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    int rc = rp_upload_state(h, pos, rot, box9);
    if (rc) b->err = h->err;
    return rc;
}

int rp_batch_download_state(void *batch, int32_t replica, double *pos, double *rot, double *box9) {
    Batch *b = static_cast<Batch *>(batch);
    Handle *h = batch_rep(b, replica);
    if (!h) return bfail(b, RP_ERR_ARG, "bad replica");
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    int rc = rp_download_state(h, pos, rot, box9);
    if (rc) b->err = h->err;
    return rc;
}

int rp_batch_set_walls(void *batch, int32_t mask) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b || mask < 0 || mask > 7) return bfail(b, RP_ERR_ARG, "wall mask outside 0..7");
    for (Handle *h : b->rep) h->walls = mask;
    return RP_OK;
}

int rp_batch_set_staging_filter(void *batch, int32_t mode) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b || mode < 0 || mode > 2) return bfail(b, RP_ERR_ARG, "bad argument");
    for (Handle *h : b->rep) h->stage_mode = mode;
    return RP_OK;
}

int rp_batch_upload_states(void *batch, const double *pos, const double *rot, const double *boxes) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b || !pos || !rot || !boxes) return bfail(b, RP_ERR_ARG, "null argument");
    RB_CUDA(b, cudaSetDevice(b->device));
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    int64_t off = 0;
    for (int r = 0; r < b->R; r++) {
        Handle *h = b->rep[r];
        const double *box9 = boxes + 9 * r;
        if (det3(box9) == 0) return bfail(b, RP_ERR_ARG, "box volume is zero");
        h->has_state = false;
        std::memcpy(h->box, box9, sizeof(h->box));
        inverse3(box9, h->inv);
        h->pcur = 0;
        h->gcur = 0;
        h->partners_valid = false;
        h->can_revert = false;
        h->log_valid = false;
        RB_CUDA(b, cudaMemcpyAsync(h->pos64[0], pos + 3 * off, sizeof(double) * 3 * h->n, cudaMemcpyHostToDevice,
                                   b->stream));
        RB_CUDA(b, cudaMemcpyAsync(h->rot64, rot + 9 * off, sizeof(double) * 9 * h->n, cudaMemcpyHostToDevice,
                                   b->stream));
        double tt[375];
        translation_table(h->box, tt);
        RB_CUDA(b, cudaMemcpyAsync(h->trans[0], tt, sizeof(tt), cudaMemcpyHostToDevice, b->stream));
        double shift[3] = {0, 0, 0};
        int rc = setup_grid(h, h->grid[0], h->box, shift);
        if (rc) return bfail(b, rc, h->err);
        h->strict_box = true;  // the rebuild checks that every particle lies inside its box
        off += h->n;
    }
    int total_items = 0, total_p = 0, total_c = 0;
    int rc = batch_tables(b, total_items, total_p, total_c);
    for (Handle *h : b->rep) h->strict_box = false;
    if (rc) return rc;
    rc = batch_copy(b);
    if (rc) return rc;
    RB_CUDA(b, cudaMemsetAsync(b->status, 0, sizeof(uint32_t) * b->R, b->stream));
    {
        BGroup grp(b, RP_KERNEL_REBUILD, 5);
        RB_CUDA(b, launch_b_rebuild(b->d_table, b->d_bases, b->d_bases + (b->R + 1), b->R, total_p, total_c,
                                    b->stream));
    }
    std::vector<uint32_t> st(b->R);
    RB_CUDA(b, cudaMemcpyAsync(st.data(), b->status, sizeof(uint32_t) * b->R, cudaMemcpyDeviceToHost, b->stream));
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    for (int r = 0; r < b->R; r++)
        if (st[r]) {
            RB_CUDA(b, cudaMemsetAsync(b->status, 0, sizeof(uint32_t) * b->R, b->stream));
            if (st[r] & ST_OUTSIDE) return bfail(b, RP_ERR_ARG, "replica " + std::to_string(r) + ": a particle lies outside the box");
            return bfail(b, RP_ERR_DEVICE, "replica " + std::to_string(r) + ": device status set");
        }
    for (Handle *h : b->rep) h->has_state = true;
    return RP_OK;
}

int rp_batch_download_states(void *batch, double *pos, double *rot, double *boxes) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b) return RP_ERR_ARG;
    for (Handle *h : b->rep)
        if (!h->has_state) return bfail(b, RP_ERR_STATE, "a replica has no state");
    RB_CUDA(b, cudaSetDevice(b->device));
    int64_t off = 0;
    for (Handle *h : b->rep) {
        if (pos)
            RB_CUDA(b, cudaMemcpyAsync(pos + 3 * off, h->pos64[h->pcur], sizeof(double) * 3 * h->n,
                                       cudaMemcpyDeviceToHost, b->stream));
        if (rot)
            RB_CUDA(b, cudaMemcpyAsync(rot + 9 * off, h->rot64, sizeof(double) * 9 * h->n, cudaMemcpyDeviceToHost,
                                       b->stream));
        off += h->n;
    }
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    if (boxes)
        for (int r = 0; r < b->R; r++) std::memcpy(boxes + 9 * r, b->rep[r]->box, sizeof(b->rep[r]->box));
    return RP_OK;
}

int rp_batch_set_timing(void *batch, int on) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b) return RP_ERR_ARG;
    RB_CUDA(b, cudaSetDevice(b->device));
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    b->tm.reset(on != 0);
    return RP_OK;
}

int rp_batch_get_timing(void *batch, double *ms, uint64_t *groups, uint64_t *launches) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b) return RP_ERR_ARG;
    RB_CUDA(b, cudaSetDevice(b->device));
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    RB_CUDA(b, b->tm.collect(ms, groups));
    if (launches) {
        uint64_t l = b->launches;
        for (Handle *h : b->rep) l += h->launches;
        *launches = l;
    }
    return RP_OK;
}

int rp_batch_count_overlaps(void *batch, int32_t replica, int early_exit, int64_t *count) {
    Batch *b = static_cast<Batch *>(batch);
    Handle *h = batch_rep(b, replica);
    if (!h) return bfail(b, RP_ERR_ARG, "bad replica");
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    int rc = rp_count_overlaps(h, early_exit, count);
    if (rc) b->err = h->err;
    return rc;
}

int rp_batch_set_tuning(void *batch, double cell_factor, int32_t warps_per_block) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b || !(cell_factor >= 1.0) || (warps_per_block != 2 && warps_per_block != 4 && warps_per_block != 8))
        return bfail(b, RP_ERR_ARG, "cell factor >= 1 and 2, 4 or 8 warps per block");
    for (Handle *h : b->rep) h->cell_factor = cell_factor;
    b->wpb = warps_per_block;
    return RP_OK;
}

int rp_batch_sweep(void *batch, const rp_sweep_params *p, rp_sweep_stats *stats) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b || !p) return bfail(b, RP_ERR_ARG, "null argument");
    int types = (p->translation_step > 0 ? 1 : 0) | (p->rotation_step > 0 ? 2 : 0);
    if (!types) return bfail(b, RP_ERR_ARG, "no move type enabled");
    if (p->flags & RP_SWEEP_ROTOTRANSLATION) {
        if (types != 3) return bfail(b, RP_ERR_ARG, "rototranslations need a translation and a rotation step");
        types = SWEEP_ROTOTRANSLATION;
    }
    for (Handle *h : b->rep)
        if (!h->has_state) return bfail(b, RP_ERR_STATE, "a replica has no state");
    RB_CUDA(b, cudaSetDevice(b->device));
    const bool log = (p->flags & RP_SWEEP_LOG) != 0;
    const int ntypes = sweep_move_types(types);
    std::vector<std::vector<int>> phases(b->R);
    std::vector<double> tstep(b->R);
    int cap = 0, maxph = 0;
    for (int r = 0; r < b->R; r++) {
        Handle *h = b->rep[r];
        double shift[3];
        uint32_t shuffle = 0;
        sweep_origin(replica_seed(p->seed, r), p->counter, shift, shuffle);
        int rc = setup_grid(h, h->grid[h->gcur], h->box, shift);
        if (rc) return bfail(b, rc, h->err);
        const GridHost &G = h->grid[h->gcur];
        phase_order(G.d, shuffle, phases[r]);
        maxph = std::max(maxph, static_cast<int>(phases[r].size()));
        cap = std::max(cap, G.cap);
        double hgt[3];
        heights_of(h->box, hgt);
        tstep[r] = std::min(p->translation_step, std::min({hgt[0], hgt[1], hgt[2]}) / 2);
        if (log) {
            int64_t before = h->log_alloc;
            RB_CUDA(b, ensure(h->d_log, h->log_alloc, ntypes * h->n));
            if (!h->d_log_codes || h->log_alloc != before) {
                cudaFree(h->d_log_codes);
                h->d_log_codes = nullptr;
                RB_CUDA(b, cudaMalloc(&h->d_log_codes, h->log_alloc));
            }
        }
    }
    // the staging capacity of every replica: two warps per block must fit
    {
        const size_t per_cap = batch_smem_per_warp(b->kind, 32) / 32;
        const int fit = static_cast<int>(static_cast<size_t>(b->smem_optin) / 2 / per_cap) / 32 * 32;
        cap = std::min(cap, fit);
    }
    int total_items = 0, total_p = 0, total_c = 0;
    int rc = batch_tables(b, total_items, total_p, total_c);
    if (rc) return rc;
    BatchRep *T = b->stage[b->cur].table;
    for (int r = 0; r < b->R; r++) {
        Handle *h = b->rep[r];
        SweepArgs &a = T[r].a;
        a.cap = cap;
        a.seed = replica_seed(p->seed, r);
        a.counter = p->counter;
        a.tstep = static_cast<float>(tstep[r]);
        a.rstep = static_cast<float>(p->rotation_step);
        a.types = types;
        a.rtab64 = b->rtab64;
        a.rtab32 = b->rtab32;
        a.rtab_mask = ROT_TABLE - 1;
        if (p->flags & RP_SWEEP_FP64_ONLY) a.fp64_only = 1;
        if (log) {
            a.log = h->d_log;
            a.log_codes = h->d_log_codes;
        }
        T[r].nphases = static_cast<int>(phases[r].size());
        for (int k = 0; k < MAX_PHASES; k++) T[r].phases[k] = k < T[r].nphases ? phases[r][k] : 0;
    }
    // the cells of phase k of every replica, numbered consecutively
    std::vector<int> phase_total(maxph, 0);
    {
        int *bases = b->stage[b->cur].bases;
        for (int k = 0; k < maxph; k++) {
            int *ibk = bases + (2 + k) * (b->R + 1);
            ibk[0] = 0;
            for (int r = 0; r < b->R; r++) {
                int act[3];
                const int items = k < T[r].nphases ? phase_cells(b->rep[r]->grid[b->rep[r]->gcur].d, T[r].phases[k], act) : 0;
                ibk[r + 1] = ibk[r] + items;
            }
            phase_total[k] = ibk[b->R];
        }
    }
    rc = batch_copy(b);
    if (rc) return rc;
    const int *pb = b->d_bases, *cb = b->d_bases + (b->R + 1);
    if (stats) RB_CUDA(b, cudaMemsetAsync(b->stats, 0, sizeof(unsigned long long) * NUM_COUNTERS * b->R, b->stream));
    {
        const bool rotations = (types & (2 | SWEEP_ROTOTRANSLATION)) != 0;
        BGroup grp(b, RP_KERNEL_REBUILD, rotations ? 6 : 5);
        RB_CUDA(b, launch_b_rebuild(b->d_table, pb, cb, b->R, total_p, total_c, b->stream));
        if (rotations)
            RB_CUDA(b, launch_rot_table(b->rtab64, b->rtab32, ROT_TABLE, p->seed, p->counter,
                                        static_cast<float>(p->rotation_step), b->stream));
    }
    RB_CUDA(b, cudaMemsetAsync(b->item_counters, 0, sizeof(int32_t) * MAX_PHASES, b->stream));
    // fewer warps per block when the staging of `cap` candidates per warp would not fit
    int wpb = b->wpb;
    while (wpb > 2 && static_cast<size_t>(wpb) * batch_smem_per_warp(b->kind, cap) > static_cast<size_t>(b->smem_optin))
        wpb /= 2;
    const int ovf_cap = static_cast<int>(OVF_SMEM / (batch_smem_per_warp(b->kind, 32) / 32)) / 32 * 32;
    for (int k = 0; k < maxph; k++) {
        const int *ib = b->d_bases + (2 + k) * (b->R + 1);
        int blocks = std::max(1, std::min((phase_total[k] + wpb - 1) / wpb, b->num_sms * (16 / wpb)));
        {
            BGroup grp(b, RP_KERNEL_SWEEP, 1);
            RB_CUDA(b, launch_b_sweep(b->d_table, ib, b->R, b->kind, k, b->item_counters + k, cap, wpb, blocks,
                                      types == SWEEP_ROTOTRANSLATION, b->stream));
        }
        {
            BGroup grp(b, RP_KERNEL_OVERFLOW, 1);
            RB_CUDA(b, launch_b_overflow(b->d_table, b->R, b->kind, k, ovf_cap, types == SWEEP_ROTOTRANSLATION,
                                         b->stream));
        }
    }
    for (int r = 0; r < b->R; r++) {
        Handle *h = b->rep[r];
        h->can_revert = false;
        h->log_valid = false;
        if (log) {
            const GridDev &g = h->grid[h->gcur].d;
            h->log_valid = true;
            h->log_types = ntypes;
            h->log_phases = phases[r];
            for (int d = 0; d < 3; d++) h->log_dims[d] = g.dims[d];
            h->log_start.resize(g.ncell + 1);
            RB_CUDA(b, cudaMemcpyAsync(h->log_start.data(), g.start, sizeof(int32_t) * (g.ncell + 1),
                                       cudaMemcpyDeviceToHost, b->stream));
        }
    }
    if (stats || log) {
        std::vector<unsigned long long> c(NUM_COUNTERS * b->R);
        std::vector<uint32_t> st(b->R);
        RB_CUDA(b, cudaMemcpyAsync(c.data(), b->stats, sizeof(unsigned long long) * NUM_COUNTERS * b->R, cudaMemcpyDeviceToHost,
                                   b->stream));
        RB_CUDA(b, cudaMemcpyAsync(st.data(), b->status, sizeof(uint32_t) * b->R, cudaMemcpyDeviceToHost, b->stream));
        RB_CUDA(b, cudaStreamSynchronize(b->stream));
        for (int r = 0; r < b->R; r++)
            if (st[r]) return bfail(b, (st[r] & ST_CAPACITY) ? RP_ERR_CAPACITY : RP_ERR_DEVICE, "device status set");
        uint64_t all_launches = b->launches;
        for (Handle *h : b->rep) all_launches += h->launches;
        if (stats)
            for (int r = 0; r < b->R; r++) {
                const unsigned long long *q = c.data() + NUM_COUNTERS * r;
                stats[r].moves = q[0];
                stats[r].accepted = q[1];
                stats[r].rejected_overlap = q[2];
                stats[r].rejected_domain = q[3];
                stats[r].pair_tests = q[4];
                stats[r].fp64_pairs = q[5];
                stats[r].translations = q[6];
                stats[r].rotations = q[7];
                stats[r].accepted_translations = q[8];
                stats[r].kernel_launches = all_launches;
            }
    }
    return RP_OK;
}

int rp_batch_sweep_log(void *batch, int32_t replica, rp_move *moves, uint8_t *codes, int64_t capacity,
                       int64_t *count) {
    Batch *b = static_cast<Batch *>(batch);
    Handle *h = batch_rep(b, replica);
    if (!h) return bfail(b, RP_ERR_ARG, "bad replica");
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    int rc = rp_sweep_log(h, moves, codes, capacity, count);
    if (rc) b->err = h->err;
    return rc;
}

int rp_batch_get_grid(void *batch, int32_t replica, rp_grid_info *info, int32_t *cells, double *bounds) {
    Batch *b = static_cast<Batch *>(batch);
    Handle *h = batch_rep(b, replica);
    if (!h) return bfail(b, RP_ERR_ARG, "bad replica");
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    int rc = rp_get_grid(h, info, cells, bounds);
    if (rc) b->err = h->err;
    return rc;
}

int rp_batch_try_scaling(void *batch, const double *boxes, const uint8_t *propose, double *dE) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b || !boxes || !propose || !dE) return bfail(b, RP_ERR_ARG, "null argument");
    RB_CUDA(b, cudaSetDevice(b->device));
    std::vector<uint8_t> upscaled(b->R, 0);
    std::vector<double> old_inv(9 * b->R);
    for (int r = 0; r < b->R; r++) {
        Handle *h = b->rep[r];
        dE[r] = 0;
        if (!propose[r]) continue;
        const double *nb = boxes + 9 * r;
        if (!h->has_state) return bfail(b, RP_ERR_STATE, "a replica has no state");
        if (det3(nb) == 0 || volume_of(nb) == 0) return bfail(b, RP_ERR_ARG, "box volume is zero");
        std::memcpy(old_inv.data() + 9 * r, h->inv, sizeof(h->inv));
        double new_inv[9];
        inverse3(nb, new_inv);
        std::memcpy(h->saved_box, h->box, sizeof(h->box));
        std::memcpy(h->saved_inv, h->inv, sizeof(h->inv));
        std::memcpy(h->box, nb, sizeof(h->box));
        std::memcpy(h->inv, new_inv, sizeof(h->inv));
        int old_g = h->gcur;
        h->pcur = 1 - h->pcur;
        h->gcur = 1 - h->gcur;
        double shift[3] = {h->grid[old_g].d.shift[0], h->grid[old_g].d.shift[1], h->grid[old_g].d.shift[2]};
        int rc = setup_grid(h, h->grid[h->gcur], h->box, shift);
        if (rc) {
            // undo this replica's switch; the replicas already switched are reverted by the caller
            std::memcpy(h->box, h->saved_box, sizeof(h->box));
            std::memcpy(h->inv, h->saved_inv, sizeof(h->inv));
            h->pcur = 1 - h->pcur;
            h->gcur = old_g;
            return bfail(b, rc, h->err);
        }
        h->can_revert = true;
        h->log_valid = false;
        h->partners_valid = false;
        upscaled[r] = box_upscaled(h->saved_box, h->box) ? 1 : 0;  // convex shapes only in a batch
    }
    int total_items = 0, total_p = 0, total_c = 0;
    int rc = batch_tables(b, total_items, total_p, total_c);
    if (rc) return rc;
    BatchRep *T = b->stage[b->cur].table;
    for (int r = 0; r < b->R; r++) {
        Handle *h = b->rep[r];
        T[r].scale = propose[r] ? 1 : 0;
        b->h_flags[r] = (propose[r] && !upscaled[r]) ? 0 : 1;  // a set flag skips the recount
        if (!propose[r]) continue;
        std::memcpy(T[r].old_inv, old_inv.data() + 9 * r, sizeof(T[r].old_inv));
        std::memcpy(T[r].new_box, h->box, sizeof(T[r].new_box));
        T[r].scale_src = h->pos64[1 - h->pcur];
        T[r].scale_dst = h->pos64[h->pcur];
        T[r].trans_dst = h->trans[h->pcur];
    }
    rc = batch_copy(b);
    if (rc) return rc;
    const int *pb = b->d_bases, *cb = b->d_bases + (b->R + 1);
    RB_CUDA(b, cudaMemcpyAsync(b->flags, b->h_flags, sizeof(int) * b->R, cudaMemcpyHostToDevice, b->stream));
    RB_CUDA(b, cudaMemsetAsync(b->counts, 0, sizeof(unsigned long long) * b->R, b->stream));
    {
        BGroup grp(b, RP_KERNEL_RESCALE, 2);
        RB_CUDA(b, launch_b_rescale(b->d_table, pb, b->R, total_p, b->stream));
    }
    {
        BGroup grp(b, RP_KERNEL_REBUILD, 5);
        RB_CUDA(b, launch_b_rebuild(b->d_table, pb, cb, b->R, total_p, total_c, b->stream));
    }
    {
        BGroup grp(b, RP_KERNEL_COUNT, 1);
        RB_CUDA(b, launch_b_count(b->d_table, pb, b->R, total_p, b->kind, 1, b->counts, b->flags, b->stream));
    }
    RB_CUDA(b, cudaMemcpyAsync(b->h_counts, b->counts, sizeof(unsigned long long) * b->R, cudaMemcpyDeviceToHost,
                               b->stream));
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    for (int r = 0; r < b->R; r++)
        if (propose[r] && !upscaled[r] && b->h_counts[r] > 0) dE[r] = std::numeric_limits<double>::infinity();
    return RP_OK;
}

int rp_batch_revert_scaling(void *batch, const uint8_t *mask) {
    Batch *b = static_cast<Batch *>(batch);
    if (!b || !mask) return bfail(b, RP_ERR_ARG, "null argument");
    RB_CUDA(b, cudaStreamSynchronize(b->stream));
    for (int r = 0; r < b->R; r++)
        if (mask[r]) {
            int rc = rp_revert_scaling(b->rep[r]);
            if (rc) return bfail(b, rc, b->rep[r]->err);
        }
    return RP_OK;
}

}  // extern "C"

namespace rp {

// The handle's FP64 state as a consistent snapshot: positions and orientations are copied
// on the device (on the handle's stream, in order with its moves) into a snapshot buffer,
// then downloaded on `side` into host memory (`pos` [n][3], `rot` [n][9], pinned for an
// asynchronous copy) while later work of the handle goes on; `done` is recorded on `side`
// after the download.  The box and the particle count are returned at once.
int state_snapshot(void *handle, double *pos, double *rot, double *box9, int64_t *n, cudaStream_t side,
                   cudaEvent_t done, std::string &err) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) {
        err = "null handle";
        return RP_ERR_ARG;
    }
    if (!h->has_state) {
        err = "no state uploaded";
        return RP_ERR_STATE;
    }
    auto cuda = [&](cudaError_t e, const char *what) {
        if (e == cudaSuccess) return false;
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return true;
    };
    if (cuda(cudaSetDevice(h->device), "cudaSetDevice")) return RP_ERR_CUDA;
    if (!h->snap64 && cuda(cudaMalloc(&h->snap64, sizeof(double) * 12 * h->n), "cudaMalloc")) return RP_ERR_CUDA;
    if (!h->snap_free && cuda(cudaEventCreateWithFlags(&h->snap_free, cudaEventDisableTiming), "cudaEventCreate"))
        return RP_ERR_CUDA;
    double *sp = h->snap64, *sr = h->snap64 + 3 * h->n;
    // the previous download out of the snapshot buffer has ended before it is overwritten
    if (cuda(cudaStreamWaitEvent(h->stream, h->snap_free, 0), "cudaStreamWaitEvent")) return RP_ERR_CUDA;
    if (cuda(cudaMemcpyAsync(sp, h->pos64[h->pcur], sizeof(double) * 3 * h->n, cudaMemcpyDeviceToDevice, h->stream),
             "cudaMemcpyAsync") ||
        cuda(cudaMemcpyAsync(sr, h->rot64, sizeof(double) * 9 * h->n, cudaMemcpyDeviceToDevice, h->stream),
             "cudaMemcpyAsync"))
        return RP_ERR_CUDA;
    cudaEvent_t copied = nullptr;
    if (cuda(cudaEventCreateWithFlags(&copied, cudaEventDisableTiming), "cudaEventCreate")) return RP_ERR_CUDA;
    bool bad = cuda(cudaEventRecord(copied, h->stream), "cudaEventRecord") ||
               cuda(cudaStreamWaitEvent(side, copied, 0), "cudaStreamWaitEvent") ||
               cuda(cudaMemcpyAsync(pos, sp, sizeof(double) * 3 * h->n, cudaMemcpyDeviceToHost, side), "cudaMemcpyAsync") ||
               cuda(cudaMemcpyAsync(rot, sr, sizeof(double) * 9 * h->n, cudaMemcpyDeviceToHost, side), "cudaMemcpyAsync") ||
               cuda(cudaEventRecord(h->snap_free, side), "cudaEventRecord") ||
               cuda(cudaEventRecord(done, side), "cudaEventRecord");
    cudaEventDestroy(copied);  // released once the recorded work completes
    if (bad) return RP_ERR_CUDA;
    std::memcpy(box9, h->box, sizeof(h->box));
    *n = h->n;
    return RP_OK;
}

// Particle count of a handle (0 for a null handle).
int64_t handle_size(void *handle) { return handle ? static_cast<Handle *>(handle)->n : 0; }

// The handle's current box (false without a state) and whether it counts overlaps.
bool handle_box(void *handle, double *box9) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !h->has_state) return false;
    std::memcpy(box9, h->box, sizeof(h->box));
    return true;
}
bool handle_counting(void *handle) { return handle && static_cast<Handle *>(handle)->counting; }
bool handle_soft(void *handle) { return handle && static_cast<Handle *>(handle)->soft != 0; }

// The current state of a handle for the observables (positions, orientations, box and its
// reference inverse), after its pending moves (in order on its stream).
struct PackingView {
    int device;
    cudaStream_t stream;
    int64_t n;
    const double *pos64;
    const double *rot64;
    double box[9], inv[9];
};
int packing_view(void *handle, PackingView *v, std::string &err) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) {
        err = "null handle";
        return RP_ERR_ARG;
    }
    if (!h->has_state) {
        err = "no state uploaded";
        return RP_ERR_STATE;
    }
    v->device = h->device;
    v->stream = h->stream;
    v->n = h->n;
    v->pos64 = h->pos64[h->pcur];
    v->rot64 = h->rot64;
    std::memcpy(v->box, h->box, sizeof(v->box));
    std::memcpy(v->inv, h->inv, sizeof(v->inv));
    return RP_OK;
}

}  // namespace rp
