// Internal layout of the engine: device structures shared by the kernels and the
// host orchestration in rp_api.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "rp_geom.cuh"
#include "rp_mlp.cuh"
#include "rp_xc.cuh"
#include "../../include/rampack_gb300.h"

namespace rp {

// Status bits a kernel may raise in the handle's device status word.
enum : uint32_t {
    ST_PARTICLE_NOT_IN_CELL = 1u << 0,  // a listed move's particle is not in its cell
    ST_BAD_CELL = 1u << 1,              // a listed move names a cell outside the grid
    ST_NUMERIC = 1u << 2,               // a non-finite coordinate was produced
    ST_CAPACITY = 1u << 3,              // a neighbourhood exceeded the largest staging capacity
    ST_OUTSIDE = 1u << 4,               // a particle lies outside the box
    ST_NOT_ROTATION = 1u << 5,          // an uploaded orientation is not a rotation (1e-6)
    ST_PORTAL_STUCK = 1u << 6,          // a convex pair's portal refinement hit its iteration limit
    ST_STAGE_TIMEOUT = 1u << 7,         // a bulk staging copy did not complete within its wait limit
};

// Constants of the FP32 filter: every comparison of the FP64 reference is decided in
// FP32 only when it clears a margin that bounds the FP32 error; otherwise the pair is
// re-decided in FP64 (the guard band).
struct FilterConsts {
    float sphere_lo, sphere_hi;   // spheres: (2r)^2 -/+ margin
    float core_lo, core_hi;       // spherocylinders: 4 r^2 -/+ margin
    float far_lo, far_hi;         // spherocylinders: (2r + l)^2 -/+ margin
    float core_thr;               // 4 r^2
    float seg_err;                // bound on |f32 - f| of the segment distance^2
    float d_min;                  // D = |u|^2 |v|^2 - (u.v)^2 below which FP64 decides
    float d_par;                  // D below which FP64 certainly takes its parallel branch
    float par_err;                // bound on that branch's excess over the true minimum
    float len;                    // spherocylinder cylinder length l
    float half_len;               // l / 2
    float cell_margin;            // relative in-cell margin of the FP32 ActiveDomain test
};

// One checkerboard cell grid with its cell list and FP32 mirror in cell order.
struct GridDev {
    int dims[3];
    int ncell;
    double shift[3];
    float fshift[3];      // shift and 1/dims in FP32 (the FP32 box-wrap test)
    float finv_dims[3];
    float cellmat[9];     // row-major box / n (column d divided by dims[d]), FP32
    float cellinv[9];     // inverse of cellmat (maps local coords to in-cell fractions)
    int32_t *count;       // [ncell]
    int32_t *start;       // [ncell + 1]
    int32_t *slot_pid;    // [n] particle of each slot (cells contiguous, pids ascending)
    int32_t *pid_slot;    // [n]
    int32_t *pid_cell;    // [n]
    int32_t *rank;        // [n] scratch: arrival rank within the cell
    float4 *mpos;         // [n] cell-local FP32 position, .w = pid bits
    float4 *maxis;        // [n] FP32 axis (orientation column 2)
    float4 *plocal;       // [n] scratch: cell-local FP32 position by pid
    double *bounds;       // ActiveDomain bounds: dim d at boundsoff[d], 2 doubles per cell
    int boundsoff[3];
    int32_t *max_occ;     // device scalar
    // the cells of each checkerboard phase by occupancy, largest first (phase-major), written
    // by the rebuild's scan; order_cnt [27 x ORDER_BINS] counts (zero between rebuilds),
    // order_off the ranges' offsets; all null where no order is kept
    int32_t *order;
    int32_t *order_cnt;
    int32_t *order_off;
    // polyspheres
    float4 *mcen;         // [n][ncen] FP32 rotated centre offsets, cell order
    float *cthr;          // [2][MAX_CEN^2] FP32 centre-pair thresholds (r_a + r_b)^2 -/+ margin
    // staging filter (cells well above the interaction range): a neighbour is staged only
    // if its distance from each face-slab of the home cell, in cell fractions times the
    // cell height stage_h[d], is at most stage_thr (the range plus a margin)
    int stage_filter;
    float stage_h[3];
    float stage_thr;
};

// A centre pair of the recount left undecided by the FP32 thresholds: body pid's centre
// aj / MAX_CEN against body pj's centre aj % MAX_CEN at FP32 separation d.
struct DeferredPair {
    int pid, pj, aj, pad;
    float4 d;
};

struct DevState {
    int64_t n;
    int kind;
    const XcShape *xc;    // generic convex bodies (kind 3): the body's geometry, device memory
    double box[9], inv[9];
    double box_zero[3];   // box * (0, 0, 0) row by row (Matrix * Vector from zero): a no-wrap correction
    double *pos64;        // [n][3]
    double *rot64;        // [n][9]
    double *trans;        // [125][3] box · m for m in {-2..2}^3
    float inv32[9];
    ExactShape ex;
    FilterConsts fc;
    uint32_t *status;
    unsigned long long *counters;  // rp_sweep_stats layout
    int strict_box;                // rebuild: flag positions outside [0, 1) relative (uploads)
    // polyspheres (kind 2): the reference's interactionCentres (orientation-rotated body
    // offsets, rotated incrementally by accepted moves) and absoluteInteractionCentres
    int ncen;
    double *cen64;                 // [n][ncen][3]
    double *abs64;                 // [n][ncen][3] (position + centre, wrapped into the box)
    const double *cthr64;          // [MAX_CEN^2] (r_a + r_b)^2, FP64 as the reference forms it
    // polyspherocylinders (PolyspherocylinderTraits): each centre a spherocylinder with a
    // body-frame half axis; circ64 [MAX_CEN^2] holds (c_a + c_b)^2 of the circumsphere radii
    int segs;
    double chax[RP_MAX_CENTRES][3];
    const double *circ64;
    // the recount's deferred FP64 centre pairs (multi-centre bodies): queued by k_count_poly,
    // decided by k_count_deferred with every lane busy; null: decided inline
    struct DeferredPair *cq_buf;
    int *cq_count;
    int cq_cap;
    // nonzero when the reference keeps no neighbour grid for this box (core/Packing.cpp:862-881):
    // it then measures sphere and polysphere-centre distances with the periodic boundary
    // conditions' own formula (pbc_distance2: per-coordinate |relative separation| folded
    // into [0, 1/2]) instead of a cell translation.  1: orthorhombic box, where that is the
    // true distance and the FP32 filter holds; 2: sheared box, where it is not, and every
    // sphere or centre pair is decided in FP64
    int pbc_fold;
    // overlap counting (Packing::toggleOverlapCounting): the cached total count, which
    // accepted moves update by their overlap delta
    int counting;
    unsigned long long *overlaps;
    // hard walls (Packing::toggleWalls): bit i walls the planes across box side i, whose unit
    // normal (side i+1 x side i+2, normalised) is wall_vec[i]; the far wall passes through
    // the corner wall_far (the sum of the sides); a particle meets the wall nearer to it
    // within wall_half (half the total interaction range); wall_radius holds the sphere,
    // spherocylinder or polysphere-centre radii and wall_half_len half the cylinder length
    int walls;
    double wall_vec[3][3];
    double wall_far[3];
    double wall_half;
    double wall_half_len;
    double wall_radius[RP_MAX_CENTRES];
    // soft part: a central potential on the interaction centres joined to the hard shape
    // (CompoundInteraction, core/interactions/CompoundInteraction.cpp:9-49): 0 none,
    // 1 RepulsiveLennardJonesInteraction, 2 SquareInverseCoreInteraction; soft_only: no hard part
    int soft, soft_only;
    double soft_eps, soft_sigma, soft_cut;   // soft_cut: sigma * std::pow(2., 1./6) (RepulsiveLennardJones)
    double soft_cut2, soft_sigma2, soft_4eps; // cut * cut, sigma * sigma, 4 * eps (the same roundings)
};

constexpr int MAX_CEN = RP_MAX_CENTRES;

// ---- checkerboard colouring ------------------------------------------------------------
// Along each dimension the cells form a ring of n cells, coloured so that neighbours differ:
// one colour for n = 1, two alternating colours for even n, and for odd n the colours
// c mod 3 (the last cell of a ring with n mod 3 = 1 takes colour 1).  A phase is one colour
// per dimension, coded p0 + 3 p1 + 9 p2; the cells of a phase never interact, since two of
// them differ in some dimension where they sit at least one cell apart.
constexpr int MAX_PHASES = 27;
RP_HD int ring_ncol(int n) { return n == 1 ? 1 : (n % 2 == 0 ? 2 : 3); }
RP_HD int ring_colour(int n, int c) {
    const int k = ring_ncol(n);
    if (k == 1) return 0;
    if (k == 2) return c & 1;
    if (n % 3 == 1 && c == n - 1) return 1;
    return c % 3;
}
RP_HD int ring_count(int n, int p) {  // cells of colour p
    const int k = ring_ncol(n);
    if (k == 1) return 1;
    if (k == 2) return n / 2;
    int cnt = (n - p + 2) / 3;
    if (n % 3 == 1) cnt += (p == 1) - (p == 0);
    return cnt;
}
RP_HD int ring_cell(int n, int p, int i) {  // the i-th cell of colour p
    const int k = ring_ncol(n);
    if (k == 1) return 0;
    if (k == 2) return 2 * i + p;
    if (n % 3 == 1 && p == 1 && i == ring_count(n, 1) - 1) return n - 1;
    return 3 * i + p;
}
RP_HD int phase_digit(int ph, int d) { return d == 0 ? ph % 3 : (d == 1 ? (ph / 3) % 3 : ph / 9); }
constexpr int ORDER_BINS = 32;  // occupancy bins of the per-phase cell order (the last holds 31 and more)
RP_HD int cell_phase(const int *dims, int cell) {
    const int cx = cell % dims[0], cy = (cell / dims[0]) % dims[1], cz = cell / (dims[0] * dims[1]);
    return ring_colour(dims[0], cx) + 3 * ring_colour(dims[1], cy) + 9 * ring_colour(dims[2], cz);
}
// per-warp polysphere scratch of the sweep (float4 units): the mover's FP32 centres
// [MAX_CEN], the centre-pair thresholds [2 MAX_CEN^2 floats], the mover's exact centres
// and absolute centres [2 x 3 MAX_CEN doubles]
constexpr int SWEEP_POLY_SCRATCH = MAX_CEN + MAX_CEN * MAX_CEN / 2 + 3 * MAX_CEN + 3 * MAX_CEN / 2;

constexpr int NUM_COUNTERS = 9;     // sweep statistics words per handle (rp_sweep_stats order)
constexpr int SWEEP_WARPS = 4;       // warps per block of the sweep kernel
constexpr int SWEEP_P1 = 4;          // candidates per lane per round of the sweep's FP32 centre pass
constexpr int SWEEP_MIN_BLOCKS = 4;  // resident blocks per SM the register budget allows
constexpr int MIRROR_ROUNDINGS = 4;  // FP32 mirror updates per particle and sweep before an exact refresh
constexpr uint32_t ROT_TABLE = 65536;  // rotations drawn per sweep (plus their inverses); at most 2^16
static_assert(ROT_TABLE <= 65536, "a rototranslation draws its table index from 16 random bits");

// SweepArgs::types: 1 translations, 2 rotations, 3 both (each particle once per type), or
// SWEEP_ROTOTRANSLATION (each particle once, translated and rotated together)
constexpr int SWEEP_ROTOTRANSLATION = 4;
__host__ __device__ inline int sweep_move_types(int types) {
    return types == SWEEP_ROTOTRANSLATION ? 1 : (types & 1) + ((types >> 1) & 1);
}

struct SweepArgs {
    DevState s;
    GridDev g;
    int phase[3];
    int active[3];
    int num_active;
    int cap;                       // staged candidates per warp
    // list mode
    const rp_move *moves;
    const int32_t *list_cells;     // cells with moves in this phase
    const int32_t *list_begin;     // [num_list + 1] ranges into moves / move_out
    const int32_t *move_out;       // original index of each (sorted) move
    int num_list;
    uint8_t *codes;
    // rng mode
    uint64_t seed, counter;
    float tstep, rstep;
    int types;                     // bit 0 translation, bit 1 rotation
    const double *rtab64;          // rotation table of this sweep: [rtab_mask + 1][9] exact FP64
    const float *rtab32;           // the same rotations rounded to FP32, padded to 12 floats
    uint32_t rtab_mask;
    rp_move *log;                  // [ntypes * n] indexed by ntypes * start[cell] + k
    uint8_t *log_codes;
    int fp64_only;
    int bulk_stage;                // stage neighbourhoods with bulk asynchronous copies (one per cell and array)
    // overflow: cells whose neighbourhood exceeds cap are appended here and rerun
    int32_t *overflow;             // [ncell]
    int32_t *overflow_count;
    const int32_t *work;           // optional explicit list of cells (overflow rerun, occupancy order)
    const int32_t *work_count;     // device-side length of `work` (null: num_work)
    int num_work;
    int32_t *next_item;            // persistent launch: shared cell counter (zeroed per launch)
    // learned ordering: best-ranked partners per particle (pre-tested before the full scan)
    const int32_t *partners;       // [n][MLP_PARTNERS] particle indices, -1 = none; NULL = off
    // pair-outcome log for training the ranking network
    float *pair_feats;             // [pair_cap][16]
    uint8_t *pair_labels;          // [pair_cap]
    unsigned long long *pair_count;
    unsigned long long pair_cap;
    int pair_every;                // log the pairs of every pair_every-th move (0 = off)
    float inv_range;
};

// The state a single unrestricted move tried (rp_try_move), kept on the device until the
// move is accepted (rp_accept_move) or another one is tried: the reference's temp shape
// slot (core/Packing.cpp:86-93) with its interaction centres (:357-361, :1041-1047).
struct SingleTry {
    double pos[3], rot[9];
    double cen[3 * RP_MAX_CENTRES], abs[3 * RP_MAX_CENTRES];
    double dE;
    int32_t particle, type, delta, valid;
    int32_t outside, pad;   // rejected by the ActiveDomain before any overlap test
};

// Arguments of one single-move test: the mover's candidates are the particles listed in the
// 27 grid cells around its position (the grid is current except for the particles moved by
// single moves since it was built, which are skipped there and tested from `disp_list`).
struct SingleArgs {
    DevState s;
    GridDev g;
    rp_move m;
    SingleTry *out;
    double temperature;   // soft sweeps: the Metropolis temperature
    const int32_t *disp_list;
    const uint8_t *disp_flag;
    int ndisp;
    float reach2;       // FP32 pre-filter of a body separation at one image: reach^2
    float box32[9];     // the box in FP32 (the images' translations in the pre-filter)
    int one_image;      // the reach is below 0.45 of every box height: one image per pair to test
    int has_domain;     // an ActiveDomain: relative bounds lo[3], hi[3] (ActiveDomain::RegionBounds)
    double dom_lo[3], dom_hi[3];
};

// A device sweep with a soft part: every move decided in FP64 (hard part, then the energy
// change), one warp per active cell of a checkerboard phase.
struct SoftSweepArgs {
    SingleArgs c;                  // state, grid, pre-filter reach, temperature (c.m, c.out unused)
    int phase[3], active[3], num_active;
    int32_t *next_item;
    uint64_t seed, counter;
    float tstep;
    int types;
    const double *rtab64;
    uint32_t rtab_mask;
    rp_move *log;
    uint8_t *log_codes;
    const int32_t *work;           // the phase's cells by occupancy, largest first (null: index order)
};

// One replica of a batched launch (rp_batch_*): its sweep arguments, this sweep's phase
// order, and its box move when the batch rescales it.  Particles, cells and sweep items of
// all replicas are numbered consecutively; the prefix offsets live in separate compact
// arrays that the kernels search.
struct alignas(16) BatchRep {
    SweepArgs a;
    int phases[MAX_PHASES];
    int nphases;
    int scale;                     // 1: this replica's positions are rescaled (box move)
    double old_inv[9], new_box[9];
    const double *scale_src;
    double *scale_dst;
    double *trans_dst;             // translation table of the new box
};
// table entries are copied into shared memory as float4 words: every entry, and the
// arguments at its start, must sit on a 16-byte boundary
static_assert(sizeof(BatchRep) % 16 == 0, "BatchRep size");
static_assert(alignof(BatchRep) == 16, "BatchRep alignment");

}  // namespace rp
