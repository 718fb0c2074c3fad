/*
 * rampack_gb300 — C ABI of the GB300 (sm_103a) hard-particle Monte Carlo
 * move-and-overlap engine.
 *
 * The entry points replace, for one packing held in GPU memory, the calls that the
 * reference's Simulation makes into Packing (core/Packing.h:143-466) on the hot path.
 * Each declaration names the reference interface it stands in for (paths relative to
 * the rampack source tree).  Plain pointers and sizes only; every call returns an int
 * status (RP_OK or a negative RP_ERR_*); rp_last_error() describes the last failure.
 *
 * Ownership: the library owns all device memory; host arrays passed in are copied
 * before the call returns.  One handle is driven by one host thread; all device work
 * of a handle is ordered on the handle's own CUDA stream.
 *
 * Layouts: positions are N x 3 doubles; orientations N x 9 doubles, row-major, so that
 * element (i, j) of Matrix<3,3> is rot[9*k + 3*i + j]; the box is 9 doubles, row-major,
 * whose columns are the box sides (core/TriclinicBox.h).
 */
#ifndef RAMPACK_GB300_H
#define RAMPACK_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RP_OK 0
#define RP_ERR_ARG (-1)          /* invalid argument: the reference throws PreconditionException */
#define RP_ERR_CUDA (-2)         /* a CUDA runtime call failed */
#define RP_ERR_STATE (-3)        /* call out of order (e.g. no state uploaded) */
#define RP_ERR_OVERLAP (-4)      /* the packing has overlaps where none are allowed */
#define RP_ERR_UNSUPPORTED (-5)  /* a configuration this engine does not handle */
#define RP_ERR_DEVICE (-6)       /* a device-side check failed (status word set by a kernel) */
#define RP_ERR_CAPACITY (-7)     /* a per-cell capacity was exceeded */
#define RP_ERR_FORMAT (-8)       /* a broken file: the reference throws RamsnapException / RamtrjException */
#define RP_ERR_IO (-9)           /* a file could not be opened, read or written */

#define RP_SHAPE_SPHERE 0
#define RP_SHAPE_SPHEROCYLINDER 1
#define RP_SHAPE_POLYSPHERE 2     /* created by rp_create_polysphere */
#define RP_SHAPE_CONVEX 3         /* generic convex body, created by rp_create_convex */
#define RP_MAX_CENTRES 8          /* spheres per polysphere */

#define RP_MOVE_TRANSLATION 0
#define RP_MOVE_ROTATION 1
#define RP_MOVE_ROTOTRANSLATION 2

/* Outcome code of one move (rp_run_moves, rp_sweep logs): the low two bits give the
 * energy class returned by Packing::tryTranslation / tryRotation / tryMove
 * (core/Packing.cpp:84-164): 0 = dE 0, 1 = overlap (+inf), 2 = outside the active
 * domain (+inf, ActiveDomain::isInside false), 3 = -inf (overlap counting only);
 * bit 7 is set when the Metropolis test accepted the move (core/Simulation.cpp:483). */
#define RP_CODE_ACCEPTED 0x80

/* Shape descriptor: the closed set of hard interactions the engine evaluates on the
 * GPU; a host caller builds it from SphereTraits(r) (core/shapes/SphereTraits.h:16) or
 * SpherocylinderTraits(l, r) (core/shapes/SpherocylinderTraits.h:16). */
typedef struct rp_shape_desc {
    int32_t kind;
    int32_t reserved;
    double radius;
    double length;
} rp_shape_desc;

/* One proposed particle move, as MoveSampler::MoveData (core/MoveSampler.h:40-49) plus
 * the Metropolis uniform that Simulation::tryMove draws for it (core/Simulation.cpp:483).
 * `domain` is the linear index of the active cell of the engine's cell grid in which
 * the move is made (rp_get_grid); it is the ActiveDomain of the move. 120 bytes. */
typedef struct rp_move {
    int32_t particle;
    int32_t type;
    int32_t domain;
    int32_t reserved;
    double translation[3];
    double rotation[9];
    double uniform;
} rp_move;

/* The engine's checkerboard cell grid (the GPU counterpart of the reference's
 * DomainDecomposition, core/DomainDecomposition.cpp:36-117). Cells are the active
 * domains; cell (x, y, z) has linear index x + dims[0] * (y + dims[1] * z). */
typedef struct rp_grid_info {
    int32_t dims[3];
    int32_t max_occupancy;
    double shift[3];           /* relative origin of cell (0, 0, 0) */
    double cell_height[3];     /* absolute cell heights */
    int64_t num_cells;
} rp_grid_info;

/* Parameters of one device-driven sweep (the GPU counterpart of one
 * Simulation::performMovesWithDomainDivision pass, core/Simulation.cpp:396-445). */
typedef struct rp_sweep_params {
    double translation_step;      /* TranslationSampler step; 0 disables translations */
    double rotation_step;         /* RotationSampler step; 0 disables rotations */
    uint64_t seed;                /* Philox key */
    uint64_t counter;             /* Philox counter base (e.g. the cycle number) */
    int32_t flags;                /* RP_SWEEP_* */
    int32_t reserved;
} rp_sweep_params;

#define RP_SWEEP_LOG 1            /* record every proposal and outcome (rp_sweep_log) */
#define RP_SWEEP_FP64_ONLY 2      /* decide every pair in FP64 (no FP32 filter) */
#define RP_SWEEP_ROTOTRANSLATION 4 /* RototranslationSampler (core/move_samplers/RototranslationSampler.cpp:22-48):
                                      N moves, each a translation and a rotation together (both steps > 0) */

typedef struct rp_sweep_stats {
    uint64_t moves;
    uint64_t accepted;
    uint64_t rejected_overlap;
    uint64_t rejected_domain;
    uint64_t pair_tests;          /* candidate pairs the FP32 filter examined (scans stop at a certain overlap) */
    uint64_t fp64_pairs;          /* pairs re-decided in FP64 (the guard band) */
    uint64_t translations;
    uint64_t rotations;
    uint64_t kernel_launches;     /* kernels this library launched (all calls since creation) */
    uint64_t accepted_translations; /* accepted translations (accepted rotations: accepted minus these) */
} rp_sweep_stats;

/* Kernel groups timed by rp_get_timing. */
#define RP_KERNEL_SWEEP 0         /* checkerboard move sweep (one launch per phase; the sweep's rotation table) */
#define RP_KERNEL_REBUILD 1       /* cell-grid rebuild (assign, scan, scatter, finish) */
#define RP_KERNEL_COUNT 2         /* all-pairs overlap recount */
#define RP_KERNEL_RESCALE 3       /* box rescale (and the kept-grid remap of a box move) */
#define RP_KERNEL_OVERFLOW 4      /* large-capacity rerun of oversized neighbourhoods */
#define RP_KERNEL_ORDER 5         /* partner ranking of the learned ordering */
#define RP_KERNEL_MLP 6           /* ranking-network training and inference */
#define RP_KERNEL_FIX 7           /* orientation renormalisation */
#define RP_KERNEL_SINGLE 8        /* unrestricted single moves (rp_try_move / rp_accept_move) */
#define RP_NUM_KERNELS 9

/* ---- lifetime ---------------------------------------------------------------------- */

/* Creates an engine for n particles of one shape on CUDA device `device`.
 * Replaces: Packing::Packing(box, shapes, bc, interaction, moveThreads, scalingThreads)
 * (core/Packing.h:152-168) together with Packing::reset (core/Packing.cpp:67-82); the
 * state itself arrives through rp_upload_state. */
int rp_create(const rp_shape_desc *shape, int64_t n, int device, void **handle);

/* Creates an engine for n polyspheres: rigid bodies of num_centres hard spheres
 * (1..RP_MAX_CENTRES) with body-frame centres (num_centres x 3) and radii.
 * Replaces: Packing::Packing(..., PolysphereTraits(sphereData)) (core/Packing.h:152-168,
 * core/shapes/PolysphereTraits.h) with Packing::setupForInteraction
 * (core/Packing.cpp:931-950); bent chains (PolysphereBananaTraits) pass their generated
 * sphere data.  Each particle carries the reference's rotated centres and absolute centres
 * (core/Packing.cpp:1035-1047, :357-361). */
int rp_create_polysphere(int32_t num_centres, const double *centres, const double *radii, int64_t n, int device,
                         void **handle);

/* Creates an engine for n polyspherocylinders: rigid bodies of num_centres hard
 * spherocylinders (1..RP_MAX_CENTRES) with body-frame centres, half axes (num_centres x 3
 * each; the segment runs from centre - half axis to centre + half axis) and radii.
 * Replaces: Packing::Packing(..., PolyspherocylinderTraits(spherocylinderData))
 * (core/shapes/PolyspherocylinderTraits.h:26-60).  The handle behaves as a polysphere one
 * (interaction centres rotated with the body) whose centre pairs are decided as
 * PolyspherocylinderTraits::overlapBetween (PolyspherocylinderTraits.cpp:102-124): inspheres
 * (r_a + r_b), circumspheres (c_a + c_b, c = r + |half axis|), then the segment distance. */
int rp_create_polyspherocylinder(int32_t num_centres, const double *centres, const double *half_axes,
                                 const double *radii, int64_t n, int device, void **handle);

/* Creates an engine for n generic convex bodies (GenericXenoCollideTraits,
 * core/shapes/GenericXenoCollideTraits.h) described by an XCBodyBuilder script: the commands
 * of XCBodyBuilder::processCommand (geometry/xenocollide/XCBodyBuilder.cpp:194-294) -- point,
 * segment, rectangle, cuboid, disk, sphere, ellipse, ellipsoid, football, saucer, move, rot,
 * sum [k], diff, wrap [k], dup k, pop, swap -- one per line or separated by ';'.  Pairs are
 * decided as XenoCollideTraits::overlapBetween (core/shapes/XenoCollideTraits.h:147-168):
 * circumspheres, inspheres, then XenoCollide's portal refinement with tolerance 1e-12, every
 * move in FP64.  Sweeps, single moves, overlap counts and counting mode, box moves, hard walls
 * (XenoCollideTraits::overlapWithWall, core/shapes/XenoCollideTraits.h:170-186) and orientation
 * fixes; not move lists, soft parts, rototranslations or the learned ordering
 * (RP_ERR_UNSUPPORTED).
 * An invalid script fails with RP_ERR_ARG and the builder's message in rp_last_error(NULL). */
int rp_create_convex(const char *script, int64_t n, int device, void **handle);

/* XenoCollideTraits::overlapBetween of the handle's convex body on n independent pairs
 * (positions n x 3, orientations n x 9, the second body at its given position: no periodic
 * image), decided on the device; out[i] = 1 for an overlap.  For parity checks of the support
 * functions and the portal refinement. */
int rp_convex_pair_overlaps(void *handle, int64_t n, const double *pos1, const double *rot1, const double *pos2,
                            const double *rot2, uint8_t *out);

/* Releases the handle and all of its device memory. */
int rp_destroy(void *handle);

/* Text of the last error on this handle (never NULL; empty when none).  With a NULL handle:
 * why the last rp_create* call of this thread failed on the device (no CUDA device, out of
 * memory, ...), else "null handle". */
const char *rp_last_error(void *handle);

/* ---- state ------------------------------------------------------------------------- */

/* Copies positions, orientations and the box to the device and builds the cell grid.
 * Replaces: Packing::reset / Packing::restore (core/Packing.cpp:67-82, :961-964).
 * Fails with RP_ERR_ARG when a particle lies outside the box (areShapesWithinBox,
 * core/Packing.cpp:1069-1075). */
int rp_upload_state(void *handle, const double *pos, const double *rot, const double *box9);

/* Copies the FP64 state back (positions, orientations, box); any pointer may be NULL.
 * Replaces: iteration over Packing (core/Packing.h:190-203) and Packing::getBox. */
int rp_download_state(void *handle, double *pos, double *rot, double *box9);

/* ---- overlap counting -------------------------------------------------------------- */

/* Counts all overlapping pairs (each pair and periodic image once); with early_exit the
 * count is 0 or 1.  Replaces: Packing::countTotalOverlaps(interaction, earlyExit)
 * (core/Packing.cpp:519-559). */
int rp_count_overlaps(void *handle, int early_exit, int64_t *out_count);

/* ---- particle moves ---------------------------------------------------------------- */

/* Rebuilds the checkerboard cell grid with the given relative shift of its origin
 * (each component in [0, 1)) and reports its layout.  Replaces the construction of
 * DomainDecomposition with a random origin (core/Simulation.cpp:401-411). */
int rp_set_grid(void *handle, const double *shift3, rp_grid_info *info);

/* Reports the current grid (info), the cell of every particle (linear cell index, n
 * int32) and the ActiveDomain bounds of every cell (6 doubles per cell: lo[3] then
 * hi[3], relative coordinates; ActiveDomain::RegionBounds, core/ActiveDomain.h:19-31).
 * Any output pointer may be NULL. */
int rp_get_grid(void *handle, rp_grid_info *info, int32_t *cell_of_particle, double *bounds);

/* Executes a list of proposed moves, in order, with the reference's semantics for hard
 * bodies: each move is Packing::tryTranslation / tryRotation / tryMove with the move's
 * cell as ActiveDomain (core/Packing.cpp:84-164), then the Metropolis test with the
 * move's uniform and Packing::acceptMove on success (core/Simulation.cpp:466-490).
 * Consecutive moves whose cells share a checkerboard colour form one phase; the cells
 * of a phase run concurrently, one warp each, and every move's particle must belong to
 * its cell.  out_codes (n bytes, optional) receives the outcome codes. */
int rp_run_moves(void *handle, const rp_move *moves, int64_t n, uint8_t *out_codes);

/* One move: Packing::tryTranslation / tryRotation / tryMove (core/Packing.cpp:84-164).
 * domain6 NULL is std::nullopt, the reference's serial path
 * (Simulation::performMovesWithoutDomainDivision, core/Simulation.cpp:365-390); otherwise an
 * ActiveDomain given by its relative bounds lo[3], hi[3] (ActiveDomain::RegionBounds
 * beg / end, core/ActiveDomain.h:19-31), which a translation or rototranslation must stay
 * inside (checked before any overlap, as the reference does).  Uses move->particle, type,
 * translation and rotation (move->domain and uniform are ignored); the tried state stays on
 * the device, and *dE receives the move's energy: 0 or +inf, in overlap counting -inf, 0 or
 * +inf (core/Packing.cpp:304-323).  One launch; synchronous.  A tried move is forgotten by
 * any call that changes the packing. */
int rp_try_move(void *handle, const rp_move *move, const double *domain6, double *dE);

/* Commits the state the last rp_try_move tried.  Replaces: Packing::acceptTranslation /
 * acceptRotation / acceptMove (core/Packing.cpp:234-302).  RP_ERR_STATE when no tried
 * move is pending.  Stream-ordered (no synchronisation); later sweeps, recounts and box
 * moves rebuild the cell grid first, later single moves do not. */
int rp_accept_move(void *handle);

/* One device-driven sweep: a random grid shift, then the 8 checkerboard phases in a
 * random order; every active cell performs (number of move types) x (occupancy) moves
 * drawn from a Philox stream.  Replaces one Simulation::performMovesWithDomainDivision
 * (core/Simulation.cpp:396-445).  stats may be NULL. */
int rp_sweep(void *handle, const rp_sweep_params *params, rp_sweep_stats *stats);

/* Copies the proposals and outcomes logged by the last rp_sweep run with RP_SWEEP_LOG,
 * in an order that replays serially to the same result (phase by phase, each cell's
 * moves in order).  *count receives the number of moves; moves/codes may be NULL to
 * query the count. */
int rp_sweep_log(void *handle, rp_move *moves, uint8_t *codes, int64_t capacity, int64_t *count);

/* ---- box moves --------------------------------------------------------------------- */

/* Rescales all positions to a new box (relative coordinates kept), rebuilds the grid
 * and recounts overlaps in one pass; *dE receives +inf on overlap and 0 otherwise.
 * A convex shape in a box that only grew is not checked, as in the reference.
 * Replaces: Packing::tryScaling(const TriclinicBox &, interaction)
 * (core/Packing.cpp:172-208). */
int rp_try_scaling(void *handle, const double *new_box9, double *dE);

/* Restores the state from before the last rp_try_scaling (buffer swap, no copy).
 * Replaces: Packing::revertScaling (core/Packing.cpp:363-371). */
int rp_revert_scaling(void *handle);

/* Overlap counting.  Replaces: Packing::toggleOverlapCounting / getCachedNumberOfOverlaps
 * (core/Packing.cpp:1049-1060).  With counting on, a move's energy is the sign of the change
 * of the mover's overlap count (core/Packing.cpp:304-323): outcome code 3 (dE = -inf, always
 * accepted) when it falls, 1 (+inf) when it grows, 0 when it stays; an accepted move adds its
 * change to the cached total; a box move recounts everything (dE = -inf / 0 / +inf by the
 * change of the total) and rp_revert_scaling restores the count.  Turning counting on counts
 * all overlaps first.  Every shape. */
int rp_set_counting(void *handle, int on);
int rp_cached_overlaps(void *handle, int64_t *count);

/* Orientation renormalisation.  Replaces: Packing::renormalizeOrientations(interaction,
 * allowOverlaps) (core/Packing.cpp:1178-1212) as Simulation::fixRotationMatrices calls it
 * (core/Simulation.cpp:750-760).  Without allow_overlaps every particle, in index order,
 * tries its orientation after three Newton-Schulz steps (core/Packing.cpp:1214-1219) as a
 * rotation move and keeps it unless it then overlaps; *rejected = the particles that kept
 * their old orientation.  With allow_overlaps the reference resets the packing with the
 * shapes as they were before the fix (so orientations do not change) and recomputes the
 * polysphere centres from the body frame; this call does the same and reports 0. */
int rp_renormalize_orientations(void *handle, int allow_overlaps, int64_t *rejected);

/* Nematic order of the current state: NematicOrder::calculate
 * (core/observables/NematicOrder.cpp:9-56).  q9 (row-major, may be NULL) receives
 * Q = 1/2 (3 <u u^T> - I) over the particles' primary axes (orientation column 2), *p2 the
 * eigenvalue of largest magnitude (Cardano, as the reference).  The sums are reduced on the
 * device in a fixed order, so Q matches the reference's serial sum to rounding (~1e-15
 * relative), not bit for bit.  Spheres have no primary axis: RP_ERR_UNSUPPORTED. */
int rp_nematic_order(void *handle, double *q9, double *p2);

/* ---- statistics --------------------------------------------------------------------- */

/* Cumulative counters of all sweeps and move lists since creation. */
int rp_get_stats(void *handle, rp_sweep_stats *stats);

/* Packing::getNeighbourGridRebuilds (core/Packing.h:423): full cell-grid rebuilds since
 * creation; and the box moves whose grid kept the old cells (same divisions and origin,
 * every particle still in its cell: one pass recomputes the FP32 cell-local positions,
 * giving the grid a rebuild would build). */
int rp_get_grid_counters(void *handle, uint64_t *rebuilds, uint64_t *remaps);

/* The cudaStream_t on which all device work of the handle runs (for the caller's own
 * CUDA events); no reference counterpart (the reference is CPU-only). */
int rp_get_stream(void *handle, void **stream);

/* Turns per-kernel-group device timing on (CUDA events recorded around every launch
 * group on the handle's stream) or off; turning it on clears the accumulated times. */
int rp_set_timing(void *handle, int on);

/* Accumulated device time (ms) and launch-group count per kernel group
 * (RP_NUM_KERNELS entries each) since timing was turned on; synchronizes the stream. */
int rp_get_timing(void *handle, double *ms, uint64_t *groups);

/* ---- learned ordering of overlap tests ----------------------------------------------
 * No reference counterpart: the reference tests a mover against its neighbour-grid cells in
 * cell order (countParticleOverlaps, core/Packing.cpp:373-430).  Here a small network (13 pair features -> 64 -> 64
 * -> 1, ReLU, BF16 weights on the tensor cores, FP32 accumulation) scores each particle's
 * in-range neighbours every few sweeps; the sweep pre-tests a mover's best-ranked
 * partners before its full neighbourhood scan and stops early only on a certain overlap, so
 * every decision, and the state after every sweep, is the plain sweep's.  The network is
 * trained on the device from pair outcomes the sweep logs (forward, backward and Adam
 * kernels of this library). */

#define RP_MLP_NPARAM 5313        /* W1[64][16], b1[64], W2[64][64], b2[64], w3[64], b3 (FP32) */
#define RP_MLP_FEATURES 16        /* per pair: 13 features, 3 zeros */

#define RP_ORDER_OFF 0            /* plain cell-order scan */
#define RP_ORDER_MLP 1            /* partners ranked by the network */
#define RP_ORDER_DISTANCE 2       /* partners ranked by centre distance (untrained ordering) */

/* Sets the network's parameters to a seeded random initialisation (He-uniform weights,
 * zero biases); the Adam state is cleared.  A new handle starts from seed 0. */
int rp_mlp_init(void *handle, uint64_t seed);

/* Copies RP_MLP_NPARAM FP32 parameters to / from the host (layout above). */
int rp_mlp_set_params(void *handle, const float *params);
int rp_mlp_get_params(void *handle, float *params);

/* Logits of n pairs (host arrays: feats n x RP_MLP_FEATURES, logits n) by the tensor-core
 * inference path the ranking uses. */
int rp_mlp_predict(void *handle, const float *feats, int64_t n, float *logits);

/* Gradient (RP_MLP_NPARAM floats) and value of the mean binary cross-entropy of the logits
 * of n labelled pairs (labels 0/1), computed by the training kernels. */
int rp_mlp_gradient(void *handle, const float *feats, const uint8_t *labels, int64_t n, float *grad,
                    float *loss);

/* Pair-outcome log: with capacity > 0, every `every`-th move of each later sweep appends
 * the pairs that reached its segment test (features before the move, label 1 if the moved
 * pair overlaps for certain, 0 if it certainly does not) until `capacity` pairs are held.
 * capacity 0 turns logging off and frees the log. */
int rp_pair_log_enable(void *handle, int64_t capacity, int32_t every);

/* Copies up to `capacity` logged pairs to the host (either pointer may be NULL) and reports
 * how many the log holds in *count; rp_pair_log_clear empties it. */
int rp_pair_log_read(void *handle, float *feats, uint8_t *labels, int64_t capacity, int64_t *count);
int rp_pair_log_clear(void *handle);

/* Trains the network on the logged pairs: `epochs` passes of Adam (learning rate lr) over
 * the log in batches of `batch` pairs, visited in a seeded shuffled order.  *loss (may be
 * NULL) receives the mean batch loss of the last epoch. */
int rp_mlp_train(void *handle, int32_t epochs, int32_t batch, float lr, uint64_t seed, float *loss);

/* Chooses the ordering of later sweeps (RP_ORDER_*), re-ranking every `every` sweeps. */
int rp_set_ordering(void *handle, int32_t mode, int32_t every);

/* ---- batched replicas -----------------------------------------------------------------
 * No single reference counterpart: many independent packings of one shape (spheres or
 * spherocylinders) advanced together, as a set of rampack Simulations would be, but with
 * every device step covering all replicas in one launch (one persistent sweep launch per
 * checkerboard phase for the whole batch).  Replica r behaves exactly as a handle would
 * under rp_sweep with the seed seed + RP_BATCH_SEED_STRIDE * r, except that all replicas draw
 * rotations from one table per sweep (from the batch seed and counter); its logged sweeps
 * replay on the reference's Packing like a handle's.  Box moves stay host-driven
 * (Simulation::tryScaling, core/Simulation.cpp:493-531): the caller proposes a box per
 * replica and the batch rescales, rebuilds and recounts all proposing replicas at once. */

/* Replica r's sweep seed: seed + 0x9E3779B97F4A7C15 * r (mod 2^64). */
#define RP_BATCH_SEED_STRIDE 0x9E3779B97F4A7C15ull

int rp_batch_create(const rp_shape_desc *shape, int32_t replicas, const int64_t *n, int device, void **batch);
int rp_batch_destroy(void *batch);
const char *rp_batch_last_error(void *batch);

/* Per replica, as rp_upload_state / rp_download_state / rp_count_overlaps / rp_get_grid /
 * rp_sweep_log on a handle. */
int rp_batch_upload_state(void *batch, int32_t replica, const double *pos, const double *rot, const double *box9);
int rp_batch_download_state(void *batch, int32_t replica, double *pos, double *rot, double *box9);
int rp_batch_count_overlaps(void *batch, int32_t replica, int early_exit, int64_t *count);
int rp_batch_get_grid(void *batch, int32_t replica, rp_grid_info *info, int32_t *cells, double *bounds);
int rp_batch_sweep_log(void *batch, int32_t replica, rp_move *moves, uint8_t *codes, int64_t capacity,
                       int64_t *count);

/* One sweep of every replica (2 N_r moves each with both steps > 0); stats (may be NULL)
 * receives one entry per replica. */
int rp_batch_sweep(void *batch, const rp_sweep_params *params, rp_sweep_stats *stats);

/* Box moves: replicas with propose[r] != 0 move to boxes[9 r ..]; dE[r] = +inf if the new
 * box makes an overlap (the caller then reverts those), else 0.  As Packing::tryScaling /
 * revertScaling per replica (core/Packing.cpp:172-208, :363-371). */
int rp_batch_try_scaling(void *batch, const double *boxes, const uint8_t *propose, double *dE);
int rp_batch_revert_scaling(void *batch, const uint8_t *mask);

/* Launch shape: checkerboard cells at least cell_factor (>= 1) interaction ranges high and
 * 2, 4 or 8 warps per block of the sweep kernel (defaults 1.0 and 4). */
int rp_batch_set_tuning(void *batch, double cell_factor, int32_t warps_per_block);
/* rp_set_staging_filter for every replica. */
int rp_batch_set_staging_filter(void *batch, int32_t mode);

/* Every replica's state at once: pos [sum n][3], rot [sum n][9] with the replicas' particles
 * in replica order, boxes [R][9].  The upload copies on the batch's stream (one copy per
 * array and replica), rebuilds every replica's cell grid in one batched launch and checks
 * that each particle lies inside its box; the download waits for the batch's work. */
int rp_batch_upload_states(void *batch, const double *pos, const double *rot, const double *boxes);
int rp_batch_download_states(void *batch, double *pos, double *rot, double *boxes);

/* Per-group device timing of the batch's own launches (RP_KERNEL_* groups), as
 * rp_set_timing / rp_get_timing; `launches` (may be null) receives the kernels launched by
 * the batch and its replicas since creation. */
int rp_batch_set_timing(void *batch, int on);
int rp_batch_get_timing(void *batch, double *ms, uint64_t *groups, uint64_t *launches);

/* ---- allocation-free overlap count ----------------------------------------------- */

/* Limits of rp_count_overlaps_static and the size of the scratch array behind it. */
#define RP_STATIC_MAX_PARTICLES 65536
#define RP_STATIC_MAX_CELLS 65536
#define RP_STATIC_SCRATCH_BYTES (5 * 1024 * 1024)

/* Counts overlapping pairs (as rp_count_overlaps) of a packing the caller already holds in
 * its own device memory, without allocating any memory.  This entry point has no
 * counterpart in the reference.  It is for callers that may not allocate: a host
 * framework that budgets or pools all device memory itself, or a stream-ordered pipeline
 * in which cudaMalloc/cudaFree would implicitly synchronise the device and stall its other
 * streams.  Inputs: d_pos (n x 3 doubles) and d_rot (n x 9 doubles) in device memory of the
 * current CUDA device (anything else, a host array for instance, is refused with
 * RP_ERR_ARG before any launch), box9 and shape on the host.  The call is synchronous: its
 * work is ordered on `stream` (a cudaStream_t, NULL for the default stream), and the call
 * waits for it and writes the count to *out_count (host).  Working memory is one fixed
 * array of RP_STATIC_SCRATCH_BYTES compiled into the library, which every GPU that loads
 * the library keeps until the process exits: n above RP_STATIC_MAX_PARTICLES is rejected
 * with RP_ERR_CAPACITY (dilute packings get cells larger than the interaction range, so the
 * grid stays within RP_STATIC_MAX_CELLS).  The first call on a device looks up the array's
 * device address (with that device current) and keeps it, so make the first call before
 * any stream capture, and make no call on a device after cudaDeviceReset.  All calls share
 * the array: calls whose GPU work overlaps (from several host threads or streams) race and
 * must be serialised by the caller. */
int rp_count_overlaps_static(const rp_shape_desc *shape, int64_t n, const double *d_pos, const double *d_rot,
                             const double *box9, int early_exit, void *stream, int64_t *out_count);

/* Packing::toggleWalls (core/Packing.cpp:1075-1084): bit i of `mask` puts hard walls on the
 * two planes across box side i (through the origin and through the far corner; periodic
 * images are kept, as in the reference).  Every move, recount, box move and orientation fix
 * then counts wall overlaps (core/Packing.cpp:1086-1139) after the pair overlaps. */
int rp_set_walls(void *handle, int32_t mask);
int rp_batch_set_walls(void *batch, int32_t mask);

/* ---- soft interactions ----------------------------------------------------------- */

#define RP_SOFT_NONE 0
#define RP_SOFT_REPULSIVE_LJ 1          /* RepulsiveLennardJonesInteraction(epsilon, sigma) (WCA) */
#define RP_SOFT_SQUARE_INVERSE_CORE 2   /* SquareInverseCoreInteraction(epsilon, sigma) */
#define RP_SOFT_LENNARD_JONES 3         /* LennardJonesInteraction: refused (no cut-off, see rp_set_soft) */

/* Joins a central potential on the shape's interaction centres (the particle position; the
 * centres of polyspheres) to its hard interaction, as CompoundShapeTraits /
 * CompoundInteraction do (core/interactions/CompoundInteraction.cpp:9-49) for casino's
 * overlap relaxation with a helper shape (frontend/modes/CasinoMode.cpp:288-289); hard = 0
 * keeps the soft part alone (SphereTraits(r, centralInteraction), PolysphereTraits(geometry,
 * centralInteraction); spheres and polyspheres).  kind RP_SOFT_NONE removes it.  Moves then
 * return the energy change (core/Packing.cpp:103-108), box moves the change of the total
 * energy (:172-207); sweeps decide every move in FP64 at the handle's temperature; move lists
 * (rp_run_moves) are refused.  Lennard-Jones is refused: it has no cut-off, so the
 * reference's particle energy sums over whatever its neighbour-grid cells hold. */
int rp_set_soft(void *handle, int32_t kind, double epsilon, double sigma, int32_t hard);
/* The Metropolis temperature of sweeps with a soft part (default 1; rp_sim sets it). */
int rp_set_temperature(void *handle, double temperature);
/* Packing::getTotalEnergy (core/Packing.cpp:689-764): the soft energy of all pairs. */
int rp_total_energy(void *handle, double *energy);

/* Cells a warp sweeps at once in the plain scans of spheres and spherocylinders: 1 (a warp
 * per cell), or 2 (each half-warp sweeps its own cell with the axes read from the FP32 mirror,
 * twice the cells in flight per SM).  Decisions and the proposal stream are the same either
 * way; learned ordering, pair logs, overlap counting, rototranslations, polyspheres and
 * neighbourhoods above the half-warp capacity keep a warp per cell. */
int rp_set_cells_per_warp(void *handle, int32_t cells);
/* Cells per warp the last sweep used (1 or 2; 0 before the first sweep). */
int rp_get_cells_per_warp(void *handle, int32_t *last);

/* Staging filter of the sweep: candidates of the 26 neighbour cells farther than the
 * interaction range from every face-slab of the mover's cell (its ActiveDomain) are not
 * staged; decisions are unchanged.  0 off, 1 (default) where cells are well above the range
 * (keeps < 90 % of the neighbourhood), 2 wherever no grid dimension has a single cell. */
int rp_set_staging_filter(void *handle, int32_t mode);
/* How a sweep stages each cell's 3x3x3 neighbourhood into shared memory: 1 with bulk
 * asynchronous copies (cp.async.bulk, one per neighbour cell and array, completing on an
 * mbarrier with a bounded wait), 0 with per-lane loads.  Decisions, states and the proposal
 * stream are the same either way; the two-cells-per-warp path, the staging filter, the FP64
 * sweeps (soft parts, convex bodies) and batched replicas always use per-lane loads.  A lost
 * copy sets a device status (RP_ERR_DEVICE) instead of waiting. */
int rp_set_bulk_staging(void *handle, int32_t on);
/* The order in which a plain sweep's persistent warps take the cells of a checkerboard phase:
 * 1 (default) by occupancy, largest first (a counting sort after each grid change, so a phase
 * ends on short cells), 0 in cell-index order.  Cells of one phase are never neighbours, so
 * decisions, logs and states are the same either way. */
int rp_set_cell_order(void *handle, int32_t on);

/* ---- the Monte Carlo cycle loop (Simulation for hard bodies) -----------------------
 *
 * Simulation::performCycle (core/Simulation.cpp:325-363) around a handle: one device sweep
 * of translations and rotations at the current step sizes, then a box move proposed by
 * the reference's TriclinicBoxScaler family from a std::mt19937 (seeded like the
 * Simulation's first generator) and pre-checked on the host (Simulation::tryScaling,
 * :493-531, incl. the overlap-counting branch); with `adjust_steps` the thermalisation's
 * step-size adaptation (Simulation::evaluateCounters, :533-607: every 100·N moves of a
 * sampler, or 100 box moves, the step grows by 1.1 above 20 % acceptance and shrinks below
 * 10 %; translations stop at half the smallest box height, rotations at pi). */
#define RP_SCALER_NONE 0
#define RP_SCALER_DELTA_TRICLINIC 1  /* TriclinicDeltaScaler (core/volume_scalers/TriclinicDeltaScaler.cpp:7-25) */
#define RP_SCALER_LOG 2              /* TriclinicAdapter + AnisotropicVolumeScaler + LogScalingFactorSampler */
#define RP_SCALER_LINEAR 3           /* TriclinicAdapter + AnisotropicVolumeScaler + LinearScalingFactorSampler */
#define RP_SCALER_DELTA_VOLUME 4     /* TriclinicAdapter + DeltaVolumeScaler */

typedef struct rp_box_scaler_desc {
    int32_t kind;            /* RP_SCALER_* */
    int32_t scale_together;  /* delta triclinic: every entry moves (1) or one random side (0) */
    int32_t num_groups;      /* log / linear: the scaling directions, 1-3 ... */
    int32_t groups[3];       /* ... each a mask of axes scaled by one factor (1 x, 2 y, 4 z; 7 isotropic) */
    int32_t independent;     /* one random direction per move (1) or the product over all (0) */
    int32_t reserved;
    double step;             /* initial step size */
} rp_box_scaler_desc;

typedef struct rp_sim_params {
    double temperature;
    double pressure;
    double translation_step;  /* initial TranslationSampler step; 0 disables translations */
    double rotation_step;     /* initial RotationSampler step; 0 disables rotations */
    rp_box_scaler_desc scaler;
    uint64_t seed;            /* the box moves' std::mt19937 seed and the sweeps' Philox key */
    int32_t rototranslation;  /* one RototranslationSampler(translation_step, rotation_step) instead of
                                 the two samplers: N moves per cycle, its step rule (RototranslationSampler.cpp:50-61) */
    int32_t reserved;
} rp_sim_params;

typedef struct rp_sim_stats {
    uint64_t cycles;          /* cycles run since creation (the sweeps' Philox counters) */
    uint64_t translations, accepted_translations, rotations, accepted_rotations;  /* rototranslations count as rotations */
    uint64_t box_moves, accepted_box_moves;
    double translation_step, rotation_step, box_step;  /* current step sizes */
    double box[9];            /* current box */
    double move_ms, scaling_ms;  /* host wall clock of the sweeps and of the box moves */
} rp_sim_stats;

int rp_sim_create(void *handle, const rp_sim_params *params, void **sim);
int rp_sim_run(void *sim, int64_t cycles, int adjust_steps, rp_sim_stats *stats);
int rp_sim_get_stats(void *sim, rp_sim_stats *stats);
int rp_sim_set_steps(void *sim, double translation_step, double rotation_step, double box_step);
int rp_sim_set_conditions(void *sim, double temperature, double pressure);
/* The cycle count a continued run starts from (the next sweep's Philox counter). */
int rp_sim_set_cycles(void *sim, uint64_t cycles);
const char *rp_sim_last_error(void *sim);
int rp_sim_destroy(void *sim);

/* The box scaler alone, as Simulation::tryScaling draws from its generator: `count` times a
 * proposal from the same `box9` followed by the Metropolis uniform (boxes [count][9],
 * uniforms [count], may be null). */
int rp_box_proposals(const rp_box_scaler_desc *scaler, uint64_t seed, const double *box9, int64_t count,
                     double *boxes, double *uniforms);

/* ---- snapshot and trajectory files (RAMSNAP text, RAMTRJ binary) ------------------
 *
 * Byte for byte the reference's formats.  Errors of these calls are described by
 * rp_io_last_error() (per host thread). */
const char *rp_io_last_error(void);

/* Packing::store → RamsnapWriter::write (core/Packing.cpp:956-959,
 * core/io/RamsnapWriter.cpp:8-48): aux entries (keys without whitespace; written in key
 * order, a repeated key keeps its last value), the box, then one line per shape.  From the
 * handle's device state (downloaded through a consistent device-side snapshot), or from
 * host arrays. */
int rp_ramsnap_write(void *handle, const char *path, int32_t naux, const char *const *keys,
                     const char *const *values);
int rp_ramsnap_write_host(const char *path, int64_t n, const double *pos, const double *rot, const double *box9,
                          int32_t naux, const char *const *keys, const char *const *values);

/* Packing::restore → RamsnapReader::read (core/Packing.cpp:961-964,
 * core/io/RamsnapReader.cpp:16-96): parses a file into an opaque snapshot (old-format
 * three-number boxes are the sides of a cuboid); the state then goes to rp_upload_state.
 * Aux strings stay valid until rp_ramsnap_free. */
int rp_ramsnap_load(const char *path, void **snap);
int rp_ramsnap_info(void *snap, int64_t *n, int32_t *naux);
int rp_ramsnap_get(void *snap, double *pos, double *rot, double *box9);
int rp_ramsnap_aux(void *snap, int32_t index, const char **key, const char **value);
int rp_ramsnap_free(void *snap);

/* RamtrjRecorder (core/io/RamtrjRecorder.cpp:9-67): a trajectory of `num_particles`
 * particles, one snapshot every `cycle_step` cycles; `append` continues an existing file
 * whose header matches.  rp_ramtrj_record takes the handle's state in order with its
 * moves and returns; the download, the Euler-angle conversion and the write run while the
 * handle goes on (one snapshot in flight; the next record, flush or close waits for it).
 * `cycle` must be (recorded snapshots + 1) · cycle_step.  Close rewrites the header. */
int rp_ramtrj_open(const char *path, int64_t num_particles, int64_t cycle_step, int append, void **rec);
int rp_ramtrj_record(void *rec, void *handle, int64_t cycle);
int rp_ramtrj_record_host(void *rec, const double *pos, const double *rot, const double *box9, int64_t cycle);
int rp_ramtrj_flush(void *rec);
int rp_ramtrj_snapshots(void *rec, int64_t *count);
int rp_ramtrj_close(void *rec);

/* RamtrjPlayer (core/io/RamtrjPlayer.cpp:11-86): the header (version = 256·major + minor)
 * of a well-formed file, and snapshot `snapshot` (from 0; the reference's cycle
 * (snapshot + 1) · cycle_step) with orientations rebuilt from the Euler angles. */
int rp_ramtrj_info(const char *path, int64_t *num_particles, int64_t *snapshots, int64_t *cycle_step,
                   int32_t *version);
int rp_ramtrj_read(const char *path, int64_t snapshot, double *pos, double *rot, double *box9);

/* ---- pair correlations (core/observables/correlation) ------------------------------- */

/* PairEnumerator implementations: RadialEnumerator (RadialEnumerator.cpp:9-29, distance
 * between focal points), LinearEnumerator (LinearEnumerator.cpp:37-67, separation
 * projected on the normal of the box faces across side `linear_axis`) and
 * LayerwiseRadialEnumerator (LayerwiseRadialEnumerator.cpp:18-46, pairs in the same layer
 * of the Miller-index planes, separation projected into the layer). */
#define RP_PAIRS_RADIAL 0
#define RP_PAIRS_LINEAR 1
#define RP_PAIRS_LAYERWISE 2
/* The BulkObservable fed with the pairs: PairDensityCorrelation (PairDensityCorrelation.cpp:
 * 4-37) or PairAveragedCorrelation (PairAveragedCorrelation.cpp:4-31) of S110Correlation,
 * S220Correlation, S221Correlation or AxesAngle (core/observables/correlation_functions). */
#define RP_CORR_DENSITY 0
#define RP_CORR_S110 1
#define RP_CORR_S220 2
#define RP_CORR_S221 3
#define RP_CORR_AXES_ANGLE 4
/* ShapeGeometry::Axis of the axis correlations: orientation · primary, orientation ·
 * secondary, or (primary ^ secondary).normalized() (core/ShapeGeometry.h:65-81). */
#define RP_AXIS_PRIMARY 0
#define RP_AXIS_SECONDARY 1
#define RP_AXIS_AUXILIARY 2

/* One correlation observable: histogram [0, max_r] in num_bins bins; `focal` is the named
 * point (ShapeGeometry::getNamedPoint) in the body frame that the enumerator measures
 * from; `primary` / `secondary` are the body-frame axes (SpherocylinderTraits: primary
 * {0, 0, 1}); `miller` is read by the layerwise enumerator, `linear_axis` (0 x, 1 y, 2 z)
 * by the linear one. */
typedef struct rp_pair_desc {
    int32_t enumerator;
    int32_t linear_axis;
    int32_t miller[3];
    int32_t function;
    int32_t axis;
    int32_t num_bins;
    int32_t flags;      /* RP_CORR_ALL_PAIRS | RP_CORR_FP64_ONLY */
    int32_t reserved;
    double max_r;
    double focal[3];
    double primary[3];
    double secondary[3];
} rp_pair_desc;

/* RP_CORR_ALL_PAIRS: no cell grid, every pair examined as the reference's loops do (the
 * counts do not change; for cross-checking the grid).  RP_CORR_FP64_ONLY: every examined
 * pair decided in FP64 (no FP32 pre-filter or binning; the results do not change). */
#define RP_CORR_ALL_PAIRS 1
#define RP_CORR_FP64_ONLY 2

/* The constructors PairDensityCorrelation(enumerator, maxR, numBins) and
 * PairAveragedCorrelation(enumerator, function, maxR, numBins) with the enumerator built
 * from the same description.  max_r > 0, 1 <= num_bins <= RP_CORR_MAX_BINS. */
#define RP_CORR_MAX_BINS 65536
int rp_correlation_create(const rp_pair_desc *desc, void **corr);
/* BulkObservable::addSnapshot on the handle's current state: the pairs are enumerated and
 * binned on the GPU (bin counts exact; the FP64 separations in the reference's operation
 * order), then the snapshot is renormalised and added as HistogramBuilder does. */
int rp_correlation_add_snapshot(void *corr, void *handle);
/* HistogramBuilder::dumpValues: bin middles, values (SUM reduction: value / snapshots
 * for the density correlation; AVERAGE: value / count for the averaged ones) and the
 * accumulated counts, num_bins each.  The values printed by the reference's print(). */
int rp_correlation_values(void *corr, double *x, double *y, uint64_t *count);
/* The last snapshot's raw bins before renormalisation: pair counts and value sums. */
int rp_correlation_last_snapshot(void *corr, uint64_t *count, double *sums);
/* Snapshots added since creation or the last clear, and the pairs the last snapshot
 * tested in FP64 (after the FP32 pre-filter). */
int rp_correlation_info(void *corr, int64_t *snapshots, int64_t *pairs_tested);
int rp_correlation_clear(void *corr);
const char *rp_correlation_last_error(void *corr);
int rp_correlation_destroy(void *corr);

#ifdef __cplusplus
}
#endif

#endif /* RAMPACK_GB300_H */
