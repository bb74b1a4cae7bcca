/*
 * direbm_gb300.h -- C ABI of the GB300 (sm_103a) DiReBM library, libdirebm_gb300.so.
 *
 * Every entry point takes plain pointers and sizes, an explicit CUDA stream (cudaStream_t passed
 * as void*; NULL means the legacy default stream) and returns an int status (DBM_OK = 0).  No
 * exception crosses the ABI; dbm_last_error() returns a message for the last failure on the
 * calling process.  Pointers named d_* are device pointers owned by the caller; the simulator
 * handle owns its own state and scratch buffers (allocated at dbm_sim_create).
 *
 * Reference interfaces replaced (berfandil/DiReBM, Python + NVIDIA Warp):
 *   direbm/warp/physics.py     collide, equilibrium, default_device
 *   direbm/warp/propagation.py disperse, create_control_points, refine_control_points, resample
 *   direbm/warp/simulator.py   GpuSimulator (__init__, step, moments)
 *   direbm/warp/lbm.py         GpuHexLBM (__init__, set_pulse, step, macroscopic)
 *   Warp library primitives    wp.utils.radix_sort_pairs / runlength_encode / array_scan
 */
#ifndef DIREBM_GB300_H
#define DIREBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------- */
#define DBM_OK 0
#define DBM_ERR_INVALID 1   /* bad argument (message in dbm_last_error) */
#define DBM_ERR_CUDA 2      /* a CUDA runtime call failed */
#define DBM_ERR_CAPACITY 3  /* a capacity would be exceeded */
#define DBM_ERR_STATE 4     /* device status word reports a fault (see dbm_sim_status) */

/* ---- enums -------------------------------------------------------------------------------- */
#define DBM_D2Q7 0   /* reference lattice: direbm/constants.py:15-36 */
#define DBM_D2Q9 1   /* standard square set (new; the reference has none) */
#define DBM_D3Q13 2  /* reference icosahedral set: direbm/lattices.py:44-61 */
#define DBM_D3Q19 3  /* standard cubic set (new) */

#define DBM_FP64 0      /* f and offsets in FP64 */
#define DBM_FP32DEV 1   /* f stored as FP32 rho + FP32 deviation from rho*W; FP32 offsets */

/* ---- library ------------------------------------------------------------------------------ */
const char* dbm_last_error(void);
int dbm_version(void);
/* Number of kernels this library has launched in this process (graph replays count their
 * kernel nodes). */
unsigned long long dbm_launch_count(void);
/* Replaces direbm/warp/physics.py:21-22 default_device(): returns the CUDA device count. */
int dbm_device_count(int* count);

/* ---- BGK physics on explicit arrays --------------------------------------------------------
 * Replaces direbm/warp/physics.py:78-97 collide(f_np, tau) / equilibrium(rho_np, u_np), whose
 * Warp kernels are _collide / _equilibrium (physics.py:45-75).  Layout is the reference's: f is
 * row-major (n, Q), u is (n, D).  In place for collide. */
int dbm_collide_f32(float* d_f, int64_t n, int lattice, float tau, void* stream);
int dbm_collide_f64(double* d_f, int64_t n, int lattice, double tau, void* stream);
int dbm_equilibrium_f32(const float* d_rho, const float* d_u, int64_t n, int lattice, float* d_out, void* stream);
int dbm_equilibrium_f64(const double* d_rho, const double* d_u, int64_t n, int lattice, double* d_out, void* stream);

/* ---- device radix sort ------------------------------------------------------------------------
 * Replaces wp.utils.radix_sort_pairs (called at direbm/warp/propagation.py:138): stable
 * ascending LSD sort of (key, value) pairs over the low `key_bits` bits.  Sorts d_keys/d_vals in
 * place, using d_tmp (size from dbm_radix_sort_tmp_bytes) as scratch. */
int64_t dbm_radix_sort_tmp_bytes(int64_t n, int key_bytes);
int dbm_radix_sort_pairs_u32(uint32_t* d_keys, uint32_t* d_vals, int64_t n, int key_bits, void* d_tmp, void* stream);
int dbm_radix_sort_pairs_u64(uint64_t* d_keys, uint32_t* d_vals, int64_t n, int key_bits, void* d_tmp, void* stream);

/* The same stable sort for callers that may not allocate device memory (no counterpart in the
 * reference).  A host program that owns all device memory in its own pool, or a latency-critical
 * loop that cannot afford the device-wide synchronisation of cudaMalloc/cudaFree, cannot provide
 * the scratch buffer dbm_radix_sort_pairs_u32 asks for.  This entry point uses a fixed scratch
 * array compiled into the library instead (about 2.2 MB held on every GPU that loads it until the
 * process exits) and never allocates or frees.  At most DBM_NOALLOC_SORT_MAX_PAIRS pairs per
 * call (larger n returns DBM_ERR_CAPACITY).  The first call on each device looks up the scratch
 * address; make it before any stream capture.  That address is cached for the life of the
 * process and stays valid only while the device's context does: after cudaDeviceReset (or any
 * teardown of the primary context) do not call this entry point again in the same process.
 * Calls share the scratch: calls that overlap on the GPU race, so order them on one stream. */
#define DBM_NOALLOC_SORT_MAX_PAIRS 262144
int dbm_radix_sort_pairs_u32_noalloc(uint32_t* d_keys, uint32_t* d_vals, int64_t n, int key_bits, void* stream);

/* ---- stage functions on explicit component arrays (FP32, 2D D2Q7 layout of the reference) ---
 * disperse: direbm/warp/propagation.py:21-36,115-127.  pos_m (M,2), f_m (M,Q) -> pos_c (Q*M,2),
 * val_c (Q*M), dir_c (Q*M), component index Q*i + k. */
int dbm_disperse_f32(const float* d_pos_m, const float* d_f_m, int64_t m, int lattice, float dx,
                     float* d_pos_c, float* d_val_c, int32_t* d_dir_c, void* stream);
/* create_control_points: direbm/warp/propagation.py:39-68,130-153.  Cell key (floor(x/cs),
 * floor(y/cs)), stable radix sort, run-length encode, exclusive scan, sequential FP32 centroid
 * per run in sorted order.  d_cp_pos needs room for nc points; *p_out receives P (this call
 * synchronises the stream, as the reference's run_count.numpy() did). */
int dbm_create_control_points_f32(const float* d_pos_c, int64_t nc, float cs, float* d_cp_pos,
                                  int64_t* p_out, void* stream);
/* refine_control_points: direbm/warp/propagation.py:77-112,249-275. */
int dbm_refine_control_points_f32(const float* d_cp_pos, int64_t p, const float* d_pos_c, const float* d_val_c,
                                  const int32_t* d_dir_c, int64_t nc, float dx, int kappa_hard,
                                  float* d_new_pos, void* stream);
/* resample: direbm/warp/propagation.py:156-246 (scatter + gap fill + emit).  The scatter keeps the
 * reference's form -- each component sends (dx - d)/sw * f to every control point within dx --
 * with its float atomics (propagation.py:186) replaced by pair records, a stable sort by (control
 * point, direction) and dbm_segmented_sum_f32, so the result is deterministic.  Synchronises the
 * stream once (the record count sizes the sort).  out_f is (P, Q). */
int dbm_resample_f32(const float* d_pos_c, const float* d_val_c, const int32_t* d_dir_c, int64_t nc,
                     const float* d_cp_pos, int64_t p, float dx, const float* d_f_rest, int lattice,
                     float eps, float* d_out_pos, float* d_out_f, void* stream);
/* Reduce-by-key: d_out[k] = sum of d_vals over the run of key k in the key-sorted d_keys (n records,
 * keys < 0xffffffff); keys without records leave d_out untouched.  Warp-level segmented scans in a
 * fixed order, no float atomics: the deterministic replacement for wp.atomic_add in the reference's
 * scatter (direbm/warp/propagation.py:186), which has no entry point of its own. */
int dbm_segmented_sum_f32(const uint32_t* d_keys, const float* d_vals, int64_t n, float* d_out, void* stream);

/* ---- hexagonal D2Q7 lattice Boltzmann ------------------------------------------------------
 * Replaces direbm/warp/lbm.py:24-105 (_lbm_collide + _lbm_stream, GpuHexLBM.step) with one
 * fused push collide-stream kernel over structure-of-arrays storage, batched over independent
 * runs.  Storage of run r, direction k, node (j, i) is at index ((r*7 + k)*nj + j)*ni + i.
 *   FP64:    d_src/d_dst are double, holding f.
 *   FP32DEV: d_src/d_dst are float, holding f - W_k*rho0 (deviation from the rest state).
 * d_tau has one entry per run (double). */
int dbm_lbm_step(int precision, const void* d_src, void* d_dst, int32_t ni, int32_t nj, int32_t runs,
                 const double* d_tau, double rho0, int32_t steps, void* d_tmp, void* stream);

/* ---- macroscopic fields --------------------------------------------------------------------
 * Replaces direbm/fields.py:17-41 (bin_fields) on the device: bins n moments (x (n,2), f (n,Q)
 * FP64) onto the grid of edge arrays ex (nex) x ey (ney) with numpy histogram2d's bin rule and
 * writes per-bin mass and momentum, indexed [iy][ix].  Bins sum their moments in input order. */
int64_t dbm_bin_fields_tmp_bytes(int64_t n);
int dbm_bin_fields_f64(const double* d_x, const double* d_f, int64_t n, int lattice, const double* d_ex, int nex,
                       const double* d_ey, int ney, double* d_mass, double* d_momx, double* d_momy, void* d_tmp,
                       void* stream);
/* The same binning in 3D (the reference bins in 2D only; its hand-off notes list 3D binning as
 * needed for macroscopic 3D fields): x (n,3), f (n,Q) FP64 with a 3D lattice, edge arrays ex, ey,
 * ez, numpy histogramdd's bin rule per axis, per-bin mass and momentum indexed [iz][iy][ix].  Bins
 * sum their moments in input order.  d_tmp: dbm_bin_fields_tmp_bytes(n) bytes. */
int dbm_bin_fields3_f64(const double* d_x, const double* d_f, int64_t n, int lattice, const double* d_ex, int nex,
                        const double* d_ey, int ney, const double* d_ez, int nez, double* d_mass, double* d_momx,
                        double* d_momy, double* d_momz, void* d_tmp, void* stream);

/* ---- the fused DiReBM simulator -----------------------------------------------------------
 * Replaces direbm/warp/simulator.py:25-77 (GpuSimulator) and the pipeline it drives.  A handle
 * holds a batch of independent instances, each a box of `dims` cells of size `cell` (periodic or
 * not); moments live as (cell, offset) sorted by cell; each step runs collide, thinning + refine,
 * a radix sort of the control points, the two-pass resampling gather and the gap fill, with no
 * host synchronisation. */
typedef struct dbm_sim dbm_sim;

typedef struct {
  int32_t lattice;     /* DBM_D2Q7 ... */
  int32_t precision;   /* DBM_FP64 / DBM_FP32DEV */
  double dx;           /* dispersion distance (reference: dx) */
  double r_res;        /* resampling / refine radius (reference: dx) */
  double cell;         /* thinning cell (reference: dx / alpha) */
  int32_t kappa_hard;  /* reference: kappa_hard (constants.py:43) */
  double eps;          /* gap-fill emptiness threshold (reference GPU path: 1e-6) */
  int64_t moment_capacity; /* >= initial moment count; raised to the cell count if smaller */
} dbm_sim_desc;

typedef struct {
  int32_t dims[3];     /* cells per axis (unused axes = 1) */
  int32_t origin[3];   /* world cell index of local cell 0 */
  int32_t periodic;    /* 1 = periodic box, 0 = bounded box (leaving it sets a status bit) */
  double tau;          /* BGK relaxation time of this instance */
  double rho_rest;     /* gap-fill rest density (reference: rho_rest) */
} dbm_instance_desc;

int dbm_sim_create(const dbm_sim_desc* desc, const dbm_instance_desc* inst, int32_t n_inst, dbm_sim** out);
int dbm_sim_destroy(dbm_sim* sim);
/* Load moments: d_inst (m) instance of each moment, d_pos (m, D) world positions, d_f (m, Q). */
int dbm_sim_set_state(dbm_sim* sim, const int32_t* d_inst, const double* d_pos, const double* d_f, int64_t m,
                      void* stream);
/* dbm_sim_set_state for moments already in cell order (the order dbm_sim_get_state writes them:
 * by instance, then cell, ties in any order): the load skips the sort.  A moment out of cell order
 * sets status bit 8, as a moment outside its box does.  Same state as dbm_sim_set_state. */
int dbm_sim_set_state_sorted(dbm_sim* sim, const int32_t* d_inst, const double* d_pos, const double* d_f,
                             int64_t m, void* stream);
/* dbm_sim_set_state with float32 positions and f, the element type of the reference's GPU simulator
 * (reference: direbm/warp/simulator.py:40-41, pos_m as wp.vec2 and f_m as wp.float32), loaded in
 * float arithmetic.  Cells and offsets are bitwise those of dbm_sim_set_state on the values widened
 * to double when the cell size is a power of two.  The FP64 store holds f widened.  The FP32DEV
 * split of f (a compensated float sum for rho, exact fmaf products for rho W) is within an ulp of
 * the float64 load's.  presorted != 0 as dbm_sim_set_state_sorted. */
int dbm_sim_set_state_f32(dbm_sim* sim, const int32_t* d_inst, const float* d_pos, const float* d_f, int64_t m,
                          int32_t presorted, void* stream);
/* Advance `steps` steps (replays a captured CUDA graph when graphs are enabled). */
int dbm_sim_step(dbm_sim* sim, int32_t steps, void* stream);
/* Synchronises `stream` and returns the current moment count. */
int dbm_sim_count(dbm_sim* sim, int64_t* m, void* stream);
/* Export the state (outputs sized by dbm_sim_count), world positions and f in FP64. */
int dbm_sim_get_state(dbm_sim* sim, int32_t* d_inst, double* d_pos, double* d_f, void* stream);
/* dbm_sim_get_state as float32 (reference: direbm/warp/simulator.py:75-77, moments() reads pos_m
 * and f_m back as float32).  Positions and FP64-store f are the float64 values rounded once; FP32DEV
 * f = rho W + dev is summed in double-float and rounded once, within an ulp of the rounded float64
 * export. */
int dbm_sim_get_state_f32(dbm_sim* sim, int32_t* d_inst, float* d_pos, float* d_f, void* stream);
/* Synchronises and returns the device status word; clears it when clear != 0.  Bits: 1 a point
 * left a bounded box, 2 a capacity was exceeded, 4 a non-finite value, 8 set_state input outside
 * its box (or, for dbm_sim_set_state_sorted, out of cell order), 16 an internal consistency check
 * failed. */
int dbm_sim_status(dbm_sim* sim, uint32_t* flags, int32_t clear, void* stream);
/* Per-instance FP64 totals: mass, then momentum per axis -> d_out (n_inst, 1 + D). */
int dbm_sim_conservation(dbm_sim* sim, double* d_out, void* stream);
/* Graph capture on/off for dbm_sim_step (default on). */
int dbm_sim_use_graphs(dbm_sim* sim, int32_t on);
/* Execution options: DBM_OPT_GRAPHS (capture steps in CUDA graphs, default 1) and DBM_OPT_TILES
 * (2D: shared-memory tiled window kernels, default 1; results are bit-identical either way). */
#define DBM_OPT_GRAPHS 1
#define DBM_OPT_TILES 2
/* DBM_OPT_TILE_WIDTH (2D): tiles of w x 256/w cells, w in {8, 16, 32, 64, 128} (default 32);
 * DBM_OPT_PERSISTENT (2D): launch the tiled kernels with a few resident blocks per SM that loop
 * over the tile list (default 0).  Neither changes any result bit; direbm_gb300.autotune picks them
 * by timing. */
#define DBM_OPT_TILE_WIDTH 3
#define DBM_OPT_PERSISTENT 4
/* DBM_OPT_KAPPA_SOFT: soft-outer spawn threshold (default 0 = off).  Replaces the CPU simulator's
 * soft_mode="spawn" / kappa_soft (direbm/reference/simulator.py:126-166; the Warp path,
 * direbm/warp/propagation.py:108, treats soft_outer as inner).  A control point with
 * kappa_hard < kappa <= value also emits one new control point 2(1 - sqrt(3)/2) dx from its
 * pre-move position, along the normalised sum of the direction vectors of its components within
 * r (none when that sum is below 1e-8).  Needs a moment capacity of 2 x cells (DBM_ERR_CAPACITY
 * otherwise); runs on the untiled kernels; the tape (dbm_tape_*) refuses a simulator with it on. */
#define DBM_OPT_KAPPA_SOFT 5
/* DBM_OPT_BRICK_WIDTH: the untiled window kernels (3D, obstacles, the soft spawn, tiles off) give
 * each block a brick of 256 cells, this many along x (a power of two, 4..32 in 3D, 8..64 in 2D;
 * default 8 in 3D, 16 in 2D); results do not depend on it.  direbm_gb300.autotune picks it. */
#define DBM_OPT_BRICK_WIDTH 6
/* DBM_OPT_SHIFTED_WINDOWS (2D, FP32 store): when every displacement c * dx / cell is a whole
 * number of cells (D2Q9 with dx = cell) and r < 2 cells, the tiled kernels build one table of
 * window rows per reference point and shift it for each direction instead of building a window
 * per (point, direction) (default 1).  Results are bit-identical either way. */
#define DBM_OPT_SHIFTED_WINDOWS 7
/* DBM_OPT_DENSE_STENCIL (2D, FP32 store, with the shifted windows): a tile whose cells each hold at
 * most two moments and two control points (in D2Q9 runs with dx = cell, almost every cell holds
 * exactly one) is staged as a dense grid -- second items in a per-tile list of 32 -- and every
 * window becomes a fixed 4 x 4 block of cells; other tiles take the row-segment loops in a second
 * launch (default 1).  Results are bit-identical either way. */
#define DBM_OPT_DENSE_STENCIL 8
int dbm_sim_get_brick_width(dbm_sim* sim, int32_t* brick_width);
int dbm_sim_set_option(dbm_sim* sim, int32_t option, int32_t value);
int dbm_sim_get_tiling(dbm_sim* sim, int32_t* tile_width, int32_t* persistent);
/* Run one step but stop after `stage` (1 collide, 2 thin+refine, 3 sort, 4 weights, 5 gather,
 * 6 emit) so intermediates can be exported with dbm_sim_trace. */
int dbm_sim_step_partial(dbm_sim* sim, int32_t stage, void* stream);
/* Run one full step stage by stage (no graph) with CUDA events recorded on the stream the kernels
 * run on; stage_ms[6] receives the durations of: collide, thin+refine, compaction+sort+finalize,
 * weights, gather, emit.  Synchronises. */
int dbm_sim_profile_step(dbm_sim* sim, float* stage_ms, void* stream);
/* Copy an internal buffer (DBM_TRACE_*) into d_dst (bytes given); *needed returns its size. */
int dbm_sim_trace(dbm_sim* sim, int32_t what, void* d_dst, int64_t bytes, int64_t* needed, void* stream);
/* Device memory held by the handle. */
int64_t dbm_sim_device_bytes(dbm_sim* sim);
/* Replace every instance's tau (n = number of instances, each > 1/2).  Synchronises.  The
 * reference fixes tau at construction (warp/simulator.py:25-44); a new tau is what a gradient
 * step on tau needs. */
int dbm_sim_set_tau(dbm_sim* sim, const double* h_tau, int32_t n);
/* Obstacles and inflow (config 3; the reference's obstacles are CPU-only, reference/boundary.py and
 * reference/simulator.py:105-117, with a specular bounce and a direction split).  A solid sphere
 * (disc in 2D) of `radius` (world units) at `center` (D world coordinates) in instance `inst`;
 * radius <= 0 removes it.  A component whose dispersion end point lies inside it bounces back: it
 * stays at its moment's position and carries the opposite direction.  Points that end a step
 * inside the solid are removed, as in the reference.  The inflow layer sets moments of the first
 * `width` cell columns to the equilibrium at velocity u (their own density).  Both take effect at
 * the next step; with an obstacle the 2D window kernels run untiled.  Synchronise. */
int dbm_sim_set_obstacle(dbm_sim* sim, int32_t inst, const double* h_center, double radius);
int dbm_sim_set_inflow(dbm_sim* sim, int32_t inst, const double* h_u, int32_t width);
/* Checkpoint / resume (the reference has none): copy the current state into a device blob of
 * *needed bytes (call with d_dst = NULL to size it; synchronises), and make such a blob the
 * current state again, bit for bit. */
int dbm_sim_snapshot(dbm_sim* sim, void* d_dst, int64_t bytes, int64_t* needed, void* stream);
int dbm_sim_restore(dbm_sim* sim, const void* d_src, int64_t bytes, void* stream);

/* ---- adjoint of the step (no reference counterpart: differentiation is future work in the
 * reference, idea.md:250) ---------------------------------------------------------------------
 * A tape records steps of a simulator: the input moments, the collided f, each component's thin
 * cell, each control point's thin cell / count / centroid / refine decision, and three neighbour
 * lists -- refine (control point and direction -> components within r of its centroid, moved
 * points only), resample (control point and direction -> components within r) and gap fill (control point ->
 * control points within r sharing an empty direction) -- with the displacement of every pair as
 * the forward step computed it.  dbm_tape_backward applies the transpose of the step's Jacobian
 * with those discrete decisions held fixed (a hand-written vector-Jacobian product of the
 * collision, the dispersion, thinning, refine, resampling weights, gather and gap fill).
 * Cotangents are FP64, row-major, in the sorted moment order of each state:
 *   g_off_out (P, D), g_f_out (P, Q): d loss / d (output offsets in cell units, output f)
 *   g_off_in (M, D), g_f_in (M, Q):  written, d loss / d (input offsets, input f)
 *   g_tau (n_inst): accumulated (+=), d loss / d tau of each instance. */
typedef struct dbm_tape dbm_tape;
int dbm_tape_create(dbm_sim* sim, dbm_tape** out);
int dbm_tape_destroy(dbm_tape* tape);
/* Forget every recorded step (device memory is kept for reuse). */
int dbm_tape_clear(dbm_tape* tape);
/* Advance the tape's simulator by one step and record it.  Synchronises. */
int dbm_tape_step(dbm_tape* tape, void* stream);
int32_t dbm_tape_length(dbm_tape* tape);
/* counts[8] of recorded step `index`: M, P, refine pairs, resample pairs, gap-fill pairs. */
int dbm_tape_counts(dbm_tape* tape, int32_t index, int64_t* counts);
int dbm_tape_backward(dbm_tape* tape, int32_t index, const double* d_g_off_out, const double* d_g_f_out,
                      double* d_g_off_in, double* d_g_f_in, double* d_g_tau, void* stream);
/* dbm_tape_step `steps` times; and every recorded step in reverse, from the cotangents of the last
 * step's output to those of the first step's input (one call per checkpoint segment). */
int dbm_tape_record(dbm_tape* tape, int32_t steps, void* stream);
/* Lists are sized from an estimate of pairs per row (grown to the largest seen; default 16).  A
 * recording whose list outgrows it is found at the next synchronisation: the call then returns
 * DBM_ERR_CAPACITY and the tape must be cleared and the segment recorded again from its start
 * state.  Setting the estimate trades memory against such retries. */
int dbm_tape_set_estimate(dbm_tape* tape, double pairs_per_row);
int dbm_tape_backward_all(dbm_tape* tape, const double* d_g_off_out, const double* d_g_f_out, double* d_g_off_in,
                          double* d_g_f_in, double* d_g_tau, void* stream);
/* Copy a recorded array (DBM_TAPE_*) of step `index` into d_dst, converted to the listed type;
 * *needed returns its size in bytes. */
int dbm_tape_export(dbm_tape* tape, int32_t index, int32_t what, void* d_dst, int64_t bytes, int64_t* needed,
                    void* stream);
#define DBM_TAPE_IN_CELL 1       /* u32[M] */
#define DBM_TAPE_IN_OFF 2        /* f64[D][M] */
#define DBM_TAPE_IN_F 3          /* f64[Q][M] (FP32DEV: rho*W + dev) */
#define DBM_TAPE_FSTAR 4         /* f64[Q][M] collided f */
#define DBM_TAPE_THIN_CELL 5     /* u32[Q][M] cell each component lands in (0xffffffff: outside) */
#define DBM_TAPE_CP_THIN 6       /* u32[P] thin cell of each output control point */
#define DBM_TAPE_CP_COUNT 7      /* u32[P] components thinned into it */
#define DBM_TAPE_CP_CEN 8        /* f64[D][P] centroid offset in its thin cell */
#define DBM_TAPE_CP_MOVED 9      /* u32[P] 1 if refine moved it */
#define DBM_TAPE_OUT_CELL 10     /* u32[P] */
#define DBM_TAPE_OUT_OFF 11      /* f64[D][P] */
#define DBM_TAPE_EMPTY 12        /* u32[P] gap-filled directions (bit k) */
#define DBM_TAPE_INV_SW 13       /* f64[Q][M] 1/sw per component (0 if dropped) */
#define DBM_TAPE_REFINE_START 14 /* u32[P*Q+1], row j*Q + k */
#define DBM_TAPE_REFINE_ITEM 15  /* u32[n] component m*Q + k */
#define DBM_TAPE_REFINE_E 16     /* f64[D][n] component minus centroid */
#define DBM_TAPE_RES_START 17    /* u32[P*Q+1], row j*Q + k */
#define DBM_TAPE_RES_ITEM 18     /* u32[n] component m*Q + k */
#define DBM_TAPE_RES_E 19        /* f64[D][n] component minus control point */
#define DBM_TAPE_GAP_START 20    /* u32[P+1] */
#define DBM_TAPE_GAP_ITEM 21     /* u32[n] neighbour control point */
#define DBM_TAPE_GAP_BITS 22     /* u32[n] directions empty in both */
#define DBM_TAPE_GAP_E 23        /* f64[D][n] neighbour minus control point */
#define DBM_TAPE_INST_START 24   /* u32[n_inst+1] first input moment of each instance */

#define DBM_TRACE_OCC 1        /* u32[ncells]   occupied flag per cell after thinning */
#define DBM_TRACE_THIN_CNT 2   /* u32[ncells]   components per occupied cell */
#define DBM_TRACE_CENTROID 3   /* real[D][ncells] centroid offset (rel. to the cell) */
#define DBM_TRACE_MASK 4       /* u32[ncells]   refine direction mask */
#define DBM_TRACE_FINAL_CELL 5 /* u32[ncells]   refined CP cell */
#define DBM_TRACE_FINAL_OFF 6  /* real[D][ncells] refined CP offset */
#define DBM_TRACE_SORTED 7     /* u32[2][P]     sorted (cell, origin cell) pairs */
#define DBM_TRACE_SW 8         /* real[Q][Mcap] 1/sw per component, 0 if dropped (FP32DEV: float) */
#define DBM_TRACE_CPF 9        /* FP64: double[Q][cap]; FP32DEV: float[2][Q][cap] (hi, lo) */
#define DBM_TRACE_EMPTY 10     /* u32[cap]      empty-direction mask per CP */
#define DBM_TRACE_FSTAR 11     /* collided f of the input moments, layout of the state */
#define DBM_TRACE_COUNTS 12    /* u32[2]: M (moments in), P (control points) */
#define DBM_TRACE_STATE_CELL 13 /* u32[Mcap]    cell of each current moment */
#define DBM_TRACE_STATE_OFF 14  /* real[D][Mcap] offsets of each current moment */
#define DBM_TRACE_IMPORT_ORDER 15 /* u32[Mcap] after dbm_sim_set_state (and before any step):
                                     input index of each sorted moment */

#ifdef __cplusplus
}
#endif

#endif /* DIREBM_GB300_H */
