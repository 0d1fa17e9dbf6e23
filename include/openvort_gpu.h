/*
 * openvort_gpu.h - C ABI of libovgpu, the GB300 (sm_103a) implementation of
 * OpenVort's vortex-filament velocity and time-step path.
 *
 * Plain C types only: pointers, sizes, doubles, ints.  No CUDA or torch type
 * crosses this boundary.  Every call returns an ov_status (0 = OV_OK); the
 * message of the last failure on a context is read with ov_last_error().
 *
 * Two layers:
 *   1. Context API (ov_ctx_*, ov_upload_*, ov_update_*, ov_rk4_step, ...):
 *      the tangle lives in HBM between calls, parameters come from an explicit
 *      ov_params, results are read back with ov_download_*.
 *   2. Drop-in layer (include/ov_dropin.h, built from ov_dropin.c): void
 *      functions with the reference's own signatures that read the
 *      reference's process-global parameters, upload, compute and download
 *      around a hidden per-process context.
 *
 * Reference interfaces replaced (OpenVort, paths within the project):
 *   update_tangents_normals  include/tangle.h:104,  src/tangle.c:509
 *   update_velocity          include/tangle.h:106,  src/tangle.c:600
 *   update_velocities        include/tangle.h:108,  src/tangle.c:733
 *   remesh                   include/tangle.h:110,  src/tangle.c:1018
 *   eliminate_small_loops    include/tangle.h:112,  src/tangle.c:1063
 *   enforce_periodic_boundaries include/tangle.h:98, src/tangle.c:793
 *   update_tangle            include/tangle.h:114-118 (static inline)
 *   rk4_step                 include/vortex_dynamics.h:21, src/vortex_dynamics.c:50
 *   reconnect                include/vortex_dynamics.h:32, src/vortex_dynamics.c:186
 *   smooth                   include/vortex_smooth.h:11, src/vortex_smooth.c:459
 *   octree_build / octree_get_vs / octree_destroy
 *                            include/octree.h:54-66, src/octree.c:139,296,41
 */
#ifndef OPENVORT_GPU_H
#define OPENVORT_GPU_H

#include <stdint.h>
#include "ov_tangle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
typedef enum ov_status {
    OV_OK = 0,
    OV_ERR_ARG = 1,      /* bad argument (null pointer, negative size, ...) */
    OV_ERR_CUDA = 2,     /* a CUDA runtime call failed */
    OV_ERR_ALLOC = 3,    /* device or host allocation failed */
    OV_ERR_DEPTH = 4,    /* two nodes share a cell at the deepest tree level (strict depth policy) */
    OV_ERR_STACK = 5,    /* a traversal exceeded its iteration bound */
    OV_ERR_NAN = 6,      /* a non-finite position or velocity was produced */
    OV_ERR_TIMEOUT = 7,  /* a bounded device wait gave up */
    OV_ERR_TOPOLOGY = 8, /* connections are not a consistent set of loops */
    OV_ERR_NODEVICE = 9, /* no CUDA device is visible */
    OV_ERR_STATE = 10    /* call made before the tangle was uploaded */
} ov_status;

/* --------------------------------------------------------------- params */
/*
 * Run parameters.  Field-for-field the process globals of the reference
 * (include/vortex_constants.h:11-60, defaults src/initial_conditions.c:12-91)
 * plus the three external-velocity configurations (vn_conf, vs_conf, vb_conf).
 */
typedef struct ov_params {
    double kappa;                     /* KAPPA [cm^2/s] */
    double vortex_width;              /* VORTEX_WIDTH, a0 [cm] */
    double alpha;                     /* alpha (mutual friction) */
    double alpha_p;                   /* alpha' (mutual friction) */
    int use_mutual_friction;          /* use_mutual_friction */
    int use_bh;                       /* use_BH: 1 = tree, 0 = direct sum */
    double bh_resolution;             /* BH_resolution, opening angle theta */
    ov_ext_vel vn;                    /* vn_conf: normal-fluid velocity */
    ov_ext_vel vs;                    /* vs_conf: external superfluid velocity */
    ov_ext_vel vb;                    /* vb_conf: boundary velocity */
    double dl_min;                    /* global_dl_min */
    double dl_max;                    /* global_dl_max */
    double rec_dist;                  /* rec_dist */
    double reconnection_angle_cutoff; /* reconnection_angle_cutoff [rad] */
    int small_loop_cutoff;            /* small_loop_cutoff */
    int use_freq_filter;              /* use_freq_filter */
    double freq_to_cutoff;            /* freq_to_cutoff */
    int num_threads;                  /* global_num_threads (host passes) */
    int pin_mode;                     /* pin_mode */
} ov_params;

/* Fill `p` with the reference's compiled-in defaults (initial_conditions.c:12-91). */
void ov_params_default(ov_params *p);

/* ------------------------------------------------------------ precision */
enum {
    OV_PREC_FP64 = 0,   /* FP64 traversal: the reference's decisions, FP64 interactions
                           (reference semantics; walk arithmetic: ov_set_walk) */
    OV_PREC_MIXED = 1,  /* FP32 traversal on grid-split positions, compensated sums,
                           FP64 for LIA, near field, guard-band decisions, RK4 update */
    OV_PREC_DD = 2      /* the mixed traversal's FP32 walk and decisions, each accepted
                           interaction and the sums in double-single (two floats, about
                           1e-14 per operation): FP64-class accuracy at FP32 speed */
};

/* Download field mask for ov_download_tangle. */
enum {
    OV_F_POS = 1, OV_F_VELS = 2, OV_F_VS = 4, OV_F_TANGENTS = 8, OV_F_NORMALS = 16,
    OV_F_TOPOLOGY = 32, OV_F_ALL = 63
};

/* Counters of the last velocity evaluation (and topology passes). */
typedef struct ov_stats {
    int64_t node_evals;        /* target nodes evaluated */
    int64_t cells;             /* cells in the linear octree */
    int64_t max_depth;         /* deepest cell level */
    int64_t visits;            /* per-target cell visits (open or accept) */
    int64_t accepts;           /* per-target monopole/leaf interactions */
    int64_t warp_steps;        /* warp-cooperative traversal iterations */
    int64_t fp64_fallbacks;    /* mixed path: guard-band decisions redone in FP64 */
    int64_t near_field_fp64;   /* mixed path: near-field interactions done in FP64 */
    int64_t out_of_root;       /* nodes outside the root box (root-only members) */
    int64_t reconnections;     /* last reconnect pass */
    int64_t remesh_added;      /* last remesh pass */
    int64_t remesh_removed;    /* last remesh pass */
    int64_t small_loops_removed;
    int64_t error_word;        /* device error flags, 0 when clean */
    int64_t reconnect_candidates;   /* last reconnect pass: nodes in candidate pairs */
    int64_t reconnect_fp64_pairs;   /* pairs the mixed-precision bound left undecided (FP64 sums) */
    int64_t reconnect_exact_pairs;  /* pairs recomputed in the reference's summation order */
    int64_t reconnect_evaluated;    /* candidate velocities the decisions used */
    int64_t wall_clipped;           /* last wall pass: nodes connected to a wall */
    int64_t wall_removed;           /* last wall pass: nodes removed behind a wall */
    int64_t injected_nodes;         /* last injection pass: nodes added */
    int64_t reconnect_lazy_evals;   /* candidate velocities decided with a bound on corrections not yet read back */
} ov_stats;

typedef struct ov_ctx ov_ctx;

/* ---------------------------------------------------------- context API */
int ov_ctx_create(ov_ctx **out, int device);
int ov_ctx_destroy(ov_ctx *ctx);
const char *ov_last_error(const ov_ctx *ctx);
int ov_set_params(ov_ctx *ctx, const ov_params *p);
int ov_set_precision(ov_ctx *ctx, int precision);
/* How OV_PREC_FP64 walks the tree.  Both give the FP64 decisions (which
   cells each node accepts, skips and opens) and FP64 interactions. */
enum {
    OV_WALK_SPLIT = 0,  /* default: the distance and opening tests in FP32 on
                           grid-split positions, the FP64 test inside their guard
                           bands; accepted cells evaluated in FP64 by full warps */
    OV_WALK_FP64 = 1    /* every test in FP64 with the reference's rounding, each
                           accepted cell evaluated where the walk meets it */
};
int ov_set_walk(ov_ctx *ctx, int walk);
int ov_get_walk(const ov_ctx *ctx);
/* RK4 steps and single evaluations (update_tangle, update_velocities) run as
   captured CUDA graphs (default on); off launches the same kernels one by
   one (identical results). */
int ov_set_rk4_graph(ov_ctx *ctx, int on);
/* Uploads and downloads read and write the caller's tangle arrays in place
   from the GPU when the device accesses pageable host memory through the
   host's page tables (Grace-based systems; default on there), else through
   one staged copy of each array; 0 forces the staged copies.  Identical
   results either way.  ov_get_host_access returns 1 when the in-place path
   is in effect. */
int ov_set_host_access(ov_ctx *ctx, int direct);
int ov_get_host_access(const ov_ctx *ctx);
/* cudaStream_t the context launches on, as an opaque pointer (for callers that
   time or order their own work against it). */
void *ov_ctx_stream(ov_ctx *ctx);

/* Copy a host tangle (reference layout) into HBM.  All node-indexed arrays
   of `t` are read for t->N slots; box and image set are taken from `t`. */
int ov_upload_tangle(ov_ctx *ctx, const ov_tangle_state *t);
/* Copy the selected fields (OV_F_* mask) back into the host tangle. The
   host arrays must hold at least the context's node capacity (ov_capacity). */
int ov_download_tangle(ov_ctx *ctx, ov_tangle_state *t, unsigned fields);
int ov_capacity(const ov_ctx *ctx);
/* Slot count of the tangle held by the context (tangle_state.N, which
   remesh may double as expand_tangle does) and its next_empty /
   total_empty bookkeeping.  A host tangle passed to ov_download_tangle must
   have at least *n_slots slots. */
int ov_tangle_info(const ov_ctx *ctx, int *n_slots, int *next_empty, int *total_empty);
/* Upload only the OV_F_* fields selected (positions and topology are all
   update_tangle needs; update_velocities also reads tangents/normals).  The
   first upload into a context, or one that changes the node count, always
   transfers positions and topology as well. */
int ov_upload_tangle_fields(ov_ctx *ctx, const ov_tangle_state *t, unsigned fields);

/* ----------------------------------------------------------- ensembles */
/* An ensemble of independent tangles held by one context.  Every entry
   point of this header then acts on all members at once: one tree per
   member built in the same launches, one persistent traversal launch over a
   (member, node tile) work queue, RK4 as one graph for all members, and the
   topology passes member by member in the reference's order.  Members share
   the box and image set and KAPPA, BH_resolution and use_BH (OV_ERR_ARG
   otherwise); every other parameter is per member.  Member i keeps its own
   slot range of ceil(N_i * headroom) slots (headroom >= 1; 2 leaves room
   for one doubling by expand_tangle without moving the other members), so
   its slot indices, next_empty and total_empty are those of the member's
   own tangle_state.  ov_upload_tangle makes a one-member context. */
int ov_upload_ensemble(ov_ctx *ctx, const ov_tangle_state *const *tangles, const ov_params *params, int n,
                       double headroom);
int ov_ensemble_size(const ov_ctx *ctx);
/* tangle_state N / next_empty / total_empty of member i */
int ov_member_info(const ov_ctx *ctx, int i, int *n_slots, int *next_empty, int *total_empty);
/* ov_download_tangle for member i (t->N must be >= the member's N) */
int ov_download_member(ov_ctx *ctx, int i, ov_tangle_state *t, unsigned fields);
/* per-member parameters (the shared ones must keep their values) */
int ov_set_member_params(ov_ctx *ctx, int i, const ov_params *p);

/* Launch shape of the traversal: warps per block (2, 4 or 8), query groups
   per node (1-27; 0 = from the node count), persistent blocks per SM (0 =
   the occupancy limit), the order of the work queue (largest member first
   or member order), and for the mixed traversal the register budget (0:
   the default; 1: fewer registers for one more resident block).  Results
   do not depend on it. */
typedef struct ov_tuning {
    int warps_per_block;
    int query_groups;
    int blocks_per_sm;
    int largest_first;
    int high_occupancy;   /* mixed traversal variant: 0 the general kernel, 1 the same under a
                             tighter register budget; 2, 3, 4 the periodic-image kernel with
                             fewer values held per lane (mirror images: as 0) with the
                             compiler's register count, 80 and 64 registers */
} ov_tuning;
int ov_get_tuning(const ov_ctx *ctx, ov_tuning *out);
int ov_set_tuning(ov_ctx *ctx, const ov_tuning *tu);
/* Time the velocity evaluation of the resident tangle(s) at time t over
   candidate launch shapes (context precision), keep the fastest, and return
   it in *best with its time in *ms_best (either may be NULL).  The
   context's velocities are overwritten. */
int ov_autotune(ov_ctx *ctx, double t, ov_tuning *best, float *ms_best);

/* ------------------------------------------------------- velocity path */
/* Tangents and normals of every node: update_tangents_normals (tangle.c:509). */
int ov_update_tangents_normals(ov_ctx *ctx);
/* Tree build + fused per-node velocity (LIA, v_s, BH over 1+n_img images,
   mutual friction): update_velocities (tangle.c:733). */
int ov_update_velocities(ov_ctx *ctx, double t);
/* update_tangle (tangle.h:114): tangents/normals then velocities. */
int ov_update_tangle(ov_ctx *ctx, double t);
/* One RK4 step (vortex_dynamics.c:50): the three further stage evaluations
   and the combine, from the velocities already held in the context (k1). */
int ov_rk4_step(ov_ctx *ctx, double t, double dt);
/* Exact FP64 direct O(N * (1+n_img)) Biot-Savart velocities of the listed
   nodes, the `tree == NULL` branch of update_velocity (tangle.c:652-687).
   Writes n vec3 to vels_out and vs_out (host arrays; either may be NULL). */
int ov_direct_velocities(ov_ctx *ctx, const int *nodes, int n, double t,
                         double *vels_out, double *vs_out);

/* The nonlocal part of the direct sum (segments of the node's own tangle and
   every image, without LIA or external/friction terms) for n nodes, as
   reconnect uses it.  precision OV_PREC_MIXED: far segments in FP32 on
   grid-split positions, near ones in FP64; OV_PREC_FP64: all in FP64.
   out (host, 5 doubles per node): the three components, a bound on each
   component's error, and the sum of the terms' magnitudes. */
int ov_direct_sums_bounded(ov_ctx *ctx, const int *nodes, int n, int precision, double *out);

/* Largest node list one ov_direct_velocities_noalloc call accepts. */
#define OV_NOALLOC_MAX_NODES 4096

/*
 * ov_direct_velocities_noalloc - the direct-sum velocities of
 * ov_direct_velocities for callers that may not allocate GPU memory.
 * This entry point has no counterpart in the reference.
 *
 * Who needs it: programs whose device memory is owned by someone else - a
 * pool or arena allocator that has reserved the GPU, a host framework that
 * hands the library its buffers once at start-up and forbids allocation
 * afterwards - and latency-bound loops that must never reach cudaMalloc,
 * which may synchronize the device.  The call takes no context, allocates
 * nothing (no cudaMalloc, no cudaFree, no allocating library routine) and
 * only launches two kernels on `stream`; the caller owns every buffer.
 *
 * Working space: the per-node partial sums live in one fixed array compiled
 * into the library (3 doubles per node, OV_NOALLOC_MAX_NODES nodes, 96 KiB),
 * which every GPU that loads the library keeps until the process exits.
 * All calls on a device share that array: two calls whose kernels overlap on
 * the GPU (different streams, no ordering between them) race and corrupt
 * each other's results.  Calls ordered on one stream are safe; each call
 * writes every partial sum it later reads, so nothing carries over.
 * The first call on each device looks up the array's device address (with
 * that device current); make that first call before any stream capture.
 * The address is kept for the life of the process: after cudaDeviceReset
 * (which unloads the library's device code) do not call this entry point
 * again in that process.
 *
 * Inputs (device pointers, n_slots node slots in the reference's indexing):
 *   d_pos       x[n_slots], y[n_slots], z[n_slots]          (SoA doubles)
 *   d_conn      forward[n_slots], reverse[n_slots]
 *   d_status    status[n_slots], pin_wall[n_slots]
 *   d_tangents  / d_normals  SoA like d_pos
 *   d_nodes     n_nodes node ids, each in [0, n_slots)
 * Outputs (device, AoS): d_vels, d_vs  n_nodes x 3 doubles (d_vs may be NULL).
 * An EMPTY slot gives zeros, as ov_direct_velocities does; a node id out of
 * range gives NaN outputs for that entry.
 * Returns OV_ERR_ARG when n_nodes > OV_NOALLOC_MAX_NODES, n_nodes < 0 or a
 * required pointer is NULL; OV_ERR_CUDA when the launch or the address
 * look-up fails.  Asynchronous: synchronize `stream` before reading outputs.
 */
int ov_direct_velocities_noalloc(const ov_params *p, const ov_domain_box *box,
                                 const ov_image_tangle *images, int n_images, int n_slots,
                                 const double *d_pos, const int *d_conn, const int *d_status,
                                 const double *d_tangents, const double *d_normals,
                                 const int *d_nodes, int n_nodes, double t,
                                 double *d_vels, double *d_vs, void *stream);

/* Barnes-Hut velocity sum of octree_get_vs (octree.c:296-356), FP64, at n
   arbitrary points: the tree of the context's current positions is built
   first when `rebuild` is non-zero (or none exists yet).  points and out are
   host arrays of n vec3.  n = 0 with rebuild = 1 only builds the tree. */
int ov_tree_velocity_at(ov_ctx *ctx, const double *points, int n, double resolution, int rebuild,
                        double *out);

/* ------------------------------------------------------ topology passes */
int ov_enforce_periodic_boundaries(ov_ctx *ctx);
int ov_eliminate_small_loops(ov_ctx *ctx);
/* reconnect (vortex_dynamics.c:186). *nrecs receives the count; if log_k /
   log_l are non-NULL the (k,l) of each reconnection is written, in order,
   up to log_cap entries. */
int ov_reconnect(ov_ctx *ctx, double t, int *nrecs, int *log_k, int *log_l, int log_cap);
/* enforce_wall_boundaries (tangle.c:966): connect nodes within rec_dist of a
   mirror wall to it (connect_to_wall, tangle.c:877) and remove nodes behind
   one.  Nothing to do when every wall is periodic or open. */
int ov_enforce_wall_boundaries(ov_ctx *ctx, double t);
/* remesh (tangle.c:1018). */
int ov_remesh(ov_ctx *ctx, double min_dist, double max_dist, double t);
/* smooth (vortex_smooth.c:459): per-loop low-pass filter when use_freq_filter. */
int ov_smooth(ov_ctx *ctx);
/* One iteration of the reference's main loop body (main.c:123-141), without
   frame output: injection (when set with ov_set_injection), wall
   boundaries, small loops, reconnect, small loops, smooth, periodic wrap,
   remesh (with wall boundaries after insertions), small loops,
   update_tangle, rk4_step, periodic wrap. */
int ov_step(ov_ctx *ctx, double t, double dt);
/* Host wall-clock milliseconds of the last ov_step, per pass: [0] small
   loops (three calls), [1] reconnect, [2] smooth, [3] periodic wrap (two
   calls), [4] remesh, [5] update_tangle, [6] rk4_step, [7] the whole step;
   reconnect's parts: [8] mirror + candidate pairs, [9] direct sums,
   [10] sequential decisions, [11] push; inside [10]: [12] reading
   corrections back, [13] launching corrections, [14] FP64 sums of
   undecided pairs, [15] reference-order recomputes.  Writes min(n, 16)
   values. */
int ov_step_times(const ov_ctx *ctx, double *ms, int n);

int ov_get_stats(const ov_ctx *ctx, ov_stats *out);

/* ------------------------------------------------------------ injection */
/* The reference's injection settings (vortex_constants.h:48-56,
   initial_conditions.c:61-68) for one tangle, with the state of its random
   stream: drand48's 48-bit state X as erand48 holds it, rand48[0] the low
   16 bits (srand48(s) leaves {0x330E, s & 0xFFFF, (s >> 16) & 0xFFFF}). */
typedef struct ov_injection {
    int loop_injection;        /* loop_injection: inject_loop on */
    double loop_frequency;     /* loop_injection_frequency: loops per unit time */
    int line_injection;        /* line_injection: inject_line_pairs on */
    int line_n;                /* line_injection_n: pairs per injection */
    double line_frequency;     /* line_injection_frequency */
    int line_polarized;        /* line_injection_polarized */
    unsigned short rand48[3];  /* the stream inject_loop / inject_line_pairs draw from */
} ov_injection;

/* add_loop (vortex_injection.c:49): a ring of (int)(4 pi r / (dl_max +
   dl_min)) FREE nodes around `center` in the plane normal to `dir`, slots
   from get_next_empty_node after doubling the member until it has that
   many EMPTY slots.  member: 0 for a single tangle. */
int ov_add_loop(ov_ctx *ctx, int member, const double center[3], const double dir[3], double r);
/* add_line_in_zdir (vortex_injection.c:267): a line along z through
   (x, y) from wall to wall, pinned (params pin_mode) at both ends;
   direction +1 runs up, -1 down. */
int ov_add_line_in_zdir(ov_ctx *ctx, int member, double x, double y, int direction);
/* Injection settings of one member (all members when member < 0); resets
   the last-injection times of inject_loop and inject_line_pairs to 0, as a
   new process starts them.  ov_get_injection returns the settings with the
   stream's current state. */
int ov_set_injection(ov_ctx *ctx, int member, const ov_injection *inj);
int ov_get_injection(const ov_ctx *ctx, int member, ov_injection *out);
/* inject_vortices (vortex_injection.c:702) for every member, in member
   order.  ov_step runs it first (main.c:123) when a member has injection
   on. */
int ov_inject_vortices(ov_ctx *ctx, double t);
/* One draw of the injection stream (drand48's recurrence on the state x,
   as erand48 draws); host only. */
double ov_erand48(unsigned short x[3]);

/* --------------------------------------------------------------- frames */
/* Frame files in the reference's text format (utils.c:68-199).  Host-only
   calls except ov_save_frame.
   ov_write_frame: save_tangle of a host tangle, loops in its order; digits
     15 writes the reference's files exactly, 17 an exact round trip.
   ov_frame_slots: the N, next_empty and total_empty that load_tangle
     leaves in a tangle made by create_tangle(n0) (any may be NULL).
   ov_read_frame: load_tangle into `t`, which must have at least that N
     slots; n0 is the slot count before the load and t->next_empty,
     t->total_empty on entry the bookkeeping before it (create_tangle(n0)
     leaves 0 and n0).
   ov_save_frame: the context's tangle (member 0) or an ensemble member. */
int ov_write_frame(const ov_tangle_state *t, const char *path, int digits);
int ov_frame_slots(const char *path, int n0, int *n_slots, int *next_empty, int *total_empty);
int ov_read_frame(const char *path, int n0, ov_tangle_state *t);
int ov_save_frame(ov_ctx *ctx, int member, const char *path, int digits);

/* -------------------------------------------------------------- timing */
/* CUDA-event timing on the context's stream (for benchmarks). */
int ov_timer_start(ov_ctx *ctx);
int ov_timer_stop(ov_ctx *ctx, float *ms);   /* synchronizes */
/* Write `bytes` of junk into a device buffer owned by the context (L2 flush). */
int ov_flush_l2(ov_ctx *ctx, size_t bytes);
int ov_synchronize(ov_ctx *ctx);
/* Number of kernels this context launched since creation. */
int64_t ov_kernel_launches(const ov_ctx *ctx);
/* Per-phase device times of the last velocity evaluation, recorded with CUDA
   events when phase timing is on: ms[0] tangents, ms[1] tree build,
   ms[2] traversal. */
int ov_set_phase_timing(ov_ctx *ctx, int on);
int ov_phase_times(ov_ctx *ctx, float ms[3]);
/* Per-target tree statistics (octree.c's walk, counted node by node): with
   counting on, every velocity evaluation outside the RK4 graph records for
   each slot the cells its 1 + n_img query points visited and the cells they
   accepted; ov_get_node_counts copies the counts of the last evaluation for
   slots [0, n) of a member (0 for a single tangle), n at most its slot count
   (OV_ERR_STATE before the first evaluation).  A target whose counts differ
   from the reference tree's took a different opening decision. */
int ov_set_node_counting(ov_ctx *ctx, int on);

/* Nodes closer than the deepest tree cell (21 levels below the root: about
   D * 5e-7 for one tangle; fewer levels in an ensemble, whose member id takes
   key bits).  OpenVort's octree keeps splitting there (octree.c:116-160) and
   never ends for two nodes at one position - which its own smoothing makes:
   with freq_to_cutoff 0.8, vortex_smooth.c:146-160 keeps only the mean of a
   closed loop of 6 to 19 nodes, so every node of it lands on one point.
   Default (strict = 0): the shared deepest cell is one leaf (its nodes'
   centre of mass and summed circulation) and the call succeeds with
   OV_EW_DEPTH (1) in ov_stats.error_word.  strict = 1: OV_ERR_DEPTH. */
int ov_set_depth_policy(ov_ctx *ctx, int strict);

/* Error-path testing: after `after` more successful device or pinned host
   allocations of this context, the next one fails as if the device were out
   of memory (no allocation is attempted); -1 switches it off.  Any allocation
   failure, real or injected, returns OV_ERR_ALLOC, frees every buffer of the
   context and leaves it holding no tangle: upload again to go on.  No
   counterpart in the reference (its allocations are unchecked malloc). */
int ov_inject_alloc_failure(ov_ctx *ctx, int after);
int ov_get_node_counts(ov_ctx *ctx, int member, unsigned *visits, unsigned *accepts, int n);
/* Measured multiply-add throughput of this GPU in TFLOP/s for FP64
   (precision OV_PREC_FP64) or FP32 (OV_PREC_MIXED): the roofline peak of
   the traversal, which is FMA-pipe bound. */
int ov_measure_fma_peak(ov_ctx *ctx, int precision, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* OPENVORT_GPU_H */
