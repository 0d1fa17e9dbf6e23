// ov_internal.cuh - shared declarations of libovgpu (not part of the C ABI).
//
// Device data layout (HBM), per tangle of `cap` node slots:
//   x,y,z            double[cap]  positions (SoA)
//   fwd,rev          int[cap]     connections
//   status,pin       int[cap]     node_status
//   tx,ty,tz nx,...  double[cap]  tangents / normals (SoA)
//   vx.. / sx..      double[cap]  vels / vs (SoA)
// Linear octree (rebuilt per evaluation):
//   keys,order       u64/int[cap] path keys and node ids, sorted by key
//   cells            Cell64[ncell] pre-order cells: COM, circulation, Lm,
//                                  subtree end (`next`) and node count
//   cells32          Cell32[ncell] FP32 copy for the mixed traversal
//   nm               double[6 cap] node moments (position, wrapped forward
//                                  segment) in id order, for the leaves
//   first,lvl8,psum  per cell: first sorted node, level, position sum
//   lvl_list         non-root, non-leaf cells grouped by level
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/openvort_gpu.h"
#include "../../include/ov_spherical.h"

#define OV_MAX_LEVEL 21                 // 3-bit digits below the root: 63 bits
#define OV_KEY_OUT (0x8000000000000000ull) // node outside the root box (| wrapped path >> 1)
#define OV_KEY_EMPTY (0xFFFFFFFFFFFFFFFFull)
#define OV_MAX_IMAGES 26
#define OV_SPH_MEMBERS 2                // spherical section: the tangle and its inner image

// device error bits (ov_stats.error_word)
enum {
    OV_EW_DEPTH = 1,      // two nodes share the deepest cell
    OV_EW_SLIVER = 2,     // a node fell in a rounding gap between child boxes
    OV_EW_WALK = 4,       // step_node walked onto an EMPTY slot or looped
    OV_EW_ITER = 8,       // traversal exceeded its iteration bound
    OV_EW_NAN = 16,       // non-finite position
    OV_EW_RUN = 32,       // sort fix-up met a run longer than its bound
    OV_EW_CELLS = 64,     // cell storage too small: host grows it and rebuilds
    OV_EW_BOUNDS = 128,   // an index failed a bounds check (access skipped)
    OV_EW_TEMP = 256,     // spherical fork: a temperature outside the He II model's range
    OV_EW_INVERT = 512    // spherical fork: inversion of a node at the origin
};

struct Cell64 {          // 64 bytes, one per cell, pre-order
    double cx, cy, cz;   // centre of mass (mean position)
    double qx, qy, qz;   // total circulation (sum of wrapped forward segments)
    double lm;           // largest side of the cell box
    int next;            // index of the first cell after this subtree
    int count;           // nodes in the cell
};

struct Cell32 {          // 48 bytes: FP32 view for the FP32 walks; a walk step reads the first 32
    float gx, gy, gz;    // COM, grid part (multiple of the grid step h)
    float thr;           // (Lm / theta)^2 (1 + 2e-5), rounded up: d^2 above it accepts the cell clear of the test's band
    float fx, fy, fz;    // COM, fine part
    int next;            // first cell after the subtree
    float qx, qy, qz;    // circulation
    float lm;            // Lm (rounded up)
};

struct CellFF {           // 64 bytes: double-single view for OV_PREC_DD
    float g[3];          // centre of mass, grid part (exact, as in Cell32)
    float fh[3], fl[3];  // centre of mass, the rest as hi + lo
    float qh[3], ql[3];  // circulation, hi + lo
    float pad;
};

// Per-member results of a forest build (tree.tt, TT_WORDS ints a member).
enum MemberWords {
    TT_NNE = 0,   // non-EMPTY nodes
    TT_M,         // nodes inside the box
    TT_START,     // first sorted position of the member
    TT_ROOT,      // root cell
    TT_END,       // one past the member's last cell
    TT_ITEM0,     // first work item of the member in the traversal queue
    TT_WORDS = 8
};

constexpr int TREE_LV_SLOTS = 32;   // levels 0..OV_MAX_LEVEL of the per-level cell lists
constexpr int TREE_INV_COUNT = 4096; // table of 1 / count for the cell means

struct TreeBuf {
    int cap = 0;
    int *tt = nullptr;           // TT_WORDS ints per member
    uint64_t *keys = nullptr, *keys_alt = nullptr;
    int *order = nullptr, *order_alt = nullptr;
    int *torder = nullptr;       // traversal order of the targets (spatial, all non-EMPTY)
    int *cpl = nullptr;          // common prefix length with the next key
    int *ncell_at = nullptr;     // cells starting at sorted position s
    int *cell_off = nullptr;     // exclusive scan of ncell_at (+1 for the root)
    int *scan_tmp = nullptr;
    int *sort_hist = nullptr;
    int cap_cells = 0;
    Cell64 *cells = nullptr;
    Cell32 *cells32 = nullptr;
    CellFF *cellsff = nullptr;
    double *psum = nullptr;      // 3 doubles per cell of more than one node: position sum (a one-node
                                 // cell's mean is its sum; every cell's circulation is a sum)
    uint8_t *lvl8 = nullptr;     // level of each cell (0 for roots)
    int *first = nullptr;        // first sorted position of each cell's nodes
    int *lvl_list = nullptr;     // non-root cells grouped by level (ascending levels)
    int *lvl_cnt = nullptr;      // TREE_LV_SLOTS cells per level, as many fill counters, then the
                                 // level sums' grid-barrier counter
    double *nm = nullptr;        // 6 doubles per node slot: position, wrapped forward segment
    double *inv_count = nullptr; // TREE_INV_COUNT entries: 1 / k, rounded (entry 0 unused)
    float *lev_tab = nullptr;    // per level: FP32 opening threshold and Lm of a box cell
    int *counters = nullptr;     // device scalars, see TreeCounters
};

// device-side scalars written by the build
enum TreeCounters {
    // cleared by every tree build
    TC_M = 0,          // nodes inside the root box (sorted prefix)
    TC_NNE,            // non-EMPTY nodes (targets)
    TC_NCELL,          // cells
    TC_MAXDEPTH,
    TC_OUT,            // nodes outside the root box
    TC_MAXRUN,
    TC_FALLBACK,       // mixed: guard-band FP64 decisions
    TC_NEAR64,         // mixed: near-field FP64 interactions
    TC_BUILD_CLEAR,    // = 8: words [0, 8) are per build
    // cleared once per API call (they accumulate over the stages of an RK4 step)
    TC_ERR = 8,        // error bits
    TC_BAD,            // first failed bounds check: code << 24 | low bits of the index
    TC_NEED,           // most cells any build needed (checked against the storage)
    TC_WORK,           // work-queue counter of the traversal (reset per launch)
    TC_ITEMS,          // work items of the traversal (written by the build)
    TC_COUNT,
    TC_STAT64 = 16,    // int offset of the 64-bit counters (per build): visits, accepts, warp steps, ...
    TC_WORDS = 32      // ints allocated
};
enum { ST_VISITS = 0, ST_ACCEPTS, ST_STEPS, ST_FALLBACK, ST_NEAR64 };

struct Geometry {
    double lo[3], hi[3], L[3];
    int periodic[3];             // low wall of the axis is periodic (seg_pwrap)
    int wall[6];
    int n_img;
    int shift[OV_MAX_IMAGES][3];
    int reflect[OV_MAX_IMAGES][3];
    int nreflect[OV_MAX_IMAGES];
    // spherical section domains (the spherical fork): seg_pwrap by angles
    int sph;                     // 1: this geometry is a spherical section
    double sph_az, sph_pl;       // half widths of the azimuth and polar ranges
    double sph_seg_max;          // 5 dl_max: longer wrapped segments stay out of the moments
};

struct NodeArrays {              // one tangle (or one RK4 stage) in HBM
    double *x = nullptr, *y = nullptr, *z = nullptr;
    double *tx = nullptr, *ty = nullptr, *tz = nullptr;
    double *nx = nullptr, *ny = nullptr, *nz = nullptr;
    double *vx = nullptr, *vy = nullptr, *vz = nullptr;
    double *sx = nullptr, *sy = nullptr, *sz = nullptr;
};

struct DevParams {               // ov_params as the kernels need them
    double kappa, a0, alpha, alpha_p, theta;
    int friction, use_bh;
    int vn_type, vs_type, vb_type;
    double vn[3], vs[3], vb[3];          // direction * strength for SIMPLE
    double vn_dir[3], vs_dir[3], vb_dir[3];   // normalised directions
    double vn_s0, vn_s1, vn_tld, vs_s0, vs_s1, vs_tld, vb_s0, vb_s1, vb_tld;
    double rec_dist;                     // reconnection candidate radius
};

// One tangle of the pool.  A single uploaded tangle is member 0 of 1; an
// ensemble keeps each member in its own contiguous slot range, so local
// index = slot - lo and the reference's slot arithmetic (next_empty, the
// doubling of expand_tangle) holds per member.
struct Member {
    int lo = 0;            // first slot
    int n = 0;             // the member's tangle_state N (its visible slots)
    int cap = 0;           // slots reserved for it (>= n; [lo+n, lo+cap) EMPTY)
    int next_empty = -1;   // tangle.h:63, local index
    int total_empty = 0;   // tangle.h:64
    ov_params params{};
    ov_injection inj{};        // injection settings and random stream
    double last_loop = 0;      // inject_loop's last injection time
    double last_line = 0;      // inject_line_pairs' last injection time
};

// Launch shape of the traversal, chosen by ov_autotune or set by the caller.
struct Tuning {
    int warps = 4;         // warps per block (2, 4 or 8)
    int groups = 0;        // query groups per node (0: from the node count)
    int blocks_per_sm = 0; // persistent blocks per SM (0: occupancy limit)
    int largest_first = 1; // work queue visits the largest member first
    int hi_occ = 0;        // mixed traversal: the tighter register budget variant
};

struct ov_ctx {
    int device = 0;
    int sm_count = 152;
    bool pageable = false;       // the device reads and writes pageable host memory (host page tables)
    bool host_direct = true;     // upload/download through the caller's arrays when pageable
    std::vector<Member> mem{Member{}};
    int key_tbits = 0;                     // member-id bits on top of the path keys
    int key_levels = OV_MAX_LEVEL;         // tree levels below each root
    int *d_tid = nullptr;                  // member of each slot (ensembles only)
    int *d_rm = nullptr;                   // remesh: slots to visit, then their count
    double *d_rm_lim = nullptr;            // remesh: (dl_min, dl_max) per member
    int rm_cap = 0, rm_lim_cap = 0;
    DevParams *d_tprm = nullptr;           // per-member parameters (ensembles only)
    int *d_qorder = nullptr;               // members in work-queue order
    int2 *d_mrange = nullptr;              // per-member slot range [lo, lo + cap)
    int tcap = 0;                          // members the per-member device arrays hold
    Tuning tune;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;            // tangents beside the tree build
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    ov_params params{};
    int precision = OV_PREC_FP64;
    int walk = OV_WALK_SPLIT;    // OV_PREC_FP64's tree walk (ov_set_walk)
    bool tree_built = false;     // the tree matches node positions (tree queries)
    std::string err;
    int cap = 0;                 // node slots
    int n_live = 0;              // slots of the uploaded tangle (<= cap)
    size_t last_h2d = 0;         // bytes of the last upload
    bool uploaded = false;
    Geometry geo{};
    int *fwd = nullptr, *rev = nullptr, *status = nullptr, *pin = nullptr;
    NodeArrays node;             // the tangle
    NodeArrays stage[3];         // RK4 stage tangles (positions, tangents, vels)
    TreeBuf tree;
    int64_t launches = 0;
    ov_stats stats{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    void *flush_buf = nullptr;
    size_t flush_bytes = 0;
    // host mirrors for the sequential topology passes (valid between
    // ov_pull_host and ov_push_device)
    std::vector<double> h_x, h_y, h_z;
    std::vector<int> h_fwd, h_rev, h_status, h_pin, h_recalc;
    bool host_valid = false;     // the mirrors equal the device positions and topology
    double step_ms[16] = {};     // host wall time of the last ov_step's passes (+ reconnect parts)
    // reconnect / smoothing scratch
    uint64_t *d_gkeys = nullptr, *d_gkeys_alt = nullptr;
    int *d_gidx = nullptr, *d_gidx_alt = nullptr;
    int *d_pairs = nullptr, *d_npairs = nullptr;
    int pair_cap = 0;
    int *d_loop_nodes = nullptr, *d_loop_off = nullptr;
    double *d_loop_buf = nullptr;
    double *d_loop_cut = nullptr;
    // long-loop smoothing (Bluestein FFT): work buffers, twiddles of size fft_M
    double2 *fft_buf = nullptr, *fft_tw = nullptr;
    size_t fft_cap = 0;
    int fft_M = 0;
    void *long_buf = nullptr;
    size_t long_cap = 0;
    int loop_cap = 0, loop_nodes_cap = 0;
    size_t loop_buf_cap = 0;
    // RK4 graph: stage times and steps live in d_time = {t+dt/2, t+dt/2,
    // t+dt, dt/2, dt, t of a single evaluation}; kernels read them when
    // time_dev_index >= 0
    cudaGraphExec_t rk4_exec = nullptr;
    unsigned long long rk4_key = 0;
    // single-evaluation graphs (tangents + tree + traversal of the context's
    // nodes): index 1 with the tangents, + 2 with phase events
    cudaGraphExec_t eval_exec[4] = {nullptr, nullptr, nullptr, nullptr};
    unsigned long long eval_key[4] = {0, 0, 0, 0};
    int64_t eval_kernels[4] = {0, 0, 0, 0};
    double *d_time = nullptr;
    double *h_time = nullptr;
    int time_dev_index = -1;
    bool use_graph = true;
    int64_t rk4_kernels = 0;     // kernels in the captured RK4 graph
    // mixed-precision grid split
    double grid_h = 0;
    // per-group partial velocity sums of the traversal (6 doubles x groups x cap)
    double *part = nullptr;
    size_t part_cap = 0;
    // reconnection velocities: candidate list, sums + bounds, corrections,
    // split positions, per-block partials
    int *rec_nodes = nullptr, *rec_pair = nullptr;
    double *rec_out = nullptr, *rec_corr = nullptr, *rec_part = nullptr;
    float *rec_split = nullptr;
    double *h_corr = nullptr;    // pinned host copy of the corrections
    size_t h_corr_cap = 0;
    double *h_pf = nullptr;      // prefetched corrections (pinned, mapped host memory)
    double *h_pf_dev = nullptr;  // the same as the device sees it
    cudaEvent_t rec_ev = nullptr;
    int rec_cap = 0, rec_split_cap = 0;
    size_t rec_part_cap = 0;
    // direct-sum scratch
    double *dsum = nullptr;
    int dsum_cap = 0;
    int *dnodes = nullptr;
    // pinned host staging
    double *h_stage = nullptr;
    size_t h_stage_bytes = 0;
    char *d_stage = nullptr;     // device copy of the host tangle's arrays as laid out there
    size_t d_stage_bytes = 0;
    // spherical sections: (r, az, pl) bounds of each tree member's root cell
    double sph_lo[OV_SPH_MEMBERS][3] = {}, sph_hi[OV_SPH_MEMBERS][3] = {};
    // nodes sharing the deepest tree cell: an error (true) or one leaf (ov_set_depth_policy)
    bool strict_depth = false;
    // allocation failure injection (ov_inject_alloc_failure): the number of
    // device or pinned allocations that still succeed before one fails; -1 off
    int alloc_fail_after = -1;
    // per-target visit / accept counters of the last evaluation (ov_set_node_counting)
    bool count_nodes = false;
    unsigned *d_node_counts = nullptr;
    size_t node_counts_cap = 0;
    // per-phase timing of the last evaluation
    bool phase_timing = false;
    cudaEvent_t ph[4] = {nullptr, nullptr, nullptr, nullptr};
};

// ------------------------------------------------------------ host helpers
int ov_fail(ov_ctx *c, int code, const char *fmt, ...);
#define OV_CUDA(ctx, call)                                                        \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess)                                                    \
            return ov_fail((ctx), OV_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, \
                           #call, cudaGetErrorString(e_));                        \
    } while (0)
#define OV_LAUNCHED(ctx) ((ctx)->launches++)

// Device and pinned host allocations.  A failure (or an injected one) frees
// every buffer the context holds and leaves it without a tangle (the next
// call must upload again), then returns OV_ERR_ALLOC: no buffer is left
// half-sized and no later launch can use one.
int ov_alloc_gate(ov_ctx *c);
int ov_alloc_failed(ov_ctx *c, const char *why, const char *what);
#define OV_ALLOC(ctx, call)                                                        \
    do {                                                                           \
        if (ov_alloc_gate(ctx)) return ov_alloc_failed((ctx), "injected failure", #call); \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            cudaGetLastError();                                                    \
            return ov_alloc_failed((ctx), cudaGetErrorString(e_), #call);          \
        }                                                                          \
    } while (0)

DevParams ov_dev_params(const ov_params &p);

inline unsigned long long *ov_stat_ptr(ov_ctx *c)
{
    return (unsigned long long *)(c->tree.counters + TC_STAT64);
}

// tree build (ov_tree.cu)
int ov_tree_reserve(ov_ctx *c, int cap);
// grow the node arrays to `cap` slots keeping their contents (topology passes)
int ov_grow_preserving(ov_ctx *c, int cap);
int ov_pull_host(ov_ctx *c);     // positions + topology -> host mirrors
int ov_push_device(ov_ctx *c, int first_new_slot);  // host mirrors -> device
int ov_eval_sync(ov_ctx *c, NodeArrays &na, double t, bool tangents);
int ov_tree_reserve_cells(ov_ctx *c, int cells);
int ov_reserve_members(ov_ctx *c, int nt);   // per-member device tables (ov_capi.cu)
int ov_upload_member_tables(ov_ctx *c);
int ov_move_device_slots(ov_ctx *c, const std::vector<Member> &old);
void ov_tree_free(TreeBuf &t);
int ov_tree_build(ov_ctx *c, const NodeArrays &na, cudaStream_t s);

// sort / scan (ov_sort.cu)
void ov_sort_keys(ov_ctx *c, TreeBuf &t, int n, cudaStream_t s);
void ov_scan_exclusive(ov_ctx *c, const int *in, int *out, int n_max, const int *n_dev, int add,
                       int *tmp, cudaStream_t s);

// velocity path (ov_velocity.cu)
void ov_launch_tangents(ov_ctx *c, const NodeArrays &na, cudaStream_t s);
int ov_launch_velocities(ov_ctx *c, const NodeArrays &na, double t, int precision, cudaStream_t s);
int ov_reserve_velocity_scratch(ov_ctx *c);
int ov_query_groups(ov_ctx *c);
int ov_traversal_blocks(ov_ctx *c, int precision, int warps, int *per_sm);
int ov_direct_sum(ov_ctx *c, const int *nodes, int n, double t, double *vels_out, double *vs_out);
// reconnection velocities (ov_velocity.cu)
int ov_rec_begin(ov_ctx *c, const int *cand, int n, double *out);
int ov_rec_exact(ov_ctx *c, int k, int l, double out[10]);
int ov_rec_correct(ov_ctx *c, int c0, int nc, const int *m, const int *f, const double *sign, int nch,
                   const int *pf, int npf);
int ov_rec_fetch(ov_ctx *c, int c0, int n, double *out);
int ov_rec_wait(ov_ctx *c);
void ov_launch_euler(ov_ctx *c, const NodeArrays &src, const double *vx, const double *vy,
                     const double *vz, double dt, NodeArrays &dst, cudaStream_t s);
void ov_launch_rk4_combine(ov_ctx *c, double dt, cudaStream_t s);
// spherical fork (ov_velocity.cu): the tangle in slots [0, n), its inner
// image in [n, 2n)
struct SphDomain {
    int n;
    double ri, ro, az, pl;       // radii, angular half widths
};
struct SphSettings {
    double kappa, a0, alpha, alpha_p, dl_min, dl_max, theta;
    int friction, use_temperature;
    double q_dot, t_bath, prof_a;
};
void ov_launch_sph_tangents(ov_ctx *c, const SphDomain &d, const SphSettings &p);
void ov_launch_sph_images(ov_ctx *c, const SphDomain &d, const SphSettings &p);
int ov_launch_sph_velocities(ov_ctx *c, const SphDomain &d, const SphSettings &p);
void ov_launch_periodic_wrap(ov_ctx *c, cudaStream_t s);

// ------------------------------------------------------------ device helpers
#ifdef __CUDACC__
// Explicitly rounded FP64 operations: never contracted into FMAs, so a
// sequence written with them has exactly the reference's rounding.
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }

// vec3_len / vec3_dot accumulation order: ((0 + a0 b0) + a1 b1) + a2 b2
__device__ __forceinline__ double dot3_ref(double a0, double a1, double a2, double b0, double b1,
                                           double b2)
{
    double o = rn_mul(a0, b0);
    o = rn_add(o, rn_mul(a1, b1));
    o = rn_add(o, rn_mul(a2, b2));
    return o;
}
__device__ __forceinline__ double len3_ref(double a0, double a1, double a2)
{
    return __dsqrt_rn(dot3_ref(a0, a1, a2, a0, a1, a2));
}

// seg_pwrap (boundaries.c:54-83): r2 moved by periods toward r1.
__device__ __forceinline__ void pwrap_dev(const Geometry &g, const double r1[3], double r2[3])
{
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!g.periodic[a]) continue;
        double L = g.L[a], hL = g.L[a] * 0.5;
        int guard = 0;
        while (rn_sub(r2[a], r1[a]) > hL && guard++ < 64) r2[a] = rn_sub(r2[a], L);
        while (rn_sub(r2[a], r1[a]) < -hL && guard++ < 128) r2[a] = rn_add(r2[a], L);
    }
}

// make_child_box (octree.c:165-232) on one box (lo,hi): child `idx` in the
// reference order BLF, BLB, BRF, BRB, TLF, TLB, TRF, TRB.
__device__ __forceinline__ void child_box_dev(const double b[3], const double t[3], int idx,
                                              double cb[3], double ct[3])
{
    double c[3], h[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        c[a] = rn_mul(rn_add(b[a], t[a]), 0.5);
        h[a] = rn_mul(rn_sub(t[a], b[a]), 0.5);   // L/2, exact
    }
    switch (idx) {
    case 0: cb[0] = rn_add(b[0], h[0]); cb[1] = b[1]; cb[2] = b[2];
            ct[0] = rn_add(c[0], h[0]); ct[1] = c[1]; ct[2] = c[2]; break;
    case 1: cb[0] = b[0]; cb[1] = b[1]; cb[2] = b[2]; ct[0] = c[0]; ct[1] = c[1]; ct[2] = c[2]; break;
    case 2: cb[0] = c[0]; cb[1] = c[1]; cb[2] = rn_sub(c[2], h[2]);
            ct[0] = t[0]; ct[1] = t[1]; ct[2] = rn_sub(t[2], h[2]); break;
    case 3: cb[0] = b[0]; cb[1] = rn_add(b[1], h[1]); cb[2] = b[2];
            ct[0] = c[0]; ct[1] = rn_add(c[1], h[1]); ct[2] = c[2]; break;
    case 4: cb[0] = c[0]; cb[1] = rn_sub(c[1], h[1]); cb[2] = c[2];
            ct[0] = t[0]; ct[1] = rn_sub(t[1], h[1]); ct[2] = t[2]; break;
    case 5: cb[0] = b[0]; cb[1] = b[1]; cb[2] = rn_add(b[2], h[2]);
            ct[0] = c[0]; ct[1] = c[1]; ct[2] = rn_add(c[2], h[2]); break;
    case 6: cb[0] = c[0]; cb[1] = c[1]; cb[2] = c[2]; ct[0] = t[0]; ct[1] = t[1]; ct[2] = t[2]; break;
    default: cb[0] = rn_sub(c[0], h[0]); cb[1] = c[1]; cb[2] = c[2];
             ct[0] = rn_sub(t[0], h[0]); ct[1] = t[1]; ct[2] = t[2]; break;
    }
}

__device__ __forceinline__ bool in_closed_box_dev(const double b[3], const double t[3], const double p[3])
{
    return p[0] >= b[0] && p[0] <= t[0] && p[1] >= b[1] && p[1] <= t[1] && p[2] >= b[2] && p[2] <= t[2];
}

// ------------------------------------------- spherical section helpers
// vec3_math.c of the spherical fork (240-282): radius, azimuth (elevation
// from the x-y plane), polar angle (in the x-y plane), and back.
__device__ __forceinline__ double sph_radius(const double v[3])
{
    return __dsqrt_rn(rn_add(rn_add(rn_mul(v[0], v[0]), rn_mul(v[1], v[1])), rn_mul(v[2], v[2])));
}
__device__ __forceinline__ double sph_azimut(const double v[3])
{
    return atan2(v[2], __dsqrt_rn(rn_add(rn_mul(v[1], v[1]), rn_mul(v[0], v[0]))));
}
__device__ __forceinline__ double sph_polar(const double v[3])
{
    if (v[0] == 0 && v[1] == 0) return 0.0;
    return atan2(v[1], v[0]);
}
__device__ __forceinline__ void sph_to_vec(double rad, double az, double pl, double out[3])
{
    const double ca = cos(az);
    out[0] = rn_mul(rn_mul(rad, ca), cos(pl));
    out[1] = rn_mul(rn_mul(rad, ca), sin(pl));
    out[2] = rn_mul(rad, sin(az));
}
// spherical_inversion: radius R^2 / r at the same angles (false for r == 0)
__device__ __forceinline__ bool sph_invert(const double v[3], double R, double out[3])
{
    const double r = sph_radius(v);
    if (r == 0) return false;
    sph_to_vec(rn_div(rn_mul(R, R), r), sph_azimut(v), sph_polar(v), out);
    return true;
}
// shifted(r, d_az, d_pl) of the spherical fork (tangle.c:622-629)
__device__ __forceinline__ void sph_rotate(const double v[3], double d_az, double d_pl, double out[3])
{
    sph_to_vec(sph_radius(v), rn_add(sph_azimut(v), d_az), rn_add(sph_polar(v), d_pl), out);
}
// seg_pwrap of the spherical fork (boundaries.c:36-72): r2's angles moved
// by whole periods (twice the half widths) toward r1's, then r2 rebuilt
// from its radius and those angles.
__device__ __forceinline__ void sph_pwrap(const Geometry &g, const double r1[3], double r2[3])
{
    const double A = g.sph_az, P = g.sph_pl;
    const double a1 = sph_azimut(r1), p1 = sph_polar(r1);
    double a2 = sph_azimut(r2), p2 = sph_polar(r2);
    const double A2 = rn_mul(2.0, A), P2 = rn_mul(2.0, P);
    int guard = 0;
    while (rn_sub(a2, a1) > A && guard++ < 64) a2 = rn_sub(a2, A2);
    while (rn_sub(a2, a1) < -A && guard++ < 128) a2 = rn_add(a2, A2);
    guard = 0;
    while (rn_sub(p2, p1) > P && guard++ < 64) p2 = rn_sub(p2, P2);
    while (rn_sub(p2, p1) < -P && guard++ < 128) p2 = rn_add(p2, P2);
    sph_to_vec(sph_radius(r2), a2, p2, r2);
}
// make_child_box of the spherical fork (octree.c:183-262) on (r, az, pl)
// bounds: child idx = 4 (upper azimuth) + 2 (upper polar) + (lower radius).
__device__ __forceinline__ void sph_child_box(const double b[3], const double t[3], int idx, double cb[3],
                                              double ct[3])
{
    const double mr = rn_div(rn_add(t[0], b[0]), 2.0), ma = rn_div(rn_add(t[1], b[1]), 2.0),
                 mp = rn_div(rn_add(t[2], b[2]), 2.0);
    if (idx & 1) { cb[0] = b[0]; ct[0] = mr; } else { cb[0] = mr; ct[0] = t[0]; }
    if (idx & 4) { cb[1] = ma; ct[1] = t[1]; } else { cb[1] = b[1]; ct[1] = ma; }
    if (idx & 2) { cb[2] = mp; ct[2] = t[2]; } else { cb[2] = b[2]; ct[2] = mp; }
}
// Lm of a spherical cell (octree.c:344-348 of the fork): the largest of the
// radial depth and the two chords at the outer radius.
__device__ __forceinline__ double sph_box_lm(const double b[3], const double t[3])
{
    const double rd = rn_sub(t[0], b[0]);
    const double az = rn_mul(rn_mul(t[0], 2.0), fabs(sin(rn_div(rn_sub(t[1], b[1]), 2.0))));
    const double pl = rn_mul(rn_mul(rn_mul(t[0], 2.0), fabs(sin(rn_div(rn_sub(t[2], b[2]), 2.0)))),
                             fabs(cos(rn_div(rn_add(t[1], b[1]), 2.0))));
    return rd > az ? (rd > pl ? rd : pl) : (az > pl ? az : pl);
}

// Largest side of a box, the reference's ternary (octree.c:302-306).
__device__ __forceinline__ double box_lm(const double b[3], const double t[3])
{
    double Lx = rn_sub(t[0], b[0]), Ly = rn_sub(t[1], b[1]), Lz = rn_sub(t[2], b[2]);
    return Lx > Ly ? (Lx > Lz ? Lx : Lz) : (Ly > Lz ? Ly : Lz);
}
#endif
