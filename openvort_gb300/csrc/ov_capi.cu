// ov_capi.cu - the C ABI of libovgpu (include/openvort_gpu.h).
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>

#include "ov_internal.cuh"
#include "ov_helium.cuh"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int ov_fail(ov_ctx *c, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

// vec3_normalize (vec3_math.c:208-217): multiply by the reciprocal length.
static void normalize_ref(const double in[3], double out[3])
{
    double s = 0;
    s += in[0] * in[0];
    s += in[1] * in[1];
    s += in[2] * in[2];
    if (in[0] == 0 && in[1] == 0 && in[2] == 0) {
        out[0] = in[0]; out[1] = in[1]; out[2] = in[2];
        return;
    }
    double inv = 1 / sqrt(s);
    for (int a = 0; a < 3; ++a) out[a] = in[a] * inv;
}

DevParams ov_dev_params(const ov_params &p)
{
    DevParams d;
    memset(&d, 0, sizeof d);
    d.kappa = p.kappa;
    d.a0 = p.vortex_width;
    d.alpha = p.alpha;
    d.alpha_p = p.alpha_p;
    d.theta = p.bh_resolution;
    d.friction = p.use_mutual_friction;
    d.use_bh = p.use_bh;
    d.rec_dist = p.rec_dist;
    const ov_ext_vel *src[3] = {&p.vn, &p.vs, &p.vb};
    int *types[3] = {&d.vn_type, &d.vs_type, &d.vb_type};
    double *dirs[3] = {d.vn_dir, d.vs_dir, d.vb_dir};
    double *s0[3] = {&d.vn_s0, &d.vs_s0, &d.vb_s0}, *s1[3] = {&d.vn_s1, &d.vs_s1, &d.vb_s1};
    double *tld[3] = {&d.vn_tld, &d.vs_tld, &d.vb_tld};
    for (int i = 0; i < 3; ++i) {
        *types[i] = src[i]->type;
        normalize_ref(src[i]->direction.p, dirs[i]);
        *s0[i] = src[i]->starting_strength;
        *s1[i] = src[i]->strength;
        *tld[i] = src[i]->time_of_linear_decrease;
    }
    return d;
}

extern "C" {

void ov_params_default(ov_params *p)
{
    memset(p, 0, sizeof *p);
    p->kappa = 9.97e-4;
    p->vortex_width = 1e-8;
    p->alpha = 0.034;
    p->alpha_p = 1.383e-2;
    p->use_mutual_friction = 1;
    p->use_bh = 1;
    p->bh_resolution = 0.4;
    p->vn.type = OV_SIMPLE;
    p->vn.strength = 10.493799;
    p->vn.direction.p[0] = 1.0;
    p->vs.type = OV_SIMPLE;
    p->vs.strength = 0.493799;
    p->vs.direction.p[0] = -1.0;
    p->vb.type = OV_NO_FLOW;
    p->dl_min = 0.5e-3;
    p->dl_max = 1.5e-3;
    p->rec_dist = 4e-4;
    p->reconnection_angle_cutoff = 5.0 * M_PI / 180.0;
    p->small_loop_cutoff = 5;
    p->use_freq_filter = 1;
    p->freq_to_cutoff = 4.0 / 5;
    p->num_threads = 1;
    p->pin_mode = OV_PINNED;
}

int ov_ctx_create(ov_ctx **out, int device)
{
    if (!out) return OV_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return OV_ERR_NODEVICE;
    }
    if (device < 0 || device >= n) return OV_ERR_ARG;
    ov_ctx *c = new ov_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    {
        int pma = 0, pmt = 0;
        cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device);
        cudaDeviceGetAttribute(&pmt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
        c->pageable = pma == 1 && pmt == 1;
    }
    ov_params_default(&c->params);
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
        delete c;
        return OV_ERR_CUDA;
    }
    *out = c;
    return OV_OK;
}

static void free_nodes(NodeArrays &a)
{
    double *ps[] = {a.x, a.y, a.z, a.tx, a.ty, a.tz, a.nx, a.ny, a.nz, a.vx, a.vy, a.vz, a.sx, a.sy, a.sz};
    for (double *p : ps)
        if (p) cudaFree(p);
    a = NodeArrays{};
}

}  // extern "C"

// Free every device and pinned buffer of the context and forget their sizes
// (streams, events and parameters stay): what the context holds after it is
// what it held when created.
// Destroy the captured graphs (buffers, layout or sizes changed).
static void ov_drop_graphs(ov_ctx *c)
{
    if (c->rk4_exec) cudaGraphExecDestroy(c->rk4_exec);
    c->rk4_exec = nullptr;
    c->rk4_key = 0;
    for (int i = 0; i < 4; ++i) {
        if (c->eval_exec[i]) cudaGraphExecDestroy(c->eval_exec[i]);
        c->eval_exec[i] = nullptr;
        c->eval_key[i] = 0;
    }
}

static void release_buffers(ov_ctx *c)
{
    cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    free_nodes(c->node);
    for (auto &s : c->stage) free_nodes(s);
    ov_tree_free(c->tree);
    void *dev[] = {c->fwd, c->rev, c->status, c->pin, c->dnodes, c->d_tid, c->d_qorder, c->d_tprm, c->d_mrange,
                   c->d_pairs, c->d_npairs, c->d_loop_off, c->d_loop_nodes, c->d_loop_buf, c->d_loop_cut,
                   c->rec_nodes, c->rec_pair, c->rec_out, c->rec_corr, c->rec_part, c->rec_split, c->fft_buf,
                   c->fft_tw, c->long_buf, c->d_rm, c->d_rm_lim, c->dsum, c->part, c->d_node_counts, c->flush_buf,
                   c->d_stage, c->d_time};
    for (void *p : dev)
        if (p) cudaFree(p);
    void *pinned[] = {c->h_stage, c->h_corr, c->h_pf, c->h_time};
    for (void *p : pinned)
        if (p) cudaFreeHost(p);
    ov_drop_graphs(c);
    c->fwd = c->rev = c->status = c->pin = c->dnodes = c->d_tid = c->d_qorder = nullptr;
    c->d_tprm = nullptr;
    c->d_mrange = nullptr;
    c->d_pairs = c->d_npairs = c->d_loop_off = c->d_loop_nodes = nullptr;
    c->d_loop_buf = c->d_loop_cut = nullptr;
    c->rec_nodes = c->rec_pair = nullptr;
    c->rec_out = c->rec_corr = c->rec_part = nullptr;
    c->rec_split = nullptr;
    c->fft_buf = c->fft_tw = nullptr;
    c->long_buf = nullptr;
    c->d_rm = nullptr;
    c->d_rm_lim = nullptr;
    c->dsum = c->part = nullptr;
    c->d_node_counts = nullptr;
    c->flush_buf = nullptr;
    c->d_stage = nullptr;
    c->d_time = nullptr;
    c->h_stage = c->h_corr = c->h_pf = c->h_pf_dev = c->h_time = nullptr;
    c->cap = c->n_live = 0;
    c->tcap = c->rm_cap = c->rm_lim_cap = c->pair_cap = c->loop_cap = c->loop_nodes_cap = 0;
    c->rec_cap = c->rec_split_cap = c->dsum_cap = 0;
    c->fft_cap = c->long_cap = c->loop_buf_cap = c->part_cap = c->rec_part_cap = c->h_corr_cap = 0;
    c->h_stage_bytes = c->d_stage_bytes = c->node_counts_cap = c->flush_bytes = 0;
    c->fft_M = 0;
    c->time_dev_index = -1;
    c->uploaded = c->tree_built = c->host_valid = false;
}

int ov_alloc_gate(ov_ctx *c)
{
    if (c->alloc_fail_after < 0) return OV_OK;
    if (c->alloc_fail_after == 0) {
        c->alloc_fail_after = -1;   // one failure, then allocations run again
        return OV_ERR_ALLOC;
    }
    --c->alloc_fail_after;
    return OV_OK;
}

int ov_alloc_failed(ov_ctx *c, const char *why, const char *what)
{
    release_buffers(c);
    return ov_fail(c, OV_ERR_ALLOC, "allocation failed (%s): %s; the context holds no tangle now", why, what);
}

extern "C" {

int ov_ctx_destroy(ov_ctx *c)
{
    if (!c) return OV_OK;
    cudaSetDevice(c->device);
    release_buffers(c);
    if (c->rec_ev) cudaEventDestroy(c->rec_ev);
    for (int i = 0; i < 4; ++i)
        if (c->ph[i]) cudaEventDestroy(c->ph[i]);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->join_ev) cudaEventDestroy(c->join_ev);
    delete c;
    return OV_OK;
}

int ov_set_depth_policy(ov_ctx *c, int strict)
{
    if (!c) return OV_ERR_ARG;
    c->strict_depth = strict != 0;
    return OV_OK;
}

int ov_inject_alloc_failure(ov_ctx *c, int after)
{
    if (!c || after < -1) return OV_ERR_ARG;
    c->alloc_fail_after = after;
    return OV_OK;
}

const char *ov_last_error(const ov_ctx *c) { return c ? c->err.c_str() : "null context"; }

int ov_set_params(ov_ctx *c, const ov_params *p)
{
    if (!c || !p) return OV_ERR_ARG;
    c->params = *p;
    for (Member &m : c->mem) m.params = *p;   // an ensemble: every member
    if (c->mem.size() > 1 && c->d_tprm) return ov_upload_member_tables(c);
    return OV_OK;
}

int ov_set_host_access(ov_ctx *c, int direct)
{
    if (!c) return OV_ERR_ARG;
    c->host_direct = direct != 0;
    return OV_OK;
}

int ov_get_host_access(const ov_ctx *c) { return c && c->pageable && c->host_direct ? 1 : 0; }

int ov_set_rk4_graph(ov_ctx *c, int on)
{
    if (!c) return OV_ERR_ARG;
    c->use_graph = on != 0;
    return OV_OK;
}

int ov_set_precision(ov_ctx *c, int precision)
{
    if (!c || (precision != OV_PREC_FP64 && precision != OV_PREC_MIXED && precision != OV_PREC_DD)) return OV_ERR_ARG;
    c->precision = precision;
    return OV_OK;
}

int ov_set_walk(ov_ctx *c, int walk)
{
    if (!c || (walk != OV_WALK_SPLIT && walk != OV_WALK_FP64)) return OV_ERR_ARG;
    c->walk = walk;
    return OV_OK;
}

int ov_get_walk(const ov_ctx *c) { return c ? c->walk : -1; }

void *ov_ctx_stream(ov_ctx *c) { return c ? (void *)c->stream : nullptr; }

int ov_capacity(const ov_ctx *c) { return c ? c->cap : 0; }

int ov_tangle_info(const ov_ctx *c, int *n_slots, int *next_empty, int *total_empty)
{
    if (!c) return OV_ERR_ARG;
    if (c->mem.size() == 1) return ov_member_info(c, 0, n_slots, next_empty, total_empty);
    // an ensemble: the whole pool
    int te = 0;
    for (const Member &m : c->mem) te += m.total_empty + (m.cap - m.n);
    if (n_slots) *n_slots = c->n_live;
    if (next_empty) *next_empty = -1;
    if (total_empty) *total_empty = te;
    return OV_OK;
}

int ov_member_info(const ov_ctx *c, int i, int *n_slots, int *next_empty, int *total_empty)
{
    if (!c || i < 0 || i >= (int)c->mem.size()) return OV_ERR_ARG;
    const Member &m = c->mem[i];
    if (n_slots) *n_slots = m.n;
    if (next_empty) *next_empty = m.next_empty;
    if (total_empty) *total_empty = m.total_empty;
    return OV_OK;
}

int ov_ensemble_size(const ov_ctx *c) { return c ? (int)c->mem.size() : 0; }

int ov_get_tuning(const ov_ctx *c, ov_tuning *out)
{
    if (!c || !out) return OV_ERR_ARG;
    out->warps_per_block = c->tune.warps;
    out->query_groups = c->tune.groups;
    out->blocks_per_sm = c->tune.blocks_per_sm;
    out->largest_first = c->tune.largest_first;
    out->high_occupancy = c->tune.hi_occ;
    return OV_OK;
}

int ov_set_tuning(ov_ctx *c, const ov_tuning *tu)
{
    if (!c || !tu) return OV_ERR_ARG;
    if ((tu->warps_per_block != 2 && tu->warps_per_block != 4 && tu->warps_per_block != 8) ||
        tu->query_groups < 0 || tu->query_groups > 27 || tu->blocks_per_sm < 0 || tu->blocks_per_sm > 64 ||
        tu->high_occupancy < 0 || tu->high_occupancy > 4)
        return ov_fail(c, OV_ERR_ARG, "tuning out of range");
    c->tune.warps = tu->warps_per_block;
    c->tune.groups = tu->query_groups;
    c->tune.blocks_per_sm = tu->blocks_per_sm;
    c->tune.largest_first = tu->largest_first != 0;
    c->tune.hi_occ = tu->high_occupancy;
    if (c->uploaded && c->mem.size() > 1) return ov_upload_member_tables(c);
    return OV_OK;
}

}  // extern "C"

static int alloc_nodes(ov_ctx *c, NodeArrays &a, int cap)
{
    size_t b = (size_t)cap * sizeof(double);
    double **ps[] = {&a.x, &a.y, &a.z, &a.tx, &a.ty, &a.tz, &a.nx, &a.ny, &a.nz, &a.vx, &a.vy, &a.vz,
                     &a.sx, &a.sy, &a.sz};
    for (double **p : ps) {
        OV_ALLOC(c, cudaMalloc(p, b));
        OV_CUDA(c, cudaMemsetAsync(*p, 0, b, c->stream));
    }
    return OV_OK;
}

static int ensure_capacity(ov_ctx *c, int cap)
{
    if (cap <= c->cap && c->node.x) return OV_OK;
    cudaStreamSynchronize(c->stream);
    free_nodes(c->node);
    for (auto &s : c->stage) free_nodes(s);
    int *is[] = {c->fwd, c->rev, c->status, c->pin};
    for (int *p : is)
        if (p) cudaFree(p);
    ov_drop_graphs(c);
    int r;
    if ((r = alloc_nodes(c, c->node, cap))) return r;
    for (auto &s : c->stage)
        if ((r = alloc_nodes(c, s, cap))) return r;
    OV_ALLOC(c, cudaMalloc(&c->fwd, (size_t)cap * 4));
    OV_ALLOC(c, cudaMalloc(&c->rev, (size_t)cap * 4));
    OV_ALLOC(c, cudaMalloc(&c->status, (size_t)cap * 4));
    OV_ALLOC(c, cudaMalloc(&c->pin, (size_t)cap * 4));
    if ((r = ov_tree_reserve(c, cap))) return r;
    c->cap = cap;
    return OV_OK;
}

int ov_grow_preserving(ov_ctx *c, int cap)
{
    if (cap <= c->cap) return OV_OK;
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    int old = c->cap;
    size_t nb = (size_t)old * sizeof(double), nn = (size_t)cap * sizeof(double);
    double **ps[] = {&c->node.x, &c->node.y, &c->node.z, &c->node.tx, &c->node.ty, &c->node.tz, &c->node.nx,
                     &c->node.ny, &c->node.nz, &c->node.vx, &c->node.vy, &c->node.vz, &c->node.sx, &c->node.sy,
                     &c->node.sz};
    for (double **p : ps) {
        double *q = nullptr;
        OV_ALLOC(c, cudaMalloc(&q, nn));
        OV_CUDA(c, cudaMemsetAsync(q, 0, nn, c->stream));
        OV_CUDA(c, cudaMemcpyAsync(q, *p, nb, cudaMemcpyDeviceToDevice, c->stream));
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaFree(*p);
        *p = q;
    }
    int **is[] = {&c->fwd, &c->rev, &c->status, &c->pin};
    for (int **p : is) {
        int *q = nullptr;
        OV_ALLOC(c, cudaMalloc(&q, (size_t)cap * 4));
        OV_CUDA(c, cudaMemsetAsync(q, 0xFF, (size_t)cap * 4, c->stream));   // -1: EMPTY / no link
        OV_CUDA(c, cudaMemcpyAsync(q, *p, (size_t)old * 4, cudaMemcpyDeviceToDevice, c->stream));
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaFree(*p);
        *p = q;
    }
    for (auto &s : c->stage) free_nodes(s);
    int r;
    for (auto &s : c->stage)
        if ((r = alloc_nodes(c, s, cap))) return r;
    ov_drop_graphs(c);
    if ((r = ov_tree_reserve(c, cap))) return r;
    c->cap = cap;
    return OV_OK;
}

static int ensure_stage(ov_ctx *c, size_t bytes)
{
    if (c->h_stage_bytes >= bytes) return OV_OK;
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    OV_ALLOC(c, cudaMallocHost(&c->h_stage, bytes));
    c->h_stage_bytes = bytes;
    return OV_OK;
}

// The device copy of a host tangle's arrays (raw layout: the five vec3 fields
// at f * n * 24 bytes, then connections and status at 120 n and 128 n).
static int ensure_dstage(ov_ctx *c, size_t bytes)
{
    if (c->d_stage_bytes >= bytes) return OV_OK;
    if (c->d_stage) cudaFree(c->d_stage);
    c->d_stage = nullptr;
    OV_ALLOC(c, cudaMalloc(&c->d_stage, bytes));
    c->d_stage_bytes = bytes;
    return OV_OK;
}

struct NodePtrs {
    double *d[15];   // x y z, vx vy vz, sx sy sz, tx ty tz, nx ny nz
    int *fwd, *rev, *status, *pin;
};

__host__ __device__ inline size_t stage_topo_off(int n) { return (size_t)n * 120; }

// Where the host-layout data of a transfer sits: the device stage (one copy
// of each host array), or the caller's arrays themselves when the device
// reads and writes pageable host memory.
struct HostView {
    ov_vec3 *f[5];           // positions, vels, vs, tangents, normals (null: absent)
    ov_neighbour *con;
    ov_node_status *st;
};

static HostView stage_view(char *stage, int n)
{
    HostView v;
    for (int f = 0; f < 5; ++f) v.f[f] = reinterpret_cast<ov_vec3 *>(stage + (size_t)f * n * 24);
    v.con = reinterpret_cast<ov_neighbour *>(stage + stage_topo_off(n));
    v.st = reinterpret_cast<ov_node_status *>(stage + stage_topo_off(n) + (size_t)n * 8);
    return v;
}

// Host layout (vec3 fields, ov_neighbour, ov_node_status) -> device arrays for
// slots [0, cap): slots past n get zeros, -1 links, EMPTY, no wall.
__global__ void k_unpack(HostView src, unsigned fields, unsigned have, int n, int cap, NodePtrs d)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cap) return;
    const unsigned bits[5] = {OV_F_POS, OV_F_VELS, OV_F_VS, OV_F_TANGENTS, OV_F_NORMALS};
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        if (!(fields & bits[f])) continue;
        const bool in = k < n && (have & bits[f]);
        for (int a = 0; a < 3; ++a) d.d[3 * f + a][k] = in ? src.f[f][k].p[a] : 0.0;
    }
    if (fields & OV_F_TOPOLOGY) {
        const bool in = k < n;
        d.fwd[k] = in ? src.con[k].forward : -1;
        d.rev[k] = in ? src.con[k].reverse : -1;
        d.status[k] = in ? src.st[k].status : OV_EMPTY;
        d.pin[k] = in ? src.st[k].pin_wall : OV_NOT_A_FACE;
    }
}

// Device slots [lo, lo + n) -> host layout, links shifted by -lo.
__global__ void k_pack(unsigned fields, int lo, int n, NodePtrs d, HostView dst)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned bits[5] = {OV_F_POS, OV_F_VELS, OV_F_VS, OV_F_TANGENTS, OV_F_NORMALS};
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        if (!(fields & bits[f]) || !dst.f[f]) continue;
        for (int a = 0; a < 3; ++a) dst.f[f][k].p[a] = d.d[3 * f + a][lo + k];
    }
    if (fields & OV_F_TOPOLOGY) {
        const int f = d.fwd[lo + k], b = d.rev[lo + k];
        dst.con[k].forward = f >= 0 ? f - lo : -1;
        dst.con[k].reverse = b >= 0 ? b - lo : -1;
        dst.st[k].status = d.status[lo + k];
        dst.st[k].pin_wall = d.pin[lo + k];
    }
}

static NodePtrs node_ptrs(ov_ctx *c)
{
    NodePtrs p;
    double *dd[15] = {c->node.x, c->node.y, c->node.z, c->node.vx, c->node.vy, c->node.vz,
                      c->node.sx, c->node.sy, c->node.sz, c->node.tx, c->node.ty, c->node.tz,
                      c->node.nx, c->node.ny, c->node.nz};
    for (int i = 0; i < 15; ++i) p.d[i] = dd[i];
    p.fwd = c->fwd; p.rev = c->rev; p.status = c->status; p.pin = c->pin;
    return p;
}

static void set_geometry(ov_ctx *c, const ov_domain_box &box, const ov_boundary_images &bimg)
{
    Geometry &g = c->geo;
    memset(&g, 0, sizeof g);
    for (int a = 0; a < 3; ++a) {
        g.lo[a] = box.bottom_left_back.p[a];
        g.hi[a] = box.top_right_front.p[a];
        g.L[a] = g.hi[a] - g.lo[a];
    }
    for (int f = 0; f < 6; ++f) g.wall[f] = box.wall[f];
    g.periodic[0] = box.wall[OV_LEFT] == OV_WALL_PERIODIC;
    g.periodic[1] = box.wall[OV_BACK] == OV_WALL_PERIODIC;
    g.periodic[2] = box.wall[OV_DOWN] == OV_WALL_PERIODIC;
    g.n_img = std::min(bimg.n, OV_MAX_IMAGES);
    for (int j = 0; j < g.n_img && bimg.images; ++j) {
        for (int a = 0; a < 3; ++a) {
            g.shift[j][a] = bimg.images[j].shift[a];
            g.reflect[j][a] = bimg.images[j].reflect[a];
        }
        g.nreflect[j] = std::min(std::max(bimg.images[j].number_of_reflects, 0), 3);
    }
    // grid step of the mixed path: a power of two with every coordinate the
    // traversal meets (box, one period either side) below 2^22 steps
    double m = 0;
    for (int a = 0; a < 3; ++a) m = std::max(m, std::max(fabs(g.lo[a]), fabs(g.hi[a])) + 2 * fabs(g.L[a]));
    int e = (int)ceil(log2(m > 0 ? m : 1.0));
    c->grid_h = ldexp(1.0, e - 22);
}

// Per-member device tables: build table, parameters, queue order, slot
// ranges, and (ensembles) the member of every slot.
int ov_reserve_members(ov_ctx *c, int nt)
{
    nt = std::max(nt, 1);
    if (c->tree.tt && c->tcap >= nt) return OV_OK;
    ov_drop_graphs(c);   // the tables move
    if (c->tree.tt) cudaFree(c->tree.tt);
    if (c->d_tprm) cudaFree(c->d_tprm);
    if (c->d_qorder) cudaFree(c->d_qorder);
    if (c->d_mrange) cudaFree(c->d_mrange);
    c->tree.tt = nullptr; c->d_tprm = nullptr; c->d_qorder = nullptr; c->d_mrange = nullptr;
    c->tcap = 0;
    OV_ALLOC(c, cudaMalloc(&c->tree.tt, (size_t)nt * TT_WORDS * 4));
    OV_CUDA(c, cudaMemset(c->tree.tt, 0, (size_t)nt * TT_WORDS * 4));
    OV_ALLOC(c, cudaMalloc(&c->d_tprm, (size_t)nt * sizeof(DevParams)));
    OV_ALLOC(c, cudaMalloc(&c->d_qorder, (size_t)nt * 4));
    OV_ALLOC(c, cudaMalloc(&c->d_mrange, (size_t)nt * sizeof(int2)));
    c->tcap = nt;
    return OV_OK;
}

int ov_upload_member_tables(ov_ctx *c)
{
    const int nt = (int)c->mem.size();
    int r;
    if ((r = ov_reserve_members(c, nt))) return r;
    // member-id bits above each key: ids 0..nt-1 are never all ones (an
    // all-ones upper half marks an EMPTY slot for the sort's fix-up)
    c->key_tbits = 0;
    if (nt > 1)
        while ((1 << c->key_tbits) <= nt) ++c->key_tbits;
    c->key_levels = std::min(OV_MAX_LEVEL, (63 - c->key_tbits) / 3);
    // (the graphs' key covers the layout, parameters and table pointers; the
    // per-slot member table of an ensemble is reallocated below)
    if (nt > 1) ov_drop_graphs(c);
    std::vector<DevParams> prm(nt);
    std::vector<int> q(nt);
    std::vector<int2> rng(nt);
    for (int i = 0; i < nt; ++i) {
        prm[i] = ov_dev_params(c->mem[i].params);
        q[i] = i;
        rng[i] = make_int2(c->mem[i].lo, c->mem[i].lo + c->mem[i].cap);
    }
    if (c->tune.largest_first)
        std::stable_sort(q.begin(), q.end(), [&](int a, int b) { return c->mem[a].n > c->mem[b].n; });
    OV_CUDA(c, cudaMemcpy(c->d_tprm, prm.data(), nt * sizeof(DevParams), cudaMemcpyHostToDevice));
    OV_CUDA(c, cudaMemcpy(c->d_qorder, q.data(), nt * 4, cudaMemcpyHostToDevice));
    OV_CUDA(c, cudaMemcpy(c->d_mrange, rng.data(), nt * sizeof(int2), cudaMemcpyHostToDevice));
    if (nt > 1) {
        if (c->d_tid) cudaFree(c->d_tid);
        c->d_tid = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->d_tid, (size_t)std::max(c->cap, 1) * 4));
        std::vector<int> tid(std::max(c->cap, 1), 0);
        for (int i = 0; i < nt; ++i)
            for (int k = 0; k < c->mem[i].cap; ++k) tid[c->mem[i].lo + k] = i;
        OV_CUDA(c, cudaMemcpy(c->d_tid, tid.data(), tid.size() * 4, cudaMemcpyHostToDevice));
    }
    return OV_OK;
}

// Move the per-slot device arrays that have no host mirror (tangents,
// normals, vels, vs) from the member layout `old` to the context's current
// one (the context already holds enough slots).
int ov_move_device_slots(ov_ctx *c, const std::vector<Member> &old)
{
    size_t n = (size_t)std::max(c->n_live, 1);
    double *tmp = nullptr;
    OV_ALLOC(c, cudaMalloc(&tmp, n * sizeof(double)));
    double *arrs[12] = {c->node.tx, c->node.ty, c->node.tz, c->node.nx, c->node.ny, c->node.nz,
                        c->node.vx, c->node.vy, c->node.vz, c->node.sx, c->node.sy, c->node.sz};
    int r = OV_OK;
    for (double *arr : arrs) {
        if (cudaMemsetAsync(tmp, 0, n * sizeof(double), c->stream) != cudaSuccess) { r = OV_ERR_CUDA; break; }
        for (size_t i = 0; i < old.size() && i < c->mem.size(); ++i) {
            size_t len = (size_t)std::min(old[i].cap, c->mem[i].cap);
            if (len && cudaMemcpyAsync(tmp + c->mem[i].lo, arr + old[i].lo, len * sizeof(double),
                                       cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
                r = OV_ERR_CUDA;
        }
        if (cudaMemcpyAsync(arr, tmp, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
            r = OV_ERR_CUDA;
    }
    cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    if (r) return ov_fail(c, r, "moving member slots failed");
    return OV_OK;
}

extern "C" {

int ov_upload_ensemble(ov_ctx *c, const ov_tangle_state *const *ts, const ov_params *params, int n,
                       double headroom)
{
    if (!c || !ts || !params || n < 1 || !(headroom >= 1.0 && headroom <= 64.0)) return OV_ERR_ARG;
    cudaSetDevice(c->device);
    for (int i = 0; i < n; ++i) {
        const ov_tangle_state *t = ts[i];
        if (!t || t->N < 0) return ov_fail(c, OV_ERR_ARG, "member %d: no tangle", i);
        if (memcmp(&t->box, &ts[0]->box, sizeof t->box) != 0 || t->bimg.n != ts[0]->bimg.n)
            return ov_fail(c, OV_ERR_ARG, "member %d: box or image set differs from member 0", i);
        for (int j = 0; j < t->bimg.n; ++j)
            if (!t->bimg.images || !ts[0]->bimg.images ||
                memcmp(&t->bimg.images[j], &ts[0]->bimg.images[j], sizeof(ov_image_tangle)) != 0)
                return ov_fail(c, OV_ERR_ARG, "member %d: image %d differs from member 0", i, j);
        const ov_params &p = params[i], &p0 = params[0];
        if (p.kappa != p0.kappa || p.bh_resolution != p0.bh_resolution || p.use_bh != p0.use_bh)
            return ov_fail(c, OV_ERR_ARG, "member %d: KAPPA, BH_resolution and use_BH must be shared", i);
    }
    std::vector<Member> mem(n);
    long long lo = 0;
    for (int i = 0; i < n; ++i) {
        Member &m = mem[i];
        m.lo = (int)lo;
        m.n = ts[i]->N;
        m.cap = std::max(m.n, (int)std::min(ceil((double)m.n * headroom), 1e9));
        m.next_empty = ts[i]->next_empty;
        m.total_empty = ts[i]->total_empty;
        m.params = params[i];
        lo += m.cap;
        if (lo > (1LL << 30)) return ov_fail(c, OV_ERR_ARG, "ensemble of more than 2^30 slots");
    }
    int r;
    for (int i = 0; i < n; ++i) {
        const ov_tangle_state *t = ts[i];
        for (int k = 0; k < t->N; ++k) {
            int f = t->connections[k].forward, b = t->connections[k].reverse, st = t->status[k].status;
            if (f < -1 || f >= t->N || b < -1 || b >= t->N || st < OV_EMPTY || st > OV_PINNED_SLIP)
                return ov_fail(c, OV_ERR_TOPOLOGY, "member %d node %d: connections (%d,%d) / status %d out of range",
                               i, k, f, b, st);
        }
    }
    const int total = (int)lo;
    if ((r = ensure_capacity(c, std::max(total, 1)))) return r;
    c->mem = mem;
    c->n_live = total;
    c->params = params[0];
    c->tree_built = false;
    c->host_valid = false;
    set_geometry(c, ts[0]->box, ts[0]->bimg);
    if ((r = ov_upload_member_tables(c))) return r;
    size_t cap = (size_t)c->cap;
    if ((r = ensure_stage(c, cap * 3 * sizeof(double) * 5 + cap * 4 * sizeof(int)))) return r;
    double *h = c->h_stage;
    int *hi = (int *)(h + 15 * cap);
    std::fill(h, h + 15 * cap, 0.0);
    std::fill(hi, hi + 2 * cap, -1);
    std::fill(hi + 2 * cap, hi + 3 * cap, (int)OV_EMPTY);
    std::fill(hi + 3 * cap, hi + 4 * cap, (int)OV_NOT_A_FACE);
    for (int i = 0; i < n; ++i) {
        const ov_tangle_state *t = ts[i];
        const size_t o = (size_t)mem[i].lo;
        const ov_vec3 *src[5] = {t->vnodes, t->vels, t->vs, t->tangents, t->normals};
        for (int f = 0; f < 5; ++f) {
            if (!src[f]) continue;
            double *dst = h + 3 * cap * f;
            for (int a = 0; a < 3; ++a)
                for (int k = 0; k < t->N; ++k) dst[a * cap + o + k] = src[f][k].p[a];
        }
        for (int k = 0; k < t->N; ++k) {
            int f = t->connections[k].forward, b = t->connections[k].reverse;
            hi[o + k] = f >= 0 ? f + (int)o : -1;
            hi[cap + o + k] = b >= 0 ? b + (int)o : -1;
            hi[2 * cap + o + k] = t->status[k].status;
            hi[3 * cap + o + k] = t->status[k].pin_wall;
        }
    }
    double *dd[15] = {c->node.x, c->node.y, c->node.z, c->node.vx, c->node.vy, c->node.vz,
                      c->node.sx, c->node.sy, c->node.sz, c->node.tx, c->node.ty, c->node.tz,
                      c->node.nx, c->node.ny, c->node.nz};
    for (int k = 0; k < 15; ++k)
        OV_CUDA(c, cudaMemcpyAsync(dd[k], h + k * cap, cap * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int *di[4] = {c->fwd, c->rev, c->status, c->pin};
    for (int i = 0; i < 4; ++i)
        OV_CUDA(c, cudaMemcpyAsync(di[i], hi + i * cap, cap * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    c->last_h2d = cap * (15 * sizeof(double) + 4 * sizeof(int));
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    c->uploaded = true;
    return OV_OK;
}

int ov_set_member_params(ov_ctx *c, int i, const ov_params *p)
{
    if (!c || !p || i < 0 || i >= (int)c->mem.size()) return OV_ERR_ARG;
    const ov_params &p0 = c->params;
    if (c->mem.size() > 1 && (p->kappa != p0.kappa || p->bh_resolution != p0.bh_resolution || p->use_bh != p0.use_bh))
        return ov_fail(c, OV_ERR_ARG, "KAPPA, BH_resolution and use_BH are shared by the members");
    c->mem[i].params = *p;
    if (c->mem.size() == 1) c->params = *p;
    if (c->uploaded && c->mem.size() > 1) return ov_upload_member_tables(c);
    return OV_OK;
}

int ov_upload_tangle(ov_ctx *c, const ov_tangle_state *t) { return ov_upload_tangle_fields(c, t, OV_F_ALL); }

int ov_upload_tangle_fields(ov_ctx *c, const ov_tangle_state *t, unsigned fields)
{
    if (!c || !t || t->N < 0) return OV_ERR_ARG;
    cudaSetDevice(c->device);
    int n = t->N;
    int r;
    int old_cap = c->cap;
    if ((r = ensure_capacity(c, std::max(n, 1)))) return r;
    if (!c->uploaded || c->cap != old_cap || c->n_live != n || c->mem.size() != 1)
        fields |= OV_F_POS | OV_F_TOPOLOGY;
    c->n_live = n;   // slots past t->N (a smaller tangle in a larger context) are EMPTY
    c->tree_built = false;
    c->host_valid = false;
    if (c->mem.size() != 1) c->mem.assign(1, Member{});
    Member &m0 = c->mem[0];
    m0.lo = 0;
    m0.n = n;
    m0.cap = n;
    m0.next_empty = t->next_empty;
    m0.total_empty = t->total_empty;
    m0.params = c->params;
    set_geometry(c, t->box, t->bimg);
    if ((r = ov_upload_member_tables(c))) return r;
    size_t cap = (size_t)c->cap;
    if (fields & OV_F_TOPOLOGY) {
        for (int k = 0; k < n; ++k) {
            int f = t->connections[k].forward, b = t->connections[k].reverse, st = t->status[k].status;
            if (f < -1 || f >= n || b < -1 || b >= n || st < OV_EMPTY || st > OV_PINNED_SLIP)
                return ov_fail(c, OV_ERR_TOPOLOGY, "node %d: connections (%d,%d) / status %d out of range", k, f, b, st);
        }
    }
    // the transposition to the device's arrays (k_unpack) reads the caller's
    // arrays in place when the device reads pageable host memory, else one
    // copy of each into the device stage
    const ov_vec3 *src[5] = {t->vnodes, t->vels, t->vs, t->tangents, t->normals};
    const unsigned bits[5] = {OV_F_POS, OV_F_VELS, OV_F_VS, OV_F_TANGENTS, OV_F_NORMALS};
    const bool direct = c->pageable && c->host_direct;
    HostView view = {};
    if (direct) {
        for (int f = 0; f < 5; ++f) view.f[f] = const_cast<ov_vec3 *>(src[f]);
        view.con = t->connections;
        view.st = t->status;
    } else {
        const size_t bytes = stage_topo_off(n) + (size_t)n * 16;
        if ((r = ensure_dstage(c, std::max(bytes, (size_t)16)))) return r;
        view = stage_view(c->d_stage, n);
    }
    unsigned have = 0;
    c->last_h2d = 0;
    for (int f = 0; f < 5; ++f) {
        if (!(fields & bits[f])) continue;
        if (src[f] && n > 0) {
            if (!direct)
                OV_CUDA(c, cudaMemcpyAsync(view.f[f], src[f], (size_t)n * 24, cudaMemcpyHostToDevice, c->stream));
            have |= bits[f];
        }
        c->last_h2d += 3 * cap * sizeof(double);
    }
    if ((fields & OV_F_TOPOLOGY) && n > 0 && !direct) {
        OV_CUDA(c, cudaMemcpyAsync(view.con, t->connections, (size_t)n * 8, cudaMemcpyHostToDevice, c->stream));
        OV_CUDA(c, cudaMemcpyAsync(view.st, t->status, (size_t)n * 8, cudaMemcpyHostToDevice, c->stream));
    }
    if (fields & OV_F_TOPOLOGY) c->last_h2d += 4 * cap * sizeof(int);
    k_unpack<<<(unsigned)((cap + 255) / 256), 256, 0, c->stream>>>(view, fields, have, n, (int)cap, node_ptrs(c));
    c->launches++;
    OV_CUDA(c, cudaGetLastError());
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    c->uploaded = true;
    return OV_OK;
}

// Copy slots [lo, lo + span) of the device pool into host tangle slots
// [0, min(span, t->N)), connections shifted by -lo; host slots past span
// become EMPTY.
static int download_range(ov_ctx *c, ov_tangle_state *t, unsigned fields, int lo, int span, int next_empty,
                          int total_empty)
{
    const int n = std::min(t->N, span);
    int r;
    const unsigned bits[5] = {OV_F_POS, OV_F_VELS, OV_F_VS, OV_F_TANGENTS, OV_F_NORMALS};
    ov_vec3 *dst[5] = {t->vnodes, t->vels, t->vs, t->tangents, t->normals};
    if (n > 0) {
        // the device's arrays transposed to the host layout (k_pack): straight
        // into the caller's arrays when the device writes pageable host
        // memory, else into the device stage and one copy each
        const bool direct = c->pageable && c->host_direct;
        HostView view = {};
        if (direct) {
            for (int f = 0; f < 5; ++f) view.f[f] = dst[f];
            view.con = t->connections;
            view.st = t->status;
        } else {
            const size_t bytes = stage_topo_off(n) + (size_t)n * 16;
            if ((r = ensure_dstage(c, std::max(bytes, (size_t)16)))) return r;
            view = stage_view(c->d_stage, n);
            for (int f = 0; f < 5; ++f)
                if (!dst[f]) view.f[f] = nullptr;
        }
        k_pack<<<(n + 255) / 256, 256, 0, c->stream>>>(fields, lo, n, node_ptrs(c), view);
        c->launches++;
        if (!direct) {
            for (int f = 0; f < 5; ++f) {
                if (!(fields & bits[f]) || !dst[f]) continue;
                OV_CUDA(c, cudaMemcpyAsync(dst[f], view.f[f], (size_t)n * 24, cudaMemcpyDeviceToHost, c->stream));
            }
            if (fields & OV_F_TOPOLOGY) {
                OV_CUDA(c, cudaMemcpyAsync(t->connections, view.con, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
                OV_CUDA(c, cudaMemcpyAsync(t->status, view.st, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
            }
        }
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    for (int f = 0; f < 5; ++f) {
        if (!(fields & bits[f]) || !dst[f]) continue;
        for (int k = n; k < t->N; ++k)
            for (int a = 0; a < 3; ++a) dst[f][k].p[a] = 0.0;
    }
    if (fields & OV_F_TOPOLOGY) {
        t->next_empty = next_empty;
        t->total_empty = total_empty;
        for (int k = n; k < t->N; ++k) {
            t->connections[k].forward = t->connections[k].reverse = -1;
            t->status[k].status = OV_EMPTY;
            t->status[k].pin_wall = OV_NOT_A_FACE;
        }
    }
    return OV_OK;
}

int ov_download_member(ov_ctx *c, int i, ov_tangle_state *t, unsigned fields)
{
    if (!c || !t || i < 0 || i >= (int)c->mem.size()) return OV_ERR_ARG;
    if (!c->uploaded) return ov_fail(c, OV_ERR_STATE, "no tangle uploaded");
    cudaSetDevice(c->device);
    const Member &m = c->mem[i];
    if (t->N < m.n)
        return ov_fail(c, OV_ERR_ARG, "host tangle has %d slots, member %d holds %d (expand it first)", t->N, i, m.n);
    // slots of the host tangle past the member's N are EMPTY
    const int span = c->mem.size() == 1 ? c->cap : m.cap;
    return download_range(c, t, fields, m.lo, span, m.next_empty, m.total_empty + (t->N - m.n));
}

int ov_download_tangle(ov_ctx *c, ov_tangle_state *t, unsigned fields)
{
    if (!c || !t) return OV_ERR_ARG;
    if (c->mem.size() > 1)
        return ov_fail(c, OV_ERR_STATE, "the context holds an ensemble: use ov_download_member");
    return ov_download_member(c, 0, t, fields);
}

}  // extern "C"

static int check_ready(ov_ctx *c)
{
    if (!c) return OV_ERR_ARG;
    if (!c->uploaded) return ov_fail(c, OV_ERR_STATE, "no tangle uploaded");
    cudaSetDevice(c->device);
    return OV_OK;
}

// Read back the device counters of the last build/evaluation into ctx->stats.
static int collect_stats(ov_ctx *c, bool sync)
{
    int host[TC_WORDS];
    if (sync) OV_CUDA(c, cudaStreamSynchronize(c->stream));
    OV_CUDA(c, cudaMemcpy(host, c->tree.counters, sizeof host, cudaMemcpyDeviceToHost));
    unsigned long long *s64 = (unsigned long long *)(host + TC_STAT64);
    c->stats.node_evals = host[TC_NNE];
    c->stats.cells = host[TC_NCELL];
    c->stats.max_depth = host[TC_MAXDEPTH];
    c->stats.out_of_root = host[TC_OUT];
    c->stats.visits = (int64_t)s64[ST_VISITS];
    c->stats.accepts = (int64_t)s64[ST_ACCEPTS];
    c->stats.warp_steps = (int64_t)s64[ST_STEPS];
    c->stats.fp64_fallbacks = (int64_t)s64[ST_FALLBACK];
    c->stats.near_field_fp64 = (int64_t)s64[ST_NEAR64];
    c->stats.error_word = host[TC_ERR];
    return OV_OK;
}

static int error_from_word(ov_ctx *c)
{
    int w = (int)c->stats.error_word;
    if (!w) return OV_OK;
    if (w & OV_EW_NAN) return ov_fail(c, OV_ERR_NAN, "non-finite node position (error word 0x%x)", w);
    if (w & OV_EW_WALK) return ov_fail(c, OV_ERR_TOPOLOGY, "filament walk reached an EMPTY slot (error word 0x%x)", w);
    if (w & OV_EW_ITER) return ov_fail(c, OV_ERR_STACK, "traversal iteration bound exceeded (error word 0x%x)", w);
    if (w & OV_EW_BOUNDS) {
        int bad = 0;
        cudaMemcpy(&bad, c->tree.counters + TC_BAD, 4, cudaMemcpyDeviceToHost);
        return ov_fail(c, OV_ERR_STATE, "device bounds check failed: code %d index %d (error word 0x%x)",
                       (bad >> 24) & 0x3F, bad & 0xFFFFFF, w);
    }
    if ((w & OV_EW_DEPTH) && c->strict_depth)
        return ov_fail(c, OV_ERR_DEPTH, "two nodes share a cell at tree level %d (error word 0x%x)", c->key_levels,
                       w);
    if (w & OV_EW_TEMP)
        return ov_fail(c, OV_ERR_ARG, "a node's temperature is outside the He II model's range (error word 0x%x)", w);
    if (w & OV_EW_INVERT)
        return ov_fail(c, OV_ERR_ARG, "spherical inversion of a node at the origin (error word 0x%x)", w);
    return OV_OK;   // sliver drops are counted, not fatal
}

// tangents + tree + traversal of one tangle on stream s (no host sync)
// Clear the error words that accumulate over one API call.
static int clear_call_words(ov_ctx *c)
{
    OV_CUDA(c, cudaMemsetAsync(c->tree.counters + TC_ERR, 0, (TC_COUNT - TC_ERR) * 4, c->stream));
    return OV_OK;
}

// The tangents run on the side stream beside the tree build (neither reads
// what the other writes); the traversal waits for both.  Phase events:
// tangents ph[0] -> ph[1] (side stream), tree ph[0] -> ph[2], traversal
// ph[2] -> ph[3].
static int eval_async(ov_ctx *c, NodeArrays &na, double t, bool tangents, cudaStream_t s)
{
    // phase events: plain records, or event-record nodes of the
    // single-evaluation graph (time slot 5); none inside the RK4 graph
    const bool in_graph = c->time_dev_index == 5;
    const bool ph = c->phase_timing && (c->time_dev_index < 0 || in_graph);
    const unsigned ev_flags = in_graph ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (ph) OV_CUDA(c, cudaEventRecordWithFlags(c->ph[0], s, ev_flags));
    if (tangents) {
        OV_CUDA(c, cudaEventRecord(c->fork_ev, s));
        OV_CUDA(c, cudaStreamWaitEvent(c->side, c->fork_ev, 0));
        ov_launch_tangents(c, na, c->side);
        if (ph) OV_CUDA(c, cudaEventRecordWithFlags(c->ph[1], c->side, ev_flags));
        OV_CUDA(c, cudaEventRecord(c->join_ev, c->side));
    } else if (ph) {
        OV_CUDA(c, cudaEventRecordWithFlags(c->ph[1], s, ev_flags));
    }
    int r = ov_tree_build(c, na, s);
    if (r) return r;
    if (ph) OV_CUDA(c, cudaEventRecordWithFlags(c->ph[2], s, ev_flags));
    if (tangents) OV_CUDA(c, cudaStreamWaitEvent(s, c->join_ev, 0));
    if ((r = ov_launch_velocities(c, na, t, c->precision, s))) return r;
    if (ph) OV_CUDA(c, cudaEventRecordWithFlags(c->ph[3], s, ev_flags));
    OV_CUDA(c, cudaGetLastError());
    return OV_OK;
}

extern "C" {
static unsigned long long graph_key(ov_ctx *c);
}

// One evaluation of the context's nodes as a captured graph (captured on
// first use and again whenever the key changes; the time comes from
// d_time[5]): one launch instead of the forty-odd kernels of the tree build
// and traversal.
static int eval_graph(ov_ctx *c, double t, bool tangents, cudaStream_t s)
{
    if (!c->d_time) {
        OV_ALLOC(c, cudaMalloc(&c->d_time, 8 * sizeof(double)));
        OV_ALLOC(c, cudaMallocHost(&c->h_time, 8 * sizeof(double)));
    }
    int r = ov_reserve_velocity_scratch(c);
    if (r) return r;
    c->h_time[5] = t;
    OV_CUDA(c, cudaMemcpyAsync(c->d_time + 5, c->h_time + 5, sizeof(double), cudaMemcpyHostToDevice, s));
    const int gi = (tangents ? 1 : 0) + (c->phase_timing ? 2 : 0);
    const unsigned long long key = graph_key(c);
    if (!c->eval_exec[gi] || key != c->eval_key[gi]) {
        if (c->eval_exec[gi]) { cudaGraphExecDestroy(c->eval_exec[gi]); c->eval_exec[gi] = nullptr; }
        cudaGraph_t g = nullptr;
        OV_CUDA(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        c->time_dev_index = 5;
        const int64_t l0 = c->launches;
        r = eval_async(c, c->node, t, tangents, s);
        c->eval_kernels[gi] = c->launches - l0;
        c->launches = l0;
        c->time_dev_index = -1;
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (r) { if (g) cudaGraphDestroy(g); return r; }
        if (e != cudaSuccess) return ov_fail(c, OV_ERR_CUDA, "evaluation graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c->eval_exec[gi], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess)
            return ov_fail(c, OV_ERR_CUDA, "evaluation graph instantiate: %s", cudaGetErrorString(e));
        c->eval_key[gi] = key;
    }
    OV_CUDA(c, cudaGraphLaunch(c->eval_exec[gi], s));
    c->launches += c->eval_kernels[gi];
    return OV_OK;
}

// Evaluate, growing the cell storage and re-running when the tree did not fit.
// The context's own nodes go through the evaluation graph unless node
// counting (host-side per-call work) is on.
int ov_eval_sync(ov_ctx *c, NodeArrays &na, double t, bool tangents)
{
    int r;
    c->tree_built = false;   // (a replayed graph does not run ov_tree_build's host side)
    const bool graph = c->use_graph && !c->count_nodes && &na == &c->node;
    for (int attempt = 0; attempt < 3; ++attempt) {
        if ((r = clear_call_words(c))) return r;
        if ((r = graph ? eval_graph(c, t, tangents, c->stream) : eval_async(c, na, t, tangents, c->stream)))
            return r;
        if ((r = collect_stats(c, true))) return r;
        if (!(c->stats.error_word & OV_EW_CELLS)) return error_from_word(c);
        int need = 0;
        OV_CUDA(c, cudaMemcpy(&need, c->tree.counters + TC_NEED, 4, cudaMemcpyDeviceToHost));
        if ((r = ov_tree_reserve_cells(c, need + need / 4 + 64))) return r;
    }
    return ov_fail(c, OV_ERR_ALLOC, "cell storage could not be sized");
}

extern "C" {

int ov_update_tangents_normals(ov_ctx *c)
{
    int r = check_ready(c);
    if (r) return r;
    OV_CUDA(c, cudaMemsetAsync(c->tree.counters, 0, TC_WORDS * 4, c->stream));
    ov_launch_tangents(c, c->node, c->stream);   // (all counter words cleared: a new call)
    OV_CUDA(c, cudaGetLastError());
    if ((r = collect_stats(c, true))) return r;
    return error_from_word(c);
}

int ov_update_velocities(ov_ctx *c, double t)
{
    int r = check_ready(c);
    if (r) return r;
    return ov_eval_sync(c, c->node, t, false);
}

int ov_update_tangle(ov_ctx *c, double t)
{
    int r = check_ready(c);
    if (r) return r;
    return ov_eval_sync(c, c->node, t, true);
}

// RK4 (vortex_dynamics.c:50-119) from k1 = the context's current vels.
// The RK4 sequence (vortex_dynamics.c:75-115) as launched on stream s:
// three Euler stages from the start positions, each followed by tangents,
// tree and velocities, then the combine.  Times come from d_time when
// time_dev_index >= 0 (graph capture).
static int rk4_sequence(ov_ctx *c, double t, double dt, cudaStream_t s)
{
    const double *vin[3][3] = {{c->node.vx, c->node.vy, c->node.vz},
                               {c->stage[0].vx, c->stage[0].vy, c->stage[0].vz},
                               {c->stage[1].vx, c->stage[1].vy, c->stage[1].vz}};
    const double tt[3] = {t + dt / 2, t + dt / 2, t + dt};
    int r;
    for (int k = 0; k < 3; ++k) {
        if (c->time_dev_index >= 0) c->time_dev_index = k;
        ov_launch_euler(c, c->node, vin[k][0], vin[k][1], vin[k][2], dt / 2, c->stage[k], s);
        if ((r = eval_async(c, c->stage[k], tt[k], true, s))) return r;
    }
    ov_launch_rk4_combine(c, dt, s);
    OV_CUDA(c, cudaGetLastError());
    return OV_OK;
}

static unsigned long long mix64(unsigned long long h, const void *p, size_t n)
{
    const unsigned char *b = (const unsigned char *)p;
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

// Identity of everything the captured graph bakes in: buffers, sizes,
// parameters, geometry, precision.
static unsigned long long graph_key(ov_ctx *c)
{
    unsigned long long h = 1469598103934665603ull;
    h = mix64(h, &c->params, sizeof c->params);
    h = mix64(h, &c->geo, sizeof c->geo);
    int ints[10] = {c->cap, c->tree.cap_cells, c->precision, (int)c->mem.size(), c->tune.warps, c->tune.groups,
                    c->tune.blocks_per_sm, c->tune.largest_first, c->tune.hi_occ, c->walk};
    h = mix64(h, ints, sizeof ints);
    for (const Member &m : c->mem) {
        int lay[3] = {m.lo, m.n, m.cap};
        h = mix64(h, lay, sizeof lay);
        h = mix64(h, &m.params, sizeof m.params);
    }
    const void *ptrs[9] = {c->node.x, c->tree.cells, c->part, c->d_time, c->d_tid, c->d_tprm, c->d_qorder, c->d_mrange,
                           c->tree.tt};
    h = mix64(h, ptrs, sizeof ptrs);
    return h;
}

int ov_rk4_step(ov_ctx *c, double t, double dt)
{
    int r = check_ready(c);
    if (r) return r;
    c->host_valid = false;
    c->tree_built = false;   // the tree buffers end up holding a stage's tree (also when a graph replays)
    cudaStream_t s = c->stream;
    if (!c->d_time) {
        OV_ALLOC(c, cudaMalloc(&c->d_time, 8 * sizeof(double)));
        OV_ALLOC(c, cudaMallocHost(&c->h_time, 8 * sizeof(double)));
    }
    if ((r = ov_reserve_velocity_scratch(c))) return r;
    for (int attempt = 0; attempt < 3; ++attempt) {
        if ((r = clear_call_words(c))) return r;
        c->h_time[0] = t + dt / 2;
        c->h_time[1] = t + dt / 2;
        c->h_time[2] = t + dt;
        c->h_time[3] = dt / 2;
        c->h_time[4] = dt;
        OV_CUDA(c, cudaMemcpyAsync(c->d_time, c->h_time, 5 * sizeof(double), cudaMemcpyHostToDevice, s));
        if (c->use_graph) {
            unsigned long long key = graph_key(c);
            if (!c->rk4_exec || key != c->rk4_key) {
                if (c->rk4_exec) { cudaGraphExecDestroy(c->rk4_exec); c->rk4_exec = nullptr; }
                cudaGraph_t g = nullptr;
                OV_CUDA(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                c->time_dev_index = 0;
                int64_t l0 = c->launches;
                r = rk4_sequence(c, t, dt, s);
                c->rk4_kernels = c->launches - l0;
                c->launches = l0;
                c->time_dev_index = -1;
                cudaError_t e = cudaStreamEndCapture(s, &g);
                if (r) { if (g) cudaGraphDestroy(g); return r; }
                if (e != cudaSuccess) return ov_fail(c, OV_ERR_CUDA, "RK4 graph capture: %s", cudaGetErrorString(e));
                e = cudaGraphInstantiate(&c->rk4_exec, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) return ov_fail(c, OV_ERR_CUDA, "RK4 graph instantiate: %s", cudaGetErrorString(e));
                c->rk4_key = key;
            }
            OV_CUDA(c, cudaGraphLaunch(c->rk4_exec, s));
            c->launches += c->rk4_kernels;
        } else {
            c->time_dev_index = 0;
            r = rk4_sequence(c, t, dt, s);
            c->time_dev_index = -1;
            if (r) return r;
        }
        if ((r = collect_stats(c, true))) return r;
        if (!(c->stats.error_word & OV_EW_CELLS)) return error_from_word(c);
        // a stage tree did not fit: the combine did not run; grow and redo
        int need = 0;
        OV_CUDA(c, cudaMemcpy(&need, c->tree.counters + TC_NEED, 4, cudaMemcpyDeviceToHost));
        if ((r = ov_tree_reserve_cells(c, need + need / 4 + 64))) return r;
    }
    return ov_fail(c, OV_ERR_ALLOC, "cell storage could not be sized");
}

// Device time of one velocity evaluation (tree + traversal) with the
// context's current tuning: best of `reps` after one warm-up.
static int time_eval(ov_ctx *c, double t, int reps, float *ms)
{
    int r;
    if ((r = ov_reserve_velocity_scratch(c))) return r;
    if ((r = ov_eval_sync(c, c->node, t, false))) return r;
    float best = 1e30f;
    for (int i = 0; i < reps; ++i) {
        if ((r = clear_call_words(c))) return r;
        OV_CUDA(c, cudaEventRecord(c->ev0, c->stream));
        if ((r = eval_async(c, c->node, t, false, c->stream))) return r;
        OV_CUDA(c, cudaEventRecord(c->ev1, c->stream));
        OV_CUDA(c, cudaEventSynchronize(c->ev1));
        float m = 0;
        OV_CUDA(c, cudaEventElapsedTime(&m, c->ev0, c->ev1));
        best = std::min(best, m);
        if ((r = collect_stats(c, false))) return r;
        if ((r = error_from_word(c))) return r;
    }
    *ms = best;
    return OV_OK;
}

int ov_autotune(ov_ctx *c, double t, ov_tuning *best_out, float *ms_best)
{
    int r = check_ready(c);
    if (r) return r;
    const Tuning saved = c->tune;
    Tuning best = c->tune;
    best.groups = ov_query_groups(c);   // resolve the default
    float best_ms = 1e30f;
    auto trial = [&](const Tuning &tu, float *ms) -> int {
        c->tune = tu;
        int rr;
        if (c->mem.size() > 1 && (rr = ov_upload_member_tables(c))) return rr;
        return time_eval(c, t, 3, ms);
    };
    if ((r = trial(best, &best_ms))) { c->tune = saved; return r; }
    // coordinate descent: block shape, query groups, blocks per SM, queue order
    const int maxg = std::min(c->geo.n_img + 1, 27);
    const int warps[3] = {2, 4, 8};
    const int groups[8] = {1, 2, 3, 4, 6, 9, 14, 27};
    for (int stage = 0; stage < 5; ++stage) {
        std::vector<Tuning> cand;
        if (stage == 0)
            for (int w : warps)
                for (int ho = 0; ho <= (c->precision == OV_PREC_MIXED ? 4 : 0); ++ho) {
                    Tuning tu = best;
                    tu.warps = w;
                    tu.hi_occ = ho;
                    cand.push_back(tu);
                }
        if (stage == 1)
            for (int g : groups)
                if (g <= maxg) { Tuning tu = best; tu.groups = g; cand.push_back(tu); }
        if (stage == 2) {
            int occ = 0;
            ov_traversal_blocks(c, c->precision, best.warps, &occ);
            for (int b : {0, occ - 1, (occ + 1) / 2})
                if (b >= 0) { Tuning tu = best; tu.blocks_per_sm = b; cand.push_back(tu); }
        }
        if (stage == 3 && c->mem.size() > 1)
            for (int lf : {1, 0}) { Tuning tu = best; tu.largest_first = lf; cand.push_back(tu); }
        if (stage == 4) {   // the block shape again, given the groups and grid picked
            for (int w : warps) { Tuning tu = best; tu.warps = w; cand.push_back(tu); }
        }
        for (const Tuning &tu : cand) {
            if (tu.warps == best.warps && tu.groups == best.groups && tu.blocks_per_sm == best.blocks_per_sm &&
                tu.largest_first == best.largest_first && tu.hi_occ == best.hi_occ)
                continue;
            float ms = 0;
            if ((r = trial(tu, &ms))) { c->tune = saved; if (c->mem.size() > 1) ov_upload_member_tables(c); return r; }
            if (ms < best_ms * 0.99f) { best_ms = ms; best = tu; }
        }
    }
    c->tune = best;
    if (c->mem.size() > 1 && (r = ov_upload_member_tables(c))) return r;
    if ((r = ov_reserve_velocity_scratch(c))) return r;
    if (best_out) ov_get_tuning(c, best_out);
    if (ms_best) *ms_best = best_ms;
    return OV_OK;
}

int ov_direct_velocities(ov_ctx *c, const int *nodes, int n, double t, double *vels_out, double *vs_out)
{
    int r = check_ready(c);
    if (r) return r;
    if (n < 0 || (n > 0 && !nodes)) return OV_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (nodes[i] < 0 || nodes[i] >= c->cap) return ov_fail(c, OV_ERR_ARG, "node %d out of range", nodes[i]);
    return ov_direct_sum(c, nodes, n, t, vels_out, vs_out);
}

int ov_enforce_periodic_boundaries(ov_ctx *c)
{
    int r = check_ready(c);
    if (r) return r;
    c->tree_built = false;
    c->host_valid = false;
    ov_launch_periodic_wrap(c, c->stream);
    OV_CUDA(c, cudaGetLastError());
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    return OV_OK;
}

int ov_get_stats(const ov_ctx *c, ov_stats *out)
{
    if (!c || !out) return OV_ERR_ARG;
    *out = c->stats;
    return OV_OK;
}

int ov_timer_start(ov_ctx *c)
{
    if (!c) return OV_ERR_ARG;
    OV_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    return OV_OK;
}

int ov_timer_stop(ov_ctx *c, float *ms)
{
    if (!c || !ms) return OV_ERR_ARG;
    OV_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    OV_CUDA(c, cudaEventSynchronize(c->ev1));
    OV_CUDA(c, cudaEventElapsedTime(ms, c->ev0, c->ev1));
    return OV_OK;
}

int ov_flush_l2(ov_ctx *c, size_t bytes)
{
    if (!c) return OV_ERR_ARG;
    if (c->flush_bytes < bytes) {
        if (c->flush_buf) cudaFree(c->flush_buf);
        c->flush_buf = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->flush_buf, bytes));
        c->flush_bytes = bytes;
    }
    static int v = 0;
    OV_CUDA(c, cudaMemsetAsync(c->flush_buf, (++v) & 0xFF, bytes, c->stream));
    return OV_OK;
}

int ov_synchronize(ov_ctx *c)
{
    if (!c) return OV_ERR_ARG;
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    return OV_OK;
}

int64_t ov_kernel_launches(const ov_ctx *c) { return c ? c->launches : 0; }

int ov_set_phase_timing(ov_ctx *c, int on)
{
    if (!c) return OV_ERR_ARG;
    if (on && !c->ph[0])
        for (int i = 0; i < 4; ++i) OV_CUDA(c, cudaEventCreate(&c->ph[i]));
    c->phase_timing = on != 0;
    return OV_OK;
}

int ov_set_node_counting(ov_ctx *c, int on)
{
    if (!c) return OV_ERR_ARG;
    c->count_nodes = on != 0;
    return OV_OK;
}

int ov_get_node_counts(ov_ctx *c, int member, unsigned *visits, unsigned *accepts, int n)
{
    if (!c || member < 0 || member >= (int)c->mem.size() || n < 0 || n > c->mem[member].n ||
        (n > 0 && (!visits || !accepts)))
        return OV_ERR_ARG;
    if (!c->count_nodes || !c->d_node_counts || c->node_counts_cap < 2 * (size_t)c->cap)
        return ov_fail(c, OV_ERR_STATE, "node counting is off or no evaluation ran since it was switched on");
    const size_t lo = (size_t)c->mem[member].lo;
    OV_CUDA(c, cudaMemcpyAsync(visits, c->d_node_counts + lo, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToHost,
                               c->stream));
    OV_CUDA(c, cudaMemcpyAsync(accepts, c->d_node_counts + c->cap + lo, (size_t)n * sizeof(unsigned),
                               cudaMemcpyDeviceToHost, c->stream));
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    return OV_OK;
}

int ov_phase_times(ov_ctx *c, float ms[3])
{
    if (!c || !ms) return OV_ERR_ARG;
    if (!c->phase_timing || !c->ph[0]) return ov_fail(c, OV_ERR_STATE, "phase timing is off");
    OV_CUDA(c, cudaEventSynchronize(c->ph[3]));
    OV_CUDA(c, cudaEventElapsedTime(&ms[0], c->ph[0], c->ph[1]));   // tangents (side stream)
    OV_CUDA(c, cudaEventElapsedTime(&ms[1], c->ph[0], c->ph[2]));   // tree build, beside them
    OV_CUDA(c, cudaEventElapsedTime(&ms[2], c->ph[2], c->ph[3]));   // traversal and finish
    return OV_OK;
}

}  // extern "C"

// ----------------------------------------------------- spherical fork
// The tangle in slots [0, N) (member 0) and its inner image in [N, 2N)
// (member 1, connections shifted by N): one forest build gives both trees.
static int sph_run(ov_ctx *c, ov_sph_tangle_state *t, const ov_sph_params *p, double time, bool tangents,
                   bool vels)
{
    (void)time;   // the fork's velocities do not depend on time
    if (!c || !t || !p || t->N < 0) return OV_ERR_ARG;
    cudaSetDevice(c->device);
    if (p->outer_surface)
        return ov_fail(c, OV_ERR_ARG,
                       "outer_surface = 1 is not supported (the reference's branch uses a null image tree)");
    const ov_sph_domain &dom = t->domain_section;
    if (!(dom.inner_radius > 0 && dom.outer_radius > dom.inner_radius && dom.azimut_angle > 0 &&
          dom.polar_angle > 0))
        return ov_fail(c, OV_ERR_ARG, "spherical section: need 0 < inner < outer radius and positive angles");
    const int N = t->N;
    if (N > 0 && (!t->vnodes || !t->vels || !t->vs || !t->tangents || !t->normals || !t->connections || !t->status))
        return OV_ERR_ARG;
    SphSettings ss;
    ss.kappa = p->kappa; ss.a0 = p->vortex_width; ss.alpha = p->alpha; ss.alpha_p = p->alpha_p;
    ss.dl_min = p->dl_min; ss.dl_max = p->dl_max; ss.theta = p->bh_resolution;
    ss.friction = p->use_mutual_friction; ss.use_temperature = p->use_temperature;
    ss.q_dot = p->q_dot; ss.t_bath = p->temp_bath; ss.prof_a = 0;
    if (p->use_temperature) {
        int terr = 0;
        ss.prof_a = helium::profile_A(p->q_dot, p->temp_bath, p->kappa, &terr);
        if (terr) return ov_fail(c, OV_ERR_ARG, "bath temperature %g K outside the He II model's range", p->temp_bath);
    }
    SphDomain sd{N, dom.inner_radius, dom.outer_radius, dom.azimut_angle, dom.polar_angle};
    if (N == 0) return OV_OK;
    int r;
    const int slots = 2 * N;
    if ((r = ensure_capacity(c, slots))) return r;
    c->uploaded = false;   // the context holds no regular tangle after this call
    c->tree_built = false;
    c->host_valid = false;
    c->n_live = slots;
    ov_params op;
    ov_params_default(&op);
    op.kappa = p->kappa; op.vortex_width = p->vortex_width; op.alpha = p->alpha; op.alpha_p = p->alpha_p;
    op.use_mutual_friction = p->use_mutual_friction; op.bh_resolution = p->bh_resolution; op.use_bh = 1;
    op.dl_min = p->dl_min; op.dl_max = p->dl_max;
    c->params = op;
    c->mem.assign(2, Member{});
    for (int m = 0; m < 2; ++m) {
        c->mem[m].lo = m * N;
        c->mem[m].n = N;
        c->mem[m].cap = N;
        c->mem[m].params = op;
    }
    Geometry &g = c->geo;
    memset(&g, 0, sizeof g);
    for (int a = 0; a < 3; ++a) { g.lo[a] = 0; g.hi[a] = 1; g.L[a] = 1; }
    g.sph = 1;
    g.sph_az = dom.azimut_angle;
    g.sph_pl = dom.polar_angle;
    g.sph_seg_max = 5 * p->dl_max;
    // grid step of the mixed path: every coordinate (|x| <= ro) below 2^22 steps
    c->grid_h = ldexp(1.0, (int)ceil(log2(dom.outer_radius)) - 22);
    const double A = dom.azimut_angle, P = dom.polar_angle;
    const double ri = dom.inner_radius, ro = dom.outer_radius;
    const double lo0[3] = {ri, -A, -P}, hi0[3] = {ro, A, P};
    const double lo1[3] = {ri * ri / ro, -A, -P}, hi1[3] = {ri, A, P};   // the inner image's section
    for (int a = 0; a < 3; ++a) {
        c->sph_lo[0][a] = lo0[a]; c->sph_hi[0][a] = hi0[a];
        c->sph_lo[1][a] = lo1[a]; c->sph_hi[1][a] = hi1[a];
    }
    if ((r = ov_upload_member_tables(c))) return r;
    // upload: positions, vels, vs, tangents, normals of the tangle (SoA), topology of both members
    const size_t cap = (size_t)c->cap;
    if ((r = ensure_stage(c, cap * 3 * sizeof(double) * 5 + cap * 4 * sizeof(int)))) return r;
    double *h = c->h_stage;
    int *hi_ = (int *)(h + 15 * cap);
    const ov_vec3 *src[5] = {t->vnodes, t->vels, t->vs, t->tangents, t->normals};
    double *dd[15] = {c->node.x, c->node.y, c->node.z, c->node.vx, c->node.vy, c->node.vz,
                      c->node.sx, c->node.sy, c->node.sz, c->node.tx, c->node.ty, c->node.tz,
                      c->node.nx, c->node.ny, c->node.nz};
    for (int f = 0; f < 5; ++f) {
        double *dst = h + 3 * cap * f;
        for (int a = 0; a < 3; ++a)
            for (int k = 0; k < N; ++k) dst[a * cap + k] = src[f][k].p[a];
        for (int a = 0; a < 3; ++a)
            OV_CUDA(c, cudaMemcpyAsync(dd[3 * f + a], dst + a * cap, (size_t)N * sizeof(double),
                                       cudaMemcpyHostToDevice, c->stream));
    }
    int *hf = hi_, *hr = hi_ + cap, *hs = hi_ + 2 * cap, *hp = hi_ + 3 * cap;
    for (int k = 0; k < N; ++k) {
        const int f = t->connections[k].forward, b = t->connections[k].reverse, st = t->status[k].status;
        if (f < -1 || f >= N || b < -1 || b >= N || st < OV_EMPTY || st > OV_PINNED_SLIP)
            return ov_fail(c, OV_ERR_TOPOLOGY, "node %d: bad connection or status", k);
        hf[k] = f; hr[k] = b; hs[k] = st; hp[k] = t->status[k].pin_wall;
        hf[N + k] = f < 0 ? -1 : f + N;
        hr[N + k] = b < 0 ? -1 : b + N;
        hs[N + k] = st;
        hp[N + k] = t->status[k].pin_wall;
    }
    for (size_t k = (size_t)slots; k < cap; ++k) {   // slots past the two members are EMPTY
        hf[k] = hr[k] = -1;
        hs[k] = OV_EMPTY;
        hp[k] = OV_NOT_A_FACE;
    }
    int *di[4] = {c->fwd, c->rev, c->status, c->pin};
    int *hsrc[4] = {hf, hr, hs, hp};
    for (int a = 0; a < 4; ++a)
        OV_CUDA(c, cudaMemcpyAsync(di[a], hsrc[a], cap * 4, cudaMemcpyHostToDevice, c->stream));
    c->last_h2d = (size_t)N * (15 * sizeof(double)) + cap * 16;
    OV_CUDA(c, cudaMemsetAsync(c->tree.counters, 0, TC_WORDS * 4, c->stream));
    if (tangents) ov_launch_sph_tangents(c, sd, ss);
    if (vels) {
        ov_launch_sph_images(c, sd, ss);
        for (int attempt = 0;; ++attempt) {
            if ((r = ov_tree_build(c, c->node, c->stream))) return r;
            if ((r = ov_launch_sph_velocities(c, sd, ss))) return r;
            OV_CUDA(c, cudaGetLastError());
            if ((r = collect_stats(c, true))) return r;
            if (!(c->stats.error_word & OV_EW_CELLS)) break;
            if (attempt == 2) return ov_fail(c, OV_ERR_ALLOC, "cell storage could not be sized");
            int need = 0;
            OV_CUDA(c, cudaMemcpy(&need, c->tree.counters + TC_NEED, 4, cudaMemcpyDeviceToHost));
            if ((r = ov_tree_reserve_cells(c, need + need / 4 + 64))) return r;
            OV_CUDA(c, cudaMemsetAsync(c->tree.counters + TC_ERR, 0, (TC_COUNT - TC_ERR) * 4, c->stream));
        }
    } else {
        OV_CUDA(c, cudaGetLastError());
        if ((r = collect_stats(c, true))) return r;
    }
    if ((r = error_from_word(c))) return r;
    // download what the reference writes: tangents, normals; vels, vs
    const int fsel[4] = {tangents ? 3 : -1, tangents ? 4 : -1, vels ? 1 : -1, vels ? 2 : -1};
    ov_vec3 *out[5] = {t->vnodes, t->vels, t->vs, t->tangents, t->normals};
    for (int q = 0; q < 4; ++q) {
        const int f = fsel[q];
        if (f < 0) continue;
        double *dst = h + 3 * cap * f;
        for (int a = 0; a < 3; ++a)
            OV_CUDA(c, cudaMemcpyAsync(dst + a * cap, dd[3 * f + a], (size_t)N * sizeof(double),
                                       cudaMemcpyDeviceToHost, c->stream));
    }
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int q = 0; q < 4; ++q) {
        const int f = fsel[q];
        if (f < 0) continue;
        const double *dsrc = h + 3 * cap * f;
        for (int k = 0; k < N; ++k)
            for (int a = 0; a < 3; ++a) out[f][k].p[a] = dsrc[a * cap + k];
    }
    return OV_OK;
}

extern "C" {

void ov_sph_params_default(ov_sph_params *p)
{
    if (!p) return;
    memset(p, 0, sizeof *p);
    p->kappa = 9.97e-4;
    p->vortex_width = 1e-8;
    p->alpha = 0.034;
    p->alpha_p = 1.383e-2;
    p->use_mutual_friction = 1;
    p->bh_resolution = 0.4;
    p->dl_min = 0.5e-3;
    p->dl_max = 1.5e-3;
    p->q_dot = 0.03;
    p->temp_bath = 1.65;
    p->use_temperature = 1;
    p->outer_surface = 0;
}

int ov_sph_update_tangents_normals(ov_ctx *c, ov_sph_tangle_state *t, const ov_sph_params *p)
{
    return sph_run(c, t, p, 0.0, true, false);
}

int ov_sph_update_velocities(ov_ctx *c, ov_sph_tangle_state *t, const ov_sph_params *p, double time)
{
    return sph_run(c, t, p, time, false, true);
}

int ov_sph_update_tangle(ov_ctx *c, ov_sph_tangle_state *t, const ov_sph_params *p, double time)
{
    return sph_run(c, t, p, time, true, true);
}

int ov_sph_helium(double T, double out[6])
{
    if (!out) return OV_ERR_ARG;
    int err = 0;
    out[0] = helium::superfluid_density(T, &err);
    out[1] = helium::total_density(T, &err);
    out[2] = helium::normal_density(T, &err);
    out[3] = helium::entropy(T, &err);
    out[4] = helium::friction_alpha(T, &err);
    out[5] = helium::friction_alpha_p(T, &err);
    return err ? OV_ERR_ARG : OV_OK;
}

}  // extern "C"
