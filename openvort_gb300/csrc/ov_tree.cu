// ov_tree.cu - GPU linear octree with the reference's exact tree semantics.
//
// OpenVort's pointer octree (src/octree.c) splits the DOMAIN box until every
// cell holds at most one node, assigning a node to the FIRST child (order
// BLF, BLB, BRF, BRB, TLF, TLB, TRF, TRB) whose closed box holds it, with
// child boxes computed by make_child_box's FP64 arithmetic (octree.c:165-232).
// A node outside the root box belongs to the root only (octree.c:116-127).
//
// Here every node gets a 63-bit path key: 21 levels x 3-bit child index in
// the reference order.  The child index at each level is read off a 62-bit
// fixed-point image of the position when the node is at least 2^-40 box
// lengths away from every face of every level (then the reference's
// rounded boxes and tie order cannot change the answer); otherwise the
// exact FP64 first-match descent of the reference is run for that node.
// Sorting the keys puts the cells of each level in contiguous ranges and in
// the reference's child order; cells are emitted in pre-order, so a cell's
// subtree is [cell+1, cell.next) and a traversal needs no stack.
//
// An ensemble builds one such tree per member in the same launches (a
// forest): the member id sits above the out-of-box bit of the key, so the
// sort groups members, and each member's sorted range gets its own root
// cell followed by its pre-order cells.  With a single member the id field
// is empty and the keys hold 21 levels; with T members it takes
// ceil(log2 T) bits and the keys hold floor((63 - bits) / 3) levels.
#include "ov_internal.cuh"

void ov_sort_keys(ov_ctx *c, TreeBuf &t, int n, cudaStream_t s);
int ov_sort_hist_ints(int cap);
int ov_scan_tmp_ints(int n_max);

namespace {

struct KeyGeom {
    double lo[3], hi[3], L[3];
    double invL[3];    // 1 / L, rounded
    double invL62[3];  // invL * 2^62 (exact)
    int fast;          // fixed-point digits allowed (rounding bound is small)
    int tb;            // member-id bits on top of the key
    int levels;        // levels the key holds
    uint64_t lvmask;   // the levels' bits in the path field
    int nt;            // members
    // spherical sections: per member (r, az, pl) bounds of the root cell
    double sb[OV_SPH_MEMBERS][3], st[OV_SPH_MEMBERS][3];
    int sph_root;      // the root cells' Lm from those bounds
    double root_lm;    // Lm of the (box) root cell
};

// bit offset of the level-`lev` digit
__device__ __forceinline__ int dsh(const KeyGeom &g, int lev) { return 63 - g.tb - 3 * lev; }
// member of a non-EMPTY key (clamped: ids come from the slot table)
__device__ __forceinline__ int key_member(const KeyGeom &g, uint64_t key)
{
    int m = g.tb ? (int)(key >> (64 - g.tb)) : 0;
    return m < g.nt ? m : g.nt - 1;
}

// 63-bit path (digit of level lev at bit 63 - 3 lev) by the reference's descent
__device__ __forceinline__ uint64_t exact_key(const double p[3], const KeyGeom &g, int *err)
{
    double b[3] = {g.lo[0], g.lo[1], g.lo[2]}, t[3] = {g.hi[0], g.hi[1], g.hi[2]};
    uint64_t key = 0;
    for (int lev = 1; lev <= g.levels; ++lev) {
        int pick = -1;
        double cb[3], ct[3];
        for (int idx = 0; idx < 8; ++idx) {
            child_box_dev(b, t, idx, cb, ct);
            if (in_closed_box_dev(cb, ct, p)) { pick = idx; break; }
        }
        if (pick < 0) {
            // rounding gap between child boxes: the reference keeps the node
            // only in this cell's ancestors; flagged, node kept in the octant
            // its coordinates point to.
            *err |= OV_EW_SLIVER;
            double c[3];
            for (int a = 0; a < 3; ++a) c[a] = rn_mul(rn_add(b[a], t[a]), 0.5);
            pick = ((p[2] > c[2]) << 2) | ((p[1] > c[1]) << 1) | ((p[0] > c[0]) ? 0 : 1);
            child_box_dev(b, t, pick, cb, ct);
        }
        key |= (uint64_t)pick << (63 - 3 * lev);
        for (int a = 0; a < 3; ++a) { b[a] = cb[a]; t[a] = ct[a]; }
    }
    return key;
}

// Path of a point u = (r, az, pl) inside member m's spherical root cell, by
// the fork's first-match descent (octree.c:126-137 with its make_child_box):
// ties go to the outer radial half and the lower angular halves.
__device__ __forceinline__ uint64_t sph_key(const double u[3], const KeyGeom &g, int m)
{
    double b[3] = {g.sb[m][0], g.sb[m][1], g.sb[m][2]}, t[3] = {g.st[m][0], g.st[m][1], g.st[m][2]};
    uint64_t key = 0;
    for (int lev = 1; lev <= g.levels; ++lev) {
        const double mr = rn_div(rn_add(t[0], b[0]), 2.0), ma = rn_div(rn_add(t[1], b[1]), 2.0),
                     mp = rn_div(rn_add(t[2], b[2]), 2.0);
        const int rl = u[0] >= mr ? 0 : 1, au = u[1] <= ma ? 0 : 1, pu = u[2] <= mp ? 0 : 1;
        const int idx = 4 * au + 2 * pu + rl;
        double cb[3], ct[3];
        sph_child_box(b, t, idx, cb, ct);
        for (int a = 0; a < 3; ++a) { b[a] = cb[a]; t[a] = ct[a]; }
        key |= (uint64_t)idx << (63 - 3 * lev);
    }
    return key;
}

__device__ __forceinline__ void node_moment(int id, const double *x, const double *y, const double *z,
                                            const int *fwd, const Geometry &geo, double out[6])
{
    double p[3] = {x[id], y[id], z[id]};
    out[0] = p[0]; out[1] = p[1]; out[2] = p[2];
    int f = fwd[id];
    if (f > -1) {
        double r2[3] = {x[f], y[f], z[f]};
        if (geo.sph) sph_pwrap(geo, p, r2);
        else pwrap_dev(geo, p, r2);
        out[3] = rn_sub(r2[0], p[0]); out[4] = rn_sub(r2[1], p[1]); out[5] = rn_sub(r2[2], p[2]);
        // the spherical fork leaves segments longer than 5 dl_max out (octree.c:316-322)
        if (geo.sph && len3_ref(out[3], out[4], out[5]) > geo.sph_seg_max) out[3] = out[4] = out[5] = 0;
    } else {
        out[3] = out[4] = out[5] = 0;
    }
}

// Path keys of all slots (EMPTY slots sort last), the member counts, and
// each live node's moment (position, wrapped forward segment) in id order,
// where the positions are read coalesced; the leaves of the tree gather it.
template <bool SPH>
__global__ void k_keys(const int *__restrict__ status, const double *__restrict__ x,
                       const double *__restrict__ y, const double *__restrict__ z, const int *__restrict__ tid,
                       int cap, KeyGeom g, uint64_t *__restrict__ keys, int *__restrict__ order,
                       int *counters, int *tt, const int *__restrict__ fwd, Geometry geo, double *__restrict__ nm)
{
    __shared__ int bc[4];   // the block's live, in-box, out-of-box counts and NaN flag
    if (threadIdx.x < 4) bc[threadIdx.x] = 0;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool live = i < cap && status[i] != OV_EMPTY;
    double p[3] = {0, 0, 0};
    if (live) { p[0] = x[i]; p[1] = y[i]; p[2] = z[i]; }
    int m = (live && tid) ? tid[i] : 0;
    double u[3] = {0, 0, 0};   // spherical sections: (r, az, pl)
    bool inside;
    if (SPH) {
        if (m < 0 || m >= OV_SPH_MEMBERS) m = 0;
        if (live) { u[0] = sph_radius(p); u[1] = sph_azimut(p); u[2] = sph_polar(p); }
        inside = live && in_closed_box_dev(g.sb[m], g.st[m], u);
    } else {
        inside = live && in_closed_box_dev(g.lo, g.hi, p);
    }
    bool bad = live && !(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]));
    // one global atomic per block for each counter (a single tree's member
    // counts are the same), one per warp and member present for a forest
    unsigned b_live = __ballot_sync(0xffffffffu, live), b_in = __ballot_sync(0xffffffffu, inside);
    unsigned peers = __match_any_sync(0xffffffffu, live ? m : -1) & b_live;
    if (lane == 0 && b_live) {
        atomicAdd(&bc[0], __popc(b_live));
        atomicAdd(&bc[1], __popc(b_in));
        atomicAdd(&bc[2], __popc(b_live & ~b_in));
    }
    if (tid && live && lane == __ffs(peers) - 1) {
        atomicAdd(&tt[m * TT_WORDS + TT_NNE], __popc(peers));
        atomicAdd(&tt[m * TT_WORDS + TT_M], __popc(peers & b_in));
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) bc[3] = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (bc[0]) {
            atomicAdd(&counters[TC_NNE], bc[0]);
            atomicAdd(&counters[TC_M], bc[1]);
            atomicAdd(&counters[TC_OUT], bc[2]);
            if (!tid) {
                atomicAdd(&tt[TT_NNE], bc[0]);
                atomicAdd(&tt[TT_M], bc[1]);
            }
        }
        if (bc[3]) atomicOr(&counters[TC_ERR], OV_EW_NAN);
    }
    if (i >= cap) return;
    order[i] = i;
    if (!live) { keys[i] = OV_KEY_EMPTY; return; }
    {
        double mo[6];
        node_moment(i, x, y, z, fwd, geo, mo);
        double2 *o = reinterpret_cast<double2 *>(nm + 6 * (size_t)i);
        o[0] = make_double2(mo[0], mo[1]);
        o[1] = make_double2(mo[2], mo[3]);
        o[2] = make_double2(mo[4], mo[5]);
    }
    const uint64_t prefix = g.tb ? (uint64_t)m << (64 - g.tb) : 0;
    if (SPH) {
        // outside the member's section: root only, ordered by the path of
        // its angles and radius clamped into the section
        double v[3];
        for (int a = 0; a < 3; ++a) {
            v[a] = fmin(fmax(u[a], g.sb[m][a]), g.st[m][a]);
            if (!(v[a] >= g.sb[m][a])) v[a] = g.sb[m][a];   // non-finite input
        }
        const uint64_t path = sph_key(v, g, m);
        if (!inside) keys[i] = prefix | (1ull << (63 - g.tb)) | (path >> (g.tb + 2));
        else keys[i] = prefix | ((path >> g.tb) & g.lvmask);
        return;
    }
    if (!inside) {
        // root-only member (octree.c:116-127).  The rest of the key orders
        // it among the other root-only nodes by the cell path of its
        // position clamped to the box, so it can be merged into the
        // traversal order beside its spatial neighbours (k_target_order).
        uint64_t k2 = 0;
        uint64_t W[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            double u = (p[a] - g.lo[a]) / g.L[a];
            u = fmin(fmax(u, 0.0), 1.0);
            if (!(u >= 0.0 && u <= 1.0)) u = 0.0;   // non-finite input
            W[a] = (uint64_t)(u * 4611686018427387904.0);
        }
#pragma unroll
        for (int lev = 1; lev <= OV_MAX_LEVEL; ++lev) {
            int sh = 62 - lev;
            uint64_t xb = (W[0] >> sh) & 1, yb = (W[1] >> sh) & 1, zb = (W[2] >> sh) & 1;
            k2 |= ((zb << 2) | (yb << 1) | (xb ^ 1)) << (63 - 3 * lev);
        }
        // (the bit below the out-of-box bit stays clear: no key but an
        // EMPTY slot's has all-ones upper bits)
        keys[i] = prefix | (1ull << (63 - g.tb)) | (k2 >> (g.tb + 2));
        return;
    }
    uint64_t U[3];
    bool safe = g.fast != 0;
    const uint64_t low = (1ull << 41) - 1, margin = 1ull << 22;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // (p - lo) / L * 2^62 clamped to [0, 2^62]: the 2^62 scaling is exact,
        // so this equals the truncated product of the clamped unit image;
        // the conversion saturates (p >= lo here)
        const double v = rn_mul(rn_sub(p[a], g.lo[a]), g.invL62[a]);
        U[a] = min((unsigned long long)__double2ull_rz(v), 1ull << 62);
        uint64_t r = U[a] & low;
        safe = safe && r >= margin && r <= low + 1 - margin;
    }
    uint64_t key = 0;
    if (safe) {
#pragma unroll
        for (int lev = 1; lev <= OV_MAX_LEVEL; ++lev) {
            int sh = 62 - lev;
            uint64_t xb = (U[0] >> sh) & 1, yb = (U[1] >> sh) & 1, zb = (U[2] >> sh) & 1;
            key |= ((zb << 2) | (yb << 1) | (xb ^ 1)) << (63 - 3 * lev);
        }
    } else {
        int err = 0;
        key = exact_key(p, g, &err);
        if (err) atomicOr(&counters[TC_ERR], err);
    }
    keys[i] = prefix | ((key >> g.tb) & g.lvmask);
}

__device__ __forceinline__ float cell_thr(double lm, double theta)
{
    const double r = lm / theta;
    return theta > 0 ? __double2float_ru(r * r * (1.0 + 2e-5)) : __int_as_float(0x7f800000);
}

// Member layout: first sorted position of each member (members in id order)
// and the first work tile of each in the traversal queue (queue order).
// Lanes also fill the per-level table of box cells (Lm = the root's Lm
// scaled by 2^-lev): the FP32 opening threshold and Lm rounded up.
__global__ void k_layout(int *tt, int nt, const int *__restrict__ qorder, int *counters, float *lev_tab,
                         double root_lm, double theta)
{
    if (blockIdx.x != 0) return;
    if (threadIdx.x < TREE_LV_SLOTS) {
        const double lm = ldexp(root_lm, -(int)threadIdx.x);
        lev_tab[threadIdx.x] = cell_thr(lm, theta);
        lev_tab[TREE_LV_SLOTS + threadIdx.x] = __double2float_ru(lm);
    }
    if (threadIdx.x != 0) return;
    int acc = 0;
    for (int m = 0; m < nt; ++m) {
        tt[m * TT_WORDS + TT_START] = acc;
        acc += tt[m * TT_WORDS + TT_NNE];
    }
    int tiles = 0;
    for (int k = 0; k < nt; ++k) {
        int m = qorder ? qorder[k] : k;
        if (m < 0 || m >= nt) { atomicOr(&counters[TC_ERR], OV_EW_BOUNDS); continue; }
        tt[m * TT_WORDS + TT_ITEM0] = tiles;
        tiles += (tt[m * TT_WORDS + TT_NNE] + 31) / 32;
    }
    counters[TC_ITEMS] = tiles;
}

// path bits of a key without member id (in-box keys) / of the clamped path
// (out-of-box keys), comparable with each other
__device__ __forceinline__ uint64_t inbox_path(const KeyGeom &g, uint64_t k)
{
    return k & ((1ull << (63 - g.tb)) - 1);
}
__device__ __forceinline__ uint64_t out_path(const KeyGeom &g, uint64_t k)
{
    return (k & ((1ull << (63 - g.tb)) - 1)) << 2;
}

// Traversal order: the in-box nodes in path order merged with the root-only
// nodes at the position of their clamped path (merge by rank; in-box first on
// ties), per member.  Out-of-box targets then share warps with their spatial
// neighbours instead of forming a few warps that span the whole box surface.
__global__ void k_target_order(const uint64_t *__restrict__ keys, const int *__restrict__ order, int cap,
                               const int *counters, const int *__restrict__ tt, KeyGeom g,
                               int *__restrict__ torder)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    int nne_all = counters[TC_NNE];
    if (s >= nne_all || s >= cap) return;
    const int *w = tt + key_member(g, keys[s]) * TT_WORDS;
    const int st = w[TT_START], M = w[TT_M], nne = w[TT_NNE];
    const int loc = s - st;
    if (loc < 0 || loc >= nne) return;   // cannot happen for a consistent build
    int nout = nne - M;
    int pos;
    if (loc < M) {
        // in-box: its rank plus the root-only nodes whose clamped path is smaller
        uint64_t k = inbox_path(g, keys[s]);
        int lo = 0, hi = nout;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (out_path(g, keys[st + M + mid]) < k) lo = mid + 1; else hi = mid;
        }
        pos = loc + lo;
    } else {
        int j = loc - M;
        uint64_t k = out_path(g, keys[s]);
        int lo = 0, hi = M;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (inbox_path(g, keys[st + mid]) <= k) lo = mid + 1; else hi = mid;
        }
        pos = j + lo;
    }
    torder[st + pos] = order[s];
}

__device__ __forceinline__ int cpl_of(const KeyGeom &g, uint64_t a, uint64_t b)
{
    uint64_t d = a ^ b;
    if (d == 0) return g.levels;
    return min((__clzll(d) - 1 - g.tb) / 3, g.levels);
}

// cpl[s] (common levels with the next in-box key of the member) and the
// number of cells that start at sorted position s: the member's root at its
// first position, then the cells of the levels the node starts.  Also counts
// the non-root, non-leaf cells of every level (lvl_cnt[lev]) for the
// per-level lists the moment sums run over, and the depth, one global atomic
// per block and counter.
__global__ void k_cpl(const uint64_t *__restrict__ keys, int cap, int *counters, const int *__restrict__ tt,
                      KeyGeom g, int *__restrict__ cpl, int *__restrict__ ncell_at, int *lvl_cnt)
{
    __shared__ int h[TREE_LV_SLOTS];
    __shared__ int bmax, bdeep;
    if (threadIdx.x < TREE_LV_SLOTS) h[threadIdx.x] = 0;
    if (threadIdx.x == 0) bmax = bdeep = 0;
    __syncthreads();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    int nne_all = counters[TC_NNE];
    int L = 0, nne = 0, lo = 1, hi = 0;
    bool deep = false;
    if (s < nne_all && s < cap) {
        uint64_t key = keys[s];
        const int *w = tt + key_member(g, key) * TT_WORDS;
        const int st = w[TT_START], M = w[TT_M];
        nne = w[TT_NNE];
        const int loc = s - st;
        if (loc < 0 || loc >= nne) {   // cannot happen for a consistent build
            cpl[s] = 0;
            ncell_at[s] = 0;
            nne = 0;
        } else if (loc < M) {
            int cn = (loc + 1 < M) ? cpl_of(g, key, keys[s + 1]) : 0;
            cpl[s] = cn;
            int cp = (loc > 0) ? cpl_of(g, keys[s - 1], key) : 0;
            L = max(cp, cn) + 1;
            if (L > g.levels) { deep = true; L = g.levels; }
            ncell_at[s] = ((nne >= 2) ? max(L - cp, 0) : 0) + (loc == 0);
            if (nne >= 2) { lo = cp + 1; hi = L - 1; }   // the non-leaf cells
        } else {
            cpl[s] = 0;
            ncell_at[s] = (loc == 0);
        }
    }
    {
        const int wlo = __reduce_min_sync(0xffffffffu, lo <= hi ? lo : OV_MAX_LEVEL + 1);
        const int whi = __reduce_max_sync(0xffffffffu, lo <= hi ? hi : 0);
        for (int lev = wlo; lev <= whi; ++lev) {
            const unsigned m = __ballot_sync(0xffffffffu, lo <= lev && lev <= hi);
            if ((threadIdx.x & 31) == 0 && m) atomicAdd(&h[lev], __popc(m));
        }
    }
    int Lmax = (nne >= 2) ? L : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) Lmax = max(Lmax, __shfl_xor_sync(0xffffffffu, Lmax, o));
    bool anydeep = __any_sync(0xffffffffu, deep);
    if ((threadIdx.x & 31) == 0) {
        if (Lmax > 0) atomicMax(&bmax, Lmax);
        if (anydeep) bdeep = 1;
    }
    __syncthreads();
    if (threadIdx.x < TREE_LV_SLOTS && h[threadIdx.x]) atomicAdd(&lvl_cnt[threadIdx.x], h[threadIdx.x]);
    if (threadIdx.x == 0) {
        if (bmax > 0) atomicMax(&counters[TC_MAXDEPTH], bmax);
        if (bdeep) atomicOr(&counters[TC_ERR], OV_EW_DEPTH);
    }
}

// FP32 view of a cell for the mixed traversal: COM split into a part on
// the grid of step h (exact in FP32) and a small remainder.  The opening
// test Lm / d < theta becomes d^2 > (Lm / theta)^2: thr holds that bound
// times (1 + 2e-5), rounded up, so that d^2 > thr accepts clear of the guard
// band and d^2 < thr (1 - 2e-5) / (1 + 2e-5) opens clear of it.
__device__ __forceinline__ void write_cell32(Cell32 *out, int ci, const double c[3], const double q[3], float thr,
                                             float lm32, int next, double h, double inv_h)
{
    double gx = rint(c[0] * inv_h) * h, gy = rint(c[1] * inv_h) * h, gz = rint(c[2] * inv_h) * h;
    float4 *o = reinterpret_cast<float4 *>(out + ci);
    o[0] = make_float4((float)gx, (float)gy, (float)gz, thr);
    o[1] = make_float4((float)(c[0] - gx), (float)(c[1] - gy), (float)(c[2] - gz), __int_as_float(next));
    o[2] = make_float4((float)q[0], (float)q[1], (float)q[2], lm32);
}

// Double-single view for the OV_PREC_DD law: the centre of mass as its grid
// part (exact in FP32) plus the rest (exact in FP64) as hi + lo floats, the
// circulation as hi + lo.
__device__ __forceinline__ void write_cellff(CellFF *out, int ci, const double c[3], const double q[3], double h,
                                             double inv_h)
{
    CellFF o;
    for (int a = 0; a < 3; ++a) {
        const double G = rint(c[a] * inv_h) * h;
        const double f = c[a] - G;
        o.g[a] = (float)G;
        o.fh[a] = (float)f;
        o.fl[a] = (float)(f - (double)o.fh[a]);
        o.qh[a] = (float)q[a];
        o.ql[a] = (float)(q[a] - (double)o.qh[a]);
    }
    o.pad = 0;
    out[ci] = o;
}

// What the traversals read of a cell once its sums are known: the means and
// the circulation in the FP64 cell, the FP32 and double-single views.
struct CellViews {
    Cell32 *c32;
    CellFF *cff;
    double h, inv_h, theta;
    const double *inv_count;   // 1 / k for k < TREE_INV_COUNT
    const float *lev_tab;      // box cells: threshold and Lm per level (null: spherical cells)
};

// Write a cell whole (64 bytes) once its sums are known: the means and the
// circulation, Lm, successor and count, then the FP32 and double-single
// views the traversals read.
// (The mean of a one-node cell is its sum: a product with 1.0.  1 / count
// comes from a table of the rounded quotients for the usual counts.)
__device__ __forceinline__ void store_cell(Cell64 *cells, int ci, const double s[6], int count, double lm, int lev,
                                           int next, const CellViews &v)
{
    double c[3] = {s[0], s[1], s[2]};
    if (count != 1) {
        const double inv = count < TREE_INV_COUNT ? v.inv_count[count] : 1.0 / (double)count;
        c[0] = rn_mul(s[0], inv); c[1] = rn_mul(s[1], inv); c[2] = rn_mul(s[2], inv);
    }
    const double q[3] = {s[3], s[4], s[5]};
    double2 *o = reinterpret_cast<double2 *>(cells + ci);
    o[0] = make_double2(c[0], c[1]);
    o[1] = make_double2(c[2], q[0]);
    o[2] = make_double2(q[1], q[2]);
    reinterpret_cast<int4 *>(cells + ci)[3] = make_int4(__double2loint(lm), __double2hiint(lm), next, count);
    if (v.c32) {
        const float thr = v.lev_tab ? v.lev_tab[lev] : cell_thr(lm, v.theta);
        const float lm32 = v.lev_tab ? v.lev_tab[TREE_LV_SLOTS + lev] : __double2float_ru(lm);
        write_cell32(v.c32, ci, c, q, thr, lm32, next, v.h, v.inv_h);
    }
    if (v.cff) write_cellff(v.cff, ci, c, q, v.h, v.inv_h);
}

__device__ __forceinline__ void store_psum(double *psum, int ci, const double acc[6])
{
    psum[3 * (size_t)ci] = acc[0];
    psum[3 * (size_t)ci + 1] = acc[1];
    psum[3 * (size_t)ci + 2] = acc[2];
}

// Add a finished cell's sums to acc (position sum, circulation sum), in
// the order of a sum over its children: a one-node cell's mean is its
// position (a product with 1.0), larger cells keep the sum in psum.
__device__ __forceinline__ void add_cell_sums(const Cell64 &c, const double *psum, int ci, double acc[6])
{
    double p0 = c.cx, p1 = c.cy, p2 = c.cz;
    if (c.count != 1) {
        p0 = psum[3 * (size_t)ci];
        p1 = psum[3 * (size_t)ci + 1];
        p2 = psum[3 * (size_t)ci + 2];
    }
    acc[0] = rn_add(acc[0], p0); acc[1] = rn_add(acc[1], p1); acc[2] = rn_add(acc[2], p2);
    acc[3] = rn_add(acc[3], c.qx); acc[4] = rn_add(acc[4], c.qy); acc[5] = rn_add(acc[5], c.qz);
}

// A node's moment as k_keys stored it (6 doubles at 48-byte stride).
__device__ __forceinline__ void load_moment(const double *nm, int id, double m[6])
{
    const double2 *q = reinterpret_cast<const double2 *>(nm + 6 * (size_t)id);
    const double2 a = q[0], b = q[1], c = q[2];
    m[0] = a.x; m[1] = a.y; m[2] = b.x; m[3] = b.y; m[4] = c.x; m[5] = c.y;
}

// Last index j in [s, end) with (keys[j] >> sh) == P, given that keys[s]
// has that prefix (keys sorted): probes at s + 1, 2, 4, ... then a binary
// search in the last gap, so a cell of c nodes costs about 2 log2(c) loads.
__device__ __forceinline__ int last_sharing(const uint64_t *keys, int s, int end, int sh, uint64_t P)
{
    int lo = s, hi = end, step = 1;
    while (true) {
        const int probe = lo + step;
        if (probe >= end) break;
        if ((keys[probe] >> sh) != P) { hi = probe; break; }
        lo = probe;
        step = step < (1 << 29) ? 2 * step : step;
    }
    while (hi - lo > 1) {
        const int mid = lo + ((hi - lo) >> 1);
        if ((keys[mid] >> sh) == P) lo = mid; else hi = mid;
    }
    return lo;
}

// Start of level `lev` in the per-level cell lists (levels ascending).
__device__ __forceinline__ int level_start(const int *lvl_cnt, int lev)
{
    int st = 0;
    for (int l = 0; l < lev; ++l) st += lvl_cnt[l];
    return st;
}

// The cells that start at each sorted position: levels cp+1 .. L of the
// node's path, each with its level, first sorted node and Lm.  The deepest,
// level L, is the node's leaf (one node, or the run of nodes sharing the
// deepest cell): it is finished here, since it depends on no other cell
// (octree.c:264-283 for a one-node cell).  The others hold at least this
// node and the next; each is entered in its level's list (lvl_list; slots
// handed out per block, any order within a level) for k_level, which sums
// their children and derives their counts and successors.
template <bool SPH>
__global__ void k_cells(const uint64_t *__restrict__ keys, const int *__restrict__ cpl,
                        const int *__restrict__ cell_off, int *counters, const int *__restrict__ tt, KeyGeom g,
                        int cap, Cell64 *__restrict__ cells, int *__restrict__ first, uint8_t *__restrict__ lvl8,
                        int *lvl_cnt, int *__restrict__ lvl_list, int cap_cells, const int *__restrict__ order,
                        const double *__restrict__ nm, double *__restrict__ psum, CellViews views)
{
    __shared__ int h[TREE_LV_SLOTS], hbase[TREE_LV_SLOTS];
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int nne_all = counters[TC_NNE];
    int ncell = cell_off[nne_all];
    if (ncell > cap_cells) {   // the same for every block
        if (s == 0) {
            atomicMax(&counters[TC_NEED], ncell);
            atomicOr(&counters[TC_ERR], OV_EW_CELLS);
        }
        return;
    }
    if (threadIdx.x < TREE_LV_SLOTS) h[threadIdx.x] = 0;
    __syncthreads();
    uint64_t key = 0;
    int st = 0, M = 0, cp = 0, L = 0;
    bool mine = false;
    if (s < nne_all && s < cap) {
        key = keys[s];
        const int *w = tt + key_member(g, key) * TT_WORDS;
        st = w[TT_START];
        M = w[TT_M];
        const int nne = w[TT_NNE], loc = s - st;
        if (loc == 0) lvl8[cell_off[s]] = 0;   // the member's root
        if (loc >= 0 && loc < M && nne >= 2) {
            cp = loc > 0 ? cpl[s - 1] : 0;
            int cn = loc + 1 < M ? cpl[s] : 0;
            L = min(max(cp, cn) + 1, g.levels);
            mine = L > cp;
        }
    }
    // the warp's range of levels; its non-leaf cells counted per level with
    // one shared atomic per warp and level
    const int lv_lo = __reduce_min_sync(0xffffffffu, mine ? cp + 1 : OV_MAX_LEVEL + 1);
    const int lv_hi = __reduce_max_sync(0xffffffffu, mine ? L : 0);
    for (int lev = lv_lo; lev < lv_hi; ++lev) {
        const unsigned m = __ballot_sync(0xffffffffu, mine && cp < lev && lev < L);
        if (lane == 0 && m) atomicAdd(&h[lev], __popc(m));
    }
    __syncthreads();
    if (threadIdx.x < TREE_LV_SLOTS) {
        const int n = h[threadIdx.x];
        hbase[threadIdx.x] = n ? level_start(lvl_cnt, threadIdx.x) +
                                     atomicAdd(&lvl_cnt[TREE_LV_SLOTS + threadIdx.x], n) : 0;
        h[threadIdx.x] = 0;
    }
    __syncthreads();
    const int loc = s - st;
    const int base = mine ? cell_off[s] + (loc == 0) : 0;
    // Box cells: Lm is the root's scaled by 2^-lev, within a few ulps of the
    // reference's rounded child boxes (octree.c:165-232); the traversals'
    // opening tests take it outside a 1e-12 band and walk the exact box
    // (cell_lm_exact) inside it.  Spherical cells: the exact box, walked from
    // the root (their Lm is not a scaled copy).
    double b[3], t[3];
    const int mem = key_member(g, key) < OV_SPH_MEMBERS ? key_member(g, key) : 0;
    if (SPH && mine) {
        for (int a = 0; a < 3; ++a) { b[a] = g.sb[mem][a]; t[a] = g.st[mem][a]; }
        for (int lev = 1; lev <= cp; ++lev) {
            double cb[3], ct[3];
            sph_child_box(b, t, (int)((key >> dsh(g, lev)) & 7), cb, ct);
            for (int a = 0; a < 3; ++a) { b[a] = cb[a]; t[a] = ct[a]; }
        }
    }
    // every cell but the leaf: level, first node, Lm, list slot (the rest is
    // k_level's)
    for (int lev = lv_lo; lev < lv_hi; ++lev) {
        const bool in = mine && cp < lev && lev < L;
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (!m) continue;
        int wofs = 0;
        if (lane == __ffs(m) - 1) wofs = atomicAdd(&h[lev], __popc(m));
        wofs = __shfl_sync(0xffffffffu, wofs, __ffs(m) - 1);
        if (!in) continue;
        const int ci = base + (lev - cp - 1);
        double lm;
        if (SPH) {
            double cb[3], ct[3];
            sph_child_box(b, t, (int)((key >> dsh(g, lev)) & 7), cb, ct);
            for (int a = 0; a < 3; ++a) { b[a] = cb[a]; t[a] = ct[a]; }
            lm = sph_box_lm(b, t);
        } else {
            lm = ldexp(g.root_lm, -lev);
        }
        first[ci] = s;
        lvl8[ci] = (uint8_t)lev;
        cells[ci].lm = lm;
        const int slot = hbase[lev] + wofs + __popc(m & ((1u << lane) - 1u));
        if (slot < cap_cells) lvl_list[slot] = ci;
        else atomicOr(&counters[TC_ERR], OV_EW_BOUNDS);
    }
    if (!mine) return;
    // the leaf: one node, or at the deepest level the run sharing its key
    const int ci = base + (L - cp - 1);
    double lm;
    if (SPH) {
        double cb[3], ct[3];
        sph_child_box(b, t, (int)((key >> dsh(g, L)) & 7), cb, ct);
        lm = sph_box_lm(cb, ct);
    } else {
        lm = ldexp(g.root_lm, -L);
    }
    first[ci] = s;
    lvl8[ci] = (uint8_t)L;
    const int sh = dsh(g, L);
    const int e = L == g.levels ? last_sharing(keys, s, st + M, sh, key >> sh) : s;
    const int count = e - s + 1, next = cell_off[e + 1];   // the member's end of cells when e + 1 == st + M
    double acc[6];
    if (count == 1) {
        load_moment(nm, order[s], acc);
    } else {
        // depth overflow: sum its nodes in sorted order
        for (int k = 0; k < 6; ++k) acc[k] = 0;
        for (int j = 0; j < count; ++j) {
            double m6[6];
            load_moment(nm, order[s + j], m6);
            for (int k = 0; k < 6; ++k) acc[k] = rn_add(acc[k], m6[k]);
        }
        store_psum(psum, ci, acc);
    }
    store_cell(cells, ci, acc, count, lm, L, next, views);
}

// Above this many slots the level sums run as one launch per level.
constexpr int kLevelLaunchSlots = 1 << 19;

// Grid-wide barrier of the cooperative k_levels (all blocks resident): one
// arrival per block on a counter cleared by the build, then a bounded wait
// for the epoch's total.  A wait that runs out sets OV_EW_ITER and returns
// false in every thread of the block, which then leaves the kernel.
constexpr unsigned kBarrierSpins = 1u << 22;   // of at least 64 ns each

__device__ __forceinline__ bool grid_barrier(unsigned *count, unsigned epoch, int *counters)
{
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0) {
        __threadfence();   // this block's sums before the arrival
        atomicAdd(count, 1u);
        const unsigned target = (epoch + 1) * gridDim.x;
        unsigned spins = 0;
        while (atomicAdd(count, 0u) < target) {
            if (++spins > kBarrierSpins) {
                atomicOr(&counters[TC_ERR], OV_EW_ITER);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();   // the other blocks' sums after it
    }
    return __syncthreads_and(ok) != 0;
}

// One non-leaf cell of the bottom-up moment sums (octree_update_means,
// octree.c:264-283, here per subtree): the sum of its children in child
// order (pre-order: ci + 1, then each child's successor, until a cell that
// is not of level lev + 1); its count is theirs and its successor the last
// child's.
__device__ __forceinline__ void level_cell(int ci, int lev, int ncell, int *counters, Cell64 *__restrict__ cells,
                                           const uint8_t *__restrict__ lvl8, double *__restrict__ psum,
                                           const CellViews &views)
{
    if (ci <= 0 || ci >= ncell) { atomicOr(&counters[TC_ERR], OV_EW_BOUNDS); return; }
    const double lm = __ldcg(&cells[ci].lm);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    int ch = ci + 1, cnt = 0, nc = 0;
    for (; nc < 8 && ch < ncell; ++nc) {
        // the child's level, cell and position sum in one round trip (the
        // sum is only used for a cell of more than one node); L2 loads: the
        // children of the previous level were written in this launch
        const int lv = __ldcg(&lvl8[ch]);
        const double2 *cc = reinterpret_cast<const double2 *>(cells + ch);
        const double2 c0 = __ldcg(cc), c1 = __ldcg(cc + 1), c2 = __ldcg(cc + 2);
        const int4 c3 = __ldcg(reinterpret_cast<const int4 *>(cells + ch) + 3);
        const double ps0 = __ldcg(&psum[3 * (size_t)ch]), ps1 = __ldcg(&psum[3 * (size_t)ch + 1]),
                     ps2 = __ldcg(&psum[3 * (size_t)ch + 2]);
        if (lv != lev + 1) break;
        const int ccount = c3.w, cnext = c3.z;
        const bool one = ccount == 1;
        acc[0] = rn_add(acc[0], one ? c0.x : ps0);
        acc[1] = rn_add(acc[1], one ? c0.y : ps1);
        acc[2] = rn_add(acc[2], one ? c1.x : ps2);
        acc[3] = rn_add(acc[3], c1.y); acc[4] = rn_add(acc[4], c2.x); acc[5] = rn_add(acc[5], c2.y);
        cnt += ccount;
        if (cnext <= ch) { nc = 9; break; }
        ch = cnext;
    }
    if (nc == 0 || nc > 8 || (nc == 8 && ch < ncell && __ldcg(&lvl8[ch]) == lev + 1)) {
        atomicOr(&counters[TC_ERR], OV_EW_BOUNDS);
        return;
    }
    store_psum(psum, ci, acc);
    store_cell(cells, ci, acc, cnt, lm, lev, ch, views);
}

// One level of the bottom-up sums per launch (large trees: the levels hold
// enough cells to fill the GPU, and launches cost less than grid barriers).
__global__ void k_level(int lev, const int *__restrict__ lvl_cnt, const int *__restrict__ lvl_list,
                        const int *__restrict__ cell_off, int *counters, int cap_cells, Cell64 *__restrict__ cells,
                        const uint8_t *__restrict__ lvl8, double *__restrict__ psum, CellViews views)
{
    const int n = lvl_cnt[lev];
    if (n == 0) return;
    const int ncell = cell_off[counters[TC_NNE]];
    if (ncell > cap_cells) return;   // flagged by k_cells; the host grows the storage
    int start = 0;
    for (int l = 0; l < lev; ++l) start += lvl_cnt[l];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ci = start + i < cap_cells ? lvl_list[start + i] : -1;
        level_cell(ci, lev, ncell, counters, cells, lvl8, psum, views);
    }
}

// The bottom-up sums of every non-leaf cell, deepest level first, in one
// cooperative launch (small trees, where a launch per level would cost more
// than the level's work): the blocks share each level's list, then meet at a
// grid barrier (levels without cells are skipped by every block alike).
// The leaves were finished by k_cells.
__global__ void k_levels(int lev_hi, const int *__restrict__ lvl_cnt, const int *__restrict__ lvl_list,
                         unsigned *barrier, const int *__restrict__ cell_off, int *counters, int cap_cells,
                         Cell64 *__restrict__ cells, const uint8_t *__restrict__ lvl8, double *__restrict__ psum,
                         CellViews views)
{
    const int ncell = cell_off[counters[TC_NNE]];
    if (ncell > cap_cells) return;   // flagged by k_cells; the host grows the storage (every block alike)
    int start = 0;
    for (int l = 0; l <= lev_hi; ++l) start += lvl_cnt[l];
    unsigned epoch = 0;
    for (int lev = lev_hi; lev >= 1; --lev) {
        const int n = lvl_cnt[lev];
        start -= n;   // level lev's list is [start, start + n)
        if (n == 0) continue;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            const int ci = start + i < cap_cells ? lvl_list[start + i] : -1;
            level_cell(ci, lev, ncell, counters, cells, lvl8, psum, views);
        }
        if (lev > 1 && !grid_barrier(barrier, epoch++, counters)) return;
    }
}

// Roots, one block per member: level-1 children plus the nodes outside the
// root box; also the one-node and empty members.
__global__ void k_root(const int *__restrict__ order, const int *__restrict__ cell_off, int *counters,
                       int *tt, const double *__restrict__ nm, KeyGeom g, Cell64 *cells, const double *psum,
                       int *first, int cap_cells, CellViews views)
{
    __shared__ double red[6][256];
    int *w = tt + blockIdx.x * TT_WORDS;
    const int M = w[TT_M], nne = w[TT_NNE], st = w[TT_START], nout = nne - M;
    const int total = cell_off[counters[TC_NNE]];
    const bool fits = total <= cap_cells;   // else flagged by k_cells; the host grows the storage
    if (blockIdx.x == 0 && threadIdx.x == 0) counters[TC_NCELL] = fits ? total : 0;
    const int root = cell_off[st], end = cell_off[st + nne];
    if (threadIdx.x == 0) {
        w[TT_ROOT] = (fits && nne > 0) ? root : 0;
        w[TT_END] = (fits && nne > 0) ? end : 0;
    }
    if (!fits || nne == 0) return;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int j = threadIdx.x; j < nout; j += blockDim.x) {
        double m[6];
        load_moment(nm, order[st + M + j], m);
        for (int k = 0; k < 6; ++k) acc[k] = rn_add(acc[k], m[k]);
    }
    if (nne == 1 && M == 1 && threadIdx.x == 0) load_moment(nm, order[st], acc);
    for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = rn_add(red[k][threadIdx.x], red[k][threadIdx.x + off]);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    double sum[6];
    for (int k = 0; k < 6; ++k) sum[k] = 0;
    if (nne >= 2) {
        for (int ch = root + 1; ch < end && ch > root; ch = cells[ch].next)
            add_cell_sums(cells[ch], psum, ch, sum);
    }
    for (int k = 0; k < 6; ++k) sum[k] = rn_add(sum[k], red[k][0]);
    Cell64 r;
    double inv = 1.0 / (double)nne;
    r.cx = rn_mul(sum[0], inv); r.cy = rn_mul(sum[1], inv); r.cz = rn_mul(sum[2], inv);
    r.qx = sum[3]; r.qy = sum[4]; r.qz = sum[5];
    const int mem = blockIdx.x < OV_SPH_MEMBERS ? blockIdx.x : 0;
    r.lm = g.sph_root ? sph_box_lm(g.sb[mem], g.st[mem]) : box_lm(g.lo, g.hi);
    r.next = end;
    r.count = nne;
    cells[root] = r;
    first[root] = st;
    const double c[3] = {r.cx, r.cy, r.cz}, q[3] = {r.qx, r.qy, r.qz};
    if (views.c32)
        write_cell32(views.c32, root, c, q, cell_thr(r.lm, views.theta), __double2float_ru(r.lm), r.next, views.h,
                     views.inv_h);
    if (views.cff) write_cellff(views.cff, root, c, q, views.h, views.inv_h);
}

}  // namespace

int ov_tree_reserve_cells(ov_ctx *c, int cells)
{
    TreeBuf &t = c->tree;
    if (t.cap_cells >= cells && t.cells) return OV_OK;
    void *ptrs[] = {t.cells, t.cells32, t.cellsff, t.psum, t.first, t.lvl_list, t.lvl8};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    t.cells = nullptr; t.cells32 = nullptr; t.cellsff = nullptr; t.first = t.lvl_list = nullptr;
    t.psum = nullptr;
    t.lvl8 = nullptr;
    t.cap_cells = 0;
    OV_ALLOC(c, cudaMalloc(&t.cells, (size_t)cells * sizeof(Cell64)));
    OV_ALLOC(c, cudaMalloc(&t.cells32, (size_t)cells * sizeof(Cell32)));
    OV_ALLOC(c, cudaMalloc(&t.cellsff, (size_t)cells * sizeof(CellFF)));
    OV_ALLOC(c, cudaMalloc(&t.psum, (size_t)cells * 3 * 8));
    OV_ALLOC(c, cudaMalloc(&t.lvl8, (size_t)cells));
    OV_ALLOC(c, cudaMalloc(&t.first, (size_t)cells * 4));
    OV_ALLOC(c, cudaMalloc(&t.lvl_list, (size_t)cells * 4));
    t.cap_cells = cells;
    return OV_OK;
}

int ov_tree_reserve(ov_ctx *c, int cap)
{
    TreeBuf &t = c->tree;
    if (t.cap >= cap && t.keys) return OV_OK;
    int *tt = t.tt;
    t.tt = nullptr;
    ov_tree_free(t);
    t.tt = tt;
    t.cap = cap;
    size_t n = (size_t)cap;
    OV_ALLOC(c, cudaMalloc(&t.keys, n * 8));
    OV_ALLOC(c, cudaMalloc(&t.keys_alt, n * 8));
    OV_ALLOC(c, cudaMalloc(&t.order, n * 4));
    OV_ALLOC(c, cudaMalloc(&t.order_alt, n * 4));
    OV_ALLOC(c, cudaMalloc(&t.torder, n * 4));
    OV_ALLOC(c, cudaMalloc(&t.cpl, n * 4 + 4));
    OV_ALLOC(c, cudaMalloc(&t.ncell_at, n * 4 + 4));
    OV_ALLOC(c, cudaMalloc(&t.cell_off, n * 4 + 8));
    OV_ALLOC(c, cudaMalloc(&t.scan_tmp, (size_t)ov_scan_tmp_ints(cap) * 4));
    OV_ALLOC(c, cudaMalloc(&t.sort_hist, (size_t)ov_sort_hist_ints(cap) * 4));
    OV_ALLOC(c, cudaMalloc(&t.counters, TC_WORDS * 4));
    OV_ALLOC(c, cudaMalloc(&t.lvl_cnt, 3 * TREE_LV_SLOTS * 4));
    OV_ALLOC(c, cudaMalloc(&t.nm, n * 6 * 8));
    OV_ALLOC(c, cudaMalloc(&t.lev_tab, 2 * TREE_LV_SLOTS * sizeof(float)));
    OV_ALLOC(c, cudaMalloc(&t.inv_count, TREE_INV_COUNT * sizeof(double)));
    {
        std::vector<double> inv(TREE_INV_COUNT, 0.0);
        for (int k = 1; k < TREE_INV_COUNT; ++k) inv[k] = 1.0 / (double)k;   // IEEE quotients, as on the device
        OV_CUDA(c, cudaMemcpy(t.inv_count, inv.data(), TREE_INV_COUNT * sizeof(double), cudaMemcpyHostToDevice));
    }
    OV_CUDA(c, cudaMemset(t.counters, 0, TC_WORDS * 4));
    // cells: about 1.3 per node for filament tangles (plus a root per
    // member); grown on demand
    return ov_tree_reserve_cells(c, 2 * cap + 64 + (int)c->mem.size());
}

void ov_tree_free(TreeBuf &t)
{
    void *ptrs[] = {t.keys, t.keys_alt, t.order, t.order_alt, t.torder, t.cpl, t.ncell_at, t.cell_off, t.scan_tmp,
                    t.sort_hist, t.cells, t.cells32, t.cellsff, t.psum, t.first, t.lvl_list, t.lvl8, t.lvl_cnt, t.nm, t.lev_tab, t.inv_count,
                    t.counters, t.tt};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    t = TreeBuf{};
}

static KeyGeom key_geom(const ov_ctx *c)
{
    const Geometry &geo = c->geo;
    KeyGeom g;
    bool fast = true;
    for (int a = 0; a < 3; ++a) {
        g.lo[a] = geo.lo[a];
        g.hi[a] = geo.hi[a];
        g.L[a] = geo.L[a];
        g.invL[a] = 1.0 / geo.L[a];
        g.invL62[a] = ldexp(g.invL[a], 62);
        // bound on how far the reference's rounded faces (21 levels) and the
        // fixed-point image (a subtraction, a product with the rounded 1/L)
        // may sit from the exact dyadic faces, in box units
        double bound = (fabs(geo.lo[a]) + fabs(geo.hi[a])) / geo.L[a] * 64 * 2.220446049250313e-16 +
                       6 * 2.220446049250313e-16;
        if (!(bound < ldexp(1.0, -44))) fast = false;
    }
    g.fast = fast ? 1 : 0;
    g.tb = c->key_tbits;
    g.levels = c->key_levels;
    g.lvmask = ((g.levels >= 21 ? ~0ull >> 1 : (1ull << (3 * g.levels)) - 1)) << (63 - g.tb - 3 * g.levels);
    g.nt = (int)c->mem.size();
    g.sph_root = c->geo.sph;
    {
        const double Lx = geo.hi[0] - geo.lo[0], Ly = geo.hi[1] - geo.lo[1], Lz = geo.hi[2] - geo.lo[2];
        g.root_lm = Lx > Ly ? (Lx > Lz ? Lx : Lz) : (Ly > Lz ? Ly : Lz);   // box_lm's ternary
    }
    for (int m = 0; m < OV_SPH_MEMBERS; ++m)
        for (int a = 0; a < 3; ++a) {
            g.sb[m][a] = c->sph_lo[m][a];
            g.st[m][a] = c->sph_hi[m][a];
        }
    return g;
}

// Build the tree (a forest for ensembles) of `na` with the context's
// topology on stream s.  Everything stays on the device, so the sequence
// can be graph-captured.
int ov_tree_build(ov_ctx *c, const NodeArrays &na, cudaStream_t s)
{
    TreeBuf &t = c->tree;
    int cap = c->cap;
    const int nt = (int)c->mem.size();
    c->tree_built = false;   // a query tree is only current until the next build
    if (!t.tt) return ov_fail(c, OV_ERR_STATE, "member table not allocated");
    KeyGeom g = key_geom(c);
    OV_CUDA(c, cudaMemsetAsync(t.counters, 0, TC_BUILD_CLEAR * 4, s));
    OV_CUDA(c, cudaMemsetAsync(t.counters + TC_STAT64, 0, (TC_WORDS - TC_STAT64) * 4, s));
    OV_CUDA(c, cudaMemsetAsync(t.tt, 0, (size_t)nt * TT_WORDS * 4, s));
    OV_CUDA(c, cudaMemsetAsync(t.lvl_cnt, 0, 3 * TREE_LV_SLOTS * 4, s));
    int nb = (cap + 255) / 256;
    if (c->geo.sph)
        k_keys<true><<<nb, 256, 0, s>>>(c->status, na.x, na.y, na.z, nt > 1 ? c->d_tid : nullptr, cap, g, t.keys,
                                        t.order, t.counters, t.tt, c->fwd, c->geo, t.nm);
    else
        k_keys<false><<<nb, 256, 0, s>>>(c->status, na.x, na.y, na.z, nt > 1 ? c->d_tid : nullptr, cap, g, t.keys,
                                         t.order, t.counters, t.tt, c->fwd, c->geo, t.nm);
    k_layout<<<1, 32, 0, s>>>(t.tt, nt, c->d_qorder, t.counters, t.lev_tab, g.root_lm, c->params.bh_resolution);
    c->launches += 2;
    ov_sort_keys(c, t, cap, s);
    k_cpl<<<nb, 256, 0, s>>>(t.keys, cap, t.counters, t.tt, g, t.cpl, t.ncell_at, t.lvl_cnt);
    k_target_order<<<nb, 256, 0, s>>>(t.keys, t.order, cap, t.counters, t.tt, g, t.torder);
    c->launches += 2;
    ov_scan_exclusive(c, t.ncell_at, t.cell_off, cap, t.counters + TC_NNE, 0, t.scan_tmp, s);
    CellViews views;
    const bool fp32_view = c->precision == OV_PREC_MIXED || c->precision == OV_PREC_DD || c->walk == OV_WALK_SPLIT;
    views.c32 = fp32_view ? t.cells32 : nullptr;
    views.cff = c->precision == OV_PREC_DD ? t.cellsff : nullptr;
    views.h = c->grid_h;
    views.inv_h = 1.0 / c->grid_h;
    views.theta = c->params.bh_resolution;
    views.inv_count = t.inv_count;
    views.lev_tab = c->geo.sph ? nullptr : t.lev_tab;
    if (c->geo.sph)
        k_cells<true><<<nb, 256, 0, s>>>(t.keys, t.cpl, t.cell_off, t.counters, t.tt, g, cap, t.cells, t.first,
                                         t.lvl8, t.lvl_cnt, t.lvl_list, t.cap_cells, t.order, t.nm, t.psum,
                                         views);
    else
        k_cells<false><<<nb, 256, 0, s>>>(t.keys, t.cpl, t.cell_off, t.counters, t.tt, g, cap, t.cells, t.first,
                                          t.lvl8, t.lvl_cnt, t.lvl_list, t.cap_cells, t.order, t.nm, t.psum,
                                          views);
    if (cap > kLevelLaunchSlots) {
        for (int lev = g.levels - 1; lev >= 1; --lev)
            k_level<<<4 * c->sm_count, 256, 0, s>>>(lev, t.lvl_cnt, t.lvl_list, t.cell_off, t.counters, t.cap_cells,
                                                    t.cells, t.lvl8, t.psum, views);
        c->launches += g.levels - 2;
    } else {
        // the level sums: one cooperative launch, every block resident
        static int per_sm = 0;
        if (!per_sm) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_levels, 256, 0);
            per_sm = per_sm > 0 ? per_sm : 1;
        }
        const int want = std::max(1, cap / 1024);   // about four non-leaf cells a thread on the fullest level
        const int grid = std::max(1, std::min(per_sm * c->sm_count, want));
        int lev_hi = g.levels - 1;
        unsigned *barrier = reinterpret_cast<unsigned *>(t.lvl_cnt + 2 * TREE_LV_SLOTS);
        void *args[] = {&lev_hi, &t.lvl_cnt, &t.lvl_list, &barrier, &t.cell_off, &t.counters, &t.cap_cells,
                        &t.cells, &t.lvl8, &t.psum, &views};
        OV_CUDA(c, cudaLaunchCooperativeKernel((const void *)k_levels, grid, 256, args, 0, s));
    }
    k_root<<<nt, 256, 0, s>>>(t.order, t.cell_off, t.counters, t.tt, t.nm, g, t.cells, t.psum, t.first, t.cap_cells,
                              views);
    c->launches += 3;
    OV_CUDA(c, cudaGetLastError());
    return OV_OK;
}
