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

#include <cuda/atomic>

void ov_sort_keys(ov_ctx *c, TreeBuf &t, int n, cudaStream_t s);
int ov_sort_hist_ints(int cap);
int ov_scan_tmp_ints(int n_max);

namespace {

struct KeyGeom {
    double lo[3], hi[3], L[3];
    double invL[3];    // 1 / L, rounded
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

template <bool SPH>
__global__ void k_keys(const int *__restrict__ status, const double *__restrict__ x,
                       const double *__restrict__ y, const double *__restrict__ z, const int *__restrict__ tid,
                       int cap, KeyGeom g, uint64_t *__restrict__ keys, int *__restrict__ order,
                       int *counters, int *tt)
{
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
    // one atomic per warp for each counter, one per member present in the warp
    unsigned b_live = __ballot_sync(0xffffffffu, live), b_in = __ballot_sync(0xffffffffu, inside);
    unsigned peers = __match_any_sync(0xffffffffu, live ? m : -1) & b_live;
    if (lane == 0 && b_live) {
        atomicAdd(&counters[TC_NNE], __popc(b_live));
        atomicAdd(&counters[TC_M], __popc(b_in));
        atomicAdd(&counters[TC_OUT], __popc(b_live & ~b_in));
    }
    if (live && lane == __ffs(peers) - 1) {
        atomicAdd(&tt[m * TT_WORDS + TT_NNE], __popc(peers));
        atomicAdd(&tt[m * TT_WORDS + TT_M], __popc(peers & b_in));
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&counters[TC_ERR], OV_EW_NAN);
    if (i >= cap) return;
    order[i] = i;
    if (!live) { keys[i] = OV_KEY_EMPTY; return; }
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
        double u = rn_mul(rn_sub(p[a], g.lo[a]), g.invL[a]);
        u = fmin(fmax(u, 0.0), 1.0);
        U[a] = (uint64_t)(u * 4611686018427387904.0);   // u * 2^62
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

// Member layout: first sorted position of each member (members in id order)
// and the first work tile of each in the traversal queue (queue order).
__global__ void k_layout(int *tt, int nt, const int *__restrict__ qorder, int *counters)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
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
// first position, then the cells of the levels the node starts.
__global__ void k_cpl(const uint64_t *__restrict__ keys, int cap, int *counters, const int *__restrict__ tt,
                      KeyGeom g, int *__restrict__ cpl, int *__restrict__ ncell_at)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    int nne_all = counters[TC_NNE];
    int L = 0, nne = 0;
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
        } else {
            cpl[s] = 0;
            ncell_at[s] = (loc == 0);
        }
    }
    int Lmax = (nne >= 2) ? L : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) Lmax = max(Lmax, __shfl_xor_sync(0xffffffffu, Lmax, o));
    bool anydeep = __any_sync(0xffffffffu, deep);
    if ((threadIdx.x & 31) == 0) {
        if (Lmax > 0) atomicMax(&counters[TC_MAXDEPTH], Lmax);
        if (anydeep) atomicOr(&counters[TC_ERR], OV_EW_DEPTH);
    }
}

// first index j in [lo, hi) with (keys[j] >> sh) > P  (keys sorted)
__device__ __forceinline__ int upper_prefix(const uint64_t *keys, int lo, int hi, int sh, uint64_t P)
{
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((keys[mid] >> sh) > P) hi = mid; else lo = mid + 1;
    }
    return lo;
}
// first index j in [lo, hi) with (keys[j] >> sh) >= P
__device__ __forceinline__ int lower_prefix(const uint64_t *keys, int lo, int hi, int sh, uint64_t P)
{
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((keys[mid] >> sh) >= P) hi = mid; else lo = mid + 1;
    }
    return lo;
}

template <bool SPH>
__global__ void k_cells(const uint64_t *__restrict__ keys, const int *__restrict__ cpl,
                        const int *__restrict__ cell_off, int *counters, const int *__restrict__ tt, KeyGeom g,
                        int cap, Cell64 *__restrict__ cells, int *__restrict__ parent, int *__restrict__ nchild,
                        int *__restrict__ arrive, int *__restrict__ first, int cap_cells)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    int nne_all = counters[TC_NNE];
    if (s >= nne_all || s >= cap) return;
    int ncell = cell_off[nne_all];
    if (ncell > cap_cells) {
        if (s == 0) {
            atomicMax(&counters[TC_NEED], ncell);
            atomicOr(&counters[TC_ERR], OV_EW_CELLS);
        }
        return;
    }
    uint64_t key = keys[s];
    const int *w = tt + key_member(g, key) * TT_WORDS;
    const int st = w[TT_START], M = w[TT_M], nne = w[TT_NNE];
    const int loc = s - st;
    if (loc < 0 || loc >= M || nne < 2) return;
    const int end = st + M;   // the member's in-box positions are [st, end)
    const int root = cell_off[st];
    int cp = loc > 0 ? cpl[s - 1] : 0;
    int cn = loc + 1 < M ? cpl[s] : 0;
    int L = min(max(cp, cn) + 1, g.levels);
    const int base = cell_off[s] + (loc == 0);
    // Box cells: Lm is the root's scaled by 2^-lev, within a few ulps of the
    // reference's rounded child boxes (octree.c:165-232); the traversals'
    // opening tests take it outside a 1e-12 band and walk the exact box
    // (cell_lm_exact) inside it.  Spherical cells: the exact box, walked from
    // the root (their Lm is not a scaled copy).
    double b[3], t[3];
    const int mem = key_member(g, key) < OV_SPH_MEMBERS ? key_member(g, key) : 0;
    if (SPH) {
        for (int a = 0; a < 3; ++a) { b[a] = g.sb[mem][a]; t[a] = g.st[mem][a]; }
        for (int lev = 1; lev <= cp; ++lev) {
            double cb[3], ct[3];
            sph_child_box(b, t, (int)((key >> dsh(g, lev)) & 7), cb, ct);
            for (int a = 0; a < 3; ++a) { b[a] = cb[a]; t[a] = ct[a]; }
        }
    }
    for (int lev = cp + 1; lev <= L; ++lev) {
        int ci = base + (lev - cp - 1);
        if (SPH) {
            double cb[3], ct[3];
            sph_child_box(b, t, (int)((key >> dsh(g, lev)) & 7), cb, ct);
            for (int a = 0; a < 3; ++a) { b[a] = cb[a]; t[a] = ct[a]; }
        }
        int sh = dsh(g, lev);
        int e = (lev < L) ? upper_prefix(keys, s + 1, end, sh, key >> sh) - 1 : s;
        if (lev == g.levels) e = upper_prefix(keys, s + 1, end, sh, key >> sh) - 1;
        Cell64 cell;
        cell.lm = SPH ? sph_box_lm(b, t) : ldexp(g.root_lm, -lev);
        cell.count = e - s + 1;
        cell.next = cell_off[e + 1];   // the member's end of cells when e + 1 == end
        cell.cx = cell.cy = cell.cz = cell.qx = cell.qy = cell.qz = 0;
        cells[ci] = cell;
        first[ci] = s;
        int par;
        if (lev == 1) par = root;
        else if (cp < lev - 1) par = ci - 1;
        else {
            int psh = dsh(g, lev - 1);
            int sp = lower_prefix(keys, st, s, psh, key >> psh);
            int cpp = sp > st ? cpl[sp - 1] : 0;
            par = cell_off[sp] + (sp == st) + (lev - 1 - cpp - 1);
        }
        parent[ci] = par;
        arrive[ci] = 0;
        atomicAdd(&nchild[par], 1);
    }
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

__device__ __forceinline__ void finalize_cell(Cell64 *cells, int ci, const double s[6], int count)
{
    double inv = 1.0 / (double)count;
    cells[ci].cx = rn_mul(s[0], inv);
    cells[ci].cy = rn_mul(s[1], inv);
    cells[ci].cz = rn_mul(s[2], inv);
    cells[ci].qx = s[3];
    cells[ci].qy = s[4];
    cells[ci].qz = s[5];
}

// Leaves from the nodes, then each parent from its children by the last
// child to arrive (one atomic per edge, no waiting).
__global__ void k_moments(const uint64_t *__restrict__ keys, const int *__restrict__ order,
                          const int *__restrict__ cpl, const int *__restrict__ cell_off, int *counters,
                          const int *__restrict__ tt, KeyGeom g, int cap,
                          const double *__restrict__ x, const double *__restrict__ y,
                          const double *__restrict__ z, const int *__restrict__ fwd, Geometry geo,
                          Cell64 *cells, const int *__restrict__ parent, const int *__restrict__ nchild,
                          int *arrive, double *csum, int cap_cells)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    int nne_all = counters[TC_NNE];
    if (s >= nne_all || s >= cap || cell_off[nne_all] > cap_cells) return;
    const int *w = tt + key_member(g, keys[s]) * TT_WORDS;
    const int st = w[TT_START], M = w[TT_M], nne = w[TT_NNE];
    const int loc = s - st;
    if (loc < 0 || loc >= M || nne < 2) return;
    const int root = cell_off[st];
    int cp = loc > 0 ? cpl[s - 1] : 0;
    int cn = loc + 1 < M ? cpl[s] : 0;
    int L = min(max(cp, cn) + 1, g.levels);
    int leaf = cell_off[s] + (loc == 0) + (L - cp - 1);
    int cnt = cells[leaf].count;
    double acc[6];
    if (cnt == 1) {
        node_moment(order[s], x, y, z, fwd, geo, acc);
    } else {
        // deepest level still shared (depth overflow): sum its nodes
        for (int k = 0; k < 6; ++k) acc[k] = 0;
        for (int j = 0; j < cnt; ++j) {
            double m[6];
            node_moment(order[s + j], x, y, z, fwd, geo, m);
            for (int k = 0; k < 6; ++k) acc[k] = rn_add(acc[k], m[k]);
        }
        if (loc > 0 && cpl[s - 1] >= L) return;   // only the first node of the run
    }
    for (int k = 0; k < 6; ++k) csum[6 * (size_t)leaf + k] = acc[k];
    finalize_cell(cells, leaf, acc, cnt);
    int cur = leaf;
    for (int guard = 0; guard < 64; ++guard) {
        int p = parent[cur];
        if (p <= root) break;
        // release this cell's sums, and (last child) acquire the siblings'
        cuda::atomic_ref<int, cuda::thread_scope_device> arr(arrive[p]);
        const int old = arr.fetch_add(1, cuda::memory_order_acq_rel);
        if (old != nchild[p] - 1) break;
        double sum[6] = {0, 0, 0, 0, 0, 0};
        int end = __ldcg(&cells[p].next);
        for (int ch = p + 1; ch != end && ch > 0; ch = __ldcg(&cells[ch].next)) {
            for (int k = 0; k < 6; ++k) sum[k] = rn_add(sum[k], __ldcg(&csum[6 * (size_t)ch + k]));
        }
        for (int k = 0; k < 6; ++k) csum[6 * (size_t)p + k] = sum[k];
        finalize_cell(cells, p, sum, __ldcg(&cells[p].count));
        cur = p;
    }
}

// Roots, one block per member: level-1 children plus the nodes outside the
// root box; also the one-node and empty members.
__global__ void k_root(const int *__restrict__ order, const int *__restrict__ cell_off, int *counters,
                       int *tt, const double *__restrict__ x, const double *__restrict__ y,
                       const double *__restrict__ z, const int *__restrict__ fwd, Geometry geo, KeyGeom g,
                       Cell64 *cells, const double *csum, int *first, int cap_cells)
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
        node_moment(order[st + M + j], x, y, z, fwd, geo, m);
        for (int k = 0; k < 6; ++k) acc[k] = rn_add(acc[k], m[k]);
    }
    if (nne == 1 && M == 1 && threadIdx.x == 0) node_moment(order[st], x, y, z, fwd, geo, acc);
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
            for (int k = 0; k < 6; ++k) sum[k] = rn_add(sum[k], csum[6 * (size_t)ch + k]);
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
}

// Double-single copy of every cell's centre of mass and circulation for
// the OV_PREC_DD law: the centre of mass as its grid part (exact in FP32)
// plus the rest (exact in FP64) as hi + lo floats, the circulation as hi + lo.
__global__ void k_cellsff(const Cell64 *__restrict__ cells, const int *counters, double h, double inv_h,
                          CellFF *__restrict__ out)
{
    int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= counters[TC_NCELL]) return;
    const Cell64 c = cells[ci];
    const double com[3] = {c.cx, c.cy, c.cz}, q[3] = {c.qx, c.qy, c.qz};
    CellFF o;
    for (int a = 0; a < 3; ++a) {
        const double G = rint(com[a] * inv_h) * h;
        const double f = com[a] - G;
        o.g[a] = (float)G;
        o.fh[a] = (float)f;
        o.fl[a] = (float)(f - (double)o.fh[a]);
        o.qh[a] = (float)q[a];
        o.ql[a] = (float)(q[a] - (double)o.qh[a]);
    }
    o.pad = 0;
    out[ci] = o;
}

// FP32 copy of every cell for the mixed traversal: COM split into a part on
// the grid of step h (exact in FP32) and a small remainder.
// The opening test Lm / d < theta becomes d^2 > (Lm / theta)^2: thr holds
// that bound times (1 + 2e-5), rounded up, so that d^2 > thr accepts clear
// of the guard band and d^2 < thr (1 - 2e-5) / (1 + 2e-5) opens clear of it.
__global__ void k_cells32(const Cell64 *__restrict__ cells, const int *counters, double h, double inv_h,
                          double theta, Cell32 *__restrict__ out)
{
    int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= counters[TC_NCELL]) return;
    Cell64 c = cells[ci];
    Cell32 o;
    double cx = c.cx, cy = c.cy, cz = c.cz;
    double gx = rint(cx * inv_h) * h, gy = rint(cy * inv_h) * h, gz = rint(cz * inv_h) * h;
    o.gx = (float)gx; o.gy = (float)gy; o.gz = (float)gz;
    const double r = c.lm / theta;
    o.thr = theta > 0 ? __double2float_ru(r * r * (1.0 + 2e-5)) : __int_as_float(0x7f800000);
    o.fx = (float)(cx - gx); o.fy = (float)(cy - gy); o.fz = (float)(cz - gz);
    o.next = c.next;
    o.qx = (float)c.qx; o.qy = (float)c.qy; o.qz = (float)c.qz;
    o.lm = __double2float_ru(c.lm);
    out[ci] = o;
}

}  // namespace

int ov_tree_reserve_cells(ov_ctx *c, int cells)
{
    TreeBuf &t = c->tree;
    if (t.cap_cells >= cells && t.cells) return OV_OK;
    void *ptrs[] = {t.cells, t.cells32, t.cellsff, t.parent, t.nchild, t.arrive, t.csum, t.first};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    t.cells = nullptr; t.cells32 = nullptr; t.cellsff = nullptr; t.parent = t.nchild = t.arrive = t.first = nullptr;
    t.csum = nullptr;
    t.cap_cells = 0;
    OV_ALLOC(c, cudaMalloc(&t.cells, (size_t)cells * sizeof(Cell64)));
    OV_ALLOC(c, cudaMalloc(&t.cells32, (size_t)cells * sizeof(Cell32)));
    OV_ALLOC(c, cudaMalloc(&t.cellsff, (size_t)cells * sizeof(CellFF)));
    OV_ALLOC(c, cudaMalloc(&t.parent, (size_t)cells * 4));
    OV_ALLOC(c, cudaMalloc(&t.nchild, (size_t)cells * 4));
    OV_ALLOC(c, cudaMalloc(&t.arrive, (size_t)cells * 4));
    OV_ALLOC(c, cudaMalloc(&t.csum, (size_t)cells * 6 * 8));
    OV_ALLOC(c, cudaMalloc(&t.first, (size_t)cells * 4));
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
    OV_CUDA(c, cudaMemset(t.counters, 0, TC_WORDS * 4));
    // cells: about 1.3 per node for filament tangles (plus a root per
    // member); grown on demand
    return ov_tree_reserve_cells(c, 2 * cap + 64 + (int)c->mem.size());
}

void ov_tree_free(TreeBuf &t)
{
    void *ptrs[] = {t.keys, t.keys_alt, t.order, t.order_alt, t.torder, t.cpl, t.ncell_at, t.cell_off, t.scan_tmp,
                    t.sort_hist, t.cells, t.cells32, t.cellsff, t.parent, t.nchild, t.arrive, t.csum, t.first,
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
    OV_CUDA(c, cudaMemsetAsync(t.nchild, 0, (size_t)t.cap_cells * 4, s));
    int nb = (cap + 255) / 256;
    if (c->geo.sph)
        k_keys<true><<<nb, 256, 0, s>>>(c->status, na.x, na.y, na.z, nt > 1 ? c->d_tid : nullptr, cap, g, t.keys,
                                        t.order, t.counters, t.tt);
    else
        k_keys<false><<<nb, 256, 0, s>>>(c->status, na.x, na.y, na.z, nt > 1 ? c->d_tid : nullptr, cap, g, t.keys,
                                         t.order, t.counters, t.tt);
    k_layout<<<1, 32, 0, s>>>(t.tt, nt, c->d_qorder, t.counters);
    c->launches += 2;
    ov_sort_keys(c, t, cap, s);
    k_cpl<<<nb, 256, 0, s>>>(t.keys, cap, t.counters, t.tt, g, t.cpl, t.ncell_at);
    k_target_order<<<nb, 256, 0, s>>>(t.keys, t.order, cap, t.counters, t.tt, g, t.torder);
    c->launches += 2;
    ov_scan_exclusive(c, t.ncell_at, t.cell_off, cap, t.counters + TC_NNE, 0, t.scan_tmp, s);
    if (c->geo.sph)
        k_cells<true><<<nb, 256, 0, s>>>(t.keys, t.cpl, t.cell_off, t.counters, t.tt, g, cap, t.cells, t.parent,
                                         t.nchild, t.arrive, t.first, t.cap_cells);
    else
        k_cells<false><<<nb, 256, 0, s>>>(t.keys, t.cpl, t.cell_off, t.counters, t.tt, g, cap, t.cells, t.parent,
                                          t.nchild, t.arrive, t.first, t.cap_cells);
    k_moments<<<nb, 256, 0, s>>>(t.keys, t.order, t.cpl, t.cell_off, t.counters, t.tt, g, cap, na.x, na.y, na.z,
                                 c->fwd, c->geo, t.cells, t.parent, t.nchild, t.arrive, t.csum, t.cap_cells);
    k_root<<<nt, 256, 0, s>>>(t.order, t.cell_off, t.counters, t.tt, na.x, na.y, na.z, c->fwd, c->geo, g, t.cells,
                              t.csum, t.first, t.cap_cells);
    c->launches += 3;
    if (c->precision == OV_PREC_MIXED || c->precision == OV_PREC_DD || c->walk == OV_WALK_SPLIT) {
        k_cells32<<<(t.cap_cells + 255) / 256, 256, 0, s>>>(t.cells, t.counters, c->grid_h, 1.0 / c->grid_h,
                                                           c->params.bh_resolution, t.cells32);
        c->launches++;
    }
    if (c->precision == OV_PREC_DD) {
        k_cellsff<<<(t.cap_cells + 255) / 256, 256, 0, s>>>(t.cells, t.counters, c->grid_h, 1.0 / c->grid_h,
                                                           t.cellsff);
        c->launches++;
    }
    OV_CUDA(c, cudaGetLastError());
    return OV_OK;
}
