// ov_velocity.cu - per-node velocity kernels.
//
//  k_tangents     update_tangent_normal (tangle.c:423-502), one node per thread
//  k_vel_fp64     update_velocity (tangle.c:600-726) fused: LIA + external
//                 v_s + Barnes-Hut over the primary and every image query
//                 point + mutual friction, one warp per 32 Morton-ordered
//                 targets sharing one cursor through the pre-order cells
//  k_rec_sums     direct sums, the tree==NULL branch (tangle.c:652-687), in
//                 (node, segment chunk) blocks; k_direct_finish adds LIA etc.
//  k_euler / k_rk4_combine / k_wrap   RK4 stages and enforce_periodic_boundaries
//
// The FP64 traversal keeps the reference's decisions bit-for-bit given the
// same cell data: Lm/d < theta, d < 1e-8 and ndot < 1e-8 are evaluated by a
// cheap test with a 1e-12 relative guard band and, inside the band, by the
// reference's own correctly rounded divisions.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "ov_internal.cuh"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_E
#define M_E 2.7182818284590452354
#endif

namespace {

struct VelArgs {
    const int *order, *counters;
    const int *tt;          // per-member build table (TT_WORDS ints a member)
    const int *qorder;      // members in work-queue order (null: id order)
    const int *tid;         // member of each slot (null: a single tangle)
    const DevParams *tprm;  // per-member parameters (null: prm)
    const int2 *mrange;     // per-member slot range [x, y) (null: [0, cap))
    int *work;              // work-queue counter
    int nt;                 // members
    int G;                  // query groups per node
    int S;                  // sub-walks per query point (FP64 split walk of a small tangle), else 1
    const Cell64 *cells;
    const Cell32 *cells32;
    const CellFF *cellsff;      // OV_PREC_DD: double-single cell data
    const double *x, *y, *z, *tx, *ty, *tz, *nx, *ny, *nz;
    double *vx, *vy, *vz, *sx, *sy, *sz;
    const int *fwd, *rev, *status, *pin;
    Geometry geo;
    DevParams prm;
    double t;
    const double *t_dev;    // when set, the time is t_dev[t_index] (graph-captured RK4)
    int t_index;
    double f4pi;            // KAPPA/4/M_PI in the reference's rounding
    double grid_h, inv_h;   // mixed path
    float shift_g[OV_MAX_IMAGES][3], shift_f[OV_MAX_IMAGES][3];   // L*shift split on the grid
    int cap;                // node slots (bounds checks)
    float th2f, near2f, f4pif;   // theta^2, near-field radius^2, KAPPA/4/pi in FP32
    float f4pi_h, f4pi_l;        // KAPPA/4/pi in double-single
    double near2;           // mixed path: squared near-field radius
    unsigned long long *stat;
    unsigned *node_counts;  // when set: visits[cap], then accepts[cap], per target slot
    // box cells store Lm scaled from the root's (null for spherical trees,
    // whose stored Lm is exact): the exact one is walked on demand
    const int *cell_first;  // first sorted position of each cell's nodes
    const uint64_t *keys;   // sorted path keys
    int key_tb;             // member-id bits above the path
    double root_lm;         // Lm of the root box
    double lm_ulp;          // 2^-44 max |box coordinate|: per-level slack of a scaled Lm
};

// Largest side of cell cp's box as the reference rounds it (make_child_box,
// octree.c:165-232; octree.c:302-306), walked from the root along the path of
// the cell's first node.  Only the opening tests within their band need it.
__device__ __noinline__ double cell_lm_exact(const VelArgs &a, const Cell64 *cp)
{
    const double lm = cp->lm;
    if (!a.cell_first) return lm;
    const int c = (int)(cp - a.cells);
    const int lev = ilogb(a.root_lm) - ilogb(lm);
    if (lev <= 0 || lev > OV_MAX_LEVEL || c < 0) return lm;
    const int s = a.cell_first[c];
    if (s < 0 || s >= a.cap) return lm;
    const uint64_t key = a.keys[s];
    double b[3] = {a.geo.lo[0], a.geo.lo[1], a.geo.lo[2]}, t[3] = {a.geo.hi[0], a.geo.hi[1], a.geo.hi[2]};
    for (int l = 1; l <= lev; ++l) {
        double cb[3], ct[3];
        child_box_dev(b, t, (int)((key >> (63 - a.key_tb - 3 * l)) & 7), cb, ct);
        for (int x = 0; x < 3; ++x) { b[x] = cb[x]; t[x] = ct[x]; }
    }
    return box_lm(b, t);
}

// Bound on |stored Lm - exact Lm| for a box cell: each level's midpoint and
// child bounds add a few roundings of the box coordinates (the parents'
// errors average, they do not add up); (lev + 2) 2^-44 max|coordinate| is
// far above them.
__device__ __forceinline__ double lm_slack(const VelArgs &a, double lm)
{
    if (!a.cell_first) return 0.0;
    return (double)(ilogb(a.root_lm) - ilogb(lm) + 2) * a.lm_ulp;
}

// Add one work item's visits and accepts of target slot id to the per-node
// counters (only when they were asked for: ov_set_node_counting).
__device__ __forceinline__ void count_node(const VelArgs &a, bool valid, int id, unsigned vis, unsigned acc)
{
    if (a.node_counts && valid) {
        atomicAdd(&a.node_counts[id], vis);
        atomicAdd(&a.node_counts[a.cap + id], acc);
    }
}

// Record the first failed bounds check (code, index) and raise the error bit.
__device__ __forceinline__ void bad_index(const VelArgs &a, int code, int idx)
{
    atomicCAS((int *)&a.counters[TC_BAD], 0, (code << 24) | (idx & 0xFFFFFF) | (1 << 30));
    atomicOr((int *)&a.counters[TC_ERR], OV_EW_BOUNDS);
}

// step_node (tangle.c:155-194) without recursion: a pinned end reverses the
// walk and mirrors the result in its wall, innermost mirror applied first.
__device__ bool step_node_dev(const VelArgs &a, int i, int where, double out[3])
{
    int walls[8];
    int nw = 0, cur = i, w = where;
    for (int guard = 0; w != 0; ++guard) {
        if (guard > 16 || cur < 0 || cur >= a.cap) return false;
        int st = a.status[cur];
        if (st == OV_FREE) {
            cur = w > 0 ? a.fwd[cur] : a.rev[cur];
            w += w > 0 ? -1 : 1;
        } else if (st == OV_PINNED || st == OV_PINNED_SLIP) {
            int nb = w > 0 ? a.fwd[cur] : a.rev[cur];
            if (nb >= 0) {
                cur = nb;
                w += w > 0 ? -1 : 1;
            } else {
                if (nw >= 8) return false;
                walls[nw++] = a.pin[cur];
                w = -w;
            }
        } else {
            return false;
        }
    }
    if (cur < 0 || cur >= a.cap || a.status[cur] == OV_EMPTY) return false;
    out[0] = a.x[cur]; out[1] = a.y[cur]; out[2] = a.z[cur];
    for (int m = nw - 1; m >= 0; --m) {
        int f = walls[m];
        if (f < 0 || f > 5) continue;
        int ax = f >> 1;
        double wpos = (f & 1) ? a.geo.hi[ax] : a.geo.lo[ax];
        out[ax] = rn_sub(rn_mul(2.0, wpos), out[ax]);
    }
    return true;
}

// FP64 hardware approximations (PTX rcp.approx / rsqrt.approx; relative
// error below 2^-20, measured on sm_103a), refined by the functions below.
__device__ __forceinline__ double rcp_seed(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
}
__device__ __forceinline__ double rsqrt_seed(double x)
{
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
}

// 1/sqrt(x) and 1/x (x normal, positive) from the hardware approximations
// (relative error below 2^-20 on sm_103a) with one third-order correction:
// for e = 1 - x y0^2, y0 (1 + e/2 + 3e^2/8) leaves 5e^3/16, and for
// e = 1 - x y0, y0 (1 + e + e^2) leaves e^3: below 2^-53 for |e| < 2^-18.
__device__ __forceinline__ double rsqrt3(double x)
{
    const double y0 = rsqrt_seed(x);
    const double e = fma(-(x * y0), y0, 1.0);
    return fma(y0 * e, fma(0.375, e, 0.5), y0);
}
__device__ __forceinline__ double rcp3(double x)
{
    const double y0 = rcp_seed(x);
    const double e = fma(-x, y0, 1.0);
    return fma(y0, fma(e, e, e), y0);
}

__device__ __forceinline__ double wrapped_len(const Geometry &g, const double r1[3], const double r2in[3])
{
    double r2[3] = {r2in[0], r2in[1], r2in[2]};
    pwrap_dev(g, r1, r2);
    return len3_ref(rn_sub(r1[0], r2[0]), rn_sub(r1[1], r2[1]), rn_sub(r1[2], r2[2]));
}

__global__ void k_tangents(VelArgs a, int cap, int *counters)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cap || a.status[k] == OV_EMPTY) return;
    const Geometry &g = a.geo;
    double s0[3] = {a.x[k], a.y[k], a.z[k]}, s1[3], s2[3], sm1[3], sm2[3];
    bool ok = step_node_dev(a, k, 1, s1) & step_node_dev(a, k, 2, s2) & step_node_dev(a, k, -1, sm1) &
              step_node_dev(a, k, -2, sm2);
    if (!ok) {
        atomicOr(&counters[TC_ERR], OV_EW_WALK);
        return;
    }
    double w2[3] = {s2[0], s2[1], s2[2]}, w1[3] = {s1[0], s1[1], s1[2]};
    double wm1[3] = {sm1[0], sm1[1], sm1[2]}, wm2[3] = {sm2[0], sm2[1], sm2[2]};
    pwrap_dev(g, s0, w2);
    pwrap_dev(g, s0, w1);
    pwrap_dev(g, s0, wm1);
    pwrap_dev(g, s0, wm2);
    double d1 = len3_ref(rn_sub(s0[0], w1[0]), rn_sub(s0[1], w1[1]), rn_sub(s0[2], w1[2]));
    double d2 = rn_add(d1, wrapped_len(g, s1, s2));
    double dm1 = len3_ref(rn_sub(s0[0], wm1[0]), rn_sub(s0[1], wm1[1]), rn_sub(s0[2], wm1[2]));
    double dm2 = rn_add(dm1, wrapped_len(g, sm1, sm2));
    double den[4] = {
        rn_mul(rn_mul(rn_mul(d2, rn_sub(d2, d1)), rn_add(dm1, d2)), rn_add(dm2, d2)),
        rn_mul(rn_mul(rn_mul(d1, rn_sub(d2, d1)), rn_add(dm1, d1)), rn_add(dm2, d1)),
        rn_mul(rn_mul(rn_mul(dm1, rn_add(dm1, d1)), rn_add(dm1, d2)), rn_sub(dm2, dm1)),
        rn_mul(rn_mul(rn_mul(dm2, rn_add(dm2, d1)), rn_add(dm2, d2)), rn_sub(dm2, dm1))};
    double c1[4] = {rn_mul(rn_mul(-d1, dm1), dm2), rn_mul(rn_mul(d2, dm1), dm2), rn_mul(rn_mul(-d1, d2), dm2),
                    rn_mul(rn_mul(d1, d2), dm1)};
    double c2[4] = {
        rn_mul(2.0, rn_sub(rn_mul(rn_sub(dm1, d1), dm2), rn_mul(d1, dm1))),
        rn_mul(-2.0, rn_sub(rn_mul(rn_sub(dm1, d2), dm2), rn_mul(d2, dm1))),
        rn_mul(2.0, rn_sub(rn_mul(rn_add(d2, d1), dm2), rn_mul(d1, d2))),
        rn_mul(-2.0, rn_sub(rn_mul(rn_add(d2, d1), dm1), rn_mul(d1, d2)))};
    // the reference divides c1 and c2 by den; one corrected reciprocal each
    // (within 2 ulp of the quotients) keeps GB300's FP64 pipe to a third
    double r1[4], r2[4];
#pragma unroll
    for (int z = 0; z < 4; ++z) {
        const double inv = rcp3(den[z]);
        r1[z] = c1[z] * inv;
        r2[z] = c2[z] * inv;
    }
    double ds[4][3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        ds[0][ax] = rn_sub(w2[ax], s0[ax]);
        ds[1][ax] = rn_sub(w1[ax], s0[ax]);
        ds[2][ax] = rn_sub(wm1[ax], s0[ax]);
        ds[3][ax] = rn_sub(wm2[ax], s0[ax]);
    }
    double tg[3], nm[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double tt = 0, nn = 0;
#pragma unroll
        for (int z = 0; z < 4; ++z) {
            tt = rn_add(tt, rn_mul(r1[z], ds[z][ax]));
            nn = rn_add(nn, rn_mul(r2[z], ds[z][ax]));
        }
        tg[ax] = tt; nm[ax] = nn;
    }
    double *T[3] = {(double *)a.tx, (double *)a.ty, (double *)a.tz};
    double *Nn[3] = {(double *)a.nx, (double *)a.ny, (double *)a.nz};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) { T[ax][k] = tg[ax]; Nn[ax][k] = nm[ax]; }
}

__device__ __forceinline__ double now(const VelArgs &a) { return a.t_dev ? a.t_dev[a.t_index] : a.t; }

// get_v (external_velocity.c:62-81)
__device__ __forceinline__ void ext_vel(int type, const double dir[3], double s1, double s0, double tld,
                                        double t, double out[3])
{
    if (type == OV_SIMPLE || type == OV_DECREASING) {
        double s = s1;
        if (type == OV_DECREASING && t < tld) s = rn_sub(s0, rn_div(rn_mul(t, rn_sub(s0, s1)), tld));
        out[0] = rn_mul(dir[0], s); out[1] = rn_mul(dir[1], s); out[2] = rn_mul(dir[2], s);
    } else {
        out[0] = out[1] = out[2] = 0;
    }
}

// shifted (tangle.c:370-414)
__device__ __forceinline__ void image_point(const Geometry &g, int j, const double p[3], double q[3])
{
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) q[ax] = rn_sub(p[ax], rn_mul(g.L[ax], (double)g.shift[j][ax]));
    for (int m = 0; m < g.nreflect[j]; ++m) {
        int f = g.reflect[j][m];
        if (f < 0 || f > 5) continue;
        int ax = f >> 1;
        double w = (f & 1) ? g.hi[ax] : g.lo[ax];
        q[ax] = rn_sub(rn_mul(2.0, w), p[ax]);
    }
}

__device__ __forceinline__ void mirror_vec(int f, double v[3])
{
    // mirror_vector_reflect (boundaries.c:201-211): normal component flips
    int ax = f >> 1;
    v[ax] = -v[ax];
}

// The segment law (octree.c:321-342 / tangle.c:536-559) for R = COM - r
// (or segment start - r) and Rp1 = R + q.  lR is |R| as the caller
// computed it.  Returns false when a filter drops the segment.
__device__ __forceinline__ bool segment_law64(const double R[3], const double Rp1[3], double lR, double f4pi,
                                              double out[3])
{
    double lRp1 = len3_ref(Rp1[0], Rp1[1], Rp1[2]);
    if (lR < 1e-8 || lRp1 < 1e-8) return false;
    double dotv = dot3_ref(R[0], R[1], R[2], Rp1[0], Rp1[1], Rp1[2]);
    double pr = rn_mul(lR, lRp1);
    // ndot = dot/lR/lRp1 < 1e-8 ?
    double thr = 1e-8 * pr;
    bool drop;
    if (dotv < thr * (1.0 - 1e-12)) drop = true;
    else if (dotv > thr * (1.0 + 1e-12)) drop = false;
    else drop = rn_div(rn_div(dotv, lR), lRp1) < 1e-8;
    if (drop) return false;
    double denom = pr * (pr + dotv);
    double sc = f4pi * (lR + lRp1) / denom;
    out[0] = (R[1] * Rp1[2] - R[2] * Rp1[1]) * sc;
    out[1] = (R[2] * Rp1[0] - R[0] * Rp1[2]) * sc;
    out[2] = (R[0] * Rp1[1] - R[1] * Rp1[0]) * sc;
    return true;
}

// 1/x (x normal and positive): two Newton-Raphson steps (20 -> 40 -> 80
// bits), full double precision without the correctly rounded sequence
__device__ __forceinline__ double recip_1_2(double x)
{
    double y = rcp_seed(x);
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// 1/sqrt(x) (x normal and positive): y <- y (3/2 - x/2 y^2)
__device__ __forceinline__ double rsqrt_nr(double x)
{
    double y = rsqrt_seed(x);
    const double h = 0.5 * x;
    y = y * fma(-h * y, y, 1.5);
    return y * fma(-h * y, y, 1.5);
}

// One Barnes-Hut query point for the 32 lanes of a warp.  `part` = lane
// takes part; returns the lane's velocity in v.
__device__ __forceinline__ void bh_query64(const VelArgs &a, const double q[3], bool part, int root, int ncell,
                                           double v[3], unsigned long long &visits,
                                           unsigned long long &accepts, unsigned long long &steps,
                                           bool &overflow)
// cells of the tree: [root, ncell)
{
    v[0] = v[1] = v[2] = 0;
    const double theta = a.prm.theta;
    int c = root;
    int resume = part ? 0 : 0x7fffffff;
    int guard = 0;
    const int guard_max = 4 * (ncell - root) + 64;
    while (c < ncell) {
        if (c < root) { bad_index(a, 5, c); break; }
        const Cell64 *cp = a.cells + c;
        double cx = __ldg(&cp->cx), cy = __ldg(&cp->cy), cz = __ldg(&cp->cz);
        double lm = __ldg(&cp->lm);
        int nxt = __ldg(&cp->next);
        if (nxt <= c || nxt > ncell) { bad_index(a, 6, c); nxt = ncell; }
        bool open = false;
        if (c >= resume) {
            ++visits;
            double dx = rn_sub(q[0], cx), dy = rn_sub(q[1], cy), dz = rn_sub(q[2], cz);
            double d = len3_ref(dx, dy, dz);
            if (d < 1e-8) {
                resume = nxt;
            } else {
                bool acc;
                if (nxt == c + 1) {
                    acc = true;   // leaf (or a cell at the deepest level)
                } else {
                    double td = theta * d;
                    const double sl = lm_slack(a, lm);
                    if (lm + sl < td * (1.0 - 1e-12)) acc = true;
                    else if (lm - sl > td * (1.0 + 1e-12)) acc = false;
                    else acc = rn_div(cell_lm_exact(a, cp), d) < theta;
                }
                if (acc) {
                    ++accepts;
                    double R[3] = {-dx, -dy, -dz};
                    double Rp1[3] = {rn_add(R[0], __ldg(&cp->qx)), rn_add(R[1], __ldg(&cp->qy)),
                                     rn_add(R[2], __ldg(&cp->qz))};
                    double w[3];
                    if (segment_law64(R, Rp1, d, a.f4pi, w)) {
                        v[0] += w[0]; v[1] += w[1]; v[2] += w[2];
                    }
                    resume = nxt;
                } else {
                    open = true;
                }
            }
        }
        ++steps;
        c = __any_sync(0xffffffffu, open) ? c + 1 : nxt;
        if (++guard > guard_max) { overflow = true; break; }
    }
}

// LIA (tangle.c:568-592) + external v_s, given the BH sums; then vels with
// mutual friction and PINNED_SLIP (tangle.c:689-725).
__device__ __forceinline__ bool finish_impl(const VelArgs &a, const DevParams &P, int id, const double p[3],
                                            const double prim[3], const double img[3], int *err, double vs_out[3],
                                            double vel_out[3])
{
    int st = a.status[id];
    if (st == OV_PINNED) {
        ext_vel(P.vb_type, P.vb_dir, P.vb_s1, P.vb_s0, P.vb_tld, now(a), vel_out);
        vs_out[0] = vs_out[1] = vs_out[2] = 0;
        return true;
    }
    double nx_[3], pv[3];
    if (!(step_node_dev(a, id, 1, nx_) && step_node_dev(a, id, -1, pv))) {
        *err |= OV_EW_WALK;
        return false;
    }
    double l_next = wrapped_len(a.geo, p, nx_);
    double l_prev = wrapped_len(a.geo, pv, p);
    double f = rn_div(rn_div(rn_mul(P.kappa,
                              log(rn_div(rn_div(rn_mul(2.0, sqrt(rn_mul(l_next, l_prev))), sqrt(M_E)), P.a0))),
                         4.0),
                    M_PI);
    double tg[3] = {a.tx[id], a.ty[id], a.tz[id]}, nm[3] = {a.nx[id], a.ny[id], a.nz[id]};
    double vs[3] = {rn_mul(rn_sub(rn_mul(tg[1], nm[2]), rn_mul(tg[2], nm[1])), f),
                    rn_mul(rn_sub(rn_mul(tg[2], nm[0]), rn_mul(tg[0], nm[2])), f),
                    rn_mul(rn_sub(rn_mul(tg[0], nm[1]), rn_mul(tg[1], nm[0])), f)};
    double ev[3];
    ext_vel(P.vs_type, P.vs_dir, P.vs_s1, P.vs_s0, P.vs_tld, now(a), ev);
    for (int ax = 0; ax < 3; ++ax) vs[ax] = rn_add(rn_add(rn_add(vs[ax], ev[ax]), prim[ax]), img[ax]);
    double vel[3] = {vs[0], vs[1], vs[2]};
    if (P.friction) {
        double vn[3];
        ext_vel(P.vn_type, P.vn_dir, P.vn_s1, P.vn_s0, P.vn_tld, now(a), vn);
        double dv[3] = {rn_sub(vn[0], vs[0]), rn_sub(vn[1], vs[1]), rn_sub(vn[2], vs[2])};
        double c1[3] = {rn_sub(rn_mul(tg[1], dv[2]), rn_mul(tg[2], dv[1])), rn_sub(rn_mul(tg[2], dv[0]), rn_mul(tg[0], dv[2])),
                        rn_sub(rn_mul(tg[0], dv[1]), rn_mul(tg[1], dv[0]))};
        for (int ax = 0; ax < 3; ++ax) vel[ax] = rn_add(vel[ax], rn_mul(c1[ax], P.alpha));
        double c2[3] = {rn_sub(rn_mul(tg[1], c1[2]), rn_mul(tg[2], c1[1])), rn_sub(rn_mul(tg[2], c1[0]), rn_mul(tg[0], c1[2])),
                        rn_sub(rn_mul(tg[0], c1[1]), rn_mul(tg[1], c1[0]))};
        double m = -P.alpha_p;
        for (int ax = 0; ax < 3; ++ax) vel[ax] = rn_add(vel[ax], rn_mul(c2[ax], m));
    }
    if (st == OV_PINNED_SLIP) {
        int f2 = a.pin[id];
        if (f2 >= 0 && f2 < 6) {
            int ax = f2 >> 1;
            double n = (f2 & 1) ? -1.0 : 1.0;
            double nv = rn_mul(n, vel[ax]);
            vel[ax] = rn_sub(vel[ax], rn_mul(n, nv));
        }
    }
    for (int ax = 0; ax < 3; ++ax) { vs_out[ax] = vs[ax]; vel_out[ax] = vel[ax]; }
    return true;
}

// finish_impl with the parameters of the node's member
__device__ __forceinline__ bool finish_node(const VelArgs &a, int id, const double p[3], const double prim[3],
                                            const double img[3], int *err, double vs_out[3], double vel_out[3])
{
    if (a.tprm) {
        int m = a.tid[id];
        if (m < 0 || m >= a.nt) { bad_index(a, 8, id); return false; }
        const DevParams P = a.tprm[m];
        return finish_impl(a, P, id, p, prim, img, err, vs_out, vel_out);
    }
    return finish_impl(a, a.prm, id, p, prim, img, err, vs_out, vel_out);
}

// Work item `it` of the traversal queue: member m, its first sorted
// position st, its node count nne, its cells [root, end), and the tile and
// query group.  Items are (group, tile) pairs, group-major: warps running at
// the same time share the query points' image set and walk nearby targets,
// so they touch the same cells.  Tiles of 32 sorted targets never cross a
// member; members come in queue order.
struct WorkItem {
    int m, st, nne, root, end, tile, grp, sub;
};

__device__ __forceinline__ WorkItem decode_item(const VelArgs &a, int it, int tiles)
{
    WorkItem w;
    const int gs = it / tiles;   // (query group, sub-walk)
    int tile = it - gs * tiles;
    w.grp = gs / a.S;
    w.sub = gs - w.grp * a.S;
    int k = 0;
    if (a.nt > 1) {
        // last member (in queue order) whose first tile is <= tile
        int lo = 0, hi = a.nt - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            int mm = a.qorder ? a.qorder[mid] : mid;
            if (a.tt[mm * TT_WORDS + TT_ITEM0] <= tile) lo = mid; else hi = mid - 1;
        }
        k = lo;
    }
    w.m = a.qorder ? a.qorder[k] : k;
    const int *t = a.tt + w.m * TT_WORDS;
    w.st = t[TT_START];
    w.nne = t[TT_NNE];
    w.root = t[TT_ROOT];
    w.end = t[TT_END];
    w.tile = tile - t[TT_ITEM0];
    return w;
}

// next work item of the warp (lane 0 takes it, all lanes get it)
__device__ __forceinline__ int next_item(const VelArgs &a)
{
    int it = 0;
    if ((threadIdx.x & 31) == 0) it = atomicAdd(a.work, 1);
    return __shfl_sync(0xffffffffu, it, 0);
}

// The 1 + n_img query points of every node (qi = 0 the node itself, qi >= 1
// image qi-1) are split over G query groups (group g takes qi = g, g+G,
// ...) so that small tangles still fill the GPU.  Persistent warps pull
// (tile, group) items from the work queue; each writes its partial sums
// (own point, images) per sorted target and k_vel_finish adds them in group
// order, so the result does not depend on which warp took which item.
// Resident blocks per SM the register budget is sized for (about 24 warps).
template <int W> constexpr int min_blocks() { return W == 2 ? 12 : (W == 4 ? 6 : 3); }
// (HI: a tighter register budget for one more block per SM, paid in spills)
template <int W, int HI> constexpr int min_blocks_mixed()
{
    return W == 2 ? (HI ? 12 : 10) : (W == 4 ? (HI ? 6 : 5) : (HI ? 3 : 2));
}

template <int W>
__global__ void __launch_bounds__(32 * W, min_blocks<W>()) k_vel_fp64(VelArgs a, double *__restrict__ part_out)
{
    const int lane = threadIdx.x & 31;
    const int tiles = a.counters[TC_ITEMS];
    const int items = tiles * a.G;
    unsigned long long visits = 0, accepts = 0, steps = 0;
    bool overflow = false;
    for (int it = next_item(a); it < items; it = next_item(a)) {
        const WorkItem w = decode_item(a, it, tiles);
        const int loc = 32 * w.tile + lane;
        const int tix = w.st + loc;
        bool valid = loc < w.nne && tix < a.cap;
        int id = valid ? a.order[tix] : 0;
        if (valid && (id < 0 || id >= a.cap)) { bad_index(a, 4, id); valid = false; id = 0; }
        const int st = valid ? a.status[id] : OV_EMPTY;
        const bool part = valid && st != OV_PINNED && st != OV_EMPTY && a.prm.use_bh;
        double p[3] = {0, 0, 0};
        if (valid) { p[0] = a.x[id]; p[1] = a.y[id]; p[2] = a.z[id]; }
        double prim[3] = {0, 0, 0}, img[3] = {0, 0, 0};
        const unsigned long long vis0 = visits, acc0 = accepts;
        for (int qi = w.grp; qi <= a.geo.n_img; qi += a.G) {
            const int j = qi - 1;
            double q[3], v[3];
            if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
            else image_point(a.geo, j, p, q);
            bh_query64(a, q, part, w.root, w.end, v, visits, accepts, steps, overflow);
            if (j < 0) {
                prim[0] = v[0]; prim[1] = v[1]; prim[2] = v[2];
            } else {
                for (int m = 0; m < a.geo.nreflect[j]; ++m) mirror_vec(a.geo.reflect[j][m], v);
                img[0] = rn_add(img[0], v[0]); img[1] = rn_add(img[1], v[1]); img[2] = rn_add(img[2], v[2]);
            }
        }
        if (valid) {
            const size_t cap = (size_t)a.cap;
            for (int ax = 0; ax < 3; ++ax) {
                part_out[((size_t)(2 * w.grp) * 3 + ax) * cap + tix] = prim[ax];
                part_out[((size_t)(2 * w.grp + 1) * 3 + ax) * cap + tix] = img[ax];
            }
        }
        count_node(a, valid, id, (unsigned)(visits - vis0), (unsigned)(accepts - acc0));
    }
    int err = overflow ? OV_EW_ITER : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        visits += __shfl_xor_sync(0xffffffffu, visits, o);
        accepts += __shfl_xor_sync(0xffffffffu, accepts, o);
        err |= __shfl_xor_sync(0xffffffffu, err, o);
    }
    if (lane == 0) {
        atomicAdd(&a.stat[ST_VISITS], visits);
        atomicAdd(&a.stat[ST_ACCEPTS], accepts);
        atomicAdd(&a.stat[ST_STEPS], steps);
        if (err) atomicOr((int *)&a.counters[TC_ERR], err);
    }
}

// Parts of split walks: each group's S parts added in part order into its
// first part's slot (one thread per group, component and target).
__global__ void k_part_sum(VelArgs a, double *__restrict__ part)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nne = min(a.counters[TC_NNE], a.cap);
    const long long per = 6LL * nne;
    if (i >= per * a.G) return;
    const int g = (int)(i / per);
    const int r = (int)(i - (long long)g * per);
    const int comp = r / nne, tix = r - comp * nne;   // comp: prim x,y,z then img x,y,z
    const size_t cap = (size_t)a.cap;
    const int half = comp / 3, ax = comp - 3 * half;
    double s = 0;
    for (int k = 0; k < a.S; ++k) {
        const size_t gs = (size_t)g * a.S + k;
        s = rn_add(s, part[((2 * gs + half) * 3 + ax) * cap + tix]);
    }
    part[((2 * (size_t)g * a.S + half) * 3 + ax) * cap + tix] = s;
}

// Sum the group partials in group order, then LIA, v_s and mutual friction.
__global__ void k_vel_finish(VelArgs a, const double *__restrict__ part_in)
{
    const int tix = blockIdx.x * blockDim.x + threadIdx.x;
    const int nne = a.counters[TC_NNE];
    if (tix >= nne || tix >= a.cap) return;
    int id = a.order[tix];
    if (id < 0 || id >= a.cap) { bad_index(a, 7, id); return; }
    const int st = a.status[id];
    if (st == OV_EMPTY) return;
    const size_t cap = (size_t)a.cap;
    double prim[3] = {0, 0, 0}, img[3] = {0, 0, 0};
    // (with parts, k_part_sum has added each group's parts into its first)
    for (int g = 0; g < a.G * a.S; g += a.S)
        for (int ax = 0; ax < 3; ++ax) {
            prim[ax] = rn_add(prim[ax], part_in[((size_t)(2 * g) * 3 + ax) * cap + tix]);
            img[ax] = rn_add(img[ax], part_in[((size_t)(2 * g + 1) * 3 + ax) * cap + tix]);
        }
    double p[3] = {a.x[id], a.y[id], a.z[id]};
    double vs[3], vel[3];
    int err = 0;
    if (finish_node(a, id, p, prim, img, &err, vs, vel)) {
        a.sx[id] = vs[0]; a.sy[id] = vs[1]; a.sz[id] = vs[2];
        a.vx[id] = vel[0]; a.vy[id] = vel[1]; a.vz[id] = vel[2];
    }
    if (err) atomicOr((int *)&a.counters[TC_ERR], err);
}

// ------------------------------------------------------------ direct sum
// Finish the direct-sum nodes (LIA, v_s, friction) into vels/vs scratch.
__global__ void k_direct_finish(VelArgs a, const int *__restrict__ nodes, int n, const double *__restrict__ sums,
                                int stride, double *__restrict__ vout, double *__restrict__ sout)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    int k = nodes[b];
    double p[3] = {a.x[k], a.y[k], a.z[k]};
    const double *sb = sums + (size_t)stride * b;
    double prim[3] = {sb[0], sb[1], sb[2]};
    double zero[3] = {0, 0, 0}, vs[3] = {0, 0, 0}, vel[3] = {0, 0, 0};
    int err = 0;
    if (a.status[k] != OV_EMPTY) finish_node(a, k, p, prim, zero, &err, vs, vel);
    for (int ax = 0; ax < 3; ++ax) {
        vout[3 * (size_t)b + ax] = vel[ax];
        sout[3 * (size_t)b + ax] = vs[ax];
    }
}

// -------------------------------------------------------------- stepping
// euler_step2 (vortex_dynamics.c:20-42): dst = src + v*dt on non-EMPTY nodes
__global__ void k_euler(const int *__restrict__ status, const double *__restrict__ x, const double *__restrict__ y,
                        const double *__restrict__ z, const double *__restrict__ vx, const double *__restrict__ vy,
                        const double *__restrict__ vz, double dt, double *__restrict__ ox, double *__restrict__ oy,
                        double *__restrict__ oz, int cap, const double *dt_dev)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cap || status[k] == OV_EMPTY) return;
    if (dt_dev) dt = *dt_dev;
    ox[k] = rn_add(x[k], rn_mul(vx[k], dt));
    oy[k] = rn_add(y[k], rn_mul(vy[k], dt));
    oz[k] = rn_add(z[k], rn_mul(vz[k], dt));
}

struct Rk4Args {
    const double *dt_dev;   // when set: the step, and the error word that vetoes the update
    const int *err;
    const int *status;
    double *x, *y, *z;
    const double *v1x, *v1y, *v1z, *v2x, *v2y, *v2z, *v3x, *v3y, *v3z, *v4x, *v4y, *v4z;
    double dt;
    int cap;
};

// vortex_dynamics.c:95-115
__global__ void k_rk4_combine(Rk4Args r)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= r.cap || r.status[k] == OV_EMPTY) return;
    // a stage whose tree did not fit its storage leaves the step undone
    if (r.err && (*r.err & OV_EW_CELLS)) return;
    double dt = r.dt_dev ? *r.dt_dev : r.dt;
    double d6 = dt / 6, d3 = dt / 3;
    double *X[3] = {r.x, r.y, r.z};
    const double *V1[3] = {r.v1x, r.v1y, r.v1z}, *V2[3] = {r.v2x, r.v2y, r.v2z};
    const double *V3[3] = {r.v3x, r.v3y, r.v3z}, *V4[3] = {r.v4x, r.v4y, r.v4z};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double mv = rn_mul(V1[ax][k], d6);
        mv = rn_add(mv, rn_mul(V2[ax][k], d3));
        mv = rn_add(mv, rn_mul(V3[ax][k], d3));
        mv = rn_add(mv, rn_mul(V4[ax][k], d6));
        X[ax][k] = rn_add(X[ax][k], mv);
    }
}

// enforce_periodic_boundaries (tangle.c:793-814)
__global__ void k_wrap(const int *__restrict__ status, double *x, double *y, double *z, Geometry g, int cap)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cap || status[k] == OV_EMPTY) return;
    double p[3] = {x[k], y[k], z[k]};
    for (int guard = 0; guard < 64; ++guard) {
        int face = -1;
        if (p[0] < g.lo[0]) face = OV_LEFT;
        if (p[0] > g.hi[0]) face = OV_RIGHT;
        if (p[1] < g.lo[1]) face = OV_BACK;
        if (p[1] > g.hi[1]) face = OV_FRONT;
        if (p[2] < g.lo[2]) face = OV_DOWN;
        if (p[2] > g.hi[2]) face = OV_UP;
        if (face > -1 && g.wall[face] != OV_WALL_PERIODIC) face = -1;
        if (face < 0) break;
        int ax = face >> 1;
        p[ax] = (face & 1) ? rn_sub(p[ax], g.L[ax]) : rn_add(p[ax], g.L[ax]);
    }
    x[k] = p[0]; y[k] = p[1]; z[k] = p[2];
}

// ----------------------------------------------------------- mixed precision
//
// Positions and centres of mass are split as p = g + f: g on a grid of step
// h = 2^k (every coordinate below 2^22 steps, so g is exact in FP32 and a
// difference of two g's is exact), f the FP32 remainder (|f| <= h/2).  A
// separation is (g_r - g_c) + (f_r - f_c): relative error ~1e-7 even for the
// nearest cells, where a plain FP32 difference of absolute positions would
// lose 4-5 digits.  Decisions (d < 1e-8, Lm/d < theta, |Rp1| < 1e-8,
// ndot < 1e-8) are taken in FP32 only outside a guard band around the
// threshold and redone exactly in FP64 inside it, so they are the FP64
// path's decisions.  Leaf interactions closer than the near-field radius
// are done in FP64.  Per-query sums use Kahan compensation.

// decision of the FP64 path for cell c: 1 skip (d < 1e-8), 2 accept, 0 open
__device__ __forceinline__ int decide64(const VelArgs &a, const Cell64 *cp, const double q[3], double theta, bool leaf,
                                        double dxyz[3], double *dout)
{
    double dx = rn_sub(q[0], __ldg(&cp->cx)), dy = rn_sub(q[1], __ldg(&cp->cy)), dz = rn_sub(q[2], __ldg(&cp->cz));
    double d = len3_ref(dx, dy, dz);
    dxyz[0] = dx; dxyz[1] = dy; dxyz[2] = dz;
    *dout = d;
    if (d < 1e-8) return 1;
    if (leaf) return 2;
    double lm = __ldg(&cp->lm);
    double td = theta * d;
    const double sl = lm_slack(a, lm);
    if (lm + sl < td * (1.0 - 1e-12)) return 2;
    if (lm - sl > td * (1.0 + 1e-12)) return 0;
    return rn_div(cell_lm_exact(a, cp), d) < theta ? 2 : 0;
}

__device__ __forceinline__ bool interact64(const Cell64 *cp, const double dxyz[3], double d, double f4pi, double w[3])
{
    double R[3] = {-dxyz[0], -dxyz[1], -dxyz[2]};
    double Rp1[3] = {rn_add(R[0], __ldg(&cp->qx)), rn_add(R[1], __ldg(&cp->qy)), rn_add(R[2], __ldg(&cp->qz))};
    return segment_law64(R, Rp1, d, f4pi, w);
}

// IEEE bits of a double: for x >= 0, or any x against a positive bound, the
// order of the bits as signed integers is the order of the values (tests on
// the integer pipe instead of the FP64 one).
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// The segment law (octree.c:321-342) for an accepted cell without the
// factor kappa / 4 pi (applied to the query point's sum), in FP64 with
// corrected hardware reciprocal square roots and reciprocal instead of the
// reference's correctly rounded sqrt and divisions (each term within a few
// ulps of the reference's).  R and Rp1 are the reference's own values.  The
// filters |Rp1| < 1e-8 and ndot < 1e-8 are decided as the reference decides
// them: near their thresholds segment_law64 redoes them with its rounding.
// |R| >= 1e-8 holds for every accepted cell (the walk's skip test).  w is
// zero when a filter drops the cell.
__device__ __forceinline__ void law64_term(const Cell64 *cp, const double q[3], double w[3])
{
    w[0] = w[1] = w[2] = 0.0;
    const double2 *c2 = reinterpret_cast<const double2 *>(cp);
    const double2 A = __ldg(c2), B = __ldg(c2 + 1), C = __ldg(c2 + 2);
    // A = (cx, cy)  B = (cz, qx)  C = (qy, qz); R = -(q - COM), rounded alike
    const double R[3] = {A.x - q[0], A.y - q[1], B.x - q[2]};
    const double P[3] = {R[0] + B.y, R[1] + C.x, R[2] + C.y};
    const double lp2 = fma(P[0], P[0], fma(P[1], P[1], P[2] * P[2]));
    const long long lp2_lo = dbits(1e-16 * (1.0 - 1e-12)), lp2_hi = dbits(1e-16 * (1.0 + 1e-12));
    const long long nd_lo = dbits(1e-8 - 1e-12), nd_hi = dbits(1e-8 + 1e-12);
    if (dbits(lp2) < lp2_lo) return;   // |Rp1| < 1e-8
    const double lR2 = fma(R[0], R[0], fma(R[1], R[1], R[2] * R[2]));
    const double dot = fma(R[0], P[0], fma(R[1], P[1], R[2] * P[2]));
    const double ra = rsqrt3(lR2), rb = rsqrt3(lp2), ab = ra * rb;
    const double nd = dot * ab;
    if (dbits(lp2) <= lp2_hi || (dbits(nd) >= nd_lo && dbits(nd) <= nd_hi)) {
        if (!segment_law64(R, P, len3_ref(R[0], R[1], R[2]), 1.0, w)) w[0] = w[1] = w[2] = 0.0;
        return;
    }
    if (dbits(nd) < nd_lo) return;   // ndot < 1e-8
    const double sc = (ra + rb) * ab * rcp3(1.0 + nd);
    w[0] = fma(R[1], P[2], -R[2] * P[1]) * sc;
    w[1] = fma(R[2], P[0], -R[0] * P[2]) * sc;
    w[2] = fma(R[0], P[1], -R[1] * P[0]) * sc;
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float v)
{
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

constexpr int kNearCap = 24;   // deferred near-field leaves per lane
// d^2 below Cell32::thr times this opens a cell clear of the guard band
constexpr float kThrLo = (1.0f - 2e-5f) / (1.0f + 2e-5f);

// ------------------------------------------------ double-single arithmetic
// A value as an unevaluated sum hi + lo of two floats (about 48 bits):
// Knuth's TwoSum, Dekker's fast TwoSum, the FMA TwoProduct, and one Newton
// step from the hardware reciprocal (square root) for 1/x and 1/sqrt(x).
// FP32 runs at 64 times the FP64 rate on GB300, so these reach FP64-class
// accuracy (about 1e-14 per operation) well above FP64's speed.
struct ff { float hi, lo; };

__device__ __forceinline__ ff ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ff ff_fast(float a, float b)   // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff x, ff y)
{
    ff s = ff_two_sum(x.hi, y.hi), t = ff_two_sum(x.lo, y.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = ff_fast(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return ff_fast(s.hi, s.lo);
}
// x + y without the second TwoSum (error relative to |x| + |y|): for sums
// whose terms do not cancel (squares, positive terms, running totals)
__device__ __forceinline__ ff ff_add_sloppy(ff x, ff y)
{
    ff s = ff_two_sum(x.hi, y.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
    return ff_fast(s.hi, s.lo);
}
// x + f for a float f
__device__ __forceinline__ ff ff_add_f(ff x, float f)
{
    ff s = ff_two_sum(x.hi, f);
    s.lo = __fadd_rn(s.lo, x.lo);
    return ff_fast(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(ff x) { return ff{-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }
__device__ __forceinline__ ff ff_mul(ff x, ff y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return ff_fast(p, e);
}
__device__ __forceinline__ ff ff_mulf(ff x, float f)
{
    const float p = __fmul_rn(x.hi, f);
    float e = __fmaf_rn(x.hi, f, -p);
    e = __fmaf_rn(x.lo, f, e);
    return ff_fast(p, e);
}
__device__ __forceinline__ ff ff_from(double v)
{
    const float h = (float)v;
    return ff{h, (float)(v - (double)h)};
}
// 1/sqrt(x), x > 0: y0 from the hardware, then y = y0 + y0 (1 - x y0^2) / 2.
// 1 - x y0^2 is of the order of y0's error: its leading part 1 - hi is exact
// and the rest needs float precision only.
__device__ __forceinline__ ff ff_rsqrt(ff x)
{
    const float y0 = rsqrtf(x.hi);
    const ff t = ff_mulf(ff_mulf(x, y0), y0);
    const float r = __fsub_rn(__fsub_rn(1.0f, t.hi), t.lo);
    return ff_fast(y0, __fmul_rn(__fmul_rn(0.5f, y0), r));
}
// 1/x: y = y0 + y0 (1 - x y0), the correction in float as above
__device__ __forceinline__ ff ff_rcp(ff x)
{
    const float y0 = __frcp_rn(x.hi);
    const ff t = ff_mulf(x, y0);
    const float r = __fsub_rn(__fsub_rn(1.0f, t.hi), t.lo);
    return ff_fast(y0, __fmul_rn(y0, r));
}

// One accepted cell in double-single: the segment law for R = COM - q,
// Rp1 = R + circulation (sc = f4pi (1/|R| + 1/|Rp1|) / (|R| |Rp1| + R.Rp1),
// w = (R x circulation) sc), added into the double-single sums acc[3].  The
// query point is split like the cell: grid part gq (exact) plus fq.
// The segment law for R (start - query) and S (segment vector) in
// double-single: w = (R x S) f4pi (1/|R| + 1/|R+S|) / (|R| |R+S| + R.(R+S)).
__device__ __forceinline__ void ff_segment(const ff R[3], const ff S[3], ff f4pi, ff w[3])
{
    ff P[3];
    for (int a = 0; a < 3; ++a) P[a] = ff_add(R[a], S[a]);
    const ff lR2 = ff_add_sloppy(ff_add_sloppy(ff_mul(R[0], R[0]), ff_mul(R[1], R[1])), ff_mul(R[2], R[2]));
    const ff lp2 = ff_add_sloppy(ff_add_sloppy(ff_mul(P[0], P[0]), ff_mul(P[1], P[1])), ff_mul(P[2], P[2]));
    const ff dot = ff_add(ff_add(ff_mul(R[0], P[0]), ff_mul(R[1], P[1])), ff_mul(R[2], P[2]));
    const ff ra = ff_rsqrt(lR2), rb = ff_rsqrt(lp2);
    const ff ab = ff_mul(ra, rb);
    const ff den = ff_add_f(ff_mul(dot, ab), 1.0f);
    const ff sc = ff_mul(ff_mul(ff_mul(f4pi, ff_add_sloppy(ra, rb)), ab), ff_rcp(den));
    const ff x[3] = {ff_sub(ff_mul(R[1], S[2]), ff_mul(R[2], S[1])), ff_sub(ff_mul(R[2], S[0]), ff_mul(R[0], S[2])),
                     ff_sub(ff_mul(R[0], S[1]), ff_mul(R[1], S[0]))};
    for (int a = 0; a < 3; ++a) w[a] = ff_mul(x[a], sc);
}

__device__ __forceinline__ void ff_law(const CellFF *cp, const float gq[3], const ff fq[3], ff f4pi, ff acc[3])
{
    const float4 *c4 = reinterpret_cast<const float4 *>(cp);
    const float4 A = __ldg(c4), B = __ldg(c4 + 1), Cc = __ldg(c4 + 2), D = __ldg(c4 + 3);
    // A = (g0, g1, g2, fh0)  B = (fh1, fh2, fl0, fl1)  Cc = (fl2, qh0, qh1, qh2)  D = (ql0, ql1, ql2, -)
    const float gc[3] = {A.x, A.y, A.z};
    const ff fc[3] = {ff{A.w, B.z}, ff{B.x, B.w}, ff{B.y, Cc.x}};
    const ff q[3] = {ff{Cc.y, D.x}, ff{Cc.z, D.y}, ff{Cc.w, D.z}};
    ff R[3], P[3];
    for (int a = 0; a < 3; ++a) {
        // grid parts differ exactly; the rest in double-single
        R[a] = ff_add_f(ff_sub(fc[a], fq[a]), __fsub_rn(gc[a], gq[a]));
        P[a] = ff_add(R[a], q[a]);
    }
    const ff lR2 = ff_add_sloppy(ff_add_sloppy(ff_mul(R[0], R[0]), ff_mul(R[1], R[1])), ff_mul(R[2], R[2]));
    const ff lp2 = ff_add_sloppy(ff_add_sloppy(ff_mul(P[0], P[0]), ff_mul(P[1], P[1])), ff_mul(P[2], P[2]));
    const ff dot = ff_add(ff_add(ff_mul(R[0], P[0]), ff_mul(R[1], P[1])), ff_mul(R[2], P[2]));
    const ff ra = ff_rsqrt(lR2), rb = ff_rsqrt(lp2);
    const ff ab = ff_mul(ra, rb);
    const ff den = ff_add_f(ff_mul(dot, ab), 1.0f);
    const ff sc = ff_mul(ff_mul(ff_mul(f4pi, ff_add_sloppy(ra, rb)), ab), ff_rcp(den));
    const ff w[3] = {ff_sub(ff_mul(R[1], q[2]), ff_mul(R[2], q[1])), ff_sub(ff_mul(R[2], q[0]), ff_mul(R[0], q[2])),
                     ff_sub(ff_mul(R[0], q[1]), ff_mul(R[1], q[0]))};
    for (int a = 0; a < 3; ++a) acc[a] = ff_add_sloppy(acc[a], ff_mul(w[a], sc));
}


// value of a (sum, compensation) pair: Kahan's sum - compensation, or a
// double-single's hi + lo
__device__ __forceinline__ double acc_value(float s, float c, bool dd)
{
    return dd ? (double)s + (double)c : (double)s - (double)c;
}

struct MixedAcc {
    float s0, s1, s2, c0, c1, c2;   // Kahan sums over every query point
    unsigned nvis, nacc, nstep, nfb, nnear;
};

// One query point (g + f split, image j; j < 0 the node itself) for the 32
// lanes of a warp.  Near-field leaves are appended to the lane's list
// (cell, image) and evaluated in FP64 after all query points.
template <bool DD>
__device__ __forceinline__ void bh_query32(const VelArgs &a, const float g[3], const float f[3], const double p[3],
                                           int j, bool part, int root, int ncell, MixedAcc &m, int *near_list,
                                           int &nnear,
                                           double w64[3], bool &overflow, const float *gqq = nullptr,
                                           const ff *qff = nullptr)
// near_list: this lane's column of a shared [kNearCap][32] array, stride 32.
// DD: accepted interactions in double-single at the query point qff, summed
// into (m.s, m.c) as (hi, lo) pairs; the near field needs no FP64 then.
{
    const float near2 = a.near2f;
    const float f4pi = a.f4pif;
    const float d2lo = 1e-16f * (1.0f - 1e-5f), d2hi = 1e-16f * (1.0f + 1e-5f);
    int c = root;
    int resume = part ? 0 : 0x7fffffff;
    const int guard_max = 4 * (ncell - root) + 64;
    int steps = 0;
    // plain FP32 sub-sums, folded into the Kahan sums every 16 warp steps
    float p0 = 0, p1 = 0, p2 = 0;
    const float2 ng01 = make_float2(-g[0], -g[1]), nf01 = make_float2(-f[0], -f[1]);
    // c only grows (nxt > c is checked), so it stays within [root, ncell)
    while (c < ncell) {
        const float4 *cp4 = reinterpret_cast<const float4 *>(a.cells32 + c);
        float4 A = __ldg(cp4), B = __ldg(cp4 + 1), Cc = __ldg(cp4 + 2);
        // A = (gx, gy, gz, thr)  B = (fx, fy, fz, next)  Cc = (qx, qy, qz, lm)
        int nxt = __float_as_int(B.w);
        if ((unsigned)(nxt - c - 1) >= (unsigned)(ncell - c)) { bad_index(a, 2, c); nxt = ncell; }
        bool open = false;
        if (c >= resume) {
            ++m.nvis;
            // x and y two-wide as R = (A - g) + (B - f), the separation's
            // negation bit for bit (round-to-nearest is symmetric)
            const float2 Rxy = __fadd2_rn(__fadd2_rn(make_float2(A.x, A.y), ng01), __fadd2_rn(make_float2(B.x, B.y), nf01));
            const float dx = -Rxy.x, dy = -Rxy.y;
            const float dz = (g[2] - A.z) + (f[2] - B.z);
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const bool leaf = (nxt == c + 1);
            // decisions taken in FP32 only when clear of their thresholds
            bool skip = d2 < d2lo;
            bool acc = !skip && (leaf || d2 > A.w);
            bool opn = !skip && !leaf && d2 < A.w * kThrLo;
            bool exact = (!skip && d2 <= d2hi) || (!skip && !acc && !opn);
            if (exact) {
                // rare: inside a guard band, decided exactly as the FP64 path
                ++m.nfb;
                double q[3], dxyz[3], d64;
                if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
                else image_point(a.geo, j, p, q);
                int dec = decide64(a, a.cells + c, q, a.prm.theta, leaf, dxyz, &d64);
                skip = dec == 1;
                acc = dec == 2;
            }
            if (acc) {
                ++m.nacc;
                const float R0 = -dx, R1 = -dy, R2 = -dz;
                const float qx = Cc.x, qy = Cc.y, qz = Cc.z;
                const float P0 = R0 + qx, P1 = R1 + qy, P2 = R2 + qz;
                const float lp2 = fmaf(P0, P0, fmaf(P1, P1, P2 * P2));
                const float dot = fmaf(R0, P0, fmaf(R1, P1, R2 * P2));
                const float ra = rsqrtf(d2), rb = rsqrtf(lp2);
                const float ab = ra * rb;
                const float nd = dot * ab;
                // the common case in one test: no deferral, the filter passing clear of its band
                bool defer = false, keep = true;
                if (exact || (!DD && leaf && d2 < near2) || lp2 < d2hi || !(nd > 1e-8f + 4e-6f)) {
                    defer = exact || (!DD && leaf && d2 < near2) || lp2 < d2hi || fabsf(nd - 1e-8f) < 4e-6f;
                    keep = nd >= 1e-8f;
                }
                if (defer) {
                    // near field, or a filter inside its guard band: FP64, after the traversal
                    ++m.nnear;
                    if (nnear < kNearCap) {
                        near_list[32 * nnear] = (c << 5) | (j + 1);
                        ++nnear;
                    } else {
                        double q[3], dxyz[3], d64, w[3];
                        if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
                        else image_point(a.geo, j, p, q);
                        decide64(a, a.cells + c, q, a.prm.theta, true, dxyz, &d64);
                        if (interact64(a.cells + c, dxyz, d64, a.f4pi, w)) {
                            w64[0] += w[0]; w64[1] += w[1]; w64[2] += w[2];
                        }
                    }
                } else if (keep) {
                    if (DD) {
                        ff acc[3] = {ff{m.s0, m.c0}, ff{m.s1, m.c1}, ff{m.s2, m.c2}};
                        ff_law(a.cellsff + c, gqq, qff, ff{a.f4pi_h, a.f4pi_l}, acc);
                        m.s0 = acc[0].hi; m.c0 = acc[0].lo;
                        m.s1 = acc[1].hi; m.c1 = acc[1].lo;
                        m.s2 = acc[2].hi; m.c2 = acc[2].lo;
                    } else {
                        const float sc = __fdividef(f4pi * (ra + rb) * ab, fmaf(dot, ab, 1.0f));
                        // R x Rp1 = R x q
                        p0 = fmaf(fmaf(R1, qz, -R2 * qy), sc, p0);
                        p1 = fmaf(fmaf(R2, qx, -R0 * qz), sc, p1);
                        p2 = fmaf(fmaf(R0, qy, -R1 * qx), sc, p2);
                    }
                }
                resume = nxt;
            } else if (skip) {
                resume = nxt;
            } else {
                open = true;
            }
        }
        ++steps;
        if ((steps & 15) == 0) {   // warp-uniform
            if (!DD) {
                kahan_add(m.s0, m.c0, p0);
                kahan_add(m.s1, m.c1, p1);
                kahan_add(m.s2, m.c2, p2);
                p0 = p1 = p2 = 0;
            }
            if (steps > guard_max) { overflow = true; break; }
        }
        c = __any_sync(0xffffffffu, open) ? c + 1 : nxt;
    }
    if (!DD) {
        kahan_add(m.s0, m.c0, p0);
        kahan_add(m.s1, m.c1, p1);
        kahan_add(m.s2, m.c2, p2);
    }
    m.nstep += steps;
}

template <int W, int HI, bool DD>
__global__ void __launch_bounds__(32 * W, (min_blocks_mixed<W, HI>())) k_vel_mixed(VelArgs a,
                                                                                  double *__restrict__ part_out)
{
    const int lane = threadIdx.x & 31;
    const int tiles = a.counters[TC_ITEMS];
    const int items = tiles * a.G;
    __shared__ int s_near[W][kNearCap * 32];   // per warp: [entry][lane]
    int *near_list = &s_near[threadIdx.x >> 5][lane];
    unsigned visits = 0, accepts = 0, steps = 0, fallback = 0, near64 = 0;   // per lane
    bool overflow = false;
    for (int it = next_item(a); it < items; it = next_item(a)) {
        const WorkItem w = decode_item(a, it, tiles);
        const int loc = 32 * w.tile + lane;
        const int tix = w.st + loc;
        bool valid = loc < w.nne && tix < a.cap;
        int id = valid ? a.order[tix] : 0;
        if (valid && (id < 0 || id >= a.cap)) { bad_index(a, 4, id); valid = false; id = 0; }
        const int st = valid ? a.status[id] : OV_EMPTY;
        const bool part = valid && st != OV_PINNED && st != OV_EMPTY && a.prm.use_bh;
        double p[3] = {0, 0, 0};
        if (valid) { p[0] = a.x[id]; p[1] = a.y[id]; p[2] = a.z[id]; }
        float g0[3], f0[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            double G = rint(p[ax] * a.inv_h) * a.grid_h;
            g0[ax] = (float)G;
            f0[ax] = (float)(p[ax] - G);
        }
        MixedAcc m = {0, 0, 0, 0, 0, 0, 0u, 0u, 0u, 0u, 0u};
        double w64[3] = {0, 0, 0};        // FP64 sums: near field and list overflow
        double img64[3] = {0, 0, 0};      // images with mirror reflections
        int nnear = 0;
        for (int qi = w.grp; qi <= a.geo.n_img; qi += a.G) {
            const int j = qi - 1;
            float g[3], f[3];
            if (j < 0) {
                for (int ax = 0; ax < 3; ++ax) { g[ax] = g0[ax]; f[ax] = f0[ax]; }
            } else {
                // image query p - L*shift: grid parts subtract exactly
                for (int ax = 0; ax < 3; ++ax) {
                    g[ax] = g0[ax] - a.shift_g[j][ax];
                    f[ax] = f0[ax] - a.shift_f[j][ax];
                }
            }
            if (j >= 0 && a.geo.nreflect[j] > 0) {
                // mirror images (wall geometries): the reflected query point split
                // on the grid, its own sums, reflected before they join the rest
                double q[3];
                image_point(a.geo, j, p, q);
                for (int ax = 0; ax < 3; ++ax) {
                    double G = rint(q[ax] * a.inv_h) * a.grid_h;
                    g[ax] = (float)G;
                    f[ax] = (float)(q[ax] - G);
                }
                MixedAcc mr = {0, 0, 0, 0, 0, 0, 0u, 0u, 0u, 0u, 0u};
                double wr[3] = {0, 0, 0};   // FP64 terms of this image when the near list is full
                ff qr[3];
                for (int ax = 0; ax < 3; ++ax) qr[ax] = ff_from(q[ax] - rint(q[ax] * a.inv_h) * a.grid_h);
                bh_query32<DD>(a, g, f, p, j, part, w.root, w.end, mr, near_list, nnear, wr, overflow, g, qr);
                double v[3] = {acc_value(mr.s0, mr.c0, DD) + wr[0], acc_value(mr.s1, mr.c1, DD) + wr[1],
                               acc_value(mr.s2, mr.c2, DD) + wr[2]};
                for (int r = 0; r < a.geo.nreflect[j]; ++r) mirror_vec(a.geo.reflect[j][r], v);
                img64[0] += v[0]; img64[1] += v[1]; img64[2] += v[2];
                m.nvis += mr.nvis; m.nacc += mr.nacc; m.nstep += mr.nstep; m.nfb += mr.nfb; m.nnear += mr.nnear;
                continue;
            }
            if (DD) {
                // the query point split as the cells are: the grid part exact, the rest
                // (exact in FP64) in double-single
                double q[3];
                if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
                else image_point(a.geo, j, p, q);
                float gq[3];
                ff qf[3];
                for (int ax = 0; ax < 3; ++ax) {
                    const double G = rint(q[ax] * a.inv_h) * a.grid_h;
                    gq[ax] = (float)G;
                    qf[ax] = ff_from(q[ax] - G);
                }
                bh_query32<DD>(a, g, f, p, j, part, w.root, w.end, m, near_list, nnear, w64, overflow, gq, qf);
            } else {
                bh_query32<DD>(a, g, f, p, j, part, w.root, w.end, m, near_list, nnear, w64, overflow);
            }
        }
        // deferred near-field interactions, all lanes together
        for (int i = 0; i < nnear && i < kNearCap; ++i) {
            int e = near_list[32 * i];
            int c = e >> 5, j = (e & 31) - 1;
            if (c < w.root || c >= w.end || j < -1 || j >= a.geo.n_img) { bad_index(a, 3, e); continue; }
            double q[3], wv[3];
            if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
            else image_point(a.geo, j, p, q);
            law64_term(a.cells + c, q, wv);   // zero when a filter drops it
            if (j >= 0)   // a mirror image's term is reflected back
                for (int r = 0; r < a.geo.nreflect[j]; ++r) mirror_vec(a.geo.reflect[j][r], wv);
            w64[0] += wv[0] * a.f4pi; w64[1] += wv[1] * a.f4pi; w64[2] += wv[2] * a.f4pi;
        }
        __syncwarp();   // the list is rewritten by the next item
        double bh[3] = {acc_value(m.s0, m.c0, DD) + w64[0] + img64[0],
                        acc_value(m.s1, m.c1, DD) + w64[1] + img64[1],
                        acc_value(m.s2, m.c2, DD) + w64[2] + img64[2]};
        if (valid) {
            const size_t cap = (size_t)a.cap;
            for (int ax = 0; ax < 3; ++ax) {
                part_out[((size_t)(2 * w.grp) * 3 + ax) * cap + tix] = bh[ax];
                part_out[((size_t)(2 * w.grp + 1) * 3 + ax) * cap + tix] = 0.0;
            }
        }
        count_node(a, valid, id, m.nvis, m.nacc);
        visits += m.nvis;
        accepts += m.nacc;
        steps += m.nstep;
        fallback += m.nfb;
        near64 += m.nnear;
    }
    int err = overflow ? OV_EW_ITER : 0;
    unsigned long long v64 = visits, a64 = accepts, f64 = fallback, n64 = near64;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v64 += __shfl_xor_sync(0xffffffffu, v64, o);
        a64 += __shfl_xor_sync(0xffffffffu, a64, o);
        f64 += __shfl_xor_sync(0xffffffffu, f64, o);
        n64 += __shfl_xor_sync(0xffffffffu, n64, o);
        err |= __shfl_xor_sync(0xffffffffu, err, o);
    }
    if (lane == 0) {
        atomicAdd(&a.stat[ST_VISITS], v64);
        atomicAdd(&a.stat[ST_ACCEPTS], a64);
        atomicAdd(&a.stat[ST_STEPS], (unsigned long long)steps);
        atomicAdd(&a.stat[ST_FALLBACK], f64);
        atomicAdd(&a.stat[ST_NEAR64], n64);
        if (err) atomicOr((int *)&a.counters[TC_ERR], err);
    }
}

// --------------------------------------- mixed precision, periodic images
// k_vel_mixed for periodic image sets, with fewer values held per lane: no
// mirror-image sums, the node's FP64 position re-read in the rare FP64
// paths instead of kept, those paths out of line, and the circulation of a
// cell read only when some lane accepts it.  Same decisions, arithmetic and
// summation order as k_vel_mixed; the register budget is a template
// parameter (more resident warps against spills), picked by the autotuner.

// (the rare paths are kept out of line: their FP64 temporaries would
// otherwise raise the register count of the walk loop)
__device__ __noinline__ void mixp_term64(const VelArgs &a, int c, int j, int id, double w64[3])
{
    double p[3] = {a.x[id], a.y[id], a.z[id]}, q[3], dxyz[3], d64, w[3];
    if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
    else image_point(a.geo, j, p, q);
    decide64(a, a.cells + c, q, a.prm.theta, true, dxyz, &d64);
    if (interact64(a.cells + c, dxyz, d64, a.f4pi, w)) {
        w64[0] += w[0]; w64[1] += w[1]; w64[2] += w[2];
    }
}

// The FP64 path's decision for cell c at node id's query point j: 1 skip,
// 2 accept, 0 open.
__device__ __noinline__ int mixp_decide64(const VelArgs &a, int c, int j, int id, bool leaf)
{
    double p[3] = {a.x[id], a.y[id], a.z[id]}, q[3], dxyz[3], d64;
    if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
    else image_point(a.geo, j, p, q);
    return decide64(a, a.cells + c, q, a.prm.theta, leaf, dxyz, &d64);
}

// An accepted cell whose term needs FP64 (near field, a decision or filter
// taken in FP64): deferred to after the walk, or evaluated now when the
// lane's deferred list is full.
__device__ __forceinline__ void mixp_defer(const VelArgs &a, MixedAcc &m, int *near_list, int &nnear, int c, int j,
                                           int id, double w64[3])
{
    ++m.nnear;
    if (nnear < kNearCap) {
        near_list[32 * nnear] = (c << 5) | (j + 1);
        ++nnear;
        return;
    }
    mixp_term64(a, c, j, id, w64);
}

// One periodic query point (g + f split; image j, j < 0 the node itself) for
// the 32 lanes of a warp.
__device__ __forceinline__ void walk_mixp(const VelArgs &a, const float g[3], const float f[3], int id, int j,
                                          bool part, int root, int ncell, MixedAcc &m, int *near_list, int &nnear,
                                          double w64[3], bool &overflow)
{
    const float near2 = a.near2f;
    const float f4pi = a.f4pif;
    const float d2lo = 1e-16f * (1.0f - 1e-5f), d2hi = 1e-16f * (1.0f + 1e-5f);
    int c = root;
    int resume = part ? 0 : 0x7fffffff;
    const int guard_max = 4 * (ncell - root) + 64;
    int steps = 0;
    // plain FP32 sub-sums, folded into the Kahan sums every 16 warp steps
    float p0 = 0, p1 = 0, p2 = 0;
    const float2 ng01 = make_float2(-g[0], -g[1]), nf01 = make_float2(-f[0], -f[1]);
    // c only grows (nxt > c is checked), so it stays within [root, ncell)
    while (c < ncell) {
        const float4 *cp4 = reinterpret_cast<const float4 *>(a.cells32 + c);
        const float4 A = __ldg(cp4), B = __ldg(cp4 + 1);
        // A = (gx, gy, gz, thr)  B = (fx, fy, fz, next)
        int nxt = __float_as_int(B.w);
        if ((unsigned)(nxt - c - 1) >= (unsigned)(ncell - c)) { bad_index(a, 2, c); nxt = ncell; }
        bool open = false;
        if (c >= resume) {
            ++m.nvis;
            // x and y two-wide as R = (A - g) + (B - f), the separation's
            // negation bit for bit (round-to-nearest is symmetric)
            const float2 Rxy = __fadd2_rn(__fadd2_rn(make_float2(A.x, A.y), ng01), __fadd2_rn(make_float2(B.x, B.y), nf01));
            const float dx = -Rxy.x, dy = -Rxy.y;
            const float dz = (g[2] - A.z) + (f[2] - B.z);
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const bool leaf = (nxt == c + 1);
            // decisions in FP32 clear of their thresholds, else as the FP64 path
            bool skip = d2 < d2lo;
            bool acc = !skip && (leaf || d2 > A.w);
            bool opn = !skip && !leaf && d2 < A.w * kThrLo;
            const bool exact = (!skip && d2 <= d2hi) || (!skip && !acc && !opn);
            if (exact) {
                ++m.nfb;
                const int dec = mixp_decide64(a, c, j, id, leaf);
                skip = dec == 1;
                acc = dec == 2;
            }
            if (acc) {
                ++m.nacc;
                if (exact || (leaf && d2 < near2)) {
                    mixp_defer(a, m, near_list, nnear, c, j, id, w64);
                } else {
                    const float4 Q = __ldg(cp4 + 2);   // (qx, qy, qz, lm)
                    const float R0 = -dx, R1 = -dy, R2 = -dz;
                    const float P0 = R0 + Q.x, P1 = R1 + Q.y, P2 = R2 + Q.z;
                    const float lp2 = fmaf(P0, P0, fmaf(P1, P1, P2 * P2));
                    const float dot = fmaf(R0, P0, fmaf(R1, P1, R2 * P2));
                    const float ra = rsqrtf(d2), rb = rsqrtf(lp2);
                    const float ab = ra * rb;
                    const float nd = dot * ab;
                    if (lp2 < d2hi || !(nd > 1e-8f + 4e-6f)) {
                        // a filter near its threshold: FP64; clearly below ndot's: dropped
                        if (lp2 < d2hi || fabsf(nd - 1e-8f) < 4e-6f) mixp_defer(a, m, near_list, nnear, c, j, id, w64);
                    } else {
                        const float sc = __fdividef(f4pi * (ra + rb) * ab, fmaf(dot, ab, 1.0f));
                        // R x Rp1 = R x q
                        p0 = fmaf(fmaf(R1, Q.z, -R2 * Q.y), sc, p0);
                        p1 = fmaf(fmaf(R2, Q.x, -R0 * Q.z), sc, p1);
                        p2 = fmaf(fmaf(R0, Q.y, -R1 * Q.x), sc, p2);
                    }
                }
                resume = nxt;
            } else if (skip) {
                resume = nxt;
            } else {
                open = true;
            }
        }
        ++steps;
        if ((steps & 15) == 0) {   // warp-uniform
            kahan_add(m.s0, m.c0, p0);
            kahan_add(m.s1, m.c1, p1);
            kahan_add(m.s2, m.c2, p2);
            p0 = p1 = p2 = 0;
            if (steps > guard_max) { overflow = true; break; }
        }
        c = __any_sync(0xffffffffu, open) ? c + 1 : nxt;
    }
    kahan_add(m.s0, m.c0, p0);
    kahan_add(m.s1, m.c1, p1);
    kahan_add(m.s2, m.c2, p2);
    m.nstep += steps;
}

// register budget: R = 0 the compiler's choice, else R registers a thread
template <int W, int R> constexpr int min_blocks_mixp() { return R == 0 ? 1 : 65536 / (32 * W * R); }

template <int W, int R>
__global__ void __launch_bounds__(32 * W, (min_blocks_mixp<W, R>())) k_vel_mixp(VelArgs a,
                                                                              double *__restrict__ part_out)
{
    const int lane = threadIdx.x & 31;
    const int tiles = a.counters[TC_ITEMS];
    const int items = tiles * a.G;
    __shared__ int s_near[W][kNearCap * 32];   // per warp: [entry][lane]
    int *near_list = &s_near[threadIdx.x >> 5][lane];
    unsigned visits = 0, accepts = 0, steps = 0, fallback = 0, near64 = 0;   // per lane
    bool overflow = false;
    for (int it = next_item(a); it < items; it = next_item(a)) {
        const WorkItem w = decode_item(a, it, tiles);
        const int loc = 32 * w.tile + lane;
        const int tix = w.st + loc;
        bool valid = loc < w.nne && tix < a.cap;
        int id = valid ? a.order[tix] : 0;
        if (valid && (id < 0 || id >= a.cap)) { bad_index(a, 4, id); valid = false; id = 0; }
        const int st = valid ? a.status[id] : OV_EMPTY;
        const bool part = valid && st != OV_PINNED && st != OV_EMPTY && a.prm.use_bh;
        float g0[3], f0[3];
        {
            double p[3] = {0, 0, 0};
            if (valid) { p[0] = a.x[id]; p[1] = a.y[id]; p[2] = a.z[id]; }
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                const double G = rint(p[ax] * a.inv_h) * a.grid_h;
                g0[ax] = (float)G;
                f0[ax] = (float)(p[ax] - G);
            }
        }
        MixedAcc m = {0, 0, 0, 0, 0, 0, 0u, 0u, 0u, 0u, 0u};
        double w64[3] = {0, 0, 0};        // FP64 terms: near field and deferred-list overflow
        int nnear = 0;
        for (int qi = w.grp; qi <= a.geo.n_img; qi += a.G) {
            const int j = qi - 1;
            float g[3], f[3];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                // image query p - L*shift: grid parts subtract exactly
                g[ax] = j < 0 ? g0[ax] : g0[ax] - a.shift_g[j][ax];
                f[ax] = j < 0 ? f0[ax] : f0[ax] - a.shift_f[j][ax];
            }
            walk_mixp(a, g, f, id, j, part, w.root, w.end, m, near_list, nnear, w64, overflow);
        }
        // deferred FP64 terms, all lanes together
        {
            double p[3] = {0, 0, 0};
            if (valid) { p[0] = a.x[id]; p[1] = a.y[id]; p[2] = a.z[id]; }
            for (int i = 0; i < nnear && i < kNearCap; ++i) {
                const int e = near_list[32 * i];
                const int c = e >> 5, j = (e & 31) - 1;
                if (c < w.root || c >= w.end || j < -1 || j >= a.geo.n_img) { bad_index(a, 3, e); continue; }
                double q[3], wv[3];
                if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
                else image_point(a.geo, j, p, q);
                law64_term(a.cells + c, q, wv);   // zero when a filter drops it
                w64[0] += wv[0] * a.f4pi; w64[1] += wv[1] * a.f4pi; w64[2] += wv[2] * a.f4pi;
            }
        }
        __syncwarp();   // the list is rewritten by the next item
        if (valid) {
            const size_t cap = (size_t)a.cap;
            const double bh[3] = {acc_value(m.s0, m.c0, false) + w64[0], acc_value(m.s1, m.c1, false) + w64[1],
                                  acc_value(m.s2, m.c2, false) + w64[2]};
            for (int ax = 0; ax < 3; ++ax) {
                part_out[((size_t)(2 * w.grp) * 3 + ax) * cap + tix] = bh[ax];
                part_out[((size_t)(2 * w.grp + 1) * 3 + ax) * cap + tix] = 0.0;
            }
        }
        count_node(a, valid, id, m.nvis, m.nacc);
        visits += m.nvis;
        accepts += m.nacc;
        steps += m.nstep;
        fallback += m.nfb;
        near64 += m.nnear;
    }
    int err = overflow ? OV_EW_ITER : 0;
    unsigned long long v64 = visits, a64 = accepts, f64 = fallback, n64 = near64;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v64 += __shfl_xor_sync(0xffffffffu, v64, o);
        a64 += __shfl_xor_sync(0xffffffffu, a64, o);
        f64 += __shfl_xor_sync(0xffffffffu, f64, o);
        n64 += __shfl_xor_sync(0xffffffffu, n64, o);
        err |= __shfl_xor_sync(0xffffffffu, err, o);
    }
    if (lane == 0) {
        atomicAdd(&a.stat[ST_VISITS], v64);
        atomicAdd(&a.stat[ST_ACCEPTS], a64);
        atomicAdd(&a.stat[ST_STEPS], (unsigned long long)steps);
        atomicAdd(&a.stat[ST_FALLBACK], f64);
        atomicAdd(&a.stat[ST_NEAR64], n64);
        if (err) atomicOr((int *)&a.counters[TC_ERR], err);
    }
}

// ------------------------------------------- FP64 path, split walk (default)
// The walk (distance and opening tests) runs in FP32 on the grid-split cells
// exactly as the mixed traversal's, with the FP64 test inside the guard
// bands, so every lane accepts, skips and opens the cells the FP64 walk
// does.  Accepted cells go to the lane's list in shared memory.  When a list
// nears its capacity, and at the end of each query point, the warp
// evaluates all lists together in FP64, 32 entries at a time whoever owns
// them (the owner's query point comes by shuffle), and every owner adds its
// own terms in walk order (the FP64 walk's summation order).  GB300 runs
// FP64 at 1/64 of the FP32 rate: this keeps the FP64 pipe for the
// interactions, in warp instructions with all lanes busy, instead of
// spending it on every visited cell and on idle lanes.

constexpr int kListCap = 64;   // accepted cells per lane between evaluations

// A warp's lists and the scratch of their evaluation (shared memory).
struct WarpLists {
    int entry[kListCap * 32];   // entry i of lane l at [32 i + l]
    unsigned row_mask[kListCap];   // row i: the lanes holding an entry i
    int row_start[kListCap];       // entries in rows before row i
    double w[32][3];               // the terms of one batch of 32 entries
};

// Evaluate the warp's lists (this lane holds n entries) at the lanes' query
// points q and add each lane's terms to its v, in entry order.
__device__ __forceinline__ void flush_lists(const VelArgs &a, WarpLists &L, int lane, int n, const double q[3],
                                            double v[3])
{
    const int nmax = __reduce_max_sync(0xffffffffu, n);
    if (nmax == 0) return;
    // rows, in entry order: row i holds the i-th entry of every lane that has one
    int total = 0;
    for (int i = 0; i < nmax; ++i) {
        const unsigned m = __ballot_sync(0xffffffffu, n > i);
        if (lane == 0) { L.row_mask[i] = m; L.row_start[i] = total; }
        total += __popc(m);
    }
    __syncwarp();
    const unsigned below = (1u << lane) - 1u;
    int own = 0;   // this lane's next entry to add
    for (int base = 0; base < total; base += 32) {
        // entry base + lane: its row (the last one starting at or before it) and owner
        const int k = base + lane;
        int owner = lane, cell = -1;
        if (k < total) {
            int lo = 0, hi = nmax - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (L.row_start[mid] <= k) lo = mid; else hi = mid - 1;
            }
            owner = __fns(L.row_mask[lo], 0, k - L.row_start[lo] + 1);
            cell = L.entry[32 * lo + owner];
        }
        double qo[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) qo[ax] = __shfl_sync(0xffffffffu, q[ax], owner);
        double w[3] = {0.0, 0.0, 0.0};
        if (cell >= 0) law64_term(a.cells + cell, qo, w);
        L.w[lane][0] = w[0]; L.w[lane][1] = w[1]; L.w[lane][2] = w[2];
        __syncwarp();
        // this lane's own entries in the batch, in order
        while (own < n) {
            const int ko = L.row_start[own] + __popc(L.row_mask[own] & below) - base;
            if (ko >= 32) break;
            v[0] += L.w[ko][0]; v[1] += L.w[ko][1]; v[2] += L.w[ko][2];
            ++own;
        }
        __syncwarp();
    }
}

// One query point (split g + f for the tests, q in FP64 for the law) for the
// 32 lanes of a warp; the lane's FP64 velocity in v.
// The split walk's decision for cell c (A, B its first 32 bytes, nxt its
// successor): the mixed traversal's FP32 tests outside their guard bands,
// the FP64 path's (decide64) inside them.  0 open, 1 skip, 2 accept.
__device__ __forceinline__ int split_decision(const VelArgs &a, int c, const float4 &A, const float4 &B, int nxt,
                                              const float g[3], const float f[3], const float2 &ng01,
                                              const float2 &nf01, const double q[3], MixedAcc &m)
{
    const float d2lo = 1e-16f * (1.0f - 1e-5f), d2hi = 1e-16f * (1.0f + 1e-5f);
    // x and y two-wide as (A - g) + (B - f) (ng01, nf01: -g and -f of x, y),
    // the separation's negation bit for bit
    const float2 Rxy = __fadd2_rn(__fadd2_rn(make_float2(A.x, A.y), ng01), __fadd2_rn(make_float2(B.x, B.y), nf01));
    const float dx = -Rxy.x, dy = -Rxy.y;
    const float dz = (g[2] - A.z) + (f[2] - B.z);
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const bool leaf = (nxt == c + 1);
    bool skip = d2 < d2lo;
    bool acc = !skip && (leaf || d2 > A.w);
    const bool opn = !skip && !leaf && d2 < A.w * kThrLo;
    if ((!skip && d2 <= d2hi) || (!skip && !acc && !opn)) {
        ++m.nfb;
        double dxyz[3], d64;
        const int dec = decide64(a, a.cells + c, q, a.prm.theta, leaf, dxyz, &d64);
        skip = dec == 1;
        acc = dec == 2;
    }
    return acc ? 2 : (skip ? 1 : 0);
}

// Where a lane of the full walk from `root` stands when the cursor reaches
// cell b: the walk visits b's ancestors (root down to b's parent) in order,
// and the first of them the lane accepts or skips keeps it out until that
// ancestor's successor (past b); a lane that opens all of them takes part
// from b on.  The decisions are the walk's own (split_decision); nothing is
// counted.
__device__ __forceinline__ int ancestor_resume(const VelArgs &a, int root, int end, int b, const float g[3],
                                               const float f[3], const double q[3])
{
    MixedAcc tmp = {0, 0, 0, 0, 0, 0, 0u, 0u, 0u, 0u, 0u};
    const float2 ng01 = make_float2(-g[0], -g[1]), nf01 = make_float2(-f[0], -f[1]);
    int c = root;
    for (int guard = 0; c < b && guard < 32 * (OV_MAX_LEVEL + 2); ++guard) {
        const float4 *cp4 = reinterpret_cast<const float4 *>(a.cells32 + c);
        const float4 A = __ldg(cp4), B = __ldg(cp4 + 1);
        int nxt = __float_as_int(B.w);
        if (nxt <= c || nxt > end) { bad_index(a, 2, c); return 0x7fffffff; }
        if (split_decision(a, c, A, B, nxt, g, f, ng01, nf01, q, tmp) != 0) return nxt;   // accepted or skipped
        // opened: on to the child holding b
        int ch = c + 1;
        for (int k = 0; k < 8; ++k) {
            const int cn = __float_as_int(__ldg(reinterpret_cast<const float4 *>(a.cells32 + ch) + 1).w);
            if (cn > b || cn <= ch) break;
            ch = cn;
        }
        c = ch;
    }
    if (c != b) { bad_index(a, 3, b); return 0x7fffffff; }
    return 0;
}

// The walk of cells [root, ncell) stops at `stop` (a sub-walk's end; ncell
// otherwise); successors are checked against ncell.  resume0: the lane takes
// part from that cell on (0: from the start; INT_MAX: not at all).
__device__ __forceinline__ void walk_split(const VelArgs &a, const float g[3], const float f[3], const double q[3],
                                           int resume0, int root, int ncell, int stop, WarpLists &L, int lane,
                                           double v[3], MixedAcc &m, bool &overflow)
{
    v[0] = v[1] = v[2] = 0;
    const float2 ng01 = make_float2(-g[0], -g[1]), nf01 = make_float2(-f[0], -f[1]);
    int c = root;
    int resume = resume0;
    const int guard_max = 4 * (ncell - root) + 64;
    int steps = 0, n = 0;
    while (c < stop) {
        if (c < root) { bad_index(a, 1, c); break; }
        const float4 *cp4 = reinterpret_cast<const float4 *>(a.cells32 + c);
        const float4 A = __ldg(cp4), B = __ldg(cp4 + 1);
        // A = (gx, gy, gz, thr)  B = (fx, fy, fz, next)
        int nxt = __float_as_int(B.w);
        if (nxt <= c || nxt > ncell) { bad_index(a, 2, c); nxt = ncell; }
        bool open = false;
        if (c >= resume) {
            ++m.nvis;
            const int dec = split_decision(a, c, A, B, nxt, g, f, ng01, nf01, q, m);
            if (dec == 2) {
                ++m.nacc;
                L.entry[32 * n + lane] = c;
                ++n;
                resume = nxt;
            } else if (dec == 1) {
                resume = nxt;
            } else {
                open = true;
            }
        }
        ++steps;
        // a lane adds at most one entry a step: room for 16 more after this test
        if ((steps & 15) == 0 && __any_sync(0xffffffffu, n > kListCap - 16)) {
            flush_lists(a, L, lane, n, q, v);
            n = 0;
        }
        c = __any_sync(0xffffffffu, open) ? c + 1 : nxt;
        if (steps > guard_max) { overflow = true; break; }
    }
    flush_lists(a, L, lane, n, q, v);
    v[0] *= a.f4pi; v[1] *= a.f4pi; v[2] *= a.f4pi;
    m.nstep += steps;
}

// Resident blocks per SM the register budget is sized for (about 20 warps)
template <int W> constexpr int min_blocks_split() { return W == 2 ? 10 : (W == 4 ? 5 : 2); }

template <int W>
__global__ void __launch_bounds__(32 * W, min_blocks_split<W>()) k_vel_split(VelArgs a, double *__restrict__ part_out)
{
    const int lane = threadIdx.x & 31;
    const int tiles = a.counters[TC_ITEMS];
    const int items = tiles * a.G * a.S;
    __shared__ WarpLists s_lists[W];
    WarpLists &lists = s_lists[threadIdx.x >> 5];
    unsigned long long visits = 0, accepts = 0, steps = 0, fallback = 0;
    bool overflow = false;
    for (int it = next_item(a); it < items; it = next_item(a)) {
        const WorkItem w = decode_item(a, it, tiles);
        const int loc = 32 * w.tile + lane;
        const int tix = w.st + loc;
        bool valid = loc < w.nne && tix < a.cap;
        int id = valid ? a.order[tix] : 0;
        if (valid && (id < 0 || id >= a.cap)) { bad_index(a, 4, id); valid = false; id = 0; }
        const int st = valid ? a.status[id] : OV_EMPTY;
        const bool part = valid && st != OV_PINNED && st != OV_EMPTY && a.prm.use_bh;
        double p[3] = {0, 0, 0};
        if (valid) { p[0] = a.x[id]; p[1] = a.y[id]; p[2] = a.z[id]; }
        float g0[3], f0[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const double G = rint(p[ax] * a.inv_h) * a.grid_h;
            g0[ax] = (float)G;
            f0[ax] = (float)(p[ax] - G);
        }
        MixedAcc m = {0, 0, 0, 0, 0, 0, 0u, 0u, 0u, 0u, 0u};
        double prim[3] = {0, 0, 0}, img[3] = {0, 0, 0};
        for (int qi = w.grp; qi <= a.geo.n_img; qi += a.G) {
            const int j = qi - 1;
            double q[3];
            float g[3], f[3];
            if (j < 0) {
                q[0] = p[0]; q[1] = p[1]; q[2] = p[2];
                for (int ax = 0; ax < 3; ++ax) { g[ax] = g0[ax]; f[ax] = f0[ax]; }
            } else {
                image_point(a.geo, j, p, q);
                if (a.geo.nreflect[j] > 0) {
                    // a mirror image: the reflected point split on the grid
                    for (int ax = 0; ax < 3; ++ax) {
                        const double G = rint(q[ax] * a.inv_h) * a.grid_h;
                        g[ax] = (float)G;
                        f[ax] = (float)(q[ax] - G);
                    }
                } else {
                    // p - L*shift: grid parts subtract exactly
                    for (int ax = 0; ax < 3; ++ax) {
                        g[ax] = g0[ax] - a.shift_g[j][ax];
                        f[ax] = f0[ax] - a.shift_f[j][ax];
                    }
                }
            }
            double v[3];
            int c0 = w.root, c1 = w.end;
            int resume0 = part ? 0 : 0x7fffffff;
            if (a.S > 1) {
                // part w.sub: an equal share of the pre-order cells; the lane's
                // state at its first cell from the walk down its ancestors
                const long long nc = (long long)(w.end - w.root);
                c0 = w.root + (int)(nc * w.sub / a.S);
                c1 = w.root + (int)(nc * (w.sub + 1) / a.S);
                if (part && c0 > w.root && c0 < c1) resume0 = ancestor_resume(a, w.root, w.end, c0, g, f, q);
            }
            walk_split(a, g, f, q, resume0, c0, w.end, c1, lists, lane, v, m, overflow);
            if (j < 0) {
                prim[0] = v[0]; prim[1] = v[1]; prim[2] = v[2];
            } else {
                for (int r = 0; r < a.geo.nreflect[j]; ++r) mirror_vec(a.geo.reflect[j][r], v);
                img[0] = rn_add(img[0], v[0]); img[1] = rn_add(img[1], v[1]); img[2] = rn_add(img[2], v[2]);
            }
        }
        if (valid) {
            const size_t cap = (size_t)a.cap, gs = (size_t)w.grp * a.S + w.sub;
            for (int ax = 0; ax < 3; ++ax) {
                part_out[((2 * gs) * 3 + ax) * cap + tix] = prim[ax];
                part_out[((2 * gs + 1) * 3 + ax) * cap + tix] = img[ax];
            }
        }
        count_node(a, valid, id, m.nvis, m.nacc);
        visits += m.nvis;
        accepts += m.nacc;
        steps += m.nstep;
        fallback += m.nfb;
    }
    int err = overflow ? OV_EW_ITER : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        visits += __shfl_xor_sync(0xffffffffu, visits, o);
        accepts += __shfl_xor_sync(0xffffffffu, accepts, o);
        fallback += __shfl_xor_sync(0xffffffffu, fallback, o);
        err |= __shfl_xor_sync(0xffffffffu, err, o);
    }
    if (lane == 0) {
        atomicAdd(&a.stat[ST_VISITS], visits);
        atomicAdd(&a.stat[ST_ACCEPTS], accepts);
        atomicAdd(&a.stat[ST_STEPS], steps);
        atomicAdd(&a.stat[ST_FALLBACK], fallback);
        if (err) atomicOr((int *)&a.counters[TC_ERR], err);
    }
}

}  // namespace

// Query groups per node: the tuned value, else enough warps for ~32 per SM
// on small tangles (~96 for the FP64 split walk, whose work items are
// longer: finer items balance the end of the launch).
int ov_query_groups(ov_ctx *c)
{
    int maxg = c->geo.n_img + 1;
    if (c->tune.groups > 0) return std::min(c->tune.groups, std::min(maxg, 27));
    int warps = (c->cap + 31) / 32;
    const bool split = c->precision == OV_PREC_FP64 && c->walk == OV_WALK_SPLIT;
    const int per_sm = split ? 96 : 32, gmax = split ? 9 : 8;
    int G = (per_sm * c->sm_count + warps - 1) / warps;
    G = G < 1 ? 1 : (G > gmax ? gmax : G);
    return std::min(G, maxg);
}

namespace {

VelArgs make_args(ov_ctx *c, const NodeArrays &na, double t, unsigned long long *stat)
{
    VelArgs a;
    a.order = c->tree.torder;
    a.counters = c->tree.counters;
    a.cells = c->tree.cells;
    a.cells32 = c->tree.cells32;
    a.cellsff = c->tree.cellsff;
    a.x = na.x; a.y = na.y; a.z = na.z;
    a.tx = na.tx; a.ty = na.ty; a.tz = na.tz;
    a.nx = na.nx; a.ny = na.ny; a.nz = na.nz;
    a.vx = na.vx; a.vy = na.vy; a.vz = na.vz;
    a.sx = na.sx; a.sy = na.sy; a.sz = na.sz;
    a.fwd = c->fwd; a.rev = c->rev; a.status = c->status; a.pin = c->pin;
    a.geo = c->geo;
    a.prm = ov_dev_params(c->params);
    a.t = t;
    a.t_dev = nullptr;
    a.t_index = 0;
    a.f4pi = c->params.kappa / 4 / M_PI;
    a.grid_h = c->grid_h;
    a.inv_h = c->grid_h > 0 ? 1.0 / c->grid_h : 0;
    double near = 2.0 * c->params.dl_max;
    a.near2 = near * near;
    for (int j = 0; j < c->geo.n_img; ++j)
        for (int ax = 0; ax < 3; ++ax) {
            double sh = c->geo.L[ax] * (double)c->geo.shift[j][ax];
            double G = c->grid_h > 0 ? rint(sh / c->grid_h) * c->grid_h : 0.0;
            a.shift_g[j][ax] = (float)G;
            a.shift_f[j][ax] = (float)(sh - G);
        }
    a.stat = stat;
    a.cap = c->cap;
    const bool ens = c->mem.size() > 1;
    a.tt = c->tree.tt;
    a.qorder = ens ? c->d_qorder : nullptr;
    a.tid = ens ? c->d_tid : nullptr;
    a.tprm = ens ? c->d_tprm : nullptr;
    a.mrange = ens ? c->d_mrange : nullptr;
    a.work = c->tree.counters + TC_WORK;
    a.nt = (int)c->mem.size();
    a.G = ov_query_groups(c);
    a.S = 1;
    a.th2f = (float)(a.prm.theta * a.prm.theta);
    a.near2f = (float)a.near2;
    a.f4pif = (float)a.f4pi;
    a.f4pi_h = (float)a.f4pi;
    a.f4pi_l = (float)(a.f4pi - (double)a.f4pi_h);
    a.node_counts = nullptr;
    a.cell_first = c->geo.sph ? nullptr : c->tree.first;
    a.keys = c->tree.keys;
    a.key_tb = c->key_tbits;
    {
        const Geometry &g = c->geo;
        const double Lx = g.hi[0] - g.lo[0], Ly = g.hi[1] - g.lo[1], Lz = g.hi[2] - g.lo[2];
        a.root_lm = Lx > Ly ? (Lx > Lz ? Lx : Lz) : (Ly > Lz ? Ly : Lz);
        double m = 0;
        for (int x = 0; x < 3; ++x) m = std::max(m, std::max(fabs(g.lo[x]), fabs(g.hi[x])));
        a.lm_ulp = ldexp(m, -44);
    }
    return a;
}

}  // namespace

void ov_launch_tangents(ov_ctx *c, const NodeArrays &na, cudaStream_t s)
{
    VelArgs a = make_args(c, na, 0.0, nullptr);
    k_tangents<<<(c->cap + 255) / 256, 256, 0, s>>>(a, c->cap, c->tree.counters);
    c->launches++;
}

// Parts per query point: the FP64 split walk of a tangle too small to fill
// the GPU with (tile, query group) items splits each walk into equal shares
// of the pre-order cells (32 parts up to 2,048 slots, 8 up to 8,192), so a
// kernel is not as long as its longest walk.
constexpr int kSubWalkSlots = 8192;
static int sub_walks_for(int cap) { return cap <= 2048 ? 32 : (cap <= kSubWalkSlots ? 8 : 1); }
static int ov_sub_walks(const ov_ctx *c, int precision)
{
    return precision == OV_PREC_FP64 && c->walk == OV_WALK_SPLIT ? sub_walks_for(c->cap) : 1;
}

int ov_reserve_velocity_scratch(ov_ctx *c)
{
    int G = ov_query_groups(c);
    size_t need = (size_t)G * sub_walks_for(c->cap) * 6 * (size_t)c->cap;
    if (c->part_cap < need) {
        if (c->part) cudaFree(c->part);
        c->part = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->part, need * sizeof(double)));
        c->part_cap = need;
    }
    return OV_OK;
}

// Traversal kernel for a precision and block shape.
typedef void (*VelKernel)(VelArgs, double *);
static bool has_mirror_images(const Geometry &g)
{
    for (int j = 0; j < g.n_img; ++j)
        if (g.nreflect[j] > 0) return true;
    return false;
}

// variant (Tuning::hi_occ) of the mixed traversal: 0 k_vel_mixed, 1 the
// same under a tighter register budget, 2-4 k_vel_mixp (periodic image sets
// only) with the compiler's register count, 80 and 64 registers
template <int R> static VelKernel mixp_kernel(int warps)
{
    if (warps == 2) return k_vel_mixp<2, R>;
    if (warps == 8) return k_vel_mixp<8, R>;
    return k_vel_mixp<4, R>;
}

static VelKernel vel_kernel(int precision, int walk, int warps, int hi_occ, bool mirror)
{
    if (precision == OV_PREC_MIXED) {
        if (hi_occ >= 2 && !mirror) return hi_occ == 2 ? mixp_kernel<0>(warps)
                                         : (hi_occ == 3 ? mixp_kernel<80>(warps) : mixp_kernel<64>(warps));
        if (hi_occ) {
            if (warps == 2) return k_vel_mixed<2, 1, false>;
            if (warps == 8) return k_vel_mixed<8, 1, false>;
            return k_vel_mixed<4, 1, false>;
        }
        if (warps == 2) return k_vel_mixed<2, 0, false>;
        if (warps == 8) return k_vel_mixed<8, 0, false>;
        return k_vel_mixed<4, 0, false>;
    }
    if (precision == OV_PREC_DD) {
        if (warps == 2) return k_vel_mixed<2, 0, true>;
        if (warps == 8) return k_vel_mixed<8, 0, true>;
        return k_vel_mixed<4, 0, true>;
    }
    if (walk == OV_WALK_SPLIT) {
        if (warps == 2) return k_vel_split<2>;
        if (warps == 8) return k_vel_split<8>;
        return k_vel_split<4>;
    }
    if (warps == 2) return k_vel_fp64<2>;
    if (warps == 8) return k_vel_fp64<8>;
    return k_vel_fp64<4>;
}

// Persistent grid: resident blocks per SM (tuned or the occupancy limit) on
// every SM, but no more blocks than there can be work items.
int ov_traversal_blocks(ov_ctx *c, int precision, int warps, int *per_sm)
{
    VelKernel k = vel_kernel(precision, c->walk, warps, c->tune.hi_occ, has_mirror_images(c->geo));
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 32 * warps, 0) != cudaSuccess || occ < 1) {
        cudaGetLastError();
        occ = 1;
    }
    int bps = c->tune.blocks_per_sm > 0 ? std::min(c->tune.blocks_per_sm, occ) : occ;
    if (per_sm) *per_sm = occ;
    long long items = ((long long)(c->cap + 31) / 32 + (long long)c->mem.size()) * ov_query_groups(c);
    long long need = (items + warps - 1) / warps;
    long long blocks = std::min((long long)bps * c->sm_count, need);
    return (int)std::max(1LL, blocks);
}

int ov_launch_velocities(ov_ctx *c, const NodeArrays &na, double t, int precision, cudaStream_t s)
{
    VelArgs a = make_args(c, na, t, ov_stat_ptr(c));
    a.S = ov_sub_walks(c, precision);
    if (c->time_dev_index >= 0) {
        a.t_dev = c->d_time;
        a.t_index = c->time_dev_index;
    }
    int r = ov_reserve_velocity_scratch(c);
    if (r) return r;
    int warps = c->tune.warps;
    if (warps != 2 && warps != 8) warps = 4;
    int blocks = ov_traversal_blocks(c, precision, warps, nullptr);
    if (c->count_nodes && c->time_dev_index < 0) {
        // per-target counters (not inside the captured RK4 graph)
        const size_t need = 2 * (size_t)c->cap;
        if (c->node_counts_cap < need) {
            if (c->d_node_counts) cudaFree(c->d_node_counts);
            c->d_node_counts = nullptr;
            c->node_counts_cap = 0;
            OV_ALLOC(c, cudaMalloc(&c->d_node_counts, need * sizeof(unsigned)));
            c->node_counts_cap = need;
        }
        OV_CUDA(c, cudaMemsetAsync(c->d_node_counts, 0, need * sizeof(unsigned), s));
        a.node_counts = c->d_node_counts;
    }
    OV_CUDA(c, cudaMemsetAsync(a.work, 0, sizeof(int), s));
    vel_kernel(precision, c->walk, warps, c->tune.hi_occ, has_mirror_images(c->geo))<<<blocks, 32 * warps, 0, s>>>(
        a, c->part);
    if (a.S > 1) {
        const long long threads = 6LL * c->cap * a.G;
        k_part_sum<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(a, c->part);
        c->launches++;
    }
    k_vel_finish<<<(c->cap + 127) / 128, 128, 0, s>>>(a, c->part);
    c->launches += 2;
    return OV_OK;
}

int ov_direct_sum_chunked(ov_ctx *c, const int *nodes, int n, double *d_out_vel, double *d_out_vs, double t);

int ov_direct_sum(ov_ctx *c, const int *nodes, int n, double t, double *vels_out, double *vs_out)
{
    if (n <= 0) return OV_OK;
    if (c->dsum_cap < n) {
        if (c->dsum) cudaFree(c->dsum);
        if (c->dnodes) cudaFree(c->dnodes);
        c->dsum = nullptr; c->dnodes = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->dsum, (size_t)n * 9 * sizeof(double)));
        OV_ALLOC(c, cudaMalloc(&c->dnodes, (size_t)n * sizeof(int)));
        c->dsum_cap = n;
    }
    double *vo = c->dsum + 3 * (size_t)n, *so = c->dsum + 6 * (size_t)n;
    int r = ov_direct_sum_chunked(c, nodes, n, vo, so, t);
    if (r) return r;
    if (vels_out)
        OV_CUDA(c, cudaMemcpyAsync(vels_out, vo, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (vs_out)
        OV_CUDA(c, cudaMemcpyAsync(vs_out, so, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    return OV_OK;
}

__global__ void __launch_bounds__(128) k_query64(VelArgs a, const double *__restrict__ pts, int n,
                                                 double *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp * 32 >= n) return;
    const int i = warp * 32 + lane;
    const bool valid = i < n;
    double q[3] = {0, 0, 0};
    if (valid) { q[0] = pts[3 * i]; q[1] = pts[3 * i + 1]; q[2] = pts[3 * i + 2]; }
    unsigned long long visits = 0, accepts = 0, steps = 0;
    bool overflow = false;
    double v[3];
    bh_query64(a, q, valid, 0, a.counters[TC_NCELL], v, visits, accepts, steps, overflow);
    if (valid) { out[3 * i] = v[0]; out[3 * i + 1] = v[1]; out[3 * i + 2] = v[2]; }
    if (overflow && lane == 0) atomicOr((int *)&a.counters[TC_ERR], OV_EW_ITER);
}

extern "C" int ov_tree_velocity_at(ov_ctx *c, const double *points, int n, double resolution, int rebuild,
                                   double *out)
{
    if (!c || n < 0 || (n > 0 && (!points || !out))) return OV_ERR_ARG;
    if (!c->uploaded) return ov_fail(c, OV_ERR_STATE, "no tangle uploaded");
    if (c->mem.size() > 1) return ov_fail(c, OV_ERR_STATE, "tree queries need a single tangle, not an ensemble");
    cudaSetDevice(c->device);
    if (rebuild || !c->tree_built) {
        OV_CUDA(c, cudaMemsetAsync(c->tree.counters + TC_ERR, 0, (TC_COUNT - TC_ERR) * 4, c->stream));
        int r = ov_tree_build(c, c->node, c->stream);
        if (r) return r;
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
        int need = 0;
        OV_CUDA(c, cudaMemcpy(&need, c->tree.counters + TC_NEED, 4, cudaMemcpyDeviceToHost));
        int err = 0;
        OV_CUDA(c, cudaMemcpy(&err, c->tree.counters + TC_ERR, 4, cudaMemcpyDeviceToHost));
        if (err & OV_EW_CELLS) {
            if ((r = ov_tree_reserve_cells(c, need + need / 4 + 64))) return r;
            if ((r = ov_tree_build(c, c->node, c->stream))) return r;
        }
        c->tree_built = true;
    }
    if (n == 0) return OV_OK;
    if (c->dsum_cap < n) {
        if (c->dsum) cudaFree(c->dsum);
        if (c->dnodes) cudaFree(c->dnodes);
        c->dsum = nullptr; c->dnodes = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->dsum, (size_t)n * 9 * sizeof(double)));
        OV_ALLOC(c, cudaMalloc(&c->dnodes, (size_t)n * sizeof(int)));
        c->dsum_cap = n;
    }
    double *dp = c->dsum, *dout = c->dsum + 3 * (size_t)n;
    OV_CUDA(c, cudaMemcpyAsync(dp, points, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    VelArgs a = make_args(c, c->node, 0.0, nullptr);
    a.prm.theta = resolution;
    int warps = (n + 31) / 32;
    k_query64<<<(warps * 32 + 127) / 128, 128, 0, c->stream>>>(a, dp, n, dout);
    c->launches++;
    OV_CUDA(c, cudaGetLastError());
    OV_CUDA(c, cudaMemcpyAsync(out, dout, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    return OV_OK;
}

// ---------------------------------------- reconnection velocities (reconnect)
//
// reconnect (vortex_dynamics.c:186-288) needs, for every candidate node, the
// direct-sum velocity of update_velocity(k, t, NULL) on the pass's current
// topology.  The sums over the pass's starting topology are computed here in
// one batch, split into (candidate, chunk of segments) blocks:
//   * mixed: segments farther than r_near from the query point in FP32 on
//     the grid-split positions (separations exact to ~1e-7 relative),
//     Kahan-summed per thread, with a rigorous bound on their error; closer
//     segments, and any whose wrap or filter sits near its threshold, in FP64;
//   * FP64: every term in FP64 (for the rare pairs the bound cannot decide).
// Rewiring changes four segments at a time; their contributions to every
// remaining candidate are added on the device after each reconnection.

namespace {

struct RecArgs {
    const double *x, *y, *z;
    const int *fwd;
    const float *sp;          // split positions: gx, gy, gz, fx, fy, fz, each [cap]
    Geometry geo;
    float shift_g[OV_MAX_IMAGES][3], shift_f[OV_MAX_IMAGES][3];
    float Lg[3], Lf[3], hL[3];   // period split on the grid, half period
    float Lfl[3];             // the rest of Lf (Lf + Lfl = L - Lg to double-single precision)
    double inv_h, grid_h;     // the grid step of the split
    double f4pi;
    float f4pif;
    float rnear2;             // squared FP64 radius
    const int *tid;
    const int2 *mrange;
    int nt, cap;
};

// grid split of every position (the mixed traversal's split, step h)
__global__ void k_split(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                        int cap, double h, double inv_h, float *__restrict__ sp)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    const double p[3] = {x[i], y[i], z[i]};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double G = rint(p[a] * inv_h) * h;
        const float fh = (float)(p[a] - G);
        sp[(size_t)a * cap + i] = (float)G;
        sp[(size_t)(3 + a) * cap + i] = fh;
        sp[(size_t)(6 + a) * cap + i] = (float)((p[a] - G) - (double)fh);   // the rest, for double-single
    }
}

__device__ __forceinline__ void member_range(const RecArgs &r, int k, int &lo, int &hi)
{
    lo = 0;
    hi = r.cap;
    if (r.tid && r.mrange) {
        int m = r.tid[k];
        if (m >= 0 && m < r.nt) { lo = r.mrange[m].x; hi = min(r.mrange[m].y, r.cap); }
        else hi = 0;
    }
}

// FP64 term: segment m -> f at image j of node position p (as k_direct)
__device__ __forceinline__ bool rec_term64(const RecArgs &r, int m, int f, int j, const double p[3], double w[3])
{
    double q[3];
    if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
    else image_point(r.geo, j, p, q);
    double s1[3] = {r.x[m], r.y[m], r.z[m]};
    double s2[3] = {r.x[f], r.y[f], r.z[f]};
    pwrap_dev(r.geo, s1, s2);
    double R[3] = {rn_sub(s1[0], q[0]), rn_sub(s1[1], q[1]), rn_sub(s1[2], q[2])};
    double Rp1[3] = {rn_sub(s2[0], q[0]), rn_sub(s2[1], q[1]), rn_sub(s2[2], q[2])};
    return segment_law64(R, Rp1, len3_ref(R[0], R[1], R[2]), r.f4pi, w);
}

// FP64 term without the reference's correctly rounded square roots and
// divisions (for whole-sum FP64 refinements): the filters are decided the
// reference's way when their test values lie near the thresholds.
__device__ __forceinline__ bool rec_term64_fast(const RecArgs &r, int m, int f, int j, const double p[3],
                                                double w[3])
{
    double q[3];
    if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
    else image_point(r.geo, j, p, q);
    double s1[3] = {r.x[m], r.y[m], r.z[m]};
    double s2[3] = {r.x[f], r.y[f], r.z[f]};
    pwrap_dev(r.geo, s1, s2);
    const double R[3] = {s1[0] - q[0], s1[1] - q[1], s1[2] - q[2]};
    const double P[3] = {s2[0] - q[0], s2[1] - q[1], s2[2] - q[2]};
    const double lR2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
    const double lp2 = P[0] * P[0] + P[1] * P[1] + P[2] * P[2];
    if (lR2 < 1.001e-16 || lp2 < 1.001e-16) return rec_term64(r, m, f, j, p, w);   // |R| < 1e-8 filter
    if (lR2 > 1e30 || lp2 > 1e30) return rec_term64(r, m, f, j, p, w);
    const double ra = rsqrt_nr(lR2), rb = rsqrt_nr(lp2), ab = ra * rb;
    const double dotv = R[0] * P[0] + R[1] * P[1] + R[2] * P[2];
    const double nd = dotv * ab;
    if (fabs(nd - 1e-8) < 1e-6) return rec_term64(r, m, f, j, p, w);   // ndot filter near its threshold
    if (nd < 1e-8) return false;
    const double sc = r.f4pi * (ra + rb) * ab * recip_1_2(1.0 + nd);
    w[0] = (R[1] * P[2] - R[2] * P[1]) * sc;
    w[1] = (R[2] * P[0] - R[0] * P[2]) * sc;
    w[2] = (R[0] * P[1] - R[1] * P[0]) * sc;
    return true;
}

constexpr int kRecThreads = 256;
constexpr int kRecVals = 7;   // 3 sums, FP32 magnitude, 3 spare (|FP64 terms|)

template <int MODE, bool MIRROR>
__global__ void __launch_bounds__(kRecThreads, 3) k_rec_sums(RecArgs r, const int *__restrict__ nodes, int n,
                                                          int span, int max_chunks, double *__restrict__ part)
// MODE: 0 FP32 far / FP64 near, 1 all FP64, 2 double-single far / FP64 near.
// MIRROR: the image set has mirror images (their query points in FP64).
{
    constexpr int force64 = MODE;
    // split query points (self, then images): (g, mirror flag), (f, 0), (f's rest, 0)
    __shared__ float4 s_q[OV_MAX_IMAGES + 1][3];
    // FP32 mode: the negated query points in pairs (0,1), (2,3), ... for the
    // two-wide FP32 instructions: -g x, y, z then -f x, y, z of both points
    __shared__ float2 s_qp[(OV_MAX_IMAGES + 2) / 2][6];
    __shared__ double red[kRecVals][kRecThreads];
    const int b = blockIdx.x, chunk = blockIdx.y;
    if (b >= n) return;
    const int k = nodes[b];
    int lo, hi;
    member_range(r, k, lo, hi);
    const int m0 = lo + chunk * span, m1 = min(hi, m0 + span);
    double *out = part + ((size_t)b * max_chunks + chunk) * kRecVals;
    if (m0 >= m1 || k < 0 || k >= r.cap) {
        if (threadIdx.x < kRecVals) out[threadIdx.x] = 0.0;
        return;
    }
    const double p[3] = {r.x[k], r.y[k], r.z[k]};
    const int nq = r.geo.n_img + 1;
    if (threadIdx.x < nq) {
        const int j = (int)threadIdx.x - 1;
        float g[3], f[3], fl[3] = {0, 0, 0};
        if (MODE == 2) {
            // double-single: the query point in FP64, split on the grid exactly
            double q[3];
            if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
            else image_point(r.geo, j, p, q);
            for (int a = 0; a < 3; ++a) {
                const double G = rint(q[a] * r.inv_h) * r.grid_h;
                g[a] = (float)G;
                f[a] = (float)(q[a] - G);
                fl[a] = (float)((q[a] - G) - (double)f[a]);
            }
        } else {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                g[a] = r.sp[(size_t)a * r.cap + k];
                f[a] = r.sp[(size_t)(3 + a) * r.cap + k];
                if (j >= 0) { g[a] -= r.shift_g[j][a]; f[a] -= r.shift_f[j][a]; }
            }
        }
        // mirror images (reflected query points): FP64 unless double-single
        const float mirror = (force64 != 2 && j >= 0 && r.geo.nreflect[j] > 0) ? 1.0f : 0.0f;
        s_q[threadIdx.x][0] = make_float4(g[0], g[1], g[2], mirror);
        s_q[threadIdx.x][1] = make_float4(f[0], f[1], f[2], 0.0f);
        s_q[threadIdx.x][2] = make_float4(fl[0], fl[1], fl[2], 0.0f);
        float *pr = reinterpret_cast<float *>(&s_qp[threadIdx.x >> 1][0]) + (threadIdx.x & 1);
        for (int a = 0; a < 3; ++a) {
            pr[2 * a] = -g[a];
            pr[2 * (3 + a)] = -f[a];
        }
    }
    __syncthreads();
    float s0 = 0, s1 = 0, s2 = 0, c0 = 0, c1 = 0, c2 = 0, mag = 0;
    double d0 = 0, d1 = 0, d2 = 0, dabs = 0;
    ff dd[3] = {ff{0, 0}, ff{0, 0}, ff{0, 0}};   // double-single terms (mode 2)
    float magdd = 0;
    const ff f4pi_ff = ff{r.f4pif, (float)(r.f4pi - (double)r.f4pif)};
    const float eps_band = 1e-3f;
    for (int m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
        const int f = r.fwd[m];
        if (f < 0 || f >= r.cap) continue;
        float ag[3], af[3], sv[3];
        ff fa[3], S[3];   // mode 2: the start's rest and the segment vector in double-single
        bool seg64 = force64 == 1;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            ag[a] = r.sp[(size_t)a * r.cap + m];
            af[a] = r.sp[(size_t)(3 + a) * r.cap + m];
            float bg = r.sp[(size_t)a * r.cap + f], bf = r.sp[(size_t)(3 + a) * r.cap + f];
            float d = (bg - ag[a]) + (bf - af[a]);
            int ws = 0;
            if (r.geo.periodic[a]) {
                // seg_pwrap: the end moved by a period toward the start
                if (fabsf(fabsf(d) - r.hL[a]) < eps_band * r.hL[a]) seg64 = true;
                if (d > r.hL[a]) { bg -= r.Lg[a]; bf -= r.Lf[a]; ws = -1; }
                else if (d < -r.hL[a]) { bg += r.Lg[a]; bf += r.Lf[a]; ws = 1; }
                if (fabsf(d) > 3.0f * r.hL[a]) seg64 = true;   // more than one period: FP64 loop
            }
            sv[a] = (bg - ag[a]) + (bf - af[a]);
            if (MODE == 2) {
                fa[a] = ff{af[a], r.sp[(size_t)(6 + a) * r.cap + m]};
                ff fb = ff{r.sp[(size_t)(3 + a) * r.cap + f], r.sp[(size_t)(6 + a) * r.cap + f]};
                if (ws) fb = ff_add(fb, ff{ws * r.Lf[a], ws * r.Lfl[a]});
                S[a] = ff_add_f(ff_sub(fb, fa[a]), __fsub_rn(bg, ag[a]));   // grid parts exact (wrapped bg)
            }
        }
        const float slen = sqrtf(fmaf(sv[0], sv[0], fmaf(sv[1], sv[1], sv[2] * sv[2])));
        const bool own = (m == k || f == k);   // the node's own segments: skipped at the primary point
        float t0 = 0, t1 = 0, t2 = 0;   // this segment's terms over the query points
        float ms = 0;                   // sum over the query points of sc |R|
        unsigned mask64 = 0;            // query points whose term is done in FP64
        int qstart = own ? 1 : 0;
        if (MODE == 0 && !own && !seg64) {
            // query points two at a time on the two-wide FP32 pipe (each
            // element rounds as the one-wide instruction); the terms of even
            // and odd points add in two chains, joined after the loop
            const float2 ag2[3] = {make_float2(ag[0], ag[0]), make_float2(ag[1], ag[1]), make_float2(ag[2], ag[2])};
            const float2 af2[3] = {make_float2(af[0], af[0]), make_float2(af[1], af[1]), make_float2(af[2], af[2])};
            const float2 sv2[3] = {make_float2(sv[0], sv[0]), make_float2(sv[1], sv[1]), make_float2(sv[2], sv[2])};
            const float2 nsv2[3] = {make_float2(-sv[0], -sv[0]), make_float2(-sv[1], -sv[1]),
                                    make_float2(-sv[2], -sv[2])};   // -R2 s1 = R2 (-s1), exactly
            float2 tt0 = make_float2(0.f, 0.f), tt1 = tt0, tt2 = tt0, mm = tt0;
            int qi = 0;
            for (; qi + 1 < nq; qi += 2) {
                const float2 *qp = s_qp[qi >> 1];
                const float2 R0 = __fadd2_rn(__fadd2_rn(ag2[0], qp[0]), __fadd2_rn(af2[0], qp[3]));
                const float2 R1 = __fadd2_rn(__fadd2_rn(ag2[1], qp[1]), __fadd2_rn(af2[1], qp[4]));
                const float2 R2 = __fadd2_rn(__fadd2_rn(ag2[2], qp[2]), __fadd2_rn(af2[2], qp[5]));
                const float2 lR2 = __ffma2_rn(R0, R0, __ffma2_rn(R1, R1, __fmul2_rn(R2, R2)));
                const float2 P0 = __fadd2_rn(R0, sv2[0]), P1 = __fadd2_rn(R1, sv2[1]), P2 = __fadd2_rn(R2, sv2[2]);
                const float2 lp2 = __ffma2_rn(P0, P0, __ffma2_rn(P1, P1, __fmul2_rn(P2, P2)));
                const float2 ra = make_float2(rsqrtf(lR2.x), rsqrtf(lR2.y)), rb = make_float2(rsqrtf(lp2.x), rsqrtf(lp2.y));
                const float2 ab = __fmul2_rn(ra, rb);
                const float2 dot = __ffma2_rn(R0, P0, __ffma2_rn(R1, P1, __fmul2_rn(R2, P2)));
                const float2 nd = __fmul2_rn(dot, ab);
                bool take[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const float l1 = e ? lR2.y : lR2.x, l2 = e ? lp2.y : lp2.x, n1 = e ? nd.y : nd.x;
                    take[e] = true;
                    if (fminf(l1, l2) < r.rnear2 || !(n1 > 1e-8f + 1e-4f) || (MIRROR && s_q[qi + e][0].w != 0.0f)) {
                        take[e] = false;
                        if (l1 < r.rnear2 || l2 < r.rnear2 || (MIRROR && s_q[qi + e][0].w != 0.0f) ||
                            fabsf(n1 - 1e-8f) < 1e-4f)
                            mask64 |= 1u << (qi + e);   // FP64 after the loop
                        // else: the ndot filter drops it (far from its threshold)
                    }
                }
                const float2 num = __fmul2_rn(__fadd2_rn(ra, rb), ab);
                const float2 den = __ffma2_rn(dot, ab, make_float2(1.0f, 1.0f));
                const float2 sc = make_float2(take[0] ? __fdividef(num.x, den.x) : 0.0f,
                                              take[1] ? __fdividef(num.y, den.y) : 0.0f);
                // R x Rp1 = R x s
                const float2 x0 = __ffma2_rn(R1, sv2[2], __fmul2_rn(R2, nsv2[1]));
                const float2 x1 = __ffma2_rn(R2, sv2[0], __fmul2_rn(R0, nsv2[2]));
                const float2 x2 = __ffma2_rn(R0, sv2[1], __fmul2_rn(R1, nsv2[0]));
                tt0 = __ffma2_rn(x0, sc, tt0);
                tt1 = __ffma2_rn(x1, sc, tt1);
                tt2 = __ffma2_rn(x2, sc, tt2);
                // sc |R| (times |s| below: >= |w|); a point left out adds
                // nothing (its 1/|R| may be infinite)
                const float2 ra_in = make_float2(take[0] ? ra.x : 0.0f, take[1] ? ra.y : 0.0f);
                mm = __ffma2_rn(sc, __fmul2_rn(lR2, ra_in), mm);
            }
            t0 = tt0.x + tt0.y;
            t1 = tt1.x + tt1.y;
            t2 = tt2.x + tt2.y;
            ms = mm.x + mm.y;
            qstart = qi;   // an odd last point below
        }
#pragma unroll 3
        for (int qi = qstart; qi < nq; ++qi) {
            const float4 qg = s_q[qi][0], qf = s_q[qi][1];
            const float R0 = (ag[0] - qg.x) + (af[0] - qf.x);
            const float R1 = (ag[1] - qg.y) + (af[1] - qf.y);
            const float R2 = (ag[2] - qg.z) + (af[2] - qf.z);
            const float lR2 = fmaf(R0, R0, fmaf(R1, R1, R2 * R2));
            const float P0 = R0 + sv[0], P1 = R1 + sv[1], P2 = R2 + sv[2];
            const float lp2 = fmaf(P0, P0, fmaf(P1, P1, P2 * P2));
            const float ra = rsqrtf(lR2), rb = rsqrtf(lp2);
            const float ab = ra * rb;
            const float dot = fmaf(R0, P0, fmaf(R1, P1, R2 * P2));
            const float nd = dot * ab;
            // the common case in one test: both ends beyond r_near, the filter
            // clear of its band and passing
            if (seg64 || fminf(lR2, lp2) < r.rnear2 || !(nd > 1e-8f + 1e-4f) || (MIRROR && qg.w != 0.0f)) {
                const bool use64 = seg64 || lR2 < r.rnear2 || lp2 < r.rnear2 || (MIRROR && qg.w != 0.0f) ||
                                   fabsf(nd - 1e-8f) < 1e-4f;   // filter near its threshold
                if (use64) {   // FP64 after the loop over the query points
                    mask64 |= 1u << qi;
                    continue;
                }
                if (nd < 1e-8f) continue;   // ndot filter (far from its threshold here)
            }
            if (MODE == 2) {
                const float4 qfl = s_q[qi][2];
                const float gq[3] = {qg.x, qg.y, qg.z}, fqh[3] = {qf.x, qf.y, qf.z}, fql[3] = {qfl.x, qfl.y, qfl.z};
                ff Rd[3], w[3];
                for (int a = 0; a < 3; ++a) Rd[a] = ff_add_f(ff_sub(fa[a], ff{fqh[a], fql[a]}), __fsub_rn(ag[a], gq[a]));
                ff_segment(Rd, S, f4pi_ff, w);
                for (int a = 0; a < 3; ++a) dd[a] = ff_add(dd[a], w[a]);
                magdd += fabsf(w[0].hi) + fabsf(w[1].hi) + fabsf(w[2].hi);
                continue;
            }
            const float sc = __fdividef((ra + rb) * ab, fmaf(dot, ab, 1.0f));   // kappa / 4 pi: on the sums
            // R x Rp1 = R x s
            t0 = fmaf(fmaf(R1, sv[2], -R2 * sv[1]), sc, t0);
            t1 = fmaf(fmaf(R2, sv[0], -R0 * sv[2]), sc, t1);
            t2 = fmaf(fmaf(R0, sv[1], -R1 * sv[0]), sc, t2);
            ms = fmaf(sc, lR2 * ra, ms);   // sc |R|; times |s| below: >= |w| (per component)
        }
        for (; mask64; mask64 &= mask64 - 1) {
            const int j = __ffs(mask64) - 2;
            double w[3];
            if (force64 == 1 ? rec_term64_fast(r, m, f, j, p, w) : rec_term64(r, m, f, j, p, w)) {
                d0 += w[0]; d1 += w[1]; d2 += w[2];
                dabs += fabs(w[0]) + fabs(w[1]) + fabs(w[2]);
            }
        }
        mag = fmaf(ms, slen, mag);
        kahan_add(s0, c0, t0);
        kahan_add(s1, c1, t1);
        kahan_add(s2, c2, t2);
    }
    // the FP32 terms lack kappa / 4 pi (one more rounding: within the bound's 1.01)
    const double f4 = r.f4pi;
    red[0][threadIdx.x] = ((double)s0 - (double)c0) * f4 + d0 + ((double)dd[0].hi + (double)dd[0].lo);
    red[1][threadIdx.x] = ((double)s1 - (double)c1) * f4 + d1 + ((double)dd[1].hi + (double)dd[1].lo);
    red[2][threadIdx.x] = ((double)s2 - (double)c2) * f4 + d2 + ((double)dd[2].hi + (double)dd[2].lo);
    red[3][threadIdx.x] = (double)mag * f4;
    red[4][threadIdx.x] = dabs;
    red[5][threadIdx.x] = (fabs((double)s0) + fabs((double)s1) + fabs((double)s2)) * f4;
    red[6][threadIdx.x] = (double)magdd;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int v = 0; v < kRecVals; ++v) red[v][threadIdx.x] += red[v][threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x < kRecVals) out[threadIdx.x] = red[threadIdx.x][0];
}

// out[5 b + {0,1,2}] = sums over the chunks in order, out[5 b + 3] = bound on
// each component's error: FP32 terms (per-term rounding, Kahan), FP64 terms
// and the FP64 reductions; out[5 b + 4] = sum of the terms' magnitudes.
__global__ void k_rec_finish(const double *__restrict__ part, int n, int max_chunks, double *__restrict__ out)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    double acc[kRecVals] = {0, 0, 0, 0, 0, 0, 0};
    for (int ch = 0; ch < max_chunks; ++ch)
        for (int v = 0; v < kRecVals; ++v) acc[v] += part[((size_t)b * max_chunks + ch) * kRecVals + v];
    const double eps32 = 5.9604644775390625e-8;
    for (int a = 0; a < 3; ++a) out[5 * (size_t)b + a] = acc[a];
    // double-single terms (acc[6]: their magnitudes): 1e-10 of each covers the
    // law's error (about 1e-13) and their running sums with a wide margin
    out[5 * (size_t)b + 3] = 1.01 * ((64.0 + 28.0) * eps32 * acc[3] + 4.0 * eps32 * acc[5]) + 1e-12 * (acc[4] + acc[3]) +
                             1.01e-10 * acc[6];
    out[5 * (size_t)b + 4] = 1.01 * (acc[3] + acc[4] + acc[6]);
}

constexpr int kRecChangeMax = 32;   // changed segments one correction launch takes (8 rewirings)
struct RecChange {
    int m[kRecChangeMax], f[kRecChangeMax];
    double sign[kRecChangeMax];
    int n;
};

// Contribution of the changed segments to candidate node k at query point j
// (j < 0 the node itself): FP32 on the split positions with the error bound
// of k_rec_sums, FP64 near the query point.  out: 3 sums, bound.
__device__ __forceinline__ void corr_point(const RecArgs &r, int k, int j, const RecChange &ch, double out[4])
{
    double acc[3] = {0, 0, 0};   // FP64 terms
    double bound = 0;
    float tf[3] = {0, 0, 0};     // FP32 terms, their magnitudes' sum sc |R| |s|
    float mag = 0;
    if (k >= 0 && k < r.cap) {
        const double p[3] = {r.x[k], r.y[k], r.z[k]};
        float qg[3], qf[3];
        for (int a = 0; a < 3; ++a) {
            qg[a] = r.sp[(size_t)a * r.cap + k];
            qf[a] = r.sp[(size_t)(3 + a) * r.cap + k];
            if (j >= 0) { qg[a] -= r.shift_g[j][a]; qf[a] -= r.shift_f[j][a]; }
        }
        for (int i = 0; i < ch.n && i < kRecChangeMax; ++i) {
            int m = ch.m[i], f = ch.f[i];
            if (m < 0 || m >= r.cap || f < 0 || f >= r.cap) continue;
            float ag[3], af[3], sv[3];
            bool use64 = false;
            for (int a = 0; a < 3; ++a) {
                ag[a] = r.sp[(size_t)a * r.cap + m];
                af[a] = r.sp[(size_t)(3 + a) * r.cap + m];
                float bg = r.sp[(size_t)a * r.cap + f], bf = r.sp[(size_t)(3 + a) * r.cap + f];
                float d = (bg - ag[a]) + (bf - af[a]);
                if (r.geo.periodic[a]) {
                    if (fabsf(fabsf(d) - r.hL[a]) < 1e-3f * r.hL[a] || fabsf(d) > 3.0f * r.hL[a]) use64 = true;
                    if (d > r.hL[a]) { bg -= r.Lg[a]; bf -= r.Lf[a]; }
                    else if (d < -r.hL[a]) { bg += r.Lg[a]; bf += r.Lf[a]; }
                }
                sv[a] = (bg - ag[a]) + (bf - af[a]);
            }
            float R[3];
            for (int a = 0; a < 3; ++a) R[a] = (ag[a] - qg[a]) + (af[a] - qf[a]);
            const float lR2 = fmaf(R[0], R[0], fmaf(R[1], R[1], R[2] * R[2]));
            const float P0 = R[0] + sv[0], P1 = R[1] + sv[1], P2 = R[2] + sv[2];
            const float lp2 = fmaf(P0, P0, fmaf(P1, P1, P2 * P2));
            use64 = use64 || lR2 < r.rnear2 || lp2 < r.rnear2 || (j >= 0 && r.geo.nreflect[j] > 0);
            float ra = 0, rb = 0, ab = 0, dot = 0, nd = 0;
            if (!use64) {
                ra = rsqrtf(lR2);
                rb = rsqrtf(lp2);
                ab = ra * rb;
                dot = fmaf(R[0], P0, fmaf(R[1], P1, R[2] * P2));
                nd = dot * ab;
                if (fabsf(nd - 1e-8f) < 1e-4f) use64 = true;
            }
            if (use64) {
                double w[3];
                if (rec_term64(r, m, f, j, p, w)) {
                    for (int a = 0; a < 3; ++a) acc[a] += ch.sign[i] * w[a];
                    bound += 1e-12 * (fabs(w[0]) + fabs(w[1]) + fabs(w[2]));
                }
                continue;
            }
            if (nd < 1e-8f) continue;
            const float sc = __fdividef(r.f4pif * (ra + rb) * ab, fmaf(dot, ab, 1.0f));
            const float slen = sqrtf(fmaf(sv[0], sv[0], fmaf(sv[1], sv[1], sv[2] * sv[2])));
            const float sg = (float)ch.sign[i];   // +-1
            tf[0] += sg * (fmaf(R[1], sv[2], -R[2] * sv[1]) * sc);
            tf[1] += sg * (fmaf(R[2], sv[0], -R[0] * sv[2]) * sc);
            tf[2] += sg * (fmaf(R[0], sv[1], -R[1] * sv[0]) * sc);
            mag += sc * slen * lR2 * ra;
        }
    }
    // per term 64 eps32 of sc |R| |s| (as k_rec_sums), plus at most 8 eps32 of
    // the same for the FP32 additions of up to 8 terms; 1.01 covers the
    // rounding of mag itself
    for (int a = 0; a < 3; ++a) out[a] = acc[a] + (double)tf[a];
    out[3] = bound + 1.01 * 72.0 * 5.9604644775390625e-8 * (double)mag;
}

// Prefetch list of a correction: candidates whose corrections go straight to
// the mapped host buffer after the update (position i: 4 doubles at 4 i).
constexpr int kPrefetchMax = 128;
struct RecPrefetch {
    int idx[kPrefetchMax];
    int n;
};

// Contributions of the changed segments to candidates [c0, c0 + nc) of the
// sorted candidate list, one thread per (candidate, query point).  part: 4
// doubles per thread (3 sums, bound).
__global__ void k_corr(RecArgs r, const int *__restrict__ cand, int c0, int nc, RecChange ch,
                       double *__restrict__ part)
{
    const int nq = r.geo.n_img + 1;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nc * nq) return;
    const int ci = idx / nq, qi = idx - ci * nq;
    double out[4];
    corr_point(r, cand[c0 + ci], qi - 1, ch, out);
    for (int a = 0; a < 4; ++a) part[(size_t)idx * 4 + a] = out[a];
}

// corr[4 c + {0,1,2}] += the query points' sums in order, corr[4 c + 3] +=
// bound; then the prefetched candidates' corrections into host memory (h_out,
// mapped: position i of the list at 4 i).
__global__ void k_corr_finish(const double *__restrict__ part, int c0, int nc, int nq, double *__restrict__ corr,
                              RecPrefetch pf, double *h_out)
{
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= nc) return;
    double acc[4] = {0, 0, 0, 0};
    for (int q = 0; q < nq; ++q)
        for (int a = 0; a < 4; ++a) acc[a] += part[((size_t)ci * nq + q) * 4 + a];
    double *cc = corr + 4 * (size_t)(c0 + ci);
    for (int a = 0; a < 3; ++a) cc[a] += acc[a];
    cc[3] += acc[3] * (1.0 + 1e-9) + 1e-15 * (fabs(acc[0]) + fabs(acc[1]) + fabs(acc[2]));
    for (int i = 0; i < pf.n && i < kPrefetchMax; ++i)
        if (pf.idx[i] == c0 + ci)
            for (int a = 0; a < 4; ++a) h_out[4 * i + a] = cc[a];
}

RecArgs make_rec_args(ov_ctx *c)
{
    RecArgs r;
    memset(&r, 0, sizeof r);
    r.x = c->node.x; r.y = c->node.y; r.z = c->node.z;
    r.fwd = c->fwd;
    r.sp = c->rec_split;
    r.geo = c->geo;
    const double h = c->grid_h;
    for (int j = 0; j < c->geo.n_img; ++j)
        for (int a = 0; a < 3; ++a) {
            double sh = c->geo.L[a] * (double)c->geo.shift[j][a];
            double G = rint(sh / h) * h;
            r.shift_g[j][a] = (float)G;
            r.shift_f[j][a] = (float)(sh - G);
        }
    for (int a = 0; a < 3; ++a) {
        double G = rint(c->geo.L[a] / h) * h;
        r.Lg[a] = (float)G;
        r.Lf[a] = (float)(c->geo.L[a] - G);
        r.Lfl[a] = (float)((c->geo.L[a] - G) - (double)r.Lf[a]);
        r.hL[a] = (float)(c->geo.L[a] * 0.5);
    }
    r.f4pi = c->params.kappa / 4 / M_PI;
    r.f4pif = (float)r.f4pi;
    r.grid_h = h;
    r.inv_h = 1.0 / h;
    // FP64 within 4 dl_max (segments are shorter than 2 dl_max after remesh)
    double dl = 0;
    for (const Member &m : c->mem) dl = std::max(dl, m.params.dl_max);
    double rn = 4.0 * std::max(dl, c->params.rec_dist);
    r.rnear2 = (float)(rn * rn);
    const bool ens = c->mem.size() > 1;
    r.tid = ens ? c->d_tid : nullptr;
    r.mrange = ens ? c->d_mrange : nullptr;
    r.nt = (int)c->mem.size();
    r.cap = c->cap;
    return r;
}

int rec_reserve(ov_ctx *c, int n, int max_chunks)
{
    size_t need_part = (size_t)std::max(n, 1) * max_chunks * kRecVals;
    const int nq = c->geo.n_img + 1;
    need_part = std::max(need_part, (size_t)std::max(n, 1) * nq * 4);
    if (c->rec_part_cap < need_part) {
        if (c->rec_part) cudaFree(c->rec_part);
        c->rec_part = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->rec_part, need_part * sizeof(double)));
        c->rec_part_cap = need_part;
    }
    if (c->rec_cap < n) {
        if (c->rec_nodes) cudaFree(c->rec_nodes);
        if (c->rec_out) cudaFree(c->rec_out);
        if (c->rec_corr) cudaFree(c->rec_corr);
        c->rec_nodes = nullptr; c->rec_out = nullptr; c->rec_corr = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->rec_nodes, (size_t)n * sizeof(int)));
        OV_ALLOC(c, cudaMalloc(&c->rec_out, (size_t)n * 5 * sizeof(double)));
        OV_ALLOC(c, cudaMalloc(&c->rec_corr, (size_t)n * 4 * sizeof(double)));
        c->rec_cap = n;
    }
    if (c->rec_split_cap < c->cap) {
        if (c->rec_split) cudaFree(c->rec_split);
        c->rec_split = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->rec_split, (size_t)c->cap * 9 * sizeof(float)));
        c->rec_split_cap = c->cap;
    }
    return OV_OK;
}

// mode: 0 mixed (FP32 far, FP64 near), 1 FP64, 2 double-single far, FP64 near
int rec_launch_sums(ov_ctx *c, const int *d_nodes, int n, int mode, double *out_host)
{
    int maxcap = 0;
    for (const Member &m : c->mem) maxcap = std::max(maxcap, c->mem.size() == 1 ? c->cap : m.cap);
    const int span = 8192;
    const int max_chunks = std::max(1, (maxcap + span - 1) / span);
    int r = rec_reserve(c, n, max_chunks);
    if (r) return r;
    RecArgs ra = make_rec_args(c);
    dim3 grid(n, max_chunks);
    bool mirror = false;
    for (int j = 0; j < c->geo.n_img; ++j) mirror = mirror || c->geo.nreflect[j] > 0;
    if (mode == 1)
        k_rec_sums<1, true><<<grid, kRecThreads, 0, c->stream>>>(ra, d_nodes, n, span, max_chunks, c->rec_part);
    else if (mode == 2 && mirror)
        k_rec_sums<2, true><<<grid, kRecThreads, 0, c->stream>>>(ra, d_nodes, n, span, max_chunks, c->rec_part);
    else if (mode == 2)
        k_rec_sums<2, false><<<grid, kRecThreads, 0, c->stream>>>(ra, d_nodes, n, span, max_chunks, c->rec_part);
    else if (mirror)
        k_rec_sums<0, true><<<grid, kRecThreads, 0, c->stream>>>(ra, d_nodes, n, span, max_chunks, c->rec_part);
    else
        k_rec_sums<0, false><<<grid, kRecThreads, 0, c->stream>>>(ra, d_nodes, n, span, max_chunks, c->rec_part);
    k_rec_finish<<<(n + 127) / 128, 128, 0, c->stream>>>(c->rec_part, n, max_chunks, c->rec_out);
    c->launches += 2;
    OV_CUDA(c, cudaGetLastError());
    OV_CUDA(c, cudaMemcpyAsync(out_host, c->rec_out, (size_t)n * 5 * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream));
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    return OV_OK;
}

}  // namespace

// Mixed-precision sums of the candidate list (kept on the device for the
// corrections): out[5 i + {0,1,2}] the sum, out[5 i + 3] a bound on each
// component's error, out[5 i + 4] the sum of the terms' magnitudes.
int ov_rec_begin(ov_ctx *c, const int *cand, int n, double *out)
{
    if (n <= 0) return OV_OK;
    int maxcap = 0;
    for (const Member &m : c->mem) maxcap = std::max(maxcap, c->mem.size() == 1 ? c->cap : m.cap);
    int r = rec_reserve(c, n, std::max(1, (maxcap + 8191) / 8192));
    if (r) return r;
    OV_CUDA(c, cudaMemcpyAsync(c->rec_nodes, cand, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    OV_CUDA(c, cudaMemsetAsync(c->rec_corr, 0, (size_t)n * 4 * sizeof(double), c->stream));
    k_split<<<(c->cap + 255) / 256, 256, 0, c->stream>>>(c->node.x, c->node.y, c->node.z, c->cap, c->grid_h,
                                                        1.0 / c->grid_h, c->rec_split);
    c->launches++;
    return rec_launch_sums(c, c->rec_nodes, n, 0, out);
}

// Tight sums of nodes k and l on the current device positions and
// connections, laid out as ov_rec_begin's: far terms in double-single (bound
// 1e-10 of their magnitudes), near ones in FP64.
int ov_rec_exact(ov_ctx *c, int k, int l, double out[10])
{
    int nodes[2] = {k, l};
    int maxcap = 0;
    for (const Member &m : c->mem) maxcap = std::max(maxcap, c->mem.size() == 1 ? c->cap : m.cap);
    int r = rec_reserve(c, 2, std::max(1, (maxcap + 8191) / 8192));
    if (r) return r;
    if (!c->rec_pair) OV_ALLOC(c, cudaMalloc(&c->rec_pair, 2 * sizeof(int)));
    OV_CUDA(c, cudaMemcpyAsync(c->rec_pair, nodes, 2 * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    // the split positions of the current device positions
    k_split<<<(c->cap + 255) / 256, 256, 0, c->stream>>>(c->node.x, c->node.y, c->node.z, c->cap, c->grid_h,
                                                        1.0 / c->grid_h, c->rec_split);
    c->launches++;
    return rec_launch_sums(c, c->rec_pair, 2, 2, out);
}

extern "C" int ov_direct_sums_bounded(ov_ctx *c, const int *nodes, int n, int precision, double *out)
{
    if (!c || n < 0 || (n > 0 && (!nodes || !out))) return OV_ERR_ARG;
    if (!c->uploaded) return ov_fail(c, OV_ERR_STATE, "no tangle uploaded");
    if (precision != OV_PREC_FP64 && precision != OV_PREC_MIXED && precision != OV_PREC_DD) return OV_ERR_ARG;
    cudaSetDevice(c->device);
    for (int i = 0; i < n; ++i)
        if (nodes[i] < 0 || nodes[i] >= c->cap) return ov_fail(c, OV_ERR_ARG, "node %d out of range", nodes[i]);
    if (n == 0) return OV_OK;
    int maxcap = 0;
    for (const Member &m : c->mem) maxcap = std::max(maxcap, c->mem.size() == 1 ? c->cap : m.cap);
    int r = rec_reserve(c, n, std::max(1, (maxcap + 8191) / 8192));
    if (r) return r;
    OV_CUDA(c, cudaMemcpyAsync(c->rec_nodes, nodes, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    k_split<<<(c->cap + 255) / 256, 256, 0, c->stream>>>(c->node.x, c->node.y, c->node.z, c->cap, c->grid_h,
                                                        1.0 / c->grid_h, c->rec_split);
    c->launches++;
    return rec_launch_sums(c, c->rec_nodes, n, precision == OV_PREC_FP64 ? 1 : (precision == OV_PREC_DD ? 2 : 0), out);
}

// ov_direct_velocities: FP64 direct sums in (node, segment chunk) blocks,
// then LIA, v_s and friction (k_direct_finish) into device arrays.
int ov_direct_sum_chunked(ov_ctx *c, const int *nodes, int n, double *d_out_vel, double *d_out_vs, double t)
{
    int maxcap = 0;
    for (const Member &m : c->mem) maxcap = std::max(maxcap, c->mem.size() == 1 ? c->cap : m.cap);
    const int span = 8192, max_chunks = std::max(1, (maxcap + span - 1) / span);
    int r = rec_reserve(c, n, max_chunks);
    if (r) return r;
    OV_CUDA(c, cudaMemcpyAsync(c->rec_nodes, nodes, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    k_split<<<(c->cap + 255) / 256, 256, 0, c->stream>>>(c->node.x, c->node.y, c->node.z, c->cap, c->grid_h,
                                                        1.0 / c->grid_h, c->rec_split);
    RecArgs ra = make_rec_args(c);
    k_rec_sums<1, true><<<dim3(n, max_chunks), kRecThreads, 0, c->stream>>>(ra, c->rec_nodes, n, span, max_chunks,
                                                                      c->rec_part);
    k_rec_finish<<<(n + 127) / 128, 128, 0, c->stream>>>(c->rec_part, n, max_chunks, c->rec_out);
    VelArgs a = make_args(c, c->node, t, nullptr);
    k_direct_finish<<<(n + 127) / 128, 128, 0, c->stream>>>(a, c->rec_nodes, n, c->rec_out, 5, d_out_vel, d_out_vs);
    c->launches += 4;
    OV_CUDA(c, cudaGetLastError());
    return OV_OK;
}

// Add the changed segments' contributions (and their error bounds) to
// candidates [c0, c0 + nc) on the device (asynchronous; ov_rec_fetch reads
// them back).
// The changed segments' contributions to candidates [c0, c0 + nc), then the
// corrections of candidates pf[0..npf) (all within that range) read back into
// the pinned, mapped buffer c->h_pf; ov_rec_wait waits for both.
int ov_rec_correct(ov_ctx *c, int c0, int nc, const int *m, const int *f, const double *sign, int nch,
                   const int *pf, int npf)
{
    if (nc <= 0) return OV_OK;
    if (npf < 0 || npf > kPrefetchMax) return ov_fail(c, OV_ERR_ARG, "reconnect: %d prefetched candidates", npf);
    if (!c->h_pf) {
        OV_ALLOC(c, cudaHostAlloc(&c->h_pf, kPrefetchMax * 4 * sizeof(double), cudaHostAllocMapped));
        OV_CUDA(c, cudaHostGetDevicePointer((void **)&c->h_pf_dev, c->h_pf, 0));
    }
    if (!c->rec_ev) OV_CUDA(c, cudaEventCreateWithFlags(&c->rec_ev, cudaEventDisableTiming));
    if (nch < 0 || nch > kRecChangeMax) return ov_fail(c, OV_ERR_ARG, "reconnect: %d changed segments", nch);
    RecChange ch;
    memset(&ch, 0, sizeof ch);
    ch.n = nch;
    for (int i = 0; i < ch.n; ++i) { ch.m[i] = m[i]; ch.f[i] = f[i]; ch.sign[i] = sign[i]; }
    RecPrefetch list;
    list.n = npf;
    for (int i = 0; i < npf; ++i) list.idx[i] = pf[i];
    RecArgs ra = make_rec_args(c);
    const int nq = c->geo.n_img + 1;
    k_corr<<<(nc * nq + 127) / 128, 128, 0, c->stream>>>(ra, c->rec_nodes, c0, nc, ch, c->rec_part);
    k_corr_finish<<<(nc + 127) / 128, 128, 0, c->stream>>>(c->rec_part, c0, nc, nq, c->rec_corr, list, c->h_pf_dev);
    c->launches += 2;
    OV_CUDA(c, cudaGetLastError());
    OV_CUDA(c, cudaEventRecord(c->rec_ev, c->stream));
    return OV_OK;
}

int ov_rec_wait(ov_ctx *c)
{
    OV_CUDA(c, cudaEventSynchronize(c->rec_ev));
    return OV_OK;
}

// Corrections of candidates [c0, c0 + n) (4 doubles each) into out.
int ov_rec_fetch(ov_ctx *c, int c0, int n, double *out)
{
    if (n <= 0) return OV_OK;
    OV_CUDA(c, cudaMemcpyAsync(out, c->rec_corr + 4 * (size_t)c0, (size_t)n * 4 * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    return OV_OK;
}

void ov_launch_euler(ov_ctx *c, const NodeArrays &src, const double *vx, const double *vy, const double *vz,
                     double dt, NodeArrays &dst, cudaStream_t s)
{
    const double *dt_dev = c->time_dev_index >= 0 ? c->d_time + 3 : nullptr;   // d_time[3] = dt/2
    k_euler<<<(c->cap + 255) / 256, 256, 0, s>>>(c->status, src.x, src.y, src.z, vx, vy, vz, dt, dst.x, dst.y,
                                                 dst.z, c->cap, dt_dev);
    c->launches++;
}

void ov_launch_rk4_combine(ov_ctx *c, double dt, cudaStream_t s)
{
    Rk4Args r;
    r.dt_dev = c->time_dev_index >= 0 ? c->d_time + 4 : nullptr;   // d_time[4] = dt
    r.err = c->tree.counters + TC_ERR;
    r.status = c->status;
    r.x = c->node.x; r.y = c->node.y; r.z = c->node.z;
    r.v1x = c->node.vx; r.v1y = c->node.vy; r.v1z = c->node.vz;
    r.v2x = c->stage[0].vx; r.v2y = c->stage[0].vy; r.v2z = c->stage[0].vz;
    r.v3x = c->stage[1].vx; r.v3y = c->stage[1].vy; r.v3z = c->stage[1].vz;
    r.v4x = c->stage[2].vx; r.v4y = c->stage[2].vy; r.v4z = c->stage[2].vz;
    r.dt = dt;
    r.cap = c->cap;
    k_rk4_combine<<<(c->cap + 255) / 256, 256, 0, s>>>(r);
    c->launches++;
}

void ov_launch_periodic_wrap(ov_ctx *c, cudaStream_t s)
{
    k_wrap<<<(c->cap + 255) / 256, 256, 0, s>>>(c->status, c->node.x, c->node.y, c->node.z, c->geo, c->cap);
    c->launches++;
}

// ----------------------------------------------------------------------------
// Direct sum without allocation (ov_direct_velocities_noalloc).
//
// For callers that cannot allocate device memory: the partial sums that
// ov_direct_velocities keeps in a context buffer live here in a fixed array
// compiled into the library.  Host code never uses the array's name as a
// pointer (on the host it is only a stand-in); the device address is looked
// up once per device and passed to the kernels.  That address belongs to the
// device's context as it was at the first call: after cudaDeviceReset the
// entry point must not be called again in the process.
// ----------------------------------------------------------------------------
#include <mutex>

static __device__ __align__(256) double g_noalloc_sums[3 * OV_NOALLOC_MAX_NODES];

namespace {

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mu;
double *g_noalloc_addr[kNoallocMaxDevices] = {};

// Sum pass: one block per listed node, every segment of the primary tangle
// and of each image; writes the node's three partial sums into `sums`.
__global__ void k_direct_noalloc(VelArgs a, const int *__restrict__ nodes, int n, int n_slots,
                                 double *__restrict__ sums)
{
    __shared__ double red[3][256];
    int b = blockIdx.x;
    if (b >= n) return;
    int k = nodes[b];
    bool ok = k >= 0 && k < n_slots;
    double acc[3] = {0, 0, 0};
    if (ok) {
        double p[3] = {a.x[k], a.y[k], a.z[k]};
        for (int j = -1; j < a.geo.n_img; ++j) {
            double q[3];
            if (j < 0) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; }
            else image_point(a.geo, j, p, q);
            for (int m = threadIdx.x; m < n_slots; m += blockDim.x) {
                int f = a.fwd[m];
                if (f < 0 || f >= n_slots) continue;
                if (j < 0 && (m == k || f == k)) continue;
                double s1[3] = {a.x[m], a.y[m], a.z[m]};
                double s2[3] = {a.x[f], a.y[f], a.z[f]};
                pwrap_dev(a.geo, s1, s2);
                double R[3] = {rn_sub(s1[0], q[0]), rn_sub(s1[1], q[1]), rn_sub(s1[2], q[2])};
                double Rp1[3] = {rn_sub(s2[0], q[0]), rn_sub(s2[1], q[1]), rn_sub(s2[2], q[2])};
                double lR = len3_ref(R[0], R[1], R[2]);
                double w[3];
                if (segment_law64(R, Rp1, lR, a.f4pi, w)) {
                    acc[0] += w[0]; acc[1] += w[1]; acc[2] += w[2];
                }
            }
        }
    }
    for (int ax = 0; ax < 3; ++ax) red[ax][threadIdx.x] = acc[ax];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int ax = 0; ax < 3; ++ax) red[ax][threadIdx.x] += red[ax][threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int ax = 0; ax < 3; ++ax) sums[3 * (size_t)b + ax] = ok ? red[ax][0] : __longlong_as_double(0x7ff8000000000000ll);
}

// Finish pass: LIA, external v_s and mutual friction on top of the sums.
__global__ void k_direct_noalloc_finish(VelArgs a, const int *__restrict__ nodes, int n, int n_slots,
                                        const double *__restrict__ sums, double *__restrict__ vout,
                                        double *__restrict__ sout)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    int k = nodes[b];
    // as k_direct_finish: an EMPTY slot gives zeros; only an id outside the
    // slot range (which the allocating call never sees) gives NaN
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    double vs[3] = {0, 0, 0}, vel[3] = {0, 0, 0};
    if (k < 0 || k >= n_slots) {
        for (int ax = 0; ax < 3; ++ax) vs[ax] = vel[ax] = nan;
    } else if (a.status[k] != OV_EMPTY) {
        double p[3] = {a.x[k], a.y[k], a.z[k]};
        double prim[3] = {sums[3 * (size_t)b], sums[3 * (size_t)b + 1], sums[3 * (size_t)b + 2]};
        double zero[3] = {0, 0, 0};
        int err = 0;
        finish_node(a, k, p, prim, zero, &err, vs, vel);
    }
    for (int ax = 0; ax < 3; ++ax) {
        vout[3 * (size_t)b + ax] = vel[ax];
        if (sout) sout[3 * (size_t)b + ax] = vs[ax];
    }
}

}  // namespace

extern "C" int ov_direct_velocities_noalloc(const ov_params *p, const ov_domain_box *box,
                                            const ov_image_tangle *images, int n_images, int n_slots,
                                            const double *d_pos, const int *d_conn, const int *d_status,
                                            const double *d_tangents, const double *d_normals,
                                            const int *d_nodes, int n_nodes, double t, double *d_vels,
                                            double *d_vs, void *stream)
{
    if (!p || !box || n_nodes < 0 || n_slots < 0 || n_images < 0 || n_images > OV_MAX_IMAGES ||
        (n_images > 0 && !images))
        return OV_ERR_ARG;
    if (n_nodes > OV_NOALLOC_MAX_NODES) return OV_ERR_ARG;   // above the fixed working space
    if (n_nodes == 0) return OV_OK;
    if (!d_pos || !d_conn || !d_status || !d_tangents || !d_normals || !d_nodes || !d_vels) return OV_ERR_ARG;

    // one-time look-up of the working array's device address on this device
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoallocMaxDevices) return OV_ERR_CUDA;
    double *sums = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void *addr = nullptr;
            if (cudaGetSymbolAddress(&addr, g_noalloc_sums) != cudaSuccess || !addr) return OV_ERR_CUDA;
            g_noalloc_addr[dev] = (double *)addr;
        }
        sums = g_noalloc_addr[dev];
    }

    VelArgs a;
    memset(&a, 0, sizeof a);
    size_t ns = (size_t)n_slots;
    a.x = d_pos; a.y = d_pos + ns; a.z = d_pos + 2 * ns;
    a.tx = d_tangents; a.ty = d_tangents + ns; a.tz = d_tangents + 2 * ns;
    a.nx = d_normals; a.ny = d_normals + ns; a.nz = d_normals + 2 * ns;
    a.fwd = d_conn; a.rev = d_conn + ns;
    a.status = d_status; a.pin = d_status + ns;
    a.cap = n_slots;
    Geometry &g = a.geo;
    for (int ax = 0; ax < 3; ++ax) {
        g.lo[ax] = box->bottom_left_back.p[ax];
        g.hi[ax] = box->top_right_front.p[ax];
        g.L[ax] = g.hi[ax] - g.lo[ax];
    }
    for (int f = 0; f < 6; ++f) g.wall[f] = box->wall[f];
    g.periodic[0] = box->wall[OV_LEFT] == OV_WALL_PERIODIC;
    g.periodic[1] = box->wall[OV_BACK] == OV_WALL_PERIODIC;
    g.periodic[2] = box->wall[OV_DOWN] == OV_WALL_PERIODIC;
    g.n_img = n_images;
    for (int j = 0; j < n_images; ++j) {
        for (int ax = 0; ax < 3; ++ax) {
            g.shift[j][ax] = images[j].shift[ax];
            g.reflect[j][ax] = images[j].reflect[ax];
        }
        int nr = images[j].number_of_reflects;
        g.nreflect[j] = nr < 0 ? 0 : (nr > 3 ? 3 : nr);
    }
    a.prm = ov_dev_params(*p);
    a.t = t;
    a.f4pi = p->kappa / 4 / M_PI;

    cudaStream_t s = (cudaStream_t)stream;
    k_direct_noalloc<<<n_nodes, 256, 0, s>>>(a, d_nodes, n_nodes, n_slots, sums);
    k_direct_noalloc_finish<<<(n_nodes + 127) / 128, 128, 0, s>>>(a, d_nodes, n_nodes, n_slots, sums, d_vels, d_vs);
    return cudaGetLastError() == cudaSuccess ? OV_OK : OV_ERR_CUDA;
}

// ------------------------------------------------ spherical section domains
//
// The spherical fork (src_spherical/ of OpenVort): the domain is a section of
// a spherical shell, inner radius ri, outer ro, azimuth and polar angle in
// (-A, A) and (-P, P); the section repeats by rotations of 2A and 2P, and the
// inner surface is a wall made by the spherical inversion of the tangle
// through ri (its own tree, subtracted).  The slot pool holds the tangle in
// member 0 and its inner image in member 1, and one forest build gives both
// trees.  Every node walks the tangle's tree at its position and at its 8
// rotated copies (results rotated back), then the image's tree at the same 9
// points, all in FP64 on the reference's decisions.  The angles go through
// the device's atan2 / sin / cos, whose last bit may differ from the host
// libm's: velocities agree to rounding, a decision exactly on a threshold
// could go the other way.
#include "ov_helium.cuh"

namespace {

struct SphArgs {
    VelArgs v;                 // tree, positions, topology (slots [0, n) the tangle)
    int n;                     // slots of the tangle
    double ri, ro;             // shell radii
    double d_az, d_pl;         // the section's full angular widths (rotation steps)
    double kappa, a0, alpha, alpha_p, dl_min, dl_max;
    int friction, use_temperature;
    double q_dot, t_bath, prof_a;   // temperature profile (use_temperature)
};

// step_node of the fork (tangle.c:155-201): a pinned end reverses the walk
// and inverts the result through its surface, innermost first.
__device__ bool sph_step_node(const SphArgs &s, int i, int where, double out[3])
{
    const VelArgs &a = s.v;
    int surf[8];
    int nw = 0, cur = i, w = where;
    for (int guard = 0; w != 0; ++guard) {
        if (guard > 16 || cur < 0 || cur >= s.n) return false;
        const int st = a.status[cur];
        if (st == OV_FREE) {
            cur = w > 0 ? a.fwd[cur] : a.rev[cur];
            w += w > 0 ? -1 : 1;
        } else if (st == OV_PINNED || st == OV_PINNED_SLIP) {
            const int nb = w > 0 ? a.fwd[cur] : a.rev[cur];
            if (nb >= 0) {
                cur = nb;
                w += w > 0 ? -1 : 1;
            } else {
                const int f = a.pin[cur];
                if (nw >= 8 || (f != 0 && f != 1)) return false;   // not on a surface
                surf[nw++] = f;
                w = -w;
            }
        } else {
            return false;
        }
    }
    if (cur < 0 || cur >= s.n || a.status[cur] == OV_EMPTY) return false;
    out[0] = a.x[cur]; out[1] = a.y[cur]; out[2] = a.z[cur];
    for (int m = nw - 1; m >= 0; --m) {
        double q[3];
        if (!sph_invert(out, surf[m] == 0 ? s.ri : s.ro, q)) return false;
        out[0] = q[0]; out[1] = q[1]; out[2] = q[2];
    }
    return true;
}

__device__ __forceinline__ double sph_wrapped_len(const Geometry &g, const double r1[3], const double r2in[3])
{
    double r2[3] = {r2in[0], r2in[1], r2in[2]};
    sph_pwrap(g, r1, r2);
    return len3_ref(rn_sub(r1[0], r2[0]), rn_sub(r1[1], r2[1]), rn_sub(r1[2], r2[2]));
}

// update_tangent_normal of the fork (tangle.c:483-560): the five-point
// finite differences of the flat geometry on angularly wrapped segments.
__global__ void k_sph_tangents(SphArgs s, int *counters)
{
    const VelArgs &a = s.v;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= s.n || a.status[k] == OV_EMPTY) return;
    const Geometry &g = a.geo;
    double s0[3] = {a.x[k], a.y[k], a.z[k]}, s1[3], s2[3], sm1[3], sm2[3];
    bool ok = sph_step_node(s, k, 1, s1) & sph_step_node(s, k, 2, s2) & sph_step_node(s, k, -1, sm1) &
              sph_step_node(s, k, -2, sm2);
    if (!ok) {
        atomicOr(&counters[TC_ERR], OV_EW_WALK);
        return;
    }
    double w2[3] = {s2[0], s2[1], s2[2]}, w1[3] = {s1[0], s1[1], s1[2]};
    double wm1[3] = {sm1[0], sm1[1], sm1[2]}, wm2[3] = {sm2[0], sm2[1], sm2[2]};
    sph_pwrap(g, s0, w2);
    sph_pwrap(g, s0, w1);
    sph_pwrap(g, s0, wm1);
    sph_pwrap(g, s0, wm2);
    double d1 = len3_ref(rn_sub(s0[0], w1[0]), rn_sub(s0[1], w1[1]), rn_sub(s0[2], w1[2]));
    double d2 = rn_add(d1, sph_wrapped_len(g, s1, s2));
    double dm1 = len3_ref(rn_sub(s0[0], wm1[0]), rn_sub(s0[1], wm1[1]), rn_sub(s0[2], wm1[2]));
    double dm2 = rn_add(dm1, sph_wrapped_len(g, sm1, sm2));
    double den[4] = {
        rn_mul(rn_mul(rn_mul(d2, rn_sub(d2, d1)), rn_add(dm1, d2)), rn_add(dm2, d2)),
        rn_mul(rn_mul(rn_mul(d1, rn_sub(d2, d1)), rn_add(dm1, d1)), rn_add(dm2, d1)),
        rn_mul(rn_mul(rn_mul(dm1, rn_add(dm1, d1)), rn_add(dm1, d2)), rn_sub(dm2, dm1)),
        rn_mul(rn_mul(rn_mul(dm2, rn_add(dm2, d1)), rn_add(dm2, d2)), rn_sub(dm2, dm1))};
    double c1[4] = {rn_mul(rn_mul(-d1, dm1), dm2), rn_mul(rn_mul(d2, dm1), dm2), rn_mul(rn_mul(-d1, d2), dm2),
                    rn_mul(rn_mul(d1, d2), dm1)};
    double c2[4] = {
        rn_mul(2.0, rn_sub(rn_mul(rn_sub(dm1, d1), dm2), rn_mul(d1, dm1))),
        rn_mul(-2.0, rn_sub(rn_mul(rn_sub(dm1, d2), dm2), rn_mul(d2, dm1))),
        rn_mul(2.0, rn_sub(rn_mul(rn_add(d2, d1), dm2), rn_mul(d1, d2))),
        rn_mul(-2.0, rn_sub(rn_mul(rn_add(d2, d1), dm1), rn_mul(d1, d2)))};
    double ds[4][3];
    for (int ax = 0; ax < 3; ++ax) {
        ds[0][ax] = rn_sub(w2[ax], s0[ax]);
        ds[1][ax] = rn_sub(w1[ax], s0[ax]);
        ds[2][ax] = rn_sub(wm1[ax], s0[ax]);
        ds[3][ax] = rn_sub(wm2[ax], s0[ax]);
    }
    double *T[3] = {(double *)a.tx, (double *)a.ty, (double *)a.tz};
    double *Nn[3] = {(double *)a.nx, (double *)a.ny, (double *)a.nz};
    for (int ax = 0; ax < 3; ++ax) {
        double tt = 0, nn = 0;
        for (int z = 0; z < 4; ++z) {
            tt = rn_add(tt, rn_mul(rn_div(c1[z], den[z]), ds[z][ax]));
            nn = rn_add(nn, rn_mul(rn_div(c2[z], den[z]), ds[z][ax]));
        }
        T[ax][k] = tt;
        Nn[ax][k] = nn;
    }
}

// The inner image (update_velocities of the fork, tangle.c:956-976):
// slot n + k holds node k inverted through the inner surface.
__global__ void k_sph_images(SphArgs s, double *x, double *y, double *z, int *counters)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= s.n || s.v.status[k] == OV_EMPTY) return;
    const double p[3] = {x[k], y[k], z[k]};
    double q[3];
    if (!sph_invert(p, s.ri, q)) {
        atomicOr(&counters[TC_ERR], OV_EW_INVERT);
        q[0] = q[1] = q[2] = 0;
    }
    x[s.n + k] = q[0]; y[s.n + k] = q[1]; z[s.n + k] = q[2];
}

__device__ __forceinline__ void sph_normalize(const double p[3], double out[3])
{
    if (p[0] == 0 && p[1] == 0 && p[2] == 0) { out[0] = out[1] = out[2] = 0; return; }
    const double m = rn_div(1.0, len3_ref(p[0], p[1], p[2]));
    for (int ax = 0; ax < 3; ++ax) out[ax] = rn_mul(p[ax], m);
}

// The 18 tree queries of update_velocity (tangle.c:669-761 of the fork,
// outer surface open), one warp per (32 targets, query): query q < 9 walks
// the tangle's tree, q >= 9 the inner image's; q % 9 == 0 at the node, else
// at rotation q % 9 - 1 (+-az, +-pl, then the corners), its result rotated
// back.  part[(q * 3 + axis) * n + node] holds the result.
__global__ void __launch_bounds__(128) k_sph_query(SphArgs s, double *__restrict__ part)
{
    const VelArgs &a = s.v;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nne = a.tt[TT_NNE];   // member 0: the tangle, first in sorted order
    const int tiles = (nne + 31) / 32;
    if (warp >= 18 * tiles) return;
    const int q = warp / tiles, tile = warp - q * tiles;
    const int loc = tile * 32 + lane;
    bool valid = loc < nne;
    int id = valid ? a.order[loc] : 0;
    if (valid && (id < 0 || id >= s.n)) { bad_index(a, 9, id); valid = false; id = 0; }
    const int st = valid ? a.status[id] : OV_EMPTY;
    const bool take = valid && st != OV_PINNED && st != OV_EMPTY;
    double p[3] = {0, 0, 0};
    if (valid) { p[0] = a.x[id]; p[1] = a.y[id]; p[2] = a.z[id]; }
    unsigned long long visits = 0, accepts = 0, steps = 0;
    bool overflow = false;
    const int m = q / 9, j = q % 9 - 1;
    const int root = a.tt[m * TT_WORDS + TT_ROOT], end = a.tt[m * TT_WORDS + TT_END];
    const bool go = take && end > root;
    double v[3], w[3];
    if (j < 0) {
        bh_query64(a, p, go, root, end, w, visits, accepts, steps, overflow);
    } else {
        const double ua = j < 2 ? (j == 0 ? 1.0 : -1.0) : (j < 4 ? 0.0 : ((j & 1) ? -1.0 : 1.0));
        const double up = j < 2 ? 0.0 : (j < 4 ? (j == 2 ? 1.0 : -1.0) : (j < 6 ? 1.0 : -1.0));
        const double da = rn_mul(ua, s.d_az), dp = rn_mul(up, s.d_pl);
        double qp[3];
        sph_rotate(p, da, dp, qp);
        bh_query64(a, qp, go, root, end, v, visits, accepts, steps, overflow);
        sph_rotate(v, -da, -dp, w);
    }
    if (a.stat) {
        for (int o = 16; o > 0; o >>= 1) {
            visits += __shfl_xor_sync(0xffffffffu, visits, o);
            accepts += __shfl_xor_sync(0xffffffffu, accepts, o);
        }
        if (lane == 0) {
            atomicAdd(&a.stat[ST_VISITS], visits);
            atomicAdd(&a.stat[ST_ACCEPTS], accepts);
            atomicAdd(&a.stat[ST_STEPS], steps);
        }
    }
    if (overflow && lane == 0) atomicOr((int *)&a.counters[TC_ERR], OV_EW_ITER);
    if (!valid) return;
    for (int ax = 0; ax < 3; ++ax) part[((size_t)q * 3 + ax) * s.n + id] = w[ax];
}

// k_sph_query in mixed precision: the query point (rotated in FP64) split on
// the grid, the FP32 walk with the FP64 path's decisions (guard bands),
// near-field leaves in FP64 after the walk.
__global__ void __launch_bounds__(128) k_sph_query_mixed(SphArgs s, double *__restrict__ part)
{
    const VelArgs &a = s.v;
    __shared__ int s_near[4][kNearCap * 32];
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int *near_list = &s_near[threadIdx.x >> 5][lane];
    const int nne = a.tt[TT_NNE];
    const int tiles = (nne + 31) / 32;
    if (warp >= 18 * tiles) return;
    const int q = warp / tiles, tile = warp - q * tiles;
    const int loc = tile * 32 + lane;
    bool valid = loc < nne;
    int id = valid ? a.order[loc] : 0;
    if (valid && (id < 0 || id >= s.n)) { bad_index(a, 9, id); valid = false; id = 0; }
    const int st = valid ? a.status[id] : OV_EMPTY;
    const bool take = valid && st != OV_PINNED && st != OV_EMPTY;
    double p[3] = {0, 0, 0};
    if (valid) { p[0] = a.x[id]; p[1] = a.y[id]; p[2] = a.z[id]; }
    const int m = q / 9, j = q % 9 - 1;
    const int root = a.tt[m * TT_WORDS + TT_ROOT], end = a.tt[m * TT_WORDS + TT_END];
    const bool go = take && end > root;
    double qp[3] = {p[0], p[1], p[2]}, da = 0, dp = 0;
    if (j >= 0) {
        const double ua = j < 2 ? (j == 0 ? 1.0 : -1.0) : (j < 4 ? 0.0 : ((j & 1) ? -1.0 : 1.0));
        const double up = j < 2 ? 0.0 : (j < 4 ? (j == 2 ? 1.0 : -1.0) : (j < 6 ? 1.0 : -1.0));
        da = rn_mul(ua, s.d_az);
        dp = rn_mul(up, s.d_pl);
        sph_rotate(p, da, dp, qp);
    }
    float g[3], f[3];
    for (int ax = 0; ax < 3; ++ax) {
        const double G = rint(qp[ax] * a.inv_h) * a.grid_h;
        g[ax] = (float)G;
        f[ax] = (float)(qp[ax] - G);
    }
    MixedAcc acc = {0, 0, 0, 0, 0, 0, 0u, 0u, 0u, 0u, 0u};
    double w64[3] = {0, 0, 0};
    int nnear = 0;
    bool overflow = false;
    bh_query32<false>(a, g, f, qp, -1, go, root, end, acc, near_list, nnear, w64, overflow);
    for (int i = 0; i < nnear && i < kNearCap; ++i) {
        const int e = near_list[32 * i];
        const int c = e >> 5;
        if (c < root || c >= end) { bad_index(a, 3, e); continue; }
        double wv[3];
        law64_term(a.cells + c, qp, wv);   // zero when a filter drops it
        w64[0] += wv[0] * a.f4pi; w64[1] += wv[1] * a.f4pi; w64[2] += wv[2] * a.f4pi;
    }
    __syncwarp();
    double v[3] = {((double)acc.s0 - (double)acc.c0) + w64[0], ((double)acc.s1 - (double)acc.c1) + w64[1],
                   ((double)acc.s2 - (double)acc.c2) + w64[2]};
    double w[3] = {v[0], v[1], v[2]};
    if (j >= 0) sph_rotate(v, -da, -dp, w);
    if (a.stat) {
        unsigned long long vis = acc.nvis, ac = acc.nacc, fb = acc.nfb, nr = acc.nnear;
        for (int o = 16; o > 0; o >>= 1) {
            vis += __shfl_xor_sync(0xffffffffu, vis, o);
            ac += __shfl_xor_sync(0xffffffffu, ac, o);
            fb += __shfl_xor_sync(0xffffffffu, fb, o);
            nr += __shfl_xor_sync(0xffffffffu, nr, o);
        }
        if (lane == 0) {
            atomicAdd(&a.stat[ST_VISITS], vis);
            atomicAdd(&a.stat[ST_ACCEPTS], ac);
            atomicAdd(&a.stat[ST_STEPS], (unsigned long long)acc.nstep);
            atomicAdd(&a.stat[ST_FALLBACK], fb);
            atomicAdd(&a.stat[ST_NEAR64], nr);
        }
    }
    if (overflow && lane == 0) atomicOr((int *)&a.counters[TC_ERR], OV_EW_ITER);
    if (!valid) return;
    for (int ax = 0; ax < 3; ++ax) part[((size_t)q * 3 + ax) * s.n + id] = w[ax];
}

// k_sph_query on the FP64 path's split walk: the rotated query point split on
// the grid for the FP32 tests (FP64 inside the guard bands), the accepted
// cells evaluated in FP64 by the whole warp.
__global__ void __launch_bounds__(128) k_sph_query_split(SphArgs s, double *__restrict__ part)
{
    const VelArgs &a = s.v;
    __shared__ WarpLists s_lists[4];
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    WarpLists &lists = s_lists[threadIdx.x >> 5];
    const int nne = a.tt[TT_NNE];
    const int tiles = (nne + 31) / 32;
    if (warp >= 18 * tiles) return;
    const int q = warp / tiles, tile = warp - q * tiles;
    const int loc = tile * 32 + lane;
    bool valid = loc < nne;
    int id = valid ? a.order[loc] : 0;
    if (valid && (id < 0 || id >= s.n)) { bad_index(a, 9, id); valid = false; id = 0; }
    const int st = valid ? a.status[id] : OV_EMPTY;
    const bool take = valid && st != OV_PINNED && st != OV_EMPTY;
    double p[3] = {0, 0, 0};
    if (valid) { p[0] = a.x[id]; p[1] = a.y[id]; p[2] = a.z[id]; }
    const int m = q / 9, j = q % 9 - 1;
    const int root = a.tt[m * TT_WORDS + TT_ROOT], end = a.tt[m * TT_WORDS + TT_END];
    const bool go = take && end > root;
    double qp[3] = {p[0], p[1], p[2]}, da = 0, dp = 0;
    if (j >= 0) {
        const double ua = j < 2 ? (j == 0 ? 1.0 : -1.0) : (j < 4 ? 0.0 : ((j & 1) ? -1.0 : 1.0));
        const double up = j < 2 ? 0.0 : (j < 4 ? (j == 2 ? 1.0 : -1.0) : (j < 6 ? 1.0 : -1.0));
        da = rn_mul(ua, s.d_az);
        dp = rn_mul(up, s.d_pl);
        sph_rotate(p, da, dp, qp);
    }
    float g[3], f[3];
    for (int ax = 0; ax < 3; ++ax) {
        const double G = rint(qp[ax] * a.inv_h) * a.grid_h;
        g[ax] = (float)G;
        f[ax] = (float)(qp[ax] - G);
    }
    MixedAcc acc = {0, 0, 0, 0, 0, 0, 0u, 0u, 0u, 0u, 0u};
    bool overflow = false;
    double v[3];
    walk_split(a, g, f, qp, go ? 0 : 0x7fffffff, root, end, end, lists, lane, v, acc, overflow);
    double w[3] = {v[0], v[1], v[2]};
    if (j >= 0) sph_rotate(v, -da, -dp, w);
    if (a.stat) {
        unsigned long long vis = acc.nvis, ac = acc.nacc, fb = acc.nfb;
        for (int o = 16; o > 0; o >>= 1) {
            vis += __shfl_xor_sync(0xffffffffu, vis, o);
            ac += __shfl_xor_sync(0xffffffffu, ac, o);
            fb += __shfl_xor_sync(0xffffffffu, fb, o);
        }
        if (lane == 0) {
            atomicAdd(&a.stat[ST_VISITS], vis);
            atomicAdd(&a.stat[ST_ACCEPTS], ac);
            atomicAdd(&a.stat[ST_STEPS], (unsigned long long)acc.nstep);
            atomicAdd(&a.stat[ST_FALLBACK], fb);
        }
    }
    if (overflow && lane == 0) atomicOr((int *)&a.counters[TC_ERR], OV_EW_ITER);
    if (!valid) return;
    for (int ax = 0; ax < 3; ++ax) part[((size_t)q * 3 + ax) * s.n + id] = w[ax];
}

// The rest of update_velocity (tangle.c:644-665, 763-865 of the fork): the
// query results summed in the fork's order, LIA with its segment-length
// limits, the temperature model, mutual friction, PINNED_SLIP.
__global__ void k_sph_finish(SphArgs s, const double *__restrict__ part)
{
    const VelArgs &a = s.v;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= s.n) return;
    const int st = a.status[id];
    if (st == OV_EMPTY) return;
    if (st == OV_PINNED) {   // the node rests; its velocity is left as it was
        a.sx[id] = a.sy[id] = a.sz[id] = 0;
        return;
    }
    const double p[3] = {a.x[id], a.y[id], a.z[id]};
    auto P = [&](int q, int ax) { return part[((size_t)q * 3 + ax) * s.n + id]; };
    double own[3], tot[3] = {0, 0, 0};
    for (int ax = 0; ax < 3; ++ax) own[ax] = P(0, ax);
    for (int q = 1; q < 9; ++q)
        for (int ax = 0; ax < 3; ++ax) tot[ax] = rn_add(tot[ax], P(q, ax));
    for (int q = 9; q < 18; ++q)
        for (int ax = 0; ax < 3; ++ax) tot[ax] = rn_sub(tot[ax], P(q, ax));
    // LIA with the fork's limits on the neighbour distances (tangle.c:581-611)
    double nx_[3], pv[3];
    if (!(sph_step_node(s, id, 1, nx_) && sph_step_node(s, id, -1, pv))) {
        atomicOr((int *)&a.counters[TC_ERR], OV_EW_WALK);
        return;
    }
    double l_next = sph_wrapped_len(a.geo, p, nx_);
    double l_prev = sph_wrapped_len(a.geo, pv, p);
    const double hi = rn_mul(4.0, s.dl_max), lo = rn_div(s.dl_min, 4.0);
    if (l_next > hi) l_next = hi;
    if (l_prev > hi) l_prev = hi;
    if (l_next < lo) l_next = lo;
    if (l_prev < lo) l_prev = lo;
    const double f = rn_div(
        rn_div(rn_mul(s.kappa, log(rn_div(rn_div(rn_mul(2.0, sqrt(rn_mul(l_next, l_prev))), sqrt(M_E)), s.a0))), 4.0),
        M_PI);
    const double tg[3] = {a.tx[id], a.ty[id], a.tz[id]}, nm[3] = {a.nx[id], a.ny[id], a.nz[id]};
    double vs[3] = {rn_mul(rn_sub(rn_mul(tg[1], nm[2]), rn_mul(tg[2], nm[1])), f),
                    rn_mul(rn_sub(rn_mul(tg[2], nm[0]), rn_mul(tg[0], nm[2])), f),
                    rn_mul(rn_sub(rn_mul(tg[0], nm[1]), rn_mul(tg[1], nm[0])), f)};
    int terr = 0;
    double T = 0, rhat[3] = {0, 0, 0};
    const double rad = sph_radius(p);
    if (s.use_temperature) {
        T = helium::temperature(rad, s.t_bath, s.prof_a);
        sph_normalize(p, rhat);
        const double vsr = helium::vs_radial(rad, T, s.q_dot, &terr);
        for (int ax = 0; ax < 3; ++ax) vs[ax] = rn_add(vs[ax], rn_mul(rhat[ax], vsr));
    }
    for (int ax = 0; ax < 3; ++ax) vs[ax] = rn_add(vs[ax], own[ax]);
    for (int ax = 0; ax < 3; ++ax) vs[ax] = rn_add(vs[ax], tot[ax]);
    double vel[3] = {vs[0], vs[1], vs[2]};
    if (s.friction) {
        double dv[3] = {0, 0, 0}, al = s.alpha, alp = s.alpha_p;
        if (s.use_temperature) {
            const double vnr = helium::vn_radial(rad, T, s.q_dot, &terr);
            for (int ax = 0; ax < 3; ++ax) dv[ax] = rn_mul(rhat[ax], vnr);
            al = helium::friction_alpha(T, &terr);
            alp = helium::friction_alpha_p(T, &terr);
        }
        for (int ax = 0; ax < 3; ++ax) dv[ax] = rn_sub(dv[ax], vs[ax]);
        double c1[3] = {rn_sub(rn_mul(tg[1], dv[2]), rn_mul(tg[2], dv[1])), rn_sub(rn_mul(tg[2], dv[0]), rn_mul(tg[0], dv[2])),
                        rn_sub(rn_mul(tg[0], dv[1]), rn_mul(tg[1], dv[0]))};
        for (int ax = 0; ax < 3; ++ax) vel[ax] = rn_add(vel[ax], rn_mul(c1[ax], al));
        double c2[3] = {rn_sub(rn_mul(tg[1], c1[2]), rn_mul(tg[2], c1[1])), rn_sub(rn_mul(tg[2], c1[0]), rn_mul(tg[0], c1[2])),
                        rn_sub(rn_mul(tg[0], c1[1]), rn_mul(tg[1], c1[0]))};
        const double mm = -alp;
        for (int ax = 0; ax < 3; ++ax) vel[ax] = rn_add(vel[ax], rn_mul(c2[ax], mm));
    }
    if (st == OV_PINNED_SLIP) {
        // surface_normal (boundaries.c:13-27 of the fork): outward from the inner surface
        double n[3];
        sph_normalize(p, n);
        if (a.pin[id] != 0) for (int ax = 0; ax < 3; ++ax) n[ax] = rn_mul(n[ax], -1.0);
        const double nv = dot3_ref(n[0], n[1], n[2], vel[0], vel[1], vel[2]);
        for (int ax = 0; ax < 3; ++ax) vel[ax] = rn_sub(vel[ax], rn_mul(n[ax], nv));
    }
    if (terr) atomicOr((int *)&a.counters[TC_ERR], OV_EW_TEMP);
    a.sx[id] = vs[0]; a.sy[id] = vs[1]; a.sz[id] = vs[2];
    a.vx[id] = vel[0]; a.vy[id] = vel[1]; a.vz[id] = vel[2];
}

SphArgs make_sph_args(ov_ctx *c, const SphDomain &d, const SphSettings &p)
{
    SphArgs s;
    s.v = make_args(c, c->node, 0.0, ov_stat_ptr(c));
    s.v.tid = nullptr; s.v.tprm = nullptr; s.v.mrange = nullptr; s.v.qorder = nullptr;
    s.n = d.n;
    s.ri = d.ri; s.ro = d.ro;
    s.d_az = 2 * d.az; s.d_pl = 2 * d.pl;
    s.kappa = p.kappa; s.a0 = p.a0; s.alpha = p.alpha; s.alpha_p = p.alpha_p;
    s.dl_min = p.dl_min; s.dl_max = p.dl_max;
    s.friction = p.friction; s.use_temperature = p.use_temperature;
    s.q_dot = p.q_dot; s.t_bath = p.t_bath; s.prof_a = p.prof_a;
    s.v.prm.theta = p.theta;
    s.v.f4pi = p.kappa / 4 / M_PI;
    return s;
}

}  // namespace

void ov_launch_sph_tangents(ov_ctx *c, const SphDomain &d, const SphSettings &p)
{
    SphArgs s = make_sph_args(c, d, p);
    k_sph_tangents<<<(d.n + 255) / 256, 256, 0, c->stream>>>(s, c->tree.counters);
    c->launches++;
}

void ov_launch_sph_images(ov_ctx *c, const SphDomain &d, const SphSettings &p)
{
    SphArgs s = make_sph_args(c, d, p);
    k_sph_images<<<(d.n + 255) / 256, 256, 0, c->stream>>>(s, c->node.x, c->node.y, c->node.z, c->tree.counters);
    c->launches++;
}

int ov_launch_sph_velocities(ov_ctx *c, const SphDomain &d, const SphSettings &p)
{
    SphArgs s = make_sph_args(c, d, p);
    const size_t need = (size_t)18 * 3 * (size_t)d.n;
    if (c->part_cap < need) {
        if (c->part) cudaFree(c->part);
        c->part = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->part, need * sizeof(double)));
        c->part_cap = need;
    }
    const long long warps = 18LL * ((d.n + 31) / 32);
    if (c->precision == OV_PREC_MIXED)
        k_sph_query_mixed<<<(unsigned)((warps + 3) / 4), 128, 0, c->stream>>>(s, c->part);
    else if (c->walk == OV_WALK_SPLIT)
        k_sph_query_split<<<(unsigned)((warps + 3) / 4), 128, 0, c->stream>>>(s, c->part);
    else
        k_sph_query<<<(unsigned)((warps + 3) / 4), 128, 0, c->stream>>>(s, c->part);
    k_sph_finish<<<(d.n + 127) / 128, 128, 0, c->stream>>>(s, c->part);
    c->launches += 2;
    return OV_OK;
}
