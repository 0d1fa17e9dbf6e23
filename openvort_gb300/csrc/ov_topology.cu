// ov_topology.cu - topology passes of the time step.
//
//  ov_reconnect           reconnect (vortex_dynamics.c:186-288)
//  ov_remesh              remesh + add_point + remove_point + slot allocation
//                         (tangle.c:1018-1061, 261-355, 201-253, 68-101)
//  ov_eliminate_small_loops (tangle.c:1063-1128)
//  ov_smooth              smooth / high_freq_cutoff / low_pass_filter
//                         (vortex_smooth.c:134-175, 183-453, 459-462)
//  ov_enforce_wall_boundaries  enforce_wall_boundaries + connect_to_wall
//                         (tangle.c:822-1016)
//  ov_add_loop, ov_add_line_in_zdir, ov_inject_vortices
//                         add_loop, add_line_in_zdir, inject_vortices
//                         (vortex_injection.c:18-100, 267-319, 702-800)
//  ov_step                one main-loop body (main.c:125-141)
//
// The reference's passes are sequential: a reconnection rewires connections
// that later candidates see, and remesh walks the slots in index order,
// visiting nodes it inserted in the same pass.  Those decisions are taken
// here on the host, in the reference's order and FP64 rounding, on host
// mirrors of positions and topology; the GPU does the parallel parts:
//   * reconnect: candidate pairs within rec_dist from a uniform grid over a
//     key sort of the nodes (cell side >= 2 rec_dist, so 27 neighbour cells
//     are enough even for nodes within rounding of a cell face), and the
//     O(N (1+n_img)) direct-sum velocities of every candidate node in one
//     batch, in mixed precision with a rigorous error bound; rewiring
//     changes four segments, whose contributions are added to every
//     remaining candidate of the member on the device; a decision the bound
//     cannot settle gets FP64 sums, and one whose dx.dv is still within the
//     error of the reference's own summation is recomputed in the
//     reference's summation order;
//   * smoothing: one block per closed loop (the loop decomposition is host
//     work): unwrap, optional detrend / odd extension, low-pass DFT on the
//     kept bins only, write back.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <chrono>
#include <vector>

#include "ov_internal.cuh"

#include <queue>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_E
#define M_E 2.7182818284590452354
#endif


namespace {

// ------------------------------------------------------------ host math
// vec3_math.c operation order; this file's host code is compiled with
// -ffp-contract=off.
inline double hdot(const double a[3], const double b[3])
{
    double o = 0;
    o += a[0] * b[0];
    o += a[1] * b[1];
    o += a[2] * b[2];
    return o;
}
inline double hlen(const double a[3]) { return sqrt(hdot(a, a)); }
inline void hsub(double r[3], const double a[3], const double b[3])
{
    for (int i = 0; i < 3; ++i) r[i] = a[i] - b[i];
}
inline void hcross(double r[3], const double u[3], const double v[3])
{
    double a0 = u[1] * v[2] - u[2] * v[1], a1 = u[2] * v[0] - u[0] * v[2], a2 = u[0] * v[1] - u[1] * v[0];
    r[0] = a0; r[1] = a1; r[2] = a2;
}

// seg_pwrap (boundaries.c:54-83)
inline void hpwrap(const Geometry &g, const double r1[3], double r2[3])
{
    for (int a = 0; a < 3; ++a) {
        if (!g.periodic[a]) continue;
        double L = g.L[a];
        int guard = 0;
        while ((r2[a] - r1[a]) > L / 2 && guard++ < 1000) r2[a] -= L;
        while ((r2[a] - r1[a]) < -L / 2 && guard++ < 2000) r2[a] += L;
    }
}
// segment_len of seg_pwrap(r1, r2): |r1 - r2'|
inline double hpwrap_len(const Geometry &g, const double r1[3], const double r2in[3])
{
    double r2[3] = {r2in[0], r2in[1], r2in[2]};
    hpwrap(g, r1, r2);
    double d[3];
    hsub(d, r1, r2);
    return hlen(d);
}

// Host mirror of the pool, seen from one member: its visible slots
// [lo, hi) and its parameters.  Indices stay pool slots.
struct Host {
    ov_ctx *c;
    int lo, hi;
    const ov_params *P;
    int N() const { return c->n_live; }
    void pos(int i, double p[3]) const { p[0] = c->h_x[i]; p[1] = c->h_y[i]; p[2] = c->h_z[i]; }
    int &fwd(int i) { return c->h_fwd[i]; }
    int &rev(int i) { return c->h_rev[i]; }
    int &st(int i) { return c->h_status[i]; }
    int &pin(int i) { return c->h_pin[i]; }
};

inline bool pinned(int s) { return s == OV_PINNED || s == OV_PINNED_SLIP; }

inline Host host_of(ov_ctx *c, int mi)
{
    const Member &m = c->mem[mi];
    return Host{c, m.lo, m.lo + m.n, &m.params};
}

// step_node (tangle.c:155-194)
bool hstep(Host &h, int i, int where, double out[3])
{
    int walls[8], nw = 0, cur = i, w = where;
    for (int guard = 0; w != 0; ++guard) {
        if (guard > 16 || cur < 0 || cur >= h.N()) return false;
        int s = h.st(cur);
        if (s == OV_FREE) {
            cur = w > 0 ? h.fwd(cur) : h.rev(cur);
            w += w > 0 ? -1 : 1;
        } else if (pinned(s)) {
            int nb = w > 0 ? h.fwd(cur) : h.rev(cur);
            if (nb >= 0) { cur = nb; w += w > 0 ? -1 : 1; }
            else {
                if (nw >= 8) return false;
                walls[nw++] = h.pin(cur);
                w = -w;
            }
        } else {
            return false;
        }
    }
    if (cur < 0 || cur >= h.N() || h.st(cur) == OV_EMPTY) return false;
    h.pos(cur, out);
    const Geometry &g = h.c->geo;
    for (int m = nw - 1; m >= 0; --m) {
        int f = walls[m];
        if (f < 0 || f > 5) continue;
        int ax = f >> 1;
        double wp = (f & 1) ? g.hi[ax] : g.lo[ax];
        out[ax] = 2 * wp - out[ax];
    }
    return true;
}

// update_tangent_normal (tangle.c:423-502)
bool htangent(Host &h, int k, double tg[3], double nm[3])
{
    const Geometry &g = h.c->geo;
    double s0[3], s1[3], s2[3], sm1[3], sm2[3];
    h.pos(k, s0);
    if (!(hstep(h, k, 1, s1) && hstep(h, k, 2, s2) && hstep(h, k, -1, sm1) && hstep(h, k, -2, sm2))) return false;
    double w2[3] = {s2[0], s2[1], s2[2]}, w1[3] = {s1[0], s1[1], s1[2]};
    double wm1[3] = {sm1[0], sm1[1], sm1[2]}, wm2[3] = {sm2[0], sm2[1], sm2[2]};
    hpwrap(g, s0, w2); hpwrap(g, s0, w1); hpwrap(g, s0, wm1); hpwrap(g, s0, wm2);
    double ds[4][3];
    hsub(ds[0], w2, s0); hsub(ds[1], w1, s0); hsub(ds[2], wm1, s0); hsub(ds[3], wm2, s0);
    double t1[3], t2[3];
    hsub(t1, s0, w1);
    double d1 = hlen(t1);
    double d2 = d1 + hpwrap_len(g, s1, s2);
    hsub(t2, s0, wm1);
    double dm1 = hlen(t2);
    double dm2 = dm1 + hpwrap_len(g, sm1, sm2);
    double den[4] = {d2 * (d2 - d1) * (dm1 + d2) * (dm2 + d2), d1 * (d2 - d1) * (dm1 + d1) * (dm2 + d1),
                     dm1 * (dm1 + d1) * (dm1 + d2) * (dm2 - dm1), dm2 * (dm2 + d1) * (dm2 + d2) * (dm2 - dm1)};
    double c1[4] = {-d1 * dm1 * dm2, d2 * dm1 * dm2, -d1 * d2 * dm2, d1 * d2 * dm1};
    double c2[4] = {2 * ((dm1 - d1) * dm2 - d1 * dm1), -2 * ((dm1 - d2) * dm2 - d2 * dm1),
                    2 * ((d2 + d1) * dm2 - d1 * d2), -2 * ((d2 + d1) * dm1 - d1 * d2)};
    for (int a = 0; a < 3; ++a) {
        double tt = 0, nn = 0;
        for (int z = 0; z < 4; ++z) {
            tt += c1[z] / den[z] * ds[z][a];
            nn += c2[z] / den[z] * ds[z][a];
        }
        tg[a] = tt;
        nm[a] = nn;
    }
    return true;
}

// get_v (external_velocity.c:62-81)
void hext(const ov_ext_vel &e, double t, double out[3])
{
    out[0] = out[1] = out[2] = 0;
    if (e.type != OV_SIMPLE && e.type != OV_DECREASING) return;
    double d[3] = {e.direction.p[0], e.direction.p[1], e.direction.p[2]};
    if (!(d[0] == 0 && d[1] == 0 && d[2] == 0)) {
        double inv = 1 / hlen(d);
        for (int a = 0; a < 3; ++a) d[a] = d[a] * inv;
    }
    double s = e.strength;
    if (e.type == OV_DECREASING && t < e.time_of_linear_decrease)
        s = e.starting_strength - t * (e.starting_strength - e.strength) / e.time_of_linear_decrease;
    for (int a = 0; a < 3; ++a) out[a] = d[a] * s;
}

// the segment law of segment_field (tangle.c:536-559)
bool hlaw(const double R[3], const double Rp1[3], double kappa, double out[3])
{
    double lR = hlen(R), lRp1 = hlen(Rp1);
    double denom = lR * lRp1 * (lR * lRp1 + hdot(R, Rp1));
    double f = kappa / 4 / M_PI;
    if (lR < 1e-8 || lRp1 < 1e-8) return false;
    if (hdot(R, Rp1) / hlen(R) / hlen(Rp1) < 1e-8) return false;
    double cr[3];
    hcross(cr, R, Rp1);
    double m = f * (lR + lRp1) / denom;
    for (int a = 0; a < 3; ++a) out[a] = cr[a] * m;
    return true;
}

// shifted (tangle.c:370-414)
void himage(const Geometry &g, int j, const double p[3], double q[3])
{
    for (int a = 0; a < 3; ++a) q[a] = p[a] - g.L[a] * g.shift[j][a];
    for (int m = 0; m < g.nreflect[j]; ++m) {
        int f = g.reflect[j][m];
        if (f < 0 || f > 5) continue;
        int ax = f >> 1;
        double w = (f & 1) ? g.hi[ax] : g.lo[ax];
        q[ax] = 2 * w - p[ax];
    }
}

// contribution of segment m -> f at point r (segment_field)
bool hsegment(Host &h, int m, int f, const double r[3], double out[3])
{
    double a[3], b[3];
    h.pos(m, a);
    h.pos(f, b);
    hpwrap(h.c->geo, a, b);
    double R[3], Rp1[3];
    hsub(R, a, r);
    hsub(Rp1, b, r);
    return hlaw(R, Rp1, h.P->kappa, out);
}

// lia_velocity (tangle.c:568-592) + external v_s, given tangent/normal
bool hlia(Host &h, int i, const double tg[3], const double nm[3], double t, double vs[3])
{
    double p[3], nx[3], pv[3];
    h.pos(i, p);
    if (!(hstep(h, i, 1, nx) && hstep(h, i, -1, pv))) return false;
    const ov_params &P = *h.P;
    double l_next = hpwrap_len(h.c->geo, p, nx);
    double l_prev = hpwrap_len(h.c->geo, pv, p);
    double f = P.kappa * log(2 * sqrt(l_next * l_prev) / sqrt(M_E) / P.vortex_width) / 4 / M_PI;
    double cr[3];
    hcross(cr, tg, nm);
    double ev[3];
    hext(P.vs, t, ev);
    for (int a = 0; a < 3; ++a) vs[a] = cr[a] * f + ev[a];
    return true;
}

// vels from vs: mutual friction and PINNED_SLIP (tangle.c:694-725)
void hfriction(Host &h, int k, const double tg[3], const double vs[3], double t, double vel[3])
{
    const ov_params &P = *h.P;
    for (int a = 0; a < 3; ++a) vel[a] = vs[a];
    if (P.use_mutual_friction) {
        double vn[3], dv[3], c1[3], c2[3];
        hext(P.vn, t, vn);
        hsub(dv, vn, vs);
        hcross(c1, tg, dv);
        for (int a = 0; a < 3; ++a) vel[a] = vel[a] + c1[a] * P.alpha;
        hcross(c2, tg, c1);
        for (int a = 0; a < 3; ++a) vel[a] = vel[a] + c2[a] * -P.alpha_p;
    }
    if (h.st(k) == OV_PINNED_SLIP) {
        int f = h.pin(k);
        if (f >= 0 && f < 6) {
            int ax = f >> 1;
            double n = (f & 1) ? -1.0 : 1.0;
            double nv = n * vel[ax];
            vel[ax] = vel[ax] - n * nv;
        }
    }
}

// update_velocity(k, tree=NULL) exactly as the reference sums it: into vs in
// segment-index order, primary then images.
bool hdirect_exact(Host &h, int k, const double tg[3], const double nm[3], double t, double vel[3])
{
    double vs[3];
    if (!hlia(h, k, tg, nm, t, vs)) return false;
    double x[3];
    h.pos(k, x);
    const Geometry &g = h.c->geo;
    for (int m = h.lo; m < h.hi; ++m) {
        int f = h.fwd(m);
        if (f == -1 || k == m || k == f) continue;
        double w[3];
        if (hsegment(h, m, f, x, w))
            for (int a = 0; a < 3; ++a) vs[a] = vs[a] + w[a];
    }
    for (int j = 0; j < g.n_img; ++j) {
        double q[3];
        himage(g, j, x, q);
        for (int m = h.lo; m < h.hi; ++m) {
            int f = h.fwd(m);
            if (f == -1) continue;
            double w[3];
            if (hsegment(h, m, f, q, w))
                for (int a = 0; a < 3; ++a) vs[a] = vs[a] + w[a];
        }
    }
    hfriction(h, k, tg, vs, t, vel);
    return true;
}

// ------------------------------------------------------------- GPU parts
struct GridGeom {
    double lo[3], L[3];
    int n[3];
    int periodic[3];
};

__global__ void k_grid_keys(const int *__restrict__ status, const double *__restrict__ x,
                            const double *__restrict__ y, const double *__restrict__ z, int n_live, int cap,
                            GridGeom gg, uint64_t *__restrict__ keys, int *__restrict__ idx)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    idx[i] = i;
    int s = i < n_live ? status[i] : OV_EMPTY;
    if (s != OV_FREE) { keys[i] = ~0ull; return; }
    double p[3] = {x[i], y[i], z[i]};
    unsigned cell[3];
    for (int a = 0; a < 3; ++a) {
        double u = (p[a] - gg.lo[a]) / gg.L[a];
        u -= floor(u);
        int ci = (int)(u * gg.n[a]);
        cell[a] = (unsigned)min(max(ci, 0), gg.n[a] - 1);
    }
    uint64_t cid = ((uint64_t)cell[2] * gg.n[1] + cell[1]) * gg.n[0] + cell[0];
    keys[i] = (cid << 32) | (uint64_t)i;
}

__device__ __forceinline__ int lower_key(const uint64_t *keys, int n, uint64_t v)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (keys[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void k_pairs(const uint64_t *__restrict__ keys, const int *__restrict__ idx, int cap,
                        const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                        GridGeom gg, Geometry geo, double rec_dist, const int *__restrict__ tid,
                        const DevParams *__restrict__ tprm, int *__restrict__ pairs, int *npairs, int pair_cap)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    uint64_t key = keys[i];
    if (key == ~0ull) return;
    int k = idx[i];
    const int mk = tid ? tid[k] : 0;   // pairs within one member, at its rec_dist
    if (tid) rec_dist = tprm[mk].rec_dist;
    uint64_t cid = key >> 32;
    int c[3] = {(int)(cid % gg.n[0]), (int)((cid / gg.n[0]) % gg.n[1]), (int)(cid / ((uint64_t)gg.n[0] * gg.n[1]))};
    double pk[3] = {x[k], y[k], z[k]};
    int lo3[3], hi3[3];
    for (int a = 0; a < 3; ++a) {
        if (gg.n[a] >= 3) { lo3[a] = -1; hi3[a] = 1; }
        else if (gg.n[a] == 2) { lo3[a] = 0; hi3[a] = 1; }
        else { lo3[a] = 0; hi3[a] = 0; }
    }
    for (int dz = lo3[2]; dz <= hi3[2]; ++dz)
        for (int dy = lo3[1]; dy <= hi3[1]; ++dy)
            for (int dx = lo3[0]; dx <= hi3[0]; ++dx) {
                int nc[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
                bool skip = false;
                for (int a = 0; a < 3; ++a) {
                    if (gg.n[a] <= 2) { nc[a] = ((nc[a] % gg.n[a]) + gg.n[a]) % gg.n[a]; continue; }
                    if (nc[a] < 0 || nc[a] >= gg.n[a]) {
                        if (!gg.periodic[a]) skip = true;
                        nc[a] = (nc[a] + gg.n[a]) % gg.n[a];
                    }
                }
                if (skip) continue;
                uint64_t ncid = ((uint64_t)nc[2] * gg.n[1] + nc[1]) * gg.n[0] + nc[0];
                int b = lower_key(keys, cap, ncid << 32), e = lower_key(keys, cap, (ncid + 1) << 32);
                for (int j = b; j < e; ++j) {
                    int l = idx[j];
                    if (l <= k) continue;
                    if (tid && tid[l] != mk) continue;
                    double v2[3] = {x[l], y[l], z[l]};
                    pwrap_dev(geo, pk, v2);
                    double d = len3_ref(rn_sub(pk[0], v2[0]), rn_sub(pk[1], v2[1]), rn_sub(pk[2], v2[2]));
                    if (d > rec_dist) continue;
                    int slot = atomicAdd(npairs, 1);
                    if (slot < pair_cap) { pairs[2 * slot] = k; pairs[2 * slot + 1] = l; }
                }
            }
}

// remesh (tangle.c:1018-1061): the slots whose lengths could make the pass
// act (remove or insert), for the host pass to visit in index order.  The
// thresholds are widened by 1e-9 relative, so the list holds every slot the
// reference's tests would act on; the host redoes each test exactly.
__global__ void k_remesh_flags(const int *__restrict__ status, const int *__restrict__ fwd,
                               const int *__restrict__ rev, const double *__restrict__ x,
                               const double *__restrict__ y, const double *__restrict__ z,
                               const int *__restrict__ tid, const double *__restrict__ lim, int nmem, Geometry geo,
                               int n, int *__restrict__ list, int *__restrict__ count, int cap_list)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || status[s] == OV_EMPTY) return;
    const int m = tid ? tid[s] : 0;
    const int nx = fwd[s], pv = rev[s];
    bool act;
    if (m < 0 || m >= nmem || nx >= n || pv >= n) {
        act = true;   // let the host see it
    } else {
        const double mn = lim[2 * m], mx = lim[2 * m + 1];
        const double p[3] = {x[s], y[s], z[s]};
        double lf = 0, lr = 0;
        if (nx >= 0) {
            double q[3] = {x[nx], y[nx], z[nx]};
            pwrap_dev(geo, p, q);
            lf = len3_ref(rn_sub(p[0], q[0]), rn_sub(p[1], q[1]), rn_sub(p[2], q[2]));
        }
        if (pv >= 0) {
            double q[3] = {x[pv], y[pv], z[pv]};
            pwrap_dev(geo, p, q);
            lr = len3_ref(rn_sub(p[0], q[0]), rn_sub(p[1], q[1]), rn_sub(p[2], q[2]));
        }
        const double up = 1.0 + 1e-9, dn = 1.0 - 1e-9;
        act = (nx >= 0 && pv >= 0 && (lf < mn * up || lr < mn * up) && (lf + lr) < mx * up) ||
              (nx >= 0 && lf > mx * dn);
    }
    if (act) {
        const int i = atomicAdd(count, 1);
        if (i < cap_list) list[i] = s;
    }
}

// eliminate_small_loops (tangle.c:1063-1128): the slots of structures the
// pass could remove from (a closed loop of at most `cutoff` nodes, or a slot
// fewer than `cutoff` forward steps from an open end or a link out of range),
// for the host pass to visit from each structure's first slot.
__global__ void k_small_flags(const int *__restrict__ status, const int *__restrict__ fwd, int n, int cutoff,
                              int *__restrict__ list, int *__restrict__ count, int cap_list)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || status[k] == OV_EMPTY) return;
    bool flag = false;
    int here = k;
    for (int st = 0; st < cutoff; ++st) {
        const int nx = fwd[here];
        if (nx < 0 || nx >= n || nx == k) { flag = true; break; }
        here = nx;
    }
    if (flag) {
        const int i = atomicAdd(count, 1);
        if (i < cap_list) list[i] = k;
    }
}

__global__ void k_zero_vel(const int *__restrict__ ids, int n, double *vx, double *vy, double *vz, double *sx,
                           double *sy, double *sz)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = ids[i];
    vx[k] = vy[k] = vz[k] = 0;
    sx[k] = sy[k] = sz[k] = 0;
}

// ---- smoothing: one block per closed loop
struct SmoothArgs {
    const int *loop_off, *loop_nodes;
    double *x, *y, *z;
    double *buf;               // 3 * 2 * total nodes
    Geometry geo;
    const double *cutoff;      // freq_to_cutoff of each loop's member
};

__global__ void __launch_bounds__(256) k_smooth(SmoothArgs a)
{
    const int lp = blockIdx.x;
    const int b0 = a.loop_off[lp], len = a.loop_off[lp + 1] - b0;
    const int *nodes = a.loop_nodes + b0;
    double *X[3];
    for (int ax = 0; ax < 3; ++ax) X[ax] = a.buf + (size_t)(2 * b0) * 3 + (size_t)ax * 2 * len;
    __shared__ int s_detrend, s_n;
    __shared__ double s_coef[3], s_c0[3];
    if (threadIdx.x == 0) {
        // unwrap along the loop (vortex_smooth.c:218-242)
        int k = nodes[0];
        double prev[3] = {a.x[k], a.y[k], a.z[k]};
        for (int ax = 0; ax < 3; ++ax) X[ax][0] = prev[ax];
        for (int j = 1; j < len; ++j) {
            int m = nodes[j];
            double r2[3] = {a.x[m], a.y[m], a.z[m]};
            double r1[3] = {X[0][j - 1], X[1][j - 1], X[2][j - 1]};
            pwrap_dev(a.geo, r1, r2);
            for (int ax = 0; ax < 3; ++ax) X[ax][j] = r2[ax];
        }
        double gx = X[0][0] - X[0][len - 1], gy = X[1][0] - X[1][len - 1], gz = X[2][0] - X[2][len - 1];
        double gap = sqrt(gx * gx + gy * gy + gz * gz);
        s_detrend = (gap > a.geo.L[0] / 2 && len > 2) ? 1 : 0;
        s_n = s_detrend ? 2 * len - 2 : len;
        if (s_detrend) {
            for (int ax = 0; ax < 3; ++ax) {
                s_coef[ax] = (X[ax][len - 1] - X[ax][0]) / (len - 1);
                s_c0[ax] = X[ax][0];
            }
        }
    }
    __syncthreads();
    const int N = s_n;
    if (s_detrend) {
        // vortex_smooth.c:252-279: subtract the chord, odd extension
        for (int j = threadIdx.x; j < len; j += blockDim.x)
            for (int ax = 0; ax < 3; ++ax)
                X[ax][j] = (j == 0 || j == len - 1) ? 0.0 : X[ax][j] - s_coef[ax] * j - s_c0[ax];
        __syncthreads();
        for (int j = threadIdx.x; j < len - 2; j += blockDim.x)
            for (int ax = 0; ax < 3; ++ax) X[ax][len + j] = -X[ax][len - 2 - j];
        __syncthreads();
    }
    // low_pass_filter (vortex_smooth.c:134-175) on the kept half-complex bins
    int cut = (int)(a.cutoff[lp] * N / 2);
    int zlo = 0, zhi = 0;
    if (N > 2 * cut + 1) {
        zlo = N / 2 - cut;
        zhi = (N % 2 == 0) ? N / 2 + 1 + cut : N / 2 + cut;
    }
    // dynamic shared memory: twiddles cos/sin(2 pi m / N) for m in [0, N),
    // cosine bins [0, N/2] and sine bins [1, (N-1)/2] per coordinate
    extern __shared__ double sh[];
    const int ncos = N / 2 + 1, nsin = (N - 1) / 2;
    double *TC = sh, *TS = sh + N;
    double *RC = sh + 2 * N, *IS = RC + 3 * ncos;   // [ax][k]
    for (int m = threadIdx.x; m < N; m += blockDim.x) sincospi(2.0 * (double)m / N, &TS[m], &TC[m]);
    __syncthreads();
    for (int kk = threadIdx.x; kk < ncos + nsin; kk += blockDim.x) {
        bool is_cos = kk < ncos;
        int k = is_cos ? kk : kk - ncos + 1;
        int hcidx = is_cos ? k : N - k;
        bool kept = !(hcidx >= zlo && hcidx < zhi);
        double acc[3] = {0, 0, 0};
        if (kept) {
            int m = 0;
            for (int j = 0; j < N; ++j) {
                double tw = is_cos ? TC[m] : -TS[m];
                for (int ax = 0; ax < 3; ++ax) acc[ax] += X[ax][j] * tw;
                m += k;
                if (m >= N) m -= N;
            }
        }
        for (int ax = 0; ax < 3; ++ax) {
            if (is_cos) RC[ax * ncos + k] = acc[ax];
            else IS[ax * nsin + (k - 1)] = acc[ax];
        }
    }
    __syncthreads();
    // highest bin that survived the cut (bins above it are all zero)
    int kmax = (zhi > zlo) ? max(zlo - 1, N - zhi) : N / 2;
    for (int j = threadIdx.x; j < len; j += blockDim.x) {
        double s[3] = {RC[0], RC[ncos], RC[2 * ncos]};
        int m = 0;
        for (int k = 1; k < N - k && k <= kmax; ++k) {
            m += j;
            if (m >= N) m -= N * (m / N);
            double cv = TC[m], sv = TS[m];
            for (int ax = 0; ax < 3; ++ax) s[ax] += 2 * (RC[ax * ncos + k] * cv - IS[ax * nsin + (k - 1)] * sv);
        }
        if (N % 2 == 0)
            for (int ax = 0; ax < 3; ++ax) s[ax] += RC[ax * ncos + N / 2] * ((j % 2) ? -1.0 : 1.0);
        double out[3];
        for (int ax = 0; ax < 3; ++ax) {
            out[ax] = s[ax] / N;
            if (s_detrend) out[ax] = out[ax] + s_coef[ax] * j + s_c0[ax];
        }
        int node = nodes[j];
        a.x[node] = out[0]; a.y[node] = out[1]; a.z[node] = out[2];
    }
}

// ---- smoothing of long loops: Bluestein DFT on an FP64 Stockham FFT
//
// A loop too long for one block's shared memory is low-pass filtered with
// the same half-complex bin mask through an exact DFT of its (arbitrary)
// length N written as a convolution of length M = 2^p >= 2N - 1 (Bluestein):
//   X_k = conj(w_k) sum_n (x_n conj(w_n)) w_(k-n),  w_n = exp(i pi n^2 / N),
// the convolution done by radix-2 Stockham FFTs (ping-pong buffers, twiddle
// table exp(-2 pi i t / M) computed once per M), the inverse by conjugation.
// Three coordinates go through each pass as a batch.

// exp(i pi n^2 / N) with n^2 reduced mod 2N exactly
__device__ __forceinline__ double2 chirp(long long n, long long N)
{
    long long r = (n * n) % (2 * N);
    double s, c;
    sincospi((double)r / (double)N, &s, &c);
    return make_double2(c, s);
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void k_twiddles(double2 *tw, int M)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M / 2) return;
    double s, c;
    sincospi(-2.0 * (double)t / (double)M, &s, &c);
    tw[t] = make_double2(c, s);
}

// b_n = w_n for |n| < N (wrapped into [0, M)), else 0
__global__ void k_chirp_filter(double2 *b, int N, int M)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= M) return;
    double2 v = make_double2(0, 0);
    if (n < N) v = chirp(n, N);
    else if (n > M - N) v = chirp(M - n, N);
    b[n] = v;
}

// a[c][n] = in[c][n] conj(w_n) (n < N), zero padded to M; in is complex
// (stride N per coordinate) or, when re != nullptr, real
__global__ void k_chirp_in(const double *re, const double2 *in, int N, int M, double2 *a)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (n >= M) return;
    double2 v = make_double2(0, 0);
    if (n < N) {
        double2 x = re ? make_double2(re[(size_t)c * N + n], 0.0) : in[(size_t)c * N + n];
        double2 w = chirp(n, N);
        v = cmul(x, make_double2(w.x, -w.y));
    }
    a[(size_t)c * M + n] = v;
}

// one radix-2 Stockham pass over `batch` sequences of length M
__global__ void k_fft_pass(const double2 *__restrict__ in, double2 *__restrict__ out, const double2 *__restrict__ tw,
                           int M, int Ns)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (j >= M / 2) return;
    const double2 *x = in + (size_t)c * M;
    double2 *y = out + (size_t)c * M;
    int k = j & (Ns - 1);
    double2 w = tw[(size_t)k * (M / (2 * Ns))];
    double2 v0 = x[j], v1 = cmul(x[j + M / 2], w);
    int d = ((j - k) << 1) + k;
    y[d] = make_double2(v0.x + v1.x, v0.y + v1.y);
    y[d + Ns] = make_double2(v0.x - v1.x, v0.y - v1.y);
}

// A[c] <- conj(A[c] * B) (the inverse transform runs as a forward one on
// the conjugate)
__global__ void k_conv_mul(double2 *A, const double2 *__restrict__ B, int M)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (n >= M) return;
    double2 v = cmul(A[(size_t)c * M + n], B[n]);
    A[(size_t)c * M + n] = make_double2(v.x, -v.y);
}

// X_k = conj(w_k) conj(c_k) / M for k < N (c = FFT of the conjugated product)
__global__ void k_chirp_out(const double2 *cbuf, int N, int M, double2 *X)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (k >= N) return;
    double2 v = cbuf[(size_t)c * M + k];
    v = make_double2(v.x / M, -v.y / M);
    double2 w = chirp(k, N);
    X[(size_t)c * N + k] = cmul(v, make_double2(w.x, -w.y));
}

// The reference's half-complex mask (vortex_smooth.c:146-160): element h of
// the R2HC array (real part of bin h for h <= N/2, imaginary part of bin
// N - h above) is zeroed for h in [zlo, zhi); the spectrum stays Hermitian.
// Writes conj(X') for the inverse transform.
__global__ void k_lowpass_mask(double2 *X, int N, int zlo, int zhi)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (k >= N) return;
    int kk = k <= N / 2 ? k : N - k;   // bin of the half-complex pair
    double2 v = X[(size_t)c * N + k];
    bool keep_re = !(kk >= zlo && kk < zhi);
    bool keep_im = kk == 0 || (2 * kk == N) || !((N - kk) >= zlo && (N - kk) < zhi);
    if (kk == 0 || 2 * kk == N) v.y = 0;
    if (!keep_re) v.x = 0;
    if (!keep_im) v.y = 0;
    X[(size_t)c * N + k] = make_double2(v.x, -v.y);
}

// positions of the loop from the filtered sequence: out = Re(y)/N (+ the
// chord of a detrended loop)
__global__ void k_long_writeback(const double2 *__restrict__ Y, int N, int len, const int *__restrict__ nodes,
                                 int detrend, double cx, double cy, double cz, double ox, double oy, double oz,
                                 double *x, double *y, double *z, int cap)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= len) return;
    int node = nodes[j];
    if (node < 0 || node >= cap) return;
    // Y = FFT(conj X') conjugated and / N on read: x_j = Re(conj(Y_j)) / N
    double o[3];
    const double co[3] = {cx, cy, cz}, c0[3] = {ox, oy, oz};
    for (int a = 0; a < 3; ++a) {
        o[a] = Y[(size_t)a * N + j].x / N;
        if (detrend) o[a] = o[a] + co[a] * j + c0[a];
    }
    x[node] = o[0]; y[node] = o[1]; z[node] = o[2];
}

}  // namespace

// ------------------------------------------------------------ host mirror
int ov_pull_host(ov_ctx *c)
{
    int n = c->n_live;
    if (c->host_valid && (int)c->h_x.size() == n && (int)c->h_status.size() == n) {
        c->h_recalc.assign(n, 0);
        return OV_OK;   // nothing changed positions or topology since the last pull / push
    }
    c->host_valid = false;
    c->h_x.resize(n); c->h_y.resize(n); c->h_z.resize(n);
    c->h_fwd.resize(n); c->h_rev.resize(n); c->h_status.resize(n); c->h_pin.resize(n);
    c->h_recalc.assign(n, 0);
    if (n == 0) return OV_OK;
    double *dd[3] = {c->node.x, c->node.y, c->node.z};
    double *hd[3] = {c->h_x.data(), c->h_y.data(), c->h_z.data()};
    for (int a = 0; a < 3; ++a)
        OV_CUDA(c, cudaMemcpyAsync(hd[a], dd[a], (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
    int *di[4] = {c->fwd, c->rev, c->status, c->pin};
    int *hi[4] = {c->h_fwd.data(), c->h_rev.data(), c->h_status.data(), c->h_pin.data()};
    for (int a = 0; a < 4; ++a)
        OV_CUDA(c, cudaMemcpyAsync(hi[a], di[a], (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    c->host_valid = true;
    return OV_OK;
}

int ov_push_device(ov_ctx *c, int pos_too)
{
    int n = c->n_live;
    c->tree_built = false;
    c->host_valid = false;
    if (n > c->cap) {
        int r = ov_grow_preserving(c, n);
        if (r) return r;
    }
    if (n == 0) return OV_OK;
    if (pos_too) {
        double *dd[3] = {c->node.x, c->node.y, c->node.z};
        double *hd[3] = {c->h_x.data(), c->h_y.data(), c->h_z.data()};
        for (int a = 0; a < 3; ++a)
            OV_CUDA(c, cudaMemcpyAsync(dd[a], hd[a], (size_t)n * 8, cudaMemcpyHostToDevice, c->stream));
    }
    int *di[4] = {c->fwd, c->rev, c->status, c->pin};
    int *hi[4] = {c->h_fwd.data(), c->h_rev.data(), c->h_status.data(), c->h_pin.data()};
    for (int a = 0; a < 4; ++a)
        OV_CUDA(c, cudaMemcpyAsync(di[a], hi[a], (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    c->host_valid = true;   // positions were pushed, or are unchanged since the pull
    return OV_OK;
}

namespace {

int ready(ov_ctx *c)
{
    if (!c) return OV_ERR_ARG;
    if (!c->uploaded) return ov_fail(c, OV_ERR_STATE, "no tangle uploaded");
    cudaSetDevice(c->device);
    return OV_OK;
}

// ------------------------------------------------------- slot allocation
// expand_tangle (tangle.c:68-101) of member mi to n slots
int hexpand(ov_ctx *c, int mi, int n);

// Give member mi room for n visible slots: a single tangle grows its host
// arrays; an ensemble member past its reserved range gets a range of 2n
// slots and the members after it move up (host mirror now, device slots
// without a mirror right away; positions and topology follow on the push).
int hrelayout(ov_ctx *c, int mi, int n)
{
    Member &m = c->mem[mi];
    if (n <= m.cap) return OV_OK;
    const int newcap = c->mem.size() == 1 ? n : 2 * n;
    const int delta = newcap - m.cap;
    const int at = m.lo + m.cap;   // first slot after the member
    const int old_total = c->n_live;
    std::vector<Member> old = c->mem;
    auto grow_d = [&](std::vector<double> &v) { v.insert(v.begin() + at, (size_t)delta, 0.0); };
    auto grow_i = [&](std::vector<int> &v, int fill) { v.insert(v.begin() + at, (size_t)delta, fill); };
    grow_d(c->h_x); grow_d(c->h_y); grow_d(c->h_z);
    grow_i(c->h_fwd, -1); grow_i(c->h_rev, -1);
    grow_i(c->h_status, OV_EMPTY); grow_i(c->h_pin, OV_NOT_A_FACE);
    grow_i(c->h_recalc, 0);
    const int total = old_total + delta;
    for (int k = 0; k < total; ++k) {
        if (c->h_fwd[k] >= at) c->h_fwd[k] += delta;
        if (c->h_rev[k] >= at) c->h_rev[k] += delta;
    }
    m.cap = newcap;
    for (size_t j = mi + 1; j < c->mem.size(); ++j) c->mem[j].lo += delta;
    c->n_live = total;
    if (c->mem.size() == 1) return OV_OK;   // a single tangle grows on the push
    int r;
    if (total > c->cap && (r = ov_grow_preserving(c, total))) return r;
    if ((r = ov_move_device_slots(c, old))) return r;
    return ov_upload_member_tables(c);
}

// search_next_empty_node (tangle.c:201-234) in member mi (returns a pool
// slot); a slot past the member's end counts as not empty where the
// reference reads status[k+1] out of bounds.
int hsearch_empty(ov_ctx *c, int mi)
{
    Member &m = c->mem[mi];
    Host h = host_of(c, mi);
    const int N = m.n, lo = m.lo;
    if (m.next_empty > 0) {
        if (m.next_empty < N && h.st(lo + m.next_empty) == OV_EMPTY) {
            int id = m.next_empty;
            if (m.next_empty + 1 < N && h.st(lo + m.next_empty + 1) == OV_EMPTY) ++m.next_empty;
            else m.next_empty = -1;
            return lo + id;
        }
    }
    for (int k = 0; k < N; ++k) {
        if (h.st(lo + k) == OV_EMPTY) {
            m.next_empty = (k + 1 < N && h.st(lo + k + 1) == OV_EMPTY) ? k + 1 : -1;
            return lo + k;
        }
    }
    return -1;
}

// get_next_empty_node (tangle.c:241-253); -1 when the pool cannot grow
int hget_empty(ov_ctx *c, int mi)
{
    int id = hsearch_empty(c, mi);
    for (int guard = 0; id < 0 || c->h_status[id] != OV_EMPTY; ++guard) {
        int n = c->mem[mi].n;
        if (guard > 40 || hexpand(c, mi, 2 * n > 0 ? 2 * n : 1)) return -1;
        id = hsearch_empty(c, mi);
    }
    return id;
}

int hexpand(ov_ctx *c, int mi, int n)
{
    int r = hrelayout(c, mi, n);
    if (r) return r;
    Member &m = c->mem[mi];
    const int old = m.n;
    for (int k = m.lo + old; k < m.lo + n; ++k) {
        c->h_status[k] = OV_EMPTY; c->h_pin[k] = OV_NOT_A_FACE;
        c->h_fwd[k] = -1; c->h_rev[k] = -1;
    }
    m.n = n;
    m.total_empty += n - old;
    int id = hget_empty(c, mi);
    if (id < 0) return ov_fail(c, OV_ERR_ALLOC, "member %d could not grow", mi);
    c->mem[mi].next_empty = id - c->mem[mi].lo;
    return OV_OK;
}

// out_of_box + periodic_shift (tangle.c:761-814, boundaries.c:113-150) on
// slots [lo, hi)
void hperiodic(ov_ctx *c, int lo, int hi)
{
    const Geometry &g = c->geo;
    for (int k = lo; k < hi; ++k) {
        if (c->h_status[k] == OV_EMPTY) continue;
        double p[3] = {c->h_x[k], c->h_y[k], c->h_z[k]};
        for (int guard = 0; guard < 1000; ++guard) {
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
            if (face % 2 == 0) p[ax] += g.L[ax];
            else p[ax] -= g.L[ax];
        }
        c->h_x[k] = p[0]; c->h_y[k] = p[1]; c->h_z[k] = p[2];
    }
}

// eliminate_small_loops (tangle.c:1063-1128) in member mi; returns nodes removed
// The pass over member mi, from the given first slots of its structures
// (sorted; every structure it could remove from): the reference visits a
// structure first at its lowest slot, and the others are left as they are.
int hsmall_loops(ov_ctx *c, int mi, const std::vector<int> &starts)
{
    Host h = host_of(c, mi);
    const int lo = h.lo, hi = h.hi, N = hi - lo;
    int removed = 0;
    if (starts.empty()) return 0;
    std::vector<char> seen(N > 0 ? N : 1, 0);
    auto mark = [&](int slot) { if (slot >= lo && slot < hi) seen[slot - lo] = 1; };
    for (int k : starts) {
        if (k < lo || k >= hi) continue;
        if (h.st(k) == OV_EMPTY || seen[k - lo]) continue;
        seen[k - lo] = 1;
        int steps = 0, here = k, nx = h.fwd(here);
        while (nx != k) {
            if (pinned(h.st(here)) && nx < 0) {
                here = k;
                nx = h.rev(here);
                while (nx >= 0) {
                    mark(here);
                    here = nx;
                    nx = h.rev(here);
                    steps++;
                }
                break;
            }
            if (nx < lo || nx >= hi) break;
            mark(here);
            here = nx;
            nx = h.fwd(here);
            steps++;
            if (steps > N) break;
        }
        if (steps < h.P->small_loop_cutoff) {
            nx = here;
            for (int guard = 0; guard <= N; ++guard) {
                int cur = nx;
                nx = h.fwd(nx);
                h.fwd(cur) = -1;
                h.rev(cur) = -1;
                h.st(cur) = OV_EMPTY;
                removed++;
                if (nx == here || nx < 0) break;
            }
        }
    }
    return removed;
}

// add_point (tangle.c:261-335) in member mi; -1 when no slot could be had
int hadd_point(ov_ctx *c, int mi, int p, std::vector<int> &new_nodes)
{
    int np = hget_empty(c, mi);
    if (np < 0) return -1;
    Host h = host_of(c, mi);
    h.st(np) = OV_FREE;
    h.pin(np) = OV_NOT_A_FACE;
    int nx = h.fwd(p);
    double tg[3], n0[3], n1[3];
    htangent(h, p, tg, n0);
    htangent(h, nx, tg, n1);
    double s0[3], s1[3];
    h.pos(p, s0);
    h.pos(nx, s1);
    hpwrap(c->geo, s0, s1);
    double dd[3];
    hsub(dd, s0, s1);
    double l = hlen(dd);
    double n[3], pos[3];
    for (int a = 0; a < 3; ++a) n[a] = (n0[a] + n1[a]) * 0.5;
    if (hlen(n) > 1e-5) {
        double R = 1 / hlen(n);
        double dR = R * R - l * l / 4;
        double delta = dR > 0 ? R - sqrt(dR) : R;
        if (!(n[0] == 0 && n[1] == 0 && n[2] == 0)) {
            double inv = 1 / hlen(n);
            for (int a = 0; a < 3; ++a) n[a] = n[a] * inv;
        }
        for (int a = 0; a < 3; ++a) n[a] = n[a] * -1;
        for (int a = 0; a < 3; ++a) pos[a] = (s0[a] + s1[a]) * 0.5 + n[a] * delta;
    } else {
        for (int a = 0; a < 3; ++a) pos[a] = (s0[a] + s1[a]) * 0.5;
    }
    c->h_x[np] = pos[0]; c->h_y[np] = pos[1]; c->h_z[np] = pos[2];
    h.rev(np) = p;
    h.fwd(np) = nx;
    h.fwd(p) = np;
    h.rev(nx) = np;
    new_nodes.push_back(np);
    return np;
}

// remove_point (tangle.c:342-355)
void hremove(ov_ctx *c, int i)
{
    Host h{c, 0, c->n_live, &c->params};
    int pv = h.rev(i), nx = h.fwd(i);
    if (pv >= 0) h.fwd(pv) = nx;
    if (nx >= 0) h.rev(nx) = pv;
    h.rev(i) = h.fwd(i) = -1;
    h.st(i) = OV_EMPTY;
}

// ------------------------------------------------------------ walls
// boundary_normals (boundaries.c:11-18): inward unit normals of the faces
const double kWallNormal[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};

inline bool solid_wall(const Geometry &g, int wall)
{
    return g.wall[wall] != OV_WALL_OPEN && g.wall[wall] != OV_WALL_PERIODIC;
}

// check_wall (tangle.c:822-838)
bool hcheck_wall(Host &h, int k, int wall)
{
    const Geometry &g = h.c->geo;
    const int ax = wall >> 1;
    double p[3];
    h.pos(k, p);
    if ((wall & 1) == 0) return p[ax] < (h.P->rec_dist + g.lo[ax]);
    return p[ax] > (g.hi[ax] - h.P->rec_dist);
}

// wall_dist (tangle.c:847-867)
double hwall_dist(Host &h, int k, int wall)
{
    const Geometry &g = h.c->geo;
    const int ax = wall >> 1;
    double p[3];
    h.pos(k, p);
    return (wall & 1) == 0 ? p[ax] - g.lo[ax] : g.hi[ax] - p[ax];
}

// The device's positions and connections brought up to the host mirror's
// (for direct sums on the current topology in the middle of a host pass).
int sync_device_geometry(ov_ctx *c)
{
    const size_t n = (size_t)c->n_live;
    if (n > (size_t)c->cap) {
        int r = ov_grow_preserving(c, (int)n);
        if (r) return r;
    }
    double *dd[3] = {c->node.x, c->node.y, c->node.z};
    const double *hd[3] = {c->h_x.data(), c->h_y.data(), c->h_z.data()};
    for (int a = 0; a < 3; ++a)
        OV_CUDA(c, cudaMemcpyAsync(dd[a], hd[a], n * 8, cudaMemcpyHostToDevice, c->stream));
    OV_CUDA(c, cudaMemcpyAsync(c->fwd, c->h_fwd.data(), n * 4, cudaMemcpyHostToDevice, c->stream));
    return OV_OK;
}

// update_velocity(k, t, NULL) on the current topology, for a sign decision
// dot(vel, n) > 0: FP64 direct sums on the GPU, and the reference's own
// summation order on the host when the sum's error could flip the sign.
int hdirect_sign(ov_ctx *c, Host &h, int k, const double tg[3], const double nm[3], double t, const double n[3],
                 double *dotv)
{
    int r;
    if ((r = sync_device_geometry(c))) return r;
    double ex[10];
    if ((r = ov_rec_exact(c, k, k, ex))) return r;
    double vs[3], vel[3];
    if (!hlia(h, k, tg, nm, t, vs)) return ov_fail(c, OV_ERR_TOPOLOGY, "walls: filament walk from %d failed", k);
    for (int a = 0; a < 3; ++a) vs[a] = vs[a] + ex[a];
    hfriction(h, k, tg, vs, t, vel);
    const double tl = hlen(tg);
    const double n_terms = (double)(h.hi - h.lo) * (h.c->geo.n_img + 1);
    const double bound = (ex[3] + n_terms * 1.1102230246251565e-16 * ex[4]) * 1.7320508075688772 * 1.01 *
                         (1.0 + fabs(h.P->alpha) * tl + fabs(h.P->alpha_p) * tl * tl);
    double d = hdot(vel, n);
    if (fabs(d) <= bound) {
        hdirect_exact(h, k, tg, nm, t, vel);
        d = hdot(vel, n);
    }
    *dotv = d;
    return OV_OK;
}

// connect_to_wall (tangle.c:877-958) in member mi; *done = 1 when clipped
int hconnect_to_wall(ov_ctx *c, int mi, int k, int wall, double t, std::vector<int> &new_nodes, int *done)
{
    *done = 0;
    Host h = host_of(c, mi);
    double tg[3], nm[3];
    if (!htangent(h, k, tg, nm)) return ov_fail(c, OV_ERR_TOPOLOGY, "walls: filament walk from %d failed", k);
    const double *n = kWallNormal[wall];
    const double d0 = hwall_dist(h, k, wall);
    // only a node in front of the wall and moving away from it is left alone
    if (d0 > 0) {
        double dv = 0;
        int r = hdirect_sign(c, h, k, tg, nm, t, n, &dv);
        if (r) return r;
        if (dv > 0) return OV_OK;
    }
    // the reference applies the integer abs() to the normalised dot product,
    // so this test only fires for a tangent exactly along the normal
    const double nd = hdot(tg, n) / hlen(tg) / hlen(n);
    if (abs((int)nd) > cos(h.P->reconnection_angle_cutoff)) return OV_OK;
    const int next = h.fwd(k), prev = h.rev(k);
    if (next < 0 || prev < 0) return OV_OK;
    const double d1 = hwall_dist(h, next, wall), dm1 = hwall_dist(h, prev, wall);
    double pk[3], pn[3], pp[3];
    h.pos(k, pk);
    h.pos(next, pn);
    h.pos(prev, pp);
    const double vd1 = hpwrap_len(c->geo, pk, pn), vdm1 = hpwrap_len(c->geo, pk, pp);
    if (vd1 < d0 + d1 && vdm1 < d0 + dm1) return OV_OK;   // the length would grow
    const int np1 = hget_empty(c, mi);
    if (np1 < 0) return OV_ERR_ALLOC;
    c->h_status[np1] = h.P->pin_mode;
    c->h_pin[np1] = wall;
    const int np2 = hget_empty(c, mi);
    if (np2 < 0) return OV_ERR_ALLOC;
    c->h_status[np2] = h.P->pin_mode;
    c->h_pin[np2] = wall;
    auto clip = [&](int dst, const double src[3], double dist) {
        double tmp[3] = {n[0] * -dist, n[1] * -dist, n[2] * -dist};
        c->h_x[dst] = src[0] + tmp[0];
        c->h_y[dst] = src[1] + tmp[1];
        c->h_z[dst] = src[2] + tmp[2];
    };
    clip(np1, pk, d0);
    std::vector<int> &rc = c->h_recalc;
    rc[k]++; rc[np1]++; rc[np2]++; rc[next]++; rc[prev]++;
    if (d1 < dm1) {
        clip(np2, pn, d1);
        c->h_fwd[k] = np1;
        c->h_fwd[np1] = -1; c->h_rev[np1] = k;
        c->h_fwd[np2] = next; c->h_rev[np2] = -1;
        c->h_rev[next] = np2;
    } else {
        clip(np2, pp, dm1);
        c->h_rev[k] = np1;
        c->h_fwd[np1] = k; c->h_rev[np1] = -1;
        c->h_fwd[np2] = -1; c->h_rev[np2] = prev;
        c->h_fwd[prev] = np2;
    }
    new_nodes.push_back(np1);
    new_nodes.push_back(np2);
    *done = 1;
    return OV_OK;
}

// enforce_wall_boundaries (tangle.c:966-1016) on member mi
int hwalls(ov_ctx *c, int mi, double t, std::vector<int> &new_nodes, int *clipped, int *removed)
{
    const Geometry &g = c->geo;
    {
        const Member &m = c->mem[mi];
        std::fill(c->h_recalc.begin() + m.lo, c->h_recalc.begin() + m.lo + m.n, 0);
    }
    for (int wall = 0; wall < 6; ++wall) {
        if (!solid_wall(g, wall)) continue;
        for (int j = 0; j < c->mem[mi].n; ++j) {   // N may grow while clipping
            Host h = host_of(c, mi);
            const int k = h.lo + j;
            const int st = h.st(k);
            if (pinned(st) || st == OV_EMPTY || c->h_recalc[k]) continue;
            if (!hcheck_wall(h, k, wall)) continue;
            int done = 0, r = hconnect_to_wall(c, mi, k, wall, t, new_nodes, &done);
            if (r) return r;
            *clipped += done;
        }
    }
    for (int wall = 0; wall < 6; ++wall) {
        if (!solid_wall(g, wall)) continue;
        for (int j = 0; j < c->mem[mi].n; ++j) {
            Host h = host_of(c, mi);
            const int k = h.lo + j;
            const int st = h.st(k);
            if (pinned(st) || st == OV_EMPTY) continue;
            if (hwall_dist(h, k, wall) < 0) {
                hremove(c, k);
                ++*removed;
            }
        }
    }
    return OV_OK;
}

inline bool any_solid_wall(const Geometry &g)
{
    for (int w = 0; w < 6; ++w)
        if (solid_wall(g, w)) return true;
    return false;
}

// remesh (tangle.c:1018-1061) of member mi: slots in index order, including
// the ones it inserts (and the range it grows into)
// The pass in index order over the member's local slots `visit` (sorted:
// every slot whose tests could act) and the slots an earlier action of the
// pass touched: a removal changes its neighbours' lengths, an insertion its
// old forward neighbour's and the new node's.  Every other slot keeps the
// lengths its test failed on, so visiting only these is the reference's pass.
int hremesh(ov_ctx *c, int mi, double min_dist, double max_dist, double time, int *added_out, int *removed_out,
            std::vector<int> &new_nodes, const std::vector<int> &visit)
{
    int added = 0, removed = 0;
    std::priority_queue<int, std::vector<int>, std::greater<int>> todo(visit.begin(), visit.end());
    int last = -1;
    while (!todo.empty()) {
        const int k = todo.top();
        todo.pop();
        if (k <= last || k >= c->mem[mi].n) continue;
        last = k;
        Host h = host_of(c, mi);
        const int s = h.lo + k;
        if (h.st(s) == OV_EMPTY) continue;
        int nx = h.fwd(s), pv = h.rev(s);
        double lf = 0, lr = 0, pk[3];
        h.pos(s, pk);
        if (nx >= 0) { double q[3]; h.pos(nx, q); lf = hpwrap_len(c->geo, pk, q); }
        if (pv >= 0) { double q[3]; h.pos(pv, q); lr = hpwrap_len(c->geo, pk, q); }
        if (nx >= 0 && pv >= 0 && ((lf < min_dist || lr < min_dist) && (lf + lr) < max_dist)) {
            hremove(c, s);
            removed++;
            if (pv - h.lo > k) todo.push(pv - h.lo);
            if (nx - h.lo > k) todo.push(nx - h.lo);
        }
        if (nx >= 0 && lf > max_dist) {
            added++;
            const int np = hadd_point(c, mi, s, new_nodes);
            if (np < 0) return OV_ERR_ALLOC;
            const int lo = host_of(c, mi).lo;
            if (np - lo > k) todo.push(np - lo);
            if (nx - lo > k) todo.push(nx - lo);
        }
    }
    if (added) {
        // points added outside the domain (tangle.c:1056-1060)
        const Member &m = c->mem[mi];
        hperiodic(c, m.lo, m.lo + m.n);
        std::fill(c->h_recalc.begin() + m.lo, c->h_recalc.begin() + m.lo + m.n, 0);
        if (any_solid_wall(c->geo)) {
            int clipped = 0, gone = 0, r = hwalls(c, mi, time, new_nodes, &clipped, &gone);
            if (r) return r;
        }
    }
    *added_out = added;
    *removed_out = removed;
    return OV_OK;
}

int ensure_pairs(ov_ctx *c, int need)
{
    if (c->pair_cap >= need && c->d_pairs) return OV_OK;
    if (c->d_pairs) cudaFree(c->d_pairs);
    c->d_pairs = nullptr;
    OV_ALLOC(c, cudaMalloc(&c->d_pairs, (size_t)need * 2 * sizeof(int)));
    if (!c->d_npairs) OV_ALLOC(c, cudaMalloc(&c->d_npairs, sizeof(int)));
    c->pair_cap = need;
    return OV_OK;
}

// candidate pairs (k < l, both FREE) with |seg_pwrap(x_k, x_l)| <= rec_dist
int find_pairs(ov_ctx *c, std::vector<std::pair<int, int>> &out)
{
    out.clear();
    int cap = c->cap;
    double rd = 0;
    for (const Member &m : c->mem) rd = std::max(rd, m.params.rec_dist);   // grid for the largest
    GridGeom gg;
    for (int a = 0; a < 3; ++a) {
        gg.lo[a] = c->geo.lo[a];
        gg.L[a] = c->geo.L[a];
        double cells = floor(c->geo.L[a] / (2.0 * rd));
        gg.n[a] = (int)std::max(1.0, std::min(cells, 1024.0));
        gg.periodic[a] = c->geo.periodic[a];
    }
    int r = ensure_pairs(c, std::max(c->pair_cap, 4 * std::max(c->n_live, 16)));
    if (r) return r;
    TreeBuf &t = c->tree;
    int nb = (cap + 255) / 256;
    k_grid_keys<<<nb, 256, 0, c->stream>>>(c->status, c->node.x, c->node.y, c->node.z, c->n_live, cap, gg, t.keys,
                                           t.order);
    c->launches++;
    ov_sort_keys(c, t, cap, c->stream);
    for (int attempt = 0; attempt < 2; ++attempt) {
        OV_CUDA(c, cudaMemsetAsync(c->d_npairs, 0, sizeof(int), c->stream));
        const bool ens = c->mem.size() > 1;
        k_pairs<<<nb, 256, 0, c->stream>>>(t.keys, t.order, cap, c->node.x, c->node.y, c->node.z, gg, c->geo, rd,
                                           ens ? c->d_tid : nullptr, ens ? c->d_tprm : nullptr, c->d_pairs,
                                           c->d_npairs, c->pair_cap);
        c->launches++;
        OV_CUDA(c, cudaGetLastError());
        int np = 0;
        OV_CUDA(c, cudaMemcpyAsync(&np, c->d_npairs, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
        if (np > c->pair_cap) {
            if ((r = ensure_pairs(c, np + np / 2))) return r;
            continue;
        }
        std::vector<int> buf(2 * (size_t)np);
        if (np)
            OV_CUDA(c, cudaMemcpy(buf.data(), c->d_pairs, (size_t)np * 2 * sizeof(int), cudaMemcpyDeviceToHost));
        out.resize(np);
        for (int i = 0; i < np; ++i) out[i] = {buf[2 * i], buf[2 * i + 1]};
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
        return OV_OK;
    }
    return ov_fail(c, OV_ERR_ALLOC, "candidate pair buffer could not be sized");
}

}  // namespace

namespace {

// Forward DFT of 3 sequences of length N (real `re` or complex `cin`, N per
// coordinate) into X (3N complex), by Bluestein over radix-2 FFTs.
int bluestein3(ov_ctx *c, const double *re, const double2 *cin, int N, double2 *X)
{
    int M = 1;
    while (M < 2 * N - 1) M <<= 1;
    if (M < 2) M = 2;
    cudaStream_t st = c->stream;
    // buffers: A, T (3M each), B, TB (M each), twiddles (M/2)
    size_t need = (size_t)8 * M;
    if (c->fft_cap < need) {
        if (c->fft_buf) cudaFree(c->fft_buf);
        c->fft_buf = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->fft_buf, need * sizeof(double2)));
        c->fft_cap = need;
        c->fft_M = 0;
    }
    double2 *A = c->fft_buf, *T = A + 3 * (size_t)M, *B = T + 3 * (size_t)M, *TB = B + M;
    double2 *tw = c->fft_tw;
    if (c->fft_M != M) {
        if (c->fft_tw) cudaFree(c->fft_tw);
        c->fft_tw = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->fft_tw, (size_t)std::max(M / 2, 1) * sizeof(double2)));
        tw = c->fft_tw;
        k_twiddles<<<(M / 2 + 255) / 256, 256, 0, st>>>(tw, M);
        c->fft_M = M;
        c->launches++;
    }
    auto fft = [&](double2 *x, double2 *y, int batch) -> double2 * {
        for (int Ns = 1; Ns < M; Ns <<= 1) {
            k_fft_pass<<<dim3((M / 2 + 255) / 256, batch), 256, 0, st>>>(x, y, tw, M, Ns);
            c->launches++;
            std::swap(x, y);
        }
        return x;   // holds the result
    };
    const dim3 gM((M + 255) / 256, 3), gN((N + 255) / 256, 3);
    k_chirp_filter<<<(M + 255) / 256, 256, 0, st>>>(B, N, M);
    k_chirp_in<<<gM, 256, 0, st>>>(re, cin, N, M, A);
    c->launches += 2;
    double2 *Bf = fft(B, TB, 1);
    double2 *Af = fft(A, T, 3);
    k_conv_mul<<<gM, 256, 0, st>>>(Af, Bf, M);
    c->launches++;
    double2 *Cf = fft(Af, Af == A ? T : A, 3);
    k_chirp_out<<<gN, 256, 0, st>>>(Cf, N, M, X);
    c->launches++;
    OV_CUDA(c, cudaGetLastError());
    return OV_OK;
}

// Loops of more than this many nodes are smoothed through the FFT path.
constexpr int kLongLoop = 1024;

// smooth one long closed loop (nodes in loop order), as k_smooth does for
// short ones: unwrap and detrend on the host mirror, filter on the GPU,
// write the positions back on the GPU
int smooth_long_loop(ov_ctx *c, const int *nodes, int len, double freq_to_cutoff)
{
    Host h{c, 0, c->n_live, &c->params};
    const Geometry &g = c->geo;
    std::vector<double> X[3];
    for (auto &v : X) v.assign((size_t)2 * len, 0.0);
    double prev[3];
    h.pos(nodes[0], prev);
    for (int a = 0; a < 3; ++a) X[a][0] = prev[a];
    for (int j = 1; j < len; ++j) {
        double r2[3], r1[3] = {X[0][j - 1], X[1][j - 1], X[2][j - 1]};
        h.pos(nodes[j], r2);
        hpwrap(g, r1, r2);
        for (int a = 0; a < 3; ++a) X[a][j] = r2[a];
    }
    double gx = X[0][0] - X[0][len - 1], gy = X[1][0] - X[1][len - 1], gz = X[2][0] - X[2][len - 1];
    double gap = sqrt(gx * gx + gy * gy + gz * gz);
    const int detrend = (gap > g.L[0] / 2 && len > 2) ? 1 : 0;
    const int N = detrend ? 2 * len - 2 : len;
    double coef[3] = {0, 0, 0}, c0[3] = {0, 0, 0};
    if (detrend) {
        for (int a = 0; a < 3; ++a) {
            coef[a] = (X[a][len - 1] - X[a][0]) / (len - 1);
            c0[a] = X[a][0];
        }
        for (int a = 0; a < 3; ++a) {
            for (int j = 0; j < len; ++j)
                X[a][j] = (j == 0 || j == len - 1) ? 0.0 : X[a][j] - coef[a] * j - c0[a];
            for (int j = 0; j < len - 2; ++j) X[a][len + j] = -X[a][len - 2 - j];
        }
    }
    std::vector<double> flat((size_t)3 * N);
    for (int a = 0; a < 3; ++a) std::copy(X[a].begin(), X[a].begin() + N, flat.begin() + (size_t)a * N);
    size_t need = (size_t)3 * N * sizeof(double) + (size_t)2 * 3 * N * sizeof(double2) + (size_t)len * sizeof(int);
    if (c->long_cap < need) {
        if (c->long_buf) cudaFree(c->long_buf);
        c->long_buf = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->long_buf, need));
        c->long_cap = need;
    }
    // complex arrays first: every double2 stays 16-byte aligned
    double2 *d_X = (double2 *)c->long_buf;
    double2 *d_Z = d_X + 3 * (size_t)N;
    double *d_re = (double *)(d_Z + 3 * (size_t)N);
    int *d_nodes = (int *)(d_re + 3 * (size_t)N);
    OV_CUDA(c, cudaMemcpyAsync(d_re, flat.data(), flat.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    OV_CUDA(c, cudaMemcpyAsync(d_nodes, nodes, (size_t)len * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    int r;
    if ((r = bluestein3(c, d_re, nullptr, N, d_X))) return r;
    // low_pass_filter's zeroed range (vortex_smooth.c:146-160)
    int cut = (int)(freq_to_cutoff * N / 2);
    int zlo = 0, zhi = 0;
    if (N > 2 * cut + 1) {
        zlo = N / 2 - cut;
        zhi = (N % 2 == 0) ? N / 2 + 1 + cut : N / 2 + cut;
    }
    const dim3 gN((N + 255) / 256, 3);
    k_lowpass_mask<<<gN, 256, 0, c->stream>>>(d_X, N, zlo, zhi);
    c->launches++;
    if ((r = bluestein3(c, nullptr, d_X, N, d_Z))) return r;
    k_long_writeback<<<(len + 255) / 256, 256, 0, c->stream>>>(d_Z, N, len, d_nodes, detrend, coef[0], coef[1],
                                                               coef[2], c0[0], c0[1], c0[2], c->node.x, c->node.y,
                                                               c->node.z, c->cap);
    c->launches++;
    OV_CUDA(c, cudaGetLastError());
    OV_CUDA(c, cudaStreamSynchronize(c->stream));   // the host buffers above go out of scope
    return OV_OK;
}

}  // namespace

namespace {

// ------------------------------------------------------------- injection
// drand48 as POSIX defines it: X <- (0x5DEECE66D X + 0xB) mod 2^48, the
// result X / 2^48; x[0] holds the low 16 bits of X.
double hrand48(unsigned short x[3])
{
    uint64_t X = (uint64_t)x[0] | (uint64_t)x[1] << 16 | (uint64_t)x[2] << 32;
    X = (0x5DEECE66DULL * X + 0xBULL) & 0xFFFFFFFFFFFFULL;
    x[0] = (unsigned short)(X & 0xFFFF);
    x[1] = (unsigned short)((X >> 16) & 0xFFFF);
    x[2] = (unsigned short)((X >> 32) & 0xFFFF);
    return ldexp((double)X, -48);
}

// vec3_normalize (vec3_math.c:208): times the reciprocal of the length
void hnormalize(double v[3])
{
    if (v[0] == 0 && v[1] == 0 && v[2] == 0) return;
    const double m = 1 / hlen(v);
    for (int i = 0; i < 3; ++i) v[i] = v[i] * m;
}

// number_of_empty_nodes (tangle.c:128) of member mi
int hcount_empty(ov_ctx *c, int mi)
{
    const Member &m = c->mem[mi];
    int n = 0;
    for (int k = m.lo; k < m.lo + m.n; ++k) n += c->h_status[k] == OV_EMPTY;
    return n;
}

// the doubling loop before add_loop / add_line_in_zdir place their nodes
int hreserve_empty(ov_ctx *c, int mi, int need)
{
    for (int guard = 0; hcount_empty(c, mi) < need; ++guard) {
        const int n = c->mem[mi].n;
        if (guard > 40) return OV_ERR_ALLOC;
        int r = hexpand(c, mi, n > 0 ? 2 * n : 1);
        if (r) return r;
    }
    return OV_OK;
}

// perpendicular (vortex_injection.c:18-40): dir's component-free part of
// (1,0,0), or of (0,1,0) when dir is along x, normalised
void hperpendicular(const double dir[3], double out[3])
{
    const double ax[2][3] = {{1, 0, 0}, {0, 1, 0}};
    for (int q = 0; q < 2; ++q) {
        const double m = -hdot(ax[q], dir);
        for (int i = 0; i < 3; ++i) out[i] = dir[i] * m;
        for (int i = 0; i < 3; ++i) out[i] = out[i] + ax[q][i];
        if (q == 0 && !(hlen(out) > 1e-8)) continue;
        hnormalize(out);
        return;
    }
}

void hset_node(ov_ctx *c, int i, const double p[3], int status)
{
    c->h_x[i] = p[0]; c->h_y[i] = p[1]; c->h_z[i] = p[2];
    c->h_status[i] = status;
}

// add_loop (vortex_injection.c:49-100) in member mi; the new slots are
// appended to `added`
int hadd_loop(ov_ctx *c, int mi, const double center[3], const double dir[3], double r, std::vector<int> &added)
{
    const ov_params &P = c->mem[mi].params;
    const int npts = (int)(4 * M_PI * r / (P.dl_max + P.dl_min));
    if (npts <= 0) return OV_OK;   // the reference would write connections[-1]
    int rc = hreserve_empty(c, mi, npts);
    if (rc) return rc;
    double zdir[3], u[3], v[3];
    hperpendicular(dir, zdir);
    hcross(u, zdir, dir);
    hcross(v, dir, u);
    hnormalize(u);
    hnormalize(v);
    int first = -1, curr = -1, last = -1;
    for (int k = 0; k < npts; ++k) {
        const double phi = 2 * M_PI / npts * k;
        const double cs = cos(phi), sn = sin(phi);
        double p[3], q[3];
        for (int i = 0; i < 3; ++i) p[i] = u[i] * (r * cs);
        for (int i = 0; i < 3; ++i) q[i] = v[i] * (r * sn);
        for (int i = 0; i < 3; ++i) p[i] = p[i] + q[i];
        for (int i = 0; i < 3; ++i) p[i] = p[i] + center[i];
        curr = hget_empty(c, mi);
        if (curr < 0) return OV_ERR_ALLOC;
        if (first < 0) first = curr;
        hset_node(c, curr, p, OV_FREE);
        if (curr != first) {
            c->h_rev[curr] = last;
            c->h_fwd[last] = curr;
        }
        last = curr;
        added.push_back(curr);
    }
    c->h_fwd[curr] = first;
    c->h_rev[first] = curr;
    return OV_OK;
}

// add_line_in_zdir (vortex_injection.c:267-319) in member mi
int hadd_line_z(ov_ctx *c, int mi, double x, double y, int direction, std::vector<int> &added)
{
    const ov_params &P = c->mem[mi].params;
    const double zmin = c->geo.lo[2], zmax = c->geo.hi[2];
    const int points = (int)(2 * (zmax - zmin) / (P.dl_max - P.dl_min));
    if (points <= 0) return OV_ERR_ARG;   // the reference divides by it
    int rc = hreserve_empty(c, mi, points);
    if (rc) return rc;
    const double dz = (zmax - zmin) / points;
    const double zstart = direction > 0 ? zmin : zmax;
    const double zend = direction > 0 ? zmax : zmin;
    double s[3] = {x, y, zstart};
    int pt = hget_empty(c, mi);
    if (pt < 0) return OV_ERR_ALLOC;
    hset_node(c, pt, s, P.pin_mode);
    c->h_pin[pt] = direction > 0 ? OV_DOWN : OV_UP;
    c->h_rev[pt] = -1;
    added.push_back(pt);
    for (int k = 1; k < points - 1; ++k) {
        const int last = pt;
        if ((pt = hget_empty(c, mi)) < 0) return OV_ERR_ALLOC;
        s[2] = zstart + direction * k * dz;
        hset_node(c, pt, s, OV_FREE);
        c->h_pin[pt] = OV_NOT_A_FACE;
        c->h_rev[pt] = last;
        c->h_fwd[last] = pt;
        added.push_back(pt);
    }
    s[2] = zend;
    const int last = pt;
    if ((pt = hget_empty(c, mi)) < 0) return OV_ERR_ALLOC;
    hset_node(c, pt, s, P.pin_mode);
    c->h_pin[pt] = direction > 0 ? OV_UP : OV_DOWN;
    c->h_rev[pt] = last;
    c->h_fwd[pt] = -1;
    c->h_fwd[last] = pt;
    added.push_back(pt);
    return OV_OK;
}

// Host mirror for a pass that may change nothing: pulled on first use.
struct LazyMirror {
    ov_ctx *c;
    bool pulled = false;
    int get()
    {
        if (pulled) return OV_OK;
        int r = ov_pull_host(c);
        if (r) return r;
        c->host_valid = false;
        pulled = true;
        return OV_OK;
    }
};

// inject_loop (vortex_injection.c:715-752) for member mi.  Three draws for
// the direction come first, whether or not it is time to inject; the build
// of the reference this follows evaluates vec3()'s three arguments from
// the last to the first.
int hinject_loop(ov_ctx *c, int mi, double t, LazyMirror &mir, std::vector<int> &added)
{
    Member &m = c->mem[mi];
    unsigned short *x = m.inj.rand48;
    double dir[3];
    dir[2] = -hrand48(x);
    dir[1] = 2 * (hrand48(x) - 0.5);
    dir[0] = 2 * (hrand48(x) - 0.5);
    hnormalize(dir);
    if (t - m.last_loop < 1 / m.inj.loop_frequency) return OV_OK;
    m.last_loop = t;
    const double left = c->geo.lo[0], right = c->geo.hi[0], back = c->geo.lo[1], front = c->geo.hi[1];
    double cent[3];
    cent[2] = c->geo.hi[2];
    cent[0] = left + (right - left) * hrand48(x);
    cent[1] = back + (front - back) * hrand48(x);
    const double D = fabs(right - left), rmin = 0.05 * D, rmax = 0.25 * D;
    const double r = rmin + (rmax - rmin) * hrand48(x);
    int rc = mir.get();
    if (rc) return rc;
    return hadd_loop(c, mi, cent, dir, r, added);
}

// inject_line_pairs (vortex_injection.c:760-800) for member mi
int hinject_lines(ov_ctx *c, int mi, double t, LazyMirror &mir, std::vector<int> &added)
{
    Member &m = c->mem[mi];
    unsigned short *x = m.inj.rand48;
    if (t - m.last_line < 1 / m.inj.line_frequency) return OV_OK;
    m.last_line = t;
    for (int k = 0; k < m.inj.line_n; ++k) {
        const double left = c->geo.lo[0], right = c->geo.hi[0], back = c->geo.lo[1], front = c->geo.hi[1];
        const double x1 = left + hrand48(x) * (right - left);
        const double x2 = left + hrand48(x) * (right - left);
        double y1, y2;
        if (m.inj.line_polarized) {
            y1 = back + (1 + hrand48(x)) * (front - back) / 2;
            y2 = back + hrand48(x) * (front - back) / 2;
        } else {
            y1 = back + hrand48(x) * (front - back);
            y2 = back + hrand48(x) * (front - back);
        }
        int rc = mir.get();
        if (rc) return rc;
        if ((rc = hadd_line_z(c, mi, x1, y1, +1, added))) return rc;
        if ((rc = hadd_line_z(c, mi, x2, y2, -1, added))) return rc;
    }
    return OV_OK;
}

// host mirror -> device after nodes were added; their velocities start at 0
int push_added(ov_ctx *c, const std::vector<int> &added)
{
    int r = ov_push_device(c, 1);
    if (r || added.empty()) return r;
    int *d = nullptr;
    OV_ALLOC(c, cudaMalloc(&d, added.size() * sizeof(int)));
    OV_CUDA(c, cudaMemcpy(d, added.data(), added.size() * sizeof(int), cudaMemcpyHostToDevice));
    k_zero_vel<<<((int)added.size() + 255) / 256, 256, 0, c->stream>>>(
        d, (int)added.size(), c->node.vx, c->node.vy, c->node.vz, c->node.sx, c->node.sy, c->node.sz);
    c->launches++;
    OV_CUDA(c, cudaGetLastError());
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(d);
    return OV_OK;
}

bool any_injection(const ov_ctx *c)
{
    for (const Member &m : c->mem)
        if (m.inj.loop_injection || m.inj.line_injection) return true;
    return false;
}

}  // namespace

extern "C" {

int ov_eliminate_small_loops(ov_ctx *c)
{
    int r = ready(c);
    if (r) return r;
    if ((r = ov_pull_host(c))) return r;
    c->host_valid = false;   // until the mirror is pushed (or found unchanged)
    int removed = 0;
    // the slots of structures the pass could remove from, from the device
    // (host and device agree here), then each structure's first slot
    const int n = c->n_live, nmem = (int)c->mem.size();
    int cutoff = 0;
    for (const Member &m : c->mem) cutoff = std::max(cutoff, m.params.small_loop_cutoff);
    std::vector<int> slots;
    if (n > 0 && cutoff > 0) {
        if (c->rm_cap < n + 1) {
            if (c->d_rm) cudaFree(c->d_rm);
            c->d_rm = nullptr;
            OV_ALLOC(c, cudaMalloc(&c->d_rm, (size_t)(n + 1) * sizeof(int)));
            c->rm_cap = n + 1;
        }
        int *d_count = c->d_rm + n;
        OV_CUDA(c, cudaMemsetAsync(d_count, 0, sizeof(int), c->stream));
        k_small_flags<<<(n + 255) / 256, 256, 0, c->stream>>>(c->status, c->fwd, n, cutoff, c->d_rm, d_count, n);
        c->launches++;
        int cnt = 0;
        OV_CUDA(c, cudaMemcpyAsync(&cnt, d_count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
        cnt = std::min(cnt, n);
        slots.resize(cnt);
        if (cnt) OV_CUDA(c, cudaMemcpy(slots.data(), c->d_rm, (size_t)cnt * sizeof(int), cudaMemcpyDeviceToHost));
    }
    std::vector<std::vector<int>> starts(nmem);
    for (int sl : slots) {
        int lo2 = 0, hi2 = nmem - 1;
        while (lo2 < hi2) {   // the member holding slot sl
            const int mid = (lo2 + hi2 + 1) >> 1;
            if (c->mem[mid].lo <= sl) lo2 = mid; else hi2 = mid - 1;
        }
        Host h = host_of(c, lo2);
        // the structure's lowest slot: forward until back or an end, then backward
        int first = sl, cur = sl, guard = 0;
        bool closed = false;
        for (int nx = h.fwd(cur); guard <= n; ++guard, nx = h.fwd(cur)) {
            if (nx == sl) { closed = true; break; }
            if (nx < h.lo || nx >= h.hi) break;
            cur = nx;
            first = std::min(first, cur);
        }
        if (!closed) {
            cur = sl;
            guard = 0;
            for (int pv = h.rev(cur); pv >= h.lo && pv < h.hi && pv != sl && guard <= n; ++guard, pv = h.rev(cur)) {
                cur = pv;
                first = std::min(first, cur);
            }
        }
        starts[lo2].push_back(first);
    }
    for (int mi = 0; mi < nmem; ++mi) {
        auto &v = starts[mi];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        removed += hsmall_loops(c, mi, v);
    }
    c->stats.small_loops_removed = removed;
    if (removed) return ov_push_device(c, 0);
    c->host_valid = true;
    return OV_OK;
}

int ov_remesh(ov_ctx *c, double min_dist, double max_dist, double t)
{
    int r = ready(c);
    if (r) return r;
    if ((r = ov_pull_host(c))) return r;
    c->host_valid = false;
    int added = 0, removed = 0;
    std::vector<int> new_nodes;
    const int nmem = (int)c->mem.size();
    std::vector<double> lim(2 * (size_t)nmem);
    for (int mi = 0; mi < nmem; ++mi) {
        // a single tangle takes the arguments; ensemble members their own dl_min / dl_max
        lim[2 * mi] = nmem == 1 ? min_dist : c->mem[mi].params.dl_min;
        lim[2 * mi + 1] = nmem == 1 ? max_dist : c->mem[mi].params.dl_max;
    }
    // the slots whose tests could act, from the device (host and device agree here)
    std::vector<std::vector<int>> visit(nmem);
    {
        const int n = c->n_live;
        if (c->rm_cap < n + 1) {
            if (c->d_rm) cudaFree(c->d_rm);
            c->d_rm = nullptr;
            OV_ALLOC(c, cudaMalloc(&c->d_rm, (size_t)(n + 1) * sizeof(int)));
            c->rm_cap = n + 1;
        }
        if (c->rm_lim_cap < 2 * nmem) {
            if (c->d_rm_lim) cudaFree(c->d_rm_lim);
            c->d_rm_lim = nullptr;
            OV_ALLOC(c, cudaMalloc(&c->d_rm_lim, 2 * (size_t)nmem * sizeof(double)));
            c->rm_lim_cap = 2 * nmem;
        }
        OV_CUDA(c, cudaMemcpyAsync(c->d_rm_lim, lim.data(), lim.size() * sizeof(double), cudaMemcpyHostToDevice,
                                   c->stream));
        int *d_count = c->d_rm + n;
        OV_CUDA(c, cudaMemsetAsync(d_count, 0, sizeof(int), c->stream));
        if (n > 0) {
            k_remesh_flags<<<(n + 255) / 256, 256, 0, c->stream>>>(c->status, c->fwd, c->rev, c->node.x, c->node.y,
                                                                   c->node.z, nmem > 1 ? c->d_tid : nullptr,
                                                                   c->d_rm_lim, nmem, c->geo, n, c->d_rm, d_count, n);
            c->launches++;
        }
        int cnt = 0;
        OV_CUDA(c, cudaMemcpyAsync(&cnt, d_count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
        cnt = std::min(cnt, n);
        std::vector<int> slots(cnt);
        if (cnt) {
            OV_CUDA(c, cudaMemcpy(slots.data(), c->d_rm, (size_t)cnt * sizeof(int), cudaMemcpyDeviceToHost));
        }
        for (int sl : slots) {
            int m = 0, lo2 = 0, hi2 = nmem - 1;
            while (lo2 < hi2) {   // the member holding slot sl
                const int mid = (lo2 + hi2 + 1) >> 1;
                if (c->mem[mid].lo <= sl) lo2 = mid; else hi2 = mid - 1;
            }
            m = lo2;
            visit[m].push_back(sl - c->mem[m].lo);
        }
        for (auto &v : visit) std::sort(v.begin(), v.end());
    }
    for (int mi = 0; mi < nmem; ++mi) {
        const double lo = lim[2 * mi], hi = lim[2 * mi + 1];
        int a = 0, d = 0;
        if ((r = hremesh(c, mi, lo, hi, t, &a, &d, new_nodes, visit[mi]))) {
            // keep host and device consistent before reporting
            ov_push_device(c, 1);
            return r == OV_ERR_ALLOC ? ov_fail(c, r, "remesh: no empty slot could be had") : r;
        }
        added += a;
        removed += d;
    }
    c->stats.remesh_added = added;
    c->stats.remesh_removed = removed;
    if (!added && !removed) {
        c->host_valid = true;
        return OV_OK;
    }
    if ((r = ov_push_device(c, 1))) return r;
    if (!new_nodes.empty()) {
        int *d = nullptr;
        OV_ALLOC(c, cudaMalloc(&d, new_nodes.size() * sizeof(int)));
        OV_CUDA(c, cudaMemcpy(d, new_nodes.data(), new_nodes.size() * sizeof(int), cudaMemcpyHostToDevice));
        k_zero_vel<<<((int)new_nodes.size() + 255) / 256, 256, 0, c->stream>>>(
            d, (int)new_nodes.size(), c->node.vx, c->node.vy, c->node.vz, c->node.sx, c->node.sy, c->node.sz);
        c->launches++;
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaFree(d);
    }
    return OV_OK;
}

int ov_reconnect(ov_ctx *c, double t, int *nrecs, int *log_k, int *log_l, int log_cap)
{
    int r = ready(c);
    if (r) return r;
    auto clk = [] { return std::chrono::steady_clock::now(); };
    auto ms_since = [&](std::chrono::steady_clock::time_point t0) {
        return std::chrono::duration<double, std::milli>(clk() - t0).count();
    };
    auto tr = clk();
    for (int i = 8; i < 16; ++i) c->step_ms[i] = 0;
    if ((r = ov_pull_host(c))) return r;
    c->host_valid = false;
    std::vector<std::pair<int, int>> pairs;
    if ((r = find_pairs(c, pairs))) return r;
    c->step_ms[8] = ms_since(tr);
    tr = clk();
    const int N = c->n_live;
    // direct sums of every candidate node on the pass's starting topology:
    // mixed precision with an error bound (rec[4 i + 3]), FP64 on demand
    std::vector<int> cand;
    cand.reserve(2 * pairs.size());
    for (auto &pr : pairs) { cand.push_back(pr.first); cand.push_back(pr.second); }
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    const int C = (int)cand.size();
    std::vector<double> rec(5 * (size_t)C);
    // corrections read back from the device (pinned: many small copies)
    if (c->h_corr_cap < 4 * (size_t)std::max(C, 1)) {
        if (c->h_corr) cudaFreeHost(c->h_corr);
        c->h_corr = nullptr;
        OV_ALLOC(c, cudaMallocHost(&c->h_corr, 4 * (size_t)std::max(C, 1) * sizeof(double)));
        c->h_corr_cap = 4 * (size_t)std::max(C, 1);
    }
    double *corr = c->h_corr;
    std::fill(corr, corr + 4 * (size_t)C, 0.0);
    // FP64 sums on the current topology (refinements), valid while
    // ex_gen[i] == gen
    std::vector<double> ex(5 * (size_t)C);
    std::vector<int> ex_gen(C, -1);
    int pushed_gen = 0;   // generation of the device's connections
    // corrections on the host are read back lazily: corr_gen[i] < gen means
    // candidate i's copy predates the last rewiring.  After each rewiring
    // the corrections of the next pairs' candidates are read back ahead
    // (pf_gen[i] == gen: waiting in the pinned prefetch buffer at pf_pos[i]).
    std::vector<int> corr_gen(C, 0), pf_gen(C, -1), pf_pos(C, 0);
    int gen = 0;
    bool pf_waited = true;
    const int kFetch = 256, kAhead = 48;   // 2 kAhead candidates at most: within the correction's read-back list
    const int kLazy = 16;                  // rewirings a copy may lack (bounded instead of read back)
    std::vector<int> ahead;
    ahead.reserve(2 * kAhead);
    struct Rewire {
        double a[4][3], b[4][3];   // the changed segments (wrapped end)
        double c[3], rho, slen;    // a sphere around them (centre, radius, 1.01 x radius), sum of lengths
    };
    std::vector<Rewire> rw;   // rewiring r: its four changed segments
    // rewirings whose corrections are not launched yet (up to 8 go in one
    // launch): their segments and the first candidate they apply to
    std::vector<int> pend_m, pend_f;
    std::vector<double> pend_s;
    int pend_from = INT_MAX, launched_gen = 0;
    size_t cur_q = 0;   // the pair being decided (the read-back list starts there)
    c->stats.reconnect_lazy_evals = 0;
    int64_t evaluated = 0;
    c->stats.reconnect_candidates = C;
    c->stats.reconnect_fp64_pairs = 0;
    c->stats.reconnect_exact_pairs = 0;
    if (C && (r = ov_rec_begin(c, cand.data(), C, rec.data()))) return r;
    c->step_ms[9] = ms_since(tr);
    tr = clk();
    auto cand_index = [&](int k) {
        return (int)(std::lower_bound(cand.begin(), cand.end(), k) - cand.begin());
    };
    std::vector<int> &recalc = c->h_recalc;
    recalc.assign(N, 0);
    const Geometry &g = c->geo;
    int nrec = 0;
    // members own contiguous slot ranges and pairs are sorted by k: each
    // member's pairs form one run, processed in the reference's order
    auto member_of = [&](int k) {
        int lo = 0, hi = (int)c->mem.size() - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (c->mem[mid].lo <= k) lo = mid; else hi = mid - 1;
        }
        return lo;
    };
    int cur_member = -1, cb = 0, ce = 0;   // the member's candidates [cb, ce)
    Host h = host_of(c, 0);
    double cos_cut = 0;

    // velocity of an unflagged candidate node on the current topology, and a
    // bound on how far it may sit from the reference's update_velocity: the
    // error of our sum plus the rounding of the reference's own sequential
    // sum of 27 N terms (at most (27 N - 1) eps64 times their magnitudes)
    // Rewirings whose corrections a candidate's copy lacks may be covered by a
    // bound instead of waiting for the device: a straight segment S at
    // distance d from a point adds at most kappa |S| / (4 pi d^2) to its
    // velocity (|dl x r| / |r|^3 <= |dl| / d^2 along it), summed over the
    // changed segments and every query point.  A pair it does not decide
    // waits for the exact corrections.
    auto pending_bound = [&](int ci, int k) -> double {
        double x[3], qs[OV_MAX_IMAGES + 1][3];
        h.pos(k, x);
        const int nq = g.n_img + 1;
        for (int a = 0; a < 3; ++a) qs[0][a] = x[a];
        for (int j = 0; j < g.n_img; ++j) himage(g, j, x, qs[j + 1]);
        double b = 0;
        for (int r = corr_gen[ci]; r < gen; ++r) {
            const Rewire &w = rw[r];
            for (int qi = 0; qi < nq; ++qi) {
                // far from the four segments' bounding sphere: every point of
                // them is at least |q - c| - rho away
                double qc[3];
                hsub(qc, qs[qi], w.c);
                const double D = sqrt(hdot(qc, qc));
                if (D > 4 * w.rho) {
                    const double d = D - w.rho;
                    b += w.slen / (d * d);
                    continue;
                }
                for (int sgi = 0; sgi < 4; ++sgi) {
                    const double *A = w.a[sgi], *B = w.b[sgi];
                    double S[3];
                    hsub(S, B, A);
                    const double s2 = hdot(S, S);
                    if (!(s2 > 0)) continue;   // a segment of zero length adds nothing
                    double QA[3];
                    hsub(QA, qs[qi], A);
                    double u = hdot(QA, S) / s2;
                    u = u < 0 ? 0 : (u > 1 ? 1 : u);
                    double d[3];
                    for (int a = 0; a < 3; ++a) d[a] = QA[a] - u * S[a];
                    const double d2 = hdot(d, d);
                    if (!(d2 > 0)) return HUGE_VAL;
                    b += sqrt(s2) / d2;
                }
            }
        }
        return b * h.P->kappa / (4 * M_PI) * (1.0 + 1e-9);
    };
    // launch the pending corrections with the read-back of the candidates of
    // the pairs from the current one on
    auto flush = [&]() -> int {
        if (pend_m.empty()) {
            launched_gen = gen;
            return OV_OK;
        }
        ahead.clear();
        for (size_t qq = cur_q; qq < pairs.size() && qq < cur_q + kAhead; ++qq) {
            for (int node : {pairs[qq].first, pairs[qq].second}) {
                int cj = cand_index(node);
                if (cj < pend_from || cj >= ce || pf_gen[cj] == gen) continue;
                pf_gen[cj] = gen;
                pf_pos[cj] = (int)ahead.size();
                ahead.push_back(cj);
            }
        }
        const int rr = ov_rec_correct(c, pend_from, ce - pend_from, pend_m.data(), pend_f.data(), pend_s.data(),
                                      (int)pend_m.size(), ahead.data(), (int)ahead.size());
        pend_m.clear(); pend_f.clear(); pend_s.clear();
        pend_from = INT_MAX;
        launched_gen = gen;
        pf_waited = false;
        return rr;
    };
    // copy the corrections of the last correction's read-back list (complete
    // once ov_rec_wait returned)
    auto take_prefetch = [&]() {
        for (size_t i = 0; i < ahead.size(); ++i) {
            const int cj = ahead[i];
            if (pf_gen[cj] != gen || corr_gen[cj] >= gen) continue;
            for (int a = 0; a < 4; ++a) corr[4 * (size_t)cj + a] = c->h_pf[4 * i + a];
            corr_gen[cj] = gen;
        }
    };
    // lazy: the copy may lack the last kLazy rewirings (covered by the bound)
    auto velocity = [&](int k, const double tg[3], const double nm[3], double vel[3], double *bound,
                        bool lazy, bool *used_lazy) -> bool {
        double vs[3];
        if (!hlia(h, k, tg, nm, t, vs)) return false;
        int ci = cand_index(k);
        static const double zero4[4] = {0, 0, 0, 0};
        const double *rc, *cc;
        double extra = 0;
        if (used_lazy) *used_lazy = false;
        if (ex_gen[ci] == gen) {
            rc = &ex[5 * (size_t)ci];   // FP64 on the current topology: no corrections
            cc = zero4;
        } else {
            if (corr_gen[ci] < gen && lazy && gen - corr_gen[ci] <= kLazy) {
                extra = pending_bound(ci, k);
                if (used_lazy) *used_lazy = true;
                ++c->stats.reconnect_lazy_evals;
            } else if (corr_gen[ci] < gen) {
                const auto tf = clk();
                if (launched_gen < gen && flush()) return false;
                if (pf_gen[ci] == gen) {
                    if (!pf_waited) {
                        if (ov_rec_wait(c)) return false;
                        pf_waited = true;
                    }
                    take_prefetch();
                } else {
                    const int n = std::min(ce, ci + kFetch) - ci;
                    if (ov_rec_fetch(c, ci, n, corr + 4 * (size_t)ci)) return false;
                    std::fill(corr_gen.begin() + ci, corr_gen.begin() + ci + n, gen);
                    pf_waited = true;   // the stream is idle now
                }
                c->step_ms[12] += ms_since(tf);
            }
            rc = &rec[5 * (size_t)ci];
            cc = &corr[4 * (size_t)ci];
        }
        ++evaluated;
        for (int a = 0; a < 3; ++a) vs[a] = vs[a] + (rc[a] + cc[a]);
        hfriction(h, k, tg, vs, t, vel);
        const double tl = hlen(tg);
        const double n_terms = (double)(h.hi - h.lo) * (g.n_img + 1);
        // the reference's rounding covers the missing terms' magnitudes too
        const double comp = rc[3] + cc[3] + n_terms * 1.1102230246251565e-16 * (rc[4] + extra) + extra;
        // the friction terms are linear in vs: |d vel| <= |d vs| (1 + alpha |t| + alpha' |t|^2)
        *bound = comp * 1.7320508075688772 * 1.01 * (1.0 + fabs(h.P->alpha) * tl + fabs(h.P->alpha_p) * tl * tl);
        return true;
    };

    size_t i = 0;
    while (i < pairs.size()) {
        int k = pairs[i].first;
        size_t e = i;
        while (e < pairs.size() && pairs[e].first == k) ++e;
        int mk = member_of(k);
        cur_q = i;
        if (mk != cur_member && cur_member >= 0 && (r = flush())) return r;
        if (mk != cur_member) {
            cur_member = mk;
            h = host_of(c, mk);
            cos_cut = cos(h.P->reconnection_angle_cutoff);
            const Member &M = c->mem[mk];
            cb = cand_index(M.lo);
            ce = cand_index(M.lo + M.cap);
        }
        int sk = h.st(k);
        if (sk == OV_EMPTY || pinned(sk) || recalc[k]) { i = e; continue; }
        for (size_t q = i; q < e; ++q) {
            cur_q = q;
            int l = pairs[q].second;
            int sl = h.st(l);
            if (sl == OV_EMPTY || pinned(sl) || h.fwd(k) == l || h.rev(k) == l || recalc[l]) continue;
            double tk[3], nk[3], tl[3], nl_[3];
            if (!htangent(h, k, tk, nk) || !htangent(h, l, tl, nl_))
                return ov_fail(c, OV_ERR_TOPOLOGY, "reconnect: filament walk from %d or %d failed", k, l);
            if (hlen(tk) < 0.5 || hlen(tl) < 0.5) continue;
            if (hdot(tk, tl) / hlen(tk) / hlen(tl) > cos_cut) continue;
            double vk[3], vl[3], bk = 0, bl = 0;
            bool lk = false, ll = false;
            if (!velocity(k, tk, nk, vk, &bk, true, &lk) || !velocity(l, tl, nl_, vl, &bl, true, &ll))
                return ov_fail(c, OV_ERR_TOPOLOGY, "reconnect: velocity of %d or %d failed", k, l);
            double v1[3], v2[3], dx[3], dv[3];
            h.pos(k, v1);
            h.pos(l, v2);
            hpwrap(g, v1, v2);
            hsub(dx, v1, v2);
            hsub(dv, vk, vl);
            double proj = hdot(dx, dv);
            if ((lk || ll) && fabs(proj) <= hlen(dx) * (bk + bl) + 1e-9 * hlen(dx) * hlen(dv)) {
                // the bound on the missing corrections does not decide: the exact ones
                if (!velocity(k, tk, nk, vk, &bk, false, nullptr) || !velocity(l, tl, nl_, vl, &bl, false, nullptr))
                    return ov_fail(c, OV_ERR_TOPOLOGY, "reconnect: velocity of %d or %d failed", k, l);
                hsub(dv, vk, vl);
                proj = hdot(dx, dv);
            }
            if (fabs(proj) <= hlen(dx) * (bk + bl) + 1e-9 * hlen(dx) * hlen(dv)) {
                // the mixed-precision sums cannot decide: FP64 sums of both
                // on the current topology (the device's connections are
                // brought up to date first)
                int ck = cand_index(k), cl = cand_index(l);
                if (ex_gen[ck] != gen || ex_gen[cl] != gen) {
                    ++c->stats.reconnect_fp64_pairs;
                    double exv[10];
                    const auto te = clk();
                    if (pushed_gen != gen) {
                        OV_CUDA(c, cudaMemcpyAsync(c->fwd, c->h_fwd.data(), (size_t)c->n_live * sizeof(int),
                                                   cudaMemcpyHostToDevice, c->stream));
                        pushed_gen = gen;
                    }
                    if ((r = ov_rec_exact(c, k, l, exv))) return r;
                    pf_waited = true;
                    c->step_ms[14] += ms_since(te);
                    for (int a = 0; a < 5; ++a) {
                        ex[5 * (size_t)ck + a] = exv[a];
                        ex[5 * (size_t)cl + a] = exv[5 + a];
                    }
                    ex_gen[ck] = ex_gen[cl] = gen;
                    velocity(k, tk, nk, vk, &bk, false, nullptr);
                    velocity(l, tl, nl_, vl, &bl, false, nullptr);
                    hsub(dv, vk, vl);
                    proj = hdot(dx, dv);
                }
            }
            if (fabs(proj) <= hlen(dx) * (bk + bl) + 1e-9 * hlen(dx) * hlen(dv)) {
                // too close to call after a different summation order: redo
                // both velocities exactly as the reference sums them
                ++c->stats.reconnect_exact_pairs;
                const auto tx = clk();
                hdirect_exact(h, k, tk, nk, t, vk);
                hdirect_exact(h, l, tl, nl_, t, vl);
                c->step_ms[15] += ms_since(tx);
                hsub(dv, vk, vl);
                proj = hdot(dx, dv);
            }
            if (proj > 0) continue;
            int kn = h.fwd(k), kp = h.rev(k), ln = h.fwd(l), lp = h.rev(l);
            // do_reconnection (vortex_dynamics.c:128-175)
            auto slen = [&](int a, int b) {
                double pa[3], pb[3];
                h.pos(a, pa);
                h.pos(b, pb);
                return hpwrap_len(g, pa, pb);
            };
            double cf1 = slen(k, l) + slen(kn, lp) - slen(k, kn) - slen(l, lp);
            double cf2 = slen(k, l) + slen(kp, ln) - slen(k, kp) - slen(l, ln);
            if (cf1 > 0 && cf2 > 0) continue;
            int cm[4], cfw[4];
            double csg[4] = {-1.0, -1.0, 1.0, 1.0};
            if (cf1 < cf2) {
                cm[0] = k; cfw[0] = kn; cm[1] = lp; cfw[1] = l;     // removed
                h.fwd(k) = l; h.rev(l) = k;
                h.rev(kn) = lp; h.fwd(lp) = kn;
                cm[2] = k; cfw[2] = l; cm[3] = lp; cfw[3] = kn;     // added
            } else {
                cm[0] = l; cfw[0] = ln; cm[1] = kp; cfw[1] = k;
                h.fwd(l) = k; h.rev(k) = l;
                h.rev(ln) = kp; h.fwd(kp) = ln;
                cm[2] = l; cfw[2] = k; cm[3] = kp; cfw[3] = ln;
            }
            // the four changed segments' contributions to the member's
            // candidates still to come (pairs are (k, l > k), sorted by k)
            const int cfrom = cand_index(k) + 1;
            const auto tc = clk();
            {
                // the four changed segments as the sums see them (wrapped end)
                Rewire rr;
                for (int sgi = 0; sgi < 4; ++sgi) {
                    h.pos(cm[sgi], rr.a[sgi]);
                    h.pos(cfw[sgi], rr.b[sgi]);
                    hpwrap(g, rr.a[sgi], rr.b[sgi]);
                }
                for (int a = 0; a < 3; ++a) rr.c[a] = rr.a[0][a];
                double rho = 0, sl = 0;
                for (int sgi = 0; sgi < 4; ++sgi) {
                    double da[3], db[3], sv[3];
                    hsub(da, rr.a[sgi], rr.c);
                    hsub(db, rr.b[sgi], rr.c);
                    hsub(sv, rr.b[sgi], rr.a[sgi]);
                    rho = std::max(rho, std::max(sqrt(hdot(da, da)), sqrt(hdot(db, db))));
                    sl += sqrt(hdot(sv, sv));
                }
                rr.rho = rho * 1.01;   // covers the rounding of the distances above
                rr.slen = sl * 1.01;
                rw.push_back(rr);
            }
            ++gen;
            if (ce > cfrom) {
                // the correction joins the pending ones (launched 8 rewirings at a
                // time, or when a pair needs the exact corrections); a launch may
                // correct candidates between two rewirings' first candidates for a
                // later rewiring too: those are not decided again in this pass
                for (int sgi = 0; sgi < 4; ++sgi) {
                    pend_m.push_back(cm[sgi]);
                    pend_f.push_back(cfw[sgi]);
                    pend_s.push_back(csg[sgi]);
                }
                pend_from = std::min(pend_from, cfrom);
                if (pend_m.size() + 4 > 32) {
                    cur_q = e;
                    if ((r = flush())) return r;
                }
            }
            c->step_ms[13] += ms_since(tc);
            recalc[k]++; recalc[h.fwd(k)]++; recalc[h.rev(k)]++; recalc[kn]++; recalc[kp]++;
            recalc[l]++; recalc[h.fwd(l)]++; recalc[h.rev(l)]++; recalc[ln]++; recalc[lp]++;
            if (log_k && log_l && nrec < log_cap) { log_k[nrec] = k; log_l[nrec] = l; }
            nrec++;
            break;
        }
        i = e;
    }
    c->stats.reconnections = nrec;
    c->stats.reconnect_evaluated = evaluated;
    if (nrecs) *nrecs = nrec;
    c->step_ms[10] = ms_since(tr);
    tr = clk();
    if (nrec) {
        r = ov_push_device(c, 0);
        c->step_ms[11] = ms_since(tr);
        return r;
    }
    c->host_valid = true;
    return OV_OK;
}

int ov_smooth(ov_ctx *c)
{
    int r = ready(c);
    if (r) return r;
    bool any = false;
    for (const Member &m : c->mem) any = any || m.params.use_freq_filter;
    if (!any) return OV_OK;
    if ((r = ov_pull_host(c))) return r;
    // closed loops of each filtering member in the reference's discovery
    // order (vortex_smooth.c:192-210)
    std::vector<int> off{0}, nodes, long_off, long_nodes;
    std::vector<double> cut, long_cut;
    int maxlen = 0;
    for (int mi = 0; mi < (int)c->mem.size(); ++mi) {
        if (!c->mem[mi].params.use_freq_filter) continue;
        Host h = host_of(c, mi);
        const int lo = h.lo, N = h.hi - h.lo;
        std::vector<char> seen(N > 0 ? N : 1, 0);
        for (int i = lo; i < h.hi; ++i) {
            if (seen[i - lo]) continue;
            if (h.st(i) == OV_EMPTY) { seen[i - lo] = 1; continue; }
            // one forward walk from i: back at i closes a loop (none of whose
            // nodes can have been seen); the end of an open line, or a node a
            // walk along the same line already passed, leaves it unsmoothed
            int len = 0;
            int m = i;
            bool closed = false;
            const size_t start = nodes.size();
            while (m >= lo && m < h.hi && !seen[m - lo] && len <= N) {
                seen[m - lo] = 1;
                nodes.push_back(m);
                ++len;
                m = h.fwd(m);
                if (m == i) { closed = true; break; }
            }
            if (!closed) {   // open line: not smoothed
                nodes.resize(start);
                continue;
            }
            if (len > kLongLoop) {
                // long loop: the FFT path, after the short ones
                long_off.push_back((int)long_nodes.size());
                long_nodes.insert(long_nodes.end(), nodes.begin() + start, nodes.end());
                long_cut.push_back(h.P->freq_to_cutoff);
                nodes.resize(start);
                continue;
            }
            off.push_back((int)nodes.size());
            cut.push_back(h.P->freq_to_cutoff);
            maxlen = std::max(maxlen, len);
        }
    }
    long_off.push_back((int)long_nodes.size());
    // long loops first (they read the host mirror, which the short-loop
    // kernel does not touch; loops share no nodes)
    for (size_t q = 0; q + 1 < long_off.size(); ++q) {
        if ((r = smooth_long_loop(c, long_nodes.data() + long_off[q], long_off[q + 1] - long_off[q], long_cut[q])))
            return r;
        c->host_valid = false;
    }
    int nloops = (int)off.size() - 1;
    if (nloops == 0) return OV_OK;
    size_t total = nodes.size();
    if (c->loop_cap < nloops + 1 || c->loop_nodes_cap < (int)total) {
        if (c->d_loop_off) cudaFree(c->d_loop_off);
        if (c->d_loop_nodes) cudaFree(c->d_loop_nodes);
        if (c->d_loop_cut) cudaFree(c->d_loop_cut);
        c->d_loop_off = nullptr; c->d_loop_nodes = nullptr; c->d_loop_cut = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->d_loop_off, (size_t)(nloops + 1) * 4));
        OV_ALLOC(c, cudaMalloc(&c->d_loop_cut, (size_t)(nloops + 1) * sizeof(double)));
        OV_ALLOC(c, cudaMalloc(&c->d_loop_nodes, std::max(total, (size_t)1) * 4));
        c->loop_cap = nloops + 1;
        c->loop_nodes_cap = (int)total;
    }
    size_t need = total * 2 * 3 * sizeof(double);
    if (c->loop_buf_cap < need) {
        if (c->d_loop_buf) cudaFree(c->d_loop_buf);
        c->d_loop_buf = nullptr;
        OV_ALLOC(c, cudaMalloc(&c->d_loop_buf, need));
        c->loop_buf_cap = need;
    }
    OV_CUDA(c, cudaMemcpyAsync(c->d_loop_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice, c->stream));
    OV_CUDA(c, cudaMemcpyAsync(c->d_loop_cut, cut.data(), cut.size() * sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
    OV_CUDA(c, cudaMemcpyAsync(c->d_loop_nodes, nodes.data(), total * 4, cudaMemcpyHostToDevice, c->stream));
    SmoothArgs a;
    a.loop_off = c->d_loop_off;
    a.loop_nodes = c->d_loop_nodes;
    a.x = c->node.x; a.y = c->node.y; a.z = c->node.z;
    a.buf = c->d_loop_buf;
    a.geo = c->geo;
    a.cutoff = c->d_loop_cut;
    int Nmax = 2 * maxlen;
    size_t shbytes = (size_t)(2 * Nmax + 3 * (Nmax / 2 + 1 + Nmax)) * sizeof(double);
    if (shbytes > 200 * 1024) return ov_fail(c, OV_ERR_ARG, "loop of %d nodes too long to smooth", maxlen);
    if (shbytes > 48 * 1024)
        OV_CUDA(c, cudaFuncSetAttribute(k_smooth, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shbytes));
    c->tree_built = false;
    c->host_valid = false;
    k_smooth<<<nloops, 256, shbytes, c->stream>>>(a);
    c->launches++;
    OV_CUDA(c, cudaGetLastError());
    OV_CUDA(c, cudaStreamSynchronize(c->stream));
    return OV_OK;
}

int ov_enforce_wall_boundaries(ov_ctx *c, double t)
{
    int r = ready(c);
    if (r) return r;
    c->stats.wall_clipped = c->stats.wall_removed = 0;
    if (!any_solid_wall(c->geo)) return OV_OK;
    if ((r = ov_pull_host(c))) return r;
    c->host_valid = false;
    std::vector<int> new_nodes;
    int clipped = 0, removed = 0;
    for (int mi = 0; mi < (int)c->mem.size(); ++mi)
        if ((r = hwalls(c, mi, t, new_nodes, &clipped, &removed))) {
            ov_push_device(c, 1);
            return r;
        }
    c->stats.wall_clipped = clipped;
    c->stats.wall_removed = removed;
    if (!clipped && !removed) {
        c->host_valid = true;   // nothing changed (direct sums synced the device to the same state)
        return OV_OK;
    }
    if ((r = ov_push_device(c, 1))) return r;
    if (!new_nodes.empty()) {
        int *d = nullptr;
        OV_ALLOC(c, cudaMalloc(&d, new_nodes.size() * sizeof(int)));
        OV_CUDA(c, cudaMemcpy(d, new_nodes.data(), new_nodes.size() * sizeof(int), cudaMemcpyHostToDevice));
        k_zero_vel<<<((int)new_nodes.size() + 255) / 256, 256, 0, c->stream>>>(
            d, (int)new_nodes.size(), c->node.vx, c->node.vy, c->node.vz, c->node.sx, c->node.sy, c->node.sz);
        c->launches++;
        OV_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaFree(d);
    }
    return OV_OK;
}

int ov_add_loop(ov_ctx *c, int member, const double center[3], const double dir[3], double r)
{
    int rc = ready(c);
    if (rc) return rc;
    if (!center || !dir || member < 0 || member >= (int)c->mem.size() || !(r >= 0)) return OV_ERR_ARG;
    if ((rc = ov_pull_host(c))) return rc;
    c->host_valid = false;
    std::vector<int> added;
    rc = hadd_loop(c, member, center, dir, r, added);
    c->stats.injected_nodes = (int64_t)added.size();
    int rp = push_added(c, added);
    if (rc) return ov_fail(c, rc, "add_loop: no empty slot could be had");
    return rp;
}

int ov_add_line_in_zdir(ov_ctx *c, int member, double x, double y, int direction)
{
    int rc = ready(c);
    if (rc) return rc;
    if (member < 0 || member >= (int)c->mem.size()) return OV_ERR_ARG;
    if ((rc = ov_pull_host(c))) return rc;
    c->host_valid = false;
    std::vector<int> added;
    rc = hadd_line_z(c, member, x, y, direction, added);
    c->stats.injected_nodes = (int64_t)added.size();
    int rp = push_added(c, added);
    if (rc) return ov_fail(c, rc, "add_line_in_zdir: %s", rc == OV_ERR_ARG ? "no nodes fit the box" : "no empty slot");
    return rp;
}

int ov_set_injection(ov_ctx *c, int member, const ov_injection *inj)
{
    if (!c || !inj || member >= (int)c->mem.size() || c->mem.empty()) return OV_ERR_ARG;
    if (inj->line_n < 0) return OV_ERR_ARG;
    for (int mi = member < 0 ? 0 : member; mi < (member < 0 ? (int)c->mem.size() : member + 1); ++mi) {
        c->mem[mi].inj = *inj;
        c->mem[mi].last_loop = c->mem[mi].last_line = 0;
    }
    return OV_OK;
}

int ov_get_injection(const ov_ctx *c, int member, ov_injection *out)
{
    if (!c || !out || member < 0 || member >= (int)c->mem.size()) return OV_ERR_ARG;
    *out = c->mem[member].inj;
    return OV_OK;
}

int ov_inject_vortices(ov_ctx *c, double t)
{
    int rc = ready(c);
    if (rc) return rc;
    c->stats.injected_nodes = 0;
    if (!any_injection(c)) return OV_OK;
    LazyMirror mir{c};
    std::vector<int> added;
    for (int mi = 0; mi < (int)c->mem.size() && !rc; ++mi) {
        if (c->mem[mi].inj.loop_injection) rc = hinject_loop(c, mi, t, mir, added);
        if (!rc && c->mem[mi].inj.line_injection) rc = hinject_lines(c, mi, t, mir, added);
    }
    c->stats.injected_nodes = (int64_t)added.size();
    int rp = mir.pulled ? push_added(c, added) : OV_OK;
    if (rc) return ov_fail(c, rc, "inject_vortices: %s", rc == OV_ERR_ARG ? "no nodes fit the box" : "no empty slot");
    return rp;
}

double ov_erand48(unsigned short x[3]) { return x ? hrand48(x) : -1.0; }

int ov_step(ov_ctx *c, double t, double dt)
{
    int r = ready(c);
    if (r) return r;
    int nrec = 0;
    // host wall time of each pass: small loops, reconnect, smooth, periodic,
    // remesh, update_tangle, rk4_step, total
    double *ms = c->step_ms;
    for (int i = 0; i < 16; ++i) ms[i] = 0;
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto since = [&](std::chrono::steady_clock::time_point t0) {
        return std::chrono::duration<double, std::milli>(now() - t0).count();
    };
    const auto t_all = now();
    auto t0 = now();
    if (any_injection(c) && (r = ov_inject_vortices(c, t))) return r;   // main.c:123
    if ((r = ov_enforce_wall_boundaries(c, 0.0))) return r;   // main.c:125 (nothing to do in a periodic box)
    if ((r = ov_eliminate_small_loops(c))) return r;
    ms[0] += since(t0); t0 = now();
    if ((r = ov_reconnect(c, 0.0, &nrec, nullptr, nullptr, 0))) return r;
    ms[1] += since(t0); t0 = now();
    if ((r = ov_eliminate_small_loops(c))) return r;
    ms[0] += since(t0); t0 = now();
    if ((r = ov_smooth(c))) return r;
    ms[2] += since(t0); t0 = now();
    if ((r = ov_enforce_periodic_boundaries(c))) return r;
    ms[3] += since(t0); t0 = now();
    if ((r = ov_remesh(c, c->params.dl_min, c->params.dl_max, 0.0))) return r;
    ms[4] += since(t0); t0 = now();
    if ((r = ov_eliminate_small_loops(c))) return r;
    ms[0] += since(t0); t0 = now();
    if ((r = ov_update_tangle(c, t))) return r;
    ms[5] += since(t0); t0 = now();
    if ((r = ov_rk4_step(c, t, dt))) return r;
    ms[6] += since(t0); t0 = now();
    if ((r = ov_enforce_periodic_boundaries(c))) return r;
    ms[3] += since(t0);
    ms[7] = since(t_all);
    c->stats.reconnections = nrec;
    return OV_OK;
}

int ov_step_times(const ov_ctx *c, double *ms, int n)
{
    if (!c || !ms || n < 0) return OV_ERR_ARG;
    for (int i = 0; i < n && i < 16; ++i) ms[i] = c->step_ms[i];
    return OV_OK;
}

}  // extern "C"
