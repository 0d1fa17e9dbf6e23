/*
 * ov_oracle.c - TEST INFRASTRUCTURE ONLY (see ov_oracle.h).
 *
 * CPU restatement of OpenVort's velocity and time-step path.  Arithmetic is
 * written in the reference's operation order (noted per function) so that a
 * build with the same flags is bit-identical to the reference; the structure
 * around it (explicit parameters, explicit recursion helpers, the DFT used
 * in place of FFTW) is this project's own.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ov_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_E
#define M_E 2.7182818284590452354
#endif

/* ------------------------------------------------------------------ vec3
 * Each helper has the rounding sequence of its vec3_math.c counterpart:
 * dot/len accumulate from 0 in x,y,z order (vec3_math.c:91-96, 167-174),
 * ndot divides by each length in turn (:104-111). */
static inline ov_vec3 V(double x, double y, double z) { ov_vec3 r = {{x, y, z}}; return r; }
static inline ov_vec3 vsub(ov_vec3 a, ov_vec3 b) { return V(a.p[0] - b.p[0], a.p[1] - b.p[1], a.p[2] - b.p[2]); }
static inline ov_vec3 vadd(ov_vec3 a, ov_vec3 b) { return V(a.p[0] + b.p[0], a.p[1] + b.p[1], a.p[2] + b.p[2]); }
static inline ov_vec3 vmul(ov_vec3 a, double m) { return V(a.p[0] * m, a.p[1] * m, a.p[2] * m); }
static inline double vdot(ov_vec3 a, ov_vec3 b)
{
    double o = 0;
    o += a.p[0] * b.p[0];
    o += a.p[1] * b.p[1];
    o += a.p[2] * b.p[2];
    return o;
}
static inline double vlen(ov_vec3 a) { return sqrt(vdot(a, a)); }
static inline double vndot(ov_vec3 a, ov_vec3 b) { return vdot(a, b) / vlen(a) / vlen(b); }
static inline ov_vec3 vcross(ov_vec3 u, ov_vec3 v)
{
    return V(u.p[1] * v.p[2] - u.p[2] * v.p[1],
             u.p[2] * v.p[0] - u.p[0] * v.p[2],
             u.p[0] * v.p[1] - u.p[1] * v.p[0]);
}
/* vec3_normalize (vec3_math.c:208): multiply by the reciprocal length. */
static inline ov_vec3 vnormalize(ov_vec3 a)
{
    if (a.p[0] == 0 && a.p[1] == 0 && a.p[2] == 0) return a;
    double d = vlen(a);
    return vmul(a, 1 / d);
}

static const ov_vec3 kInwardNormal[6] = {
    {{1, 0, 0}}, {{-1, 0, 0}}, {{0, 1, 0}}, {{0, -1, 0}}, {{0, 0, 1}}, {{0, 0, -1}}};

/* ------------------------------------------------------------- geometry */

/* seg_pwrap (boundaries.c:54-83): move r2 by whole periods until it lies
 * within half a period of r1, per axis whose low wall is periodic.  The
 * bound on the loop only matters for non-finite input. */
static inline ov_vec3 pwrap(const ov_domain_box *box, ov_vec3 r1, ov_vec3 r2)
{
    static const int low_face[3] = {OV_LEFT, OV_BACK, OV_DOWN};
    for (int a = 0; a < 3; ++a) {
        if (box->wall[low_face[a]] != OV_WALL_PERIODIC) continue;
        double L = box->top_right_front.p[a] - box->bottom_left_back.p[a];
        int guard = 0;
        while ((r2.p[a] - r1.p[a]) > L / 2 && guard++ < 100000) r2.p[a] -= L;
        while ((r2.p[a] - r1.p[a]) < -L / 2 && guard++ < 200000) r2.p[a] += L;
    }
    return r2;
}
/* segment_len (vec3_math.h:94) of a wrapped segment: |r1 - r2|. */
static inline double pwrap_len(const ov_domain_box *box, ov_vec3 r1, ov_vec3 r2)
{
    return vlen(vsub(r1, pwrap(box, r1, r2)));
}

/* mirror_shift (boundaries.c:159-193) */
static ov_vec3 mirror_point(ov_vec3 v, const ov_domain_box *box, int wall)
{
    int axis = wall / 2;
    if (wall < 0 || wall > 5) return v;
    double w = (wall % 2 == 0) ? box->bottom_left_back.p[axis] : box->top_right_front.p[axis];
    v.p[axis] = 2 * w - v.p[axis];
    return v;
}

/* mirror_vector_reflect (boundaries.c:201-211) */
static ov_vec3 mirror_vector(ov_vec3 v, int wall)
{
    double nc = vdot(v, kInwardNormal[wall]);
    return vadd(v, vmul(kInwardNormal[wall], -2 * nc));
}

/* step_node (tangle.c:155-194): position `where` steps along the filament;
 * a pinned end is walked back and mirrored in its wall. */
ov_vec3 orc_step_node(const ov_tangle_state *t, int i, int where)
{
    if (where == 0) return t->vnodes[i];
    int st = t->status[i].status;
    if (st == OV_FREE) {
        if (where > 0) return orc_step_node(t, t->connections[i].forward, where - 1);
        return orc_step_node(t, t->connections[i].reverse, where + 1);
    }
    if (st == OV_PINNED || st == OV_PINNED_SLIP) {
        ov_vec3 back;
        if (where > 0) {
            if (t->connections[i].forward >= 0)
                return orc_step_node(t, t->connections[i].forward, where - 1);
            back = orc_step_node(t, i, -where);
        } else {
            if (t->connections[i].reverse >= 0)
                return orc_step_node(t, t->connections[i].reverse, where + 1);
            back = orc_step_node(t, i, -where);
        }
        return mirror_point(back, &t->box, t->status[i].pin_wall);
    }
    return V(0, 0, 0);
}

/* shifted (tangle.c:370-414): query point moved into an image tangle. */
static ov_vec3 image_point(const ov_image_tangle *img, const ov_tangle_state *t, ov_vec3 r)
{
    ov_vec3 rs = r;
    double Ls[3];
    for (int a = 0; a < 3; ++a) Ls[a] = t->box.top_right_front.p[a] - t->box.bottom_left_back.p[a];
    for (int a = 0; a < 3; ++a) rs.p[a] -= Ls[a] * img->shift[a];
    for (int m = 0; m < img->number_of_reflects; ++m) {
        int f = img->reflect[m];
        if (f < 0 || f > 5) continue;
        int axis = f / 2;
        double w = (f % 2 == 0) ? t->box.bottom_left_back.p[axis] : t->box.top_right_front.p[axis];
        rs.p[axis] = 2 * w - r.p[axis];
    }
    return rs;
}

/* get_v (external_velocity.c:62-81) */
static ov_vec3 ext_velocity(const ov_ext_vel *c, double time)
{
    switch (c->type) {
    case OV_SIMPLE:
        return vmul(vnormalize(c->direction), c->strength);
    case OV_DECREASING: {
        double s;
        if (time < c->time_of_linear_decrease)
            s = c->starting_strength - time * (c->starting_strength - c->strength) / c->time_of_linear_decrease;
        else
            s = c->strength;
        return vmul(vnormalize(c->direction), s);
    }
    default:
        return V(0, 0, 0);
    }
}

/* --------------------------------------------------------------- pool */

/* create_tangle (tangle.c:27-61) */
void orc_tangle_create(ov_tangle_state *t, int n)
{
    t->vnodes = (ov_vec3 *)malloc(sizeof(ov_vec3) * n);
    t->vels = (ov_vec3 *)malloc(sizeof(ov_vec3) * n);
    t->vs = (ov_vec3 *)malloc(sizeof(ov_vec3) * n);
    t->tangents = (ov_vec3 *)malloc(sizeof(ov_vec3) * n);
    t->normals = (ov_vec3 *)malloc(sizeof(ov_vec3) * n);
    t->recalculate = (int *)malloc(sizeof(int) * n);
    t->status = (ov_node_status *)malloc(sizeof(ov_node_status) * n);
    t->connections = (ov_neighbour *)malloc(sizeof(ov_neighbour) * n);
    for (int k = 0; k < n; ++k) {
        t->status[k].status = OV_EMPTY;
        t->status[k].pin_wall = OV_NOT_A_FACE;
        t->connections[k].forward = -1;
        t->connections[k].reverse = -1;
    }
    memset(&t->box, 0, sizeof(t->box));
    t->box.top_right_front = V(1, 1, 1);
    t->bimg.images = NULL;
    t->bimg.n = 0;
    t->N = n;
    t->next_empty = 0;
    t->total_empty = n;
}

void orc_tangle_free(ov_tangle_state *t)
{
    free(t->vnodes); free(t->vels); free(t->vs); free(t->tangents); free(t->normals);
    free(t->connections); free(t->recalculate); free(t->status);
    t->vnodes = t->vels = t->vs = t->tangents = t->normals = NULL;
    t->connections = NULL; t->recalculate = NULL; t->status = NULL;
}

/* search_next_empty_node (tangle.c:201-234).  The reference's linear scan
 * reads status[k+1] even for k = N-1; here a slot past the end counts as
 * not empty. */
static int search_empty(ov_tangle_state *t)
{
    if (t->next_empty > 0) {
        if (t->next_empty < t->N && t->status[t->next_empty].status == OV_EMPTY) {
            int id = t->next_empty;
            if (t->next_empty + 1 < t->N && t->status[t->next_empty + 1].status == OV_EMPTY)
                ++t->next_empty;
            else
                t->next_empty = -1;
            return id;
        }
    }
    for (int k = 0; k < t->N; ++k) {
        if (t->status[k].status == OV_EMPTY) {
            if (k + 1 < t->N && t->status[k + 1].status == OV_EMPTY) t->next_empty = k + 1;
            else t->next_empty = -1;
            return k;
        }
    }
    return -1;
}

/* get_next_empty_node (tangle.c:241-253) */
int orc_get_next_empty_node(ov_tangle_state *t)
{
    int id = search_empty(t);
    while (id < 0 || t->status[id].status != OV_EMPTY) {
        orc_tangle_expand(t, 2 * t->N);
        id = search_empty(t);
    }
    return id;
}

/* expand_tangle (tangle.c:68-101) */
void orc_tangle_expand(ov_tangle_state *t, int n)
{
    int old = t->N;
    t->vnodes = (ov_vec3 *)realloc(t->vnodes, sizeof(ov_vec3) * n);
    t->vels = (ov_vec3 *)realloc(t->vels, sizeof(ov_vec3) * n);
    t->vs = (ov_vec3 *)realloc(t->vs, sizeof(ov_vec3) * n);
    t->tangents = (ov_vec3 *)realloc(t->tangents, sizeof(ov_vec3) * n);
    t->normals = (ov_vec3 *)realloc(t->normals, sizeof(ov_vec3) * n);
    t->recalculate = (int *)realloc(t->recalculate, sizeof(int) * n);
    t->status = (ov_node_status *)realloc(t->status, sizeof(ov_node_status) * n);
    t->connections = (ov_neighbour *)realloc(t->connections, sizeof(ov_neighbour) * n);
    for (int k = old; k < n; ++k) {
        t->status[k].status = OV_EMPTY;
        t->status[k].pin_wall = OV_NOT_A_FACE;
        t->connections[k].forward = -1;
        t->connections[k].reverse = -1;
    }
    t->N = n;
    t->total_empty += n - old;
    t->next_empty = orc_get_next_empty_node(t);
}

/* ----------------------------------------------------------- tangents */

/* update_tangent_normal (tangle.c:423-502): fourth-order finite differences
 * on the non-uniform 5-point stencil k-2..k+2. */
void orc_update_tangent_normal(ov_tangle_state *t, int k)
{
    if (t->status[k].status == OV_EMPTY) return;
    const ov_domain_box *box = &t->box;
    ov_vec3 s0 = t->vnodes[k];
    ov_vec3 s1 = orc_step_node(t, k, 1);
    ov_vec3 s2 = orc_step_node(t, k, 2);
    ov_vec3 sm1 = orc_step_node(t, k, -1);
    ov_vec3 sm2 = orc_step_node(t, k, -2);

    /* ds[j] = wrapped(end) - start, stencil order {+2, +1, -1, -2} */
    ov_vec3 w2 = pwrap(box, s0, s2), w1 = pwrap(box, s0, s1);
    ov_vec3 wm1 = pwrap(box, s0, sm1), wm2 = pwrap(box, s0, sm2);
    ov_vec3 ds[4] = {vsub(w2, s0), vsub(w1, s0), vsub(wm1, s0), vsub(wm2, s0)};

    double d1 = vlen(vsub(s0, w1));
    double d2 = d1 + pwrap_len(box, s1, s2);
    double dm1 = vlen(vsub(s0, wm1));
    double dm2 = dm1 + pwrap_len(box, sm1, sm2);

    double den[4] = {
        d2 * (d2 - d1) * (dm1 + d2) * (dm2 + d2),
        d1 * (d2 - d1) * (dm1 + d1) * (dm2 + d1),
        dm1 * (dm1 + d1) * (dm1 + d2) * (dm2 - dm1),
        dm2 * (dm2 + d1) * (dm2 + d2) * (dm2 - dm1)};
    double c1[4] = {-d1 * dm1 * dm2, d2 * dm1 * dm2, -d1 * d2 * dm2, d1 * d2 * dm1};
    double c2[4] = {
        2 * ((dm1 - d1) * dm2 - d1 * dm1),
        -2 * ((dm1 - d2) * dm2 - d2 * dm1),
        2 * ((d2 + d1) * dm2 - d1 * d2),
        -2 * ((d2 + d1) * dm1 - d1 * d2)};

    for (int a = 0; a < 3; ++a) {
        double tg = 0, nm = 0;
        for (int z = 0; z < 4; ++z) {
            tg += c1[z] / den[z] * ds[z].p[a];
            nm += c2[z] / den[z] * ds[z].p[a];
        }
        t->tangents[k].p[a] = tg;
        t->normals[k].p[a] = nm;
    }
}

void orc_update_tangents_normals(ov_tangle_state *t)
{
    for (int i = 0; i < t->N; ++i) orc_update_tangent_normal(t, i);
}

/* --------------------------------------------------------------- octree */

struct orc_cell {
    int n, cap;
    int *ids;
    ov_vec3 com;
    ov_vec3 circ;
    ov_domain_box box;
    orc_cell *child[8];
};

static orc_cell *cell_new(int cap)
{
    orc_cell *c = (orc_cell *)calloc(1, sizeof(orc_cell));
    c->cap = cap > 0 ? cap : 8;
    c->ids = (int *)malloc(sizeof(int) * c->cap);
    return c;
}

static void cell_push(orc_cell *c, int id)
{
    if (c->n == c->cap) {
        c->cap *= 2;
        c->ids = (int *)realloc(c->ids, sizeof(int) * c->cap);
    }
    c->ids[c->n++] = id;
}

void orc_octree_destroy(orc_cell *c)
{
    if (!c) return;
    for (int i = 0; i < 8; ++i) orc_octree_destroy(c->child[i]);
    free(c->ids);
    free(c);
}

/* make_child_box (octree.c:165-232).  Child order BLF, BLB, BRF, BRB, TLF,
 * TLB, TRF, TRB; each child is built from the parent's corners, centre
 * c = (blb+trf)*0.5 and half sides L/2 exactly as there, so the boxes carry
 * the same rounding. */
static ov_domain_box child_box(const ov_domain_box *pb, int idx)
{
    ov_vec3 b = pb->bottom_left_back, t = pb->top_right_front;
    ov_vec3 c = vmul(vadd(b, t), 0.5);
    ov_vec3 L = vsub(t, b);
    ov_domain_box cb = *pb;
    switch (idx) {
    case 0: cb.bottom_left_back = b; cb.bottom_left_back.p[0] += L.p[0] / 2;
            cb.top_right_front = c; cb.top_right_front.p[0] += L.p[0] / 2; break;
    case 1: cb.bottom_left_back = b; cb.top_right_front = c; break;
    case 2: cb.bottom_left_back = c; cb.bottom_left_back.p[2] -= L.p[2] / 2;
            cb.top_right_front = t; cb.top_right_front.p[2] -= L.p[2] / 2; break;
    case 3: cb.bottom_left_back = b; cb.bottom_left_back.p[1] += L.p[1] / 2;
            cb.top_right_front = c; cb.top_right_front.p[1] += L.p[1] / 2; break;
    case 4: cb.bottom_left_back = c; cb.bottom_left_back.p[1] -= L.p[1] / 2;
            cb.top_right_front = t; cb.top_right_front.p[1] -= L.p[1] / 2; break;
    case 5: cb.bottom_left_back = b; cb.bottom_left_back.p[2] += L.p[2] / 2;
            cb.top_right_front = c; cb.top_right_front.p[2] += L.p[2] / 2; break;
    case 6: cb.bottom_left_back = c; cb.top_right_front = t; break;
    default: cb.bottom_left_back = c; cb.bottom_left_back.p[0] -= L.p[0] / 2;
             cb.top_right_front = t; cb.top_right_front.p[0] -= L.p[0] / 2; break;
    }
    return cb;
}

/* in_octree_box (octree.c:88-104): closed on every face. */
static inline int in_closed_box(const ov_domain_box *b, const ov_vec3 *v)
{
    return v->p[0] >= b->bottom_left_back.p[0] && v->p[0] <= b->top_right_front.p[0] &&
           v->p[1] >= b->bottom_left_back.p[1] && v->p[1] <= b->top_right_front.p[1] &&
           v->p[2] >= b->bottom_left_back.p[2] && v->p[2] <= b->top_right_front.p[2];
}

/* octree_inner_sort (octree.c:110-133): split until a cell holds <= 1 node;
 * a node goes to the first child whose closed box holds it, and a node held
 * by no child (outside the root box) stays only in the ancestors. */
static void cell_split(orc_cell *c, const ov_tangle_state *t, int depth)
{
    if (c->n <= 1) return;
    if (depth > 200) {
        fprintf(stderr, "oracle octree: depth limit (coincident nodes)\n");
        return;
    }
    int cap = c->cap / 8;
    if (cap == 0) cap = 8;
    for (int i = 0; i < 8; ++i) {
        c->child[i] = cell_new(cap);
        c->child[i]->box = child_box(&c->box, i);
    }
    for (int k = 0; k < c->n; ++k) {
        int id = c->ids[k];
        for (int i = 0; i < 8; ++i) {
            if (in_closed_box(&c->child[i]->box, &t->vnodes[id])) {
                cell_push(c->child[i], id);
                break;
            }
        }
    }
    for (int i = 0; i < 8; ++i) cell_split(c->child[i], t, depth + 1);
}

/* octree_update_means (octree.c:258-286): COM = sum of positions in
 * node-id order times 1/N; circulation = sum of wrapped forward segments. */
static void cell_moments(orc_cell *c, const ov_tangle_state *t)
{
    if (!c || c->n == 0) return;
    ov_vec3 s = V(0, 0, 0);
    for (int k = 0; k < c->n; ++k) s = vadd(s, t->vnodes[c->ids[k]]);
    c->com = vmul(s, 1.0 / c->n);
    ov_vec3 q = V(0, 0, 0);
    for (int k = 0; k < c->n; ++k) {
        int id = c->ids[k];
        int f = t->connections[id].forward;
        if (f > -1) {
            ov_vec3 r2 = pwrap(&t->box, t->vnodes[id], t->vnodes[f]);
            q = vadd(q, vsub(r2, t->vnodes[id]));
        }
    }
    c->circ = q;
    for (int i = 0; i < 8; ++i) cell_moments(c->child[i], t);
}

/* octree_build (octree.c:139-158): root holds every non-EMPTY node and the
 * domain box. */
orc_cell *orc_octree_build(const ov_tangle_state *t)
{
    orc_cell *root = cell_new(t->N);
    for (int k = 0; k < t->N; ++k)
        if (t->status[k].status != OV_EMPTY) cell_push(root, k);
    root->box = t->box;
    cell_split(root, t, 0);
    cell_moments(root, t);
    return root;
}

/* The segment law shared by the tree monopole (octree.c:321-342) and the
 * direct sum (tangle.c:536-559): velocity at the origin of R induced by the
 * straight segment from R to Rp1, with the reference's three filters. */
static inline ov_vec3 segment_law(ov_vec3 R, ov_vec3 Rp1, double kappa)
{
    double lR = vlen(R);
    double lRp1 = vlen(Rp1);
    double denom = lR * lRp1 * (lR * lRp1 + vdot(R, Rp1));
    double f = kappa / 4 / M_PI;
    if (lR < 1e-8 || lRp1 < 1e-8) return V(0, 0, 0);
    if (vndot(R, Rp1) < 1e-8) return V(0, 0, 0);
    return vmul(vcross(R, Rp1), f * (lR + lRp1) / denom);
}

/* octree_get_vs (octree.c:296-356) */
void orc_octree_get_vs(const ov_tangle_state *t, const orc_cell *c, const ov_vec3 *r,
                       double resolution, const ov_params *p, ov_vec3 *res)
{
    *res = V(0, 0, 0);
    if (c->n == 0) return;
    double Lx = c->box.top_right_front.p[0] - c->box.bottom_left_back.p[0];
    double Ly = c->box.top_right_front.p[1] - c->box.bottom_left_back.p[1];
    double Lz = c->box.top_right_front.p[2] - c->box.bottom_left_back.p[2];
    double Lm = Lx > Ly ? (Lx > Lz ? Lx : Lz) : (Ly > Lz ? Ly : Lz);
    double d = vlen(vsub(*r, c->com));
    if (d < 1e-8) return;
    if (Lm / d < resolution || c->n == 1) {
        ov_vec3 R = vsub(c->com, *r);
        ov_vec3 Rp1 = vadd(R, c->circ);
        *res = segment_law(R, Rp1, p->kappa);
        return;
    }
    ov_vec3 sum = V(0, 0, 0), part;
    for (int i = 0; i < 8; ++i) {
        orc_octree_get_vs(t, c->child[i], r, resolution, p, &part);
        sum = vadd(sum, part);
    }
    *res = sum;
}

static void count_walk(const orc_cell *c, const ov_vec3 *r, double resolution, orc_counts *o)
{
    if (c->n == 0) return;
    o->visits++;
    double Lx = c->box.top_right_front.p[0] - c->box.bottom_left_back.p[0];
    double Ly = c->box.top_right_front.p[1] - c->box.bottom_left_back.p[1];
    double Lz = c->box.top_right_front.p[2] - c->box.bottom_left_back.p[2];
    double Lm = Lx > Ly ? (Lx > Lz ? Lx : Lz) : (Ly > Lz ? Ly : Lz);
    double d = vlen(vsub(*r, c->com));
    if (d < 1e-8) return;
    if (Lm / d < resolution || c->n == 1) { o->accepts++; return; }
    for (int i = 0; i < 8; ++i) count_walk(c->child[i], r, resolution, o);
}

static void count_cells(const orc_cell *c, int depth, orc_counts *o)
{
    if (!c || c->n == 0) return;
    o->cells++;
    if (depth > o->max_depth) o->max_depth = depth;
    for (int i = 0; i < 8; ++i) count_cells(c->child[i], depth + 1, o);
}

/* Interaction statistics of the reference tree: visits/accepts summed over
 * all non-EMPTY targets and their 1+n_img query points. */
void orc_count_interactions(const ov_tangle_state *t, double resolution, orc_counts *out)
{
    memset(out, 0, sizeof(*out));
    orc_cell *tree = orc_octree_build(t);
    count_cells(tree, 0, out);
    for (int k = 0; k < t->N; ++k) {
        if (t->status[k].status == OV_EMPTY) continue;
        count_walk(tree, &t->vnodes[k], resolution, out);
        for (int j = 0; j < t->bimg.n; ++j) {
            ov_vec3 q = image_point(&t->bimg.images[j], t, t->vnodes[k]);
            count_walk(tree, &q, resolution, out);
        }
    }
    orc_octree_destroy(tree);
}

/* Per-target visits and accepts of the reference tree (the counts of
 * orc_count_interactions, node by node): visits[k], accepts[k] over node k's
 * 1 + n_img query points; zero for EMPTY slots.  threads <= 0: one. */
void orc_node_interactions(const ov_tangle_state *t, double resolution, int threads, long long *visits,
                           long long *accepts)
{
    orc_cell *tree = orc_octree_build(t);
    const int nthr = threads > 0 ? threads : 1;
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 64)
    for (int k = 0; k < t->N; ++k) {
        orc_counts o;
        memset(&o, 0, sizeof o);
        if (t->status[k].status != OV_EMPTY) {
            count_walk(tree, &t->vnodes[k], resolution, &o);
            for (int j = 0; j < t->bimg.n; ++j) {
                ov_vec3 q = image_point(&t->bimg.images[j], t, t->vnodes[k]);
                count_walk(tree, &q, resolution, &o);
            }
        }
        visits[k] = o.visits;
        accepts[k] = o.accepts;
    }
    orc_octree_destroy(tree);
}

/* ------------------------------------------------------------- velocity */

/* lia_velocity (tangle.c:568-592) */
static ov_vec3 lia(const ov_tangle_state *t, int i, const ov_params *p)
{
    ov_vec3 x = t->vnodes[i];
    ov_vec3 nx = orc_step_node(t, i, +1);
    ov_vec3 pv = orc_step_node(t, i, -1);
    double l_next = pwrap_len(&t->box, x, nx);
    double l_prev = pwrap_len(&t->box, pv, x);
    double f = p->kappa * log(2 * sqrt(l_next * l_prev) / sqrt(M_E) / p->vortex_width) / 4 / M_PI;
    return vmul(vcross(t->tangents[i], t->normals[i]), f);
}

/* segment_field (tangle.c:525-560): segment m -> forward(m) seen from r. */
static inline ov_vec3 segment_field(const ov_tangle_state *t, int m, ov_vec3 r, double kappa)
{
    int nx = t->connections[m].forward;
    if (nx == -1) return V(0, 0, 0);
    ov_vec3 a = t->vnodes[m];
    ov_vec3 b = pwrap(&t->box, a, t->vnodes[nx]);
    return segment_law(vsub(a, r), vsub(b, r), kappa);
}

/* update_velocity (tangle.c:600-726) */
void orc_update_velocity(ov_tangle_state *t, int k, double time, const orc_cell *tree,
                         const ov_params *p)
{
    int st = t->status[k].status;
    if (st == OV_EMPTY) return;
    if (st == OV_PINNED) {
        t->vs[k] = V(0, 0, 0);
        t->vels[k] = ext_velocity(&p->vb, time);
        return;
    }
    t->vs[k] = lia(t, k, p);
    t->vs[k] = vadd(t->vs[k], ext_velocity(&p->vs, time));

    ov_vec3 images = V(0, 0, 0);
    if (p->use_bh && tree) {
        ov_vec3 v;
        orc_octree_get_vs(t, tree, &t->vnodes[k], p->bh_resolution, p, &v);
        t->vs[k] = vadd(t->vs[k], v);
        for (int j = 0; j < t->bimg.n; ++j) {
            const ov_image_tangle *img = &t->bimg.images[j];
            ov_vec3 q = image_point(img, t, t->vnodes[k]);
            orc_octree_get_vs(t, tree, &q, p->bh_resolution, p, &v);
            for (int m = 0; m < img->number_of_reflects; ++m) v = mirror_vector(v, img->reflect[m]);
            images = vadd(images, v);
        }
    } else {
        /* Direct sum, accumulated straight into vs[k]: the primary tangle
         * skips the two segments touching k, the images skip nothing and
         * (as in the reference) are added without the mirror reflection. */
        ov_vec3 x = t->vnodes[k];
        for (int m = 0; m < t->N; ++m) {
            int f = t->connections[m].forward;
            if (f == -1 || k == m || k == f) continue;
            t->vs[k] = vadd(t->vs[k], segment_field(t, m, x, p->kappa));
        }
        for (int j = 0; j < t->bimg.n; ++j) {
            ov_vec3 q = image_point(&t->bimg.images[j], t, x);
            for (int m = 0; m < t->N; ++m) {
                if (t->connections[m].forward == -1) continue;
                t->vs[k] = vadd(t->vs[k], segment_field(t, m, q, p->kappa));
            }
        }
    }
    t->vs[k] = vadd(t->vs[k], images);
    t->vels[k] = t->vs[k];

    if (p->use_mutual_friction) {
        ov_vec3 dv = vsub(ext_velocity(&p->vn, time), t->vs[k]);
        ov_vec3 tg = t->tangents[k];
        t->vels[k] = vadd(t->vels[k], vmul(vcross(tg, dv), p->alpha));
        t->vels[k] = vadd(t->vels[k], vmul(vcross(tg, vcross(tg, dv)), -p->alpha_p));
    }
    if (st == OV_PINNED_SLIP) {
        ov_vec3 n = kInwardNormal[t->status[k].pin_wall];
        double nv = vdot(n, t->vels[k]);
        t->vels[k] = vsub(t->vels[k], vmul(n, nv));
    }
}

/* update_velocities (tangle.c:733-749) */
void orc_update_velocities(ov_tangle_state *t, double time, const ov_params *p)
{
    orc_cell *tree = p->use_bh ? orc_octree_build(t) : NULL;
    int nthr = p->num_threads > 0 ? p->num_threads : 1;
    int i;
#pragma omp parallel for num_threads(nthr) schedule(static)
    for (i = 0; i < t->N; ++i) orc_update_velocity(t, i, time, tree, p);
    orc_octree_destroy(tree);
}

void orc_direct_velocities(ov_tangle_state *t, const int *nodes, int n, double time,
                           const ov_params *p)
{
    int nthr = p->num_threads > 0 ? p->num_threads : 1;
    int i;
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 1)
    for (i = 0; i < n; ++i) orc_update_velocity(t, nodes[i], time, NULL, p);
}

/* ------------------------------------------------------------------ RK4 */

/* euler_step2 (vortex_dynamics.c:20-42) */
static void euler_into(ov_tangle_state *dst, const ov_tangle_state *src, double dt, const ov_vec3 *vel)
{
    for (int k = 0; k < src->N; ++k) {
        if (src->status[k].status == OV_EMPTY) continue;
        dst->vnodes[k] = vadd(src->vnodes[k], vmul(vel[k], dt));
    }
}

/* rk4_step (vortex_dynamics.c:50-119): stage times t+dt/2, t+dt/2, t+dt and
 * every stage displaced by dt/2 from the start (k4 included), stage
 * positions left unwrapped, combine dt/6, dt/3, dt/3, dt/6. */
void orc_rk4_step(ov_tangle_state *t, double time, double dt, const ov_params *p)
{
    int N = t->N;
    ov_tangle_state st[3];
    for (int s = 0; s < 3; ++s) {
        orc_tangle_create(&st[s], N);
        st[s].bimg = t->bimg;
        st[s].box = t->box;
        for (int k = 0; k < N; ++k) {
            st[s].status[k] = t->status[k];
            st[s].connections[k] = t->connections[k];
        }
    }
    euler_into(&st[0], t, dt / 2, t->vels);
    orc_update_tangents_normals(&st[0]);
    orc_update_velocities(&st[0], time + dt / 2, p);
    euler_into(&st[1], t, dt / 2, st[0].vels);
    orc_update_tangents_normals(&st[1]);
    orc_update_velocities(&st[1], time + dt / 2, p);
    euler_into(&st[2], t, dt / 2, st[1].vels);
    orc_update_tangents_normals(&st[2]);
    orc_update_velocities(&st[2], time + dt, p);

    for (int k = 0; k < N; ++k) {
        if (t->status[k].status == OV_EMPTY) continue;
        ov_vec3 mv = vmul(t->vels[k], dt / 6);
        mv = vadd(mv, vmul(st[0].vels[k], dt / 3));
        mv = vadd(mv, vmul(st[1].vels[k], dt / 3));
        mv = vadd(mv, vmul(st[2].vels[k], dt / 6));
        t->vnodes[k] = vadd(t->vnodes[k], mv);
    }
    for (int s = 0; s < 3; ++s) orc_tangle_free(&st[s]);
}

/* ------------------------------------------------------------ reconnect */

/* do_reconnection (vortex_dynamics.c:128-175) */
static int rewire(ov_tangle_state *t, int k, int l)
{
    int kf = t->connections[k].forward, kr = t->connections[k].reverse;
    int lf = t->connections[l].forward, lr = t->connections[l].reverse;
    const ov_domain_box *b = &t->box;
#define SLEN(x, y) pwrap_len(b, t->vnodes[x], t->vnodes[y])
    double cf1 = SLEN(k, l) + SLEN(kf, lr) - SLEN(k, kf) - SLEN(l, lr);
    double cf2 = SLEN(k, l) + SLEN(kr, lf) - SLEN(k, kr) - SLEN(l, lf);
#undef SLEN
    if (cf1 > 0 && cf2 > 0) return 0;
    if (cf1 < cf2) {
        t->connections[k].forward = l;
        t->connections[l].reverse = k;
        t->connections[kf].reverse = lr;
        t->connections[lr].forward = kf;
    } else {
        t->connections[l].forward = k;
        t->connections[k].reverse = l;
        t->connections[lf].reverse = kr;
        t->connections[kr].forward = lf;
    }
    return 1;
}

static inline int is_pinned(int st) { return st == OV_PINNED || st == OV_PINNED_SLIP; }

/* reconnect (vortex_dynamics.c:186-288): sequential pair scan; tangents and
 * direct-sum velocities of the candidates are recomputed on the current
 * (already rewired) tangle. */
int orc_reconnect(ov_tangle_state *t, double time, const ov_params *p,
                  int *log_k, int *log_l, int log_cap)
{
    int nrec = 0;
    for (int k = 0; k < t->N; ++k) t->recalculate[k] = 0;
    double cos_cut = cos(p->reconnection_angle_cutoff);
    for (int k = 0; k < t->N; ++k) {
        int sk = t->status[k].status;
        if (sk == OV_EMPTY || is_pinned(sk) || t->recalculate[k]) continue;
        for (int l = k + 1; l < t->N; ++l) {
            int sl = t->status[l].status;
            if (sl == OV_EMPTY || is_pinned(sl) || t->connections[k].forward == l ||
                t->connections[k].reverse == l || t->recalculate[l])
                continue;
            ov_vec3 v1 = t->vnodes[k];
            ov_vec3 v2 = pwrap(&t->box, v1, t->vnodes[l]);
            if (vlen(vsub(v1, v2)) > p->rec_dist) continue;

            orc_update_tangent_normal(t, k);
            orc_update_tangent_normal(t, l);
            ov_vec3 d1 = t->tangents[k], d2 = t->tangents[l];
            if (vlen(d1) < 0.5 || vlen(d2) < 0.5) continue;
            if (vndot(d1, d2) > cos_cut) continue;

            orc_update_velocity(t, k, time, NULL, p);
            orc_update_velocity(t, l, time, NULL, p);
            ov_vec3 dx = vsub(v1, v2);
            ov_vec3 dv = vsub(t->vels[k], t->vels[l]);
            if (vdot(dx, dv) > 0) continue;

            int kn = t->connections[k].forward, kp = t->connections[k].reverse;
            int ln = t->connections[l].forward, lp = t->connections[l].reverse;
            if (!rewire(t, k, l)) continue;

            t->recalculate[k]++;
            t->recalculate[t->connections[k].forward]++;
            t->recalculate[t->connections[k].reverse]++;
            t->recalculate[kn]++;
            t->recalculate[kp]++;
            t->recalculate[l]++;
            t->recalculate[t->connections[l].forward]++;
            t->recalculate[t->connections[l].reverse]++;
            t->recalculate[ln]++;
            t->recalculate[lp]++;
            if (log_k && nrec < log_cap) { log_k[nrec] = k; log_l[nrec] = l; }
            nrec++;
            break;
        }
    }
    return nrec;
}

/* --------------------------------------------------------------- remesh */

/* add_point (tangle.c:261-335): new node on the circle through p and its
 * forward neighbour with the mean curvature of the two. */
static int insert_after(ov_tangle_state *t, int p)
{
    int np = orc_get_next_empty_node(t);
    t->status[np].status = OV_FREE;
    t->status[np].pin_wall = OV_NOT_A_FACE;
    int nx = t->connections[p].forward;
    orc_update_tangent_normal(t, p);
    orc_update_tangent_normal(t, nx);
    ov_vec3 s0pp = t->normals[p], s1pp = t->normals[nx];
    ov_vec3 s0 = t->vnodes[p];
    ov_vec3 s1 = pwrap(&t->box, s0, t->vnodes[nx]);
    double l = vlen(vsub(s0, s1));
    ov_vec3 n = vmul(vadd(s0pp, s1pp), 0.5);
    ov_vec3 pos;
    if (vlen(n) > 1e-5) {
        double R = 1 / vlen(n);
        double dR = R * R - l * l / 4;
        double delta = dR > 0 ? R - sqrt(dR) : R;
        n = vnormalize(n);
        n = vmul(n, -1);
        ov_vec3 a = vmul(vadd(s0, s1), 0.5);
        pos = vadd(a, vmul(n, delta));
    } else {
        pos = vmul(vadd(s0, s1), 0.5);
    }
    t->vnodes[np] = pos;
    t->vs[np] = V(0, 0, 0);
    t->vels[np] = V(0, 0, 0);
    t->connections[np].reverse = p;
    t->connections[np].forward = nx;
    t->connections[p].forward = np;
    t->connections[nx].reverse = np;
    return np;
}

/* remove_point (tangle.c:342-355) */
static void drop_node(ov_tangle_state *t, int i)
{
    int pv = t->connections[i].reverse, nx = t->connections[i].forward;
    if (pv >= 0) t->connections[pv].forward = nx;
    if (nx >= 0) t->connections[nx].reverse = pv;
    t->connections[i].reverse = t->connections[i].forward = -1;
    t->status[i].status = OV_EMPTY;
}

/* out_of_box (tangle.c:761-787): the last out-of-range face in the order
 * -x,+x,-y,+y,-z,+z wins; non-periodic faces report -1. */
static int face_outside(const ov_tangle_state *t, const ov_vec3 *w)
{
    const double *lo = t->box.bottom_left_back.p, *hi = t->box.top_right_front.p;
    int face = -1;
    if (w->p[0] < lo[0]) face = OV_LEFT;
    if (w->p[0] > hi[0]) face = OV_RIGHT;
    if (w->p[1] < lo[1]) face = OV_BACK;
    if (w->p[1] > hi[1]) face = OV_FRONT;
    if (w->p[2] < lo[2]) face = OV_DOWN;
    if (w->p[2] > hi[2]) face = OV_UP;
    if (face > -1 && t->box.wall[face] != OV_WALL_PERIODIC) face = -1;
    return face;
}

/* enforce_periodic_boundaries (tangle.c:793-814) with periodic_shift
 * (boundaries.c:113-150). */
void orc_enforce_periodic_boundaries(ov_tangle_state *t)
{
    for (int k = 0; k < t->N; ++k) {
        if (t->status[k].status == OV_EMPTY) continue;
        int face, guard = 0;
        while ((face = face_outside(t, &t->vnodes[k])) >= 0 && guard++ < 100000) {
            int axis = face / 2;
            double L = t->box.top_right_front.p[axis] - t->box.bottom_left_back.p[axis];
            if (face % 2 == 0) t->vnodes[k].p[axis] += L;
            else t->vnodes[k].p[axis] -= L;
        }
    }
}

/* remesh (tangle.c:1018-1061).  The pass re-reads N, so nodes inserted at
 * higher indices are visited in the same pass. */
void orc_remesh(ov_tangle_state *t, double min_dist, double max_dist, double time,
                const ov_params *p, int *n_added, int *n_removed)
{
    (void)time; (void)p;
    int added = 0, removed = 0;
    for (int k = 0; k < t->N; ++k) {
        if (t->status[k].status == OV_EMPTY) continue;
        int nx = t->connections[k].forward, pv = t->connections[k].reverse;
        double lf = 0, lr = 0;
        if (nx >= 0) lf = pwrap_len(&t->box, t->vnodes[k], t->vnodes[nx]);
        if (pv >= 0) lr = pwrap_len(&t->box, t->vnodes[k], t->vnodes[pv]);
        if (nx >= 0 && pv >= 0 && ((lf < min_dist || lr < min_dist) && (lf + lr) < max_dist)) {
            drop_node(t, k);
            removed++;
        }
        if (nx >= 0 && lf > max_dist) {
            added++;
            int np = insert_after(t, k);
            orc_update_tangent_normal(t, np);
        }
    }
    if (added) {
        orc_enforce_periodic_boundaries(t);
        /* enforce_wall_boundaries: only its reset of `recalculate` has an
         * effect when every wall is periodic (tangle.c:968-974). */
        for (int k = 0; k < t->N; ++k) t->recalculate[k] = 0;
    }
    if (n_added) *n_added = added;
    if (n_removed) *n_removed = removed;
}

/* eliminate_small_loops (tangle.c:1063-1128) */
int orc_eliminate_small_loops(ov_tangle_state *t, const ov_params *p)
{
    int removed_nodes = 0;
    char *seen = (char *)calloc(t->N > 0 ? t->N : 1, 1);
    for (int k = 0; k < t->N; ++k) {
        if (t->status[k].status == OV_EMPTY || seen[k]) continue;
        seen[k] = 1;
        int steps = 0;
        int here = k, nx = t->connections[here].forward;
        while (nx != k) {
            if (is_pinned(t->status[here].status) && nx < 0) {
                here = k;
                nx = t->connections[here].reverse;
                while (nx >= 0) {
                    seen[here] = 1;
                    here = nx;
                    nx = t->connections[here].reverse;
                    steps++;
                }
                break;
            }
            if (nx < 0) break; /* open end on a free node: not a valid tangle */
            seen[here] = 1;
            here = nx;
            nx = t->connections[here].forward;
            steps++;
        }
        if (steps < p->small_loop_cutoff) {
            nx = here;
            for (;;) {
                int cur = nx;
                nx = t->connections[nx].forward;
                t->connections[cur].forward = -1;
                t->connections[cur].reverse = -1;
                t->status[cur].status = OV_EMPTY;
                removed_nodes++;
                if (nx == here || nx < 0) break;
            }
        }
    }
    free(seen);
    return removed_nodes;
}

/* ------------------------------------------------------------ smoothing */

/* low_pass_filter (vortex_smooth.c:134-175).  The reference asks FFTW for a
 * real-to-real transform and documents the half-complex (R2HC) layout; this
 * restatement uses a direct R2HC DFT, zeroes the same middle bins and
 * applies the unnormalised HC2R inverse, then divides by N. */
void orc_low_pass_filter(double *in, int n, double freq_to_cutoff)
{
    if (n <= 0) return;
    double *hc = (double *)calloc(n, sizeof(double));
    for (int k = 0; k <= n / 2; ++k) {
        double re = 0, im = 0;
        for (int j = 0; j < n; ++j) {
            long long m = ((long long)j * k) % n;
            double ang = 2 * M_PI * (double)m / n;
            re += in[j] * cos(ang);
            im -= in[j] * sin(ang);
        }
        hc[k] = re;
        if (k > 0 && k < n - k) hc[n - k] = im;
    }
    int cut = (int)(freq_to_cutoff * n / 2);
    if (n > 2 * cut + 1) {
        int hi = (n % 2 == 0) ? n / 2 + 1 + cut : n / 2 + cut;
        for (int i = n / 2 - cut; i < hi; ++i) hc[i] = 0;
    }
    for (int j = 0; j < n; ++j) {
        double s = hc[0];
        for (int k = 1; k < n - k; ++k) {
            long long m = ((long long)j * k) % n;
            double ang = 2 * M_PI * (double)m / n;
            s += 2 * (hc[k] * cos(ang) - hc[n - k] * sin(ang));
        }
        if (n % 2 == 0) s += hc[n / 2] * ((j % 2) ? -1.0 : 1.0);
        in[j] = s / n;
    }
    free(hc);
}

/* high_freq_cutoff (vortex_smooth.c:183-453) for closed loops: unwrap the
 * loop by seg_pwrap from its first node, filter x, y, z as functions of the
 * node index, write back.  A loop whose unwrapped ends are more than half a
 * box apart is treated as the reference does: detrended, odd-extended to
 * 2L-2 samples, filtered, trend restored.  Open (wall-pinned) lines are out
 * of scope for periodic boxes and are left untouched. */
void orc_smooth(ov_tangle_state *t, const ov_params *p)
{
    if (!p->use_freq_filter) return;
    char *seen = (char *)calloc(t->N > 0 ? t->N : 1, 1);
    for (int i = 0; i < t->N; ++i) {
        if (seen[i]) continue;
        if (t->status[i].status == OV_EMPTY) { seen[i] = 1; continue; }
        /* is_vortex_open (vortex_smooth.c:24-39) */
        int j = i;
        while (t->connections[j].reverse != i && t->connections[j].reverse != -1)
            j = t->connections[j].reverse;
        if (t->connections[j].reverse == -1) { seen[i] = 1; continue; }
        int len = 1;
        for (int m = t->connections[i].forward; m != i; m = t->connections[m].forward) len++;
        double *c[3];
        for (int a = 0; a < 3; ++a) c[a] = (double *)malloc(sizeof(double) * (2 * len + 2));
        int k = i;
        for (int a = 0; a < 3; ++a) c[a][0] = t->vnodes[k].p[a];
        seen[k] = 1;
        k = t->connections[k].forward;
        for (int s = 1; s < len; ++s) {
            ov_vec3 prev = V(c[0][s - 1], c[1][s - 1], c[2][s - 1]);
            ov_vec3 w = pwrap(&t->box, prev, t->vnodes[k]);
            for (int a = 0; a < 3; ++a) c[a][s] = w.p[a];
            seen[k] = 1;
            k = t->connections[k].forward;
        }
        ov_vec3 gap = V(c[0][0] - c[0][len - 1], c[1][0] - c[1][len - 1], c[2][0] - c[2][len - 1]);
        double halfx = (t->box.top_right_front.p[0] - t->box.bottom_left_back.p[0]) / 2;
        if (vlen(gap) > halfx && len > 2) {
            double coef[3], c0[3];
            for (int a = 0; a < 3; ++a) {
                coef[a] = (c[a][len - 1] - c[a][0]) / (len - 1);
                c0[a] = c[a][0];
                c[a][len - 1] = 0;
                c[a][0] = 0;
                for (int s = 1; s < len - 1; ++s) c[a][s] = c[a][s] - coef[a] * s - c0[a];
                for (int s = 0; s < len - 2; ++s) c[a][len + s] = -c[a][len - 2 - s];
                orc_low_pass_filter(c[a], 2 * len - 2, p->freq_to_cutoff);
                for (int s = 0; s < len; ++s) c[a][s] = c[a][s] + coef[a] * s + c0[a];
            }
        } else {
            for (int a = 0; a < 3; ++a) orc_low_pass_filter(c[a], len, p->freq_to_cutoff);
        }
        k = i;
        for (int s = 0; s < len; ++s) {
            for (int a = 0; a < 3; ++a) t->vnodes[k].p[a] = c[a][s];
            k = t->connections[k].forward;
        }
        for (int a = 0; a < 3; ++a) free(c[a]);
    }
    free(seen);
}

/* One main-loop body (main.c:125-141) for a fully periodic box with no
 * injection: walls are no-ops there (tangle.c:974). */
void orc_step(ov_tangle_state *t, double time, double dt, const ov_params *p, int *n_recs)
{
    orc_eliminate_small_loops(t, p);
    int r = orc_reconnect(t, 0.0, p, NULL, NULL, 0);
    if (n_recs) *n_recs = r;
    orc_eliminate_small_loops(t, p);
    orc_smooth(t, p);
    orc_enforce_periodic_boundaries(t);
    orc_remesh(t, p->dl_min, p->dl_max, 0.0, p, NULL, NULL);
    orc_eliminate_small_loops(t, p);
    orc_update_tangents_normals(t);
    orc_update_velocities(t, time, p);
    orc_rk4_step(t, time, dt, p);
    orc_enforce_periodic_boundaries(t);
}

/* ------------------------------------------------------------ injection */

/* perpendicular + add_loop (vortex_injection.c:18-103) */
void orc_add_loop(ov_tangle_state *t, const ov_vec3 *center, const ov_vec3 *dir, double r,
                  const ov_params *p)
{
    int npts = (int)(4 * M_PI * r / (p->dl_max + p->dl_min));
    for (;;) {
        int empty = 0;
        for (int k = 0; k < t->N; ++k) empty += t->status[k].status == OV_EMPTY;
        if (empty >= npts) break;
        orc_tangle_expand(t, 2 * t->N);
    }
    ov_vec3 ex = V(1, 0, 0), ey = V(0, 1, 0);
    ov_vec3 z = vadd(vmul(*dir, -vdot(ex, *dir)), ex);
    if (vlen(z) > 1e-8) z = vnormalize(z);
    else z = vnormalize(vadd(vmul(*dir, -vdot(ey, *dir)), ey));
    ov_vec3 u = vcross(z, *dir);
    ov_vec3 v = vnormalize(vcross(*dir, u)); /* built from u before u is normalised */
    u = vnormalize(u);
    int first = -1, last = -1, cur = -1;
    for (int k = 0; k < npts; ++k) {
        double phi = 2 * M_PI / npts * k;
        double c = cos(phi), s = sin(phi);
        ov_vec3 pt = vadd(vadd(vmul(u, r * c), vmul(v, r * s)), *center);
        cur = orc_get_next_empty_node(t);
        if (first < 0) first = cur;
        t->status[cur].status = OV_FREE;
        t->vnodes[cur] = pt;
        if (cur != first) {
            t->connections[cur].reverse = last;
            t->connections[last].forward = cur;
        }
        last = cur;
    }
    t->connections[cur].forward = first;
    t->connections[first].reverse = cur;
}
