/*
 * ov_oracle_sph.c - TEST INFRASTRUCTURE ONLY (see ov_oracle.h).
 *
 * CPU restatement of the velocity path of OpenVort's spherical fork
 * (src_spherical/): the section-of-shell geometry (vec3_math.c:240-282,
 * boundaries.c:13-72), its octree over (radius, azimuth, polar angle)
 * boxes (octree.c), step_node / update_tangent_normal / lia_velocity /
 * update_velocity / update_velocities (tangle.c:156-1042) with the outer
 * surface open, and the He II temperature model (temperature_functions.c).
 * Arithmetic follows the fork's operation order, so a build with the same
 * flags and libm reproduces the fork's results.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ov_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_E
#define M_E 2.7182818284590452354
#endif

typedef ov_vec3 V3;

static inline V3 mk(double x, double y, double z) { V3 r = {{x, y, z}}; return r; }
static inline V3 add3(V3 a, V3 b) { return mk(a.p[0] + b.p[0], a.p[1] + b.p[1], a.p[2] + b.p[2]); }
static inline V3 sub3(V3 a, V3 b) { return mk(a.p[0] - b.p[0], a.p[1] - b.p[1], a.p[2] - b.p[2]); }
static inline V3 mul3(V3 a, double m) { return mk(a.p[0] * m, a.p[1] * m, a.p[2] * m); }
static inline double dot3(V3 a, V3 b)
{
    double o = 0;
    for (int k = 0; k < 3; ++k) o += a.p[k] * b.p[k];
    return o;
}
static inline double len3(V3 a) { return sqrt(dot3(a, a)); }
static inline V3 cross3(V3 u, V3 v)
{
    return mk(u.p[1] * v.p[2] - u.p[2] * v.p[1], u.p[2] * v.p[0] - u.p[0] * v.p[2],
              u.p[0] * v.p[1] - u.p[1] * v.p[0]);
}
static inline V3 unit3(V3 v)
{
    if (v.p[0] == 0 && v.p[1] == 0 && v.p[2] == 0) return v;
    return mul3(v, 1 / len3(v));
}

/* ------------------------------------------------------ section geometry */
static inline double s_radius(V3 v) { return sqrt(v.p[0] * v.p[0] + v.p[1] * v.p[1] + v.p[2] * v.p[2]); }
static inline double s_azimut(V3 v) { return atan2(v.p[2], sqrt(v.p[1] * v.p[1] + v.p[0] * v.p[0])); }
static inline double s_polar(V3 v)
{
    if (v.p[0] == 0 && v.p[1] == 0) return 0.0;
    return atan2(v.p[1], v.p[0]);
}
static inline V3 s_vec(double r, double az, double pl)
{
    return mk(r * cos(az) * cos(pl), r * cos(az) * sin(pl), r * sin(az));
}
static inline V3 s_invert(V3 v, double R)
{
    double r = s_radius(v);
    return s_vec(R * R / r, s_azimut(v), s_polar(v));
}
static inline V3 s_rotate(V3 v, double daz, double dpl)
{
    return s_vec(s_radius(v), s_azimut(v) + daz, s_polar(v) + dpl);
}
/* seg_pwrap: r2 rebuilt from its radius and angles moved toward r1's */
static V3 s_pwrap(const ov_sph_domain *d, V3 r1, V3 r2)
{
    double a1 = s_azimut(r1), a2 = s_azimut(r2);
    while (a2 - a1 > d->azimut_angle) a2 -= 2 * d->azimut_angle;
    while (a2 - a1 < -d->azimut_angle) a2 += 2 * d->azimut_angle;
    double p1 = s_polar(r1), p2 = s_polar(r2);
    while (p2 - p1 > d->polar_angle) p2 -= 2 * d->polar_angle;
    while (p2 - p1 < -d->polar_angle) p2 += 2 * d->polar_angle;
    return s_vec(s_radius(r2), a2, p2);
}
static inline double s_dist(V3 a, V3 b) { return len3(sub3(a, b)); }

/* step_node: a pinned end walks back and inverts through its surface */
static V3 s_step(const ov_sph_tangle_state *t, int i, int where)
{
    if (where == 0) return t->vnodes[i];
    int st = t->status[i].status;
    if (st == OV_FREE) {
        if (where > 0) return s_step(t, t->connections[i].forward, where - 1);
        return s_step(t, t->connections[i].reverse, where + 1);
    }
    V3 out;
    if (where > 0) {
        if (t->connections[i].forward >= 0) return s_step(t, t->connections[i].forward, where - 1);
        out = s_step(t, i, -where);
    } else {
        if (t->connections[i].reverse >= 0) return s_step(t, t->connections[i].reverse, where + 1);
        out = s_step(t, i, -where);
    }
    if (t->status[i].pin_wall == 0) return s_invert(out, t->domain_section.inner_radius);
    return s_invert(out, t->domain_section.outer_radius);
}

/* ------------------------------------------------------------- tangents */
static void s_tangent_normal(ov_sph_tangle_state *t, int k)
{
    if (t->status[k].status == OV_EMPTY) return;
    const ov_sph_domain *d = &t->domain_section;
    V3 s0 = t->vnodes[k], s1 = s_step(t, k, 1), s2 = s_step(t, k, 2);
    V3 sm1 = s_step(t, k, -1), sm2 = s_step(t, k, -2);
    V3 w2 = s_pwrap(d, s0, s2), w1 = s_pwrap(d, s0, s1), wm1 = s_pwrap(d, s0, sm1), wm2 = s_pwrap(d, s0, sm2);
    V3 ds[4] = {sub3(w2, s0), sub3(w1, s0), sub3(wm1, s0), sub3(wm2, s0)};
    double d1 = s_dist(s0, w1);
    double d2 = d1 + s_dist(s1, s_pwrap(d, s1, s2));
    double dm1 = s_dist(s0, wm1);
    double dm2 = dm1 + s_dist(sm1, s_pwrap(d, sm1, sm2));
    double den[4] = {d2 * (d2 - d1) * (dm1 + d2) * (dm2 + d2), d1 * (d2 - d1) * (dm1 + d1) * (dm2 + d1),
                     dm1 * (dm1 + d1) * (dm1 + d2) * (dm2 - dm1), dm2 * (dm2 + d1) * (dm2 + d2) * (dm2 - dm1)};
    double c1[4] = {-d1 * dm1 * dm2, d2 * dm1 * dm2, -d1 * d2 * dm2, d1 * d2 * dm1};
    double c2[4] = {2 * ((dm1 - d1) * dm2 - d1 * dm1), -2 * ((dm1 - d2) * dm2 - d2 * dm1),
                    2 * ((d2 + d1) * dm2 - d1 * d2), -2 * ((d2 + d1) * dm1 - d1 * d2)};
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

/* --------------------------------------------------- section octree */
typedef struct scell {
    int n, cap;
    int *ids;
    double b[6];   /* inner, outer, +az, -az, +pl, -pl */
    V3 com, circ;
    struct scell *child[8];
} scell;

static scell *sc_new(int cap)
{
    scell *c = (scell *)calloc(1, sizeof(scell));
    c->cap = cap > 0 ? cap : 8;
    c->ids = (int *)malloc(sizeof(int) * c->cap);
    return c;
}
static void sc_push(scell *c, int id)
{
    if (c->n == c->cap) {
        c->cap *= 2;
        c->ids = (int *)realloc(c->ids, sizeof(int) * c->cap);
    }
    c->ids[c->n++] = id;
}
static void sc_free(scell *c)
{
    if (!c) return;
    for (int i = 0; i < 8; ++i) sc_free(c->child[i]);
    free(c->ids);
    free(c);
}
/* child idx: bit 0 the inner radial half, bit 1 the upper polar half,
 * bit 2 the upper azimuth half (the fork's BLF..TRB order) */
static void sc_child(const double *pb, int idx, double *cb)
{
    double mr = (pb[1] + pb[0]) / 2, ma = (pb[2] + pb[3]) / 2, mp = (pb[4] + pb[5]) / 2;
    cb[0] = (idx & 1) ? pb[0] : mr;
    cb[1] = (idx & 1) ? mr : pb[1];
    cb[2] = (idx & 4) ? pb[2] : ma;
    cb[3] = (idx & 4) ? ma : pb[3];
    cb[4] = (idx & 2) ? pb[4] : mp;
    cb[5] = (idx & 2) ? mp : pb[5];
}
static int sc_holds(const double *b, V3 v)
{
    double r = s_radius(v), az = s_azimut(v), pl = s_polar(v);
    return r >= b[0] && r <= b[1] && az >= b[3] && az <= b[2] && pl >= b[5] && pl <= b[4];
}
static void sc_split(scell *c, const ov_sph_tangle_state *t, int depth)
{
    if (c->n <= 1 || depth > 200) return;
    int cap = c->cap / 8;
    if (cap == 0) cap = 8;
    for (int i = 0; i < 8; ++i) {
        c->child[i] = sc_new(cap);
        sc_child(c->b, i, c->child[i]->b);
    }
    for (int k = 0; k < c->n; ++k)
        for (int i = 0; i < 8; ++i)
            if (sc_holds(c->child[i]->b, t->vnodes[c->ids[k]])) {
                sc_push(c->child[i], c->ids[k]);
                break;
            }
    for (int i = 0; i < 8; ++i) sc_split(c->child[i], t, depth + 1);
}
static void sc_moments(scell *c, const ov_sph_tangle_state *t, double dl_max)
{
    if (!c || c->n == 0) return;
    V3 s = mk(0, 0, 0);
    for (int k = 0; k < c->n; ++k) s = add3(s, t->vnodes[c->ids[k]]);
    c->com = mul3(s, 1.0 / c->n);
    V3 q = mk(0, 0, 0);
    for (int k = 0; k < c->n; ++k) {
        int id = c->ids[k], f = t->connections[id].forward;
        if (f > -1) {
            V3 ds = sub3(s_pwrap(&t->domain_section, t->vnodes[id], t->vnodes[f]), t->vnodes[id]);
            if (!(len3(ds) > 5 * dl_max)) q = add3(q, ds);
        }
    }
    c->circ = q;
    for (int i = 0; i < 8; ++i) sc_moments(c->child[i], t, dl_max);
}
static scell *sc_build(const ov_sph_tangle_state *t, double dl_max)
{
    scell *root = sc_new(t->N);
    for (int k = 0; k < t->N; ++k)
        if (t->status[k].status != OV_EMPTY) sc_push(root, k);
    const ov_sph_domain *d = &t->domain_section;
    root->b[0] = d->inner_radius; root->b[1] = d->outer_radius;
    root->b[2] = d->azimut_angle; root->b[3] = -d->azimut_angle;
    root->b[4] = d->polar_angle; root->b[5] = -d->polar_angle;
    sc_split(root, t, 0);
    sc_moments(root, t, dl_max);
    return root;
}
static V3 sc_vs(const scell *c, V3 r, double theta, double kappa)
{
    if (!c || c->n == 0) return mk(0, 0, 0);
    double rd = c->b[1] - c->b[0];
    double az = c->b[1] * 2 * fabs(sin((c->b[2] - c->b[3]) / 2));
    double pl = c->b[1] * 2 * fabs(sin((c->b[4] - c->b[5]) / 2)) * fabs(cos((c->b[2] + c->b[3]) / 2));
    double Lm = rd > az ? (rd > pl ? rd : pl) : (az > pl ? az : pl);
    double d = s_dist(r, c->com);
    if (d < 1e-8) return mk(0, 0, 0);
    if (Lm / d < theta || c->n == 1) {
        V3 R = sub3(c->com, r), Rp1 = add3(R, c->circ);
        double lR = len3(R), lRp1 = len3(Rp1);
        double denom = lR * lRp1 * (lR * lRp1 + dot3(R, Rp1));
        double f = kappa / 4 / M_PI;
        if (lR < 1e-8 || lRp1 < 1e-8) return mk(0, 0, 0);
        if (dot3(R, Rp1) / len3(R) / len3(Rp1) < 1e-8) return mk(0, 0, 0);
        return mul3(cross3(R, Rp1), f * (lR + lRp1) / denom);
    }
    V3 tot = mk(0, 0, 0);
    for (int i = 0; i < 8; ++i) tot = add3(tot, sc_vs(c->child[i], r, theta, kappa));
    return tot;
}

/* ------------------------------------------------------ He II model */
static double spline(int len, const double *A, const double *Q, double x, int *err)
{
    int N = len - 5 - 1;
    if (x < Q[4] || x > Q[N + 5]) { *err = 1; return 0.0; }
    int I = 0, J = N + 1;
    while (J - I > 1) {
        int K = (I + J) / 2;
        if (x >= Q[K + 4]) I = K; else J = K;
    }
    double D[32];
    int JP3 = J + 3;
    for (int i = J; i <= JP3; ++i) D[i] = A[i];
    for (int K = 1; K <= 3; ++K)
        for (int i = J; i <= JP3 - K; ++i)
            D[i] = ((x - Q[i + K]) * D[i + 1] + (Q[i + 4] - x) * D[i]) / (Q[i + 4] - Q[i + K]);
    return D[J];
}
static const double LAMBDA = 2.1768;
static double he_super(double T, int *err)
{
    static const double Q[26] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.443, 0.9012, 1.5419, 1.7540, 1.918, 2.111, 2.156991,
                                 2.173218, 2.175647, 2.176358, 2.176568, 2.176692, 2.176766, 2.176791, 2.176798,
                                 2.176799, 2.17679999, 2.1768, 2.1768, 2.1768, 2.1768};
    static const double A[26] = {0.0, 1.451275432822459e-1, 1.451334563362309e-1, 1.449759191497576e-1,
                                 1.455008000684433e-1, 1.4075e-1, 1.095e-1, 8.15e-2, 5.30e-2, 2.1e-2, 8.904576e-3,
                                 3.053214e-3, 1.494043e-3, 8.342826e-4, 5.10686e-4, 2.8379e-4, 1.287426e-4,
                                 5.202569e-5, 2.153580e-5, 8.564206e-6, 3.567958e-6, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (!(T >= 0.0 && T <= LAMBDA)) { *err = 1; return 0.0; }
    return spline(26, A, Q, T, err) * 1000;
}
static double he_total(double T, int *err)
{
    static const double a1[3] = {0.0, -7.57537e-3, 6.87483e-3}, a2[3] = {0.0, -7.94605e-3, 5.07051e-3};
    static const double b1[8] = {0.0, 3.79937e-3, 1.86557e-3, 4.88345e-3, 0.0, 0.0, 0.0, 0.0};
    static const double b2[8] = {0.0, -30.3511e-3, -10.2326e-3, -3.00636e-3, 0.240720e-3, -2.45749e-3, 1.53454e-3,
                                 -0.308182e-3};
    static const double m[5] = {0.0, -1.26935e-5, 7.12413e-5, -16.7461e-5, 8.75342e-5};
    if (!(T >= 0 && T <= 4.9)) { *err = 1; return 0.0; }
    double t = T - LAMBDA, ro = 0.0;
    if (T < 1.344) {
        for (int i = 1; i <= 4; ++i) ro = ro + m[i] * pow(T, i + 1);
        ro = ro + 0.1451397;
    } else {
        const double *a = T <= LAMBDA ? a1 : a2, *b = T <= LAMBDA ? b1 : b2;
        double dro = 0;
        for (int i = 1; i <= 2; ++i)
            if (t != 0) dro = dro + a[i] * pow(t, i) * log(fabs(t));
        for (int i = 1; i <= 7; ++i) dro = dro + b[i] * pow(t, i);
        ro = 0.1461087 * (dro + 1);
    }
    return ro * 1000;
}
static double he_entropy(double T, int *err)
{
    static const double Q[30] = {0.0, 0.10000, 0.10000, 0.10000, 0.10000, 0.11123, 0.21625, 0.27672, 0.44817,
                                 0.56369, 0.71969, 0.85360, 1.00186, 1.40184, 1.72912, 1.99887, 2.07775, 2.15384,
                                 2.17680, 2.17680, 2.17680, 2.21160, 2.34820, 2.69075, 4.38277, 4.76361, 5.00000,
                                 5.0, 5.0, 5.0};
    static const double A[30] = {0.0, 6.60e-6, 7.60e-6, 1.60e-5, 4.61413e-5, 1.8400e-4, 4.68675e-4, 0.00121,
                                 0.00236, 0.00561, 0.01978, 0.08337, 0.35824, 0.76882, 1.17803, 1.38629, 1.53613,
                                 1.58271, 1.62419, 1.72261, 1.91862, 2.53529, 3.16601, 4.10379, 4.44077, 4.61570,
                                 0.0, 0.0, 0.0, 0.0};
    if (!(T >= 0.1 && T <= 5.0)) { *err = 1; return 0.0; }
    return spline(30, A, Q, T, err) * 1000;
}
static double he_normal(double T, int *err)
{
    if (!(T >= 1.1 && T <= LAMBDA)) { *err = 1; return 0.0; }
    return he_total(T, err) - he_super(T, err);
}
static double he_alpha(double T, int *err)
{
    static const double Q[12] = {0.0, -5.0, -5.0, -5.0, -5.0, -2.5, -2.0, -0.8, -0.387958059947, -0.387958059947,
                                 -0.387958059947, -0.387958059947};
    static const double A[12] = {0.0, 1.31928144433, 1.12452707801, 0.639314792565, 0.313383532495,
                                 -0.162687403543, 0.092047691284, 0.188452616588, 0.0, 0.0, 0.0, 0.0};
    if (!(T >= 1.3 && T < LAMBDA)) { *err = 1; return 0.0; }
    double b = T <= 2.167 ? pow(10, spline(12, A, Q, log10(1 - T / LAMBDA), err))
                          : 0.47 * pow(1 - T / LAMBDA, -0.33);
    return (b / 2) * (1 - he_super(T, err) / he_total(T, err));
}
static double he_alpha_p(double T, int *err)
{
    static const double Q[13] = {0.0, -5.0, -5.0, -5.0, -5.0, -3.55, -3.2, -2.5, -1.0, -0.384067377871,
                                 -0.384067377871, -0.384067377871, -0.384067377871};
    static const double A[13] = {0.0, -8.47218032526e-2, 0.931621715174, 0.973263359433, 1.10543591819,
                                 1.15904485127, 1.18311634566, 1.17480594214, 1.19458392766, 0.0, 0.0, 0.0, 0.0};
    if (!(T >= 1.3 && T < LAMBDA)) { *err = 1; return 0.0; }
    double b = T <= 2.134 ? pow(10, spline(13, A, Q, log10(1 - T / LAMBDA), err)) - 15
                          : -0.34 * pow(1 - T / LAMBDA, -0.33) + 1.01;
    return (b / 2) * (1 - he_super(T, err) / he_total(T, err));
}

/* ------------------------------------------------------------ velocity */
typedef struct sph_ctx {
    const ov_sph_params *p;
    double T_A;   /* the profile's A (bath terms) */
} sph_ctx;

static void s_velocity(ov_sph_tangle_state *t, const ov_sph_tangle_state *img, int k, const scell *tree,
                       const scell *itree, const sph_ctx *sc, int *err)
{
    const ov_sph_params *p = sc->p;
    int st = t->status[k].status;
    if (st == OV_EMPTY) return;
    if (st == OV_PINNED) { t->vs[k] = mk(0, 0, 0); return; }
    const ov_sph_domain *dom = &t->domain_section;
    /* LIA with the fork's segment-length limits */
    V3 x = t->vnodes[k], nx = s_step(t, k, 1), pv = s_step(t, k, -1);
    double l_next = s_dist(x, s_pwrap(dom, x, nx)), l_prev = s_dist(pv, s_pwrap(dom, pv, x));
    if (l_next > 4 * p->dl_max) l_next = 4 * p->dl_max;
    if (l_prev > 4 * p->dl_max) l_prev = 4 * p->dl_max;
    if (l_next < p->dl_min / 4) l_next = p->dl_min / 4;
    if (l_prev < p->dl_min / 4) l_prev = p->dl_min / 4;
    double f = p->kappa * log(2 * sqrt(l_next * l_prev) / sqrt(M_E) / p->vortex_width) / 4 / M_PI;
    V3 vs = mul3(cross3(t->tangents[k], t->normals[k]), f);
    double T = 0;
    double rr = s_radius(x) * 0.01;
    if (p->use_temperature) {
        T = p->temp_bath + sc->T_A / 5 * pow(rr, -5);
        double v_s = -p->q_dot * he_normal(T, err) /
                     (T * he_entropy(T, err) * he_super(T, err) * he_total(T, err) * 4 * M_PI * pow(rr, 2));
        vs = add3(vs, mul3(unit3(x), v_s * 100));
    }
    vs = add3(vs, sc_vs(tree, x, p->bh_resolution, p->kappa));
    double daz = 2 * dom->azimut_angle, dpl = 2 * dom->polar_angle;
    static const double sa[8] = {1, -1, 0, 0, 1, -1, 1, -1}, sp[8] = {0, 0, 1, -1, 1, 1, -1, -1};
    V3 tot = mk(0, 0, 0);
    for (int j = 0; j < 8; ++j) {
        V3 q = s_rotate(x, sa[j] * daz, sp[j] * dpl);
        tot = add3(tot, s_rotate(sc_vs(tree, q, p->bh_resolution, p->kappa), -sa[j] * daz, -sp[j] * dpl));
    }
    tot = sub3(tot, sc_vs(itree, x, p->bh_resolution, p->kappa));
    for (int j = 0; j < 8; ++j) {
        V3 q = s_rotate(x, sa[j] * daz, sp[j] * dpl);
        tot = sub3(tot, s_rotate(sc_vs(itree, q, p->bh_resolution, p->kappa), -sa[j] * daz, -sp[j] * dpl));
    }
    vs = add3(vs, tot);
    t->vs[k] = vs;
    V3 vel = vs;
    if (p->use_mutual_friction) {
        V3 dv = mk(0, 0, 0);
        double a = p->alpha, ap = p->alpha_p;
        if (p->use_temperature) {
            double v_n = p->q_dot / (T * he_entropy(T, err) * he_total(T, err) * 4 * M_PI * pow(rr, 2));
            dv = mul3(unit3(x), v_n * 100);
            a = he_alpha(T, err);
            ap = he_alpha_p(T, err);
        }
        dv = sub3(dv, vs);
        V3 tg = t->tangents[k];
        vel = add3(vel, mul3(cross3(tg, dv), a));
        vel = add3(vel, mul3(cross3(tg, cross3(tg, dv)), -ap));
    }
    if (st == OV_PINNED_SLIP) {
        V3 n = unit3(x);
        if (t->status[k].pin_wall != 0) n = mul3(n, -1);
        vel = sub3(vel, mul3(n, dot3(n, vel)));
    }
    t->vels[k] = vel;
    (void)img;
}

int orc_sph_update_tangle(ov_sph_tangle_state *t, const ov_sph_params *p, double time, int threads, int tangents)
{
    (void)time;
    if (!t || !p || p->outer_surface) return -1;
    const int N = t->N;
    if (tangents)
        for (int k = 0; k < N; ++k) s_tangent_normal(t, k);
    sph_ctx sc = {p, 0.0};
    int err = 0;
    if (p->use_temperature) {
        double Tb = p->temp_bath;
        double vn = p->q_dot / (Tb * he_entropy(Tb, &err) * he_total(Tb, &err) * 4 * M_PI);
        double g = (155.8 * Tb - 75) * 10000;
        sc.T_A = he_alpha(Tb, &err) * (p->kappa * 0.0001) * pow(g, 2) *
                 pow(he_total(Tb, &err) * vn / he_super(Tb, &err), 3) / he_entropy(Tb, &err);
    }
    /* the inner image: the tangle inverted through the inner surface */
    ov_sph_tangle_state img = *t;
    img.vnodes = (V3 *)malloc(sizeof(V3) * (N > 0 ? N : 1));
    for (int k = 0; k < N; ++k)
        if (t->status[k].status != OV_EMPTY) img.vnodes[k] = s_invert(t->vnodes[k], t->domain_section.inner_radius);
    double ri = t->domain_section.inner_radius, ro = t->domain_section.outer_radius;
    img.domain_section.outer_radius = ri;
    img.domain_section.inner_radius = ri * ri / ro;
    scell *tree = sc_build(t, p->dl_max), *itree = sc_build(&img, p->dl_max);
    int k;
#pragma omp parallel for num_threads(threads > 0 ? threads : 1) reduction(| : err) schedule(dynamic, 64)
    for (k = 0; k < N; ++k) {
        int e = 0;
        s_velocity(t, &img, k, tree, itree, &sc, &e);
        err |= e;
    }
    sc_free(tree);
    sc_free(itree);
    free(img.vnodes);
    return err ? -2 : 0;
}

int orc_sph_helium(double T, double out[6])
{
    int err = 0;
    out[0] = he_super(T, &err);
    out[1] = he_total(T, &err);
    out[2] = he_normal(T, &err);
    out[3] = he_entropy(T, &err);
    out[4] = he_alpha(T, &err);
    out[5] = he_alpha_p(T, &err);
    return err ? -1 : 0;
}
