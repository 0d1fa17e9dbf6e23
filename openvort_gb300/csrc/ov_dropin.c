/*
 * ov_dropin.c - OpenVort's own entry points backed by libovgpu
 * (declarations and linking: include/ov_dropin.h).
 *
 * Parameters come from the reference's process globals at every call, as
 * the reference reads them; the caller's tangle_state is uploaded, the GPU
 * computes, and the fields the reference function writes are copied back.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/openvort_gpu.h"
#include "../../include/ov_dropin.h"

/* The reference's globals (include/vortex_constants.h:11-60,
   include/external_velocity.h:33-37), defined by its initial_conditions.c. */
extern double VORTEX_WIDTH, KAPPA, alpha, alpha_p, global_dl_min, global_dl_max, rec_dist;
extern double reconnection_angle_cutoff, freq_to_cutoff, BH_resolution;
extern int use_mutual_friction, use_BH, small_loop_cutoff, use_freq_filter, global_num_threads, pin_mode;
extern ov_ext_vel vn_conf, vs_conf, vb_conf;
/* injection settings (include/vortex_constants.h:48-56) */
extern int loop_injection, line_injection, line_injection_n, line_injection_polarized;
extern double loop_injection_frequency, line_injection_frequency;

static ov_ctx *g_ctx = NULL;
static int g_status = OV_OK;

int ovd_last_status(void) { return g_status; }

static int report(int rc, const char *what)
{
    g_status = rc;
    if (rc != OV_OK)
        fprintf(stderr, "libovgpu %s: error %d: %s\n", what, rc, g_ctx ? ov_last_error(g_ctx) : "no context");
    return rc;
}

static ov_ctx *context(void)
{
    if (!g_ctx) {
        const char *dev = getenv("OV_DEVICE");
        int rc = ov_ctx_create(&g_ctx, dev ? atoi(dev) : 0);
        if (rc != OV_OK) {
            g_ctx = NULL;
            report(rc, "context");
            return NULL;
        }
    }
    ov_params p;
    memset(&p, 0, sizeof p);
    p.kappa = KAPPA;
    p.vortex_width = VORTEX_WIDTH;
    p.alpha = alpha;
    p.alpha_p = alpha_p;
    p.use_mutual_friction = use_mutual_friction;
    p.use_bh = use_BH;
    p.bh_resolution = BH_resolution;
    p.vn = vn_conf;
    p.vs = vs_conf;
    p.vb = vb_conf;
    p.dl_min = global_dl_min;
    p.dl_max = global_dl_max;
    p.rec_dist = rec_dist;
    p.reconnection_angle_cutoff = reconnection_angle_cutoff;
    p.small_loop_cutoff = small_loop_cutoff;
    p.use_freq_filter = use_freq_filter;
    p.freq_to_cutoff = freq_to_cutoff;
    p.num_threads = global_num_threads;
    p.pin_mode = pin_mode;
    ov_set_params(g_ctx, &p);
    return g_ctx;
}

/* expand_tangle's effect on the arrays (tangle.c:68-98): realloc to n
   slots, new slots EMPTY; the bookkeeping comes back from the context. */
static int grow_host(ov_tangle_state *t, int n)
{
#define GROW(field, type)                                                   \
    do {                                                                    \
        void *q = realloc(t->field, sizeof(type) * (size_t)n);              \
        if (!q) return OV_ERR_ALLOC;                                        \
        t->field = (type *)q;                                               \
    } while (0)
    GROW(vnodes, ov_vec3); GROW(vels, ov_vec3); GROW(vs, ov_vec3);
    GROW(tangents, ov_vec3); GROW(normals, ov_vec3);
    GROW(recalculate, int); GROW(status, ov_node_status); GROW(connections, ov_neighbour);
#undef GROW
    for (int k = t->N; k < n; ++k) {
        t->status[k].status = OV_EMPTY;
        t->status[k].pin_wall = OV_NOT_A_FACE;
        t->connections[k].forward = -1;
        t->connections[k].reverse = -1;
        t->recalculate[k] = 0;
    }
    t->N = n;
    return OV_OK;
}

static int sync_back(ov_tangle_state *t, unsigned fields)
{
    int n = 0;
    ov_tangle_info(g_ctx, &n, NULL, NULL);
    if (n > t->N) {
        int rc = grow_host(t, n);
        if (rc) return rc;
    }
    return ov_download_tangle(g_ctx, t, fields);
}

#define TRY(call, what)                                 \
    do {                                                \
        int rc_ = (call);                               \
        if (rc_ != OV_OK) { report(rc_, what); return; } \
    } while (0)
#define TRYV(call, what, val)                           \
    do {                                                \
        int rc_ = (call);                               \
        if (rc_ != OV_OK) { report(rc_, what); return val; } \
    } while (0)

void ovd_update_tangents_normals(ov_tangle_state *t)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "update_tangents_normals");
    TRY(ov_update_tangents_normals(c), "update_tangents_normals");
    TRY(ov_download_tangle(c, t, OV_F_TANGENTS | OV_F_NORMALS), "update_tangents_normals");
    g_status = OV_OK;
}

void ovd_update_velocities(ov_tangle_state *t, double time)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY | OV_F_TANGENTS | OV_F_NORMALS), "update_velocities");
    TRY(ov_update_velocities(c, time), "update_velocities");
    TRY(ov_download_tangle(c, t, OV_F_VELS | OV_F_VS), "update_velocities");
    g_status = OV_OK;
}

void ovd_update_velocity(ov_tangle_state *t, int k, double time, void *tree)
{
    ov_ctx *c = context();
    if (!c) return;
    if (k < 0 || k >= t->N || t->status[k].status == OV_EMPTY) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY | OV_F_TANGENTS | OV_F_NORMALS), "update_velocity");
    if (!tree || !use_BH) {
        double v[3], s[3];
        TRY(ov_direct_velocities(c, &k, 1, time, v, s), "update_velocity");
        memcpy(t->vels[k].p, v, sizeof v);
        memcpy(t->vs[k].p, s, sizeof s);
    } else {
        /* the tree branch is the per-node body of update_velocities */
        ov_vec3 keep_v, keep_s;
        TRY(ov_update_velocities(c, time), "update_velocity");
        ov_vec3 *vv = (ov_vec3 *)malloc(sizeof(ov_vec3) * (size_t)t->N);
        ov_vec3 *ss = (ov_vec3 *)malloc(sizeof(ov_vec3) * (size_t)t->N);
        if (!vv || !ss) { free(vv); free(ss); report(OV_ERR_ALLOC, "update_velocity"); return; }
        ov_tangle_state tmp = *t;
        tmp.vels = vv;
        tmp.vs = ss;
        int rc = ov_download_tangle(c, &tmp, OV_F_VELS | OV_F_VS);
        keep_v = vv[k];
        keep_s = ss[k];
        free(vv);
        free(ss);
        if (rc) { report(rc, "update_velocity"); return; }
        t->vels[k] = keep_v;
        t->vs[k] = keep_s;
    }
    g_status = OV_OK;
}

void ovd_rk4_step(ov_tangle_state *t, double time, double dt)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY | OV_F_VELS), "rk4_step");
    TRY(ov_rk4_step(c, time, dt), "rk4_step");
    TRY(ov_download_tangle(c, t, OV_F_POS), "rk4_step");
    g_status = OV_OK;
}

int ovd_reconnect(ov_tangle_state *t, double time)
{
    ov_ctx *c = context();
    if (!c) return 0;
    int n = 0;
    TRYV(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "reconnect", 0);
    TRYV(ov_reconnect(c, time, &n, NULL, NULL, 0), "reconnect", 0);
    TRYV(ov_download_tangle(c, t, OV_F_TOPOLOGY), "reconnect", 0);
    for (int k = 0; k < t->N; ++k) t->recalculate[k] = 0;
    g_status = OV_OK;
    return n;
}

void ovd_remesh(ov_tangle_state *t, double min_dist, double max_dist, double time)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY | OV_F_VELS | OV_F_VS), "remesh");
    TRY(ov_remesh(c, min_dist, max_dist, time), "remesh");
    TRY(sync_back(t, OV_F_POS | OV_F_TOPOLOGY | OV_F_VELS | OV_F_VS), "remesh");
    g_status = OV_OK;
}

void ovd_eliminate_small_loops(ov_tangle_state *t)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "eliminate_small_loops");
    TRY(ov_eliminate_small_loops(c), "eliminate_small_loops");
    TRY(ov_download_tangle(c, t, OV_F_TOPOLOGY), "eliminate_small_loops");
    g_status = OV_OK;
}

void ovd_enforce_periodic_boundaries(ov_tangle_state *t)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "enforce_periodic_boundaries");
    TRY(ov_enforce_periodic_boundaries(c), "enforce_periodic_boundaries");
    TRY(ov_download_tangle(c, t, OV_F_POS), "enforce_periodic_boundaries");
    g_status = OV_OK;
}

void ovd_smooth(ov_tangle_state *t)
{
    if (!use_freq_filter) return;
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "smooth");
    TRY(ov_smooth(c), "smooth");
    TRY(ov_download_tangle(c, t, OV_F_POS), "smooth");
    g_status = OV_OK;
}

void ovd_enforce_wall_boundaries(ov_tangle_state *t, double time)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "enforce_wall_boundaries");
    TRY(ov_enforce_wall_boundaries(c, time), "enforce_wall_boundaries");
    TRY(sync_back(t, OV_F_POS | OV_F_TOPOLOGY), "enforce_wall_boundaries");
    g_status = OV_OK;
}

/* Frame files need no GPU. */
void ovd_save_tangle(const char *filename, ov_tangle_state *t)
{
    report(ov_write_frame(t, filename, 15), "save_tangle");
}

int ovd_load_tangle(const char *filename, ov_tangle_state *t)
{
    int n = 0;
    TRYV(ov_frame_slots(filename, t->N, &n, NULL, NULL), "load_tangle", -1);
    const int n0 = t->N;
    if (n > t->N) TRYV(grow_host(t, n), "load_tangle", -1);
    TRYV(ov_read_frame(filename, n0, t), "load_tangle", -1);
    g_status = OV_OK;
    return 0;
}

void ovd_add_loop(ov_tangle_state *t, ov_vec3 *center, ov_vec3 *dir, double r)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "add_loop");
    TRY(ov_add_loop(c, 0, center->p, dir->p, r), "add_loop");
    TRY(sync_back(t, OV_F_POS | OV_F_TOPOLOGY), "add_loop");
    g_status = OV_OK;
}

void ovd_add_line_in_zdir(ov_tangle_state *t, double x, double y, int direction)
{
    ov_ctx *c = context();
    if (!c) return;
    TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "add_line_in_zdir");
    TRY(ov_add_line_in_zdir(c, 0, x, y, direction), "add_line_in_zdir");
    TRY(sync_back(t, OV_F_POS | OV_F_TOPOLOGY), "add_line_in_zdir");
    g_status = OV_OK;
}

/* vec3_normalize (vec3_math.c:208) */
static void normalize3(double v[3])
{
    if (v[0] == 0 && v[1] == 0 && v[2] == 0) return;
    double d = 0;
    for (int k = 0; k < 3; ++k) d += v[k] * v[k];
    const double m = 1 / sqrt(d);
    for (int k = 0; k < 3; ++k) v[k] = v[k] * m;
}

/* inject_vortices (vortex_injection.c:702-800) drawing from the process's
   own drand48 stream, so the draws interleave with the rest of the
   program's as they do in the reference.  The direction's three draws are
   taken last component first, the order in which the reference build
   (gcc, x86-64) evaluates vec3()'s arguments. */
void ovd_inject_vortices(ov_tangle_state *t, double time)
{
    static double last_loop = 0, last_line = 0;
    ov_ctx *c = NULL;
    const double left = t->box.bottom_left_back.p[0], right = t->box.top_right_front.p[0];
    const double back = t->box.bottom_left_back.p[1], front = t->box.top_right_front.p[1];
    g_status = OV_OK;
    if (loop_injection) {
        double dir[3];
        dir[2] = -drand48();
        dir[1] = 2 * (drand48() - 0.5);
        dir[0] = 2 * (drand48() - 0.5);
        normalize3(dir);
        if (!(time - last_loop < 1 / loop_injection_frequency)) {
            last_loop = time;
            double cent[3];
            cent[2] = t->box.top_right_front.p[2];
            cent[0] = left + (right - left) * drand48();
            cent[1] = back + (front - back) * drand48();
            const double D = fabs(right - left), rmin = 0.05 * D, rmax = 0.25 * D;
            const double r = rmin + (rmax - rmin) * drand48();
            if (!(c = context())) return;
            TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "inject_vortices");
            TRY(ov_add_loop(c, 0, cent, dir, r), "inject_vortices");
        }
    }
    if (line_injection && !(time - last_line < 1 / line_injection_frequency)) {
        last_line = time;
        for (int k = 0; k < line_injection_n; ++k) {
            const double x1 = left + drand48() * (right - left);
            const double x2 = left + drand48() * (right - left);
            double y1, y2;
            if (line_injection_polarized) {
                y1 = back + (1 + drand48()) * (front - back) / 2;
                y2 = back + drand48() * (front - back) / 2;
            } else {
                y1 = back + drand48() * (front - back);
                y2 = back + drand48() * (front - back);
            }
            if (!c) {
                if (!(c = context())) return;
                TRY(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "inject_vortices");
            }
            TRY(ov_add_line_in_zdir(c, 0, x1, y1, +1), "inject_vortices");
            TRY(ov_add_line_in_zdir(c, 0, x2, y2, -1), "inject_vortices");
        }
    }
    if (c) TRY(sync_back(t, OV_F_POS | OV_F_TOPOLOGY), "inject_vortices");
}

/* The octree API: the tree lives in the context; the handle only marks
   that ovd_octree_build ran for this tangle. */
typedef struct ovd_tree { const ov_tangle_state *tangle; } ovd_tree;

void *ovd_octree_build(const ov_tangle_state *t)
{
    ov_ctx *c = context();
    if (!c) return NULL;
    TRYV(ov_upload_tangle_fields(c, t, OV_F_POS | OV_F_TOPOLOGY), "octree_build", NULL);
    TRYV(ov_tree_velocity_at(c, NULL, 0, BH_resolution, 1, NULL), "octree_build", NULL);
    ovd_tree *h = (ovd_tree *)malloc(sizeof *h);
    if (h) h->tangle = t;
    g_status = OV_OK;
    return h;
}

void ovd_octree_get_vs(const ov_tangle_state *t, const void *tree, const ov_vec3 *r, double resolution, ov_vec3 *res)
{
    (void)t;
    res->p[0] = res->p[1] = res->p[2] = 0;
    if (!tree || !g_ctx) return;
    double out[3];
    TRY(ov_tree_velocity_at(g_ctx, r->p, 1, resolution, 0, out), "octree_get_vs");
    memcpy(res->p, out, sizeof out);
    g_status = OV_OK;
}

void ovd_octree_destroy(void *tree) { free(tree); }

#ifdef OV_DROPIN_WRAP
/* Linker redirection targets: -Wl,--wrap=<name> routes the reference's
   calls of <name> here. */
void __wrap_update_tangents_normals(ov_tangle_state *t) { ovd_update_tangents_normals(t); }
void __wrap_update_velocities(ov_tangle_state *t, double time) { ovd_update_velocities(t, time); }
void __wrap_update_velocity(ov_tangle_state *t, int k, double time, void *tree) { ovd_update_velocity(t, k, time, tree); }
void __wrap_rk4_step(ov_tangle_state *t, double time, double dt) { ovd_rk4_step(t, time, dt); }
int __wrap_reconnect(ov_tangle_state *t, double time) { return ovd_reconnect(t, time); }
void __wrap_remesh(ov_tangle_state *t, double a, double b, double time) { ovd_remesh(t, a, b, time); }
void __wrap_eliminate_small_loops(ov_tangle_state *t) { ovd_eliminate_small_loops(t); }
void __wrap_enforce_periodic_boundaries(ov_tangle_state *t) { ovd_enforce_periodic_boundaries(t); }
void __wrap_smooth(ov_tangle_state *t) { ovd_smooth(t); }
void *__wrap_octree_build(const ov_tangle_state *t) { return ovd_octree_build(t); }
void __wrap_octree_get_vs(const ov_tangle_state *t, const void *tree, const ov_vec3 *r, double res_, ov_vec3 *res)
{
    ovd_octree_get_vs(t, tree, r, res_, res);
}
void __wrap_octree_destroy(void *tree) { ovd_octree_destroy(tree); }
void __wrap_enforce_wall_boundaries(ov_tangle_state *t, double time) { ovd_enforce_wall_boundaries(t, time); }
void __wrap_save_tangle(const char *f, ov_tangle_state *t) { ovd_save_tangle(f, t); }
int __wrap_load_tangle(const char *f, ov_tangle_state *t) { return ovd_load_tangle(f, t); }
void __wrap_add_loop(ov_tangle_state *t, ov_vec3 *c, ov_vec3 *d, double r) { ovd_add_loop(t, c, d, r); }
void __wrap_add_line_in_zdir(ov_tangle_state *t, double x, double y, int d) { ovd_add_line_in_zdir(t, x, y, d); }
void __wrap_inject_vortices(ov_tangle_state *t, double time) { ovd_inject_vortices(t, time); }
#endif
