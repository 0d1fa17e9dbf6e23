/*
 * ov_oracle.h - TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of OpenVort's vortex-filament velocity and time-step path,
 * used as the checker for the GPU library (tests, the smoke check and the
 * CPU-baseline leg of the benchmark).  Nothing in the shipped library links
 * or calls this code.
 *
 * Each function follows the reference function named in its comment (paths
 * within the OpenVort project) with the same floating-point operation order,
 * so that, built with the same compiler flags, its results are bit-identical
 * to the reference's.  That is checked against the reference compiled from
 * its own sources (oracle/Makefile -> oracle/_ref/libovref.so) by
 * tests/test_oracle_pin.py.
 *
 * Parameters are passed explicitly (ov_params) instead of through process
 * globals, so several tangles with different parameters can be run from one
 * process.
 */
#ifndef OV_ORACLE_H
#define OV_ORACLE_H

#include "../include/ov_tangle.h"
#include "../include/openvort_gpu.h"
#include "../include/ov_spherical.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_cell orc_cell;

/* Tree statistics accumulated by orc_count_interactions. */
typedef struct orc_counts {
    long long visits;   /* calls of the traversal on non-empty cells */
    long long accepts;  /* monopole / leaf evaluations */
    int max_depth;
    long long cells;
} orc_counts;

/* tangle pool: create_tangle / expand_tangle / free_tangle (tangle.c:27-117) */
void orc_tangle_create(ov_tangle_state *t, int n);
void orc_tangle_expand(ov_tangle_state *t, int n);
void orc_tangle_free(ov_tangle_state *t);
int orc_get_next_empty_node(ov_tangle_state *t);

/* geometry */
ov_vec3 orc_step_node(const ov_tangle_state *t, int i, int where);

/* octree (octree.c) */
orc_cell *orc_octree_build(const ov_tangle_state *t);
void orc_octree_destroy(orc_cell *tree);
void orc_octree_get_vs(const ov_tangle_state *t, const orc_cell *tree, const ov_vec3 *r,
                       double resolution, const ov_params *p, ov_vec3 *res);
void orc_count_interactions(const ov_tangle_state *t, double resolution, orc_counts *out);
/* the same counts per target node (visits[N], accepts[N]) */
void orc_node_interactions(const ov_tangle_state *t, double resolution, int threads, long long *visits,
                           long long *accepts);

/* velocity path (tangle.c) */
void orc_update_tangent_normal(ov_tangle_state *t, int k);
void orc_update_tangents_normals(ov_tangle_state *t);
void orc_update_velocity(ov_tangle_state *t, int k, double time, const orc_cell *tree,
                         const ov_params *p);
void orc_update_velocities(ov_tangle_state *t, double time, const ov_params *p);
/* update_velocity(..., tree=NULL) for the listed nodes only (direct sum). */
void orc_direct_velocities(ov_tangle_state *t, const int *nodes, int n, double time,
                           const ov_params *p);

/* time stepping and topology (vortex_dynamics.c, tangle.c) */
void orc_rk4_step(ov_tangle_state *t, double time, double dt, const ov_params *p);
int orc_reconnect(ov_tangle_state *t, double time, const ov_params *p,
                  int *log_k, int *log_l, int log_cap);
void orc_remesh(ov_tangle_state *t, double min_dist, double max_dist, double time,
                const ov_params *p, int *n_added, int *n_removed);
int orc_eliminate_small_loops(ov_tangle_state *t, const ov_params *p);
void orc_enforce_periodic_boundaries(ov_tangle_state *t);
void orc_smooth(ov_tangle_state *t, const ov_params *p);
void orc_low_pass_filter(double *in, int n, double freq_to_cutoff);
void orc_step(ov_tangle_state *t, double time, double dt, const ov_params *p,
              int *n_recs);

/* add_loop (vortex_injection.c:49): ring geometry used by the small config. */
/* The spherical fork's update_tangents_normals (tangents != 0) and
   update_velocities with the outer surface open (ov_oracle_sph.c). */
int orc_sph_update_tangle(ov_sph_tangle_state *t, const ov_sph_params *p, double time, int threads, int tangents);
/* Its He II model at T: superfluid, total, normal density, entropy, alpha, alpha'. */
int orc_sph_helium(double T, double out[6]);

void orc_add_loop(ov_tangle_state *t, const ov_vec3 *center, const ov_vec3 *dir, double r,
                  const ov_params *p);

#ifdef __cplusplus
}
#endif
#endif
