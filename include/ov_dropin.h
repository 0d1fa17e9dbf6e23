/*
 * ov_dropin.h - OpenVort's own entry points, backed by libovgpu.
 *
 * Each function has the signature of the reference function named beside
 * it and the same in-place effect on the caller's tangle_state; parameters
 * are read from the reference's process globals (KAPPA, alpha, BH_resolution,
 * vn_conf, ... declared in the reference's include/vortex_constants.h and
 * external_velocity.h) at every call, as the reference reads them.
 *
 * Link ov_dropin.o (openvort_gb300/lib/libovdropin.a) and libovgpu.so into
 * the reference program and redirect its calls with the linker, e.g.
 *   -Wl,--wrap=update_velocities -Wl,--wrap=rk4_step ...
 * after compiling ov_dropin.c with -DOV_DROPIN_WRAP, which adds the
 * __wrap_<name> aliases.
 *
 * Failures: the reference functions are void; these print one line to
 * stderr and leave the status in ovd_last_status() (0 = OV_OK).
 * One hidden context per process on device $OV_DEVICE (default 0).
 */
#ifndef OV_DROPIN_H
#define OV_DROPIN_H

#include "ov_tangle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* update_tangents_normals   include/tangle.h:104, src/tangle.c:509 */
void ovd_update_tangents_normals(ov_tangle_state *tangle);
/* update_velocities         include/tangle.h:108, src/tangle.c:733 */
void ovd_update_velocities(ov_tangle_state *tangle, double t);
/* update_velocity           include/tangle.h:106, src/tangle.c:600
   (tree == NULL: direct sum; otherwise a tree from ovd_octree_build) */
void ovd_update_velocity(ov_tangle_state *tangle, int k, double t, void *tree);
/* rk4_step                  include/vortex_dynamics.h:21, src/vortex_dynamics.c:50 */
void ovd_rk4_step(ov_tangle_state *tangle, double t, double dt);
/* reconnect                 include/vortex_dynamics.h:32, src/vortex_dynamics.c:186 */
int ovd_reconnect(ov_tangle_state *tangle, double t);
/* remesh                    include/tangle.h:110, src/tangle.c:1018 (may grow the
   tangle's arrays with realloc, as expand_tangle does) */
void ovd_remesh(ov_tangle_state *tangle, double min_dist, double max_dist, double time);
/* eliminate_small_loops     include/tangle.h:112, src/tangle.c:1063 */
void ovd_eliminate_small_loops(ov_tangle_state *tangle);
/* enforce_periodic_boundaries include/tangle.h:98, src/tangle.c:793 */
void ovd_enforce_periodic_boundaries(ov_tangle_state *tangle);
/* smooth                    include/vortex_smooth.h:11, src/vortex_smooth.c:459 */
void ovd_smooth(ov_tangle_state *tangle);
/* octree_build / octree_get_vs / octree_destroy   include/octree.h:54-66 */
void *ovd_octree_build(const ov_tangle_state *tangle);
void ovd_octree_get_vs(const ov_tangle_state *tangle, const void *tree, const ov_vec3 *r,
                       double resolution, ov_vec3 *res);
void ovd_octree_destroy(void *tree);
/* enforce_wall_boundaries   include/tangle.h:100, src/tangle.c:966 (may grow the arrays) */
void ovd_enforce_wall_boundaries(ov_tangle_state *tangle, double time);
/* save_tangle / load_tangle include/utils.h:17-18, src/utils.c:132-199 (no GPU;
   load_tangle grows the arrays with realloc as expand_tangle does) */
void ovd_save_tangle(const char *filename, ov_tangle_state *tangle);
int ovd_load_tangle(const char *filename, ov_tangle_state *tangle);
/* add_loop / add_line_in_zdir  include/vortex_injection.h:13, 23,
   src/vortex_injection.c:49, 267 (may grow the arrays) */
void ovd_add_loop(ov_tangle_state *tangle, ov_vec3 *center, ov_vec3 *dir, double r);
void ovd_add_line_in_zdir(ov_tangle_state *tangle, double x, double y, int direction);
/* inject_vortices           include/vortex_injection.h:35, src/vortex_injection.c:702
   (settings from the reference's loop_injection / line_injection globals,
   draws from the process's drand48 stream) */
void ovd_inject_vortices(ov_tangle_state *tangle, double t);
/* status of the last ovd_* call (an ov_status value) */
int ovd_last_status(void);

#ifdef __cplusplus
}
#endif
#endif
