/*
 * ov_spherical.h - the velocity path of OpenVort's spherical fork on the GPU.
 *
 * The fork (src_spherical/, include_spherical/ of OpenVort) simulates a
 * section of a spherical shell: inner radius ri, outer radius ro, azimuth
 * (elevation from the x-y plane) in [-A, A] and polar angle (in the x-y
 * plane) in [-P, P].  The section repeats under rotations by 2A and 2P, and
 * the inner surface is a wall represented by the spherical inversion of the
 * tangle through ri.  Its tangle_state holds the section instead of the
 * box and its image tables; node_status.pin_wall holds the fork's
 * pin_surface (-1 none, 0 INNER, 1 OUTER).
 *
 * Reference layout this mirrors:
 *   struct node_status     include_spherical/boundaries.h:34-37
 *   struct domain          include_spherical/boundaries.h:42-47
 *   struct tangle_state    include_spherical/tangle.h:30-43
 *
 * Each call uploads the caller's tangle, computes on the GPU and writes the
 * fields the reference function writes back into the caller's arrays.
 */
#ifndef OV_SPHERICAL_H
#define OV_SPHERICAL_H

#include "openvort_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { OV_NOT_A_SURFACE = -1, OV_INNER = 0, OV_OUTER = 1 };

typedef struct ov_sph_domain {
    double inner_radius;
    double outer_radius;
    double azimut_angle;   /* half width A of the azimuth range [rad] */
    double polar_angle;    /* half width P of the polar range [rad] */
} ov_sph_domain;

typedef struct ov_sph_tangle_state {
    ov_vec3 *vnodes;
    ov_vec3 *vels;
    ov_vec3 *vs;
    ov_vec3 *tangents;
    ov_vec3 *normals;
    int *recalculate;
    ov_neighbour *connections;
    ov_node_status *status;
    ov_sph_domain domain_section;
    int N;
    int next_empty;
    int total_empty;
} ov_sph_tangle_state;

/* The fork's globals on this path (src_spherical/initial_conditions.c:11-71). */
typedef struct ov_sph_params {
    double kappa;              /* KAPPA [cm^2/s] */
    double vortex_width;       /* VORTEX_WIDTH [cm] */
    double alpha, alpha_p;     /* mutual friction without the temperature model */
    int use_mutual_friction;
    double bh_resolution;      /* BH_resolution (theta) */
    double dl_min, dl_max;     /* global_dl_min / global_dl_max */
    double q_dot;              /* heat source power [W] */
    double temp_bath;          /* bath temperature [K] */
    int use_temperature;       /* temperature model: v_s, v_n, alpha(T), alpha'(T) */
    int outer_surface;         /* must be 0: the outer surface open */
} ov_sph_params;

/* The fork's defaults (initial_conditions.c:11-71). */
void ov_sph_params_default(ov_sph_params *p);

/* update_tangents_normals   src_spherical/tangle.c:563-572 (update_tangent_normal 483-556) */
int ov_sph_update_tangents_normals(ov_ctx *ctx, ov_sph_tangle_state *tangle, const ov_sph_params *p);
/* update_velocities         src_spherical/tangle.c:950-1042 (update_velocity
   638-865; tangents and normals as stored in `tangle`) */
int ov_sph_update_velocities(ov_ctx *ctx, ov_sph_tangle_state *tangle, const ov_sph_params *p, double t);
/* update_tangle             include_spherical/tangle.h:99-103 */
int ov_sph_update_tangle(ov_ctx *ctx, ov_sph_tangle_state *tangle, const ov_sph_params *p, double t);
/* The temperature model at T (host): superfluid, total and normal density
   [kg m^-3], entropy, alpha(T), alpha'(T) (temperature_functions.c:49-209);
   OV_ERR_ARG outside its range. */
int ov_sph_helium(double T, double out[6]);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
#define OV_SPH_ASSERT(c, m) static_assert(c, m)
#else
#define OV_SPH_ASSERT(c, m) _Static_assert(c, m)
#endif
OV_SPH_ASSERT(sizeof(ov_sph_domain) == 32, "struct domain");
OV_SPH_ASSERT(offsetof(ov_sph_tangle_state, domain_section) == 64, "tangle_state.domain_section");
OV_SPH_ASSERT(offsetof(ov_sph_tangle_state, N) == 96, "tangle_state.N");
OV_SPH_ASSERT(sizeof(ov_sph_tangle_state) == 112, "struct tangle_state");
#undef OV_SPH_ASSERT

#endif
