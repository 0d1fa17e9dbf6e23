/*
 * ov_tangle.h - binary-compatible mirror of OpenVort's host tangle state.
 *
 * The GPU library is a drop-in behind OpenVort's own entry points, so it must
 * read and write the caller's `struct tangle_state` in place.  These types
 * restate that layout under `ov_` names (so both headers can coexist in one
 * translation unit); the static asserts at the bottom pin every offset that
 * the library touches.
 *
 * Reference layout this mirrors (OpenVort, paths within the project):
 *   struct vec3            include/vec3_math.h:16-18
 *   struct neighbour_t     include/tangle.h:39-42
 *   node_status_t, boundary_faces, wall_type, struct node_status,
 *   struct domain_box, struct image_tangle, struct boundary_images
 *                          include/boundaries.h:18-80
 *   struct tangle_state    include/tangle.h:47-66
 */
#ifndef OV_TANGLE_H
#define OV_TANGLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Node status values (boundaries.h:50-55). */
enum { OV_EMPTY = -1, OV_FREE = 0, OV_PINNED = 1, OV_PINNED_SLIP = 2 };

/* Box faces (boundaries.h:30-38): LEFT -x, RIGHT +x, BACK -y, FRONT +y, DOWN -z, UP +z. */
enum { OV_NOT_A_FACE = -1, OV_LEFT = 0, OV_RIGHT, OV_BACK, OV_FRONT, OV_DOWN, OV_UP };

/* Wall types (boundaries.h:21-25). */
enum { OV_WALL_OPEN = 0, OV_WALL_PERIODIC = 1, OV_WALL_MIRROR = 2 };

/* External velocity kinds (external_velocity.h:26-30). */
enum { OV_NO_FLOW = 0, OV_SIMPLE = 1, OV_DECREASING = 2 };

typedef struct ov_vec3 { double p[3]; } ov_vec3;

typedef struct ov_neighbour { int forward; int reverse; } ov_neighbour;

typedef struct ov_node_status { int status; int pin_wall; } ov_node_status;

typedef struct ov_domain_box {
    ov_vec3 bottom_left_back;
    ov_vec3 top_right_front;
    int wall[6];
} ov_domain_box;

typedef struct ov_image_tangle {
    int shift[3];
    int reflect[3];
    int number_of_reflects;
} ov_image_tangle;

typedef struct ov_boundary_images {
    const ov_image_tangle *images;
    int n;
} ov_boundary_images;

typedef struct ov_tangle_state {
    ov_vec3 *vnodes;
    ov_vec3 *vels;
    ov_vec3 *vs;
    ov_vec3 *tangents;
    ov_vec3 *normals;
    int *recalculate;
    ov_neighbour *connections;
    ov_node_status *status;
    ov_domain_box box;
    ov_boundary_images bimg;
    int N;
    int next_empty;
    int total_empty;
} ov_tangle_state;

/* Layout of OpenVort's `struct ext_vel_param` (external_velocity.h:13-19). */
typedef struct ov_ext_vel {
    int type;
    double strength;
    double time_of_linear_decrease;
    double starting_strength;
    ov_vec3 direction;
} ov_ext_vel;

#ifndef __cplusplus
#define OV_STATIC_ASSERT _Static_assert
#else
#define OV_STATIC_ASSERT static_assert
#endif
OV_STATIC_ASSERT(sizeof(ov_vec3) == 24, "vec3 layout");
OV_STATIC_ASSERT(sizeof(ov_neighbour) == 8, "neighbour_t layout");
OV_STATIC_ASSERT(sizeof(ov_node_status) == 8, "node_status layout");
OV_STATIC_ASSERT(sizeof(ov_domain_box) == 72, "domain_box layout");
OV_STATIC_ASSERT(sizeof(ov_image_tangle) == 28, "image_tangle layout");
OV_STATIC_ASSERT(offsetof(ov_tangle_state, box) == 64, "tangle_state.box offset");
OV_STATIC_ASSERT(offsetof(ov_tangle_state, bimg) == 136, "tangle_state.bimg offset");
OV_STATIC_ASSERT(offsetof(ov_tangle_state, N) == 152, "tangle_state.N offset");
OV_STATIC_ASSERT(sizeof(ov_tangle_state) == 168, "tangle_state size");
OV_STATIC_ASSERT(sizeof(ov_ext_vel) == 56, "ext_vel_param layout");

#ifdef __cplusplus
}
#endif
#endif /* OV_TANGLE_H */
