/*
 * A reference-side program that keeps OpenVort's own main-loop calls
 * (main.c:125-141) and is linked with -Wl,--wrap=... so those calls run on
 * libovgpu.  Built and run by tests/test_dropin_link.py.
 */
#include <stdio.h>

#include "initial_conditions.h"
#include "tangle.h"
#include "vortex_constants.h"
#include "vortex_dynamics.h"
#include "vortex_injection.h"
#include "vortex_smooth.h"

int main(void)
{
    struct tangle_state t;
    create_tangle(&t, 512);
    for (int w = 0; w < 6; ++w) t.box.wall[w] = WALL_PERIODIC;
    t.box.bottom_left_back = vec3(0, 0, 0);
    t.box.top_right_front = vec3(0.1, 0.1, 0.1);
    t.bimg = periodic_26;
    struct vec3 c = vec3(0.05, 0.05, 0.05), d = vec3(1, 0, 0);
    add_loop(&t, &c, &d, 0.02);
    double time = 0, dt = 5e-5;
    for (int s = 0; s < 3; ++s) {
        eliminate_small_loops(&t);
        reconnect(&t, 0.0);
        eliminate_small_loops(&t);
        smooth(&t);
        enforce_periodic_boundaries(&t);
        remesh(&t, global_dl_min, global_dl_max, 0.0);
        eliminate_small_loops(&t);
        update_tangle(&t, time);
        rk4_step(&t, time, dt);
        enforce_periodic_boundaries(&t);
        time += dt;
    }
    printf("nodes %d  x0 %.17g\n", number_of_used_nodes(&t), t.vnodes[0].p[0]);
    free_tangle(&t);
    return 0;
}
