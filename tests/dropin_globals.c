/*
 * Stand-in for the reference's global parameter definitions
 * (src/initial_conditions.c:12-91 of OpenVort) so the drop-in layer can be
 * exercised without the reference program: same names, types and defaults.
 * Tests set them through ctypes before each call, as a reference program
 * would through its configuration.
 */
#include "../include/ov_tangle.h"

double VORTEX_WIDTH = 1e-8;
double KAPPA = 9.97e-4;
int global_num_threads = 32;
int use_mutual_friction = 1;
double alpha = 0.034;
double alpha_p = 1.383e-2;
double global_dl_min = 0.5e-3;
double global_dl_max = 1.5e-3;
double reconnection_angle_cutoff = 5.0 * 3.14159265358979323846 / 180.0;
double rec_dist = 4e-4;
int small_loop_cutoff = 5;
int pin_mode = OV_PINNED;
int use_freq_filter = 1;
double freq_to_cutoff = 4.0 / 5;
int use_BH = 1;
double BH_resolution = 0.4;
ov_ext_vel vn_conf = {OV_SIMPLE, 10.493799, 0, 0, {{1.0, 0, 0}}};
ov_ext_vel vb_conf = {OV_NO_FLOW, 0, 0, 0, {{0, 0, 0}}};
ov_ext_vel vs_conf = {OV_SIMPLE, 0.493799, 0, 0, {{-1.0, 0, 0}}};
int loop_injection = 0;
double loop_injection_frequency = 1;
int line_injection = 0;
int line_injection_n = 1;
double line_injection_frequency = 1;
int line_injection_polarized = 0;
