// ov_helium.cuh - the spherical fork's temperature model of He II
// (src_spherical/temperature_functions.c of OpenVort), for host and device.
//
// Densities, entropy and the mutual-friction coefficients are cubic
// B-splines (de Boor's recursion over the knots Q and coefficients A) or
// the fork's closed forms; the numbers in the tables are the fork's, the
// model the velocities depend on.  The temperature of a node follows the
// heat-flux profile T(r) = T_bath + A / 5 (r / 1 m)^-5, with A fixed by the
// bath temperature (computed once on the host).  Out-of-range temperatures,
// on which the fork exits the process, set *err.
//
// Arithmetic goes through hd_* so that device code is not contracted into
// FMAs (host code is compiled with -ffp-contract=off).
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define OV_HD __host__ __device__
#else
#define OV_HD
#endif

namespace helium {

#ifdef __CUDA_ARCH__
OV_HD inline double hd_add(double a, double b) { return __dadd_rn(a, b); }
OV_HD inline double hd_sub(double a, double b) { return __dsub_rn(a, b); }
OV_HD inline double hd_mul(double a, double b) { return __dmul_rn(a, b); }
OV_HD inline double hd_div(double a, double b) { return __ddiv_rn(a, b); }
#else
OV_HD inline double hd_add(double a, double b) { return a + b; }
OV_HD inline double hd_sub(double a, double b) { return a - b; }
OV_HD inline double hd_mul(double a, double b) { return a * b; }
OV_HD inline double hd_div(double a, double b) { return a / b; }
#endif

constexpr double kLambda = 2.1768;   // temp_la, the lambda point [K]
constexpr double kPi = 3.14159265358979323846;

// Spline (temperature_functions.c:11-47): de Boor's recursion on the knot
// interval holding x; `len` entries in A and Q (A zero-padded).
OV_HD inline double spline(int len, const double *A, const double *Q, double x, int *err)
{
    const int N = len - 5 - 1;
    if (x < Q[4] || x > Q[N + 5]) {
        *err = 1;
        return 0.0;
    }
    int I = 0, J = N + 1;
    while (J - I > 1) {
        const int K = (I + J) / 2;
        if (x >= Q[K + 4]) I = K;
        else J = K;
    }
    const int JP3 = J + 3;
    double D[32];
    for (int i = J; i <= JP3; ++i) D[i] = A[i];
    for (int K = 1; K <= 3; ++K) {
        const int JPL = JP3 - K;
        for (int i = J; i <= JPL; ++i)
            D[i] = hd_div(hd_add(hd_mul(hd_sub(x, Q[i + K]), D[i + 1]), hd_mul(hd_sub(Q[i + 4], x), D[i])),
                          hd_sub(Q[i + 4], Q[i + K]));
    }
    return D[J];
}

// superfluid_density (temperature_functions.c:49-65) [kg m^-3]
OV_HD inline double superfluid_density(double T, int *err)
{
    if (!(T >= 0.0 && T <= kLambda)) { *err = 1; return 0.0; }
    const double Q[26] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.443, 0.9012, 1.5419, 1.7540, 1.918, 2.111, 2.156991, 2.173218,
                          2.175647, 2.176358, 2.176568, 2.176692, 2.176766, 2.176791, 2.176798, 2.176799, 2.17679999,
                          2.1768, 2.1768, 2.1768, 2.1768};
    const double A[26] = {0.0, 1.451275432822459e-1, 1.451334563362309e-1, 1.449759191497576e-1,
                          1.455008000684433e-1, 1.4075e-1, 1.095e-1, 8.15e-2, 5.30e-2, 2.1e-2, 8.904576e-3,
                          3.053214e-3, 1.494043e-3, 8.342826e-4, 5.10686e-4, 2.8379e-4, 1.287426e-4, 5.202569e-5,
                          2.153580e-5, 8.564206e-6, 3.567958e-6, 0.0, 0.0, 0.0, 0.0, 0.0};
    return hd_mul(spline(26, A, Q, T, err), 1000.0);
}

// total_density (temperature_functions.c:67-121) [kg m^-3]
OV_HD inline double total_density(double T, int *err)
{
    if (!(T >= 0 && T <= 4.9)) { *err = 1; return 0.0; }
    const double ro_0 = 0.1451397, ro_la = 0.1461087;
    const double a1[3] = {0.0, -7.57537e-3, 6.87483e-3};
    const double a2[3] = {0.0, -7.94605e-3, 5.07051e-3};
    const double b1[8] = {0.0, 3.79937e-3, 1.86557e-3, 4.88345e-3, 0.0, 0.0, 0.0, 0.0};
    const double b2[8] = {0.0, -30.3511e-3, -10.2326e-3, -3.00636e-3, 0.240720e-3, -2.45749e-3, 1.53454e-3,
                          -0.308182e-3};
    const double m[5] = {0.0, -1.26935e-5, 7.12413e-5, -16.7461e-5, 8.75342e-5};
    const double t = hd_sub(T, kLambda);
    double ro = 0.0;
    if (T < 1.344) {
        for (int i = 1; i <= 4; ++i) ro = hd_add(ro, hd_mul(m[i], pow(T, (double)(i + 1))));
        ro = hd_add(ro, ro_0);
    } else {
        const double *a = T <= kLambda ? a1 : a2;
        const double *b = T <= kLambda ? b1 : b2;
        double dro = 0;
        for (int i = 1; i <= 2; ++i)
            if (t != 0) dro = hd_add(dro, hd_mul(hd_mul(a[i], pow(t, (double)i)), log(fabs(t))));
        for (int i = 1; i <= 7; ++i) dro = hd_add(dro, hd_mul(b[i], pow(t, (double)i)));
        ro = hd_mul(ro_la, hd_add(dro, 1.0));
    }
    return hd_mul(ro, 1000.0);
}

// normal_density (temperature_functions.c:123-137)
OV_HD inline double normal_density(double T, int *err)
{
    if (!(T >= 1.1 && T <= kLambda)) { *err = 1; return 0.0; }
    return hd_sub(total_density(T, err), superfluid_density(T, err));
}

// entropy (temperature_functions.c:139-152)
OV_HD inline double entropy(double T, int *err)
{
    if (!(T >= 0.1 && T <= 5.0)) { *err = 1; return 0.0; }
    const double Q[30] = {0.0, 0.10000, 0.10000, 0.10000, 0.10000, 0.11123, 0.21625, 0.27672, 0.44817, 0.56369,
                          0.71969, 0.85360, 1.00186, 1.40184, 1.72912, 1.99887, 2.07775, 2.15384, 2.17680, 2.17680,
                          2.17680, 2.21160, 2.34820, 2.69075, 4.38277, 4.76361, 5.00000, 5.0, 5.0, 5.0};
    const double A[30] = {0.0, 6.60e-6, 7.60e-6, 1.60e-5, 4.61413e-5, 1.8400e-4, 4.68675e-4, 0.00121, 0.00236,
                          0.00561, 0.01978, 0.08337, 0.35824, 0.76882, 1.17803, 1.38629, 1.53613, 1.58271, 1.62419,
                          1.72261, 1.91862, 2.53529, 3.16601, 4.10379, 4.44077, 4.61570, 0.0, 0.0, 0.0, 0.0};
    return hd_mul(spline(30, A, Q, T, err), 1000.0);
}

// mutual_firction_alpha (temperature_functions.c:154-180)
OV_HD inline double friction_alpha(double T, int *err)
{
    if (!(T >= 1.3 && T < kLambda)) { *err = 1; return 0.0; }
    double b;
    if (T <= 2.167) {
        const double ep = log10(hd_sub(1.0, hd_div(T, kLambda)));
        const double Q[12] = {0.0, -5.0, -5.0, -5.0, -5.0, -2.5, -2.0, -0.8, -0.387958059947, -0.387958059947,
                              -0.387958059947, -0.387958059947};
        const double A[12] = {0.0, 1.31928144433, 1.12452707801, 0.639314792565, 0.313383532495, -0.162687403543,
                              0.092047691284, 0.188452616588, 0.0, 0.0, 0.0, 0.0};
        b = pow(10.0, spline(12, A, Q, ep, err));
    } else {
        b = hd_mul(0.47, pow(hd_sub(1.0, hd_div(T, kLambda)), -0.33));
    }
    return hd_mul(hd_div(b, 2.0), hd_sub(1.0, hd_div(superfluid_density(T, err), total_density(T, err))));
}

// mutual_firction_alpha_p (temperature_functions.c:182-209)
OV_HD inline double friction_alpha_p(double T, int *err)
{
    if (!(T >= 1.3 && T < kLambda)) { *err = 1; return 0.0; }
    double b;
    if (T <= 2.134) {
        const double ep = log10(hd_sub(1.0, hd_div(T, kLambda)));
        const double Q[13] = {0.0, -5.0, -5.0, -5.0, -5.0, -3.55, -3.2, -2.5, -1.0, -0.384067377871,
                              -0.384067377871, -0.384067377871, -0.384067377871};
        const double A[13] = {0.0, -8.47218032526e-2, 0.931621715174, 0.973263359433, 1.10543591819,
                              1.15904485127, 1.18311634566, 1.17480594214, 1.19458392766, 0.0, 0.0, 0.0, 0.0};
        b = hd_sub(pow(10.0, spline(13, A, Q, ep, err)), 15.0);
    } else {
        b = hd_add(hd_mul(-0.34, pow(hd_sub(1.0, hd_div(T, kLambda)), -0.33)), 1.01);
    }
    return hd_mul(hd_div(b, 2.0), hd_sub(1.0, hd_div(superfluid_density(T, err), total_density(T, err))));
}

// gamma (temperature_functions.c:254-258) [m^-2]
OV_HD inline double gamma_coef(double T) { return hd_mul(hd_sub(hd_mul(155.8, T), 75.0), 10000.0); }

// A of get_temperature (temperature_functions.c:260-270): the bath terms
OV_HD inline double profile_A(double q_dot, double T_bath, double kappa, int *err)
{
    const double e = entropy(T_bath, err), rho = total_density(T_bath, err);
    const double vn = hd_div(q_dot, hd_mul(hd_mul(hd_mul(hd_mul(T_bath, e), rho), 4.0), kPi));
    const double g = gamma_coef(T_bath);
    double A = hd_mul(friction_alpha(T_bath, err), hd_mul(kappa, 0.0001));
    A = hd_mul(A, pow(g, 2.0));
    A = hd_mul(A, pow(hd_div(hd_mul(total_density(T_bath, err), vn), superfluid_density(T_bath, err)), 3.0));
    return hd_div(A, entropy(T_bath, err));
}

// get_temperature at radius r [cm]
OV_HD inline double temperature(double r_cm, double T_bath, double A)
{
    const double x = hd_mul(r_cm, 0.01);
    return hd_add(T_bath, hd_mul(hd_div(A, 5.0), pow(x, -5.0)));
}

// |v_n| and |v_s| [cm/s] along the radial unit vector at radius r [cm]
// (get_vn, get_vs: temperature_functions.c:216-252)
OV_HD inline double vn_radial(double r_cm, double T, double q_dot, int *err)
{
    const double r = hd_mul(r_cm, 0.01);
    const double den = hd_mul(hd_mul(hd_mul(hd_mul(hd_mul(T, entropy(T, err)), total_density(T, err)), 4.0), kPi),
                              pow(r, 2.0));
    return hd_mul(hd_div(q_dot, den), 100.0);
}
OV_HD inline double vs_radial(double r_cm, double T, double q_dot, int *err)
{
    const double r = hd_mul(r_cm, 0.01);
    const double den = hd_mul(
        hd_mul(hd_mul(hd_mul(hd_mul(hd_mul(T, entropy(T, err)), superfluid_density(T, err)), total_density(T, err)),
                      4.0),
               kPi),
        pow(r, 2.0));
    return hd_mul(hd_div(hd_mul(-q_dot, normal_density(T, err)), den), 100.0);
}

}  // namespace helium
