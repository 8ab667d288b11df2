/*
 * ddgi_exact.h — host-side definitions whose exact floating-point result is
 * part of the contract of ddgi_update.
 *
 * Closest-hit instance and triangle IDs are required to be bit-identical
 * between the CUDA path and any CPU implementation of the same update.  That
 * only holds if both trace bit-identical rays, so the inputs of the ray
 * generation are fixed here, computed once on the host in double precision
 * and rounded to float:
 *
 *  - the per-update ray-direction table: the rotated spherical Fibonacci set
 *    of src/shaders/irradiance.glsl:52-64 and src/shaders/traceProbes.rgen:36
 *    (the reference stores the same table in its `rayDirection` image,
 *    src/shaders/traceProbes.rgen:46-47);
 *  - the world-to-object transform of an instance (the reference gets it from
 *    the ray-tracing driver as gl_WorldToObjectEXT).
 *
 * Compile users of this header with -ffp-contract=off: the functions below
 * assume every operation is rounded separately.
 */
#ifndef DDGI_EXACT_H
#define DDGI_EXACT_H

#include <math.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Golden-ratio constant of sphericalFibonacci (irradiance.glsl:53). */
#define DDGI_PHI_MINUS_ONE 0.61803398874989484820

/* Ray direction `i` of `n`: M * sphericalFibonacci(i, n), M row-major 3x3.
 * Written as (x, y, z, 1) into out[0..3]. */
static inline void ddgi_ray_direction(const float m[9], uint32_t i, uint32_t n, float out[4]) {
    const double two_pi = 6.283185307179586476925;
    double a = (double)i * DDGI_PHI_MINUS_ONE;
    double frac = a - floor(a);
    double phi = two_pi * frac;
    double cos_theta = 1.0 - (2.0 * (double)i + 1.0) / (double)n;
    double s2 = 1.0 - cos_theta * cos_theta;
    if (s2 < 0.0) s2 = 0.0;
    if (s2 > 1.0) s2 = 1.0;
    double sin_theta = sqrt(s2);
    double v[3] = {cos(phi) * sin_theta, sin(phi) * sin_theta, cos_theta};
    for (int r = 0; r < 3; ++r) {
        double acc = (double)m[3 * r + 0] * v[0];
        acc = acc + (double)m[3 * r + 1] * v[1];
        acc = acc + (double)m[3 * r + 2] * v[2];
        out[r] = (float)acc;
    }
    out[3] = 1.0f;
}

static inline void ddgi_ray_direction_table(const float m[9], uint32_t n, float* out4) {
    for (uint32_t i = 0; i < n; ++i) ddgi_ray_direction(m, i, n, out4 + 4 * i);
}

/* Inverse of a row-major 3x4 affine transform [A | t] -> [A^-1 | -A^-1 t].
 * Returns 0 when A is singular (|det| below 1e-30), 1 otherwise. */
static inline int ddgi_affine_inverse(const float o2w[12], float w2o[12]) {
    double a[3][3], t[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) a[r][c] = (double)o2w[4 * r + c];
        t[r] = (double)o2w[4 * r + 3];
    }
    double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    double det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
    if (!(fabs(det) > 1e-30)) return 0;
    double inv[3][3];
    inv[0][0] = c00 / det;
    inv[1][0] = c01 / det;
    inv[2][0] = c02 / det;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
    for (int r = 0; r < 3; ++r) {
        double tr = -(inv[r][0] * t[0] + inv[r][1] * t[1] + inv[r][2] * t[2]);
        for (int c = 0; c < 3; ++c) w2o[4 * r + c] = (float)inv[r][c];
        w2o[4 * r + 3] = (float)tr;
    }
    return 1;
}

#ifdef __cplusplus
}
#endif

#endif /* DDGI_EXACT_H */
