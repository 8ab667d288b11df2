/*
 * ddgi_exact.h — host-side definitions whose exact floating-point result is
 * part of the contract of ddgi_update.
 *
 * Closest-hit instance and triangle IDs are required to be bit-identical
 * between the CUDA path and any CPU implementation of the same update.  That
 * only holds if both trace bit-identical rays, so the inputs of the ray
 * generation are fixed here, computed once on the host:
 *
 *  - the per-update ray-direction table: the rotated spherical Fibonacci set
 *    of src/shaders/irradiance.glsl:52-64 and src/shaders/traceProbes.rgen:36,
 *    evaluated in float operation by operation as the shaders write it (the
 *    reference stores the same table in its `rayDirection` image,
 *    src/shaders/traceProbes.rgen:46-47);
 *  - the world-to-object transform of an instance (the reference gets it from
 *    the ray-tracing driver as gl_WorldToObjectEXT), in double, rounded.
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

/* Ray direction `i` of `n`: M * sphericalFibonacci(i, n), M row-major 3x3,
 * written as (x, y, z, 1) into out[0..3].  The float operations of
 * irradiance.glsl:52-64 (pi = 3.1415926538f, common.glsl:4) in their order,
 * each rounded separately:
 *   PHI = sqrt(5) * 0.5 + 0.5;  a = i * (PHI - 1);  phi = (2 pi) (a - floor(a))
 *   cosTheta = 1 - (2 i + 1) * (1 / n);  sinTheta = sqrt(clamp(1 - cosTheta^2, 0, 1))
 *   v = (cos(phi) sinTheta, sin(phi) sinTheta, cosTheta)
 * with cos and sin of the float phi correctly rounded (evaluated in double,
 * then rounded: the most accurate result GLSL permits, and the same on every
 * host); then the rotation as mat3 * vec3 (traceProbes.rgen:36), column 0 * x
 * + column 1 * y + column 2 * z. */
static inline void ddgi_ray_direction(const float m[9], uint32_t i, uint32_t n, float out[4]) {
    const float phi_golden = sqrtf(5.0f) * 0.5f + 0.5f;
    const float fi = (float)i;
    const float a = fi * (phi_golden - 1.0f);
    const float frac = a - floorf(a);
    const float phi = (2.0f * 3.1415926538f) * frac;
    const float cos_theta = 1.0f - (2.0f * fi + 1.0f) * (1.0f / (float)n);
    float s2 = 1.0f - cos_theta * cos_theta;
    if (s2 < 0.0f) s2 = 0.0f;
    if (s2 > 1.0f) s2 = 1.0f;
    const float sin_theta = sqrtf(s2);
    const float v[3] = {(float)cos((double)phi) * sin_theta, (float)sin((double)phi) * sin_theta, cos_theta};
    for (int r = 0; r < 3; ++r) out[r] = (m[3 * r + 0] * v[0] + m[3 * r + 1] * v[1]) + m[3 * r + 2] * v[2];
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

/*
 * Storage rounding of the reference-format atlas (ddgi_precision
 * DDGI_PRECISION_REFERENCE_FORMAT).  The reference keeps its irradiance atlas
 * in VK_FORMAT_B10G11R11_UFLOAT_PACK32 images and its depth atlas in
 * VK_FORMAT_R16G16_SFLOAT images (src/IrradianceProbes.cpp:41-63), so every
 * texel it stores is rounded to those formats and the next update's bounce
 * lookup reads the rounded values.  The functions below give the value a
 * float becomes in such a format: 5-bit exponent (bias 15, subnormals below
 * 2^-14), `mbits` stored mantissa bits (6 for the 11-bit red and green
 * channels, 5 for the 10-bit blue channel, 10 for a half), rounding to
 * nearest with ties to even, overflow (2^16 and above after rounding) to
 * infinity; the unsigned 11/10-bit formats store negative values (and -0)
 * as 0.  NaN stays NaN.  The same code runs on the host and in CUDA kernels.
 */
#if defined(__CUDACC__)
#define DDGI_HD __host__ __device__
#else
#define DDGI_HD
#endif

DDGI_HD static inline uint32_t ddgi_float_bits(float f) {
    union {
        float f;
        uint32_t u;
    } v;
    v.f = f;
    return v.u;
}

DDGI_HD static inline float ddgi_bits_float(uint32_t u) {
    union {
        float f;
        uint32_t u;
    } v;
    v.u = u;
    return v.f;
}

DDGI_HD static inline float ddgi_round_small_float(float x, int mbits, int is_unsigned) {
    const uint32_t u = ddgi_float_bits(x);
    const uint32_t sign = u & 0x80000000u;
    uint32_t a = u & 0x7fffffffu;
    if (a >= 0x7f800000u) { /* infinity or NaN */
        if (a > 0x7f800000u) return x;
        return (is_unsigned && sign) ? 0.0f : x;
    }
    if (is_unsigned && sign) return 0.0f;
    if (a < 0x38800000u) {
        /* below 2^-14: multiples of 2^-(14 + mbits); the scalings are exact */
        const float up = ddgi_bits_float((uint32_t)(127 + 14 + mbits) << 23);
        const float down = ddgi_bits_float((uint32_t)(127 - 14 - mbits) << 23);
        const float r = rintf(ddgi_bits_float(a) * up) * down;
        a = ddgi_float_bits(r);
    } else {
        const int drop = 23 - mbits;
        a += ((1u << (drop - 1)) - 1u) + ((a >> drop) & 1u);
        a &= ~((1u << drop) - 1u);
        if (a >= 0x47800000u) a = 0x7f800000u;
    }
    return ddgi_bits_float(a | sign);
}

/* One colour texel of the reference-format atlas: R and G as unsigned 11-bit
 * floats, B as an unsigned 10-bit float (the format has no alpha; reads
 * return 1). */
DDGI_HD static inline float ddgi_round_r11(float x) { return ddgi_round_small_float(x, 6, 1); }
DDGI_HD static inline float ddgi_round_b10(float x) { return ddgi_round_small_float(x, 5, 1); }
/* One depth channel of the reference-format atlas (R16G16_SFLOAT). */
DDGI_HD static inline float ddgi_round_half(float x) { return ddgi_round_small_float(x, 10, 0); }

#ifdef __cplusplus
}
#endif

#endif /* DDGI_EXACT_H */
