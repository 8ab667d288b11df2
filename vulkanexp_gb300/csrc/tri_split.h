// tri_split.h — conservative bounds of the part of a triangle between two
// planes perpendicular to one axis: the reference split of the spatial-split
// tree builders, the host one (sbvh.cu) and the device one (gbuild.cu), which
// evaluate exactly these float operations and so produce the same trees.
//
// The part of a triangle T with slo <= x_k <= shi is the convex hull of T's
// vertices inside the slab and the crossings of T's edges with the two
// planes (Stich, Friedrich & Dietrich 2009, "Spatial splits in bounding
// volume hierarchies"; the reference split of Embree's SBVH builder works
// the same way).  A crossing p + t (q - p), t = (pl - p_k) / (q_k - p_k), is
// evaluated from the triangle's own float vertices with interval
// arithmetic: every operation rounded to nearest and then widened by one
// ulp on each side (nextafterf), which contains the exact result; t is
// clamped to [0, 1].  The box is therefore a superset of the exact part,
// wider by a few ulps of the coordinates only, and the crossing's own axis
// is the plane exactly.  Callers intersect it with the reference's box (the
// triangle's part inside earlier split planes), which keeps it conservative:
// box(T within the slab) contains T within the slab and the earlier planes.
#pragma once

#include <math.h>

#include "../../include/ddgi_exact.h"

namespace ddgi {

DDGI_HD static inline float ts_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
DDGI_HD static inline float ts_sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
DDGI_HD static inline float ts_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
DDGI_HD static inline float ts_div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
DDGI_HD static inline float ts_down(float x) { return nextafterf(x, -INFINITY); }
DDGI_HD static inline float ts_up(float x) { return nextafterf(x, INFINITY); }
DDGI_HD static inline float ts_min4(float a, float b, float c, float d) { return fminf(fminf(a, b), fminf(c, d)); }
DDGI_HD static inline float ts_max4(float a, float b, float c, float d) { return fmaxf(fmaxf(a, b), fmaxf(c, d)); }

// Bounds of the part of triangle `tri` (9 floats: v0, v1, v2) with
// slo <= x_k <= shi; lo[k] > hi[k] when the triangle misses the slab.
DDGI_HD static inline void tri_slab_bounds(const float* tri, int k, float slo, float shi, float lo[3], float hi[3]) {
    for (int a = 0; a < 3; ++a) {
        lo[a] = INFINITY;
        hi[a] = -INFINITY;
    }
    for (int v = 0; v < 3; ++v) {
        const float* p = tri + 3 * v;
        if (p[k] >= slo && p[k] <= shi)
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], p[a]);
                hi[a] = fmaxf(hi[a], p[a]);
            }
    }
    for (int e = 0; e < 3; ++e) {
        const float* p = tri + 3 * e;
        const float* q = tri + 3 * (e == 2 ? 0 : e + 1);
        for (int s = 0; s < 2; ++s) {
            const float pl = s ? shi : slo;
            if (!((p[k] < pl && q[k] > pl) || (p[k] > pl && q[k] < pl))) continue;
            // t = (pl - p_k) / (q_k - p_k), in (0, 1) exactly
            const float n = ts_sub(pl, p[k]), d = ts_sub(q[k], p[k]);
            const float nlo = ts_down(n), nhi = ts_up(n), dlo = ts_down(d), dhi = ts_up(d);
            float t0 = 0.0f, t1 = 1.0f;
            if (dlo > 0.0f || dhi < 0.0f) {
                const float c0 = ts_div(nlo, dlo), c1 = ts_div(nlo, dhi), c2 = ts_div(nhi, dlo), c3 = ts_div(nhi, dhi);
                t0 = fmaxf(0.0f, ts_down(ts_min4(c0, c1, c2, c3)));
                t1 = fminf(1.0f, ts_up(ts_max4(c0, c1, c2, c3)));
            }
            for (int a = 0; a < 3; ++a) {
                if (a == k) {
                    lo[a] = fminf(lo[a], pl);
                    hi[a] = fmaxf(hi[a], pl);
                    continue;
                }
                const float dd = ts_sub(q[a], p[a]);
                const float ddlo = ts_down(dd), ddhi = ts_up(dd);
                const float m0 = ts_mul(ddlo, t0), m1 = ts_mul(ddlo, t1), m2 = ts_mul(ddhi, t0), m3 = ts_mul(ddhi, t1);
                const float mlo = ts_down(ts_min4(m0, m1, m2, m3)), mhi = ts_up(ts_max4(m0, m1, m2, m3));
                lo[a] = fminf(lo[a], ts_down(ts_add(p[a], mlo)));
                hi[a] = fmaxf(hi[a], ts_up(ts_add(p[a], mhi)));
            }
        }
    }
}

// The spatial-split builders' reference split: the box of the part of the
// triangle inside `slab` along axis k (tri_slab_bounds), intersected with
// the slab in every axis (the reference's box with axis k narrowed).
DDGI_HD static inline void tri_split_box(const float* tri, int k, const float slab_lo[3], const float slab_hi[3],
                                         float out_lo[3], float out_hi[3]) {
    tri_slab_bounds(tri, k, slab_lo[k], slab_hi[k], out_lo, out_hi);
    for (int a = 0; a < 3; ++a) {
        out_lo[a] = fmaxf(out_lo[a], slab_lo[a]);
        out_hi[a] = fminf(out_hi[a], slab_hi[a]);
    }
}

}  // namespace ddgi
