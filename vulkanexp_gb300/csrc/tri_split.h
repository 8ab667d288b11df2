// tri_split.h — conservative bounds of the parts of a triangle on either
// side of a plane perpendicular to one axis: the reference split of the
// spatial-split tree builders, the host one (sbvh.cu) and the device one
// (gbuild.cu), which evaluate exactly these float operations and so produce
// the same trees.
//
// The part of a triangle T on one side of a plane is the convex hull of T's
// vertices on that side and the crossings of T's edges with the plane (the
// reference split of Stich, Friedrich & Dietrich 2009, "Spatial splits in
// bounding volume hierarchies", as in Embree's SBVH builder).  A crossing
// p + t (q - p), t = (pl - p_k) / (q_k - p_k), is evaluated from the
// triangle's own float vertices with interval arithmetic: every operation
// rounded to nearest and then widened by one ulp on each side (nextafterf),
// which contains the exact result; t is clamped to [0, 1], and the
// crossing's own axis is the plane exactly.  The boxes therefore contain
// the exact parts and are wider by a few ulps of the coordinates only.  A
// builder intersects them with the reference's box (which bounds the
// triangle's part inside earlier split planes), which keeps them
// conservative: the part of T inside the reference and below a plane lies
// in box(T below the plane) and in the reference's box; the part between
// two planes lies in box(T above the lower one) and box(T below the upper
// one).
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

// Bounds of the parts of triangle `tri` (9 floats: v0, v1, v2) on either
// side of the plane x_K = pl: below (x_K <= pl) into llo/lhi, above
// (x_K >= pl) into glo/ghi.  A side the triangle misses stays empty (lo
// +inf, hi -inf).  K is a template argument so that a device caller keeps
// the triangle in registers.
template <int K>
DDGI_HD static inline void tri_plane_bounds_k(const float* tri, float pl, float llo[3], float lhi[3], float glo[3],
                                              float ghi[3]) {
    for (int a = 0; a < 3; ++a) {
        llo[a] = glo[a] = INFINITY;
        lhi[a] = ghi[a] = -INFINITY;
    }
    for (int v = 0; v < 3; ++v) {
        const float* p = tri + 3 * v;
        if (p[K] <= pl)
            for (int a = 0; a < 3; ++a) {
                llo[a] = fminf(llo[a], p[a]);
                lhi[a] = fmaxf(lhi[a], p[a]);
            }
        if (p[K] >= pl)
            for (int a = 0; a < 3; ++a) {
                glo[a] = fminf(glo[a], p[a]);
                ghi[a] = fmaxf(ghi[a], p[a]);
            }
    }
    for (int e = 0; e < 3; ++e) {
        const float* p = tri + 3 * e;
        const float* q = tri + 3 * (e == 2 ? 0 : e + 1);
        if (!((p[K] < pl && q[K] > pl) || (p[K] > pl && q[K] < pl))) continue;
        // t = (pl - p_K) / (q_K - p_K), in (0, 1) exactly
        const float n = ts_sub(pl, p[K]), d = ts_sub(q[K], p[K]);
        const float nlo = ts_down(n), nhi = ts_up(n), dlo = ts_down(d), dhi = ts_up(d);
        float t0 = 0.0f, t1 = 1.0f;
        if (dlo > 0.0f || dhi < 0.0f) {
            const float c0 = ts_div(nlo, dlo), c1 = ts_div(nlo, dhi), c2 = ts_div(nhi, dlo), c3 = ts_div(nhi, dhi);
            t0 = fmaxf(0.0f, ts_down(ts_min4(c0, c1, c2, c3)));
            t1 = fminf(1.0f, ts_up(ts_max4(c0, c1, c2, c3)));
        }
        for (int a = 0; a < 3; ++a) {
            float clo = pl, chi = pl;  // the crossing's own axis is the plane exactly
            if (a != K) {
                const float dd = ts_sub(q[a], p[a]);
                const float ddlo = ts_down(dd), ddhi = ts_up(dd);
                const float m0 = ts_mul(ddlo, t0), m1 = ts_mul(ddlo, t1), m2 = ts_mul(ddhi, t0), m3 = ts_mul(ddhi, t1);
                clo = ts_down(ts_add(p[a], ts_down(ts_min4(m0, m1, m2, m3))));
                chi = ts_up(ts_add(p[a], ts_up(ts_max4(m0, m1, m2, m3))));
            }
            llo[a] = fminf(llo[a], clo);
            lhi[a] = fmaxf(lhi[a], chi);
            glo[a] = fminf(glo[a], clo);
            ghi[a] = fmaxf(ghi[a], chi);
        }
    }
}

DDGI_HD static inline void tri_plane_bounds(const float* tri, int k, float pl, float llo[3], float lhi[3], float glo[3],
                                            float ghi[3]) {
    if (k == 0) tri_plane_bounds_k<0>(tri, pl, llo, lhi, glo, ghi);
    else if (k == 1) tri_plane_bounds_k<1>(tri, pl, llo, lhi, glo, ghi);
    else tri_plane_bounds_k<2>(tri, pl, llo, lhi, glo, ghi);
}

// A reference box bounding the triangle's part inside `slab` (a reference's
// box with axis k narrowed to [slab_lo[k], slab_hi[k]]): the slab
// intersected with the triangle's bounds above slab_lo[k] and below
// slab_hi[k].  lo > hi in some axis when that leaves nothing.
DDGI_HD static inline void tri_split_box(const float* tri, int k, const float slab_lo[3], const float slab_hi[3],
                                         float out_lo[3], float out_hi[3]) {
    float llo[3], lhi[3], glo[3], ghi[3];
    for (int a = 0; a < 3; ++a) {
        out_lo[a] = slab_lo[a];
        out_hi[a] = slab_hi[a];
    }
    tri_plane_bounds(tri, k, slab_lo[k], llo, lhi, glo, ghi);
    for (int a = 0; a < 3; ++a) {
        out_lo[a] = fmaxf(out_lo[a], glo[a]);
        out_hi[a] = fminf(out_hi[a], ghi[a]);
    }
    tri_plane_bounds(tri, k, slab_hi[k], llo, lhi, glo, ghi);
    for (int a = 0; a < 3; ++a) {
        out_lo[a] = fmaxf(out_lo[a], llo[a]);
        out_hi[a] = fminf(out_hi[a], lhi[a]);
    }
}

}  // namespace ddgi
