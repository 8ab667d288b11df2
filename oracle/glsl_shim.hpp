// glsl_shim.hpp — GLSL vector types and built-in functions in C++, enough to
// compile the reference's own shader helper files (src/shaders/common.glsl,
// ProbeGrid.glsl, irradiance.glsl, pbrMetallicRoughness.glsl, sky.glsl)
// unchanged on the host, so that the oracle's restatements of them can be
// checked against the reference's code; glsl_compute.hpp and glsl_rt.hpp
// build the compute, fragment and ray-tracing stages on it.  Test
// infrastructure: built by oracle/build_ref_glsl.py into oracle/_ref/,
// loaded only by tests and the fixture generator.
//
// The shader files are included inside namespace glsl, so unqualified calls
// (cos, sqrt, max, ...) find the overloads below and never the C library's.
// GLSL semantics kept: float literals are float (the build passes
// -fsingle-precision-constant), int and uint operands convert to float in
// mixed arithmetic, swizzles read and assign (v.xy = ...), and textureLod
// filters bilinearly with REPEAT addressing, as the reference's atlas
// sampler is set up (src/RaytracingDescriptors.hpp:63, 70), with exact
// weights (the checker's convention; hardware uses 8-bit fractions).
#pragma once

#include <math.h>
#include <stdint.h>

namespace glsl {

typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;

// Swizzle proxies: storage aliasing the vector's components.
template <int N, int A, int B>
struct swz2 {
    float e[N];
    operator vec2() const;
    swz2& operator=(const vec2& v);
};
template <int N, int A, int B, int C>
struct swz3 {
    float e[N];
    operator vec3() const;
    swz3& operator=(const vec3& v);
};

struct vec2 {
    union {
        struct {
            float x, y;
        };
        struct {
            float r, g;
        };
        swz2<2, 0, 1> xy;
        swz2<2, 1, 0> yx;
    };
    vec2() { x = y = 0.0f; }
    vec2(float s) { x = y = s; }
    vec2(float a, float b) {
        x = a;
        y = b;
    }
    vec2(const vec2& o) {
        x = o.x;
        y = o.y;
    }
    vec2& operator=(const vec2& o) {
        x = o.x;
        y = o.y;
        return *this;
    }
    explicit vec2(const struct ivec2& v);
    float& operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
};

struct vec3 {
    union {
        struct {
            float x, y, z;
        };
        struct {
            float r, g, b;
        };
        swz2<3, 0, 1> xy;
        swz2<3, 1, 0> yx;
        swz3<3, 0, 1, 2> xyz;
        swz3<3, 0, 1, 2> rgb;
    };
    vec3() { x = y = z = 0.0f; }
    vec3(float a, const vec2& v) {
        x = a;
        y = v.x;
        z = v.y;
    }
    explicit vec3(const struct vec4& v);
    float& operator[](unsigned i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](unsigned i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3(float s) { x = y = z = s; }
    vec3(float a, float b, float c) {
        x = a;
        y = b;
        z = c;
    }
    vec3(const vec2& v, float c) {
        x = v.x;
        y = v.y;
        z = c;
    }
    vec3(const vec3& o) {
        x = o.x;
        y = o.y;
        z = o.z;
    }
    vec3& operator=(const vec3& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        return *this;
    }
    explicit vec3(const struct ivec3& v);
    vec3& operator+=(const vec3& o) {
        x += o.x, y += o.y, z += o.z;
        return *this;
    }
    vec3& operator-=(const vec3& o) {
        x -= o.x, y -= o.y, z -= o.z;
        return *this;
    }
    vec3& operator*=(const vec3& o) {
        x *= o.x, y *= o.y, z *= o.z;
        return *this;
    }
    vec3& operator*=(float s) {
        x *= s, y *= s, z *= s;
        return *this;
    }
};

struct vec4 {
    union {
        struct {
            float x, y, z, w;
        };
        struct {
            float r, g, b, a;
        };
        swz2<4, 0, 1> xy;
        swz2<4, 0, 1> rg;
        swz2<4, 1, 2> yz;
        swz2<4, 2, 3> zw;
        swz3<4, 0, 1, 2> xyz;
        swz3<4, 0, 1, 2> rgb;
        swz3<4, 1, 2, 3> yzw;
    };
    vec4() { x = y = z = w = 0.0f; }
    vec4(float s) { x = y = z = w = s; }
    vec4(float a_, float b_, float c_, float d_) {
        x = a_;
        y = b_;
        z = c_;
        w = d_;
    }
    vec4(const vec2& v, float c_, float d_) {
        x = v.x;
        y = v.y;
        z = c_;
        w = d_;
    }
    vec4(const vec3& v, float d_) {
        x = v.x;
        y = v.y;
        z = v.z;
        w = d_;
    }
    vec4(const vec4& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        w = o.w;
    }
    vec4& operator=(const vec4& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        w = o.w;
        return *this;
    }
    vec4& operator*=(const vec4& o) {
        x *= o.x, y *= o.y, z *= o.z, w *= o.w;
        return *this;
    }
};
inline vec3::vec3(const vec4& v) {
    x = v.x;
    y = v.y;
    z = v.z;
}

template <int N, int A, int B>
swz2<N, A, B>::operator vec2() const {
    return vec2(e[A], e[B]);
}
template <int N, int A, int B>
swz2<N, A, B>& swz2<N, A, B>::operator=(const vec2& v) {
    const float a = v.x, b = v.y;  // v may alias this storage
    e[A] = a;
    e[B] = b;
    return *this;
}
template <int N, int A, int B, int C>
swz3<N, A, B, C>::operator vec3() const {
    return vec3(e[A], e[B], e[C]);
}
template <int N, int A, int B, int C>
swz3<N, A, B, C>& swz3<N, A, B, C>::operator=(const vec3& v) {
    const float a = v.x, b = v.y, c = v.z;
    e[A] = a;
    e[B] = b;
    e[C] = c;
    return *this;
}
template <int N, int A, int B, int C>
swz3<N, A, B, C>& operator+=(swz3<N, A, B, C>& s, const vec3& v) {
    const float a = v.x, b = v.y, c = v.z;
    s.e[A] += a;
    s.e[B] += b;
    s.e[C] += c;
    return s;
}

struct uvec2 {
    uint x, y;
};
struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int s) : x(s), y(s) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const uvec2& v) : x((int)v.x), y((int)v.y) {}
};
struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int s) : x(s), y(s), z(s) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
    explicit ivec3(const struct uvec3& v);
};
struct bvec3 {
    bool x, y, z;
};

inline vec2::vec2(const ivec2& v) {
    x = (float)v.x;
    y = (float)v.y;
}
inline vec3::vec3(const ivec3& v) {
    x = (float)v.x;
    y = (float)v.y;
    z = (float)v.z;
}

// ---- arithmetic ----
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(const vec2& a, const vec2& b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator+(const vec2& a, float s) { return vec2(a.x + s, a.y + s); }
inline vec2 operator-(const vec2& a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator/(const vec2& a, float s) { return vec2(a.x / s, a.y / s); }
inline vec2 operator+(float s, const vec2& a) { return vec2(s + a.x, s + a.y); }
inline vec2 operator-(float s, const vec2& a) { return vec2(s - a.x, s - a.y); }
inline vec2 operator*(float s, const vec2& a) { return vec2(s * a.x, s * a.y); }

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator+(float s, const vec3& a) { return vec3(s + a.x, s + a.y, s + a.z); }
inline vec3 operator-(float s, const vec3& a) { return vec3(s - a.x, s - a.y, s - a.z); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
// int vectors promote to float in mixed arithmetic
inline vec3 operator*(const ivec3& a, const vec3& b) { return vec3(a) * b; }
inline vec3 operator/(const vec3& a, const ivec3& b) { return a / vec3(b); }

inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator-(const vec4& a, const vec4& b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(const vec4& a, const vec4& b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator*(float s, const vec4& a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }

inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator*(int s, const ivec2& a) { return ivec2(s * a.x, s * a.y); }
inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator-(const ivec3& a, int s) { return ivec3(a.x - s, a.y - s, a.z - s); }
inline ivec3 operator&(const ivec3& a, const ivec3& b) { return ivec3(a.x & b.x, a.y & b.y, a.z & b.z); }

// ---- built-ins ----
inline float abs(float v) { return fabsf(v); }
inline vec2 abs(const vec2& v) { return vec2(fabsf(v.x), fabsf(v.y)); }
inline vec3 abs(const vec3& v) { return vec3(fabsf(v.x), fabsf(v.y), fabsf(v.z)); }
inline float sign(float v) { return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f); }
inline vec3 sign(const vec3& v) { return vec3(sign(v.x), sign(v.y), sign(v.z)); }
inline float floor(float v) { return floorf(v); }
inline float sqrt(float v) { return sqrtf(v); }
inline vec3 sqrt(const vec3& v) { return vec3(sqrtf(v.x), sqrtf(v.y), sqrtf(v.z)); }
inline float cos(float v) { return cosf(v); }
inline float sin(float v) { return sinf(v); }
inline float acos(float v) { return acosf(v); }
inline float atan(float v) { return atanf(v); }
inline float exp(float v) { return expf(v); }
inline vec3 exp(const vec3& v) { return vec3(expf(v.x), expf(v.y), expf(v.z)); }
inline float pow(float a, float b) { return powf(a, b); }
inline float min(float a, float b) { return a < b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }
inline float clamp(float v, float lo, float hi) { return min(max(v, lo), hi); }
inline vec3 clamp(const vec3& v, const vec3& lo, const vec3& hi) {
    return vec3(clamp(v.x, lo.x, hi.x), clamp(v.y, lo.y, hi.y), clamp(v.z, lo.z, hi.z));
}
inline float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline vec3 mix(const vec3& a, const vec3& b, float t) { return a * (1.0f - t) + b * t; }
inline vec3 mix(const vec3& a, const vec3& b, const vec3& t) { return a * (1.0f - t) + b * t; }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const vec3& v) { return sqrtf(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v * (1.0f / length(v)); }
inline vec3 reflect(const vec3& i, const vec3& n) { return i - 2.0f * dot(n, i) * n; }
inline bool isinf(float v) { return __builtin_isinf(v) != 0; }
inline bool isnan(float v) { return __builtin_isnan(v) != 0; }
inline bvec3 isinf(const vec3& v) { return bvec3{isinf(v.x), isinf(v.y), isinf(v.z)}; }
inline bvec3 isnan(const vec3& v) { return bvec3{isnan(v.x), isnan(v.y), isnan(v.z)}; }
inline bvec3 lessThan(const vec3& a, const vec3& b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec3 greaterThan(const ivec3& a, const ivec3& b) { return bvec3{a.x > b.x, a.y > b.y, a.z > b.z}; }
inline bool any(const bvec3& v) { return v.x || v.y || v.z; }

// ---- sampling ----
struct sampler2D {
    const float* texels;  // row-major, `channels` floats per texel
    int width, height, channels;
};
inline vec4 textureLod(const sampler2D& s, const vec2& uv, float) {
    const float x = uv.x * (float)s.width - 0.5f, y = uv.y * (float)s.height - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    auto wrap = [](long i, long n) {
        const long r = i % n;
        return r < 0 ? r + n : r;
    };
    const long i0 = wrap((long)fx, s.width), i1 = wrap((long)fx + 1, s.width);
    const long j0 = wrap((long)fy, s.height), j1 = wrap((long)fy + 1, s.height);
    float out[4] = {0.0f, 0.0f, 0.0f, 1.0f};
    for (int c = 0; c < s.channels && c < 4; ++c) {
        const float t00 = s.texels[((size_t)j0 * s.width + i0) * s.channels + c];
        const float t10 = s.texels[((size_t)j0 * s.width + i1) * s.channels + c];
        const float t01 = s.texels[((size_t)j1 * s.width + i0) * s.channels + c];
        const float t11 = s.texels[((size_t)j1 * s.width + i1) * s.channels + c];
        const float top = t00 * (1.0f - ax) + t10 * ax, bot = t01 * (1.0f - ax) + t11 * ax;
        out[c] = top * (1.0f - ay) + bot * ay;
    }
    return vec4(out[0], out[1], out[2], out[3]);
}

}  // namespace glsl
