// adjoint.cu — reverse-mode gradients of a colour-atlas loss through K
// recurrent probe updates, with the hit set held fixed.
//
// Forward of one update k (FP32 form, all probes), for a probe ray:
//   miss:      x = sky
//   backface:  x = 0
//   front hit: base = emissive + spec(albedo) * sampleProbes_k-1(reflect)
//                              + diffuse(albedo) * sampleProbes_k-1(normal)
//              x = shadowed ? base : (base + pbr(albedo) * sun) * fade
// and the colour blend of every interior texel t of the probe:
//   atlas_k[t] = (1 - h) * sum_r w[t][r] x_r / W_t + h * atlas_k-1[t]
// followed by the border copy.  The depth atlas does not depend on albedo,
// sun or sky once the hits are fixed, so only the colour chain is reversed.
//
// Reverse step k, given G_k = dL/d atlas_k:
//   k_border_fold     border gradients go to their source interior texels;
//   k_blend_adjoint   G_k-1 (interior) = h G_k, g_x[r] = (1-h) sum_t w W^-1 G;
//   k_ray_adjoint     g_x -> albedo, sun and sky gradients, and the two
//                     sampleProbes lookups scatter into G_k-1 (atomics).
// atlas_k-1 itself is restored from a checkpoint and replayed (k_replay_shade
// + the FP32 blend), so no hit is traced again.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "kernels.h"
#include "shade.cuh"

namespace ddgi {

namespace {

using AtlasF32 = AtlasView<ColorTexF32, DepthTexF32>;
constexpr uint32_t kShadowBit = 1u << 30;
constexpr uint32_t kBackBit = 1u << 31;
constexpr uint32_t kPrimMask = (1u << 28) - 1u;

__device__ __forceinline__ float night_fade(const DeviceLight& L) {
    return L.dir[1] < 0.0f ? 1.0f - clampf(-L.dir[1], 0.0f, 0.1f) / 0.1f : 1.0f;
}

// One ray record from a recorded hit (the forward's shading, no traversal).
__global__ void __launch_bounds__(128) k_replay_shade(DeviceScene sc, DeviceGrid g, DeviceLight L,
                                                      const float4* __restrict__ dirs,
                                                      const uint32_t* __restrict__ states, AtlasF32 at,
                                                      const float4* __restrict__ thit,
                                                      const uint32_t* __restrict__ prim, float4* rays, uint32_t total,
                                                      uint32_t* err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const uint32_t R = g.rays, slot = i / R, ray = i - slot * R;
    float4 th = thit[i];
    uint32_t pb = prim[i], inst = __float_as_uint(th.w);
    float4 rec;
    if (inst == 0xFFFFFFFFu) {
        rec = make_float4(L.sky[0], L.sky[1], L.sky[2], -1.0f);
    } else if (pb & kBackBit) {
        rec = make_float4(0.0f, 0.0f, 0.0f, th.x * 0.80f);
    } else {
        float4 d4 = dirs[ray];
        SurfaceShade s;
        shade_surface(sc, g, L, states, at, probe_origin_exact(g, slot), f3(d4.x, d4.y, d4.z), th.x, th.y, th.z, inst,
                      pb & kPrimMask, &s, err);
        float3 c = (pb & kShadowBit) ? s.base : lit_color(s);
        rec = make_float4(c.x, c.y, c.z, th.x);
    }
    rays[i] = rec;
}

// Adjoint of the border copy: a border texel's gradient belongs to the
// interior texel it was copied from.
__global__ void k_border_fold(DeviceGrid g, float4* gatlas) {
    const uint32_t probe = blockIdx.x;
    const uint32_t rx = (uint32_t)g.res[0], rxy = (uint32_t)(g.res[0] * g.res[1]);
    const int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
    const int n = (int)g.color_res, tile = iy * g.res[0] + ix;
    const int nb = 4 + 4 * (n - 2);
    const size_t ox = (size_t)n * tile, oy = (size_t)n * iz;
    for (int e = threadIdx.x; e < nb; e += blockDim.x) {
        int4 b = border_entry(e, n);
        float4* dst = gatlas + (oy + b.y) * g.color_w + ox + b.x;
        float4* src = gatlas + (oy + b.w) * g.color_w + ox + b.z;
        float4 v = *dst;
        *dst = make_float4(0, 0, 0, 0);
        atomicAdd(&src->x, v.x);
        atomicAdd(&src->y, v.y);
        atomicAdd(&src->z, v.z);
    }
}

// Adjoint of the colour blend + hysteresis of one probe (block = probe).
__global__ void __launch_bounds__(256) k_blend_adjoint(DeviceGrid g, const float4* __restrict__ dirs,
                                                       const float4* __restrict__ gk, float4* gprev, float4* gx) {
    extern __shared__ float smem[];
    const uint32_t R = g.rays;
    const int n = (int)g.color_res - 2, nt = n * n;
    float* s_td = smem;            // nt x 3
    float* s_g = s_td + 3 * nt;    // nt x 3, already divided by W_t
    const uint32_t probe = blockIdx.x;
    const uint32_t rx = (uint32_t)g.res[0], rxy = (uint32_t)(g.res[0] * g.res[1]);
    const int ix = (int)(probe % rx), iy = (int)((probe % rxy) / rx), iz = (int)(probe / rxy);
    const int cres = (int)g.color_res, tile = iy * g.res[0] + ix;
    const size_t ox = (size_t)cres * tile, oy = (size_t)cres * iz;
    const float hy = g.hyst;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        int tx = t % n, ty = t / n;
        float sc = texel_scale((uint32_t)n), ce = 0.5f * (float)(n - 1);
        float3 td = oct_decode(sc * ((float)tx - ce), sc * ((float)ty - ce));
        float W = 0.0f;
        for (uint32_t r = 0; r < R; ++r) {  // ray order, as the forward sums it
            float4 d = dirs[r];
            W += fmaxf(0.0f, td.x * d.x + td.y * d.y + td.z * d.z);
        }
        float inv = W > 1e-3f ? 1.0f / W : 1.0f;
        size_t ti = (oy + 1 + ty) * g.color_w + ox + 1 + tx;
        float4 gv = gk[ti];
        gprev[ti] = make_float4(hy * gv.x, hy * gv.y, hy * gv.z, 0.0f);
        s_td[3 * t] = td.x;
        s_td[3 * t + 1] = td.y;
        s_td[3 * t + 2] = td.z;
        s_g[3 * t] = (1.0f - hy) * gv.x * inv;
        s_g[3 * t + 1] = (1.0f - hy) * gv.y * inv;
        s_g[3 * t + 2] = (1.0f - hy) * gv.z * inv;
    }
    const int nb = 4 + 4 * (cres - 2);
    for (int e = threadIdx.x; e < nb; e += blockDim.x) {
        int4 b = border_entry(e, cres);
        gprev[(oy + b.y) * g.color_w + ox + b.x] = make_float4(0, 0, 0, 0);
    }
    __syncthreads();
    for (uint32_t r = threadIdx.x; r < R; r += blockDim.x) {
        float4 d = dirs[r];
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
        for (int t = 0; t < nt; ++t) {
            float w = fmaxf(0.0f, s_td[3 * t] * d.x + s_td[3 * t + 1] * d.y + s_td[3 * t + 2] * d.z);
            a0 += w * s_g[3 * t];
            a1 += w * s_g[3 * t + 1];
            a2 += w * s_g[3 * t + 2];
        }
        gx[(size_t)probe * R + r] = make_float4(a0, a1, a2, 0.0f);
    }
}

// sampleProbes (irradiance.glsl:145-237) evaluated and differentiated with
// respect to the colour atlas: returns the value, and adds
// d(value)/d(texel) . gout into gatlas.  The weights depend only on geometry
// and the depth atlas (constants here); d sqrt(c)/dc at c = 0 is taken as 0
// (such texels receive only zero radiance whatever the parameters).
__device__ float3 sample_probes_vjp(float3 position, float3 normal, float3 toCamera, const DeviceGrid& g,
                                    const uint32_t* states, const AtlasF32& at, float3 gout, float4* gatlas) {
    float3 cs = abs3(f3(g.cell[0], g.cell[1], g.cell[2]));
    float3 gridCoords = (position - f3(g.mn[0], g.mn[1], g.mn[2])) / cs;
    if (!(gridCoords.x >= 0.0f && gridCoords.y >= 0.0f && gridCoords.z >= 0.0f)) return f3(0, 0, 0);
    float3 biasedPosition = position + (normal + toCamera) * g.bias;
    int fx = (int)fminf(gridCoords.x, 16777216.0f), fy = (int)fminf(gridCoords.y, 16777216.0f),
        fz = (int)fminf(gridCoords.z, 16777216.0f);
    float3 alpha = (position - grid_probe_pos(g, fx, fy, fz)) / cs;
    alpha = f3(clampf(alpha.x, 0.0f, 1.0f), clampf(alpha.y, 0.0f, 1.0f), clampf(alpha.z, 0.0f, 1.0f));
    const float uvsx = (float)(g.res[0] * g.res[1]), uvsy = (float)g.res[2];
    const float cr = (float)g.color_res, dr = (float)g.depth_res;
    const float cscale = (float)(g.color_res - 2) / cr;
    const float dscale = (float)(g.depth_res - 2) / dr;
    const float2 nuv = sphere_to_oct_uv(normal);
    float3 S = f3(0, 0, 0), Sf = f3(0, 0, 0);
    float W = 0.0f, Wf = 0.0f;
    // pass 0: sums; pass 1: scatter
    for (int pass = 0; pass < 2; ++pass) {
        float3 coef_f = f3(0, 0, 0), coef = f3(0, 0, 0);
        if (pass == 1) {
            float n = W > 1e-3f ? 1.0f / W : 1.0f, nf = Wf > 1e-3f ? 1.0f / Wf : 1.0f;
            float a = 8.0f * clampf(W, 0.0f, 1.0f / 8.0f);
            // d out / d s_i = (1-a) 2 Sf nf^2 wf_i + a 2 S n^2 w_i, per channel
            coef_f = Sf * (2.0f * (1.0f - a) * nf * nf) * gout;
            coef = S * (2.0f * a * n * n) * gout;
        }
#pragma unroll 1
        for (int i = 0; i < 8; ++i) {
            int ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;
            int px = fx + ox, py = fy + oy, pz = fz + oz;
            if (px > g.res[0] - 1 || py > g.res[1] - 1 || pz > g.res[2] - 1) continue;
            uint32_t lin = (uint32_t)(px + g.res[0] * py + g.res[0] * g.res[1] * pz);
            if (__ldg(states + lin) == 0) continue;
            float3 probePosition = grid_probe_pos(g, px, py, pz);
            float3 directionToProbe = norm3(probePosition - position);
            float3 biasedDirectionToProbe = probePosition - biasedPosition;
            float2 duv = sphere_to_oct_uv(-norm3(biasedDirectionToProbe));
            int tile = py * g.res[0] + px;
            float cu = ((float)((int)g.color_res * tile + 1) / cr + cscale * nuv.x) / uvsx;
            float cv = ((float)((int)g.color_res * pz + 1) / cr + cscale * nuv.y) / uvsy;
            float du = ((float)((int)g.depth_res * tile + 1) / dr + dscale * duv.x) / uvsx;
            float dv = ((float)((int)g.depth_res * pz + 1) / dr + dscale * duv.y) / uvsy;
            float3 tri = f3(ox ? alpha.x : 1.0f - alpha.x, oy ? alpha.y : 1.0f - alpha.y, oz ? alpha.z : 1.0f - alpha.z);
            float weight = 1.0f;
            float bfw = fmaxf(0.0001f, (dot3(directionToProbe, normal) + 1.0f) * 0.5f);
            weight *= bfw * bfw + 0.2f;
            float fallbackWeight = weight;
            float depth[2];
            bilinear<2>(at.depth, g.depth_w, g.depth_h, du, dv, depth);
            float mean = depth[0];
            float variance = fabsf(depth[0] * depth[0] - depth[1]);
            float dist = len3(probePosition - biasedPosition);
            float dm = fmaxf(dist - mean, 0.0001f);
            float cheb = variance / (variance + dm * dm);
            cheb = fmaxf(cheb * cheb * cheb, 0.0f);
            weight *= (dist <= mean) ? 1.0f : cheb;
            weight = fmaxf(0.000001f, weight);
            const float crush = 0.2f;
            if (weight < crush) weight *= weight * weight * (1.0f / (crush * crush));
            float triw = tri.x * tri.y * tri.z + 0.001f;
            weight *= triw;
            fallbackWeight *= triw;
            // bilinear colour fetch (REPEAT) with its texel weights
            float x = cu * (float)g.color_w - 0.5f, y = cv * (float)g.color_h - 0.5f;
            float fx0 = floorf(x), fy0 = floorf(y);
            float ax = x - fx0, ay = y - fy0;
            int iw = (int)g.color_w, ih = (int)g.color_h;
            int i0 = wrap_repeat((int)fx0, iw), i1 = wrap_repeat((int)fx0 + 1, iw);
            int j0 = wrap_repeat((int)fy0, ih), j1 = wrap_repeat((int)fy0 + 1, ih);
            size_t t00 = (size_t)j0 * g.color_w + i0, t10 = (size_t)j0 * g.color_w + i1;
            size_t t01 = (size_t)j1 * g.color_w + i0, t11 = (size_t)j1 * g.color_w + i1;
            float b00 = (1.0f - ax) * (1.0f - ay), b10 = ax * (1.0f - ay), b01 = (1.0f - ax) * ay, b11 = ax * ay;
            float col[3];
            bilinear<3>(at.color, g.color_w, g.color_h, cu, cv, col);
            float3 s = f3(sqrtf(col[0]), sqrtf(col[1]), sqrtf(col[2]));
            if (pass == 0) {
                S = S + s * weight;
                W += weight;
                Sf = Sf + s * fallbackWeight;
                Wf += fallbackWeight;
            } else {
                float3 ds = coef_f * fallbackWeight + coef * weight;  // dL/ds_i
                float3 dc = f3(s.x > 0.0f ? ds.x / (2.0f * s.x) : 0.0f, s.y > 0.0f ? ds.y / (2.0f * s.y) : 0.0f,
                               s.z > 0.0f ? ds.z / (2.0f * s.z) : 0.0f);
                const size_t tt[4] = {t00, t10, t01, t11};
                const float bw[4] = {b00, b10, b01, b11};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (bw[q] == 0.0f) continue;
                    atomicAdd(&gatlas[tt[q]].x, dc.x * bw[q]);
                    atomicAdd(&gatlas[tt[q]].y, dc.y * bw[q]);
                    atomicAdd(&gatlas[tt[q]].z, dc.z * bw[q]);
                }
            }
        }
    }
    float n = W > 1e-3f ? 1.0f / W : 1.0f, nf = Wf > 1e-3f ? 1.0f / Wf : 1.0f;
    float3 fin = S * n, fb = Sf * nf;
    fin = fin * fin;
    fb = fb * fb;
    return mix3(fb, fin, 8.0f * clampf(W, 0.0f, 1.0f / 8.0f));
}

// Vector-Jacobian product of pbrMetallicRoughness with respect to albedo
// (pbrMetallicRoughness.glsl:43-84), for a general metalness.
__device__ float3 pbr_albedo_vjp(float3 n, float3 v, float3 lightColor, float3 lightDir, float3 albedo, float metal,
                                 float rough, float3 gout) {
    const float pi = DDGI_PI;
    float3 spec = mix3(f3(0.04f, 0.04f, 0.04f), albedo, metal);
    int jmax = spec.x >= spec.y ? 0 : 1;
    float smax = fmaxf(spec.x, spec.y);
    if (!(smax >= spec.z)) jmax = 2;
    smax = fmaxf(smax, spec.z);
    float r90raw = smax * 25.0f;
    float dr90 = (r90raw > 0.0f && r90raw < 1.0f) ? 25.0f * metal : 0.0f;
    float r90 = clampf(r90raw, 0.0f, 1.0f);
    float alphaRoughness = rough * rough;
    float3 l = norm3(lightDir);
    float3 h = norm3(l + v);
    float NdotL = clampf(dot3(n, l), 0.001f, 1.0f);
    float NdotV = clampf(fabsf(dot3(n, v)), 0.001f, 1.0f);
    float NdotH = clampf(dot3(n, h), 0.0f, 1.0f);
    float VdotH = clampf(dot3(v, h), 0.0f, 1.0f);
    float x = clampf(1.0f - VdotH, 0.0f, 1.0f);
    float x2 = x * x;
    float p5 = x2 * x2 * x;
    float3 F = spec + (f3(r90, r90, r90) - spec) * p5;
    float a2 = alphaRoughness * alphaRoughness;
    float attL = 2.0f * NdotL / (NdotL + sqrtf(a2 + (1.0f - a2) * (NdotL * NdotL)));
    float attV = 2.0f * NdotV / (NdotV + sqrtf(a2 + (1.0f - a2) * (NdotV * NdotV)));
    float a = NdotH * alphaRoughness;
    float k = alphaRoughness / ((1.0f - NdotH * NdotH) + a * a);
    float D = clampf(k * k * (1.0f / pi), 0.0f, 4.0f);
    float GD4 = attL * attV * D / (4.0f * NdotL * NdotV);
    float3 dcol = albedo * (1.0f - 0.04f) * (1.0f - metal);
    float3 e = gout * lightColor * NdotL;
    float3 q = f3(GD4 - dcol.x / pi, GD4 - dcol.y / pi, GD4 - dcol.z / pi);
    float3 ga = f3(e.x * (1.0f - F.x), e.y * (1.0f - F.y), e.z * (1.0f - F.z)) * ((1.0f - 0.04f) * (1.0f - metal) / pi);
    ga = ga + e * q * (metal * (1.0f - p5));
    float sumq = e.x * q.x + e.y * q.y + e.z * q.z;
    float extra = p5 * dr90 * sumq;
    if (jmax == 0) ga.x += extra;
    else if (jmax == 1) ga.y += extra;
    else ga.z += extra;
    return ga;
}

// Parameter gradients and the bounce scatter of every ray of one update.
// grad layout (doubles): albedo [material_count][3], sun [3], sky [3].
__global__ void __launch_bounds__(128) k_ray_adjoint(DeviceScene sc, DeviceGrid g, DeviceLight L,
                                                     const float4* __restrict__ dirs,
                                                     const uint32_t* __restrict__ states, AtlasF32 at,
                                                     const float4* __restrict__ thit, const uint32_t* __restrict__ prim,
                                                     const float4* __restrict__ gx, float4* gatlas, double* grad,
                                                     uint32_t total, bool smem_albedo, uint32_t* err) {
    extern __shared__ double s_grad[];  // [M*3 if smem_albedo] + sun[3] + sky[3]
    const uint32_t M3 = smem_albedo ? sc.material_count * 3 : 0;
    for (uint32_t k = threadIdx.x; k < M3 + 6; k += blockDim.x) s_grad[k] = 0.0;
    __syncthreads();
    double* s_sun = s_grad + M3;
    double* s_sky = s_sun + 3;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < total) {
        const uint32_t R = g.rays, slot = i / R, ray = i - slot * R;
        float4 th = thit[i];
        uint32_t pb = prim[i], inst = __float_as_uint(th.w);
        float4 gv = gx[i];
        float3 gxi = f3(gv.x, gv.y, gv.z);
        if (inst == 0xFFFFFFFFu) {
            atomicAdd(&s_sky[0], (double)gxi.x);
            atomicAdd(&s_sky[1], (double)gxi.y);
            atomicAdd(&s_sky[2], (double)gxi.z);
        } else if (!(pb & kBackBit) && (gxi.x != 0.0f || gxi.y != 0.0f || gxi.z != 0.0f)) {
            float4 d4 = dirs[ray];
            float3 dir = f3(d4.x, d4.y, d4.z);
            Surface s;
            if (surface_at(sc, probe_origin_exact(g, slot), dir, th.x, th.y, th.z, inst, pb & kPrimMask, &s, err)) {
                const bool shadowed = (pb & kShadowBit) != 0;
                const float fade = night_fade(L);
                const float3 sun = f3(L.color[0], L.color[1], L.color[2]);
                const float3 ldir = f3(L.dir[0], L.dir[1], L.dir[2]);
                float3 spec = mix3(f3(0.04f, 0.04f, 0.04f), s.albedo, s.metal);
                float3 diffuse = s.albedo * (1.0f - 0.04f) * (1.0f - s.metal);
                float3 g_base = shadowed ? gxi : gxi * fade;
                float3 g_pbr = shadowed ? f3(0, 0, 0) : gxi * fade;
                float3 reflectDir = dir - s.normal * (2.0f * dot3(s.normal, dir));
                float3 refl = sample_probes_vjp(s.position, reflectDir, -dir, g, states, at, g_base * spec, gatlas);
                float3 ind = sample_probes_vjp(s.position, s.normal, -dir, g, states, at, g_base * diffuse, gatlas);
                float3 ga = g_base * (refl * s.metal + ind * ((1.0f - 0.04f) * (1.0f - s.metal)));
                if (!shadowed) {
                    float3 v = norm3(-dir);
                    ga = ga + pbr_albedo_vjp(s.normal, v, sun, ldir, s.albedo, s.metal, s.rough, g_pbr);
                    float3 factor = pbr_metallic_roughness(s.normal, v, f3(1, 1, 1), ldir, s.albedo, s.metal, s.rough);
                    atomicAdd(&s_sun[0], (double)(g_pbr.x * factor.x));
                    atomicAdd(&s_sun[1], (double)(g_pbr.y * factor.y));
                    atomicAdd(&s_sun[2], (double)(g_pbr.z * factor.z));
                }
                double* ag = smem_albedo ? s_grad + 3 * s.material : grad + 3 * (size_t)s.material;
                atomicAdd(ag + 0, (double)ga.x);
                atomicAdd(ag + 1, (double)ga.y);
                atomicAdd(ag + 2, (double)ga.z);
            }
        }
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < M3 + 6; k += blockDim.x) {
        double v = s_grad[k];
        if (v != 0.0) atomicAdd(grad + (k < M3 ? k : sc.material_count * 3 + (k - M3)), v);
    }
}

}  // namespace

cudaError_t launch_replay_update(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L, const float4* dirs,
                                 uint32_t* states, float4* color, float2* depth, const float4* thit,
                                 const uint32_t* prim, float4* rays, uint32_t* err, cudaStream_t st) {
    const uint32_t P = (uint32_t)(g.res[0] * g.res[1] * g.res[2]);
    const uint32_t total = P * g.rays;
    AtlasF32 at{{color}, {depth}};
    k_replay_shade<<<(total + 127) / 128, 128, 0, st>>>(sc, g, L, dirs, states, at, thit, prim, rays, total, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_blend_fp32(g, nullptr, P, rays, dirs, states, color, depth, st);
}

cudaError_t launch_adjoint_step(const DeviceScene& sc, const DeviceGrid& g, const DeviceLight& L, const float4* dirs,
                                const uint32_t* states, const float4* color_prev, const float2* depth_prev,
                                const float4* thit, const uint32_t* prim, float4* gk, float4* gprev, float4* gx,
                                double* grad, uint32_t* err, cudaStream_t st) {
    const uint32_t P = (uint32_t)(g.res[0] * g.res[1] * g.res[2]);
    const uint32_t total = P * g.rays;
    k_border_fold<<<P, 64, 0, st>>>(g, gk);
    const uint32_t nt = (g.color_res - 2) * (g.color_res - 2);
    k_blend_adjoint<<<P, 256, sizeof(float) * 6 * nt, st>>>(g, dirs, gk, gprev, gx);
    AtlasF32 at{{color_prev}, {depth_prev}};
    const bool smem_albedo = sc.material_count <= 1024;
    size_t smem = sizeof(double) * ((smem_albedo ? sc.material_count * 3 : 0) + 6);
    k_ray_adjoint<<<(total + 127) / 128, 128, smem, st>>>(sc, g, L, dirs, states, at, thit, prim, gx, gprev, grad,
                                                          total, smem_albedo, err);
    return cudaGetLastError();
}

}  // namespace ddgi
