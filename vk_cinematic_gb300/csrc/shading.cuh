// Per-vertex shading of the path tracer (device code), shared by the
// wavefront stages, the reference-order tile kernel and the batch kernel.
//
// ComputeRadianceForPath (src/simd_path_tracer.cpp:107-175) evaluates each
// path vertex from its own data plus the clamped radiance of the next
// vertex.  vertex_terms computes the per-vertex part - emission E, the
// response A = kD*albedo/pi + specular and the cosine - and path_radiance
// runs the reverse pass radiance = E + (A * clamp(radiance_next)) * cos, the
// reference's expression in the reference's order.
#pragma once

#include "gbsp_common.cuh"
#include "traverse.cuh"

namespace gbsp {

// ---------------------------------------------------------------------------
// Material evaluation (src/sp_material_system.cpp:59-105, image.h:3-18)
// ---------------------------------------------------------------------------
__device__ __forceinline__ V3 texel_nearest(const MaterialView &mv, int slot, float u, float v)
{
    TextureDesc t = mv.textures[slot];
    float fx = u * (float)t.width;
    float fy = v * (float)t.height;
    uint32_t x = (uint32_t)floorf(fx);
    uint32_t y = (uint32_t)floorf(fy);
    uint64_t idx = (uint64_t)y * t.width + x;
    uint64_t maxIdx = (uint64_t)t.width * t.height - 1;  // the reference may read index W*H
    if (idx > maxIdx) idx = maxIdx;
    float4 p = __ldg(mv.texels + t.offset + idx);
    return v3(p.x, p.y, p.z);
}

__device__ __forceinline__ V3 sky_radiance(const SkyParams &s, V3 dir)
{
    float t = rclamp(0.5f * (dir.y + 1.0f), 0.0f, 1.0f);
    V3 c = add(s.bottom, mul(sub(s.top, s.bottom), t));
    if (dot(dir, s.sunDir) >= s.cosSunRadius) c = add(c, s.sunRadiance);
    return c;
}

// Albedo of the material in `slot` at uv (sp_EvaluateMaterial's albedo).
__device__ __forceinline__ V3 material_albedo(const MaterialView &mv, int slot, float uvx, float uvy)
{
    if (slot < 0) return v3(0.0f, 0.0f, 0.0f);
    const DeviceMaterial &m = mv.materials[slot];
    return m.albedoTex >= 0 ? texel_nearest(mv, m.albedoTex, uvx, uvy)
                            : v3(m.albedo[0], m.albedo[1], m.albedo[2]);
}

// Per-vertex terms of ComputeRadianceForPath for the material in `slot`.
__device__ __forceinline__ void vertex_terms(const MaterialView &mv, int slot, V3 N, V3 L, V3 V,
    float uvx, float uvy, float4 &ec, float4 &aa)
{
    V3 albedo = v3(0.0f, 0.0f, 0.0f), emission;
    float roughness = 0.0f;
    if (slot < 0) {
        emission = v3(1.0f, 0.0f, 1.0f);  // missing material: magenta
    } else {
        const DeviceMaterial &m = mv.materials[slot];
        albedo = m.albedoTex >= 0 ? texel_nearest(mv, m.albedoTex, uvx, uvy)
                                  : v3(m.albedo[0], m.albedo[1], m.albedo[2]);
        if (m.emissionTex == -2) {
            emission = sky_radiance(mv.sky, neg(V));
        } else if (m.emissionTex >= 0) {
            V3 dir = neg(V);  // src/math_lib.h:849-884
            float inc = atan2f(sqrtf(dir.x * dir.x + dir.z * dir.z), dir.y);
            float az = atan2f(dir.z, dir.x);
            if (az < 0.0f) az += 2.0f * kPi;
            float eu = az / (2.0f * kPi);
            float ev = cosf(inc) * 0.5f + 0.5f;
            ev = 1.0f - ev;
            emission = mul(texel_nearest(mv, m.emissionTex, eu, ev), 1.0f);
        } else {
            emission = v3(m.emission[0], m.emission[1], m.emission[2]);
        }
        roughness = m.roughness;
    }
    float cosine = rmax(0.0f, dot(N, L));
    V3 H = normalize(add(L, V));
    // FresnelSchlick(max(H.V, 0), 0.04) (src/simd_path_tracer.cpp:65-70)
    float p5 = powf(1.0f - rmax(dot(H, V), 0.0f), 5.0f);
    float F0 = 0.04f;
    float Fs = F0 + (1.0f - F0) * p5;
    V3 F = v3(Fs, Fs, Fs);
    V3 kD = sub(v3(1.0f, 1.0f, 1.0f), F);
    // DistributionGGX (:72-84)
    float a = roughness * roughness;
    float a2 = a * a;
    float NdotH = rmax(dot(N, H), 0.0f);
    float NdotH2 = NdotH * NdotH;
    float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
    denom = kPi * denom * denom;
    float NDF = a2 / denom;
    // GeometrySmith (:86-105)
    float NdotV = rmax(dot(N, V), 0.0f);
    float NdotL = rmax(dot(N, L), 0.0f);
    float r1 = roughness + 1.0f;
    float k = (r1 * r1) / 8.0f;
    float ggx2 = NdotV / (NdotV * (1.0f - k) + k);
    float ggx1 = NdotL / (NdotL * (1.0f - k) + k);
    float G = ggx1 * ggx2;
    V3 numerator = mul(F, NDF * G);
    float denominator = 4.0f * rmax(dot(N, V), 0.0f) * rmax(dot(N, L), 0.0f) + 0.0001f;
    V3 specular = mul(numerator, 1.0f / denominator);
    float oneOverPi = 1.0f / kPi;
    V3 A = add(mul(hadamard(kD, albedo), oneOverPi), specular);
    ec = make_float4(emission.x, emission.y, emission.z, cosine);
    aa = make_float4(A.x, A.y, A.z, 0.0f);
}

// One step of the reverse pass: radiance = E + (A * clamp(radiance)) * cosine.
__device__ __forceinline__ V3 radiance_step(V3 radiance, float4 ec, float4 aa, float clampValue)
{
    V3 Li = radiance;
    if (clampValue != 0.0f)
        Li = v3(rclamp(Li.x, 0.0f, clampValue), rclamp(Li.y, 0.0f, clampValue),
            rclamp(Li.z, 0.0f, clampValue));
    return add(v3(ec.x, ec.y, ec.z), mul(hadamard(v3(aa.x, aa.y, aa.z), Li), ec.w));
}

// Reverse pass over stored vertex terms.
__device__ __forceinline__ V3 path_radiance(const float4 *vertE, const float4 *vertA,
    size_t stride, uint32_t p, uint32_t len, float clampValue)
{
    V3 radiance = v3(0.0f, 0.0f, 0.0f);
    for (int i = (int)len - 1; i >= 0; i--)
        radiance = radiance_step(radiance, vertE[(size_t)i * stride + p],
            vertA[(size_t)i * stride + p], clampValue);
    return radiance;
}

// The same with the last vertex's terms given (not stored) and the len - 1
// before it read from memory.
__device__ __forceinline__ V3 path_radiance_last(const float4 *vertE, const float4 *vertA,
    size_t stride, uint32_t p, uint32_t len, float4 lastE, float4 lastA, float clampValue)
{
    V3 radiance = radiance_step(v3(0.0f, 0.0f, 0.0f), lastE, lastA, clampValue);
    for (int i = (int)len - 2; i >= 0; i--)
        radiance = radiance_step(radiance, vertE[(size_t)i * stride + p],
            vertA[(size_t)i * stride + p], clampValue);
    return radiance;
}

// One whole path in one thread: the body of the reference's per-sample loop
// (src/simd_path_tracer.cpp:208-324) - jitter and camera ray drawn from
// `rng`, up to maxBounces closest-hit queries, per-vertex terms, reverse pass.
template <int kMaxBounces, bool kWT = false>
__device__ __forceinline__ V3 trace_full_path(const SceneView &sv, const MaterialView &mv,
    const CameraParams &cam, uint32_t x, uint32_t y, uint32_t &rng, uint32_t maxBounces,
    float clampValue, uint32_t *status, TraceCounters &cnt, uint32_t &rays, uint32_t &hits)
{
    float4 vE[kMaxBounces], vA[kMaxBounces];
    V3 o, d;
    camera_ray(cam, x, y, rng, o, d);
    uint32_t len = 0;
    if (maxBounces > (uint32_t)kMaxBounces) maxBounces = kMaxBounces;
    for (uint32_t b = 0; b < maxBounces; b++) {
        RayHit h = trace_closest<true, kWT>(sv, o, d, status, cnt);
        rays++;
        float4 ec, aa;
        if (h.prim >= 0 && h.t > 0.0f) {
            hits++;
            V3 n;
            float ux, uy;
            hit_surface(sv, h, n, ux, uy);
            V3 pos = add(o, mul(d, h.t));
            V3 dir = random_hemisphere(n, rng);
            vertex_terms(mv, mv.instanceSlot[h.inst], n, dir, neg(d), ux, uy, ec, aa);
            vE[len] = ec;
            vA[len] = aa;
            len++;
            o = add(pos, mul(n, 0.0001f));
            d = dir;
        } else {
            vertex_terms(mv, mv.backgroundSlot, v3(0, 0, 0), v3(0, 0, 0), neg(d), 0.0f, 0.0f, ec,
                aa);
            vE[len] = ec;
            vA[len] = aa;
            len++;
            break;
        }
    }
    return path_radiance(vE, vA, 1, 0, len, clampValue);
}

}  // namespace gbsp
