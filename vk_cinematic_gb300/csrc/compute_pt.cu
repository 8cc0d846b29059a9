// The reference's compute-shader path tracer (src/shaders/test_compute.comp.glsl)
// as a CUDA kernel.
//
// Semantics kept from the shader: one 16x16 (configurable) tile per work item,
// the tile's RNG seeded (tileIndex + 1) * 0xF51C0E49 and drawn in scanline
// order through the tile (2 jitter draws per pixel, 3 per hit), a brute-force
// closest hit over every entity's triangles in entity order (no BVH, no
// back-face culling, strict < so the first triangle wins ties), three bounces,
// hard-coded materials (0 red albedo, 2 checkerboard texture, 5 white light)
// and the normalize(N + rand3) bounce.
//
// GB300 layout: the tile's RNG chain makes its pixels sequential, so a whole
// warp works on one tile and splits each ray's triangle loop across its
// lanes: lane l tests triangles l, l+32, ... (its own strict-< minimum), then
// a warp reduction on (t, triangle index) gives the sequential loop's answer
// (smallest t, lowest index among equal t).  The eight warps of a block trace
// their rays in step so that every chunk of 256 triangles is staged into
// shared memory once for eight rays.  Triangles are pre-expanded per mesh
// into structure-of-arrays a, e1 = b - a, e2 = c - a (the same IEEE
// subtractions the shader performs), so staging is coalesced; texture
// coordinates are read only for the winner.  All other per-ray work is
// warp-uniform.
//
// Built-ins are fixed to one IEEE definition shared with the oracle (dot in
// x, y, z order; normalize = v * (1 / sqrt(dot)); mat4 * vec4 summed over
// columns 0..3; GLSL max(x, y) = x < y ? y : x) and compiled without
// contraction.

#include <vector>

#include "gbsp_internal.h"

namespace gbsp {
namespace cpt {

constexpr float kF32Max = 3.402823466e+38f;
constexpr uint32_t kMaterialRed = 0, kMaterialCheckerBoard = 2, kMaterialWhiteLight = 5,
                   kMaterialBlack = 6;
constexpr int kMaxBounces = 3;
constexpr int kWarpsPerBlock = 8;
constexpr int kChunk = 32 * kWarpsPerBlock;  // triangles staged per step (one per thread)

struct EntityDev {
    float model[16];
    float inv[16];
    uint32_t triBegin, triCount, material, pad;
};

struct TriSoA {
    const float *ax, *ay, *az, *e1x, *e1y, *e1z, *e2x, *e2y, *e2z;
    const float2 *uv;  // 3 per triangle
};

struct View {
    V3 right, up, position, center;
    float halfWidth, halfHeight, halfPixelWidth, halfPixelHeight, invW, invH;
    uint32_t width, height, tileW, tileH, tileCountX;
};

struct Counters {
    unsigned long long *rays, *hits, *tests, *paths;
};

__device__ __forceinline__ float cdot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V3 ccross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3 cnormalize(V3 v)
{
    float inv = 1.0f / sqrtf(cdot(v, v));
    return v3(v.x * inv, v.y * inv, v.z * inv);
}
__device__ __forceinline__ float glsl_max(float x, float y) { return x < y ? y : x; }

__device__ __forceinline__ V3 mat_mul(const float *m, V3 v, float w)
{
    V3 r;
    r.x = ((__ldg(m + 0) * v.x + __ldg(m + 4) * v.y) + __ldg(m + 8) * v.z) + __ldg(m + 12) * w;
    r.y = ((__ldg(m + 1) * v.x + __ldg(m + 5) * v.y) + __ldg(m + 9) * v.z) + __ldg(m + 13) * w;
    r.z = ((__ldg(m + 2) * v.x + __ldg(m + 6) * v.y) + __ldg(m + 10) * v.z) + __ldg(m + 14) * w;
    return r;
}

struct Rng {
    uint32_t s;
    __device__ __forceinline__ float bilateral()
    {
        uint32_t x = s;
        x ^= x << 13;
        x ^= x >> 17;
        x ^= x << 5;
        s = x;
        float u = __uint2float_rn(x) / 4294967296.0f;  // float(x) / float(U32_MAX)
        return -1.0f + 2.0f * u;
    }
};

__device__ __forceinline__ float wrap_coord(float u, uint32_t n, int32_t &i0, int32_t &i1)
{
    float x = u * (float)n - 0.5f;
    if (!(fabsf(x) < 1.0e9f)) {
        i0 = 0;
        i1 = n > 1 ? 1 : 0;
        return 0.0f;
    }
    float f = floorf(x);
    float a = x - f;
    long long i = (long long)f;
    long long m = ((i % (long long)n) + (long long)n) % (long long)n;
    i0 = (int32_t)m;
    i1 = (int32_t)((m + 1) % (long long)n);
    return a;
}

// Vulkan linear filter at the base level with REPEAT addressing (the
// reference's defaultSampler, src/vulkan_renderer.cpp:986-1001).
__device__ V3 sample_bilinear(const float4 *tex, uint32_t w, uint32_t h, float u, float v)
{
    if (!tex || !w || !h) return v3(0.0f, 0.0f, 0.0f);
    int32_t x0, x1, y0, y1;
    float a = wrap_coord(u, w, x0, x1);
    float b = wrap_coord(v, h, y0, y1);
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float4 t00 = __ldg(&tex[(size_t)y0 * w + x0]), t10 = __ldg(&tex[(size_t)y0 * w + x1]);
    float4 t01 = __ldg(&tex[(size_t)y1 * w + x0]), t11 = __ldg(&tex[(size_t)y1 * w + x1]);
    V3 r = v3(t00.x * w00, t00.y * w00, t00.z * w00);
    r = v3(r.x + t10.x * w10, r.y + t10.y * w10, r.z + t10.z * w10);
    r = v3(r.x + t01.x * w01, r.y + t01.y * w01, r.z + t01.z * w01);
    r = v3(r.x + t11.x * w11, r.y + t11.y * w11, r.z + t11.z * w11);
    return r;
}

struct SceneHit {
    float t;
    uint32_t material;
    V3 normal;
    float u, v;
};

struct PathVertex {
    uint32_t material;
    V3 incoming, normal;
    float u, v;
};

// Radiance of a finished path (test_compute.comp.glsl:441-481).
__device__ __forceinline__ V3 path_radiance_cpt(const PathVertex *path, int len,
    const float4 *__restrict__ tex, uint32_t texW, uint32_t texH)
{
    V3 radiance = v3(0.0f, 0.0f, 0.0f);
    for (int i = len - 1; i >= 0; i--) {
        V3 emission = v3(0.0f, 0.0f, 0.0f), albedo = v3(0.0f, 0.0f, 0.0f);
        uint32_t m = path[i].material;
        if (m == kMaterialRed)
            albedo = v3(0.18f, 0.1f, 0.1f);
        else if (m == kMaterialCheckerBoard)
            albedo = sample_bilinear(tex, texW, texH, path[i].u, path[i].v);
        else if (m == kMaterialWhiteLight)
            emission = v3(1.0f, 1.0f, 1.0f);
        float cosine = glsl_max(0.0f, cdot(path[i].normal, path[i].incoming));
        radiance = v3(emission.x + (albedo.x * radiance.x) * cosine,
            emission.y + (albedo.y * radiance.y) * cosine,
            emission.z + (albedo.z * radiance.z) * cosine);
    }
    return radiance;
}

// Block-lockstep kernel: the kWarpsPerBlock warps of a block own one tile
// each and trace their current rays together.  The brute-force triangle
// loop is the same sequence for every ray (entity by entity, triangle by
// triangle), so the block stages each chunk of kChunk triangles (9 floats
// each: a, e1, e2) into shared memory once - double-buffered, the next chunk
// loading while this one is tested - and every warp tests its own ray
// against it, lane l taking triangles l, l + 32, ...  Per warp the order of
// triangles, the strict-< minimum and every RNG draw are those of the
// shader's sequential loops, so results are unchanged; a warp whose tile is
// done keeps staging chunks for the others until the whole block is done.
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_compute_pt(const EntityDev *__restrict__ ents,
    uint32_t entityCount, TriSoA tri, const float4 *__restrict__ tex, uint32_t texW, uint32_t texH,
    View view, const uint32_t *__restrict__ tiles, uint32_t tileCount, float4 *__restrict__ image,
    Counters counters)
{
    __shared__ float sTri[2][9][kChunk];
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t item = blockIdx.x * kWarpsPerBlock + (tid >> 5);
    bool active = item < tileCount;
    uint32_t minX = 0, minY = 0, maxX = 0, maxY = 0, tileIndex = 0;
    if (active) {
        tileIndex = __ldg(&tiles[item]);
        uint32_t tx = tileIndex % view.tileCountX, ty = tileIndex / view.tileCountX;
        minX = tx * view.tileW;
        minY = ty * view.tileH;
        maxX = min(view.width, (tx + 1) * view.tileW);
        maxY = min(view.height, (ty + 1) * view.tileH);
        active = minX < maxX && minY < maxY;
    }
    Rng rng{(tileIndex + 1u) * 0xF51C0E49u};
    uint64_t rays = 0, hits = 0, tests = 0, paths = 0;
    uint32_t x = minX, y = minY;
    int len = 0, bounce = 0;
    PathVertex path[kMaxBounces];
    V3 o = v3(0.0f, 0.0f, 0.0f), d = v3(0.0f, 0.0f, 0.0f);
    // camera ray of pixel (x, y): test_compute.comp.glsl:510-540
    auto start_pixel = [&]() {
        float px = (float)x + 0.5f, py = (float)y + 0.5f;
        float jx = view.halfPixelWidth * rng.bilateral();
        float jy = view.halfPixelHeight * rng.bilateral();
        px = px + jx;
        py = py + jy;
        float fx = px * view.invW, fy = py * view.invH;
        fy = 1.0f - fy;
        fx = fx * 2.0f - 1.0f;
        fy = fy * 2.0f - 1.0f;
        V3 filmP = view.center;
        float sx = view.halfWidth * fx, sy = view.halfHeight * fy;
        filmP = v3(filmP.x + view.right.x * sx, filmP.y + view.right.y * sx,
            filmP.z + view.right.z * sx);
        filmP = v3(filmP.x + view.up.x * sy, filmP.y + view.up.y * sy, filmP.z + view.up.z * sy);
        o = view.position;
        d = cnormalize(v3(filmP.x - o.x, filmP.y - o.y, filmP.z - o.z));
        len = 0;
        bounce = 0;
    };
    if (active) start_pixel();
    // stage the triangles [c, c + n) of entity e into buffer buf
    auto stage = [&](uint32_t e, uint32_t c, int buf) {
        const EntityDev &ent = ents[e];
        uint32_t count = __ldg(&ent.triCount);
        uint32_t n = count - c < (uint32_t)kChunk ? count - c : (uint32_t)kChunk;
        if ((uint32_t)tid < n) {
            uint32_t g = __ldg(&ent.triBegin) + c + tid;
            sTri[buf][0][tid] = __ldg(tri.ax + g);
            sTri[buf][1][tid] = __ldg(tri.ay + g);
            sTri[buf][2][tid] = __ldg(tri.az + g);
            sTri[buf][3][tid] = __ldg(tri.e1x + g);
            sTri[buf][4][tid] = __ldg(tri.e1y + g);
            sTri[buf][5][tid] = __ldg(tri.e1z + g);
            sTri[buf][6][tid] = __ldg(tri.e2x + g);
            sTri[buf][7][tid] = __ldg(tri.e2y + g);
            sTri[buf][8][tid] = __ldg(tri.e2z + g);
        }
    };

    for (uint32_t guard = 0; guard < (1u << 30); guard++) {
        if (!__syncthreads_or(active)) break;
        // ---- trace: test_compute.comp.glsl:320-430, all warps in step
        SceneHit res;
        res.t = kF32Max;
        res.material = kMaterialBlack;
        res.normal = v3(0.0f, 0.0f, 0.0f);
        res.u = res.v = 0.0f;
        if (entityCount) {
            uint32_t e = 0, c = 0;
            int buf = 0;
            V3 lo = mat_mul(ents[0].inv, o, 1.0f);
            V3 ld = cnormalize(mat_mul(ents[0].inv, d, 0.0f));
            float bestT = kF32Max, bestU = 0.0f, bestV = 0.0f;
            uint32_t bestK = 0xFFFFFFFFu;
            stage(0, 0, 0);
            __syncthreads();
            while (e < entityCount) {
                const EntityDev &ent = ents[e];
                const uint32_t count = __ldg(&ent.triCount);
                // next chunk: the rest of this entity, else the next entity (an
                // entity without triangles is one empty chunk)
                uint32_t ne = e, nc = c + kChunk;
                if (nc >= count) {
                    ne = e + 1;
                    nc = 0;
                }
                if (ne < entityCount) stage(ne, nc, buf ^ 1);
                if (active) {
                    uint32_t n = count - c < (uint32_t)kChunk ? count - c : (uint32_t)kChunk;
                    if (c == 0) tests += count;
                    for (uint32_t j = lane; j < n; j += 32) {
                        V3 a = v3(sTri[buf][0][j], sTri[buf][1][j], sTri[buf][2][j]);
                        V3 e1 = v3(sTri[buf][3][j], sTri[buf][4][j], sTri[buf][5][j]);
                        V3 e2 = v3(sTri[buf][6][j], sTri[buf][7][j], sTri[buf][8][j]);
                        V3 T = v3(lo.x - a.x, lo.y - a.y, lo.z - a.z);
                        V3 p = ccross(ld, e2);
                        V3 q = ccross(T, e1);
                        float mx = cdot(q, e2), my = cdot(p, T), mz = cdot(q, ld);
                        float det = 1.0f / cdot(p, e1);
                        float t = det * mx, u = det * my, v = det * mz;
                        float w = 1.0f - u - v;
                        if (u >= 0.0f && u <= 1.0f && v >= 0.0f && v <= 1.0f && w >= 0.0f &&
                            w <= 1.0f && t >= 0.0f && t < kF32Max && t < bestT) {
                            bestT = t;
                            bestU = u;
                            bestV = v;
                            bestK = c + j;
                        }
                    }
                    if (ne != e) {
                        // entity e done: the sequential loop's answer, then world space
#pragma unroll
                        for (int off = 16; off; off >>= 1) {
                            float ot = __shfl_xor_sync(0xFFFFFFFFu, bestT, off);
                            uint32_t ok = __shfl_xor_sync(0xFFFFFFFFu, bestK, off);
                            if (ot < bestT || (ot == bestT && ok < bestK)) {
                                bestT = ot;
                                bestK = ok;
                            }
                        }
                        float meshT = kF32Max, meshU = 0.0f, meshV = 0.0f;
                        V3 localNormal = v3(0.0f, 0.0f, 0.0f);
                        if (bestK != 0xFFFFFFFFu) {
                            int src = (int)(bestK & 31u);
                            float u = __shfl_sync(0xFFFFFFFFu, bestU, src);
                            float v = __shfl_sync(0xFFFFFFFFu, bestV, src);
                            uint32_t g = __ldg(&ent.triBegin) + bestK;
                            V3 e1 = v3(__ldg(tri.e1x + g), __ldg(tri.e1y + g), __ldg(tri.e1z + g));
                            V3 e2 = v3(__ldg(tri.e2x + g), __ldg(tri.e2y + g), __ldg(tri.e2z + g));
                            localNormal = cnormalize(ccross(e1, e2));
                            float w = 1.0f - u - v;
                            float2 t0 = __ldg(&tri.uv[(size_t)g * 3 + 0]);
                            float2 t1 = __ldg(&tri.uv[(size_t)g * 3 + 1]);
                            float2 t2 = __ldg(&tri.uv[(size_t)g * 3 + 2]);
                            meshT = bestT;
                            meshU = (t0.x * w + t1.x * u) + t2.x * v;
                            meshV = (t0.y * w + t1.y * u) + t2.y * v;
                        }
                        V3 localHit = v3(lo.x + ld.x * meshT, lo.y + ld.y * meshT,
                            lo.z + ld.z * meshT);
                        V3 worldHit = mat_mul(ent.model, localHit, 1.0f);
                        float t = cdot(v3(worldHit.x - o.x, worldHit.y - o.y, worldHit.z - o.z), d);
                        V3 worldNormal = cnormalize(mat_mul(ent.model, localNormal, 0.0f));
                        if (t >= 0.0f && t < res.t) {
                            res.t = t;
                            res.material = __ldg(&ent.material);
                            res.normal = worldNormal;
                            res.u = meshU;
                            res.v = meshV;
                        }
                        if (ne < entityCount) {
                            lo = mat_mul(ents[ne].inv, o, 1.0f);
                            ld = cnormalize(mat_mul(ents[ne].inv, d, 0.0f));
                            bestT = kF32Max;
                            bestU = bestV = 0.0f;
                            bestK = 0xFFFFFFFFu;
                        }
                    }
                }
                __syncthreads();  // chunk consumed, next chunk staged
                e = ne;
                c = nc;
                buf ^= 1;
            }
        }
        if (!active) continue;
        // ---- shade: test_compute.comp.glsl:558-600 (warp-uniform)
        rays++;
        bool more = false;
        if (res.t > 0.0f && res.t < kF32Max) {
            hits++;
            float r0 = rng.bilateral();
            float r1 = rng.bilateral();
            float r2 = rng.bilateral();
            V3 dir = cnormalize(v3(res.normal.x + r0, res.normal.y + r1, res.normal.z + r2));
            if (cdot(dir, res.normal) < 0.0f) dir = v3(-dir.x, -dir.y, -dir.z);
            path[len].material = res.material;
            path[len].normal = res.normal;
            path[len].incoming = dir;
            path[len].u = res.u;
            path[len].v = res.v;
            len++;
            V3 wp = v3(o.x + d.x * res.t, o.y + d.y * res.t, o.z + d.z * res.t);
            o = v3(wp.x + res.normal.x * 0.001f, wp.y + res.normal.y * 0.001f,
                wp.z + res.normal.z * 0.001f);
            d = dir;
            bounce++;
            more = bounce < kMaxBounces;
        } else {
            path[len].material = kMaterialBlack;
            path[len].normal = v3(0.0f, 0.0f, 0.0f);
            path[len].incoming = v3(0.0f, 0.0f, 0.0f);
            path[len].u = path[len].v = 0.0f;
            len++;
        }
        if (more) continue;
        V3 radiance = path_radiance_cpt(path, len, tex, texW, texH);
        paths++;
        if (lane == 0)
            image[(size_t)y * view.width + x] = make_float4(0.0f + radiance.x * 1.0f,
                0.0f + radiance.y * 1.0f, 0.0f + radiance.z * 1.0f, 1.0f);
        // next pixel of the tile in scanline order
        if (++x >= maxX) {
            x = minX;
            y++;
        }
        if (y >= maxY)
            active = false;
        else
            start_pixel();
    }
    if (lane == 0) {
        atomicAdd(counters.rays, (unsigned long long)rays);
        atomicAdd(counters.hits, (unsigned long long)hits);
        atomicAdd(counters.tests, (unsigned long long)tests);
        atomicAdd(counters.paths, (unsigned long long)paths);
    }
}

}  // namespace cpt
}  // namespace gbsp

using namespace gbsp;

struct gbsp_cpt_scene {
    gbsp_runtime *rt = nullptr;
    uint32_t entityCount = 0, texW = 0, texH = 0;
    uint64_t triangleCount = 0;
    DeviceBuffer<cpt::EntityDev> entities;
    DeviceBuffer<float> soa;  // 9 component arrays of triangleCount floats
    DeviceBuffer<float2> uv;
    DeviceBuffer<float4> tex;
    DeviceBuffer<uint32_t> tiles;
};

extern "C" {

int gbsp_cpt_scene_create(gbsp_runtime *rt, const gbsp_vertex *vertices, uint32_t vertexCount,
    const uint32_t *indices, uint32_t indexCount, const gbsp_cpt_mesh *meshes, uint32_t meshCount,
    const float *modelMatrices, const float *invModelMatrices, uint32_t matrixCount,
    const gbsp_cpt_entity *entities, uint32_t entityCount, const float *checkerBoard,
    uint32_t texWidth, uint32_t texHeight, gbsp_cpt_scene **out)
{
    if (!rt || !out) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if ((entityCount && (!entities || !meshes || !modelMatrices || !invModelMatrices)) ||
        (indexCount && !indices) || (vertexCount && !vertices))
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL array with a non-zero count");
    if ((texWidth || texHeight) && (!checkerBoard || !texWidth || !texHeight))
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "texture needs pixels, width and height");
    // triangles per mesh, expanded once (entities share meshes)
    std::vector<uint64_t> meshBegin(meshCount), meshTris(meshCount);
    uint64_t total = 0;
    for (uint32_t m = 0; m < meshCount; m++) {
        const gbsp_cpt_mesh &mesh = meshes[m];
        uint64_t tris = mesh.indexCount / 3;
        if ((uint64_t)mesh.indicesOffset + tris * 3 > indexCount)
            return set_error(GBSP_ERR_INVALID_ARGUMENT, "mesh %u: indices out of range", m);
        for (uint64_t k = 0; k < tris * 3; k++) {
            uint64_t vi = (uint64_t)indices[mesh.indicesOffset + k] + mesh.vertexDataOffset;
            if (vi >= vertexCount)
                return set_error(GBSP_ERR_INVALID_ARGUMENT, "mesh %u: vertex index out of range", m);
        }
        meshBegin[m] = total;
        meshTris[m] = tris;
        total += tris;
    }
    if (total > 0xFFFFFFF0ull) return set_error(GBSP_ERR_CAPACITY, "too many triangles");
    std::vector<cpt::EntityDev> ents(entityCount);
    for (uint32_t e = 0; e < entityCount; e++) {
        const gbsp_cpt_entity &en = entities[e];
        if (en.meshIndex >= meshCount || en.modelMatrixIndex >= matrixCount)
            return set_error(GBSP_ERR_INVALID_ARGUMENT, "entity %u: mesh or matrix out of range", e);
        cpt::EntityDev &d = ents[e];
        for (int k = 0; k < 16; k++) {
            d.model[k] = modelMatrices[(size_t)en.modelMatrixIndex * 16 + k];
            d.inv[k] = invModelMatrices[(size_t)en.modelMatrixIndex * 16 + k];
        }
        d.triBegin = (uint32_t)meshBegin[en.meshIndex];
        d.triCount = (uint32_t)meshTris[en.meshIndex];
        d.material = en.materialId;
        d.pad = 0;
    }
    std::vector<float> soa((size_t)total * 9);
    std::vector<float2> uv((size_t)total * 3);
    for (uint32_t m = 0; m < meshCount; m++) {
        const gbsp_cpt_mesh &mesh = meshes[m];
        for (uint64_t k = 0; k < meshTris[m]; k++) {
            uint64_t g = meshBegin[m] + k;
            const gbsp_vertex *v[3];
            for (int j = 0; j < 3; j++)
                v[j] = &vertices[indices[mesh.indicesOffset + k * 3 + j] + mesh.vertexDataOffset];
            const float *a = v[0]->position, *b = v[1]->position, *c = v[2]->position;
            float comp[9] = {a[0], a[1], a[2], b[0] - a[0], b[1] - a[1], b[2] - a[2], c[0] - a[0],
                c[1] - a[1], c[2] - a[2]};
            for (int j = 0; j < 9; j++) soa[(size_t)j * total + g] = comp[j];
            for (int j = 0; j < 3; j++) uv[g * 3 + j] = make_float2(v[j]->uv[0], v[j]->uv[1]);
        }
    }
    int rrc = runtime_retain(rt);
    if (rrc) return rrc;
    gbsp_cpt_scene *s = new gbsp_cpt_scene();
    s->rt = rt;
    s->entityCount = entityCount;
    s->triangleCount = total;
    s->texW = texWidth;
    s->texH = texHeight;
    cudaStream_t st = rt->stream;
    int rc = GBSP_OK;
    if (entityCount) rc = s->entities.upload(ents.data(), ents.size(), st);
    if (!rc && total) rc = s->soa.upload(soa.data(), soa.size(), st);
    if (!rc && total) rc = s->uv.upload(uv.data(), uv.size(), st);
    if (!rc && texWidth)
        rc = s->tex.upload(reinterpret_cast<const float4 *>(checkerBoard),
            (size_t)texWidth * texHeight, st);
    if (!rc && cudaStreamSynchronize(st) != cudaSuccess)
        rc = set_error(GBSP_ERR_CUDA, "compute path tracer scene upload failed");
    if (rc) {
        delete s;
        runtime_release(rt);
        return rc;
    }
    *out = s;
    return GBSP_OK;
}

int gbsp_cpt_scene_destroy(gbsp_cpt_scene *scene)
{
    if (!scene) return GBSP_OK;
    gbsp_runtime *rt = scene->rt;
    cudaStreamSynchronize(rt->stream);
    delete scene;
    runtime_release(rt);
    return GBSP_OK;
}

int gbsp_cpt_render_tiles(gbsp_cpt_scene *scene, const gbsp_cpt_view *view,
    const uint32_t *tileIndices, uint32_t tileCount, float *deviceImage, gbsp_metrics *metrics)
{
    if (!scene || !view || (tileCount && (!tileIndices || !deviceImage)))
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!view->width || !view->height || !view->tileWidth || !view->tileHeight ||
        view->width < view->tileWidth)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad image or tile size");
    gbsp_runtime *rt = scene->rt;
    cudaStream_t s = rt->stream;
    if (!tileCount) return GBSP_OK;
    int rc = scene->tiles.upload(tileIndices, tileCount, s);
    if (rc) return rc;
    // main() of the shader: film and camera (test_compute.comp.glsl:615-668)
    cpt::View v;
    float planeW = (float)view->width, planeH = (float)view->height;
    float filmWidth = 1.0f, filmHeight = 1.0f;
    if (planeW > planeH)
        filmHeight = planeH / planeW;
    else if (planeW < planeH)
        filmWidth = planeW / planeH;
    const float *ct = view->cameraTransform;
    v.right = v3(ct[0], ct[1], ct[2]);
    v.up = v3(ct[4], ct[5], ct[6]);
    V3 forward = v3(ct[8], ct[9], ct[10]);
    v.position = v3(ct[12], ct[13], ct[14]);
    v.halfWidth = filmWidth * 0.5f;
    v.halfHeight = filmHeight * 0.5f;
    v.halfPixelWidth = 0.5f / planeW;
    v.halfPixelHeight = 0.5f / planeH;
    float fd = view->filmDistance;
    v.center = v3(v.position.x + forward.x * fd, v.position.y + forward.y * fd,
        v.position.z + forward.z * fd);
    v.invW = 1.0f / planeW;
    v.invH = 1.0f / planeH;
    v.width = view->width;
    v.height = view->height;
    v.tileW = view->tileWidth;
    v.tileH = view->tileHeight;
    v.tileCountX = view->width / view->tileWidth;
    cpt::TriSoA tri;
    uint64_t n = scene->triangleCount;
    const float *base = scene->soa.ptr;
    const float **comp[9] = {&tri.ax, &tri.ay, &tri.az, &tri.e1x, &tri.e1y, &tri.e1z, &tri.e2x,
        &tri.e2y, &tri.e2z};
    for (int j = 0; j < 9; j++) *comp[j] = base ? base + (size_t)j * n : nullptr;
    tri.uv = scene->uv.ptr;
    cpt::Counters c;
    c.rays = rt->dCounters + GBSP_METRIC_RAYS_TRACED;
    c.hits = rt->dCounters + GBSP_METRIC_RAY_HIT_COUNT;
    c.tests = rt->dCounters + GBSP_METRIC_TRIANGLE_TESTS;
    c.paths = rt->dCounters + GBSP_METRIC_PATHS_TRACED;
    GBSP_CUDA_TRY(cudaMemsetAsync(rt->dCounters, 0, sizeof(unsigned long long) * GBSP_METRIC_COUNT, s));
    if (metrics) GBSP_CUDA_TRY(cudaEventRecord(rt->ev[0], s));
    uint32_t grid = (tileCount + cpt::kWarpsPerBlock - 1) / cpt::kWarpsPerBlock;
    cpt::k_compute_pt<<<grid, 32 * cpt::kWarpsPerBlock, 0, s>>>(scene->entities.ptr,
        scene->entityCount, tri, scene->tex.ptr, scene->texW, scene->texH, v, scene->tiles.ptr,
        tileCount, reinterpret_cast<float4 *>(deviceImage), c);
    GBSP_CUDA_TRY(cudaGetLastError());
    if (!metrics) return GBSP_OK;
    GBSP_CUDA_TRY(cudaEventRecord(rt->ev[1], s));
    unsigned long long cnt[GBSP_METRIC_COUNT];
    GBSP_CUDA_TRY(cudaMemcpyAsync(cnt, rt->dCounters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, rt->ev[0], rt->ev[1]);
    for (int i = 0; i < GBSP_METRIC_COUNT; i++) metrics->values[i] += cnt[i];
    metrics->values[GBSP_METRIC_RAY_MISS_COUNT] +=
        cnt[GBSP_METRIC_RAYS_TRACED] - cnt[GBSP_METRIC_RAY_HIT_COUNT];
    metrics->values[GBSP_METRIC_ELAPSED_NS] += (uint64_t)((double)ms * 1.0e6);
    metrics->values[GBSP_METRIC_KERNEL_LAUNCHES] += 1;
    return GBSP_OK;
}

}  // extern "C"
