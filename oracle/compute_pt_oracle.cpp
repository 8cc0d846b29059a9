// Oracle for the compute path tracer: TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of the reference's GPU compute-shader path tracer
// (src/shaders/test_compute.comp.glsl): one invocation per 16x16 tile, RNG
// seeded (tileIndex + 1) * 0xF51C0E49 and drawn in scanline order through the
// tile, brute-force closest hit over every entity's triangles (no BVH, no
// back-face culling), diffuse-only shading with hard-coded material ids and a
// normalize(N + rand3) bounce.  Only tests and the CPU-baseline leg of the
// benchmark use it.
//
// The shader's built-ins have implementation-defined precision in Vulkan, so
// this restatement fixes one IEEE single-precision definition of each and the
// CUDA kernel follows the same one (both without contraction):
//   dot(a, b)        (a.x*b.x + a.y*b.y) + a.z*b.z
//   normalize(v)     v * (1 / sqrt(dot(v, v)))
//   m * vec4(v, w)   ((c0*v.x + c1*v.y) + c2*v.z) + c3*w, per row
//   GLSL argument evaluation is left to right (GLSL 4.50 section 6.1), so in
//   vec2(hw * RandomBilateral(), hh * RandomBilateral()) x draws first.
// Values the shader leaves uninitialised (the normal and uv of a mesh without
// a hit, the fields of a miss vertex) are zero here.  Texture sampling is the
// Vulkan linear filter at the base level with REPEAT addressing, written from
// the Vulkan specification's formula with exact weights; hardware samplers
// quantise the weights, so checkerboard pixels are not pinned to a Vulkan
// device (none can be brought up on this machine).

#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

struct V3 {
    float x, y, z;
};
struct V2 {
    float x, y;
};

V3 v3(float x, float y, float z) { return V3{x, y, z}; }
V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
V3 hadamard(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
V3 cross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
V3 normalize(V3 v)
{
    float inv = 1.0f / std::sqrt(dot(v, v));
    return mul(v, inv);
}
// GLSL max(x, y): "y if x < y, otherwise x" (GLSL 4.50 section 8.3)
float glsl_max(float x, float y) { return x < y ? y : x; }

// column-major 4x4: m[c*4 + r]
V3 mat_mul(const float *m, V3 v, float w)
{
    V3 r;
    r.x = ((m[0] * v.x + m[4] * v.y) + m[8] * v.z) + m[12] * w;
    r.y = ((m[1] * v.x + m[5] * v.y) + m[9] * v.z) + m[13] * w;
    r.z = ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * w;
    return r;
}

const float kF32Max = 3.402823466e+38f;

// test_compute.comp.glsl:117-135
struct Rng {
    uint32_t s;
    uint32_t next()
    {
        uint32_t x = s;
        x ^= x << 13;
        x ^= x >> 17;
        x ^= x << 5;
        s = x;
        return x;
    }
    float unilateral() { return (float)next() / (float)0xFFFFFFFFu; }
    float bilateral() { return -1.0f + 2.0f * unilateral(); }
};

struct TriResult {
    float t;
    V2 uv;
    V3 normal;
};

// test_compute.comp.glsl:167-198 (no back-face test)
TriResult intersect_triangle(V3 o, V3 d, V3 a, V3 b, V3 c)
{
    TriResult r;
    r.t = -1.0f;
    r.uv = V2{0.0f, 0.0f};
    r.normal = v3(0.0f, 0.0f, 0.0f);
    V3 T = sub(o, a);
    V3 e1 = sub(b, a);
    V3 e2 = sub(c, a);
    V3 p = cross(d, e2);
    V3 q = cross(T, e1);
    V3 m = v3(dot(q, e2), dot(p, T), dot(q, d));
    float det = 1.0f / dot(p, e1);
    float t = det * m.x;
    float u = det * m.y;
    float v = det * m.z;
    float w = 1.0f - u - v;
    if (u >= 0.0f && u <= 1.0f && v >= 0.0f && v <= 1.0f && w >= 0.0f && w <= 1.0f) {
        r.t = t;
        r.normal = normalize(cross(e1, e2));
        r.uv = V2{u, v};
    }
    return r;
}

struct Mesh {
    uint32_t indexCount, indicesOffset, vertexDataOffset;
};
struct Entity {
    uint32_t meshIndex, materialId, modelMatrixIndex;
};

struct Scene {
    const float *vertices;  // VertexPNT: px py pz nx ny nz tx ty
    const uint32_t *indices;
    const Mesh *meshes;
    const float *model;  // 16 floats per matrix
    const float *invModel;
    const Entity *entities;
    uint32_t entityCount;
    const float *tex;  // RGBA32F checkerboard
    uint32_t texW, texH;
};

V3 vpos(const Scene &s, uint32_t i)
{
    const float *v = s.vertices + (size_t)i * 8;
    return v3(v[0], v[1], v[2]);
}
V2 vuv(const Scene &s, uint32_t i)
{
    const float *v = s.vertices + (size_t)i * 8;
    return V2{v[6], v[7]};
}

// test_compute.comp.glsl:265-310
TriResult intersect_mesh(const Scene &s, const Mesh &mesh, V3 o, V3 d)
{
    TriResult best;
    best.t = kF32Max;
    best.uv = V2{0.0f, 0.0f};
    best.normal = v3(0.0f, 0.0f, 0.0f);
    uint32_t triCount = mesh.indexCount / 3;
    for (uint32_t k = 0; k < triCount; k++) {
        uint32_t i0 = s.indices[k * 3 + 0 + mesh.indicesOffset] + mesh.vertexDataOffset;
        uint32_t i1 = s.indices[k * 3 + 1 + mesh.indicesOffset] + mesh.vertexDataOffset;
        uint32_t i2 = s.indices[k * 3 + 2 + mesh.indicesOffset] + mesh.vertexDataOffset;
        TriResult r = intersect_triangle(o, d, vpos(s, i0), vpos(s, i1), vpos(s, i2));
        if (r.t >= 0.0f && r.t < kF32Max && r.t < best.t) {
            best = r;
            float w = 1.0f - r.uv.x - r.uv.y;
            V2 t0 = vuv(s, i0), t1 = vuv(s, i1), t2 = vuv(s, i2);
            best.uv.x = (t0.x * w + t1.x * r.uv.x) + t2.x * r.uv.y;
            best.uv.y = (t0.y * w + t1.y * r.uv.x) + t2.y * r.uv.y;
        }
    }
    return best;
}

struct SceneHit {
    float t;
    uint32_t material;
    V3 normal;
    V2 uv;
};

const uint32_t kMaterialRed = 0, kMaterialCheckerBoard = 2, kMaterialWhiteLight = 5,
               kMaterialBlack = 6;

// test_compute.comp.glsl:320-430 (the live part: the entity loop)
SceneHit intersect_scene(const Scene &s, V3 o, V3 d, uint64_t *triTests)
{
    SceneHit res;
    res.t = kF32Max;
    res.material = kMaterialBlack;
    res.normal = v3(0.0f, 0.0f, 0.0f);
    res.uv = V2{0.0f, 0.0f};
    for (uint32_t e = 0; e < s.entityCount; e++) {
        const Entity &ent = s.entities[e];
        const Mesh &mesh = s.meshes[ent.meshIndex];
        const float *model = s.model + (size_t)ent.modelMatrixIndex * 16;
        const float *inv = s.invModel + (size_t)ent.modelMatrixIndex * 16;
        V3 lo = mat_mul(inv, o, 1.0f);
        V3 ld = normalize(mat_mul(inv, d, 0.0f));
        TriResult tr = intersect_mesh(s, mesh, lo, ld);
        if (triTests) *triTests += mesh.indexCount / 3;
        V3 localHit = add(lo, mul(ld, tr.t));
        V3 worldHit = mat_mul(model, localHit, 1.0f);
        float t = dot(sub(worldHit, o), d);
        V3 worldNormal = normalize(mat_mul(model, tr.normal, 0.0f));
        if (t >= 0.0f && t < res.t) {
            res.t = t;
            res.material = ent.materialId;
            res.normal = worldNormal;
            res.uv = tr.uv;
        }
    }
    return res;
}

// Texel coordinate of the Vulkan linear filter along one axis: i0 =
// floor(u * n - 0.5) and i1 = i0 + 1, each wrapped with REPEAT (i mod n);
// returns the fraction.  A non-finite or huge coordinate samples texel 0.
float wrap_coord(float u, uint32_t n, int32_t *i0, int32_t *i1)
{
    float x = u * (float)n - 0.5f;
    if (!(std::fabs(x) < 1.0e9f)) {
        *i0 = 0;
        *i1 = n > 1 ? 1 : 0;
        return 0.0f;
    }
    float f = std::floor(x);
    float a = x - f;
    int64_t i = (int64_t)f;
    int64_t m = ((i % (int64_t)n) + (int64_t)n) % (int64_t)n;
    *i0 = (int32_t)m;
    *i1 = (int32_t)((m + 1) % (int64_t)n);
    return a;
}

// Vulkan linear filter, base level, REPEAT (the reference's defaultSampler,
// src/vulkan_renderer.cpp:986-1001): tau = (1-a)(1-b) t00 + a(1-b) t10 +
// (1-a) b t01 + a b t11.
V3 sample_bilinear(const Scene &s, V2 uv)
{
    if (!s.tex || !s.texW || !s.texH) return v3(0.0f, 0.0f, 0.0f);
    int32_t x0, x1, y0, y1;
    float a = wrap_coord(uv.x, s.texW, &x0, &x1);
    float b = wrap_coord(uv.y, s.texH, &y0, &y1);
    auto texel = [&](int32_t x, int32_t y) {
        const float *p = s.tex + ((size_t)y * s.texW + (size_t)x) * 4;
        return v3(p[0], p[1], p[2]);
    };
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b,
          w11 = a * b;
    V3 r = mul(texel(x0, y0), w00);
    r = add(r, mul(texel(x1, y0), w10));
    r = add(r, mul(texel(x0, y1), w01));
    r = add(r, mul(texel(x1, y1), w11));
    return r;
}

struct PathVertex {
    uint32_t material;
    V3 incoming, normal;
    V2 uv;
};

const int kMaxBounces = 3;

// test_compute.comp.glsl:441-481
V3 radiance_for_path(const Scene &s, const PathVertex *path, int len)
{
    V3 radiance = v3(0.0f, 0.0f, 0.0f);
    for (int i = len - 1; i >= 0; i--) {
        const PathVertex &vx = path[i];
        V3 emission = v3(0.0f, 0.0f, 0.0f), albedo = v3(0.0f, 0.0f, 0.0f);
        if (vx.material == kMaterialRed)
            albedo = v3(0.18f, 0.1f, 0.1f);
        else if (vx.material == kMaterialCheckerBoard)
            albedo = sample_bilinear(s, vx.uv);
        else if (vx.material == kMaterialWhiteLight)
            emission = v3(1.0f, 1.0f, 1.0f);
        float cosine = glsl_max(0.0f, dot(vx.normal, vx.incoming));
        radiance = add(emission, mul(hadamard(albedo, radiance), cosine));
    }
    return radiance;
}

}  // namespace

extern "C" {

// One tile of test_compute.comp.glsl:PathTraceTile + main (lines 510-671):
// tile (tileIndex % (width / tileW), tileIndex / (width / tileW)), clipped to
// the image; the camera is the 4 columns of cameraTransform (right, up,
// forward, position; column-major 16 floats).  Writes RGBA32F pixels of the
// tile into image (width * height * 4).  counters: [rays, hits, triangle
// tests] (may be NULL).
void oracle_compute_pt_tiles(const float *vertices, const uint32_t *indices,
    const uint32_t *meshes, const float *model, const float *invModel,
    const uint32_t *entities, uint32_t entityCount, const float *tex, uint32_t texW,
    uint32_t texH, const float *cameraTransform, uint32_t width, uint32_t height,
    uint32_t tileW, uint32_t tileH, float filmDistance, const uint32_t *tileIndices,
    uint32_t tileCount, float *image, uint64_t *counters)
{
    Scene s;
    s.vertices = vertices;
    s.indices = indices;
    s.meshes = reinterpret_cast<const Mesh *>(meshes);
    s.model = model;
    s.invModel = invModel;
    s.entities = reinterpret_cast<const Entity *>(entities);
    s.entityCount = entityCount;
    s.tex = tex;
    s.texW = texW;
    s.texH = texH;

    float planeW = (float)width, planeH = (float)height;
    float filmWidth = 1.0f, filmHeight = 1.0f;
    if (planeW > planeH)
        filmHeight = planeH / planeW;
    else if (planeW < planeH)
        filmWidth = planeW / planeH;
    const float *ct = cameraTransform;
    V3 right = v3(ct[0], ct[1], ct[2]);
    V3 up = v3(ct[4], ct[5], ct[6]);
    V3 forward = v3(ct[8], ct[9], ct[10]);
    V3 position = v3(ct[12], ct[13], ct[14]);
    float halfWidth = filmWidth * 0.5f, halfHeight = filmHeight * 0.5f;
    float halfPixelWidth = 0.5f / planeW, halfPixelHeight = 0.5f / planeH;
    V3 center = add(position, mul(forward, filmDistance));
    float invW = 1.0f / planeW, invH = 1.0f / planeH;
    uint32_t tileCountX = width / tileW;
    uint64_t rays = 0, hits = 0, tests = 0;

    for (uint32_t q = 0; q < tileCount; q++) {
        uint32_t tileIndex = tileIndices[q];
        uint32_t tx = tileIndex % tileCountX, ty = tileIndex / tileCountX;
        uint32_t minX = tx * tileW, minY = ty * tileH;
        uint32_t maxX = (tx + 1) * tileW < width ? (tx + 1) * tileW : width;
        uint32_t maxY = (ty + 1) * tileH < height ? (ty + 1) * tileH : height;
        Rng rng{(tileIndex + 1u) * 0xF51C0E49u};
        for (uint32_t y = minY; y < maxY; y++) {
            for (uint32_t x = minX; x < maxX; x++) {
                float px = (float)x + 0.5f, py = (float)y + 0.5f;
                float jx = halfPixelWidth * rng.bilateral();
                float jy = halfPixelHeight * rng.bilateral();
                px = px + jx;
                py = py + jy;
                float fx = px * invW, fy = py * invH;
                fy = 1.0f - fy;
                fx = fx * 2.0f - 1.0f;
                fy = fy * 2.0f - 1.0f;
                V3 filmP = center;
                filmP = add(filmP, mul(right, halfWidth * fx));
                filmP = add(filmP, mul(up, halfHeight * fy));
                V3 o = position;
                V3 d = normalize(sub(filmP, o));
                PathVertex path[kMaxBounces];
                int len = 0;
                for (int b = 0; b < kMaxBounces; b++) {
                    SceneHit h = intersect_scene(s, o, d, &tests);
                    rays++;
                    if (h.t > 0.0f && h.t < kF32Max) {
                        hits++;
                        PathVertex vx;
                        vx.material = h.material;
                        vx.normal = h.normal;
                        vx.uv = h.uv;
                        float r0 = rng.bilateral();
                        float r1 = rng.bilateral();
                        float r2 = rng.bilateral();
                        V3 dir = normalize(add(h.normal, v3(r0, r1, r2)));
                        if (dot(dir, h.normal) < 0.0f) dir = neg(dir);
                        vx.incoming = dir;
                        path[len++] = vx;
                        V3 wp = add(o, mul(d, h.t));
                        o = add(wp, mul(h.normal, 0.001f));
                        d = dir;
                    } else {
                        PathVertex vx;
                        vx.material = kMaterialBlack;
                        vx.incoming = v3(0.0f, 0.0f, 0.0f);
                        vx.normal = v3(0.0f, 0.0f, 0.0f);
                        vx.uv = V2{0.0f, 0.0f};
                        path[len++] = vx;
                        break;
                    }
                }
                V3 r = radiance_for_path(s, path, len);
                // totalRadiance += radiance * (1 / 1)
                V3 total = add(v3(0.0f, 0.0f, 0.0f), mul(r, 1.0f / 1.0f));
                float *out = image + ((size_t)y * width + x) * 4;
                out[0] = total.x;
                out[1] = total.y;
                out[2] = total.z;
                out[3] = 1.0f;
            }
        }
    }
    if (counters) {
        counters[0] += rays;
        counters[1] += hits;
        counters[2] += tests;
    }
}

}  // extern "C"
