// Shared device/host definitions of the GB300 path tracer.
//
// Arithmetic here reproduces the reference's single-precision expressions
// operation for operation: the library is compiled with --fmad=false (and
// the host side with -ffp-contract=off) so no a*b+c is fused unless a
// function asks for fmaf explicitly, and every min/max is the reference's
// "a < b ? a : b" form (src/math_utils.h:5-15), whose NaN behaviour differs
// from fminf/fmaxf.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define GBSP_HD __host__ __device__ __forceinline__

namespace gbsp {

constexpr float kPi = 3.14159265359f;          // src/math_lib.h:6
constexpr float kEpsilon = 1.19209290e-07f;    // FLT_EPSILON, src/math_lib.h:7
constexpr uint32_t kNoTexture = 0xFFFFFFFFu;
constexpr uint32_t kSkyTexture = 0xFFFFFFFEu;

// ---------------------------------------------------------------------------
// Scalar / vector helpers
// ---------------------------------------------------------------------------
GBSP_HD float rmin(float a, float b) { return a < b ? a : b; }
GBSP_HD float rmax(float a, float b) { return a > b ? a : b; }
GBSP_HD float rclamp(float x, float lo, float hi) { return rmin(rmax(x, lo), hi); }

struct V3 {
    float x, y, z;
};
GBSP_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
GBSP_HD V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
GBSP_HD V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
GBSP_HD V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
GBSP_HD V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
GBSP_HD V3 hadamard(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
// src/math_lib.h:461-477
GBSP_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GBSP_HD V3 cross(V3 a, V3 b)
{
    return v3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z),
        (a.x * b.y) - (a.y * b.x));
}
GBSP_HD V3 vmin(V3 a, V3 b) { return v3(rmin(a.x, b.x), rmin(a.y, b.y), rmin(a.z, b.z)); }
GBSP_HD V3 vmax(V3 a, V3 b) { return v3(rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z)); }
GBSP_HD float max_component(V3 a) { return rmax(a.x, rmax(a.y, a.z)); }
GBSP_HD float min_component(V3 a) { return rmin(a.x, rmin(a.y, a.z)); }
GBSP_HD V3 inverse(V3 a) { return v3(1.0f / a.x, 1.0f / a.y, 1.0f / a.z); }
// src/math_lib.h:503-512
GBSP_HD V3 normalize(V3 v, float *lengthOut = nullptr)
{
    float len = sqrtf(dot(v, v));
    if (lengthOut) *lengthOut = len;
    V3 r = v3(0.0f, 0.0f, 0.0f);
    if (len > kEpsilon) r = mul(v, 1.0f / len);
    return r;
}

// 3x4 affine transform, rows of the reference's column-major mat4:
// row i = (m[i], m[4+i], m[8+i], m[12+i]).  Point / vector transforms
// follow the 4-term dot of src/math_lib.h:238-247, 381-398, 748-758.
struct Affine {
    float r[12];
};
GBSP_HD V3 transform_point(const Affine &m, V3 p)
{
    return v3(((m.r[0] * p.x + m.r[1] * p.y) + m.r[2] * p.z) + m.r[3] * 1.0f,
        ((m.r[4] * p.x + m.r[5] * p.y) + m.r[6] * p.z) + m.r[7] * 1.0f,
        ((m.r[8] * p.x + m.r[9] * p.y) + m.r[10] * p.z) + m.r[11] * 1.0f);
}
GBSP_HD V3 transform_vector(const Affine &m, V3 d)
{
    return v3(((m.r[0] * d.x + m.r[1] * d.y) + m.r[2] * d.z) + m.r[3] * 0.0f,
        ((m.r[4] * d.x + m.r[5] * d.y) + m.r[6] * d.z) + m.r[7] * 0.0f,
        ((m.r[8] * d.x + m.r[9] * d.y) + m.r[10] * d.z) + m.r[11] * 0.0f);
}

// ---------------------------------------------------------------------------
// RNG (src/math_utils.h:184-214) and per-sample seeding
// ---------------------------------------------------------------------------
GBSP_HD uint32_t xorshift32(uint32_t &s)
{
    uint32_t x = s;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    s = x;
    return x;
}
GBSP_HD float random_unilateral(uint32_t &s)
{
    float num = (float)(xorshift32(s) >> 1);
    float den = (float)(0xFFFFFFFFu >> 1);
    return num / den;
}
GBSP_HD float random_bilateral(uint32_t &s) { return -1.0f + 2.0f * random_unilateral(s); }

// PCG-style integer hash (Jarzynski & Olano, "Hash Functions for GPU
// Rendering", JCGT 9(3), 2020), chained over (seed, x, y, sample); a zero
// state (the fixed point of XorShift32) is replaced by a constant.
GBSP_HD uint32_t pcg_hash(uint32_t v)
{
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
GBSP_HD uint32_t sample_seed(uint32_t seed, uint32_t x, uint32_t y, uint32_t s)
{
    uint32_t h = pcg_hash(seed);
    h = pcg_hash(h ^ x);
    h = pcg_hash(h ^ y);
    h = pcg_hash(h ^ s);
    return h != 0u ? h : 0x6D2B79F5u;
}

// src/math_lib.h:932-959 (+ MapSphericalToCartesianCoordinates :864-871)
GBSP_HD V3 random_hemisphere(V3 n, uint32_t &s)
{
    float theta = kPi * random_unilateral(s);
    float phi = kPi * random_bilateral(s);
    float st = sinf(theta);
    V3 d;
    d.x = st * cosf(phi);
    d.z = st * sinf(phi);
    d.y = cosf(theta);
    if (dot(d, n) < 0.0f) d = neg(d);
    return d;
}

// Neumaier-compensated sum (per colour channel) for per-pixel accumulation.
struct CSum {
    float s, c;
};
GBSP_HD void csum_add(CSum &a, float x)
{
    float t = a.s + x;
    if (fabsf(a.s) >= fabsf(x))
        a.c += (a.s - t) + x;
    else
        a.c += (x - t) + a.s;
    a.s = t;
}
GBSP_HD float csum_value(const CSum &a) { return a.s + a.c; }

// ---------------------------------------------------------------------------
// Camera (src/simd_path_tracer.cpp:1-63)
// ---------------------------------------------------------------------------
struct CameraParams {
    V3 right, up, forward, position, filmCenter;
    float halfPixelWidth, halfPixelHeight, halfFilmWidth, halfFilmHeight;
    uint32_t width, height;
};

GBSP_HD V3 film_position(const CameraParams &c, float px, float py)
{
    float fx = px / (float)c.width;
    float fy = py / (float)c.height;
    fy = 1.0f - fy;
    fx = fx * 2.0f - 1.0f;
    fy = fy * 2.0f - 1.0f;
    V3 r = mul(c.right, c.halfFilmWidth * fx);
    r = add(r, mul(c.up, c.halfFilmHeight * fy));
    r = add(r, c.filmCenter);
    return r;
}

// Primary ray of one sample: jitter (two draws, y first - the reference's
// argument evaluation order, src/simd_path_tracer.cpp:219-222), film point,
// normalised direction.
GBSP_HD void camera_ray(const CameraParams &c, uint32_t x, uint32_t y, uint32_t &rng,
    V3 &o, V3 &d)
{
    float jy = c.halfPixelHeight * random_bilateral(rng);
    float jx = c.halfPixelWidth * random_bilateral(rng);
    float px = (float)x + 0.5f;
    float py = (float)y + 0.5f;
    px = px + jx;
    py = py + jy;
    V3 f = film_position(c, px, py);
    o = c.position;
    d = normalize(sub(f, c.position));
}

// ---------------------------------------------------------------------------
// Intersection primitives
// ---------------------------------------------------------------------------
// src/simd.h:198-271 for one box: hit iff max(0, max(tmin)) <= min(tmax)
// with t0 = (lo - o) * invd; returns the entry distance or -1.
GBSP_HD float slab_entry(V3 lo, V3 hi, V3 o, V3 invd)
{
    float t0x = (lo.x - o.x) * invd.x, t1x = (hi.x - o.x) * invd.x;
    float t0y = (lo.y - o.y) * invd.y, t1y = (hi.y - o.y) * invd.y;
    float t0z = (lo.z - o.z) * invd.z, t1z = (hi.z - o.z) * invd.z;
    float mnx = t0x < t1x ? t0x : t1x, mxx = t0x > t1x ? t0x : t1x;
    float mny = t0y < t1y ? t0y : t1y, mxy = t0y > t1y ? t0y : t1y;
    float mnz = t0z < t1z ? t0z : t1z, mxz = t0z > t1z ? t0z : t1z;
    float tn = rmax(0.0f, rmax(mnx, rmax(mny, mnz)));
    float tf = rmin(mxx, rmin(mxy, mxz));
    return tn <= tf ? tn : -1.0f;
}

// The slab test of interior nodes for rays whose inverse direction is finite:
// the same arithmetic with min / max instructions (fminf / fmaxf) in place of
// the reference's `a < b ? a : b` form.  The two differ only when an operand
// is NaN or the operands are zeros of opposite sign; with finite boxes, a
// finite origin and a finite inverse direction no NaN can arise, and signed
// zeros compare equal, so every decision and entry distance is the same.
// Leaves (the triangle box gate) keep slab_entry.
GBSP_HD float slab_entry_node(V3 lo, V3 hi, V3 o, V3 invd)
{
    float t0x = (lo.x - o.x) * invd.x, t1x = (hi.x - o.x) * invd.x;
    float t0y = (lo.y - o.y) * invd.y, t1y = (hi.y - o.y) * invd.y;
    float t0z = (lo.z - o.z) * invd.z, t1z = (hi.z - o.z) * invd.z;
    float tn = fmaxf(fmaxf(0.0f, fminf(t0x, t1x)), fmaxf(fminf(t0y, t1y), fminf(t0z, t1z)));
    float tf = fminf(fmaxf(t0x, t1x), fminf(fmaxf(t0y, t1y), fmaxf(t0z, t1z)));
    return tn <= tf ? tn : -1.0f;
}

// The same test with the exit distance scaled by 1 + 2 gamma(3) (Ize, "Robust
// BVH Ray Traversal", JCGT 2(2), 2013): a rounded slab test can no longer
// reject a ray that touches the box, which the watertight mode relies on.
GBSP_HD float slab_entry_robust(V3 lo, V3 hi, V3 o, V3 invd)
{
    float t0x = (lo.x - o.x) * invd.x, t1x = (hi.x - o.x) * invd.x;
    float t0y = (lo.y - o.y) * invd.y, t1y = (hi.y - o.y) * invd.y;
    float t0z = (lo.z - o.z) * invd.z, t1z = (hi.z - o.z) * invd.z;
    float mnx = t0x < t1x ? t0x : t1x, mxx = t0x > t1x ? t0x : t1x;
    float mny = t0y < t1y ? t0y : t1y, mxy = t0y > t1y ? t0y : t1y;
    float mnz = t0z < t1z ? t0z : t1z, mxz = t0z > t1z ? t0z : t1z;
    float tn = rmax(0.0f, rmax(mnx, rmax(mny, mnz)));
    float tf = rmin(mxx, rmin(mxy, mxz)) * 1.0000004f;
    return tn <= tf ? tn : -1.0f;
}

struct TriHit {
    float t, u, v;
    bool hit;
};

// src/ray_intersection.cpp:156-190 with e1, e2 from the stored vertices and
// the precomputed face normal n = cross(e1, e2).
GBSP_HD TriHit ray_triangle_mt(V3 o, V3 d, V3 a, V3 b, V3 c, V3 n)
{
    TriHit r;
    V3 T = sub(o, a);
    V3 e1 = sub(b, a);
    V3 e2 = sub(c, a);
    V3 p = cross(d, e2);
    V3 q = cross(T, e1);
    float mx = dot(q, e2), my = dot(p, T), mz = dot(q, d);
    float det = 1.0f / dot(p, e1);
    r.t = det * mx;
    r.u = det * my;
    r.v = det * mz;
    float w = 1.0f - r.u - r.v;
    float f = dot(d, n);
    r.hit = r.u >= 0.0f && r.u <= 1.0f && r.v >= 0.0f && r.v <= 1.0f && w >= 0.0f &&
            w <= 1.0f && f < 0.0f;
    return r;
}

// Watertight ray/triangle test (Woop, Benthin and Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013): the vertices are translated
// to the ray origin and sheared so the ray runs along +z, and the 2D edge
// functions U, V, W decide the hit; an edge function that rounds to exactly
// zero is recomputed in double precision, so a ray through a shared edge or
// vertex hits at least one of the triangles that share it.  Two-sided edge
// test, then the reference's face culling (dot(d, n) < 0 with the stored
// n = cross(b - a, c - a)); u, v are the weights of b and c, as in
// ray_triangle_mt.
GBSP_HD float axis_of(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

GBSP_HD TriHit ray_triangle_watertight(V3 o, V3 d, V3 a, V3 b, V3 c, V3 n)
{
    TriHit r;
    r.hit = false;
    r.t = r.u = r.v = 0.0f;
    float ax_ = fabsf(d.x), ay_ = fabsf(d.y), az_ = fabsf(d.z);
    int kz = ax_ > ay_ ? (ax_ > az_ ? 0 : 2) : (ay_ > az_ ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    float dz = axis_of(d, kz);
    if (dz < 0.0f) {
        int tmp = kx;
        kx = ky;
        ky = tmp;
    }
    float sx = axis_of(d, kx) / dz, sy = axis_of(d, ky) / dz, sz = 1.0f / dz;
    V3 A = sub(a, o), B = sub(b, o), C = sub(c, o);
    float Az = axis_of(A, kz), Bz = axis_of(B, kz), Cz = axis_of(C, kz);
    float Ax = axis_of(A, kx) - sx * Az, Ay = axis_of(A, ky) - sy * Az;
    float Bx = axis_of(B, kx) - sx * Bz, By = axis_of(B, ky) - sy * Bz;
    float Cx = axis_of(C, kx) - sx * Cz, Cy = axis_of(C, ky) - sy * Cz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return r;
    float det = U + V + W;
    if (det == 0.0f) return r;
    float T = (U * (sz * Az) + V * (sz * Bz)) + W * (sz * Cz);
    float inv = 1.0f / det;
    r.t = T * inv;
    r.u = V * inv;
    r.v = W * inv;
    r.hit = dot(d, n) < 0.0f;
    return r;
}

// ---------------------------------------------------------------------------
// Device scene layout
// ---------------------------------------------------------------------------
// BVH node of width 4 * Q children, Q = 2 (8-wide) or Q = 1 (4-wide, the
// reference's width, src/bvh.h:4-12): structure of arrays inside the node,
// 7 * Q float4 loaded with 128-bit loads.  Float4 number c * Q + q of a node
// holds component c of its children 4q .. 4q+3, with c = 0..5 the child
// boxes' lo.x, hi.x, lo.y, hi.y, lo.z, hi.z and c = 6 the child words:
//   < 0x80000000  internal node index (in nodes of the same width)
//   0xFFFFFFFF    empty slot
//   otherwise     leaf: bits 30..3 first primitive, bits 2..0 count - 1
// An 8-wide node is 224 bytes = 7 x 32 B sectors, a 4-wide node 112 bytes.
constexpr uint32_t kNodeComponents = 7;
constexpr uint32_t kMaxNodeQuads = 2;
GBSP_HD size_t node_offset(uint32_t ref, uint32_t quads)
{
    return (size_t)ref * kNodeComponents * quads;
}
// The 8-wide node as a struct (the same bytes as Q = 2 above).
struct __align__(16) Node8 {
    float lox[8], hix[8], loy[8], hiy[8], loz[8], hiz[8];
    uint32_t child[8];
};
static_assert(sizeof(Node8) == 224, "Node8 is 224 bytes");
constexpr uint32_t kEmptyChild = 0xFFFFFFFFu;
constexpr uint32_t kLeafFlag = 0x80000000u;
// Mesh leaves hold at most this many triangles (the leaf count field has 3
// bits).  Smaller leaves trade triangle tests for node visits: on the 1080p
// benchmark scene 2 gave 1.82 tests and 6.71 visits per ray and 1,468
// Msamples/s, 4 gave 2.42 / 6.45 and 1,427, 8 gave 4.73 / 5.94 and 1,336.
constexpr uint32_t kMaxLeafPrims = 2;
GBSP_HD bool child_is_leaf(uint32_t c) { return (c & kLeafFlag) != 0u; }
GBSP_HD uint32_t leaf_first(uint32_t c) { return (c & 0x7FFFFFFFu) >> 3; }
GBSP_HD uint32_t leaf_count(uint32_t c) { return (c & 7u) + 1u; }
GBSP_HD uint32_t make_leaf(uint32_t first, uint32_t count)
{
    return kLeafFlag | (first << 3) | (count - 1u);
}

// Triangle in leaf order: three float4 = vertex a, b, c with the face normal
// n = cross(b - a, c - a) in the w lanes (48 bytes).
struct __align__(16) TriRecord {
    float4 a_nx, b_ny, c_nz;
};

// Shading attributes of a triangle in leaf order: vertex normals and uvs.
struct __align__(16) TriAttr {
    float4 n0_n1x;   // n0.xyz, n1.x
    float4 n1yz_n2;  // n1.y, n1.z, n2.x, n2.y
    float4 n2z_uv0;  // n2.z, uv0.x, uv0.y, uv1.x
    float4 uv1y_uv2; // uv1.y, uv2.x, uv2.y, pad
};

// Objects are stored in object-BVH leaf order; objectIndex is the caller's
// index (order of add_object calls).
struct __align__(16) Instance {
    Affine inv;          // inverse model matrix rows
    Affine model;        // model matrix rows
    float lo[3], hi[3];  // world AABB (src/aabb.h:29-58)
    uint32_t blasRoot;   // node index of the mesh's root in the node pool
    uint32_t materialId; // the reference's material id (resolved per render)
    uint32_t objectIndex;
    uint32_t smooth;     // mesh uses interpolated vertex normals
};

// Resolved material (id lookup done at upload time, first match wins as in
// src/sp_material_system.cpp:15-28).
struct __align__(16) DeviceMaterial {
    float albedo[3];
    int32_t albedoTex;    // texture slot or -1
    float emission[3];
    int32_t emissionTex;  // texture slot, -1 none, -2 analytic sky
    float roughness;
    uint32_t present;     // 0 => missing material (magenta emission)
    uint32_t pad[2];
};

struct TextureDesc {
    uint64_t offset;  // in float4 texels
    uint32_t width, height;
};

struct SkyParams {
    V3 bottom, top, sunDir;
    float cosSunRadius;
    V3 sunRadiance;
};

// Everything a kernel needs to trace and shade against one scene.
struct SceneView {
    const float4 *nodes;         // node pool (all mesh BVHs + object BVH), nodeQuads wide
    uint32_t nodeQuads;          // 2: 8-wide nodes, 1: 4-wide nodes
    const TriRecord *tris;       // leaf-ordered triangles of all meshes
    const TriAttr *attrs;        // per triangle, same order
    const uint32_t *triIds;      // leaf order -> the mesh's own triangle index
    const Instance *instances;
    uint32_t tlasRoot;           // node index of the object BVH root, or kEmptyChild
    uint32_t instanceCount;
    uint32_t watertight;         // 1: ray_triangle_watertight, 0: the reference's MT
};

struct MaterialView {
    const int32_t *instanceSlot;  // per instance (leaf order): material slot or -1
    const DeviceMaterial *materials;
    uint32_t materialCount;
    const float4 *texels;
    const TextureDesc *textures;
    uint32_t textureCount;
    int32_t backgroundSlot;  // -1 = missing
    SkyParams sky;
    uint32_t haveSky;
};

// Kernel status bits (host turns them into GBSP_ERR_DEVICE_STATUS).
constexpr uint32_t kStatusStackOverflow = 1u;
constexpr uint32_t kStatusQueueOverflow = 2u;
constexpr uint32_t kStatusBadIndex = 4u;
constexpr uint32_t kStatusBuildLoop = 8u;
constexpr uint32_t kStatusRayStepLimit = 16u;  // a ray exceeded the per-ray step cap

}  // namespace gbsp
