// Oracle port: TEST INFRASTRUCTURE ONLY (see sp_oracle.h).
//
// A restatement of vk_cinematic's CPU path-tracing hot path.  Each function
// cites the reference file:line it follows.  Operation order inside every
// expression matches the reference's so that, compiled with
// -ffp-contract=off, results agree bit for bit with the reference's own
// code (only libm's sinf/cosf/powf/atan2f/sqrtf are shared).

#include "sp_oracle.h"
#include "sample_seed.h"

#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

const float kPi = 3.14159265359f;      // math_lib.h:6
const float kEpsilon = FLT_EPSILON;    // math_lib.h:7
const float kF32Max = FLT_MAX;
const uint32_t kNoTexture = 0xFFFFFFFFu;
const uint32_t kSkyTexture = 0xFFFFFFFEu;

// ---------------------------------------------------------------------------
// Scalar and vector arithmetic (math_utils.h, math_lib.h)
// ---------------------------------------------------------------------------
inline float fmin_ref(float a, float b) { return a < b ? a : b; }  // math_utils.h:5-9
inline float fmax_ref(float a, float b) { return a > b ? a : b; }  // math_utils.h:11-15
inline float clamp_ref(float x, float lo, float hi) { return fmin_ref(fmax_ref(x, lo), hi); }

struct F3
{
    float x, y, z;
};
struct F2
{
    float x, y;
};
struct F4
{
    float x, y, z, w;
};
struct M4
{
    float m[16];  // column-major, m[col*4 + row] (math_lib.h:93-97)
};

inline F3 f3(float x, float y, float z) { return F3{x, y, z}; }
inline F3 f3s(float s) { return F3{s, s, s}; }
inline F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline F3 operator-(F3 a) { return f3(-a.x, -a.y, -a.z); }
inline F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
inline F3 operator*(float s, F3 a) { return a * s; }
inline F3 hadamard(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }  // math_lib.h:461
inline F3 cross3(F3 a, F3 b)  // math_lib.h:467-477
{
    return f3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z),
        (a.x * b.y) - (a.y * b.x));
}
inline F3 normalize3(F3 v)  // math_lib.h:503-512
{
    float len = sqrtf(dot3(v, v));
    F3 r = {0, 0, 0};
    if (len > kEpsilon) r = v * (1.0f / len);
    return r;
}
inline F3 vmin3(F3 a, F3 b) { return f3(fmin_ref(a.x, b.x), fmin_ref(a.y, b.y), fmin_ref(a.z, b.z)); }
inline F3 vmax3(F3 a, F3 b) { return f3(fmax_ref(a.x, b.x), fmax_ref(a.y, b.y), fmax_ref(a.z, b.z)); }
inline float max_component(F3 a) { return fmax_ref(a.x, fmax_ref(a.y, a.z)); }  // math_lib.h:918
inline float min_component(F3 a) { return fmin_ref(a.x, fmin_ref(a.y, a.z)); }  // math_lib.h:924
inline F3 inverse3(F3 a) { return f3(1.0f / a.x, 1.0f / a.y, 1.0f / a.z); }     // math_lib.h:911
inline F3 clamp3(F3 v, float lo, float hi)
{
    return f3(clamp_ref(v.x, lo, hi), clamp_ref(v.y, lo, hi), clamp_ref(v.z, lo, hi));
}
inline F3 ld3(const float *p) { return f3(p[0], p[1], p[2]); }
inline void st3(float *o, F3 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }

inline float dot4(const float *a, const float *b)  // math_lib.h:238-247
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
}

M4 m4_identity()
{
    M4 r = {};
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
    return r;
}
M4 m4_scale(F3 s)  // math_lib.h:212-221
{
    M4 r = {};
    r.m[0] = s.x;
    r.m[5] = s.y;
    r.m[10] = s.z;
    r.m[15] = 1.0f;
    return r;
}
M4 m4_translate(F3 t)  // math_lib.h:228-236
{
    M4 r = m4_identity();
    r.m[12] = t.x;
    r.m[13] = t.y;
    r.m[14] = t.z;
    return r;
}
M4 m4_mul(const M4 &a, const M4 &b)  // math_lib.h:250-270
{
    M4 r = {};
    for (int i = 0; i < 4; i++)
    {
        float row[4] = {a.m[0 * 4 + i], a.m[1 * 4 + i], a.m[2 * 4 + i], a.m[3 * 4 + i]};
        for (int c = 0; c < 4; c++) r.m[c * 4 + i] = dot4(row, b.m + c * 4);
    }
    return r;
}
F4 m4_apply(const M4 &a, F4 v)  // math_lib.h:381-398
{
    float vv[4] = {v.x, v.y, v.z, v.w};
    float out[4];
    for (int i = 0; i < 4; i++)
    {
        float row[4] = {a.m[0 * 4 + i], a.m[1 * 4 + i], a.m[2 * 4 + i], a.m[3 * 4 + i]};
        out[i] = dot4(row, vv);
    }
    return F4{out[0], out[1], out[2], out[3]};
}
F3 transform_point(F3 p, const M4 &m)  // math_lib.h:754-758
{
    F4 v = m4_apply(m, F4{p.x, p.y, p.z, 1.0f});
    return f3(v.x, v.y, v.z);
}
F3 transform_vector(F3 d, const M4 &m)  // math_lib.h:748-752
{
    F4 v = m4_apply(m, F4{d.x, d.y, d.z, 0.0f});
    return f3(v.x, v.y, v.z);
}

// Quaternions (math_lib.h:556-623): x, y, z = vector part, w = scalar part
F4 quat_mul(F4 p, F4 q)  // math_lib.h:565-571
{
    F3 pv = f3(p.x, p.y, p.z), qv = f3(q.x, q.y, q.z);
    F3 v = p.w * qv + q.w * pv + cross3(pv, qv);
    float s = p.w * q.w - dot3(pv, qv);
    return F4{v.x, v.y, v.z, s};
}
F4 quat_conj(F4 p) { return F4{-p.x, -p.y, -p.z, p.w}; }
F3 rotate_vector(F3 v, F4 p)  // math_lib.h:588-593
{
    F4 q = {v.x, v.y, v.z, 0.0f};
    F4 r = quat_mul(quat_mul(p, q), quat_conj(p));
    return f3(r.x, r.y, r.z);
}
M4 m4_rotate(F4 q)  // math_lib.h:602-623
{
    M4 r = m4_identity();
    float x = q.x, y = q.y, z = q.z, w = q.w;
    r.m[0] = 1.0f - 2.0f * y * y - 2.0f * z * z;
    r.m[1] = 2.0f * x * y + 2.0f * z * w;
    r.m[2] = 2.0f * x * z - 2.0f * y * w;
    r.m[4] = 2.0f * x * y - 2.0f * z * w;
    r.m[5] = 1.0f - 2.0f * x * x - 2.0f * z * z;
    r.m[6] = 2.0f * y * z + 2.0f * x * w;
    r.m[8] = 2.0f * x * z + 2.0f * y * w;
    r.m[9] = 2.0f * y * z - 2.0f * x * w;
    r.m[10] = 1.0f - 2.0f * x * x - 2.0f * y * y;
    return r;
}
inline F4 ld4(const float *p) { return F4{p[0], p[1], p[2], p[3]}; }

// ---------------------------------------------------------------------------
// RNG (math_utils.h:184-214)
// ---------------------------------------------------------------------------
inline uint32_t xorshift32(uint32_t *s)
{
    uint32_t x = *s;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    *s = x;
    return x;
}
inline float random_unilateral(uint32_t *s)
{
    float num = (float)(xorshift32(s) >> 1);
    float den = (float)(0xFFFFFFFFu >> 1);
    return num / den;
}
inline float random_bilateral(uint32_t *s) { return -1.0f + 2.0f * random_unilateral(s); }

// math_lib.h:932-959 with MapSphericalToCartesianCoordinates (:864-871)
F3 random_hemisphere(F3 normal, uint32_t *s)
{
    float theta = kPi * random_unilateral(s);
    float phi = kPi * random_bilateral(s);
    F3 dir;
    dir.x = sinf(theta) * cosf(phi);
    dir.z = sinf(theta) * sinf(phi);
    dir.y = cosf(theta);
    if (dot3(dir, normal) < 0.0f) dir = -dir;
    return dir;
}

// ---------------------------------------------------------------------------
// Camera (simd_path_tracer.cpp:1-63)
// ---------------------------------------------------------------------------
struct Camera
{
    F3 right, up, forward, position, filmCenter;
    float halfPixelWidth, halfPixelHeight, halfFilmWidth, halfFilmHeight;
    uint32_t width, height;
};

Camera configure_camera(uint32_t width, uint32_t height, F3 pos, F4 rot,
    float filmDistance)
{
    Camera c = {};
    c.width = width;
    c.height = height;
    c.position = pos;
    c.right = rotate_vector(f3(1, 0, 0), rot);
    c.up = rotate_vector(f3(0, 1, 0), rot);
    c.forward = rotate_vector(f3(0, 0, -1), rot);
    c.filmCenter = pos + c.forward * filmDistance;
    c.halfPixelWidth = 0.5f / (float)width;
    c.halfPixelHeight = 0.5f / (float)height;
    float fw = 1.0f, fh = 1.0f;
    if (width > height)
        fh = (float)height / (float)width;
    else if (width < height)
        fw = (float)width / (float)height;
    c.halfFilmWidth = 0.5f * fw;
    c.halfFilmHeight = 0.5f * fh;
    return c;
}

F3 film_position(const Camera &c, F2 p)  // simd_path_tracer.cpp:38-63
{
    float fx = p.x / (float)c.width;
    float fy = p.y / (float)c.height;
    fy = 1.0f - fy;
    fx = fx * 2.0f - 1.0f;
    fy = fy * 2.0f - 1.0f;
    F3 r = (c.halfFilmWidth * fx) * c.right;
    r = r + (c.halfFilmHeight * fy) * c.up;
    r = r + c.filmCenter;
    return r;
}

// ---------------------------------------------------------------------------
// Intersection primitives
// ---------------------------------------------------------------------------
struct TriHit
{
    float t;
    F2 uv;
    F3 normal;
};

// ray_intersection.cpp:156-190 (Moller-Trumbore, back-face culled)
TriHit ray_triangle_mt(F3 o, F3 d, F3 a, F3 b, F3 c)
{
    TriHit r = {};
    r.t = -1.0f;
    F3 T = o - a;
    F3 e1 = b - a;
    F3 e2 = c - a;
    F3 p = cross3(d, e2);
    F3 q = cross3(T, e1);
    F3 n = cross3(e1, e2);
    float mx = dot3(q, e2), my = dot3(p, T), mz = dot3(q, d);
    float det = 1.0f / dot3(p, e1);
    float t = det * mx;
    float u = det * my;
    float v = det * mz;
    float w = 1.0f - u - v;
    float f = dot3(d, n);
    if (u >= 0.0f && u <= 1.0f && v >= 0.0f && v <= 1.0f && w >= 0.0f &&
        w <= 1.0f && f < 0.0f)
    {
        r.t = t;
        r.normal = n;
        r.uv = F2{u, v};
    }
    return r;
}

// Watertight test of Woop, Benthin and Wald (JCGT 2013), restated for the
// optional intersection mode (no reference counterpart): translate to the ray
// origin, shear so the ray runs along +z (kz = largest |d| component, x / y
// swapped when d[kz] < 0 to keep the winding), 2D edge functions U, V, W with
// a double-precision recompute when one rounds to exactly zero, two-sided
// edge test, then the same face culling as ray_triangle_mt; uv = weights of
// b and c.
TriHit ray_triangle_watertight(F3 o, F3 d, F3 a, F3 b, F3 c)
{
    TriHit r = {};
    r.t = -1.0f;
    const float dv[3] = {d.x, d.y, d.z};
    float mx_ = std::fabs(d.x), my_ = std::fabs(d.y), mz_ = std::fabs(d.z);
    int kz = mx_ > my_ ? (mx_ > mz_ ? 0 : 2) : (my_ > mz_ ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (dv[kz] < 0.0f) std::swap(kx, ky);
    float sx = dv[kx] / dv[kz], sy = dv[ky] / dv[kz], sz = 1.0f / dv[kz];
    F3 A3 = a - o, B3 = b - o, C3 = c - o;
    const float A[3] = {A3.x, A3.y, A3.z}, B[3] = {B3.x, B3.y, B3.z}, C[3] = {C3.x, C3.y, C3.z};
    float ax = A[kx] - sx * A[kz], ay = A[ky] - sy * A[kz];
    float bx = B[kx] - sx * B[kz], by = B[ky] - sy * B[kz];
    float cx = C[kx] - sx * C[kz], cy = C[ky] - sy * C[kz];
    float U = cx * by - cy * bx, V = ax * cy - ay * cx, W = bx * ay - by * ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f)
    {
        U = (float)((double)cx * (double)by - (double)cy * (double)bx);
        V = (float)((double)ax * (double)cy - (double)ay * (double)cx);
        W = (float)((double)bx * (double)ay - (double)by * (double)ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return r;
    float det = U + V + W;
    if (det == 0.0f) return r;
    float T = (U * (sz * A[kz]) + V * (sz * B[kz])) + W * (sz * C[kz]);
    float inv = 1.0f / det;
    F3 n = cross3(b - a, c - a);
    if (!(dot3(d, n) < 0.0f)) return r;
    r.t = T * inv;
    r.uv = F2{V * inv, W * inv};
    r.normal = n;
    return r;
}

// simd.h:198-271: 4-box slab test; hit iff max(0, max(tmin)) <= min(tmax)
inline bool slab_hit(F3 bmin, F3 bmax, F3 o, F3 invd)
{
    float t0x = (bmin.x - o.x) * invd.x, t1x = (bmax.x - o.x) * invd.x;
    float t0y = (bmin.y - o.y) * invd.y, t1y = (bmax.y - o.y) * invd.y;
    float t0z = (bmin.z - o.z) * invd.z, t1z = (bmax.z - o.z) * invd.z;
    // _mm_min_ps(a, b) = a < b ? a : b, _mm_max_ps(a, b) = a > b ? a : b
    F3 tmin = f3(t0x < t1x ? t0x : t1x, t0y < t1y ? t0y : t1y, t0z < t1z ? t0z : t1z);
    F3 tmax = f3(t0x > t1x ? t0x : t1x, t0y > t1y ? t0y : t1y, t0z > t1z ? t0z : t1z);
    return fmax_ref(0.0f, max_component(tmin)) <= min_component(tmax);
}

uint32_t aabb4(const F3 *bmin, const F3 *bmax, F3 o, F3 invd)
{
    uint32_t mask = 0;
    for (int i = 0; i < 4; i++)
        if (slab_hit(bmin[i], bmax[i], o, invd)) mask |= 1u << i;
    return mask;
}

// aabb.h:29-58 (corner order kept; the min/max fold is order dependent for -0)
void transform_aabb(F3 bmin, F3 bmax, F3 pos, F4 rot, F3 scale, F3 *omin, F3 *omax)
{
    M4 model = m4_mul(m4_mul(m4_translate(pos), m4_rotate(rot)), m4_scale(scale));
    F3 v[8] = {f3(bmin.x, bmin.y, bmin.z), f3(bmax.x, bmin.y, bmin.z),
        f3(bmax.x, bmin.y, bmax.z), f3(bmin.x, bmin.y, bmax.z),
        f3(bmin.x, bmax.y, bmin.z), f3(bmax.x, bmax.y, bmin.z),
        f3(bmax.x, bmax.y, bmax.z), f3(bmin.x, bmax.y, bmax.z)};
    F3 lo = transform_point(v[0], model), hi = lo;
    for (int i = 1; i < 8; i++)
    {
        F3 t = transform_point(v[i], model);
        lo = vmin3(lo, t);
        hi = vmax3(hi, t);
    }
    *omin = lo;
    *omax = hi;
}

// ---------------------------------------------------------------------------
// BVH: agglomerative 4-ary build and all-hits query (bvh.cpp)
// ---------------------------------------------------------------------------
struct BvhNode
{
    F3 min, max;
    int32_t child[4];  // -1 = none
    uint32_t leafIndex;
};

struct BvhTree
{
    std::vector<BvhNode> nodes;
    int32_t root = -1;
};

// bvh.cpp:37-60: the sort payload has the reference's 16-byte layout so the
// C library's qsort makes exactly the same moves.
struct DistPair
{
    float distSq;
    uint32_t pad;
    uint64_t node;
};
static_assert(sizeof(DistPair) == 16, "DistPair must match bvh_NodeDistSqPair");

int compare_dist_desc(const void *p1, const void *p2)
{
    DistPair a = *(const DistPair *)p1;
    DistPair b = *(const DistPair *)p2;
    if (a.distSq < b.distSq) return 1;
    if (a.distSq > b.distSq) return -1;
    return 0;
}

// bvh.cpp:51-200
BvhTree bvh_build(const F3 *mins, const F3 *maxs, uint32_t count)
{
    BvhTree tree;
    if (count == 0) return tree;
    tree.nodes.reserve((size_t)count * 2);
    std::vector<DistPair> buf[2];
    buf[0].resize(count);
    buf[1].resize(count);
    uint32_t n[2] = {count, 0};
    int rd = 0, wr = 1;
    for (uint32_t i = 0; i < count; i++)
    {
        BvhNode node = {mins[i], maxs[i], {-1, -1, -1, -1}, i};
        tree.nodes.push_back(node);
        buf[rd][i].node = i;
        buf[rd][i].distSq = 0.0f;
        buf[rd][i].pad = 0;
    }
    int32_t last = (int32_t)buf[rd][0].node;
    for (uint32_t depth = 0; depth < 256; depth++)
    {
        n[wr] = 0;
        while (n[rd] > 0)
        {
            uint32_t index = n[rd] - 1;
            int32_t cur = (int32_t)buf[rd][index].node;
            F3 centroid = (tree.nodes[cur].max + tree.nodes[cur].min) * 0.5f;
            uint32_t sortCount = n[rd] - 1;
            for (uint32_t i = 0; i < sortCount; i++)  // bvh.cpp:62-75
            {
                const BvhNode &o = tree.nodes[buf[rd][i].node];
                F3 c = (o.max + o.min) * 0.5f;
                F3 d = c - centroid;
                buf[rd][i].distSq = dot3(d, d);
            }
            qsort(buf[rd].data(), sortCount, sizeof(DistPair), compare_dist_desc);
            uint32_t nb = sortCount < 3 ? sortCount : 3;
            if (nb > 0)
            {
                BvhNode parent = {tree.nodes[cur].min, tree.nodes[cur].max,
                    {cur, -1, -1, -1}, 0xFFFFFFFFu};
                for (uint32_t i = 0; i < nb; i++)
                {
                    int32_t nbIdx = (int32_t)buf[rd][index - (i + 1)].node;
                    parent.min = vmin3(parent.min, tree.nodes[nbIdx].min);
                    parent.max = vmax3(parent.max, tree.nodes[nbIdx].max);
                    parent.child[i + 1] = nbIdx;
                }
                tree.nodes.push_back(parent);
                last = (int32_t)tree.nodes.size() - 1;
                buf[wr][n[wr]].node = (uint64_t)last;
                n[wr]++;
                n[rd] -= nb + 1;
            }
            else
            {
                buf[wr][n[wr]].node = (uint64_t)cur;
                n[wr]++;
                n[rd]--;
            }
        }
        if (n[wr] > 1)
        {
            int t = rd;
            rd = wr;
            wr = t;
        }
        else
        {
            break;
        }
    }
    tree.root = last;
    return tree;
}

struct BvhQuery
{
    bool error;
    uint32_t count;
    uint32_t aabbTests;
};

// bvh.cpp:203-311 (SIMD box path, USE_BVH_SIMD_RAY_INTERSECT_AABB = 1)
BvhQuery bvh_query(const BvhTree &tree, F3 o, F3 d, uint32_t *leaves,
    uint32_t maxHits, std::vector<int32_t> *stackA, std::vector<int32_t> *stackB)
{
    BvhQuery r = {false, 0, 0};
    std::vector<int32_t> *stk[2] = {stackA, stackB};
    stk[0]->clear();
    stk[1]->clear();
    int rd = 0, wr = 1;
    F3 invd = inverse3(d);
    if (tree.root >= 0)
    {
        const BvhNode &root = tree.nodes[tree.root];
        if (slab_hit(root.min, root.max, o, invd)) stk[0]->push_back(tree.root);
    }
    while (!stk[rd]->empty())
    {
        int32_t ni = stk[rd]->back();
        stk[rd]->pop_back();
        const BvhNode &node = tree.nodes[ni];
        if (node.child[0] >= 0)
        {
            uint32_t childCount = 0;
            for (int i = 0; i < 4; i++)
                if (node.child[i] >= 0) childCount++;
            r.aabbTests += childCount;
            for (uint32_t i = 0; i < childCount; i++)
            {
                const BvhNode &c = tree.nodes[node.child[i]];
                if (slab_hit(c.min, c.max, o, invd)) stk[wr]->push_back(node.child[i]);
            }
        }
        else
        {
            if (r.count < maxHits)
            {
                leaves[r.count++] = node.leafIndex;
            }
            else
            {
                r.error = true;
                break;
            }
        }
        if (stk[rd]->empty())
        {
            int t = rd;
            rd = wr;
            wr = t;
        }
    }
    return r;
}

// ---------------------------------------------------------------------------
// Materials (sp_material_system.cpp, image.h)
// ---------------------------------------------------------------------------
struct Material
{
    F3 albedo;
    uint32_t albedoTexture;
    F3 emission;
    uint32_t emissionTexture;
    float roughness;
};
static_assert(sizeof(Material) == 36, "Material must match sp_Material");

struct Texture
{
    std::vector<float> rgba;  // one spare row: the reference may read index W*H
    uint32_t width, height;
};

struct Sky
{
    F3 bottom, top, sunDir;
    float cosSunRadius;
    F3 sunRadiance;
};

struct PathVertex  // sp_material_system.h:22-30
{
    uint32_t materialId;
    F3 worldPosition;
    F3 outgoingDir;
    F3 incomingDir;
    F3 normal;
    F2 uv;
};
static_assert(sizeof(PathVertex) == 60, "PathVertex must match sp_PathVertex");

// image.h:3-18: x = floor(u*W), y = floor(v*H), no clamp (x == W allowed)
F3 sample_nearest(const Texture &t, F2 uv)
{
    float fx = uv.x * t.width;
    float fy = uv.y * t.height;
    uint32_t x = (uint32_t)floorf(fx);
    uint32_t y = (uint32_t)floorf(fy);
    size_t idx = (size_t)y * t.width + x;
    size_t maxIdx = (size_t)t.width * (t.height + 1) - 1;
    if (idx > maxIdx) idx = maxIdx;
    const float *p = t.rgba.data() + 4 * idx;
    return f3(p[0], p[1], p[2]);
}

// Analytic sky: linear vertical gradient plus a sun disc.
F3 sky_radiance(const Sky &s, F3 dir)
{
    float t = clamp_ref(0.5f * (dir.y + 1.0f), 0.0f, 1.0f);
    F3 c = s.bottom + (s.top - s.bottom) * t;
    if (dot3(dir, s.sunDir) >= s.cosSunRadius) c = c + s.sunRadiance;
    return c;
}

// ---------------------------------------------------------------------------
// World
// ---------------------------------------------------------------------------
struct Mesh
{
    std::vector<F3> pos;
    std::vector<F3> nrm;
    std::vector<F2> uv;
    std::vector<uint32_t> idx;
    bool smooth;
    BvhTree tree;
    F3 aabbMin, aabbMax;  // sp_scene.cpp:57-75 (vertex AABB)
};

struct Object
{
    int mesh;
    uint32_t material;
    M4 model, invModel;
    F3 aabbMin, aabbMax;
};

struct World
{
    std::vector<Mesh> meshes;
    std::vector<Object> objects;
    BvhTree broadphase;
    std::vector<uint32_t> materialKeys;
    std::vector<Material> materials;
    std::vector<uint32_t> textureKeys;
    std::vector<Texture> textures;
    uint32_t backgroundMaterialId = 0;
    Sky sky = {};
    bool haveSky = false;
    oracle_options opt = {1, 3, 10.0f, 32, 128};
    bool buildMeshBvh = true;  // false: meshes are only queried by brute force
    bool watertight = false;   // brute-force queries use ray_triangle_watertight
};

const Material *find_material(const World &w, uint32_t id)  // sp_material_system.cpp:15-28
{
    for (size_t i = 0; i < w.materialKeys.size(); i++)
        if (w.materialKeys[i] == id) return &w.materials[i];
    return nullptr;
}
const Texture *find_texture(const World &w, uint32_t id)  // sp_material_system.cpp:30-43
{
    for (size_t i = 0; i < w.textureKeys.size(); i++)
        if (w.textureKeys[i] == id) return &w.textures[i];
    return nullptr;
}

struct MaterialOut
{
    F3 albedo, emission;
    float roughness;
};

// sp_material_system.cpp:59-105
MaterialOut evaluate_material(const World &w, const Material &m, const PathVertex &v)
{
    MaterialOut o = {};
    const Texture *at = find_texture(w, m.albedoTexture);
    const Texture *et = find_texture(w, m.emissionTexture);
    o.albedo = at ? sample_nearest(*at, v.uv) : m.albedo;
    if (m.emissionTexture == kSkyTexture && w.haveSky && !et)
    {
        o.emission = sky_radiance(w.sky, -v.outgoingDir);
    }
    else if (et)
    {
        F3 dir = -v.outgoingDir;  // math_lib.h:849-884
        float inc = atan2f(sqrtf(dir.x * dir.x + dir.z * dir.z), dir.y);
        float az = atan2f(dir.z, dir.x);
        if (az < 0.0f) az += 2.0f * kPi;
        F2 uv = {az / (2.0f * kPi), cosf(inc) * 0.5f + 0.5f};
        uv.y = 1.0f - uv.y;
        o.emission = sample_nearest(*et, uv) * 1.0f;
    }
    else
    {
        o.emission = m.emission;
    }
    o.roughness = m.roughness;
    return o;
}

// simd_path_tracer.cpp:65-105
F3 fresnel_schlick(float cosTheta, F3 F0)
{
    return F0 + (f3s(1.0f) - F0) * powf(1.0f - cosTheta, 5.0f);
}
float distribution_ggx(F3 N, F3 H, float roughness)
{
    float a = roughness * roughness;
    float a2 = a * a;
    float NdotH = fmax_ref(dot3(N, H), 0.0f);
    float NdotH2 = NdotH * NdotH;
    float num = a2;
    float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
    denom = kPi * denom * denom;
    return num / denom;
}
float geometry_schlick_ggx(float NdotV, float roughness)
{
    float r = (roughness + 1.0f);
    float k = (r * r) / 8.0f;
    float num = NdotV;
    float denom = NdotV * (1.0f - k) + k;
    return num / denom;
}
float geometry_smith(F3 N, F3 V, F3 L, float roughness)
{
    float NdotV = fmax_ref(dot3(N, V), 0.0f);
    float NdotL = fmax_ref(dot3(N, L), 0.0f);
    return geometry_schlick_ggx(NdotL, roughness) * geometry_schlick_ggx(NdotV, roughness);
}

// simd_path_tracer.cpp:107-175
F3 radiance_for_path(const World &w, const PathVertex *path, uint32_t len)
{
    F3 radiance = {0, 0, 0};
    for (int32_t i = (int32_t)len - 1; i >= 0; i--)
    {
        const PathVertex &v = path[i];
        MaterialOut mo = {};
        const Material *m = find_material(w, v.materialId);
        if (m)
            mo = evaluate_material(w, *m, v);
        else
            mo.emission = f3(1, 0, 1);
        float cosine = fmax_ref(0.0f, dot3(v.normal, v.incomingDir));
        F3 Li = radiance;
        if (w.opt.radiance_clamp != 0.0f) Li = clamp3(Li, 0.0f, w.opt.radiance_clamp);
        F3 L = v.incomingDir, N = v.normal, V = v.outgoingDir;
        F3 H = normalize3(L + V);
        F3 F = fresnel_schlick(fmax_ref(dot3(H, V), 0.0f), f3s(0.04f));
        F3 kD = f3s(1.0f) - F;
        float oneOverPi = 1.0f / kPi;
        float NDF = distribution_ggx(N, H, mo.roughness);
        float G = geometry_smith(N, V, L, mo.roughness);
        F3 numerator = NDF * G * F;
        float denominator = 4.0f * fmax_ref(dot3(N, V), 0.0f) * fmax_ref(dot3(N, L), 0.0f) + 0.0001f;
        F3 specular = numerator * (1.0f / denominator);
        radiance = mo.emission +
                   hadamard(hadamard(kD, mo.albedo) * oneOverPi + specular, Li) * cosine;
    }
    return radiance;
}

// ---------------------------------------------------------------------------
// Scene queries (sp_scene.cpp:127-339)
// ---------------------------------------------------------------------------
struct QueryScratch
{
    std::vector<uint32_t> leaves;
    std::vector<int32_t> stackA, stackB;
    std::vector<uint32_t> objects;
};

struct MeshHit
{
    TriHit hit;
    int32_t triangle;
    // another candidate of this mesh hit at exactly hit.t (the reference's
    // strict '<' keeps the first one found, so the winner is order-dependent)
    bool tied;
};

// sp_scene.cpp:127-227; returns -100 style errors through ok=false
MeshHit intersect_mesh(const World &w, const Mesh &mesh, F3 o, F3 d,
    QueryScratch &s, uint64_t *metrics, bool *ok)
{
    MeshHit best = {};
    best.hit.t = -1.0f;
    best.triangle = -1;
    best.tied = false;
    s.leaves.resize(w.opt.max_midphase);
    BvhQuery q = bvh_query(mesh.tree, o, d, s.leaves.data(), w.opt.max_midphase,
        &s.stackA, &s.stackB);
    if (metrics) metrics[10] += q.aabbTests;
    if (q.error) *ok = false;
    for (uint32_t i = 0; i < q.count; i++)
    {
        uint32_t tri = s.leaves[i];
        uint32_t i0 = mesh.idx[tri * 3 + 0], i1 = mesh.idx[tri * 3 + 1], i2 = mesh.idx[tri * 3 + 2];
        TriHit h = ray_triangle_mt(o, d, mesh.pos[i0], mesh.pos[i1], mesh.pos[i2]);
        if (h.t > 0.0f)
        {
            if (h.t == best.hit.t) best.tied = true;
            if (h.t < best.hit.t || best.hit.t < 0.0f)
            {
                best.hit = h;
                best.triangle = (int32_t)tri;
                best.tied = false;
                float wgt = 1.0f - h.uv.x - h.uv.y;
                F2 uv;
                uv.x = mesh.uv[i0].x * wgt + mesh.uv[i1].x * h.uv.x + mesh.uv[i2].x * h.uv.y;
                uv.y = mesh.uv[i0].y * wgt + mesh.uv[i1].y * h.uv.x + mesh.uv[i2].y * h.uv.y;
                if (mesh.smooth)
                {
                    F3 n = mesh.nrm[i0] * wgt + mesh.nrm[i1] * h.uv.x + mesh.nrm[i2] * h.uv.y;
                    best.hit.normal = normalize3(n);
                }
                best.hit.uv = uv;
            }
        }
    }
    return best;
}

struct SceneHit
{
    float t;
    uint32_t materialId;
    F3 normal;
    F2 uv;
    int32_t object, triangle;
    // the best t is an exact tie: two objects at the same world t, or two
    // triangles of the winning object at the same object-space t
    bool tied;
};

// sp_scene.cpp:229-339
SceneHit intersect_scene(const World &w, F3 o, F3 d, QueryScratch &s,
    uint64_t *metrics, bool *ok)
{
    SceneHit r = {};
    r.t = -1.0f;
    r.object = -1;
    r.triangle = -1;
    r.tied = false;
    s.objects.resize(w.opt.max_broadphase);
    BvhQuery q = bvh_query(w.broadphase, o, d, s.objects.data(), w.opt.max_broadphase,
        &s.stackA, &s.stackB);
    if (q.error) *ok = false;
    for (uint32_t i = 0; i < q.count; i++)
    {
        uint32_t oi = s.objects[i];
        const Object &obj = w.objects[oi];
        F3 lo = transform_point(o, obj.invModel);
        F3 ld = normalize3(transform_vector(d, obj.invModel));
        MeshHit mh = intersect_mesh(w, w.meshes[obj.mesh], lo, ld, s, metrics, ok);
        if (metrics) metrics[11]++;
        if (mh.hit.t >= 0.0f)
        {
            F3 localHit = lo + ld * mh.hit.t;
            F3 worldHit = transform_point(localHit, obj.model);
            float t = dot3(worldHit - o, d);
            F3 wn = normalize3(transform_vector(mh.hit.normal, obj.model));
            if (r.t >= 0.0f && t == r.t) r.tied = true;
            if (t < r.t || r.t < 0.0f)
            {
                r.tied = mh.tied;
                r.t = t;
                r.materialId = obj.material;
                r.normal = wn;
                r.uv = mh.hit.uv;
                r.object = (int32_t)oi;
                r.triangle = mh.triangle;
            }
        }
    }
    return r;
}

// ---------------------------------------------------------------------------
// Path tracing (simd_path_tracer.cpp:178-345)
// ---------------------------------------------------------------------------
// One path; draws from *rng exactly as the reference loop body does.
F3 trace_path(const World &w, const Camera &cam, uint32_t x, uint32_t y,
    uint32_t *rng, QueryScratch &s, std::vector<PathVertex> &path,
    uint64_t *metrics, bool *ok)
{
    // simd_path_tracer.cpp:219-222.  The two jitter draws are arguments of
    // one Vec2 call; GCC evaluates them right to left, so the y jitter takes
    // the first draw.
    float jy = cam.halfPixelHeight * random_bilateral(rng);
    float jx = cam.halfPixelWidth * random_bilateral(rng);
    F2 pp = {(float)x + 0.5f, (float)y + 0.5f};
    pp.x = pp.x + jx;
    pp.y = pp.y + jy;
    F3 filmP = film_position(cam, pp);
    F3 ro = cam.position;
    F3 rd = normalize3(filmP - cam.position);
    uint32_t len = 0;
    path.assign(w.opt.max_bounces + 1, PathVertex{});
    for (uint32_t b = 0; b < w.opt.max_bounces; b++)
    {
        SceneHit h = intersect_scene(w, ro, rd, s, metrics, ok);
        if (metrics) metrics[2]++;
        PathVertex &v = path[len++];
        if (h.t > 0.0f)
        {
            v.materialId = h.materialId;
            v.worldPosition = ro + rd * h.t;
            v.outgoingDir = -rd;
            v.normal = h.normal;
            v.uv = h.uv;
            F3 dir = random_hemisphere(h.normal, rng);
            v.incomingDir = dir;
            float bias = 0.0001f;
            ro = v.worldPosition + h.normal * bias;
            rd = dir;
            if (metrics) metrics[3]++;
        }
        else
        {
            v.materialId = w.backgroundMaterialId;
            v.outgoingDir = -rd;
            if (metrics) metrics[4]++;
            break;
        }
    }
    F3 r = radiance_for_path(w, path.data(), len);
    if (metrics) metrics[1]++;
    return r;
}

void path_trace_tile(const World &w, const Camera &cam, const uint32_t *tile,
    uint32_t *rng, float *pixels, uint64_t *metrics, bool *ok)
{
    QueryScratch s;
    std::vector<PathVertex> path;
    uint32_t maxX = tile[2] < cam.width ? tile[2] : cam.width;
    uint32_t maxY = tile[3] < cam.height ? tile[3] : cam.height;
    uint32_t spp = w.opt.spp;
    for (uint32_t y = tile[1]; y < maxY; y++)
    {
        for (uint32_t x = tile[0]; x < maxX; x++)
        {
            F3 total = {0, 0, 0};
            for (uint32_t smp = 0; smp < spp; smp++)
            {
                F3 r = trace_path(w, cam, x, y, rng, s, path, metrics, ok);
                total = total + r * (1.0f / (float)spp);
            }
            float *o = pixels + 4 * ((size_t)x + (size_t)y * cam.width);
            o[0] = total.x;
            o[1] = total.y;
            o[2] = total.z;
            o[3] = 1.0f;
        }
    }
}

// Hash-per-sample pixel: Neumaier-summed radiance * (1/spp) over samples.
void hashed_pixel(const World &w, const Camera &cam, uint32_t x, uint32_t y,
    uint32_t seed, int nanPolicy, QueryScratch &s, std::vector<PathVertex> &path,
    float *o, uint32_t *nans, uint64_t *metrics, float *perSample, bool *ok)
{
    uint32_t spp = w.opt.spp;
    float invSpp = 1.0f / (float)spp;
    OracleSum acc[3] = {};
    for (uint32_t smp = 0; smp < spp; smp++)
    {
        uint32_t rng = oracle_sample_seed(seed, x, y, smp);
        F3 r = trace_path(w, cam, x, y, &rng, s, path, metrics, ok);
        if (perSample) st3(perSample + 3 * smp, r);
        if (std::isnan(r.x) || std::isnan(r.y) || std::isnan(r.z))
        {
            (*nans)++;
            if (nanPolicy == 0) continue;
        }
        oracle_sum_add(&acc[0], r.x * invSpp);
        oracle_sum_add(&acc[1], r.y * invSpp);
        oracle_sum_add(&acc[2], r.z * invSpp);
    }
    o[0] = oracle_sum_value(&acc[0]);
    o[1] = oracle_sum_value(&acc[1]);
    o[2] = oracle_sum_value(&acc[2]);
    o[3] = 1.0f;
}

double now_seconds()
{
    return std::chrono::duration<double>(
        std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// ===========================================================================
// extern "C" surface
// ===========================================================================
extern "C" {

uint32_t oracle_xorshift32(uint32_t *state) { return xorshift32(state); }
float oracle_random_unilateral(uint32_t *state) { return random_unilateral(state); }
float oracle_random_bilateral(uint32_t *state) { return random_bilateral(state); }
uint32_t oracle_sample_seed_c(uint32_t seed, uint32_t x, uint32_t y, uint32_t s)
{
    return oracle_sample_seed(seed, x, y, s);
}

void oracle_configure_camera(uint32_t width, uint32_t height, const float *pos,
    const float *rot, float filmDistance, float *out)
{
    Camera c = configure_camera(width, height, ld3(pos), ld4(rot), filmDistance);
    st3(out + 0, c.right);
    st3(out + 3, c.up);
    st3(out + 6, c.forward);
    st3(out + 9, c.position);
    st3(out + 12, c.filmCenter);
    out[15] = c.halfPixelWidth;
    out[16] = c.halfPixelHeight;
    out[17] = c.halfFilmWidth;
    out[18] = c.halfFilmHeight;
}

void oracle_film_positions(uint32_t width, uint32_t height, const float *pos,
    const float *rot, float filmDistance, uint32_t count, const float *pixel,
    float *out)
{
    Camera c = configure_camera(width, height, ld3(pos), ld4(rot), filmDistance);
    for (uint32_t i = 0; i < count; i++)
        st3(out + 3 * i, film_position(c, F2{pixel[2 * i], pixel[2 * i + 1]}));
}

void oracle_ray_triangle_mt(const float *o, const float *d, const float *a,
    const float *b, const float *c, float *out)
{
    TriHit h = ray_triangle_mt(ld3(o), ld3(d), ld3(a), ld3(b), ld3(c));
    out[0] = h.t;
    st3(out + 1, h.normal);
    out[4] = h.uv.x;
    out[5] = h.uv.y;
}

uint32_t oracle_aabb4(const float *mins, const float *maxs, const float *o,
    const float *invd)
{
    F3 bmin[4], bmax[4];
    for (int i = 0; i < 4; i++)
    {
        bmin[i] = ld3(mins + 3 * i);
        bmax[i] = ld3(maxs + 3 * i);
    }
    return aabb4(bmin, bmax, ld3(o), ld3(invd));
}

void oracle_hemisphere(uint32_t *state, const float *normal, float *out)
{
    st3(out, random_hemisphere(ld3(normal), state));
}

void oracle_transform_aabb(const float *bmin, const float *bmax,
    const float *pos, const float *rot, const float *scale, float *out)
{
    F3 lo, hi;
    transform_aabb(ld3(bmin), ld3(bmax), ld3(pos), ld4(rot), ld3(scale), &lo, &hi);
    st3(out, lo);
    st3(out + 3, hi);
}

void oracle_object_matrices(const float *pos, const float *rot,
    const float *scale, float *out)
{
    F3 p = ld3(pos), s = ld3(scale);
    F4 q = ld4(rot);
    M4 model = m4_mul(m4_mul(m4_translate(p), m4_rotate(q)), m4_scale(s));
    M4 inv = m4_mul(m4_mul(m4_scale(inverse3(s)), m4_rotate(quat_conj(q))), m4_translate(-p));
    memcpy(out, model.m, 64);
    memcpy(out + 16, inv.m, 64);
}

int oracle_bvh_build_flat(const float *mins, const float *maxs, uint32_t count,
    float *outNodes, uint32_t maxNodes)
{
    std::vector<F3> lo(count), hi(count);
    for (uint32_t i = 0; i < count; i++)
    {
        lo[i] = ld3(mins + 3 * i);
        hi[i] = ld3(maxs + 3 * i);
    }
    BvhTree t = bvh_build(lo.data(), hi.data(), count);
    std::vector<int32_t> order, stack;
    std::vector<int32_t> pre(t.nodes.size(), -1);
    if (t.root >= 0) stack.push_back(t.root);
    while (!stack.empty())
    {
        int32_t n = stack.back();
        stack.pop_back();
        pre[n] = (int32_t)order.size();
        order.push_back(n);
        for (int i = 3; i >= 0; i--)
            if (t.nodes[n].child[i] >= 0) stack.push_back(t.nodes[n].child[i]);
    }
    if (order.size() > maxNodes) return -1;
    for (size_t i = 0; i < order.size(); i++)
    {
        const BvhNode &n = t.nodes[order[i]];
        float *o = outNodes + 11 * i;
        st3(o, n.min);
        st3(o + 3, n.max);
        for (int c = 0; c < 4; c++)
        {
            int32_t idx = n.child[c] >= 0 ? pre[n.child[c]] : -1;
            memcpy(o + 6 + c, &idx, 4);
        }
        memcpy(o + 10, &n.leafIndex, 4);
    }
    return (int)order.size();
}

int oracle_bvh_query(const float *mins, const float *maxs, uint32_t count,
    uint32_t rayCount, const float *rays, uint32_t maxHits, uint32_t *out)
{
    std::vector<F3> lo(count), hi(count);
    for (uint32_t i = 0; i < count; i++)
    {
        lo[i] = ld3(mins + 3 * i);
        hi[i] = ld3(maxs + 3 * i);
    }
    BvhTree t = bvh_build(lo.data(), hi.data(), count);
    std::vector<uint32_t> leaves(maxHits ? maxHits : 1);
    std::vector<int32_t> a, b;
    for (uint32_t r = 0; r < rayCount; r++)
    {
        BvhQuery q = bvh_query(t, ld3(rays + 6 * r), ld3(rays + 6 * r + 3),
            leaves.data(), maxHits, &a, &b);
        uint32_t *o = out + (uint64_t)r * (3 + maxHits);
        o[0] = q.count;
        o[1] = q.error ? 1 : 0;
        o[2] = q.aabbTests;
        for (uint32_t i = 0; i < q.count; i++) o[3 + i] = leaves[i];
    }
    return 0;
}

void *oracle_world_create(void) { return new World(); }
void oracle_world_destroy(void *w) { delete (World *)w; }

int oracle_world_add_mesh(void *wp, const float *vertices, uint32_t vertexCount,
    const uint32_t *indices, uint32_t indexCount, int smooth)
{
    World &w = *(World *)wp;
    if (indexCount % 3 != 0 || vertexCount == 0) return -1;
    Mesh m;
    m.smooth = smooth != 0;
    m.pos.resize(vertexCount);
    m.nrm.resize(vertexCount);
    m.uv.resize(vertexCount);
    for (uint32_t i = 0; i < vertexCount; i++)
    {
        const float *v = vertices + 8 * i;
        m.pos[i] = ld3(v);
        m.nrm[i] = ld3(v + 3);
        m.uv[i] = F2{v[6], v[7]};
    }
    m.idx.assign(indices, indices + indexCount);
    for (uint32_t i = 0; i < indexCount; i++)
        if (indices[i] >= vertexCount) return -1;
    uint32_t triCount = indexCount / 3;
    std::vector<F3> lo(triCount), hi(triCount);
    for (uint32_t i = 0; i < triCount; i++)  // sp_scene.cpp:21-54
    {
        F3 a = m.pos[m.idx[3 * i]], b = m.pos[m.idx[3 * i + 1]], c = m.pos[m.idx[3 * i + 2]];
        lo[i] = vmin3(a, vmin3(b, c));
        hi[i] = vmax3(a, vmax3(b, c));
    }
    if (w.buildMeshBvh) m.tree = bvh_build(lo.data(), hi.data(), triCount);
    m.aabbMin = m.pos[0];
    m.aabbMax = m.pos[0];
    for (uint32_t i = 1; i < vertexCount; i++)
    {
        m.aabbMin = vmin3(m.aabbMin, m.pos[i]);
        m.aabbMax = vmax3(m.aabbMax, m.pos[i]);
    }
    w.meshes.push_back(std::move(m));
    return (int)w.meshes.size() - 1;
}

int oracle_world_add_object(void *wp, int mesh, uint32_t material,
    const float *pos, const float *rot, const float *scale)
{
    World &w = *(World *)wp;
    if (mesh < 0 || mesh >= (int)w.meshes.size()) return -1;
    Object o = {};
    o.mesh = mesh;
    o.material = material;
    F3 p = ld3(pos), s = ld3(scale);
    F4 q = ld4(rot);
    transform_aabb(w.meshes[mesh].aabbMin, w.meshes[mesh].aabbMax, p, q, s,
        &o.aabbMin, &o.aabbMax);
    o.model = m4_mul(m4_mul(m4_translate(p), m4_rotate(q)), m4_scale(s));
    o.invModel = m4_mul(m4_mul(m4_scale(inverse3(s)), m4_rotate(quat_conj(q))), m4_translate(-p));
    w.objects.push_back(o);
    return 0;
}

int oracle_world_build(void *wp)
{
    World &w = *(World *)wp;
    std::vector<F3> lo, hi;
    for (const Object &o : w.objects)
    {
        lo.push_back(o.aabbMin);
        hi.push_back(o.aabbMax);
    }
    w.broadphase = bvh_build(lo.data(), hi.data(), (uint32_t)lo.size());
    return 0;
}

int oracle_world_register_material(void *wp, const void *material, uint32_t id)
{
    World &w = *(World *)wp;
    Material m;
    memcpy(&m, material, sizeof(m));
    w.materialKeys.push_back(id);
    w.materials.push_back(m);
    return 0;
}

int oracle_world_register_texture(void *wp, const float *rgba, uint32_t width,
    uint32_t height, uint32_t id)
{
    World &w = *(World *)wp;
    Texture t;
    t.width = width;
    t.height = height;
    t.rgba.assign((size_t)width * (height + 1) * 4, 0.0f);
    memcpy(t.rgba.data(), rgba, sizeof(float) * 4 * (size_t)width * height);
    w.textureKeys.push_back(id);
    w.textures.push_back(std::move(t));
    return 0;
}

void oracle_world_set_background(void *wp, uint32_t id)
{
    ((World *)wp)->backgroundMaterialId = id;
}

void oracle_world_set_sky(void *wp, const float *p)
{
    World &w = *(World *)wp;
    w.sky.bottom = ld3(p);
    w.sky.top = ld3(p + 3);
    w.sky.sunDir = ld3(p + 6);
    w.sky.cosSunRadius = p[9];
    w.sky.sunRadiance = ld3(p + 10);
    w.haveSky = true;
}

void oracle_world_set_options(void *wp, const oracle_options *opt)
{
    ((World *)wp)->opt = *opt;
}

int oracle_world_intersect(void *wp, uint32_t rayCount, const float *rays,
    float *out, uint32_t *materialOut, uint64_t *metrics)
{
    World &w = *(World *)wp;
    QueryScratch s;
    bool ok = true;
    uint64_t m[12] = {};
    for (uint32_t r = 0; r < rayCount; r++)
    {
        SceneHit h = intersect_scene(w, ld3(rays + 6 * r), ld3(rays + 6 * r + 3), s, m, &ok);
        out[6 * r] = h.t;
        st3(out + 6 * r + 1, h.normal);
        out[6 * r + 4] = h.uv.x;
        out[6 * r + 5] = h.uv.y;
        materialOut[r] = h.materialId;
    }
    if (metrics) memcpy(metrics, m, sizeof(m));
    return ok ? 0 : -100;
}

int oracle_world_closest(void *wp, uint32_t rayCount, const float *rays,
    float *tOut, int32_t *objectOut, int32_t *triangleOut, int32_t *tiedOut)
{
    World &w = *(World *)wp;
    QueryScratch s;
    bool ok = true;
    for (uint32_t r = 0; r < rayCount; r++)
    {
        SceneHit h = intersect_scene(w, ld3(rays + 6 * r), ld3(rays + 6 * r + 3), s, nullptr, &ok);
        tOut[r] = h.t;
        objectOut[r] = h.object;
        triangleOut[r] = h.triangle;
        if (tiedOut) tiedOut[r] = h.tied ? 1 : 0;
    }
    return ok ? 0 : -100;
}

int oracle_world_path_trace_tile(void *wp, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    const uint32_t *tile, uint32_t *rngState, float *pixels, uint64_t *metrics)
{
    World &w = *(World *)wp;
    Camera cam = configure_camera(width, height, ld3(camPos), ld4(camRot), filmDistance);
    uint64_t m[12] = {};
    bool ok = true;
    path_trace_tile(w, cam, tile, rngState, pixels, m, &ok);
    if (metrics) memcpy(metrics, m, sizeof(m));
    return ok ? 0 : -100;
}

int oracle_world_path_trace_hashed(void *wp, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    const uint32_t *region, uint32_t seed, int nanPolicy, float *out,
    uint32_t *nanCount, uint64_t *metrics, float *perSample)
{
    World &w = *(World *)wp;
    Camera cam = configure_camera(width, height, ld3(camPos), ld4(camRot), filmDistance);
    QueryScratch s;
    std::vector<PathVertex> path;
    uint64_t m[12] = {};
    uint32_t nans = 0;
    bool ok = true;
    uint64_t k = 0;
    for (uint32_t y = region[1]; y < region[3]; y++)
        for (uint32_t x = region[0]; x < region[2]; x++)
        {
            hashed_pixel(w, cam, x, y, seed, nanPolicy, s, path,
                out + 4 * ((size_t)x + (size_t)y * width), &nans, m,
                perSample ? perSample + 3 * k * w.opt.spp : nullptr, &ok);
            k++;
        }
    if (nanCount) *nanCount = nans;
    if (metrics) memcpy(metrics, m, sizeof(m));
    return ok ? 0 : -100;
}

void oracle_world_radiance_for_path(void *wp, const void *vertices,
    uint32_t count, float *out)
{
    World &w = *(World *)wp;
    std::vector<PathVertex> path(count);
    memcpy(path.data(), vertices, sizeof(PathVertex) * count);
    st3(out, radiance_for_path(w, path.data(), count));
}

// Renders the listed 64x64-style tiles (ids in row-major tile order) on a
// pool of threads that pop tile indices from an atomic counter, each tile
// with the application's per-tile RNG reset (src/main.cpp:731-759).
static double render_tile_ids(World &w, uint32_t width, uint32_t height, const float *camPos,
    const float *camRot, float filmDistance, uint32_t tileSize, const uint32_t *ids,
    uint32_t firstTile, uint32_t tileCount, uint32_t threads, float *pixels, uint64_t *metrics)
{
    Camera cam = configure_camera(width, height, ld3(camPos), ld4(camRot), filmDistance);
    uint32_t tilesX = (width + tileSize - 1) / tileSize;
    std::atomic<uint32_t> next(0);
    std::vector<std::vector<uint64_t>> tm(threads, std::vector<uint64_t>(12, 0));
    std::atomic<bool> allOk(true);
    double t0 = now_seconds();
    auto worker = [&](uint32_t ti) {
        for (;;)
        {
            uint32_t k = next.fetch_add(1);
            if (k >= tileCount) break;
            uint32_t tid = ids ? ids[k] : firstTile + k;
            uint32_t tx = tid % tilesX, ty = tid / tilesX;
            uint32_t tile[4] = {tx * tileSize, ty * tileSize,
                tx * tileSize + tileSize < width ? tx * tileSize + tileSize : width,
                ty * tileSize + tileSize < height ? ty * tileSize + tileSize : height};
            uint32_t rng = 0xF51C0E49u;  // main.cpp:738-739
            bool ok = true;
            path_trace_tile(w, cam, tile, &rng, pixels, tm[ti].data(), &ok);
            if (!ok) allOk = false;
        }
    };
    std::vector<std::thread> pool;
    for (uint32_t i = 0; i < threads; i++) pool.emplace_back(worker, i);
    for (auto &t : pool) t.join();
    double dt = now_seconds() - t0;
    if (metrics)
    {
        memset(metrics, 0, 12 * sizeof(uint64_t));
        for (auto &v : tm)
            for (int i = 0; i < 12; i++) metrics[i] += v[i];
    }
    return allOk ? dt : -dt;
}

double oracle_world_render_tiles_mt(void *wp, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    uint32_t tileSize, uint32_t firstTile, uint32_t tileCount,
    uint32_t threads, float *pixels, uint64_t *metrics)
{
    return render_tile_ids(*(World *)wp, width, height, camPos, camRot, filmDistance, tileSize,
        nullptr, firstTile, tileCount, threads, pixels, metrics);
}

double oracle_world_render_tile_list(void *wp, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    uint32_t tileSize, const uint32_t *tileIds, uint32_t tileCount,
    uint32_t threads, float *pixels, uint64_t *metrics)
{
    return render_tile_ids(*(World *)wp, width, height, camPos, camRot, filmDistance, tileSize,
        tileIds, 0, tileCount, threads, pixels, metrics);
}

double oracle_world_render_hashed_mt(void *wp, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    uint32_t seed, uint32_t rowBegin, uint32_t rowEnd, uint32_t threads,
    float *out, uint64_t *metrics)
{
    World &w = *(World *)wp;
    Camera cam = configure_camera(width, height, ld3(camPos), ld4(camRot), filmDistance);
    std::atomic<uint32_t> next(rowBegin);
    std::vector<std::vector<uint64_t>> tm(threads, std::vector<uint64_t>(12, 0));
    std::atomic<bool> allOk(true);
    double t0 = now_seconds();
    auto worker = [&](uint32_t ti) {
        QueryScratch s;
        std::vector<PathVertex> path;
        uint32_t nans = 0;
        bool ok = true;
        for (;;)
        {
            uint32_t y = next.fetch_add(1);
            if (y >= rowEnd) break;
            for (uint32_t x = 0; x < width; x++)
                hashed_pixel(w, cam, x, y, seed, 0, s, path,
                    out + 4 * ((size_t)x + (size_t)y * width), &nans,
                    tm[ti].data(), nullptr, &ok);
        }
        if (!ok) allOk = false;
    };
    std::vector<std::thread> pool;
    for (uint32_t i = 0; i < threads; i++) pool.emplace_back(worker, i);
    for (auto &t : pool) t.join();
    double dt = now_seconds() - t0;
    if (metrics)
    {
        memset(metrics, 0, 12 * sizeof(uint64_t));
        for (auto &v : tm)
            for (int i = 0; i < 12; i++) metrics[i] += v[i];
    }
    return allOk ? dt : -dt;
}

void oracle_world_set_build_bvh(void *wp, int on) { ((World *)wp)->buildMeshBvh = on != 0; }
void oracle_world_set_watertight(void *wp, int on) { ((World *)wp)->watertight = on != 0; }

void oracle_ray_triangle_watertight(const float *o, const float *d, const float *a,
    const float *b, const float *c, float *out)
{
    TriHit h = ray_triangle_watertight(ld3(o), ld3(d), ld3(a), ld3(b), ld3(c));
    out[0] = h.t;
    out[1] = h.uv.x;
    out[2] = h.uv.y;
}

// One channel of ToColor (src/math_lib.h:525-528): floor(c * 255) cast to
// u8.  The reference's cast is defined for results in [0, 255]; outside it
// (and for NaN, which the device's fminf/fmaxf send to 0) the value is clamped.
static uint32_t to_color_channel(float c)
{
    float f = floorf(c * 255.0f);
    if (!(f >= 0.0f)) f = 0.0f;
    if (f > 255.0f) f = 255.0f;
    return (uint32_t)f;
}

// ToColor (src/math_lib.h:523-532) over n RGBA pixels, packed A8B8G8R8.
void oracle_to_color(const float *rgba, uint64_t n, uint32_t *out)
{
    for (uint64_t i = 0; i < n; i++)
    {
        const float *c = rgba + 4 * i;
        out[i] = (to_color_channel(c[3]) << 24) | (to_color_channel(c[2]) << 16) |
                 (to_color_channel(c[1]) << 8) | to_color_channel(c[0]);
    }
}

// PerformToneMapping (src/shaders/post_processing.frag.glsl:19-26) restated
// in C, then ToColor (src/math_lib.h:523-532) with the shader's alpha of 1.
void oracle_tonemap(const float *frame, uint64_t pixels, uint32_t *out)
{
    for (uint64_t i = 0; i < pixels; i++)
    {
        const float *c = frame + 4 * i;
        float m[4];
        for (int k = 0; k < 3; k++)
        {
            float x = c[k] * 1.0f;
            x = x / (1.0f + x);
            m[k] = powf(x, 1.0f / 2.2f);
        }
        m[3] = 1.0f;
        oracle_to_color(m, 1, out + i);
    }
}

// Closest hit without BVHs: every object whose world box passes the slab
// test, every triangle whose own box passes it in object space (the set the
// reference's BVH queries return), Moller-Trumbore, smallest object-space t
// per object (ties to the lower triangle index), world t, smallest world t
// (ties to the lower object index).  Threads split the rays.
int oracle_world_closest_brute(void *wp, uint32_t rayCount, const float *rays,
    uint32_t threads, float *tOut, int32_t *objectOut, int32_t *triangleOut, int32_t *tiedOut)
{
    const World &w = *(const World *)wp;
    std::atomic<uint32_t> next(0);
    auto worker = [&]() {
        for (;;)
        {
            uint32_t r = next.fetch_add(1);
            if (r >= rayCount) break;
            F3 o = ld3(rays + 6 * (size_t)r), d = ld3(rays + 6 * (size_t)r + 3);
            F3 invd = inverse3(d);
            float best = INFINITY;
            int32_t bestObj = -1, bestTri = -1;
            bool tied = false;
            for (size_t oi = 0; oi < w.objects.size(); oi++)
            {
                const Object &obj = w.objects[oi];
                // the box gates are rounded slab tests; the watertight mode tests
                // every triangle so that no gate can reject an edge or vertex ray
                if (!w.watertight && !slab_hit(obj.aabbMin, obj.aabbMax, o, invd)) continue;
                const Mesh &mesh = w.meshes[obj.mesh];
                F3 lo = transform_point(o, obj.invModel);
                F3 ld = normalize3(transform_vector(d, obj.invModel));
                F3 linvd = inverse3(ld);
                float lbest = -1.0f;
                int32_t ltri = -1;
                bool ltied = false;
                uint32_t triCount = (uint32_t)(mesh.idx.size() / 3);
                for (uint32_t t = 0; t < triCount; t++)
                {
                    F3 a = mesh.pos[mesh.idx[3 * t]], b = mesh.pos[mesh.idx[3 * t + 1]],
                       c = mesh.pos[mesh.idx[3 * t + 2]];
                    if (!w.watertight &&
                        !slab_hit(vmin3(a, vmin3(b, c)), vmax3(a, vmax3(b, c)), lo, linvd))
                        continue;
                    TriHit h = w.watertight ? ray_triangle_watertight(lo, ld, a, b, c)
                                            : ray_triangle_mt(lo, ld, a, b, c);
                    if (h.t > 0.0f && h.t == lbest) ltied = true;
                    if (h.t > 0.0f && (h.t < lbest || lbest < 0.0f))
                    {
                        lbest = h.t;
                        ltri = (int32_t)t;
                        ltied = false;
                    }
                }
                if (ltri < 0) continue;
                F3 worldHit = transform_point(lo + ld * lbest, obj.model);
                float tw = dot3(worldHit - o, d);
                if (tw == best) tied = true;
                if (tw < best)
                {
                    best = tw;
                    bestObj = (int32_t)oi;
                    bestTri = ltri;
                    tied = ltied;
                }
            }
            tOut[r] = bestObj >= 0 ? best : -1.0f;
            objectOut[r] = bestObj;
            triangleOut[r] = bestTri;
            if (tiedOut) tiedOut[r] = tied ? 1 : 0;
        }
    };
    std::vector<std::thread> pool;
    for (uint32_t i = 0; i < (threads ? threads : 1); i++) pool.emplace_back(worker);
    for (auto &t : pool) t.join();
    return 0;
}

}  // extern "C"
