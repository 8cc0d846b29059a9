// Reference harness: TEST INFRASTRUCTURE ONLY.
//
// Compiles the unmodified vk_cinematic hot-path sources (from the reference
// tree, passed as -I<reference>/src by oracle/Makefile) into a shared library
// with a flat extern "C" surface, so that tests and the golden-vector script
// can drive the reference's own code. Nothing in the product links this.
//
// The translation unit mirrors how the reference's own unit tests build the
// path tracer (unit_tests/test_simd_path_tracer.cpp:1-31): include the headers,
// then the .cpp files, as one unity build.  The compile-time switches are the
// application's (src/config.h:25-53) except SAMPLES_PER_PIXEL, which expands to
// a harness variable so one build can run any sample count.
//
// The reference aborts on Assert failure (src/platform.h:18-22).  The harness
// turns SIGABRT raised inside a harness call into an error return so that an
// overflow of the reference's fixed capacities (32 broadphase / 128 midphase
// hits, src/sp_scene.cpp:139,240) does not take down the test process.

#include <csetjmp>
#include <csignal>
#include <cstdarg>
#include <cstring>
#include <cstdlib>
#include <vector>

#include "sample_seed.h"

static unsigned int g_harness_spp = 1;

#define USE_MT_RAY_TRIANGLE_INTERSECT 1
#define USE_BVH_SIMD_RAY_INTERSECT_AABB 1
#define RADIANCE_CLAMP 10
#define SAMPLES_PER_PIXEL g_harness_spp
#define SP_DEBUG_BROADPHASE_INTERSECTION_COUNT 0
#define SP_DEBUG_SURFACE_NORMAL 0
#define SP_DEBUG_MIDPHASE_INTERSECTION_COUNT 0
#define SP_DEBUG_PATH_LENGTH 0
#define SP_DEBUG_COSINE 0

#include "platform.h"
#include "math_lib.h"
#include "tile.h"
#include "memory_pool.h"
#include "bvh.h"
#include "ray_intersection.h"
#include "asset_loader/asset_loader.h"
#include "image.h"
#include "mesh.h"
#include "sp_scene.h"
#include "sp_material_system.h"
#include "simd_path_tracer.h"
#include "sp_metrics.h"
#include "simd.h"
#include "aabb.h"

#include "memory_pool.cpp"
#include "ray_intersection.cpp"
#include "bvh.cpp"
#include "sp_scene.cpp"
#include "sp_material_system.cpp"
#include "simd_path_tracer.cpp"
#include "mesh_generation.cpp"

// src/cubemap.cpp twice: the application's uniform (phi, theta) irradiance
// integration (src/config.h:43) and the random-sampling variant behind the
// same switch.
#define IRRADIANCE_CUBEMAP_USE_UNIFORM_SAMPLING 1
namespace ref_cube_uniform {
#include "cubemap.cpp"
}
#undef IRRADIANCE_CUBEMAP_USE_UNIFORM_SAMPLING
#define IRRADIANCE_CUBEMAP_USE_UNIFORM_SAMPLING 0
namespace ref_cube_random {
#include "cubemap.cpp"
}
#undef IRRADIANCE_CUBEMAP_USE_UNIFORM_SAMPLING

// ---------------------------------------------------------------------------
// Abort capture
// ---------------------------------------------------------------------------
static sigjmp_buf g_abort_jmp;
static volatile sig_atomic_t g_abort_armed = 0;
static char g_last_log[512];

static void HarnessLog(const char *fmt, ...)
{
    va_list args;
    va_start(args, fmt);
    vsnprintf(g_last_log, sizeof(g_last_log), fmt, args);
    va_end(args);
}

static void OnAbort(int)
{
    if (g_abort_armed)
    {
        g_abort_armed = 0;
        siglongjmp(g_abort_jmp, 1);
    }
    signal(SIGABRT, SIG_DFL);
    raise(SIGABRT);
}

#define GUARDED_BEGIN                                                          \
    LogMessage = HarnessLog;                                                   \
    signal(SIGABRT, OnAbort);                                                  \
    if (sigsetjmp(g_abort_jmp, 1) != 0)                                        \
    {                                                                          \
        return -100;                                                           \
    }                                                                          \
    g_abort_armed = 1;
#define GUARDED_END g_abort_armed = 0;

static vec3 V3(const float *p) { return Vec3(p[0], p[1], p[2]); }
static void Put3(float *o, vec3 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }

extern "C" {

const char *ref_last_log(void) { return g_last_log; }

// --- RNG (src/math_utils.h:184-214) ---------------------------------------
uint32_t ref_xorshift32(uint32_t *state)
{
    RandomNumberGenerator rng = {*state};
    u32 r = XorShift32(&rng);
    *state = rng.state;
    return r;
}
float ref_random_unilateral(uint32_t *state)
{
    RandomNumberGenerator rng = {*state};
    f32 r = RandomUnilateral(&rng);
    *state = rng.state;
    return r;
}
float ref_random_bilateral(uint32_t *state)
{
    RandomNumberGenerator rng = {*state};
    f32 r = RandomBilateral(&rng);
    *state = rng.state;
    return r;
}

// --- Camera (src/simd_path_tracer.cpp:1-63) --------------------------------
// out: right(3) up(3) forward(3) position(3) filmCenter(3)
//      halfPixelWidth halfPixelHeight halfFilmWidth halfFilmHeight  (19 floats)
void ref_configure_camera(uint32_t width, uint32_t height, const float *pos,
    const float *rot, float filmDistance, float *out)
{
    ImagePlane plane = {};
    plane.width = width;
    plane.height = height;
    sp_Camera cam = {};
    quat q = Vec4(rot[0], rot[1], rot[2], rot[3]);
    sp_ConfigureCamera(&cam, &plane, V3(pos), q, filmDistance);
    Put3(out + 0, cam.basis.right);
    Put3(out + 3, cam.basis.up);
    Put3(out + 6, cam.basis.forward);
    Put3(out + 9, cam.position);
    Put3(out + 12, cam.filmCenter);
    out[15] = cam.halfPixelWidth;
    out[16] = cam.halfPixelHeight;
    out[17] = cam.halfFilmWidth;
    out[18] = cam.halfFilmHeight;
}

void ref_film_positions(uint32_t width, uint32_t height, const float *pos,
    const float *rot, float filmDistance, uint32_t count, const float *pixel,
    float *out)
{
    ImagePlane plane = {};
    plane.width = width;
    plane.height = height;
    sp_Camera cam = {};
    quat q = Vec4(rot[0], rot[1], rot[2], rot[3]);
    sp_ConfigureCamera(&cam, &plane, V3(pos), q, filmDistance);
    for (u32 i = 0; i < count; i++)
    {
        vec2 p = Vec2(pixel[2 * i], pixel[2 * i + 1]);
        vec3 f = {};
        sp_CalculateFilmPositions(&cam, &f, &p, 1);
        Put3(out + 3 * i, f);
    }
}

// Quaternion helpers, so tests build rotations with the reference's own code
void ref_quat_axis_angle(const float *axis, float angle, float *out)
{
    quat q = Quat(V3(axis), angle);
    out[0] = q.x; out[1] = q.y; out[2] = q.z; out[3] = q.w;
}

// --- Intersection primitives ----------------------------------------------
// out: t, normal(3), u, v
void ref_ray_triangle_mt(const float *o, const float *d, const float *a,
    const float *b, const float *c, float *out)
{
    RayIntersectTriangleResult r =
        RayIntersectTriangleMT(V3(o), V3(d), V3(a), V3(b), V3(c));
    out[0] = r.t;
    Put3(out + 1, r.normal);
    out[4] = r.uv.x;
    out[5] = r.uv.y;
}

uint32_t ref_aabb4(const float *mins, const float *maxs, const float *o,
    const float *invd)
{
    vec3 bmin[4], bmax[4];
    for (int i = 0; i < 4; i++)
    {
        bmin[i] = V3(mins + 3 * i);
        bmax[i] = V3(maxs + 3 * i);
    }
    return simd_RayIntersectAabb4(bmin, bmax, V3(o), V3(invd));
}

void ref_inverse3(const float *d, float *out) { Put3(out, Inverse(V3(d))); }
void ref_normalize3(const float *d, float *out) { Put3(out, Normalize(V3(d))); }

float ref_ray_aabb_scalar(const float *bmin, const float *bmax, const float *o,
    const float *d)
{
    return RayIntersectAabb(V3(bmin), V3(bmax), V3(o), V3(d));
}

void ref_transform_aabb(const float *bmin, const float *bmax, const float *pos,
    const float *rot, const float *scale, float *out)
{
    quat q = Vec4(rot[0], rot[1], rot[2], rot[3]);
    Aabb r = TransformAabb(V3(bmin), V3(bmax), V3(pos), q, V3(scale));
    Put3(out, r.min);
    Put3(out + 3, r.max);
}

// model(16) then inverse model(16), column-major as the reference stores mat4
void ref_object_matrices(const float *pos, const float *rot,
    const float *scale, float *out)
{
    vec3 p = V3(pos);
    quat q = Vec4(rot[0], rot[1], rot[2], rot[3]);
    vec3 s = V3(scale);
    mat4 m = Translate(p) * Rotate(q) * Scale(s);
    mat4 inv = Scale(Inverse(s)) * Rotate(Conjugate(q)) * Translate(-p);
    memcpy(out, m.data, 64);
    memcpy(out + 16, inv.data, 64);
}

void ref_hemisphere(uint32_t *state, const float *normal, float *out)
{
    RandomNumberGenerator rng = {*state};
    vec3 d = RandomDirectionOnHemisphere(V3(normal), &rng);
    *state = rng.state;
    Put3(out, d);
}

// --- Procedural meshes (src/mesh_generation.cpp) ---------------------------
// vertices: 8 floats each (position, normal, uv) = VertexPNT
int ref_icosphere(uint32_t level, float *vertices, uint32_t *indices,
    uint32_t *vertexCount, uint32_t *indexCount)
{
    GUARDED_BEGIN
    static u8 *buffer = (u8 *)calloc(1, Megabytes(8));
    MemoryArena arena = {};
    InitializeMemoryArena(&arena, buffer, Megabytes(8));
    MeshData m = CreateIcosahedronMesh(level, &arena);
    memcpy(vertices, m.vertices, sizeof(VertexPNT) * m.vertexCount);
    memcpy(indices, m.indices, sizeof(u32) * m.indexCount);
    *vertexCount = m.vertexCount;
    *indexCount = m.indexCount;
    GUARDED_END
    return 0;
}

int ref_plane_mesh(float *vertices, uint32_t *indices)
{
    static u8 buffer[4096];
    MemoryArena arena = {};
    InitializeMemoryArena(&arena, buffer, sizeof(buffer));
    MeshData m = CreatePlaneMesh(&arena);
    memcpy(vertices, m.vertices, sizeof(VertexPNT) * m.vertexCount);
    memcpy(indices, m.indices, sizeof(u32) * m.indexCount);
    return (int)m.vertexCount;
}

// --- BVH (src/bvh.cpp) -------------------------------------------------------
// Builds a tree and flattens it in pre-order.  Per node 11 words:
// min(3 f32) max(3 f32) child[4] (pre-order index or -1) leafIndex (u32).
// Returns the node count, or a negative error.
int ref_bvh_build_flat(const float *mins, const float *maxs, uint32_t count,
    float *outNodes, uint32_t maxNodes)
{
    GUARDED_BEGIN
    u64 cap = (u64)count * 10 * sizeof(bvh_Node) + (u64)count * 64 + 4096;
    void *mem = calloc(1, cap);
    MemoryArena arena = {};
    InitializeMemoryArena(&arena, mem, cap);
    std::vector<vec3> bmin(count), bmax(count);
    for (u32 i = 0; i < count; i++)
    {
        bmin[i] = V3(mins + 3 * i);
        bmax[i] = V3(maxs + 3 * i);
    }
    bvh_Tree tree = bvh_CreateTree(&arena, bmin.data(), bmax.data(), count);
    // pre-order flatten
    std::vector<bvh_Node *> order;
    std::vector<bvh_Node *> stack;
    if (tree.root) stack.push_back(tree.root);
    while (!stack.empty())
    {
        bvh_Node *n = stack.back();
        stack.pop_back();
        order.push_back(n);
        for (int i = 3; i >= 0; i--)
            if (n->children[i]) stack.push_back(n->children[i]);
    }
    if (order.size() > maxNodes)
    {
        free(mem);
        GUARDED_END
        return -1;
    }
    for (size_t i = 0; i < order.size(); i++)
    {
        bvh_Node *n = order[i];
        float *o = outNodes + 11 * i;
        Put3(o, n->min);
        Put3(o + 3, n->max);
        for (int c = 0; c < 4; c++)
        {
            int idx = -1;
            if (n->children[c])
            {
                for (size_t j = 0; j < order.size(); j++)
                    if (order[j] == n->children[c]) { idx = (int)j; break; }
            }
            memcpy(o + 6 + c, &idx, 4);
        }
        memcpy(o + 10, &n->leafIndex, 4);
    }
    free(mem);
    GUARDED_END
    return (int)order.size();
}

// Build + query: leaf indices hit by each ray in the reference's order.
// out per ray: count, errorOccurred, aabbTestCount, then up to maxHits indices.
int ref_bvh_query(const float *mins, const float *maxs, uint32_t count,
    uint32_t rayCount, const float *rays, uint32_t maxHits, uint32_t *out)
{
    GUARDED_BEGIN
    u64 cap = (u64)count * 10 * sizeof(bvh_Node) + (u64)count * 64 + 4096;
    void *mem = calloc(1, cap);
    MemoryArena arena = {};
    InitializeMemoryArena(&arena, mem, cap);
    std::vector<vec3> bmin(count), bmax(count);
    for (u32 i = 0; i < count; i++)
    {
        bmin[i] = V3(mins + 3 * i);
        bmax[i] = V3(maxs + 3 * i);
    }
    bvh_Tree tree = {};
    if (count > 0)
        tree = bvh_CreateTree(&arena, bmin.data(), bmax.data(), count);
    std::vector<bvh_Node *> hits(maxHits ? maxHits : 1);
    for (u32 r = 0; r < rayCount; r++)
    {
        bvh_IntersectRayResult res = bvh_IntersectRay(&tree, V3(rays + 6 * r),
            V3(rays + 6 * r + 3), hits.data(), maxHits);
        uint32_t *o = out + (u64)r * (3 + maxHits);
        o[0] = res.count;
        o[1] = res.errorOccurred;
        o[2] = res.aabbTestCount;
        for (u32 i = 0; i < res.count; i++) o[3 + i] = hits[i]->leafIndex;
    }
    free(mem);
    GUARDED_END
    return 0;
}

// --- Scene / materials / path tracing -------------------------------------
struct RefWorld
{
    MemoryArena arena;
    sp_Scene scene;
    sp_MaterialSystem materials;
    std::vector<sp_Mesh> meshes;
    std::vector<void *> owned;
};

void *ref_world_create(uint64_t arenaBytes)
{
    RefWorld *w = new RefWorld();
    void *mem = calloc(1, arenaBytes);
    InitializeMemoryArena(&w->arena, mem, arenaBytes);
    w->owned.push_back(mem);
    memset(&w->scene, 0, sizeof(w->scene));
    memset(&w->materials, 0, sizeof(w->materials));
    sp_InitializeScene(&w->scene, &w->arena);
    return w;
}

void ref_world_destroy(void *p)
{
    RefWorld *w = (RefWorld *)p;
    for (void *m : w->owned) free(m);
    delete w;
}

// vertices: VertexPNT (8 floats).  The reference keeps pointers, so copy.
int ref_world_add_mesh(void *p, const float *vertices, uint32_t vertexCount,
    const uint32_t *indices, uint32_t indexCount, int smooth)
{
    RefWorld *w = (RefWorld *)p;
    GUARDED_BEGIN
    VertexPNT *v = (VertexPNT *)malloc(sizeof(VertexPNT) * vertexCount);
    u32 *idx = (u32 *)malloc(sizeof(u32) * indexCount);
    memcpy(v, vertices, sizeof(VertexPNT) * vertexCount);
    memcpy(idx, indices, sizeof(u32) * indexCount);
    w->owned.push_back(v);
    w->owned.push_back(idx);
    sp_Mesh mesh = sp_CreateMesh(v, vertexCount, idx, indexCount, smooth);
    u64 tempBytes = (u64)indexCount / 3 * 2 * sizeof(vec3) * 2 + 4096;
    MemoryArena temp = SubAllocateArena(&w->arena, tempBytes);
    sp_BuildMeshMidphase(&mesh, &w->arena, &temp);
    w->meshes.push_back(mesh);
    GUARDED_END
    return (int)w->meshes.size() - 1;
}

int ref_world_add_object(void *p, int mesh, uint32_t material,
    const float *pos, const float *rot, const float *scale)
{
    RefWorld *w = (RefWorld *)p;
    GUARDED_BEGIN
    quat q = Vec4(rot[0], rot[1], rot[2], rot[3]);
    sp_AddObjectToScene(&w->scene, w->meshes[mesh], material, V3(pos), q,
        V3(scale));
    GUARDED_END
    return 0;
}

int ref_world_build(void *p)
{
    RefWorld *w = (RefWorld *)p;
    GUARDED_BEGIN
    sp_BuildSceneBroadphase(&w->scene);
    GUARDED_END
    return 0;
}

// material: albedo(3) albedoTexture(u32) emission(3) emissionTexture(u32)
//           roughness = 9 words, same layout as sp_Material
int ref_world_register_material(void *p, const void *material, uint32_t id)
{
    RefWorld *w = (RefWorld *)p;
    sp_Material m;
    memcpy(&m, material, sizeof(m));
    return sp_RegisterMaterial(&w->materials, m, id) ? 0 : -1;
}

int ref_world_register_texture(void *p, const float *rgba, uint32_t width,
    uint32_t height, uint32_t id)
{
    RefWorld *w = (RefWorld *)p;
    // one spare pixel row so the reference's u == 1.0 read stays in memory
    u64 bytes = (u64)width * (height + 1) * 4 * sizeof(float);
    float *pix = (float *)calloc(1, bytes);
    memcpy(pix, rgba, (u64)width * height * 4 * sizeof(float));
    w->owned.push_back(pix);
    HdrImage img = {pix, width, height};
    return sp_RegisterTexture(&w->materials, img, id) ? 0 : -1;
}

void ref_world_set_background(void *p, uint32_t id)
{
    ((RefWorld *)p)->materials.backgroundMaterialId = id;
}

// out per ray: t, normal(3), u, v (6 floats); materialOut per ray
int ref_world_intersect(void *p, uint32_t rayCount, const float *rays,
    float *out, uint32_t *materialOut, uint64_t *metrics)
{
    RefWorld *w = (RefWorld *)p;
    GUARDED_BEGIN
    sp_Metrics m = {};
    for (u32 r = 0; r < rayCount; r++)
    {
        sp_RayIntersectSceneResult res = sp_RayIntersectScene(
            &w->scene, V3(rays + 6 * r), V3(rays + 6 * r + 3), &m);
        out[6 * r] = res.t;
        Put3(out + 6 * r + 1, res.normal);
        out[6 * r + 4] = res.uv.x;
        out[6 * r + 5] = res.uv.y;
        materialOut[r] = res.materialId;
    }
    if (metrics) memcpy(metrics, m.values, sizeof(m.values));
    GUARDED_END
    return 0;
}

// The reference tile entry point, as the application calls it
// (src/main.cpp:731-759): camera + tile + caller RNG state + spp.
// pixels: width*height*4 floats, written only inside the tile.
int ref_world_path_trace_tile(void *p, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    const uint32_t *tile, uint32_t *rngState, uint32_t spp, float *pixels,
    uint64_t *metrics)
{
    RefWorld *w = (RefWorld *)p;
    GUARDED_BEGIN
    ImagePlane plane = {};
    plane.width = width;
    plane.height = height;
    plane.pixels = (vec4 *)pixels;
    sp_Camera cam = {};
    quat q = Vec4(camRot[0], camRot[1], camRot[2], camRot[3]);
    sp_ConfigureCamera(&cam, &plane, V3(camPos), q, filmDistance);
    sp_Context ctx = {};
    ctx.camera = &cam;
    ctx.scene = &w->scene;
    ctx.materialSystem = &w->materials;
    Tile t = {tile[0], tile[1], tile[2], tile[3]};
    RandomNumberGenerator rng = {*rngState};
    sp_Metrics m = {};
    g_harness_spp = spp;
    sp_PathTraceTile(&ctx, t, &rng, &m);
    *rngState = rng.state;
    if (metrics) memcpy(metrics, m.values, sizeof(m.values));
    GUARDED_END
    return 0;
}

// Hash-per-sample rendering with the reference's own tile routine: every
// (x, y, sample) is one call of sp_PathTraceTile on a 1x1 tile with
// SAMPLES_PER_PIXEL = 1 and the RNG state set from oracle_sample_seed.
// Samples whose radiance has a NaN component contribute zero and are counted
// (nanPolicy 0) or are summed as they are (nanPolicy 1, what the reference
// itself does).  region = x0, y0, x1, y1.  out: width*height*4 floats
// (only the region is written).  perSample (optional): region pixels in
// row-major order x spp x 3 floats, the raw per-sample radiance.
int ref_world_path_trace_hashed(void *p, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    const uint32_t *region, uint32_t spp, uint32_t seed, int nanPolicy,
    float *out, uint32_t *nanCount, uint64_t *metrics, float *perSample)
{
    RefWorld *w = (RefWorld *)p;
    GUARDED_BEGIN
    ImagePlane plane = {};
    plane.width = width;
    plane.height = height;
    std::vector<vec4> scratch((size_t)width * height);
    plane.pixels = scratch.data();
    sp_Camera cam = {};
    quat q = Vec4(camRot[0], camRot[1], camRot[2], camRot[3]);
    sp_ConfigureCamera(&cam, &plane, V3(camPos), q, filmDistance);
    sp_Context ctx = {};
    ctx.camera = &cam;
    ctx.scene = &w->scene;
    ctx.materialSystem = &w->materials;
    sp_Metrics total = {};
    g_harness_spp = 1;
    f32 invSpp = 1.0f / (f32)spp;
    u32 nans = 0;
    u64 k = 0;
    for (u32 y = region[1]; y < region[3]; y++)
    {
        for (u32 x = region[0]; x < region[2]; x++)
        {
            OracleSum acc[3] = {};
            for (u32 s = 0; s < spp; s++)
            {
                RandomNumberGenerator rng = {oracle_sample_seed(seed, x, y, s)};
                sp_Metrics m = {};
                Tile t = {x, y, x + 1, y + 1};
                sp_PathTraceTile(&ctx, t, &rng, &m);
                for (int i = 1; i < SP_MAX_METRICS; i++)
                    total.values[i] += m.values[i];
                total.values[0] += m.values[0];
                vec4 r = scratch[x + y * width];
                if (perSample)
                {
                    perSample[3 * k + 0] = r.x;
                    perSample[3 * k + 1] = r.y;
                    perSample[3 * k + 2] = r.z;
                }
                k++;
                b32 isNan = std::isnan(r.x) || std::isnan(r.y) || std::isnan(r.z);
                if (isNan)
                {
                    nans++;
                    if (nanPolicy == 0) continue;
                }
                oracle_sum_add(&acc[0], r.x * invSpp);
                oracle_sum_add(&acc[1], r.y * invSpp);
                oracle_sum_add(&acc[2], r.z * invSpp);
            }
            float *o = out + 4 * ((size_t)x + (size_t)y * width);
            o[0] = oracle_sum_value(&acc[0]);
            o[1] = oracle_sum_value(&acc[1]);
            o[2] = oracle_sum_value(&acc[2]);
            o[3] = 1.0f;
        }
    }
    if (nanCount) *nanCount = nans;
    if (metrics) memcpy(metrics, total.values, sizeof(total.values));
    GUARDED_END
    return 0;
}

uint32_t ref_sample_seed(uint32_t seed, uint32_t x, uint32_t y, uint32_t s)
{
    return oracle_sample_seed(seed, x, y, s);
}

// Radiance of one explicit path (src/simd_path_tracer.cpp:107-175).
// vertex: materialId(u32) worldPosition(3) outgoingDir(3) incomingDir(3)
//         normal(3) uv(2) = 15 words, the sp_PathVertex layout.
void ref_world_radiance_for_path(void *p, const void *vertices,
    uint32_t count, float *out)
{
    RefWorld *w = (RefWorld *)p;
    std::vector<sp_PathVertex> path(count);
    memcpy(path.data(), vertices, sizeof(sp_PathVertex) * count);
    vec3 r = ComputeRadianceForPath(path.data(), count, &w->materials);
    Put3(out, r);
}

// ToColor (src/math_lib.h:523-532) over n RGBA pixels; the reference's cast
// to u8 is defined for channels whose floor(c * 255) lies in [0, 255].
void ref_to_color(const float *rgba, uint64_t n, uint32_t *out)
{
    for (uint64_t i = 0; i < n; i++)
    {
        const float *c = rgba + 4 * i;
        out[i] = ToColor(Vec4(c[0], c[1], c[2], c[3]));
    }
}

int ref_sizeof(int which)
{
    switch (which)
    {
    case 0: return sizeof(sp_Material);
    case 1: return sizeof(sp_PathVertex);
    case 2: return sizeof(VertexPNT);
    case 3: return sizeof(bvh_Node);
    default: return -1;
    }
}

} // extern "C"

// --- Cube maps (src/cubemap.cpp:108-291) ------------------------------------
// equirect: RGBA32F eqWidth x eqHeight; out: 6 faces of width x height RGBA32F.
extern "C" {

static int ref_cube_common(int which, const float *equirect, uint32_t eqWidth,
    uint32_t eqHeight, uint32_t width, uint32_t height, uint32_t spp, float *out)
{
    GUARDED_BEGIN
    HdrImage eq = {};
    eq.width = eqWidth;
    eq.height = eqHeight;
    eq.pixels = (f32 *)equirect;
    uint64_t bytes = (uint64_t)width * height * 16 * 6 + 4096;
    void *mem = calloc(1, bytes);
    MemoryArena arena = {};
    InitializeMemoryArena(&arena, mem, bytes);
    HdrImage faces[6];
    if (which == 0) {
        ref_cube_uniform::HdrCubeMap c = ref_cube_uniform::CreateCubeMap(eq, &arena, width, height);
        for (int i = 0; i < 6; i++) faces[i] = c.images[i];
    } else if (which == 1) {
        ref_cube_uniform::HdrCubeMap c =
            ref_cube_uniform::CreateIrradianceCubeMap(eq, &arena, width, height, spp);
        for (int i = 0; i < 6; i++) faces[i] = c.images[i];
    } else {
        ref_cube_random::HdrCubeMap c =
            ref_cube_random::CreateIrradianceCubeMap(eq, &arena, width, height, spp);
        for (int i = 0; i < 6; i++) faces[i] = c.images[i];
    }
    for (int i = 0; i < 6; i++)
        memcpy(out + (size_t)i * width * height * 4, faces[i].pixels,
            (size_t)width * height * 16);
    free(mem);
    GUARDED_END
    return 0;
}

int ref_create_cube_map(const float *equirect, uint32_t eqWidth, uint32_t eqHeight,
    uint32_t width, uint32_t height, float *out)
{
    return ref_cube_common(0, equirect, eqWidth, eqHeight, width, height, 0, out);
}

// mode 0: uniform (phi, theta) grid (the application's setting); 1: random
int ref_create_irradiance_cube_map(const float *equirect, uint32_t eqWidth,
    uint32_t eqHeight, uint32_t width, uint32_t height, uint32_t spp, uint32_t mode, float *out)
{
    return ref_cube_common(mode == 0 ? 1 : 2, equirect, eqWidth, eqHeight, width, height, spp,
        out);
}

}  // extern "C"
