// sp_gpu.h - vk_cinematic's sp_* path-tracer API on the GB300 library.
//
// A C++ caller that builds the reference's path tracer as a unity build
// (src/main.cpp:227-243, unit_tests/test_simd_path_tracer.cpp:22-31) swaps
// the sp_scene / sp_material_system / simd_path_tracer / sp_metrics headers
// and .cpp files for this header and links libgbsp.so.  The reference's
// platform and math types (vec3, quat, VertexPNT, Tile,
// RandomNumberGenerator, MemoryArena, HdrImage) keep coming from its own
// headers; define SP_GPU_STANDALONE to get layout-identical stand-ins
// instead (for callers without the reference tree).
//
// Semantics are the reference's: sp_PathTraceTile draws from the caller's
// RNG in the reference's pixel/sample/bounce order (GBSP_RNG_TILE_SEQUENTIAL)
// with SAMPLES_PER_PIXEL samples (1 if the macro is undefined) and 3
// bounces; sp_gpu::options() changes those per process.  Objects, meshes and
// materials are uploaded to the device when the scene's broadphase is built.
#pragma once

#include <stdint.h>
#include <string.h>

#include <utility>
#include <vector>

#include "gbsp.h"

#ifdef SP_GPU_STANDALONE
typedef uint8_t u8;
typedef uint32_t u32;
typedef uint64_t u64;
typedef int32_t i32;
typedef float f32;
typedef u32 b32;
union vec2 {
    struct { f32 x, y; };
    f32 data[2];
};
union vec3 {
    struct { f32 x, y, z; };
    f32 data[3];
};
union vec4 {
    struct { f32 x, y, z, w; };
    struct { vec3 xyz; f32 w_; };
    f32 data[4];
};
typedef vec4 quat;
struct VertexPNT {
    vec3 position;
    vec3 normal;
    vec2 textureCoord;
};
struct Tile {
    u32 minX, minY, maxX, maxY;
};
struct RandomNumberGenerator {
    u32 state;
};
struct MemoryArena {
    void *base;
    u64 size;
    u64 capacity;
};
struct HdrImage {
    float *pixels;
    uint32_t width;
    uint32_t height;
};
#endif

static_assert(sizeof(VertexPNT) == sizeof(gbsp_vertex), "VertexPNT layout");

namespace sp_gpu {

// Process-wide runtime on device 0 (created on first use).
inline gbsp_runtime *runtime()
{
    static gbsp_runtime *rt = nullptr;
    if (!rt) gbsp_runtime_create(0, nullptr, &rt);
    return rt;
}

// Options used by sp_PathTraceTile.
inline gbsp_options &options()
{
    static gbsp_options opt = [] {
        gbsp_options o;
        gbsp_options_default(&o);
        o.rng_mode = GBSP_RNG_TILE_SEQUENTIAL;
        o.nan_policy = GBSP_NAN_PROPAGATE;
        o.max_bounces = 3;
#ifdef SAMPLES_PER_PIXEL
        o.spp = SAMPLES_PER_PIXEL;
#else
        o.spp = 1;
#endif
        return o;
    }();
    return opt;
}

// Status of the last sp_* call that talked to the device (0 = success).
inline int &last_status()
{
    static int s = 0;
    return s;
}

inline u32 next_mesh_key()
{
    static u32 k = 0;
    return ++k;
}

}  // namespace sp_gpu

// ---- sp_Mesh / sp_Scene (src/sp_scene.h:3-29) -------------------------------
struct sp_Mesh {
    VertexPNT *vertices;  // caller memory, read at sp_BuildSceneBroadphase
    u32 *indices;
    u32 vertexCount;
    u32 indexCount;
    b32 useSmoothShading;
    u32 key;  // assigned by sp_BuildMeshMidphase
};

struct sp_GpuObject {
    sp_Mesh mesh;
    u32 material;
    vec3 position;
    quat orientation;
    vec3 scale;
};

struct sp_Scene {
    gbsp_scene *handle;
    std::vector<sp_GpuObject> *objects;
    std::vector<std::pair<u32, u32>> *uploaded;  // mesh key -> device mesh
    u32 objectCount;
};

struct sp_RayIntersectSceneResult {
    f32 t;
    u32 materialId;
    vec3 normal;
    vec2 uv;
};

inline void sp_InitializeScene(sp_Scene *scene, MemoryArena *)
{
    if (!scene->handle) gbsp_scene_create(sp_gpu::runtime(), &scene->handle);
    if (!scene->objects) scene->objects = new std::vector<sp_GpuObject>();
    if (!scene->uploaded) scene->uploaded = new std::vector<std::pair<u32, u32>>();
}

inline sp_Mesh sp_CreateMesh(VertexPNT *vertices, u32 vertexCount, u32 *indices,
    u32 indexCount, b32 useSmoothShading = false)
{
    sp_Mesh m = {};
    m.vertices = vertices;
    m.vertexCount = vertexCount;
    m.indices = indices;
    m.indexCount = indexCount;
    m.useSmoothShading = useSmoothShading;
    return m;
}

// The mesh BVH is built on the device when the mesh is first used by a scene.
inline void sp_BuildMeshMidphase(sp_Mesh *mesh, MemoryArena *, MemoryArena *)
{
    mesh->key = sp_gpu::next_mesh_key();
}

inline void sp_AddObjectToScene(sp_Scene *scene, sp_Mesh mesh, u32 material, vec3 position,
    quat orientation, vec3 scale)
{
    sp_InitializeScene(scene, nullptr);
    scene->objects->push_back(sp_GpuObject{mesh, material, position, orientation, scale});
    scene->objectCount = (u32)scene->objects->size();
}

inline void sp_BuildSceneBroadphase(sp_Scene *scene)
{
    sp_InitializeScene(scene, nullptr);
    int rc = gbsp_clear_objects(scene->handle);
    for (const sp_GpuObject &o : *scene->objects) {
        u32 dev = 0xFFFFFFFFu;
        for (auto &kv : *scene->uploaded)
            if (o.mesh.key != 0 && kv.first == o.mesh.key) dev = kv.second;
        if (dev == 0xFFFFFFFFu) {
            rc = rc ? rc : gbsp_create_mesh(scene->handle, (const gbsp_vertex *)o.mesh.vertices,
                o.mesh.vertexCount, o.mesh.indices, o.mesh.indexCount, o.mesh.useSmoothShading,
                &dev);
            if (o.mesh.key != 0) scene->uploaded->push_back({o.mesh.key, dev});
        }
        rc = rc ? rc : gbsp_add_object_to_scene(scene->handle, dev, o.material, o.position.data,
            o.orientation.data, o.scale.data);
    }
    rc = rc ? rc : gbsp_build_scene_broadphase(scene->handle);
    sp_gpu::last_status() = rc;
}

// ---- materials (src/sp_material_system.h:3-46) -----------------------------
struct sp_Material {
    vec3 albedo;
    u32 albedoTexture;
    vec3 emission;
    u32 emissionTexture;
    f32 roughness;
};
static_assert(sizeof(sp_Material) == sizeof(gbsp_material), "sp_Material layout");

struct sp_MaterialSystem {
    gbsp_material_system *handle;
    u32 backgroundMaterialId;
};

inline void sp_gpu_material_init(sp_MaterialSystem *ms)
{
    if (!ms->handle) gbsp_material_system_create(sp_gpu::runtime(), &ms->handle);
}

inline b32 sp_RegisterMaterial(sp_MaterialSystem *ms, sp_Material material, u32 id)
{
    sp_gpu_material_init(ms);
    return gbsp_register_material(ms->handle, (const gbsp_material *)&material, id) == GBSP_OK;
}

inline b32 sp_RegisterTexture(sp_MaterialSystem *ms, HdrImage image, u32 id)
{
    sp_gpu_material_init(ms);
    return gbsp_register_texture(ms->handle, image.pixels, image.width, image.height, id) == GBSP_OK;
}

// ---- camera and tile entry (src/simd_path_tracer.h, .cpp) -------------------
struct ImagePlane {
    vec4 *pixels;
    u32 width;
    u32 height;
};

struct Basis {
    vec3 right;
    vec3 up;
    vec3 forward;
};

struct sp_Camera {
    Basis basis;
    vec3 position;
    vec3 filmCenter;
    ImagePlane *imagePlane;
    f32 halfPixelWidth;
    f32 halfPixelHeight;
    f32 halfFilmWidth;
    f32 halfFilmHeight;
};

struct sp_Context {
    sp_Camera *camera;
    sp_Scene *scene;
    sp_MaterialSystem *materialSystem;
};

enum {
    sp_Metric_CyclesElapsed,
    sp_Metric_PathsTraced,
    sp_Metric_RaysTraced,
    sp_Metric_RayHitCount,
    sp_Metric_RayMissCount,
    sp_Metric_CyclesElapsed_RayIntersectScene,
    sp_Metric_CyclesElapsed_RayIntersectBroadphase,
    sp_Metric_CyclesElapsed_RayIntersectMesh,
    sp_Metric_CyclesElapsed_RayIntersectMeshMidphase,
    sp_Metric_CyclesElapsed_RayIntersectTriangle,
    sp_Metric_RayIntersectMesh_MidphaseAabbTestCount,
    sp_Metric_RayIntersectMesh_TestsPerformed,
    SP_MAX_METRICS,
};

// Cycle slots hold nanoseconds of device time.
struct sp_Metrics {
    u64 values[SP_MAX_METRICS];
};

inline gbsp_camera sp_gpu_camera(const sp_Camera *c, gbsp_image_plane *plane)
{
    gbsp_camera g;
    memcpy(g.right, c->basis.right.data, 12);
    memcpy(g.up, c->basis.up.data, 12);
    memcpy(g.forward, c->basis.forward.data, 12);
    memcpy(g.position, c->position.data, 12);
    memcpy(g.filmCenter, c->filmCenter.data, 12);
    g.imagePlane = plane;
    g.halfPixelWidth = c->halfPixelWidth;
    g.halfPixelHeight = c->halfPixelHeight;
    g.halfFilmWidth = c->halfFilmWidth;
    g.halfFilmHeight = c->halfFilmHeight;
    return g;
}

inline void sp_ConfigureCamera(sp_Camera *camera, ImagePlane *imagePlane, vec3 position,
    quat rotation, f32 filmDistance)
{
    gbsp_image_plane plane = {(float *)imagePlane->pixels, imagePlane->width, imagePlane->height};
    gbsp_camera g;
    gbsp_configure_camera(&g, &plane, position.data, rotation.data, filmDistance);
    camera->imagePlane = imagePlane;
    memcpy(camera->basis.right.data, g.right, 12);
    memcpy(camera->basis.up.data, g.up, 12);
    memcpy(camera->basis.forward.data, g.forward, 12);
    memcpy(camera->position.data, g.position, 12);
    memcpy(camera->filmCenter.data, g.filmCenter, 12);
    camera->halfPixelWidth = g.halfPixelWidth;
    camera->halfPixelHeight = g.halfPixelHeight;
    camera->halfFilmWidth = g.halfFilmWidth;
    camera->halfFilmHeight = g.halfFilmHeight;
}

inline u32 sp_CalculateFilmPositions(sp_Camera *camera, vec3 *filmPositions,
    vec2 *pixelPositions, u32 count)
{
    gbsp_image_plane plane = {nullptr, camera->imagePlane->width, camera->imagePlane->height};
    gbsp_camera g = sp_gpu_camera(camera, &plane);
    return gbsp_calculate_film_positions(&g, (float *)filmPositions, (const float *)pixelPositions,
        count);
}

inline void sp_gpu_add_metrics(sp_Metrics *out, const gbsp_metrics &m)
{
    if (!out) return;
    out->values[sp_Metric_CyclesElapsed] += m.values[GBSP_METRIC_ELAPSED_NS];
    out->values[sp_Metric_PathsTraced] += m.values[GBSP_METRIC_PATHS_TRACED];
    out->values[sp_Metric_RaysTraced] += m.values[GBSP_METRIC_RAYS_TRACED];
    out->values[sp_Metric_RayHitCount] += m.values[GBSP_METRIC_RAY_HIT_COUNT];
    out->values[sp_Metric_RayMissCount] += m.values[GBSP_METRIC_RAY_MISS_COUNT];
    out->values[sp_Metric_CyclesElapsed_RayIntersectScene] += m.values[GBSP_METRIC_INTERSECT_SCENE_NS];
    out->values[sp_Metric_RayIntersectMesh_MidphaseAabbTestCount] +=
        m.values[GBSP_METRIC_MIDPHASE_BOX_TESTS];
    out->values[sp_Metric_RayIntersectMesh_TestsPerformed] +=
        m.values[GBSP_METRIC_MESH_TESTS_PERFORMED];
}

// replaces sp_PathTraceTile (src/simd_path_tracer.cpp:178-345)
inline void sp_PathTraceTile(sp_Context *ctx, Tile tile, RandomNumberGenerator *rng,
    sp_Metrics *metrics)
{
    sp_Scene *scene = ctx->scene;
    if (!scene->handle) sp_BuildSceneBroadphase(scene);  // a scene never built is empty
    sp_gpu_material_init(ctx->materialSystem);
    gbsp_set_background_material(ctx->materialSystem->handle,
        ctx->materialSystem->backgroundMaterialId);
    ImagePlane *ip = ctx->camera->imagePlane;
    gbsp_image_plane plane = {(float *)ip->pixels, ip->width, ip->height};
    gbsp_camera cam = sp_gpu_camera(ctx->camera, &plane);
    gbsp_context g = {&cam, scene->handle, ctx->materialSystem->handle, sp_gpu::runtime(),
        &sp_gpu::options()};
    gbsp_tile t = {tile.minX, tile.minY, tile.maxX, tile.maxY};
    gbsp_rng r = {rng->state};
    gbsp_metrics m = {};
    sp_gpu::last_status() = gbsp_path_trace_tile(&g, t, &r, &m);
    rng->state = r.state;
    sp_gpu_add_metrics(metrics, m);
}

// replaces sp_RayIntersectScene (src/sp_scene.cpp:229-339) for one ray
inline sp_RayIntersectSceneResult sp_RayIntersectScene(sp_Scene *scene, vec3 rayOrigin,
    vec3 rayDirection, sp_Metrics *metrics)
{
    sp_RayIntersectSceneResult r = {};
    r.t = -1.0f;
    if (!scene->handle) return r;
    float ray[6] = {rayOrigin.x, rayOrigin.y, rayOrigin.z, rayDirection.x, rayDirection.y,
        rayDirection.z};
    float out[6];
    u32 mat = 0;
    gbsp_metrics m = {};
    sp_gpu::last_status() = gbsp_ray_intersect_scene(scene->handle, 1, ray, out, &mat, &m);
    if (sp_gpu::last_status() != GBSP_OK) return r;
    r.t = out[0];
    r.normal.x = out[1];
    r.normal.y = out[2];
    r.normal.z = out[3];
    r.uv.x = out[4];
    r.uv.y = out[5];
    r.materialId = mat;
    sp_gpu_add_metrics(metrics, m);
    return r;
}
