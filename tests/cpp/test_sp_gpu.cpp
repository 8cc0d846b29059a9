// The reference's path-tracer unit tests (unit_tests/test_simd_path_tracer.cpp)
// restated against include/sp_gpu.h, i.e. run through the GB300 library the
// way a vk_cinematic caller would after swapping its sp_* includes.
// Built and run by tests/test_sp_gpu_cpp.py on a GPU host.

#define SP_GPU_STANDALONE
#include "sp_gpu.h"

#include <cmath>
#include <cstdio>

static int g_failures = 0;
static int g_tests = 0;
#define CHECK(cond)                                                        \
    do {                                                                   \
        if (!(cond)) {                                                     \
            printf("  FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);       \
            g_failures++;                                                  \
        }                                                                  \
    } while (0)

static vec3 V3(f32 x, f32 y, f32 z) { vec3 v; v.x = x; v.y = y; v.z = z; return v; }
static vec2 V2(f32 x, f32 y) { vec2 v; v.x = x; v.y = y; return v; }
static quat QuatIdentity() { quat q; q.x = q.y = q.z = 0; q.w = 1; return q; }
static quat QuatAxisAngle(vec3 a, f32 angle)
{
    quat q;
    q.x = a.x * sinf(angle * 0.5f);
    q.y = a.y * sinf(angle * 0.5f);
    q.z = a.z * sinf(angle * 0.5f);
    q.w = cosf(angle * 0.5f);
    return q;
}
static bool Near(f32 a, f32 b) { return fabsf(a - b) <= 1.1920929e-7f; }
static bool NearV(vec3 a, vec3 b) { return Near(a.x, b.x) && Near(a.y, b.y) && Near(a.z, b.z); }

// test_simd_path_tracer.cpp:49-87
static void TestPathTraceSingleColor()
{
    vec4 pixels[16] = {};
    ImagePlane imagePlane = {pixels, 4, 4};
    sp_Camera camera = {};
    camera.imagePlane = &imagePlane;
    sp_Scene scene = {};
    sp_MaterialSystem materialSystem = {};
    sp_Context ctx = {&camera, &scene, &materialSystem};
    RandomNumberGenerator rng = {};
    sp_Metrics metrics = {};
    Tile tile = {0, 0, 4, 4};
    sp_PathTraceTile(&ctx, tile, &rng, &metrics);
    CHECK(sp_gpu::last_status() == 0);
    for (int i = 0; i < 16; i++)
        CHECK(pixels[i].x == 1 && pixels[i].y == 0 && pixels[i].z == 1 && pixels[i].w == 1);
}

// test_simd_path_tracer.cpp:89-135
static void TestPathTraceTile()
{
    vec4 pixels[16] = {};
    ImagePlane imagePlane = {pixels, 4, 4};
    sp_Camera camera = {};
    camera.imagePlane = &imagePlane;
    sp_Scene scene = {};
    sp_MaterialSystem materialSystem = {};
    sp_Context ctx = {&camera, &scene, &materialSystem};
    RandomNumberGenerator rng = {};
    sp_Metrics metrics = {};
    Tile tile = {1, 1, 3, 3};
    sp_PathTraceTile(&ctx, tile, &rng, &metrics);
    for (int y = 0; y < 4; y++)
        for (int x = 0; x < 4; x++) {
            bool in = x >= 1 && x < 3 && y >= 1 && y < 3;
            vec4 p = pixels[x + 4 * y];
            if (in)
                CHECK(p.x == 1 && p.y == 0 && p.z == 1 && p.w == 1);
            else
                CHECK(p.x == 0 && p.y == 0 && p.z == 0 && p.w == 0);
        }
    // metrics per call (test_simd_path_tracer.cpp:333-368)
    CHECK(metrics.values[sp_Metric_PathsTraced] == 4);
    CHECK(metrics.values[sp_Metric_CyclesElapsed] > 0);
}

// test_simd_path_tracer.cpp:137-168
static void TestConfigureCamera()
{
    vec4 pixels[16] = {};
    ImagePlane imagePlane = {pixels, 4, 2};
    sp_Camera camera = {};
    sp_ConfigureCamera(&camera, &imagePlane, V3(0, 2, 0), QuatIdentity(), 0.1f);
    CHECK(camera.imagePlane == &imagePlane);
    CHECK(NearV(camera.position, V3(0, 2, 0)));
    CHECK(NearV(camera.basis.right, V3(1, 0, 0)));
    CHECK(NearV(camera.basis.up, V3(0, 1, 0)));
    CHECK(NearV(camera.basis.forward, V3(0, 0, -1)));
    CHECK(NearV(camera.filmCenter, V3(0, 2, -0.1f)));
    CHECK(Near(camera.halfPixelWidth, 0.125f));
    CHECK(Near(camera.halfPixelHeight, 0.25f));
    CHECK(Near(camera.halfFilmWidth, 0.5f));
    CHECK(Near(camera.halfFilmHeight, 0.25f));
}

// test_simd_path_tracer.cpp:170-200
static void TestCalculateFilmP()
{
    vec4 pixels[16] = {};
    ImagePlane imagePlane = {pixels, 4, 4};
    sp_Camera camera = {};
    sp_ConfigureCamera(&camera, &imagePlane, V3(0, 2, 0), QuatIdentity(), 0.1f);
    vec3 film[4] = {};
    vec2 px[4] = {V2(0.5f, 0.5f), V2(1.5f, 0.5f), V2(0.5f, 1.5f), V2(3.5f, 3.5f)};
    CHECK(sp_CalculateFilmPositions(&camera, film, px, 4) == 4);
    CHECK(NearV(film[0], V3(-0.375f, 2.375f, -0.1f)));
    CHECK(NearV(film[3], V3(0.375f, 1.625f, -0.1f)));
}

// test_simd_path_tracer.cpp:216-276
static void TestRayIntersectScene()
{
    sp_Scene scene = {};
    sp_InitializeScene(&scene, nullptr);
    VertexPNT vertices[3] = {
        {V3(-0.5f, -0.5f, 0), V3(0, 0, 1), V2(0, 0)},
        {V3(0.5f, -0.5f, 0), V3(0, 0, 1), V2(0, 0)},
        {V3(0.0f, 0.5f, 0), V3(0, 0, 1), V2(0, 0)},
    };
    u32 indices[3] = {0, 1, 2};
    u32 material = 53;
    sp_Mesh meshes[2];
    meshes[0] = sp_CreateMesh(vertices, 3, indices, 3);
    meshes[1] = sp_CreateMesh(vertices, 3, indices, 3);
    sp_BuildMeshMidphase(&meshes[0], nullptr, nullptr);
    sp_BuildMeshMidphase(&meshes[1], nullptr, nullptr);
    sp_AddObjectToScene(&scene, meshes[0], material, V3(0, 2, -5), QuatIdentity(), V3(1, 1, 1));
    sp_AddObjectToScene(&scene, meshes[1], material, V3(0, 2, -15),
        QuatAxisAngle(V3(0, 1, 0), 3.14159265359f * 0.25f), V3(2, 2, 2));
    sp_BuildSceneBroadphase(&scene);
    CHECK(sp_gpu::last_status() == 0);
    sp_Metrics metrics = {};
    sp_RayIntersectSceneResult r = sp_RayIntersectScene(&scene, V3(0, 2, 0), V3(0, 0, -1), &metrics);
    CHECK(r.t >= 0.0f);
    CHECK(fabsf(r.t - 5.0f) < 1e-5f);
    CHECK(r.materialId == material);
    CHECK(NearV(r.normal, V3(0, 0, 1)));
}

// test_simd_path_tracer.cpp:370-396 (through a one-object scene)
static void TestRayIntersectMesh()
{
    sp_Scene scene = {};
    VertexPNT vertices[3] = {
        {V3(-0.5f, -0.5f, 0), V3(0, 0, 1), V2(0, 0)},
        {V3(0.5f, -0.5f, 0), V3(0, 0, 1), V2(0, 0)},
        {V3(0.0f, 0.5f, 0), V3(0, 0, 1), V2(0, 0)},
    };
    u32 indices[3] = {0, 1, 2};
    sp_Mesh mesh = sp_CreateMesh(vertices, 3, indices, 3);
    sp_BuildMeshMidphase(&mesh, nullptr, nullptr);
    sp_AddObjectToScene(&scene, mesh, 1, V3(0, 0, 0), QuatIdentity(), V3(1, 1, 1));
    sp_BuildSceneBroadphase(&scene);
    sp_RayIntersectSceneResult r =
        sp_RayIntersectScene(&scene, V3(0, 0, 10), V3(0, 0, -1), nullptr);
    CHECK(r.t >= 0.0f);
    // back-face culling (src/ray_intersection.cpp:181-182): from behind, no hit
    sp_RayIntersectSceneResult b =
        sp_RayIntersectScene(&scene, V3(0, 0, -10), V3(0, 0, 1), nullptr);
    CHECK(b.t < 0.0f);
}

// A lit scene through the tile entry point: an emissive background and a
// diffuse triangle; the pixel through the triangle is darker than the sky.
static void TestPathTraceLitScene()
{
    const u32 W = 16, H = 16;
    static vec4 pixels[W * H];
    ImagePlane imagePlane = {pixels, W, H};
    sp_Camera camera = {};
    sp_ConfigureCamera(&camera, &imagePlane, V3(0, 0, 2), QuatIdentity(), 0.5f);
    sp_Scene scene = {};
    VertexPNT vertices[3] = {
        {V3(-0.5f, -0.5f, 0), V3(0, 0, 1), V2(0, 0)},
        {V3(0.5f, -0.5f, 0), V3(0, 0, 1), V2(1, 0)},
        {V3(0.0f, 0.5f, 0), V3(0, 0, 1), V2(0, 1)},
    };
    u32 indices[3] = {0, 1, 2};
    sp_Mesh mesh = sp_CreateMesh(vertices, 3, indices, 3);
    sp_BuildMeshMidphase(&mesh, nullptr, nullptr);
    sp_AddObjectToScene(&scene, mesh, 1, V3(0, 0, 0), QuatIdentity(), V3(1, 1, 1));
    sp_BuildSceneBroadphase(&scene);
    sp_MaterialSystem ms = {};
    sp_Material bg = {};
    bg.emission = V3(1, 1, 1);
    bg.albedoTexture = bg.emissionTexture = 0xFFFFFFFFu;
    sp_Material diffuse = {};
    diffuse.albedo = V3(0.5f, 0.5f, 0.5f);
    diffuse.albedoTexture = diffuse.emissionTexture = 0xFFFFFFFFu;
    CHECK(sp_RegisterMaterial(&ms, bg, 0));
    CHECK(sp_RegisterMaterial(&ms, diffuse, 1));
    ms.backgroundMaterialId = 0;
    sp_Context ctx = {&camera, &scene, &ms};
    RandomNumberGenerator rng = {0xF51C0E49u};
    sp_Metrics metrics = {};
    sp_PathTraceTile(&ctx, Tile{0, 0, W, H}, &rng, &metrics);
    CHECK(sp_gpu::last_status() == 0);
    CHECK(rng.state != 0xF51C0E49u);  // the caller's stream advanced
    vec4 sky = pixels[0];
    vec4 centre = pixels[W / 2 + (H / 2) * W];
    CHECK(sky.x == 1.0f);
    CHECK(centre.x > 0.0f && centre.x < 1.0f);
    CHECK(metrics.values[sp_Metric_RaysTraced] ==
          metrics.values[sp_Metric_RayHitCount] + metrics.values[sp_Metric_RayMissCount]);
}

#define RUN(t)                                   \
    do {                                         \
        int before = g_failures;                 \
        t();                                     \
        g_tests++;                               \
        printf("%s %s\n", #t, g_failures == before ? "PASS" : "FAIL"); \
    } while (0)

int main()
{
    RUN(TestPathTraceSingleColor);
    RUN(TestPathTraceTile);
    RUN(TestConfigureCamera);
    RUN(TestCalculateFilmP);
    RUN(TestRayIntersectScene);
    RUN(TestRayIntersectMesh);
    RUN(TestPathTraceLitScene);
    printf("%d tests, %d failures\n", g_tests, g_failures);
    return g_failures == 0 ? 0 : 1;
}
