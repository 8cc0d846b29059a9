// Oracle port: TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of vk_cinematic's path-tracing hot path (the sp_* scene,
// BVH, material and tile path-tracing code), written for this project and
// checked bit for bit against the reference's own code (oracle/_ref, built
// from the reference sources) and against golden vectors captured from it.
// Only tests, the smoke check and the CPU-baseline leg of the benchmark use
// it; the product never links it.
//
// Everything is plain IEEE single precision with one rounding per operation
// (built with -ffp-contract=off), and every min/max is the reference's
// "a < b ? a : b" form, whose NaN behaviour differs from fminf/fmaxf.

#pragma once
#include <cstdint>

#ifdef __cplusplus
extern "C" {
#endif

// Runtime knobs the reference only has as compile-time constants.
typedef struct
{
    uint32_t spp;              // SAMPLES_PER_PIXEL (simd_path_tracer.cpp:194)
    uint32_t max_bounces;      // 3 in the reference (simd_path_tracer.cpp:195)
    float radiance_clamp;      // RADIANCE_CLAMP 10 (config.h:37); 0 = off
    uint32_t max_broadphase;   // 32 (sp_scene.cpp:240)
    uint32_t max_midphase;     // 128 (sp_scene.cpp:139)
} oracle_options;

// RNG (math_utils.h:184-214)
uint32_t oracle_xorshift32(uint32_t *state);
float oracle_random_unilateral(uint32_t *state);
float oracle_random_bilateral(uint32_t *state);
uint32_t oracle_sample_seed_c(uint32_t seed, uint32_t x, uint32_t y, uint32_t s);

// Camera (simd_path_tracer.cpp:1-63); same 19-float layout as the harness
void oracle_configure_camera(uint32_t width, uint32_t height, const float *pos,
    const float *rot, float filmDistance, float *out);
void oracle_film_positions(uint32_t width, uint32_t height, const float *pos,
    const float *rot, float filmDistance, uint32_t count, const float *pixel,
    float *out);

// Primitives
void oracle_ray_triangle_mt(const float *o, const float *d, const float *a,
    const float *b, const float *c, float *out);
uint32_t oracle_aabb4(const float *mins, const float *maxs, const float *o,
    const float *invd);
void oracle_hemisphere(uint32_t *state, const float *normal, float *out);
void oracle_transform_aabb(const float *bmin, const float *bmax,
    const float *pos, const float *rot, const float *scale, float *out);
void oracle_object_matrices(const float *pos, const float *rot,
    const float *scale, float *out);

// BVH (bvh.cpp)
int oracle_bvh_build_flat(const float *mins, const float *maxs, uint32_t count,
    float *outNodes, uint32_t maxNodes);
int oracle_bvh_query(const float *mins, const float *maxs, uint32_t count,
    uint32_t rayCount, const float *rays, uint32_t maxHits, uint32_t *out);

// World = scene + material system
void *oracle_world_create(void);
void oracle_world_destroy(void *w);
int oracle_world_add_mesh(void *w, const float *vertices, uint32_t vertexCount,
    const uint32_t *indices, uint32_t indexCount, int smooth);
int oracle_world_add_object(void *w, int mesh, uint32_t material,
    const float *pos, const float *rot, const float *scale);
int oracle_world_build(void *w);
int oracle_world_register_material(void *w, const void *material, uint32_t id);
int oracle_world_register_texture(void *w, const float *rgba, uint32_t width,
    uint32_t height, uint32_t id);
void oracle_world_set_background(void *w, uint32_t id);
// Analytic sky for the emission-texture id 0xFFFFFFFE (an extension of
// sp_EvaluateMaterial): params = bottom(3) top(3) sunDir(3) cosSunRadius
// sunRadiance(3) = 13 floats.
void oracle_world_set_sky(void *w, const float *params);
void oracle_world_set_options(void *w, const oracle_options *opt);
int oracle_world_intersect(void *w, uint32_t rayCount, const float *rays,
    float *out, uint32_t *materialOut, uint64_t *metrics);
int oracle_world_path_trace_tile(void *w, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    const uint32_t *tile, uint32_t *rngState, float *pixels,
    uint64_t *metrics);
int oracle_world_path_trace_hashed(void *w, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    const uint32_t *region, uint32_t seed, int nanPolicy, float *out,
    uint32_t *nanCount, uint64_t *metrics, float *perSample);
void oracle_world_radiance_for_path(void *w, const void *vertices,
    uint32_t count, float *out);

// Multi-threaded frame render in the application's tile mode
// (main.cpp:731-844): 64x64 tiles taken from an atomic counter, every tile's
// RNG reset to 0xF51C0E49.  Renders tiles [firstTile, firstTile+tileCount)
// of the row-major tile list.  Returns wall seconds; metrics summed.
double oracle_world_render_tiles_mt(void *w, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    uint32_t tileSize, uint32_t firstTile, uint32_t tileCount,
    uint32_t threads, float *pixels, uint64_t *metrics);

// Same, over an explicit list of tile ids (row-major tile order).
double oracle_world_render_tile_list(void *w, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    uint32_t tileSize, const uint32_t *tileIds, uint32_t tileCount,
    uint32_t threads, float *pixels, uint64_t *metrics);

// Same, hash-per-sample seeding (what the GPU path computes).
double oracle_world_render_hashed_mt(void *w, uint32_t width, uint32_t height,
    const float *camPos, const float *camRot, float filmDistance,
    uint32_t seed, uint32_t rowBegin, uint32_t rowEnd, uint32_t threads,
    float *out, uint64_t *metrics);

// Closest hit for a ray batch through the reference's scene query: out per
// ray is the world t (-1 miss), the winning object and its triangle index;
// tiedOut (optional) flags rays whose best t is an exact tie between two
// candidates (two objects at the same world t, or two triangles of the
// winning object at the same object-space t), where the reference's winner
// depends on its BVH order.
int oracle_world_closest(void *w, uint32_t rayCount, const float *rays,
    float *tOut, int32_t *objectOut, int32_t *triangleOut, int32_t *tiedOut);

// Meshes added after this call skip the reference's O(n^2 log n) BVH build
// (they can then only be queried with oracle_world_closest_brute).
void oracle_world_set_build_bvh(void *w, int on);
// Brute-force queries use the watertight triangle test (Woop et al. 2013).
void oracle_world_set_watertight(void *w, int on);
// out = t (-1 miss), u, v of the watertight test with the reference's culling.
void oracle_ray_triangle_watertight(const float *o, const float *d, const float *a,
    const float *b, const float *c, float *out);
// 8-bit packing of RGBA pixels (ToColor), and the display conversion:
// Reinhard + gamma 1/2.2, then that packing.
void oracle_to_color(const float *rgba, uint64_t n, uint32_t *out);
void oracle_tonemap(const float *frame, uint64_t pixels, uint32_t *out);
int oracle_world_closest_brute(void *w, uint32_t rayCount, const float *rays,
    uint32_t threads, float *tOut, int32_t *objectOut, int32_t *triangleOut, int32_t *tiedOut);

#ifdef __cplusplus
}
#endif
