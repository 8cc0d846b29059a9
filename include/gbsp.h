/* gbsp.h - C ABI of the GB300 path tracer (libgbsp.so).
 *
 * A drop-in for the CPU path-tracing hot path of vk_cinematic: the sp_Scene
 * build (mesh midphase + scene broadphase BVHs), the sp_MaterialSystem
 * registries and the tile entry point sp_PathTraceTile with its per-sample
 * RNG.  Every entry point is plain C: opaque handles, plain pointers and
 * sizes, an int status.  Each declaration names the reference interface it
 * replaces as file:line inside the vk_cinematic tree.
 *
 * Semantics kept from the reference: camera model, XorShift32 draws, the
 * Moller-Trumbore back-face-culled triangle test with the per-triangle AABB
 * slab gate, the two-level (object / mesh) query with its local-space
 * re-normalisation and world-space t, material evaluation, and the shading
 * estimator of ComputeRadianceForPath including RADIANCE_CLAMP.
 *
 * Differences, all deliberate:
 *  - the library copies geometry at mesh creation and owns device memory;
 *  - capacities are runtime sizes, not the reference's compile-time 32
 *    objects / 32 materials / 16 textures / 3 bounces / 32 and 128 BVH hits;
 *  - no call aborts: errors come back as a negative status, with a message
 *    from gbsp_last_error_string();
 *  - spp, bounces, seeding mode and NaN policy are per-call options.
 */
#ifndef GBSP_H
#define GBSP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBSP_VERSION 1

/* Status codes (0 = success). */
#define GBSP_OK 0
#define GBSP_ERR_INVALID_ARGUMENT (-1)
#define GBSP_ERR_OUT_OF_MEMORY (-2)
#define GBSP_ERR_CAPACITY (-3)
#define GBSP_ERR_CUDA (-4)
#define GBSP_ERR_DEVICE_STATUS (-5) /* a kernel reported a bounded-loop or stack limit */
#define GBSP_ERR_NOT_READY (-6)     /* scene broadphase not built since the last change */
#define GBSP_ERR_NO_DEVICE (-7)

/* Texture id meaning "no texture" (the reference uses U32_MAX). */
#define GBSP_NO_TEXTURE 0xFFFFFFFFu
/* Emission-texture id selecting the analytic sky (extension). */
#define GBSP_SKY_TEXTURE 0xFFFFFFFEu

/* Seeding modes. */
#define GBSP_RNG_HASH_PER_SAMPLE 0u   /* state = hash(seed, x, y, sample) */
#define GBSP_RNG_TILE_SEQUENTIAL 1u   /* one stream per tile, drawn in the
                                         reference's pixel/sample/bounce order */
/* NaN policy for a sample whose radiance has a NaN component. */
#define GBSP_NAN_ZERO 0u      /* contributes 0, counted in metrics */
#define GBSP_NAN_PROPAGATE 1u /* summed as is (what the reference does) */

/* Metric slots, same order as the reference's sp_Metrics (src/sp_metrics.h:3-41).
 * Cycle slots hold nanoseconds of device time on this library. */
#define GBSP_METRIC_ELAPSED_NS 0
#define GBSP_METRIC_PATHS_TRACED 1
#define GBSP_METRIC_RAYS_TRACED 2
#define GBSP_METRIC_RAY_HIT_COUNT 3
#define GBSP_METRIC_RAY_MISS_COUNT 4
#define GBSP_METRIC_INTERSECT_SCENE_NS 5
#define GBSP_METRIC_BROADPHASE_NODE_VISITS 6   /* top-level node visits */
#define GBSP_METRIC_SHADE_NS 7
#define GBSP_METRIC_MIDPHASE_NODE_VISITS 8     /* mesh-level node visits */
#define GBSP_METRIC_TRIANGLE_TESTS 9
#define GBSP_METRIC_MIDPHASE_BOX_TESTS 10
#define GBSP_METRIC_MESH_TESTS_PERFORMED 11
#define GBSP_METRIC_NAN_SAMPLES 12
#define GBSP_METRIC_TRACE_LAUNCHES 13          /* closest-hit kernel launches */
#define GBSP_METRIC_KERNEL_LAUNCHES 14         /* all kernels the call launched */
#define GBSP_METRIC_COUNT 16

/* gbsp_options.flags */
#define GBSP_FLAG_STAGE_TIMING 1u  /* fill the *_NS metric slots per stage
                                      (CUDA events around each launch) */
#define GBSP_FLAG_AOV 2u           /* also write first-hit G-buffers, averaged over
                                      the samples (gbsp_frame_aov_device_pointer) */
/* Closest-hit scheduling (same results, different speed).  By default primary
 * rays (coherent) run one ray per lane until the warp's 32 rays are done, and
 * bounce rays (incoherent) run per-lane: a lane fetches its next ray as soon as
 * its current one is done.  The flags force one scheduling for every bounce. */
#define GBSP_FLAG_TRACE_PER_LANE 4u
#define GBSP_FLAG_TRACE_PER_WARP 8u
/* Sort each bounce's ray queue by direction octant before tracing it (same
 * results; rays of a warp then share the tree's near-to-far child order). */
#define GBSP_FLAG_SORT_DIRECTIONS 16u

typedef struct gbsp_runtime gbsp_runtime;
typedef struct gbsp_scene gbsp_scene;
typedef struct gbsp_material_system gbsp_material_system;

/* VertexPNT (src/mesh.h:10-15): 32 bytes. */
typedef struct {
    float position[3];
    float normal[3];
    float uv[2];
} gbsp_vertex;

/* Tile (src/tile.h:3-9). */
typedef struct {
    uint32_t minX, minY, maxX, maxY;
} gbsp_tile;

/* RandomNumberGenerator (src/math_utils.h:184-187). */
typedef struct {
    uint32_t state;
} gbsp_rng;

/* sp_Metrics (src/sp_metrics.h:44-48), widened to GBSP_METRIC_COUNT slots. */
typedef struct {
    uint64_t values[GBSP_METRIC_COUNT];
} gbsp_metrics;

/* sp_Material (src/sp_material_system.h:3-12): 36 bytes, same layout. */
typedef struct {
    float albedo[3];
    uint32_t albedoTexture;
    float emission[3];
    uint32_t emissionTexture;
    float roughness;
} gbsp_material;

/* ImagePlane (src/simd_path_tracer.h:3-8).  pixels is host memory holding
 * width*height RGBA32F values, or NULL to keep the frame on the device. */
typedef struct {
    float *pixels;
    uint32_t width;
    uint32_t height;
} gbsp_image_plane;

/* sp_Camera (src/simd_path_tracer.h:17-32). */
typedef struct {
    float right[3], up[3], forward[3];
    float position[3];
    float filmCenter[3];
    gbsp_image_plane *imagePlane;
    float halfPixelWidth, halfPixelHeight;
    float halfFilmWidth, halfFilmHeight;
} gbsp_camera;

/* Per-call knobs that the reference fixes at compile time. */
typedef struct {
    uint32_t spp;            /* SAMPLES_PER_PIXEL (src/simd_path_tracer.cpp:194) */
    uint32_t max_bounces;    /* 3 in the reference (src/simd_path_tracer.cpp:195) */
    uint32_t seed;           /* hash seed for GBSP_RNG_HASH_PER_SAMPLE */
    uint32_t rng_mode;       /* GBSP_RNG_* */
    uint32_t nan_policy;     /* GBSP_NAN_* */
    float radiance_clamp;    /* RADIANCE_CLAMP (src/config.h:37); 0 disables */
    uint32_t wave_paths;     /* paths in flight per wave (0 = library default, 2^25:
                              * about 270 bytes of device memory per path at 5 bounces,
                              * never more paths than the render has) */
    uint32_t flags;          /* GBSP_FLAG_* */
} gbsp_options;

/* sp_Context (src/simd_path_tracer.h:34-46) plus the runtime and options. */
typedef struct {
    gbsp_camera *camera;
    gbsp_scene *scene;
    gbsp_material_system *materialSystem;
    gbsp_runtime *runtime;
    const gbsp_options *options;
} gbsp_context;

/* ---- runtime -------------------------------------------------------------- */
/* Device, stream and work buffers.  stream may be NULL (the library creates
 * one) or a cudaStream_t cast to void*. No reference counterpart: the
 * reference runs on host threads (src/main.cpp:790-817). */
int gbsp_runtime_create(int device, void *stream, gbsp_runtime **out);
int gbsp_runtime_destroy(gbsp_runtime *rt);
int gbsp_runtime_synchronize(gbsp_runtime *rt);
/* The stream the library launches on (a cudaStream_t). */
void *gbsp_runtime_stream(gbsp_runtime *rt);
/* Message for the last failing call on this thread. */
const char *gbsp_last_error_string(void);
int gbsp_version(void);
void gbsp_options_default(gbsp_options *opt);

/* ---- camera (host, same arithmetic as the reference) --------------------- */
/* replaces sp_ConfigureCamera (src/simd_path_tracer.cpp:1-36) */
int gbsp_configure_camera(gbsp_camera *camera, gbsp_image_plane *imagePlane,
    const float position[3], const float rotation[4], float filmDistance);
/* replaces sp_CalculateFilmPositions (src/simd_path_tracer.cpp:38-63) */
uint32_t gbsp_calculate_film_positions(const gbsp_camera *camera,
    float *filmPositions, const float *pixelPositions, uint32_t count);

/* ---- scene ------------------------------------------------------------------ */
/* replaces sp_InitializeScene (src/sp_scene.cpp:1-5) */
int gbsp_scene_create(gbsp_runtime *rt, gbsp_scene **out);
int gbsp_scene_destroy(gbsp_scene *scene);
/* Triangle test of every query and render of this scene.  REFERENCE_MT
 * (default) is RayIntersectTriangleMT (src/ray_intersection.cpp:156-190), the
 * test the bit-exact parity gate runs; WATERTIGHT is the watertight test of
 * Woop, Benthin and Wald (JCGT 2013), which cannot let a ray slip between
 * triangles sharing an edge (same face culling).  No reference counterpart. */
#define GBSP_ISECT_REFERENCE_MT 0u
#define GBSP_ISECT_WATERTIGHT 1u
int gbsp_scene_set_intersection(gbsp_scene *scene, uint32_t mode);
/* Node width of the BVHs the scene's queries and renders walk: 8 (default)
 * or 4 (the reference's width, src/bvh.h:4-12).  Every mesh and object BVH
 * is built at both widths from one binary tree (same leaves, same triangle
 * order), so switching is free and never changes a result: images, hit
 * records and ids are bit-identical at either width; only the work per ray
 * differs.  gbsp_batch_autotune picks it per batch item.  No reference
 * counterpart (the reference's width is fixed at 4). */
int gbsp_scene_set_node_width(gbsp_scene *scene, uint32_t width);
uint32_t gbsp_scene_node_width(const gbsp_scene *scene);
/* replaces sp_CreateMesh + sp_BuildMeshMidphase (src/sp_scene.cpp:8-54):
 * copies the vertices and indices to the device and builds the mesh BVH
 * there.  *meshOut receives the mesh handle used by add_object. */
int gbsp_create_mesh(gbsp_scene *scene, const gbsp_vertex *vertices,
    uint32_t vertexCount, const uint32_t *indices, uint32_t indexCount,
    int useSmoothShading, uint32_t *meshOut);
/* replaces sp_AddObjectToScene (src/sp_scene.cpp:77-117) */
int gbsp_add_object_to_scene(gbsp_scene *scene, uint32_t mesh,
    uint32_t material, const float position[3], const float orientation[4],
    const float scale[3]);
/* Removes every object (meshes stay); lets a caller rebuild the object set
 * per frame as src/main.cpp:1529-1556 does. */
int gbsp_clear_objects(gbsp_scene *scene);
/* replaces sp_BuildSceneBroadphase (src/sp_scene.cpp:119-125): uploads the
 * objects and builds the object BVH on the device. */
int gbsp_build_scene_broadphase(gbsp_scene *scene);
/* Object and triangle counts of the committed scene. */
int gbsp_scene_info(const gbsp_scene *scene, uint32_t *objects,
    uint64_t *triangles, uint32_t *meshNodes, uint32_t *maxDepth);

/* ---- queries -------------------------------------------------------------- */
/* replaces sp_RayIntersectScene (src/sp_scene.cpp:229-339) for a batch of
 * rays in host memory: rays = count * (origin xyz, direction xyz).
 * resultOut = count * (t, normal xyz, u, v), t = -1 on a miss;
 * materialOut = count material ids. */
int gbsp_ray_intersect_scene(gbsp_scene *scene, uint32_t count,
    const float *rays, float *resultOut, uint32_t *materialOut,
    gbsp_metrics *metrics);
/* Closest hit for rays already in device memory (no reference counterpart as
 * a batch; the per-ray rules are sp_RayIntersectScene's).  rays: count *
 * (ox, oy, oz, pad, dx, dy, dz, pad) float; tOut: world t (-1 miss);
 * triangleOut: the mesh's triangle index (-1 miss); objectOut may be NULL.
 * Launches on the runtime's stream and returns without synchronising. */
int gbsp_intersect_closest_device(gbsp_scene *scene, uint32_t count,
    const float *rays, float *tOut, int32_t *triangleOut, int32_t *objectOut);

/* ---- materials -------------------------------------------------------------- */
int gbsp_material_system_create(gbsp_runtime *rt, gbsp_material_system **out);
int gbsp_material_system_destroy(gbsp_material_system *ms);
/* replaces sp_RegisterMaterial (src/sp_material_system.cpp:1-13) */
int gbsp_register_material(gbsp_material_system *ms,
    const gbsp_material *material, uint32_t id);
/* replaces sp_RegisterTexture (src/sp_material_system.cpp:45-57); rgba is
 * width*height RGBA32F, copied. */
int gbsp_register_texture(gbsp_material_system *ms, const float *rgba,
    uint32_t width, uint32_t height, uint32_t id);
/* replaces the backgroundMaterialId field (src/sp_material_system.h:45) */
int gbsp_set_background_material(gbsp_material_system *ms, uint32_t id);
/* Analytic sky used by materials whose emissionTexture is GBSP_SKY_TEXTURE
 * (extension): params = bottom rgb, top rgb, sun direction xyz (unit),
 * cos(sun radius), sun radiance rgb. */
int gbsp_set_procedural_sky(gbsp_material_system *ms, const float params[13]);

/* ---- path tracing ----------------------------------------------------------- */
/* replaces sp_PathTraceTile (src/simd_path_tracer.cpp:178-345).  Renders
 * the tile into ctx->camera->imagePlane->pixels (host) and adds to
 * *metrics.  With GBSP_RNG_TILE_SEQUENTIAL the tile draws from *rng in the
 * reference's order and *rng is advanced; with GBSP_RNG_HASH_PER_SAMPLE
 * every sample is seeded from options->seed and *rng is left unchanged. */
int gbsp_path_trace_tile(const gbsp_context *ctx, gbsp_tile tile,
    gbsp_rng *rng, gbsp_metrics *metrics);
/* Whole image in one call (the caller's 510-tile loop of src/main.cpp:819-844
 * in one device pass).  The frame stays on the device (gbsp_frame_device_pointer)
 * and is also copied to imagePlane->pixels when that is not NULL. */
int gbsp_path_trace_frame(const gbsp_context *ctx, gbsp_metrics *metrics);
/* Many tiles of one frame in one device pass (hash-per-sample seeding only):
 * the caller's per-tile loop of src/main.cpp:819-844 for an arbitrary subset
 * of tiles, e.g. the tiles a denoised frame must serve from plain samples.
 * Each tile is clipped to the image and rendered exactly as
 * gbsp_path_trace_tile renders it (bit-identical pixels); tiles should not
 * overlap.  Results land in the runtime's frame buffer
 * (gbsp_frame_device_pointer) and, when imagePlane->pixels is not NULL, in
 * those host pixels.  metrics NULL and no host pixels: asynchronous. */
int gbsp_path_trace_tile_list(const gbsp_context *ctx, const gbsp_tile *tiles, uint32_t count,
    gbsp_metrics *metrics);
/* One pass of options->spp samples per pixel over the tile whose samples
 * split in two images (extension, hash-per-sample seeding only): the mean of
 * samples [0, firstSpp) goes to the runtime's frame buffer (and the
 * G-buffers with GBSP_FLAG_AOV) - bit-identical to gbsp_path_trace_tile with
 * options->spp = firstSpp - and the mean of samples [firstSpp, spp) to
 * deviceImage2 (device memory, imagePlane->width x height RGBA32F; only the
 * tile is written).  E.g. a denoiser's input and an independent check render
 * in one launch sequence.  metrics NULL and no host pixels: asynchronous. */
int gbsp_path_trace_tile_split(const gbsp_context *ctx, gbsp_tile tile, uint32_t firstSpp,
    float *deviceImage2, gbsp_metrics *metrics);
/* The same with a sample count per tile (extension): tile i is rendered
 * exactly as gbsp_path_trace_tile renders it with options->spp = spp[i]
 * (bit-identical pixels; spp[i] = 0 skips the tile), all tiles in one device
 * pass - e.g. a denoised frame's fallback tiles, each topped up to the
 * sample count its check estimated. */
int gbsp_path_trace_tile_list_spp(const gbsp_context *ctx, const gbsp_tile *tiles,
    const uint32_t *spp, uint32_t count, gbsp_metrics *metrics);
/* Tile render that allocates no memory.  No counterpart in the reference: it
 * is for callers that must not allocate device memory per call - e.g. a
 * render loop that runs under a fixed device-memory budget, or that cannot
 * afford the device-wide synchronisation an allocation may cause - but can
 * still hand the library its inputs and an output image.  Same result as
 * gbsp_path_trace_tile in GBSP_RNG_HASH_PER_SAMPLE mode, written into
 * deviceImage (device memory, imagePlane->width * imagePlane->height
 * RGBA32F, 16-byte aligned; only the tile is written).  The working memory is
 * one fixed array inside libgbsp that every GPU loading the library holds
 * until exit (about 5.8 MB): at most 16384 paths in flight, 8 bounces and
 * 4096 objects; larger requests fail with GBSP_ERR_CAPACITY.  The scene's
 * broadphase must be built and the material system uploaded by an earlier
 * render (else GBSP_ERR_NOT_READY).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress), so make that first call
 * before any stream capture.  All calls share the array: calls that overlap
 * on the GPU (other threads, other runtimes on the same device) race and
 * must be serialised by the caller.  The call waits for its own work and
 * leaves the caller's current device as it found it.  Options: the trace
 * scheduling flags apply as in gbsp_path_trace_tile; GBSP_FLAG_AOV is
 * rejected (GBSP_ERR_INVALID_ARGUMENT: no G-buffer output here);
 * GBSP_FLAG_SORT_DIRECTIONS and GBSP_FLAG_STAGE_TIMING have no effect, so
 * the ELAPSED_NS, INTERSECT_SCENE_NS and SHADE_NS metric slots stay zero;
 * every other metric slot is filled as by gbsp_path_trace_tile. */
int gbsp_path_trace_tile_noalloc(const gbsp_context *ctx, gbsp_tile tile,
    float *deviceImage, gbsp_metrics *metrics);
/* Device pointer of the runtime's last frame (width*height RGBA32F). */
const float *gbsp_frame_device_pointer(gbsp_runtime *rt);
/* Device pointer of the last frame's G-buffers when GBSP_FLAG_AOV was set:
 * width*height*8 floats per pixel = albedo rgb, depth (world t of the first
 * hit), normal xyz, fraction of samples whose first ray hit; means over the
 * samples (misses contribute zeros).  No reference counterpart: input of the
 * learned denoiser. */
const float *gbsp_frame_aov_device_pointer(gbsp_runtime *rt);
/* Copies a w x h window at (x0, y0) of the last frame (and of its G-buffers
 * when dstAov is not NULL) into packed device arrays, on the runtime's stream. */
int gbsp_frame_copy_region(gbsp_runtime *rt, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h,
    float *dstRadiance, float *dstAov);

/* ---- batched rendering ---------------------------------------------------------- */
/* Many scenes and images of uneven size rendered by one persistent kernel
 * launch that pulls pixels from a global atomic queue, launched through a
 * captured CUDA graph.  No reference counterpart: the reference renders one
 * frame at a time through its tile queue (src/main.cpp:819-844).  Every item
 * renders exactly what gbsp_path_trace_frame renders for it in
 * GBSP_RNG_HASH_PER_SAMPLE mode (bit-identical images). */
typedef struct gbsp_batch gbsp_batch;

typedef struct {
    gbsp_scene *scene;                     /* broadphase built */
    gbsp_material_system *materialSystem;
    const gbsp_camera *camera;             /* camera->imagePlane gives the size */
    gbsp_options options;                  /* hash-per-sample mode, <= 16 bounces */
    float *deviceImage;                    /* width*height RGBA32F, device memory */
} gbsp_batch_item;

typedef struct {
    uint32_t block;        /* threads per block: 64, 128 or 256 */
    uint32_t chunk;        /* pixels a thread takes per queue pop: 1..8 */
    uint32_t blocksPerSm;  /* persistent grid = SM count * blocksPerSm; 0 (wavefront
                              kernel only): each kernel at the blocks the SMs hold */
    uint32_t useGraph;     /* 1 = replay a captured CUDA graph */
    uint32_t kernel;       /* GBSP_BATCH_WAVEFRONT, GBSP_BATCH_PATH_STATE or
                              GBSP_BATCH_THREAD_PER_PIXEL */
    uint32_t wavePaths;    /* wavefront: paths per wave (0 = 2^25) */
} gbsp_batch_config;

/* gbsp_batch_config.kernel: one thread traces a whole pixel (all samples,
 * bounces and traversal) at a time; or every lane runs a state machine whose
 * steps (one traversal stack pop, one shading event) the warp executes
 * together for the lanes in the same phase, refilling finished lanes with
 * new pixels.  Both give identical images. */
#define GBSP_BATCH_THREAD_PER_PIXEL 0u
#define GBSP_BATCH_PATH_STATE 1u
/* the frame renderer's stages (generate, per-bounce closest hit and shading
 * over compacted queues, accumulate) over waves that pack the paths of
 * several items; the whole sequence is one CUDA graph (default) */
#define GBSP_BATCH_WAVEFRONT 2u

int gbsp_batch_create(gbsp_runtime *rt, const gbsp_batch_item *items, uint32_t count,
    gbsp_batch **out);
int gbsp_batch_destroy(gbsp_batch *batch);
int gbsp_batch_set_config(gbsp_batch *batch, const gbsp_batch_config *config);
int gbsp_batch_get_config(const gbsp_batch *batch, gbsp_batch_config *config);
/* First picks each item's BVH node width (8 or 4): the item's frame is
 * timed alone at both widths (spp capped at 8) and the faster is kept; then
 * times every candidate configuration (36: thread-per-pixel block x chunk x
 * blocks per SM, path-state block x blocks per SM, wavefront blocks per SM x
 * wave size 2^22..2^25) over `trials` launches each and keeps the fastest;
 * *best receives it.  Items start at their scene's gbsp_scene_set_node_width. */
int gbsp_batch_autotune(gbsp_batch *batch, uint32_t trials, gbsp_batch_config *best);
/* Node width per item (`widths` has one entry per item: 4 or 8), as chosen by
 * gbsp_batch_autotune or set by the caller.  Images do not depend on it. */
int gbsp_batch_set_node_widths(gbsp_batch *batch, const uint32_t *widths);
int gbsp_batch_get_node_widths(const gbsp_batch *batch, uint32_t *widths);
/* Renders every item.  metrics NULL: asynchronous on the runtime's stream. */
int gbsp_batch_launch(gbsp_batch *batch, gbsp_metrics *metrics);

/* ---- compute-shader path tracer ------------------------------------------------- */
/* The reference's GPU compute path tracer, src/shaders/test_compute.comp.glsl,
 * as CUDA: replaces its Vulkan dispatch (src/vulkan_renderer.cpp:1340-1368:
 * up to 64 tile indices in push constants, one invocation per tile) and the
 * descriptor bindings of its scene buffers (test_compute.comp.glsl:60-100).
 * Brute-force closest hit over every entity's triangles, RNG chained through
 * each tile, three bounces, hard-coded material ids (0 red, 2 checkerboard,
 * 5 white light, others black). */
typedef struct gbsp_cpt_scene gbsp_cpt_scene;

typedef struct {                 /* Mesh, test_compute.comp.glsl:46-51 */
    uint32_t indexCount;
    uint32_t indicesOffset;      /* in indices */
    uint32_t vertexDataOffset;   /* in vertices */
} gbsp_cpt_mesh;

typedef struct {                 /* Entity, test_compute.comp.glsl:53-58 */
    uint32_t meshIndex;
    uint32_t materialId;
    uint32_t modelMatrixIndex;
} gbsp_cpt_entity;

typedef struct {
    uint32_t width, height;          /* IMAGE_WIDTH / IMAGE_HEIGHT (256 x 192 in the shader) */
    uint32_t tileWidth, tileHeight;  /* TILE_WIDTH / TILE_HEIGHT (16) */
    float filmDistance;              /* 0.8 in the shader */
    float cameraTransform[16];       /* column-major: right, up, forward, position
                                        (ComputeShaderUniformBuffer, src/main.cpp:686-693) */
} gbsp_cpt_view;

/* Copies the scene buffers to the device.  Matrices are column-major 4x4,
 * 16 floats each; checkerBoard is an RGBA32F texture sampled with the
 * reference's linear/REPEAT sampler (NULL with size 0: albedo 0). */
int gbsp_cpt_scene_create(gbsp_runtime *rt, const gbsp_vertex *vertices, uint32_t vertexCount,
    const uint32_t *indices, uint32_t indexCount, const gbsp_cpt_mesh *meshes, uint32_t meshCount,
    const float *modelMatrices, const float *invModelMatrices, uint32_t matrixCount,
    const gbsp_cpt_entity *entities, uint32_t entityCount, const float *checkerBoard,
    uint32_t texWidth, uint32_t texHeight, gbsp_cpt_scene **out);
int gbsp_cpt_scene_destroy(gbsp_cpt_scene *scene);
/* Renders the tiles tileIndices[0..tileCount) (host array; tile i covers
 * (i % (width / tileWidth), i / (width / tileWidth)), clipped to the image)
 * into deviceImage (width * height RGBA32F, device memory).  Pixels outside
 * the listed tiles are left as they are.  metrics NULL: asynchronous. */
int gbsp_cpt_render_tiles(gbsp_cpt_scene *scene, const gbsp_cpt_view *view,
    const uint32_t *tileIndices, uint32_t tileCount, float *deviceImage, gbsp_metrics *metrics);

/* ---- cube maps ------------------------------------------------------------------- */
/* Equirectangular RGBA32F image (eqWidth x eqHeight, row 0 = top) -> six
 * faces (face-major: 6 x height x width RGBA32F, faces +X -X +Y -Y +Z -Z).
 * Device pointers, 16-byte aligned; asynchronous on `stream` (a
 * cudaStream_t, NULL = default stream). */
/* replaces CreateCubeMap (src/cubemap.cpp:235-291) */
int gbsp_create_cube_map(void *stream, const float *equirect, uint32_t eqWidth, uint32_t eqHeight,
    uint32_t width, uint32_t height, float *faces);
/* replaces CreateIrradianceCubeMap (src/cubemap.cpp:106-233).  mode
 * GBSP_IRRADIANCE_UNIFORM integrates the (phi, theta) grid of step 0.1 (the
 * application's IRRADIANCE_CUBEMAP_USE_UNIFORM_SAMPLING 1, src/config.h:43;
 * samplesPerPixel unused); GBSP_IRRADIANCE_RANDOM draws samplesPerPixel
 * offsets per texel from one XorShift32 stream seeded 0x45BA12F3 in face,
 * row, column order, as the reference does. */
#define GBSP_IRRADIANCE_UNIFORM 0u
#define GBSP_IRRADIANCE_RANDOM 1u
int gbsp_create_irradiance_cube_map(void *stream, const float *equirect, uint32_t eqWidth,
    uint32_t eqHeight, uint32_t width, uint32_t height, uint32_t samplesPerPixel, uint32_t mode,
    float *faces);
/* XorShift32 (src/math_utils.h:184-192) advanced `steps` times in
 * O(log steps) GF(2) matrix products.  Host function, no device needed; no
 * reference counterpart. */
uint32_t gbsp_xorshift32_jump(uint32_t state, uint64_t steps);

/* ---- display ------------------------------------------------------------------------ */
/* Tone maps an RGBA32F frame (device memory) into packed 8-bit RGBA (device
 * memory): replaces PerformToneMapping of src/shaders/post_processing.frag.glsl:19-26
 * (Reinhard, gamma 1/2.2) and ToColor (src/math_lib.h:523-532). */
int gbsp_tonemap(void *stream, const float *frame, uint64_t pixels, uint32_t *out);

/* ---- learned denoiser ----------------------------------------------------------- */
/* Kernels of a kernel-predicting CNN denoiser (8 conv3x3 layers, 48 channels,
 * softmax 5x5 filter) trained on this path tracer's low/high-spp frames.
 * No reference counterpart.  All pointers are device memory, BF16 values
 * travel as uint16_t.  `stream` is a cudaStream_t (NULL = default stream).
 * Calls are asynchronous.  Layouts: frames (radiance RGBA32F, G-buffers,
 * denoised output) and FP32 logits are NHWC; activations and their gradients
 * (features, conv inputs and BF16 / FP32-gradient outputs, dLogits) are
 * channel-group-planar, [B][H][C/8][W][8]: each 8-channel group of an image
 * row is one contiguous plane of W pixels. */
#define GBSP_DN_EPI_BF16_BIAS_RELU 0  /* BF16 out = relu(conv + bias) */
#define GBSP_DN_EPI_F32_BIAS 1        /* FP32 out = conv + bias */
#define GBSP_DN_EPI_F32 2             /* FP32 out = conv */
/* features[p] = log1p(radiance), albedo, normal, depth/(1+depth), 6 zeros
 * (16 BF16, planar) from an RGBA32F frame and its G-buffers (8 floats per
 * pixel); `pixels` is a whole number of rows of `width` pixels. */
int gbsp_dn_features(void *stream, const float *radiance, const float *aov, uint64_t pixels,
    uint32_t width, uint16_t *out);
/* out[p][co] = sum_tap,ci in[p+off(tap)][ci] * w[tap][co][ci] (zero padded),
 * with the epilogue above.  Instantiated for (cin, cout) = (16,48), (48,48),
 * (48,32) and, for data gradients, (48,48)/(32,48) with GBSP_DN_EPI_F32. */
int gbsp_dn_conv3x3_forward(void *stream, const uint16_t *in, uint32_t B, uint32_t H, uint32_t W,
    uint32_t cin, const uint16_t *weights, const float *bias, uint32_t cout, int epilogue,
    uint16_t *outBf16, float *outF32);
/* The same convolution on the 5th-generation tensor cores (tcgen05.mma,
 * accumulator in tensor memory), 128-pixel tiles; tensors 16-byte aligned.
 * Same instantiations and epilogues. */
int gbsp_dn_conv3x3_forward_tc(void *stream, const uint16_t *in, uint32_t B, uint32_t H,
    uint32_t W, uint32_t cin, const uint16_t *weights, const float *bias, uint32_t cout,
    int epilogue, uint16_t *outBf16, float *outF32);
/* The logits layer (cin -> 32, FP32 accumulators + bias) fused with the 5x5
 * kernel-prediction filter: out[p] = sum_k softmax(logits[p][0..24])_k *
 * noisy[p + off5x5(k)] (edge-clamped), RGBA32F, without storing the logits.
 * Bit-identical to gbsp_dn_conv3x3_forward_tc (epilogue 1) + gbsp_dn_filter.
 * cin = 48. */
int gbsp_dn_conv3x3_filter_tc(void *stream, const uint16_t *in, uint32_t B, uint32_t H,
    uint32_t W, uint32_t cin, const uint16_t *weights, const float *bias, const float *noisy,
    float *out);
/* Diagnostic: clock cycles per 128 x n x 16 BF16 tcgen05.mma when `issuers`
 * (1 or 2) threads of one CTA each issue `iters` of them back to back into
 * their own tensor-memory accumulator (n = 16, 32, 48, 64, 96, 128, 144, 256);
 * the A operand starts (aOffset16 % 64) 16-byte units past a 1 KB boundary,
 * and from aOffset16 = 64 on the MMAs alternate between two A tiles 4 KB apart.
 * cyclesPerMma receives one value per issuer.  Synchronises the device. */
int gbsp_dn_tc_rate(uint32_t n, uint32_t iters, uint32_t issuers, uint32_t aOffset16,
    double *cyclesPerMma);
/* Reads and clears the denoiser kernels' device status word (1 = a tensor-core
 * completion wait ran out); GBSP_ERR_DEVICE_STATUS when it was set. */
int gbsp_dn_status(uint32_t *status);
/* Plain path tracing checks the denoiser: A (the denoiser's input)
 * and C are independent plain renders with the same spp, denoised = D(A);
 * per tile x tile block (tile <= 16) the tile's relMSE is estimated as
 * mean(((D - C)^2 - (A - C)^2 / 2) / (D^2 + 0.01)) (the second term removes
 * C's own variance); a tile whose estimate exceeds `bound` by more than two
 * standard errors of the tile mean (from the spread of its per-pixel terms)
 * is served from the plain samples (A + C) / 2.  Frames are RGBA32F
 * (B x H x W); tileErr receives the estimate and flags 1 for a tile that
 * fell back, one value per tile (row-major per image). */
int gbsp_dn_tile_fallback(void *stream, const float *denoised, const float *plainA,
    const float *plainC, uint32_t B, uint32_t H, uint32_t W, uint32_t tile, float bound,
    float *out, float *tileErr, uint32_t *flags);
/* The served-output check: per tile x tile block (tile <= 16) of B denoised
 * frames D (H x W RGBA32F), judged by the plain path tracer from A, the
 * plain render D was denoised from (sppA samples per pixel), and C, an
 * independent plain render (sppC).  tileErr receives the tile's estimated
 * relMSE (unbiased: (D - C)^2 less C's variance, over D^2 + 0.01), flags 1
 * where the estimate exceeds `bound` by more than two standard errors, and
 * needSpp the plain samples per pixel that bring the tile to `bound`
 * (`margin` times the per-sample relMSE estimated from A - C, over bound;
 * 1..maxSpp).  No reference counterpart. */
int gbsp_dn_tile_check(void *stream, const float *denoised, const float *plainA, uint32_t sppA,
    const float *plainC, uint32_t sppC, uint32_t B, uint32_t H, uint32_t W, uint32_t tile,
    float bound, float margin, uint32_t maxSpp, float *tileErr, uint32_t *flags, uint32_t *needSpp);
/* The served frame: D where flags[t] is 0; elsewhere the mean of all plain
 * samples of the pixel, (sppA A + sppC C + sppF[t] F) / (sppA + sppC +
 * sppF[t]), F the fallback render of the flagged tiles (NULL: none). */
int gbsp_dn_tile_merge(void *stream, const float *denoised, const float *plainA, uint32_t sppA,
    const float *plainC, uint32_t sppC, const float *fallback, const uint32_t *sppF, uint32_t B,
    uint32_t H, uint32_t W, uint32_t tile, const uint32_t *flags, float *out);
/* wt[8-tap][ci][co] = w[tap][co][ci]: weights of the data-gradient conv. */
int gbsp_dn_flip_transpose(void *stream, const uint16_t *w, uint32_t cout, uint32_t cin,
    uint16_t *wt);
/* out = dAct * (act > 0), as BF16. */
int gbsp_dn_relu_backward(void *stream, const float *dAct, const uint16_t *act, uint64_t n,
    uint16_t *out);
/* dW[tap][co][ci] += sum_p dOut[p][co] * in[p+off(tap)][ci]; dBias[co] += sum_p dOut[p][co]. */
int gbsp_dn_conv3x3_weight_grad(void *stream, const uint16_t *in, const uint16_t *dOut,
    uint32_t B, uint32_t H, uint32_t W, uint32_t cin, uint32_t cout, float *dW, float *dBias);
/* The same gradient on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32
 * accumulators): per-CTA partial sums added in a fixed order, so repeated calls give
 * identical results.  Same shapes as gbsp_dn_conv3x3_weight_grad. */
int gbsp_dn_conv3x3_weight_grad_tc(void *stream, const uint16_t *in, const uint16_t *dOut,
    uint32_t B, uint32_t H, uint32_t W, uint32_t cin, uint32_t cout, float *dW, float *dBias);
/* The same weight and bias gradients on the 5th-generation tensor cores
 * (tcgen05.mma, FP32 accumulators in tensor memory): all nine taps of a
 * 64-pixel input-row chunk as one GEMM, M = (tap row, input channel), N =
 * (tap column, output channel), K = pixels, with both operands read by the
 * tensor core straight from TMA-loaded boxes of the channel-group-planar
 * tensors (MN-major: eight channels of one pixel per 16-byte row) and the
 * bias gradient from an extra row of ones; per-CTA partial sums added in a
 * fixed order (deterministic).  Tensors 16-byte aligned.  No reference
 * counterpart. */
int gbsp_dn_conv3x3_weight_grad_tcgen05(void *stream, const uint16_t *in, const uint16_t *dOut,
    uint32_t B, uint32_t H, uint32_t W, uint32_t cin, uint32_t cout, float *dW, float *dBias);
/* out[p] = sum_k softmax(logits[p][0..24])_k * noisy[p + off5x5(k)] (edge-clamped);
 * logits have 32 channels per pixel. */
int gbsp_dn_filter(void *stream, const float *logits, const float *noisy, uint32_t B, uint32_t H,
    uint32_t W, float *out);
/* Gradient of relMSE = mean((out - target)^2 / (target^2 + 0.01)) with respect
 * to the logits (BF16, 32 channels); adds the unnormalised loss to *lossSum. */
int gbsp_dn_relmse_backward(void *stream, const float *logits, const float *noisy,
    const float *target, uint32_t B, uint32_t H, uint32_t W, uint16_t *dLogits, float *lossSum);
/* One Adam step on n parameters (FP32 master copy, optional BF16 mirror). */
int gbsp_dn_adam(void *stream, float *param, uint16_t *paramBf16, const float *grad, float *m,
    float *v, uint64_t n, float lr, float beta1, float beta2, float eps, uint32_t step);

/* ---- procedural meshes (src/mesh_generation.cpp) ------------------------------ */
/* CreateIcosahedronMesh (src/mesh_generation.cpp:220-337) without its 2048
 * vertex cap.  Pass NULL arrays to get the counts only. */
int gbsp_icosphere(uint32_t level, gbsp_vertex *vertices, uint32_t *indices,
    uint32_t *vertexCount, uint32_t *indexCount);
/* CreatePlaneMesh (src/mesh_generation.cpp:1-21): 4 vertices, 6 indices. */
int gbsp_plane_mesh(gbsp_vertex vertices[4], uint32_t indices[6]);

/* The per-sample RNG state used by GBSP_RNG_HASH_PER_SAMPLE. */
uint32_t gbsp_sample_seed(uint32_t seed, uint32_t x, uint32_t y,
    uint32_t sample);

#ifdef __cplusplus
}
#endif
#endif /* GBSP_H */
