// C ABI of the GB300 path tracer: host objects, scene build and entry points.
//
// Host arithmetic that must match the reference bit for bit (camera basis,
// object matrices, object AABBs) is compiled with -ffp-contract=off and
// follows the reference's expression order.

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "gbsp_internal.h"

namespace gbsp {

static thread_local char g_error[512] = "";

int set_error(int status, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_error(cudaError_t e, const char *what)
{
    return set_error(e == cudaErrorMemoryAllocation ? GBSP_ERR_OUT_OF_MEMORY : GBSP_ERR_CUDA,
        "%s: %s", what, cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// Host math: quaternion and mat4 in the reference's layout and order
// (src/math_lib.h:201-270, 556-623)
// ---------------------------------------------------------------------------
namespace {

struct Q4 {
    float x, y, z, w;
};
struct M4 {
    float m[16];  // column-major
};

Q4 quat_mul(Q4 p, Q4 q)
{
    V3 pv = v3(p.x, p.y, p.z), qv = v3(q.x, q.y, q.z);
    V3 v = add(add(mul(qv, p.w), mul(pv, q.w)), cross(pv, qv));
    float s = p.w * q.w - dot(pv, qv);
    return Q4{v.x, v.y, v.z, s};
}
Q4 quat_conj(Q4 p) { return Q4{-p.x, -p.y, -p.z, p.w}; }
V3 rotate_vector(V3 v, Q4 p)
{
    Q4 q = {v.x, v.y, v.z, 0.0f};
    Q4 r = quat_mul(quat_mul(p, q), quat_conj(p));
    return v3(r.x, r.y, r.z);
}
M4 m4_identity()
{
    M4 r = {};
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
    return r;
}
M4 m4_scale(V3 s)
{
    M4 r = {};
    r.m[0] = s.x;
    r.m[5] = s.y;
    r.m[10] = s.z;
    r.m[15] = 1.0f;
    return r;
}
M4 m4_translate(V3 t)
{
    M4 r = m4_identity();
    r.m[12] = t.x;
    r.m[13] = t.y;
    r.m[14] = t.z;
    return r;
}
float dot4(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3]; }
M4 m4_mul(const M4 &a, const M4 &b)
{
    M4 r = {};
    for (int i = 0; i < 4; i++) {
        float row[4] = {a.m[i], a.m[4 + i], a.m[8 + i], a.m[12 + i]};
        for (int c = 0; c < 4; c++) r.m[c * 4 + i] = dot4(row, b.m + c * 4);
    }
    return r;
}
M4 m4_rotate(Q4 q)
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
Affine rows_of(const M4 &m)
{
    Affine a;
    for (int i = 0; i < 3; i++) {
        a.r[4 * i + 0] = m.m[i];
        a.r[4 * i + 1] = m.m[4 + i];
        a.r[4 * i + 2] = m.m[8 + i];
        a.r[4 * i + 3] = m.m[12 + i];
    }
    return a;
}
V3 ld3(const float *p) { return v3(p[0], p[1], p[2]); }

// src/aabb.h:29-58
void transform_aabb(V3 bmin, V3 bmax, const M4 &model, V3 &omin, V3 &omax)
{
    Affine a = rows_of(model);
    V3 c[8] = {v3(bmin.x, bmin.y, bmin.z), v3(bmax.x, bmin.y, bmin.z), v3(bmax.x, bmin.y, bmax.z),
        v3(bmin.x, bmin.y, bmax.z), v3(bmin.x, bmax.y, bmin.z), v3(bmax.x, bmax.y, bmin.z),
        v3(bmax.x, bmax.y, bmax.z), v3(bmin.x, bmax.y, bmax.z)};
    V3 lo = transform_point(a, c[0]), hi = lo;
    for (int i = 1; i < 8; i++) {
        V3 t = transform_point(a, c[i]);
        lo = vmin(lo, t);
        hi = vmax(hi, t);
    }
    omin = lo;
    omax = hi;
}

int check_stream_status(gbsp_runtime *rt)
{
    uint32_t st = 0;
    GBSP_CUDA_TRY(cudaMemcpyAsync(&st, rt->dStatus, 4, cudaMemcpyDeviceToHost, rt->stream));
    GBSP_CUDA_TRY(cudaStreamSynchronize(rt->stream));
    if (st) {
        GBSP_CUDA_TRY(cudaMemsetAsync(rt->dStatus, 0, 4, rt->stream));
        return set_error(GBSP_ERR_DEVICE_STATUS,
            "device status 0x%x (1 = traversal stack overflow, 2 = queue overflow, 4 = bad index, "
            "8 = build capacity, 16 = per-ray step cap)",
            st);
    }
    return GBSP_OK;
}

}  // namespace

int resolve_material(const gbsp_material_system *ms, uint32_t id)
{
    for (size_t i = 0; i < ms->keys.size(); i++)
        if (ms->keys[i] == id) return (int)i;  // first match, src/sp_material_system.cpp:15-28
    return -1;
}

static int resolve_texture(const gbsp_material_system *ms, uint32_t id)
{
    for (size_t i = 0; i < ms->textureKeys.size(); i++)
        if (ms->textureKeys[i] == id) return (int)i;
    return -1;
}

int material_view(gbsp_material_system *ms, MaterialView *out)
{
    cudaStream_t s = ms->rt->stream;
    int rc;
    if (ms->dirty) {
        std::vector<DeviceMaterial> dm(ms->materials.size());
        for (size_t i = 0; i < dm.size(); i++) {
            const gbsp_material &m = ms->materials[i];
            DeviceMaterial &d = dm[i];
            memset(&d, 0, sizeof(d));
            memcpy(d.albedo, m.albedo, 12);
            memcpy(d.emission, m.emission, 12);
            d.roughness = m.roughness;
            d.albedoTex = resolve_texture(ms, m.albedoTexture);
            int et = resolve_texture(ms, m.emissionTexture);
            if (et < 0 && m.emissionTexture == kSkyTexture && ms->haveSky) et = -2;
            d.emissionTex = et;
            d.present = 1;
        }
        std::vector<TextureDesc> td(ms->texturePixels.size());
        uint64_t off = 0;
        for (size_t i = 0; i < td.size(); i++) {
            td[i].offset = off;
            td[i].width = ms->textureW[i];
            td[i].height = ms->textureH[i];
            off += (uint64_t)ms->textureW[i] * ms->textureH[i];
        }
        std::vector<float4> texels(off ? off : 1);
        for (size_t i = 0; i < td.size(); i++)
            memcpy(texels.data() + td[i].offset, ms->texturePixels[i].data(),
                ms->texturePixels[i].size() * sizeof(float));
        if ((rc = ms->dMaterials.upload(dm.data(), dm.size(), s)) ||
            (rc = ms->dTextures.upload(td.data(), td.size(), s)) ||
            (rc = ms->dTexels.upload(texels.data(), texels.size(), s)))
            return rc;
        GBSP_CUDA_TRY(cudaStreamSynchronize(s));
        ms->dirty = false;
    }
    out->materials = ms->dMaterials.ptr;
    out->materialCount = (uint32_t)ms->materials.size();
    out->texels = ms->dTexels.ptr;
    out->textures = ms->dTextures.ptr;
    out->textureCount = (uint32_t)ms->texturePixels.size();
    out->backgroundSlot = resolve_material(ms, ms->backgroundId);
    out->sky = ms->sky;
    out->haveSky = ms->haveSky ? 1u : 0u;
    out->instanceSlot = nullptr;
    return GBSP_OK;
}

}  // namespace gbsp

using namespace gbsp;

extern "C" {

const char *gbsp_last_error_string(void) { return gbsp::g_error; }
int gbsp_version(void) { return GBSP_VERSION; }

void gbsp_options_default(gbsp_options *opt)
{
    if (!opt) return;
    memset(opt, 0, sizeof(*opt));
    opt->spp = 1;
    opt->max_bounces = 3;
    opt->seed = 0;
    opt->rng_mode = GBSP_RNG_HASH_PER_SAMPLE;
    opt->nan_policy = GBSP_NAN_ZERO;
    opt->radiance_clamp = 10.0f;
    opt->wave_paths = 0;
}

int gbsp_runtime_create(int device, void *stream, gbsp_runtime **out)
{
    if (!out) return set_error(GBSP_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return set_error(GBSP_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    if (device < 0 || device >= n)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "device %d of %d", device, n);
    GBSP_CUDA_TRY(cudaSetDevice(device));
    gbsp_runtime *rt = new gbsp_runtime();
    rt->device = device;
    if (stream) {
        rt->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&rt->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete rt;
            return cuda_error(e, "cudaStreamCreate");
        }
        rt->ownsStream = true;
    }
    cudaDeviceGetAttribute(&rt->smCount, cudaDevAttrMultiProcessorCount, device);
    e = cudaMalloc((void **)&rt->dStatus, 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&rt->dCounters, sizeof(unsigned long long) * (GBSP_METRIC_COUNT + 16));
    if (e == cudaSuccess) e = cudaMemset(rt->dStatus, 0, 4);
    if (e == cudaSuccess) e = cudaMemset(rt->dCounters, 0, sizeof(unsigned long long) * (GBSP_METRIC_COUNT + 16));
    if (e != cudaSuccess) {
        gbsp_runtime_destroy(rt);
        return cuda_error(e, "runtime allocation");
    }
    for (auto &ev : rt->ev) cudaEventCreate(&ev);
    *out = rt;
    return GBSP_OK;
}

}  // extern "C"

static std::mutex g_runtimeMutex;

static void runtime_teardown(gbsp_runtime *rt)
{
    cudaStreamSynchronize(rt->stream);
    rt->rayO.release();
    rt->rayD.release();
    rt->hitA.release();
    rt->hitInst.release();
    rt->vertE.release();
    rt->vertA.release();
    rt->pathRad.release();
    rt->queueCounts.release();
    rt->frame.release();
    rt->aov.release();
    rt->pathAov.release();
    rt->sortHist.release();
    cudaStreamSynchronize(rt->stream);
    if (rt->dStatus) cudaFree(rt->dStatus);
    if (rt->dCounters) cudaFree(rt->dCounters);
    for (auto &ev : rt->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : rt->evPool) cudaEventDestroy(ev);
    if (rt->ownsStream) cudaStreamDestroy(rt->stream);
    delete rt;
}

// Drops one reference; the last one tears the runtime down.
void gbsp::runtime_release(gbsp_runtime *rt)
{
    bool last;
    {
        std::lock_guard<std::mutex> lock(g_runtimeMutex);
        last = --rt->refs == 0;
    }
    if (last) runtime_teardown(rt);
}

int gbsp::runtime_retain(gbsp_runtime *rt)
{
    std::lock_guard<std::mutex> lock(g_runtimeMutex);
    if (rt->closed) return set_error(GBSP_ERR_INVALID_ARGUMENT, "runtime already destroyed");
    rt->refs++;
    return GBSP_OK;
}

extern "C" {

int gbsp_runtime_destroy(gbsp_runtime *rt)
{
    if (!rt) return GBSP_OK;
    {
        std::lock_guard<std::mutex> lock(g_runtimeMutex);
        if (rt->closed) return set_error(GBSP_ERR_INVALID_ARGUMENT, "runtime destroyed twice");
        rt->closed = true;
    }
    runtime_release(rt);
    return GBSP_OK;
}

int gbsp_runtime_synchronize(gbsp_runtime *rt)
{
    if (!rt) return set_error(GBSP_ERR_INVALID_ARGUMENT, "runtime is NULL");
    GBSP_CUDA_TRY(cudaStreamSynchronize(rt->stream));
    return check_stream_status(rt);
}

void *gbsp_runtime_stream(gbsp_runtime *rt) { return rt ? (void *)rt->stream : nullptr; }

// ---- camera -----------------------------------------------------------------
int gbsp_configure_camera(gbsp_camera *camera, gbsp_image_plane *imagePlane,
    const float position[3], const float rotation[4], float filmDistance)
{
    if (!camera || !imagePlane || !position || !rotation)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument to gbsp_configure_camera");
    Q4 q = {rotation[0], rotation[1], rotation[2], rotation[3]};
    V3 pos = ld3(position);
    camera->imagePlane = imagePlane;
    memcpy(camera->position, position, 12);
    V3 r = rotate_vector(v3(1, 0, 0), q);
    V3 u = rotate_vector(v3(0, 1, 0), q);
    V3 f = rotate_vector(v3(0, 0, -1), q);
    V3 fc = add(pos, mul(f, filmDistance));
    memcpy(camera->right, &r, 12);
    memcpy(camera->up, &u, 12);
    memcpy(camera->forward, &f, 12);
    memcpy(camera->filmCenter, &fc, 12);
    camera->halfPixelWidth = 0.5f / (float)imagePlane->width;
    camera->halfPixelHeight = 0.5f / (float)imagePlane->height;
    float fw = 1.0f, fh = 1.0f;
    if (imagePlane->width > imagePlane->height)
        fh = (float)imagePlane->height / (float)imagePlane->width;
    else if (imagePlane->width < imagePlane->height)
        fw = (float)imagePlane->width / (float)imagePlane->height;
    camera->halfFilmWidth = 0.5f * fw;
    camera->halfFilmHeight = 0.5f * fh;
    return GBSP_OK;
}

static CameraParams camera_params(const gbsp_camera *c)
{
    CameraParams p;
    p.right = ld3(c->right);
    p.up = ld3(c->up);
    p.forward = ld3(c->forward);
    p.position = ld3(c->position);
    p.filmCenter = ld3(c->filmCenter);
    p.halfPixelWidth = c->halfPixelWidth;
    p.halfPixelHeight = c->halfPixelHeight;
    p.halfFilmWidth = c->halfFilmWidth;
    p.halfFilmHeight = c->halfFilmHeight;
    p.width = c->imagePlane ? c->imagePlane->width : 0;
    p.height = c->imagePlane ? c->imagePlane->height : 0;
    return p;
}

uint32_t gbsp_calculate_film_positions(const gbsp_camera *camera, float *filmPositions,
    const float *pixelPositions, uint32_t count)
{
    if (!camera || !camera->imagePlane || !filmPositions || !pixelPositions) return 0;
    CameraParams p = camera_params(camera);
    for (uint32_t i = 0; i < count; i++) {
        V3 f = film_position(p, pixelPositions[2 * i], pixelPositions[2 * i + 1]);
        memcpy(filmPositions + 3 * i, &f, 12);
    }
    return count;
}

uint32_t gbsp_sample_seed(uint32_t seed, uint32_t x, uint32_t y, uint32_t sample)
{
    return sample_seed(seed, x, y, sample);
}

// ---- scene --------------------------------------------------------------------
int gbsp_scene_create(gbsp_runtime *rt, gbsp_scene **out)
{
    if (!rt || !out) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = runtime_retain(rt);
    if (rc) return rc;
    gbsp_scene *s = new gbsp_scene();
    s->rt = rt;
    *out = s;
    return GBSP_OK;
}

int gbsp_scene_set_intersection(gbsp_scene *scene, uint32_t mode)
{
    if (!scene) return set_error(GBSP_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (mode != GBSP_ISECT_REFERENCE_MT && mode != GBSP_ISECT_WATERTIGHT)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "unknown intersection mode %u", mode);
    scene->isectMode = mode;
    return GBSP_OK;
}

int gbsp_scene_set_node_width(gbsp_scene *scene, uint32_t width)
{
    if (!scene) return set_error(GBSP_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (width != 4 && width != 8)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "node width %u (4 or 8)", width);
    scene->nodeWidth = width;
    return GBSP_OK;
}

uint32_t gbsp_scene_node_width(const gbsp_scene *scene)
{
    return scene ? scene->nodeWidth : 0u;
}

int gbsp_scene_destroy(gbsp_scene *scene)
{
    if (!scene) return GBSP_OK;
    gbsp_runtime *rt = scene->rt;
    cudaStreamSynchronize(rt->stream);
    delete scene;  // device buffers are freed in stream order on rt's stream
    runtime_release(rt);
    return GBSP_OK;
}

}  // extern "C"

// Grows a device buffer to hold used + extra elements, keeping the first used.
template <typename T>
static int append_device(DeviceBuffer<T> &buf, size_t used, size_t extra, cudaStream_t s)
{
    if (used + extra <= buf.count && buf.ptr) return GBSP_OK;
    DeviceBuffer<T> grown;
    int rc = grown.reserve((used + extra) * 3 / 2 + 16, s);
    if (rc) return rc;
    if (used) GBSP_CUDA_TRY(cudaMemcpyAsync(grown.ptr, buf.ptr, used * sizeof(T), cudaMemcpyDeviceToDevice, s));
    buf.release();
    buf.ptr = grown.ptr;
    buf.count = grown.count;
    buf.stream = s;
    grown.ptr = nullptr;
    grown.count = 0;
    return GBSP_OK;
}

extern "C" {

int gbsp_create_mesh(gbsp_scene *scene, const gbsp_vertex *vertices, uint32_t vertexCount,
    const uint32_t *indices, uint32_t indexCount, int useSmoothShading, uint32_t *meshOut)
{
    if (!scene || !vertices || !indices || vertexCount == 0)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL or empty mesh");
    if (indexCount == 0 || indexCount % 3 != 0)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "index count %u is not a positive multiple of 3",
            indexCount);
    for (uint32_t i = 0; i < indexCount; i++)
        if (indices[i] >= vertexCount)
            return set_error(GBSP_ERR_INVALID_ARGUMENT, "index %u = %u out of range (%u vertices)", i,
                indices[i], vertexCount);
    gbsp_runtime *rt = scene->rt;
    cudaStream_t s = rt->stream;
    uint32_t triCount = indexCount / 3;
    if (scene->triCount + triCount >= (1ull << 28))
        return set_error(GBSP_ERR_CAPACITY, "more than 2^28 triangles in one scene");
    int rc;
    DeviceBuffer<gbsp_vertex> dv;
    DeviceBuffer<uint32_t> di, order;
    DeviceBuffer<float4> lo, hi;
    if ((rc = dv.upload(vertices, vertexCount, s)) || (rc = di.upload(indices, indexCount, s)) ||
        (rc = lo.reserve(triCount, s)) || (rc = hi.reserve(triCount, s)))
        return rc;
    if ((rc = mesh_prepare(s, dv.ptr, di.ptr, triCount, lo.ptr, hi.ptr))) return rc;
    // the object BVH lives after the mesh nodes and is rebuilt on commit
    scene->committed = false;
    for (int w = 0; w < kNodeWidths; w++) scene->tlasRoot[w] = kEmptyChild;
    const uint32_t nodeBase[kNodeWidths] = {scene->meshNodeCount[0], scene->meshNodeCount[1]};
    WideTree trees[kNodeWidths];
    // triangle boxes on the host too (the same min/max as k_mesh_prepare), for
    // the host SAH build
    std::vector<float4> hlo(triCount), hhi(triCount);
    for (uint32_t t = 0; t < triCount; t++) {
        V3 a = ld3(vertices[indices[3 * t]].position), b = ld3(vertices[indices[3 * t + 1]].position),
           c = ld3(vertices[indices[3 * t + 2]].position);
        V3 mn = vmin(a, vmin(b, c)), mx = vmax(a, vmax(b, c));
        hlo[t] = make_float4(mn.x, mn.y, mn.z, 0.0f);
        hhi[t] = make_float4(mx.x, mx.y, mx.z, 0.0f);
    }
    if ((rc = build_wide_bvh(s, lo.ptr, hi.ptr, triCount, kMaxLeafPrims, scene->nodes, nodeBase,
             trees, &order, rt->dStatus, hlo.data(), hhi.data())))
        return rc;
    uint64_t triBase = scene->triCount;
    if ((rc = append_device(scene->tris, triBase, triCount, s)) ||
        (rc = append_device(scene->attrs, triBase, triCount, s)) ||
        (rc = append_device(scene->triIds, triBase, triCount, s)))
        return rc;
    if ((rc = mesh_emit(s, dv.ptr, di.ptr, triCount, order.ptr, scene->tris.ptr + triBase,
             scene->attrs.ptr + triBase, scene->triIds.ptr + triBase, (uint32_t)triBase)))
        return rc;
    for (int w = 0; w < kNodeWidths; w++)
        if ((rc = offset_nodes(s, scene->nodes[w], trees[w].nodeCount, nodeBase[w],
                 (uint32_t)triBase)))
            return rc;
    gbsp_mesh_info mi;
    for (int w = 0; w < kNodeWidths; w++) {
        mi.rootNode[w] = nodeBase[w];
        mi.nodeCount[w] = trees[w].nodeCount;
        mi.depth[w] = trees[w].depth;
    }
    mi.triFirst = (uint32_t)triBase;
    mi.triCount = triCount;
    mi.smooth = useSmoothShading != 0;
    // vertex AABB over all vertices (src/sp_scene.cpp:57-75)
    V3 mn = ld3(vertices[0].position), mx = mn;
    for (uint32_t i = 1; i < vertexCount; i++) {
        mn = vmin(mn, ld3(vertices[i].position));
        mx = vmax(mx, ld3(vertices[i].position));
    }
    memcpy(mi.aabbMin, &mn, 12);
    memcpy(mi.aabbMax, &mx, 12);
    scene->meshes.push_back(mi);
    for (int w = 0; w < kNodeWidths; w++) {
        scene->meshNodeCount[w] += trees[w].nodeCount;
        scene->maxDepth[w] = std::max(scene->maxDepth[w], trees[w].depth);
    }
    scene->triCount += triCount;
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    if (meshOut) *meshOut = (uint32_t)scene->meshes.size() - 1;
    return check_stream_status(rt);
}

int gbsp_add_object_to_scene(gbsp_scene *scene, uint32_t mesh, uint32_t material,
    const float position[3], const float orientation[4], const float scale[3])
{
    if (!scene || !position || !orientation || !scale)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (mesh >= scene->meshes.size())
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "mesh %u of %zu", mesh, scene->meshes.size());
    gbsp_object_info o;
    o.mesh = mesh;
    o.material = material;
    memcpy(o.position, position, 12);
    memcpy(o.rotation, orientation, 16);
    memcpy(o.scale, scale, 12);
    V3 p = ld3(position), sc = ld3(scale);
    Q4 q = {orientation[0], orientation[1], orientation[2], orientation[3]};
    // src/sp_scene.cpp:77-117
    M4 model = m4_mul(m4_mul(m4_translate(p), m4_rotate(q)), m4_scale(sc));
    M4 inv = m4_mul(m4_mul(m4_scale(inverse(sc)), m4_rotate(quat_conj(q))), m4_translate(neg(p)));
    const gbsp_mesh_info &mi = scene->meshes[mesh];
    V3 lo, hi;
    transform_aabb(ld3(mi.aabbMin), ld3(mi.aabbMax), model, lo, hi);
    Instance &in = o.inst;
    memset(&in, 0, sizeof(in));
    in.inv = rows_of(inv);
    in.model = rows_of(model);
    memcpy(in.lo, &lo, 12);
    memcpy(in.hi, &hi, 12);
    in.blasRoot = mi.rootNode[0];  // per width when the instances are uploaded
    in.materialId = material;
    in.objectIndex = (uint32_t)scene->objects.size();
    in.smooth = mi.smooth ? 1u : 0u;
    scene->objects.push_back(o);
    scene->committed = false;
    return GBSP_OK;
}

int gbsp_clear_objects(gbsp_scene *scene)
{
    if (!scene) return set_error(GBSP_ERR_INVALID_ARGUMENT, "scene is NULL");
    scene->objects.clear();
    scene->committed = false;
    return GBSP_OK;
}

int gbsp_build_scene_broadphase(gbsp_scene *scene)
{
    if (!scene) return set_error(GBSP_ERR_INVALID_ARGUMENT, "scene is NULL");
    gbsp_runtime *rt = scene->rt;
    cudaStream_t s = rt->stream;
    uint32_t n = (uint32_t)scene->objects.size();
    for (int w = 0; w < kNodeWidths; w++) {
        scene->totalNodeCount[w] = scene->meshNodeCount[w];
        scene->tlasRoot[w] = kEmptyChild;
        scene->tlasDepth[w] = 0;
    }
    if (n == 0) {
        scene->committed = true;
        return GBSP_OK;
    }
    std::vector<float4> lo(n), hi(n);
    for (uint32_t i = 0; i < n; i++) {
        const Instance &in = scene->objects[i].inst;
        lo[i] = make_float4(in.lo[0], in.lo[1], in.lo[2], 0.0f);
        hi[i] = make_float4(in.hi[0], in.hi[1], in.hi[2], 0.0f);
    }
    int rc;
    DeviceBuffer<float4> dlo, dhi;
    DeviceBuffer<uint32_t> order;
    if ((rc = dlo.upload(lo.data(), n, s)) || (rc = dhi.upload(hi.data(), n, s))) return rc;
    WideTree trees[kNodeWidths];
    if ((rc = build_wide_bvh(s, dlo.ptr, dhi.ptr, n, 1, scene->nodes, scene->meshNodeCount, trees,
             &order, rt->dStatus, lo.data(), hi.data())))
        return rc;
    for (int w = 0; w < kNodeWidths; w++)
        if ((rc = offset_nodes(s, scene->nodes[w], trees[w].nodeCount, scene->meshNodeCount[w], 0)))
            return rc;
    std::vector<uint32_t> ord(n);
    GBSP_CUDA_TRY(cudaMemcpyAsync(ord.data(), order.ptr, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<Instance> inst(n);
    for (uint32_t j = 0; j < n; j++)
        if (ord[j] >= n) return set_error(GBSP_ERR_DEVICE_STATUS, "object order out of range");
    for (int w = 0; w < kNodeWidths; w++) {
        for (uint32_t j = 0; j < n; j++) {
            const gbsp_object_info &o = scene->objects[ord[j]];
            inst[j] = o.inst;
            inst[j].blasRoot = scene->meshes[o.mesh].rootNode[w];
        }
        if ((rc = scene->instances[w].upload(inst.data(), n, s))) return rc;
        scene->tlasRoot[w] = scene->meshNodeCount[w];
        scene->tlasDepth[w] = trees[w].depth;
        scene->totalNodeCount[w] = scene->meshNodeCount[w] + trees[w].nodeCount;
    }
    scene->leafOrder = ord;
    scene->committed = true;
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    return check_stream_status(rt);
}

int gbsp_scene_info(const gbsp_scene *scene, uint32_t *objects, uint64_t *triangles,
    uint32_t *meshNodes, uint32_t *maxDepth)
{
    if (!scene) return set_error(GBSP_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (objects) *objects = (uint32_t)scene->objects.size();
    if (triangles) {
        uint64_t t = 0;
        for (const auto &o : scene->objects) t += scene->meshes[o.mesh].triCount;
        *triangles = t;
    }
    int w = width_index(scene->nodeWidth);
    if (meshNodes) *meshNodes = scene->meshNodeCount[w];
    if (maxDepth) *maxDepth = scene->maxDepth[w] + scene->tlasDepth[w];
    return GBSP_OK;
}

// ---- queries ---------------------------------------------------------------------
static int need_committed(const gbsp_scene *scene)
{
    if (!scene) return set_error(GBSP_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (!scene->committed)
        return set_error(GBSP_ERR_NOT_READY,
            "scene changed since gbsp_build_scene_broadphase (call it before querying)");
    return GBSP_OK;
}

static int counters_begin(gbsp_runtime *rt, bool stageTiming = false)
{
    rt->begin_call(stageTiming);
    GBSP_CUDA_TRY(cudaMemsetAsync(rt->dCounters, 0, sizeof(unsigned long long) * GBSP_METRIC_COUNT,
        rt->stream));
    return GBSP_OK;
}

static int counters_end(gbsp_runtime *rt, gbsp_metrics *metrics, float elapsedMs)
{
    if (!metrics) return GBSP_OK;
    unsigned long long c[GBSP_METRIC_COUNT];
    GBSP_CUDA_TRY(cudaMemcpyAsync(c, rt->dCounters, sizeof(c), cudaMemcpyDeviceToHost, rt->stream));
    GBSP_CUDA_TRY(cudaStreamSynchronize(rt->stream));
    for (int i = 0; i < GBSP_METRIC_COUNT; i++) metrics->values[i] += c[i];
    metrics->values[GBSP_METRIC_ELAPSED_NS] += (uint64_t)((double)elapsedMs * 1.0e6);
    metrics->values[GBSP_METRIC_KERNEL_LAUNCHES] += rt->launches;
    metrics->values[GBSP_METRIC_TRACE_LAUNCHES] += rt->traceLaunches;
    double traceMs = 0.0, shadeMs = 0.0;
    for (auto &sp : rt->traceSpans) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt->evPool[sp.first], rt->evPool[sp.second]) == cudaSuccess)
            traceMs += ms;
    }
    for (auto &sp : rt->shadeSpans) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, rt->evPool[sp.first], rt->evPool[sp.second]) == cudaSuccess)
            shadeMs += ms;
    }
    metrics->values[GBSP_METRIC_INTERSECT_SCENE_NS] += (uint64_t)(traceMs * 1.0e6);
    metrics->values[GBSP_METRIC_SHADE_NS] += (uint64_t)(shadeMs * 1.0e6);
    return GBSP_OK;
}

int gbsp_intersect_closest_device(gbsp_scene *scene, uint32_t count, const float *rays,
    float *tOut, int32_t *triangleOut, int32_t *objectOut)
{
    int rc = need_committed(scene);
    if (rc) return rc;
    if (count && !rays) return set_error(GBSP_ERR_INVALID_ARGUMENT, "rays is NULL");
    if (((uintptr_t)rays & 15u) != 0)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "rays must be 16-byte aligned");
    gbsp_runtime *rt = scene->rt;
    if ((rc = counters_begin(rt))) return rc;
    return launch_intersect(rt->stream, scene->view(), count, reinterpret_cast<const float4 *>(rays),
        tOut, triangleOut, objectOut, nullptr, nullptr, nullptr, rt->smCount, rt->dCounters,
        rt->dStatus);
}

int gbsp_ray_intersect_scene(gbsp_scene *scene, uint32_t count, const float *rays, float *resultOut,
    uint32_t *materialOut, gbsp_metrics *metrics)
{
    int rc = need_committed(scene);
    if (rc) return rc;
    if (count == 0) return GBSP_OK;
    if (!rays || !resultOut) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    gbsp_runtime *rt = scene->rt;
    cudaStream_t s = rt->stream;
    std::vector<float4> packed(2 * (size_t)count);
    for (uint32_t i = 0; i < count; i++) {
        const float *r = rays + 6 * (size_t)i;
        packed[2 * i] = make_float4(r[0], r[1], r[2], 0.0f);
        packed[2 * i + 1] = make_float4(r[3], r[4], r[5], 0.0f);
    }
    DeviceBuffer<float4> dr;
    DeviceBuffer<float> dattr;
    DeviceBuffer<uint32_t> dmat;
    if ((rc = dr.upload(packed.data(), packed.size(), s)) ||
        (rc = dattr.reserve(6 * (size_t)count, s)) || (rc = dmat.reserve(count, s)))
        return rc;
    if ((rc = counters_begin(rt))) return rc;
    GBSP_CUDA_TRY(cudaEventRecord(rt->ev[0], s));
    if ((rc = launch_intersect(s, scene->view(), count, dr.ptr, nullptr, nullptr, nullptr, dattr.ptr,
             dmat.ptr, nullptr, rt->smCount, rt->dCounters, rt->dStatus)))
        return rc;
    GBSP_CUDA_TRY(cudaEventRecord(rt->ev[1], s));
    GBSP_CUDA_TRY(cudaMemcpyAsync(resultOut, dattr.ptr, 24 * (size_t)count, cudaMemcpyDeviceToHost, s));
    if (materialOut)
        GBSP_CUDA_TRY(cudaMemcpyAsync(materialOut, dmat.ptr, 4 * (size_t)count, cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, rt->ev[0], rt->ev[1]);
    if ((rc = counters_end(rt, metrics, ms))) return rc;
    return check_stream_status(rt);
}

// ---- materials ------------------------------------------------------------------------
int gbsp_material_system_create(gbsp_runtime *rt, gbsp_material_system **out)
{
    if (!rt || !out) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = runtime_retain(rt);
    if (rc) return rc;
    gbsp_material_system *ms = new gbsp_material_system();
    ms->rt = rt;
    *out = ms;
    return GBSP_OK;
}

int gbsp_material_system_destroy(gbsp_material_system *ms)
{
    if (!ms) return GBSP_OK;
    gbsp_runtime *rt = ms->rt;
    cudaStreamSynchronize(rt->stream);
    delete ms;
    runtime_release(rt);
    return GBSP_OK;
}

int gbsp_register_material(gbsp_material_system *ms, const gbsp_material *material, uint32_t id)
{
    if (!ms || !material) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (ms->materials.size() >= (1u << 24))
        return set_error(GBSP_ERR_CAPACITY, "material registry full");
    ms->keys.push_back(id);
    ms->materials.push_back(*material);
    ms->dirty = true;
    return GBSP_OK;
}

int gbsp_register_texture(gbsp_material_system *ms, const float *rgba, uint32_t width,
    uint32_t height, uint32_t id)
{
    if (!ms || !rgba || !width || !height)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL or empty texture");
    ms->textureKeys.push_back(id);
    ms->texturePixels.emplace_back(rgba, rgba + (size_t)width * height * 4);
    ms->textureW.push_back(width);
    ms->textureH.push_back(height);
    ms->dirty = true;
    return GBSP_OK;
}

int gbsp_set_background_material(gbsp_material_system *ms, uint32_t id)
{
    if (!ms) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    ms->backgroundId = id;
    return GBSP_OK;
}

int gbsp_set_procedural_sky(gbsp_material_system *ms, const float params[13])
{
    if (!ms || !params) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    ms->sky.bottom = ld3(params);
    ms->sky.top = ld3(params + 3);
    ms->sky.sunDir = ld3(params + 6);
    ms->sky.cosSunRadius = params[9];
    ms->sky.sunRadiance = ld3(params + 10);
    ms->haveSky = true;
    ms->dirty = true;
    return GBSP_OK;
}

// ---- path tracing --------------------------------------------------------------------------
static int prepare_render(const gbsp_context *ctx, gbsp_options &opt, MaterialView &mv,
    DeviceBuffer<int32_t> &slots)
{
    if (!ctx || !ctx->camera || !ctx->camera->imagePlane || !ctx->scene || !ctx->materialSystem ||
        !ctx->runtime)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "incomplete context");
    if (ctx->options)
        opt = *ctx->options;
    else
        gbsp_options_default(&opt);
    int rc = need_committed(ctx->scene);
    if (rc) return rc;
    if (ctx->scene->rt != ctx->runtime || ctx->materialSystem->rt != ctx->runtime)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "scene, materials and context use different runtimes");
    if ((rc = material_view(ctx->materialSystem, &mv))) return rc;
    const gbsp_scene *sc = ctx->scene;
    std::vector<int32_t> hs(std::max<size_t>(1, sc->objects.size()), -1);
    for (size_t j = 0; j < sc->leafOrder.size(); j++)
        hs[j] = resolve_material(ctx->materialSystem, sc->objects[sc->leafOrder[j]].material);
    if ((rc = slots.upload(hs.data(), hs.size(), ctx->runtime->stream))) return rc;
    mv.instanceSlot = slots.ptr;
    return GBSP_OK;
}

static int ensure_frame(gbsp_runtime *rt, uint32_t w, uint32_t h, bool aov = false)
{
    int rc = rt->frame.reserve((size_t)w * h, rt->stream);
    if (rc) return rc;
    if (aov && (rc = rt->aov.reserve(2 * (size_t)w * h, rt->stream))) return rc;
    rt->frameW = w;
    rt->frameH = h;
    return GBSP_OK;
}

static float4 *aov_target(gbsp_runtime *rt, const gbsp_options &opt)
{
    return (opt.flags & GBSP_FLAG_AOV) ? rt->aov.ptr : nullptr;
}

int gbsp_path_trace_tile(const gbsp_context *ctx, gbsp_tile tile, gbsp_rng *rng,
    gbsp_metrics *metrics)
{
    gbsp_options opt;
    MaterialView mv;
    DeviceBuffer<int32_t> slots;
    int rc = prepare_render(ctx, opt, mv, slots);
    if (rc) return rc;
    gbsp_runtime *rt = ctx->runtime;
    cudaStream_t s = rt->stream;
    gbsp_image_plane *ip = ctx->camera->imagePlane;
    uint32_t x0 = tile.minX, y0 = tile.minY;
    uint32_t x1 = std::min(tile.maxX, ip->width), y1 = std::min(tile.maxY, ip->height);
    if ((rc = ensure_frame(rt, ip->width, ip->height, (opt.flags & GBSP_FLAG_AOV) != 0))) return rc;
    if ((rc = counters_begin(rt, (opt.flags & GBSP_FLAG_STAGE_TIMING) != 0))) return rc;
    GBSP_CUDA_TRY(cudaEventRecord(rt->ev[0], s));
    bool seq = opt.rng_mode == GBSP_RNG_TILE_SEQUENTIAL;
    if (seq && !rng) return set_error(GBSP_ERR_INVALID_ARGUMENT, "tile-sequential mode needs an RNG");
    if (x1 > x0 && y1 > y0) {
        if ((rc = render_frame(rt, ctx->scene->view(), mv, camera_params(ctx->camera), opt, x0, y0,
                 x1, y1, rt->frame.ptr, ip->width, seq ? &rng->state : nullptr,
                 seq ? nullptr : aov_target(rt, opt))))
            return rc;
    }
    GBSP_CUDA_TRY(cudaEventRecord(rt->ev[1], s));
    if (ip->pixels && x1 > x0 && y1 > y0) {
        size_t pitch = (size_t)ip->width * sizeof(float4);
        GBSP_CUDA_TRY(cudaMemcpy2DAsync(ip->pixels + 4 * ((size_t)y0 * ip->width + x0), pitch,
            rt->frame.ptr + (size_t)y0 * ip->width + x0, pitch, (size_t)(x1 - x0) * sizeof(float4),
            y1 - y0, cudaMemcpyDeviceToHost, s));
    }
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, rt->ev[0], rt->ev[1]);
    if ((rc = counters_end(rt, metrics, ms))) return rc;
    return check_stream_status(rt);
}

int gbsp_path_trace_tile_split(const gbsp_context *ctx, gbsp_tile tile, uint32_t firstSpp,
    float *deviceImage2, gbsp_metrics *metrics)
{
    if (!deviceImage2) return set_error(GBSP_ERR_INVALID_ARGUMENT, "deviceImage2 is NULL");
    gbsp_options opt;
    MaterialView mv;
    DeviceBuffer<int32_t> slots;
    int rc = prepare_render(ctx, opt, mv, slots);
    if (rc) return rc;
    if (opt.rng_mode != GBSP_RNG_HASH_PER_SAMPLE)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "split renders seed hash-per-sample only");
    if (firstSpp == 0 || firstSpp >= (opt.spp ? opt.spp : 1u))
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "first spp %u of %u", firstSpp, opt.spp);
    gbsp_runtime *rt = ctx->runtime;
    cudaStream_t s = rt->stream;
    gbsp_image_plane *ip = ctx->camera->imagePlane;
    uint32_t x0 = tile.minX, y0 = tile.minY;
    uint32_t x1 = std::min(tile.maxX, ip->width), y1 = std::min(tile.maxY, ip->height);
    if ((rc = ensure_frame(rt, ip->width, ip->height, (opt.flags & GBSP_FLAG_AOV) != 0))) return rc;
    if ((rc = counters_begin(rt, (opt.flags & GBSP_FLAG_STAGE_TIMING) != 0))) return rc;
    GBSP_CUDA_TRY(cudaEventRecord(rt->ev[0], s));
    if (x1 > x0 && y1 > y0 &&
        (rc = render_frame(rt, ctx->scene->view(), mv, camera_params(ctx->camera), opt, x0, y0, x1,
             y1, rt->frame.ptr, ip->width, nullptr, aov_target(rt, opt), firstSpp,
             reinterpret_cast<float4 *>(deviceImage2))))
        return rc;
    GBSP_CUDA_TRY(cudaEventRecord(rt->ev[1], s));
    if (ip->pixels && x1 > x0 && y1 > y0) {
        size_t pitch = (size_t)ip->width * sizeof(float4);
        GBSP_CUDA_TRY(cudaMemcpy2DAsync(ip->pixels + 4 * ((size_t)y0 * ip->width + x0), pitch,
            rt->frame.ptr + (size_t)y0 * ip->width + x0, pitch, (size_t)(x1 - x0) * sizeof(float4),
            y1 - y0, cudaMemcpyDeviceToHost, s));
    }
    if (!metrics && !ip->pixels) return GBSP_OK;
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, rt->ev[0], rt->ev[1]);
    if ((rc = counters_end(rt, metrics, ms))) return rc;
    return check_stream_status(rt);
}

static int tile_list(const gbsp_context *ctx, const gbsp_tile *tiles, const uint32_t *spp,
    uint32_t count, gbsp_metrics *metrics)
{
    if (count && !tiles) return set_error(GBSP_ERR_INVALID_ARGUMENT, "tiles is NULL");
    gbsp_options opt;
    MaterialView mv;
    DeviceBuffer<int32_t> slots;
    int rc = prepare_render(ctx, opt, mv, slots);
    if (rc) return rc;
    if (opt.rng_mode != GBSP_RNG_HASH_PER_SAMPLE)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "tile lists render hash-per-sample only");
    if (opt.flags & GBSP_FLAG_AOV)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "tile lists write no G-buffers (GBSP_FLAG_AOV)");
    gbsp_runtime *rt = ctx->runtime;
    cudaStream_t s = rt->stream;
    gbsp_image_plane *ip = ctx->camera->imagePlane;
    std::vector<uint4> rects;
    std::vector<uint32_t> rectSpp;
    rects.reserve(count);
    for (uint32_t i = 0; i < count; i++) {
        uint32_t x0 = tiles[i].minX, y0 = tiles[i].minY;
        uint32_t x1 = std::min(tiles[i].maxX, ip->width), y1 = std::min(tiles[i].maxY, ip->height);
        if (x1 <= x0 || y1 <= y0 || (spp && spp[i] == 0)) continue;
        rects.push_back(make_uint4(x0, y0, x1 - x0, y1 - y0));
        if (spp) rectSpp.push_back(spp[i]);
    }
    if ((rc = ensure_frame(rt, ip->width, ip->height))) return rc;
    rt->begin_call(false);
    if (metrics && (rc = counters_begin(rt, (opt.flags & GBSP_FLAG_STAGE_TIMING) != 0))) return rc;
    if (metrics) GBSP_CUDA_TRY(cudaEventRecord(rt->ev[0], s));
    if ((rc = render_tile_list(rt, ctx->scene->view(), mv, camera_params(ctx->camera), opt, rects,
             rt->frame.ptr, ip->width, spp ? &rectSpp : nullptr)))
        return rc;
    if (metrics) GBSP_CUDA_TRY(cudaEventRecord(rt->ev[1], s));
    if (ip->pixels) {
        size_t pitch = (size_t)ip->width * sizeof(float4);
        for (const uint4 &r : rects)
            GBSP_CUDA_TRY(cudaMemcpy2DAsync(ip->pixels + 4 * ((size_t)r.y * ip->width + r.x), pitch,
                rt->frame.ptr + (size_t)r.y * ip->width + r.x, pitch, (size_t)r.z * sizeof(float4),
                r.w, cudaMemcpyDeviceToHost, s));
    }
    if (!metrics && !ip->pixels) return GBSP_OK;
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.0f;
    if (metrics) cudaEventElapsedTime(&ms, rt->ev[0], rt->ev[1]);
    if ((rc = counters_end(rt, metrics, ms))) return rc;
    return check_stream_status(rt);
}

int gbsp_path_trace_tile_list(const gbsp_context *ctx, const gbsp_tile *tiles, uint32_t count,
    gbsp_metrics *metrics)
{
    return tile_list(ctx, tiles, nullptr, count, metrics);
}

int gbsp_path_trace_tile_list_spp(const gbsp_context *ctx, const gbsp_tile *tiles,
    const uint32_t *spp, uint32_t count, gbsp_metrics *metrics)
{
    if (count && !spp) return set_error(GBSP_ERR_INVALID_ARGUMENT, "spp is NULL");
    return tile_list(ctx, tiles, spp, count, metrics);
}

int gbsp_path_trace_frame(const gbsp_context *ctx, gbsp_metrics *metrics)
{
    gbsp_options opt;
    MaterialView mv;
    DeviceBuffer<int32_t> slots;
    int rc = prepare_render(ctx, opt, mv, slots);
    if (rc) return rc;
    gbsp_runtime *rt = ctx->runtime;
    cudaStream_t s = rt->stream;
    gbsp_image_plane *ip = ctx->camera->imagePlane;
    if ((rc = ensure_frame(rt, ip->width, ip->height, (opt.flags & GBSP_FLAG_AOV) != 0))) return rc;
    rt->begin_call(false);
    if (metrics && (rc = counters_begin(rt, (opt.flags & GBSP_FLAG_STAGE_TIMING) != 0))) return rc;
    if (metrics) GBSP_CUDA_TRY(cudaEventRecord(rt->ev[0], s));
    bool seq = opt.rng_mode == GBSP_RNG_TILE_SEQUENTIAL;
    if ((rc = render_frame(rt, ctx->scene->view(), mv, camera_params(ctx->camera), opt, 0, 0,
             ip->width, ip->height, rt->frame.ptr, ip->width, nullptr,
             seq ? nullptr : aov_target(rt, opt))))
        return rc;
    if (metrics) GBSP_CUDA_TRY(cudaEventRecord(rt->ev[1], s));
    if (ip->pixels)
        GBSP_CUDA_TRY(cudaMemcpyAsync(ip->pixels, rt->frame.ptr,
            (size_t)ip->width * ip->height * sizeof(float4), cudaMemcpyDeviceToHost, s));
    if (!metrics && !ip->pixels) {
        // fully asynchronous: errors surface at gbsp_runtime_synchronize;
        // the slot table is freed in stream order behind the kernels
        return GBSP_OK;
    }
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.0f;
    if (metrics) cudaEventElapsedTime(&ms, rt->ev[0], rt->ev[1]);
    if ((rc = counters_end(rt, metrics, ms))) return rc;
    return check_stream_status(rt);
}

const float *gbsp_frame_aov_device_pointer(gbsp_runtime *rt)
{
    return rt ? reinterpret_cast<const float *>(rt->aov.ptr) : nullptr;
}

int gbsp_frame_copy_region(gbsp_runtime *rt, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h,
    float *dstRadiance, float *dstAov)
{
    if (!rt || !dstRadiance) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (x0 + w > rt->frameW || y0 + h > rt->frameH || !rt->frame.ptr)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "region outside the last frame");
    size_t srcPitch = (size_t)rt->frameW * sizeof(float4);
    GBSP_CUDA_TRY(cudaMemcpy2DAsync(dstRadiance, (size_t)w * sizeof(float4),
        rt->frame.ptr + (size_t)y0 * rt->frameW + x0, srcPitch, (size_t)w * sizeof(float4), h,
        cudaMemcpyDeviceToDevice, rt->stream));
    if (dstAov) {
        if (!rt->aov.ptr || rt->aov.count < 2 * (size_t)rt->frameW * rt->frameH)
            return set_error(GBSP_ERR_NOT_READY, "no G-buffers: render with GBSP_FLAG_AOV");
        GBSP_CUDA_TRY(cudaMemcpy2DAsync(dstAov, (size_t)w * 2 * sizeof(float4),
            rt->aov.ptr + 2 * ((size_t)y0 * rt->frameW + x0), 2 * srcPitch,
            (size_t)w * 2 * sizeof(float4), h, cudaMemcpyDeviceToDevice, rt->stream));
    }
    return GBSP_OK;
}

const float *gbsp_frame_device_pointer(gbsp_runtime *rt)
{
    return rt ? reinterpret_cast<const float *>(rt->frame.ptr) : nullptr;
}

// ---- procedural meshes (src/mesh_generation.cpp) ---------------------------------------------
static gbsp_vertex unit_vertex(V3 p)  // CreateUnitVertex, src/mesh_generation.cpp:206-213
{
    V3 n = normalize(p);
    gbsp_vertex v;
    memcpy(v.position, &n, 12);
    memcpy(v.normal, &n, 12);
    v.uv[0] = n.x;
    v.uv[1] = n.y;
    return v;
}

int gbsp_icosphere(uint32_t level, gbsp_vertex *vertices, uint32_t *indices, uint32_t *vertexCount,
    uint32_t *indexCount)
{
    if (level > 10) return set_error(GBSP_ERR_CAPACITY, "icosphere level %u > 10", level);
    uint64_t faces = 20ull << (2 * level);
    uint64_t verts = 12 + 60 * (((1ull << (2 * level)) - 1) / 3);
    if (vertexCount) *vertexCount = (uint32_t)verts;
    if (indexCount) *indexCount = (uint32_t)(faces * 3);
    if (!vertices || !indices) return GBSP_OK;
    float t = (1.0f + sqrtf(5.0f)) * 0.5f;
    V3 base[12] = {v3(-1, t, 0), v3(1, t, 0), v3(-1, -t, 0), v3(1, -t, 0), v3(0, -1, t),
        v3(0, 1, t), v3(0, -1, -t), v3(0, 1, -t), v3(t, 0, -1), v3(t, 0, 1), v3(-t, 0, -1),
        v3(-t, 0, 1)};
    for (int i = 0; i < 12; i++) vertices[i] = unit_vertex(base[i]);
    static const uint32_t f0[60] = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11,
        4, 11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4,
        11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    std::vector<uint32_t> cur(f0, f0 + 60), next;
    uint32_t count = 12;
    for (uint32_t l = 0; l < level; l++) {
        size_t nf = cur.size() / 3;
        next.resize(nf * 12);
        for (size_t j = 0; j < nf; j++) {
            uint32_t a = cur[3 * j], b = cur[3 * j + 1], c = cur[3 * j + 2];
            uint32_t e[6] = {a, b, b, c, c, a};
            uint32_t added[3];
            for (int k = 0; k < 3; k++) {
                V3 u = add(ld3(vertices[e[2 * k]].position), ld3(vertices[e[2 * k + 1]].position));
                vertices[count] = unit_vertex(u);
                added[k] = count++;
            }
            uint32_t *o = next.data() + 12 * j;
            o[0] = a, o[1] = added[0], o[2] = added[2];
            o[3] = b, o[4] = added[1], o[5] = added[0];
            o[6] = c, o[7] = added[2], o[8] = added[1];
            o[9] = added[0], o[10] = added[1], o[11] = added[2];
        }
        cur.swap(next);
    }
    memcpy(indices, cur.data(), cur.size() * 4);
    return GBSP_OK;
}

int gbsp_plane_mesh(gbsp_vertex vertices[4], uint32_t indices[6])
{
    if (!vertices || !indices) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    const float v[4][8] = {{-0.5f, -0.5f, 0, 0, 0, 1, 0, 0}, {0.5f, -0.5f, 0, 0, 0, 1, 1, 0},
        {0.5f, 0.5f, 0, 0, 0, 1, 1, 1}, {-0.5f, 0.5f, 0, 0, 0, 1, 0, 1}};
    memcpy(vertices, v, sizeof(v));
    const uint32_t i[6] = {0, 1, 2, 2, 3, 0};
    memcpy(indices, i, sizeof(i));
    return GBSP_OK;
}

}  // extern "C"
