// Host-side objects behind the gbsp C ABI.
#pragma once

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbsp.h"
#include "gbsp_common.cuh"

namespace gbsp {

// Sets the thread's last error message and returns the status.
int set_error(int status, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);
#define GBSP_CUDA_TRY(call)                                            \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return ::gbsp::cuda_error(e_, #call);   \
    } while (0)

// Owning device allocation (stream-ordered).
template <typename T>
struct DeviceBuffer {
    T *ptr = nullptr;
    size_t count = 0;  // elements allocated
    cudaStream_t stream = nullptr;

    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    ~DeviceBuffer() { release(); }

    void release()
    {
        if (ptr) cudaFreeAsync(ptr, stream);
        ptr = nullptr;
        count = 0;
    }
    // Grows to at least n elements; contents are not kept.
    int reserve(size_t n, cudaStream_t s)
    {
        if (n <= count && ptr) return GBSP_OK;
        release();
        stream = s;
        size_t bytes = (n ? n : 1) * sizeof(T);
        cudaError_t e = cudaMallocAsync((void **)&ptr, bytes, s);
        if (e != cudaSuccess) {
            ptr = nullptr;
            return set_error(e == cudaErrorMemoryAllocation ? GBSP_ERR_OUT_OF_MEMORY : GBSP_ERR_CUDA,
                "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        }
        count = n ? n : 1;
        return GBSP_OK;
    }
    int upload(const T *host, size_t n, cudaStream_t s)
    {
        int rc = reserve(n, s);
        if (rc) return rc;
        if (n) GBSP_CUDA_TRY(cudaMemcpyAsync(ptr, host, n * sizeof(T), cudaMemcpyHostToDevice, s));
        return GBSP_OK;
    }
};

struct Counters;  // device metric block

// Paths per wave of the wavefront renderers when the caller leaves it to the
// library: 2^25 (about 9 GB of wave state at 5 bounces).  Larger waves have
// fewer bounce tails and launches: a 1080p x 64-spp frame measured 1,304,
// 1,355, 1,378 and 1,391 Msamples/s at 2^22, 2^23, 2^24 and 2^25 paths.
constexpr uint32_t kDefaultWavePaths = 1u << 25;

// BVH node widths the library builds for every mesh and object BVH: index 0
// holds the 8-wide trees (2 quads per node), index 1 the 4-wide trees.
constexpr int kNodeWidths = 2;
constexpr uint32_t kWidthQuads[kNodeWidths] = {2, 1};
inline int width_index(uint32_t width) { return width == 4 ? 1 : 0; }

// Device node pool of one width (layout in gbsp_common.cuh).
struct NodePool {
    DeviceBuffer<float4> buf;
    uint32_t quads = 2;
    float4 *node(uint32_t i) const { return buf.ptr + node_offset(i, quads); }
};

struct WideTree {
    uint32_t nodeCount = 0;
    uint32_t depth = 0;
};

}  // namespace gbsp

// A runtime lives until gbsp_runtime_destroy has been called AND every scene
// and material system created on it has been destroyed (reference count).
struct gbsp_runtime {
    int refs = 1;                       // guarded by the API's runtime mutex
    bool closed = false;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool ownsStream = false;
    int smCount = 0;
    uint32_t *dStatus = nullptr;        // kernel status word
    unsigned long long *dCounters = nullptr;  // GBSP_METRIC_COUNT u64 counters
    cudaEvent_t ev[8] = {};
    // wavefront state, grown on demand
    gbsp::DeviceBuffer<float4> rayO, rayD;         // two queues back to back
    gbsp::DeviceBuffer<int4> hitA;                 // t, u, v, prim
    gbsp::DeviceBuffer<int> hitInst;
    gbsp::DeviceBuffer<uint32_t> sortHist;       // octant histograms of the ray sort
    gbsp::DeviceBuffer<float4> vertE;              // emission xyz, cosine
    gbsp::DeviceBuffer<float4> vertA;              // response xyz
    gbsp::DeviceBuffer<float4> pathRad;            // radiance per path
    gbsp::DeviceBuffer<unsigned int> queueCounts;  // small control block
    gbsp::DeviceBuffer<float4> frame;              // last frame, RGBA32F
    gbsp::DeviceBuffer<float4> aov;                // 2 per pixel when GBSP_FLAG_AOV
    gbsp::DeviceBuffer<float4> pathAov;            // 2 per path of a wave
    uint32_t frameW = 0, frameH = 0;
    // launch accounting and optional per-stage timing of the current call
    uint64_t launches = 0, traceLaunches = 0;
    std::vector<cudaEvent_t> evPool;
    size_t evUsed = 0;
    std::vector<std::pair<int, int>> traceSpans, shadeSpans;  // event index pairs
    bool stageTiming = false;
    int stage_event(cudaStream_t s)  // records and returns an event index, -1 on failure
    {
        if (evUsed == evPool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            evPool.push_back(e);
        }
        if (cudaEventRecord(evPool[evUsed], s) != cudaSuccess) return -1;
        return (int)evUsed++;
    }
    void begin_call(bool timing)
    {
        launches = traceLaunches = 0;
        evUsed = 0;
        traceSpans.clear();
        shadeSpans.clear();
        stageTiming = timing;
    }
};

struct gbsp_mesh_info {
    uint32_t rootNode[gbsp::kNodeWidths];   // in the scene's node pool of each width
    uint32_t triFirst;     // first triangle in the pool
    uint32_t triCount;
    uint32_t nodeCount[gbsp::kNodeWidths];
    uint32_t depth[gbsp::kNodeWidths];
    bool smooth;
    float aabbMin[3], aabbMax[3];  // vertex AABB (src/sp_scene.cpp:57-75)
};

struct gbsp_object_info {
    uint32_t mesh;
    uint32_t material;
    float position[3], rotation[4], scale[3];
    gbsp::Instance inst;
};

struct gbsp_scene {
    gbsp_runtime *rt = nullptr;
    std::vector<gbsp_mesh_info> meshes;
    std::vector<gbsp_object_info> objects;
    // node pools, one per width: mesh BVHs first, then the object BVH
    // (rebuilt per commit); renders use the pool of nodeWidth
    gbsp::NodePool nodes[gbsp::kNodeWidths];
    uint32_t meshNodeCount[gbsp::kNodeWidths] = {0, 0};   // nodes used by meshes
    uint32_t totalNodeCount[gbsp::kNodeWidths] = {0, 0};
    gbsp::DeviceBuffer<gbsp::TriRecord> tris;
    gbsp::DeviceBuffer<gbsp::TriAttr> attrs;
    gbsp::DeviceBuffer<uint32_t> triIds;
    uint64_t triCount = 0;
    // instances in object-BVH leaf order, one array per width (they differ
    // only in the mesh root node index)
    gbsp::DeviceBuffer<gbsp::Instance> instances[gbsp::kNodeWidths];
    uint32_t tlasRoot[gbsp::kNodeWidths] = {gbsp::kEmptyChild, gbsp::kEmptyChild};
    uint32_t tlasDepth[gbsp::kNodeWidths] = {0, 0};
    uint32_t maxDepth[gbsp::kNodeWidths] = {0, 0};
    uint32_t nodeWidth = 8;       // 8 or 4
    bool committed = false;
    uint32_t isectMode = GBSP_ISECT_REFERENCE_MT;
    std::vector<uint32_t> leafOrder;  // object-BVH leaf position -> object index
    gbsp_scene()
    {
        for (int w = 0; w < gbsp::kNodeWidths; w++) nodes[w].quads = gbsp::kWidthQuads[w];
    }
    // resolved material slots depend on the material system; objects keep ids
    gbsp::SceneView view(uint32_t width = 0) const
    {
        int w = gbsp::width_index(width ? width : nodeWidth);
        gbsp::SceneView v;
        v.nodes = nodes[w].buf.ptr;
        v.nodeQuads = nodes[w].quads;
        v.tris = tris.ptr;
        v.attrs = attrs.ptr;
        v.triIds = triIds.ptr;
        v.instances = instances[w].ptr;
        v.tlasRoot = tlasRoot[w];
        v.instanceCount = (uint32_t)objects.size();
        v.watertight = isectMode == GBSP_ISECT_WATERTIGHT ? 1u : 0u;
        return v;
    }
};

struct gbsp_material_system {
    gbsp_runtime *rt = nullptr;
    std::vector<uint32_t> keys;
    std::vector<gbsp_material> materials;
    std::vector<uint32_t> textureKeys;
    std::vector<std::vector<float>> texturePixels;
    std::vector<uint32_t> textureW, textureH;
    uint32_t backgroundId = 0;
    gbsp::SkyParams sky = {};
    bool haveSky = false;
    bool dirty = true;
    gbsp::DeviceBuffer<gbsp::DeviceMaterial> dMaterials;
    gbsp::DeviceBuffer<float4> dTexels;
    gbsp::DeviceBuffer<gbsp::TextureDesc> dTextures;
};

namespace gbsp {

// bvh_build.cu
// Builds the wide BVHs (8- and 4-wide, from one binary tree) over n
// primitive boxes (dLo/dHi on the device).  The binary tree is a binned-SAH
// tree built on the host when the host copies of the boxes (hLo/hHi) are
// given and n <= 2^20, else a linear BVH built on the device.  Tree w is
// appended to pools[w] at nodeBase[w] (growing the pool, keeping its
// contents), with node indices relative to nodeBase[w]; trees[w] receives
// its node count and depth.  Returns the primitive order (sorted position
// -> primitive) both trees' leaves index.
int build_wide_bvh(cudaStream_t s, const float4 *dLo, const float4 *dHi, uint32_t n,
    uint32_t leafMax, NodePool *pools, const uint32_t *nodeBase, WideTree *trees,
    DeviceBuffer<uint32_t> *orderOut, uint32_t *dStatus, const float4 *hLo = nullptr,
    const float4 *hHi = nullptr);
// Triangle boxes + records for a mesh: positions from VertexPNT, indices.
int mesh_prepare(cudaStream_t s, const gbsp_vertex *dVerts, const uint32_t *dIdx,
    uint32_t triCount, float4 *dLo, float4 *dHi);
int mesh_emit(cudaStream_t s, const gbsp_vertex *dVerts, const uint32_t *dIdx,
    uint32_t triCount, const uint32_t *dOrder, TriRecord *dTris, TriAttr *dAttrs,
    uint32_t *dTriIds, uint32_t triBase);
// Moves nodeCount nodes at nodeBase of a pool from relative to absolute
// indices (child node indices += nodeBase, leaf first += leafBase).
int offset_nodes(cudaStream_t s, NodePool &pool, uint32_t nodeCount, uint32_t nodeBase,
    uint32_t leafBase);

// trace.cu
// Reference counting of runtimes: scenes, material systems, batches and
// compute-path-tracer scenes hold a reference so that a runtime destroyed
// first stays alive (stream and buffers) until its last dependent goes.
int runtime_retain(gbsp_runtime *rt);
void runtime_release(gbsp_runtime *rt);

int launch_intersect(cudaStream_t s, const SceneView &sv, uint32_t count, const float4 *rays,
    float *tOut, int32_t *triOut, int32_t *objOut, float *attrOut, uint32_t *matOut,
    const Instance *instHost, int smCount, unsigned long long *counters, uint32_t *dStatus);

// pathtrace.cu
int render_frame(gbsp_runtime *rt, const SceneView &sv, const MaterialView &mv,
    const CameraParams &cam, const gbsp_options &opt, uint32_t x0, uint32_t y0, uint32_t x1,
    uint32_t y1, float4 *dImage, uint32_t imageWidth, uint32_t *rngState,
    float4 *dAov = nullptr, uint32_t splitSpp = 0, float4 *dImage2 = nullptr);

// Renders the listed rectangles (x0, y0, width, height), hash-per-sample
// seeding, into dImage (imageWidth pixels per row) in one wave sequence:
// opt.spp samples per pixel, or (*tileSpp)[i] for tile i when tileSpp is given.
int render_tile_list(gbsp_runtime *rt, const SceneView &sv, const MaterialView &mv,
    const CameraParams &cam, const gbsp_options &opt, const std::vector<uint4> &tiles,
    float4 *dImage, uint32_t imageWidth, const std::vector<uint32_t> *tileSpp = nullptr);

// api.cu
int material_view(gbsp_material_system *ms, MaterialView *out);
int resolve_material(const gbsp_material_system *ms, uint32_t id);

}  // namespace gbsp
