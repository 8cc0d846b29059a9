// Batched rendering of many scenes of uneven size in one persistent launch.
//
// Work unit = one pixel of one item (all of its samples, traced one after
// another in one thread, each seeded from hash(seed, x, y, sample)), so the
// per-pixel sum is the same ordered Neumaier sum as the wavefront path and
// every image is bit-identical to a single-scene render.  The items' pixels
// are numbered back to back; warps pop 32*chunk of them at a time from one
// global 64-bit atomic counter until the total is exhausted, which balances
// items of 1 to 256 spp and 1 to 8 bounces without any host involvement.
// The reset + kernel pair is captured once into a CUDA graph and replayed.

#include <algorithm>
#include <vector>

#include "wavefront.cuh"

namespace gbsp {

constexpr int kBatchMaxBounces = 16;

struct BatchItemDev {
    SceneView sv;
    MaterialView mv;
    CameraParams cam;
    float4 *image;
    uint64_t pixelBase;
    uint64_t pathBase;  // first path of this item in the batch's path numbering
    uint32_t width, height, spp, maxBounces, seed, nanPolicy;
    float clampValue, invSpp;
};

// ---------------------------------------------------------------------------
// Batched wavefront.  The items' paths are numbered back to back (item,
// pixel, sample) and cut into waves of whole pixels; a wave may hold the
// tail of one item and the heads of the next ones.  Every wave runs the
// frame renderer's stages - generate, then per bounce the closest-hit and
// shading kernels over one compacted queue, then accumulate - with each path
// finding its scene, materials, bounce count and clamp through its item
// (ManyScenes), so small scenes share waves instead of each running its own
// short launches, and the whole sequence replays as one CUDA graph.  Per
// pixel the same ordered Neumaier sum over the same per-sample seeds as a
// single-scene render: images are bit-identical.
// ---------------------------------------------------------------------------
struct ManyScenes {
    const BatchItemDev *items;
    const uint32_t *pathItem;
    __device__ __forceinline__ const SceneView &scene(uint32_t p) const
    {
        return items[__ldg(pathItem + p)].sv;
    }
    __device__ __forceinline__ const MaterialView &materials(uint32_t p) const
    {
        return items[__ldg(pathItem + p)].mv;
    }
    __device__ __forceinline__ uint32_t bounces(uint32_t p) const
    {
        return items[__ldg(pathItem + p)].maxBounces;
    }
    __device__ __forceinline__ float clamp(uint32_t p) const
    {
        return items[__ldg(pathItem + p)].clampValue;
    }
};

struct BatchWave {
    uint64_t pathBase, pixBase;
    uint32_t paths, pixels, maxBounces;
};

__device__ __forceinline__ uint32_t find_item_by_path(const BatchItemDev *items, uint32_t n,
    uint64_t gp)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (items[mid].pathBase <= gp)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ uint32_t find_item_by_pixel(const BatchItemDev *items, uint32_t n,
    uint64_t gq)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (items[mid].pixelBase <= gq)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(256) k_bgenerate(const BatchItemDev *__restrict__ items,
    uint32_t itemCount, BatchWave wave, WaveBuffers wb, uint32_t *pathItem)
{
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= wave.paths) return;
    uint64_t gp = wave.pathBase + p;
    uint32_t k = find_item_by_path(items, itemCount, gp);
    const BatchItemDev &it = items[k];
    uint64_t lp = gp - it.pathBase;
    uint64_t pix = lp / it.spp;
    uint32_t s = (uint32_t)(lp % it.spp);
    uint32_t x = (uint32_t)(pix % it.width), y = (uint32_t)(pix / it.width);
    uint32_t rng = sample_seed(it.seed, x, y, s);
    V3 o, d;
    camera_ray(it.cam, x, y, rng, o, d);
    wb.rayO[p] = make_float4(o.x, o.y, o.z, __int_as_float((int)p));
    wb.rayD[p] = make_float4(d.x, d.y, d.z, __uint_as_float(rng));
    pathItem[p] = k;
}

__global__ void __launch_bounds__(256) k_baccumulate(const BatchItemDev *__restrict__ items,
    uint32_t itemCount, BatchWave wave, WaveBuffers wb, unsigned long long *counters)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nans = 0;
    if (k < wave.pixels) {
        uint64_t gq = wave.pixBase + k;
        const BatchItemDev &it = items[find_item_by_pixel(items, itemCount, gq)];
        uint64_t lq = gq - it.pixelBase;
        uint32_t x = (uint32_t)(lq % it.width), y = (uint32_t)(lq / it.width);
        size_t first = (size_t)(it.pathBase + lq * it.spp - wave.pathBase);
        CSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
        for (uint32_t s = 0; s < it.spp; s++) {
            float4 r = wb.pathRad[first + s];
            if (isnan(r.x) || isnan(r.y) || isnan(r.z)) {
                nans++;
                if (it.nanPolicy == GBSP_NAN_ZERO) continue;
            }
            csum_add(acc[0], r.x * it.invSpp);
            csum_add(acc[1], r.y * it.invSpp);
            csum_add(acc[2], r.z * it.invSpp);
        }
        it.image[(size_t)y * it.width + x] =
            make_float4(csum_value(acc[0]), csum_value(acc[1]), csum_value(acc[2]), 1.0f);
    }
    for (int off = 16; off; off >>= 1) nans += __shfl_xor_sync(0xFFFFFFFFu, nans, off);
    if ((threadIdx.x & 31) == 0 && nans)
        atomicAdd(&counters[GBSP_METRIC_NAN_SAMPLES], (unsigned long long)nans);
}

// zero-bounce items: every path of the wave has radiance 0
__global__ void k_bzero(WaveBuffers wb, uint32_t paths)
{
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < paths) wb.pathRad[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void k_batch_reset(unsigned long long *work, unsigned long long *counters)
{
    if (threadIdx.x == 0) *work = 0;
    if (threadIdx.x < GBSP_METRIC_COUNT) counters[threadIdx.x] = 0;
}

template <bool kWT>
__global__ void __launch_bounds__(256) k_batch(const BatchItemDev *__restrict__ items,
    uint32_t itemCount, uint64_t totalPixels, uint32_t chunk, unsigned long long *work,
    unsigned long long *counters, uint32_t *status)
{
    int lane = threadIdx.x & 31;
    TraceCounters cnt = {0, 0, 0, 0, 0};
    uint32_t rays = 0, hits = 0, paths = 0, nans = 0;
    uint64_t step = 32ull * chunk;
    for (uint64_t guard = 0; guard <= totalPixels / step + 1; guard++) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(work, (unsigned long long)step);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= totalPixels) break;
        for (uint32_t c = 0; c < chunk; c++) {
            uint64_t pix = base + (uint64_t)c * 32 + lane;  // neighbouring lanes, neighbouring pixels
            if (pix >= totalPixels) continue;
            uint32_t lo = 0, hi = itemCount - 1;
            while (lo < hi) {
                uint32_t mid = (lo + hi + 1) >> 1;
                if (items[mid].pixelBase <= pix)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const BatchItemDev &it = items[lo];
            uint64_t local = pix - it.pixelBase;
            uint32_t x = (uint32_t)(local % it.width), y = (uint32_t)(local / it.width);
            CSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
            for (uint32_t s = 0; s < it.spp; s++) {
                uint32_t rng = sample_seed(it.seed, x, y, s);
                V3 r = trace_full_path<kBatchMaxBounces, kWT>(it.sv, it.mv, it.cam, x, y, rng,
                    it.maxBounces, it.clampValue, status, cnt, rays, hits);
                paths++;
                if (isnan(r.x) || isnan(r.y) || isnan(r.z)) {
                    nans++;
                    if (it.nanPolicy == GBSP_NAN_ZERO) continue;
                }
                csum_add(acc[0], r.x * it.invSpp);
                csum_add(acc[1], r.y * it.invSpp);
                csum_add(acc[2], r.z * it.invSpp);
            }
            it.image[(size_t)y * it.width + x] =
                make_float4(csum_value(acc[0]), csum_value(acc[1]), csum_value(acc[2]), 1.0f);
        }
    }
    uint32_t v[10] = {rays, hits, paths, nans, cnt.topNodes, cnt.meshNodes, cnt.triTests,
        cnt.boxTests, cnt.meshTests, 0};
#pragma unroll
    for (int k = 0; k < 9; k++)
        for (int off = 16; off; off >>= 1) v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
    if (lane == 0) {
        atomicAdd(&counters[GBSP_METRIC_RAYS_TRACED], (unsigned long long)v[0]);
        atomicAdd(&counters[GBSP_METRIC_RAY_HIT_COUNT], (unsigned long long)v[1]);
        atomicAdd(&counters[GBSP_METRIC_RAY_MISS_COUNT], (unsigned long long)(v[0] - v[1]));
        atomicAdd(&counters[GBSP_METRIC_PATHS_TRACED], (unsigned long long)v[2]);
        atomicAdd(&counters[GBSP_METRIC_NAN_SAMPLES], (unsigned long long)v[3]);
        atomicAdd(&counters[GBSP_METRIC_BROADPHASE_NODE_VISITS], (unsigned long long)v[4]);
        atomicAdd(&counters[GBSP_METRIC_MIDPHASE_NODE_VISITS], (unsigned long long)v[5]);
        atomicAdd(&counters[GBSP_METRIC_TRIANGLE_TESTS], (unsigned long long)v[6]);
        atomicAdd(&counters[GBSP_METRIC_MIDPHASE_BOX_TESTS], (unsigned long long)v[7]);
        atomicAdd(&counters[GBSP_METRIC_MESH_TESTS_PERFORMED], (unsigned long long)v[8]);
    }
}

// ---------------------------------------------------------------------------
// Path state machine variant.  Every lane owns one pixel at a time and walks
// its samples, paths, bounces and traversal as a sequence of small steps:
// one stack pop of the closest-hit traversal (object or mesh level), or one
// shading event.  The warp executes either a traversal step for the lanes
// that are tracing or a shading step for the lanes whose query finished
// (once at least half of the warp waits for it, or nobody traces), so the
// instructions of a step are shared by most lanes; lanes that finish a pixel
// take the next ones from the global queue (one atomicAdd per refill).
// Per lane the sequence of operations - and so every result bit - is the
// one of trace_full_path.
// ---------------------------------------------------------------------------
constexpr int kSmRefill = 8;
// A ray of a validated tree needs far fewer steps (every node is popped at
// most once per object entry); past this cap the ray is ended with the best
// hit so far and the status word records it.
constexpr uint32_t kMaxRaySteps = 1u << 22;
constexpr uint64_t kMaxBatchIterations = 1ull << 34;
constexpr int kSmShade = 16;

template <bool kWT>
__global__ void __launch_bounds__(128) k_batch_sm(const BatchItemDev *__restrict__ items,
    uint32_t itemCount, uint64_t totalPixels, unsigned long long *work,
    unsigned long long *counters, uint32_t *status)
{
    const int lane = threadIdx.x & 31;
    const uint32_t laneMaskLt = (1u << lane) - 1u;
    TraceCounters cnt = {0, 0, 0, 0, 0};
    uint32_t rays = 0, hitsCnt = 0, paths = 0, nans = 0;
    // lane state
    int phase = 0;  // 0 idle, 1 tracing, 2 query done
    uint32_t it = 0, x = 0, y = 0, s = 0, rng = 0, b = 0, len = 0;
    CSum acc[3];
    float4 vE[kBatchMaxBounces], vA[kBatchMaxBounces];
    V3 o = v3(0, 0, 0), d = v3(0, 0, 0), invd = v3(0, 0, 0);
    // traversal state
    StackEntry stack[kStackSize];
    int sp = 0, tmode = 1, base = 0;
    float bestT = kInf, bestU = 0, bestV = 0;
    int32_t bestPrim = -1, bestInst = -1;
    uint32_t inst = 0;
    V3 lo = v3(0, 0, 0), ld = v3(0, 0, 0), linvd = v3(0, 0, 0);
    float llen = 0, lBestT = kInf, lU = 0, lV = 0;
    int32_t lPrim = -1;
    bool exhausted = false;

    uint32_t steps = 0;
    auto trace_begin = [&](const SceneView &sv) {
        steps = 0;
        invd = inverse(d);
        bestT = kInf;
        bestU = bestV = 0.0f;
        bestPrim = bestInst = -1;
        sp = 0;
        if (sv.tlasRoot != kEmptyChild) {
            stack[0] = StackEntry{sv.tlasRoot, 0.0f};
            sp = 1;
        }
        tmode = 1;
        phase = 1;
    };
    bool emptyPath = false;  // max_bounces 0: the sample has no query at all
    auto start_sample = [&](const BatchItemDev &itd) {
        rng = sample_seed(itd.seed, x, y, s);
        camera_ray(itd.cam, x, y, rng, o, d);
        b = 0;
        len = 0;
        emptyPath = itd.maxBounces == 0;
        if (emptyPath)
            phase = 2;
        else
            trace_begin(itd.sv);
    };

    bool finished = false;
    for (uint64_t guard = 0; guard < kMaxBatchIterations; guard++) {
        // One iteration = one convergence point: every lane passes the
        // __syncwarp and the three ballots exactly once, and each lane's step
        // is a function call without early exits from the loop, so votes
        // and shuffles always see the whole warp at the same instruction.
        __syncwarp();
        // ---- refill idle lanes with pixels
        uint32_t idle = __ballot_sync(0xFFFFFFFFu, phase == 0);
        if (idle && !exhausted && (__popc(idle) >= kSmRefill || idle == 0xFFFFFFFFu)) {
            uint32_t n = __popc(idle);
            int leader = __ffs(idle) - 1;
            unsigned long long first = 0;
            if (lane == leader) first = atomicAdd(work, (unsigned long long)n);
            first = __shfl_sync(0xFFFFFFFFu, first, leader);
            if (first + n >= totalPixels) exhausted = true;
            if (phase == 0) {
                uint64_t pix = first + __popc(idle & laneMaskLt);
                if (pix < totalPixels) {
                    uint32_t lo_ = 0, hi_ = itemCount - 1;
                    while (lo_ < hi_) {
                        uint32_t mid = (lo_ + hi_ + 1) >> 1;
                        if (items[mid].pixelBase <= pix)
                            lo_ = mid;
                        else
                            hi_ = mid - 1;
                    }
                    it = lo_;
                    const BatchItemDev &itd = items[it];
                    uint64_t local = pix - itd.pixelBase;
                    x = (uint32_t)(local % itd.width);
                    y = (uint32_t)(local / itd.width);
                    s = 0;
                    acc[0] = acc[1] = acc[2] = CSum{0.0f, 0.0f};
                    start_sample(itd);
                }
            }
        }
        uint32_t tmask = __ballot_sync(0xFFFFFFFFu, phase == 1);
        uint32_t smask = __ballot_sync(0xFFFFFFFFu, phase == 2);
        if (!tmask && !smask && exhausted) {
            finished = true;
            break;
        }
        bool doShade = smask && (__popc(smask) >= kSmShade || !tmask);
        const BatchItemDev &itd = items[it];
        // ---- one shading event
        auto shade_step = [&]() {
            float4 ec, aa;
            bool more = false;
            bool hit = false;
            if (!emptyPath) {
                rays++;
                hit = bestPrim >= 0 && bestT > 0.0f;
            }
            if (hit) {
                hitsCnt++;
                RayHit h;
                h.t = bestT;
                h.u = bestU;
                h.v = bestV;
                h.prim = bestPrim;
                h.inst = bestInst;
                V3 n;
                float ux, uy;
                hit_surface(itd.sv, h, n, ux, uy);
                V3 pos = add(o, mul(d, h.t));
                V3 dir = random_hemisphere(n, rng);
                vertex_terms(itd.mv, itd.mv.instanceSlot[h.inst], n, dir, neg(d), ux, uy, ec, aa);
                vE[len] = ec;
                vA[len] = aa;
                len++;
                if (b + 1 < itd.maxBounces && b + 1 < (uint32_t)kBatchMaxBounces) {
                    o = add(pos, mul(n, 0.0001f));
                    d = dir;
                    b++;
                    more = true;
                    trace_begin(itd.sv);
                }
            } else if (!emptyPath) {
                vertex_terms(itd.mv, itd.mv.backgroundSlot, v3(0, 0, 0), v3(0, 0, 0), neg(d), 0.0f,
                    0.0f, ec, aa);
                vE[len] = ec;
                vA[len] = aa;
                len++;
            }
            if (more) return;
            V3 r = path_radiance(vE, vA, 1, 0, len, itd.clampValue);
            paths++;
            bool isNan = isnan(r.x) || isnan(r.y) || isnan(r.z);
            if (isNan) nans++;
            if (!isNan || itd.nanPolicy != GBSP_NAN_ZERO) {
                csum_add(acc[0], r.x * itd.invSpp);
                csum_add(acc[1], r.y * itd.invSpp);
                csum_add(acc[2], r.z * itd.invSpp);
            }
            s++;
            if (s < itd.spp) {
                start_sample(itd);
            } else {
                itd.image[(size_t)y * itd.width + x] =
                    make_float4(csum_value(acc[0]), csum_value(acc[1]), csum_value(acc[2]), 1.0f);
                phase = 0;
            }
        };
        // ---- one traversal step (trace_closest's stack walk, one pop per call)
        auto trace_step = [&]() {
            const SceneView &sv = itd.sv;
            if (++steps > kMaxRaySteps) {
                atomicOr(status, kStatusRayStepLimit);
                tmode = 1;
                sp = 0;
                steps = 0;
            }
            if (tmode == 2 && sp == base) {
                if (lPrim >= 0) {
                    const Instance &in = sv.instances[inst];
                    Affine model;
#pragma unroll
                    for (int k = 0; k < 12; k++) model.r[k] = __ldg(&in.model.r[k]);
                    V3 worldHit = transform_point(model, add(lo, mul(ld, lBestT)));
                    float tw = dot(sub(worldHit, o), d);
                    if (tw < bestT || (tw == bestT && (int32_t)inst < bestInst)) {
                        bestT = tw;
                        bestU = lU;
                        bestV = lV;
                        bestPrim = lPrim;
                        bestInst = (int32_t)inst;
                    }
                }
                tmode = 1;
                return;
            }
            if (tmode == 1 && sp == 0) {
                phase = 2;
                return;
            }
            sp--;
            const StackEntry top = stack[sp];
            uint32_t ref = top.ref;
            float te = top.t;
            float bound = tmode == 1 ? prune_bound(bestT) : prune_bound(rmin(lBestT, bestT * llen));
            if (te > bound) return;
            if (!child_is_leaf(ref)) {
                if (tmode == 1)
                    cnt.topNodes++;
                else
                    cnt.meshNodes++;
                V3 ro = tmode == 1 ? o : lo;
                V3 ri = tmode == 1 ? invd : linvd;
                visit_node<true, kWT>(sv.nodes, sv.nodeQuads, ref, ro, ri, bound, stack, sp, status,
                    cnt);
                return;
            }
            if (tmode == 1) {
                inst = leaf_first(ref);
                const Instance &in = sv.instances[inst];
                Affine inv;
#pragma unroll
                for (int k = 0; k < 12; k++) inv.r[k] = __ldg(&in.inv.r[k]);
                lo = transform_point(inv, o);
                ld = normalize(transform_vector(inv, d), &llen);
                linvd = inverse(ld);
                cnt.meshTests++;
                lBestT = kInf;
                lU = lV = 0.0f;
                lPrim = -1;
                base = sp;
                if (sp >= kStackSize) {
                    atomicOr(status, kStatusStackOverflow);
                    return;
                }
                stack[sp] = StackEntry{__ldg(&in.blasRoot), 0.0f};
                sp++;
                tmode = 2;
                return;
            }
            visit_leaf<true, kWT>(sv, ref, lo, ld, linvd, lBestT, lU, lV, lPrim, cnt);
        };
        if (doShade && phase == 2)
            shade_step();
        else if (!doShade && phase == 1)
            trace_step();
    }
    if (!finished && lane == 0) atomicOr(status, kStatusQueueOverflow);
    __syncwarp();
    uint32_t v[9] = {rays, hitsCnt, paths, nans, cnt.topNodes, cnt.meshNodes, cnt.triTests,
        cnt.boxTests, cnt.meshTests};
#pragma unroll
    for (int k = 0; k < 9; k++)
        for (int off = 16; off; off >>= 1) v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
    if (lane == 0) {
        atomicAdd(&counters[GBSP_METRIC_RAYS_TRACED], (unsigned long long)v[0]);
        atomicAdd(&counters[GBSP_METRIC_RAY_HIT_COUNT], (unsigned long long)v[1]);
        atomicAdd(&counters[GBSP_METRIC_RAY_MISS_COUNT], (unsigned long long)(v[0] - v[1]));
        atomicAdd(&counters[GBSP_METRIC_PATHS_TRACED], (unsigned long long)v[2]);
        atomicAdd(&counters[GBSP_METRIC_NAN_SAMPLES], (unsigned long long)v[3]);
        atomicAdd(&counters[GBSP_METRIC_BROADPHASE_NODE_VISITS], (unsigned long long)v[4]);
        atomicAdd(&counters[GBSP_METRIC_MIDPHASE_NODE_VISITS], (unsigned long long)v[5]);
        atomicAdd(&counters[GBSP_METRIC_TRIANGLE_TESTS], (unsigned long long)v[6]);
        atomicAdd(&counters[GBSP_METRIC_MIDPHASE_BOX_TESTS], (unsigned long long)v[7]);
        atomicAdd(&counters[GBSP_METRIC_MESH_TESTS_PERFORMED], (unsigned long long)v[8]);
    }
}

}  // namespace gbsp

using namespace gbsp;

struct gbsp_batch {
    gbsp_runtime *rt = nullptr;
    std::vector<gbsp_batch_item> items;
    DeviceBuffer<BatchItemDev> dItems;
    DeviceBuffer<int32_t> dSlots;
    DeviceBuffer<unsigned long long> dWork;
    uint64_t totalPixels = 0, totalPaths = 0;
    gbsp_batch_config cfg = {128, 1, 8, 1, GBSP_BATCH_WAVEFRONT, 0};
    cudaGraphExec_t exec = nullptr;
    bool watertight = false;  // every item's scene uses the same triangle test
    // batched wavefront
    std::vector<BatchItemDev> hostItems;
    std::vector<BatchWave> waves;
    uint32_t waveCap = 0, waveBounces = 0;
    DeviceBuffer<float4> rayO, rayD, vertE, vertA, pathRad;
    DeviceBuffer<int4> hitA;
    DeviceBuffer<int> hitInst;
    DeviceBuffer<uint32_t> pathItem;
    std::vector<uint32_t> nodeWidth;  // per item: BVH node width its scene view walks
};

static void drop_graph(gbsp_batch *b);

// Points every item's scene view at the BVHs of its chosen node width,
// re-uploads the item table and drops the captured graph (re-captured on
// the next launch).
static int apply_node_widths(gbsp_batch *b)
{
    for (size_t i = 0; i < b->items.size(); i++)
        b->hostItems[i].sv = b->items[i].scene->view(b->nodeWidth[i]);
    drop_graph(b);
    return b->dItems.upload(b->hostItems.data(), b->hostItems.size(), b->rt->stream);
}

// Node width per item, timed on the item's own frame: the frame renderer
// draws the item at each width (its spp capped at 8 for the probe; per-ray
// work does not depend on the sample count) and the faster width is kept.
static int tune_node_widths(gbsp_batch *b, uint32_t trials)
{
    gbsp_runtime *rt = b->rt;
    cudaStream_t s = rt->stream;
    for (size_t i = 0; i < b->items.size(); i++) {
        const gbsp_batch_item &it = b->items[i];
        const BatchItemDev &d = b->hostItems[i];
        gbsp_options o = it.options;
        o.spp = std::min(o.spp ? o.spp : 1u, 8u);
        o.flags = 0;
        float bestMs = 3.0e38f;
        uint32_t bestWidth = b->nodeWidth[i];
        for (uint32_t width : {8u, 4u}) {
            SceneView sv = it.scene->view(width);
            int rc = render_frame(rt, sv, d.mv, d.cam, o, 0, 0, d.width, d.height, d.image, d.width,
                nullptr);
            if (rc) return rc;
            GBSP_CUDA_TRY(cudaEventRecord(rt->ev[2], s));
            for (uint32_t t = 0; t < trials; t++)
                if ((rc = render_frame(rt, sv, d.mv, d.cam, o, 0, 0, d.width, d.height, d.image,
                         d.width, nullptr)))
                    return rc;
            GBSP_CUDA_TRY(cudaEventRecord(rt->ev[3], s));
            GBSP_CUDA_TRY(cudaEventSynchronize(rt->ev[3]));
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, rt->ev[2], rt->ev[3]);
            if (ms < bestMs) {
                bestMs = ms;
                bestWidth = width;
            }
        }
        b->nodeWidth[i] = bestWidth;
    }
    return apply_node_widths(b);
}

// Cuts the items' paths into waves of whole pixels of at most `cap` paths
// and reserves the wave buffers (once).
static int plan_waves(gbsp_batch *b)
{
    const std::vector<BatchItemDev> &dev = b->hostItems;
    uint64_t want = b->cfg.wavePaths ? b->cfg.wavePaths : kDefaultWavePaths;
    uint64_t cap = std::min<uint64_t>(want, std::max<uint64_t>(b->totalPaths, 1));
    uint32_t maxSpp = 1, maxB = 1;
    for (const BatchItemDev &d : dev) {
        maxSpp = std::max(maxSpp, d.spp);
        maxB = std::max(maxB, d.maxBounces);
    }
    cap = std::max<uint64_t>(cap, maxSpp);
    b->waves.clear();
    BatchWave w = {0, 0, 0, 0, 0};
    for (const BatchItemDev &d : dev) {
        uint64_t pixels = (uint64_t)d.width * d.height;
        for (uint64_t q = 0; q < pixels;) {
            if (w.paths + (uint64_t)d.spp > cap) {
                b->waves.push_back(w);
                w = {w.pathBase + w.paths, w.pixBase + w.pixels, 0, 0, 0};
            }
            // as many whole pixels of this item as still fit
            uint64_t fit = std::min<uint64_t>(pixels - q, (cap - w.paths) / d.spp);
            w.paths += (uint32_t)(fit * d.spp);
            w.pixels += (uint32_t)fit;
            w.maxBounces = std::max(w.maxBounces, d.maxBounces);
            q += fit;
        }
    }
    if (w.paths) b->waves.push_back(w);
    b->waveCap = (uint32_t)cap;
    b->waveBounces = maxB;
    cudaStream_t s = b->rt->stream;
    size_t c = cap;
    int rc;
    if ((rc = b->rayO.reserve(2 * c, s)) || (rc = b->rayD.reserve(2 * c, s)) ||
        (rc = b->hitA.reserve(c, s)) || (rc = b->hitInst.reserve(c, s)) ||
        (rc = b->pathItem.reserve(c, s)) || (rc = b->vertE.reserve((size_t)maxB * c, s)) ||
        (rc = b->vertA.reserve((size_t)maxB * c, s)) || (rc = b->pathRad.reserve(c, s)))
        return rc;
    return GBSP_OK;
}

static void enqueue_wavefront(gbsp_batch *b)
{
    gbsp_runtime *rt = b->rt;
    cudaStream_t s = rt->stream;
    unsigned long long *counters = rt->dCounters;
    unsigned int *ctl = reinterpret_cast<unsigned int *>(rt->dCounters + GBSP_METRIC_COUNT);
    WaveBuffers wb;
    wb.rayO = b->rayO.ptr;
    wb.rayD = b->rayD.ptr;
    wb.hitA = b->hitA.ptr;
    wb.hitInst = b->hitInst.ptr;
    wb.vertE = b->vertE.ptr;
    wb.vertA = b->vertA.ptr;
    wb.pathRad = b->pathRad.ptr;
    wb.pathAov = nullptr;
    wb.cap = b->waveCap;
    ManyScenes src = {b->dItems.ptr, b->pathItem.ptr};
    uint32_t n = (uint32_t)b->items.size();
    // blocksPerSm 0: every kernel at the blocks the SMs hold (occupancy)
    const bool resident = b->cfg.blocksPerSm == 0;
    const int grid = rt->smCount * (int)b->cfg.blocksPerSm;
    const int shadeGrid = resident ? shade_grid<ManyScenes>(rt->smCount) : grid;
    for (const BatchWave &w : b->waves) {
        k_reset_ctl<<<1, 32, 0, s>>>(ctl, w.paths);
        if (w.maxBounces == 0) {
            k_bzero<<<(w.paths + 255) / 256, 256, 0, s>>>(wb, w.paths);
        } else {
            k_bgenerate<<<(w.paths + 255) / 256, 256, 0, s>>>(b->dItems.ptr, n, w, wb,
                b->pathItem.ptr);
        }
        for (uint32_t bn = 0; bn < w.maxBounces; bn++) {
            int inQ = (bn & 1) ? kCtlQueue1 : kCtlQueue0;
            int outQ = (bn & 1) ? kCtlQueue0 : kCtlQueue1;
            const float4 *qO = wb.rayO + ((bn & 1) ? wb.cap : 0);
            const float4 *qD = wb.rayD + ((bn & 1) ? wb.cap : 0);
            k_reset_stage<<<1, 1, 0, s>>>(ctl, outQ);
            // primary rays per warp, bounce rays per lane (the frame renderer's default)
            launch_trace_stage(bn > 0, b->watertight,
                resident ? trace_grid<ManyScenes>(bn > 0, b->watertight, rt->smCount) : grid, s,
                src, qO, qD, ctl + inQ, wb.hitA, wb.hitInst, ctl, counters, rt->dStatus);
            k_shade<<<shadeGrid, 128, 0, s>>>(src, wb, bn, inQ, ctl, counters);
        }
        k_baccumulate<<<(w.pixels + 255) / 256, 256, 0, s>>>(b->dItems.ptr, n, w, wb, counters);
    }
}

static void drop_graph(gbsp_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
}

static int enqueue(gbsp_batch *b)
{
    gbsp_runtime *rt = b->rt;
    cudaStream_t s = rt->stream;
    k_batch_reset<<<1, 32, 0, s>>>(b->dWork.ptr, rt->dCounters);
    int grid = rt->smCount * (int)b->cfg.blocksPerSm;
    if (b->cfg.kernel == GBSP_BATCH_WAVEFRONT)
        enqueue_wavefront(b);
    else if (b->cfg.kernel == GBSP_BATCH_PATH_STATE)
        (b->watertight ? k_batch_sm<true> : k_batch_sm<false>)<<<grid, b->cfg.block, 0, s>>>(
            b->dItems.ptr, (uint32_t)b->items.size(),
            b->totalPixels, b->dWork.ptr, rt->dCounters, rt->dStatus);
    else
        (b->watertight ? k_batch<true> : k_batch<false>)<<<grid, b->cfg.block, 0, s>>>(
            b->dItems.ptr, (uint32_t)b->items.size(),
            b->totalPixels, b->cfg.chunk, b->dWork.ptr, rt->dCounters, rt->dStatus);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

static int launch_once(gbsp_batch *b)
{
    cudaStream_t s = b->rt->stream;
    if (!b->cfg.useGraph) return enqueue(b);
    if (!b->exec) {
        cudaGraph_t g = nullptr;
        GBSP_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue(b);
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return cuda_error(e, "cudaGraphInstantiate");
        }
    }
    GBSP_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    return GBSP_OK;
}

static int check_config(const gbsp_batch_config *c)
{
    if (c->kernel != GBSP_BATCH_THREAD_PER_PIXEL && c->kernel != GBSP_BATCH_PATH_STATE &&
        c->kernel != GBSP_BATCH_WAVEFRONT)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "unknown batch kernel %u", c->kernel);
    if (c->block != 64 && c->block != 128 && c->block != 256)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "block must be 64, 128 or 256");
    if (c->kernel == GBSP_BATCH_PATH_STATE && c->block > 128)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "the path-state kernel takes 64 or 128 threads");
    if (c->chunk < 1 || c->chunk > 8) return set_error(GBSP_ERR_INVALID_ARGUMENT, "chunk must be 1..8");
    if (c->blocksPerSm > 32 || (c->blocksPerSm == 0 && c->kernel != GBSP_BATCH_WAVEFRONT))
        return set_error(GBSP_ERR_INVALID_ARGUMENT,
            "blocksPerSm must be 1..32 (0: occupancy, wavefront kernel only)");
    return GBSP_OK;
}

extern "C" {

int gbsp_batch_create(gbsp_runtime *rt, const gbsp_batch_item *items, uint32_t count,
    gbsp_batch **out)
{
    if (!rt || !items || !count || !out) return set_error(GBSP_ERR_INVALID_ARGUMENT, "empty batch");
    *out = nullptr;
    int rrc = runtime_retain(rt);
    if (rrc) return rrc;
    gbsp_batch *b = new gbsp_batch();
    b->rt = rt;
    b->items.assign(items, items + count);
    std::vector<BatchItemDev> dev(count);
    std::vector<int32_t> slots;
    std::vector<size_t> slotOffset(count);
    uint64_t base = 0;
    int rc = GBSP_OK;
    for (uint32_t i = 0; i < count && !rc; i++) {
        const gbsp_batch_item &it = items[i];
        if (!it.scene || !it.materialSystem || !it.camera || !it.camera->imagePlane ||
            !it.deviceImage) {
            rc = set_error(GBSP_ERR_INVALID_ARGUMENT, "batch item %u is incomplete", i);
            break;
        }
        if (!it.scene->committed || it.scene->rt != rt || it.materialSystem->rt != rt) {
            rc = set_error(GBSP_ERR_NOT_READY, "batch item %u: scene not built or other runtime", i);
            break;
        }
        if (it.options.rng_mode != GBSP_RNG_HASH_PER_SAMPLE ||
            it.options.max_bounces > (uint32_t)kBatchMaxBounces) {
            rc = set_error(GBSP_ERR_INVALID_ARGUMENT,
                "batch item %u: hash-per-sample seeding and at most %d bounces", i,
                kBatchMaxBounces);
            break;
        }
        bool wt = it.scene->isectMode == GBSP_ISECT_WATERTIGHT;
        if (i == 0) b->watertight = wt;
        if (wt != b->watertight) {
            rc = set_error(GBSP_ERR_INVALID_ARGUMENT,
                "batch item %u: all items must use the same intersection mode", i);
            break;
        }
        MaterialView mv;
        if ((rc = material_view(it.materialSystem, &mv))) break;
        slotOffset[i] = slots.size();
        const gbsp_scene *sc = it.scene;
        for (size_t j = 0; j < sc->leafOrder.size(); j++)
            slots.push_back(resolve_material(it.materialSystem, sc->objects[sc->leafOrder[j]].material));
        slots.push_back(-1);
        BatchItemDev &d = dev[i];
        d.sv = sc->view();
        d.mv = mv;
        const gbsp_camera *c = it.camera;
        d.cam.right = v3(c->right[0], c->right[1], c->right[2]);
        d.cam.up = v3(c->up[0], c->up[1], c->up[2]);
        d.cam.forward = v3(c->forward[0], c->forward[1], c->forward[2]);
        d.cam.position = v3(c->position[0], c->position[1], c->position[2]);
        d.cam.filmCenter = v3(c->filmCenter[0], c->filmCenter[1], c->filmCenter[2]);
        d.cam.halfPixelWidth = c->halfPixelWidth;
        d.cam.halfPixelHeight = c->halfPixelHeight;
        d.cam.halfFilmWidth = c->halfFilmWidth;
        d.cam.halfFilmHeight = c->halfFilmHeight;
        d.cam.width = c->imagePlane->width;
        d.cam.height = c->imagePlane->height;
        d.image = reinterpret_cast<float4 *>(it.deviceImage);
        d.pixelBase = base;
        d.pathBase = b->totalPaths;
        d.width = c->imagePlane->width;
        d.height = c->imagePlane->height;
        d.spp = it.options.spp ? it.options.spp : 1;
        d.maxBounces = it.options.max_bounces;
        d.seed = it.options.seed;
        d.nanPolicy = it.options.nan_policy;
        d.clampValue = it.options.radiance_clamp;
        d.invSpp = 1.0f / (float)d.spp;
        base += (uint64_t)d.width * d.height;
        b->totalPaths += (uint64_t)d.width * d.height * d.spp;
    }
    if (!rc && base == 0) rc = set_error(GBSP_ERR_INVALID_ARGUMENT, "batch has no pixels");
    cudaStream_t s = rt->stream;
    if (!rc) rc = b->dSlots.upload(slots.data(), slots.size(), s);
    if (!rc) {
        for (uint32_t i = 0; i < count; i++) dev[i].mv.instanceSlot = b->dSlots.ptr + slotOffset[i];
        rc = b->dItems.upload(dev.data(), dev.size(), s);
    }
    if (!rc) rc = b->dWork.reserve(1, s);
    if (!rc) {
        b->hostItems = dev;
        b->totalPixels = base;
        b->nodeWidth.resize(count);
        for (uint32_t i = 0; i < count; i++) b->nodeWidth[i] = items[i].scene->nodeWidth;
        rc = plan_waves(b);
    }
    if (!rc && cudaStreamSynchronize(s) != cudaSuccess)
        rc = set_error(GBSP_ERR_CUDA, "batch upload failed");
    if (rc) {
        delete b;
        runtime_release(rt);
        return rc;
    }
    b->totalPixels = base;
    *out = b;
    return GBSP_OK;
}

int gbsp_batch_destroy(gbsp_batch *batch)
{
    if (!batch) return GBSP_OK;
    gbsp_runtime *rt = batch->rt;
    cudaStreamSynchronize(rt->stream);
    drop_graph(batch);
    delete batch;
    runtime_release(rt);
    return GBSP_OK;
}

int gbsp_batch_set_config(gbsp_batch *batch, const gbsp_batch_config *config)
{
    if (!batch || !config) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = check_config(config);
    if (rc) return rc;
    bool replan = config->wavePaths != batch->cfg.wavePaths;
    batch->cfg = *config;
    drop_graph(batch);
    if (replan) return plan_waves(batch);
    return GBSP_OK;
}

int gbsp_batch_get_config(const gbsp_batch *batch, gbsp_batch_config *config)
{
    if (!batch || !config) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    *config = batch->cfg;
    return GBSP_OK;
}

int gbsp_batch_launch(gbsp_batch *batch, gbsp_metrics *metrics)
{
    if (!batch) return set_error(GBSP_ERR_INVALID_ARGUMENT, "batch is NULL");
    gbsp_runtime *rt = batch->rt;
    cudaStream_t s = rt->stream;
    if (metrics) GBSP_CUDA_TRY(cudaEventRecord(rt->ev[0], s));
    int rc = launch_once(batch);
    if (rc) return rc;
    if (!metrics) return GBSP_OK;
    GBSP_CUDA_TRY(cudaEventRecord(rt->ev[1], s));
    unsigned long long c[GBSP_METRIC_COUNT];
    uint32_t st = 0;
    GBSP_CUDA_TRY(cudaMemcpyAsync(c, rt->dCounters, sizeof(c), cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaMemcpyAsync(&st, rt->dStatus, 4, cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    if (st) {
        cudaMemsetAsync(rt->dStatus, 0, 4, s);
        return set_error(GBSP_ERR_DEVICE_STATUS, "device status 0x%x in the batch kernel", st);
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, rt->ev[0], rt->ev[1]);
    for (int i = 0; i < GBSP_METRIC_COUNT; i++) metrics->values[i] += c[i];
    metrics->values[GBSP_METRIC_ELAPSED_NS] += (uint64_t)((double)ms * 1.0e6);
    metrics->values[GBSP_METRIC_KERNEL_LAUNCHES] += 2;
    return GBSP_OK;
}

int gbsp_batch_set_node_widths(gbsp_batch *batch, const uint32_t *widths)
{
    if (!batch || !widths) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    for (size_t i = 0; i < batch->items.size(); i++)
        if (widths[i] != 4 && widths[i] != 8)
            return set_error(GBSP_ERR_INVALID_ARGUMENT, "item %zu: node width %u (4 or 8)", i,
                widths[i]);
    batch->nodeWidth.assign(widths, widths + batch->items.size());
    return apply_node_widths(batch);
}

int gbsp_batch_get_node_widths(const gbsp_batch *batch, uint32_t *widths)
{
    if (!batch || !widths) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    for (size_t i = 0; i < batch->items.size(); i++) widths[i] = batch->nodeWidth[i];
    return GBSP_OK;
}

int gbsp_batch_autotune(gbsp_batch *batch, uint32_t trials, gbsp_batch_config *best)
{
    if (!batch) return set_error(GBSP_ERR_INVALID_ARGUMENT, "batch is NULL");
    gbsp_runtime *rt = batch->rt;
    cudaStream_t s = rt->stream;
    if (trials == 0) trials = 1;
    int wrc = tune_node_widths(batch, trials);
    if (wrc) return wrc;
    gbsp_batch_config keep = batch->cfg;
    // candidates: thread-per-pixel (block x chunk x blocks per SM), path state
    // (block <= 128 x blocks per SM), wavefront (blocks per SM x wave size)
    std::vector<gbsp_batch_config> cands;
    for (uint32_t ps : {2u, 4u, 8u}) {
        for (uint32_t bl : {64u, 128u, 256u})
            for (uint32_t ch : {1u, 4u})
                cands.push_back({bl, ch, ps, keep.useGraph, GBSP_BATCH_THREAD_PER_PIXEL, keep.wavePaths});
        for (uint32_t bl : {64u, 128u})
            cands.push_back({bl, 1, ps, keep.useGraph, GBSP_BATCH_PATH_STATE, keep.wavePaths});
        for (uint32_t wave : {1u << 22, 1u << 23, 1u << 24, 1u << 25})
            cands.push_back({128, 1, ps, keep.useGraph, GBSP_BATCH_WAVEFRONT, wave});
    }
    for (uint32_t wave : {1u << 24, 1u << 25})
        cands.push_back({128, 1, 0, keep.useGraph, GBSP_BATCH_WAVEFRONT, wave});
    gbsp_batch_config bestCfg = keep;
    float bestMs = 3.0e38f;
    for (const gbsp_batch_config &c : cands) {
        bool replan = c.wavePaths != batch->cfg.wavePaths;
        batch->cfg = c;
        drop_graph(batch);
        int rc = replan ? plan_waves(batch) : GBSP_OK;
        if (!rc) rc = launch_once(batch);  // warm-up (and graph capture)
        if (rc) return rc;
        GBSP_CUDA_TRY(cudaEventRecord(rt->ev[2], s));
        for (uint32_t t = 0; t < trials; t++)
            if ((rc = launch_once(batch))) return rc;
        GBSP_CUDA_TRY(cudaEventRecord(rt->ev[3], s));
        GBSP_CUDA_TRY(cudaEventSynchronize(rt->ev[3]));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, rt->ev[2], rt->ev[3]);
        if (ms < bestMs) {
            bestMs = ms;
            bestCfg = c;
        }
    }
    bool replan = bestCfg.wavePaths != batch->cfg.wavePaths;
    batch->cfg = bestCfg;
    drop_graph(batch);
    if (replan) {
        int rc = plan_waves(batch);
        if (rc) return rc;
    }
    if (best) *best = bestCfg;
    uint32_t st = 0;
    GBSP_CUDA_TRY(cudaMemcpyAsync(&st, rt->dStatus, 4, cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    if (st) return set_error(GBSP_ERR_DEVICE_STATUS, "device status 0x%x while tuning", st);
    return GBSP_OK;
}

}  // extern "C"
