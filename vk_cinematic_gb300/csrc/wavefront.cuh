// Wave kernels shared by the frame renderer (pathtrace.cu) and the batched
// wavefront (batch.cu).  See pathtrace.cu for the stage structure.  The
// trace and shade kernels are templates over a scene source: OneScene for a
// frame, a per-path item table for a batch of scenes.
#pragma once

#include "gbsp_internal.h"
#include "traverse.cuh"
#include "shading.cuh"

namespace gbsp {

// Work/queue control words (u32) behind the metric counters.
enum Ctl : int {
    kCtlTraceWork = 0,
    kCtlShadeWork = 1,
    kCtlQueue0 = 2,
    kCtlQueue1 = 3,
    kCtlCount = 8
};

struct WaveBuffers {
    // a queued ray carries its path's state: the path id and the RNG state ride
    // in the w lanes, and its path length is the bounce number of the queue
    float4 *rayO;      // 2 * cap: (origin, path id bits)
    float4 *rayD;      // 2 * cap: (direction, RNG state bits)
    int4 *hitA;        // cap: (t, u, v, prim) bits
    int *hitInst;      // cap
    float4 *vertE;     // maxBounces * cap: (emission xyz, cosine), vertices of paths that go on
    float4 *vertA;     // maxBounces * cap: (A xyz, 0)
    float4 *pathRad;   // cap
    float4 *pathAov;   // 2 * cap first-hit G-buffer per path, or null
    uint32_t cap;
};

struct WaveParams {
    CameraParams cam;
    uint32_t x0, y0, regionW;
    // optional list of rectangles rendered instead of the region: tile i is
    // (x0, y0, width, height) = tiles[i], its pixels numbered row-major from
    // tileStart[i] (an exclusive prefix sum over the tiles' pixel counts)
    const uint4 *tiles;
    const uint64_t *tileStart;
    uint32_t tileCount;
    // optional per-tile sample counts of a tile list: tile i renders
    // tileSpp[i] samples per pixel, its paths numbered pixel-major from
    // tilePath[i] (an exclusive prefix sum over pixels x spp); null: `spp`
    // samples for every pixel
    const uint32_t *tileSpp;
    const uint64_t *tilePath;
    uint64_t pixelBase;   // first pixel (row-major in the region) of this wave
    uint32_t pixels;      // pixels in this wave
    uint64_t pathBase;    // first path of this wave (with tileSpp)
    uint32_t paths;       // paths in this wave
    uint32_t spp;
    uint32_t maxBounces;
    uint32_t seed;
    float clampValue;
    uint32_t nanPolicy;
    float invSpp;
    float4 *aovImage;     // 2 float4 per image pixel, or null
    // split accumulation (0: off): samples [0, splitSpp) of a pixel go to the
    // image (and the G-buffers), samples [splitSpp, spp) to image2
    uint32_t splitSpp;
    float4 *image2;
};

// Scene source of the wave kernels: everything a path needs from its scene.
// OneScene: one scene for the whole launch (a frame or a tile).
struct OneScene {
    SceneView sv;
    MaterialView mv;
    uint32_t maxBounces;
    float clampValue;
    __device__ __forceinline__ const SceneView &scene(uint32_t) const { return sv; }
    __device__ __forceinline__ const MaterialView &materials(uint32_t) const { return mv; }
    __device__ __forceinline__ uint32_t bounces(uint32_t) const { return maxBounces; }
    __device__ __forceinline__ float clamp(uint32_t) const { return clampValue; }
};

// ---------------------------------------------------------------------------
// Stage kernels
// ---------------------------------------------------------------------------
static __global__ void k_reset_ctl(unsigned int *ctl, uint32_t queue0)
{
    if (threadIdx.x < kCtlCount) ctl[threadIdx.x] = 0;
    __syncthreads();
    if (threadIdx.x == 0) ctl[kCtlQueue0] = queue0;
}

static __global__ void k_reset_stage(unsigned int *ctl, int outQueue)
{
    ctl[kCtlTraceWork] = 0;
    ctl[kCtlShadeWork] = 0;
    ctl[outQueue] = 0;
}

// ---------------------------------------------------------------------------
// Stable counting sort of a ray queue by direction octant (sign bits of d),
// so that the lanes of a warp walk the tree with the same near-to-far child
// order.  Queue order otherwise follows path order (neighbouring pixels'
// samples), which the sort keeps within each octant.  Three launches over a
// fixed grid of kSortBlocks blocks (the count lives on the device):
// per-block octant histograms, one exclusive scan over (octant, block), and
// the scatter, which ranks rays inside each 256-ray tile with warp ballots.
constexpr int kSortBlocks = 512;

__device__ __forceinline__ uint32_t dir_octant(float4 d)
{
    return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
}

__device__ __forceinline__ void sort_chunk(uint32_t n, uint32_t &begin, uint32_t &end)
{
    uint32_t chunk = (n + kSortBlocks - 1) / kSortBlocks;
    chunk = (chunk + 255u) & ~255u;
    begin = min(n, blockIdx.x * chunk);
    end = min(n, begin + chunk);
}

static __global__ void __launch_bounds__(256) k_octant_count(const float4 *__restrict__ rayD,
    const unsigned int *ctl, int queue, uint32_t *hist)
{
    __shared__ uint32_t sh[8];
    if (threadIdx.x < 8) sh[threadIdx.x] = 0;
    __syncthreads();
    uint32_t begin, end;
    sort_chunk(ctl[queue], begin, end);
    for (uint32_t i = begin + threadIdx.x; i < end; i += 256) atomicAdd(&sh[dir_octant(rayD[i])], 1u);
    __syncthreads();
    if (threadIdx.x < 8) hist[threadIdx.x * kSortBlocks + blockIdx.x] = sh[threadIdx.x];
}

// Exclusive scan of hist[8][kSortBlocks] in (octant, block) order; also
// publishes the count as the destination queue's length.
static __global__ void __launch_bounds__(1024) k_octant_scan(uint32_t *hist, unsigned int *ctl,
    int srcQueue, int dstQueue)
{
    constexpr int kPer = 8 * kSortBlocks / 1024;
    __shared__ uint32_t warpSum[32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t v[kPer], sum = 0;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        v[k] = hist[t * kPer + k];
        sum += v[k];
    }
    uint32_t incl = sum;
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) warpSum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warpSum[lane], wi = w;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t o = __shfl_up_sync(0xFFFFFFFFu, wi, off);
            if (lane >= off) wi += o;
        }
        warpSum[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = warpSum[warp] + incl - sum;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        hist[t * kPer + k] = run;
        run += v[k];
    }
    if (t == 0) ctl[dstQueue] = ctl[srcQueue];
}

static __global__ void __launch_bounds__(256) k_octant_scatter(const float4 *__restrict__ srcO,
    const float4 *__restrict__ srcD, const unsigned int *ctl, int queue,
    const uint32_t *__restrict__ offsets, float4 *__restrict__ dstO, float4 *__restrict__ dstD)
{
    __shared__ uint32_t base[8], warpCount[8][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < 8) base[threadIdx.x] = offsets[threadIdx.x * kSortBlocks + blockIdx.x];
    uint32_t begin, end;
    sort_chunk(ctl[queue], begin, end);
    __syncthreads();
    for (uint32_t t0 = begin; t0 < end; t0 += 256) {
        const uint32_t i = t0 + threadIdx.x;
        const bool valid = i < end;
        float4 o = make_float4(0, 0, 0, 0), d = o;
        uint32_t oct = 8u;
        if (valid) {
            o = srcO[i];
            d = srcD[i];
            oct = dir_octant(d);
        }
        uint32_t rank = 0;
#pragma unroll
        for (uint32_t k = 0; k < 8; k++) {
            uint32_t m = __ballot_sync(0xFFFFFFFFu, oct == k);
            if (lane == 0) warpCount[k][warp] = __popc(m);
            if (oct == k) rank = __popc(m & ((1u << lane) - 1u));
        }
        __syncthreads();
        if (valid) {
            uint32_t before = 0;
            for (int w = 0; w < warp; w++) before += warpCount[oct][w];
            const uint32_t dst = base[oct] + before + rank;
            dstO[dst] = o;
            dstD[dst] = d;
        }
        __syncthreads();
        if (threadIdx.x < 8) {
            uint32_t tot = 0;
            for (int w = 0; w < 8; w++) tot += warpCount[threadIdx.x][w];
            base[threadIdx.x] += tot;
        }
        __syncthreads();
    }
}

// Image position of pixel `pix` of a wave's pixel numbering: row-major in
// the region, or in the tile list (binary search over the tiles' first
// pixels).
// The tile holding item `key` of a list numbered by the exclusive prefix sum
// `start` (binary search: the last tile whose start is <= key).
__device__ __forceinline__ uint32_t tile_of(const uint64_t *start, uint32_t count, uint64_t key)
{
    uint32_t lo = 0, hi = count - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(start + mid) <= key)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void tile_pixel(const WaveParams &wp, uint32_t t, uint64_t local,
    uint32_t &x, uint32_t &y)
{
    const uint4 r = __ldg(wp.tiles + t);
    x = r.x + (uint32_t)(local % r.z);
    y = r.y + (uint32_t)(local / r.z);
}

__device__ __forceinline__ void wave_pixel(const WaveParams &wp, uint64_t pix, uint32_t &x,
    uint32_t &y)
{
    if (!wp.tiles) {
        x = wp.x0 + (uint32_t)(pix % wp.regionW);
        y = wp.y0 + (uint32_t)(pix / wp.regionW);
        return;
    }
    const uint32_t t = tile_of(wp.tileStart, wp.tileCount, pix);
    tile_pixel(wp, t, pix - __ldg(wp.tileStart + t), x, y);
}

static __global__ void __launch_bounds__(256) k_generate(WaveParams wp, WaveBuffers wb)
{
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= wp.paths) return;
    uint32_t x, y, s;
    if (wp.tileSpp) {
        const uint64_t gp = wp.pathBase + p;
        const uint32_t t = tile_of(wp.tilePath, wp.tileCount, gp);
        const uint32_t n = __ldg(wp.tileSpp + t);
        const uint64_t local = gp - __ldg(wp.tilePath + t), lp = local / n;
        s = (uint32_t)(local - lp * n);
        tile_pixel(wp, t, lp, x, y);
    } else {
        s = p % wp.spp;
        wave_pixel(wp, wp.pixelBase + p / wp.spp, x, y);
    }
    uint32_t rng = sample_seed(wp.seed, x, y, s);
    V3 o, d;
    camera_ray(wp.cam, x, y, rng, o, d);
    wb.rayO[p] = make_float4(o.x, o.y, o.z, __int_as_float((int)p));
    wb.rayD[p] = make_float4(d.x, d.y, d.z, __uint_as_float(rng));
}

// Closest hit, 32 queued rays per warp (primary rays by default).  7 blocks of
// 128 per SM (72 registers): 1,521 Msamples/s on the 1080p benchmark frame
// against 1,516 at 6 blocks and 1,521 at 8 (which spills more).
template <class Src, bool kWT>
__global__ void __launch_bounds__(128, 7) k_trace(Src src, const float4 *__restrict__ rayO,
    const float4 *__restrict__ rayD, const unsigned int *queueCount, int4 *hitA, int *hitInst,
    unsigned int *ctl, unsigned long long *counters, uint32_t *status)
{
    int lane = threadIdx.x & 31;
    uint32_t count = *queueCount;
    TraceCounters cnt = {0, 0, 0, 0, 0};
    uint32_t done = 0, hits = 0;
    for (uint32_t guard = 0; guard <= count / 32 + 1; guard++) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&ctl[kCtlTraceWork], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= count) break;
        uint32_t i = base + lane;
        if (i < count) {
            float4 o4 = rayO[i], d4 = rayD[i];
            const SceneView &sv = src.scene((uint32_t)__float_as_int(o4.w));
            RayHit h = trace_closest<true, kWT>(sv, v3(o4.x, o4.y, o4.z), v3(d4.x, d4.y, d4.z),
                status, cnt);
            hitA[i] = make_int4(__float_as_int(h.t), __float_as_int(h.u), __float_as_int(h.v),
                h.prim);
            hitInst[i] = h.inst;
            done++;
            hits += (h.prim >= 0 && h.t > 0.0f) ? 1u : 0u;
        }
    }
    uint32_t v[7] = {done, hits, cnt.topNodes, cnt.meshNodes, cnt.triTests, cnt.boxTests,
        cnt.meshTests};
#pragma unroll
    for (int k = 0; k < 7; k++)
        for (int off = 16; off; off >>= 1) v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
    if (lane == 0) {
        atomicAdd(&counters[GBSP_METRIC_RAYS_TRACED], (unsigned long long)v[0]);
        atomicAdd(&counters[GBSP_METRIC_RAY_HIT_COUNT], (unsigned long long)v[1]);
        atomicAdd(&counters[GBSP_METRIC_RAY_MISS_COUNT], (unsigned long long)(v[0] - v[1]));
        atomicAdd(&counters[GBSP_METRIC_BROADPHASE_NODE_VISITS], (unsigned long long)v[2]);
        atomicAdd(&counters[GBSP_METRIC_MIDPHASE_NODE_VISITS], (unsigned long long)v[3]);
        atomicAdd(&counters[GBSP_METRIC_TRIANGLE_TESTS], (unsigned long long)v[4]);
        atomicAdd(&counters[GBSP_METRIC_MIDPHASE_BOX_TESTS], (unsigned long long)v[5]);
        atomicAdd(&counters[GBSP_METRIC_MESH_TESTS_PERFORMED], (unsigned long long)v[6]);
    }
}

// Per-lane variant of k_trace (bounce rays by default).  Every lane keeps
// its own ray and stack and advances by single steps (one stack pop: an
// object- or mesh-level node visit, entering an object, one triangle leaf,
// leaving an object); a lane whose ray is done takes the next queue index
// straight away, so short rays no longer wait for the warp's longest one.
// The fetch is a warp-aggregated atomic over the lanes that are idle at that
// moment (__activemask), and a lane leaves the loop as soon as the queue is
// exhausted: there is no whole-warp vote or shuffle inside the loop.  Same
// candidate sets, arithmetic and tie rules as trace_closest, hence the same
// hit records.  8 blocks of 128 per SM (64 registers): on the 1080p benchmark
// frame 8 blocks gave 1,516 Msamples/s against 1,468 at 7 (72 registers) and
// 1,461 at 9 (56 registers, which spill).
constexpr uint32_t kMaxLaneRaySteps = 1u << 22;
constexpr int kLaneThreads = 128;  // block size of k_trace_lane
constexpr uint32_t kMaxLaneIterations = 1u << 28;

template <class Src, bool kWT>
__global__ void __launch_bounds__(kLaneThreads, 8) k_trace_lane(Src src, const float4 *__restrict__ rayO,
    const float4 *__restrict__ rayD, const unsigned int *queueCount, int4 *hitA, int *hitInst,
    unsigned int *ctl, unsigned long long *counters, uint32_t *status)
{
    const int lane = threadIdx.x & 31;
    const uint32_t laneMaskLt = (1u << lane) - 1u;
    const uint32_t count = *queueCount;
    unsigned int *work = &ctl[kCtlTraceWork];
    TraceCounters cnt = {0, 0, 0, 0, 0};
    uint32_t done = 0, hits = 0;
    StackEntry stack[kStackSize];
    // State a lane touches only when it fetches a ray, enters or leaves an
    // object, or stores a hit, kept in shared memory on purpose: the walk
    // itself then holds just the current level's ray, bounds and stack
    // pointer in registers.  (In a local array its stores were written
    // through to L2; shared memory keeps them on the SM: 1,556 against
    // 1,552 Msamples/s on the 1080p benchmark frame.)  Word w of the lane
    // is column threadIdx.x of row w, so a warp's accesses to one word are
    // contiguous.  Words: world origin 0-2, direction 3-5, inverse direction
    // 6-8; best hit over objects u 9, v 10, triangle 11, object 12; queue
    // slot 13; object being walked 14; its best triangle's u 15, v 16.
    __shared__ uint32_t coldWords[17 * kLaneThreads];
    struct ColdWords {
        volatile uint32_t *p;
        __device__ __forceinline__ volatile uint32_t &operator[](int w) const
        {
            return p[w * kLaneThreads];
        }
    };
    const ColdWords cold{coldWords + threadIdx.x};
    // next: the entry to visit next (the nearest child of the last node
    // visit, or a root), kept out of the stack; ref kEmptyChild when none
    StackEntry next = StackEntry{kEmptyChild, 0.0f};
    int sp = 0, base = 0;
    int mode = 0;  // 0 needs a ray, 1 object level, 2 mesh level
    uint32_t steps = 0;
    // the ray of the level being walked: world (mode 1) or object space (mode 2)
    V3 ro = v3(0, 0, 0), rinvd = v3(0, 0, 0), ld = v3(0, 0, 0);
    float bestT = kInf;
    float len = 0.0f, lBestT = kInf;
    int32_t lPrim = -1;
    uint32_t pathId = 0;
    bool drained = false;
    const auto put3 = [&](int w, V3 v) {
        cold[w] = __float_as_uint(v.x);
        cold[w + 1] = __float_as_uint(v.y);
        cold[w + 2] = __float_as_uint(v.z);
    };
    const auto get3 = [&](int w) {
        return v3(__uint_as_float(cold[w]), __uint_as_float(cold[w + 1]),
            __uint_as_float(cold[w + 2]));
    };
    for (uint32_t it = 0; it < kMaxLaneIterations; it++) {
        if (mode == 0) {
            unsigned int m = __activemask();
            int leader = __ffs(m) - 1;
            uint32_t first = 0;
            if (lane == leader) first = atomicAdd(work, (unsigned int)__popc(m));
            first = __shfl_sync(m, first, leader);
            uint32_t idx = first + __popc(m & laneMaskLt);
            if (idx >= count) {
                drained = true;
                break;
            }
            steps = 0;
            float4 o4 = rayO[idx], d4 = rayD[idx];
            ro = v3(o4.x, o4.y, o4.z);
            const V3 d = v3(d4.x, d4.y, d4.z);
            pathId = (uint32_t)__float_as_int(o4.w);
            rinvd = inverse(d);
            put3(0, ro);
            put3(3, d);
            put3(6, rinvd);
            cold[9] = 0u;
            cold[10] = 0u;
            cold[11] = 0xFFFFFFFFu;
            cold[12] = 0xFFFFFFFFu;
            cold[13] = idx;
            bestT = kInf;
            sp = 0;
            next = StackEntry{src.scene(pathId).tlasRoot, 0.0f};
            mode = 1;
        }
        if (++steps > kMaxLaneRaySteps) {
            atomicOr(status, kStatusRayStepLimit);
            mode = 1;
            sp = 0;  // store the best hit found so far
            next.ref = kEmptyChild;
        }
        const bool levelDone = sp == (mode == 2 ? base : 0) && next.ref == kEmptyChild;
        if (mode == 2 && levelDone) {
            // leaving an object: its closest triangle goes back to world space
            const V3 o = get3(0);
            if (lPrim >= 0) {
                const uint32_t inst = cold[14];
                const Instance &in = src.scene(pathId).instances[inst];
                Affine model;
#pragma unroll
                for (int k = 0; k < 12; k++) model.r[k] = __ldg(&in.model.r[k]);
                V3 worldHit = transform_point(model, add(ro, mul(ld, lBestT)));
                float tw = dot(sub(worldHit, o), get3(3));
                if (tw < bestT || (tw == bestT && (int32_t)inst < (int32_t)cold[12])) {
                    bestT = tw;
                    cold[9] = cold[15];
                    cold[10] = cold[16];
                    cold[11] = (uint32_t)lPrim;
                    cold[12] = inst;
                }
            }
            ro = o;
            rinvd = get3(6);
            mode = 1;
        } else if (mode == 1 && levelDone) {
            const int32_t bestPrim = (int32_t)cold[11];
            const uint32_t slot = cold[13];
            hitA[slot] = make_int4(__float_as_int(bestT), (int)cold[9], (int)cold[10], bestPrim);
            hitInst[slot] = (int)cold[12];
            done++;
            hits += (bestPrim >= 0 && bestT > 0.0f) ? 1u : 0u;
            mode = 0;
        } else {
            StackEntry top;
            if (next.ref != kEmptyChild) {
                top = next;
                next.ref = kEmptyChild;
            } else {
                sp--;
                top = stack[sp];
            }
            uint32_t ref = top.ref;
            float te = top.t;
            float bound = mode == 1 ? prune_bound(bestT) : prune_bound(rmin(lBestT, bestT * len));
            if (te > bound) {
                // pruned
            } else if (!child_is_leaf(ref)) {
                if (mode == 1)
                    cnt.topNodes++;
                else
                    cnt.meshNodes++;
                next = visit_node<true, kWT, true>(src.scene(pathId).nodes,
                    src.scene(pathId).nodeQuads, ref, ro, rinvd, bound, stack, sp, status, cnt);
            } else if (mode == 1) {
                // an object whose world box passed: enter its mesh
                const uint32_t inst = leaf_first(ref);
                cold[14] = inst;
                const Instance &in = src.scene(pathId).instances[inst];
                Affine inv;
#pragma unroll
                for (int k = 0; k < 12; k++) inv.r[k] = __ldg(&in.inv.r[k]);
                const V3 d = get3(3);
                ro = transform_point(inv, ro);
                ld = normalize(transform_vector(inv, d), &len);
                rinvd = inverse(ld);
                cnt.meshTests++;
                lBestT = kInf;
                lPrim = -1;
                base = sp;
                next = StackEntry{__ldg(&in.blasRoot), 0.0f};
                mode = 2;
            } else {
                visit_leaf_uv<true, kWT>(src.scene(pathId), ref, ro, ld, rinvd, lBestT, lPrim,
                    [&](float u, float v) {
                        cold[15] = __float_as_uint(u);
                        cold[16] = __float_as_uint(v);
                    },
                    cnt);
            }
        }
    }
    if (!drained) atomicOr(status, kStatusQueueOverflow);
    __syncwarp();
    uint32_t v[7] = {done, hits, cnt.topNodes, cnt.meshNodes, cnt.triTests, cnt.boxTests,
        cnt.meshTests};
#pragma unroll
    for (int k = 0; k < 7; k++)
        for (int off = 16; off; off >>= 1) v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
    if (lane == 0) {
        atomicAdd(&counters[GBSP_METRIC_RAYS_TRACED], (unsigned long long)v[0]);
        atomicAdd(&counters[GBSP_METRIC_RAY_HIT_COUNT], (unsigned long long)v[1]);
        atomicAdd(&counters[GBSP_METRIC_RAY_MISS_COUNT], (unsigned long long)(v[0] - v[1]));
        atomicAdd(&counters[GBSP_METRIC_BROADPHASE_NODE_VISITS], (unsigned long long)v[2]);
        atomicAdd(&counters[GBSP_METRIC_MIDPHASE_NODE_VISITS], (unsigned long long)v[3]);
        atomicAdd(&counters[GBSP_METRIC_TRIANGLE_TESTS], (unsigned long long)v[4]);
        atomicAdd(&counters[GBSP_METRIC_MIDPHASE_BOX_TESTS], (unsigned long long)v[5]);
        atomicAdd(&counters[GBSP_METRIC_MESH_TESTS_PERFORMED], (unsigned long long)v[6]);
    }
}

template <class Src>
__global__ void __launch_bounds__(128) k_shade(Src src, WaveBuffers wb, uint32_t bounce, int inQueue,
    unsigned int *ctl, unsigned long long *counters)
{
    int lane = threadIdx.x & 31;
    uint32_t count = ctl[inQueue];
    int outQueue = inQueue == kCtlQueue0 ? kCtlQueue1 : kCtlQueue0;
    const float4 *inO = wb.rayO + (inQueue == kCtlQueue0 ? 0 : wb.cap);
    const float4 *inD = wb.rayD + (inQueue == kCtlQueue0 ? 0 : wb.cap);
    float4 *outO = wb.rayO + (inQueue == kCtlQueue0 ? wb.cap : 0);
    float4 *outD = wb.rayD + (inQueue == kCtlQueue0 ? wb.cap : 0);
    uint32_t finished = 0;
    for (uint32_t guard = 0; guard <= count / 32 + 1; guard++) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&ctl[kCtlShadeWork], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= count) break;
        uint32_t i = base + lane;
        bool active = i < count;
        bool cont = false;
        float4 newO = make_float4(0, 0, 0, 0), newD = make_float4(0, 0, 0, 0);
        uint32_t p = 0;
        if (active) {
            float4 o4 = inO[i], d4 = inD[i];
            p = (uint32_t)__float_as_int(o4.w);
            const SceneView &sv = src.scene(p);
            const MaterialView &mv = src.materials(p);
            bool lastBounce = bounce + 1 >= src.bounces(p);
            int4 hA = wb.hitA[i];
            RayHit h;
            h.t = __int_as_float(hA.x);
            h.u = __int_as_float(hA.y);
            h.v = __int_as_float(hA.z);
            h.prim = hA.w;
            h.inst = wb.hitInst[i];
            V3 o = v3(o4.x, o4.y, o4.z), d = v3(d4.x, d4.y, d4.z);
            // every path in this queue has `bounce` vertices so far
            const uint32_t len = bounce;
            float4 ec, aa;
            if (h.prim >= 0 && h.t > 0.0f) {
                // hit vertex (src/simd_path_tracer.cpp:268-288)
                V3 n;
                float ux, uy;
                hit_surface(sv, h, n, ux, uy);
                V3 pos = add(o, mul(d, h.t));
                uint32_t rng = __float_as_uint(d4.w);
                V3 dir = random_hemisphere(n, rng);
                int slot = mv.instanceSlot[h.inst];
                vertex_terms(mv, slot, n, dir, neg(d), ux, uy, ec, aa);
                V3 no = add(pos, mul(n, 0.0001f));
                newO = make_float4(no.x, no.y, no.z, __int_as_float((int)p));
                newD = make_float4(dir.x, dir.y, dir.z, __uint_as_float(rng));
                cont = !lastBounce;
                if (wb.pathAov && bounce == 0) {
                    V3 al = material_albedo(mv, slot, ux, uy);
                    wb.pathAov[2 * (size_t)p] = make_float4(al.x, al.y, al.z, h.t);
                    wb.pathAov[2 * (size_t)p + 1] = make_float4(n.x, n.y, n.z, 1.0f);
                }
            } else {
                // miss: background vertex, path ends (:302-314)
                vertex_terms(mv, mv.backgroundSlot, v3(0, 0, 0), v3(0, 0, 0), neg(d), 0.0f, 0.0f,
                    ec, aa);
                if (wb.pathAov && bounce == 0) {
                    wb.pathAov[2 * (size_t)p] = make_float4(0, 0, 0, 0);
                    wb.pathAov[2 * (size_t)p + 1] = make_float4(0, 0, 0, 0);
                }
            }
            if (cont) {
                wb.vertE[(size_t)len * wb.cap + p] = ec;
                wb.vertA[(size_t)len * wb.cap + p] = aa;
            } else {
                // the path ends at this vertex: the reverse pass starts from it
                V3 r = path_radiance_last(wb.vertE, wb.vertA, wb.cap, p, len + 1, ec, aa,
                    src.clamp(p));
                wb.pathRad[p] = make_float4(r.x, r.y, r.z, 0.0f);
                finished++;
            }
        }
        // compaction: one atomic per warp for the continuing rays
        uint32_t mask = __ballot_sync(0xFFFFFFFFu, cont);
        uint32_t outBase = 0;
        if (lane == 0 && mask) outBase = atomicAdd(&ctl[outQueue], (unsigned)__popc(mask));
        outBase = __shfl_sync(0xFFFFFFFFu, outBase, 0);
        if (cont) {
            uint32_t slot = outBase + __popc(mask & ((1u << lane) - 1u));
            outO[slot] = newO;
            outD[slot] = newD;
        }
    }
    for (int off = 16; off; off >>= 1) finished += __shfl_xor_sync(0xFFFFFFFFu, finished, off);
    if (lane == 0 && finished)
        atomicAdd(&counters[GBSP_METRIC_PATHS_TRACED], (unsigned long long)finished);
}

static __global__ void __launch_bounds__(256) k_accumulate(WaveParams wp, WaveBuffers wb, float4 *image,
    uint32_t imageWidth, unsigned long long *counters)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nans = 0;
    if (k < wp.pixels) {
        uint64_t pix = wp.pixelBase + k;
        uint32_t x, y, n = wp.spp;
        size_t first = (size_t)k * wp.spp;  // this pixel's first path in the wave
        float inv = wp.invSpp;
        if (wp.tileSpp) {
            const uint32_t t = tile_of(wp.tileStart, wp.tileCount, pix);
            const uint64_t lp = pix - __ldg(wp.tileStart + t);
            n = __ldg(wp.tileSpp + t);
            first = (size_t)(__ldg(wp.tilePath + t) + lp * n - wp.pathBase);
            inv = 1.0f / (float)n;
            tile_pixel(wp, t, lp, x, y);
        } else {
            wave_pixel(wp, pix, x, y);
        }
        // with a split, the image holds the first splitSpp samples, image2 the rest
        const uint32_t nFirst = wp.splitSpp ? wp.splitSpp : n;
        if (wp.splitSpp) inv = 1.0f / (float)nFirst;
        CSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
        for (uint32_t s = 0; s < nFirst; s++) {
            float4 r = wb.pathRad[first + s];
            if (isnan(r.x) || isnan(r.y) || isnan(r.z)) {
                nans++;
                if (wp.nanPolicy == GBSP_NAN_ZERO) continue;
            }
            csum_add(acc[0], r.x * inv);
            csum_add(acc[1], r.y * inv);
            csum_add(acc[2], r.z * inv);
        }
        image[(size_t)y * imageWidth + x] =
            make_float4(csum_value(acc[0]), csum_value(acc[1]), csum_value(acc[2]), 1.0f);
        if (wp.splitSpp) {
            const float inv2 = 1.0f / (float)(n - nFirst);
            CSum acc2[3] = {{0, 0}, {0, 0}, {0, 0}};
            for (uint32_t s = nFirst; s < n; s++) {
                float4 r = wb.pathRad[first + s];
                if (isnan(r.x) || isnan(r.y) || isnan(r.z)) {
                    nans++;
                    if (wp.nanPolicy == GBSP_NAN_ZERO) continue;
                }
                csum_add(acc2[0], r.x * inv2);
                csum_add(acc2[1], r.y * inv2);
                csum_add(acc2[2], r.z * inv2);
            }
            wp.image2[(size_t)y * imageWidth + x] =
                make_float4(csum_value(acc2[0]), csum_value(acc2[1]), csum_value(acc2[2]), 1.0f);
        }
        if (wp.aovImage) {
            float4 a = make_float4(0, 0, 0, 0), b = make_float4(0, 0, 0, 0);
            for (uint32_t s = 0; s < nFirst; s++) {
                float4 u = wb.pathAov[2 * (first + s)];
                float4 v = wb.pathAov[2 * (first + s) + 1];
                a = make_float4(a.x + u.x, a.y + u.y, a.z + u.z, a.w + u.w);
                b = make_float4(b.x + v.x, b.y + v.y, b.z + v.z, b.w + v.w);
            }
            float is = inv;
            size_t o = 2 * ((size_t)y * imageWidth + x);
            wp.aovImage[o] = make_float4(a.x * is, a.y * is, a.z * is, a.w * is);
            wp.aovImage[o + 1] = make_float4(b.x * is, b.y * is, b.z * is, b.w * is);
        }
    }
    for (int off = 16; off; off >>= 1) nans += __shfl_xor_sync(0xFFFFFFFFu, nans, off);
    if ((threadIdx.x & 31) == 0 && nans)
        atomicAdd(&counters[GBSP_METRIC_NAN_SAMPLES], (unsigned long long)nans);
}

// Persistent grid of k_shade: every block an SM can hold (the kernel waits on
// scattered loads, so more resident warps hide more of that latency).
template <class Src>
int shade_grid(int smCount)
{
    static int perSm = 0;
    if (perSm == 0) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shade<Src>, 128, 0) !=
                cudaSuccess || n < 1)
            n = 8;
        perSm = n;
    }
    return smCount * perSm;
}

// Persistent grid of the closest-hit kernel launch_trace_stage picks: every
// block the SMs hold at once (blocks beyond that would only start once others
// have drained the queue).
template <class K>
int resident_blocks_per_sm(K kernel)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, 128, 0) != cudaSuccess || n < 1)
        n = 6;
    return n;
}

template <class Src>
int trace_grid(bool perLane, bool watertight, int smCount)
{
    static const int lane[2] = {resident_blocks_per_sm(k_trace_lane<Src, false>),
        resident_blocks_per_sm(k_trace_lane<Src, true>)};
    static const int warp[2] = {resident_blocks_per_sm(k_trace<Src, false>),
        resident_blocks_per_sm(k_trace<Src, true>)};
    return smCount * (perLane ? lane[watertight ? 1 : 0] : warp[watertight ? 1 : 0]);
}

// Launches the closest-hit kernel of one bounce: per-warp or per-lane
// scheduling, reference MT or watertight triangle test (template arguments,
// so neither choice costs the other anything).
template <class Src>
void launch_trace_stage(bool perLane, bool watertight, int grid, cudaStream_t s, const Src &src,
    const float4 *qO, const float4 *qD, const unsigned int *queueCount, int4 *hitA, int *hitInst,
    unsigned int *ctl, unsigned long long *counters, uint32_t *status)
{
    if (perLane) {
        if (watertight)
            k_trace_lane<Src, true><<<grid, kLaneThreads, 0, s>>>(src, qO, qD, queueCount, hitA, hitInst,
                ctl, counters, status);
        else
            k_trace_lane<Src, false><<<grid, kLaneThreads, 0, s>>>(src, qO, qD, queueCount, hitA, hitInst,
                ctl, counters, status);
    } else {
        if (watertight)
            k_trace<Src, true><<<grid, 128, 0, s>>>(src, qO, qD, queueCount, hitA, hitInst, ctl,
                counters, status);
        else
            k_trace<Src, false><<<grid, 128, 0, s>>>(src, qO, qD, queueCount, hitA, hitInst, ctl,
                counters, status);
    }
}

}  // namespace gbsp
