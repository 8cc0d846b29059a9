// Wavefront path tracer: the tile loop of sp_PathTraceTile
// (src/simd_path_tracer.cpp:178-345) split into stages over a wave of paths.
//
//   generate   one thread per (pixel, sample): seed, jitter, camera ray
//   trace      persistent closest-hit kernel pulling 32 rays per warp from a
//              global atomic counter
//   shade      persistent: surface attributes, hemisphere sample, material
//              and BRDF terms of the path vertex; continuing rays are
//              compacted into the next queue with one atomic per warp
//              (ballot + popc); finished paths are evaluated at once
//   accumulate one thread per pixel: Neumaier sum of sample * (1/spp)
//
// A wave holds a run of whole pixels with all their samples, so the
// accumulation is a deterministic, ordered sum per pixel.  Bounce counts and
// queue sizes stay on the device: a wave is enqueued with no host round trip.
//
// ComputeRadianceForPath (src/simd_path_tracer.cpp:107-175) evaluates each
// vertex from its own data plus the clamped radiance of the next vertex.
// The per-vertex part is computed at shade time and stored as
// E (emission), A (kD*albedo/pi + specular) and the cosine; the reverse pass
// then is radiance = E + (A * clamp(radiance_next)) * cos, the reference's
// expression in the reference's order.

#include <algorithm>
#include <mutex>

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
    float4 *rayO;      // 2 * cap: (origin, path id bits)
    float4 *rayD;      // 2 * cap: (direction, 0)
    int4 *hitA;        // cap: (t, u, v, prim) bits
    int *hitInst;      // cap
    uint32_t *pathRng; // cap
    uint32_t *pathLen; // cap
    float4 *vertE;     // maxBounces * cap: (emission xyz, cosine)
    float4 *vertA;     // maxBounces * cap: (A xyz, 0)
    float4 *pathRad;   // cap
    float4 *pathAov;   // 2 * cap first-hit G-buffer per path, or null
    uint32_t cap;
};

struct WaveParams {
    CameraParams cam;
    uint32_t x0, y0, regionW;
    uint64_t pixelBase;   // first pixel (row-major in the region) of this wave
    uint32_t pixels;      // pixels in this wave
    uint32_t spp;
    uint32_t maxBounces;
    uint32_t seed;
    float clampValue;
    uint32_t nanPolicy;
    float invSpp;
    float4 *aovImage;     // 2 float4 per image pixel, or null
};

// ---------------------------------------------------------------------------
// Stage kernels
// ---------------------------------------------------------------------------
__global__ void k_reset_ctl(unsigned int *ctl, uint32_t queue0)
{
    if (threadIdx.x < kCtlCount) ctl[threadIdx.x] = 0;
    __syncthreads();
    if (threadIdx.x == 0) ctl[kCtlQueue0] = queue0;
}

__global__ void k_reset_stage(unsigned int *ctl, int outQueue)
{
    ctl[kCtlTraceWork] = 0;
    ctl[kCtlShadeWork] = 0;
    ctl[outQueue] = 0;
}

__global__ void __launch_bounds__(256) k_generate(WaveParams wp, WaveBuffers wb)
{
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t paths = wp.pixels * wp.spp;
    if (p >= paths) return;
    uint64_t pix = wp.pixelBase + p / wp.spp;
    uint32_t s = p % wp.spp;
    uint32_t x = wp.x0 + (uint32_t)(pix % wp.regionW);
    uint32_t y = wp.y0 + (uint32_t)(pix / wp.regionW);
    uint32_t rng = sample_seed(wp.seed, x, y, s);
    V3 o, d;
    camera_ray(wp.cam, x, y, rng, o, d);
    wb.rayO[p] = make_float4(o.x, o.y, o.z, __int_as_float((int)p));
    wb.rayD[p] = make_float4(d.x, d.y, d.z, 0.0f);
    wb.pathRng[p] = rng;
    wb.pathLen[p] = 0;
}

__global__ void __launch_bounds__(128) k_trace(SceneView sv, const float4 *__restrict__ rayO,
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
            RayHit h = trace_closest<true>(sv, v3(o4.x, o4.y, o4.z), v3(d4.x, d4.y, d4.z), status,
                cnt);
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

// Per-lane variant of k_trace (GBSP_FLAG_TRACE_PER_LANE).  Every lane keeps
// its own ray and stack and advances by single steps (one stack pop: an
// object- or mesh-level node visit, entering an object, one triangle leaf,
// leaving an object); a lane whose ray is done takes the next queue index
// straight away, so short rays no longer wait for the warp's longest one.
// The fetch is a warp-aggregated atomic over the lanes that are idle at that
// moment (__activemask), and a lane leaves the loop as soon as the queue is
// exhausted: there is no whole-warp vote or shuffle inside the loop.  Same
// candidate sets, arithmetic and tie rules as trace_closest, hence the same
// hit records.
constexpr uint32_t kMaxLaneRaySteps = 1u << 22;
constexpr uint32_t kMaxLaneIterations = 1u << 28;

__global__ void __launch_bounds__(128) k_trace_lane(SceneView sv, const float4 *__restrict__ rayO,
    const float4 *__restrict__ rayD, const unsigned int *queueCount, int4 *hitA, int *hitInst,
    unsigned int *ctl, unsigned long long *counters, uint32_t *status)
{
    const int lane = threadIdx.x & 31;
    const uint32_t laneMaskLt = (1u << lane) - 1u;
    const uint32_t count = *queueCount;
    unsigned int *work = &ctl[kCtlTraceWork];
    TraceCounters cnt = {0, 0, 0, 0, 0};
    uint32_t done = 0, hits = 0;
    uint32_t stackRef[kStackSize];
    float stackT[kStackSize];
    int sp = 0, base = 0;
    int mode = 0;  // 0 needs a ray, 1 object level, 2 mesh level
    uint32_t slot = 0, steps = 0, inst = 0;
    V3 o = v3(0, 0, 0), d = v3(0, 0, 0), invd = v3(0, 0, 0);
    float bestT = kInf, bestU = 0.0f, bestV = 0.0f;
    int32_t bestPrim = -1, bestInst = -1;
    V3 lo = v3(0, 0, 0), ld = v3(0, 0, 0), linvd = v3(0, 0, 0);
    float len = 0.0f, lBestT = kInf, lU = 0.0f, lV = 0.0f;
    int32_t lPrim = -1;
    bool drained = false;
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
            slot = idx;
            steps = 0;
            float4 o4 = rayO[idx], d4 = rayD[idx];
            o = v3(o4.x, o4.y, o4.z);
            d = v3(d4.x, d4.y, d4.z);
            invd = inverse(d);
            bestT = kInf;
            bestU = bestV = 0.0f;
            bestPrim = bestInst = -1;
            sp = 0;
            if (sv.tlasRoot != kEmptyChild) {
                stackRef[0] = sv.tlasRoot;
                stackT[0] = 0.0f;
                sp = 1;
            }
            mode = 1;
        }
        if (++steps > kMaxLaneRaySteps) {
            atomicOr(status, kStatusRayStepLimit);
            mode = 1;
            sp = 0;  // store the best hit found so far
        }
        if (mode == 2 && sp == base) {
            // leaving an object: its closest triangle goes back to world space
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
            mode = 1;
        } else if (mode == 1 && sp == 0) {
            hitA[slot] = make_int4(__float_as_int(bestT), __float_as_int(bestU),
                __float_as_int(bestV), bestPrim);
            hitInst[slot] = bestInst;
            done++;
            hits += (bestPrim >= 0 && bestT > 0.0f) ? 1u : 0u;
            mode = 0;
        } else {
            sp--;
            uint32_t ref = stackRef[sp];
            float te = stackT[sp];
            float bound = mode == 1 ? prune_bound(bestT) : prune_bound(rmin(lBestT, bestT * len));
            if (te > bound) {
                // pruned
            } else if (!child_is_leaf(ref)) {
                if (mode == 1)
                    cnt.topNodes++;
                else
                    cnt.meshNodes++;
                visit_node<true>(sv.nodes, ref, mode == 1 ? o : lo, mode == 1 ? invd : linvd,
                    bound, stackRef, stackT, sp, status, cnt);
            } else if (mode == 1) {
                // an object whose world box passed: enter its mesh
                inst = leaf_first(ref);
                const Instance &in = sv.instances[inst];
                Affine inv;
#pragma unroll
                for (int k = 0; k < 12; k++) inv.r[k] = __ldg(&in.inv.r[k]);
                lo = transform_point(inv, o);
                ld = normalize(transform_vector(inv, d), &len);
                linvd = inverse(ld);
                cnt.meshTests++;
                lBestT = kInf;
                lU = lV = 0.0f;
                lPrim = -1;
                base = sp;
                if (sp >= kStackSize) {
                    atomicOr(status, kStatusStackOverflow);
                } else {
                    stackRef[sp] = __ldg(&in.blasRoot);
                    stackT[sp] = 0.0f;
                    sp++;
                    mode = 2;
                }
            } else {
                visit_leaf<true>(sv, ref, lo, ld, linvd, lBestT, lU, lV, lPrim, cnt);
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

__global__ void __launch_bounds__(128) k_shade(SceneView sv, MaterialView mv, WaveParams wp,
    WaveBuffers wb, uint32_t bounce, int inQueue, unsigned int *ctl, unsigned long long *counters)
{
    int lane = threadIdx.x & 31;
    uint32_t count = ctl[inQueue];
    int outQueue = inQueue == kCtlQueue0 ? kCtlQueue1 : kCtlQueue0;
    const float4 *inO = wb.rayO + (inQueue == kCtlQueue0 ? 0 : wb.cap);
    const float4 *inD = wb.rayD + (inQueue == kCtlQueue0 ? 0 : wb.cap);
    float4 *outO = wb.rayO + (inQueue == kCtlQueue0 ? wb.cap : 0);
    float4 *outD = wb.rayD + (inQueue == kCtlQueue0 ? wb.cap : 0);
    bool lastBounce = bounce + 1 >= wp.maxBounces;
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
            int4 hA = wb.hitA[i];
            RayHit h;
            h.t = __int_as_float(hA.x);
            h.u = __int_as_float(hA.y);
            h.v = __int_as_float(hA.z);
            h.prim = hA.w;
            h.inst = wb.hitInst[i];
            V3 o = v3(o4.x, o4.y, o4.z), d = v3(d4.x, d4.y, d4.z);
            uint32_t len = wb.pathLen[p];
            float4 ec, aa;
            if (h.prim >= 0 && h.t > 0.0f) {
                // hit vertex (src/simd_path_tracer.cpp:268-288)
                V3 n;
                float ux, uy;
                hit_surface(sv, h, n, ux, uy);
                V3 pos = add(o, mul(d, h.t));
                uint32_t rng = wb.pathRng[p];
                V3 dir = random_hemisphere(n, rng);
                wb.pathRng[p] = rng;
                int slot = mv.instanceSlot[h.inst];
                vertex_terms(mv, slot, n, dir, neg(d), ux, uy, ec, aa);
                V3 no = add(pos, mul(n, 0.0001f));
                newO = make_float4(no.x, no.y, no.z, __int_as_float((int)p));
                newD = make_float4(dir.x, dir.y, dir.z, 0.0f);
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
            wb.vertE[(size_t)len * wb.cap + p] = ec;
            wb.vertA[(size_t)len * wb.cap + p] = aa;
            len++;
            wb.pathLen[p] = len;
            if (!cont) {
                V3 r = path_radiance(wb.vertE, wb.vertA, wb.cap, p, len, wp.clampValue);
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

__global__ void __launch_bounds__(256) k_accumulate(WaveParams wp, WaveBuffers wb, float4 *image,
    uint32_t imageWidth, unsigned long long *counters)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nans = 0;
    if (k < wp.pixels) {
        uint64_t pix = wp.pixelBase + k;
        uint32_t x = wp.x0 + (uint32_t)(pix % wp.regionW);
        uint32_t y = wp.y0 + (uint32_t)(pix / wp.regionW);
        CSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
        for (uint32_t s = 0; s < wp.spp; s++) {
            float4 r = wb.pathRad[(size_t)k * wp.spp + s];
            if (isnan(r.x) || isnan(r.y) || isnan(r.z)) {
                nans++;
                if (wp.nanPolicy == GBSP_NAN_ZERO) continue;
            }
            csum_add(acc[0], r.x * wp.invSpp);
            csum_add(acc[1], r.y * wp.invSpp);
            csum_add(acc[2], r.z * wp.invSpp);
        }
        image[(size_t)y * imageWidth + x] =
            make_float4(csum_value(acc[0]), csum_value(acc[1]), csum_value(acc[2]), 1.0f);
        if (wp.aovImage) {
            float4 a = make_float4(0, 0, 0, 0), b = make_float4(0, 0, 0, 0);
            for (uint32_t s = 0; s < wp.spp; s++) {
                float4 u = wb.pathAov[2 * ((size_t)k * wp.spp + s)];
                float4 v = wb.pathAov[2 * ((size_t)k * wp.spp + s) + 1];
                a = make_float4(a.x + u.x, a.y + u.y, a.z + u.z, a.w + u.w);
                b = make_float4(b.x + v.x, b.y + v.y, b.z + v.z, b.w + v.w);
            }
            float is = wp.invSpp;
            size_t o = 2 * ((size_t)y * imageWidth + x);
            wp.aovImage[o] = make_float4(a.x * is, a.y * is, a.z * is, a.w * is);
            wp.aovImage[o + 1] = make_float4(b.x * is, b.y * is, b.z * is, b.w * is);
        }
    }
    for (int off = 16; off; off >>= 1) nans += __shfl_xor_sync(0xFFFFFFFFu, nans, off);
    if ((threadIdx.x & 31) == 0 && nans)
        atomicAdd(&counters[GBSP_METRIC_NAN_SAMPLES], (unsigned long long)nans);
}

// ---------------------------------------------------------------------------
// Reference-order tile mode: one thread walks one tile exactly like
// sp_PathTraceTile, drawing every random number from one XorShift32 stream.
// ---------------------------------------------------------------------------
constexpr int kMaxSeqBounces = 16;

__global__ void __launch_bounds__(64) k_tile_sequential(SceneView sv, MaterialView mv,
    CameraParams cam, const uint4 *tiles, uint32_t tileCount, uint32_t *rngStates, uint32_t spp,
    uint32_t maxBounces, float clampValue, float4 *image, uint32_t imageWidth,
    unsigned long long *counters, uint32_t *status)
{
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tileCount) return;
    uint4 tile = tiles[t];
    uint32_t rng = rngStates[t];
    uint32_t maxX = tile.z < cam.width ? tile.z : cam.width;
    uint32_t maxY = tile.w < cam.height ? tile.w : cam.height;
    float4 vE[kMaxSeqBounces], vA[kMaxSeqBounces];
    TraceCounters cnt = {0, 0, 0, 0, 0};
    uint64_t rays = 0, hits = 0, paths = 0;
    for (uint32_t y = tile.y; y < maxY; y++) {
        for (uint32_t x = tile.x; x < maxX; x++) {
            V3 total = v3(0, 0, 0);
            for (uint32_t s = 0; s < spp; s++) {
                V3 o, d;
                camera_ray(cam, x, y, rng, o, d);
                uint32_t len = 0;
                for (uint32_t b = 0; b < maxBounces; b++) {
                    RayHit h = trace_closest<true>(sv, o, d, status, cnt);
                    rays++;
                    float4 ec, aa;
                    if (h.prim >= 0 && h.t > 0.0f) {
                        hits++;
                        V3 n;
                        float ux, uy;
                        hit_surface(sv, h, n, ux, uy);
                        V3 pos = add(o, mul(d, h.t));
                        V3 dir = random_hemisphere(n, rng);
                        vertex_terms(mv, mv.instanceSlot[h.inst], n, dir, neg(d), ux, uy, ec, aa);
                        vE[len] = ec;
                        vA[len] = aa;
                        len++;
                        o = add(pos, mul(n, 0.0001f));
                        d = dir;
                    } else {
                        vertex_terms(mv, mv.backgroundSlot, v3(0, 0, 0), v3(0, 0, 0), neg(d), 0.0f,
                            0.0f, ec, aa);
                        vE[len] = ec;
                        vA[len] = aa;
                        len++;
                        break;
                    }
                }
                V3 r = path_radiance(vE, vA, 1, 0, len, clampValue);
                total = add(total, mul(r, 1.0f / (float)spp));
                paths++;
            }
            image[(size_t)y * imageWidth + x] = make_float4(total.x, total.y, total.z, 1.0f);
        }
    }
    rngStates[t] = rng;
    atomicAdd(&counters[GBSP_METRIC_RAYS_TRACED], (unsigned long long)rays);
    atomicAdd(&counters[GBSP_METRIC_RAY_HIT_COUNT], (unsigned long long)hits);
    atomicAdd(&counters[GBSP_METRIC_RAY_MISS_COUNT], (unsigned long long)(rays - hits));
    atomicAdd(&counters[GBSP_METRIC_PATHS_TRACED], (unsigned long long)paths);
    atomicAdd(&counters[GBSP_METRIC_TRIANGLE_TESTS], (unsigned long long)cnt.triTests);
    atomicAdd(&counters[GBSP_METRIC_MIDPHASE_BOX_TESTS], (unsigned long long)cnt.boxTests);
    atomicAdd(&counters[GBSP_METRIC_MESH_TESTS_PERFORMED], (unsigned long long)cnt.meshTests);
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
static int ensure_wave_buffers(gbsp_runtime *rt, uint32_t cap, uint32_t maxBounces)
{
    cudaStream_t s = rt->stream;
    int rc;
    if ((rc = rt->rayO.reserve(2 * (size_t)cap, s)) || (rc = rt->rayD.reserve(2 * (size_t)cap, s)) ||
        (rc = rt->hitA.reserve(cap, s)) || (rc = rt->hitInst.reserve(cap, s)) ||
        (rc = rt->pathRng.reserve(cap, s)) || (rc = rt->pathLen.reserve(cap, s)) ||
        (rc = rt->vertE.reserve((size_t)maxBounces * cap, s)) ||
        (rc = rt->vertA.reserve((size_t)maxBounces * cap, s)) ||
        (rc = rt->pathRad.reserve(cap, s)))
        return rc;
    return GBSP_OK;
}

int render_frame(gbsp_runtime *rt, const SceneView &sv, const MaterialView &mv,
    const CameraParams &cam, const gbsp_options &opt, uint32_t x0, uint32_t y0, uint32_t x1,
    uint32_t y1, float4 *dImage, uint32_t imageWidth, uint32_t *rngState, float4 *dAov)
{
    cudaStream_t s = rt->stream;
    unsigned long long *counters = rt->dCounters;
    unsigned int *ctl = reinterpret_cast<unsigned int *>(rt->dCounters + GBSP_METRIC_COUNT);
    if (x1 <= x0 || y1 <= y0) return GBSP_OK;
    uint32_t spp = opt.spp ? opt.spp : 1;
    uint32_t maxBounces = opt.max_bounces;
    if (maxBounces == 0) {
        // no bounce at all: every path has zero vertices and zero radiance
        maxBounces = 0;
    }
    if (opt.rng_mode == GBSP_RNG_TILE_SEQUENTIAL) {
        if (maxBounces > (uint32_t)kMaxSeqBounces)
            return set_error(GBSP_ERR_CAPACITY, "tile-sequential mode supports at most %d bounces",
                kMaxSeqBounces);
        // tiles of 64x64 in row-major order (src/tile.h:11-42), each starting
        // from the caller's RNG state (src/main.cpp:738-739); with one tile
        // the state is advanced and returned (sp_PathTraceTile semantics)
        std::vector<uint4> tiles;
        uint32_t tw = rngState ? (x1 - x0) : 64u, th = rngState ? (y1 - y0) : 64u;
        for (uint32_t ty = y0; ty < y1; ty += th)
            for (uint32_t tx = x0; tx < x1; tx += tw)
                tiles.push_back(make_uint4(tx, ty, std::min(tx + tw, x1), std::min(ty + th, y1)));
        std::vector<uint32_t> states(tiles.size(), rngState ? *rngState : 0xF51C0E49u);
        DeviceBuffer<uint4> dTiles;
        DeviceBuffer<uint32_t> dStates;
        int rc;
        if ((rc = dTiles.upload(tiles.data(), tiles.size(), s)) ||
            (rc = dStates.upload(states.data(), states.size(), s)))
            return rc;
        uint32_t n = (uint32_t)tiles.size();
        k_tile_sequential<<<(n + 63) / 64, 64, 0, s>>>(sv, mv, cam, dTiles.ptr, n, dStates.ptr, spp,
            maxBounces, opt.radiance_clamp, dImage, imageWidth, counters, rt->dStatus);
        GBSP_CUDA_TRY(cudaGetLastError());
        rt->launches += 1;
        if (rngState) {
            GBSP_CUDA_TRY(cudaMemcpyAsync(rngState, dStates.ptr, 4, cudaMemcpyDeviceToHost, s));
            GBSP_CUDA_TRY(cudaStreamSynchronize(s));
        }
        return GBSP_OK;
    }

    uint64_t regionPixels = (uint64_t)(x1 - x0) * (y1 - y0);
    uint64_t waveTarget = opt.wave_paths ? opt.wave_paths : (1u << 22);
    uint64_t pixelsPerWave = std::max<uint64_t>(1, waveTarget / spp);
    pixelsPerWave = std::min<uint64_t>(pixelsPerWave, regionPixels);
    uint64_t capWide = pixelsPerWave * spp;
    if (capWide > 0x7FFFFFFFull)
        return set_error(GBSP_ERR_CAPACITY, "wave of %llu paths is too large",
            (unsigned long long)capWide);
    uint32_t cap = (uint32_t)capWide;
    int rc = ensure_wave_buffers(rt, cap, std::max<uint32_t>(maxBounces, 1));
    if (rc) return rc;
    WaveBuffers wb;
    wb.rayO = rt->rayO.ptr;
    wb.rayD = rt->rayD.ptr;
    wb.hitA = rt->hitA.ptr;
    wb.hitInst = rt->hitInst.ptr;
    wb.pathRng = rt->pathRng.ptr;
    wb.pathLen = rt->pathLen.ptr;
    wb.vertE = rt->vertE.ptr;
    wb.vertA = rt->vertA.ptr;
    wb.pathRad = rt->pathRad.ptr;
    wb.pathAov = nullptr;
    if (dAov) {
        if ((rc = rt->pathAov.reserve(2 * (size_t)cap, s))) return rc;
        wb.pathAov = rt->pathAov.ptr;
    }
    wb.cap = cap;
    WaveParams wp;
    wp.cam = cam;
    wp.x0 = x0;
    wp.y0 = y0;
    wp.regionW = x1 - x0;
    wp.spp = spp;
    wp.maxBounces = maxBounces;
    wp.seed = opt.seed;
    wp.clampValue = opt.radiance_clamp;
    wp.nanPolicy = opt.nan_policy;
    wp.invSpp = 1.0f / (float)spp;
    wp.aovImage = dAov;
    int persistentGrid = rt->smCount * 8;
    bool timing = rt->stageTiming;
    for (uint64_t pb = 0; pb < regionPixels; pb += pixelsPerWave) {
        wp.pixelBase = pb;
        wp.pixels = (uint32_t)std::min<uint64_t>(pixelsPerWave, regionPixels - pb);
        uint32_t paths = wp.pixels * spp;
        if (maxBounces == 0) {
            GBSP_CUDA_TRY(cudaMemsetAsync(wb.pathRad, 0, sizeof(float4) * (size_t)paths, s));
        } else {
            k_reset_ctl<<<1, 32, 0, s>>>(ctl, paths);
            k_generate<<<(paths + 255) / 256, 256, 0, s>>>(wp, wb);
            rt->launches += 2;
            for (uint32_t b = 0; b < maxBounces; b++) {
                int inQ = (b & 1) ? kCtlQueue1 : kCtlQueue0;
                int outQ = (b & 1) ? kCtlQueue0 : kCtlQueue1;
                const float4 *qO = wb.rayO + ((b & 1) ? cap : 0);
                const float4 *qD = wb.rayD + ((b & 1) ? cap : 0);
                k_reset_stage<<<1, 1, 0, s>>>(ctl, outQ);
                int e0 = timing ? rt->stage_event(s) : -1;
                if (opt.flags & GBSP_FLAG_TRACE_PER_LANE)
                    k_trace_lane<<<persistentGrid, 128, 0, s>>>(sv, qO, qD, ctl + inQ, wb.hitA,
                        wb.hitInst, ctl, counters, rt->dStatus);
                else
                    k_trace<<<persistentGrid, 128, 0, s>>>(sv, qO, qD, ctl + inQ, wb.hitA,
                        wb.hitInst, ctl, counters, rt->dStatus);
                int e1 = timing ? rt->stage_event(s) : -1;
                k_shade<<<persistentGrid, 128, 0, s>>>(sv, mv, wp, wb, b, inQ, ctl, counters);
                int e2 = timing ? rt->stage_event(s) : -1;
                if (timing && e0 >= 0 && e1 >= 0 && e2 >= 0) {
                    rt->traceSpans.emplace_back(e0, e1);
                    rt->shadeSpans.emplace_back(e1, e2);
                }
                rt->launches += 3;
                rt->traceLaunches += 1;
            }
        }
        k_accumulate<<<(wp.pixels + 255) / 256, 256, 0, s>>>(wp, wb, dImage, imageWidth, counters);
        rt->launches += 1;
        GBSP_CUDA_TRY(cudaGetLastError());
    }
    return GBSP_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free tile render (gbsp_path_trace_tile_noalloc).
//
// Its working memory is this one file-scope device array, laid out below.
// Host code never uses the symbol as an address: the device address comes
// from cudaGetSymbolAddress, once per device, with that device current.
// ---------------------------------------------------------------------------
constexpr uint32_t kNoAllocMaxPaths = 16384;
constexpr uint32_t kNoAllocMaxBounces = 8;
constexpr uint32_t kNoAllocMaxObjects = 4096;
constexpr size_t kNoAllocAlign = 256;

constexpr size_t na_align(size_t x) { return (x + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign; }
constexpr size_t kNaCtl = 0;  // metric counters + control words + status
constexpr size_t kNaCtlBytes = sizeof(unsigned long long) * (GBSP_METRIC_COUNT + 16) + 16;
constexpr size_t kNaSlots = na_align(kNaCtl + kNaCtlBytes);
constexpr size_t kNaRayO = na_align(kNaSlots + 4 * (size_t)kNoAllocMaxObjects);
constexpr size_t kNaRayD = na_align(kNaRayO + 2 * 16 * (size_t)kNoAllocMaxPaths);
constexpr size_t kNaHitA = na_align(kNaRayD + 2 * 16 * (size_t)kNoAllocMaxPaths);
constexpr size_t kNaHitInst = na_align(kNaHitA + 16 * (size_t)kNoAllocMaxPaths);
constexpr size_t kNaRng = na_align(kNaHitInst + 4 * (size_t)kNoAllocMaxPaths);
constexpr size_t kNaLen = na_align(kNaRng + 4 * (size_t)kNoAllocMaxPaths);
constexpr size_t kNaVertE = na_align(kNaLen + 4 * (size_t)kNoAllocMaxPaths);
constexpr size_t kNaVertA = na_align(kNaVertE + 16 * (size_t)kNoAllocMaxBounces * kNoAllocMaxPaths);
constexpr size_t kNaRad = na_align(kNaVertA + 16 * (size_t)kNoAllocMaxBounces * kNoAllocMaxPaths);
constexpr size_t kNoAllocBytes = na_align(kNaRad + 16 * (size_t)kNoAllocMaxPaths);

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocBytes];

static int noalloc_scratch(int device, unsigned char **out)
{
    static std::mutex lock;
    static unsigned char *addr[64] = {};
    if (device < 0 || device >= 64) return set_error(GBSP_ERR_INVALID_ARGUMENT, "device %d", device);
    std::lock_guard<std::mutex> g(lock);
    if (!addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noallocScratch)");
        addr[device] = (unsigned char *)p;
    }
    *out = addr[device];
    return GBSP_OK;
}

}  // namespace gbsp

using namespace gbsp;

extern "C" int gbsp_path_trace_tile_noalloc(const gbsp_context *ctx, gbsp_tile tile,
    float *deviceImage, gbsp_metrics *metrics)
{
    if (!ctx || !ctx->camera || !ctx->camera->imagePlane || !ctx->scene || !ctx->materialSystem ||
        !ctx->runtime || !deviceImage)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "incomplete context or NULL image");
    if (((uintptr_t)deviceImage & 15u) != 0)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "deviceImage must be 16-byte aligned");
    gbsp_options opt;
    if (ctx->options)
        opt = *ctx->options;
    else
        gbsp_options_default(&opt);
    gbsp_runtime *rt = ctx->runtime;
    const gbsp_scene *sc = ctx->scene;
    gbsp_material_system *ms = ctx->materialSystem;
    if (!sc->committed)
        return set_error(GBSP_ERR_NOT_READY, "scene changed since gbsp_build_scene_broadphase");
    if (ms->dirty)
        return set_error(GBSP_ERR_NOT_READY,
            "materials not uploaded: render once with gbsp_path_trace_tile or _frame first");
    if (sc->rt != rt || ms->rt != rt)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "scene, materials and context use different runtimes");
    if (opt.rng_mode != GBSP_RNG_HASH_PER_SAMPLE)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "the allocation-free entry renders hash-per-sample only");
    uint32_t spp = opt.spp ? opt.spp : 1;
    if (spp > kNoAllocMaxPaths || opt.max_bounces > kNoAllocMaxBounces ||
        sc->objects.size() > kNoAllocMaxObjects)
        return set_error(GBSP_ERR_CAPACITY,
            "allocation-free render limits: spp <= %u, bounces <= %u, objects <= %u (got %u, %u, %zu)",
            kNoAllocMaxPaths, kNoAllocMaxBounces, kNoAllocMaxObjects, spp, opt.max_bounces,
            sc->objects.size());
    const gbsp_image_plane *ip = ctx->camera->imagePlane;
    uint32_t x0 = tile.minX, y0 = tile.minY;
    uint32_t x1 = tile.maxX < ip->width ? tile.maxX : ip->width;
    uint32_t y1 = tile.maxY < ip->height ? tile.maxY : ip->height;
    if (x1 <= x0 || y1 <= y0) return GBSP_OK;

    GBSP_CUDA_TRY(cudaSetDevice(rt->device));
    unsigned char *base = nullptr;
    int rc = noalloc_scratch(rt->device, &base);
    if (rc) return rc;
    cudaStream_t s = rt->stream;
    unsigned long long *counters = reinterpret_cast<unsigned long long *>(base + kNaCtl);
    unsigned int *ctl = reinterpret_cast<unsigned int *>(counters + GBSP_METRIC_COUNT);
    uint32_t *status = reinterpret_cast<uint32_t *>(base + kNaCtl + kNaCtlBytes - 16);
    int32_t *slots = reinterpret_cast<int32_t *>(base + kNaSlots);
    // the array keeps the previous call's contents: zero what must start at zero
    GBSP_CUDA_TRY(cudaMemsetAsync(base + kNaCtl, 0, kNaCtlBytes, s));

    // material slots per object in leaf order, built on the host stack
    int32_t hostSlots[kNoAllocMaxObjects];
    size_t nObj = sc->leafOrder.size();
    for (size_t j = 0; j < nObj; j++)
        hostSlots[j] = resolve_material(ms, sc->objects[sc->leafOrder[j]].material);
    if (nObj) GBSP_CUDA_TRY(cudaMemcpyAsync(slots, hostSlots, 4 * nObj, cudaMemcpyHostToDevice, s));

    MaterialView mv;
    mv.instanceSlot = slots;
    mv.materials = ms->dMaterials.ptr;
    mv.materialCount = (uint32_t)ms->materials.size();
    mv.texels = ms->dTexels.ptr;
    mv.textures = ms->dTextures.ptr;
    mv.textureCount = (uint32_t)ms->texturePixels.size();
    mv.backgroundSlot = resolve_material(ms, ms->backgroundId);
    mv.sky = ms->sky;
    mv.haveSky = ms->haveSky ? 1u : 0u;

    const gbsp_camera *c = ctx->camera;
    CameraParams cam;
    cam.right = v3(c->right[0], c->right[1], c->right[2]);
    cam.up = v3(c->up[0], c->up[1], c->up[2]);
    cam.forward = v3(c->forward[0], c->forward[1], c->forward[2]);
    cam.position = v3(c->position[0], c->position[1], c->position[2]);
    cam.filmCenter = v3(c->filmCenter[0], c->filmCenter[1], c->filmCenter[2]);
    cam.halfPixelWidth = c->halfPixelWidth;
    cam.halfPixelHeight = c->halfPixelHeight;
    cam.halfFilmWidth = c->halfFilmWidth;
    cam.halfFilmHeight = c->halfFilmHeight;
    cam.width = ip->width;
    cam.height = ip->height;

    WaveBuffers wb;
    wb.rayO = reinterpret_cast<float4 *>(base + kNaRayO);
    wb.rayD = reinterpret_cast<float4 *>(base + kNaRayD);
    wb.hitA = reinterpret_cast<int4 *>(base + kNaHitA);
    wb.hitInst = reinterpret_cast<int *>(base + kNaHitInst);
    wb.pathRng = reinterpret_cast<uint32_t *>(base + kNaRng);
    wb.pathLen = reinterpret_cast<uint32_t *>(base + kNaLen);
    wb.vertE = reinterpret_cast<float4 *>(base + kNaVertE);
    wb.vertA = reinterpret_cast<float4 *>(base + kNaVertA);
    wb.pathRad = reinterpret_cast<float4 *>(base + kNaRad);
    wb.pathAov = nullptr;
    uint32_t pixelsPerWave = kNoAllocMaxPaths / spp;
    wb.cap = pixelsPerWave * spp;

    WaveParams wp;
    wp.cam = cam;
    wp.x0 = x0;
    wp.y0 = y0;
    wp.regionW = x1 - x0;
    wp.spp = spp;
    wp.maxBounces = opt.max_bounces;
    wp.seed = opt.seed;
    wp.clampValue = opt.radiance_clamp;
    wp.nanPolicy = opt.nan_policy;
    wp.invSpp = 1.0f / (float)spp;
    wp.aovImage = nullptr;
    SceneView sv = sc->view();
    float4 *image = reinterpret_cast<float4 *>(deviceImage);
    uint64_t regionPixels = (uint64_t)(x1 - x0) * (y1 - y0);
    int grid = rt->smCount * 8;
    for (uint64_t pb = 0; pb < regionPixels; pb += pixelsPerWave) {
        wp.pixelBase = pb;
        uint64_t left = regionPixels - pb;
        wp.pixels = (uint32_t)(left < pixelsPerWave ? left : pixelsPerWave);
        uint32_t paths = wp.pixels * spp;
        if (opt.max_bounces == 0) {
            GBSP_CUDA_TRY(cudaMemsetAsync(wb.pathRad, 0, sizeof(float4) * (size_t)paths, s));
        } else {
            k_reset_ctl<<<1, 32, 0, s>>>(ctl, paths);
            k_generate<<<(paths + 255) / 256, 256, 0, s>>>(wp, wb);
            for (uint32_t b = 0; b < opt.max_bounces; b++) {
                int inQ = (b & 1) ? kCtlQueue1 : kCtlQueue0;
                int outQ = (b & 1) ? kCtlQueue0 : kCtlQueue1;
                k_reset_stage<<<1, 1, 0, s>>>(ctl, outQ);
                k_trace<<<grid, 128, 0, s>>>(sv, wb.rayO + ((b & 1) ? wb.cap : 0),
                    wb.rayD + ((b & 1) ? wb.cap : 0), ctl + inQ, wb.hitA, wb.hitInst, ctl,
                    counters, status);
                k_shade<<<grid, 128, 0, s>>>(sv, mv, wp, wb, b, inQ, ctl, counters);
            }
        }
        k_accumulate<<<(wp.pixels + 255) / 256, 256, 0, s>>>(wp, wb, image, ip->width, counters);
        GBSP_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long hostCounters[GBSP_METRIC_COUNT];
    uint32_t st = 0;
    GBSP_CUDA_TRY(cudaMemcpyAsync(hostCounters, counters, sizeof(hostCounters), cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaMemcpyAsync(&st, status, 4, cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    if (st)
        return set_error(GBSP_ERR_DEVICE_STATUS, "device status 0x%x in the allocation-free render", st);
    if (metrics)
        for (int i = 0; i < GBSP_METRIC_COUNT; i++) metrics->values[i] += hostCounters[i];
    return GBSP_OK;
}
