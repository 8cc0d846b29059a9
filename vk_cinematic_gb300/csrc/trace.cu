// Batched closest-hit ray casting (config 2 and sp_RayIntersectScene batches).
//
// Small batches: k_intersect, a persistent kernel whose warps take 32 rays at
// a time from a global atomic counter until the batch is exhausted (the
// counter only grows, so each warp loops at most count/32 times).  Large
// batches of (typically incoherent) rays go through the wavefront's per-lane
// closest-hit kernel instead, where a lane fetches its next ray as soon as
// its current one is done: the rays are split into the queue layout, traced,
// and the queue-ordered hits turned into the requested outputs.  Rays are
// (origin, pad, direction, pad) float4 pairs, read with 128-bit loads.

#include "gbsp_internal.h"
#include "traverse.cuh"
#include "wavefront.cuh"

namespace gbsp {

__device__ __forceinline__ void warp_add_counters(unsigned long long *counters,
    const TraceCounters &c, uint32_t rays, uint32_t hits)
{
    uint32_t v[7] = {rays, hits, c.topNodes, c.meshNodes, c.triTests, c.boxTests, c.meshTests};
#pragma unroll
    for (int k = 0; k < 7; k++)
        for (int off = 16; off; off >>= 1) v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
    if ((threadIdx.x & 31) == 0) {
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

template <bool kWT>
__global__ void __launch_bounds__(128) k_intersect(SceneView sv, const float4 *__restrict__ rays,
    uint32_t count, float *tOut, int32_t *triOut, int32_t *objOut, float *attrOut,
    uint32_t *matOut, unsigned int *work, unsigned long long *counters, uint32_t *status)
{
    int lane = threadIdx.x & 31;
    TraceCounters cnt = {0, 0, 0, 0, 0};
    uint32_t rays_done = 0, hits = 0;
    for (uint32_t guard = 0; guard <= count / 32 + 1; guard++) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= count) break;
        uint32_t i = base + lane;
        if (i < count) {
            float4 o4 = __ldg(rays + 2 * (size_t)i), d4 = __ldg(rays + 2 * (size_t)i + 1);
            RayHit h = trace_closest<true, kWT>(sv, v3(o4.x, o4.y, o4.z), v3(d4.x, d4.y, d4.z), status,
                cnt);
            bool hit = h.prim >= 0;
            rays_done++;
            hits += hit ? 1u : 0u;
            if (tOut) tOut[i] = hit ? h.t : -1.0f;
            if (triOut) triOut[i] = hit ? (int32_t)__ldg(sv.triIds + h.prim) : -1;
            const Instance *in = hit ? sv.instances + h.inst : nullptr;
            if (objOut) objOut[i] = hit ? (int32_t)__ldg(&in->objectIndex) : -1;
            if (attrOut) {
                float *a = attrOut + 6 * (size_t)i;
                if (hit) {
                    V3 n;
                    float ux, uy;
                    hit_surface(sv, h, n, ux, uy);
                    a[0] = h.t;
                    a[1] = n.x;
                    a[2] = n.y;
                    a[3] = n.z;
                    a[4] = ux;
                    a[5] = uy;
                } else {
                    a[0] = -1.0f;
                    a[1] = a[2] = a[3] = a[4] = a[5] = 0.0f;
                }
            }
            if (matOut) matOut[i] = hit ? __ldg(&in->materialId) : 0u;
        }
    }
    warp_add_counters(counters, cnt, rays_done, hits);
}

// Ray pairs -> queue layout (origin with path id 0, direction).
__global__ void __launch_bounds__(256) k_split_rays(const float4 *__restrict__ rays, uint32_t count,
    float4 *__restrict__ o, float4 *__restrict__ d)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
    o[i] = make_float4(a.x, a.y, a.z, 0.0f);
    d[i] = make_float4(b.x, b.y, b.z, 0.0f);
}

// Queue-ordered hits -> the per-ray outputs of k_intersect (same values).
__global__ void __launch_bounds__(256) k_intersect_outputs(SceneView sv, const int4 *__restrict__ hitA,
    const int *__restrict__ hitInst, uint32_t count, float *tOut, int32_t *triOut, int32_t *objOut,
    float *attrOut, uint32_t *matOut)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int4 hA = hitA[i];
    RayHit h;
    h.t = __int_as_float(hA.x);
    h.u = __int_as_float(hA.y);
    h.v = __int_as_float(hA.z);
    h.prim = hA.w;
    h.inst = hitInst[i];
    bool hit = h.prim >= 0;
    if (tOut) tOut[i] = hit ? h.t : -1.0f;
    if (triOut) triOut[i] = hit ? (int32_t)__ldg(sv.triIds + h.prim) : -1;
    const Instance *in = hit ? sv.instances + h.inst : nullptr;
    if (objOut) objOut[i] = hit ? (int32_t)__ldg(&in->objectIndex) : -1;
    if (attrOut) {
        float *a = attrOut + 6 * (size_t)i;
        if (hit) {
            V3 n;
            float ux, uy;
            hit_surface(sv, h, n, ux, uy);
            a[0] = h.t;
            a[1] = n.x;
            a[2] = n.y;
            a[3] = n.z;
            a[4] = ux;
            a[5] = uy;
        } else {
            a[0] = -1.0f;
            a[1] = a[2] = a[3] = a[4] = a[5] = 0.0f;
        }
    }
    if (matOut) matOut[i] = hit ? __ldg(&in->materialId) : 0u;
}

// Batches from this size on take the per-lane path.
constexpr uint32_t kPerLaneBatch = 1u << 16;

static int launch_intersect_per_lane(cudaStream_t s, const SceneView &sv, uint32_t count,
    const float4 *rays, float *tOut, int32_t *triOut, int32_t *objOut, float *attrOut,
    uint32_t *matOut, int smCount, unsigned long long *counters, uint32_t *dStatus)
{
    // one allocation: O, D, hits (16 B each per ray), instance ids, control block
    const size_t n = count;
    const size_t bytes = n * (16 + 16 + 16 + 4) + sizeof(unsigned int) * kCtlCount + 64;
    unsigned char *tmp = nullptr;
    GBSP_CUDA_TRY(cudaMallocAsync((void **)&tmp, bytes, s));
    float4 *o = reinterpret_cast<float4 *>(tmp);
    float4 *d = o + n;
    int4 *hitA = reinterpret_cast<int4 *>(d + n);
    int *hitInst = reinterpret_cast<int *>(hitA + n);
    unsigned int *ctl = reinterpret_cast<unsigned int *>(
        (reinterpret_cast<uintptr_t>(hitInst + n) + 63) & ~(uintptr_t)63);
    OneScene one = {};
    one.sv = sv;
    const int blocks = (int)((n + 255) / 256);
    k_split_rays<<<blocks, 256, 0, s>>>(rays, count, o, d);
    k_reset_ctl<<<1, 32, 0, s>>>(ctl, count);
    launch_trace_stage(true, sv.watertight != 0, smCount * 8, s, one, o, d, ctl + kCtlQueue0, hitA,
        hitInst, ctl, counters, dStatus);
    k_intersect_outputs<<<blocks, 256, 0, s>>>(sv, hitA, hitInst, count, tOut, triOut, objOut,
        attrOut, matOut);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(tmp, s);
    GBSP_CUDA_TRY(e);
    return GBSP_OK;
}

int launch_intersect(cudaStream_t s, const SceneView &sv, uint32_t count, const float4 *rays,
    float *tOut, int32_t *triOut, int32_t *objOut, float *attrOut, uint32_t *matOut,
    const Instance *, int smCount, unsigned long long *counters, uint32_t *dStatus)
{
    if (!count) return GBSP_OK;
    if (count >= kPerLaneBatch)
        return launch_intersect_per_lane(s, sv, count, rays, tOut, triOut, objOut, attrOut, matOut,
            smCount, counters, dStatus);
    // the work counter lives in the last counter slot's neighbour block
    unsigned int *work = reinterpret_cast<unsigned int *>(counters + GBSP_METRIC_COUNT);
    GBSP_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(unsigned int), s));
    int grid = smCount * 8;
    uint64_t needed = ((uint64_t)count + 127) / 128;
    if ((uint64_t)grid > needed) grid = (int)needed;
    auto kern = sv.watertight ? k_intersect<true> : k_intersect<false>;
    kern<<<grid, 128, 0, s>>>(sv, rays, count, tOut, triOut, objOut, attrOut, matOut, work,
        counters, dStatus);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

}  // namespace gbsp
