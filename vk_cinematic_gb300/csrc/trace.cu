// Batched closest-hit ray casting (config 2 and sp_RayIntersectScene batches).
//
// Persistent kernel: a grid sized to the SM count; every warp takes 32 rays
// at a time from a global atomic counter until the batch is exhausted (the
// counter only grows, so each warp loops at most count/32 times).  Rays are
// (origin, pad, direction, pad) float4 pairs, read with 128-bit loads.

#include "gbsp_internal.h"
#include "traverse.cuh"

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

int launch_intersect(cudaStream_t s, const SceneView &sv, uint32_t count, const float4 *rays,
    float *tOut, int32_t *triOut, int32_t *objOut, float *attrOut, uint32_t *matOut,
    const Instance *, int smCount, unsigned long long *counters, uint32_t *dStatus)
{
    if (!count) return GBSP_OK;
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
