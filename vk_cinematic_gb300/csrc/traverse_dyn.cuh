// Closest-hit traversal with per-lane dynamic ray fetch (device code).
//
// Same results as trace_closest (traverse.cuh) - same candidate sets, same
// arithmetic, same tie rules - but organised for SIMT efficiency on
// incoherent rays.  Every lane carries its own ray and traversal state and
// the warp loops over single steps (one stack pop: an object- or mesh-level
// node visit, entering an object, or one triangle leaf).  Node visits at
// both levels share one code path (the lane picks its world or object-space
// ray), so lanes at different levels still run the same instructions.
// When a lane finishes its ray it becomes idle; once a quarter of the warp is
// idle (or all of it), the warp takes that many new rays from the global
// queue with one atomicAdd, so short rays no longer wait for the warp's
// longest one (Aila & Laine, "Understanding the efficiency of ray traversal
// on GPUs", HPG 2009, persistent threads with dynamic fetch).
#pragma once

#include "traverse.cuh"

namespace gbsp {

constexpr int kRefillIdleLanes = 8;
// A ray of a validated tree needs far fewer steps (every node is popped at
// most once per object entry); past this cap the ray is ended with the best
// hit so far and the status word records it.
constexpr uint32_t kMaxRaySteps = 1u << 22;

template <class Policy>
__device__ __forceinline__ void dyn_trace_loop(Policy &pol, const SceneView &sv, uint32_t count,
    unsigned int *work, uint32_t *status, TraceCounters &cnt, uint32_t &done, uint32_t &hitCount)
{
    const int lane = threadIdx.x & 31;
    const uint32_t laneMaskLt = (1u << lane) - 1u;
    uint32_t stackRef[kStackSize];
    float stackT[kStackSize];
    int sp = 0;
    int mode = 0;  // 0 idle, 1 object level, 2 mesh level
    uint32_t slot = 0;
    V3 o = v3(0, 0, 0), d = v3(0, 0, 0), invd = v3(0, 0, 0);
    float bestT = kInf, bestU = 0.0f, bestV = 0.0f;
    int32_t bestPrim = -1, bestInst = -1;
    // mesh-level state
    uint32_t inst = 0;
    V3 lo = v3(0, 0, 0), ld = v3(0, 0, 0), linvd = v3(0, 0, 0);
    float len = 0.0f, lBestT = kInf, lU = 0.0f, lV = 0.0f;
    int32_t lPrim = -1;
    int base = 0;
    uint32_t steps = 0;
    bool exhausted = false;
    for (uint32_t guard = 0; guard < (1u << 30); guard++) {
        // ---- refill idle lanes (warp-uniform control flow)
        uint32_t idle = __ballot_sync(0xFFFFFFFFu, mode == 0);
        if (idle && !exhausted && (__popc(idle) >= kRefillIdleLanes || idle == 0xFFFFFFFFu)) {
            uint32_t n = __popc(idle);
            int leader = __ffs(idle) - 1;
            uint32_t first = 0;
            if (lane == leader) first = atomicAdd(work, n);
            first = __shfl_sync(0xFFFFFFFFu, first, leader);
            if (first + n >= count) exhausted = true;
            if (mode == 0) {
                uint32_t idx = first + __popc(idle & laneMaskLt);
                if (idx < count) {
                    slot = idx;
                    steps = 0;
                    pol.load(idx, o, d);
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
            }
        }
        uint32_t active = __ballot_sync(0xFFFFFFFFu, mode != 0);
        if (!active) {
            if (exhausted) break;
            continue;
        }
        if (mode == 0) continue;
        if (++steps > kMaxRaySteps) {
            atomicOr(status, kStatusRayStepLimit);
            mode = 1;
            sp = 0;  // the next step stores the best hit found so far
            steps = 0;
        }

        // ---- one step for this lane
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
            continue;
        }
        if (mode == 1 && sp == 0) {
            RayHit h;
            h.t = bestT;
            h.u = bestU;
            h.v = bestV;
            h.prim = bestPrim;
            h.inst = bestInst;
            pol.store(slot, h, sv);
            done++;
            hitCount += (bestPrim >= 0 && bestT > 0.0f) ? 1u : 0u;
            mode = 0;
            continue;
        }
        sp--;
        uint32_t ref = stackRef[sp];
        float te = stackT[sp];
        float bound = mode == 1 ? prune_bound(bestT) : prune_bound(rmin(lBestT, bestT * len));
        if (te > bound) continue;
        if (!child_is_leaf(ref)) {
            if (mode == 1) {
                cnt.topNodes++;
            } else {
                cnt.meshNodes++;
            }
            V3 ro = mode == 1 ? o : lo;
            V3 ri = mode == 1 ? invd : linvd;
            visit_node<true>(sv.nodes, ref, ro, ri, bound, stackRef, stackT, sp, status, cnt);
            continue;
        }
        if (mode == 1) {
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
                continue;
            }
            stackRef[sp] = __ldg(&in.blasRoot);
            stackT[sp] = 0.0f;
            sp++;
            mode = 2;
            continue;
        }
        visit_leaf<true>(sv, ref, lo, ld, linvd, lBestT, lU, lV, lPrim, cnt);
    }
}

}  // namespace gbsp
