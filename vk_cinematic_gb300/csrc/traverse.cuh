// Closest-hit traversal of the two-level scene (device code).
//
// Semantics follow sp_RayIntersectScene / sp_RayIntersectMesh
// (src/sp_scene.cpp:127-339):
//   * an object is a candidate iff its world AABB passes the reference's
//     slab test (src/simd.h:198-271) for the world ray;
//   * the ray enters object space through the inverse model matrix and its
//     direction is re-normalised there (src/sp_scene.cpp:274-276);
//   * a triangle is a candidate iff its own AABB passes the slab test in
//     object space (the reference collects exactly those BVH leaves,
//     src/bvh.cpp:203-311) and the Moller-Trumbore test hits with t > 0;
//   * per object the smallest object-space t wins, its hit point goes back
//     to world space and t = dot(worldHit - o, d) (src/sp_scene.cpp:302-308);
//     the smallest world t over objects wins.
// Node boxes here are exact unions of the reference's leaf boxes, and the
// slab test is monotone in the box, so interior tests never drop a leaf the
// reference would test.  Unlike the reference, the walk is ordered and
// prunes boxes that start beyond the best hit so far; pruning keeps a
// relative margin of 2^-10 so that a triangle whose rounded t lands just
// under its box's rounded entry distance is still tested.  Exact t ties go
// to the lower triangle (or object) index instead of the reference's
// BVH-order-dependent first find.
#pragma once

#include "gbsp_common.cuh"

namespace gbsp {

constexpr int kStackSize = 96;

// One traversal stack entry: a node or leaf reference and its entry
// distance, kept together so that a push or a pop is one 8-byte access.
struct __align__(8) StackEntry {
    uint32_t ref;
    float t;
};
constexpr float kInf = __builtin_huge_valf();

struct RayHit {
    float t;       // world t, +inf = miss
    float u, v;    // barycentrics of the winning triangle
    int32_t prim;  // leaf-order triangle index in the pool, -1 = miss
    int32_t inst;  // instance index (object-BVH leaf order), -1 = miss
};

struct TraceCounters {
    uint32_t topNodes, meshNodes, boxTests, triTests, meshTests;
};

__device__ __forceinline__ float prune_bound(float t) { return t + t * 0.0009765625f; }

// Tests the children of a node (4 per quad, `quads` = 1 or 2) against the
// ray, pushing hits nearest-last.  kWT: the watertight mode's robust slab
// test.  With kKeepNearest the nearest hit child is not pushed but returned
// (ref kEmptyChild when no child is hit), for the caller to visit straight
// away: one stack store and load fewer per node visit.  Without it the
// return value is an empty entry.
// kFastSlab: slab_entry_node instead of the reference's slab_entry (see
// visit_node for when that is allowed).
template <bool kCount, bool kWT, bool kKeepNearest, bool kFastSlab>
__device__ __forceinline__ StackEntry visit_node_impl(const float4 *__restrict__ pool,
    uint32_t quads, uint32_t ref, V3 o, V3 invd, float bound, StackEntry *stack, int &sp,
    uint32_t *status, TraceCounters &cnt)
{
    const float4 *p = pool + node_offset(ref, quads);
    // a node pushes at most 4 * quads entries: one room check per visit instead
    // of one per push (a walk out of room reports the overflow and skips the node)
    if (sp > kStackSize - 4 * (int)kMaxNodeQuads) {
        atomicOr(status, kStatusStackOverflow);
        return StackEntry{kEmptyChild, 0.0f};
    }
    uint32_t nearRef = kEmptyChild;
    float nearT = kInf;
#pragma unroll
    for (int half = 0; half < (int)kMaxNodeQuads; half++) {
        if (half >= (int)quads) break;
        float4 lx = __ldg(p + 0 * quads + half), hx = __ldg(p + 1 * quads + half);
        float4 ly = __ldg(p + 2 * quads + half), hy = __ldg(p + 3 * quads + half);
        float4 lz = __ldg(p + 4 * quads + half), hz = __ldg(p + 5 * quads + half);
        uint4 ch = __ldg(reinterpret_cast<const uint4 *>(p + 6 * quads + half));
        float lxs[4] = {lx.x, lx.y, lx.z, lx.w}, hxs[4] = {hx.x, hx.y, hx.z, hx.w};
        float lys[4] = {ly.x, ly.y, ly.z, ly.w}, hys[4] = {hy.x, hy.y, hy.z, hy.w};
        float lzs[4] = {lz.x, lz.y, lz.z, lz.w}, hzs[4] = {hz.x, hz.y, hz.z, hz.w};
        uint32_t chs[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t c = chs[k];
            if (c == kEmptyChild) continue;
            if (kCount) cnt.boxTests++;
            V3 bl = v3(lxs[k], lys[k], lzs[k]), bh = v3(hxs[k], hys[k], hzs[k]);
            float te = kWT ? slab_entry_robust(bl, bh, o, invd)
                           : (kFastSlab ? slab_entry_node(bl, bh, o, invd)
                                        : slab_entry(bl, bh, o, invd));
            if (te < 0.0f || te > bound) continue;
            if (te < nearT) {
                if (nearRef != kEmptyChild) {
                    stack[sp] = StackEntry{nearRef, nearT};
                    sp++;
                }
                nearRef = c;
                nearT = te;
            } else {
                stack[sp] = StackEntry{c, te};
                sp++;
            }
        }
    }
    if constexpr (kKeepNearest) {
        return StackEntry{nearRef, nearT};
    } else {
        if (nearRef != kEmptyChild) {
            stack[sp] = StackEntry{nearRef, nearT};
            sp++;
        }
        return StackEntry{kEmptyChild, 0.0f};
    }
}

// Interior nodes take the min/max-instruction slab test when every component
// of the inverse direction is finite: then no NaN can arise and it decides
// exactly as the reference's form.  A ray with a zero direction component (an
// infinite inverse, where (lo - o) * invd can be NaN and the reference's form
// has its own NaN rules) keeps the reference's form, whose decisions below a
// node are a superset of its leaves'.
template <bool kCount, bool kWT = false, bool kKeepNearest = false>
__device__ __forceinline__ StackEntry visit_node(const float4 *__restrict__ pool, uint32_t quads,
    uint32_t ref, V3 o, V3 invd, float bound, StackEntry *stack, int &sp, uint32_t *status,
    TraceCounters &cnt)
{
    if (kWT || !(isfinite(invd.x) && isfinite(invd.y) && isfinite(invd.z)))
        return visit_node_impl<kCount, kWT, kKeepNearest, false>(pool, quads, ref, o, invd, bound,
            stack, sp, status, cnt);
    return visit_node_impl<kCount, kWT, kKeepNearest, true>(pool, quads, ref, o, invd, bound,
        stack, sp, status, cnt);
}

// Triangle candidates of one mesh leaf, in object space.  kWT: the
// watertight test on every candidate (no box gate: a rounded box test could
// reject an edge ray); otherwise the reference's gate and MT test.  A closer
// hit updates bestT and bestPrim and hands its barycentrics to keepUV(u, v).
template <bool kCount, bool kWT, class KeepUV>
__device__ __forceinline__ void visit_leaf_uv(const SceneView &sv, uint32_t ref, V3 lo, V3 ld,
    V3 linvd, float &bestT, int32_t &bestPrim, KeepUV keepUV, TraceCounters &cnt)
{
    uint32_t first = leaf_first(ref), count = leaf_count(ref);
    for (uint32_t k = 0; k < count; k++) {
        uint32_t j = first + k;
        const float4 *tp = reinterpret_cast<const float4 *>(sv.tris + j);
        float4 A = __ldg(tp + 0), B = __ldg(tp + 1), C = __ldg(tp + 2);
        V3 a = v3(A.x, A.y, A.z), b = v3(B.x, B.y, B.z), c = v3(C.x, C.y, C.z);
        if (kCount) cnt.triTests++;
        TriHit h;
        if constexpr (kWT) {
            h = ray_triangle_watertight(lo, ld, a, b, c, v3(A.w, B.w, C.w));
        } else {
            // the three conditions of a hit, cheapest first (each is a pure
            // predicate, so the order changes no result): the face culling of
            // RayIntersectTriangleMT (src/ray_intersection.cpp:181-182), the
            // triangle's own box (the reference only reaches triangles whose
            // box passes), then the test itself
            if (!(dot(ld, v3(A.w, B.w, C.w)) < 0.0f)) continue;
            V3 bl = vmin(a, vmin(b, c)), bh = vmax(a, vmax(b, c));
            if (slab_entry(bl, bh, lo, linvd) < 0.0f) continue;
            h = ray_triangle_mt(lo, ld, a, b, c, v3(A.w, B.w, C.w));
        }
        if (!h.hit || !(h.t > 0.0f)) continue;
        bool take = h.t < bestT;
        if (!take && h.t == bestT && bestPrim >= 0)
            take = __ldg(sv.triIds + j) < __ldg(sv.triIds + bestPrim);
        if (take) {
            bestT = h.t;
            keepUV(h.u, h.v);
            bestPrim = (int32_t)j;
        }
    }
}

template <bool kCount, bool kWT = false>
__device__ __forceinline__ void visit_leaf(const SceneView &sv, uint32_t ref, V3 lo, V3 ld,
    V3 linvd, float &bestT, float &bestU, float &bestV, int32_t &bestPrim, TraceCounters &cnt)
{
    visit_leaf_uv<kCount, kWT>(sv, ref, lo, ld, linvd, bestT, bestPrim,
        [&](float u, float v) {
            bestU = u;
            bestV = v;
        },
        cnt);
}

template <bool kCount, bool kWT = false>
__device__ RayHit trace_closest(const SceneView &sv, V3 o, V3 d, uint32_t *status,
    TraceCounters &cnt)
{
    RayHit best;
    best.t = kInf;
    best.u = best.v = 0.0f;
    best.prim = -1;
    best.inst = -1;
    if (sv.tlasRoot == kEmptyChild) return best;
    StackEntry stack[kStackSize];
    // State used only when entering or leaving an object, kept in memory
    // (local, L1-resident) on purpose so that the walks hold just the current
    // level's ray, bounds and stack in registers.  Words: world origin 0-2,
    // direction 3-5, inverse direction 6-8; best hit over objects u 9, v 10,
    // triangle 11, object 12; the object's best triangle's u 13, v 14.
    volatile uint32_t cold[15];
    const auto put3 = [&](int w, V3 v) {
        cold[w] = __float_as_uint(v.x);
        cold[w + 1] = __float_as_uint(v.y);
        cold[w + 2] = __float_as_uint(v.z);
    };
    const auto get3 = [&](int w) {
        return v3(__uint_as_float(cold[w]), __uint_as_float(cold[w + 1]),
            __uint_as_float(cold[w + 2]));
    };
    int sp = 0;
    V3 invd = inverse(d);
    put3(0, o);
    put3(3, d);
    put3(6, invd);
    cold[9] = 0u;
    cold[10] = 0u;
    cold[11] = 0xFFFFFFFFu;
    cold[12] = 0xFFFFFFFFu;
    // the entry to visit next (the nearest child of the last node visit),
    // kept out of the stack
    StackEntry next = StackEntry{sv.tlasRoot, 0.0f};
    const float4 *__restrict__ nodes = sv.nodes;
    const uint32_t quads = sv.nodeQuads;
    // trees are validated at build time (children after parents), so the
    // walk is finite; the guard only bounds it against corrupted memory
    for (int guard = 0; next.ref != kEmptyChild || sp > 0; guard++) {
        if (guard >= (1 << 20)) {
            atomicOr(status, kStatusStackOverflow);
            break;
        }
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
        if (te > prune_bound(best.t)) continue;
        if (!child_is_leaf(ref)) {
            if (kCount) cnt.topNodes++;
            next = visit_node<kCount, kWT, true>(nodes, quads, ref, o, invd, prune_bound(best.t),
                stack, sp, status, cnt);
            continue;
        }
        // an object whose world box passed: descend into its mesh
        uint32_t inst = leaf_first(ref);
        const Instance &in = sv.instances[inst];
        Affine inv, model;
#pragma unroll
        for (int k = 0; k < 12; k++) inv.r[k] = __ldg(&in.inv.r[k]);
        const V3 lo = transform_point(inv, o);
        float len;
        const V3 ld = normalize(transform_vector(inv, get3(3)), &len);
        const V3 linvd = inverse(ld);
        if (kCount) cnt.meshTests++;
        float lBestT = kInf;
        int32_t lPrim = -1;
        float localBound = best.t * len;
        const int base = sp;
        StackEntry lnext = StackEntry{__ldg(&in.blasRoot), 0.0f};
        for (int guard = 0; (lnext.ref != kEmptyChild || sp > base) && guard < (1 << 22); guard++) {
            StackEntry top2;
            if (lnext.ref != kEmptyChild) {
                top2 = lnext;
                lnext.ref = kEmptyChild;
            } else {
                sp--;
                top2 = stack[sp];
            }
            uint32_t r2 = top2.ref;
            float t2 = top2.t;
            float bound = prune_bound(rmin(lBestT, localBound));
            if (t2 > bound) continue;
            if (!child_is_leaf(r2)) {
                if (kCount) cnt.meshNodes++;
                lnext = visit_node<kCount, kWT, true>(nodes, quads, r2, lo, linvd, bound, stack, sp,
                    status, cnt);
            } else {
                visit_leaf_uv<kCount, kWT>(sv, r2, lo, ld, linvd, lBestT, lPrim,
                    [&](float u, float v) {
                        cold[13] = __float_as_uint(u);
                        cold[14] = __float_as_uint(v);
                    },
                    cnt);
            }
        }
        sp = base;
        // the world ray comes back from memory: it was not held through the mesh walk
        o = get3(0);
        invd = get3(6);
        if (lPrim < 0) continue;
#pragma unroll
        for (int k = 0; k < 12; k++) model.r[k] = __ldg(&in.model.r[k]);
        V3 localHit = add(lo, mul(ld, lBestT));
        V3 worldHit = transform_point(model, localHit);
        float tw = dot(sub(worldHit, o), get3(3));
        if (tw < best.t || (tw == best.t && (int32_t)inst < (int32_t)cold[12])) {
            best.t = tw;
            cold[9] = cold[13];
            cold[10] = cold[14];
            cold[11] = (uint32_t)lPrim;
            cold[12] = inst;
        }
    }
    best.u = __uint_as_float(cold[9]);
    best.v = __uint_as_float(cold[10]);
    best.prim = (int32_t)cold[11];
    best.inst = (int32_t)cold[12];
    return best;
}

// World-space normal and uv of a hit (src/sp_scene.cpp:189-215, 302-312).
__device__ __forceinline__ void hit_surface(const SceneView &sv, const RayHit &h, V3 &normal,
    float &uvx, float &uvy)
{
    const Instance &in = sv.instances[h.inst];
    const float4 *tp = reinterpret_cast<const float4 *>(sv.tris + h.prim);
    float4 A = __ldg(tp + 0), B = __ldg(tp + 1), C = __ldg(tp + 2);
    const float4 *ap = reinterpret_cast<const float4 *>(sv.attrs + h.prim);
    float4 a0 = __ldg(ap + 0), a1 = __ldg(ap + 1), a2 = __ldg(ap + 2), a3 = __ldg(ap + 3);
    float w = 1.0f - h.u - h.v;
    // uv0 = (a2.y, a2.z), uv1 = (a2.w, a3.x), uv2 = (a3.y, a3.z)
    uvx = a2.y * w + a2.w * h.u + a3.y * h.v;
    uvy = a2.z * w + a3.x * h.u + a3.z * h.v;
    V3 ln = v3(A.w, B.w, C.w);
    if (__ldg(&in.smooth)) {
        V3 n0 = v3(a0.x, a0.y, a0.z), n1 = v3(a0.w, a1.x, a1.y), n2 = v3(a1.z, a1.w, a2.x);
        ln = normalize(add(add(mul(n0, w), mul(n1, h.u)), mul(n2, h.v)));
    }
    Affine model;
#pragma unroll
    for (int k = 0; k < 12; k++) model.r[k] = __ldg(&in.model.r[k]);
    normal = normalize(transform_vector(model, ln));
}

}  // namespace gbsp
