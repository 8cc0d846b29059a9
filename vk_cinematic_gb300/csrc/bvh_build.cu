// Device BVH construction.
//
// The reference builds its 4-ary BVHs on the CPU by agglomerative nearest-
// neighbour merging (src/bvh.cpp:51-200, O(n^2 log n)).  Query results do not
// depend on the tree shape: the reference returns every leaf whose box the
// ray passes and the closest triangle among those, so any hierarchy of exact
// box unions plus the per-triangle box test in the traversal gives the same
// candidate set.  Here the tree is a linear BVH:
//   1. per-primitive boxes and centroids, centroid bounds;
//   2. 30-bit Morton codes, sorted with a stable LSD radix sort (8-bit digits,
//      per-block ranks from __match_any_sync);
//   3. the binary radix tree of Karras (HPG 2012), one thread per node;
//   4. bottom-up box refit with one atomic arrival counter per node;
//   5. top-down collapse into wide nodes, once per node width (8 and 4)
//      from the same binary tree: each wide node repeatedly opens its
//      largest-area child until it has W children; subtrees of at most
//      leafMax primitives become leaves.  Leaves index the primitives in the
//      sorted Morton order, which both widths share, so one triangle pool
//      serves the trees of both widths.
// Every loop is bounded by the primitive count or log2 of it.

#include <algorithm>
#include <cstdio>
#include <vector>

#include "gbsp_internal.h"

namespace gbsp {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;  // elements per thread per tile
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortWarps = kSortThreads / 32;

__global__ void radix_histogram(const uint32_t *keys, uint32_t n, int shift, uint32_t *hist,
    uint32_t numBlocks)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; k++) {
        uint64_t i = base + (uint64_t)k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * numBlocks + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of hist (digit-major, block-minor) in one block.
__global__ void radix_scan(uint32_t *hist, uint32_t total)
{
    __shared__ uint32_t partial[1024];
    uint32_t per = (total + blockDim.x - 1) / blockDim.x;
    uint32_t begin = threadIdx.x * per;
    uint32_t end = begin + per < total ? begin + per : total;
    uint32_t s = 0;
    for (uint32_t i = begin; i < end; i++) s += hist[i];
    partial[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
        uint32_t v = threadIdx.x >= off ? partial[threadIdx.x - off] : 0;
        __syncthreads();
        partial[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? partial[threadIdx.x - 1] : 0;
    for (uint32_t i = begin; i < end; i++) {
        uint32_t v = hist[i];
        hist[i] = run;
        run += v;
    }
}

// Stable scatter: ranks within a tile are taken in element order, round by
// round (each round = one element per thread, warps in order).
__global__ void radix_scatter(const uint32_t *keysIn, const uint32_t *valsIn, uint32_t *keysOut,
    uint32_t *valsOut, uint32_t n, int shift, const uint32_t *hist, uint32_t numBlocks)
{
    __shared__ uint32_t base[256];
    __shared__ uint32_t wc[kSortWarps][257];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    base[threadIdx.x] = hist[(uint64_t)threadIdx.x * numBlocks + blockIdx.x];
    for (int w = 0; w < kSortWarps; w++) wc[w][threadIdx.x] = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kSortWarps; w++) wc[w][256] = 0;
    __syncthreads();
    uint64_t tile = (uint64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; r++) {
        uint64_t i = tile + (uint64_t)r * kSortThreads + threadIdx.x;
        bool valid = i < n;
        uint32_t key = valid ? keysIn[i] : 0u;
        uint32_t digit = valid ? ((key >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        int leader = __ffs(peers) - 1;
        if (lane == leader) wc[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = base[digit] + rank;
            for (int w = 0; w < warp; w++) pos += wc[w][digit];
            keysOut[pos] = key;
            valsOut[pos] = valsIn[i];
        }
        __syncthreads();
        uint32_t add = 0;
        for (int w = 0; w < kSortWarps; w++) {
            add += wc[w][threadIdx.x];
            wc[w][threadIdx.x] = 0;
        }
        base[threadIdx.x] += add;
        if (threadIdx.x == 0)
            for (int w = 0; w < kSortWarps; w++) wc[w][256] = 0;
        __syncthreads();
    }
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// Centroid bounds as ordered-int atomics (floats mapped to monotone ints).
__device__ __forceinline__ int float_to_ordered(float f)
{
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ordered_to_float(int i)
{
    return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF);
}

__global__ void centroid_bounds(const float4 *lo, const float4 *hi, uint32_t n, int *bounds)
{
    float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = lo[i], b = hi[i];
        float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        for (int k = 0; k < 3; k++) {
            mn[k] = fminf(mn[k], c[k]);
            mx[k] = fmaxf(mx[k], c[k]);
        }
    }
    for (int k = 0; k < 3; k++) {
        for (int off = 16; off; off >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], off));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], off));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; k++) {
            atomicMin(&bounds[k], float_to_ordered(mn[k]));
            atomicMax(&bounds[3 + k], float_to_ordered(mx[k]));
        }
    }
}

__global__ void morton_codes(const float4 *lo, const float4 *hi, uint32_t n, const int *bounds,
    uint32_t *codes, uint32_t *ids)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float bmin[3], ext[3];
    for (int k = 0; k < 3; k++) {
        bmin[k] = ordered_to_float(bounds[k]);
        float e = ordered_to_float(bounds[3 + k]) - bmin[k];
        ext[k] = e > 0.0f ? e : 1.0f;
    }
    float4 a = lo[i], b = hi[i];
    float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
    uint32_t q[3];
    for (int k = 0; k < 3; k++) {
        float u = (c[k] - bmin[k]) / ext[k];
        u = fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f);
        q[k] = (uint32_t)u;
    }
    codes[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    ids[i] = i;
}

// Karras' common-prefix length with index tie-break.
__device__ __forceinline__ int delta(const uint32_t *codes, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + __clz((uint32_t)(i ^ j));
    return __clz(a ^ b);
}

// Binary child reference: bit 31 set = leaf (sorted position), else internal.
constexpr uint32_t kBinLeaf = 0x80000000u;

__global__ void karras_hierarchy(const uint32_t *codes, int n, uint32_t *left, uint32_t *right,
    uint32_t *parent, uint32_t *first, uint32_t *last)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(codes, n, i, i - d);
    int lmax = 2;
    while (delta(codes, n, i, i + lmax * d) > dmin && lmax < (1 << 30)) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(codes, n, i, j);
    int s = 0;
    for (int div = 2; div < (1 << 30); div <<= 1) {
        int t = (l + div - 1) / div;
        if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    int gamma = i + s * d + (d < 0 ? d : 0);
    int lo = i < j ? i : j, hi = i < j ? j : i;
    uint32_t lc = (lo == gamma) ? (kBinLeaf | (uint32_t)gamma) : (uint32_t)gamma;
    uint32_t rc = (hi == gamma + 1) ? (kBinLeaf | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    left[i] = lc;
    right[i] = rc;
    first[i] = (uint32_t)lo;
    last[i] = (uint32_t)hi;
    // parents: internal nodes in [0, n-1), leaves in [n-1, 2n-1)
    parent[(lc & kBinLeaf) ? (n - 1) + (lc & ~kBinLeaf) : lc] = (uint32_t)i;
    parent[(rc & kBinLeaf) ? (n - 1) + (rc & ~kBinLeaf) : rc] = (uint32_t)i;
}

__device__ __forceinline__ void child_box(uint32_t c, const float4 *nodeLo, const float4 *nodeHi,
    const float4 *primLo, const float4 *primHi, const uint32_t *order, float4 &lo, float4 &hi)
{
    if (c & kBinLeaf) {
        uint32_t p = order[c & ~kBinLeaf];
        lo = primLo[p];
        hi = primHi[p];
    } else {
        lo = nodeLo[c];
        hi = nodeHi[c];
    }
}

// Exact box unions with the reference's min/max form.
__device__ __forceinline__ float4 min4(float4 a, float4 b)
{
    return make_float4(rmin(a.x, b.x), rmin(a.y, b.y), rmin(a.z, b.z), 0.0f);
}
__device__ __forceinline__ float4 max4(float4 a, float4 b)
{
    return make_float4(rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z), 0.0f);
}

__global__ void refit(int n, const uint32_t *left, const uint32_t *right, const uint32_t *parent,
    const float4 *primLo, const float4 *primHi, const uint32_t *order, float4 *nodeLo,
    float4 *nodeHi, uint32_t *arrivals, uint32_t *status)
{
    int leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n) return;
    uint32_t node = parent[(n - 1) + leaf];
    for (int guard = 0; guard < n; guard++) {
        __threadfence();
        if (atomicAdd(&arrivals[node], 1u) == 0u) return;  // first arrival stops
        __threadfence();
        float4 al, ah, bl, bh;
        child_box(left[node], nodeLo, nodeHi, primLo, primHi, order, al, ah);
        child_box(right[node], nodeLo, nodeHi, primLo, primHi, order, bl, bh);
        // volatile-free: the other child's box was published before its
        // thread's atomicAdd (fenced above)
        nodeLo[node] = min4(al, bl);
        nodeHi[node] = max4(ah, bh);
        if (node == 0) return;
        node = parent[node];
    }
    atomicOr(status, kStatusBuildLoop);
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi)
{
    float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

struct CollapseItem {
    uint32_t bin;   // binary internal node
    uint32_t wide;  // output wide node (relative index)
};

// Writes one node of width 4 * quads (layout in gbsp_common.cuh).
__device__ void store_node(float4 *dst, uint32_t quads, const float *lo, const float *hi,
    const uint32_t *child)
{
    for (uint32_t q = 0; q < quads; q++) {
        const uint32_t b = 4 * q;
        dst[0 * quads + q] = make_float4(lo[3 * b + 0], lo[3 * (b + 1) + 0], lo[3 * (b + 2) + 0],
            lo[3 * (b + 3) + 0]);
        dst[1 * quads + q] = make_float4(hi[3 * b + 0], hi[3 * (b + 1) + 0], hi[3 * (b + 2) + 0],
            hi[3 * (b + 3) + 0]);
        dst[2 * quads + q] = make_float4(lo[3 * b + 1], lo[3 * (b + 1) + 1], lo[3 * (b + 2) + 1],
            lo[3 * (b + 3) + 1]);
        dst[3 * quads + q] = make_float4(hi[3 * b + 1], hi[3 * (b + 1) + 1], hi[3 * (b + 2) + 1],
            hi[3 * (b + 3) + 1]);
        dst[4 * quads + q] = make_float4(lo[3 * b + 2], lo[3 * (b + 1) + 2], lo[3 * (b + 2) + 2],
            lo[3 * (b + 3) + 2]);
        dst[5 * quads + q] = make_float4(hi[3 * b + 2], hi[3 * (b + 1) + 2], hi[3 * (b + 2) + 2],
            hi[3 * (b + 3) + 2]);
        dst[6 * quads + q] = make_float4(__uint_as_float(child[b]), __uint_as_float(child[b + 1]),
            __uint_as_float(child[b + 2]), __uint_as_float(child[b + 3]));
    }
}

__device__ __forceinline__ uint32_t node_child(const float4 *node, uint32_t quads, uint32_t c)
{
    const float4 v = node[6 * quads + c / 4];
    const float f = (c & 3) == 0 ? v.x : (c & 3) == 1 ? v.y : (c & 3) == 2 ? v.z : v.w;
    return __float_as_uint(f);
}

template <int W>
__global__ void collapse_level(const CollapseItem *in, uint32_t inCount, CollapseItem *out,
    uint32_t *outCount, uint32_t *nodeCounter, uint32_t nodeCapacity, const uint32_t *left,
    const uint32_t *right, const uint32_t *first, const uint32_t *last, const float4 *nodeLo,
    const float4 *nodeHi, const float4 *primLo, const float4 *primHi, const uint32_t *order,
    uint32_t leafMax, float4 *nodes, uint32_t *status)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= inCount) return;
    CollapseItem item = in[k];
    uint32_t ch[W];
    float4 clo[W], chi[W];
    int cnt = 2;
    ch[0] = left[item.bin];
    ch[1] = right[item.bin];
    child_box(ch[0], nodeLo, nodeHi, primLo, primHi, order, clo[0], chi[0]);
    child_box(ch[1], nodeLo, nodeHi, primLo, primHi, order, clo[1], chi[1]);
    while (cnt < W) {
        int best = -1;
        float bestArea = -1.0f;
        for (int c = 0; c < cnt; c++) {
            if (ch[c] & kBinLeaf) continue;
            float a = half_area(clo[c], chi[c]);
            if (a > bestArea) {
                bestArea = a;
                best = c;
            }
        }
        if (best < 0) break;
        uint32_t b = ch[best];
        ch[best] = left[b];
        child_box(ch[best], nodeLo, nodeHi, primLo, primHi, order, clo[best], chi[best]);
        ch[cnt] = right[b];
        child_box(ch[cnt], nodeLo, nodeHi, primLo, primHi, order, clo[cnt], chi[cnt]);
        cnt++;
    }
    // the node's internal children get consecutive indices (and work-list
    // slots) from one atomic each, so that siblings lie side by side in memory
    uint32_t internal = 0;
    for (int c = 0; c < cnt; c++) {
        const uint32_t r = ch[c];
        if (!(r & kBinLeaf) && last[r] - first[r] + 1u > leafMax) internal++;
    }
    const uint32_t w = internal ? atomicAdd(nodeCounter, internal) : 0u;
    // children past the capacity are reported and left out, and get no slot
    const uint32_t fit = w >= nodeCapacity ? 0u : min(internal, nodeCapacity - w);
    const uint32_t slot = fit ? atomicAdd(outCount, fit) : 0u;
    uint32_t taken = 0;
    float lo[3 * W], hi[3 * W];
    uint32_t child[W];
    for (int c = 0; c < W; c++) {
        if (c >= cnt) {
            lo[3 * c] = lo[3 * c + 1] = lo[3 * c + 2] = 1.0f;
            hi[3 * c] = hi[3 * c + 1] = hi[3 * c + 2] = 0.0f;
            child[c] = kEmptyChild;
            continue;
        }
        lo[3 * c] = clo[c].x;
        lo[3 * c + 1] = clo[c].y;
        lo[3 * c + 2] = clo[c].z;
        hi[3 * c] = chi[c].x;
        hi[3 * c + 1] = chi[c].y;
        hi[3 * c + 2] = chi[c].z;
        uint32_t r = ch[c];
        if (r & kBinLeaf) {
            child[c] = make_leaf(r & ~kBinLeaf, 1u);
        } else if (last[r] - first[r] + 1u <= leafMax) {
            child[c] = make_leaf(first[r], last[r] - first[r] + 1u);
        } else {
            if (taken >= fit) {
                atomicOr(status, kStatusBuildLoop);
                child[c] = kEmptyChild;
                continue;
            }
            child[c] = w + taken;
            out[slot + taken] = CollapseItem{r, w + taken};
            taken++;
        }
    }
    store_node(nodes + node_offset(item.wide, W / 4), W / 4, lo, hi, child);
}

// Structural check of a freshly built tree (relative indices): every
// internal child index is greater than its parent's and below the node
// count, every leaf range lies inside the primitives.  Children are always
// allocated after their parent, so this rules out cycles and makes every
// traversal loop finite.
__global__ void validate_nodes(const float4 *nodes, uint32_t quads, uint32_t count,
    uint32_t prims, uint32_t *status)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float4 *n = nodes + node_offset(i, quads);
    for (uint32_t c = 0; c < 4 * quads; c++) {
        uint32_t r = node_child(n, quads, c);
        if (r == kEmptyChild) continue;
        bool ok = child_is_leaf(r) ? (leaf_first(r) + leaf_count(r) <= prims)
                                   : (r > i && r < count);
        if (!ok) atomicOr(status, kStatusBadIndex);
    }
}

__global__ void single_leaf_root(const float4 *lo, const float4 *hi, float4 *nodes, uint32_t quads)
{
    float l[24], h[24];
    uint32_t child[8];
    for (int c = 0; c < 8; c++) {
        l[3 * c] = l[3 * c + 1] = l[3 * c + 2] = 1.0f;
        h[3 * c] = h[3 * c + 1] = h[3 * c + 2] = 0.0f;
        child[c] = kEmptyChild;
    }
    l[0] = lo[0].x;
    l[1] = lo[0].y;
    l[2] = lo[0].z;
    h[0] = hi[0].x;
    h[1] = hi[0].y;
    h[2] = hi[0].z;
    child[0] = make_leaf(0, 1);
    store_node(nodes, quads, l, h, child);
}

__global__ void init_bounds(int *b)
{
    if (threadIdx.x < 3) b[threadIdx.x] = 0x7FFFFFFF;  // ordered +max
    else if (threadIdx.x < 6) b[threadIdx.x] = (int)0x80000000;
}

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// Triangle boxes (src/sp_scene.cpp:21-54: min/max of the three positions).
__global__ void k_mesh_prepare(const gbsp_vertex *v, const uint32_t *idx, uint32_t triCount,
    float4 *lo, float4 *hi)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= triCount) return;
    const float *a = v[idx[3 * i + 0]].position;
    const float *b = v[idx[3 * i + 1]].position;
    const float *c = v[idx[3 * i + 2]].position;
    V3 A = v3(a[0], a[1], a[2]), B = v3(b[0], b[1], b[2]), C = v3(c[0], c[1], c[2]);
    V3 mn = vmin(A, vmin(B, C));
    V3 mx = vmax(A, vmax(B, C));
    lo[i] = make_float4(mn.x, mn.y, mn.z, 0.0f);
    hi[i] = make_float4(mx.x, mx.y, mx.z, 0.0f);
}

int mesh_prepare(cudaStream_t s, const gbsp_vertex *dVerts, const uint32_t *dIdx,
    uint32_t triCount, float4 *dLo, float4 *dHi)
{
    if (!triCount) return GBSP_OK;
    k_mesh_prepare<<<blocks_for(triCount, 256), 256, 0, s>>>(dVerts, dIdx, triCount, dLo, dHi);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

// Leaf-ordered triangle records and attributes; offsets the mesh's nodes into
// the pool (node indices += nodeBase, leaf first += triBase).
__global__ void k_mesh_emit(const gbsp_vertex *v, const uint32_t *idx, uint32_t triCount,
    const uint32_t *order, TriRecord *tris, TriAttr *attrs, uint32_t *triIds)
{
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= triCount) return;
    uint32_t t = order[j];
    const gbsp_vertex &va = v[idx[3 * t + 0]];
    const gbsp_vertex &vb = v[idx[3 * t + 1]];
    const gbsp_vertex &vc = v[idx[3 * t + 2]];
    V3 A = v3(va.position[0], va.position[1], va.position[2]);
    V3 B = v3(vb.position[0], vb.position[1], vb.position[2]);
    V3 C = v3(vc.position[0], vc.position[1], vc.position[2]);
    V3 n = cross(sub(B, A), sub(C, A));  // src/ray_intersection.cpp:162-168
    TriRecord r;
    r.a_nx = make_float4(A.x, A.y, A.z, n.x);
    r.b_ny = make_float4(B.x, B.y, B.z, n.y);
    r.c_nz = make_float4(C.x, C.y, C.z, n.z);
    tris[j] = r;
    TriAttr at;
    at.n0_n1x = make_float4(va.normal[0], va.normal[1], va.normal[2], vb.normal[0]);
    at.n1yz_n2 = make_float4(vb.normal[1], vb.normal[2], vc.normal[0], vc.normal[1]);
    at.n2z_uv0 = make_float4(vc.normal[2], va.uv[0], va.uv[1], vb.uv[0]);
    at.uv1y_uv2 = make_float4(vb.uv[1], vc.uv[0], vc.uv[1], 0.0f);
    attrs[j] = at;
    triIds[j] = t;
}

__global__ void k_offset_nodes(float4 *nodes, uint32_t quads, uint32_t count, uint32_t nodeBase,
    uint32_t leafBase)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float4 *n = nodes + node_offset(i, quads);
    for (uint32_t q = 0; q < quads; q++) {
        float4 &v = n[6 * quads + q];
        float *w = &v.x;
        for (int k = 0; k < 4; k++) {
            uint32_t r = __float_as_uint(w[k]);
            if (r == kEmptyChild) continue;
            r = child_is_leaf(r) ? make_leaf(leaf_first(r) + leafBase, leaf_count(r)) : r + nodeBase;
            w[k] = __uint_as_float(r);
        }
    }
}

int offset_nodes(cudaStream_t s, NodePool &pool, uint32_t nodeCount, uint32_t nodeBase,
    uint32_t leafBase)
{
    if (!nodeCount) return GBSP_OK;
    k_offset_nodes<<<blocks_for(nodeCount, 128), 128, 0, s>>>(pool.node(nodeBase), pool.quads,
        nodeCount, nodeBase, leafBase);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int mesh_emit(cudaStream_t s, const gbsp_vertex *dVerts, const uint32_t *dIdx, uint32_t triCount,
    const uint32_t *dOrder, TriRecord *dTris, TriAttr *dAttrs, uint32_t *dTriIds, uint32_t triBase)
{
    k_mesh_emit<<<blocks_for(triCount, 256), 256, 0, s>>>(dVerts, dIdx, triCount, dOrder, dTris,
        dAttrs, dTriIds);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

// Grows a node pool to at least `nodes` nodes, keeping its contents.
static int grow_pool(cudaStream_t s, NodePool &pool, size_t nodes)
{
    size_t want = nodes * kNodeComponents * pool.quads;
    if (want <= pool.buf.count && pool.buf.ptr) return GBSP_OK;
    DeviceBuffer<float4> grown;
    int rc = grown.reserve(want * 3 / 2 + 64, s);
    if (rc) return rc;
    if (pool.buf.ptr && pool.buf.count)
        GBSP_CUDA_TRY(cudaMemcpyAsync(grown.ptr, pool.buf.ptr, pool.buf.count * sizeof(float4),
            cudaMemcpyDeviceToDevice, s));
    pool.buf.release();
    pool.buf.ptr = grown.ptr;
    pool.buf.count = grown.count;
    pool.buf.stream = s;
    grown.ptr = nullptr;
    grown.count = 0;
    return GBSP_OK;
}

// Binary tree in the form the collapse reads: internal nodes 0 .. n-2 (root
// 0), child references with kBinLeaf for a primitive (its sorted position),
// each internal node's range [first, last] of sorted positions and its box,
// and order[sorted position] = primitive.
struct HostBinaryTree {
    std::vector<uint32_t> left, right, first, last, order;
    std::vector<float4> lo, hi;
};

// Top-down binned SAH build (Wald, "On fast construction of SAH-based
// bounding volume hierarchies", 2007) of the binary tree over n >= 2
// primitive boxes, split down to single primitives: at every node the
// primitives' centroids are binned into kSahBins slabs along each axis, and
// the split between bins that minimises area(left) x count(left) +
// area(right) x count(right) partitions the node's range (a median split
// when every centroid coincides).  Node boxes are exact unions.
// 64 bins: on the 1080p benchmark scene 16, 32, 64 and 128 bins gave 6.71,
// 6.48, 6.45 and 6.44 node visits per ray (1,518, 1,542, 1,547 and 1,550
// Msamples/s) for a host build time that grows with the bin count.
constexpr int kSahBins = 64;
// Above this many primitives the device LBVH (Morton order, Karras tree)
// is built instead: the host build's time grows as n log n on one core.
constexpr uint32_t kSahMaxPrims = 1u << 20;

static float half_area_host(const float4 &lo, const float4 &hi)
{
    float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

static void sah_binary_tree(const float4 *plo, const float4 *phi, uint32_t n, HostBinaryTree &t)
{
    t.left.assign(n - 1, 0);
    t.right.assign(n - 1, 0);
    t.first.assign(n - 1, 0);
    t.last.assign(n - 1, 0);
    t.lo.assign(n - 1, make_float4(0, 0, 0, 0));
    t.hi.assign(n - 1, make_float4(0, 0, 0, 0));
    t.order.resize(n);
    std::vector<float> cen(3 * (size_t)n);
    for (uint32_t i = 0; i < n; i++) {
        t.order[i] = i;
        cen[3 * (size_t)i + 0] = (plo[i].x + phi[i].x) * 0.5f;
        cen[3 * (size_t)i + 1] = (plo[i].y + phi[i].y) * 0.5f;
        cen[3 * (size_t)i + 2] = (plo[i].z + phi[i].z) * 0.5f;
    }
    struct Job {
        uint32_t node, begin, end;
    };
    std::vector<Job> jobs;
    jobs.push_back({0, 0, n});
    uint32_t next = 1;
    const float inf = 3.0e38f;
    while (!jobs.empty()) {
        const Job j = jobs.back();
        jobs.pop_back();
        float4 blo = make_float4(inf, inf, inf, 0), bhi = make_float4(-inf, -inf, -inf, 0);
        float cmin[3] = {inf, inf, inf}, cmax[3] = {-inf, -inf, -inf};
        for (uint32_t k = j.begin; k < j.end; k++) {
            const uint32_t p = t.order[k];
            blo = make_float4(rmin(blo.x, plo[p].x), rmin(blo.y, plo[p].y), rmin(blo.z, plo[p].z), 0);
            bhi = make_float4(rmax(bhi.x, phi[p].x), rmax(bhi.y, phi[p].y), rmax(bhi.z, phi[p].z), 0);
            for (int a = 0; a < 3; a++) {
                cmin[a] = std::min(cmin[a], cen[3 * (size_t)p + a]);
                cmax[a] = std::max(cmax[a], cen[3 * (size_t)p + a]);
            }
        }
        t.lo[j.node] = blo;
        t.hi[j.node] = bhi;
        t.first[j.node] = j.begin;
        t.last[j.node] = j.end - 1;
        int bestAxis = -1, bestBin = 0;
        float bestCost = inf;
        for (int a = 0; a < 3; a++) {
            const float ext = cmax[a] - cmin[a];
            if (!(ext > 0.0f)) continue;
            const float scale = (float)kSahBins / ext;
            uint32_t cnt[kSahBins] = {};
            float4 lo[kSahBins], hi[kSahBins];
            for (int b = 0; b < kSahBins; b++) {
                lo[b] = make_float4(inf, inf, inf, 0);
                hi[b] = make_float4(-inf, -inf, -inf, 0);
            }
            for (uint32_t k = j.begin; k < j.end; k++) {
                const uint32_t p = t.order[k];
                const int b = std::min(kSahBins - 1, (int)((cen[3 * (size_t)p + a] - cmin[a]) * scale));
                cnt[b]++;
                lo[b] = make_float4(std::min(lo[b].x, plo[p].x), std::min(lo[b].y, plo[p].y),
                    std::min(lo[b].z, plo[p].z), 0);
                hi[b] = make_float4(std::max(hi[b].x, phi[p].x), std::max(hi[b].y, phi[p].y),
                    std::max(hi[b].z, phi[p].z), 0);
            }
            // suffix areas and counts, then a prefix sweep
            float rArea[kSahBins];
            uint32_t rCnt[kSahBins];
            float4 rl = make_float4(inf, inf, inf, 0), rh = make_float4(-inf, -inf, -inf, 0);
            uint32_t rc = 0;
            for (int b = kSahBins - 1; b > 0; b--) {
                rc += cnt[b];
                rl = make_float4(std::min(rl.x, lo[b].x), std::min(rl.y, lo[b].y), std::min(rl.z, lo[b].z), 0);
                rh = make_float4(std::max(rh.x, hi[b].x), std::max(rh.y, hi[b].y), std::max(rh.z, hi[b].z), 0);
                rCnt[b] = rc;
                rArea[b] = rc ? half_area_host(rl, rh) : 0.0f;
            }
            float4 ll = make_float4(inf, inf, inf, 0), lh = make_float4(-inf, -inf, -inf, 0);
            uint32_t lc = 0;
            for (int b = 0; b < kSahBins - 1; b++) {
                lc += cnt[b];
                ll = make_float4(std::min(ll.x, lo[b].x), std::min(ll.y, lo[b].y), std::min(ll.z, lo[b].z), 0);
                lh = make_float4(std::max(lh.x, hi[b].x), std::max(lh.y, hi[b].y), std::max(lh.z, hi[b].z), 0);
                if (lc == 0 || rCnt[b + 1] == 0) continue;
                const float cost = half_area_host(ll, lh) * (float)lc + rArea[b + 1] * (float)rCnt[b + 1];
                if (cost < bestCost) {
                    bestCost = cost;
                    bestAxis = a;
                    bestBin = b;
                }
            }
        }
        uint32_t mid = j.begin + (j.end - j.begin) / 2;
        if (bestAxis >= 0) {
            const float scale = (float)kSahBins / (cmax[bestAxis] - cmin[bestAxis]);
            const float c0 = cmin[bestAxis];
            uint32_t *it = std::partition(t.order.data() + j.begin, t.order.data() + j.end,
                [&](uint32_t p) {
                    return std::min(kSahBins - 1, (int)((cen[3 * (size_t)p + bestAxis] - c0) * scale)) <=
                        bestBin;
                });
            const uint32_t m = (uint32_t)(it - t.order.data());
            if (m > j.begin && m < j.end) mid = m;
        }
        const uint32_t ranges[2][2] = {{j.begin, mid}, {mid, j.end}};
        for (int side = 0; side < 2; side++) {
            const uint32_t b = ranges[side][0], e = ranges[side][1];
            uint32_t ref;
            if (e - b == 1) {
                ref = kBinLeaf | b;
            } else {
                ref = next++;
                jobs.push_back({ref, b, e});
            }
            (side ? t.right : t.left)[j.node] = ref;
        }
    }
}

int build_wide_bvh(cudaStream_t s, const float4 *dLo, const float4 *dHi, uint32_t n,
    uint32_t leafMax, NodePool *pools, const uint32_t *nodeBase, WideTree *trees,
    DeviceBuffer<uint32_t> *orderOut, uint32_t *dStatus, const float4 *hLo, const float4 *hHi)
{
    if (n == 0) return set_error(GBSP_ERR_INVALID_ARGUMENT, "BVH over zero primitives");
    if (n >= (1u << 27)) return set_error(GBSP_ERR_CAPACITY, "BVH over %u primitives (max 2^27)", n);
    int rc;
    uint32_t capacity = n > 1 ? n - 1 : 1;  // wide nodes never exceed binary internal nodes
    for (int w = 0; w < kNodeWidths; w++)
        if ((rc = grow_pool(s, pools[w], (size_t)nodeBase[w] + capacity))) return rc;
    if ((rc = orderOut->reserve(n, s))) return rc;
    if (n == 1) {
        for (int w = 0; w < kNodeWidths; w++) {
            single_leaf_root<<<1, 1, 0, s>>>(dLo, dHi, pools[w].node(nodeBase[w]), pools[w].quads);
            trees[w].nodeCount = 1;
            trees[w].depth = 1;
        }
        GBSP_CUDA_TRY(cudaGetLastError());
        uint32_t zero = 0;
        GBSP_CUDA_TRY(cudaMemcpyAsync(orderOut->ptr, &zero, 4, cudaMemcpyHostToDevice, s));
        GBSP_CUDA_TRY(cudaStreamSynchronize(s));
        return GBSP_OK;
    }

    DeviceBuffer<uint32_t> codes[2], vals[2], hist, left, right, parent, first, last, arrivals,
        counters;
    DeviceBuffer<int> bounds;
    DeviceBuffer<float4> nodeLo, nodeHi;
    DeviceBuffer<CollapseItem> q[2];
    uint32_t sortBlocks = (n + kSortTile - 1) / kSortTile;
    if ((rc = codes[0].reserve(n, s)) || (rc = codes[1].reserve(n, s)) ||
        (rc = vals[0].reserve(n, s)) || (rc = vals[1].reserve(n, s)) ||
        (rc = hist.reserve((size_t)256 * sortBlocks, s)) || (rc = left.reserve(n, s)) ||
        (rc = right.reserve(n, s)) || (rc = parent.reserve(2 * (size_t)n, s)) ||
        (rc = first.reserve(n, s)) || (rc = last.reserve(n, s)) ||
        (rc = arrivals.reserve(n, s)) || (rc = counters.reserve(4, s)) ||
        (rc = bounds.reserve(6, s)) || (rc = nodeLo.reserve(n, s)) ||
        (rc = nodeHi.reserve(n, s)) || (rc = q[0].reserve(capacity, s)) ||
        (rc = q[1].reserve(capacity, s)))
        return rc;

    const uint32_t *order = nullptr;
    if (hLo && hHi && n <= kSahMaxPrims) {
        // binned SAH tree on the host (the host boxes are the device ones)
        HostBinaryTree ht;
        sah_binary_tree(hLo, hHi, n, ht);
        GBSP_CUDA_TRY(cudaMemcpyAsync(left.ptr, ht.left.data(), 4 * (size_t)(n - 1),
            cudaMemcpyHostToDevice, s));
        GBSP_CUDA_TRY(cudaMemcpyAsync(right.ptr, ht.right.data(), 4 * (size_t)(n - 1),
            cudaMemcpyHostToDevice, s));
        GBSP_CUDA_TRY(cudaMemcpyAsync(first.ptr, ht.first.data(), 4 * (size_t)(n - 1),
            cudaMemcpyHostToDevice, s));
        GBSP_CUDA_TRY(cudaMemcpyAsync(last.ptr, ht.last.data(), 4 * (size_t)(n - 1),
            cudaMemcpyHostToDevice, s));
        GBSP_CUDA_TRY(cudaMemcpyAsync(nodeLo.ptr, ht.lo.data(), sizeof(float4) * (n - 1),
            cudaMemcpyHostToDevice, s));
        GBSP_CUDA_TRY(cudaMemcpyAsync(nodeHi.ptr, ht.hi.data(), sizeof(float4) * (n - 1),
            cudaMemcpyHostToDevice, s));
        GBSP_CUDA_TRY(cudaMemcpyAsync(vals[0].ptr, ht.order.data(), 4 * (size_t)n,
            cudaMemcpyHostToDevice, s));
        // the host vectors must outlive the copies
        GBSP_CUDA_TRY(cudaStreamSynchronize(s));
        order = vals[0].ptr;
    } else {
        init_bounds<<<1, 32, 0, s>>>(bounds.ptr);
        centroid_bounds<<<min(blocks_for(n, 256), 1024u), 256, 0, s>>>(dLo, dHi, n, bounds.ptr);
        morton_codes<<<blocks_for(n, 256), 256, 0, s>>>(dLo, dHi, n, bounds.ptr, codes[0].ptr,
            vals[0].ptr);
        GBSP_CUDA_TRY(cudaGetLastError());
        int cur = 0;
        for (int shift = 0; shift < 32; shift += 8) {
            radix_histogram<<<sortBlocks, kSortThreads, 0, s>>>(codes[cur].ptr, n, shift, hist.ptr,
                sortBlocks);
            radix_scan<<<1, 1024, 0, s>>>(hist.ptr, 256 * sortBlocks);
            radix_scatter<<<sortBlocks, kSortThreads, 0, s>>>(codes[cur].ptr, vals[cur].ptr,
                codes[cur ^ 1].ptr, vals[cur ^ 1].ptr, n, shift, hist.ptr, sortBlocks);
            cur ^= 1;
        }
        GBSP_CUDA_TRY(cudaGetLastError());
        const uint32_t *sorted = codes[cur].ptr;
        order = vals[cur].ptr;
        karras_hierarchy<<<blocks_for(n - 1, 256), 256, 0, s>>>(sorted, (int)n, left.ptr,
            right.ptr, parent.ptr, first.ptr, last.ptr);
        GBSP_CUDA_TRY(cudaMemsetAsync(arrivals.ptr, 0, 4 * (size_t)n, s));
        refit<<<blocks_for(n, 256), 256, 0, s>>>((int)n, left.ptr, right.ptr, parent.ptr, dLo,
            dHi, order, nodeLo.ptr, nodeHi.ptr, arrivals.ptr, dStatus);
        GBSP_CUDA_TRY(cudaGetLastError());
    }

    // collapse the same binary tree once per width, level by level;
    // counters: [0] node counter, [1..2] queue counts
    for (int w = 0; w < kNodeWidths; w++) {
        float4 *out = pools[w].node(nodeBase[w]);
        uint32_t init[4] = {1, 0, 0, 0};
        GBSP_CUDA_TRY(cudaMemcpyAsync(counters.ptr, init, 16, cudaMemcpyHostToDevice, s));
        CollapseItem rootItem = {0, 0};
        GBSP_CUDA_TRY(cudaMemcpyAsync(q[0].ptr, &rootItem, sizeof(rootItem), cudaMemcpyHostToDevice,
            s));
        uint32_t inCount = 1, depth = 0;
        int qi = 0;
        while (inCount > 0) {
            if (depth > 200)
                return set_error(GBSP_ERR_DEVICE_STATUS, "BVH collapse exceeded 200 levels");
            GBSP_CUDA_TRY(cudaMemsetAsync(counters.ptr + 1 + (qi ^ 1), 0, 4, s));
            auto kern = pools[w].quads == 2 ? collapse_level<8> : collapse_level<4>;
            kern<<<blocks_for(inCount, 128), 128, 0, s>>>(q[qi].ptr, inCount, q[qi ^ 1].ptr,
                counters.ptr + 1 + (qi ^ 1), counters.ptr, capacity, left.ptr, right.ptr,
                first.ptr, last.ptr, nodeLo.ptr, nodeHi.ptr, dLo, dHi, order, leafMax, out, dStatus);
            GBSP_CUDA_TRY(cudaGetLastError());
            GBSP_CUDA_TRY(cudaMemcpyAsync(&inCount, counters.ptr + 1 + (qi ^ 1), 4,
                cudaMemcpyDeviceToHost, s));
            GBSP_CUDA_TRY(cudaStreamSynchronize(s));
            qi ^= 1;
            depth++;
        }
        uint32_t used = 0;
        GBSP_CUDA_TRY(cudaMemcpyAsync(&used, counters.ptr, 4, cudaMemcpyDeviceToHost, s));
        GBSP_CUDA_TRY(cudaStreamSynchronize(s));
        if (used > capacity) used = capacity;
        validate_nodes<<<blocks_for(used, 128), 128, 0, s>>>(out, pools[w].quads, used, n, dStatus);
        GBSP_CUDA_TRY(cudaGetLastError());
        trees[w].nodeCount = used;
        trees[w].depth = depth;
    }
    GBSP_CUDA_TRY(cudaMemcpyAsync(orderOut->ptr, order, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s));
    uint32_t st = 0;
    GBSP_CUDA_TRY(cudaMemcpyAsync(&st, dStatus, 4, cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    if (st & kStatusBuildLoop)
        return set_error(GBSP_ERR_DEVICE_STATUS, "BVH build exceeded its node capacity");
    if (st & kStatusBadIndex)
        return set_error(GBSP_ERR_DEVICE_STATUS, "BVH build produced an invalid child reference");
    return GBSP_OK;
}

}  // namespace gbsp
