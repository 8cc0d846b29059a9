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

#include "wavefront.cuh"

namespace gbsp {

// ---------------------------------------------------------------------------
// Reference-order tile mode: one thread walks one tile exactly like
// sp_PathTraceTile, drawing every random number from one XorShift32 stream.
// ---------------------------------------------------------------------------
constexpr int kMaxSeqBounces = 16;

template <bool kWT>
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
                    RayHit h = trace_closest<true, kWT>(sv, o, d, status, cnt);
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
        (rc = rt->vertE.reserve((size_t)maxBounces * cap, s)) ||
        (rc = rt->vertA.reserve((size_t)maxBounces * cap, s)) ||
        (rc = rt->pathRad.reserve(cap, s)))
        return rc;
    return GBSP_OK;
}

// One wave of a render: a run of whole pixels (numbered row-major through the
// region or tile list) and the paths of their samples.
struct WavePlan {
    uint64_t pixelBase, pathBase;
    uint32_t pixels, paths;
};

static int uniform_waves(uint64_t pixels, uint32_t spp, uint64_t waveTarget,
    std::vector<WavePlan> &waves);
static int variable_waves(const std::vector<uint4> &tiles, const std::vector<uint32_t> &spp,
    uint64_t waveTarget, std::vector<WavePlan> &waves);
static int render_waves(gbsp_runtime *rt, const SceneView &sv, const MaterialView &mv,
    const CameraParams &cam, const gbsp_options &opt, WaveParams wp,
    const std::vector<WavePlan> &waves, float4 *dImage, uint32_t imageWidth, float4 *dAov);

int render_frame(gbsp_runtime *rt, const SceneView &sv, const MaterialView &mv,
    const CameraParams &cam, const gbsp_options &opt, uint32_t x0, uint32_t y0, uint32_t x1,
    uint32_t y1, float4 *dImage, uint32_t imageWidth, uint32_t *rngState, float4 *dAov,
    uint32_t splitSpp, float4 *dImage2)
{
    cudaStream_t s = rt->stream;
    unsigned long long *counters = rt->dCounters;
    if (x1 <= x0 || y1 <= y0) return GBSP_OK;
    uint32_t spp = opt.spp ? opt.spp : 1;
    if (splitSpp && (splitSpp >= spp || !dImage2 || opt.rng_mode == GBSP_RNG_TILE_SEQUENTIAL))
        return set_error(GBSP_ERR_INVALID_ARGUMENT,
            "a split render needs 0 < first spp < spp, a second image and hash-per-sample seeding");
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
        auto seqKernel = sv.watertight ? k_tile_sequential<true> : k_tile_sequential<false>;
        seqKernel<<<(n + 63) / 64, 64, 0, s>>>(sv, mv, cam, dTiles.ptr, n, dStates.ptr, spp,
            maxBounces, opt.radiance_clamp, dImage, imageWidth, counters, rt->dStatus);
        GBSP_CUDA_TRY(cudaGetLastError());
        rt->launches += 1;
        if (rngState) {
            GBSP_CUDA_TRY(cudaMemcpyAsync(rngState, dStates.ptr, 4, cudaMemcpyDeviceToHost, s));
            GBSP_CUDA_TRY(cudaStreamSynchronize(s));
        }
        return GBSP_OK;
    }

    WaveParams wp;
    wp.x0 = x0;
    wp.y0 = y0;
    wp.regionW = x1 - x0;
    wp.tiles = nullptr;
    wp.tileStart = nullptr;
    wp.tileCount = 0;
    wp.tileSpp = nullptr;
    wp.tilePath = nullptr;
    wp.splitSpp = splitSpp;
    wp.image2 = splitSpp ? dImage2 : nullptr;
    std::vector<WavePlan> waves;
    int rc = uniform_waves((uint64_t)(x1 - x0) * (y1 - y0), spp, opt.wave_paths, waves);
    if (rc) return rc;
    return render_waves(rt, sv, mv, cam, opt, wp, waves, dImage, imageWidth, dAov);
}

int render_tile_list(gbsp_runtime *rt, const SceneView &sv, const MaterialView &mv,
    const CameraParams &cam, const gbsp_options &opt, const std::vector<uint4> &tiles,
    float4 *dImage, uint32_t imageWidth, const std::vector<uint32_t> *tileSpp)
{
    if (tiles.empty()) return GBSP_OK;
    if (tileSpp && tileSpp->size() != tiles.size())
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "one spp per tile");
    std::vector<uint64_t> start(tiles.size()), pathStart;
    uint64_t total = 0;
    for (size_t i = 0; i < tiles.size(); i++) {
        start[i] = total;
        total += (uint64_t)tiles[i].z * tiles[i].w;
    }
    if (total == 0) return GBSP_OK;
    std::vector<WavePlan> waves;
    int rc;
    if (tileSpp) {
        pathStart.resize(tiles.size());
        uint64_t paths = 0;
        for (size_t i = 0; i < tiles.size(); i++) {
            if ((*tileSpp)[i] == 0) return set_error(GBSP_ERR_INVALID_ARGUMENT, "tile spp 0");
            pathStart[i] = paths;
            paths += (uint64_t)tiles[i].z * tiles[i].w * (*tileSpp)[i];
        }
        rc = variable_waves(tiles, *tileSpp, opt.wave_paths, waves);
    } else {
        rc = uniform_waves(total, opt.spp ? opt.spp : 1, opt.wave_paths, waves);
    }
    if (rc) return rc;
    cudaStream_t s = rt->stream;
    DeviceBuffer<uint4> dTiles;
    DeviceBuffer<uint64_t> dStart, dPath;
    DeviceBuffer<uint32_t> dSpp;
    if ((rc = dTiles.upload(tiles.data(), tiles.size(), s)) ||
        (rc = dStart.upload(start.data(), start.size(), s)))
        return rc;
    if (tileSpp && ((rc = dSpp.upload(tileSpp->data(), tileSpp->size(), s)) ||
                       (rc = dPath.upload(pathStart.data(), pathStart.size(), s))))
        return rc;
    WaveParams wp;
    wp.x0 = wp.y0 = 0;
    wp.regionW = 1;
    wp.tiles = dTiles.ptr;
    wp.tileStart = dStart.ptr;
    wp.tileCount = (uint32_t)tiles.size();
    wp.tileSpp = tileSpp ? dSpp.ptr : nullptr;
    wp.tilePath = tileSpp ? dPath.ptr : nullptr;
    wp.splitSpp = 0;
    wp.image2 = nullptr;
    // the lists are freed in stream order behind the kernels that read them
    return render_waves(rt, sv, mv, cam, opt, wp, waves, dImage, imageWidth, nullptr);
}

// Waves of `spp` samples per pixel over `pixels` pixels: as many whole pixels
// per wave as fit in waveTarget paths (default kDefaultWavePaths), at least one.
static int uniform_waves(uint64_t pixels, uint32_t spp, uint64_t waveTarget,
    std::vector<WavePlan> &waves)
{
    if (!waveTarget) waveTarget = kDefaultWavePaths;
    const uint64_t perWave = std::min<uint64_t>(std::max<uint64_t>(1, waveTarget / spp), pixels);
    if (perWave * spp > 0x7FFFFFFFull)
        return set_error(GBSP_ERR_CAPACITY, "wave of %llu paths is too large",
            (unsigned long long)(perWave * spp));
    waves.clear();
    for (uint64_t pb = 0; pb < pixels; pb += perWave) {
        const uint32_t n = (uint32_t)std::min<uint64_t>(perWave, pixels - pb);
        waves.push_back(WavePlan{pb, pb * spp, n, n * spp});
    }
    return GBSP_OK;
}

// Waves over a tile list whose tile i renders spp[i] samples per pixel: tiles
// in order, each wave as many whole pixels as fit in waveTarget paths (at
// least one pixel), so that a pixel's samples never straddle two waves.
static int variable_waves(const std::vector<uint4> &tiles, const std::vector<uint32_t> &spp,
    uint64_t waveTarget, std::vector<WavePlan> &waves)
{
    if (!waveTarget) waveTarget = kDefaultWavePaths;
    uint32_t maxSpp = 0;
    for (uint32_t v : spp) maxSpp = std::max(maxSpp, v);
    const uint64_t cap = std::max<uint64_t>(waveTarget, maxSpp);
    if (cap > 0x7FFFFFFFull)
        return set_error(GBSP_ERR_CAPACITY, "wave of %llu paths is too large",
            (unsigned long long)cap);
    waves.clear();
    WavePlan cur{0, 0, 0, 0};
    uint64_t pixel = 0, path = 0;
    for (size_t i = 0; i < tiles.size(); i++) {
        uint64_t left = (uint64_t)tiles[i].z * tiles[i].w;
        while (left > 0) {
            uint64_t fit = (cap - cur.paths) / spp[i];
            if (fit == 0) {
                waves.push_back(cur);
                cur = WavePlan{pixel, path, 0, 0};
                continue;
            }
            const uint64_t k = std::min(fit, left);
            cur.pixels += (uint32_t)k;
            cur.paths += (uint32_t)(k * spp[i]);
            pixel += k;
            path += k * spp[i];
            left -= k;
        }
    }
    if (cur.pixels) waves.push_back(cur);
    return GBSP_OK;
}

static int render_waves(gbsp_runtime *rt, const SceneView &sv, const MaterialView &mv,
    const CameraParams &cam, const gbsp_options &opt, WaveParams wp,
    const std::vector<WavePlan> &waves, float4 *dImage, uint32_t imageWidth, float4 *dAov)
{
    cudaStream_t s = rt->stream;
    unsigned long long *counters = rt->dCounters;
    unsigned int *ctl = reinterpret_cast<unsigned int *>(rt->dCounters + GBSP_METRIC_COUNT);
    const uint32_t spp = opt.spp ? opt.spp : 1;
    const uint32_t maxBounces = opt.max_bounces;
    uint32_t cap = 1;
    for (const WavePlan &w : waves) cap = std::max(cap, w.paths);
    int rc = ensure_wave_buffers(rt, cap, std::max<uint32_t>(maxBounces, 1));
    if (rc) return rc;
    WaveBuffers wb;
    wb.rayO = rt->rayO.ptr;
    wb.rayD = rt->rayD.ptr;
    wb.hitA = rt->hitA.ptr;
    wb.hitInst = rt->hitInst.ptr;
    wb.vertE = rt->vertE.ptr;
    wb.vertA = rt->vertA.ptr;
    wb.pathRad = rt->pathRad.ptr;
    wb.pathAov = nullptr;
    if (dAov) {
        if ((rc = rt->pathAov.reserve(2 * (size_t)cap, s))) return rc;
        wb.pathAov = rt->pathAov.ptr;
    }
    wb.cap = cap;
    wp.cam = cam;
    wp.spp = spp;
    wp.maxBounces = maxBounces;
    wp.seed = opt.seed;
    wp.clampValue = opt.radiance_clamp;
    wp.nanPolicy = opt.nan_policy;
    wp.invSpp = 1.0f / (float)spp;
    wp.aovImage = dAov;
    OneScene one = {sv, mv, maxBounces, opt.radiance_clamp};
    const int shadeGrid = shade_grid<OneScene>(rt->smCount);
    const bool sortDirs = (opt.flags & GBSP_FLAG_SORT_DIRECTIONS) != 0 && maxBounces > 1;
    if (sortDirs && (rc = rt->sortHist.reserve(8 * (size_t)kSortBlocks, s))) return rc;
    bool timing = rt->stageTiming;
    for (const WavePlan &w : waves) {
        wp.pixelBase = w.pixelBase;
        wp.pixels = w.pixels;
        wp.pathBase = w.pathBase;
        wp.paths = w.paths;
        const uint32_t paths = w.paths;
        if (maxBounces == 0) {
            GBSP_CUDA_TRY(cudaMemsetAsync(wb.pathRad, 0, sizeof(float4) * (size_t)paths, s));
        } else {
            k_reset_ctl<<<1, 32, 0, s>>>(ctl, paths);
            k_generate<<<(paths + 255) / 256, 256, 0, s>>>(wp, wb);
            rt->launches += 2;
            for (uint32_t b = 0; b < maxBounces; b++) {
                // sorted queues: shade always writes queue 1, the sort moves it to queue 0
                const uint32_t side = sortDirs ? 0u : (b & 1u);
                int inQ = side ? kCtlQueue1 : kCtlQueue0;
                int outQ = side ? kCtlQueue0 : kCtlQueue1;
                const float4 *qO = wb.rayO + (side ? cap : 0);
                const float4 *qD = wb.rayD + (side ? cap : 0);
                k_reset_stage<<<1, 1, 0, s>>>(ctl, outQ);
                int e0 = timing ? rt->stage_event(s) : -1;
                bool perLane = (opt.flags & GBSP_FLAG_TRACE_PER_LANE) ||
                    (!(opt.flags & GBSP_FLAG_TRACE_PER_WARP) && b > 0);
                launch_trace_stage(perLane, sv.watertight != 0,
                    trace_grid<OneScene>(perLane, sv.watertight != 0, rt->smCount), s, one, qO, qD,
                    ctl + inQ, wb.hitA, wb.hitInst, ctl, counters, rt->dStatus);
                int e1 = timing ? rt->stage_event(s) : -1;
                k_shade<<<shadeGrid, 128, 0, s>>>(one, wb, b, inQ, ctl, counters);
                if (sortDirs && b + 1 < maxBounces) {
                    k_octant_count<<<kSortBlocks, 256, 0, s>>>(wb.rayD + cap, ctl, kCtlQueue1,
                        rt->sortHist.ptr);
                    k_octant_scan<<<1, 1024, 0, s>>>(rt->sortHist.ptr, ctl, kCtlQueue1, kCtlQueue0);
                    k_octant_scatter<<<kSortBlocks, 256, 0, s>>>(wb.rayO + cap, wb.rayD + cap, ctl,
                        kCtlQueue1, rt->sortHist.ptr, wb.rayO, wb.rayD);
                    rt->launches += 3;
                }
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
constexpr size_t kNaVertE = na_align(kNaHitInst + 4 * (size_t)kNoAllocMaxPaths);
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

// Makes a device current for the scope of a call and restores the caller's
// current device on every return.
struct CurrentDeviceScope {
    int previous = -1;
    bool changed = false;
    cudaError_t enter(int device)
    {
        cudaError_t e = cudaGetDevice(&previous);
        if (e != cudaSuccess) return e;
        if (previous == device) return cudaSuccess;
        e = cudaSetDevice(device);
        changed = e == cudaSuccess;
        return e;
    }
    ~CurrentDeviceScope()
    {
        if (changed) cudaSetDevice(previous);
    }
};

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
    if (opt.flags & GBSP_FLAG_AOV)
        return set_error(GBSP_ERR_INVALID_ARGUMENT,
            "the allocation-free entry writes no G-buffers (GBSP_FLAG_AOV)");
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

    CurrentDeviceScope deviceScope;
    GBSP_CUDA_TRY(deviceScope.enter(rt->device));
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
    wp.tiles = nullptr;
    wp.tileStart = nullptr;
    wp.tileCount = 0;
    wp.tileSpp = nullptr;
    wp.tilePath = nullptr;
    wp.splitSpp = 0;
    wp.image2 = nullptr;
    wp.spp = spp;
    wp.maxBounces = opt.max_bounces;
    wp.seed = opt.seed;
    wp.clampValue = opt.radiance_clamp;
    wp.nanPolicy = opt.nan_policy;
    wp.invSpp = 1.0f / (float)spp;
    wp.aovImage = nullptr;
    OneScene one = {sc->view(), mv, opt.max_bounces, opt.radiance_clamp};
    float4 *image = reinterpret_cast<float4 *>(deviceImage);
    uint64_t regionPixels = (uint64_t)(x1 - x0) * (y1 - y0);
    int grid = rt->smCount * 8;
    uint64_t launches = 0, traceLaunches = 0;
    for (uint64_t pb = 0; pb < regionPixels; pb += pixelsPerWave) {
        wp.pixelBase = pb;
        uint64_t left = regionPixels - pb;
        wp.pixels = (uint32_t)(left < pixelsPerWave ? left : pixelsPerWave);
        uint32_t paths = wp.pixels * spp;
        wp.pathBase = pb * spp;
        wp.paths = paths;
        if (opt.max_bounces == 0) {
            GBSP_CUDA_TRY(cudaMemsetAsync(wb.pathRad, 0, sizeof(float4) * (size_t)paths, s));
        } else {
            k_reset_ctl<<<1, 32, 0, s>>>(ctl, paths);
            k_generate<<<(paths + 255) / 256, 256, 0, s>>>(wp, wb);
            launches += 2;
            for (uint32_t b = 0; b < opt.max_bounces; b++) {
                int inQ = (b & 1) ? kCtlQueue1 : kCtlQueue0;
                int outQ = (b & 1) ? kCtlQueue0 : kCtlQueue1;
                k_reset_stage<<<1, 1, 0, s>>>(ctl, outQ);
                // the same per-bounce scheduling choice as the regular entry points
                // (it changes the order of work, not the results)
                bool perLane = (opt.flags & GBSP_FLAG_TRACE_PER_LANE) ||
                    (!(opt.flags & GBSP_FLAG_TRACE_PER_WARP) && b > 0);
                launch_trace_stage(perLane, one.sv.watertight != 0, grid, s, one,
                    wb.rayO + ((b & 1) ? wb.cap : 0), wb.rayD + ((b & 1) ? wb.cap : 0), ctl + inQ,
                    wb.hitA, wb.hitInst, ctl, counters, status);
                k_shade<<<shade_grid<OneScene>(rt->smCount), 128, 0, s>>>(one, wb, b, inQ, ctl,
                    counters);
                launches += 3;
                traceLaunches += 1;
            }
        }
        k_accumulate<<<(wp.pixels + 255) / 256, 256, 0, s>>>(wp, wb, image, ip->width, counters);
        launches += 1;
        GBSP_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long hostCounters[GBSP_METRIC_COUNT];
    uint32_t st = 0;
    GBSP_CUDA_TRY(cudaMemcpyAsync(hostCounters, counters, sizeof(hostCounters), cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaMemcpyAsync(&st, status, 4, cudaMemcpyDeviceToHost, s));
    GBSP_CUDA_TRY(cudaStreamSynchronize(s));
    if (st)
        return set_error(GBSP_ERR_DEVICE_STATUS, "device status 0x%x in the allocation-free render", st);
    hostCounters[GBSP_METRIC_TRACE_LAUNCHES] += traceLaunches;
    hostCounters[GBSP_METRIC_KERNEL_LAUNCHES] += launches;
    if (metrics)
        for (int i = 0; i < GBSP_METRIC_COUNT; i++) metrics->values[i] += hostCounters[i];
    return GBSP_OK;
}
