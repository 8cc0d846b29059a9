// Cube maps from an equirectangular HDR image: the reference's CreateCubeMap
// and CreateIrradianceCubeMap (src/cubemap.cpp:106-291) as CUDA kernels.
//
// CreateCubeMap: one thread per output texel (6 faces x height x width),
// face direction -> (azimuth, inclination) -> clamp-to-edge bilinear sample.
//
// CreateIrradianceCubeMap, uniform mode (the application's setting): the
// (phi, theta) grid of step 0.1 is accumulated in float exactly as the
// reference's loops do (63 x 16 = 1,008 samples) and its tangent-space
// directions and cos(theta) sin(theta) weights are tabulated once per block
// in shared memory; one warp integrates one texel, lane l taking samples l,
// l + 32, ..., then a shuffle tree sums the lanes.  The 32 MB source image
// stays L2-resident (129 MB L2), so the kernel is bound by texel fetches from
// L2 and the per-sample atan2/sqrt.
//
// Random mode: the reference draws 3 numbers per sample from ONE XorShift32
// stream for the whole cube (face, row, column, sample order).  Every texel
// draws exactly 3 * samplesPerPixel numbers, so texel i starts at state
// J^i * s0 with J = M^(3 * samplesPerPixel), M the 32 x 32 GF(2) matrix of one
// XorShift32 step; the host tabulates J^(2^k) and each thread jumps to its
// texel's state with at most 32 GF(2) matrix-vector products, then runs its
// samples sequentially.
//
// Transcendentals are CUDA's sinf/cosf/atan2f (their last bits differ from
// glibc's), so results match the reference to within those differences;
// everything else follows the reference's operation order without
// contraction.

#include <vector>

#include "gbsp_internal.h"

namespace gbsp {
namespace cube {

constexpr float kRadianceClamp = 10.0f;  // RADIANCE_CLAMP, src/config.h:37
constexpr int kMaxGridSamples = 1024;
constexpr int kIrrWarps = 8;

struct Basis {
    V3 forward, up, right;
};

// MapCubeMapLayerIndexToBasisVectors (src/cubemap.cpp:56-103)
__device__ __forceinline__ Basis face_basis(uint32_t layer)
{
    switch (layer) {
    case 0: return Basis{v3(1, 0, 0), v3(0, 1, 0), v3(0, 0, -1)};
    case 1: return Basis{v3(-1, 0, 0), v3(0, 1, 0), v3(0, 0, 1)};
    case 2: return Basis{v3(0, 1, 0), v3(0, 0, -1), v3(1, 0, 0)};
    case 3: return Basis{v3(0, -1, 0), v3(0, 0, 1), v3(1, 0, 0)};
    case 4: return Basis{v3(0, 0, 1), v3(0, 1, 0), v3(1, 0, 0)};
    default: return Basis{v3(0, 0, -1), v3(0, 1, 0), v3(-1, 0, 0)};
    }
}

struct Image {
    const float4 *pixels;
    uint32_t width, height;
};

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t)
{
    float s = 1.0f - t;
    return make_float4(a.x * s + b.x * t, a.y * s + b.y * t, a.z * s + b.z * t, a.w * s + b.w * t);
}

// SampleImageBilinear (src/image.h:34-73), clamp-to-edge
__device__ __forceinline__ float4 sample_bilinear(const Image &im, float u, float v)
{
    float px = (u * (float)im.width) - 0.5f;
    float py = (v * (float)im.height) - 0.5f;
    px = rmax(px, 0.0f);
    py = rmax(py, 0.0f);
    uint32_t x0 = (uint32_t)floorf(px), x1 = x0 + 1;
    uint32_t y0 = (uint32_t)floorf(py), y1 = y0 + 1;
    float fx = px - (float)x0, fy = py - (float)y0;
    x1 = min(x1, im.width - 1);
    y1 = min(y1, im.height - 1);
    x0 = min(x0, im.width - 1);  // u <= 1 keeps the reference's x0 in range too
    y0 = min(y0, im.height - 1);
    float4 a = __ldg(&im.pixels[(size_t)y0 * im.width + x0]);
    float4 b = __ldg(&im.pixels[(size_t)y0 * im.width + x1]);
    float4 c = __ldg(&im.pixels[(size_t)y1 * im.width + x0]);
    float4 d = __ldg(&im.pixels[(size_t)y1 * im.width + x1]);
    return lerp4(lerp4(a, b, fx), lerp4(c, d, fx), fy);
}

// ToSphericalCoordinates + MapToEquirectangular + y flip
// (src/math_lib.h:849-884, src/cubemap.cpp:176-178)
__device__ __forceinline__ void direction_uv(V3 d, float &u, float &v)
{
    float inc = atan2f(sqrtf(d.x * d.x + d.z * d.z), d.y);
    float az = atan2f(d.z, d.x);
    if (az < 0.0f) az += 2.0f * kPi;
    u = az / (2.0f * kPi);
    v = 1.0f - (cosf(inc) * 0.5f + 0.5f);
}

__device__ __forceinline__ V3 face_direction(const Basis &b, uint32_t x, uint32_t y,
    uint32_t width, uint32_t height)
{
    float fx = (float)x / (float)width;
    float fy = (float)y / (float)height;
    fy = 1.0f - fy;
    fx = fx * 2.0f - 1.0f;
    fy = fy * 2.0f - 1.0f;
    return normalize(add(add(b.forward, mul(b.right, fx)), mul(b.up, fy)));
}

__global__ void k_cube_map(Image im, uint32_t width, uint32_t height, float4 *__restrict__ out)
{
    uint64_t total = 6ull * width * height;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)(i % width);
        uint32_t y = (uint32_t)((i / width) % height);
        uint32_t layer = (uint32_t)(i / ((uint64_t)width * height));
        V3 dir = face_direction(face_basis(layer), x, y, width, height);
        float u, v;
        direction_uv(dir, u, v);
        out[i] = sample_bilinear(im, u, v);
    }
}

// Uniform grid: table entries (t.x, t.y = cos(theta), t.z, sin(theta)) of
// MapSphericalToCartesianCoordinates (src/math_lib.h:864-871).
__global__ void __launch_bounds__(32 * kIrrWarps) k_irradiance_uniform(Image im, uint32_t width,
    uint32_t height, const float2 *__restrict__ grid, uint32_t gridCount, float4 *__restrict__ out)
{
    __shared__ float4 table[kMaxGridSamples];
    for (uint32_t k = threadIdx.x; k < gridCount; k += blockDim.x) {
        float phi = grid[k].x, theta = grid[k].y;
        float st = sinf(theta);
        float4 e;
        e.x = st * cosf(phi);
        e.z = st * sinf(phi);
        e.y = cosf(theta);
        e.w = st;
        table[k] = e;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    uint64_t total = 6ull * width * height;
    uint64_t warpId = blockIdx.x * (uint64_t)kIrrWarps + (threadIdx.x >> 5);
    uint64_t warps = (uint64_t)gridDim.x * kIrrWarps;
    for (uint64_t i = warpId; i < total; i += warps) {
        uint32_t x = (uint32_t)(i % width);
        uint32_t y = (uint32_t)((i / width) % height);
        uint32_t layer = (uint32_t)(i / ((uint64_t)width * height));
        Basis b = face_basis(layer);
        V3 normal = face_direction(b, x, y, width, height);
        V3 tangent = normalize(cross(b.up, normal));
        V3 bitangent = normalize(cross(normal, tangent));
        V3 irr = v3(0.0f, 0.0f, 0.0f);
        for (uint32_t k = lane; k < gridCount; k += 32) {
            float4 e = table[k];
            V3 w = add(add(mul(normal, e.y), mul(tangent, e.x)), mul(bitangent, e.z));
            float u, v;
            direction_uv(w, u, v);
            float4 s = sample_bilinear(im, u, v);
            V3 rad = v3(rclamp(s.x, 0.0f, kRadianceClamp), rclamp(s.y, 0.0f, kRadianceClamp),
                rclamp(s.z, 0.0f, kRadianceClamp));
            irr = add(irr, mul(mul(rad, e.y), e.w));  // radiance * Cos(theta) * Sin(theta)
        }
#pragma unroll
        for (int off = 16; off; off >>= 1) {
            irr.x += __shfl_xor_sync(0xFFFFFFFFu, irr.x, off);
            irr.y += __shfl_xor_sync(0xFFFFFFFFu, irr.y, off);
            irr.z += __shfl_xor_sync(0xFFFFFFFFu, irr.z, off);
        }
        if (lane == 0) {
            float invCount = 1.0f / (float)gridCount;
            out[i] = make_float4((kPi * irr.x) * invCount, (kPi * irr.y) * invCount,
                (kPi * irr.z) * invCount, 1.0f);
        }
    }
}

struct JumpTable {
    uint32_t col[32][32];  // col[k][c]: column c of J^(2^k)
};

__device__ __forceinline__ uint32_t gf2_apply(const uint32_t *cols, uint32_t s)
{
    uint32_t r = 0;
#pragma unroll
    for (int c = 0; c < 32; c++) r ^= (s >> c & 1u) ? cols[c] : 0u;
    return r;
}

__global__ void k_irradiance_random(Image im, uint32_t width, uint32_t height, uint32_t spp,
    const JumpTable *__restrict__ jumps, uint32_t seed, float4 *__restrict__ out)
{
    uint64_t total = 6ull * width * height;
    float contribution = 1.0f / (float)spp;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)(i % width);
        uint32_t y = (uint32_t)((i / width) % height);
        uint32_t layer = (uint32_t)(i / ((uint64_t)width * height));
        uint32_t rng = seed;
        for (int k = 0; k < 32 && (i >> k); k++)
            if ((i >> k) & 1u) rng = gf2_apply(jumps->col[k], rng);
        V3 dir = face_direction(face_basis(layer), x, y, width, height);
        V3 irr = v3(0.0f, 0.0f, 0.0f);
        for (uint32_t k = 0; k < spp; k++) {
            // Vec3(RandomBilateral() x3) with GCC's right-to-left argument order
            float oz = random_bilateral(rng);
            float oy = random_bilateral(rng);
            float ox = random_bilateral(rng);
            V3 sd = normalize(add(dir, v3(ox, oy, oz)));
            if (dot(sd, dir) < 0.0f) sd = neg(sd);
            float cosine = rmax(dot(dir, sd), 0.0f);
            float u, v;
            direction_uv(sd, u, v);
            float4 s = sample_bilinear(im, u, v);
            V3 rad = v3(rclamp(s.x * cosine, 0.0f, kRadianceClamp),
                rclamp(s.y * cosine, 0.0f, kRadianceClamp), rclamp(s.z * cosine, 0.0f, kRadianceClamp));
            irr = add(irr, mul(rad, contribution));
        }
        out[i] = make_float4(irr.x, irr.y, irr.z, 1.0f);
    }
}

// ---- host: GF(2) jump-ahead of XorShift32 --------------------------------
using Mat = std::vector<uint32_t>;  // 32 columns

static uint32_t apply(const Mat &m, uint32_t s)
{
    uint32_t r = 0;
    for (int c = 0; c < 32; c++)
        if (s >> c & 1u) r ^= m[c];
    return r;
}

static Mat multiply(const Mat &a, const Mat &b)
{
    Mat r(32);
    for (int c = 0; c < 32; c++) r[c] = apply(a, b[c]);
    return r;
}

static Mat step_matrix()
{
    Mat m(32);
    for (int c = 0; c < 32; c++) {
        uint32_t s = 1u << c;
        m[c] = xorshift32(s);
    }
    return m;
}

static Mat power(Mat base, uint64_t n)
{
    Mat r(32);
    for (int c = 0; c < 32; c++) r[c] = 1u << c;
    while (n) {
        if (n & 1) r = multiply(r, base);
        base = multiply(base, base);
        n >>= 1;
    }
    return r;
}

}  // namespace cube
}  // namespace gbsp

using namespace gbsp;

static int check_image(const float *equirect, uint32_t eqW, uint32_t eqH, uint32_t w, uint32_t h,
    const float *faces)
{
    if (!eqW || !eqH || !w || !h) return set_error(GBSP_ERR_INVALID_ARGUMENT, "empty image");
    if (!equirect || !faces) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL image");
    if (((uintptr_t)equirect | (uintptr_t)faces) & 15u)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "images must be 16-byte aligned");
    return GBSP_OK;
}

static int grid_for(uint64_t work, int block)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t want = (work + block - 1) / block;
    uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * 16;
    return (int)(want < cap ? (want ? want : 1) : cap);
}

extern "C" {

uint32_t gbsp_xorshift32_jump(uint32_t state, uint64_t steps)
{
    return cube::apply(cube::power(cube::step_matrix(), steps), state);
}

int gbsp_create_cube_map(void *stream, const float *equirect, uint32_t eqWidth, uint32_t eqHeight,
    uint32_t width, uint32_t height, float *faces)
{
    int rc = check_image(equirect, eqWidth, eqHeight, width, height, faces);
    if (rc) return rc;
    cube::Image im{reinterpret_cast<const float4 *>(equirect), eqWidth, eqHeight};
    uint64_t total = 6ull * width * height;
    cube::k_cube_map<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(im, width, height,
        reinterpret_cast<float4 *>(faces));
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_create_irradiance_cube_map(void *stream, const float *equirect, uint32_t eqWidth,
    uint32_t eqHeight, uint32_t width, uint32_t height, uint32_t samplesPerPixel, uint32_t mode,
    float *faces)
{
    int rc = check_image(equirect, eqWidth, eqHeight, width, height, faces);
    if (rc) return rc;
    if (mode != GBSP_IRRADIANCE_UNIFORM && mode != GBSP_IRRADIANCE_RANDOM)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "unknown irradiance mode %u", mode);
    if (mode == GBSP_IRRADIANCE_RANDOM && samplesPerPixel == 0)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "samplesPerPixel must be positive");
    cudaStream_t s = (cudaStream_t)stream;
    cube::Image im{reinterpret_cast<const float4 *>(equirect), eqWidth, eqHeight};
    uint64_t total = 6ull * width * height;
    if (total >> 32) return set_error(GBSP_ERR_CAPACITY, "cube map too large");
    if (mode == GBSP_IRRADIANCE_UNIFORM) {
        // the reference's loops: phi, theta += 0.1f in float (src/cubemap.cpp:155-160)
        std::vector<float2> grid;
        const float delta = 0.1f;
        for (float phi = 0.0f; phi < 2.0f * kPi; phi += delta)
            for (float theta = 0.0f; theta < 0.5f * kPi; theta += delta)
                grid.push_back(make_float2(phi, theta));
        if (grid.size() > (size_t)cube::kMaxGridSamples)
            return set_error(GBSP_ERR_CAPACITY, "sample grid too large");
        float2 *dGrid = nullptr;
        GBSP_CUDA_TRY(cudaMallocAsync((void **)&dGrid, grid.size() * sizeof(float2), s));
        cudaError_t e = cudaMemcpyAsync(dGrid, grid.data(), grid.size() * sizeof(float2),
            cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            int block = 32 * cube::kIrrWarps;
            uint64_t blocks = (total + cube::kIrrWarps - 1) / cube::kIrrWarps;
            int gridBlocks = grid_for(blocks * block, block);
            cube::k_irradiance_uniform<<<gridBlocks, block, 0, s>>>(im, width, height, dGrid,
                (uint32_t)grid.size(), reinterpret_cast<float4 *>(faces));
            e = cudaGetLastError();
        }
        cudaFreeAsync(dGrid, s);
        if (e != cudaSuccess) return cuda_error(e, "irradiance (uniform)");
        return GBSP_OK;
    }
    // random mode: jump table J^(2^k), J = M^(3 spp); host copy waits for the upload
    cube::JumpTable table;
    cube::Mat j = cube::power(cube::step_matrix(), 3ull * samplesPerPixel);
    for (int k = 0; k < 32; k++) {
        for (int c = 0; c < 32; c++) table.col[k][c] = j[c];
        j = cube::multiply(j, j);
    }
    cube::JumpTable *dTable = nullptr;
    GBSP_CUDA_TRY(cudaMallocAsync((void **)&dTable, sizeof(table), s));
    cudaError_t e = cudaMemcpyAsync(dTable, &table, sizeof(table), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // `table` lives on this stack frame
    if (e == cudaSuccess) {
        cube::k_irradiance_random<<<grid_for(total, 128), 128, 0, s>>>(im, width, height,
            samplesPerPixel, dTable, 0x45BA12F3u, reinterpret_cast<float4 *>(faces));
        e = cudaGetLastError();
    }
    cudaFreeAsync(dTable, s);
    if (e != cudaSuccess) return cuda_error(e, "irradiance (random)");
    return GBSP_OK;
}

}  // extern "C"
