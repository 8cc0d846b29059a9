// Oracle for the cube-map builders: TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of the reference's CreateCubeMap and
// CreateIrradianceCubeMap (src/cubemap.cpp:106-291): equirectangular HDR
// image -> six cube faces, and the diffuse irradiance cube map integrated
// either on the uniform (phi, theta) grid with step 0.1 (the application's
// setting, src/config.h:43) or with random hemisphere offsets from one RNG
// stream seeded 0x45BA12F3.  Built with -ffp-contract=off and the host's
// libm, so on the same host it reproduces the reference bit for bit (checked
// against oracle/_ref).  Only tests and the benchmark's CPU leg use it.

#include <cmath>
#include <cstdint>
#include <cstring>

extern "C" float oracle_random_bilateral(uint32_t *state);

namespace {

const float kPi = 3.14159265359f;        // src/math_lib.h:6
const float kEpsilon = 1.19209290e-07f;  // FLT_EPSILON
const float kRadianceClamp = 10.0f;      // RADIANCE_CLAMP, src/config.h:37

struct V3 {
    float x, y, z;
};
struct V4 {
    float x, y, z, w;
};

V3 v3(float x, float y, float z) { return V3{x, y, z}; }
V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b)
{
    return v3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
V3 normalize(V3 v)
{
    float len = std::sqrt(dot(v, v));
    V3 r = v3(0.0f, 0.0f, 0.0f);
    if (len > kEpsilon) r = mul(v, 1.0f / len);
    return r;
}
float rmin(float a, float b) { return a < b ? a : b; }
float rmax(float a, float b) { return a > b ? a : b; }
float rclamp(float x, float lo, float hi) { return rmin(rmax(x, lo), hi); }

struct Basis {
    V3 forward, up, right;
};

// MapCubeMapLayerIndexToBasisVectors (src/cubemap.cpp:56-103)
Basis face_basis(uint32_t layer)
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
    const float *pixels;
    uint32_t width, height;
};

V4 texel(const Image &im, uint32_t x, uint32_t y)
{
    const float *p = im.pixels + ((size_t)y * im.width + x) * 4;
    return V4{p[0], p[1], p[2], p[3]};
}

V4 lerp(V4 a, V4 b, float t)
{
    float s = 1.0f - t;
    return V4{a.x * s + b.x * t, a.y * s + b.y * t, a.z * s + b.z * t, a.w * s + b.w * t};
}

// SampleImageBilinear (src/image.h:34-73), clamp-to-edge
V4 sample_bilinear(const Image &im, float u, float v)
{
    float px = (u * (float)im.width) - 0.5f;
    float py = (v * (float)im.height) - 0.5f;
    px = rmax(px, 0.0f);
    py = rmax(py, 0.0f);
    uint32_t x0 = (uint32_t)std::floor(px), x1 = x0 + 1;
    uint32_t y0 = (uint32_t)std::floor(py), y1 = y0 + 1;
    float fx = px - (float)x0, fy = py - (float)y0;
    x1 = x1 < im.width - 1 ? x1 : im.width - 1;
    y1 = y1 < im.height - 1 ? y1 : im.height - 1;
    // the reference asserts x0 < width; u <= 1 keeps it there
    if (x0 > im.width - 1) x0 = im.width - 1;
    if (y0 > im.height - 1) y0 = im.height - 1;
    V4 t0 = lerp(texel(im, x0, y0), texel(im, x1, y0), fx);
    V4 t1 = lerp(texel(im, x0, y1), texel(im, x1, y1), fx);
    return lerp(t0, t1, fy);
}

// ToSphericalCoordinates + MapToEquirectangular + the y flip
// (src/math_lib.h:849-884, src/cubemap.cpp:176-178)
void direction_uv(V3 d, float *u, float *v)
{
    float inc = std::atan2(std::sqrt(d.x * d.x + d.z * d.z), d.y);
    float az = std::atan2(d.z, d.x);
    if (az < 0.0f) az += 2.0f * kPi;
    *u = az / (2.0f * kPi);
    float vv = std::cos(inc) * 0.5f + 0.5f;
    *v = 1.0f - vv;
}

V3 face_direction(const Basis &b, uint32_t x, uint32_t y, uint32_t width, uint32_t height)
{
    float fx = (float)x / (float)width;
    float fy = (float)y / (float)height;
    fy = 1.0f - fy;
    fx = fx * 2.0f - 1.0f;
    fy = fy * 2.0f - 1.0f;
    V3 dir = add(add(b.forward, mul(b.right, fx)), mul(b.up, fy));
    return normalize(dir);
}

}  // namespace

extern "C" {

// CreateCubeMap (src/cubemap.cpp:235-291): out = 6 faces x height x width RGBA32F
void oracle_create_cube_map(const float *equirect, uint32_t eqWidth, uint32_t eqHeight,
    uint32_t width, uint32_t height, float *out)
{
    Image im{equirect, eqWidth, eqHeight};
    for (uint32_t layer = 0; layer < 6; layer++) {
        Basis b = face_basis(layer);
        for (uint32_t y = 0; y < height; y++)
            for (uint32_t x = 0; x < width; x++) {
                V3 dir = face_direction(b, x, y, width, height);
                float u, v;
                direction_uv(dir, &u, &v);
                V4 s = sample_bilinear(im, u, v);
                float *o = out + (((size_t)layer * height + y) * width + x) * 4;
                o[0] = s.x;
                o[1] = s.y;
                o[2] = s.z;
                o[3] = s.w;
            }
    }
}

// CreateIrradianceCubeMap (src/cubemap.cpp:106-233).  mode 0: the uniform
// (phi, theta) grid; mode 1: samplesPerPixel random offsets per texel, one
// XorShift32 stream for the whole cube in face, row, column, sample order.
void oracle_create_irradiance_cube_map(const float *equirect, uint32_t eqWidth,
    uint32_t eqHeight, uint32_t width, uint32_t height, uint32_t samplesPerPixel, uint32_t mode,
    float *out)
{
    Image im{equirect, eqWidth, eqHeight};
    float contribution = 1.0f / (float)samplesPerPixel;
    uint32_t rng = 0x45BA12F3u;
    for (uint32_t layer = 0; layer < 6; layer++) {
        Basis b = face_basis(layer);
        for (uint32_t y = 0; y < height; y++)
            for (uint32_t x = 0; x < width; x++) {
                V3 dir = face_direction(b, x, y, width, height);
                V3 irr = v3(0.0f, 0.0f, 0.0f);
                if (mode == 0) {
                    V3 normal = dir;
                    V3 tangent = normalize(cross(b.up, normal));
                    V3 bitangent = normalize(cross(normal, tangent));
                    const float delta = 0.1f;
                    uint32_t count = 0;
                    for (float phi = 0.0f; phi < 2.0f * kPi; phi += delta)
                        for (float theta = 0.0f; theta < 0.5f * kPi; theta += delta) {
                            V3 t;
                            t.x = std::sin(theta) * std::cos(phi);
                            t.z = std::sin(theta) * std::sin(phi);
                            t.y = std::cos(theta);
                            V3 w = add(add(mul(normal, t.y), mul(tangent, t.x)), mul(bitangent, t.z));
                            float u, v;
                            direction_uv(w, &u, &v);
                            V4 s = sample_bilinear(im, u, v);
                            V3 rad = v3(rclamp(s.x, 0.0f, kRadianceClamp),
                                rclamp(s.y, 0.0f, kRadianceClamp), rclamp(s.z, 0.0f, kRadianceClamp));
                            float c = std::cos(theta), sn = std::sin(theta);
                            irr = add(irr, mul(mul(rad, c), sn));
                            count++;
                        }
                    irr = mul(v3(kPi * irr.x, kPi * irr.y, kPi * irr.z), 1.0f / (float)count);
                } else {
                    for (uint32_t k = 0; k < samplesPerPixel; k++) {
                        // Vec3(RandomBilateral(), x3): GCC evaluates the
                        // arguments right to left, so z takes the first draw
                        float oz = oracle_random_bilateral(&rng);
                        float oy = oracle_random_bilateral(&rng);
                        float ox = oracle_random_bilateral(&rng);
                        V3 sd = normalize(add(dir, v3(ox, oy, oz)));
                        if (dot(sd, dir) < 0.0f) sd = v3(-sd.x, -sd.y, -sd.z);
                        float cosine = rmax(dot(dir, sd), 0.0f);
                        float u, v;
                        direction_uv(sd, &u, &v);
                        V4 s = sample_bilinear(im, u, v);
                        V3 rad = v3(rclamp(s.x * cosine, 0.0f, kRadianceClamp),
                            rclamp(s.y * cosine, 0.0f, kRadianceClamp),
                            rclamp(s.z * cosine, 0.0f, kRadianceClamp));
                        irr = add(irr, mul(rad, contribution));
                    }
                }
                float *o = out + (((size_t)layer * height + y) * width + x) * 4;
                o[0] = irr.x;
                o[1] = irr.y;
                o[2] = irr.z;
                o[3] = 1.0f;
            }
    }
}

}  // extern "C"
