// TEST INFRASTRUCTURE ONLY (shared by the reference harness and the oracle
// port, never by the product).
//
// Per-sample RNG seeding and per-pixel accumulation used by the "hash per
// sample" rendering mode.  The reference seeds one XorShift32 stream per
// 64x64 tile (src/main.cpp:738-739) and draws sequentially; the hash mode
// instead starts every (x, y, sample) path from its own state so that paths
// are independent.  The product's device code carries its own statement of
// the same mapping; tests check that the two agree.

#pragma once
#include <cmath>
#include <cstdint>

// PCG-style integer hash from Jarzynski & Olano, "Hash Functions for GPU
// Rendering", JCGT 9(3), 2020 (the "pcg" entry of their comparison).
static inline uint32_t oracle_pcg_hash(uint32_t v)
{
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

// Chained hash of (seed, x, y, sample).  XorShift32 has a fixed point at 0,
// so a zero hash is replaced by a fixed non-zero constant.
static inline uint32_t oracle_sample_seed(
    uint32_t seed, uint32_t x, uint32_t y, uint32_t sample)
{
    uint32_t h = oracle_pcg_hash(seed);
    h = oracle_pcg_hash(h ^ x);
    h = oracle_pcg_hash(h ^ y);
    h = oracle_pcg_hash(h ^ sample);
    return h != 0u ? h : 0x6D2B79F5u;
}

// Neumaier-compensated float sum, one per colour channel.
struct OracleSum
{
    float s;
    float c;
};

static inline void oracle_sum_add(OracleSum *a, float x)
{
    float t = a->s + x;
    if (std::fabs(a->s) >= std::fabs(x))
        a->c += (a->s - t) + x;
    else
        a->c += (x - t) + a->s;
    a->s = t;
}

static inline float oracle_sum_value(const OracleSum *a) { return a->s + a->c; }
