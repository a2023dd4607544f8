// The reference's host noise stream, for BG3_NOISE_INJECT runs that replay the reference
// exactly without its code: Norm (RNG/Norm.cpp:59-86), the Marsaglia polar method in float over
// MTRand (RNG/MersenneTwister.cpp), seeded with the parameter file's seed
// (Core/SingleThreadedSpikingModel.cpp:30).  Host code only; built with -ffp-contract=off like
// the rest of the library so that every product and sum rounds as the reference's do.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <new>

#include "bg3.h"

namespace {

// MT19937 (Matsumoto and Nishimura 1998) with Knuth's seeding: the state is refilled 624 words
// at a time, and the block's words are tempered and turned into uniforms in one loop.
struct Mt {
    uint32_t s[624];
    float u[624];
    int next = 624;

    explicit Mt(uint32_t seed)
    {
        s[0] = seed;
        for (uint32_t i = 1; i < 624; i++) s[i] = 1812433253u * (s[i - 1] ^ (s[i - 1] >> 30)) + i;
        refill();
    }
    static uint32_t mix(uint32_t far, uint32_t hi, uint32_t lo)
    {
        uint32_t y = (hi & 0x80000000u) | (lo & 0x7fffffffu);
        return far ^ (y >> 1) ^ ((0u - (lo & 1u)) & 0x9908b0dfu);
    }
    void refill()
    {
        int i = 0;
        for (; i < 227; i++) s[i] = mix(s[i + 397], s[i], s[i + 1]);
        for (; i < 623; i++) s[i] = mix(s[i - 227], s[i], s[i + 1]);
        s[623] = mix(s[396], s[623], s[0]);
        // MTRand::rand as BrainGrid declares it (BGFLOAT): the tempered word over 2^32 - 1 in
        // double, rounded to float
        for (int i = 0; i < 624; i++) {
            uint32_t y = s[i];
            y ^= y >> 11;
            y ^= (y << 7) & 0x9d2c5680u;
            y ^= (y << 15) & 0xefc60000u;
            y ^= y >> 18;
            u[i] = (float)((double)(float)y * (1.0 / 4294967295.0));
        }
        next = 0;
    }
    float uniform()
    {
        if (next == 624) refill();
        return u[next++];
    }
};

}  // namespace

struct bg3_norm {
    Mt mt;
    float mu, sigma;
    bool odd = true;  // Norm's constructor (RNG/Norm.h:70): the first call computes a pair
    float x2 = 0.0f;
    bg3_norm(uint32_t seed, float m, float s) : mt(seed), mu(m), sigma(s) {}

    float draw()
    {
        if ((odd = !odd)) return mu + sigma * x2;
        float v1, v2, w;
        do {
            float u1 = mt.uniform();
            float u2 = mt.uniform();
            v1 = 2 * u1 - 1;
            v2 = 2 * u2 - 1;
            w = v1 * v1 + v2 * v2;
        } while (w > 1);
        float y = std::sqrt(-2 * std::log(w) / w);
        float x1 = v1 * y;
        x2 = v2 * y;
        return mu + sigma * x1;
    }
};

extern "C" int bg3_norm_create(uint32_t seed, float mu, float sigma, bg3_norm **out)
{
    if (!out) return BG3_EINVAL;
    *out = new (std::nothrow) bg3_norm(seed, mu, sigma);
    return *out ? BG3_OK : BG3_ENOMEM;
}

extern "C" int bg3_norm_fill(bg3_norm *g, float *values, int64_t n)
{
    if (!g || n < 0 || (n && !values)) return BG3_EINVAL;
    for (int64_t i = 0; i < n; i++) values[i] = g->draw();
    return BG3_OK;
}

extern "C" void bg3_norm_destroy(bg3_norm *g) { delete g; }
