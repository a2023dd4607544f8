// The reference's host noise stream, for BG3_NOISE_INJECT runs that replay the reference
// exactly without its code: Norm (RNG/Norm.cpp:59-86), the Marsaglia polar method in float over
// MTRand (RNG/MersenneTwister.cpp), seeded with the parameter file's seed
// (Core/SingleThreadedSpikingModel.cpp:30).  Host code only; built with -ffp-contract=off like
// the rest of the library so that every product and sum rounds as the reference's do (and with
// the host compiler's -O3, which vectorises the generator's recurrence; the values are the
// integer recurrence's and the same float operations either way).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <new>
#include <thread>
#include <vector>

#include "bg3.h"

namespace {

// MT19937 (Matsumoto and Nishimura 1998) with Knuth's seeding: the state is refilled 624 words
// at a time (twist), and each word is tempered and turned into a uniform as MTRand::rand does.
struct Mt {
    uint32_t s[624];
    int next = 624;

    explicit Mt(uint32_t seed)
    {
        s[0] = seed;
        for (uint32_t i = 1; i < 624; i++) s[i] = 1812433253u * (s[i - 1] ^ (s[i - 1] >> 30)) + i;
    }
    static uint32_t mix(uint32_t far, uint32_t hi, uint32_t lo)
    {
        uint32_t y = (hi & 0x80000000u) | (lo & 0x7fffffffu);
        return far ^ (y >> 1) ^ ((0u - (lo & 1u)) & 0x9908b0dfu);
    }
    void twist()
    {
        int i = 0;
        for (; i < 227; i++) s[i] = mix(s[i + 397], s[i], s[i + 1]);
        for (; i < 623; i++) s[i] = mix(s[i - 227], s[i], s[i + 1]);
        s[623] = mix(s[396], s[623], s[0]);
        next = 0;
    }
    // The same recurrence from a block of 624 words (prev) into the next block (out, another
    // array): each loop reads only words that are already final, so the compiler vectorises it.
    static void next_block(const uint32_t *__restrict prev, uint32_t *__restrict out)
    {
        for (int i = 0; i < 227; i++) out[i] = mix(prev[i + 397], prev[i], prev[i + 1]);
        for (int i = 227; i < 454; i++) out[i] = mix(out[i - 227], prev[i], prev[i + 1]);
        for (int i = 454; i < 623; i++) out[i] = mix(out[i - 227], prev[i], prev[i + 1]);
        out[623] = mix(out[396], prev[623], out[0]);
    }
    // MTRand::rand as BrainGrid declares it (BGFLOAT): the tempered word over 2^32 - 1 in
    // double, rounded to float
    static float uniform_of(uint32_t y)
    {
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        return (float)((double)(float)y * (1.0 / 4294967295.0));
    }
    uint32_t word()
    {
        if (next == 624) twist();
        return s[next++];
    }
};

}  // namespace

// One attempt of the polar method on the uniform pair (u1, u2): whether it is accepted and,
// if so, the pair of normal values it yields (RNG/Norm.cpp:59-86, in float as the reference).
static inline bool polar_pair(float u1, float u2, float &x1, float &x2)
{
    const float v1 = 2 * u1 - 1;
    const float v2 = 2 * u2 - 1;
    const float w = v1 * v1 + v2 * v2;
    if (w > 1) return false;
    const float y = std::sqrt(-2 * std::log(w) / w);
    x1 = v1 * y;
    x2 = v2 * y;
    return true;
}
// Whether that attempt is accepted (the same arithmetic, without the logarithm).
static inline bool polar_accepts(float u1, float u2)
{
    const float v1 = 2 * u1 - 1;
    const float v2 = 2 * u2 - 1;
    return !(v1 * v1 + v2 * v2 > 1);
}

struct bg3_norm {
    Mt mt;
    float mu, sigma;
    bool odd = true;  // Norm's constructor (RNG/Norm.h:70): the first call computes a pair
    float x2 = 0.0f;
    std::vector<uint32_t> wbuf;  // generator words taken out and not yet consumed
    size_t wpos = 0;
    bg3_norm(uint32_t seed, float m, float s) : mt(seed), mu(m), sigma(s) {}

    float uniform()
    {
        if (wpos < wbuf.size()) return Mt::uniform_of(wbuf[wpos++]);
        return Mt::uniform_of(mt.word());
    }

    float draw()
    {
        if ((odd = !odd)) return mu + sigma * x2;
        float x1;
        for (;;) {
            const float u1 = uniform();
            const float u2 = uniform();
            if (polar_pair(u1, u2, x1, x2)) break;
        }
        return mu + sigma * x1;
    }

    // Appends at least k more words of the generator to wbuf: the current block's words not yet
    // taken, then whole blocks generated in place (no copy of the state), the last one kept as
    // the generator's state.
    void buffer_words(size_t k)
    {
        wbuf.erase(wbuf.begin(), wbuf.begin() + (ptrdiff_t)wpos);
        wpos = 0;
        if (mt.next < 624) {
            const size_t r = (size_t)(624 - mt.next);
            wbuf.insert(wbuf.end(), mt.s + mt.next, mt.s + 624);
            mt.next = 624;
            k = k > r ? k - r : 0;
        }
        const size_t nb = (k + 623) / 624;
        if (!nb) return;
        const size_t old = wbuf.size();
        wbuf.resize(old + nb * 624);
        uint32_t *dst = wbuf.data() + old;
        Mt::next_block(mt.s, dst);
        for (size_t b = 1; b < nb; b++) Mt::next_block(dst + (b - 1) * 624, dst + b * 624);
        std::copy(dst + (nb - 1) * 624, dst + nb * 624, mt.s);
    }

    // The next 2P values of the stream as P whole pairs (odd must be true: no value pending).
    // Only the generator's recurrence runs in order on this thread.  Tempering, the polar
    // attempts and the logarithms are independent per pair of words, so threads take ranges of
    // word pairs: a first pass counts each range's accepted attempts, which gives every range the
    // place of its pairs in the output, and a second writes them there: the same values in the
    // same order as 2P sequential draws.
    void fill_pairs(float *out, int64_t P)
    {
        const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        int64_t done = 0;
        while (done < P) {
            const int64_t need = P - done;
            // 4/pi attempts per accepted pair on average (the acceptance of the polar method is
            // pi/4), plus six standard deviations: few attempts are made and not used
            const size_t attempts =
                (size_t)(1.2733 * (double)need + 6.0 * std::sqrt((double)need) + 64.0);
            if (wbuf.size() - wpos < 2 * attempts) buffer_words(2 * attempts - (wbuf.size() - wpos));
            const uint32_t *w = wbuf.data() + wpos;
            const int64_t A = (int64_t)((wbuf.size() - wpos) / 2);
            const int T = (int)std::max<int64_t>(1, std::min<int64_t>(hw, A / 16384));
            std::vector<int64_t> cnt(T, 0), off(T, 0), take(T, 0), last(T, -1);
            // ranges 1.. on threads of their own, range 0 here; ranges whose thread could not be
            // started run here too, so every started thread is joined
            auto parallel = [&](auto &&fn) {
                std::vector<std::thread> th;
                th.reserve((size_t)T);
                int k = 1;
                try {
                    for (; k < T; k++) th.emplace_back(fn, k);
                } catch (...) {
                }
                for (int j = k; j < T; j++) fn(j);
                fn(0);
                for (auto &x : th) x.join();
            };
            parallel([&](int k) {
                const int64_t lo = A * k / T, hi = A * (k + 1) / T;
                int64_t c = 0;
                for (int64_t j = lo; j < hi; j++)
                    c += polar_accepts(Mt::uniform_of(w[2 * j]), Mt::uniform_of(w[2 * j + 1])) ? 1 : 0;
                cnt[k] = c;
            });
            int64_t got = 0;
            for (int k = 0; k < T; k++) {
                off[k] = got;
                take[k] = std::min<int64_t>(cnt[k], need - got);
                got += take[k];
            }
            parallel([&](int k) {
                if (take[k] <= 0) return;
                const int64_t lo = A * k / T, hi = A * (k + 1) / T;
                float *o = out + 2 * (done + off[k]);
                int64_t c = 0;
                float a, b;
                for (int64_t j = lo; j < hi && c < take[k]; j++) {
                    if (!polar_pair(Mt::uniform_of(w[2 * j]), Mt::uniform_of(w[2 * j + 1]), a, b)) continue;
                    o[2 * c] = mu + sigma * a;
                    o[2 * c + 1] = mu + sigma * b;
                    c++;
                    last[k] = j;
                }
            });
            int64_t used = A;
            if (got == need)  // the attempts after the last pair taken stay unread
                for (int k = T - 1; k >= 0; k--)
                    if (take[k] > 0) {
                        used = last[k] + 1;
                        break;
                    }
            wpos += 2 * (size_t)used;
            done += got;
        }
    }
};

extern "C" int bg3_norm_create(uint32_t seed, float mu, float sigma, bg3_norm **out)
{
    if (!out) return BG3_EINVAL;
    *out = new (std::nothrow) bg3_norm(seed, mu, sigma);
    return *out ? BG3_OK : BG3_ENOMEM;
}

// Large fills run the polar attempts on several host threads (bg3_norm::fill_pairs); the values
// are the sequential stream's, whatever the split of a stream into calls.
extern "C" int bg3_norm_fill(bg3_norm *g, float *values, int64_t n)
{
    if (!g || n < 0 || (n && !values)) return BG3_EINVAL;
    int64_t i = 0;
    if (i < n && !g->odd) values[i++] = g->draw();  // the pending second value of a pair
    const int64_t pairs = (n - i) / 2;
    if (pairs >= 65536) {
        try {
            g->fill_pairs(values + i, pairs);
        } catch (...) {  // no thread or no memory: the caller gets an error, the stream is lost
            return BG3_ENOMEM;
        }
        i += 2 * pairs;
    }
    for (; i < n; i++) values[i] = g->draw();
    return BG3_OK;
}

extern "C" void bg3_norm_destroy(bg3_norm *g) { delete g; }
