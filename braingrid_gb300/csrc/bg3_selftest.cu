// Self-test of the integer-pipe binary64 arithmetic (SoftD, bg3_internal.cuh) against the
// hardware: random operands (random signs, mantissas, exponents in [-300, 300]) and operand pairs
// that nearly cancel, for add, multiply and the conversion to float.
#include "../../include/bg3.h"
#include "bg3_internal.cuh"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    // SplitMix64 finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom number
    // generators", OOPSLA 2014)
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ double rand_double(uint64_t r, int emin, int emax)
{
    const uint64_t span = (uint64_t)(emax - emin + 1);
    const uint64_t ex = (uint64_t)(emin + (int)((r >> 52) % span) + 1023);
    return __longlong_as_double((long long)((r & 0x800fffffffffffffull) | (ex << 52)));
}

__global__ void k_softd_test(uint64_t n, uint64_t seed, unsigned long long *bad)
{
    unsigned long long local[4] = {0, 0, 0, 0};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r1 = mix64(seed ^ (2 * i)), r2 = mix64(seed ^ (2 * i + 1));
        const double a = rand_double(r1, -300, 300);
        double b = rand_double(r2, -300, 300);
        if ((r2 & 3ull) == 0) {  // nearly cancelling pair: -a with a few low bits changed
            b = __longlong_as_double((long long)(((uint64_t)__double_as_longlong(a) ^ (r2 >> 54)) ^
                                                 0x8000000000000000ull));
        } else if ((r2 & 3ull) == 1) {  // close exponents
            b = __longlong_as_double((long long)(((uint64_t)__double_as_longlong(b) & 0x800fffffffffffffull) |
                                                 ((uint64_t)__double_as_longlong(a) & 0x7ff0000000000000ull)));
        }
        bool ok = true;
        const SoftD sa = sd_from_double(a, ok), sb = sd_from_double(b, ok);
        const SoftD ss = sd_add(sa, sb, ok), sm = sd_mul(sa, sb, ok);
        if (!ok) {
            local[3]++;
            continue;
        }
        const double hs = __dadd_rn(a, b), hm = __dmul_rn(a, b);
        const uint64_t es = ((uint64_t)ss.s << 63) | (ss.m ? ((uint64_t)(ss.e + 1023) << 52) | (ss.m & 0xfffffffffffffull) : 0ull);
        const uint64_t em = ((uint64_t)sm.s << 63) | (sm.m ? ((uint64_t)(sm.e + 1023) << 52) | (sm.m & 0xfffffffffffffull) : 0ull);
        if (es != (uint64_t)__double_as_longlong(hs)) local[0]++;
        if (em != (uint64_t)__double_as_longlong(hm)) local[1]++;
        // conversion to float of a double in the float range
        const double c = rand_double(r1 ^ r2, -120, 120);
        bool okc = true;
        const float fc = sd_to_float(sd_from_double(c, okc), okc);
        if (okc && __float_as_uint(fc) != __float_as_uint(__double2float_rn(c))) local[2]++;
        if (!okc) local[3]++;
    }
    for (int k = 0; k < 4; k++)
        if (local[k]) atomicAdd(&bad[k], local[k]);
}

}  // namespace

extern "C" int bg3_selftest_binary64(uint64_t samples, uint64_t seed, uint64_t *counts)
{
    if (!counts) return BG3_EINVAL;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 4 * sizeof(unsigned long long)) != cudaSuccess) return BG3_ENOMEM;
    cudaMemset(d, 0, 4 * sizeof(unsigned long long));
    k_softd_test<<<152 * 8, 256>>>(samples, seed, d);
    unsigned long long h[4];
    const cudaError_t e1 = cudaDeviceSynchronize();
    const cudaError_t e2 = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e1 != cudaSuccess || e2 != cudaSuccess) return BG3_ECUDA;
    for (int k = 0; k < 4; k++) counts[k] = h[k];
    return BG3_OK;
}
