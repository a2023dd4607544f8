// Self-tests.  bg3_selftest_binary64: the integer-pipe binary64 arithmetic (SoftD,
// bg3_internal.cuh) against the hardware on random operands (random signs, mantissas, exponents
// in [-300, 300]) and operand pairs that nearly cancel, for add, multiply and the conversion to
// float.  bg3_selftest_timeout: the bounded mbarrier wait of the step kernels, run out on purpose.
#include "../../include/bg3.h"
#include "bg3_internal.cuh"
#include "bg3_ptx.cuh"

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

// A wait that nothing ends: an mbarrier expecting one arrival that never comes, waited on by a
// warp with the step kernels' bounded wait at limit_ns.  No copy targets the barrier, so the
// block may leave it pending; the kernel records whether the wait gave up and how long it took,
// and returns.
__global__ void k_wait_test(unsigned long long limit_ns, unsigned long long *out)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        bg3::mbar_init(&bar, 1);
        bg3::fence_mbar_init();
    }
    __syncthreads();
    const unsigned long long t0 = bg3::global_ns();
    const bool done = bg3::mbar_wait(&bar, 0u, limit_ns);
    const unsigned long long t1 = bg3::global_ns();
    if (threadIdx.x == 0) {
        out[0] = done ? 0ull : (unsigned long long)BG3_ERR_TIMEOUT;
        out[1] = t1 - t0;
    }
}

}  // namespace

extern "C" int bg3_selftest_timeout(uint64_t limit_ns, uint32_t *status, uint64_t *waited_ns)
{
    if (!status || !waited_ns || limit_ns == 0 || limit_ns > 2000000000ull) return BG3_EINVAL;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return BG3_ENOMEM;
    k_wait_test<<<1, 32>>>((unsigned long long)limit_ns, d);
    unsigned long long h[2] = {0, 0};
    const cudaError_t e1 = cudaDeviceSynchronize();
    const cudaError_t e2 = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e1 != cudaSuccess || e2 != cudaSuccess) return BG3_ECUDA;
    *status = (uint32_t)h[0];
    *waited_ns = h[1];
    return BG3_OK;
}

extern "C" int bg3_selftest_binary64(uint64_t samples, uint64_t seed, uint64_t *counts)
{
    if (!counts) return BG3_EINVAL;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 4 * sizeof(unsigned long long)) != cudaSuccess) return BG3_ENOMEM;
    if (cudaMemset(d, 0, 4 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaFree(d);
        return BG3_ECUDA;
    }
    k_softd_test<<<152 * 8, 256>>>(samples, seed, d);
    unsigned long long h[4];
    const cudaError_t e1 = cudaDeviceSynchronize();
    const cudaError_t e2 = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e1 != cudaSuccess || e2 != cudaSuccess) return BG3_ECUDA;
    for (int k = 0; k < 4; k++) counts[k] = h[k];
    return BG3_OK;
}
