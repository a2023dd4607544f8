// Self-tests.  bg3_selftest_binary64: the integer-pipe binary64 arithmetic (SoftD,
// bg3_internal.cuh) against the hardware on random operands (random signs, mantissas, exponents
// in [-300, 300]) and operand pairs that nearly cancel, for add, multiply and the conversion to
// float.  bg3_selftest_izhikevich: the Izhikevich update's double expression evaluated on the
// integer pipe and in float-float arithmetic, against the FP64 pipe.  bg3_selftest_timeout: the bounded mbarrier wait of the step kernels, run out on purpose.
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

// The Izhikevich update's double expression (izh_v_fp64) against its integer-pipe restatement
// (neuron_apply's IZH_SOFT branch) and its float-float evaluation (izh_v_ff), on random membrane
// potentials in [-100, 60] mV, recovery variables in [-40, 40], C3 in [0.02, 0.5] and summation
// inputs C2 sp in [-0.05, 0.05] V, a quarter of them drawn near the values where the float
// rounding is close (v with few mantissa bits).
__device__ __forceinline__ float izh_v_soft(float Vint, float u, float C3, float c2sp, bool &ok)
{
    constexpr SoftD K004 = {0x147ae147ae147bull, -5, 0u};
    constexpr SoftD K140 = {0x11800000000000ull, 7, 0u};
    constexpr SoftD K0001 = {0x10624dd2f1a9fcull, -10, 0u};
    const SoftD vd = sd_from_float(Vint, ok);
    SoftD t = sd_mul(K004, vd, ok);
    t = sd_mul(t, vd, ok);
    t = sd_add(t, sd_from_float(5.0f * Vint, ok), ok);
    t = sd_add(t, K140, ok);
    SoftD nu = sd_from_float(u, ok);
    nu.s ^= 1u;
    t = sd_add(t, nu, ok);
    t = sd_mul(sd_from_float(C3, ok), t, ok);
    const float Vb = sd_to_float(sd_add(vd, t, ok), ok);
    SoftD w = sd_mul(sd_from_float(Vb, ok), K0001, ok);
    w = sd_add(w, sd_from_float(c2sp, ok), ok);
    return sd_to_float(w, ok);
}

__global__ void k_izh_test(uint64_t n, uint64_t seed, unsigned long long *bad)
{
    unsigned long long local[4] = {0, 0, 0, 0};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r1 = mix64(seed ^ (2 * i)), r2 = mix64(seed ^ (2 * i + 1));
        const float f1 = (float)(r1 >> 40) * 0x1p-24f, f2 = (float)((r1 >> 16) & 0xffffffull) * 0x1p-24f;
        const float f3 = (float)(r2 >> 40) * 0x1p-24f, f4 = (float)((r2 >> 16) & 0xffffffull) * 0x1p-24f;
        float Vint = -100.0f + 160.0f * f1;
        if ((r2 & 3ull) == 0) Vint = __uint_as_float(__float_as_uint(Vint) & 0xffffff00u);
        const float u = -40.0f + 80.0f * f2, C3 = 0.02f + 0.48f * f3, c2sp = -0.05f + 0.1f * f4;
        const float hw = izh_v_fp64(Vint, u, C3, c2sp);
        bool ok = true;
        const float sw = izh_v_soft(Vint, u, C3, c2sp, ok);
        if (ok && __float_as_uint(sw) != __float_as_uint(hw)) local[0]++;
        bool ffok = false;
        const float fv = izh_v_ff(Vint, u, C3, c2sp, ffok);
        if (!ffok) local[2]++;
        else if (__float_as_uint(fv) != __float_as_uint(hw)) local[1]++;
        if (!ok) local[3]++;
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

extern "C" int bg3_selftest_izhikevich(uint64_t samples, uint64_t seed, uint64_t *counts)
{
    if (!counts) return BG3_EINVAL;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 4 * sizeof(unsigned long long)) != cudaSuccess) return BG3_ENOMEM;
    if (cudaMemset(d, 0, 4 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaFree(d);
        return BG3_ECUDA;
    }
    k_izh_test<<<152 * 8, 256>>>(samples, seed, d);
    unsigned long long h[4];
    const cudaError_t e1 = cudaDeviceSynchronize();
    const cudaError_t e2 = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e1 != cudaSuccess || e2 != cudaSuccess) return BG3_ECUDA;
    for (int k = 0; k < 4; k++) counts[k] = h[k];
    return BG3_OK;
}
