// Allocation-free variant of the outgoing synapse map build (bg3_outgoing_map_noalloc).
//
// Some callers cannot allocate device memory at the point where they need the map: a host
// runtime that hands all device memory out of its own pool and forbids the library from calling
// cudaMalloc/cudaFree behind its back, or a real-time loop that must not take the allocator's
// locks.  This entry point takes the caller's device buffers for its inputs and
// outputs and allocates nothing: its only scratch (one counter per source neuron) lives in a
// file-scope __device__ array of fixed size, which every GPU that loads the library holds until
// the process exits.
//
// Limits and sharing:
//   * at most BG3_NOALLOC_MAX_NEURONS neurons, and n_neurons * max_syn at most 2^32 (slot ids
//     are 32-bit, as the reference's BGSIZE): more is rejected with BG3_EINVAL before any work
//     is queued; a source with more than BG3_NOALLOC_MAX_FANOUT synapses (known only on the
//     device) sets bit 1 of the caller's status word and its run of the map stays unsorted;
//   * every call uses the same scratch array and leaves the last call's counters in it; each
//     call clears what it needs first, but two calls whose work overlaps on the GPU (different
//     streams, or different host threads on one device) race on it and must be serialised by
//     the caller;
//   * the first call on each device looks up the array's device address (cudaGetSymbolAddress)
//     with that device current and keeps it for the life of the process; make that first call
//     before any stream capture.  A cudaDeviceReset invalidates the kept address: a process that
//     resets a device must not call this entry point on it again;
//   * an error left pending by earlier CUDA calls of the process is cleared on entry, so that a
//     launch failure reported here is this call's own.
#include <cstdio>
#include <mutex>

#include "../../include/bg3.h"
#include "bg3_internal.cuh"

namespace {

constexpr int NOALLOC_THREADS = 256;

static __device__ __align__(256) uint32_t g_fill_scratch[BG3_NOALLOC_MAX_NEURONS];

std::mutex g_addr_mutex;
uint32_t *g_addr[64] = {};  // device address of g_fill_scratch, per device ordinal

int scratch_address(uint32_t **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return BG3_ECUDA;
    }
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_fill_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return BG3_ECUDA;
        }
        g_addr[dev] = (uint32_t *)p;
    }
    *out = g_addr[dev];
    return BG3_OK;
}

__global__ void k_na_zero(uint32_t *fill, uint32_t *cnt, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        fill[i] = 0u;
        cnt[i] = 0u;
    }
}

// in-use slots of row d are 0 .. counts[d] - 1 (reference layout, slot id d * max_syn + k)
__global__ void k_na_count(const int32_t *src, const uint32_t *counts, int n, int max_syn,
                           uint32_t *cnt, uint32_t *bad)
{
    const size_t total = (size_t)n * max_syn;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int d = (int)(i / max_syn), k = (int)(i % max_syn);
        if (k >= (int)counts[d]) continue;
        const int s = src[i];
        if (s < 0 || s >= n) { atomicOr(bad, 1u); continue; }
        atomicAdd(&cnt[s], 1u);
    }
}

__global__ void __launch_bounds__(1024) k_na_scan(const uint32_t *cnt, uint32_t *begin, int n,
                                                  uint32_t *bad)
{
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < n; b += 1024) {
        const int i = b + threadIdx.x;
        const uint32_t v = (i < n) ? cnt[i] : 0u;
        if (v > BG3_NOALLOC_MAX_FANOUT) atomicOr(bad, 2u);
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = wsum[lane], z = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            wsum[lane] = z - w;
        }
        __syncthreads();
        const uint32_t c = carry;
        if (i < n) begin[i] = c + wsum[warp] + x - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c + wsum[31] + x;
        __syncthreads();
    }
}

__global__ void k_na_fill(const int32_t *src, const uint32_t *counts, int n, int max_syn,
                          const uint32_t *begin, uint32_t *fill, uint32_t *map)
{
    const size_t total = (size_t)n * max_syn;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int d = (int)(i / max_syn), k = (int)(i % max_syn);
        if (k >= (int)counts[d]) continue;
        const int s = src[i];
        if (s < 0 || s >= n) continue;
        map[begin[s] + atomicAdd(&fill[s], 1u)] = (uint32_t)i;
    }
}

// Each source's slot ids in ascending order (the order AllSynapses::createSynapseImap produces,
// Synapses/AllSynapses.cpp:223-293): one CTA per source, bitonic sort in shared memory.
__global__ void __launch_bounds__(NOALLOC_THREADS) k_na_sort(const uint32_t *begin,
                                                             const uint32_t *cnt, uint32_t *map)
{
    __shared__ uint32_t key[BG3_NOALLOC_MAX_FANOUT];
    const uint32_t b = begin[blockIdx.x], c = cnt[blockIdx.x];
    if (c <= 1 || c > BG3_NOALLOC_MAX_FANOUT) return;
    uint32_t p2 = 1;
    while (p2 < c) p2 <<= 1;
    for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) key[i] = (i < c) ? map[b + i] : 0xffffffffu;
    __syncthreads();
    for (uint32_t k = 2; k <= p2; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) {
                const uint32_t l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const uint32_t a = key[i], e = key[l];
                    if ((a > e) == up) {
                        key[i] = e;
                        key[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (uint32_t i = threadIdx.x; i < c; i += blockDim.x) map[b + i] = key[i];
}

}  // namespace

extern "C" int bg3_outgoing_map_noalloc(const int32_t *src_dev, const uint32_t *counts_dev,
                                        int32_t n_neurons, int32_t max_syn, uint32_t *begin_dev,
                                        uint32_t *count_dev, uint32_t *map_dev,
                                        uint32_t *status_dev, void *stream)
{
    if (!src_dev || !counts_dev || !begin_dev || !count_dev || !map_dev || !status_dev ||
        n_neurons <= 0 || max_syn < 0)
        return BG3_EINVAL;
    if (n_neurons > BG3_NOALLOC_MAX_NEURONS) {
        fprintf(stderr, "bg3_outgoing_map_noalloc: %d neurons exceed the fixed scratch of %d\n",
                n_neurons, BG3_NOALLOC_MAX_NEURONS);
        return BG3_EINVAL;
    }
    if ((uint64_t)n_neurons * (uint64_t)max_syn > (1ull << 32)) {
        fprintf(stderr, "bg3_outgoing_map_noalloc: %d x %d slots do not fit 32-bit slot ids\n",
                n_neurons, max_syn);
        return BG3_EINVAL;
    }
    cudaGetLastError();  // an earlier call's pending error is not this call's
    uint32_t *fill = nullptr;
    int rc = scratch_address(&fill);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = (n_neurons + NOALLOC_THREADS - 1) / NOALLOC_THREADS;
    const int sb = 152 * 8;
    if (cudaMemsetAsync(status_dev, 0, sizeof(uint32_t), s) != cudaSuccess) return BG3_ECUDA;
    k_na_zero<<<nb, NOALLOC_THREADS, 0, s>>>(fill, count_dev, n_neurons);
    if (cudaGetLastError() != cudaSuccess) return BG3_ECUDA;
    k_na_count<<<sb, NOALLOC_THREADS, 0, s>>>(src_dev, counts_dev, n_neurons, max_syn, count_dev, status_dev);
    if (cudaGetLastError() != cudaSuccess) return BG3_ECUDA;
    k_na_scan<<<1, 1024, 0, s>>>(count_dev, begin_dev, n_neurons, status_dev);
    if (cudaGetLastError() != cudaSuccess) return BG3_ECUDA;
    k_na_fill<<<sb, NOALLOC_THREADS, 0, s>>>(src_dev, counts_dev, n_neurons, max_syn, begin_dev, fill, map_dev);
    if (cudaGetLastError() != cudaSuccess) return BG3_ECUDA;
    k_na_sort<<<n_neurons, NOALLOC_THREADS, 0, s>>>(begin_dev, count_dev, map_dev);
    if (cudaGetLastError() != cudaSuccess) return BG3_ECUDA;
    return BG3_OK;
}
