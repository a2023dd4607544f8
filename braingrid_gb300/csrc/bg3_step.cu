// Per-step kernels of the spiking hot path: neuron integration, spike propagation, synapse sweep.
//
// One simulation step t is three launches on the network's stream:
//   k_neurons_*  (t)  LIF integration / refractory / fire; spikers compacted into a list
//   k_fanout     (t)  one warp per spiking neuron sets bit (t + delay) & 31 of each outgoing
//                     synapse's delay queue (each synapse has a single source, so no two warps
//                     touch one queue word)
//   k_sweep      (t)  per 32-dest tile: pop the step's queue bit, DS facilitation/depression on a
//                     hit, psr *= decay, and the ordered sum psr -> summation point of each dest;
//                     the last tile to finish advances the device step counter.
#include "bg3_internal.cuh"

namespace bg3 {

// ---- neurons ---------------------------------------------------------------------------------
enum { BR_REFRACTORY = 0, BR_FIRE = 1, BR_INTEGRATE = 2 };

// AllLIFNeurons::advanceNeuron branch selection (Neurons/AllLIFNeurons.cpp:31-35).
__device__ __forceinline__ int lif_branch(const NetDev &n, int i)
{
    if (n.refr[i] > 0) return BR_REFRACTORY;
    if (n.Vm[i] >= n.Vthresh[i]) return BR_FIRE;
    return BR_INTEGRATE;
}

// AllLIFNeurons::advanceNeuron / fire and AllSpikingNeurons::fire
// (Neurons/AllLIFNeurons.cpp:20-77, Neurons/AllSpikingNeurons.cpp:155-172).  Returns true when
// the neuron fired.  The library is built with -fmad=false: each operation rounds on its own.
__device__ __forceinline__ bool lif_apply(const NetDev &n, int i, int br, float noise,
                                          unsigned long long t)
{
    bool fired = false;
    if (br == BR_REFRACTORY) {
        n.refr[i] = n.refr[i] - 1;
    } else if (br == BR_FIRE) {
        int cnt = n.spikeCount[i];
        int idx = (cnt + n.spikeCountOffset[i]) % n.max_spikes;
        n.history[(size_t)i * n.max_spikes + idx] = t;
        cnt += 1;
        n.spikeCount[i] = cnt;
        if (cnt >= n.max_spikes) set_err(n, 1u << 0);
        n.refr[i] = (int)((double)(n.Trefract[i] / n.dt) + 0.5);
        n.Vm[i] = n.Vreset[i];
        fired = true;
    } else {
        float sp = n.sp[i];
        sp = sp + n.I0[i];
        sp = sp + noise * n.Inoise[i];
        n.Vm[i] = n.C1[i] * n.Vm[i] + n.C2[i] * sp;
    }
    n.sp[i] = 0.0f;
    return fired;
}

__device__ __forceinline__ void push_spike(const NetDev &n, bool fired)
{
    unsigned mask = __ballot_sync(0xffffffffu, fired);
    if (!mask) return;
    int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == __ffs(mask) - 1) base = atomicAdd(n.nspikes, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
    if (fired) {
        int pos = base + __popc(mask & ((1u << lane) - 1));
        if (pos < n.N) n.spikes[pos] = (int)(blockIdx.x * blockDim.x + threadIdx.x);
        else set_err(n, 1u << 5);
    }
}

// Device-noise mode: one N(0,1) draw per neuron per step, keyed by (seed, step, neuron).
__global__ void __launch_bounds__(256) k_neurons_device(const NetDev *nets)
{
    const NetDev &n = nets[0];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long t = *n.step;
    bool fired = false;
    if (i < n.N) {
        int br = lif_branch(n, i);
        float noise = (br == BR_INTEGRATE) ? normal_device(n.noise_seed, t, i) : 0.0f;
        fired = lif_apply(n, i, br, noise, t);
    }
    push_spike(n, fired);
}

// Injected-noise mode: the reference CPU draws one value per integrating neuron while walking
// neurons from N-1 down to 0 (Neurons/AllSpikingNeurons.cpp:104).  One CTA walks the neurons in
// chunks of 1024 from the top; a block scan of the "integrates" flags gives each neuron the
// number of integrating neurons above it, i.e. its position in the stream.
__global__ void __launch_bounds__(1024) k_neurons_inject(const NetDev *nets)
{
    const NetDev &n = nets[0];
    __shared__ int warp_tot[32];
    __shared__ long long s_running;
    unsigned long long t = *n.step;
    unsigned long long cursor = *n.noise_cursor;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_running = 0;
    __syncthreads();
    for (int top = n.N - 1; top >= 0; top -= 1024) {
        int i = top - (int)threadIdx.x;
        int br = (i >= 0) ? lif_branch(n, i) : BR_REFRACTORY;
        bool integ = (i >= 0) && br == BR_INTEGRATE;
        unsigned m = __ballot_sync(0xffffffffu, integ);
        int in_warp = __popc(m & ((1u << lane) - 1));
        if (lane == 31) warp_tot[warp] = __popc(m);
        __syncthreads();
        if (warp == 0) {
            int v = warp_tot[lane];
            int x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            warp_tot[lane] = x - v;  // exclusive prefix of warp totals
        }
        __syncthreads();
        long long running = s_running;
        long long rank = running + warp_tot[warp] + in_warp;
        bool fired = false;
        if (i >= 0) {
            float noise = 0.0f;
            if (integ) {
                long long pos = (long long)cursor + rank;
                if (pos < n.noise_len) noise = n.noise_buf[pos];
                else set_err(n, 1u << 3);
            }
            fired = lif_apply(n, i, br, noise, t);
        }
        // compaction: neuron id, not thread id
        unsigned fm = __ballot_sync(0xffffffffu, fired);
        if (fm) {
            int b = 0;
            if (lane == __ffs(fm) - 1) b = atomicAdd(n.nspikes, __popc(fm));
            b = __shfl_sync(0xffffffffu, b, __ffs(fm) - 1);
            if (fired) {
                int pos = b + __popc(fm & ((1u << lane) - 1));
                if (pos < n.N) n.spikes[pos] = i;
                else set_err(n, 1u << 5);
            }
        }
        __syncthreads();
        if (threadIdx.x == 1023) s_running = running + warp_tot[31] + __popc(m);
        __syncthreads();
    }
    if (threadIdx.x == 0) *n.noise_cursor = cursor + (unsigned long long)s_running;
}

// ---- spike propagation -----------------------------------------------------------------------
// AllSpikingSynapses::preSpikeHit over the outgoing map (Neurons/AllSpikingNeurons.cpp:117-128,
// Synapses/AllSpikingSynapses.cpp:261-279).  Global-phase queues: bit (t + total_delay) & 31.
__global__ void __launch_bounds__(256) k_fanout(const NetDev *nets)
{
    const NetDev &n = nets[0];
    unsigned long long t = *n.step;
    int ns = min(*n.nspikes, n.N);
    int lane = threadIdx.x & 31;
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nw = (gridDim.x * blockDim.x) >> 5;
    for (int s = gw; s < ns; s += nw) {
        int i = n.spikes[s];
        uint32_t b = n.outBegin[i], c = n.outCount[i];
        for (uint32_t j = lane; j < c; j += 32) {
            uint32_t e = n.outMap[b + j];
            uint32_t pos = e & BG3_POS_MASK;
            uint32_t bit = 1u << ((uint32_t)(t + (e >> BG3_DELAY_SHIFT)) & 31u);
            uint32_t q = n.queue[pos];
            if (q & bit) set_err(n, 1u << 1);
            n.queue[pos] = q | bit;
        }
    }
}

// ---- synapse sweep ---------------------------------------------------------------------------
// AllDSSynapses::changePSR (Synapses/AllDSSynapses.cpp:227-247).
__device__ __forceinline__ float ds_hit(const NetDev &n, size_t p, float psr, float decay,
                                        unsigned long long t)
{
    float u = n.u[p], r = n.r[p];
    unsigned long long last = n.lastSpike[p];
    if (last != BG3_ULONG_MAX) {
        float isi = (float)(t - last) * n.dt;
        float D = n.D[p], F = n.F[p], U = n.U[p];
        r = 1.0f + (r * (1.0f - u) - 1.0f) * exp_cr(-isi / D);
        u = U + u * (1.0f - U) * exp_cr(-isi / F);
        n.r[p] = r;
        n.u[p] = u;
    }
    n.lastSpike[p] = t;
    return psr + ((n.W[p] / decay) * u * r);
}

constexpr int SW_DESTS = 32;   // dests per tile (one per lane)
constexpr int SW_WARPS = 8;    // warps per CTA
constexpr int SW_ROWS = 64;    // rows per chunk; each warp takes SW_ROWS / SW_WARPS of them
constexpr int SW_RPW = SW_ROWS / SW_WARPS;

// AllSpikingSynapses::advanceSynapse / isSpikeQueue over every in-use synapse
// (Synapses/AllSpikingSynapses.cpp:242-319) with the summation of AllSynapses::advanceSynapses
// (Synapses/AllSynapses.cpp:325-331): sp[d] = ((0 + psr_0) + psr_1) + ... in slot order, the
// order the reference accumulates in.  All warps update psr for a 64-row chunk (loads first, so
// each thread keeps 8 x 3 loads in flight), the chunk is staged in shared memory, and warp 0
// adds it in row order for its 32 dests.
template <int SYN>
__global__ void __launch_bounds__(SW_WARPS * 32) k_sweep(const NetDev *nets)
{
    const NetDev &n = nets[0];
    __shared__ float stage[SW_ROWS][SW_DESTS + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int d = blockIdx.x * SW_DESTS + lane;
    const bool valid = d < n.N;
    const unsigned long long t = *n.step;
    const uint32_t bit = 1u << ((uint32_t)t & 31u);
    const int cnt = valid ? (int)n.count[d] : 0;
    const int kmax = __reduce_max_sync(0xffffffffu, cnt);
    const size_t N = (size_t)n.N;
    float acc = 0.0f;
    for (int kb = 0; kb < kmax; kb += SW_ROWS) {
        float ps[SW_RPW], dc[SW_RPW];
        uint32_t q[SW_RPW];
#pragma unroll
        for (int j = 0; j < SW_RPW; j++) {
            int k = kb + warp + j * SW_WARPS;
            if (k < cnt) {
                size_t p = (size_t)k * N + d;
                ps[j] = n.psr[p];
                dc[j] = n.decay[p];
                q[j] = n.queue[p];
            }
        }
#pragma unroll
        for (int j = 0; j < SW_RPW; j++) {
            int k = kb + warp + j * SW_WARPS;
            if (k < cnt) {
                size_t p = (size_t)k * N + d;
                float v = ps[j];
                if (q[j] & bit) {
                    n.queue[p] = q[j] & ~bit;
                    if (SYN == 1) v = ds_hit(n, p, v, dc[j], t);
                    else v = v + n.W[p] / dc[j];
                }
                v = v * dc[j];
                n.psr[p] = v;
                stage[warp + j * SW_WARPS][lane] = v;
            }
        }
        __syncthreads();
        if (warp == 0) {
            int kend = min(SW_ROWS, cnt - kb);
            for (int kk = 0; kk < kend; kk++) acc = acc + stage[kk][lane];
        }
        __syncthreads();
    }
    if (warp == 0 && valid) n.sp[d] = acc;
    // the last tile to finish advances the step and clears the spike list
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(n.sweep_done, 1u);
        if (prev == gridDim.x - 1) {
            *n.step = t + 1;
            *n.nspikes = 0;
            *n.sweep_done = 0;
            __threadfence();
        }
    }
}

// ---- launchers -------------------------------------------------------------------------------
int fanout_blocks() { return 2 * 152; }

void launch_step(const NetDev &h, const NetDev *d_net, cudaStream_t s)
{
    if (h.noise_mode == 1)
        k_neurons_inject<<<1, 1024, 0, s>>>(d_net);
    else
        k_neurons_device<<<(h.N + 255) / 256, 256, 0, s>>>(d_net);
    k_fanout<<<fanout_blocks(), 256, 0, s>>>(d_net);
    if (h.syn_kind == 1)
        k_sweep<1><<<h.ntiles, SW_WARPS * 32, 0, s>>>(d_net);
    else
        k_sweep<0><<<h.ntiles, SW_WARPS * 32, 0, s>>>(d_net);
}

void launch_step_parts(const NetDev &h, const NetDev *d_net, cudaStream_t s, cudaEvent_t ev[4])
{
    cudaEventRecord(ev[0], s);
    if (h.noise_mode == 1)
        k_neurons_inject<<<1, 1024, 0, s>>>(d_net);
    else
        k_neurons_device<<<(h.N + 255) / 256, 256, 0, s>>>(d_net);
    cudaEventRecord(ev[1], s);
    k_fanout<<<fanout_blocks(), 256, 0, s>>>(d_net);
    cudaEventRecord(ev[2], s);
    if (h.syn_kind == 1)
        k_sweep<1><<<h.ntiles, SW_WARPS * 32, 0, s>>>(d_net);
    else
        k_sweep<0><<<h.ntiles, SW_WARPS * 32, 0, s>>>(d_net);
    cudaEventRecord(ev[3], s);
}

}  // namespace bg3
