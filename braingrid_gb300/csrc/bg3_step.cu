// Per-step kernels of the spiking hot path.
//
// One simulation step t on the network's stream:
//   k_deliver    (t)  spike arrival: for every delay class D, the neurons that fired at step
//                     t - D (spike ring) deliver to their outgoing synapses of that class; a hit
//                     runs AllDSSynapses::changePSR on the synapse (one 32-byte EvSlot).
//   k_sweep      (t)  per 32-dest tile, TMA-pipelined: psr *= decay for every slot row and the
//                     ordered sum into each dest's summation point; in device-noise mode the
//                     epilogue also integrates the tile's neurons for step t + 1 (they need only
//                     their own summation point), so a step costs two launches.
//   k_neurons_*  (t)  standalone neuron integration: the first step of a bg3_step call and every
//                     step in injected-noise mode (the noise order needs a scan over all neurons).
// In device-noise mode a call runs neurons(t0), k_deliver(t0), then (k_sweep(t), k_deliver(t+1))
// pairs, each delivery a programmatic dependent that overlaps the sweep before it, and a last
// unfused sweep.  The step counter: an unfused sweep advances it; after a fused sweep the next
// delivery does.  The delivery's own copy, dstep, which it reads before the sweep ahead of it
// ends, is advanced by that sweep's first tile as soon as the sweep's wait is over.
#include <cuda.h>
#include <algorithm>
#include <utility>
#include "bg3_internal.cuh"
#include "bg3_ptx.cuh"

namespace bg3 {

// The delivery pass of step t + 1 starts (programmatically) during the sweep of step t and reads
// its step from dstep before that sweep ends.  The sweep's first tile advances dstep once the
// delivery of step t has finished (after pdl_wait) and before any CTA of the sweep releases the
// next launch (the fence makes the store visible first; the caller's barrier keeps the other
// threads of the CTA from triggering before it).
__device__ __forceinline__ void dstep_advance(const NetDev &n, bool me, unsigned long long t)
{
    if (me) {
        *n.dstep = t + 1;
        __threadfence();
    }
}

// The batched kernels find their network's descriptor in global memory (nets[k]); read there
// field by field, every field is a dependent load (the plain kernels take theirs as a kernel
// parameter).  Each block serves one network and first copies its descriptor into shared
// memory with all its threads, 16 bytes each.
static_assert(sizeof(NetDev) % 16 == 0, "descriptor copied in 16-byte words");
__device__ __forceinline__ void block_copy_desc(NetDev *dst, const NetDev *src)
{
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (int k = threadIdx.x; k < (int)(sizeof(NetDev) / 16); k += blockDim.x) d4[k] = s4[k];
    __syncthreads();
}

// Spiking neurons whose spikes arrive at step t (one work item of the delivery pass per neuron
// and delay class), from the spike ring.  A pass with at most DLV_LIGHT_ITEMS of them is light:
// it starts during the TMA sweep before it and lets the sweep after it start early.  A heavy pass
// does neither: launched early it would sit on SMs whose shared memory / L1 split is set for the
// TMA sweep, and run its random accesses with little L1 (measured: 161 us per step instead of 95
// at ~1,000 spiking neurons per step).  The thin sweeps hold no shared memory and always release.
constexpr int DLV_LIGHT_ITEMS = 128;
// Whether the delivery of step t is light, computed by a whole warp (one delay class per lane).
// The spikes it counts are at least one step old, so their counts are final during the sweep of
// step t - 1.
// Lanes 1-31 of a warp (lane 0 is busy elsewhere), one delay class per lane.
__device__ __forceinline__ bool delivery_light(const NetDev &n, unsigned long long t)
{
    const int c = (int)(threadIdx.x & 31) - 1;
    int m = 0;
    if (c < n.n_delays) {
        const int D = n.ltab[c];
        if (D > 0 && (unsigned long long)D <= t)
            m = min(n.ring_n[(t - (unsigned long long)D) & (BG3_RING - 1)], n.N);
    }
    return __reduce_add_sync(0xfffffffeu, m) <= DLV_LIGHT_ITEMS;
}
// The other warps of a TMA sweep CTA act on that decision when they see it (a flag in shared
// memory: -1 undecided, 0 heavy, 1 light) without waiting for it; returns true once decided.
__device__ __forceinline__ bool release_if_light(const int *flag)
{
    const int f = *(const volatile int *)flag;
    if (f < 0) return false;
    if (f == 1) pdl_trigger();
    return true;
}

// ---- standalone neuron kernels ---------------------------------------------------------------
// Device-noise mode: one N(0,1) draw per neuron per step, keyed by (seed, step, neuron).
__global__ void __launch_bounds__(256) k_neurons_device(const __grid_constant__ NetDev n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long t = *n.step;
    bool fired = false;
    if (i < n.N) {
        NeuronIn x;
        neuron_load(n, i, x);
        const int br = neuron_branch(x);
        float noise = (br == BR_INTEGRATE) ? normal_device(n.noise_seed, t, i) : 0.0f;
        fired = neuron_apply(n, i, x, br, input_apply(n, i, x, t, n.sp[i]), noise, t,
                                 izh_mode(n, i));
        n.sp[i] = 0.0f;
    }
    ring_push(n, t, fired, i);
}

// Injected-noise mode: the reference CPU draws one value per integrating neuron while walking
// neurons from N-1 down to 0 (Neurons/AllSpikingNeurons.cpp:104).  One CTA walks the neurons in
// chunks of 1024 from the top; a block scan of the "integrates" flags gives each neuron the
// number of integrating neurons above it, i.e. its position in the stream.
__global__ void __launch_bounds__(1024) k_neurons_inject(const __grid_constant__ NetDev n)
{
    __shared__ int warp_tot[32];
    __shared__ long long s_running;
    unsigned long long t = *n.step;
    unsigned long long cursor = *n.noise_cursor;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_running = 0;
    __syncthreads();
    for (int top = n.N - 1; top >= 0; top -= 1024) {
        int i = top - (int)threadIdx.x;
        NeuronIn x;
        if (i >= 0) neuron_load(n, i, x);
        int br = (i >= 0) ? neuron_branch(x) : BR_REFRACTORY;
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
                else set_err(n, ERR_NOISE_EXHAUSTED);
            }
            fired = neuron_apply(n, i, x, br, input_apply(n, i, x, t, n.sp[i]), noise, t,
                                 izh_mode(n, i));
            n.sp[i] = 0.0f;
        }
        ring_push(n, t, fired, i);
        __syncthreads();
        if (threadIdx.x == 1023) s_running = running + warp_tot[31] + __popc(m);
        __syncthreads();
    }
    if (threadIdx.x == 0) *n.noise_cursor = cursor + (unsigned long long)s_running;
}

// Injected-noise mode for larger networks: the same stream positions from two passes over
// 1024-neuron chunks taken from the top (chunk b holds neurons N-1-1024b down to N-1024(b+1)).
// The count pass stores each chunk's number of integrating neurons, and the cursor at the start
// of the step, in the map builder's scratch (outFill, unused between map builds); the apply
// pass gives each neuron the integrating neurons of the chunks above it plus those above it in
// its own chunk, and advances the cursor by the step's total.
static const int INJ_CHUNK = 1024;

__global__ void __launch_bounds__(1024) k_neurons_inject_count(const __grid_constant__ NetDev n)
{
    const int b = blockIdx.x;
    const int i = n.N - 1 - b * INJ_CHUNK - (int)threadIdx.x;
    bool integ = false;
    if (i >= 0) {
        NeuronIn x;
        neuron_load(n, i, x);
        integ = neuron_branch(x) == BR_INTEGRATE;
    }
    const int c = __syncthreads_count(integ);
    if (threadIdx.x == 0) {
        n.outFill[b] = (uint32_t)c;
        if (b == 0) {
            const unsigned long long cur = *n.noise_cursor;
            n.outFill[gridDim.x] = (uint32_t)cur;
            n.outFill[gridDim.x + 1] = (uint32_t)(cur >> 32);
        }
    }
}

__global__ void __launch_bounds__(1024) k_neurons_inject_apply(const __grid_constant__ NetDev n)
{
    __shared__ int warp_tot[32];
    __shared__ long long s_above;
    const int b = blockIdx.x, nb = gridDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long t = *n.step;
    const unsigned long long cursor =
        (unsigned long long)n.outFill[nb] | ((unsigned long long)n.outFill[nb + 1] << 32);
    if (warp == 0) {
        long long a = 0;
        for (int k = lane; k < b; k += 32) a += n.outFill[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) s_above = a;
    }
    const int i = n.N - 1 - b * INJ_CHUNK - (int)threadIdx.x;
    NeuronIn x;
    if (i >= 0) neuron_load(n, i, x);
    const int br = (i >= 0) ? neuron_branch(x) : BR_REFRACTORY;
    const bool integ = (i >= 0) && br == BR_INTEGRATE;
    const unsigned m = __ballot_sync(0xffffffffu, integ);
    const int in_warp = __popc(m & ((1u << lane) - 1));
    if (lane == 31) warp_tot[warp] = __popc(m);
    __syncthreads();
    if (warp == 0) {
        const int v = warp_tot[lane];
        int y = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += z;
        }
        warp_tot[lane] = y - v;  // exclusive prefix of warp totals
    }
    __syncthreads();
    bool fired = false;
    if (i >= 0) {
        float noise = 0.0f;
        if (integ) {
            const long long pos = (long long)cursor + s_above + warp_tot[warp] + in_warp;
            if (pos < n.noise_len) noise = n.noise_buf[pos];
            else set_err(n, ERR_NOISE_EXHAUSTED);
        }
        fired = neuron_apply(n, i, x, br, input_apply(n, i, x, t, n.sp[i]), noise, t,
                                 izh_mode(n, i));
        n.sp[i] = 0.0f;
    }
    ring_push(n, t, fired, i);
    if (b == 0 && threadIdx.x == 0) {
        long long tot = 0;
        for (int k = 0; k < nb; k++) tot += n.outFill[k];
        *n.noise_cursor = cursor + (unsigned long long)tot;
    }
}

// ---- STDP ------------------------------------------------------------------------------------
// AllSTDPSynapses::advanceSynapse / stdpLearning (Synapses/AllSTDPSynapses.cpp:283-472) and the
// device form advanceSTDPSynapsesDevice (AllSynapsesDeviceFuncs_d.cu:100-380).  The only
// difference between the two builds is the type of the spike times in the interval arithmetic:
// uint64_t on the host (a pre-spike walk interval wraps to a huge positive value), int64_t on
// the device.  Each float / double operation rounds as in the reference; the exp factors come
// from the host library's tables.

// getSpikeHistory (Neurons/AllSpikingNeurons.cpp:182-188) for off in [-max_spikes, -1];
// co = spikeCount + spikeCountOffset.
__device__ __forceinline__ unsigned long long hist_at(const NetDev &n, int i, int co, int off)
{
    const int x = (co + n.max_spikes + off) % n.max_spikes;
    return n.history[(size_t)i * n.max_spikes + x];
}

// W^mu with mu = 0, the only exponent a network accepts (set_stdp_type refuses others)
__device__ __forceinline__ float pow_mu(float, float) { return 1.0f; }

// One stdpLearning call with delta = dk steps (dk the signed interval; 0 when not a small count),
// in two parts.  stdp_inc: the weight change, which W does not enter (W^mu = 1): false when delta
// lies within the gap (W unchanged, no clamp), else epost * epre * dw in double.  stdp_apply: W
// plus that change, rounded to float, then the clamps.  So the walks below can find a walk's
// changes before W is known and apply them in order after.
__device__ __forceinline__ bool stdp_inc(const StdpConst &c, float delta, float epost, float epre,
                                         long long dk, double &inc)
{
    const double d = (double)delta;
    float dw;
    if (d < (double)(-c.gap)) {
        const double e = (dk < 0 && -dk < (long long)c.dlen_neg) ? c.dneg[-dk] : exp(d / (double)c.tauneg);
        dw = (float)((double)(pow_mu(0.0f, c.muneg) * c.Aneg) * e);
    } else if (d > (double)c.gap) {
        const double e = (dk > 0 && dk < (long long)c.dlen_pos) ? c.dpos[dk] : exp(-d / (double)c.taupos);
        dw = (float)((double)(pow_mu(0.0f, c.mupos) * c.Apos) * e);
    } else {
        return false;
    }
    inc = (double)epost * (double)epre * (double)dw;
    return true;
}
__device__ __forceinline__ float stdp_apply(const StdpConst &c, float W, double inc)
{
    W = (float)((double)W + inc);
    if ((c.Wex < 0.0f && W > 0.0f) || (c.Wex > 0.0f && W < 0.0f)) W = 0.0f;
    if (fabsf(W) > fabsf(c.Wex)) W = c.Wex;
    return W;
}
__device__ __forceinline__ float stdp_learn(const StdpConst &c, float W, float delta, float epost,
                                            float epre, long long dk)
{
    double inc;
    return stdp_inc(c, delta, epost, epre, dk, inc) ? stdp_apply(c, W, inc) : W;
}

// A neuron's history entries -1 .. -4 read together (those of them that exist: off >= -ms), so
// that a walk's first steps do not wait on one load each; hist_get takes the rest from memory.
struct Hist4 {
    unsigned long long h0, h1, h2, h3;
};
__device__ __forceinline__ void hist_load4(const NetDev &n, int i, int co, Hist4 &c)
{
    const int ms = n.max_spikes;
    c.h0 = hist_at(n, i, co, -1);  // max_spikes >= 1
    c.h1 = ms >= 2 ? hist_at(n, i, co, -2) : BG3_ULONG_MAX;
    c.h2 = ms >= 3 ? hist_at(n, i, co, -3) : BG3_ULONG_MAX;
    c.h3 = ms >= 4 ? hist_at(n, i, co, -4) : BG3_ULONG_MAX;
}
// entry off (-ms <= off <= -1)
__device__ __forceinline__ unsigned long long hist_get(const NetDev &n, int i, int co, int off,
                                                       const Hist4 &c)
{
    return off == -1 ? c.h0 : off == -2 ? c.h1 : off == -3 ? c.h2 : off == -4 ? c.h3
                                                                    : hist_at(n, i, co, off);
}

// The fPre branch: a spike from pre arrives at the synapse onto post at step t.  Returns W.
__device__ float stdp_pre(const NetDev &n, const StdpConst &c, float W, int pre, int post,
                          unsigned long long t)
{
    const int ms = n.max_spikes;
    const int cpost = n.spikeCount[post] + n.spikeCountOffset[post];
    if (!n.stdp_signed) {
        // Every interval (spikeHistory - step) wraps to ~1.8e15 s (or is 0 at step t): each
        // learning call potentiates by exactly zero and applies the clamps, so only whether one
        // happens matters: the walk runs while entries -k and -(k+1) are valid.
        const unsigned long long h1 = hist_at(n, post, cpost, -1);
        const unsigned long long h2 = hist_at(n, post, cpost, -2);
        if (hist_at(n, post, cpost, -ms) != BG3_ULONG_MAX) set_err(n, ERR_STDP_RING);
        bool learn;
        if (c.useFD) {
            const unsigned long long h3 = hist_at(n, post, cpost, -3);
            learn = h1 != BG3_ULONG_MAX && h2 != BG3_ULONG_MAX && (h1 != t || h3 != BG3_ULONG_MAX);
        } else {
            learn = h1 != BG3_ULONG_MAX && (h1 != t || h2 != BG3_ULONG_MAX);
        }
        if (learn) {
            // potentiation by (float)(x * exp(-huge)) = +-0; epost * epre >= 0 keeps dw's sign
            const float dw = (float)((double)(pow_mu(c.Wex - W, c.mupos) * c.Apos) * 0.0);
            W = (float)((double)W + (double)dw);
            if ((c.Wex < 0.0f && W > 0.0f) || (c.Wex > 0.0f && W < 0.0f)) W = 0.0f;
            if (fabsf(W) > fabsf(c.Wex)) W = c.Wex;
        }
        return W;
    }
    const int cpre = n.spikeCount[pre] + n.spikeCountOffset[pre];
    Hist4 hp;
    hist_load4(n, post, cpost, hp);
    const unsigned long long sp2 = hist_at(n, pre, cpre, -2);
    float epre = 1.0f;
    if ((long long)sp2 > 0 && c.useFD)
        epre = (float)(1.0 - (double)exp_interval(n, t - sp2, true, c.tauspre));
    for (int off = -1;; --off) {
        if (off < -ms) { set_err(n, ERR_STDP_RING); break; }
        const unsigned long long sh = hist_get(n, post, cpost, off, hp);
        if (sh == BG3_ULONG_MAX) break;
        const long long dk = (long long)(sh - t);
        const float delta = (float)dk * n.dt;
        if ((double)delta <= -3.0 * (double)c.tauneg) break;
        float epost = 1.0f;
        if (c.useFD) {
            if (off - 1 < -ms) { set_err(n, ERR_STDP_RING); break; }
            const unsigned long long sh2 = hist_get(n, post, cpost, off - 1, hp);
            if (sh2 == BG3_ULONG_MAX) break;
            epost = (float)(1.0 - (double)exp_interval(n, sh - sh2, true, c.tauspost));
        }
        W = stdp_learn(c, W, delta, epost, epre, dk);
    }
    return W;
}

// The fPost branch: post fired at step t; walk the pre history (both builds agree here).  The
// walk does not depend on W, so it runs in two parts: stdp_post_prep reads everything it needs
// (spike counts, histories, tables) and makes its first four steps, keeping their weight changes;
// stdp_post_finish applies them to W and makes any further steps.  The post-spike pass calls
// the first before its wait on the delivery of the same step (the one writer of W there).
constexpr int POST_STEPS = 4;
struct PostPrep {
    double inc0, inc1, inc2, inc3;  // the changes of steps 1 .. 4 (those with a bit in mask)
    float epost;
    int cpre;
    int mask;                       // bit k: step k + 1 changed W
    int next;                       // 0: the walk has ended; else the entry it continues from
};
__device__ __forceinline__ void stdp_post_prep(const NetDev &n, const StdpConst &c, int pre,
                                               int post, int total_delay, unsigned long long t,
                                               PostPrep &q)
{
    const int ms = n.max_spikes;
    const bool sgn = n.stdp_signed != 0;
    const int cpost = n.spikeCount[post] + n.spikeCountOffset[post];
    const int cpre = n.spikeCount[pre] + n.spikeCountOffset[pre];
    const unsigned long long q2 = hist_at(n, post, cpost, -2);
    Hist4 hp;
    hist_load4(n, pre, cpre, hp);
    float epost = 1.0f;
    const bool ok = sgn ? ((long long)q2 > 0) : (q2 != BG3_ULONG_MAX);
    if (ok && c.useFD) epost = (float)(1.0 - (double)exp_interval(n, t - q2, sgn, c.tauspost));
    q.epost = epost;
    q.cpre = cpre;
    q.mask = 0;
    q.next = 0;
    q.inc0 = q.inc1 = q.inc2 = q.inc3 = 0.0;
#pragma unroll
    for (int k = 0; k < POST_STEPS; k++) {
        const int off = -1 - k;
        if (off < -ms) { set_err(n, ERR_STDP_RING); return; }
        const unsigned long long sh = hist_get(n, pre, cpre, off, hp);
        if (sh == BG3_ULONG_MAX) return;
        const unsigned long long dd = t - (unsigned long long)(long long)total_delay - sh;
        const float delta = (sgn ? (float)(long long)dd : (float)dd) * n.dt;
        if (delta <= 0.0f || (double)delta >= 3.0 * (double)c.taupos) return;
        float epre = 1.0f;
        if (c.useFD) {
            if (off - 1 < -ms) { set_err(n, ERR_STDP_RING); return; }
            const unsigned long long sh2 = hist_get(n, pre, cpre, off - 1, hp);
            if (sh2 == BG3_ULONG_MAX) return;
            epre = (float)(1.0 - (double)exp_interval(n, sh - sh2, sgn, c.tauspre));
        }
        double inc;
        if (stdp_inc(c, delta, epost, epre, (long long)dd, inc)) {
            q.mask |= 1 << k;
            if (k == 0) q.inc0 = inc;
            else if (k == 1) q.inc1 = inc;
            else if (k == 2) q.inc2 = inc;
            else q.inc3 = inc;
        }
    }
    q.next = -1 - POST_STEPS;
}
__device__ __forceinline__ float stdp_post_finish(const NetDev &n, const StdpConst &c, float W,
                                                  int pre, int total_delay, unsigned long long t,
                                                  const PostPrep &q)
{
    if (q.mask & 1) W = stdp_apply(c, W, q.inc0);
    if (q.mask & 2) W = stdp_apply(c, W, q.inc1);
    if (q.mask & 4) W = stdp_apply(c, W, q.inc2);
    if (q.mask & 8) W = stdp_apply(c, W, q.inc3);
    if (!q.next) return W;
    const int ms = n.max_spikes;
    const bool sgn = n.stdp_signed != 0;
    for (int off = q.next;; --off) {
        if (off < -ms) { set_err(n, ERR_STDP_RING); break; }
        const unsigned long long sh = hist_at(n, pre, q.cpre, off);
        if (sh == BG3_ULONG_MAX) break;
        const unsigned long long dd = t - (unsigned long long)(long long)total_delay - sh;
        const float delta = (sgn ? (float)(long long)dd : (float)dd) * n.dt;
        if (delta <= 0.0f || (double)delta >= 3.0 * (double)c.taupos) break;
        float epre = 1.0f;
        if (c.useFD) {
            if (off - 1 < -ms) { set_err(n, ERR_STDP_RING); break; }
            const unsigned long long sh2 = hist_at(n, pre, q.cpre, off - 1);
            if (sh2 == BG3_ULONG_MAX) break;
            epre = (float)(1.0 - (double)exp_interval(n, sh - sh2, sgn, c.tauspre));
        }
        W = stdp_learn(c, W, delta, q.epost, epre, (long long)dd);
    }
    return W;
}
__device__ float stdp_post(const NetDev &n, const StdpConst &c, float W, int pre, int post,
                           int total_delay, unsigned long long t)
{
    PostPrep q;
    stdp_post_prep(n, c, pre, post, total_delay, t, q);
    return stdp_post_finish(n, c, W, pre, total_delay, t, q);
}

// ---- spike arrival ---------------------------------------------------------------------------
// Arrival of a spike emitted at step tf on plane slot p at step t: the isSpikeQueue hit of
// AllSpikingSynapses::advanceSynapse (Synapses/AllSpikingSynapses.cpp:297-319) followed by
// changePSR — AllDSSynapses.cpp:227-247 for DS and dynamic STDP, AllSpikingSynapses.cpp:327-334
// for spiking and STDP synapses; the STDP kinds (2, 3) first run the fPre learning walk.
// The STDP kinds' arrival in two parts: stdp_hit_prep reads what passes before the previous sweep
// wrote (the event slot; the DS update of u and r for dynamic STDP), stdp_hit_finish what that
// sweep writes (psr; the post neuron's spikes, which the fPre walk reads) and stores.  The
// delivery pass calls the first before its wait on that sweep.
struct StdpHit {
    EvSlot e;
    const StdpConst *c;
    float dec, u, r;
    int d;
    bool ok;
};
template <int SYN>
__device__ __forceinline__ void stdp_hit_prep(const NetDev &n, uint32_t p, uint32_t tf, uint32_t t,
                                              StdpHit &h)
{
    h.e = n.ev[p];
    h.ok = (int32_t)(tf - h.e.born) >= 0;  // else the synapse did not exist when the spike left
    if (!h.ok) return;
    h.dec = n.dtab[h.e.dcls];
    h.c = &n.stdp[n.stype[p]];
    int k;
    pos_slot(p, n.Mq, k, h.d);
    h.u = h.e.u;
    h.r = h.e.r;
    if (SYN == 3 && h.e.last != BG3_NO_SPIKE32) ds_update(n, h.e, t - h.e.last, h.u, h.r);
}
template <int SYN>
__device__ __forceinline__ void stdp_hit_finish(const NetDev &n, uint32_t p, unsigned long long t64,
                                                int src, const StdpHit &h)
{
    if (!h.ok) return;
    float ps = n.psr[p];
    const float W = stdp_pre(n, *h.c, h.e.W, src, h.d, t64);
    n.ev[p].W = W;
    if (SYN == 3) {
        ps = ps + ((W / h.dec) * h.u * h.r);
        EvSlot *q = &n.ev[p];
        q->u = h.u;
        q->r = h.r;
        q->last = (uint32_t)t64;
    } else {
        ps = ps + W / h.dec;
    }
    n.psr[p] = ps;
}

template <int SYN>
__device__ __forceinline__ void deliver_hit(const NetDev &n, uint32_t p, uint32_t tf,
                                            unsigned long long t64, int src)
{
    if (SYN >= 2) {
        StdpHit h;
        stdp_hit_prep<SYN>(n, p, tf, (uint32_t)t64, h);
        stdp_hit_finish<SYN>(n, p, t64, src, h);
        return;
    }
    const uint32_t t = (uint32_t)t64;
    EvSlot e = n.ev[p];
    if ((int32_t)(tf - e.born) < 0) return;  // the synapse did not exist when the spike left
    float dec = n.dtab[e.dcls];
    float ps = n.psr[p];
    if (SYN >= 2) {
        int k, d;
        pos_slot(p, n.Mq, k, d);
        e.W = stdp_pre(n, n.stdp[n.stype[p]], e.W, src, d, t64);
        n.ev[p].W = e.W;
    }
    if (SYN == 1 || SYN == 3) {
        float u = e.u, r = e.r;
        if (e.last != BG3_NO_SPIKE32) ds_update(n, e, t - e.last, u, r);
        ps = ps + ((e.W / dec) * u * r);
        EvSlot *q = &n.ev[p];
        q->u = u;
        q->r = r;
        q->last = t;
    } else {
        ps = ps + e.W / dec;
    }
    n.psr[p] = ps;
}

// Spike arrivals of one step.  The work items are (delay class c, neuron that fired at t - D_c)
// pairs; each item's outgoing synapses of the class are cut into chunks of DLV_CHUNK that one warp
// delivers, four per lane with their loads issued together.  A block takes up to DLV_GROUP items
// at a time (fewer when the step has few spikes, so that they spread over the blocks), scans their
// chunk counts and lets its warps take the chunks in turn; so a burst of high-fan-out neurons
// keeps every warp of the grid busy instead of one warp per neuron walking its synapses 32 at a
// time.  Each synapse has one source, which fires at most once per step, so no two lanes touch
// one slot.  Block 0 also clears ring slot t + 1 for the next neuron pass.
//
// Spiking and DS synapses: the pass starts while the previous sweep is still running (its launch
// is a programmatic dependent of that sweep).  Everything an arrival needs except psr depends only
// on spikes at least one step old (written by earlier sweeps), the outgoing map and the synapse's
// event slot (written only by earlier delivery passes, which have finished: a sweep releases its
// dependent only after its own wait on the delivery before it).  So the item table, the slot
// positions, the DS update of u, r and the last-spike step, and the psr increment are done first;
// pdl_wait() then waits for the sweep, and only the psr read-modify-write comes after it.  The
// step comes from the pass's own counter (dstep), since the sweep advances `step` at its end.
// STDP kinds prepare the same way and wait before their pre-spike walks, which read the post
// neurons' latest spikes.
constexpr int DLV_CHUNK = 128;
constexpr int DLV_GROUP = 32;

struct Arrivals {
    uint32_t p[4];
    float add[4];
    bool ok[4];
};

// Event-state part of the arrivals of one chunk (lane's four synapses): slot positions, the
// isSpikeQueue/changePSR arithmetic of the spiking and DS synapses up to the psr increment
// (AllSpikingSynapses.cpp:327-334, AllDSSynapses.cpp:227-247), and the event-slot update.
template <int SYN>
__device__ __forceinline__ void deliver_prep(const NetDev &n, uint32_t b, uint32_t k, uint32_t base,
                                             uint32_t tf, uint32_t t, int lane, Arrivals &a)
{
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const uint32_t j = base + (uint32_t)lane + 32u * u;
        a.ok[u] = j < k;
        a.p[u] = a.ok[u] ? n.outMap[b + j] : 0u;
    }
    EvSlot e[4];
#pragma unroll
    for (int u = 0; u < 4; u++)
        if (a.ok[u]) e[u] = n.ev[a.p[u]];
#pragma unroll
    for (int u = 0; u < 4; u++) a.ok[u] = a.ok[u] && (int32_t)(tf - e[u].born) >= 0;
    float xr[4], xu[4], dec[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
        if (!a.ok[u]) continue;
        dec[u] = n.dtab[e[u].dcls];
        if (SYN == 1 && e[u].last != BG3_NO_SPIKE32) {
            const uint32_t ki = t - e[u].last;
            const int c = e[u].pcls;
            xr[u] = exp_tab(n, n.p_xD[c], ki, n.p_D[c]);
            xu[u] = exp_tab(n, n.p_xF[c], ki, n.p_F[c]);
        }
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
        if (!a.ok[u]) continue;
        if (SYN == 1) {
            float uu = e[u].u, r = e[u].r;
            if (e[u].last != BG3_NO_SPIKE32) {
                const float U = n.p_U[e[u].pcls];
                r = 1.0f + (r * (1.0f - uu) - 1.0f) * xr[u];
                uu = U + uu * (1.0f - U) * xu[u];
            }
            a.add[u] = (e[u].W / dec[u]) * uu * r;
            EvSlot *w = &n.ev[a.p[u]];
            w->u = uu;
            w->r = r;
            w->last = t;
        } else {
            a.add[u] = e[u].W / dec[u];
        }
    }
}

// psr part: psr += increment (the four loads issued together).
__device__ __forceinline__ void deliver_apply(const NetDev &n, const Arrivals &a)
{
    float ps[4];
#pragma unroll
    for (int u = 0; u < 4; u++)
        if (a.ok[u]) ps[u] = n.psr[a.p[u]];
#pragma unroll
    for (int u = 0; u < 4; u++)
        if (a.ok[u]) n.psr[a.p[u]] = ps[u] + a.add[u];
}

template <int SYN>
__device__ __forceinline__ void deliver_net(const NetDev &n, int bid, int nb, bool early_cfg)
{
    __shared__ uint32_t s_pref[DLV_GROUP], s_beg[DLV_GROUP], s_cnt[DLV_GROUP], s_tf[DLV_GROUP];
    __shared__ int32_t s_src[DLV_GROUP];
    __shared__ int s_moff[BG3_MAX_DELAYS + 1];
    bool waited = false;
    const unsigned long long t = *n.dstep;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (threadIdx.x == 0) {
        int off = 0;
        for (int c = 0; c < n.n_delays; c++) {
            s_moff[c] = off;
            const int D = n.ltab[c];
            if (D > 0 && (unsigned long long)D <= t)
                off += min(n.ring_n[(t - (unsigned long long)D) & (BG3_RING - 1)], n.N);
        }
        s_moff[n.n_delays] = off;
    }
    __syncthreads();
    const int M = s_moff[n.n_delays];
    // Early start pays while the step's arrivals are few (light, see DLV_LIGHT_ITEMS).  A heavy
    // pass waits first, and does not release the next sweep early either: that sweep's CTAs
    // would hold the SMs' shared memory, and so the L1 its random accesses need.
    const bool light = M <= DLV_LIGHT_ITEMS;
    if (!waited && !(early_cfg && light)) {
        pdl_wait();
        if (light) pdl_trigger();
        waited = true;
    }
    const int G = max(1, min(DLV_GROUP, (M + nb - 1) / nb));
    for (int g0 = bid * G; g0 < M; g0 += nb * G) {
        const int items = min(G, M - g0);
        if (warp == 0) {
            uint32_t chunks = 0;
            if (lane < items) {
                const int idx = g0 + lane;
                int c = 0;
                while (idx >= s_moff[c + 1]) c++;
                const unsigned long long tf = t - (unsigned long long)n.ltab[c];
                const int slot = (int)(tf & (BG3_RING - 1));
                const int i = n.ring[(size_t)slot * n.N + (idx - s_moff[c])];
                const size_t ci = (size_t)c * n.N + i;
                const uint32_t k = n.outCount[ci];
                s_beg[lane] = n.outBegin[ci];
                s_cnt[lane] = k;
                s_src[lane] = i;
                s_tf[lane] = (uint32_t)tf;
                chunks = (k + DLV_CHUNK - 1) / DLV_CHUNK;
            }
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, chunks, o);
                if (lane >= o) chunks += v;
            }
            s_pref[lane] = chunks;
        }
        __syncthreads();
        const uint32_t total = s_pref[31];
        for (uint32_t ch = warp; ch < total; ch += nwarps) {
            int lo = 0, hi = items - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (s_pref[mid] > ch) hi = mid;
                else lo = mid + 1;
            }
            const uint32_t first = lo ? s_pref[lo - 1] : 0u;
            const uint32_t base = (ch - first) * DLV_CHUNK;
            if (SYN >= 2) {  // STDP: the pre-spike walks go one synapse at a time
                const uint32_t end = min(s_cnt[lo], base + (uint32_t)DLV_CHUNK);
                for (uint32_t j = base + lane; j < end; j += 32) {
                    const uint32_t p = n.outMap[s_beg[lo] + j];
                    StdpHit h;
                    stdp_hit_prep<SYN>(n, p, s_tf[lo], (uint32_t)t, h);
                    if (!waited) {
                        pdl_wait();  // the walks read the post neurons' spikes of the sweep before
                        pdl_trigger();
                        waited = true;
                    }
                    stdp_hit_finish<SYN>(n, p, t, s_src[lo], h);
                }
            } else {
                Arrivals a;
                deliver_prep<SYN>(n, s_beg[lo], s_cnt[lo], base, s_tf[lo], (uint32_t)t, lane, a);
                if (!waited) {
                    pdl_wait();  // the previous sweep has finished with psr
                    pdl_trigger();
                    waited = true;
                }
                deliver_apply(n, a);
            }
        }
        __syncthreads();
    }
    if (!waited) {
        pdl_wait();
        pdl_trigger();
    }
    if (threadIdx.x == 0) {
        if (bid == 0) {
            // the step counter reaches t here: a fused sweep before this pass left it at t - 1
            const unsigned long long st = *n.step;
            if (st + 1 == t) {
                *n.step = t;
                if (t >= 0xffffff00ull) set_err(n, ERR_STEP_RANGE);
            } else if (st != t) {
                set_err(n, ERR_STEP_SYNC);  // internal check
            }
            n.ring_n[(t + 1) & (BG3_RING - 1)] = 0;
        }
    }
}

template <int SYN>
__global__ void __launch_bounds__(256) k_deliver(const __grid_constant__ NetDev n, int early)
{
    deliver_net<SYN>(n, blockIdx.x, gridDim.x, early != 0);
}

// Batched form: grid.y indexes the network, so the networks' delivery passes run side by side.
template <int SYN>
__global__ void __launch_bounds__(256) k_deliver_batch(const NetDev *nets, int early)
{
    __shared__ __align__(16) NetDev s_net;
    block_copy_desc(&s_net, nets + blockIdx.y);
    deliver_net<SYN>(s_net, blockIdx.x, gridDim.x, early != 0);
}

// The fPost branch (AllSTDPSynapses.cpp:368-418) for every in-use synapse onto a neuron that
// fired at step t (postSpikeHit marks them all, AllSpikingNeurons.cpp:128-138, with
// total_delayPost 0, so the post queue is read in the same step).  One warp per fired neuron,
// one lane per incoming synapse; runs after the arrivals of step t (the fPre branch comes first
// in the reference) and before the sweep.
//
// The pass is a programmatic dependent of the delivery, which launches it only once the sweep
// before has finished: the step (the delivery's own counter, dstep, which only that sweep
// advances), the fired neurons, every spike count and history are final when it starts; only W
// is written by the delivery.  So each synapse's walk is prepared (stdp_post_prep) before the
// wait on the delivery, and W is read, learned and stored after it.
__device__ __forceinline__ void stdp_post_net(const NetDev &n, int gw, int nw)
{
    const unsigned long long t = *n.dstep;
    const int slot = (int)(t & (BG3_RING - 1));
    const int m = min(n.ring_n[slot], n.N);
    const int32_t *ids = n.ring + (size_t)slot * n.N;
    const int lane = threadIdx.x & 31;
    bool waited = false;
    for (int s = gw; s < m; s += nw) {
        const int d = ids[s];
        const int cnt = (int)n.count[d];
        for (int k = lane; k < cnt; k += 32) {
            const size_t p = slot_pos(k, d, n.Mq);
            const StdpConst &c = n.stdp[n.stype[p]];
            const int pre = n.src[p];
            const int delay = n.ltab[n.lcls[p]];
            PostPrep q;
            stdp_post_prep(n, c, pre, d, delay, t, q);
            if (!waited) {
                pdl_wait();
                pdl_trigger();
                waited = true;
            }
            n.ev[p].W = stdp_post_finish(n, c, n.ev[p].W, pre, delay, t, q);
        }
    }
    if (!waited) {
        pdl_wait();
        pdl_trigger();
    }
}

__global__ void __launch_bounds__(256) k_stdp_post(const __grid_constant__ NetDev n)
{
    stdp_post_net(n, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5);
}

__global__ void __launch_bounds__(256) k_stdp_post_batch(const NetDev *nets)
{
    __shared__ __align__(16) NetDev s_net;
    block_copy_desc(&s_net, nets + blockIdx.y);
    stdp_post_net(s_net, (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                  (gridDim.x * blockDim.x) >> 5);
}

// Batched standalone neuron pass (device noise): grid.y indexes the network.
__global__ void __launch_bounds__(256) k_neurons_device_batch(const NetDev *nets)
{
    __shared__ __align__(16) NetDev s_net;
    block_copy_desc(&s_net, nets + blockIdx.y);
    const NetDev &n = s_net;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x * blockDim.x >= (unsigned)n.N) return;  // whole warp-aligned block beyond N
    unsigned long long t = *n.step;
    bool fired = false;
    if (i < n.N) {
        NeuronIn x;
        neuron_load(n, i, x);
        const int br = neuron_branch(x);
        float noise = (br == BR_INTEGRATE) ? normal_device(n.noise_seed, t, i) : 0.0f;
        fired = neuron_apply(n, i, x, br, input_apply(n, i, x, t, n.sp[i]), noise, t,
                                 izh_mode(n, i));
        n.sp[i] = 0.0f;
    }
    ring_push(n, t, fired, i);
}

// ---- synapse sweep ---------------------------------------------------------------------------
constexpr int SW_DESTS = 32;   // dests per tile (one per lane)
constexpr int SW_ROWS = 64;    // slot rows per TMA chunk
constexpr int SW_QUADS = SW_ROWS / 4;

constexpr int SW_SCALE_WARPS = 4;
constexpr int SW_THREADS = 32 * (2 + SW_SCALE_WARPS);
// a chunk of a D-dest tile: 64 rows of psr and of the decay class
__host__ __device__ constexpr uint32_t sw_psr_bytes(int D) { return (uint32_t)(SW_ROWS * D * 4); }
// a chunk: psr [16 quads][D] float4, then classes [16 quads][D] 16-bit (four 4-bit codes)
__host__ __device__ constexpr uint32_t sw_chunk_bytes(int D) { return (uint32_t)(SW_ROWS * D * 4 + SW_QUADS * D * 2); }
// dynamic shared memory: stages (psr | class), decay table, barriers; +128 for alignment
// ST chunks in flight per D-dest tile; for D = 32: 4 (42 KB, five CTAs per SM), 6 (63 KB,
// three), 8 (83 KB, two); D = 16 halves the stages
constexpr size_t sw_smem(int st, int D)
{
    return (size_t)st * sw_chunk_bytes(D) + BG3_MAX_DCLS * 4 + 3 * (size_t)st * 8 + 16 + 128;
}

// AllSpikingSynapses::advanceSynapse's "psr *= decay" for every in-use synapse, and the
// summation of AllSynapses::advanceSynapses (Synapses/AllSynapses.cpp:325-331):
// sp[d] = ((0 + psr_0) + psr_1) + ... in slot order, the reference's accumulation order.
//
// One CTA per tile of 32 dests, three warp roles over a 6-stage shared-memory ring of chunks
// (64 rows x 32 dests = 16 row quads of psr and of the decay class):
//   warp 0      lane 0 issues the 2-D TMA loads of each chunk (mbarrier full[s]);
//   warps 1-4   scale 4 quads each in place, psr *= decay[class] (then arrive on scaled[s]);
//   warp 5      adds the 64 rows of each chunk in row order (one lane per dest), writes the chunk
//               back with a TMA store and releases the stage (empty[s]); its epilogue stores the
//               sums, or with FUSE integrates the tile's neurons for step t + 1.
// Rows past a dest's in-use count hold +0.0f (never written otherwise), and adding +0.0f leaves
// a sum that started at +0.0f unchanged, so the sum warp adds all 64 rows of every chunk.  The
// prologue overlaps the previous kernel's tail; the step's data is touched after pdl_wait().
// Every mbarrier wait is bounded (about 1 s); on expiry the error word is set and the CTA drains.
// Tile epilogue: the sums go to the summation points or, with FUSE, straight into the neuron
// update of step t + 1 (device noise); the step counter advances here only when unfused (a fused
// sweep's next delivery advances it).
// x: the dest's neuron values (neuron_load after pdl_wait), noise: its N(0,1) draw for step t+1.
// FF: the epilogue may evaluate Izhikevich neurons in float-float arithmetic; the TMA sweep's
// sum warp has no registers to spare for it and uses the FP64 pipe instead (the same bits).
template <bool FUSE, bool FF = true>
__device__ __forceinline__ void sweep_finish(const NetDev &n, int d, bool valid, float acc,
                                             unsigned long long t, int lane, const NeuronIn &x,
                                             float noise, int tiles)
{
    if (FUSE) {
        const unsigned long long t1 = t + 1;
        bool fired = false;
        if (valid) {
            // the summation point stays 0: the call's first neuron pass cleared it, and a fused
            // sweep hands its sum to the update directly
            const int br = neuron_branch(x);
            fired = neuron_apply<FF>(n, d, x, br, input_apply(n, d, x, t1, acc),
                                     br == BR_INTEGRATE ? noise : 0.0f, t1, izh_mode(n, d));
        }
        ring_push(n, t1, fired, d);
    } else if (valid) {
        gst(&n.sp[d], acc);
    }
    // A fused sweep is always followed by the next step's delivery, which advances the step
    // counter after its wait; an unfused one (the last step of a call, injected noise) advances it
    // here, from the network's last tile.
    if (!FUSE && lane == 0) {
        __threadfence();
        unsigned prev = atomicAdd(n.sweep_done, 1u);
        if (prev == (unsigned)tiles - 1) {
            *n.step = t + 1;
            *n.sweep_done = 0;
            if (t + 1 >= 0xffffff00ull) set_err(n, ERR_STEP_RANGE);
            __threadfence();
        }
    }
}

template <bool FUSE, int SW_STAGES, int D>
__device__ __forceinline__ void sweep_tile(const NetDev &n, const CUtensorMap *tm_psr,
                                           const CUtensorMap *tm_cls, const int tile,
                                           uint8_t *smem_raw)
{
    constexpr uint32_t CH = sw_chunk_bytes(D), PB = sw_psr_bytes(D);
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
    float *s_dtab = (float *)(smem + (size_t)SW_STAGES * CH);
    uint64_t *full = (uint64_t *)(s_dtab + BG3_MAX_DCLS);
    uint64_t *scaled = full + SW_STAGES;
    uint64_t *empty = scaled + SW_STAGES;
    int *s_issued = (int *)(empty + SW_STAGES);
    int *s_light = s_issued + 1;  // the next delivery is light: -1 undecided, 0 no, 1 yes
    auto st_psr = [&](int s) { return (float *)(smem + (size_t)s * CH); };
    auto st_cls = [&](int s) { return smem + (size_t)s * CH + PB; };
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int d0 = tile * D;
    const int d = d0 + lane;
    const bool valid = lane < D && d < n.N;
    const int t32 = d0 >> 5, lx = d0 & 31;  // 32-dest plane tile and the first lane within it
    for (int i = threadIdx.x; i < n.n_dcls; i += blockDim.x) s_dtab[i] = n.dtab[i];
    const int cnt = valid ? (int)n.count[d] : 0;
    const int kmax = __reduce_max_sync(0xffffffffu, cnt);
    const int nch = (kmax + SW_ROWS - 1) / SW_ROWS;
    if (threadIdx.x == 0) {
        for (int s = 0; s < SW_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&scaled[s], SW_SCALE_WARPS);
            mbar_init(&empty[s], 1);
        }
        fence_mbar_init();
        *s_issued = 0;
        *s_light = -1;
    }
    __syncthreads();
    pdl_wait();  // spike delivery for this step has finished writing psr
    const unsigned long long t = *n.step;
    dstep_advance(n, tile == 0 && threadIdx.x == 0, t);
    __syncthreads();
    // The producer's idle lanes decide whether the next delivery is light (delivery_light); every
    // warp releases it (pdl_trigger) once it sees a light decision; a heavy one starts when this
    // sweep has ended.

    if (warp == 0) {  // ---------------------------------------------------------- producer
        auto issue = [&](int c) {
            const int s = c % SW_STAGES;
            mbar_expect_tx(&full[s], CH);
            tma_load_3d(st_psr(s), tm_psr, lx * 4, c * SW_QUADS, t32, &full[s]);
            tma_load_3d(st_cls(s), tm_cls, lx, c * SW_QUADS, t32, &full[s]);
            *(volatile int *)s_issued = c + 1;
        };
        if (lane == 0) {
            const int first = min(nch, SW_STAGES);
            for (int c = 0; c < first; c++) issue(c);  // free stages: no wait
            bool decided = false;
            for (int c = first; c < nch; c++) {
                if (!decided) decided = release_if_light(s_light);
                if (!mbar_wait(&empty[c % SW_STAGES], (uint32_t)((c / SW_STAGES - 1) & 1))) {
                    set_err(n, ERR_TIMEOUT);
                    break;
                }
                issue(c);
            }
        } else {
            const bool light = delivery_light(n, t + 1);
            if (lane == 1) *(volatile int *)s_light = light ? 1 : 0;
            if (light) pdl_trigger();
        }
        return;
    }

    if (warp <= SW_SCALE_WARPS) {  // --------------------------------------------- scale warps
        // a chunk is [16 quads][D dests] entries of (float4 psr, 16-bit class quad); each scale
        // warp takes a quarter of them, J per lane
        constexpr int E = SW_QUADS * D / SW_SCALE_WARPS, J = E / 32;
        const int e0 = (warp - 1) * E;
        bool decided = false;
        for (int c = 0; c < nch; c++) {
            const int s = c % SW_STAGES;
            if (!decided) decided = release_if_light(s_light);
            if (!mbar_wait(&full[s], (uint32_t)((c / SW_STAGES) & 1))) {
                set_err(n, ERR_TIMEOUT);
                break;
            }
            float4 *ps4 = reinterpret_cast<float4 *>(st_psr(s));                 // [16 quads][D]
            const uint16_t *cw = reinterpret_cast<const uint16_t *>(st_cls(s));  // [16 quads][D]
            float4 pv[J];
            uint32_t cv[J];
#pragma unroll
            for (int j = 0; j < J; j++) {
                pv[j] = ps4[e0 + j * 32 + lane];
                cv[j] = cw[e0 + j * 32 + lane];
            }
#pragma unroll
            for (int j = 0; j < J; j++) {
                pv[j].x = pv[j].x * s_dtab[cv[j] & 15u];
                pv[j].y = pv[j].y * s_dtab[(cv[j] >> 4) & 15u];
                pv[j].z = pv[j].z * s_dtab[(cv[j] >> 8) & 15u];
                pv[j].w = pv[j].w * s_dtab[(cv[j] >> 12) & 15u];
            }
#pragma unroll
            for (int j = 0; j < J; j++) ps4[e0 + j * 32 + lane] = pv[j];
            fence_async_smem();  // the TMA store (async proxy) must see these writes
            __syncwarp();
            if (lane == 0) mbar_arrive(&scaled[s]);
        }
        return;
    }

    // ------------------------------------------------------------------------------- sum warp
    NeuronIn x;
    float noise = 0.0f;
    if (FUSE && valid) {
        neuron_load(n, d, x);  // in flight while the chunks stream
        noise = normal_device(n.noise_seed, t + 1, d);
    }
    float acc = 0.0f;
    int done = 0;
    bool decided = false;
    for (int c = 0; c < nch; c++) {
        const int s = c % SW_STAGES;
        if (!decided) decided = release_if_light(s_light);
        if (!mbar_wait(&scaled[s], (uint32_t)((c / SW_STAGES) & 1))) {
            set_err(n, ERR_TIMEOUT);
            break;
        }
        done = c + 1;
        const float4 *ps4 = reinterpret_cast<const float4 *>(st_psr(s));
        if (lane < D) {
            float4 pv[SW_QUADS];
#pragma unroll
            for (int q = 0; q < SW_QUADS; q++) pv[q] = ps4[q * D + lane];
#pragma unroll
            for (int q = 0; q < SW_QUADS; q++) {
                acc = acc + pv[q].x;
                acc = acc + pv[q].y;
                acc = acc + pv[q].z;
                acc = acc + pv[q].w;
            }
        }
        __syncwarp();
        if (lane == 0) {
            tma_store_3d(tm_psr, lx * 4, c * SW_QUADS, t32, st_psr(s));
            bulk_commit();
            if (c >= 1) {
                bulk_wait_read1();
                mbar_arrive(&empty[(c - 1) % SW_STAGES]);
            }
        }
        __syncwarp();
    }
    if (lane == 0) bulk_wait_read_all();
    __syncwarp();
    if (done < nch) {
        // error path: wait (bounded) for the loads already issued before the smem goes away
        if (lane == 0) {
            int issued = *(volatile int *)s_issued;
            for (int c = done; c < issued; c++)
                if (!mbar_wait(&full[c % SW_STAGES], (uint32_t)((c / SW_STAGES) & 1))) break;
        }
        __syncwarp();
    }

    sweep_finish<FUSE, false>(n, d, valid, acc, t, lane, x, noise, n.ntiles * (SW_DESTS / D));
}

// psr *= decay for the first nq row quads of a 32-dest tile and the sum of each dest's rows in
// row order (one lane per dest; a row quad is one coalesced 16-byte load per lane).  between()
// runs once the first four row quads' loads are issued and before their data is used: work that
// needs no row data (the neuron pass's noise draw) then hides their latency.
template <typename F>
__device__ __forceinline__ float thin_rows(const NetDev &n, const int tile, const int nq,
                                           const int lane, F &&between)
{
    // this tile's row quads: [Mq][32 lanes] float4 of psr, 16 bits of class codes
    float4 *P = reinterpret_cast<float4 *>(n.psr) + (size_t)tile * n.Mq * 32 + lane;
    const uint16_t *C = reinterpret_cast<const uint16_t *>(n.dcls) + (size_t)tile * n.Mq * 32 + lane;
    float acc = 0.0f;
    float4 v[4];
    uint32_t c[4];
    auto load = [&](int q) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (q + j < nq) {
                v[j] = P[(size_t)(q + j) * 32];
                c[j] = C[(size_t)(q + j) * 32];
            }
        }
    };
    auto apply = [&](int q) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (q + j < nq) {
                v[j].x = v[j].x * __ldg(&n.dtab[c[j] & 15u]);
                v[j].y = v[j].y * __ldg(&n.dtab[(c[j] >> 4) & 15u]);
                v[j].z = v[j].z * __ldg(&n.dtab[(c[j] >> 8) & 15u]);
                v[j].w = v[j].w * __ldg(&n.dtab[(c[j] >> 12) & 15u]);
                gst(&P[(size_t)(q + j) * 32], v[j]);
                acc = acc + v[j].x;
                acc = acc + v[j].y;
                acc = acc + v[j].z;
                acc = acc + v[j].w;
            }
        }
    };
    if (nq > 0) load(0);  // nq is the warp's: a uniform branch
    between();
    if (nq > 0) apply(0);
    for (int q = 4; q < nq; q += 4) {
        load(q);
        apply(q);
    }
    return acc;
}

// The same without work in between (the one-CTA path): row quads in groups of four.
__device__ __forceinline__ float thin_rows(const NetDev &n, const int tile, const int nq,
                                           const int lane)
{
    float4 *P = reinterpret_cast<float4 *>(n.psr) + (size_t)tile * n.Mq * 32 + lane;
    const uint16_t *C = reinterpret_cast<const uint16_t *>(n.dcls) + (size_t)tile * n.Mq * 32 + lane;
    float acc = 0.0f;
    for (int q = 0; q < nq; q += 4) {
        float4 v[4];
        uint32_t c[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (q + j < nq) {
                v[j] = P[(size_t)(q + j) * 32];
                c[j] = C[(size_t)(q + j) * 32];
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (q + j < nq) {
                v[j].x = v[j].x * __ldg(&n.dtab[c[j] & 15u]);
                v[j].y = v[j].y * __ldg(&n.dtab[(c[j] >> 4) & 15u]);
                v[j].z = v[j].z * __ldg(&n.dtab[(c[j] >> 8) & 15u]);
                v[j].w = v[j].w * __ldg(&n.dtab[(c[j] >> 12) & 15u]);
                gst(&P[(size_t)(q + j) * 32], v[j]);
                acc = acc + v[j].x;
                acc = acc + v[j].y;
                acc = acc + v[j].z;
                acc = acc + v[j].w;
            }
        }
    }
    return acc;
}

// Thin networks (at most THIN_QUADS row quads per dest): one warp per 32-dest tile.  A row quad
// of a tile is 512 contiguous bytes of the plane (and 64 of the class plane), so the warp reads
// it with one coalesced 16-byte load per lane, scales it, writes it back and adds it in row
// order; the same epilogue as sweep_tile.  The noise draw runs while the neuron state and the
// first row quads are in flight.  Lanes past N sit in the last tile's padding, whose
// slots stay +0.0f.  For these networks a TMA pipeline per 32 dests would spend most of its time
// in set-up.
// Before it: the kernel's pdl_wait (spike delivery for this step has finished writing psr), the
// dstep advance by the network's tile 0 and the block barrier, then pdl_trigger.
template <bool FUSE>
__device__ __forceinline__ void sweep_thin_tile(const NetDev &n, const int tile, const int nq,
                                                const unsigned long long t)
{
    const int lane = threadIdx.x & 31;
    const int d = tile * SW_DESTS + lane;
    const bool valid = d < n.N;
    NeuronIn x;
    float noise = 0.0f;
    if (FUSE && valid) neuron_load(n, d, x);  // in flight with the row loads
    const float acc = thin_rows(n, tile, nq, lane, [&] {
        if (FUSE && valid) noise = normal_device(n.noise_seed, t + 1, d);
    });
    sweep_finish<FUSE>(n, d, valid, acc, t, lane, x, noise, n.ntiles);
}


template <int SYN, bool FUSE, int ST, int D>
__global__ void __launch_bounds__(SW_THREADS) k_sweep(const __grid_constant__ NetDev n,
                                                      const __grid_constant__ CUtensorMap tm_psr,
                                                      const __grid_constant__ CUtensorMap tm_cls)
{
    extern __shared__ uint8_t smem_raw[];
    sweep_tile<FUSE, ST, D>(n, &tm_psr, &tm_cls, blockIdx.x, smem_raw);
}

// Batched form: one launch sweeps every tile of every network of a batch.  tiles[b] = (network,
// tile); maps holds each network's two tensor maps (psr, class) in global memory; the block's
// network descriptor is copied into shared memory first (block_copy_desc).
template <bool FUSE, int ST>
__global__ void __launch_bounds__(SW_THREADS) k_sweep_batch(const NetDev *nets,
                                                            const CUtensorMap *maps,
                                                            const int2 *tiles)
{
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(16) NetDev s_net;
    const int2 tr = tiles[blockIdx.x];
    block_copy_desc(&s_net, nets + tr.x);
    sweep_tile<FUSE, ST, SW_DESTS>(s_net, &maps[2 * tr.x], &maps[2 * tr.x + 1], tr.y, smem_raw);
}

// Row-quad count of a thin tile (read before pdl_wait: the counts change only between calls).
__device__ __forceinline__ int thin_quads(const NetDev &n, int tile)
{
    const int d = tile * SW_DESTS + (int)(threadIdx.x & 31);
    const int cnt = d < n.N ? (int)n.count[d] : 0;
    return (__reduce_max_sync(0xffffffffu, cnt) + 3) >> 2;
}

template <bool FUSE>
__global__ void __launch_bounds__(1024) k_sweep_thin(const __grid_constant__ NetDev n)
{
    const int tile = blockIdx.x * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5);
    const bool active = tile < n.ntiles;
    const int nq = active ? thin_quads(n, tile) : 0;
    pdl_wait();
    const unsigned long long t = *n.step;
    dstep_advance(n, tile == 0 && (threadIdx.x & 31) == 0, t);
    __syncthreads();
    pdl_trigger();  // no shared memory held: an early next delivery keeps its L1
    if (active) sweep_thin_tile<FUSE>(n, tile, nq, t);
}

// Batched thin tiles: tiles[i] = (network, tile), one warp each.  Every block's entries belong to
// one network (the tile table pads each network's run to whole blocks with tile -1 entries,
// which do nothing), so the block shares one copy of the descriptor in shared memory.
template <bool FUSE>
__global__ void __launch_bounds__(1024) k_sweep_thin_batch(const NetDev *nets, const int2 *tiles,
                                                           int count)
{
    __shared__ __align__(16) NetDev s_net;
    const int first = blockIdx.x * (int)(blockDim.x >> 5);
    const int i = first + (int)(threadIdx.x >> 5);
    const int2 tr = i < count ? tiles[i] : make_int2(0, -1);
    const bool active = tr.y >= 0;
    block_copy_desc(&s_net, nets + tiles[min(first, count - 1)].x);
    const NetDev &n = s_net;
    const int nq = active ? thin_quads(n, tr.y) : 0;
    pdl_wait();
    const unsigned long long t = *n.step;
    dstep_advance(n, active && tr.y == 0 && (threadIdx.x & 31) == 0, t);
    __syncthreads();
    pdl_trigger();  // 1.7 KB of shared memory held: an early next delivery keeps its L1
    if (active) sweep_thin_tile<FUSE>(n, tr.y, nq, t);
}

bool sweep_is_thin(const NetDev &h, const LaunchCfg &c) { return h.Mq <= c.thin_max_quads; }

// ---- small networks: many steps per launch ----------------------------------------------------
// A network of at most SMALL_MAX_N neurons whose synapse planes hold at most the launch
// configuration's small_max_slots slots is advanced by one CTA through many steps in one launch.
// Each step runs the passes of a bg3_step call in their order — the neuron pass (device noise as
// k_neurons_device, injected noise as k_neurons_inject), the spike arrivals and, for the STDP
// kinds, the post-spike learning (as deliver_net and stdp_post_net), and the synapse sweep with
// the summation (thin_rows) — with block barriers between them, which also make each pass's
// global writes visible to the next.  A step of a 100-neuron network is then a few microseconds
// of on-chip latency instead of two or three kernel launches.  The step counter, its delivery
// copy and the injected stream's cursor are kept in registers and stored at the end.  No thread
// waits on another block, so nothing here can wait forever.
// Up to SMALL_THREADS threads: a network of N neurons gets N rounded up to whole warps (at least
// two), so that a small one pays for few warps at each barrier.
constexpr int SMALL_THREADS = 512;
constexpr int SMALL_WARPS = SMALL_THREADS / 32;

// ring_push with the spike counts of the ring's slots held in shared memory (the one-CTA path
// keeps them there for the whole launch and stores them back at its end).
__device__ __forceinline__ void ring_push_smem(const NetDev &n, int *s_ring_n,
                                               unsigned long long t, bool fired, int i)
{
    const unsigned mask = __ballot_sync(0xffffffffu, fired);
    if (!mask) return;
    const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
    const int slot = (int)(t & (BG3_RING - 1));
    int base = 0;
    if (lane == leader) base = atomicAdd(&s_ring_n[slot], __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (fired) {
        const int pos = base + __popc(mask & ((1u << lane) - 1));
        if (pos < n.N) n.ring[(size_t)slot * n.N + pos] = i;
        else set_err(n, ERR_SPIKE_LIST);
    }
}

// Injected noise: the reference CPU order, neurons walked from the top in chunks of the block
// (k_neurons_inject with the launch's block); returns the step's number of draws.
__device__ __forceinline__ long long small_neurons_inject(const NetDev &n, unsigned long long t,
                                                          unsigned long long cursor,
                                                          int *warp_tot, long long *s_running,
                                                          int *s_ring_n)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) *s_running = 0;
    __syncthreads();
    const int nt = (int)blockDim.x, nw = nt >> 5;
    for (int top = n.N - 1; top >= 0; top -= nt) {
        const int i = top - (int)threadIdx.x;
        NeuronIn x;
        if (i >= 0) neuron_load(n, i, x);
        const int br = (i >= 0) ? neuron_branch(x) : BR_REFRACTORY;
        const bool integ = (i >= 0) && br == BR_INTEGRATE;
        const unsigned m = __ballot_sync(0xffffffffu, integ);
        const int in_warp = __popc(m & ((1u << lane) - 1));
        if (lane == 31) warp_tot[warp] = __popc(m);
        __syncthreads();
        if (warp == 0) {
            const int v = lane < nw ? warp_tot[lane] : 0;
            int y = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int z = __shfl_up_sync(0xffffffffu, y, o);
                if (lane >= o) y += z;
            }
            if (lane < nw) warp_tot[lane] = y - v;  // exclusive prefix of warp totals
        }
        __syncthreads();
        const long long running = *s_running;
        bool fired = false;
        if (i >= 0) {
            float noise = 0.0f;
            if (integ) {
                const long long pos = (long long)cursor + running + warp_tot[warp] + in_warp;
                if (pos < n.noise_len) noise = n.noise_buf[pos];
                else set_err(n, ERR_NOISE_EXHAUSTED);
            }
            fired = neuron_apply(n, i, x, br, input_apply(n, i, x, t, n.sp[i]), noise, t,
                                 izh_mode(n, i));
            n.sp[i] = 0.0f;
        }
        ring_push_smem(n, s_ring_n, t, fired, i);
        __syncthreads();
        if ((int)threadIdx.x == nt - 1) *s_running = running + warp_tot[warp] + __popc(m);
        __syncthreads();
    }
    return *s_running;
}

template <int SYN, bool INJECT>
__global__ void __launch_bounds__(SMALL_THREADS) k_small_run(const __grid_constant__ NetDev n,
                                                             int nsteps)
{
    __shared__ int warp_tot[SMALL_WARPS];
    __shared__ long long s_running;
    __shared__ int s_moff[BG3_MAX_DELAYS + 1];
    __shared__ int s_ring_n[BG3_RING];        // the ring's spike counts, stored back at the end
    __shared__ int s_ltab[BG3_MAX_DELAYS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthreads = (int)blockDim.x, nwarps = nthreads >> 5;
    unsigned long long t = *n.step;
    unsigned long long cursor = INJECT ? *n.noise_cursor : 0ull;
    for (int k = tid; k < BG3_RING; k += nthreads) s_ring_n[k] = n.ring_n[k];
    if (tid < BG3_MAX_DELAYS) s_ltab[tid] = tid < n.n_delays ? n.ltab[tid] : 0;
    __syncthreads();
    for (int s = 0; s < nsteps; s++, t++) {
        // ---- neuron pass of step t
        if (INJECT) {
            cursor += (unsigned long long)small_neurons_inject(n, t, cursor, warp_tot, &s_running,
                                                               s_ring_n);
        } else {
            for (int i0 = 0; i0 < n.N; i0 += nthreads) {
                const int i = i0 + tid;
                bool fired = false;
                if (i < n.N) {
                    NeuronIn x;
                    neuron_load(n, i, x);
                    const int br = neuron_branch(x);
                    const float noise = (br == BR_INTEGRATE) ? normal_device(n.noise_seed, t, i) : 0.0f;
                    fired = neuron_apply(n, i, x, br, input_apply(n, i, x, t, n.sp[i]), noise, t,
                                 izh_mode(n, i));
                    n.sp[i] = 0.0f;
                }
                ring_push_smem(n, s_ring_n, t, fired, i);
            }
        }
        __syncthreads();
        if (warp == 0) {
            // arrival items per delay class, then their offsets
            int m = 0;
            if (lane < n.n_delays) {
                const int D = s_ltab[lane];
                if (D > 0 && (unsigned long long)D <= t)
                    m = min(s_ring_n[(t - (unsigned long long)D) & (BG3_RING - 1)], n.N);
            }
            int x = m;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane <= n.n_delays) s_moff[lane] = x - m;  // exclusive prefix; the last is M
        }
        __syncthreads();
        // ---- spike arrivals of step t: one warp per (delay class, neuron that fired) item;
        // every synapse has one source, which fired once, so no two lanes touch one slot
        const int M = s_moff[n.n_delays];
        for (int item = warp; item < M; item += nwarps) {
            int c = 0;
            while (item >= s_moff[c + 1]) c++;
            const unsigned long long tf = t - (unsigned long long)s_ltab[c];
            const int src = n.ring[(size_t)(tf & (BG3_RING - 1)) * n.N + (item - s_moff[c])];
            const size_t ci = (size_t)c * n.N + src;
            const uint32_t b = n.outBegin[ci], k = n.outCount[ci];
            for (uint32_t j = (uint32_t)lane; j < k; j += 32)
                deliver_hit<SYN>(n, n.outMap[b + j], (uint32_t)tf, t, src);
        }
        if (tid == 0) s_ring_n[(t + 1) & (BG3_RING - 1)] = 0;  // for the next neuron pass
        __syncthreads();
        if (SYN >= 2) {
            // post-spike learning of the neurons that fired at step t, after the arrivals
            const int slot = (int)(t & (BG3_RING - 1));
            const int m = min(s_ring_n[slot], n.N);
            for (int e = warp; e < m; e += nwarps) {
                const int d = n.ring[(size_t)slot * n.N + e];
                const int cnt = (int)n.count[d];
                for (int k = lane; k < cnt; k += 32) {
                    const size_t p = slot_pos(k, d, n.Mq);
                    n.ev[p].W = stdp_post(n, n.stdp[n.stype[p]], n.ev[p].W, n.src[p], d,
                                          n.ltab[n.lcls[p]], t);
                }
            }
            __syncthreads();
        }
        // ---- synapse sweep and summation of step t: one warp per 32-dest tile
        for (int tile = warp; tile < n.ntiles; tile += nwarps) {
            const float acc = thin_rows(n, tile, thin_quads(n, tile), lane);
            const int d = tile * SW_DESTS + lane;
            if (d < n.N) n.sp[d] = acc;
        }
        __syncthreads();
    }
    for (int k = tid; k < BG3_RING; k += nthreads) n.ring_n[k] = s_ring_n[k];
    if (tid == 0) {
        *n.step = t;
        *n.dstep = t;
        if (INJECT) *n.noise_cursor = cursor;
        if (t >= 0xffffff00ull) set_err(n, ERR_STEP_RANGE);
    }
}

bool small_eligible(const NetDev &h, const LaunchCfg &c)
{
    return h.N <= SMALL_MAX_N && (long long)h.Np * h.Mq * 4 <= (long long)c.small_max_slots;
}

// nsteps steps of a small network in one launch (small_eligible).
void launch_small(const NetDev &h, int nsteps, cudaStream_t s)
{
    const bool inj = h.noise_mode == 1;
    const int SMALL_THREADS = std::max(64, std::min(bg3::SMALL_THREADS, (h.N + 31) / 32 * 32));
    switch (h.syn_kind * 2 + (inj ? 1 : 0)) {
    case 2: k_small_run<1, false><<<1, SMALL_THREADS, 0, s>>>(h, nsteps); break;
    case 3: k_small_run<1, true><<<1, SMALL_THREADS, 0, s>>>(h, nsteps); break;
    case 4: k_small_run<2, false><<<1, SMALL_THREADS, 0, s>>>(h, nsteps); break;
    case 5: k_small_run<2, true><<<1, SMALL_THREADS, 0, s>>>(h, nsteps); break;
    case 6: k_small_run<3, false><<<1, SMALL_THREADS, 0, s>>>(h, nsteps); break;
    case 7: k_small_run<3, true><<<1, SMALL_THREADS, 0, s>>>(h, nsteps); break;
    case 1: k_small_run<0, true><<<1, SMALL_THREADS, 0, s>>>(h, nsteps); break;
    default: k_small_run<0, false><<<1, SMALL_THREADS, 0, s>>>(h, nsteps); break;
    }
}

// ---- launchers -------------------------------------------------------------------------------

int neuron_launches(const NetDev &h) { return (h.noise_mode == 1 && h.N > 2 * INJ_CHUNK) ? 2 : 1; }

void launch_neurons(const NetDev &h, cudaStream_t s)
{
    if (h.noise_mode == 1 && h.N > 2 * INJ_CHUNK) {
        const int nb = (h.N + INJ_CHUNK - 1) / INJ_CHUNK;
        k_neurons_inject_count<<<nb, INJ_CHUNK, 0, s>>>(h);
        k_neurons_inject_apply<<<nb, INJ_CHUNK, 0, s>>>(h);
    } else if (h.noise_mode == 1)
        k_neurons_inject<<<1, 1024, 0, s>>>(h);
    else
        k_neurons_device<<<(h.N + 255) / 256, 256, 0, s>>>(h);
}

template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kern)(KArgs...), dim3 grid, int block, size_t smem, cudaStream_t s,
                       Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.gridDim = grid;
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// Spike arrivals of the step, then (STDP kinds) the post-spike learning pass.
void launch_deliver(const NetDev &h, const LaunchCfg &c, cudaStream_t s)
{
    const int g = c.deliver_blocks, e = c.deliver_early;
    switch (h.syn_kind) {
    case 1: launch_pdl(k_deliver<1>, g, 256, 0, s, h, e); break;
    case 2: launch_pdl(k_deliver<2>, g, 256, 0, s, h, e); break;
    case 3: launch_pdl(k_deliver<3>, g, 256, 0, s, h, e); break;
    default: launch_pdl(k_deliver<0>, g, 256, 0, s, h, e); break;
    }
    if (h.syn_kind >= 2) launch_pdl(k_stdp_post, g, 256, 0, s, h);
}

template <typename K>
static void allow_smem(K kern, int st, int D)
{
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sw_smem(st, D));
}

template <int SYN, bool FUSE, int ST, int D>
static void launch_sweep_t(const NetDev &h, const CUtensorMap &tp, const CUtensorMap &tc, cudaStream_t s)
{
    static bool attr_set = false;
    if (!attr_set) {
        allow_smem(k_sweep<SYN, FUSE, ST, D>, ST, D);
        attr_set = true;
    }
    launch_pdl(k_sweep<SYN, FUSE, ST, D>, h.ntiles * (SW_DESTS / D), SW_THREADS, sw_smem(ST, D), s,
               h, tp, tc);
}

template <bool FUSE, int ST>
static void launch_sweep_batch_thick(const NetDev *nets, const CUtensorMap *maps, const int2 *tiles,
                                     int n_thick, cudaStream_t s)
{
    static bool attr_set = false;
    if (!attr_set) {
        allow_smem(k_sweep_batch<FUSE, ST>, ST, SW_DESTS);
        attr_set = true;
    }
    launch_pdl(k_sweep_batch<FUSE, ST>, n_thick, SW_THREADS, sw_smem(ST, SW_DESTS), s, nets, maps, tiles);
}

template <bool FUSE>
static void launch_sweep_batch_t(const NetDev *nets, const CUtensorMap *maps, const int2 *tiles,
                                 int n_thick, int n_thin, const LaunchCfg &c, cudaStream_t s)
{
    if (n_thick > 0) {
        if (c.sweep_stages == 4) launch_sweep_batch_thick<FUSE, 4>(nets, maps, tiles, n_thick, s);
        else if (c.sweep_stages == 8) launch_sweep_batch_thick<FUSE, 8>(nets, maps, tiles, n_thick, s);
        else launch_sweep_batch_thick<FUSE, 6>(nets, maps, tiles, n_thick, s);
    }
    if (n_thin > 0) {
        const int w = c.thin_warps;
        launch_pdl(k_sweep_thin_batch<FUSE>, (n_thin + w - 1) / w, 32 * w, 0, s, nets,
                   (const int2 *)(tiles + n_thick), n_thin);
    }
}

void launch_neurons_batch(const NetDev *nets, int count, int max_n, cudaStream_t s)
{
    k_neurons_device_batch<<<dim3((max_n + 255) / 256, count), 256, 0, s>>>(nets);
}

void launch_deliver_batch(int syn_kind, const NetDev *nets, int count, const LaunchCfg &c,
                          cudaStream_t s)
{
    // per network: four plain grids shared out over the batch (blocks without items exit at
    // once, so a quiet network costs little)
    const int per_net = std::max(2, std::min(c.deliver_blocks, 4 * c.deliver_blocks / std::max(count, 1)));
    const dim3 grid(per_net, count);
    const int e = c.deliver_early;
    switch (syn_kind) {
    case 1: launch_pdl(k_deliver_batch<1>, grid, 256, 0, s, nets, e); break;
    case 2: launch_pdl(k_deliver_batch<2>, grid, 256, 0, s, nets, e); break;
    case 3: launch_pdl(k_deliver_batch<3>, grid, 256, 0, s, nets, e); break;
    default: launch_pdl(k_deliver_batch<0>, grid, 256, 0, s, nets, e); break;
    }
    if (syn_kind >= 2) launch_pdl(k_stdp_post_batch, grid, 256, 0, s, nets);
}

void launch_sweep_batch(const NetDev *nets, const CUtensorMap *maps, const int2 *tiles, int n_thick,
                        int n_thin, bool fuse, const LaunchCfg &c, cudaStream_t s)
{
    if (fuse) launch_sweep_batch_t<true>(nets, maps, tiles, n_thick, n_thin, c, s);
    else launch_sweep_batch_t<false>(nets, maps, tiles, n_thick, n_thin, c, s);
}

template <int SYN, bool FUSE, int D>
static void launch_sweep_st(const NetDev &h, const CUtensorMap &tp, const CUtensorMap &tc,
                            const LaunchCfg &c, cudaStream_t s)
{
    if (c.sweep_stages == 4) launch_sweep_t<SYN, FUSE, 4, D>(h, tp, tc, s);
    else if (c.sweep_stages == 8) launch_sweep_t<SYN, FUSE, 8, D>(h, tp, tc, s);
    else launch_sweep_t<SYN, FUSE, 6, D>(h, tp, tc, s);
}

// tp/tc: the tensor maps of 32-dest boxes, tp16/tc16 those of 16-dest boxes
void launch_sweep(const NetDev &h, const CUtensorMap &tp, const CUtensorMap &tc,
                  const CUtensorMap &tp16, const CUtensorMap &tc16, bool fuse,
                  const LaunchCfg &c, cudaStream_t s)
{
    if (sweep_is_thin(h, c)) {
        const int w = c.thin_warps;
        const int blocks = (h.ntiles + w - 1) / w;
        if (fuse) launch_pdl(k_sweep_thin<true>, blocks, 32 * w, 0, s, h);
        else launch_pdl(k_sweep_thin<false>, blocks, 32 * w, 0, s, h);
        return;
    }
    // the synapse kind does not change the sweep: one instantiation serves all kinds
    if (c.sweep_dests == 16) {
        if (fuse) launch_sweep_st<1, true, 16>(h, tp16, tc16, c, s);
        else launch_sweep_st<1, false, 16>(h, tp16, tc16, c, s);
    } else {
        if (fuse) launch_sweep_st<1, true, SW_DESTS>(h, tp, tc, c, s);
        else launch_sweep_st<1, false, SW_DESTS>(h, tp, tc, c, s);
    }
}

}  // namespace bg3
