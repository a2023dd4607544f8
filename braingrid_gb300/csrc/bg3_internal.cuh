// Internal device-side layout and helpers of libbg3.
//
// HBM layout of one network (all arrays owned by bg3_net, allocated once at bg3_create):
//
//   neurons (n = N)       SoA float/int arrays, neuron index contiguous.
//   synapse slot planes   slot (dest d, row k) lives at plane index p = k * N + d ("ELL" order):
//                         a warp that walks 32 consecutive dests of one row k reads 128
//                         contiguous bytes per field.  The reference slot id is d * maxSyn + k.
//   delay queues          one uint32 ring per slot, stored in the GLOBAL step phase: a spike
//                         due at step t sits at bit (t & 31).  The reference keeps a per-slot
//                         read index (delayIdx) instead; with phase0 = (creation step) & 31 the
//                         two are related by q_global = rotl(q_ref, phase0) and
//                         delayIdx = (t - phase0) & 31, so the hot sweep needs neither the
//                         index read nor its write.
//   outgoing map          CSR by source neuron; entry = plane index | (total_delay << 27).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define BG3_ULONG_MAX 0xffffffffffffffffull
#define BG3_DELAY_SHIFT 27
#define BG3_POS_MASK ((1u << BG3_DELAY_SHIFT) - 1u)

struct NetDev {
    int32_t N, max_syn, max_spikes, neuron_kind, syn_kind, noise_mode;
    float dt, epoch_duration;
    uint32_t noise_seed;
    int32_t ntiles;           // sweep tiles of 32 dests
    // step counter and the last-CTA barrier of the sweep
    unsigned long long *step;
    uint32_t *sweep_done;
    uint32_t *err;
    // neurons
    float *Vm, *Vthresh, *Vreset, *I0, *Inoise, *C1, *C2, *Trefract, *sp;
    int32_t *refr, *spikeCount, *spikeCountOffset;
    unsigned long long *history;   // [N][max_spikes]
    int8_t *ntype;                 // 1 INH, 2 EXC
    // spikes of the current step
    int32_t *spikes, *nspikes;
    // synapse planes
    float *psr, *decay, *W, *U, *D, *F, *u, *r;
    uint32_t *queue;
    unsigned long long *lastSpike;
    int32_t *src;
    int8_t *stype;
    uint8_t *phase0;
    uint8_t *sdelay;               // total_delay of the slot (steps)
    uint32_t *count;               // in-use prefix length per dest
    // outgoing CSR
    uint32_t *outBegin, *outCount, *outMap;
    uint32_t *outFill;
    // growth
    float *radii, *rates, *xloc, *yloc;
    float g_epsilon, g_beta, g_rho, g_target_rate, g_min_radius, g_start_radius, g_max_rate;
    // recorder
    float *burstiness, *spikes_hist, *rates_hist, *radii_hist;
    int32_t n_burst_bins, n_spike_bins, max_epochs;
    // injected noise
    const float *noise_buf;
    unsigned long long *noise_cursor;
    long long noise_len;
    // per-type constants for synapses created on the device
    float t_tau[4], t_decay[4], t_U[4], t_D[4], t_F[4], t_u0, t_r0;
    int32_t t_delay[4];
};

// ---- exact-rounding helpers -----------------------------------------------------------------
// The library is compiled with -fmad=false so that every a*b+c is two rounded operations, as in
// the reference's x86-64 build.  expf of the reference's host library is correctly rounded for
// almost every argument; evaluating exp in double and rounding once reproduces that.
__device__ __forceinline__ float exp_cr(float x) { return (float)exp((double)x); }
__device__ __forceinline__ float acos_cr(float x) { return (float)acos((double)x); }
__device__ __forceinline__ float sin_cr(float x) { return (float)sin((double)x); }

// ---- counter-based normal generator (device noise mode) --------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11): key = (seed, seed ^ 0x5bd1e995), counter = (neuron, step lo, step hi, 0).
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int i = 0; i < 10; i++) {
        uint32_t hi0 = __umulhi(M0, c[0]), lo0 = M0 * c[0];
        uint32_t hi1 = __umulhi(M1, c[2]), lo1 = M1 * c[2];
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += W0; k1 += W1;
    }
}
// One N(0,1) value by the Box-Muller transform of two 32-bit uniforms.
__device__ __forceinline__ float normal_device(uint32_t seed, unsigned long long step, int i)
{
    uint32_t c[4] = {(uint32_t)i, (uint32_t)step, (uint32_t)(step >> 32), 0u};
    philox4x32_10(c, seed, seed ^ 0x5bd1e995u);
    float u1 = ((float)(c[0] >> 8) + 0.5f) * (1.0f / 16777216.0f);  // (0,1)
    float u2 = (float)(c[1] >> 8) * (1.0f / 16777216.0f);           // [0,1)
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

__device__ __forceinline__ void set_err(const NetDev &n, uint32_t bit) { atomicOr(n.err, bit); }
