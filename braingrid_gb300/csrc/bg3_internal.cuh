// Internal device-side layout and helpers of libbg3.
//
// HBM layout of one network (arrays owned by bg3_net, allocated once at bg3_create):
//
//   neurons               SoA float/int arrays, neuron index contiguous.
//   synapse slot planes   tile-major ELL with row quads: dests are grouped in tiles of 32; slot
//                         (dest d, row k) of tile T = d / 32 lives at
//                         p = ((T * Mq + k / 4) * 32 + d % 32) * 4 + k % 4, Mq = max_syn / 4
//                         rounded up.  One 16-byte load gives a lane four consecutive rows of its
//                         dest; a tile's row quads are one contiguous stream of Mq x 512 bytes,
//                         so the sweep reads long sequential runs (a 64-row chunk of a tile is
//                         8 KB of psr and 2 KB of classes, one 3-D TMA box each).  The reference
//                         slot id of (d, k) is d * maxSyn + k.
//   hot per-slot state    psr (f32) and a one-byte decay class (index into a per-network table
//                         of decay factors): 9 bytes per synapse per step.
//   event per-slot state  EvSlot (32 B, one sector): W, u, r, last spike step, birth step, and
//                         the slot's decay class and DS parameter class (U, D, F and their exp
//                         tables live in a per-network table) — read only when a spike is
//                         delivered, so a delivery touches two lines: its EvSlot and its psr.
//   spike propagation     instead of a 32-bit delay queue per synapse, the ids of the neurons
//                         that fired at each of the last 64 steps are kept in a ring; the
//                         outgoing map is grouped by delay class, so at step t the synapses of
//                         delay D that receive a spike are the outgoing synapses (class D) of the
//                         neurons in ring slot (t - D) & 63.  A synapse receives the spike only
//                         if it existed when the spike was emitted (birth step <= emit step),
//                         which is what the reference's per-synapse queue encodes.  The
//                         reference's delayQueue / delayIdx are rebuilt from the ring on download.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define BG3_ULONG_MAX 0xffffffffffffffffull
#define BG3_NO_SPIKE32 0xffffffffu
#define BG3_RING 64          // spike-list ring depth (steps); delays must be < 32
#define BG3_MAX_DCLS 16      // decay classes (4-bit codes in the class plane)
#define BG3_MAX_DELAYS 8     // delay classes
#define BG3_MAX_EXPC 16      // time constants with an exp table
#define BG3_EXP_LEN 262144   // steps covered by an exp table (26 s at dt = 0.1 ms)
#define BG3_DEXP_LEN 8192    // steps covered by a double exp table (STDP windows)
#define BG3_MAX_PCLS 16      // distinct (U, D, F) triples of DS synapses

// STDP constants of one synapse type (AllSTDPSynapses.h:350-420); createSynapse gives every
// synapse the same values (AllSTDPSynapses.cpp:252-273), so they are held per type.
struct StdpConst {
    float Apos, Aneg, gap, tauspost, tauspre, taupos, tauneg, Wex, mupos, muneg;
    int32_t useFD;
    int32_t dlen_pos, dlen_neg;      // entries of the double tables (0: none)
    const double *dpos, *dneg;       // exp(-(k dt) / taupos), exp(-(k dt) / tauneg)
};

struct __align__(32) EvSlot {
    float W, u, r;
    uint32_t last;   // step of the last delivered spike, BG3_NO_SPIKE32 = none (ULONG_MAX)
    uint32_t born;   // step at which the synapse was created (low 32 bits)
    uint8_t dcls;    // decay class (the plane's class byte, for the delivery)
    uint8_t pcls;    // (U, D, F) class
    uint16_t pad0;
    uint32_t pad1, pad2;
};

// Launch configuration of the step and growth kernels (bg3_launch_cfg of the C-ABI; chosen by
// the autotuner or set by the caller).
struct LaunchCfg {
    int32_t sweep_stages;     // chunks in flight per TMA sweep tile: 4, 6 or 8
    int32_t thin_max_quads;   // networks with at most this many row quads take the thin sweep
    int32_t thin_warps;       // warps per block of the thin sweep (1 .. 32)
    int32_t deliver_blocks;   // blocks of the delivery grid (a batch shares 4x this out)
    int32_t growth_threads;   // threads per block of the overlap pass: 128, 256 or 512
    int32_t sweep_dests;      // dests per TMA sweep tile of a single network: 16 or 32
    int32_t deliver_early;    // 1: spiking/DS delivery prepares its arrivals during the previous
                              // sweep, 0: it starts after it
    int32_t izh_hw_every;     // Izhikevich update: every k-th 32-neuron tile in hardware FP64,
                              // the others on the integer pipe (0: all on the integer pipe);
                              // -1: float-float arithmetic, FP64 only for uncertain roundings
    int32_t small_max_slots;  // networks of at most SMALL_MAX_N neurons and this many synapse
                              // slots run many steps per launch in one CTA (0: never)
};
constexpr int SMALL_MAX_N = 2048;
constexpr LaunchCfg LAUNCH_DEFAULT = {6, 16, 8, 304, 256, 32, 1, -1, 65536};

// plane position of slot (dest d, row k) and its inverse (Mq row quads per dest)
__host__ __device__ __forceinline__ size_t slot_pos(int k, int d, int Mq)
{
    const size_t t = (size_t)(d >> 5) * (size_t)Mq + (size_t)(k >> 2);  // tile row quad
    return (((t << 5) | (size_t)(d & 31)) << 2) | (size_t)(k & 3);
}
// The class plane holds a 4-bit decay class per slot position p: nibble p & 7 of word p >> 3,
// so one 16-bit half-word carries the four rows of one dest's row quad.
__host__ __device__ __forceinline__ uint32_t cls_get(const uint32_t *plane, size_t p)
{
    return (plane[p >> 3] >> (4u * (uint32_t)(p & 7))) & 15u;
}
__host__ __device__ __forceinline__ void cls_put(uint32_t *plane, size_t p, uint32_t c)
{
    plane[p >> 3] |= (c & 15u) << (4u * (uint32_t)(p & 7));  // the nibble must be 0 before
}
__host__ __device__ __forceinline__ void pos_slot(size_t p, int Mq, int &k, int &d)
{
    const size_t q = p >> 2;
    const size_t t = q >> 5;
    d = (int)((t / (size_t)Mq) << 5) | (int)(q & 31);
    k = (int)((t % (size_t)Mq) << 2) | (int)(p & 3);
}

struct NetDev {
    int32_t N, Np, max_syn, max_spikes, neuron_kind, syn_kind, noise_mode;
    int32_t Mq;                    // row quads per dest: ceil(max_syn / 4)
    float dt, epoch_duration;
    uint32_t noise_seed;
    int32_t ntiles;                // sweep tiles of 32 dests
    int32_t izh_hw_every;          // LaunchCfg::izh_hw_every, for the fused neuron pass
    int32_t n_dcls, n_delays;
    // step counter and the last-CTA barrier of the sweep
    unsigned long long *step;
    uint32_t *sweep_done;
    // the delivery pass's own copy of the step counter: a delivery prepares its arrivals while
    // the previous sweep, which may advance `step`, is still running
    unsigned long long *dstep;
    uint32_t *err;
    // neurons
    float *Vm, *Vthresh, *Vreset, *I0, *Inoise, *C1, *C2, *Trefract, *sp;
    int32_t *refr, *spikeCount, *spikeCountOffset;
    unsigned long long *history;   // [N][max_spikes]
    int8_t *ntype;                 // 1 INH, 2 EXC
    // Izhikevich neurons only (NULL for LIF): a, b, c, d, recovery variable u, C3 = dt * 1000
    float *Aconst, *Bconst, *Cconst, *Dconst, *u_izh, *C3;
    // spike ring: ids of the neurons that fired at step t are ring[(t & 63) * N + i]
    int32_t *ring, *ring_n;
    // synapse planes (index slot_pos(k, d, Mq), Np * Mq * 4 entries)
    float *psr;
    uint32_t *dcls;                // decay class, 4 bits per slot: nibble p (cls_get / cls_or)
    uint8_t *lcls;                 // delay class
    EvSlot *ev;
    int32_t *src;
    int8_t *stype;
    uint32_t *count;               // in-use prefix length per dest
    float *dtab;                   // decay factor per decay class [BG3_MAX_DCLS]
    int32_t *ltab;                 // delay (steps) per delay class [BG3_MAX_DELAYS]
    // outgoing CSR per (delay class, source): index c * N + i
    uint32_t *outBegin, *outCount, *outMap, *outFill;
    // growth
    float *radii, *rates, *xloc, *yloc;
    // the layout is the reference's grid (xloc = i % grid_w, yloc = i / grid_w), so the overlap
    // scan of a destination can stop at the sources beyond the largest radius; 0 otherwise
    int32_t grid_w, grid_h;
    float *grow_rmax;  // [1]: the largest radius of the epoch's growth pass
    float g_epsilon, g_beta, g_rho, g_target_rate, g_min_radius, g_start_radius, g_max_rate;
    float *grow_exp;   // [max_spikes + 1]: the outgrowth exp for each spike count (host libm)
    // recorder
    float *burstiness, *spikes_hist, *rates_hist, *radii_hist;
    int32_t n_burst_bins, n_spike_bins, max_epochs;
    // injected noise
    const float *noise_buf;
    unsigned long long *noise_cursor;
    long long noise_len;
    // per-type constants for synapses created on the device
    float t_tau[4], t_U[4], t_D[4], t_F[4], t_u0, t_r0;
    int32_t t_dcls[4], t_lcls[4];
    // external input: 0 none, 1 regular (Inputs/SInputRegular), 2 Poisson (Inputs/SInputPoisson)
    int32_t input_kind;
    float *reg_values;
    int32_t *reg_shift;
    int32_t reg_dur, reg_cycle, reg_c0;    // cycle position reg_c0 at step reg_t0
    unsigned long long reg_t0;
    uint8_t *pois_mask;
    int32_t *pois_nisi;
    float pois_lambda;
    uint32_t pois_seed;
    unsigned long long pois_t0;            // step of bg3_input_poisson (masked-out synapses stay)
    float *in_psr, *in_decay;
    uint32_t *in_queue;                    // global-phase delay queue of the input synapse
    uint8_t *in_delay;
    EvSlot *in_ev;
    int32_t *isi_begin, *isi_vals, *isi_cursor;  // injected ISI draws (NULL: device generator)
    // exp(-(k dt) / tau) for k < BG3_EXP_LEN, one table per time constant, filled by the host's
    // libm expf (the function the reference's host build calls for these factors)
    int32_t n_expc;
    float expc_tau[BG3_MAX_EXPC];
    const float *expc_tab[BG3_MAX_EXPC];
    // STDP kinds: per-type constants; stdp_signed selects the reference device build's signed
    // spike-time arithmetic instead of its host build's unsigned one
    StdpConst stdp[4];
    int32_t stdp_signed;
    // DS parameter classes: (U, D, F) and the exp tables of D and F (NULL past the limit)
    int32_t n_pcls;
    int32_t t_pcls[4];               // class of the per-type constants (synapses growth creates)
    float p_U[BG3_MAX_PCLS], p_D[BG3_MAX_PCLS], p_F[BG3_MAX_PCLS];
    const float *p_xD[BG3_MAX_PCLS], *p_xF[BG3_MAX_PCLS];
};

// device error word bits (mirrored in include/bg3.h)
enum : uint32_t {
    ERR_HISTORY_OVERFLOW = 1u << 0,
    ERR_ROW_FULL = 1u << 2,
    ERR_NOISE_EXHAUSTED = 1u << 3,
    ERR_NEGATIVE_AREA = 1u << 4,
    ERR_SPIKE_LIST = 1u << 5,
    ERR_TIMEOUT = 1u << 6,
    ERR_STEP_RANGE = 1u << 7,
    ERR_ISI_EXHAUSTED = 1u << 8,
    ERR_STDP_RING = 1u << 9,
    ERR_STEP_SYNC = 1u << 10,
};

// ---- exact-rounding helpers -----------------------------------------------------------------
// The library is compiled with -fmad=false so that every a*b+c is two rounded operations, as in
// the reference's x86-64 build.  expf of the reference's host library is correctly rounded for
// almost every argument; evaluating exp in double and rounding once reproduces that.
__device__ __forceinline__ float exp_cr(float x) { return (float)exp((double)x); }
__device__ __forceinline__ float acos_cr(float x) { return (float)acos((double)x); }
__device__ __forceinline__ float sin_cr(float x) { return (float)sin((double)x); }

// expf(-((float)k * dt) / tau): the DS facilitation / depression factors and the STDP
// efficacies all take this form with k a whole number of steps.  Time constants registered by
// the host are read from their table, so the value is the host library's own rounding; others
// (and k beyond the table) fall back to the correctly rounded value.
__device__ __forceinline__ float exp_steps(const NetDev &n, uint32_t k, float tau)
{
    if (k < (uint32_t)BG3_EXP_LEN) {
        for (int c = 0; c < n.n_expc; c++)
            if (n.expc_tau[c] == tau) return __ldg(n.expc_tab[c] + k);
    }
    const float x = (float)k * n.dt;
    return exp_cr(-x / tau);
}

// expf(-((float)k * dt) / tau) from the table of a DS parameter class.
__device__ __forceinline__ float exp_tab(const NetDev &n, const float *tab, uint32_t k, float tau)
{
    if (tab && k < (uint32_t)BG3_EXP_LEN) return __ldg(tab + k);
    const float x = (float)k * n.dt;
    return exp_cr(-x / tau);
}

// AllDSSynapses::changePSR's facilitation / depression update of u and r
// (Synapses/AllDSSynapses.cpp:235-241) for a spike k steps after the previous one.
__device__ __forceinline__ void ds_update(const NetDev &n, const EvSlot &e, uint32_t k,
                                          float &u, float &r)
{
    const int c = e.pcls;
    const float U = n.p_U[c];
    r = 1.0f + (r * (1.0f - u) - 1.0f) * exp_tab(n, n.p_xD[c], k, n.p_D[c]);
    u = U + u * (1.0f - U) * exp_tab(n, n.p_xF[c], k, n.p_F[c]);
}

// expf(-(x dt) / tau) for a spike-time difference u held as uint64 (host build) or int64
// (device build): x = (float)u or (float)(int64)u.
__device__ __forceinline__ float exp_interval(const NetDev &n, unsigned long long u, bool sgn,
                                              float tau)
{
    if (u < (unsigned long long)BG3_EXP_LEN) return exp_steps(n, (uint32_t)u, tau);
    const float x = (sgn ? (float)(long long)u : (float)u) * n.dt;
    return exp_cr(-x / tau);
}

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
// One N(0,1) value by the Box-Muller transform of two 24-bit uniforms.
__device__ __forceinline__ float normal_device(uint32_t seed, unsigned long long step, int i)
{
    uint32_t c[4] = {(uint32_t)i, (uint32_t)step, (uint32_t)(step >> 32), 0u};
    philox4x32_10(c, seed, seed ^ 0x5bd1e995u);
    float u1 = ((float)(c[0] >> 8) + 0.5f) * (1.0f / 16777216.0f);  // (0,1)
    float u2 = (float)(c[1] >> 8) * (1.0f / 16777216.0f);           // [0,1)
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

__device__ __forceinline__ void set_err(const NetDev &n, uint32_t bit) { atomicOr(n.err, bit); }

// A store to global memory as such (st.global, the default write-back policy).  The batched
// kernels read their network's descriptor from shared memory; a plain store through a pointer
// taken from it is a generic store, which as far as the compiler knows may write shared memory,
// so every descriptor field would be read again after it.
template <typename T>
__device__ __forceinline__ void gst(T *p, T v)
{
    __stwb(p, v);
}

// ---- exact float <-> double conversions on the integer pipe ---------------------------------
// GB300's FP64 pipe is narrow and the Izhikevich update (which the reference evaluates partly in
// double) is bound by it; its conversions are done with integer operations instead.  Both are
// exact restatements of IEEE 754: widening a normal float only re-biases the exponent (+896) and
// shifts the mantissa; narrowing rounds the 52-bit mantissa to 23 bits, to nearest, ties to even,
// with the carry into the exponent.  Zero, subnormal, infinite and NaN inputs, and results
// outside the normal float range, take the hardware conversion.
__device__ __forceinline__ double f2d_exact(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)f;
    const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    const uint32_t lo = b << 29;
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ float d2f_rn(double d)
{
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e < 1 || e > 254) return (float)d;
    // 52-bit mantissa m = [hi 20 bits][lo 32 bits]; keep the top 23, round on the other 29
    const uint32_t mhi = hi & 0xfffffu;
    uint32_t m23 = (mhi << 3) | (lo >> 29);
    const uint32_t rest = lo & 0x1fffffffu;  // 29 dropped bits
    const uint32_t half = 0x10000000u;
    uint32_t bits = (hi & 0x80000000u) | ((uint32_t)e << 23) | m23;
    if (rest > half || (rest == half && (m23 & 1u))) bits += 1u;  // may carry into the exponent
    if (((bits >> 23) & 0xffu) == 0xffu) return (float)d;           // rounded up to infinity
    return __uint_as_float(bits);
}

// ---- IEEE 754 binary64 add and multiply on the integer pipe ---------------------------------
// The Izhikevich update evaluates part of its expression in double (as the reference does);
// GB300's FP64 pipe is a small fraction of its FP32 rate, so these few operations are restated
// in integer arithmetic: a finite nonzero double is (-1)^s * m * 2^(e - 52) with a 53-bit
// m in [2^52, 2^53); products are formed exactly (106 bits) and sums with 10 guard bits plus a
// sticky bit, then rounded to nearest, ties to even — the definition of IEEE 754 rounding, so the
// results are the hardware's bit for bit.  Zero is m = 0.  Anything else (subnormal, infinite,
// NaN, or an exponent leaving the normal range) sets ok = false and the caller recomputes with
// hardware doubles.
struct SoftD {
    uint64_t m;
    int32_t e;
    uint32_t s;
};

__device__ __forceinline__ SoftD sd_from_float(float f, bool &ok)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t ex = (b >> 23) & 0xffu, fr = b & 0x7fffffu;
    SoftD r;
    r.s = b >> 31;
    if (ex == 0u) {
        if (fr) ok = false;  // subnormal
        r.m = 0;
        r.e = 0;
        return r;
    }
    if (ex == 0xffu) ok = false;
    r.m = (uint64_t)(fr | 0x800000u) << 29;
    r.e = (int32_t)ex - 127;
    return r;
}

__device__ __forceinline__ SoftD sd_from_double(double x, bool &ok)
{
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const uint32_t ex = (uint32_t)(b >> 52) & 0x7ffu;
    const uint64_t fr = b & 0xfffffffffffffull;
    SoftD r;
    r.s = (uint32_t)(b >> 63);
    if (ex == 0u) {
        if (fr) ok = false;
        r.m = 0;
        r.e = 0;
        return r;
    }
    if (ex == 0x7ffu) ok = false;
    r.m = fr | (1ull << 52);
    r.e = (int32_t)ex - 1023;
    return r;
}

__device__ __forceinline__ void sd_round(SoftD &r, uint64_t rem, uint64_t half, bool &ok)
{
    if (rem > half || (rem == half && (r.m & 1ull))) {
        r.m += 1ull;
        if (r.m == (1ull << 53)) {
            r.m >>= 1;
            r.e += 1;
        }
    }
    if (r.e > 1023 || r.e < -1022) ok = false;
}

__device__ __forceinline__ SoftD sd_mul(SoftD a, SoftD b, bool &ok)
{
    SoftD r;
    r.s = a.s ^ b.s;
    if (a.m == 0 || b.m == 0) {
        r.m = 0;
        r.e = 0;
        return r;
    }
    const uint64_t lo = a.m * b.m, hi = __umul64hi(a.m, b.m);  // product in [2^104, 2^106)
    const int sh = (hi >> 41) ? 53 : 52;
    r.e = a.e + b.e + (sh - 52);
    r.m = (hi << (64 - sh)) | (lo >> sh);
    const uint64_t rem = lo & ((1ull << sh) - 1ull);
    sd_round(r, rem, 1ull << (sh - 1), ok);
    return r;
}

__device__ __forceinline__ SoftD sd_add(SoftD a, SoftD b, bool &ok)
{
    if (b.m == 0) {
        if (a.m == 0) a.s &= b.s;  // +0 + -0 = +0, -0 + -0 = -0
        return a;
    }
    if (a.m == 0) return b;
    // A: the operand of larger magnitude
    if (b.e > a.e || (b.e == a.e && b.m > a.m)) {
        const SoftD t = a;
        a = b;
        b = t;
    }
    const int d = a.e - b.e;
    const uint64_t ma = a.m << 10;  // leading bit at 62
    uint64_t mb = b.m << 10;
    if (d >= 63) {
        mb = 1ull;  // only the sticky bit survives
    } else if (d > 0) {
        const uint64_t lost = mb & ((1ull << d) - 1ull);
        mb = (mb >> d) | (lost ? 1ull : 0ull);
    }
    SoftD r;
    r.s = a.s;
    r.e = a.e;
    uint64_t S;
    if (a.s == b.s) {
        S = ma + mb;
        if (S >> 63) {
            S = (S >> 1) | (S & 1ull);
            r.e += 1;
        }
    } else {
        S = ma - mb;
        if (S == 0) {  // exact cancellation gives +0 in round-to-nearest
            r.m = 0;
            r.e = 0;
            r.s = 0;
            return r;
        }
        const int k = __clzll((long long)S) - 1;  // bring the leading bit back to 62
        S <<= k;
        r.e -= k;
    }
    r.m = S >> 10;
    sd_round(r, S & 0x3ffull, 0x200ull, ok);
    return r;
}

// (float) of the double, rounded to nearest, ties to even.
__device__ __forceinline__ float sd_to_float(SoftD a, bool &ok)
{
    if (a.m == 0) return __uint_as_float(a.s << 31);
    uint32_t m = (uint32_t)(a.m >> 29);
    const uint64_t rem = a.m & ((1ull << 29) - 1ull);
    int e = a.e;
    if (rem > (1ull << 28) || (rem == (1ull << 28) && (m & 1u))) {
        m += 1u;
        if (m == (1u << 24)) {
            m >>= 1;
            e += 1;
        }
    }
    if (e < -126 || e > 127) {
        ok = false;
        return 0.0f;
    }
    return __uint_as_float((a.s << 31) | ((uint32_t)(e + 127) << 23) | (m & 0x7fffffu));
}

// ---- neuron update (shared by the standalone kernels and the sweep epilogues) ---------------
enum { BR_REFRACTORY = 0, BR_FIRE = 1, BR_INTEGRATE = 2 };

// The values one neuron's update reads, loaded together with independent loads (neuron_load) so
// that their latency overlaps other work — in the sweeps, the synapse loads of the same step.
struct NeuronIn {
    float Vm, Vthresh, Trefract, I0, Inoise, C1, C2;
    int32_t refr;
    float A, B, Cc, Dd, u, C3;          // Izhikevich
    int32_t reg_shift;                  // regular input
    float reg_value;
    int32_t nisi;                       // Poisson input
    uint32_t q;
    float ipsr, idec;
    uint8_t pmask, idelay;
};

__device__ __forceinline__ void neuron_load(const NetDev &n, int i, NeuronIn &x)
{
    x.Vm = n.Vm[i];
    x.Vthresh = n.Vthresh[i];
    x.refr = n.refr[i];
    x.Trefract = n.Trefract[i];
    x.I0 = n.I0[i];
    x.Inoise = n.Inoise[i];
    x.C2 = n.C2[i];
    if (n.neuron_kind == 1) {
        x.A = n.Aconst[i];
        x.B = n.Bconst[i];
        x.Cc = n.Cconst[i];
        x.Dd = n.Dconst[i];
        x.u = n.u_izh[i];
        x.C3 = n.C3[i];
    } else {
        x.C1 = n.C1[i];
    }
    if (n.input_kind == 1) {
        x.reg_shift = n.reg_shift[i];
        x.reg_value = n.reg_values[i];
    } else if (n.input_kind == 2) {
        x.pmask = n.pois_mask[i];
        x.nisi = n.pois_nisi[i];
        x.q = n.in_queue[i];
        x.ipsr = n.in_psr[i];
        x.idec = n.in_decay[i];
        x.idelay = n.in_delay[i];
    }
}

// AllLIFNeurons::advanceNeuron branch selection (Neurons/AllLIFNeurons.cpp:31-35; the same for
// AllIZHNeurons, Neurons/AllIZHNeurons.cpp:577-583).
__device__ __forceinline__ int neuron_branch(const NeuronIn &x)
{
    if (x.refr > 0) return BR_REFRACTORY;
    if (x.Vm >= x.Vthresh) return BR_FIRE;
    return BR_INTEGRATE;
}

// AllLIFNeurons::advanceNeuron / fire and AllSpikingNeurons::fire
// (Neurons/AllLIFNeurons.cpp:20-77, Neurons/AllSpikingNeurons.cpp:155-172), and for Izhikevich
// neurons AllIZHNeurons::advanceNeuron / fire (Neurons/AllIZHNeurons.cpp:570-655), with the
// summation point value passed in.  Each float operation rounds on its own (-fmad=false) and the
// double promotions of the reference's expressions are kept.  Returns true when the neuron
// fired.  The caller stores sp = 0 afterwards.
// The Izhikevich update's double expression on the FP64 pipe: Vb = (float)(v + C3 (0.04 v v +
// (double)(5 v) + 140 - u)), then (float)((double)Vb * 0.001 + (double)(C2 sp)).
__device__ __forceinline__ float izh_v_fp64(float Vint, float u, float C3, float c2sp)
{
    const double v = (double)Vint;
    const float Vh = (float)(v + (double)C3 * (0.04 * v * v + (double)(5.0f * Vint) + 140.0 - (double)u));
    return (float)((double)Vh * 0.001 + (double)c2sp);
}

// ---- the Izhikevich double expression in float-float arithmetic ------------------------------
// A float-float value is hi + lo with |lo| <= ulp(hi) / 2 (Dekker, "A floating-point technique
// for extending the available precision", 1971; Knuth's two-sum): about 48 significant bits, kept
// with FP32 additions and fused multiply-adds (each fmaf rounds once, so two_prod's error term is
// exact; -fmad=false stops only the contraction of separate operations).  The chain of the
// reference's double operations is evaluated this way to within a bound E of the reference's own
// double result; where that result's float rounding is certain (the value lies more than E away
// from every rounding boundary, the midpoints between floats) the float is returned, and
// otherwise ok = false and the caller evaluates the expression in hardware FP64.  The same bits
// as the double evaluation, with the FP64 pipe used only for the rare uncertain values.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b)
{
    const float s = a + b, bb = s - a;
    return FF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b)  // |a| >= |b| or a == 0
{
    const float s = a + b;
    return FF{s, b - (s - a)};
}
__device__ __forceinline__ FF ff_add_f(FF a, float b)
{
    FF s = ff_two_sum(a.hi, b);
    s.lo = s.lo + a.lo;
    return ff_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ FF ff_mul_f(FF a, float b)
{
    const float p = a.hi * b;
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return ff_fast_two_sum(p, e);
}
// Rounds a float-float value to float when no rounding boundary lies within err of it.
__device__ __forceinline__ bool ff_round(FF a, float err, float &out)
{
    const uint32_t m = __float_as_uint(a.hi) & 0x7fffffffu;
    if (m < 0x00800001u || m >= 0x7f000000u || !(err < 1e30f)) return false;  // tiny, huge, NaN
    const float up = __uint_as_float(m + 1u) - __uint_as_float(m);    // gap above |hi|
    const float dn = __uint_as_float(m) - __uint_as_float(m - 1u);    // gap below |hi|
    const bool neg = (__float_as_uint(a.hi) >> 31) != 0u;
    // distances from hi + lo to the midpoints above and below hi (on the real line)
    const float half_hi = 0.5f * (neg ? dn : up), half_lo = 0.5f * (neg ? up : dn);
    if (half_hi - a.lo <= err || half_lo + a.lo <= err) return false;
    out = a.hi;
    return true;
}

// (float)(v + C3 (0.04 v v + (double)(5 v) + 140 - u)) and (float)((double)Vb * 0.001 + c2sp)
// as izh_v_fp64 computes them, from float-float arithmetic: the constants 0.04 and 0.001 as
// three floats (exact to ~2^-72); every operation of the chain adds at most ~2^-46 of the
// magnitudes it combines and the reference's seven double roundings ~2^-53 each, so
// E = 2^-40 x (|C3| x M + |Vb|), M = 0.04 v^2 + 5 |v| + 140 + |u|, bounds the distance to the
// reference's double with a wide margin (and likewise for the second expression).
__device__ __forceinline__ float izh_v_ff(float Vint, float u, float C3, float c2sp, bool &ok)
{
    // the double constants split into three floats each (their sum is the double exactly)
    constexpr float K04H = (float)0.04, K04M = (float)(0.04 - (double)K04H),
                    K04L = (float)(0.04 - (double)K04H - (double)K04M);
    constexpr float K001H = (float)0.001, K001M = (float)(0.001 - (double)K001H),
                    K001L = (float)(0.001 - (double)K001H - (double)K001M);
    ok = true;
    if (!(fabsf(Vint) < 1e4f) || !(fabsf(u) < 1e4f) || !(fabsf(C3) < 1e4f) || !(fabsf(c2sp) < 1e4f)) {
        ok = false;
        return 0.0f;
    }
    FF t = ff_mul_f(FF{K04H, K04M}, Vint);
    t.lo = __fmaf_rn(K04L, Vint, t.lo);
    t = ff_mul_f(t, Vint);
    const float v5 = 5.0f * Vint;
    t = ff_add_f(t, v5);
    t = ff_add_f(t, 140.0f);
    t = ff_add_f(t, -u);
    t = ff_mul_f(t, C3);
    t = ff_add_f(t, Vint);
    const float M = 0.04f * Vint * Vint + fabsf(v5) + 140.0f + fabsf(u);
    float Vb;
    if (!ff_round(t, (fabsf(C3) * M + fabsf(t.hi)) * 0x1p-40f, Vb)) {
        ok = false;
        return 0.0f;
    }
    FF w = ff_mul_f(FF{K001H, K001M}, Vb);
    w.lo = __fmaf_rn(K001L, Vb, w.lo);
    w = ff_add_f(w, c2sp);
    float Vnew;
    if (!ff_round(w, (fabsf(Vb) * 0.001f + fabsf(c2sp)) * 0x1p-40f, Vnew)) {
        ok = false;
        return 0.0f;
    }
    return Vnew;
}

// How a neuron's Izhikevich double expression is evaluated: the integer-pipe restatement, the
// hardware FP64 pipe, or float-float arithmetic with the FP64 pipe for uncertain roundings (the
// same bits every way).
enum { IZH_SOFT = 0, IZH_HW = 1, IZH_FF = 2 };
__device__ __forceinline__ int izh_mode(const NetDev &n, int i)
{
    if (n.izh_hw_every < 0) return IZH_FF;
    if (n.izh_hw_every > 0 && ((i >> 5) % n.izh_hw_every) == 0) return IZH_HW;
    return IZH_SOFT;
}

// mode: IZH_SOFT, IZH_HW or IZH_FF (izh_mode); the same bits every way.  FFOK = false compiles
// the float-float branch out (IZH_FF then takes the FP64 pipe), for kernels without registers
// to spare.
template <bool FFOK = true>
__device__ __forceinline__ bool neuron_apply(const NetDev &n, int i, const NeuronIn &x, int br,
                                             float sp, float noise, unsigned long long t,
                                             int mode = IZH_SOFT)
{
    const bool izh = n.neuron_kind == 1;
    if (br == BR_REFRACTORY) {
        gst(&n.refr[i], x.refr - 1);
        return false;
    }
    if (br == BR_FIRE) {
        int cnt = n.spikeCount[i];
        int idx = (cnt + n.spikeCountOffset[i]) % n.max_spikes;
        gst(&n.history[(size_t)i * n.max_spikes + idx], t);
        cnt += 1;
        gst(&n.spikeCount[i], cnt);
        if (cnt >= n.max_spikes) set_err(n, ERR_HISTORY_OVERFLOW);
        gst(&n.refr[i], (int)((double)(x.Trefract / n.dt) + 0.5));
        if (izh) {
            gst(&n.Vm[i], (float)((double)x.Cc * 0.001));
            gst(&n.u_izh[i], x.u + x.Dd);
        } else {
            gst(&n.Vm[i], n.Vreset[i]);
        }
        return true;
    }
    sp = sp + x.I0;
    sp = sp + noise * x.Inoise;
    if (izh) {
        // Vm in mV; dv = C3 (0.04 v^2 + 5 v + 140 - u) evaluated in double, du = C3 a (b v - u)
        const float Vint = x.Vm * 1000.0f;
        const float u = x.u, C3 = x.C3;
        // Vb = (float)(v + C3 * (0.04 v v + (double)(5 v) + 140 - u)), then
        // Vm = (float)((double)Vb * 0.001 + (double)(C2 sp)), each double operation rounded once
        // the double constants 0.04, 140.0 and 0.001 as (mantissa, exponent, sign)
        float Vnew;
        bool ffok = false;
        if (FFOK && mode == IZH_FF) {
            Vnew = izh_v_ff(Vint, u, C3, x.C2 * sp, ffok);
            if (!ffok) Vnew = izh_v_fp64(Vint, u, C3, x.C2 * sp);  // uncertain rounding
        } else if (mode == IZH_HW || mode == IZH_FF) {
            Vnew = izh_v_fp64(Vint, u, C3, x.C2 * sp);
        } else {
            constexpr SoftD K004 = {0x147ae147ae147bull, -5, 0u};
            constexpr SoftD K140 = {0x11800000000000ull, 7, 0u};
            constexpr SoftD K0001 = {0x10624dd2f1a9fcull, -10, 0u};
            bool ok = true;
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
            w = sd_add(w, sd_from_float(x.C2 * sp, ok), ok);
            Vnew = sd_to_float(w, ok);
            if (!ok) Vnew = izh_v_fp64(Vint, u, C3, x.C2 * sp);  // outside the restated range
        }
        gst(&n.u_izh[i], u + C3 * x.A * (x.B * Vint - u));
        gst(&n.Vm[i], Vnew);
    } else {
        gst(&n.Vm[i], x.C1 * x.Vm + x.C2 * sp);
    }
    return false;
}

// ---- external input, applied to the summation point before the neuron update ----------------
// One Poisson inter-spike interval in steps (HostSInputPoisson.cpp:81-84): exponential with mean
// lambda ms, rejected while U <= exp(-isi^2 / 32).  Injected draws replay the reference's own
// sequence; otherwise a Philox stream keyed by (seed, neuron, draw index).
__device__ __forceinline__ int32_t next_isi(const NetDev &n, int i)
{
    const int32_t k = n.isi_cursor[i];
    gst(&n.isi_cursor[i], k + 1);
    if (n.isi_begin) {
        const int32_t p = n.isi_begin[i] + k;
        if (p < n.isi_begin[i + 1]) return n.isi_vals[p];
        set_err(n, ERR_ISI_EXHAUSTED);
        return 0x3fffffff;
    }
    for (uint32_t a = 0; a < 64; a++) {
        uint32_t c[4] = {(uint32_t)i, (uint32_t)k, a, 0x9e3779b9u};
        philox4x32_10(c, n.pois_seed, n.pois_seed ^ 0x85ebca6bu);
        float u1 = ((float)(c[0] >> 8) + 1.0f) * (1.0f / 16777216.0f);  // (0,1]
        float u2 = (float)(c[1] >> 8) * (1.0f / 16777216.0f);
        float isi = -n.pois_lambda * logf(u1);
        if (u2 > expf(-(isi * isi) / 32.0f)) return (int32_t)((double)((isi / 1000.0f) / n.dt) + 0.5);
    }
    return (int32_t)((double)((n.pois_lambda / 1000.0f) / n.dt) + 0.5);
}

// HostSInputRegular::inputStimulus (Inputs/HostSInputRegular.cpp:59-80) and
// HostSInputPoisson::inputStimulus (Inputs/HostSInputPoisson.cpp:60-94) for neuron i at step t:
// returns the summation point after the input.
__device__ __forceinline__ float input_apply(const NetDev &n, int i, const NeuronIn &x,
                                             unsigned long long t, float sp)
{
    if (n.input_kind == 1) {
        const int cyc = (int)(((unsigned long long)n.reg_c0 + (t - n.reg_t0)) % (unsigned long long)n.reg_cycle);
        const int sh = x.reg_shift;
        if (cyc >= sh && cyc < (sh + n.reg_dur) % n.reg_cycle) sp = sp + x.reg_value;
    } else if (n.input_kind == 2 && x.pmask) {
        int32_t c = x.nisi - 1;
        uint32_t q = x.q;
        if (c <= 0) {
            q |= 1u << ((uint32_t)(t + x.idelay) & 31u);
            c = next_isi(n, i);
        }
        gst(&n.pois_nisi[i], c);
        const uint32_t bit = 1u << ((uint32_t)t & 31u);
        float psr = x.ipsr;
        const float dec = x.idec;
        if (q & bit) {
            q &= ~bit;
            EvSlot e = n.in_ev[i];
            float u = e.u, r = e.r;
            if (e.last != BG3_NO_SPIKE32) ds_update(n, e, (uint32_t)t - e.last, u, r);
            psr = psr + ((e.W / dec) * u * r);
            gst(&n.in_ev[i].u, u);
            gst(&n.in_ev[i].r, r);
            gst(&n.in_ev[i].last, (uint32_t)t);
        }
        gst(&n.in_queue[i], q);
        psr = psr * dec;
        gst(&n.in_psr[i], psr);
        sp = sp + psr;
    }
    return sp;
}

// Append the firing lanes' neuron ids to ring slot (t & 63) (warp-aggregated atomic).
__device__ __forceinline__ void ring_push(const NetDev &n, unsigned long long t, bool fired, int i)
{
    unsigned mask = __ballot_sync(0xffffffffu, fired);
    if (!mask) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    int slot = (int)(t & (BG3_RING - 1));
    int base = 0;
    if (lane == leader) base = atomicAdd(&n.ring_n[slot], __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (fired) {
        int pos = base + __popc(mask & ((1u << lane) - 1));
        if (pos < n.N) gst(&n.ring[(size_t)slot * n.N + pos], i);
        else set_err(n, ERR_SPIKE_LIST);
    }
}
