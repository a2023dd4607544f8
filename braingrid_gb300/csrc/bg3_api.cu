// C-ABI of libbg3: handle lifetime, conversion between the reference's slot layout and the
// device plane layout, and the launch sequences of a step and of an epoch.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "../../include/bg3.h"
#include "bg3_internal.cuh"

namespace bg3 {
void launch_neurons(const NetDev &h, cudaStream_t s);
int neuron_launches(const NetDev &h);
void launch_deliver(const NetDev &h, const LaunchCfg &c, cudaStream_t s);
void launch_sweep(const NetDev &h, const CUtensorMap &tp, const CUtensorMap &tc,
                  const CUtensorMap &tp16, const CUtensorMap &tc16, bool fuse, const LaunchCfg &c,
                  cudaStream_t s);
void launch_neurons_batch(const NetDev *nets, int count, int max_n, cudaStream_t s);
void launch_deliver_batch(int syn_kind, const NetDev *nets, int count, const LaunchCfg &c,
                          cudaStream_t s);
void launch_sweep_batch(const NetDev *nets, const CUtensorMap *maps, const int2 *tiles, int n_thick,
                        int n_thin, bool fuse, const LaunchCfg &c, cudaStream_t s);
bool sweep_is_thin(const NetDev &h, const LaunchCfg &c);
bool small_eligible(const NetDev &h, const LaunchCfg &c);
void launch_small(const NetDev &h, int nsteps, cudaStream_t s);
void launch_growth(const NetDev &h, const NetDev *d_net, int epoch, int add_threads, cudaStream_t s);
void launch_rebuild_maps(const NetDev &h, const NetDev *d_net, cudaStream_t s);
void launch_scale_weights(const NetDev &h, float f, cudaStream_t s);
void launch_record(const NetDev &h, const NetDev *d_net, cudaStream_t s);
}  // namespace bg3

static const int GRAPH_STEPS = 32;  // fused steps captured per CUDA graph replay
static const int SMALL_STEPS = 4096;  // steps per launch of a small network (bg3::launch_small)

// kernels one step launches after its neuron pass: delivery (+ post-spike STDP) and the sweep
static inline int step_kernels(int syn_kind) { return syn_kind >= BG3_SYN_STDP ? 3 : 2; }

struct bg3_net {
    bg3_net_desc desc;
    NetDev h;                 // host copy of the device descriptor
    NetDev *d = nullptr;      // device copy
    cudaStream_t stream = nullptr;
    std::vector<std::pair<void *, size_t>> allocs;  // device allocations and their sizes
    LaunchCfg cfg = LAUNCH_DEFAULT;
    CUtensorMap tm_psr, tm_cls, tm_psr16, tm_cls16;  // 32- and 16-dest sweep boxes
    std::vector<float> dtab;  // decay factor per decay class
    std::vector<int> ltab;    // delay per delay class
    long long noise_cap = 0;
    float *noise_dev = nullptr;
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float ms_neurons = 0, ms_fanout = 0, ms_sweep = 0;
    long long launches = 0;
    void *flush_buf = nullptr, *scrub_buf = nullptr;
    size_t flush_size = 0;
    cudaGraphExec_t graph = nullptr;
    std::vector<std::tuple<int, int, uint32_t, uint32_t>> exp_keys;  // exp tables this net holds
    uint64_t bytes = 0;                                                 // device bytes allocated
};

#define CK(x)                                                                            \
    do {                                                                                 \
        cudaError_t e_ = (x);                                                            \
        if (e_ != cudaSuccess) {                                                         \
            fprintf(stderr, "bg3: %s failed: %s\n", #x, cudaGetErrorString(e_));         \
            return BG3_ECUDA;                                                            \
        }                                                                                \
    } while (0)

template <typename T>
static int dalloc(bg3_net *n, T **p, size_t count, int fill = 0)
{
    void *q = nullptr;
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
        cudaGetLastError();
        return BG3_ENOMEM;
    }
    n->allocs.push_back(std::make_pair(q, bytes));
    n->bytes += bytes;
    if (cudaMemsetAsync(q, fill, bytes, n->stream) != cudaSuccess) return BG3_ECUDA;
    *p = (T *)q;
    return BG3_OK;
}

static void drop_graph(bg3_net *n);
// The step kernels take the descriptor by value (captured into the step graph); the growth
// kernels read the device copy.  Any change drops the captured graph.
static int push_desc(bg3_net *n)
{
    drop_graph(n);
    CK(cudaMemcpyAsync(n->d, &n->h, sizeof(NetDev), cudaMemcpyHostToDevice, n->stream));
    return BG3_OK;
}

template <typename T>
static int h2d(bg3_net *n, T *dst, const T *src, size_t count)
{
    if (!src || !count) return BG3_OK;
    CK(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, n->stream));
    return BG3_OK;
}
template <typename T>
static int d2h(bg3_net *n, T *dst, const T *src, size_t count)
{
    if (!dst || !count) return BG3_OK;
    CK(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, n->stream));
    return BG3_OK;
}

static void drop_graph(bg3_net *n)
{
    if (n->graph) cudaGraphExecDestroy(n->graph);
    n->graph = nullptr;
}

// decay / delay class tables (host copy is the source of truth; pushed on change)
static int push_tables(bg3_net *n)
{
    n->h.n_dcls = (int)n->dtab.size();
    n->h.n_delays = (int)n->ltab.size();
    int rc;
    if ((rc = h2d(n, n->h.dtab, n->dtab.data(), n->dtab.size())) ||
        (rc = h2d(n, n->h.ltab, n->ltab.data(), n->ltab.size())))
        return rc;
    drop_graph(n);
    return push_desc(n);
}
static int decay_class(bg3_net *n, float v)
{
    uint32_t b;
    memcpy(&b, &v, 4);
    for (size_t i = 0; i < n->dtab.size(); i++) {
        uint32_t c;
        memcpy(&c, &n->dtab[i], 4);
        if (c == b) return (int)i;
    }
    if (n->dtab.size() >= BG3_MAX_DCLS) return -1;
    n->dtab.push_back(v);
    return (int)n->dtab.size() - 1;
}
// ---- exp tables ------------------------------------------------------------------------------
// expf(-((float)k * dt) / tau) for k < BG3_EXP_LEN, evaluated by this host's libm in the order
// the reference's DS and STDP code evaluates it (AllDSSynapses.cpp:239-240,
// AllSTDPSynapses.cpp:322,345,370,394).  One device table per (device, dt, tau), shared by all
// networks of the process and freed with the last one.
struct ExpTable {
    void *dev = nullptr;
    int refs = 0;
};
// key: (device, kind, dt bits, tau bits); kind 0 = float expf table, 1 = double exp table
using ExpKey = std::tuple<int, int, uint32_t, uint32_t>;
static std::mutex g_exp_mu;
static std::map<ExpKey, ExpTable> g_exp;

static uint32_t fbits(float v)
{
    uint32_t b;
    memcpy(&b, &v, 4);
    return b;
}

// Registers tau with the network; returns 0, or BG3_ENOMEM / BG3_ECUDA.  A tau that is not
// positive and finite, or one past BG3_MAX_EXPC classes, is left to the device fallback.
// Returns the shared device table of (kind, dt, tau), creating it on first use; the caller
// records the key in n->exp_keys.
template <typename T>
static int exp_table(bg3_net *n, int kind, float tau, int len, const T **out)
{
    int dev = 0;
    CK(cudaGetDevice(&dev));
    const float dt = n->h.dt;
    ExpKey key = std::make_tuple(dev, kind, fbits(dt), fbits(tau));
    std::lock_guard<std::mutex> lock(g_exp_mu);
    ExpTable &t = g_exp[key];
    if (!t.dev) {
        std::vector<T> v(len);
        for (int k = 0; k < len; k++) {
            const float x = (float)k * dt;
            if (kind == 0) v[k] = (T)expf(-x / tau);            // expf(-isi / tau), float isi
            else v[k] = (T)exp(-(double)x / (double)tau);     // exp(-delta / tau), double delta
        }
        if (cudaMalloc(&t.dev, v.size() * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            g_exp.erase(key);
            return BG3_ENOMEM;
        }
        if (cudaMemcpy(t.dev, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(t.dev);
            g_exp.erase(key);
            return BG3_ECUDA;
        }
    }
    t.refs++;
    n->exp_keys.push_back(key);
    *out = (const T *)t.dev;
    return BG3_OK;
}

static int exp_class(bg3_net *n, float tau)
{
    NetDev &h = n->h;
    if (!(tau > 0.0f) || !std::isfinite(tau)) return BG3_OK;
    for (int c = 0; c < h.n_expc; c++)
        if (fbits(h.expc_tau[c]) == fbits(tau)) return BG3_OK;
    if (h.n_expc >= BG3_MAX_EXPC) return BG3_OK;
    const float *tab = nullptr;
    int rc = exp_table<float>(n, 0, tau, BG3_EXP_LEN, &tab);
    if (rc) return rc;
    h.expc_tau[h.n_expc] = tau;
    h.expc_tab[h.n_expc] = tab;
    h.n_expc++;
    return push_desc(n);
}

// Per-type STDP constants: the float tables of tauspre / tauspost and the double tables of
// taupos / tauneg (exp(-delta / taupos), exp(delta / tauneg) over a 3 tau window).
// The weight-dependence exponents mu+ and mu- must be 0 (the reference's only values,
// Synapses/AllSTDPSynapses.cpp:252-273): the reference raises W to them with the host libm's
// pow, which no device function reproduces bit for bit, so other values are refused
// (BG3_EUNSUPPORTED) rather than run with a different rounding.
static int set_stdp_type(bg3_net *n, int type, const StdpConst &in)
{
    if (!(in.mupos == 0.0f) || !(in.muneg == 0.0f)) return BG3_EUNSUPPORTED;
    StdpConst c = in;
    int rc;
    if ((rc = exp_class(n, c.tauspre)) || (rc = exp_class(n, c.tauspost))) return rc;
    c.dpos = c.dneg = nullptr;
    c.dlen_pos = c.dlen_neg = 0;
    if (c.taupos > 0.0f && std::isfinite(c.taupos)) {
        if ((rc = exp_table<double>(n, 1, c.taupos, BG3_DEXP_LEN, &c.dpos))) return rc;
        c.dlen_pos = BG3_DEXP_LEN;
    }
    if (c.tauneg > 0.0f && std::isfinite(c.tauneg)) {
        if ((rc = exp_table<double>(n, 1, c.tauneg, BG3_DEXP_LEN, &c.dneg))) return rc;
        c.dlen_neg = BG3_DEXP_LEN;
    }
    n->h.stdp[type] = c;
    return push_desc(n);
}

// DS parameter class of (U, D, F): index into the network's table, adding it (with the exp
// tables of D and F) on first use.  Returns the class, or a negative status.
static int param_class(bg3_net *n, float U, float D, float F)
{
    NetDev &h = n->h;
    for (int c = 0; c < h.n_pcls; c++)
        if (fbits(h.p_U[c]) == fbits(U) && fbits(h.p_D[c]) == fbits(D) && fbits(h.p_F[c]) == fbits(F))
            return c;
    if (h.n_pcls >= BG3_MAX_PCLS) return BG3_EUNSUPPORTED;
    const float *xd = nullptr, *xf = nullptr;
    int rc;
    if (D > 0.0f && std::isfinite(D) && (rc = exp_table<float>(n, 0, D, BG3_EXP_LEN, &xd))) return rc;
    if (F > 0.0f && std::isfinite(F) && (rc = exp_table<float>(n, 0, F, BG3_EXP_LEN, &xf))) return rc;
    const int c = h.n_pcls++;
    h.p_U[c] = U;
    h.p_D[c] = D;
    h.p_F[c] = F;
    h.p_xD[c] = xd;
    h.p_xF[c] = xf;
    if ((rc = push_desc(n))) return rc;
    return c;
}

static void exp_release(bg3_net *n)
{
    std::lock_guard<std::mutex> lock(g_exp_mu);
    for (auto &key : n->exp_keys) {
        auto it = g_exp.find(key);
        if (it == g_exp.end()) continue;
        if (--it->second.refs == 0) {
            cudaFree(it->second.dev);
            g_exp.erase(it);
        }
    }
    n->exp_keys.clear();
    n->h.n_expc = 0;
}

static int delay_class(bg3_net *n, int D)
{
    for (size_t i = 0; i < n->ltab.size(); i++)
        if (n->ltab[i] == D) return (int)i;
    if (n->ltab.size() >= BG3_MAX_DELAYS || D < 1 || D > 31) return -1;
    n->ltab.push_back(D);
    return (int)n->ltab.size() - 1;
}

static int make_tensor_maps(bg3_net *n)
{
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess || !fn || q != cudaDriverEntryPointSuccess)
        return BG3_ECUDA;
    auto encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    const NetDev &h = n->h;
    // tile-major planes as 3-D tensors [tiles][Mq quads][32 dests x 4 rows] (psr, floats) and
    // [tiles][Mq quads][32 dests] (classes, 16-bit words of four 4-bit codes); a box is 16 quads
    // of one tile (32 or 16 dests); quads past Mq read as zero and are not written
    const cuuint64_t T = (cuuint64_t)h.ntiles, Q = (cuuint64_t)std::max(h.Mq, 1);
    cuuint64_t dims_f[3] = {128, Q, T}, dims_b[3] = {32, Q, T};
    cuuint64_t st_f[2] = {512, Q * 512}, st_b[2] = {64, Q * 64};
    cuuint32_t box_f[3] = {128, 16, 1}, box_b[3] = {32, 16, 1};
    cuuint32_t box_f16[3] = {64, 16, 1}, box_b16[3] = {16, 16, 1};
    cuuint32_t es[3] = {1, 1, 1};
    struct { CUtensorMap *m; CUtensorMapDataType ty; void *base; cuuint64_t *dims, *st; cuuint32_t *box; } maps[4] = {
        {&n->tm_psr, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, h.psr, dims_f, st_f, box_f},
        {&n->tm_cls, CU_TENSOR_MAP_DATA_TYPE_UINT16, h.dcls, dims_b, st_b, box_b},
        {&n->tm_psr16, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, h.psr, dims_f, st_f, box_f16},
        {&n->tm_cls16, CU_TENSOR_MAP_DATA_TYPE_UINT16, h.dcls, dims_b, st_b, box_b16}};
    for (auto &m : maps)
        if (encode(m.m, m.ty, 3, m.base, m.dims, m.st, m.box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return BG3_ECUDA;
    return BG3_OK;
}

extern "C" {

const char *bg3_status_string(int s)
{
    switch (s) {
    case BG3_OK: return "ok";
    case BG3_EINVAL: return "invalid argument or state";
    case BG3_ENOMEM: return "device allocation failed";
    case BG3_ECUDA: return "CUDA call failed";
    case BG3_ENOISE: return "injected noise stream exhausted";
    case BG3_EDEVICE: return "device error word set";
    case BG3_EUNSUPPORTED: return "unsupported model combination";
    case BG3_ECANCELED: return "job cancelled";
    default: return "unknown status";
    }
}

int bg3_create(const bg3_net_desc *desc, bg3_net **out)
{
    if (!desc || !out) return BG3_EINVAL;
    *out = nullptr;
    const bg3_net_desc &D = *desc;
    if (D.n_neurons <= 0 || D.max_syn_per_neuron < 0 || D.delta_t <= 0 || D.epoch_duration <= 0)
        return BG3_EINVAL;
    if ((((size_t)D.n_neurons + 31) / 32 * 32) * (((size_t)D.max_syn_per_neuron + 3) / 4 * 4) >=
        (1ull << 32))
        return BG3_EINVAL;  // plane positions are 32-bit
    if (D.neuron_kind != BG3_NEURON_LIF && D.neuron_kind != BG3_NEURON_IZH) return BG3_EUNSUPPORTED;
    if (D.synapse_kind < BG3_SYN_SPIKING || D.synapse_kind > BG3_SYN_DYNSTDP) return BG3_EUNSUPPORTED;
    if (D.noise_mode != BG3_NOISE_DEVICE && D.noise_mode != BG3_NOISE_INJECT) return BG3_EINVAL;
    int max_spikes = (int)(D.epoch_duration * (float)D.max_firing_rate);
    if (max_spikes <= 0) return BG3_EINVAL;

    bg3_net *n = new (std::nothrow) bg3_net();
    if (!n) return BG3_ENOMEM;
    n->desc = D;
    if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete n;
        return BG3_ECUDA;
    }
    NetDev &h = n->h;
    memset(&h, 0, sizeof(h));
    const size_t N = (size_t)D.n_neurons;
    const size_t Np = (N + 31) / 32 * 32;
    const size_t Mq = ((size_t)D.max_syn_per_neuron + 3) / 4;
    const size_t S = Np * Mq * 4;
    h.N = D.n_neurons;
    h.Np = (int)Np;
    h.max_syn = D.max_syn_per_neuron;
    h.Mq = (int)Mq;
    h.max_spikes = max_spikes;
    h.neuron_kind = D.neuron_kind;
    h.syn_kind = D.synapse_kind;
    h.noise_mode = D.noise_mode;
    h.noise_seed = D.noise_seed;
    h.dt = D.delta_t;
    h.epoch_duration = D.epoch_duration;
    h.ntiles = (int)(Np / 32);
    h.max_epochs = D.max_epochs;
    h.izh_hw_every = n->cfg.izh_hw_every;
    h.n_burst_bins = (int)((float)D.max_epochs * D.epoch_duration);
    h.n_spike_bins = (int)((float)D.max_epochs * D.epoch_duration * 100.0f);
    int rc = 0;
#define A(ptr, cnt) if ((rc = dalloc(n, &h.ptr, (cnt))) != 0) goto fail;
    A(step, 1) A(sweep_done, 1) A(dstep, 1) A(err, 1) A(noise_cursor, 1)
    A(Vm, N) A(Vthresh, N) A(Vreset, N) A(I0, N) A(Inoise, N) A(C1, N) A(C2, N) A(Trefract, N)
    A(sp, N) A(refr, N) A(spikeCount, N) A(spikeCountOffset, N) A(ntype, N)
    A(ring, N * BG3_RING) A(ring_n, BG3_RING)
    A(psr, S) A(dcls, S / 8) A(lcls, S) A(ev, S) A(src, S) A(stype, S) A(count, N)
    A(dtab, BG3_MAX_DCLS) A(ltab, BG3_MAX_DELAYS)
    A(outBegin, N * BG3_MAX_DELAYS) A(outCount, N * BG3_MAX_DELAYS) A(outFill, N * BG3_MAX_DELAYS)
    A(outMap, S)
    A(radii, N) A(rates, N) A(xloc, N) A(yloc, N) A(grow_exp, (size_t)max_spikes + 1)
    A(grow_rmax, 1)
    A(burstiness, (size_t)std::max(h.n_burst_bins, 1)) A(spikes_hist, (size_t)std::max(h.n_spike_bins, 1))
    A(rates_hist, (size_t)(D.max_epochs + 1) * N) A(radii_hist, (size_t)(D.max_epochs + 1) * N)
    if (D.neuron_kind == BG3_NEURON_IZH) {
        A(Aconst, N) A(Bconst, N) A(Cconst, N) A(Dconst, N) A(u_izh, N) A(C3, N)
    }
#undef A
    if ((rc = dalloc(n, &h.history, N * (size_t)max_spikes, 0xff)) != 0) goto fail;
    if (cudaMalloc((void **)&n->d, sizeof(NetDev)) != cudaSuccess) { rc = BG3_ENOMEM; goto fail; }
    // type constants of createSynapse at this deltaT (Synapses/AllSpikingSynapses.cpp:192-240,
    // AllDSSynapses.cpp:180-218); decay = exp(-deltaT / tau) on the host, as the reference does
    {
        const float tau[4] = {6e-3f, 6e-3f, 3e-3f, 3e-3f};
        const float dly[4] = {0.8e-3f, 0.8e-3f, 0.8e-3f, 1.5e-3f};
        const float U[4] = {0.32f, 0.25f, 0.05f, 0.5f}, Dd[4] = {0.144f, 0.7f, 0.125f, 1.1f},
                    F[4] = {0.06f, 0.02f, 1.2f, 0.05f};
        for (int t = 0; t < 4; t++) {
            h.t_tau[t] = tau[t];
            h.t_dcls[t] = decay_class(n, expf(-D.delta_t / tau[t]));
            h.t_lcls[t] = delay_class(n, (int)(dly[t] / D.delta_t) + 1);
            if (h.t_lcls[t] < 0) { rc = BG3_EINVAL; goto fail; }
            h.t_U[t] = U[t];
            h.t_D[t] = Dd[t];
            h.t_F[t] = F[t];
        }
        h.t_u0 = 0.4f;
        h.t_r0 = 1.0f;
    }
    if ((rc = make_tensor_maps(n)) != 0) goto fail;
    if (cudaMemcpy(n->d, &h, sizeof(NetDev), cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = BG3_ECUDA;
        goto fail;
    }
    for (int t = 0; t < 4 && (h.syn_kind == BG3_SYN_DS || h.syn_kind == BG3_SYN_DYNSTDP); t++) {
        const int c = param_class(n, h.t_U[t], h.t_D[t], h.t_F[t]);
        if (c < 0) { rc = c; goto fail; }
        h.t_pcls[t] = c;
    }
    // AllSTDPSynapses::createSynapse constants (Synapses/AllSTDPSynapses.cpp:256-272)
    for (int t = 0; t < 4 && h.syn_kind >= BG3_SYN_STDP; t++) {
        StdpConst c = {};
        c.Apos = 0.5f; c.Aneg = -0.5f; c.gap = 2e-3f;
        c.tauspost = 75e-3f; c.tauspre = 34e-3f; c.taupos = 15e-3f; c.tauneg = 35e-3f;
        c.Wex = 1.0f; c.mupos = 0.0f; c.muneg = 0.0f; c.useFD = 1;
        if ((rc = set_stdp_type(n, t, c))) goto fail;
    }
    if ((rc = push_tables(n)) != 0) goto fail;
    if (cudaStreamSynchronize(n->stream) != cudaSuccess) { rc = BG3_ECUDA; goto fail; }
    *out = n;
    return BG3_OK;
fail:
    cudaGetLastError();
    bg3_destroy(n);
    return rc;
}

// Device bytes bg3_create allocates for desc, plus an external input's arrays (Poisson 54 B or
// regular 8 B per neuron); mirrors the allocation list of bg3_create.
int64_t bg3_net_footprint(const bg3_net_desc *desc)
{
    if (!desc || desc->n_neurons <= 0 || desc->max_syn_per_neuron < 0 || desc->delta_t <= 0 ||
        desc->epoch_duration <= 0)
        return BG3_EINVAL;
    const bg3_net_desc &D = *desc;
    const uint64_t N = (uint64_t)D.n_neurons;
    const uint64_t Np = (N + 31) / 32 * 32;
    const uint64_t S = Np * (((uint64_t)D.max_syn_per_neuron + 3) / 4) * 4;
    const int64_t ms = (int64_t)(D.epoch_duration * (float)D.max_firing_rate);
    if (ms <= 0) return BG3_EINVAL;
    const uint64_t nb = (uint64_t)std::max((int)((float)D.max_epochs * D.epoch_duration), 1);
    const uint64_t ns = (uint64_t)std::max((int)((float)D.max_epochs * D.epoch_duration * 100.0f), 1);
    const uint64_t E1 = (uint64_t)D.max_epochs + 1;
    uint64_t b = 8 + 4 + 8 + 4 + 8;                       // step, sweep_done, dstep, err, cursor
    b += N * (9 * 4 + 3 * 4 + 1);                                  // neuron SoA + ntype
    b += N * BG3_RING * 4 + BG3_RING * 4;                          // spike ring
    b += S * (4 + 1 + sizeof(EvSlot) + 4 + 1 + 4) + S / 2 + N * 4; // planes, outMap, count
    b += BG3_MAX_DCLS * 4 + BG3_MAX_DELAYS * 4 + 3 * N * BG3_MAX_DELAYS * 4;
    b += 4 * N * 4 + ((uint64_t)ms + 1) * 4;                       // growth arrays, grow_exp
    b += (nb + ns) * 4 + 2 * E1 * N * 4;                           // recorder
    if (D.neuron_kind == BG3_NEURON_IZH) b += 6 * N * 4;
    b += N * (uint64_t)ms * 8;                                     // spike history
    b += sizeof(NetDev) + 54 * N;                                  // descriptor, input
    return (int64_t)b;
}

uint64_t bg3_net_bytes(bg3_net *n) { return n ? n->bytes + sizeof(NetDev) : 0; }

int bg3_set_device(int32_t device)
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return BG3_ECUDA;
    }
    if (device < 0 || device >= count) return BG3_EINVAL;
    CK(cudaSetDevice(device));
    return BG3_OK;
}

int bg3_get_desc(bg3_net *n, bg3_net_desc *desc)
{
    if (!n || !desc) return BG3_EINVAL;
    *desc = n->desc;
    return BG3_OK;
}

int bg3_destroy(bg3_net *n)
{
    if (!n) return BG3_EINVAL;
    if (n->stream) cudaStreamSynchronize(n->stream);
    drop_graph(n);
    exp_release(n);
    for (auto &a : n->allocs)
        if (a.first) cudaFree(a.first);
    if (n->d) cudaFree(n->d);
    if (n->noise_dev) cudaFree(n->noise_dev);
    if (n->flush_buf) cudaFree(n->flush_buf);
    if (n->scrub_buf) cudaFree(n->scrub_buf);
    for (int i = 0; i < 4; i++)
        if (n->ev[i]) cudaEventDestroy(n->ev[i]);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
    return BG3_OK;
}

// ---- uploads --------------------------------------------------------------------------------
int bg3_upload_lif(bg3_net *n, const bg3_lif_arrays *a)
{
    if (!n || !a) return BG3_EINVAL;
    size_t N = n->h.N;
    int rc;
    NetDev &h = n->h;
    if ((rc = h2d(n, h.Vm, a->Vm, N)) || (rc = h2d(n, h.Vthresh, a->Vthresh, N)) ||
        (rc = h2d(n, h.Vreset, a->Vreset, N)) || (rc = h2d(n, h.I0, a->I0, N)) ||
        (rc = h2d(n, h.Inoise, a->Inoise, N)) || (rc = h2d(n, h.C1, a->C1, N)) ||
        (rc = h2d(n, h.C2, a->C2, N)) || (rc = h2d(n, h.Trefract, a->Trefract, N)) ||
        (rc = h2d(n, h.sp, a->summation, N)) || (rc = h2d(n, h.refr, a->nStepsInRefr, N)) ||
        (rc = h2d(n, h.spikeCount, a->spikeCount, N)) ||
        (rc = h2d(n, h.spikeCountOffset, a->spikeCountOffset, N)) ||
        (rc = h2d(n, (uint64_t *)h.history, a->history, N * (size_t)h.max_spikes)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_upload_izh(bg3_net *n, const bg3_izh_arrays *a)
{
    if (!n || !a) return BG3_EINVAL;
    if (n->h.neuron_kind != BG3_NEURON_IZH) return BG3_EUNSUPPORTED;
    size_t N = n->h.N;
    NetDev &h = n->h;
    int rc;
    if ((rc = h2d(n, h.Aconst, a->Aconst, N)) || (rc = h2d(n, h.Bconst, a->Bconst, N)) ||
        (rc = h2d(n, h.Cconst, a->Cconst, N)) || (rc = h2d(n, h.Dconst, a->Dconst, N)) ||
        (rc = h2d(n, h.u_izh, a->u, N)) || (rc = h2d(n, h.C3, a->C3, N)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_upload_layout(bg3_net *n, const float *x, const float *y, const int32_t *ntype)
{
    if (!n || !x || !y || !ntype) return BG3_EINVAL;
    size_t N = n->h.N;
    std::vector<int8_t> t(N);
    for (size_t i = 0; i < N; i++) {
        if (ntype[i] != 1 && ntype[i] != 2) return BG3_EINVAL;
        t[i] = (int8_t)ntype[i];
    }
    // the reference's grid (Layouts/Layout.cpp:41-52: xloc = i % width, yloc = i / width)?
    const int W = n->desc.width, H = n->desc.height;
    bool grid = W > 0 && H > 0 && (size_t)W * (size_t)H == N;
    for (size_t i = 0; grid && i < N; i++)
        grid = x[i] == (float)(i % (size_t)W) && y[i] == (float)(i / (size_t)W);
    n->h.grid_w = grid ? W : 0;
    n->h.grid_h = grid ? H : 0;
    int rc;
    if ((rc = h2d(n, n->h.xloc, x, N)) || (rc = h2d(n, n->h.yloc, y, N)) ||
        (rc = h2d(n, n->h.ntype, t.data(), N)) || (rc = push_desc(n)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_set_type_constants(bg3_net *n, const bg3_type_constants *c)
{
    if (!n || !c) return BG3_EINVAL;
    for (int t = 0; t < 4; t++) {
        int dc = decay_class(n, c->decay[t]);
        int lc = delay_class(n, c->total_delay[t]);
        if (dc < 0 || lc < 0) return BG3_EINVAL;
        n->h.t_tau[t] = c->tau[t];
        n->h.t_dcls[t] = dc;
        n->h.t_lcls[t] = lc;
        n->h.t_U[t] = c->U[t];
        n->h.t_D[t] = c->D[t];
        n->h.t_F[t] = c->F[t];
        if (n->h.syn_kind == BG3_SYN_DS || n->h.syn_kind == BG3_SYN_DYNSTDP) {
            const int pc = param_class(n, c->U[t], c->D[t], c->F[t]);
            if (pc < 0) return pc;
            n->h.t_pcls[t] = pc;
        }
    }
    n->h.t_u0 = c->u0;
    n->h.t_r0 = c->r0;
    int rc = push_tables(n);
    if (rc) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

// Converts the reference's per-synapse delay queues into the device's spike ring and birth
// steps.  Queue bit b of a synapse with read index di is checked (delivered) o = (b - di) & 31
// steps from now, so its source fired at tf = step + o - D.  A synapse that lacks the bit of a
// spike its source emitted while its queue would have recorded it did not exist yet: its birth
// step is step - di (the reference's delayIdx counts steps since creation, mod 32).
int bg3_upload_synapses(bg3_net *n, const bg3_synapse_arrays *a, uint64_t step)
{
    if (!n || !a || !a->in_use || !a->src || !a->type || !a->W || !a->psr || !a->decay ||
        !a->delayQueue || !a->delayIdx || !a->total_delay)
        return BG3_EINVAL;
    if (step >= 0xffffff00ull) return BG3_EINVAL;
    const size_t N = n->h.N, Np = n->h.Np, M = n->h.max_syn, S = Np * (size_t)n->h.Mq * 4;
    const bool ds = n->h.syn_kind == BG3_SYN_DS || n->h.syn_kind == BG3_SYN_DYNSTDP;
    if (ds && (!a->U || !a->D || !a->F || !a->u || !a->r || !a->lastSpike)) return BG3_EINVAL;
    std::vector<float> psr(S, 0.f);
    std::vector<uint32_t> dc(S / 8, 0u);
    std::vector<uint8_t> lc(S, 0);
    std::vector<EvSlot> ev(S);
    std::vector<int32_t> src(S, 0);
    std::vector<int8_t> st(S, 0);
    std::vector<uint32_t> count(N, 0u);
    memset(ev.data(), 0, S * sizeof(EvSlot));
    // fired[s] bit j: neuron s fired at step - 1 - j (j < 32), from the queues
    std::vector<uint32_t> fired(N, 0u);
    uint32_t seenU = 0xffffffffu, seenD = 0xffffffffu, seenF = 0xffffffffu;  // last (U, D, F)
    int seenC = 0;
    for (size_t d = 0; d < N; d++) {
        size_t c = 0;
        while (c < M && a->in_use[d * M + c]) c++;
        for (size_t k = c; k < M; k++)
            if (a->in_use[d * M + k]) return BG3_EINVAL;  // in-use slots must be a prefix
        if (a->counts && a->counts[d] != c) return BG3_EINVAL;
        count[d] = (uint32_t)c;
        for (size_t k = 0; k < c; k++) {
            size_t i = d * M + k, p = slot_pos((int)k, (int)d, (int)n->h.Mq);
            int D = a->total_delay[i], di = a->delayIdx[i];
            if (a->src[i] < 0 || (size_t)a->src[i] >= N || a->type[i] < 0 || a->type[i] > 3 ||
                D < 1 || D > 31 || di < 0 || di > 31)
                return BG3_EINVAL;
            int dcl = decay_class(n, a->decay[i]), lcl = delay_class(n, D);
            if (dcl < 0) return BG3_EUNSUPPORTED;  // more than BG3_MAX_DCLS decay factors
            if (lcl < 0) return BG3_EINVAL;
            psr[p] = a->psr[i];
            cls_put(dc.data(), p, (uint32_t)dcl);
            lc[p] = (uint8_t)lcl;
            src[p] = a->src[i];
            st[p] = (int8_t)a->type[i];
            EvSlot &e = ev[p];
            e.W = a->W[i];
            e.born = (uint32_t)(step - (uint64_t)di - 32u);
            e.dcls = (uint8_t)dcl;
            if (ds) {
                e.u = a->u[i];
                e.r = a->r[i];
                if (fbits(a->U[i]) != seenU || fbits(a->D[i]) != seenD || fbits(a->F[i]) != seenF) {
                    seenC = param_class(n, a->U[i], a->D[i], a->F[i]);
                    if (seenC < 0) return seenC;
                    seenU = fbits(a->U[i]);
                    seenD = fbits(a->D[i]);
                    seenF = fbits(a->F[i]);
                }
                e.pcls = (uint8_t)seenC;
                uint64_t ls = a->lastSpike[i];
                if (ls != BG3_ULONG_MAX && ls >= BG3_NO_SPIKE32) return BG3_EINVAL;
                e.last = (ls == BG3_ULONG_MAX) ? BG3_NO_SPIKE32 : (uint32_t)ls;
            } else {
                e.last = BG3_NO_SPIKE32;
            }
            uint32_t q = a->delayQueue[i];
            for (int b = 0; b < 32; b++) {
                if (!((q >> b) & 1u)) continue;
                int o = (b - di) & 31;
                if (o >= D || (uint64_t)(D - o) > step) return BG3_EINVAL;  // not a past spike
                fired[a->src[i]] |= 1u << (D - o - 1);
            }
        }
    }
    for (size_t d = 0; d < N; d++) {
        for (size_t k = 0; k < count[d]; k++) {
            size_t i = d * M + k, p = slot_pos((int)k, (int)d, (int)n->h.Mq);
            int D = a->total_delay[i], di = a->delayIdx[i];
            uint32_t f = fired[a->src[i]], q = a->delayQueue[i];
            for (int j = 0; j < D; j++) {
                if (!((f >> j) & 1u)) continue;
                int o = D - 1 - j;  // pending spike from step - 1 - j, due in o steps
                if ((q >> ((di + o) & 31)) & 1u) continue;
                // missing: the synapse was created after that spike (step - di > step - 1 - j)
                if (di > j) return BG3_EINVAL;
                ev[p].born = (uint32_t)(step - (uint64_t)di);
            }
        }
    }
    std::vector<int32_t> ring(N * BG3_RING, 0), ring_n(BG3_RING, 0);
    for (size_t s = 0; s < N; s++)
        for (int j = 0; j < 32; j++)
            if ((fired[s] >> j) & 1u) {
                int slot = (int)((step - 1 - (uint64_t)j) & (BG3_RING - 1));
                ring[(size_t)slot * N + ring_n[slot]++] = (int32_t)s;
            }
    NetDev &h = n->h;
    int rc;
    if ((rc = push_tables(n))) return rc;
    if ((rc = h2d(n, h.psr, psr.data(), S)) || (rc = h2d(n, h.dcls, dc.data(), S / 8)) ||
        (rc = h2d(n, h.lcls, lc.data(), S)) || (rc = h2d(n, h.ev, ev.data(), S)) ||
        (rc = h2d(n, h.src, src.data(), S)) || (rc = h2d(n, h.stype, st.data(), S)) ||
        (rc = h2d(n, h.count, count.data(), N)) || (rc = h2d(n, h.ring, ring.data(), ring.size())) ||
        (rc = h2d(n, h.ring_n, ring_n.data(), ring_n.size())))
        return rc;
    unsigned long long s64 = step;
    CK(cudaMemcpyAsync(h.step, &s64, sizeof(s64), cudaMemcpyHostToDevice, n->stream));
    CK(cudaMemcpyAsync(h.dstep, &s64, sizeof(s64), cudaMemcpyHostToDevice, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    bg3::launch_rebuild_maps(h, n->d, n->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_upload_growth(bg3_net *n, const bg3_growth_params *p, const float *radii,
                      const float *rates)
{
    if (!n || (!p && !radii && !rates)) return BG3_EINVAL;
    NetDev &h = n->h;
    size_t N = h.N;
    int rc;
    if (p) {
        h.g_epsilon = p->epsilon; h.g_beta = p->beta; h.g_rho = p->rho;
        h.g_target_rate = p->target_rate; h.g_min_radius = p->min_radius;
        h.g_start_radius = p->start_radius; h.g_max_rate = p->max_rate;
        // ConnGrowth::updateConns' exp((epsilon - rate / maxRate) / beta) for rate = count / T
        // (Connections/ConnGrowth.cpp:300-306), one value per possible spike count
        std::vector<float> ge((size_t)h.max_spikes + 1);
        for (int c = 0; c <= h.max_spikes; c++) {
            const float rate = (float)c / h.epoch_duration;
            ge[c] = expf((h.g_epsilon - rate / h.g_max_rate) / h.g_beta);
        }
        if ((rc = h2d(n, h.grow_exp, ge.data(), ge.size()))) return rc;
    }
    if ((rc = h2d(n, h.radii, radii, N)) || (rc = h2d(n, h.rates, rates, N))) return rc;
    // recorder row 0 holds the start values (XmlGrowthRecorder::initDefaultValues / initValues)
    if ((rc = h2d(n, h.radii_hist, radii, N)) || (rc = h2d(n, h.rates_hist, rates, N))) return rc;
    if ((rc = push_desc(n))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_upload_weights(bg3_net *n, const float *Wref)
{
    if (!n || !Wref) return BG3_EINVAL;
    const size_t N = n->h.N, Np = n->h.Np, M = n->h.max_syn, S = Np * (size_t)n->h.Mq * 4;
    std::vector<uint32_t> count(N);
    std::vector<EvSlot> ev(S);
    int rc;
    if ((rc = d2h(n, count.data(), n->h.count, N)) || (rc = d2h(n, ev.data(), n->h.ev, S))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    for (size_t d = 0; d < N; d++)
        for (size_t k = 0; k < count[d]; k++) ev[slot_pos((int)k, (int)d, (int)n->h.Mq)].W = Wref[d * M + k];
    if ((rc = h2d(n, n->h.ev, ev.data(), S))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_scale_weights(bg3_net *n, float factor)
{
    if (!n) return BG3_EINVAL;
    bg3::launch_scale_weights(n->h, factor, n->stream);
    n->launches += 1;
    CK(cudaGetLastError());
    return BG3_OK;
}

int bg3_set_noise_mode(bg3_net *n, int32_t mode, uint32_t seed)
{
    if (!n || (mode != BG3_NOISE_DEVICE && mode != BG3_NOISE_INJECT)) return BG3_EINVAL;
    CK(cudaStreamSynchronize(n->stream));
    // an injected stream starts empty: values pushed for the old mode are dropped
    if (n->noise_dev) CK(cudaFree(n->noise_dev));
    n->noise_dev = nullptr;
    n->noise_cap = 0;
    n->h.noise_buf = nullptr;
    n->h.noise_len = 0;
    unsigned long long zero = 0;
    CK(cudaMemcpyAsync(n->h.noise_cursor, &zero, sizeof(zero), cudaMemcpyHostToDevice, n->stream));
    n->h.noise_mode = mode;
    n->h.noise_seed = seed;
    n->desc.noise_mode = mode;
    n->desc.noise_seed = seed;
    int rc = push_desc(n);
    if (rc) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_push_noise(bg3_net *n, const float *v, int64_t cnt)
{
    if (!n || (!v && cnt) || cnt < 0 || n->h.noise_mode != BG3_NOISE_INJECT) return BG3_EINVAL;
    // drop consumed values, then append: always into a fresh buffer (no overlapping copies)
    unsigned long long cur = 0;
    CK(cudaMemcpyAsync(&cur, n->h.noise_cursor, sizeof(cur), cudaMemcpyDeviceToHost, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    long long keep = n->h.noise_len - (long long)cur;
    if (keep < 0) keep = 0;
    long long need = keep + cnt;
    float *old = n->noise_dev;
    float *buf = nullptr;
    if (cudaMalloc(&buf, (size_t)std::max<long long>(need, 1) * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return BG3_ENOMEM;
    }
    if (keep) CK(cudaMemcpyAsync(buf, old + cur, (size_t)keep * sizeof(float), cudaMemcpyDeviceToDevice, n->stream));
    if (cnt) CK(cudaMemcpyAsync(buf + keep, v, (size_t)cnt * sizeof(float), cudaMemcpyHostToDevice, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    if (old) cudaFree(old);
    n->noise_cap = need;
    n->noise_dev = buf;
    n->h.noise_buf = buf;
    n->h.noise_len = need;
    unsigned long long zero = 0;
    CK(cudaMemcpyAsync(n->h.noise_cursor, &zero, sizeof(zero), cudaMemcpyHostToDevice, n->stream));
    int rc = push_desc(n);
    if (rc) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_noise_pending(bg3_net *n, int64_t *pending)
{
    if (!n || !pending) return BG3_EINVAL;
    *pending = 0;
    if (n->h.noise_mode != BG3_NOISE_INJECT || !n->noise_dev) return BG3_OK;
    unsigned long long cur = 0;
    CK(cudaMemcpyAsync(&cur, n->h.noise_cursor, sizeof(cur), cudaMemcpyDeviceToHost, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    const long long left = n->h.noise_len - (long long)cur;
    *pending = left > 0 ? left : 0;
    return BG3_OK;
}

// ---- external input -------------------------------------------------------------------------
int bg3_input_regular(bg3_net *n, const float *values, const int32_t *shifts, int32_t dur,
                      int32_t cycle, int32_t in_cycle)
{
    if (!n || !values || !shifts || dur < 0 || cycle <= 0 || in_cycle < 0 || in_cycle >= cycle)
        return BG3_EINVAL;
    NetDev &h = n->h;
    const size_t N = h.N;
    int rc;
    if (!h.reg_values) {
        if ((rc = dalloc(n, &h.reg_values, N)) || (rc = dalloc(n, &h.reg_shift, N))) return rc;
    }
    if ((rc = h2d(n, h.reg_values, values, N)) || (rc = h2d(n, h.reg_shift, shifts, N))) return rc;
    unsigned long long step = 0;
    CK(cudaMemcpyAsync(&step, h.step, sizeof(step), cudaMemcpyDeviceToHost, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    h.input_kind = 1;
    h.reg_dur = dur;
    h.reg_cycle = cycle;
    h.reg_c0 = in_cycle;
    h.reg_t0 = step;
    if ((rc = push_desc(n))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

static inline uint32_t rotl32(uint32_t x, unsigned r) { r &= 31u; return r ? (x << r) | (x >> (32 - r)) : x; }
static inline uint32_t rotr32(uint32_t x, unsigned r) { r &= 31u; return r ? (x >> r) | (x << (32 - r)) : x; }

int bg3_input_poisson(bg3_net *n, const bg3_poisson_arrays *a, float lambda, uint32_t seed,
                      uint64_t step)
{
    if (!n || !a || !a->nISIs || !a->total_delay || !a->delayIdx || !a->delayQueue || !a->W ||
        !a->psr || !a->decay || !a->U || !a->D || !a->F || !a->u || !a->r || !a->lastSpike ||
        lambda <= 0 || step >= 0xffffff00ull)
        return BG3_EINVAL;
    NetDev &h = n->h;
    const size_t N = h.N;
    int rc;
    if (!h.pois_mask) {
        if ((rc = dalloc(n, &h.pois_mask, N)) || (rc = dalloc(n, &h.pois_nisi, N)) ||
            (rc = dalloc(n, &h.in_psr, N)) || (rc = dalloc(n, &h.in_decay, N)) ||
            (rc = dalloc(n, &h.in_queue, N)) || (rc = dalloc(n, &h.in_delay, N)) ||
            (rc = dalloc(n, &h.in_ev, N)) || (rc = dalloc(n, &h.isi_cursor, N)))
            return rc;
    }
    std::vector<uint8_t> mask(N), dl(N);
    std::vector<uint32_t> q(N);
    std::vector<EvSlot> ev(N);
    for (size_t i = 0; i < N; i++) {
        if (a->total_delay[i] < 1 || a->total_delay[i] > 31 || a->delayIdx[i] < 0 || a->delayIdx[i] > 31)
            return BG3_EINVAL;
        uint64_t ls = a->lastSpike[i];
        if (ls != BG3_ULONG_MAX && ls >= BG3_NO_SPIKE32) return BG3_EINVAL;
        mask[i] = a->masks ? (a->masks[i] ? 1 : 0) : 1;
        dl[i] = (uint8_t)a->total_delay[i];
        unsigned phase = (unsigned)((step - (uint64_t)a->delayIdx[i]) & 31u);
        q[i] = rotl32(a->delayQueue[i], phase);
        EvSlot &e = ev[i];
        e.W = a->W[i]; e.u = a->u[i]; e.r = a->r[i];
        e.last = (ls == BG3_ULONG_MAX) ? BG3_NO_SPIKE32 : (uint32_t)ls;
        e.born = (uint32_t)(step - (uint64_t)a->delayIdx[i]);
        const int pc = param_class(n, a->U[i], a->D[i], a->F[i]);
        if (pc < 0) return pc;
        e.pcls = (uint8_t)pc;
    }
    if ((rc = h2d(n, h.pois_mask, mask.data(), N)) || (rc = h2d(n, h.pois_nisi, a->nISIs, N)) ||
        (rc = h2d(n, h.in_psr, a->psr, N)) || (rc = h2d(n, h.in_decay, a->decay, N)) ||
        (rc = h2d(n, h.in_queue, q.data(), N)) || (rc = h2d(n, h.in_delay, dl.data(), N)) ||
        (rc = h2d(n, h.in_ev, ev.data(), N)))
        return rc;
    CK(cudaMemsetAsync(h.isi_cursor, 0, N * sizeof(int32_t), n->stream));
    h.input_kind = 2;
    h.pois_lambda = lambda;
    h.pois_seed = seed;
    h.pois_t0 = step;
    if ((rc = push_desc(n))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_push_poisson_isis(bg3_net *n, const int32_t *begin, const int32_t *isis)
{
    if (!n || !begin || (!isis && begin[n->h.N] > 0) || n->h.input_kind != 2) return BG3_EINVAL;
    NetDev &h = n->h;
    const size_t N = h.N;
    const size_t total = (size_t)begin[N];
    int rc;
    if (!h.isi_begin && (rc = dalloc(n, &h.isi_begin, N + 1))) return rc;
    if (h.isi_vals) {  // replace the previous draws
        cudaStreamSynchronize(n->stream);
        for (auto &p : n->allocs)
            if (p.first == (void *)h.isi_vals) {
                cudaFree(p.first);
                n->bytes -= p.second;
                p = std::make_pair((void *)nullptr, (size_t)0);
            }
        h.isi_vals = nullptr;
    }
    if ((rc = dalloc(n, &h.isi_vals, std::max<size_t>(total, 1)))) return rc;
    if ((rc = h2d(n, h.isi_begin, begin, N + 1)) || (rc = h2d(n, h.isi_vals, isis, total))) return rc;
    CK(cudaMemsetAsync(h.isi_cursor, 0, N * sizeof(int32_t), n->stream));
    if ((rc = push_desc(n))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_download_poisson(bg3_net *n, bg3_poisson_arrays *a)
{
    if (!n || !a || n->h.input_kind != 2) return BG3_EINVAL;
    NetDev &h = n->h;
    const size_t N = h.N;
    std::vector<uint8_t> mask(N), dl(N);
    std::vector<uint32_t> q(N);
    std::vector<EvSlot> ev(N);
    std::vector<float> psr(N), dec(N);
    std::vector<int32_t> nisi(N);
    unsigned long long step = 0;
    int rc;
    if ((rc = d2h(n, mask.data(), h.pois_mask, N)) || (rc = d2h(n, nisi.data(), h.pois_nisi, N)) ||
        (rc = d2h(n, psr.data(), h.in_psr, N)) || (rc = d2h(n, dec.data(), h.in_decay, N)) ||
        (rc = d2h(n, q.data(), h.in_queue, N)) || (rc = d2h(n, dl.data(), h.in_delay, N)) ||
        (rc = d2h(n, ev.data(), h.in_ev, N)) || (rc = d2h(n, &step, h.step, 1)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    for (size_t i = 0; i < N; i++) {
        const EvSlot &e = ev[i];
        uint32_t phase = e.born & 31u;
        if (a->masks) a->masks[i] = mask[i];
        if (a->nISIs) a->nISIs[i] = nisi[i];
        if (a->total_delay) a->total_delay[i] = dl[i];
        // the reference advances the read index only of masked-in neurons' input synapses
        const uint32_t now = mask[i] ? (uint32_t)step : (uint32_t)h.pois_t0;
        if (a->delayIdx) a->delayIdx[i] = (int32_t)((now - e.born) & 31u);
        if (a->delayQueue) a->delayQueue[i] = rotr32(q[i], phase);
        if (a->W) a->W[i] = e.W;
        if (a->psr) a->psr[i] = psr[i];
        if (a->decay) a->decay[i] = dec[i];
        if (a->U) a->U[i] = h.p_U[e.pcls];
        if (a->D) a->D[i] = h.p_D[e.pcls];
        if (a->F) a->F[i] = h.p_F[e.pcls];
        if (a->u) a->u[i] = e.u;
        if (a->r) a->r[i] = e.r;
        if (a->lastSpike) a->lastSpike[i] = (e.last == BG3_NO_SPIKE32) ? BG3_ULONG_MAX : (uint64_t)e.last;
    }
    return BG3_OK;
}

// ---- hot path -------------------------------------------------------------------------------
// Device-noise mode: neurons(t0), then per step deliver + sweep whose epilogue integrates the
// next step's neurons, the last sweep without that epilogue.  Runs of interior steps replay a
// CUDA graph of GRAPH_STEPS (deliver, fused sweep) pairs.  Injected-noise mode: neurons,
// deliver, sweep for every step, GRAPH_STEPS of them per graph replay.
static int run_steps(bg3_net *n, int64_t nsteps)
{
    if (nsteps <= 0) return BG3_OK;
    const NetDev &h = n->h;
    if (bg3::small_eligible(h, n->cfg)) {
        // a small network: up to SMALL_STEPS whole steps per launch, one CTA
        for (int64_t left = nsteps; left > 0;) {
            const int k = (int)std::min<int64_t>(left, SMALL_STEPS);
            bg3::launch_small(h, k, n->stream);
            n->launches += 1;
            left -= k;
        }
        CK(cudaGetLastError());
        return BG3_OK;
    }
    if (h.noise_mode == BG3_NOISE_INJECT) {
        // (neurons, deliver, sweep) per step; runs of GRAPH_STEPS steps replay a captured graph
        // (the injected stream's cursor lives on the device, and a push or any other change of
        // the descriptor drops the graph)
        auto one = [&]() {
            bg3::launch_neurons(h, n->stream);
            bg3::launch_deliver(h, n->cfg, n->stream);
            bg3::launch_sweep(h, n->tm_psr, n->tm_cls, n->tm_psr16, n->tm_cls16, false, n->cfg, n->stream);
        };
        int64_t left = nsteps;
        if (left >= GRAPH_STEPS && !n->graph) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(n->stream, cudaStreamCaptureModeThreadLocal));
            for (int i = 0; i < GRAPH_STEPS; i++) one();
            CK(cudaStreamEndCapture(n->stream, &g));
            cudaError_t e = cudaGraphInstantiate(&n->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { n->graph = nullptr; return BG3_ECUDA; }
        }
        while (n->graph && left >= GRAPH_STEPS) {
            CK(cudaGraphLaunch(n->graph, n->stream));
            left -= GRAPH_STEPS;
        }
        for (; left > 0; left--) one();
        n->launches += (bg3::neuron_launches(h) + step_kernels(h.syn_kind)) * nsteps;
        CK(cudaGetLastError());
        return BG3_OK;
    }
    // neuron pass and arrivals of the first step, then (fused sweep of step t, arrivals of step
    // t + 1) pairs, so that each delivery pass overlaps the sweep before it, then the last sweep
    bg3::launch_neurons(h, n->stream);
    bg3::launch_deliver(h, n->cfg, n->stream);
    int64_t interior = nsteps - 1;
    if (interior >= GRAPH_STEPS && !n->graph) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(n->stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < GRAPH_STEPS; i++) {
            bg3::launch_sweep(h, n->tm_psr, n->tm_cls, n->tm_psr16, n->tm_cls16, true, n->cfg, n->stream);
            bg3::launch_deliver(h, n->cfg, n->stream);
        }
        CK(cudaStreamEndCapture(n->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&n->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { n->graph = nullptr; return BG3_ECUDA; }
    }
    while (n->graph && interior >= GRAPH_STEPS) {
        CK(cudaGraphLaunch(n->graph, n->stream));
        interior -= GRAPH_STEPS;
    }
    for (int64_t i = 0; i < interior; i++) {
        bg3::launch_sweep(h, n->tm_psr, n->tm_cls, n->tm_psr16, n->tm_cls16, true, n->cfg, n->stream);
        bg3::launch_deliver(h, n->cfg, n->stream);
    }
    bg3::launch_sweep(h, n->tm_psr, n->tm_cls, n->tm_psr16, n->tm_cls16, false, n->cfg, n->stream);
    n->launches += 1 + step_kernels(h.syn_kind) * nsteps;
    CK(cudaGetLastError());
    return BG3_OK;
}

int bg3_step(bg3_net *n, int64_t nsteps)
{
    if (!n || nsteps < 0) return BG3_EINVAL;
    return run_steps(n, nsteps);
}

int bg3_epoch_growth(bg3_net *n, int32_t epoch)
{
    if (!n || epoch < 0) return BG3_EINVAL;
    bg3::launch_growth(n->h, n->d, epoch, n->cfg.growth_threads, n->stream);
    n->launches += 8;
    CK(cudaGetLastError());
    return BG3_OK;
}

int bg3_epoch_record(bg3_net *n)
{
    if (!n) return BG3_EINVAL;
    bg3::launch_record(n->h, n->d, n->stream);
    n->launches += 1;
    CK(cudaGetLastError());
    return BG3_OK;
}

// ---- downloads ------------------------------------------------------------------------------
int bg3_sync(bg3_net *n)
{
    if (!n) return BG3_EINVAL;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_get_step(bg3_net *n, uint64_t *step)
{
    if (!n || !step) return BG3_EINVAL;
    unsigned long long s = 0;
    CK(cudaMemcpyAsync(&s, n->h.step, sizeof(s), cudaMemcpyDeviceToHost, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    *step = s;
    return BG3_OK;
}

int bg3_error_word(bg3_net *n, uint32_t *err)
{
    if (!n || !err) return BG3_EINVAL;
    CK(cudaMemcpyAsync(err, n->h.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_download_lif(bg3_net *n, bg3_lif_arrays *a)
{
    if (!n || !a) return BG3_EINVAL;
    size_t N = n->h.N;
    NetDev &h = n->h;
    int rc;
    if ((rc = d2h(n, a->Vm, h.Vm, N)) || (rc = d2h(n, a->Vthresh, h.Vthresh, N)) ||
        (rc = d2h(n, a->Vreset, h.Vreset, N)) || (rc = d2h(n, a->I0, h.I0, N)) ||
        (rc = d2h(n, a->Inoise, h.Inoise, N)) || (rc = d2h(n, a->C1, h.C1, N)) ||
        (rc = d2h(n, a->C2, h.C2, N)) || (rc = d2h(n, a->Trefract, h.Trefract, N)) ||
        (rc = d2h(n, a->summation, h.sp, N)) || (rc = d2h(n, a->nStepsInRefr, h.refr, N)) ||
        (rc = d2h(n, a->spikeCount, h.spikeCount, N)) ||
        (rc = d2h(n, a->spikeCountOffset, h.spikeCountOffset, N)) ||
        (rc = d2h(n, a->history, (const uint64_t *)h.history, N * (size_t)h.max_spikes)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_download_izh(bg3_net *n, bg3_izh_arrays *a)
{
    if (!n || !a) return BG3_EINVAL;
    if (n->h.neuron_kind != BG3_NEURON_IZH) return BG3_EUNSUPPORTED;
    size_t N = n->h.N;
    NetDev &h = n->h;
    int rc;
    if ((rc = d2h(n, a->Aconst, h.Aconst, N)) || (rc = d2h(n, a->Bconst, h.Bconst, N)) ||
        (rc = d2h(n, a->Cconst, h.Cconst, N)) || (rc = d2h(n, a->Dconst, h.Dconst, N)) ||
        (rc = d2h(n, a->u, h.u_izh, N)) || (rc = d2h(n, a->C3, h.C3, N)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

// Rebuilds the reference's delayQueue / delayIdx from the spike ring and birth steps: a spike
// emitted at tf >= birth is due at tf + D; at step t it sits at bit (delayIdx + tf + D - t) & 31
// with delayIdx = (t - birth) & 31.
int bg3_download_synapses(bg3_net *n, bg3_synapse_arrays *a)
{
    if (!n || !a) return BG3_EINVAL;
    const size_t N = n->h.N, Np = n->h.Np, M = n->h.max_syn, S = Np * (size_t)n->h.Mq * 4;
    NetDev &h = n->h;
    std::vector<float> psr(S);
    std::vector<uint32_t> dc(S / 8);
    std::vector<uint8_t> lc(S);
    std::vector<EvSlot> ev(S);
    std::vector<int32_t> src(S), ring(N * BG3_RING), ring_n(BG3_RING);
    std::vector<int8_t> st(S);
    std::vector<uint32_t> count(N);
    unsigned long long step = 0;
    const bool ds = h.syn_kind == BG3_SYN_DS || h.syn_kind == BG3_SYN_DYNSTDP;
    int rc;
    if ((rc = d2h(n, psr.data(), h.psr, S)) || (rc = d2h(n, dc.data(), h.dcls, S / 8)) ||
        (rc = d2h(n, lc.data(), h.lcls, S)) || (rc = d2h(n, ev.data(), h.ev, S)) ||
        (rc = d2h(n, src.data(), h.src, S)) || (rc = d2h(n, st.data(), h.stype, S)) ||
        (rc = d2h(n, count.data(), h.count, N)) || (rc = d2h(n, &step, h.step, 1)) ||
        (rc = d2h(n, ring.data(), h.ring, ring.size())) ||
        (rc = d2h(n, ring_n.data(), h.ring_n, ring_n.size())))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    // fired[s] bit j: neuron s fired at step - 1 - j
    std::vector<uint32_t> fired(N, 0u);
    for (int j = 0; j < 32 && (uint64_t)j < step; j++) {
        int slot = (int)((step - 1 - (uint64_t)j) & (BG3_RING - 1));
        for (int q = 0; q < std::min<int>(ring_n[slot], (int)N); q++)
            fired[ring[(size_t)slot * N + q]] |= 1u << j;
    }
    for (size_t d = 0; d < N; d++) {
        if (a->counts) a->counts[d] = count[d];
        for (size_t k = 0; k < M; k++) {
            size_t i = d * M + k, p = slot_pos((int)k, (int)d, (int)n->h.Mq);
            bool used = k < count[d];
            if (a->in_use) a->in_use[i] = used ? 1 : 0;
            if (!used) continue;
            const EvSlot &e = ev[p];
            int D = n->ltab[lc[p]];
            uint32_t di = (uint32_t)((uint32_t)step - e.born) & 31u;
            uint32_t q = 0;
            for (int j = 0; j < D; j++) {
                if (!((fired[src[p]] >> j) & 1u)) continue;
                uint32_t tf = (uint32_t)(step - 1 - (uint64_t)j);
                if ((int32_t)(tf - e.born) < 0) continue;
                q |= 1u << ((di + (uint32_t)(D - 1 - j)) & 31u);
            }
            if (a->src) a->src[i] = src[p];
            if (a->type) a->type[i] = st[p];
            if (a->W) a->W[i] = e.W;
            if (a->psr) a->psr[i] = psr[p];
            if (a->decay) a->decay[i] = n->dtab[cls_get(dc.data(), p)];
            if (a->total_delay) a->total_delay[i] = D;
            if (a->delayIdx) a->delayIdx[i] = (int32_t)di;
            if (a->delayQueue) a->delayQueue[i] = q;
            if (a->tau) a->tau[i] = h.t_tau[st[p] & 3];
            if (!ds) continue;  // the DS fields exist for DS and dynamic STDP synapses only
            if (a->U) a->U[i] = h.p_U[e.pcls];
            if (a->D) a->D[i] = h.p_D[e.pcls];
            if (a->F) a->F[i] = h.p_F[e.pcls];
            if (a->u) a->u[i] = e.u;
            if (a->r) a->r[i] = e.r;
            if (a->lastSpike) a->lastSpike[i] = (e.last == BG3_NO_SPIKE32) ? BG3_ULONG_MAX : (uint64_t)e.last;
        }
    }
    return BG3_OK;
}

// ---- STDP --------------------------------------------------------------------------------------
static StdpConst stdp_from(const bg3_stdp_constants *c, int t)
{
    StdpConst s = {};
    s.Apos = c->Apos[t]; s.Aneg = c->Aneg[t]; s.gap = c->STDPgap[t];
    s.tauspost = c->tauspost[t]; s.tauspre = c->tauspre[t];
    s.taupos = c->taupos[t]; s.tauneg = c->tauneg[t];
    s.Wex = c->Wex[t]; s.mupos = c->mupos[t]; s.muneg = c->muneg[t];
    s.useFD = c->useFroemkeDanSTDP[t] ? 1 : 0;
    return s;
}

int bg3_set_stdp_constants(bg3_net *n, const bg3_stdp_constants *c)
{
    if (!n || !c) return BG3_EINVAL;
    if (n->h.syn_kind < BG3_SYN_STDP) return BG3_EUNSUPPORTED;
    for (int t = 0; t < 4; t++) {
        int rc = set_stdp_type(n, t, stdp_from(c, t));
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_set_stdp_arithmetic(bg3_net *n, int mode)
{
    if (!n || (mode != BG3_STDP_HOST && mode != BG3_STDP_DEVICE)) return BG3_EINVAL;
    if (n->h.syn_kind < BG3_SYN_STDP) return BG3_EUNSUPPORTED;
    n->h.stdp_signed = mode == BG3_STDP_DEVICE;
    int rc = push_desc(n);
    if (rc) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

// The reference's STDP fields per slot; every in-use synapse of one type must carry the same
// constants, an empty post queue, total_delayPost 0 and delayIdxPost == delayIdx (what
// createSynapse and the step produce).  Anything else is BG3_EUNSUPPORTED.
int bg3_upload_stdp(bg3_net *n, const bg3_synapse_arrays *syn, const bg3_stdp_arrays *a)
{
    if (!n || !syn || !a || !syn->in_use || !syn->type || !syn->delayIdx || !a->delayQueuePost ||
        !a->delayIdxPost || !a->total_delayPost || !a->tauspost || !a->tauspre || !a->taupos ||
        !a->tauneg || !a->STDPgap || !a->Wex || !a->Aneg || !a->Apos || !a->mupos || !a->muneg ||
        !a->useFroemkeDanSTDP)
        return BG3_EINVAL;
    if (n->h.syn_kind < BG3_SYN_STDP) return BG3_EUNSUPPORTED;
    const size_t S = (size_t)n->h.N * n->h.max_syn;
    bool seen[4] = {false, false, false, false};
    bg3_stdp_constants c;
    memset(&c, 0, sizeof(c));
    for (size_t i = 0; i < S; i++) {
        if (!syn->in_use[i]) continue;
        const int t = syn->type[i];
        if (t < 0 || t > 3) return BG3_EINVAL;
        if (a->delayQueuePost[i] != 0 || a->total_delayPost[i] != 0 ||
            a->delayIdxPost[i] != syn->delayIdx[i])
            return BG3_EUNSUPPORTED;
        const float v[10] = {a->Apos[i], a->Aneg[i], a->STDPgap[i], a->tauspost[i], a->tauspre[i],
                             a->taupos[i], a->tauneg[i], a->Wex[i], a->mupos[i], a->muneg[i]};
        float *dst[10] = {&c.Apos[t], &c.Aneg[t], &c.STDPgap[t], &c.tauspost[t], &c.tauspre[t],
                          &c.taupos[t], &c.tauneg[t], &c.Wex[t], &c.mupos[t], &c.muneg[t]};
        const int fd = a->useFroemkeDanSTDP[i] ? 1 : 0;
        if (!seen[t]) {
            for (int k = 0; k < 10; k++) *dst[k] = v[k];
            c.useFroemkeDanSTDP[t] = fd;
            seen[t] = true;
            continue;
        }
        for (int k = 0; k < 10; k++)
            if (fbits(*dst[k]) != fbits(v[k])) return BG3_EUNSUPPORTED;
        if (c.useFroemkeDanSTDP[t] != fd) return BG3_EUNSUPPORTED;
    }
    for (int t = 0; t < 4; t++) {
        if (!seen[t]) continue;
        int rc = set_stdp_type(n, t, stdp_from(&c, t));
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_download_stdp(bg3_net *n, bg3_stdp_arrays *a)
{
    if (!n || !a) return BG3_EINVAL;
    if (n->h.syn_kind < BG3_SYN_STDP) return BG3_EUNSUPPORTED;
    const NetDev &h = n->h;
    const size_t N = h.N, Np = h.Np, M = h.max_syn, S = Np * (size_t)h.Mq * 4;
    std::vector<EvSlot> ev(S);
    std::vector<int8_t> st(S);
    std::vector<uint32_t> count(N);
    unsigned long long step = 0;
    int rc;
    if ((rc = d2h(n, ev.data(), h.ev, S)) || (rc = d2h(n, st.data(), h.stype, S)) ||
        (rc = d2h(n, count.data(), h.count, N)) || (rc = d2h(n, &step, h.step, 1)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    for (size_t d = 0; d < N; d++) {
        for (size_t k = 0; k < M && k < count[d]; k++) {
            const size_t i = d * M + k, p = slot_pos((int)k, (int)d, (int)n->h.Mq);
            const StdpConst &c = h.stdp[st[p] & 3];
            if (a->delayQueuePost) a->delayQueuePost[i] = 0;
            if (a->delayIdxPost) a->delayIdxPost[i] = (int32_t)(((uint32_t)step - ev[p].born) & 31u);
            if (a->total_delayPost) a->total_delayPost[i] = 0;
            if (a->tauspost) a->tauspost[i] = c.tauspost;
            if (a->tauspre) a->tauspre[i] = c.tauspre;
            if (a->taupos) a->taupos[i] = c.taupos;
            if (a->tauneg) a->tauneg[i] = c.tauneg;
            if (a->STDPgap) a->STDPgap[i] = c.gap;
            if (a->Wex) a->Wex[i] = c.Wex;
            if (a->Aneg) a->Aneg[i] = c.Aneg;
            if (a->Apos) a->Apos[i] = c.Apos;
            if (a->mupos) a->mupos[i] = c.mupos;
            if (a->muneg) a->muneg[i] = c.muneg;
            if (a->useFroemkeDanSTDP) a->useFroemkeDanSTDP[i] = (uint8_t)c.useFD;
        }
    }
    return BG3_OK;
}

int64_t bg3_total_synapses(bg3_net *n)
{
    if (!n) return BG3_EINVAL;
    std::vector<uint32_t> count(n->h.N);
    if (cudaMemcpyAsync(count.data(), n->h.count, count.size() * 4, cudaMemcpyDeviceToHost, n->stream) != cudaSuccess ||
        cudaStreamSynchronize(n->stream) != cudaSuccess)
        return BG3_ECUDA;
    int64_t t = 0;
    for (uint32_t c : count) t += c;
    return t;
}

// The device keeps the outgoing map grouped by (delay class, source) with plane slots in
// arbitrary order (delivery does not depend on it) and the incoming map implicitly as the in-use
// row prefixes.  Both are returned in the reference's order: slot ids d * maxSyn + k, ascending
// within each source; incoming in dest-major slot order (Synapses/AllSynapses.cpp:223-293).
int bg3_download_maps(bg3_net *n, bg3_index_maps *m)
{
    if (!n || !m) return BG3_EINVAL;
    const size_t N = n->h.N, Np = n->h.Np, M = n->h.max_syn;
    const size_t C = n->ltab.size();
    std::vector<uint32_t> ob(N * C), oc(N * C), count(N);
    int rc;
    if ((rc = d2h(n, ob.data(), n->h.outBegin, N * C)) || (rc = d2h(n, oc.data(), n->h.outCount, N * C)) ||
        (rc = d2h(n, count.data(), n->h.count, N)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    size_t total = 0;
    for (uint32_t c : count) total += c;
    std::vector<uint32_t> om(std::max<size_t>(total, 1));
    if (total && (rc = d2h(n, om.data(), n->h.outMap, total))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    uint32_t acc = 0;
    for (size_t i = 0; i < N; i++) {
        std::vector<uint32_t> ids;
        for (size_t c = 0; c < C; c++)
            for (uint32_t j = 0; j < oc[c * N + i]; j++) {
                int k, d;
                pos_slot(om[ob[c * N + i] + j], (int)n->h.Mq, k, d);
                ids.push_back((uint32_t)((size_t)d * M + (size_t)k));
            }
        std::sort(ids.begin(), ids.end());
        if (m->outgoingSynapseBegin) m->outgoingSynapseBegin[i] = acc;
        if (m->outgoingSynapseCount) m->outgoingSynapseCount[i] = (uint32_t)ids.size();
        if (m->outgoingSynapseIndexMap)
            for (size_t j = 0; j < ids.size(); j++) m->outgoingSynapseIndexMap[acc + j] = ids[j];
        acc += (uint32_t)ids.size();
    }
    acc = 0;
    for (size_t d = 0; d < N; d++) {
        if (m->incomingSynapseBegin) m->incomingSynapseBegin[d] = acc;
        if (m->incomingSynapseCount) m->incomingSynapseCount[d] = count[d];
        if (m->incomingSynapseIndexMap)
            for (uint32_t k = 0; k < count[d]; k++) m->incomingSynapseIndexMap[acc + k] = (uint32_t)(d * M + k);
        acc += count[d];
    }
    return BG3_OK;
}

int bg3_download_growth(bg3_net *n, float *radii, float *rates)
{
    if (!n) return BG3_EINVAL;
    int rc;
    if ((rc = d2h(n, radii, n->h.radii, n->h.N)) || (rc = d2h(n, rates, n->h.rates, n->h.N))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_download_state(bg3_net *n, const bg3_state_view *v)
{
    if (!n || !v || (!v->radii != !v->rates)) return BG3_EINVAL;
    if ((v->izh && n->h.neuron_kind != BG3_NEURON_IZH) ||
        (v->stdp && n->h.syn_kind < BG3_SYN_STDP))
        return BG3_EINVAL;
    int rc = BG3_OK;
    if (v->neurons && (rc = bg3_download_lif(n, v->neurons))) return rc;
    if (v->izh && (rc = bg3_download_izh(n, v->izh))) return rc;
    if (v->synapses && (rc = bg3_download_synapses(n, v->synapses))) return rc;
    if (v->stdp && (rc = bg3_download_stdp(n, v->stdp))) return rc;
    if (v->maps && (rc = bg3_download_maps(n, v->maps))) return rc;
    if (v->radii && (rc = bg3_download_growth(n, v->radii, v->rates))) return rc;
    return BG3_OK;
}

int bg3_download_histories(bg3_net *n, float *burst, float *spikes, float *rh, float *radh)
{
    if (!n) return BG3_EINVAL;
    NetDev &h = n->h;
    size_t rows = (size_t)(h.max_epochs + 1) * h.N;
    int rc;
    if ((rc = d2h(n, burst, h.burstiness, (size_t)h.n_burst_bins)) ||
        (rc = d2h(n, spikes, h.spikes_hist, (size_t)h.n_spike_bins)) ||
        (rc = d2h(n, rh, h.rates_hist, rows)) || (rc = d2h(n, radh, h.radii_hist, rows)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

// ---- batched form ---------------------------------------------------------------------------
// Many networks advanced together: per step one delivery launch and one sweep launch cover every
// network (per-network descriptors and tensor maps in device tables, a (network, tile) table
// ordered heaviest tile first).  Member handles keep their own state and remain usable on their
// own; the batch orders its stream after theirs and theirs after its own.
struct bg3_batch {
    std::vector<bg3_net *> nets;
    NetDev *d_nets = nullptr;
    CUtensorMap *d_maps = nullptr;
    int2 *d_tiles = nullptr;
    int ntiles = 0, n_thick = 0, max_n = 0, syn_kind = 1;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev = nullptr;
    void *flush_buf = nullptr, *scrub_buf = nullptr;
    size_t flush_size = 0;
    long long launches = 0;
    LaunchCfg cfg = LAUNCH_DEFAULT;
};

static int batch_refresh(bg3_batch *b)
{
    std::vector<NetDev> hd;
    std::vector<CUtensorMap> maps;
    std::vector<std::pair<int, int2>> tiles;  // (rows, (net, tile))
    for (size_t k = 0; k < b->nets.size(); k++) {
        bg3_net *n = b->nets[k];
        hd.push_back(n->h);
        hd.back().izh_hw_every = b->cfg.izh_hw_every;
        maps.push_back(n->tm_psr);
        maps.push_back(n->tm_cls);
        std::vector<uint32_t> count(n->h.N);
        CK(cudaMemcpy(count.data(), n->h.count, count.size() * 4, cudaMemcpyDeviceToHost));
        for (int t = 0; t < n->h.ntiles; t++) {
            uint32_t m = 0;
            for (int d = t * 32; d < std::min(n->h.N, t * 32 + 32); d++) m = std::max(m, count[d]);
            tiles.push_back(std::make_pair((int)m, make_int2((int)k, t)));
        }
    }
    // TMA-swept tiles first, heaviest first; then the tiles of thin networks (one warp each) in
    // (network, tile) order, each network's run padded with (network, -1) entries to whole blocks
    // of the thin sweep, so that a block serves one network
    std::vector<int2> thin;
    const int w = b->cfg.thin_warps;
    for (auto &t : tiles) {
        if (!bg3::sweep_is_thin(b->nets[t.second.x]->h, b->cfg)) continue;
        thin.push_back(t.second);
        if (t.second.y == b->nets[t.second.x]->h.ntiles - 1)
            while (thin.size() % w) thin.push_back(make_int2(t.second.x, -1));
    }
    std::stable_sort(tiles.begin(), tiles.end(),
                     [](const std::pair<int, int2> &a, const std::pair<int, int2> &c) { return a.first > c.first; });
    std::vector<int2> tl;
    for (auto &t : tiles)
        if (!bg3::sweep_is_thin(b->nets[t.second.x]->h, b->cfg)) tl.push_back(t.second);
    b->n_thick = (int)tl.size();
    tl.insert(tl.end(), thin.begin(), thin.end());
    if ((int)tl.size() != b->ntiles) {
        if (b->d_tiles) cudaFree(b->d_tiles);
        b->d_tiles = nullptr;
        if (cudaMalloc(&b->d_tiles, std::max<size_t>(tl.size(), 1) * sizeof(int2)) != cudaSuccess) {
            cudaGetLastError();
            return BG3_ENOMEM;
        }
        b->ntiles = (int)tl.size();
    }
    CK(cudaMemcpyAsync(b->d_nets, hd.data(), hd.size() * sizeof(NetDev), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(b->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(b->d_tiles, tl.data(), tl.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    return BG3_OK;
}

// order the batch stream after every member stream (enter) or every member after it (leave)
static int batch_order(bg3_batch *b, bool enter)
{
    for (bg3_net *n : b->nets) {
        CK(cudaEventRecord(b->ev, enter ? n->stream : b->stream));
        CK(cudaStreamWaitEvent(enter ? b->stream : n->stream, b->ev, 0));
    }
    return BG3_OK;
}

int bg3_batch_create(bg3_net *const *nets, int32_t count, bg3_batch **out)
{
    if (!nets || count <= 0 || !out) return BG3_EINVAL;
    *out = nullptr;
    for (int k = 0; k < count; k++) {
        if (!nets[k] || nets[k]->h.noise_mode != BG3_NOISE_DEVICE ||
            nets[k]->h.syn_kind != nets[0]->h.syn_kind)
            return BG3_EINVAL;
        for (int j = 0; j < k; j++)
            if (nets[j] == nets[k]) return BG3_EINVAL;
    }
    bg3_batch *b = new (std::nothrow) bg3_batch();
    if (!b) return BG3_ENOMEM;
    b->nets.assign(nets, nets + count);
    b->syn_kind = nets[0]->h.syn_kind;
    for (bg3_net *n : b->nets) b->max_n = std::max(b->max_n, n->h.N);
    int rc = BG3_ECUDA;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) != cudaSuccess)
        goto fail;
    rc = BG3_ENOMEM;
    if (cudaMalloc(&b->d_nets, count * sizeof(NetDev)) != cudaSuccess ||
        cudaMalloc(&b->d_maps, 2 * count * sizeof(CUtensorMap)) != cudaSuccess)
        goto fail;
    for (bg3_net *n : b->nets) cudaStreamSynchronize(n->stream);
    if ((rc = batch_refresh(b)) != 0) goto fail;
    *out = b;
    return BG3_OK;
fail:
    cudaGetLastError();
    bg3_batch_destroy(b);
    return rc;
}

int bg3_batch_destroy(bg3_batch *b)
{
    if (!b) return BG3_EINVAL;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->d_nets) cudaFree(b->d_nets);
    if (b->d_maps) cudaFree(b->d_maps);
    if (b->d_tiles) cudaFree(b->d_tiles);
    if (b->flush_buf) cudaFree(b->flush_buf);
    if (b->scrub_buf) cudaFree(b->scrub_buf);
    if (b->ev) cudaEventDestroy(b->ev);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return BG3_OK;
}

int bg3_batch_refresh(bg3_batch *b)
{
    if (!b) return BG3_EINVAL;
    int rc = batch_order(b, true);
    if (rc) return rc;
    CK(cudaStreamSynchronize(b->stream));
    return batch_refresh(b);
}

// (fused sweep of step t, arrivals of step t + 1) pairs: each delivery pass overlaps the sweep
// before it
static void batch_interior(bg3_batch *b, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        bg3::launch_sweep_batch(b->d_nets, b->d_maps, b->d_tiles, b->n_thick, b->ntiles - b->n_thick, true, b->cfg, b->stream);
        bg3::launch_deliver_batch(b->syn_kind, b->d_nets, (int)b->nets.size(), b->cfg, b->stream);
    }
}

int bg3_batch_step(bg3_batch *b, int64_t nsteps)
{
    if (!b || nsteps < 0) return BG3_EINVAL;
    if (nsteps == 0) return BG3_OK;
    int rc = batch_order(b, true);
    if (rc) return rc;
    const int M = (int)b->nets.size();
    bg3::launch_neurons_batch(b->d_nets, M, b->max_n, b->stream);
    bg3::launch_deliver_batch(b->syn_kind, b->d_nets, M, b->cfg, b->stream);
    int64_t interior = nsteps - 1;
    if (interior >= GRAPH_STEPS && !b->graph) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        batch_interior(b, GRAPH_STEPS);
        CK(cudaStreamEndCapture(b->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { b->graph = nullptr; return BG3_ECUDA; }
    }
    while (b->graph && interior >= GRAPH_STEPS) {
        CK(cudaGraphLaunch(b->graph, b->stream));
        interior -= GRAPH_STEPS;
    }
    batch_interior(b, interior);
    bg3::launch_sweep_batch(b->d_nets, b->d_maps, b->d_tiles, b->n_thick, b->ntiles - b->n_thick, false, b->cfg, b->stream);
    const int sweeps = (b->n_thick > 0) + (b->ntiles > b->n_thick);
    b->launches += 1 + (step_kernels(b->syn_kind) - 1 + sweeps) * nsteps;
    CK(cudaGetLastError());
    return batch_order(b, false);
}

int bg3_batch_sync(bg3_batch *b)
{
    if (!b) return BG3_EINVAL;
    CK(cudaStreamSynchronize(b->stream));
    return BG3_OK;
}

int64_t bg3_batch_launches(bg3_batch *b) { return b ? b->launches : BG3_EINVAL; }

// ---- benchmarking ---------------------------------------------------------------------------
__global__ void k_scrub(const float4 *p, size_t n4, float *sink)
{
    float acc = 0.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        float4 v = p[i];
        acc += v.x + v.y + v.z + v.w;
    }
    if (acc == 12345.678f) *sink = acc;  // keeps the loads; practically never true
}

int bg3_bench_steps(bg3_net *n, int64_t nsteps, int64_t flush_bytes, float *step_ms,
                    float *kernel_ms)
{
    if (!n || nsteps < 0 || !step_ms) return BG3_EINVAL;
    if (flush_bytes > 0 && (size_t)flush_bytes > n->flush_size) {
        if (n->flush_buf) cudaFree(n->flush_buf);
        if (n->scrub_buf) cudaFree(n->scrub_buf);
        n->flush_buf = n->scrub_buf = nullptr;
        n->flush_size = 0;
        if (cudaMalloc(&n->flush_buf, (size_t)flush_bytes) != cudaSuccess ||
            cudaMalloc(&n->scrub_buf, (size_t)flush_bytes + 16) != cudaSuccess) {
            cudaGetLastError();
            return BG3_ENOMEM;
        }
        CK(cudaMemsetAsync(n->scrub_buf, 0, (size_t)flush_bytes + 16, n->stream));
        n->flush_size = (size_t)flush_bytes;
    }
    const NetDev &h = n->h;
    const bool inject = h.noise_mode == BG3_NOISE_INJECT;
    std::vector<cudaEvent_t> ev((size_t)nsteps * 3);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (int64_t s = 0; s < nsteps; s++) {
        if (flush_bytes > 0) {
            // evict L2: write a buffer larger than L2, then read another one so the step does
            // not pay for writing back the flush's dirty lines
            CK(cudaMemsetAsync(n->flush_buf, (int)(s & 0xff), (size_t)flush_bytes, n->stream));
            k_scrub<<<2 * 152, 512, 0, n->stream>>>((const float4 *)n->scrub_buf,
                                                   (size_t)flush_bytes / 16,
                                                   (float *)((char *)n->scrub_buf + flush_bytes));
        }
        cudaEvent_t *e = &ev[(size_t)s * 3];
        const bool last = s == nsteps - 1;
        if (!inject && s == 0) bg3::launch_neurons(h, n->stream);
        CK(cudaEventRecord(e[0], n->stream));
        if (inject || kernel_ms) {
            // three events per step: [neurons (injected-noise mode)] deliver | sweep; in
            // device-noise mode the neuron pass runs in the previous sweep's epilogue
            if (inject) bg3::launch_neurons(h, n->stream);
            bg3::launch_deliver(h, n->cfg, n->stream);
            if (kernel_ms) CK(cudaEventRecord(e[1], n->stream));
            bg3::launch_sweep(h, n->tm_psr, n->tm_cls, n->tm_psr16, n->tm_cls16, !inject && !last, n->cfg, n->stream);
        } else {
            // as bg3_step runs them: the sweep of step s and the arrivals of step s + 1, which
            // overlap it (the first step's arrivals open the first timed region)
            if (s == 0) bg3::launch_deliver(h, n->cfg, n->stream);
            bg3::launch_sweep(h, n->tm_psr, n->tm_cls, n->tm_psr16, n->tm_cls16, !last, n->cfg, n->stream);
            if (!last) bg3::launch_deliver(h, n->cfg, n->stream);
        }
        CK(cudaEventRecord(e[2], n->stream));
    }
    n->launches += (step_kernels(h.syn_kind) + (inject ? 1 : 0)) * nsteps + (inject ? 0 : 1);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(n->stream));
    for (int64_t s = 0; s < nsteps; s++) {
        cudaEvent_t *e = &ev[(size_t)s * 3];
        CK(cudaEventElapsedTime(&step_ms[s], e[0], e[2]));
        if (kernel_ms) {
            kernel_ms[3 * s] = 0.0f;
            CK(cudaEventElapsedTime(&kernel_ms[3 * s + 1], e[0], e[1]));
            CK(cudaEventElapsedTime(&kernel_ms[3 * s + 2], e[1], e[2]));
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return BG3_OK;
}

int bg3_batch_bench_steps(bg3_batch *b, int64_t nsteps, int64_t flush_bytes, float *step_ms)
{
    if (!b || nsteps < 0 || !step_ms) return BG3_EINVAL;
    if (flush_bytes > 0 && (size_t)flush_bytes > b->flush_size) {
        if (b->flush_buf) cudaFree(b->flush_buf);
        if (b->scrub_buf) cudaFree(b->scrub_buf);
        b->flush_buf = b->scrub_buf = nullptr;
        b->flush_size = 0;
        if (cudaMalloc(&b->flush_buf, (size_t)flush_bytes) != cudaSuccess ||
            cudaMalloc(&b->scrub_buf, (size_t)flush_bytes + 16) != cudaSuccess) {
            cudaGetLastError();
            return BG3_ENOMEM;
        }
        CK(cudaMemsetAsync(b->scrub_buf, 0, (size_t)flush_bytes + 16, b->stream));
        b->flush_size = (size_t)flush_bytes;
    }
    int rc = batch_order(b, true);
    if (rc) return rc;
    const int M = (int)b->nets.size();
    std::vector<cudaEvent_t> ev((size_t)nsteps * 2);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    bg3::launch_neurons_batch(b->d_nets, M, b->max_n, b->stream);
    for (int64_t s = 0; s < nsteps; s++) {
        if (flush_bytes > 0) {
            CK(cudaMemsetAsync(b->flush_buf, (int)(s & 0xff), (size_t)flush_bytes, b->stream));
            k_scrub<<<2 * 152, 512, 0, b->stream>>>((const float4 *)b->scrub_buf, (size_t)flush_bytes / 16,
                                                   (float *)((char *)b->scrub_buf + flush_bytes));
        }
        // the sweep of step s and the arrivals of step s + 1, which overlap it, as bg3_batch_step
        // runs them (the first step's arrivals open the first timed region)
        CK(cudaEventRecord(ev[2 * s], b->stream));
        if (s == 0) bg3::launch_deliver_batch(b->syn_kind, b->d_nets, M, b->cfg, b->stream);
        bg3::launch_sweep_batch(b->d_nets, b->d_maps, b->d_tiles, b->n_thick, b->ntiles - b->n_thick, s < nsteps - 1, b->cfg, b->stream);
        if (s < nsteps - 1) bg3::launch_deliver_batch(b->syn_kind, b->d_nets, M, b->cfg, b->stream);
        CK(cudaEventRecord(ev[2 * s + 1], b->stream));
    }
    const int sweeps = (b->n_thick > 0) + (b->ntiles > b->n_thick);
    b->launches += 1 + (step_kernels(b->syn_kind) - 1 + sweeps) * nsteps;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(b->stream));
    for (int64_t s = 0; s < nsteps; s++) CK(cudaEventElapsedTime(&step_ms[s], ev[2 * s], ev[2 * s + 1]));
    for (auto &e : ev) cudaEventDestroy(e);
    return batch_order(b, false);
}

int bg3_enable_timing(bg3_net *n, int on)
{
    if (!n) return BG3_EINVAL;
    n->timing = on != 0;
    return BG3_OK;
}

int bg3_kernel_times(bg3_net *n, float *a, float *b, float *c, int64_t *launches)
{
    if (!n) return BG3_EINVAL;
    if (a) *a = n->ms_neurons;
    if (b) *b = n->ms_fanout;
    if (c) *c = n->ms_sweep;
    if (launches) *launches = n->launches;
    return BG3_OK;
}

}  // extern "C"

// ---- launch configuration and autotuning ------------------------------------------------------
static bool cfg_valid(const bg3_launch_cfg *c)
{
    return c && (c->sweep_stages == 4 || c->sweep_stages == 6 || c->sweep_stages == 8) &&
           c->thin_max_quads >= 1 && c->thin_max_quads <= 4096 && c->thin_warps >= 1 &&
           c->thin_warps <= 32 && c->deliver_blocks >= 1 && c->deliver_blocks <= 65535 &&
           (c->growth_threads == 128 || c->growth_threads == 256 || c->growth_threads == 512) &&
           (c->sweep_dests == 16 || c->sweep_dests == 32) &&
           (c->deliver_early == 0 || c->deliver_early == 1) && c->izh_hw_every >= -1 &&
           c->izh_hw_every <= 8 && c->small_max_slots >= 0;
}
static LaunchCfg cfg_from(const bg3_launch_cfg &c)
{
    return LaunchCfg{c.sweep_stages, c.thin_max_quads, c.thin_warps, c.deliver_blocks,
                     c.growth_threads, c.sweep_dests, c.deliver_early, c.izh_hw_every,
                     c.small_max_slots};
}
static bg3_launch_cfg cfg_to(const LaunchCfg &c)
{
    bg3_launch_cfg o;
    o.sweep_stages = c.sweep_stages;
    o.thin_max_quads = c.thin_max_quads;
    o.thin_warps = c.thin_warps;
    o.deliver_blocks = c.deliver_blocks;
    o.growth_threads = c.growth_threads;
    o.sweep_dests = c.sweep_dests;
    o.deliver_early = c.deliver_early;
    o.izh_hw_every = c.izh_hw_every;
    o.small_max_slots = c.small_max_slots;
    return o;
}

int bg3_get_launch(bg3_net *n, bg3_launch_cfg *c)
{
    if (!n || !c) return BG3_EINVAL;
    *c = cfg_to(n->cfg);
    return BG3_OK;
}

int bg3_set_launch(bg3_net *n, const bg3_launch_cfg *c)
{
    if (!n || !cfg_valid(c)) return BG3_EINVAL;
    CK(cudaStreamSynchronize(n->stream));
    n->cfg = cfg_from(*c);
    n->h.izh_hw_every = n->cfg.izh_hw_every;
    drop_graph(n);
    return BG3_OK;
}

int bg3_batch_get_launch(bg3_batch *b, bg3_launch_cfg *c)
{
    if (!b || !c) return BG3_EINVAL;
    *c = cfg_to(b->cfg);
    return BG3_OK;
}

int bg3_batch_set_launch(bg3_batch *b, const bg3_launch_cfg *c)
{
    if (!b || !cfg_valid(c)) return BG3_EINVAL;
    CK(cudaStreamSynchronize(b->stream));
    b->cfg = cfg_from(*c);
    return batch_refresh(b);  // the thin / TMA split and the thin tile table depend on it
}

// A device-side copy of a network's whole state (every allocation plus the injected-noise
// buffer), for trials that must leave the network as it was.
struct StateCopy {
    void *buf = nullptr;
    std::vector<std::pair<void *, size_t>> parts;
};

static int state_save(bg3_net *n, StateCopy &sc)
{
    sc.parts.clear();
    for (auto &a : n->allocs)
        if (a.first) sc.parts.push_back(a);
    if (n->noise_dev) sc.parts.push_back(std::make_pair((void *)n->noise_dev, (size_t)n->noise_cap * sizeof(float)));
    size_t tot = 0;
    for (auto &p : sc.parts) tot += p.second;
    CK(cudaStreamSynchronize(n->stream));
    if (cudaMalloc(&sc.buf, std::max<size_t>(tot, 1)) != cudaSuccess) {
        cudaGetLastError();
        sc.buf = nullptr;
        return BG3_ENOMEM;
    }
    size_t off = 0;
    for (auto &p : sc.parts) {
        CK(cudaMemcpyAsync((char *)sc.buf + off, p.first, p.second, cudaMemcpyDeviceToDevice, n->stream));
        off += p.second;
    }
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

static int state_load(bg3_net *n, const StateCopy &sc)
{
    size_t off = 0;
    for (auto &p : sc.parts) {
        CK(cudaMemcpyAsync(p.first, (const char *)sc.buf + off, p.second, cudaMemcpyDeviceToDevice, n->stream));
        off += p.second;
    }
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

static void state_free(StateCopy &sc)
{
    if (sc.buf) cudaFree(sc.buf);
    sc.buf = nullptr;
}

// Coordinate search over the launch parameters; trial(cfg) returns a time (ms) or < 0 on error.
template <typename Trial>
static int tune(LaunchCfg &cur, bool thick, bool thin, int mq, bool batch, bool izh, Trial trial,
                float &best_ms)
{
    float t = trial(cur);
    if (t < 0) return (int)t;
    best_ms = t;
    auto try_param = [&](int LaunchCfg::*field, std::initializer_list<int> values) -> int {
        const int keep = cur.*field;
        int best_v = keep;
        for (int v : values) {
            if (v == keep) continue;
            cur.*field = v;
            const float tv = trial(cur);
            if (tv < 0) return (int)tv;
            if (tv < best_ms) { best_ms = tv; best_v = v; }
        }
        cur.*field = best_v;
        return BG3_OK;
    };
    int rc;
    if (thick && !batch && (rc = try_param(&LaunchCfg::sweep_dests, {16, 32}))) return rc;
    if (thick && (rc = try_param(&LaunchCfg::sweep_stages, {4, 6, 8}))) return rc;
    if (mq > 4 && mq <= 64 && (rc = try_param(&LaunchCfg::thin_max_quads, {mq - 1, mq}))) return rc;
    if ((thin || mq <= 64) && (rc = try_param(&LaunchCfg::thin_warps, {4, 8, 16}))) return rc;
    if ((rc = try_param(&LaunchCfg::deliver_blocks, {152, 304, 608}))) return rc;
    if ((rc = try_param(&LaunchCfg::deliver_early, {0, 1}))) return rc;
    if (izh && (rc = try_param(&LaunchCfg::izh_hw_every, {-1, 0, 1, 2, 3, 4}))) return rc;
    return BG3_OK;
}

// Warm-up long enough to capture the step graph outside the timed region, then steps timed.
static float time_steps(bg3_net *n, int32_t steps)
{
    if (bg3_step(n, GRAPH_STEPS + 3) != BG3_OK) return -1.0f;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return -1.0f;
    cudaEventRecord(a, n->stream);
    int rc = bg3_step(n, steps);
    cudaEventRecord(b, n->stream);
    float ms = -1.0f;
    if (rc == BG3_OK && cudaEventSynchronize(b) == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms < 0 ? -1.0f : ms / (float)steps;
}

int bg3_autotune(bg3_net *n, int32_t steps, int32_t tune_growth, bg3_launch_cfg *best,
                 float *best_ms)
{
    if (!n || steps < 1) return BG3_EINVAL;
    StateCopy sc;
    int rc = state_save(n, sc);
    if (rc) return rc;
    const NetDev &h = n->h;
    LaunchCfg cur = n->cfg;
    auto trial = [&](const LaunchCfg &c) -> float {
        if (state_load(n, sc) != BG3_OK) return -1.0f;
        n->cfg = c;
        n->h.izh_hw_every = c.izh_hw_every;
        drop_graph(n);
        return time_steps(n, steps);
    };
    float ms = 0.0f;
    rc = tune(cur, !bg3::sweep_is_thin(h, cur), bg3::sweep_is_thin(h, cur), h.Mq, false,
              h.neuron_kind == BG3_NEURON_IZH, trial, ms);
    if (rc == BG3_OK && tune_growth) {
        // the overlap pass: one growth pass per candidate block size from the saved state
        float best_g = -1.0f;
        int best_t = cur.growth_threads;
        for (int t : {128, 256, 512}) {
            if (state_load(n, sc) != BG3_OK) { rc = BG3_ECUDA; break; }
            cudaEvent_t a, b;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, n->stream);
            bg3::launch_growth(h, n->d, 0, t, n->stream);
            cudaEventRecord(b, n->stream);
            float g = -1.0f;
            if (cudaEventSynchronize(b) == cudaSuccess) cudaEventElapsedTime(&g, a, b);
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            if (g >= 0 && (best_g < 0 || g < best_g)) { best_g = g; best_t = t; }
        }
        cur.growth_threads = best_t;
    }
    int rc2 = state_load(n, sc);
    state_free(sc);
    n->cfg = cur;
    n->h.izh_hw_every = cur.izh_hw_every;
    drop_graph(n);
    if (rc) return rc;
    if (rc2) return rc2;
    if (best) *best = cfg_to(cur);
    if (best_ms) *best_ms = ms;
    return BG3_OK;
}

static float time_batch_steps(bg3_batch *b, int32_t steps)
{
    if (bg3_batch_step(b, GRAPH_STEPS + 3) != BG3_OK) return -1.0f;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return -1.0f;
    cudaEventRecord(e0, b->stream);
    int rc = bg3_batch_step(b, steps);
    cudaEventRecord(e1, b->stream);
    float ms = -1.0f;
    if (rc == BG3_OK && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms < 0 ? -1.0f : ms / (float)steps;
}

int bg3_batch_autotune(bg3_batch *b, int32_t steps, bg3_launch_cfg *best, float *best_ms)
{
    if (!b || steps < 1) return BG3_EINVAL;
    std::vector<StateCopy> sc(b->nets.size());
    int rc = BG3_OK;
    for (size_t k = 0; k < b->nets.size() && rc == BG3_OK; k++) rc = state_save(b->nets[k], sc[k]);
    bool thick = false, thin = false, izh = false;
    int mq = 1 << 30;
    for (bg3_net *n : b->nets) {
        izh = izh || n->h.neuron_kind == BG3_NEURON_IZH;
        if (bg3::sweep_is_thin(n->h, b->cfg)) thin = true;
        else thick = true;
        mq = std::min(mq, n->h.Mq);
    }
    LaunchCfg cur = b->cfg;
    auto trial = [&](const LaunchCfg &c) -> float {
        for (size_t k = 0; k < b->nets.size(); k++)
            if (state_load(b->nets[k], sc[k]) != BG3_OK) return -1.0f;
        // the thin / TMA split, the thin tile table's padding to blocks and the descriptors'
        // Izhikevich option depend on these
        const bool split = b->cfg.thin_max_quads != c.thin_max_quads ||
                           b->cfg.thin_warps != c.thin_warps ||
                           b->cfg.izh_hw_every != c.izh_hw_every;
        b->cfg = c;
        if (split && batch_refresh(b) != BG3_OK) return -1.0f;
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        return time_batch_steps(b, steps);
    };
    float ms = 0.0f;
    if (rc == BG3_OK) rc = tune(cur, thick, thin, thin ? 1 << 30 : mq, true, izh, trial, ms);
    int rc2 = BG3_OK;
    for (size_t k = 0; k < b->nets.size(); k++) {
        if (sc[k].buf && state_load(b->nets[k], sc[k]) != BG3_OK) rc2 = BG3_ECUDA;
        state_free(sc[k]);
    }
    b->cfg = cur;
    int rc3 = batch_refresh(b);
    if (rc) return rc;
    if (rc2) return rc2;
    if (rc3) return rc3;
    if (best) *best = cfg_to(cur);
    if (best_ms) *best_ms = ms;
    return BG3_OK;
}

// ---- checkpoints ------------------------------------------------------------------------------
// Every device array of a network, by its NetDev field.  A checkpoint holds each one's bytes with
// the size of its allocation; bg3_checkpoint_save refuses a network holding an allocation that
// this list does not name, so a new array cannot be left out silently.
#define BG3_NET_ARRAYS(X)                                                                         \
    X(step) X(sweep_done) X(dstep) X(err) X(noise_cursor) X(Vm) X(Vthresh) X(Vreset) X(I0) X(Inoise)       \
    X(C1) X(C2) X(Trefract) X(sp) X(refr) X(spikeCount) X(spikeCountOffset) X(history) X(ntype)   \
    X(Aconst) X(Bconst) X(Cconst) X(Dconst) X(u_izh) X(C3) X(ring) X(ring_n) X(psr) X(dcls)       \
    X(lcls) X(ev) X(src) X(stype) X(count) X(dtab) X(ltab) X(outBegin) X(outCount) X(outMap)      \
    X(outFill) X(radii) X(rates) X(xloc) X(yloc) X(grow_exp) X(grow_rmax) X(burstiness)           \
    X(spikes_hist)                                                                                \
    X(rates_hist) X(radii_hist) X(reg_values) X(reg_shift) X(pois_mask) X(pois_nisi) X(in_psr)    \
    X(in_decay) X(in_queue) X(in_delay) X(in_ev) X(isi_begin) X(isi_vals) X(isi_cursor)

#define BG3_COUNT_ONE(f) +1
static const uint32_t CKPT_ARRAYS = 0 BG3_NET_ARRAYS(BG3_COUNT_ONE);
#undef BG3_COUNT_ONE

struct CkptHeader {
    char magic[8];             // "BG3CKPT"
    uint32_t version;          // CKPT_VERSION
    uint32_t netdev_bytes;     // sizeof(NetDev) of the writing library
    uint64_t total_bytes;      // whole checkpoint
    bg3_net_desc desc;
    LaunchCfg cfg;
    int64_t noise_count;       // injected noise values held (consumed ones included)
    uint32_t n_dtab, n_ltab;   // decay / delay class tables
    uint32_t n_arrays;         // CKPT_ARRAYS
    uint32_t pad;
    uint64_t checksum;         // FNV-1a 64 of every byte after the header
};
static_assert(sizeof(CkptHeader) == 144, "checkpoint header layout");
static const uint32_t CKPT_VERSION = 5;
static const char CKPT_MAGIC[8] = {'B', 'G', '3', 'C', 'K', 'P', 'T', 0};

static uint64_t fnv1a64(const char *p, uint64_t n)
{
    uint64_t h = 0xcbf29ce484222325ull;
    for (uint64_t i = 0; i < n; i++) {
        h ^= (uint8_t)p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

static size_t alloc_size(const bg3_net *n, const void *p)
{
    if (!p) return 0;
    for (auto &a : n->allocs)
        if (a.first == p) return a.second;
    return 0;
}

static void afree(bg3_net *n, const void *p)
{
    for (auto &a : n->allocs)
        if (a.first && a.first == p) {
            cudaFree(a.first);
            n->bytes -= a.second;
            a = std::make_pair((void *)nullptr, (size_t)0);
        }
}

// Gives field an allocation of exactly `bytes` (none for 0), keeping one of that size.
template <typename T>
static int aresize(bg3_net *n, T *&field, size_t bytes)
{
    if (field && alloc_size(n, field) == bytes) return BG3_OK;
    if (field) afree(n, field);
    field = nullptr;
    if (!bytes) return BG3_OK;
    if (bytes % sizeof(T)) return BG3_EINVAL;
    return dalloc(n, &field, bytes / sizeof(T));
}

// Index of each array in the checkpoint's list.
enum CkptArray {
#define BG3_ENUM_ONE(f) CKA_##f,
    BG3_NET_ARRAYS(BG3_ENUM_ONE)
#undef BG3_ENUM_ONE
    CKA_COUNT
};

// Arrays that an external input or its injected intervals add after bg3_create: a checkpoint
// may hold them where the live network does not (or the reverse).  Every other array must have
// the live network's allocation size exactly, so that no buffer a tensor map, a captured graph
// or a kernel bound was derived from changes size.
static bool ckpt_optional(int i)
{
    switch (i) {
    case CKA_reg_values: case CKA_reg_shift: case CKA_pois_mask: case CKA_pois_nisi:
    case CKA_in_psr: case CKA_in_decay: case CKA_in_queue: case CKA_in_delay: case CKA_in_ev:
    case CKA_isi_begin: case CKA_isi_vals: case CKA_isi_cursor:
        return true;
    default:
        return false;
    }
}

// The allocation size an optional array has when present (dalloc's max(count, 1) elements);
// 0 for isi_vals, whose length is the number of intervals drawn ahead.
static uint64_t ckpt_optional_size(int i, uint64_t N)
{
    switch (i) {
    case CKA_reg_values: case CKA_reg_shift: case CKA_pois_nisi: case CKA_in_psr:
    case CKA_in_decay: case CKA_in_queue: case CKA_isi_cursor:
        return 4 * N;
    case CKA_pois_mask: case CKA_in_delay: return N;
    case CKA_in_ev: return N * sizeof(EvSlot);
    case CKA_isi_begin: return 4 * (N + 1);
    default: return 0;
    }
}

// Element i of an array held in a checkpoint's bytes (which need not be aligned).
template <typename T>
static T ckpt_get(const char *base, uint64_t i)
{
    T v;
    memcpy(&v, base + i * sizeof(T), sizeof(T));
    return v;
}

// Checks the index-like contents of a checkpoint (every value a kernel uses to address memory)
// against the live network's shape.  Returns BG3_OK or BG3_EINVAL; reads host bytes only.
static int ckpt_check_contents(const bg3_net *n, const NetDev &sv, const char *const *ap,
                               const uint64_t *as, int64_t noise_count)
{
    const uint64_t N = (uint64_t)n->h.N, Np = (uint64_t)n->h.Np, Mq = (uint64_t)n->h.Mq;
    const uint64_t S = Np * Mq * 4;
    // per-dest in-use prefix and the slots behind it
    for (uint64_t d = 0; d < N; d++) {
        const uint32_t c = ckpt_get<uint32_t>(ap[CKA_count], d);
        if (c > (uint32_t)n->h.max_syn) return BG3_EINVAL;
        for (uint32_t k = 0; k < c; k++) {
            const uint64_t q = slot_pos((int)k, (int)d, (int)Mq);
            const int32_t s = ckpt_get<int32_t>(ap[CKA_src], q);
            const int8_t t = ckpt_get<int8_t>(ap[CKA_stype], q);
            const uint8_t l = ckpt_get<uint8_t>(ap[CKA_lcls], q);
            const uint32_t dw = ckpt_get<uint32_t>(ap[CKA_dcls], q >> 3);
            const uint32_t dc = (dw >> (4u * (uint32_t)(q & 7))) & 15u;
            EvSlot e;
            memcpy(&e, ap[CKA_ev] + q * sizeof(EvSlot), sizeof(EvSlot));
            if (s < 0 || (uint64_t)s >= N || t < 0 || t > 3 || l >= (uint8_t)sv.n_delays ||
                dc >= (uint32_t)sv.n_dcls || e.dcls >= (uint8_t)sv.n_dcls ||
                (sv.n_pcls > 0 && e.pcls >= (uint8_t)sv.n_pcls))
                return BG3_EINVAL;
        }
    }
    // spike ring: per slot a count and that many neuron ids
    for (uint64_t r = 0; r < BG3_RING; r++) {
        const int32_t m = ckpt_get<int32_t>(ap[CKA_ring_n], r);
        if (m < 0 || (uint64_t)m > N) return BG3_EINVAL;
        for (int32_t i = 0; i < m; i++) {
            const int32_t id = ckpt_get<int32_t>(ap[CKA_ring], r * N + (uint64_t)i);
            if (id < 0 || (uint64_t)id >= N) return BG3_EINVAL;
        }
    }
    // outgoing map: runs inside the map, entries inside the planes
    const uint64_t om = as[CKA_outMap] / 4;
    for (uint64_t i = 0; i < N * BG3_MAX_DELAYS; i++) {
        const uint64_t b = ckpt_get<uint32_t>(ap[CKA_outBegin], i);
        const uint64_t c = ckpt_get<uint32_t>(ap[CKA_outCount], i);
        if (b + c > om) return BG3_EINVAL;
    }
    for (uint64_t i = 0; i < om; i++)
        if (ckpt_get<uint32_t>(ap[CKA_outMap], i) >= S) return BG3_EINVAL;
    // injected noise and intervals: cursors inside what is held
    if (ckpt_get<unsigned long long>(ap[CKA_noise_cursor], 0) > (unsigned long long)noise_count)
        return BG3_EINVAL;
    if (as[CKA_isi_begin]) {
        const uint64_t nv = as[CKA_isi_vals] / 4;
        int32_t prev = 0;
        for (uint64_t i = 0; i <= N; i++) {
            const int32_t b = ckpt_get<int32_t>(ap[CKA_isi_begin], i);
            if (b < prev || (uint64_t)b > nv) return BG3_EINVAL;
            prev = b;
        }
    }
    if (as[CKA_isi_cursor])
        for (uint64_t i = 0; i < N; i++)
            if (ckpt_get<int32_t>(ap[CKA_isi_cursor], i) < 0) return BG3_EINVAL;
    if (as[CKA_in_delay])
        for (uint64_t i = 0; i < N; i++)
            if (ckpt_get<uint8_t>(ap[CKA_in_delay], i) > 31) return BG3_EINVAL;
    return BG3_OK;
}

extern "C" {

int bg3_checkpoint_save(bg3_net *n, void *buf, uint64_t cap, uint64_t *len)
{
    if (!n || !len) return BG3_EINVAL;
    CK(cudaStreamSynchronize(n->stream));
    const NetDev &h = n->h;
    uint64_t arrays = 0, named = 0;
#define BG3_SIZE_ONE(f) { const size_t s = alloc_size(n, h.f); arrays += 8 + s; named += s; }
    BG3_NET_ARRAYS(BG3_SIZE_ONE)
#undef BG3_SIZE_ONE
    if (named != n->bytes) return BG3_EUNSUPPORTED;  // an allocation outside the list
    const int64_t noise = (n->noise_dev && h.noise_len > 0) ? h.noise_len : 0;
    const uint64_t total = sizeof(CkptHeader) + sizeof(NetDev) + n->dtab.size() * sizeof(float) +
                           n->ltab.size() * sizeof(int32_t) + (uint64_t)noise * sizeof(float) + arrays;
    *len = total;
    if (!buf) return BG3_OK;
    if (cap < total) return BG3_EINVAL;
    char *p = (char *)buf;
    CkptHeader hd;
    memset(&hd, 0, sizeof(hd));
    memcpy(hd.magic, CKPT_MAGIC, 8);
    hd.version = CKPT_VERSION;
    hd.netdev_bytes = (uint32_t)sizeof(NetDev);
    hd.total_bytes = total;
    hd.desc = n->desc;
    hd.cfg = n->cfg;
    hd.noise_count = noise;
    hd.n_dtab = (uint32_t)n->dtab.size();
    hd.n_ltab = (uint32_t)n->ltab.size();
    hd.n_arrays = CKPT_ARRAYS;
    p += sizeof(hd);
    memcpy(p, &h, sizeof(NetDev));  // scalars; its pointers mean nothing to a reader
    p += sizeof(NetDev);
    memcpy(p, n->dtab.data(), n->dtab.size() * sizeof(float));
    p += n->dtab.size() * sizeof(float);
    memcpy(p, n->ltab.data(), n->ltab.size() * sizeof(int32_t));
    p += n->ltab.size() * sizeof(int32_t);
    if (noise) {
        CK(cudaMemcpy(p, n->noise_dev, (size_t)noise * sizeof(float), cudaMemcpyDeviceToHost));
        p += (size_t)noise * sizeof(float);
    }
#define BG3_SAVE_ONE(f)                                                                           \
    {                                                                                             \
        const uint64_t s = alloc_size(n, h.f);                                                    \
        memcpy(p, &s, 8);                                                                         \
        p += 8;                                                                                   \
        if (s) CK(cudaMemcpy(p, h.f, s, cudaMemcpyDeviceToHost));                                 \
        p += s;                                                                                   \
    }
    BG3_NET_ARRAYS(BG3_SAVE_ONE)
#undef BG3_SAVE_ONE
    hd.checksum = fnv1a64((const char *)buf + sizeof(hd), total - sizeof(hd));
    memcpy(buf, &hd, sizeof(hd));
    return BG3_OK;
}

// Loads in two phases.  The first reads and checks everything against the live network without
// changing it: the header and checksum, every shape scalar of the saved descriptor, every
// array's size (only an external input's arrays may differ, see ckpt_optional) and every
// index-like value (ckpt_check_contents).  Any mismatch returns BG3_EINVAL with the network
// untouched.  The second drops the captured graph, copies the arrays, takes the exp tables of the
// saved time constants and only then installs the saved scalars; a CUDA or allocation failure in
// it leaves the network unusable (destroy it), never pointing at another process's memory.
int bg3_checkpoint_load(bg3_net *n, const void *buf, uint64_t len)
{
    if (!n || !buf || len < sizeof(CkptHeader) + sizeof(NetDev)) return BG3_EINVAL;
    const char *p = (const char *)buf, *end = p + len;
    CkptHeader hd;
    memcpy(&hd, p, sizeof(hd));
    if (memcmp(hd.magic, CKPT_MAGIC, 8) || hd.version != CKPT_VERSION ||
        hd.netdev_bytes != sizeof(NetDev) || hd.total_bytes != len || hd.n_arrays != CKPT_ARRAYS ||
        memcmp(&hd.desc, &n->desc, sizeof(bg3_net_desc)) || hd.n_dtab > BG3_MAX_DCLS ||
        hd.n_ltab > BG3_MAX_DELAYS || hd.noise_count < 0)
        return BG3_EINVAL;
    if (hd.checksum != fnv1a64(p + sizeof(hd), len - sizeof(hd))) return BG3_EINVAL;
    const bg3_launch_cfg lc = cfg_to(hd.cfg);
    if (!cfg_valid(&lc)) return BG3_EINVAL;
    p += sizeof(hd);
    NetDev sv;
    memcpy(&sv, p, sizeof(NetDev));
    p += sizeof(NetDev);
    // noise_count is bounded by the bytes left before it enters any product
    if ((uint64_t)hd.noise_count > (uint64_t)(end - p) / sizeof(float)) return BG3_EINVAL;
    const uint64_t fixed = hd.n_dtab * sizeof(float) + hd.n_ltab * sizeof(int32_t) +
                           (uint64_t)hd.noise_count * sizeof(float);
    if ((uint64_t)(end - p) < fixed) return BG3_EINVAL;
    const char *dtab = p, *ltab = p + hd.n_dtab * sizeof(float);
    const char *noise = p + hd.n_dtab * sizeof(float) + hd.n_ltab * sizeof(int32_t);
    p += fixed;
    NetDev &h = n->h;
    // shape scalars: what the live allocations, tensor maps and launch geometry derive from
    if (sv.N != h.N || sv.Np != h.Np || sv.max_syn != h.max_syn || sv.max_spikes != h.max_spikes ||
        sv.Mq != h.Mq || sv.ntiles != h.ntiles || sv.neuron_kind != h.neuron_kind ||
        sv.syn_kind != h.syn_kind || fbits(sv.dt) != fbits(h.dt) ||
        sv.n_burst_bins != h.n_burst_bins || sv.n_spike_bins != h.n_spike_bins ||
        sv.max_epochs != h.max_epochs || sv.n_dcls != (int32_t)hd.n_dtab ||
        sv.n_delays != (int32_t)hd.n_ltab || sv.n_expc < 0 || sv.n_expc > BG3_MAX_EXPC ||
        sv.n_pcls < 0 || sv.n_pcls > BG3_MAX_PCLS || sv.input_kind < 0 || sv.input_kind > 2 ||
        sv.grid_w < 0 || sv.grid_h < 0 || (long long)sv.grid_w * sv.grid_h != (sv.grid_w ? sv.N : 0))
        return BG3_EINVAL;
    for (int t = 0; t < 4; t++)
        if (sv.t_dcls[t] < 0 || sv.t_dcls[t] >= BG3_MAX_DCLS || sv.t_lcls[t] < 0 ||
            sv.t_lcls[t] >= BG3_MAX_DELAYS || sv.t_pcls[t] < 0 || sv.t_pcls[t] >= BG3_MAX_PCLS ||
            sv.stdp[t].dlen_pos < 0 || sv.stdp[t].dlen_pos > BG3_DEXP_LEN ||
            sv.stdp[t].dlen_neg < 0 || sv.stdp[t].dlen_neg > BG3_DEXP_LEN ||
            !(sv.stdp[t].mupos == 0.0f) || !(sv.stdp[t].muneg == 0.0f))
            return BG3_EINVAL;
    for (uint32_t i = 0; i < hd.n_ltab; i++) {
        const int32_t D = ckpt_get<int32_t>(ltab, i);
        if (D < 1 || D > 31) return BG3_EINVAL;
    }
    // the array list: sizes first
    const char *ap[CKA_COUNT];
    uint64_t as[CKA_COUNT];
    const uint64_t N = (uint64_t)h.N;
    for (int i = 0; i < CKA_COUNT; i++) {
        uint64_t s;
        if ((uint64_t)(end - p) < 8) return BG3_EINVAL;
        memcpy(&s, p, 8);
        p += 8;
        if ((uint64_t)(end - p) < s) return BG3_EINVAL;
        ap[i] = p;
        as[i] = s;
        p += s;
    }
    if (p != end) return BG3_EINVAL;
    {
        uint64_t live[CKA_COUNT];
#define BG3_LIVE_ONE(f) live[CKA_##f] = alloc_size(n, h.f);
        BG3_NET_ARRAYS(BG3_LIVE_ONE)
#undef BG3_LIVE_ONE
        for (int i = 0; i < CKA_COUNT; i++) {
            if (as[i] == live[i]) continue;
            if (!ckpt_optional(i)) return BG3_EINVAL;
            const uint64_t want = ckpt_optional_size(i, N);
            if (as[i] != 0 && (want ? as[i] != want : (as[i] % 4) != 0)) return BG3_EINVAL;
        }
    }
    // an input's arrays come as a set, and the descriptor's input kind agrees with them
    const bool reg = as[CKA_reg_values] && as[CKA_reg_shift];
    const bool pois = as[CKA_pois_mask] && as[CKA_pois_nisi] && as[CKA_in_psr] &&
                      as[CKA_in_decay] && as[CKA_in_queue] && as[CKA_in_delay] && as[CKA_in_ev] &&
                      as[CKA_isi_cursor];
    if ((sv.input_kind == 1 && !reg) || (sv.input_kind == 2 && !pois) ||
        (as[CKA_isi_begin] != 0) != (as[CKA_isi_vals] != 0) || (as[CKA_isi_begin] && !pois))
        return BG3_EINVAL;
    int rc = ckpt_check_contents(n, sv, ap, as, hd.noise_count);
    if (rc) return rc;

    // ---- second phase: nothing above changed the network ----
    CK(cudaStreamSynchronize(n->stream));
    drop_graph(n);
#define BG3_LOAD_ONE(f)                                                                           \
    {                                                                                             \
        if ((rc = aresize(n, h.f, (size_t)as[CKA_##f]))) return rc;                               \
        if (as[CKA_##f])                                                                          \
            CK(cudaMemcpy((void *)h.f, ap[CKA_##f], (size_t)as[CKA_##f], cudaMemcpyHostToDevice)); \
    }
    BG3_NET_ARRAYS(BG3_LOAD_ONE)
#undef BG3_LOAD_ONE
    if (n->noise_dev) cudaFree(n->noise_dev);
    n->noise_dev = nullptr;
    n->noise_cap = 0;
    h.noise_buf = nullptr;
    h.noise_len = 0;
    if (hd.noise_count) {
        if (cudaMalloc(&n->noise_dev, (size_t)hd.noise_count * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            n->noise_dev = nullptr;
            return BG3_ENOMEM;
        }
        CK(cudaMemcpy(n->noise_dev, noise, (size_t)hd.noise_count * sizeof(float),
                      cudaMemcpyHostToDevice));
        n->noise_cap = hd.noise_count;
    }
    // the saved scalars with this network's pointers; exp tables of the saved time constants
    // taken before the old ones are released, so that a failure leaves the old ones in place
    NetDev nh = sv;
#define BG3_KEEP_ONE(f) nh.f = h.f;
    BG3_NET_ARRAYS(BG3_KEEP_ONE)
#undef BG3_KEEP_ONE
    nh.noise_buf = n->noise_dev;
    nh.noise_len = hd.noise_count;
    std::vector<ExpKey> old_keys;
    old_keys.swap(n->exp_keys);
    auto fail = [&](int code) {
        const int32_t keep = h.n_expc;
        exp_release(n);                 // the tables taken for nh
        h.n_expc = keep;
        n->exp_keys.swap(old_keys);     // h keeps its own
        return code;
    };
    for (int c = 0; c < nh.n_expc; c++)
        if ((rc = exp_table<float>(n, 0, nh.expc_tau[c], BG3_EXP_LEN, &nh.expc_tab[c])))
            return fail(rc);
    for (int t = 0; t < 4; t++) {
        StdpConst &st = nh.stdp[t];
        st.dpos = st.dneg = nullptr;
        if (st.dlen_pos && (rc = exp_table<double>(n, 1, st.taupos, BG3_DEXP_LEN, &st.dpos)))
            return fail(rc);
        if (st.dlen_neg && (rc = exp_table<double>(n, 1, st.tauneg, BG3_DEXP_LEN, &st.dneg)))
            return fail(rc);
    }
    for (int c = 0; c < nh.n_pcls; c++) {
        nh.p_xD[c] = nh.p_xF[c] = nullptr;
        if (nh.p_D[c] > 0.0f && std::isfinite(nh.p_D[c]) &&
            (rc = exp_table<float>(n, 0, nh.p_D[c], BG3_EXP_LEN, &nh.p_xD[c])))
            return fail(rc);
        if (nh.p_F[c] > 0.0f && std::isfinite(nh.p_F[c]) &&
            (rc = exp_table<float>(n, 0, nh.p_F[c], BG3_EXP_LEN, &nh.p_xF[c])))
            return fail(rc);
    }
    {
        std::vector<ExpKey> taken;
        taken.swap(n->exp_keys);
        n->exp_keys.swap(old_keys);
        exp_release(n);                 // the old tables
        n->exp_keys.swap(taken);
    }
    h = nh;
    n->dtab.resize(hd.n_dtab);
    n->ltab.resize(hd.n_ltab);
    if (hd.n_dtab) memcpy(n->dtab.data(), dtab, hd.n_dtab * sizeof(float));
    if (hd.n_ltab) memcpy(n->ltab.data(), ltab, hd.n_ltab * sizeof(int32_t));
    n->cfg = hd.cfg;
    if ((rc = push_desc(n))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

}  // extern "C"
