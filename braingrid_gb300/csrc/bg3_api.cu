// C-ABI of libbg3: handle lifetime, host <-> device conversion between the reference's slot
// layout and the device plane layout, and the launch sequence of a step and of an epoch.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/bg3.h"
#include "bg3_internal.cuh"

namespace bg3 {
void launch_step(const NetDev &h, const NetDev *d_net, cudaStream_t s);
void launch_step_parts(const NetDev &h, const NetDev *d_net, cudaStream_t s, cudaEvent_t ev[4]);
void launch_growth(const NetDev &h, const NetDev *d_net, int epoch, cudaStream_t s);
void launch_rebuild_maps(const NetDev &h, const NetDev *d_net, cudaStream_t s);
}  // namespace bg3


struct bg3_net {
    bg3_net_desc desc;
    NetDev h;                 // host copy of the device descriptor
    NetDev *d = nullptr;      // device copy
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    long long noise_cap = 0;  // capacity of the injected-noise buffer (values)
    float *noise_dev = nullptr;
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float ms_neurons = 0, ms_fanout = 0, ms_sweep = 0;
    long long launches = 0;
    void *flush_buf = nullptr;
    size_t flush_size = 0;
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
    n->allocs.push_back(q);
    if (cudaMemsetAsync(q, fill, bytes, n->stream) != cudaSuccess) return BG3_ECUDA;
    *p = (T *)q;
    return BG3_OK;
}

static int push_desc(bg3_net *n)
{
    CK(cudaMemcpyAsync(n->d, &n->h, sizeof(NetDev), cudaMemcpyHostToDevice, n->stream));
    return BG3_OK;
}

template <typename T>
static int h2d(bg3_net *n, T *dst, const T *src, size_t count)
{
    if (!src) return BG3_OK;
    CK(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, n->stream));
    return BG3_OK;
}
template <typename T>
static int d2h(bg3_net *n, T *dst, const T *src, size_t count)
{
    if (!dst) return BG3_OK;
    CK(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, n->stream));
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
    if ((size_t)D.n_neurons * (size_t)D.max_syn_per_neuron > (size_t)BG3_POS_MASK) return BG3_EINVAL;
    if (D.neuron_kind != BG3_NEURON_LIF) return BG3_EUNSUPPORTED;
    if (D.synapse_kind != BG3_SYN_DS && D.synapse_kind != BG3_SYN_SPIKING) return BG3_EUNSUPPORTED;
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
    const size_t N = (size_t)D.n_neurons, S = N * (size_t)D.max_syn_per_neuron;
    h.N = D.n_neurons;
    h.max_syn = D.max_syn_per_neuron;
    h.max_spikes = max_spikes;
    h.neuron_kind = D.neuron_kind;
    h.syn_kind = D.synapse_kind;
    h.noise_mode = D.noise_mode;
    h.noise_seed = D.noise_seed;
    h.dt = D.delta_t;
    h.epoch_duration = D.epoch_duration;
    h.ntiles = (int)((N + 31) / 32);
    h.max_epochs = D.max_epochs;
    h.n_burst_bins = (int)((float)D.max_epochs * D.epoch_duration);
    h.n_spike_bins = (int)((float)D.max_epochs * D.epoch_duration * 100.0f);
    int rc = 0;
#define A(ptr, cnt) if ((rc = dalloc(n, &h.ptr, (cnt))) != 0) goto fail;
#define AF(ptr, cnt, f) if ((rc = dalloc(n, &h.ptr, (cnt), (f))) != 0) goto fail;
    A(step, 1) A(sweep_done, 1) A(err, 1) A(nspikes, 1) A(noise_cursor, 1)
    A(Vm, N) A(Vthresh, N) A(Vreset, N) A(I0, N) A(Inoise, N) A(C1, N) A(C2, N) A(Trefract, N)
    A(sp, N) A(refr, N) A(spikeCount, N) A(spikeCountOffset, N) A(ntype, N) A(spikes, N)
    AF(history, N * (size_t)max_spikes, 0xff)
    A(psr, S) A(decay, S) A(W, S) A(U, S) A(D, S) A(F, S) A(u, S) A(r, S) A(queue, S)
    A(lastSpike, S) A(src, S) A(stype, S) A(phase0, S) A(sdelay, S) A(count, N)
    A(outBegin, N) A(outCount, N) A(outMap, S) A(outFill, N)
    A(radii, N) A(rates, N) A(xloc, N) A(yloc, N)
    A(burstiness, (size_t)std::max(h.n_burst_bins, 1)) A(spikes_hist, (size_t)std::max(h.n_spike_bins, 1))
    A(rates_hist, (size_t)(D.max_epochs + 1) * N) A(radii_hist, (size_t)(D.max_epochs + 1) * N)
#undef A
#undef AF
    if (cudaMalloc((void **)&n->d, sizeof(NetDev)) != cudaSuccess) { rc = BG3_ENOMEM; goto fail; }
    // default type constants: tau, delay, U/D/F from createSynapse with this deltaT
    {
        const float tau[4] = {6e-3f, 6e-3f, 3e-3f, 3e-3f};
        const float dly[4] = {0.8e-3f, 0.8e-3f, 0.8e-3f, 1.5e-3f};
        const float U[4] = {0.32f, 0.25f, 0.05f, 0.5f}, Dd[4] = {0.144f, 0.7f, 0.125f, 1.1f},
                    F[4] = {0.06f, 0.02f, 1.2f, 0.05f};
        for (int t = 0; t < 4; t++) {
            h.t_tau[t] = tau[t];
            h.t_decay[t] = expf(-D.delta_t / tau[t]);
            h.t_delay[t] = (int)(dly[t] / D.delta_t) + 1;
            h.t_U[t] = U[t];
            h.t_D[t] = Dd[t];
            h.t_F[t] = F[t];
        }
        h.t_u0 = 0.4f;
        h.t_r0 = 1.0f;
    }
    if ((rc = push_desc(n)) != 0) goto fail;
    if (cudaStreamSynchronize(n->stream) != cudaSuccess) { rc = BG3_ECUDA; goto fail; }
    *out = n;
    return BG3_OK;
fail:
    cudaGetLastError();
    bg3_destroy(n);
    return rc;
}

int bg3_destroy(bg3_net *n)
{
    if (!n) return BG3_EINVAL;
    if (n->stream) cudaStreamSynchronize(n->stream);
    for (void *p : n->allocs) cudaFree(p);
    if (n->d) cudaFree(n->d);
    if (n->noise_dev) cudaFree(n->noise_dev);
    if (n->flush_buf) cudaFree(n->flush_buf);
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

int bg3_upload_layout(bg3_net *n, const float *x, const float *y, const int32_t *ntype)
{
    if (!n || !x || !y || !ntype) return BG3_EINVAL;
    size_t N = n->h.N;
    std::vector<int8_t> t(N);
    for (size_t i = 0; i < N; i++) {
        if (ntype[i] != 1 && ntype[i] != 2) return BG3_EINVAL;
        t[i] = (int8_t)ntype[i];
    }
    int rc;
    if ((rc = h2d(n, n->h.xloc, x, N)) || (rc = h2d(n, n->h.yloc, y, N)) ||
        (rc = h2d(n, n->h.ntype, t.data(), N)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_set_type_constants(bg3_net *n, const bg3_type_constants *c)
{
    if (!n || !c) return BG3_EINVAL;
    for (int t = 0; t < 4; t++) {
        if (c->total_delay[t] < 1 || c->total_delay[t] > 31) return BG3_EINVAL;
        n->h.t_tau[t] = c->tau[t];
        n->h.t_decay[t] = c->decay[t];
        n->h.t_delay[t] = c->total_delay[t];
        n->h.t_U[t] = c->U[t];
        n->h.t_D[t] = c->D[t];
        n->h.t_F[t] = c->F[t];
    }
    n->h.t_u0 = c->u0;
    n->h.t_r0 = c->r0;
    int rc = push_desc(n);
    if (rc) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

static inline uint32_t rotl32(uint32_t x, unsigned r) { r &= 31u; return r ? (x << r) | (x >> (32 - r)) : x; }
static inline uint32_t rotr32(uint32_t x, unsigned r) { r &= 31u; return r ? (x >> r) | (x << (32 - r)) : x; }

int bg3_upload_synapses(bg3_net *n, const bg3_synapse_arrays *a, uint64_t step)
{
    if (!n || !a || !a->in_use || !a->src || !a->type || !a->W || !a->psr || !a->decay ||
        !a->delayQueue || !a->delayIdx || !a->total_delay)
        return BG3_EINVAL;
    const size_t N = n->h.N, M = n->h.max_syn, S = N * M;
    const bool ds = n->h.syn_kind == BG3_SYN_DS;
    if (ds && (!a->U || !a->D || !a->F || !a->u || !a->r || !a->lastSpike)) return BG3_EINVAL;
    std::vector<float> psr(S, 0.f), decay(S, 0.f), W(S, 0.f), U(S, 0.f), Dd(S, 0.f), F(S, 0.f),
        u(S, 0.f), r(S, 0.f);
    std::vector<uint32_t> queue(S, 0u), count(N, 0u);
    std::vector<unsigned long long> last(S, BG3_ULONG_MAX);
    std::vector<int32_t> src(S, 0);
    std::vector<int8_t> st(S, 0);
    std::vector<uint8_t> ph(S, 0), dl(S, 0);
    for (size_t d = 0; d < N; d++) {
        size_t c = 0;
        while (c < M && a->in_use[d * M + c]) c++;
        for (size_t k = c; k < M; k++)
            if (a->in_use[d * M + k]) return BG3_EINVAL;  // in-use slots must be a prefix
        if (a->counts && a->counts[d] != c) return BG3_EINVAL;
        count[d] = (uint32_t)c;
        for (size_t k = 0; k < c; k++) {
            size_t i = d * M + k, p = k * N + d;
            if (a->src[i] < 0 || (size_t)a->src[i] >= N || a->type[i] < 0 || a->type[i] > 3 ||
                a->total_delay[i] < 1 || a->total_delay[i] > 31 || a->delayIdx[i] < 0 ||
                a->delayIdx[i] > 31)
                return BG3_EINVAL;
            unsigned phase = (unsigned)((step - (uint64_t)a->delayIdx[i]) & 31u);
            psr[p] = a->psr[i];
            decay[p] = a->decay[i];
            W[p] = a->W[i];
            queue[p] = rotl32(a->delayQueue[i], phase);
            src[p] = a->src[i];
            st[p] = (int8_t)a->type[i];
            ph[p] = (uint8_t)phase;
            dl[p] = (uint8_t)a->total_delay[i];
            if (ds) {
                U[p] = a->U[i]; Dd[p] = a->D[i]; F[p] = a->F[i]; u[p] = a->u[i]; r[p] = a->r[i];
                last[p] = a->lastSpike[i];
            }
        }
    }
    NetDev &h = n->h;
    int rc;
    if ((rc = h2d(n, h.psr, psr.data(), S)) || (rc = h2d(n, h.decay, decay.data(), S)) ||
        (rc = h2d(n, h.W, W.data(), S)) || (rc = h2d(n, h.U, U.data(), S)) ||
        (rc = h2d(n, h.D, Dd.data(), S)) || (rc = h2d(n, h.F, F.data(), S)) ||
        (rc = h2d(n, h.u, u.data(), S)) || (rc = h2d(n, h.r, r.data(), S)) ||
        (rc = h2d(n, h.queue, queue.data(), S)) || (rc = h2d(n, h.lastSpike, last.data(), S)) ||
        (rc = h2d(n, h.src, src.data(), S)) || (rc = h2d(n, h.stype, st.data(), S)) ||
        (rc = h2d(n, h.phase0, ph.data(), S)) || (rc = h2d(n, h.sdelay, dl.data(), S)) ||
        (rc = h2d(n, h.count, count.data(), N)))
        return rc;
    unsigned long long s64 = step;
    CK(cudaMemcpyAsync(h.step, &s64, sizeof(s64), cudaMemcpyHostToDevice, n->stream));
    bg3::launch_rebuild_maps(h, n->d, n->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_upload_growth(bg3_net *n, const bg3_growth_params *p, const float *radii,
                      const float *rates)
{
    if (!n || !p) return BG3_EINVAL;
    NetDev &h = n->h;
    h.g_epsilon = p->epsilon; h.g_beta = p->beta; h.g_rho = p->rho;
    h.g_target_rate = p->target_rate; h.g_min_radius = p->min_radius;
    h.g_start_radius = p->start_radius; h.g_max_rate = p->max_rate;
    size_t N = h.N;
    int rc;
    if ((rc = h2d(n, h.radii, radii, N)) || (rc = h2d(n, h.rates, rates, N))) return rc;
    // recorder row 0 holds the start values (XmlGrowthRecorder::initDefaultValues / initValues)
    if (radii) CK(cudaMemcpyAsync(h.radii_hist, radii, N * sizeof(float), cudaMemcpyHostToDevice, n->stream));
    if (rates) CK(cudaMemcpyAsync(h.rates_hist, rates, N * sizeof(float), cudaMemcpyHostToDevice, n->stream));
    if ((rc = push_desc(n))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return BG3_OK;
}

int bg3_upload_weights(bg3_net *n, const float *Wref)
{
    if (!n || !Wref) return BG3_EINVAL;
    const size_t N = n->h.N, M = n->h.max_syn, S = N * M;
    std::vector<uint32_t> count(N);
    std::vector<float> W(S);
    int rc;
    if ((rc = d2h(n, count.data(), n->h.count, N)) || (rc = d2h(n, W.data(), n->h.W, S))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    for (size_t d = 0; d < N; d++)
        for (size_t k = 0; k < count[d]; k++) W[k * N + d] = Wref[d * M + k];
    if ((rc = h2d(n, n->h.W, W.data(), S))) return rc;
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

// ---- hot path -------------------------------------------------------------------------------
int bg3_step(bg3_net *n, int64_t nsteps)
{
    if (!n || nsteps < 0) return BG3_EINVAL;
    if (n->timing) {
        for (int i = 0; i < 4; i++)
            if (!n->ev[i]) CK(cudaEventCreate(&n->ev[i]));
        n->ms_neurons = n->ms_fanout = n->ms_sweep = 0;
        for (int64_t s = 0; s < nsteps; s++) {
            bg3::launch_step_parts(n->h, n->d, n->stream, n->ev);
            CK(cudaEventSynchronize(n->ev[3]));
            float a, b, c;
            cudaEventElapsedTime(&a, n->ev[0], n->ev[1]);
            cudaEventElapsedTime(&b, n->ev[1], n->ev[2]);
            cudaEventElapsedTime(&c, n->ev[2], n->ev[3]);
            n->ms_neurons += a; n->ms_fanout += b; n->ms_sweep += c;
        }
    } else {
        for (int64_t s = 0; s < nsteps; s++) bg3::launch_step(n->h, n->d, n->stream);
    }
    n->launches += 3 * nsteps;
    CK(cudaGetLastError());
    return BG3_OK;
}

int bg3_epoch_growth(bg3_net *n, int32_t epoch)
{
    if (!n || epoch < 0) return BG3_EINVAL;
    bg3::launch_growth(n->h, n->d, epoch, n->stream);
    n->launches += 8;
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

int bg3_download_synapses(bg3_net *n, bg3_synapse_arrays *a)
{
    if (!n || !a) return BG3_EINVAL;
    const size_t N = n->h.N, M = n->h.max_syn, S = N * M;
    NetDev &h = n->h;
    std::vector<float> psr(S), decay(S), W(S), U(S), Dd(S), F(S), u(S), r(S);
    std::vector<uint32_t> queue(S), count(N);
    std::vector<unsigned long long> last(S);
    std::vector<int32_t> src(S);
    std::vector<int8_t> st(S);
    std::vector<uint8_t> ph(S), dl(S);
    unsigned long long step = 0;
    int rc;
    if ((rc = d2h(n, psr.data(), h.psr, S)) || (rc = d2h(n, decay.data(), h.decay, S)) ||
        (rc = d2h(n, W.data(), h.W, S)) || (rc = d2h(n, U.data(), h.U, S)) ||
        (rc = d2h(n, Dd.data(), h.D, S)) || (rc = d2h(n, F.data(), h.F, S)) ||
        (rc = d2h(n, u.data(), h.u, S)) || (rc = d2h(n, r.data(), h.r, S)) ||
        (rc = d2h(n, queue.data(), h.queue, S)) || (rc = d2h(n, last.data(), h.lastSpike, S)) ||
        (rc = d2h(n, src.data(), h.src, S)) || (rc = d2h(n, st.data(), h.stype, S)) ||
        (rc = d2h(n, ph.data(), h.phase0, S)) || (rc = d2h(n, dl.data(), h.sdelay, S)) ||
        (rc = d2h(n, count.data(), h.count, N)) || (rc = d2h(n, &step, h.step, 1)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    for (size_t d = 0; d < N; d++) {
        if (a->counts) a->counts[d] = count[d];
        for (size_t k = 0; k < M; k++) {
            size_t i = d * M + k, p = k * N + d;
            bool used = k < count[d];
            if (a->in_use) a->in_use[i] = used ? 1 : 0;
            if (!used) continue;
            if (a->src) a->src[i] = src[p];
            if (a->type) a->type[i] = st[p];
            if (a->W) a->W[i] = W[p];
            if (a->psr) a->psr[i] = psr[p];
            if (a->decay) a->decay[i] = decay[p];
            if (a->total_delay) a->total_delay[i] = dl[p];
            if (a->delayIdx) a->delayIdx[i] = (int32_t)((step - ph[p]) & 31u);
            if (a->delayQueue) a->delayQueue[i] = rotr32(queue[p], ph[p]);
            if (a->tau) a->tau[i] = h.t_tau[st[p] & 3];
            if (a->U) a->U[i] = U[p];
            if (a->D) a->D[i] = Dd[p];
            if (a->F) a->F[i] = F[p];
            if (a->u) a->u[i] = u[p];
            if (a->r) a->r[i] = r[p];
            if (a->lastSpike) a->lastSpike[i] = last[p];
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

// The device keeps the outgoing map as plane positions grouped by source in arbitrary order
// (spike propagation does not depend on it) and the incoming map implicitly as the in-use row
// prefixes.  Both are returned in the reference's order: slot ids d * maxSyn + k, ascending
// within each source; incoming in dest-major slot order (Synapses/AllSynapses.cpp:223-293).
int bg3_download_maps(bg3_net *n, bg3_index_maps *m)
{
    if (!n || !m) return BG3_EINVAL;
    const size_t N = n->h.N, M = n->h.max_syn;
    std::vector<uint32_t> ob(N), oc(N), count(N);
    int rc;
    if ((rc = d2h(n, ob.data(), n->h.outBegin, N)) || (rc = d2h(n, oc.data(), n->h.outCount, N)) ||
        (rc = d2h(n, count.data(), n->h.count, N)))
        return rc;
    CK(cudaStreamSynchronize(n->stream));
    size_t total = 0;
    for (uint32_t c : count) total += c;
    std::vector<uint32_t> om(std::max<size_t>(total, 1));
    if (total && (rc = d2h(n, om.data(), n->h.outMap, total))) return rc;
    CK(cudaStreamSynchronize(n->stream));
    for (size_t i = 0; i < N; i++) {
        if (m->outgoingSynapseBegin) m->outgoingSynapseBegin[i] = ob[i];
        if (m->outgoingSynapseCount) m->outgoingSynapseCount[i] = oc[i];
        std::vector<uint32_t> ids(oc[i]);
        for (uint32_t j = 0; j < oc[i]; j++) {
            uint32_t p = om[ob[i] + j] & BG3_POS_MASK;
            ids[j] = (uint32_t)((p % N) * M + p / N);
        }
        std::sort(ids.begin(), ids.end());
        if (m->outgoingSynapseIndexMap)
            for (uint32_t j = 0; j < oc[i]; j++) m->outgoingSynapseIndexMap[ob[i] + j] = ids[j];
    }
    uint32_t acc = 0;
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

int bg3_bench_steps(bg3_net *n, int64_t nsteps, int64_t flush_bytes, float *step_ms,
                    float *kernel_ms)
{
    if (!n || nsteps < 0 || !step_ms) return BG3_EINVAL;
    if (flush_bytes > 0 && (size_t)flush_bytes > n->flush_size) {
        if (n->flush_buf) cudaFree(n->flush_buf);
        n->flush_buf = nullptr;
        n->flush_size = 0;
        if (cudaMalloc(&n->flush_buf, (size_t)flush_bytes) != cudaSuccess) {
            cudaGetLastError();
            return BG3_ENOMEM;
        }
        n->flush_size = (size_t)flush_bytes;
    }
    const int per = kernel_ms ? 4 : 2;
    std::vector<cudaEvent_t> ev((size_t)nsteps * per);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (int64_t s = 0; s < nsteps; s++) {
        if (flush_bytes > 0)
            CK(cudaMemsetAsync(n->flush_buf, (int)(s & 0xff), (size_t)flush_bytes, n->stream));
        cudaEvent_t *e = &ev[(size_t)s * per];
        if (kernel_ms) {
            bg3::launch_step_parts(n->h, n->d, n->stream, e);
        } else {
            CK(cudaEventRecord(e[0], n->stream));
            bg3::launch_step(n->h, n->d, n->stream);
            CK(cudaEventRecord(e[1], n->stream));
        }
    }
    n->launches += 3 * nsteps;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(n->stream));
    for (int64_t s = 0; s < nsteps; s++) {
        cudaEvent_t *e = &ev[(size_t)s * per];
        CK(cudaEventElapsedTime(&step_ms[s], e[0], e[per - 1]));
        if (kernel_ms)
            for (int k = 0; k < 3; k++) CK(cudaEventElapsedTime(&kernel_ms[3 * s + k], e[k], e[k + 1]));
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return BG3_OK;
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
