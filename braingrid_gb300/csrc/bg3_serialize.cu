// The reference's checkpoint stream (include/bg3.h: bg3_serialize, bg3_deserialize): the bytes
// Model::serialize writes (Core/Model.cpp:85-98), produced from and read back into a network
// through the public C-ABI.  Host code only.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/bg3.h"

namespace {

const int32_t LENGTH_OF_DELAYQUEUE = 32;  // Synapses/AllSpikingSynapses.h:355

// Writes NUL-terminated values; counts the bytes whether or not they fit.
struct Out {
    char *buf;
    uint64_t cap, len = 0;
    void put(const char *t, int k)
    {
        if (buf && len + (uint64_t)k + 1 <= cap) {
            memcpy(buf + len, t, (size_t)k);
            buf[len + (uint64_t)k] = 0;  // std::ends
        }
        len += (uint64_t)k + 1;
    }
    // std::ostream << float: the float converted to double, "%.*g" with the default precision 6
    void f(float v)
    {
        char t[48];
        put(t, snprintf(t, sizeof t, "%.*g", 6, (double)v));
    }
    void i(long long v)
    {
        char t[24];
        put(t, snprintf(t, sizeof t, "%lld", v));
    }
    void u(unsigned long long v)
    {
        char t[24];
        put(t, snprintf(t, sizeof t, "%llu", v));
    }
};

// Reads NUL-terminated values; any malformed or missing value sets bad.
struct In {
    const char *p, *end;
    bool bad = false;
    const char *tok(const char **tend)
    {
        if (bad) return nullptr;
        const char *q = (const char *)memchr(p, 0, (size_t)(end - p));
        if (!q || q == p) {
            bad = true;
            return nullptr;
        }
        const char *t = p;
        *tend = q;
        p = q + 1;
        return t;
    }
    float f()
    {
        const char *e, *t = tok(&e);
        if (!t) return 0.0f;
        char *stop;
        errno = 0;
        const float v = strtof(t, &stop);  // what std::istream >> float parses
        if (stop != e) bad = true;
        return v;
    }
    long long i()
    {
        const char *e, *t = tok(&e);
        if (!t) return 0;
        char *stop;
        errno = 0;
        const long long v = strtoll(t, &stop, 10);
        if (stop != e || errno) bad = true;
        return v;
    }
    unsigned long long u()
    {
        const char *e, *t = tok(&e);
        if (!t || *t == '-') {
            bad = true;
            return 0;
        }
        char *stop;
        errno = 0;
        const unsigned long long v = strtoull(t, &stop, 10);
        if (stop != e || errno) bad = true;
        return v;
    }
};

struct Nets {
    size_t N, M, S;
    bool izh, dyn, stdp;
};

Nets shape(const bg3_net_desc &d)
{
    Nets s;
    s.N = (size_t)d.n_neurons;
    s.M = (size_t)d.max_syn_per_neuron;
    s.S = s.N * s.M;
    s.izh = d.neuron_kind == BG3_NEURON_IZH;
    s.dyn = d.synapse_kind == BG3_SYN_DS || d.synapse_kind == BG3_SYN_DYNSTDP;
    s.stdp = d.synapse_kind == BG3_SYN_STDP || d.synapse_kind == BG3_SYN_DYNSTDP;
    return s;
}

// Host copies of everything the stream holds, in the reference layouts.
struct State {
    std::vector<float> Vm, Vthresh, Vreset, I0, Inoise, C1, C2, Trefract;
    std::vector<int32_t> refr;
    std::vector<float> A, B, C, D, u_izh, C3;
    std::vector<uint8_t> in_use;
    std::vector<int32_t> src, type, delayIdx, total_delay;
    std::vector<float> W, psr, decay, tau, U, Dd, F, u, r;
    std::vector<uint32_t> queue, counts;
    std::vector<uint64_t> lastSpike;
    std::vector<uint32_t> queuePost;
    std::vector<int32_t> delayIdxPost, total_delayPost;
    std::vector<float> tauspost, tauspre, taupos, tauneg, gap, Wex, Aneg, Apos, mupos, muneg;
    std::vector<uint8_t> useFD;
    std::vector<float> radii, rates;

    void size(const Nets &s)
    {
        for (auto *v : {&Vm, &Vthresh, &Vreset, &I0, &Inoise, &C1, &C2, &Trefract, &radii, &rates})
            v->assign(s.N, 0.0f);
        refr.assign(s.N, 0);
        if (s.izh)
            for (auto *v : {&A, &B, &C, &D, &u_izh, &C3}) v->assign(s.N, 0.0f);
        in_use.assign(s.S, 0);
        for (auto *v : {&src, &type, &delayIdx, &total_delay}) v->assign(s.S, 0);
        for (auto *v : {&W, &psr, &decay, &tau, &U, &Dd, &F, &u, &r}) v->assign(s.S, 0.0f);
        queue.assign(s.S, 0u);
        counts.assign(s.N, 0u);
        lastSpike.assign(s.S, 0);
        if (s.stdp) {
            queuePost.assign(s.S, 0u);
            delayIdxPost.assign(s.S, 0);
            total_delayPost.assign(s.S, 0);
            for (auto *v : {&tauspost, &tauspre, &taupos, &tauneg, &gap, &Wex, &Aneg, &Apos, &mupos,
                            &muneg})
                v->assign(s.S, 0.0f);
            useFD.assign(s.S, 0);
        }
    }
    bg3_synapse_arrays syn()
    {
        bg3_synapse_arrays a;
        a.in_use = in_use.data();
        a.src = src.data();
        a.type = type.data();
        a.delayIdx = delayIdx.data();
        a.total_delay = total_delay.data();
        a.W = W.data();
        a.psr = psr.data();
        a.decay = decay.data();
        a.tau = tau.data();
        a.delayQueue = queue.data();
        a.counts = counts.data();
        a.U = U.data();
        a.D = Dd.data();
        a.F = F.data();
        a.u = u.data();
        a.r = r.data();
        a.lastSpike = lastSpike.data();
        return a;
    }
    bg3_stdp_arrays stdp_arrays()
    {
        bg3_stdp_arrays a;
        a.delayQueuePost = queuePost.data();
        a.delayIdxPost = delayIdxPost.data();
        a.total_delayPost = total_delayPost.data();
        a.tauspost = tauspost.data();
        a.tauspre = tauspre.data();
        a.taupos = taupos.data();
        a.tauneg = tauneg.data();
        a.STDPgap = gap.data();
        a.Wex = Wex.data();
        a.Aneg = Aneg.data();
        a.Apos = Apos.data();
        a.mupos = mupos.data();
        a.muneg = muneg.data();
        a.useFroemkeDanSTDP = useFD.data();
        return a;
    }
    bg3_lif_arrays lif()
    {
        bg3_lif_arrays a;
        memset(&a, 0, sizeof(a));
        a.Vm = Vm.data();
        a.Vthresh = Vthresh.data();
        a.Vreset = Vreset.data();
        a.I0 = I0.data();
        a.Inoise = Inoise.data();
        a.C1 = C1.data();
        a.C2 = C2.data();
        a.Trefract = Trefract.data();
        a.nStepsInRefr = refr.data();
        return a;
    }
    bg3_izh_arrays izh_arrays()
    {
        bg3_izh_arrays a;
        a.Aconst = A.data();
        a.Bconst = B.data();
        a.Cconst = C.data();
        a.Dconst = D.data();
        a.u = u_izh.data();
        a.C3 = C3.data();
        return a;
    }
};

int download(bg3_net *net, const Nets &s, bool growth, State &st)
{
    st.size(s);
    int rc;
    bg3_lif_arrays la = st.lif();
    if ((rc = bg3_download_lif(net, &la))) return rc;
    if (s.izh) {
        bg3_izh_arrays ia = st.izh_arrays();
        if ((rc = bg3_download_izh(net, &ia))) return rc;
    }
    bg3_synapse_arrays sa = st.syn();
    if (!s.dyn) sa.U = sa.D = sa.F = sa.u = sa.r = nullptr, sa.lastSpike = nullptr;
    if ((rc = bg3_download_synapses(net, &sa))) return rc;
    if (s.stdp) {
        bg3_stdp_arrays ta = st.stdp_arrays();
        if ((rc = bg3_download_stdp(net, &ta))) return rc;
    }
    if (growth && (rc = bg3_download_growth(net, st.radii.data(), st.rates.data()))) return rc;
    return BG3_OK;
}

inline float at(const float *a, size_t i) { return a ? a[i] : 0.0f; }

}  // namespace

extern "C" {

int bg3_serialize(bg3_net *net, const bg3_if_fields *setup, int32_t conn, char *buf, uint64_t cap,
                  uint64_t *len)
{
    if (!net || !len || (conn != BG3_CONN_STATIC && conn != BG3_CONN_GROWTH)) return BG3_EINVAL;
    bg3_net_desc d;
    int rc;
    if ((rc = bg3_get_desc(net, &d))) return rc;
    const Nets s = shape(d);
    State st;
    if ((rc = download(net, s, conn == BG3_CONN_GROWTH, st))) return rc;
    bg3_if_fields none;
    memset(&none, 0, sizeof(none));
    const bg3_if_fields &x = setup ? *setup : none;
    Out o{buf, cap};
    o.i((long long)s.N);  // Model::serialize: totalNeurons
    for (size_t i = 0; i < s.N; i++) {
        // AllIFNeurons::writeNeuron (Neurons/AllIFNeurons.cpp:594-613)
        o.f(at(x.Cm, i)); o.f(at(x.Rm, i)); o.f(st.Vthresh[i]); o.f(at(x.Vrest, i));
        o.f(st.Vreset[i]); o.f(at(x.Vinit, i)); o.f(st.Trefract[i]); o.f(st.Inoise[i]);
        o.f(at(x.Iinject, i)); o.f(at(x.Isyn, i)); o.i(st.refr[i]); o.f(st.C1[i]); o.f(st.C2[i]);
        o.f(st.I0[i]); o.f(st.Vm[i]);
        o.i(0);  // hasFired: cleared in the step that sets it (AllSpikingNeurons.cpp:144)
        o.f(at(x.Tau, i));
        if (s.izh) {
            // AllIZHNeurons::writeNeuron (Neurons/AllIZHNeurons.cpp:551-561)
            o.f(st.A[i]); o.f(st.B[i]); o.f(st.C[i]); o.f(st.D[i]); o.f(st.u_izh[i]); o.f(st.C3[i]);
        }
    }
    // AllSynapses::serialize (Synapses/AllSynapses.cpp:163-177): dest rows in order, the first
    // synapse_counts[dest] slots of each
    long long total = 0;
    for (size_t i = 0; i < s.N; i++) total += st.counts[i];
    o.i(total);
    for (size_t dst = 0; dst < s.N; dst++)
        for (uint32_t k = 0; k < st.counts[dst]; k++) {
            const size_t j = dst * s.M + k;
            // AllSynapses::writeSynapse (:207-215)
            o.i(st.src[j]); o.i((long long)dst); o.f(st.W[j]); o.f(st.psr[j]); o.i(st.type[j]);
            o.i(st.in_use[j] ? 1 : 0);
            // AllSpikingSynapses::writeSynapse (Synapses/AllSpikingSynapses.cpp:168-178)
            o.f(st.decay[j]); o.i(st.total_delay[j]); o.u(st.queue[j]); o.i(st.delayIdx[j]);
            o.i(LENGTH_OF_DELAYQUEUE); o.f(st.tau[j]);
            if (s.stdp) {
                // AllSTDPSynapses::writeSynapse (Synapses/AllSTDPSynapses.cpp:209-228)
                o.i(st.total_delayPost[j]); o.u(st.queuePost[j]); o.i(st.delayIdxPost[j]);
                o.i(LENGTH_OF_DELAYQUEUE); o.f(st.tauspost[j]); o.f(st.tauspre[j]);
                o.f(st.taupos[j]); o.f(st.tauneg[j]); o.f(st.gap[j]); o.f(st.Wex[j]);
                o.f(st.Aneg[j]); o.f(st.Apos[j]); o.f(st.mupos[j]); o.f(st.muneg[j]);
                o.i(st.useFD[j] ? 1 : 0);
            }
            if (s.dyn) {
                // AllDSSynapses::writeSynapse (Synapses/AllDSSynapses.cpp:142-152) and
                // AllDynamicSTDPSynapses::writeSynapse (AllDynamicSTDPSynapses.cpp:142-152)
                o.u(st.lastSpike[j]); o.f(st.r[j]); o.f(st.u[j]); o.f(st.Dd[j]); o.f(st.U[j]);
                o.f(st.F[j]);
            }
        }
    if (conn == BG3_CONN_GROWTH) {
        // ConnGrowth::serialize (Connections/ConnGrowth.cpp:254-265)
        for (size_t i = 0; i < s.N; i++) o.f(st.radii[i]);
        for (size_t i = 0; i < s.N; i++) o.f(st.rates[i]);
    }
    *len = o.len;
    if (buf && o.len > cap) return BG3_EINVAL;
    return BG3_OK;
}

int bg3_deserialize(bg3_net *net, const char *buf, uint64_t len, int32_t conn, uint64_t current_step,
                    bg3_if_fields *setup_out)
{
    if (!net || !buf || (conn != BG3_CONN_STATIC && conn != BG3_CONN_GROWTH)) return BG3_EINVAL;
    bg3_net_desc d;
    int rc;
    if ((rc = bg3_get_desc(net, &d))) return rc;
    const Nets s = shape(d);
    State st;
    st.size(s);
    std::vector<float> Cm(s.N), Rm(s.N), Vrest(s.N), Vinit(s.N), Iinject(s.N), Isyn(s.N), Tau(s.N);
    In in{buf, buf + len};
    if (in.i() != (long long)s.N) return BG3_EINVAL;  // Simulator::deserialize: totalNeurons
    for (size_t i = 0; i < s.N && !in.bad; i++) {
        // AllIFNeurons::readNeuron (Neurons/AllIFNeurons.cpp:552-572)
        Cm[i] = in.f(); Rm[i] = in.f(); st.Vthresh[i] = in.f(); Vrest[i] = in.f();
        st.Vreset[i] = in.f(); Vinit[i] = in.f(); st.Trefract[i] = in.f(); st.Inoise[i] = in.f();
        Iinject[i] = in.f(); Isyn[i] = in.f(); st.refr[i] = (int32_t)in.i(); st.C1[i] = in.f();
        st.C2[i] = in.f(); st.I0[i] = in.f(); st.Vm[i] = in.f();
        if (in.i() != 0) return BG3_EUNSUPPORTED;  // hasFired: only false between steps
        Tau[i] = in.f();
        if (s.izh) {
            // AllIZHNeurons::readNeuron (Neurons/AllIZHNeurons.cpp:519-529)
            st.A[i] = in.f(); st.B[i] = in.f(); st.C[i] = in.f(); st.D[i] = in.f();
            st.u_izh[i] = in.f(); st.C3[i] = in.f();
        }
    }
    const long long total = in.i();
    if (in.bad || total < 0 || (unsigned long long)total > s.S) return BG3_EINVAL;
    for (long long q = 0; q < total && !in.bad; q++) {
        // the writer's layout (AllSynapses::writeSynapse and the subclasses' fields); the
        // synapse goes to the next slot of its dest row
        const long long sr = in.i(), dst = in.i();
        if (in.bad || sr < 0 || (size_t)sr >= s.N || dst < 0 || (size_t)dst >= s.N ||
            st.counts[dst] >= s.M)
            return BG3_EINVAL;
        const size_t j = (size_t)dst * s.M + st.counts[dst]++;
        st.src[j] = (int32_t)sr;
        st.W[j] = in.f(); st.psr[j] = in.f(); st.type[j] = (int32_t)in.i();
        if (in.i() != 1) return BG3_EINVAL;  // only in-use synapses are written
        st.in_use[j] = 1;
        st.decay[j] = in.f(); st.total_delay[j] = (int32_t)in.i(); st.queue[j] = (uint32_t)in.u();
        st.delayIdx[j] = (int32_t)in.i();
        if (in.i() != LENGTH_OF_DELAYQUEUE) return BG3_EUNSUPPORTED;
        st.tau[j] = in.f();
        if (s.stdp) {
            st.total_delayPost[j] = (int32_t)in.i(); st.queuePost[j] = (uint32_t)in.u();
            st.delayIdxPost[j] = (int32_t)in.i();
            if (in.i() != LENGTH_OF_DELAYQUEUE) return BG3_EUNSUPPORTED;
            st.tauspost[j] = in.f(); st.tauspre[j] = in.f(); st.taupos[j] = in.f();
            st.tauneg[j] = in.f(); st.gap[j] = in.f(); st.Wex[j] = in.f(); st.Aneg[j] = in.f();
            st.Apos[j] = in.f(); st.mupos[j] = in.f(); st.muneg[j] = in.f();
            st.useFD[j] = in.i() ? 1 : 0;
        }
        if (s.dyn) {
            st.lastSpike[j] = in.u(); st.r[j] = in.f(); st.u[j] = in.f(); st.Dd[j] = in.f();
            st.U[j] = in.f(); st.F[j] = in.f();
        }
    }
    if (conn == BG3_CONN_GROWTH) {
        // ConnGrowth::deserialize (Connections/ConnGrowth.cpp:235-246)
        for (size_t i = 0; i < s.N; i++) st.radii[i] = in.f();
        for (size_t i = 0; i < s.N; i++) st.rates[i] = in.f();
    }
    if (in.bad || in.p != in.end) return BG3_EINVAL;

    bg3_lif_arrays la = st.lif();
    if ((rc = bg3_upload_lif(net, &la))) return rc;
    if (s.izh) {
        bg3_izh_arrays ia = st.izh_arrays();
        if ((rc = bg3_upload_izh(net, &ia))) return rc;
    }
    bg3_synapse_arrays sa = st.syn();
    if ((rc = bg3_upload_synapses(net, &sa, current_step))) return rc;
    if (s.stdp) {
        bg3_stdp_arrays ta = st.stdp_arrays();
        if ((rc = bg3_upload_stdp(net, &sa, &ta))) return rc;
    }
    if (conn == BG3_CONN_GROWTH &&
        (rc = bg3_upload_growth(net, nullptr, st.radii.data(), st.rates.data())))
        return rc;
    // the library keeps some fields per synapse type or as classes: a stream whose values it
    // cannot hold exactly (a tau that is not its type's) is refused
    State back;
    if ((rc = download(net, s, false, back))) return rc;
    for (size_t dst = 0; dst < s.N; dst++)
        for (uint32_t k = 0; k < st.counts[dst]; k++) {
            const size_t j = dst * s.M + k;
            if (memcmp(&back.tau[j], &st.tau[j], 4) || memcmp(&back.decay[j], &st.decay[j], 4) ||
                back.queue[j] != st.queue[j] || back.delayIdx[j] != st.delayIdx[j])
                return BG3_EUNSUPPORTED;
            if (s.dyn && (memcmp(&back.U[j], &st.U[j], 4) || memcmp(&back.Dd[j], &st.Dd[j], 4) ||
                          memcmp(&back.F[j], &st.F[j], 4)))
                return BG3_EUNSUPPORTED;
        }
    if (setup_out) {
        const std::vector<float> *src[7] = {&Cm, &Rm, &Vrest, &Vinit, &Iinject, &Isyn, &Tau};
        float *dst[7] = {setup_out->Cm, setup_out->Rm, setup_out->Vrest, setup_out->Vinit,
                         setup_out->Iinject, setup_out->Isyn, setup_out->Tau};
        for (int f = 0; f < 7; f++)
            if (dst[f]) memcpy(dst[f], src[f]->data(), s.N * sizeof(float));
    }
    return BG3_OK;
}

}  // extern "C"
