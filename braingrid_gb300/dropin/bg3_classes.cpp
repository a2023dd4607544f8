// The device-side members of the reference's neuron, synapse and connection classes, as their
// USE_GPU declarations name them (Neurons/IAllNeurons.h:89-142, Neurons/AllSpikingNeurons.h:
// 76-106, Neurons/AllIFNeurons.h:120-190, Neurons/AllIZHNeurons.h:168-240, Synapses/
// IAllSynapses.h:125-221, Synapses/AllSpikingSynapses.h:163-260 and the DS, STDP and dynamic
// STDP subclasses, Connections/ConnGrowth.h:167-182), defined on the bg3 C-ABI.  They replace
// Neurons/*_d.cu, Synapses/*_d.cu and Connections/ConnGrowth_d.cu.
//
// Every `void*` device struct is the network's bg3_net handle (bg3_dropin.h).  Uploads and
// downloads move the classes' own host arrays, in the reference layout, through one call each;
// the library converts to and from its device layout.
#include <cstring>
#include <vector>

#include "AllDSSynapses.h"
#include "AllDynamicSTDPSynapses.h"
#include "AllIFNeurons.h"
#include "AllIZHNeurons.h"
#include "AllLIFNeurons.h"
#include "AllSTDPSynapses.h"
#include "AllSpikingNeurons.h"
#include "AllSpikingSynapses.h"
#include "ConnGrowth.h"
#include "Global.h"
#include "bg3_dropin.h"

namespace {

int max_spikes_of(const SimulationInfo *si)
{
    return static_cast<int>(si->epochDuration * si->maxFiringRate);  // the recorder's ring length
}

bg3_lif_arrays if_arrays(AllIFNeurons &n)
{
    bg3_lif_arrays a;
    memset(&a, 0, sizeof(a));
    a.Vm = n.Vm; a.Vthresh = n.Vthresh; a.Vreset = n.Vreset; a.I0 = n.I0; a.Inoise = n.Inoise;
    a.C1 = n.C1; a.C2 = n.C2; a.Trefract = n.Trefract; a.summation = n.summation_map;
    a.nStepsInRefr = n.nStepsInRefr; a.spikeCount = n.spikeCount;
    a.spikeCountOffset = n.spikeCountOffset;
    return a;
}

bg3_izh_arrays izh_arrays(AllIZHNeurons &z)
{
    bg3_izh_arrays a = {z.Aconst, z.Bconst, z.Cconst, z.Dconst, z.u, z.C3};
    return a;
}

void neurons_to_device(AllIFNeurons &n, void *dev, const SimulationInfo *si)
{
    bg3_net *net = bg3_dropin_net(dev, "copyNeuronHostToDevice");
    const int ms = max_spikes_of(si);
    std::vector<uint64_t> flat;
    bg3_dropin_pack_history(n.spike_history, si->totalNeurons, ms, flat);
    bg3_lif_arrays a = if_arrays(n);
    a.history = flat.data();
    bg3_dropin_check(bg3_upload_lif(net, &a), "bg3_upload_lif");
    if (AllIZHNeurons *z = dynamic_cast<AllIZHNeurons *>(&n)) {
        bg3_izh_arrays za = izh_arrays(*z);
        bg3_dropin_check(bg3_upload_izh(net, &za), "bg3_upload_izh");
    }
}

void neurons_to_host(AllIFNeurons &n, void *dev, const SimulationInfo *si)
{
    bg3_net *net = bg3_dropin_net(dev, "copyNeuronDeviceToHost");
    const int ms = max_spikes_of(si);
    std::vector<uint64_t> flat((size_t)si->totalNeurons * ms);
    bg3_lif_arrays a = if_arrays(n);
    a.history = flat.data();
    bg3_dropin_check(bg3_download_lif(net, &a), "bg3_download_lif");
    bg3_dropin_unpack_history(flat, si->totalNeurons, ms, n.spike_history);
    if (AllIZHNeurons *z = dynamic_cast<AllIZHNeurons *>(&n)) {
        bg3_izh_arrays za = izh_arrays(*z);
        bg3_dropin_check(bg3_download_izh(net, &za), "bg3_download_izh");
    }
    // the step that sets hasFired also clears it (Neurons/AllSpikingNeurons.cpp:144)
    memset(n.hasFired, 0, sizeof(bool) * si->totalNeurons);
}

void history_to_host(AllSpikingNeurons &n, void *dev, const SimulationInfo *si)
{
    bg3_net *net = bg3_dropin_net(dev, "copyNeuronDeviceSpikeHistoryToHost");
    const int ms = max_spikes_of(si);
    std::vector<uint64_t> flat((size_t)si->totalNeurons * ms);
    bg3_lif_arrays a;
    memset(&a, 0, sizeof(a));
    a.history = flat.data();
    bg3_dropin_check(bg3_download_lif(net, &a), "bg3_download_lif");
    bg3_dropin_unpack_history(flat, si->totalNeurons, ms, n.spike_history);
}

void counts_to_host(AllSpikingNeurons &n, void *dev)
{
    bg3_lif_arrays a;
    memset(&a, 0, sizeof(a));
    a.spikeCount = n.spikeCount;
    a.spikeCountOffset = n.spikeCountOffset;
    bg3_dropin_check(bg3_download_lif(bg3_dropin_net(dev, "copyNeuronDeviceSpikeCountsToHost"), &a),
                     "bg3_download_lif");
}

// The device's spike counts become 0 and its ring offsets the host's, which the recorder has
// just advanced (AllSpikingNeurons::clearSpikeCounts on the host, then this, as
// Neurons/AllSpikingNeurons_d.cu does).
void clear_counts(AllSpikingNeurons &n, void *dev, const SimulationInfo *si)
{
    std::vector<int> zero(si->totalNeurons, 0);
    bg3_lif_arrays a;
    memset(&a, 0, sizeof(a));
    a.spikeCount = zero.data();
    a.spikeCountOffset = n.spikeCountOffset;
    bg3_dropin_check(bg3_upload_lif(bg3_dropin_net(dev, "clearNeuronSpikeCounts"), &a),
                     "bg3_upload_lif");
}

void bind(void **dev, const char *what)
{
    bg3_dropin_net(dev ? *dev : NULL, what);  // the handle must already be there
}

// One fused step: neuron integration with spike detection, spike propagation, the synapse sweep
// and the summation (the reference's advanceNeurons, advanceSynapses and calcSummationMap).
void one_step(void *dev)
{
    bg3_dropin_check(bg3_step(bg3_dropin_net(dev, "advanceNeurons"), 1), "bg3_step");
}

bg3_synapse_arrays slot_arrays(AllSpikingSynapses &s)
{
    bg3_synapse_arrays a;
    memset(&a, 0, sizeof(a));
    a.in_use = reinterpret_cast<uint8_t *>(s.in_use);  // bool is one byte on every target
    a.src = s.sourceNeuronIndex;
    a.type = reinterpret_cast<int32_t *>(s.type);     // the synapseType enum is an int
    a.delayIdx = s.delayIdx;
    a.total_delay = s.total_delay;
    a.W = s.W; a.psr = s.psr; a.decay = s.decay; a.tau = s.tau;
    a.delayQueue = s.delayQueue;
    a.counts = s.synapse_counts;
    if (AllDSSynapses *d = dynamic_cast<AllDSSynapses *>(&s)) {
        a.U = d->U; a.D = d->D; a.F = d->F; a.u = d->u; a.r = d->r;
        a.lastSpike = d->lastSpike;
    } else if (AllDynamicSTDPSynapses *d = dynamic_cast<AllDynamicSTDPSynapses *>(&s)) {
        a.U = d->U; a.D = d->D; a.F = d->F; a.u = d->u; a.r = d->r;
        a.lastSpike = d->lastSpike;
    }
    return a;
}

bg3_stdp_arrays stdp_arrays(AllSTDPSynapses &p)
{
    bg3_stdp_arrays a = {p.delayQueuePost, p.delayIdxPost, p.total_delayPost, p.tauspost,
                         p.tauspre, p.taupos, p.tauneg, p.STDPgap, p.Wex, p.Aneg, p.Apos,
                         p.mupos, p.muneg, reinterpret_cast<uint8_t *>(p.useFroemkeDanSTDP)};
    return a;
}

void synapses_to_device(AllSpikingSynapses &s, void *dev)
{
    bg3_net *net = bg3_dropin_net(dev, "copySynapseHostToDevice");
    bg3_synapse_arrays a = slot_arrays(s);
    bg3_dropin_check(bg3_upload_synapses(net, &a, g_simulationStep), "bg3_upload_synapses");
    if (AllSTDPSynapses *p = dynamic_cast<AllSTDPSynapses *>(&s)) {
        bg3_stdp_arrays pa = stdp_arrays(*p);
        bg3_dropin_check(bg3_upload_stdp(net, &a, &pa), "bg3_upload_stdp");
    }
}

void total_counts(AllSpikingSynapses &s, const SimulationInfo *si)
{
    BGSIZE t = 0;
    for (int i = 0; i < si->totalNeurons; i++) t += s.synapse_counts[i];
    s.total_synapse_counts = t;
}

void synapses_to_host(AllSpikingSynapses &s, void *dev, const SimulationInfo *si)
{
    bg3_net *net = bg3_dropin_net(dev, "copySynapseDeviceToHost");
    bg3_synapse_arrays a = slot_arrays(s);
    bg3_dropin_check(bg3_download_synapses(net, &a), "bg3_download_synapses");
    if (AllSTDPSynapses *p = dynamic_cast<AllSTDPSynapses *>(&s)) {
        bg3_stdp_arrays pa = stdp_arrays(*p);
        bg3_dropin_check(bg3_download_stdp(net, &pa), "bg3_download_stdp");
    }
    // the host fields the device does not keep: a slot's dest is its row (Synapses/
    // AllSynapses.cpp:367), its summation point that dest's (AllSpikingSynapses.cpp:196)
    const BGSIZE M = s.maxSynapsesPerNeuron;
    for (int d = 0; d < si->totalNeurons; d++)
        for (BGSIZE k = 0; k < s.synapse_counts[d]; k++) {
            const BGSIZE i = (BGSIZE)d * M + k;
            s.destNeuronIndex[i] = d;
            if (si->pSummationMap) s.summationPoint[i] = &si->pSummationMap[d];
        }
    total_counts(s, si);
}

void unused_form(const char *what)
{
    fprintf(stderr, "%s: the (num_neurons, maxSynapsesPerNeuron) form copies a stand-alone "
            "synapse layer; with libbg3 an input's synapse layer lives in the network "
            "(bg3_input_poisson)\n", what);
    exit(EXIT_FAILURE);
}

}  // namespace

// ---- neurons ----------------------------------------------------------------------------------
// The device state is created once for the whole network by GPUSpikingModel::setupSim
// (bg3_create); allocation binds to that handle and deletion leaves it to the model.
void AllIFNeurons::allocNeuronDeviceStruct(void **dev, SimulationInfo *) { bind(dev, "allocNeuronDeviceStruct"); }
void AllIFNeurons::deleteNeuronDeviceStruct(void *, const SimulationInfo *) {}
void AllIFNeurons::copyNeuronHostToDevice(void *dev, const SimulationInfo *si) { neurons_to_device(*this, dev, si); }
void AllIFNeurons::copyNeuronDeviceToHost(void *dev, const SimulationInfo *si) { neurons_to_host(*this, dev, si); }
void AllIFNeurons::copyNeuronDeviceSpikeHistoryToHost(void *dev, const SimulationInfo *si) { history_to_host(*this, dev, si); }
void AllIFNeurons::copyNeuronDeviceSpikeCountsToHost(void *dev, const SimulationInfo *) { counts_to_host(*this, dev); }
void AllIFNeurons::clearNeuronSpikeCounts(void *dev, const SimulationInfo *si) { clear_counts(*this, dev, si); }
void AllIFNeurons::advanceNeurons(IAllSynapses &, void *dev, void *, const SimulationInfo *, float *, SynapseIndexMap *) { one_step(dev); }

void AllLIFNeurons::advanceNeurons(IAllSynapses &, void *dev, void *, const SimulationInfo *, float *, SynapseIndexMap *) { one_step(dev); }

void AllIZHNeurons::allocNeuronDeviceStruct(void **dev, SimulationInfo *) { bind(dev, "allocNeuronDeviceStruct"); }
void AllIZHNeurons::deleteNeuronDeviceStruct(void *, const SimulationInfo *) {}
void AllIZHNeurons::copyNeuronHostToDevice(void *dev, const SimulationInfo *si) { neurons_to_device(*this, dev, si); }
void AllIZHNeurons::copyNeuronDeviceToHost(void *dev, const SimulationInfo *si) { neurons_to_host(*this, dev, si); }
void AllIZHNeurons::copyNeuronDeviceSpikeHistoryToHost(void *dev, const SimulationInfo *si) { history_to_host(*this, dev, si); }
void AllIZHNeurons::copyNeuronDeviceSpikeCountsToHost(void *dev, const SimulationInfo *) { counts_to_host(*this, dev); }
void AllIZHNeurons::clearNeuronSpikeCounts(void *dev, const SimulationInfo *si) { clear_counts(*this, dev, si); }
void AllIZHNeurons::advanceNeurons(IAllSynapses &, void *dev, void *, const SimulationInfo *, float *, SynapseIndexMap *) { one_step(dev); }

// Whether spikes propagate back to the synapses (STDP): the synapse class says so
// (AllSpikingSynapses::allowBackPropagation).  The library reads it from the synapse kind.
void AllSpikingNeurons::setAdvanceNeuronsDeviceParams(IAllSynapses &synapses)
{
    m_fAllowBackPropagation = dynamic_cast<AllSpikingSynapses &>(synapses).allowBackPropagation();
}

// ---- synapses ---------------------------------------------------------------------------------
// One set of definitions serves every synapse class: the copies look at the object's dynamic
// class for its DS and STDP fields.  advanceSynapses does no separate work: the synapse sweep and
// the summation run inside the fused step that advanceNeurons launched.  The synapse class is
// part of the network's shape (bg3_net_desc.synapse_kind), so setSynapseClassID has nothing to set.
#define BG3_SYNAPSE_MEMBERS(C)                                                                     \
    void C::allocSynapseDeviceStruct(void **dev, const SimulationInfo *) { bind(dev, "allocSynapseDeviceStruct"); } \
    void C::allocSynapseDeviceStruct(void **, int, int) { unused_form(#C "::allocSynapseDeviceStruct"); } \
    void C::deleteSynapseDeviceStruct(void *) {}                                                   \
    void C::copySynapseHostToDevice(void *dev, const SimulationInfo *) { synapses_to_device(*this, dev); } \
    void C::copySynapseHostToDevice(void *, int, int) { unused_form(#C "::copySynapseHostToDevice"); } \
    void C::copySynapseDeviceToHost(void *dev, const SimulationInfo *si) { synapses_to_host(*this, dev, si); } \
    void C::setSynapseClassID() {}

BG3_SYNAPSE_MEMBERS(AllSpikingSynapses)
BG3_SYNAPSE_MEMBERS(AllDSSynapses)
BG3_SYNAPSE_MEMBERS(AllSTDPSynapses)
BG3_SYNAPSE_MEMBERS(AllDynamicSTDPSynapses)
#undef BG3_SYNAPSE_MEMBERS

void AllSpikingSynapses::copyDeviceSynapseCountsToHost(void *dev, const SimulationInfo *si)
{
    bg3_synapse_arrays a;
    memset(&a, 0, sizeof(a));
    a.counts = synapse_counts;
    bg3_dropin_check(bg3_download_synapses(bg3_dropin_net(dev, "copyDeviceSynapseCountsToHost"), &a),
                     "bg3_download_synapses");
    total_counts(*this, si);
}

void AllSpikingSynapses::copyDeviceSynapseSumIdxToHost(void *dev, const SimulationInfo *)
{
    bg3_synapse_arrays a;
    memset(&a, 0, sizeof(a));
    a.src = sourceNeuronIndex;
    a.in_use = reinterpret_cast<uint8_t *>(in_use);
    bg3_dropin_check(bg3_download_synapses(bg3_dropin_net(dev, "copyDeviceSynapseSumIdxToHost"), &a),
                     "bg3_download_synapses");
}

void AllSpikingSynapses::advanceSynapses(void *, void *, void *, const SimulationInfo *) {}
void AllSTDPSynapses::advanceSynapses(void *, void *, void *, const SimulationInfo *) {}
void AllSpikingSynapses::setAdvanceSynapsesDeviceParams() { setSynapseClassID(); }

// ---- connections ------------------------------------------------------------------------------
// The epoch's growth pass on the device, as one call: firing rates and radii (the work of
// ConnGrowth::updateConns), frontiers and overlap areas (updateFrontiers, updateOverlap), weights
// of existing synapses and the synapses new overlaps create (this member in the reference,
// Connections/ConnGrowth_d.cu:18-61), the index maps, and the growth recorder's device
// histories.  The new radii and rates come back into this object (the recorder reads them);
// the host's distance, area and weight matrices are neither read nor written.
void ConnGrowth::updateSynapsesWeights(const int num_neurons, IAllNeurons &, IAllSynapses &,
                                       const SimulationInfo *si, AllSpikingNeuronsDeviceProperties *dev,
                                       AllSpikingSynapsesDeviceProperties *, Layout *)
{
    bg3_net *net = bg3_dropin_net(dev, "ConnGrowth::updateSynapsesWeights");
    bg3_dropin_check(bg3_epoch_growth(net, si->currentStep), "bg3_epoch_growth");
    std::vector<float> r(num_neurons), q(num_neurons);
    bg3_dropin_check(bg3_download_growth(net, r.data(), q.data()), "bg3_download_growth");
    for (int i = 0; i < num_neurons; i++) {
        (*radii)[i] = r[i];
        (*rates)[i] = q[i];
    }
}
