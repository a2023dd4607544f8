// The reference's GPU stimulus classes (Inputs/GpuSInputRegular.h, Inputs/GpuSInputPoisson.h,
// created by Inputs/FSInput.cpp:86-100 under USE_GPU) on libbg3; they replace
// Inputs/GpuSInputRegular.cu and Inputs/GpuSInputPoisson.cu.
//
// The library applies an external input inside the neuron pass of every step, so init hands the
// input's host arrays to the network once and inputStimulus, which the Simulator calls before
// every step (Core/Simulator.cpp:178-182), has nothing left to do; the cycle position of a regular
// input and the interval counters of a Poisson input advance on the device.
#include <cstring>

#include "AllDSSynapses.h"
#include "GPUSpikingModel.h"
#include "GpuSInputPoisson.h"
#include "GpuSInputRegular.h"
#include "Layout.h"
#include "bg3_dropin.h"

namespace {

// The network of the run's model (GPUSpikingModel::setupSim runs before the input's init,
// Core/Simulator.cpp:36-45).
bg3_net *model_net(SimulationInfo *psi, const char *what)
{
    return bg3_dropin_net(bg3_dropin_model_network(psi->model), what);
}

}  // namespace

// ---- regular pulses ----------------------------------------------------------------------------
GpuSInputRegular::GpuSInputRegular(SimulationInfo *psi, TiXmlElement *parms) : SInputRegular(psi, parms) {}

GpuSInputRegular::~GpuSInputRegular() {}

// The per-neuron values and phase shifts the constructor read (Inputs/SInputRegular.cpp:20-112)
// and the cycle position now; the network adds values[i] to neuron i's summation point while its
// shifted pulse window is open, as the reference's inputStimulusDevice does.
void GpuSInputRegular::init(SimulationInfo *psi)
{
    SInputRegular::init(psi);
    if (!fSInput) return;
    bg3_dropin_check(bg3_input_regular(model_net(psi, "GpuSInputRegular::init"), values,
                                       nShiftValues, nStepsDuration, nStepsCycle, nStepsInCycle),
                     "bg3_input_regular");
}

void GpuSInputRegular::term(SimulationInfo *psi) { SInputRegular::term(psi); }

void GpuSInputRegular::inputStimulus(SimulationInfo *) {}

// ---- Poisson drive -----------------------------------------------------------------------------
GpuSInputPoisson::GpuSInputPoisson(SimulationInfo *psi, TiXmlElement *parms) : SInputPoisson(psi, parms) {}

GpuSInputPoisson::~GpuSInputPoisson() {}

// The input synapse layer of SInputPoisson::init (Inputs/SInputPoisson.cpp:124-146): one DS
// synapse per neuron, EI onto inhibitory and EE onto excitatory neurons, source 0, weight
// `weight` nA.  The reference places neuron i's synapse at slot maxSynapsesPerNeuron * i of a
// one-slot-per-neuron object, outside it whenever maxSynapsesPerNeuron > 1; here it is slot i.
// The network then draws each neuron's intervals with its own generator keyed by the run's seed
// (the reference's GPU input seeds curand with the wall clock, Inputs/GpuSInputPoisson.cu:54).
void GpuSInputPoisson::init(SimulationInfo *psi)
{
    if (!fSInput) return;
    const int N = psi->totalNeurons;
    AllDSSynapses *layer = new AllDSSynapses(N, 1);
    m_synapses = layer;
    Layout *layout = psi->model->getLayout();
    for (int i = 0; i < N; i++) {
        const synapseType type = layout->neuron_type_map[i] == INH ? EI : EE;
        layer->createSynapse(i, 0, i, &psi->pSummationMap[i], psi->deltaT, type);
        layer->W[i] = weight * AllSynapses::SYNAPSE_STRENGTH_ADJUSTMENT;
    }
    bg3_poisson_arrays a;
    memset(&a, 0, sizeof(a));
    a.masks = reinterpret_cast<uint8_t *>(masks);
    a.nISIs = nISIs;
    a.total_delay = layer->total_delay;
    a.delayIdx = layer->delayIdx;
    a.delayQueue = layer->delayQueue;
    a.W = layer->W;
    a.psr = layer->psr;
    a.decay = layer->decay;
    a.U = layer->U; a.D = layer->D; a.F = layer->F; a.u = layer->u; a.r = layer->r;
    a.lastSpike = layer->lastSpike;
    bg3_dropin_check(bg3_input_poisson(model_net(psi, "GpuSInputPoisson::init"), &a, lambda,
                                       (uint32_t)psi->seed, g_simulationStep),
                     "bg3_input_poisson");
}

void GpuSInputPoisson::term(SimulationInfo *psi)
{
    if (fSInput) SInputPoisson::term(psi);
}

void GpuSInputPoisson::inputStimulus(SimulationInfo *) {}
