// GPUSpikingModel on libbg3: the drop-in for the reference's Core/GPUSpikingModel.cu.
//
// Compiled by g++ with -DUSE_GPU against the reference's own headers, unchanged.  Its class
// declaration is the reference's Core/GPUSpikingModel.h (which includes the CUDA sample header
// Book.h only under __CUDACC__, never defined here), so BGDriver (Core/BGDriver.cpp:204-208),
// Simulator and the XML parameter files drive this model exactly as they drive the reference's.
// Nothing of the reference's CUDA code is compiled or linked: the GPU work goes through the C-ABI
// of include/bg3.h.
//
// What the model does on each interface call (Core/IModel.h:64-151):
//   setupSim           host setup as the reference (Model::setupSim), then one bg3_net for the
//                      whole network, filled from the host objects through the classes' own
//                      copy*HostToDevice members (bg3_classes.cpp); an STDP class's constants
//                      come from the parameter file's <BG3Params><STDPParams> where it has one
//                      (read_bg3_params), and <BG3Params><ParameterDraw>r_squared</ParameterDraw>
//                      gives Izhikevich neurons Izhikevich's r^2 spread (redraw_izh_r_squared);
//   advance            queues the step; queued steps run as one bg3_step call (CUDA-graph replays
//                      inside the library) when BG3_STEPS_PER_CALL steps have queued, or when the
//                      state is next observed (epoch end, checkpoint, cleanup);
//   updateConnections  the spike counts and histories the recorder reads come back to the host,
//                      then the epoch's growth pass runs on the device (ConnGrowth) and its radii
//                      and rates come back; a static network only rolls its device counters;
//   updateHistory      the reference recorder (Model::updateHistory) on those host copies, then
//                      the device spike counts are cleared as the reference's model does;
//   deserialize        Model::deserialize into the host objects, then a fresh upload;
//   cleanupSim         the whole device state back into the host objects, then the network is
//                      freed (Core/GPUSpikingModel.cu:82-99).
//
// Noise.  By default the model feeds the reference's own noise stream: Norm(0, 1, seed), the
// generator the reference's single-threaded model creates (Core/SingleThreadedSpikingModel.cpp:
// 30), drawn by the library's restatement of it (bg3_norm_*, the same values: MT19937 and the
// polar method in float, with large fills spread over host threads), and the library consumes it
// in the reference's CPU order, so a run matches the single-threaded reference spike for spike.
// The values are drawn ahead on the host while the GPU runs the previous steps.  With
// BG3_NOISE=device the library's own generator (keyed by seed, step and neuron, one draw per
// neuron per step like the reference GPU model's) is used instead and the host draws nothing.
//
// Checkpoints.  The reference's Model::serialize writes the host objects; when the run writes a
// checkpoint (a memOutputFileName is set), the last epoch's updateHistory copies the whole device
// state back into them first, so the stream holds the final state.
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "AllDSSynapses.h"
#include "AllDynamicSTDPSynapses.h"
#include "AllIFNeurons.h"
#include "AllIZHNeurons.h"
#include "AllSTDPSynapses.h"
#include "ConnGrowth.h"
#include "GPUSpikingModel.h"
#include "Global.h"
#include "bg3_dropin.h"
#include "tinyxml.h"

namespace {

// What this model keeps beside the reference's class layout (whose members are the reference's
// device pointers): the network, the queued steps and the noise drawn ahead.
// Values of <BG3Params><STDPParams> by name (absent names keep createSynapse's values).
typedef std::map<std::string, double> StdpParams;

struct ModelState {
    bg3_net *net;
    bg3_norm *gen;                        // the reference's noise stream (reference noise only)
    StdpParams stdp;                      // the parameter file's STDP constants
    bool reference_noise;
    int64_t chunk;                        // steps per bg3_step call
    int64_t queued;                       // steps advance() queued and not yet launched
    std::vector<float> drawn;             // noise values drawn ahead, not yet pushed
    int64_t held_at_launch;               // values the device held when the last steps launched
    ModelState() : net(NULL), gen(NULL), reference_noise(true), chunk(1000), queued(0),
                   held_at_launch(0) {}
};

std::map<const GPUSpikingModel *, ModelState> g_state;

ModelState &state_of(const GPUSpikingModel *m) { return g_state[m]; }

int32_t neuron_kind(IAllNeurons *n)
{
    if (dynamic_cast<AllIZHNeurons *>(n)) return BG3_NEURON_IZH;
    if (dynamic_cast<AllIFNeurons *>(n)) return BG3_NEURON_LIF;
    fprintf(stderr, "GPUSpikingModel: neuron class not supported by libbg3\n");
    exit(EXIT_FAILURE);
}

int32_t synapse_kind(IAllSynapses *s)
{
    if (dynamic_cast<AllDynamicSTDPSynapses *>(s)) return BG3_SYN_DYNSTDP;
    if (dynamic_cast<AllSTDPSynapses *>(s)) return BG3_SYN_STDP;
    if (dynamic_cast<AllDSSynapses *>(s)) return BG3_SYN_DS;
    if (dynamic_cast<AllSpikingSynapses *>(s)) return BG3_SYN_SPIKING;
    fprintf(stderr, "GPUSpikingModel: synapse class not supported by libbg3\n");
    exit(EXIT_FAILURE);
}

// A fresh object of the network's synapse class, for reading what its createSynapse gives each
// synapse type.
AllSpikingSynapses *scratch_synapses(int32_t kind)
{
    switch (kind) {
    case BG3_SYN_DYNSTDP: return new AllDynamicSTDPSynapses(1, 4);
    case BG3_SYN_STDP: return new AllSTDPSynapses(1, 4);
    case BG3_SYN_DS: return new AllDSSynapses(1, 4);
    default: return new AllSpikingSynapses(1, 4);
    }
}

// <BG3Params>, a child of the parameter file's root element: the reference's readers take their
// elements by name (<SimInfoParams>, Core/SimulationInfo.cpp:24; <ModelParams>,
// Core/FClassOfCategory.cpp:249) and never visit it.  <BG3Params><STDPParams> holds any of the
// names below: the constants of every synapse of an STDP class, in place of the ones
// AllSTDPSynapses::createSynapse writes (Synapses/AllSTDPSynapses.cpp:252-273); Wex is WexInh for
// synapses from inhibitory neurons (II, IE) and WexExc otherwise, as braingrid_gb300.config
// reads the same element.  <BG3Params><ParameterDraw> is "ranges" (the reference's flat ranges)
// or "r_squared" (redraw_izh_r_squared below).
const char *const STDP_NAMES[] = {"Apos", "Aneg", "STDPgap", "tauspost", "tauspre", "taupos",
                                  "tauneg", "WexExc", "WexInh", "mupos", "muneg",
                                  "useFroemkeDanSTDP"};

void refuse(const std::string &file, const std::string &what)
{
    fprintf(stderr, "%s: <BG3Params>: %s\n", file.c_str(), what.c_str());
    exit(EXIT_FAILURE);
}

StdpParams read_bg3_params(const std::string &file, bool &r_squared)
{
    StdpParams out;
    r_squared = false;
    TiXmlDocument doc(file.c_str());
    if (!doc.LoadFile()) return out;  // the reference's reader has already reported it
    TiXmlElement *root = doc.FirstChildElement();
    TiXmlElement *bp = root ? root->FirstChildElement("BG3Params") : NULL;
    if (!bp) return out;
    for (TiXmlElement *e = bp->FirstChildElement(); e; e = e->NextSiblingElement()) {
        if (e->ValueStr() == "ParameterDraw") {
            const std::string how = e->GetText() ? e->GetText() : "";
            if (how != "ranges" && how != "r_squared")
                refuse(file, "<ParameterDraw> must be ranges or r_squared");
            r_squared = how == "r_squared";
            continue;
        }
        if (e->ValueStr() != "STDPParams")
            refuse(file, "<" + e->ValueStr() + "> is not applied by this driver");
        for (TiXmlElement *f = e->FirstChildElement(); f; f = f->NextSiblingElement()) {
            const std::string name = f->ValueStr();
            bool known = false;
            for (size_t k = 0; k < sizeof(STDP_NAMES) / sizeof(STDP_NAMES[0]); k++)
                known = known || name == STDP_NAMES[k];
            const char *text = f->GetText();
            if (!known || !text) refuse(file, "unknown or empty <STDPParams> element <" + name + ">");
            out[name] = atof(text);
        }
    }
    return out;
}

// The file's value for name, else dflt; as a float, the way the reference reads parameters.
float stdp_value(const StdpParams &p, const char *name, float dflt)
{
    StdpParams::const_iterator it = p.find(name);
    return it == p.end() ? dflt : (float)it->second;
}

// Writes the file's STDP constants into the host synapses the reference's setup made (before
// they are uploaded).
void apply_stdp_to_host(IAllSynapses *syn, const StdpParams &p)
{
    AllSTDPSynapses *s = dynamic_cast<AllSTDPSynapses *>(syn);
    if (!s || p.empty()) return;
    const BGSIZE total = (BGSIZE)s->count_neurons * s->maxSynapsesPerNeuron;
    for (BGSIZE i = 0; i < total; i++) {
        if (!s->in_use[i]) continue;
        const bool inh_src = s->type[i] == II || s->type[i] == IE;
        s->Apos[i] = stdp_value(p, "Apos", s->Apos[i]);
        s->Aneg[i] = stdp_value(p, "Aneg", s->Aneg[i]);
        s->STDPgap[i] = stdp_value(p, "STDPgap", s->STDPgap[i]);
        s->tauspost[i] = stdp_value(p, "tauspost", s->tauspost[i]);
        s->tauspre[i] = stdp_value(p, "tauspre", s->tauspre[i]);
        s->taupos[i] = stdp_value(p, "taupos", s->taupos[i]);
        s->tauneg[i] = stdp_value(p, "tauneg", s->tauneg[i]);
        s->Wex[i] = stdp_value(p, inh_src ? "WexInh" : "WexExc", s->Wex[i]);
        s->mupos[i] = stdp_value(p, "mupos", s->mupos[i]);
        s->muneg[i] = stdp_value(p, "muneg", s->muneg[i]);
        s->useFroemkeDanSTDP[i] = stdp_value(p, "useFroemkeDanSTDP", s->useFroemkeDanSTDP[i] ? 1.0f : 0.0f) != 0.0f;
    }
}

// <ParameterDraw>r_squared</ParameterDraw>: Izhikevich's (2003) heterogeneous parameters.  The
// reference's AllIZHNeurons::createNeuron (Neurons/AllIZHNeurons.cpp:412-432) draws a, b, c, d
// from flat ranges, four inRange draws after the six of AllIFNeurons::createNeuron and, for a
// starter neuron, its two more (Neurons/AllIFNeurons.cpp:401-439).  This draw keeps those draws
// (so the generator's stream, and everything drawn after the neurons, is unchanged) and takes
// the first of the four as r = inRange(0, 1): excitatory a = 0.02, b = 0.2, c = -65 + 15 r r,
// d = 8 - 6 r r; inhibitory a = 0.02 + 0.08 r, b = 0.25 - 0.05 r, c = -65, d = 2, in float, left
// to right.  r is replayed here from a copy of the generator taken before the neurons drew, in
// their order, and the host neurons take the four values before they are uploaded.  Returns the
// FNV-1a hash of the four arrays' bytes (a, then b, c, d), which the log line reports.
//
// A copy of the generator that draws on its own: MTRand's implicit copy keeps the original's
// read pointer into the original's state, so the copy points it into its own state, where
// MTRand keeps it (pNext = state + N - left, RNG/MersenneTwister.cpp:93-99,278-290).  (MTRand's
// save and load are declared inline and defined only inside the RNG's own file.)
struct GeneratorCopy : MTRand {
    explicit GeneratorCopy(const MTRand &from) : MTRand(from) { pNext = state + (N - left); }
};

uint64_t redraw_izh_r_squared(AllIZHNeurons *n, const Layout *layout, const MTRand &saved, int count)
{
    GeneratorCopy g(saved);
    for (int i = 0; i < count; i++) {
        for (int k = 0; k < (layout->starter_map[i] ? 8 : 6); k++) g();
        const BGFLOAT r = g.inRange(0, 1);
        for (int k = 0; k < 3; k++) g();
        if (layout->neuron_type_map[i] == EXC) {
            n->Aconst[i] = 0.02f;
            n->Bconst[i] = 0.2f;
            n->Cconst[i] = -65.0f + 15.0f * r * r;
            n->Dconst[i] = 8.0f - 6.0f * r * r;
        } else {
            n->Aconst[i] = 0.02f + 0.08f * r;
            n->Bconst[i] = 0.25f - 0.05f * r;
            n->Cconst[i] = -65.0f;
            n->Dconst[i] = 2.0f;
        }
    }
    uint64_t h = 1469598103934665603ull;
    const BGFLOAT *arrays[4] = {n->Aconst, n->Bconst, n->Cconst, n->Dconst};
    for (int a = 0; a < 4; a++) {
        const unsigned char *b = reinterpret_cast<const unsigned char *>(arrays[a]);
        for (size_t k = 0; k < (size_t)count * sizeof(BGFLOAT); k++) h = (h ^ b[k]) * 1099511628211ull;
    }
    return h;
}

// The per-type constants of synapses the device growth pass creates, taken from the reference's
// own createSynapse (one synapse of each type II, IE, EI, EE on a scratch object), so that they
// are the reference's values for this deltaT by construction; the STDP ones then take the
// parameter file's <BG3Params> values (fp), like the synapses the host setup made.
void set_type_constants(bg3_net *net, int32_t kind, const SimulationInfo *si, const StdpParams &fp)
{
    AllSpikingSynapses *s = scratch_synapses(kind);
    BGFLOAT sp = 0;
    for (int t = 0; t < 4; t++) s->createSynapse(t, 0, 0, &sp, si->deltaT, (synapseType)t);
    bg3_type_constants c;
    memset(&c, 0, sizeof(c));
    for (int t = 0; t < 4; t++) {
        c.tau[t] = s->tau[t];
        c.decay[t] = s->decay[t];
        c.total_delay[t] = s->total_delay[t];
    }
    const BGFLOAT *U = NULL, *D = NULL, *F = NULL, *u = NULL, *r = NULL;
    if (AllDSSynapses *d = dynamic_cast<AllDSSynapses *>(s)) {
        U = d->U; D = d->D; F = d->F; u = d->u; r = d->r;
    } else if (AllDynamicSTDPSynapses *d = dynamic_cast<AllDynamicSTDPSynapses *>(s)) {
        U = d->U; D = d->D; F = d->F; u = d->u; r = d->r;
    }
    if (U) {
        for (int t = 0; t < 4; t++) {
            c.U[t] = U[t];
            c.D[t] = D[t];
            c.F[t] = F[t];
        }
        c.u0 = u[0];
        c.r0 = r[0];
    }
    bg3_dropin_check(bg3_set_type_constants(net, &c), "bg3_set_type_constants");
    if (AllSTDPSynapses *p = dynamic_cast<AllSTDPSynapses *>(s)) {
        bg3_stdp_constants k;
        memset(&k, 0, sizeof(k));
        for (int t = 0; t < 4; t++) {
            k.Apos[t] = p->Apos[t]; k.Aneg[t] = p->Aneg[t]; k.STDPgap[t] = p->STDPgap[t];
            k.tauspost[t] = p->tauspost[t]; k.tauspre[t] = p->tauspre[t];
            k.taupos[t] = p->taupos[t]; k.tauneg[t] = p->tauneg[t]; k.Wex[t] = p->Wex[t];
            k.mupos[t] = p->mupos[t]; k.muneg[t] = p->muneg[t];
            k.useFroemkeDanSTDP[t] = p->useFroemkeDanSTDP[t] ? 1 : 0;
        }
        if (!fp.empty()) {  // the parameter file's constants (apply_stdp_to_host, per type)
            for (int t = 0; t < 4; t++) {
                k.Apos[t] = stdp_value(fp, "Apos", k.Apos[t]);
                k.Aneg[t] = stdp_value(fp, "Aneg", k.Aneg[t]);
                k.STDPgap[t] = stdp_value(fp, "STDPgap", k.STDPgap[t]);
                k.tauspost[t] = stdp_value(fp, "tauspost", k.tauspost[t]);
                k.tauspre[t] = stdp_value(fp, "tauspre", k.tauspre[t]);
                k.taupos[t] = stdp_value(fp, "taupos", k.taupos[t]);
                k.tauneg[t] = stdp_value(fp, "tauneg", k.tauneg[t]);
                k.Wex[t] = stdp_value(fp, (t == II || t == IE) ? "WexInh" : "WexExc", k.Wex[t]);
                k.mupos[t] = stdp_value(fp, "mupos", k.mupos[t]);
                k.muneg[t] = stdp_value(fp, "muneg", k.muneg[t]);
                k.useFroemkeDanSTDP[t] = stdp_value(fp, "useFroemkeDanSTDP", (float)k.useFroemkeDanSTDP[t]) != 0.0f;
            }
        }
        bg3_dropin_check(bg3_set_stdp_constants(net, &k), "bg3_set_stdp_constants");
    }
    delete s;
}

int64_t env_int(const char *name, int64_t dflt)
{
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    char *end = NULL;
    const long long x = strtoll(v, &end, 10);
    return (end && !*end && x > 0) ? (int64_t)x : dflt;
}

void draw(bg3_norm *gen, std::vector<float> &out, int64_t n)
{
    const size_t old = out.size();
    out.resize(old + (size_t)n);
    bg3_dropin_check(bg3_norm_fill(gen, &out[old], n), "bg3_norm_fill");
}

}  // namespace

bg3_net *bg3_dropin_model_network(IModel *model)
{
    GPUSpikingModel *m = dynamic_cast<GPUSpikingModel *>(model);
    if (!m) return NULL;
    std::map<const GPUSpikingModel *, ModelState>::iterator it = g_state.find(m);
    return it == g_state.end() ? NULL : it->second.net;
}

GPUSpikingModel::GPUSpikingModel(Connections *conns, IAllNeurons *neurons, IAllSynapses *synapses,
                                 Layout *layout)
    : Model(conns, neurons, synapses, layout), randNoise_d(NULL), synapseIndexMapDevice(NULL),
      m_allSynapsesDevice(NULL), m_allNeuronsDevice(NULL)
{
}

GPUSpikingModel::~GPUSpikingModel()
{
    std::map<const GPUSpikingModel *, ModelState>::iterator it = g_state.find(this);
    if (it != g_state.end()) {
        if (it->second.net) bg3_destroy(it->second.net);
        if (it->second.gen) bg3_norm_destroy(it->second.gen);
        g_state.erase(it);
    }
}

// The network's device state: one bg3_net for neurons, synapses, maps and growth state, which
// both device-struct pointers stand for (Core/GPUSpikingModel.cu:28-47 allocates the two SoA
// structs and the noise array instead).  The host arrays go over through the classes' own copy
// members; the index maps are rebuilt on the device from the synapse slots.
void GPUSpikingModel::allocDeviceStruct(void **allNeuronsDevice, void **allSynapsesDevice,
                                        SimulationInfo *sim_info)
{
    ModelState &st = state_of(this);
    bg3_net_desc d;
    memset(&d, 0, sizeof(d));
    d.n_neurons = sim_info->totalNeurons;
    d.max_syn_per_neuron = sim_info->maxSynapsesPerNeuron;
    d.width = sim_info->width;
    d.height = sim_info->height;
    d.epoch_duration = sim_info->epochDuration;
    d.delta_t = sim_info->deltaT;
    d.max_firing_rate = sim_info->maxFiringRate;
    d.max_epochs = sim_info->maxSteps;
    d.neuron_kind = neuron_kind(m_neurons);
    d.synapse_kind = synapse_kind(m_synapses);
    d.noise_mode = st.reference_noise ? BG3_NOISE_INJECT : BG3_NOISE_DEVICE;
    d.noise_seed = (uint32_t)sim_info->seed;
    bg3_dropin_check(bg3_create(&d, &st.net), "bg3_create");
    *allNeuronsDevice = st.net;
    *allSynapsesDevice = st.net;
    m_neurons->allocNeuronDeviceStruct(allNeuronsDevice, sim_info);
    m_synapses->allocSynapseDeviceStruct(allSynapsesDevice, sim_info);

    std::vector<int32_t> types(sim_info->totalNeurons);
    for (int i = 0; i < sim_info->totalNeurons; i++) types[i] = m_layout->neuron_type_map[i];
    bg3_dropin_check(bg3_upload_layout(st.net, &(*m_layout->xloc)[0], &(*m_layout->yloc)[0],
                                       types.data()),
                     "bg3_upload_layout");
    set_type_constants(st.net, d.synapse_kind, sim_info, st.stdp);
    m_neurons->copyNeuronHostToDevice(*allNeuronsDevice, sim_info);
    m_synapses->copySynapseHostToDevice(*allSynapsesDevice, sim_info);
    if (ConnGrowth *g = dynamic_cast<ConnGrowth *>(m_conns)) {
        bg3_growth_params gp;
        gp.epsilon = g->m_growth.epsilon;
        gp.beta = g->m_growth.beta;
        gp.rho = g->m_growth.rho;
        gp.target_rate = g->m_growth.targetRate;
        gp.min_radius = g->m_growth.minRadius;
        gp.start_radius = g->m_growth.startRadius;
        gp.max_rate = g->m_growth.maxRate;
        bg3_dropin_check(bg3_upload_growth(st.net, &gp, &(*g->radii)[0], &(*g->rates)[0]),
                         "bg3_upload_growth");
    }
}

// Copies the device state back into the host objects and frees the network
// (Core/GPUSpikingModel.cu:56-74).
void GPUSpikingModel::deleteDeviceStruct(void **allNeuronsDevice, void **allSynapsesDevice,
                                         SimulationInfo *sim_info)
{
    ModelState &st = state_of(this);
    m_neurons->copyNeuronDeviceToHost(*allNeuronsDevice, sim_info);
    m_neurons->deleteNeuronDeviceStruct(*allNeuronsDevice, sim_info);
    m_synapses->copySynapseDeviceToHost(*allSynapsesDevice, sim_info);
    m_synapses->deleteSynapseDeviceStruct(*allSynapsesDevice);
    bg3_dropin_check(bg3_destroy(st.net), "bg3_destroy");
    st.net = NULL;
    *allNeuronsDevice = NULL;
    *allSynapsesDevice = NULL;
}

void GPUSpikingModel::setupSim(SimulationInfo *sim_info)
{
    ModelState &st = state_of(this);
    const std::string &file = sim_info->stateInputFileName;
    bool r_squared = false;
    st.stdp = read_bg3_params(file, r_squared);
    if (!st.stdp.empty()) {
        if (!dynamic_cast<AllSTDPSynapses *>(m_synapses))
            refuse(file, "STDPParams given for a synapse class without STDP");
        fprintf(stderr, "BG3Params: %d STDP constants from %s\n", (int)st.stdp.size(), file.c_str());
    }
    AllIZHNeurons *izh = dynamic_cast<AllIZHNeurons *>(m_neurons);
    if (r_squared && !izh) refuse(file, "ParameterDraw given for a neuron class other than AllIZHNeurons");
    // The host setup comes first and the device is selected after it (the reference selects it
    // first; nothing in the host setup touches the device).
    if (r_squared) {
        // Model::setupSim's steps (Core/Model.cpp:136-158, with Model::createAllNeurons,
        // Core/Model.cpp:117-129), with the generator's state saved before the neurons draw
        m_neurons->setupNeurons(sim_info);
        m_synapses->setupSynapses(sim_info);
        m_layout->setupLayout(sim_info);
        if (sim_info->simRecorder != NULL) sim_info->simRecorder->initDefaultValues();
        m_layout->generateNeuronTypeMap(sim_info->totalNeurons);
        m_layout->initStarterMap(sim_info->totalNeurons);
        const GeneratorCopy saved(rng);
        m_neurons->createAllNeurons(sim_info, m_layout);
        m_conns->setupConnections(sim_info, m_layout, m_neurons, m_synapses);
        m_synapses->createSynapseImap(m_synapseIndexMap, sim_info);
        const uint64_t h = redraw_izh_r_squared(izh, m_layout, saved, sim_info->totalNeurons);
        fprintf(stderr, "BG3Params: Izhikevich r^2 draw for %d neurons (a, b, c, d FNV-1a %016llx)\n",
                sim_info->totalNeurons, (unsigned long long)h);
    } else {
        Model::setupSim(sim_info);
    }
    apply_stdp_to_host(m_synapses, st.stdp);
    bg3_dropin_check(bg3_set_device(g_deviceId), "bg3_set_device");
    const char *noise = getenv("BG3_NOISE");
    st.reference_noise = !(noise && std::string(noise) == "device");
    st.chunk = env_int("BG3_STEPS_PER_CALL", 1000);
    st.queued = 0;
    st.drawn.clear();
    st.held_at_launch = 0;
    if (st.gen) bg3_norm_destroy(st.gen);
    st.gen = NULL;
    if (st.reference_noise)
        bg3_dropin_check(bg3_norm_create((uint32_t)sim_info->seed, 0.0f, 1.0f, &st.gen),
                         "bg3_norm_create");
    allocDeviceStruct((void **)&m_allNeuronsDevice, (void **)&m_allSynapsesDevice, sim_info);
    m_neurons->setAdvanceNeuronsDeviceParams(*m_synapses);
    m_synapses->setAdvanceSynapsesDeviceParams();
}

// Runs the steps advance() queued.  With the reference's noise the device must hold one value
// per neuron per queued step (each step consumes at most that); the values drawn ahead go over
// first, any shortfall is drawn now, and after the launch the next call's values are drawn while
// the GPU runs: enough to hold two calls' worth, so the device never runs short and never piles
// up more than that.
static void run_queued(ModelState &st, const SimulationInfo *si)
{
    if (!st.queued) return;
    const int64_t N = si->totalNeurons;
    if (st.reference_noise) {
        if (!st.drawn.empty())
            bg3_dropin_check(bg3_push_noise(st.net, st.drawn.data(), (int64_t)st.drawn.size()),
                             "bg3_push_noise");
        st.drawn.clear();
        int64_t held = 0;
        bg3_dropin_check(bg3_noise_pending(st.net, &held), "bg3_noise_pending");
        if (held < N * st.queued) {
            draw(st.gen, st.drawn, N * st.queued - held);
            bg3_dropin_check(bg3_push_noise(st.net, st.drawn.data(), (int64_t)st.drawn.size()),
                             "bg3_push_noise");
            st.drawn.clear();
            held = N * st.queued;
        }
        st.held_at_launch = held;
    }
    bg3_dropin_check(bg3_step(st.net, st.queued), "bg3_step");
    if (st.reference_noise) {
        const int64_t want = 2 * N * st.chunk - st.held_at_launch;
        if (want > 0) draw(st.gen, st.drawn, want);   // overlaps the steps just launched
    }
    st.queued = 0;
}

void GPUSpikingModel::advance(const SimulationInfo *sim_info)
{
    ModelState &st = state_of(this);
    if (++st.queued >= st.chunk) run_queued(st, sim_info);
}

// Fused into the sweep of every step (the reference's calcSummationMapDevice,
// Core/GPUSpikingModel.cu:382-416): nothing is left to do here.
void GPUSpikingModel::calcSummationMap(const SimulationInfo *) {}

void GPUSpikingModel::updateConnections(const SimulationInfo *sim_info)
{
    ModelState &st = state_of(this);
    run_queued(st, sim_info);
    AllSpikingNeurons *sn = dynamic_cast<AllSpikingNeurons *>(m_neurons);
    sn->copyNeuronDeviceSpikeCountsToHost(m_allNeuronsDevice, sim_info);
    sn->copyNeuronDeviceSpikeHistoryToHost(m_allNeuronsDevice, sim_info);
    if (dynamic_cast<ConnGrowth *>(m_conns)) {
        m_conns->updateSynapsesWeights(sim_info->totalNeurons, *m_neurons, *m_synapses, sim_info,
                                       m_allNeuronsDevice, m_allSynapsesDevice, m_layout);
    } else {
        // no growth: the device's own recorder histories and its spike-count roll
        bg3_dropin_check(bg3_epoch_record(st.net), "bg3_epoch_record");
    }
    uint32_t err = 0;
    bg3_dropin_check(bg3_error_word(st.net, &err), "bg3_error_word");
    if (err) {
        fprintf(stderr, "GPUSpikingModel: device error word 0x%x after epoch %d\n", err,
                sim_info->currentStep);
        exit(EXIT_FAILURE);
    }
}

void GPUSpikingModel::updateHistory(const SimulationInfo *sim_info)
{
    Model::updateHistory(sim_info);
    dynamic_cast<AllSpikingNeurons *>(m_neurons)->clearNeuronSpikeCounts(m_allNeuronsDevice, sim_info);
    if (sim_info->currentStep == sim_info->maxSteps && !sim_info->memOutputFileName.empty()) {
        // the driver writes the checkpoint from the host objects next (Core/BGDriver.cpp:110-116)
        m_neurons->copyNeuronDeviceToHost(m_allNeuronsDevice, sim_info);
        m_synapses->copySynapseDeviceToHost(m_allSynapsesDevice, sim_info);
    }
}

void GPUSpikingModel::deserialize(istream &input, const SimulationInfo *sim_info)
{
    Model::deserialize(input, sim_info);
    m_neurons->copyNeuronHostToDevice(m_allNeuronsDevice, sim_info);
    m_synapses->copySynapseHostToDevice(m_allSynapsesDevice, sim_info);
    if (ConnGrowth *g = dynamic_cast<ConnGrowth *>(m_conns))
        bg3_dropin_check(bg3_upload_growth(state_of(this).net, NULL, &(*g->radii)[0],
                                           &(*g->rates)[0]),
                         "bg3_upload_growth");
}

void GPUSpikingModel::cleanupSim(SimulationInfo *sim_info)
{
    ModelState &st = state_of(this);
    run_queued(st, sim_info);
    deleteDeviceStruct((void **)&m_allNeuronsDevice, (void **)&m_allSynapsesDevice, sim_info);
    st.drawn.clear();
    Model::cleanupSim(sim_info);
}
