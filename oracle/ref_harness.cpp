// Step-locked state dumper around the reference single-threaded simulator.
//
// Test infrastructure only (the checker): it links the reference's own objects (built by
// oracle/ref.mk from the reference sources) and replays what Core/BGDriver.cpp:49-158 and
// Core/Simulator.cpp:94-186 do, but one step at a time, writing the model state to a binary
// dump that tests/golden/make_golden.py and the oracle tests read.
//
//   bg_ref_harness -t config.xml -o dump.bin [-s stim.xml] [--epochs E] [--tsim SECONDS]
//                  [--dump-every K] [--dump-syn-every K] [--radii R] [--maxsyn M]
//                  [--record-noise] [--steps-limit S] [--serialize FILE]
//
// --serialize writes the reference's checkpoint stream (Simulator::serialize, Core/
// Simulator.cpp:225-232) at the end of the run, where Core/BGDriver.cpp:110-116 writes it.
//
// Dump format: "BGR1", then records: name[24] (NUL padded), dtype char ('f' float32,
// 'd' float64, 'i' int32, 'I' uint32, 'Q' uint64, 'B' uint8), 7 pad bytes, uint64 count,
// uint64 step, then count elements.  A record named "end" closes the file.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <cstring>
#include <string>
#include <vector>
#include <climits>

#include "Global.h"
#include "SimulationInfo.h"
#include "Simulator.h"
#include "SingleThreadedSpikingModel.h"
#include "FClassOfCategory.h"
#include "FSInput.h"
#include "ISInput.h"
#include "AllIFNeurons.h"
#include "AllIZHNeurons.h"
#include "AllSpikingNeurons.h"
#include "AllSpikingSynapses.h"
#include "AllDSSynapses.h"
#include "AllSTDPSynapses.h"
#include "AllDynamicSTDPSynapses.h"
#include "ConnGrowth.h"
#include "Layout.h"
#include "IRecorder.h"
#include "tinyxml.h"
#include "HostSInputPoisson.h"

// ---------------------------------------------------------------------------------------------
static FILE *g_out = NULL;

static void rec_raw(const char *name, char dt, size_t esz, uint64_t n, uint64_t step, const void *p)
{
    char hdr[24 + 8];
    memset(hdr, 0, sizeof(hdr));
    strncpy(hdr, name, 23);
    hdr[24] = dt;
    fwrite(hdr, 1, sizeof(hdr), g_out);
    fwrite(&n, 8, 1, g_out);
    fwrite(&step, 8, 1, g_out);
    if (n) fwrite(p, esz, n, g_out);
}
static void rec(const char *name, uint64_t step, const float *p, uint64_t n) { rec_raw(name, 'f', 4, n, step, p); }
static void rec(const char *name, uint64_t step, const double *p, uint64_t n) { rec_raw(name, 'd', 8, n, step, p); }
static void rec(const char *name, uint64_t step, const int *p, uint64_t n) { rec_raw(name, 'i', 4, n, step, p); }
static void rec(const char *name, uint64_t step, const uint32_t *p, uint64_t n) { rec_raw(name, 'I', 4, n, step, p); }
static void rec(const char *name, uint64_t step, const uint64_t *p, uint64_t n) { rec_raw(name, 'Q', 8, n, step, p); }
static void rec_bool(const char *name, uint64_t step, const bool *p, uint64_t n)
{
    std::vector<unsigned char> b(n);
    for (uint64_t i = 0; i < n; i++) b[i] = p[i] ? 1 : 0;
    rec_raw(name, 'B', 1, n, step, n ? &b[0] : NULL);
}

// Noise stream recorder: the reference draws N(0,1) through the virtual Norm::operator()
// (RNG/Norm.h:77), so a subclass sees every value in consumption order.
class RecordingNorm : public Norm {
public:
    RecordingNorm(BGFLOAT m, BGFLOAT s, uint32_t seed) : Norm(m, s, seed) {}
    virtual BGFLOAT operator()() { BGFLOAT v = Norm::operator()(); drawn.push_back(v); return v; }
    std::vector<BGFLOAT> drawn;
};

// The reference's HostSInputPoisson (Inputs/HostSInputPoisson.cpp:60-94, SInputPoisson.cpp:129-146)
// with one documented fix: its one-slot-per-neuron synapse object is indexed by neuron, not by
// maxSynapsesPerNeuron * neuron (out of bounds whenever maxSynapsesPerNeuron > 1).  Everything
// else — rng draws, rejection rule, synapse creation, the DS advance — is the reference's code.
class FixedPoissonInput : public HostSInputPoisson {
public:
    FixedPoissonInput(SimulationInfo *psi, TiXmlElement *parms) : HostSInputPoisson(psi, parms) {}
    virtual void init(SimulationInfo *psi)
    {
        if (!fSInput) return;
        m_synapses = new AllDSSynapses(psi->totalNeurons, 1);
        for (int i = 0; i < psi->totalNeurons; i++) {
            synapseType type = (psi->model->getLayout()->neuron_type_map[i] == INH) ? EI : EE;
            BGFLOAT *sum_point = &(psi->pSummationMap[i]);
            m_synapses->createSynapse((BGSIZE)i, 0, i, sum_point, psi->deltaT, type);
            dynamic_cast<AllSynapses *>(m_synapses)->W[i] = weight * AllSynapses::SYNAPSE_STRENGTH_ADJUSTMENT;
        }
    }
    virtual void inputStimulus(SimulationInfo *psi)
    {
        if (!fSInput) return;
        for (int i = 0; i < psi->totalNeurons; i++) {
            if (!masks[i]) continue;
            if (--nISIs[i] <= 0) {
                dynamic_cast<AllSpikingSynapses *>(m_synapses)->preSpikeHit((BGSIZE)i);
                BGFLOAT isi = -lambda * log(rng.inRange(0, 1));
                while (rng.inRange(0, 1) <= exp(-(isi * isi) / 32))
                    isi = -lambda * log(rng.inRange(0, 1));
                nISIs[i] = static_cast<int>((isi / 1000) / psi->deltaT + 0.5);
            }
            m_synapses->advanceSynapse((BGSIZE)i, psi, NULL);
        }
    }
    int *isis() { return nISIs; }
    AllDSSynapses *syn() { return dynamic_cast<AllDSSynapses *>(m_synapses); }
};

static ISInput *make_input(SimulationInfo *si)
{
    if (si->stimulusInputFileName.empty()) return NULL;
    TiXmlDocument doc(si->stimulusInputFileName.c_str());
    if (!doc.LoadFile()) return NULL;
    TiXmlElement *parms = doc.FirstChildElement("InputParams");
    if (!parms) return NULL;
    TiXmlElement *m = parms->FirstChildElement("IMethod");
    std::string name;
    if (m && m->QueryValueAttribute("name", &name) == TIXML_SUCCESS && name == "SInputPoisson")
        return new FixedPoissonInput(si, parms);
    return FSInput::get()->CreateInstance(si);
}

static void dump_input(SimulationInfo *si, uint64_t t)
{
    FixedPoissonInput *p = dynamic_cast<FixedPoissonInput *>(si->pInput);
    if (!p || !p->syn()) return;
    int N = si->totalNeurons;
    AllDSSynapses *s = p->syn();
    rec("in.nisi", t, p->isis(), N);
    rec("in.psr", t, s->psr, N); rec("in.u", t, s->u, N); rec("in.r", t, s->r, N);
    rec("in.lastSpike", t, s->lastSpike, N); rec("in.queue", t, s->delayQueue, N);
    rec("in.delayIdx", t, s->delayIdx, N);
}

// Exposes the protected members of Core/Model.h:134-169.
class HarnessModel : public SingleThreadedSpikingModel {
public:
    HarnessModel(Connections *c, IAllNeurons *n, IAllSynapses *s, Layout *l)
        : SingleThreadedSpikingModel(c, n, s, l) {}
    IAllNeurons *neurons() { return m_neurons; }
    IAllSynapses *synapses() { return m_synapses; }
    Connections *conns() { return m_conns; }
    Layout *layout() { return m_layout; }
    SynapseIndexMap *imap() { return m_synapseIndexMap; }
};

static bool create_instances(TiXmlDocument *doc, SimulationInfo *si)
{
    TiXmlElement *parms = doc->FirstChildElement()->FirstChildElement("ModelParams");
    if (!parms) return false;
    IAllNeurons *neurons = NULL; IAllSynapses *synapses = NULL; Connections *conns = NULL; Layout *layout = NULL;
    const TiXmlNode *p = NULL;
    while ((p = parms->IterateChildren(p)) != NULL) {
        if (strcmp(p->Value(), "NeuronsParams") == 0) neurons = FClassOfCategory::get()->createNeurons(p);
        else if (strcmp(p->Value(), "SynapsesParams") == 0) synapses = FClassOfCategory::get()->createSynapses(p);
        else if (strcmp(p->Value(), "ConnectionsParams") == 0) conns = FClassOfCategory::get()->createConnections(p);
        else if (strcmp(p->Value(), "LayoutParams") == 0) layout = FClassOfCategory::get()->createLayout(p);
    }
    if (!neurons || !synapses || !conns || !layout) return false;
    si->model = new HarnessModel(conns, neurons, synapses, layout);
    return true;
}

// ---------------------------------------------------------------------------------------------
static void dump_setup(HarnessModel *m, SimulationInfo *si)
{
    int N = si->totalNeurons;
    uint64_t t = g_simulationStep;
    int hdr[6] = {N, si->maxSynapsesPerNeuron, si->width, si->height,
                  (int)(si->epochDuration * si->maxFiringRate), si->maxSteps};
    rec("hdr", t, hdr, 6);
    BGFLOAT f[3] = {si->epochDuration, si->deltaT, (BGFLOAT)si->maxFiringRate};
    rec("hdrf", t, f, 3);
    Layout *L = m->layout();
    std::vector<int> types(N), starter(N);
    std::vector<BGFLOAT> x(N), y(N);
    for (int i = 0; i < N; i++) {
        types[i] = L->neuron_type_map[i];
        starter[i] = L->starter_map[i] ? 1 : 0;
        x[i] = (*L->xloc)[i];
        y[i] = (*L->yloc)[i];
    }
    rec("ntype", t, &types[0], N);
    rec("starter", t, &starter[0], N);
    rec("xloc", t, &x[0], N);
    rec("yloc", t, &y[0], N);
    AllIFNeurons *nf = dynamic_cast<AllIFNeurons *>(m->neurons());
    if (nf) {
        rec("Vm", t, nf->Vm, N); rec("Vthresh", t, nf->Vthresh, N); rec("Vreset", t, nf->Vreset, N);
        rec("Vrest", t, nf->Vrest, N); rec("Vinit", t, nf->Vinit, N); rec("I0", t, nf->I0, N);
        rec("Inoise", t, nf->Inoise, N); rec("Iinject", t, nf->Iinject, N); rec("C1", t, nf->C1, N);
        rec("C2", t, nf->C2, N); rec("Trefract", t, nf->Trefract, N); rec("Rm", t, nf->Rm, N);
        rec("Cm", t, nf->Cm, N); rec("Tau", t, nf->Tau, N); rec("refr", t, nf->nStepsInRefr, N);
    }
    AllIZHNeurons *nz = dynamic_cast<AllIZHNeurons *>(m->neurons());
    if (nz) {
        rec("Aconst", t, nz->Aconst, N); rec("Bconst", t, nz->Bconst, N); rec("Cconst", t, nz->Cconst, N);
        rec("Dconst", t, nz->Dconst, N); rec("u", t, nz->u, N); rec("C3", t, nz->C3, N);
    }
    ConnGrowth *g = dynamic_cast<ConnGrowth *>(m->conns());
    if (g) {
        std::vector<BGFLOAT> r(N);
        for (int i = 0; i < N; i++) r[i] = (*g->radii)[i];
        rec("radii", t, &r[0], N);
        BGFLOAT gp[7] = {g->m_growth.epsilon, g->m_growth.beta, g->m_growth.rho, g->m_growth.targetRate,
                         g->m_growth.minRadius, g->m_growth.startRadius, g->m_growth.maxRate};
        rec("growth", t, gp, 7);
    }
}

static void dump_neurons_step(HarnessModel *m, SimulationInfo *si, uint64_t t)
{
    int N = si->totalNeurons;
    AllIFNeurons *nf = dynamic_cast<AllIFNeurons *>(m->neurons());
    AllSpikingNeurons *ns = dynamic_cast<AllSpikingNeurons *>(m->neurons());
    AllNeurons *na = dynamic_cast<AllNeurons *>(m->neurons());
    if (nf) { rec("s.Vm", t, nf->Vm, N); rec("s.refr", t, nf->nStepsInRefr, N); }
    AllIZHNeurons *nz = dynamic_cast<AllIZHNeurons *>(m->neurons());
    if (nz) rec("s.u", t, nz->u, N);
    if (ns) rec("s.spikeCount", t, ns->spikeCount, N);
    if (na) rec("s.sp", t, na->summation_map, N);
}

static void dump_synapses(HarnessModel *m, SimulationInfo *si, uint64_t t, const char *pfx)
{
    int N = si->totalNeurons;
    uint64_t S = (uint64_t)N * si->maxSynapsesPerNeuron;
    char nm[64];
#define R(field, ptr) do { snprintf(nm, sizeof nm, "%s%s", pfx, field); rec(nm, t, ptr, S); } while (0)
    AllSynapses *sa = dynamic_cast<AllSynapses *>(m->synapses());
    if (!sa || S == 0) return;
    snprintf(nm, sizeof nm, "%sin_use", pfx); rec_bool(nm, t, sa->in_use, S);
    R("psr", sa->psr); R("W", sa->W); R("src", sa->sourceNeuronIndex); R("dest", sa->destNeuronIndex);
    std::vector<int> ty(S);
    for (uint64_t i = 0; i < S; i++) ty[i] = sa->in_use[i] ? (int)sa->type[i] : -1;
    R("type", &ty[0]);
    snprintf(nm, sizeof nm, "%scounts", pfx); rec(nm, t, sa->synapse_counts, (uint64_t)N);
    AllSpikingSynapses *ss = dynamic_cast<AllSpikingSynapses *>(m->synapses());
    if (ss) {
        R("decay", ss->decay); R("tau", ss->tau); R("total_delay", ss->total_delay);
        R("queue", ss->delayQueue); R("delayIdx", ss->delayIdx); R("ldelayQueue", ss->ldelayQueue);
    }
    AllDSSynapses *ds = dynamic_cast<AllDSSynapses *>(m->synapses());
    if (ds) { R("lastSpike", ds->lastSpike); R("r", ds->r); R("u", ds->u); R("D", ds->D); R("U", ds->U); R("F", ds->F); }
    AllSTDPSynapses *sp = dynamic_cast<AllSTDPSynapses *>(m->synapses());
    if (sp) {
        R("queuePost", sp->delayQueuePost); R("delayIdxPost", sp->delayIdxPost);
        R("total_delayPost", sp->total_delayPost); R("tauspost", sp->tauspost); R("tauspre", sp->tauspre);
        R("taupos", sp->taupos); R("tauneg", sp->tauneg); R("STDPgap", sp->STDPgap); R("Wex", sp->Wex);
        R("Aneg", sp->Aneg); R("Apos", sp->Apos); R("mupos", sp->mupos); R("muneg", sp->muneg);
    }
    AllDynamicSTDPSynapses *dd = dynamic_cast<AllDynamicSTDPSynapses *>(m->synapses());
    if (dd) { R("lastSpike", dd->lastSpike); R("r", dd->r); R("u", dd->u); R("D", dd->D); R("U", dd->U); R("F", dd->F); }
#undef R
}

static void dump_epoch(HarnessModel *m, SimulationInfo *si, uint64_t t, const char *pfx)
{
    int N = si->totalNeurons;
    char nm[64];
#define NM(s) (snprintf(nm, sizeof nm, "%s%s", pfx, s), nm)
    ConnGrowth *g = dynamic_cast<ConnGrowth *>(m->conns());
    if (g) {
        std::vector<BGFLOAT> r(N), q(N);
        for (int i = 0; i < N; i++) { r[i] = (*g->radii)[i]; q[i] = (*g->rates)[i]; }
        rec(NM("radii"), t, &r[0], N);
        rec(NM("rates"), t, &q[0], N);
    }
    AllSpikingNeurons *ns = dynamic_cast<AllSpikingNeurons *>(m->neurons());
    if (ns) {
        rec(NM("spikeCount"), t, ns->spikeCount, N);
        rec(NM("spikeCountOffset"), t, ns->spikeCountOffset, N);
        int maxs = (int)(si->epochDuration * si->maxFiringRate);
        std::vector<uint64_t> h((size_t)N * maxs);
        for (int i = 0; i < N; i++) memcpy(&h[(size_t)i * maxs], ns->spike_history[i], 8 * (size_t)maxs);
        rec(NM("history"), t, &h[0], h.size());
    }
    dump_synapses(m, si, t, pfx);
    SynapseIndexMap *im = m->imap();
    AllSynapses *sa = dynamic_cast<AllSynapses *>(m->synapses());
    if (im && sa) {
        uint64_t tot = sa->total_synapse_counts;
        rec(NM("inMap"), t, im->incomingSynapseIndexMap, tot);
        rec(NM("inBegin"), t, im->incomingSynapseBegin, (uint64_t)N);
        rec(NM("inCount"), t, im->incomingSynapseCount, (uint64_t)N);
        rec(NM("outMap"), t, im->outgoingSynapseIndexMap, tot);
        rec(NM("outBegin"), t, im->outgoingSynapseBegin, (uint64_t)N);
        rec(NM("outCount"), t, im->outgoingSynapseCount, (uint64_t)N);
    }
#undef NM
}

// Parameter override (a documented deviation): the reference hard-codes its STDP constants in
// AllSTDPSynapses::createSynapse (Synapses/AllSTDPSynapses.cpp:252-273) and reads none from the
// configuration.  Synapses are only created by growth here, so setting the constants of every
// in-use synapse right after each growth pass is the same as creating them with these values.
// Wex takes the source's sign: WexE for EI/EE synapses, WexI for II/IE.
static void override_stdp(HarnessModel *m, SimulationInfo *si, const BGFLOAT *p)
{
    AllSTDPSynapses *sp = dynamic_cast<AllSTDPSynapses *>(m->synapses());
    if (!sp) return;
    uint64_t S = (uint64_t)si->totalNeurons * si->maxSynapsesPerNeuron;
    for (uint64_t i = 0; i < S; i++) {
        if (!sp->in_use[i]) continue;
        sp->Apos[i] = p[0]; sp->Aneg[i] = p[1]; sp->STDPgap[i] = p[2];
        sp->tauspost[i] = p[3]; sp->tauspre[i] = p[4]; sp->taupos[i] = p[5]; sp->tauneg[i] = p[6];
        sp->Wex[i] = (sp->type[i] == II || sp->type[i] == IE) ? p[8] : p[7];
        sp->mupos[i] = p[9]; sp->muneg[i] = p[10];
    }
}

int main(int argc, char **argv)
{
    std::string cfg, out, stim, ser;
    BGFLOAT stdp_p[11];
    int n_stdp = 0;
    int epochs = -1, dump_every = 0, dump_syn_every = 0, maxsyn = -1;
    long steps_limit = -1;
    double tsim = -1, radii = -1;
    bool record_noise = false;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "-t") cfg = argv[++i];
        else if (a == "-o") out = argv[++i];
        else if (a == "-s") stim = argv[++i];
        else if (a == "--epochs") epochs = atoi(argv[++i]);
        else if (a == "--tsim") tsim = atof(argv[++i]);
        else if (a == "--dump-every") dump_every = atoi(argv[++i]);
        else if (a == "--dump-syn-every") dump_syn_every = atoi(argv[++i]);
        else if (a == "--radii") radii = atof(argv[++i]);
        else if (a == "--maxsyn") maxsyn = atoi(argv[++i]);
        else if (a == "--record-noise") record_noise = true;
        else if (a == "--serialize") ser = argv[++i];
        else if (a == "--steps-limit") steps_limit = atol(argv[++i]);
        else if (a == "--stdp") {
            // Apos,Aneg,STDPgap,tauspost,tauspre,taupos,tauneg,WexE,WexI,mupos,muneg
            std::string v = argv[++i];
            n_stdp = 0;
            for (size_t p = 0; n_stdp < 11 && p <= v.size();) {
                size_t q = v.find(',', p);
                if (q == std::string::npos) q = v.size();
                stdp_p[n_stdp++] = (BGFLOAT)atof(v.substr(p, q - p).c_str());
                p = q + 1;
            }
            if (n_stdp != 11) { fprintf(stderr, "--stdp wants 11 values\n"); return 2; }
        }
        else { fprintf(stderr, "unknown arg %s\n", a.c_str()); return 2; }
    }
    if (cfg.empty() || out.empty()) { fprintf(stderr, "usage: -t cfg -o out\n"); return 2; }

    SimulationInfo *si = new SimulationInfo();
    si->stateInputFileName = cfg;
    si->stimulusInputFileName = stim;
    TiXmlDocument doc(cfg.c_str());
    if (!doc.LoadFile()) { fprintf(stderr, "cannot load %s\n", cfg.c_str()); return 1; }
    if (!si->readParameters(&doc)) return 1;
    if (epochs > 0) si->maxSteps = epochs;
    if (tsim > 0) si->epochDuration = (BGFLOAT)tsim;
    if (maxsyn > 0) si->maxSynapsesPerNeuron = maxsyn;
    if (!create_instances(&doc, si)) { fprintf(stderr, "class creation failed\n"); return 1; }
    if (!FClassOfCategory::get()->readParameters(&doc)) { fprintf(stderr, "param read failed\n"); return 1; }
    si->stateOutputFileName = out + ".xml";
    si->simRecorder = si->model->getConnections()->createRecorder(si);
    si->pInput = make_input(si);

    Simulator *sim = new Simulator();
    sim->setup(si);
    HarnessModel *m = static_cast<HarnessModel *>(si->model);

    // Replace the noise generator by an identically seeded recorder
    // (Core/SingleThreadedSpikingModel.cpp:30 constructs Norm(0, 1, seed) and draws nothing).
    RecordingNorm *rn = new RecordingNorm(0, 1, si->seed);
    delete rgNormrnd[0];
    rgNormrnd[0] = rn;

    if (n_stdp) override_stdp(m, si, stdp_p);  // synapses made by setupConnections (ConnStatic)
    ConnGrowth *g = dynamic_cast<ConnGrowth *>(m->conns());
    if (g && radii > 0)
        for (int i = 0; i < si->totalNeurons; i++) (*g->radii)[i] = (BGFLOAT)radii;

    g_out = fopen(out.c_str(), "wb");
    fwrite("BGR1", 1, 4, g_out);
    dump_setup(m, si);
    dump_synapses(m, si, g_simulationStep, "i.");

    long steps_done = 0;
    for (int epoch = 1; epoch <= si->maxSteps; epoch++) {
        si->currentStep = epoch;
        uint64_t endStep = g_simulationStep + static_cast<uint64_t>(si->epochDuration / si->deltaT);
        while (g_simulationStep < endStep) {
            size_t before = rn->drawn.size();
            if (si->pInput != NULL) si->pInput->inputStimulus(si);
            si->model->advance(si);
            uint64_t t = g_simulationStep;
            g_simulationStep++;
            if (record_noise) {
                int cnt = (int)(rn->drawn.size() - before);
                rec("n.count", t, &cnt, 1);
                if (cnt) rec("n.vals", t, &rn->drawn[before], (uint64_t)cnt);
            }
            if (dump_every > 0 && (t % dump_every) == 0) {
                dump_neurons_step(m, si, t);
                dump_input(si, t);
            }
            if (dump_syn_every > 0 && (t % dump_syn_every) == 0) dump_synapses(m, si, t, "s.");
            steps_done++;
            if (steps_limit > 0 && steps_done >= steps_limit) break;
        }
        if (steps_limit > 0 && steps_done >= steps_limit) break;
        // record spike history and counts before the recorder consumes them
        dump_epoch(m, si, g_simulationStep, "pre.");
        si->model->updateConnections(si);
        if (n_stdp) override_stdp(m, si, stdp_p);
        dump_epoch(m, si, g_simulationStep, "grow.");   // after growth, before the recorder
        si->model->updateHistory(si);
        dump_epoch(m, si, g_simulationStep, "post.");   // after the recorder (radius clamp, count roll)
    }
    rec_raw("end", 'B', 1, 0, g_simulationStep, NULL);
    fclose(g_out);
    if (si->pInput) { si->pInput->term(si); }
    sim->saveData(si);
    if (!ser.empty()) {
        std::ofstream mo(ser.c_str(), std::ofstream::binary | std::ofstream::trunc);
        sim->serialize(mo, si);
        mo.close();
    }
    if (si->simRecorder) si->simRecorder->term();
    return 0;
}
