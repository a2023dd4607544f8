/* CPU oracle for the BrainGrid per-step spiking hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference single-threaded simulator, used as the checker for the
 * CUDA path.  Each function cites the reference file:line it follows (paths relative to the
 * reference project root).  Pinned bit-for-bit against dumps of the compiled reference
 * (tests/golden/, generated by tests/golden/make_golden.py with oracle/ref_harness.cpp).
 *
 * Arithmetic is kept in the reference's types and order: BGFLOAT = float
 * (Utils/BGTypes.h:20-21), each float operation rounded on its own (compile with
 * -ffp-contract=off), double only where the reference promotes (double literals).
 */
#include "bg_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#define ULONG_MAX_U64 0xffffffffffffffffULL
#define LDELAYQUEUE 32 /* LENGTH_OF_DELAYQUEUE, Synapses/AllSpikingSynapses.h */

/* ============================== RNG ============================== */
/* MTRand::initialize + reload (RNG/MersenneTwister.cpp:260-291): the standard MT19937. */
static uint32_t mt_twist(uint32_t m, uint32_t s0, uint32_t s1)
{
    return m ^ (((s0 & 0x80000000u) | (s1 & 0x7fffffffu)) >> 1) ^ ((0u - (s1 & 1u)) & 0x9908b0dfu);
}
static void mt_reload(bgo_mt *m)
{
    uint32_t *s = m->s;
    int i;
    for (i = 0; i < 624 - 397; i++) s[i] = mt_twist(s[i + 397], s[i], s[i + 1]);
    for (; i < 623; i++) s[i] = mt_twist(s[i + 397 - 624], s[i], s[i + 1]);
    s[623] = mt_twist(s[396], s[623], s[0]);
    m->left = 624;
    m->next = 0;
}
void bgo_mt_seed(bgo_mt *m, uint32_t seed)
{
    m->s[0] = seed;
    for (int i = 1; i < 624; i++) m->s[i] = 1812433253u * (m->s[i - 1] ^ (m->s[i - 1] >> 30)) + (uint32_t)i;
    mt_reload(m);
}
/* MTRand::randInt (RNG/MersenneTwister.cpp): tempering of the next state word. */
uint32_t bgo_mt_randint(bgo_mt *m)
{
    if (m->left == 0) mt_reload(m);
    --m->left;
    uint32_t y = m->s[m->next++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    return y ^ (y >> 18);
}
/* MTRand::rand: float(randInt) * (1.0/4294967295.0) evaluated in double, returned as float. */
float bgo_mt_rand(bgo_mt *m)
{
    return (float)((double)(float)bgo_mt_randint(m) * (1.0 / 4294967295.0));
}
/* MTRand::inRange: val *= (max - min); val += min, all float. */
float bgo_mt_inrange(bgo_mt *m, float lo, float hi)
{
    float v = bgo_mt_rand(m);
    float range = hi - lo;
    v *= range;
    v += lo;
    return v;
}
/* Norm::operator() (RNG/Norm.cpp:59-86): Marsaglia polar method, values returned in pairs. */
void bgo_norm_init(bgo_norm *n, float mu, float sigma, uint32_t seed)
{
    bgo_mt_seed(&n->mt, seed);
    n->odd = 1;
    n->mu = mu;
    n->sigma = sigma;
    n->x2 = 0.0f;
}
float bgo_norm_next(bgo_norm *n)
{
    if ((n->odd = !n->odd)) return n->mu + n->sigma * n->x2;
    float u1, u2, v1, v2, w, y, x1;
    do {
        u1 = bgo_mt_rand(&n->mt);
        u2 = bgo_mt_rand(&n->mt);
        v1 = 2.0f * u1 - 1.0f;
        v2 = 2.0f * u2 - 1.0f;
        w = v1 * v1 + v2 * v2;
    } while (w > 1.0f);
    y = sqrtf(-2.0f * logf(w) / w);
    x1 = v1 * y;
    n->x2 = v2 * y;
    return n->mu + n->sigma * x1;
}
void bgo_norm_fill(uint32_t seed, float *out, int64_t cnt)
{
    bgo_norm n;
    bgo_norm_init(&n, 0.0f, 1.0f, seed);
    for (int64_t i = 0; i < cnt; i++) out[i] = bgo_norm_next(&n);
}

/* ============================== state ============================== */
struct bgo_net {
    int N, max_syn, width, height, max_spikes, max_epochs, neuron_kind, syn_kind;
    float epoch_duration, delta_t;
    int max_firing_rate;
    uint64_t step;
    int flags;
    bgo_mt rng;      /* global `MTRand rng(1)` (Utils/Global.cpp:79) */
    bgo_norm noise;  /* rgNormrnd[0] = Norm(0, 1, seed) (Core/SingleThreadedSpikingModel.cpp:30) */
    float *noise_rec;
    int64_t noise_cap, noise_n;
    /* layout */
    float *xloc, *yloc;
    int *ntype, *starter;
    /* IF neurons (Neurons/AllIFNeurons.h:279-362) */
    float *Vm, *Vthresh, *Vreset, *Vrest, *Vinit, *I0, *Inoise, *Iinject, *C1, *C2, *Trefract;
    float *Rm, *Cm, *Tau, *sp;
    float *Aconst, *Bconst, *Cconst, *Dconst, *u_izh, *C3; /* Neurons/AllIZHNeurons.h:380-472 */
    int *refr, *spikeCount, *spikeCountOffset;
    uint8_t *hasFired;
    uint64_t *history; /* [N][max_spikes] */
    /* synapse slots, iSyn = dest * max_syn + k (Synapses/AllSynapses.cpp:367) */
    uint8_t *in_use;
    int *src, *dest, *type, *total_delay, *delayIdx, *ldelayQueue;
    float *W, *psr, *decay, *tau, *r, *u, *D, *U, *F;
    uint32_t *queue, *counts;
    uint64_t *lastSpike;
    /* STDP slots (Synapses/AllSTDPSynapses.h:330-420), allocated for the STDP kinds only */
    int *total_delayPost, *delayIdxPost, *ldelayQueuePost;
    uint32_t *queuePost;
    float *tauspost, *tauspre, *taupos, *tauneg, *STDPgap, *Wex, *Aneg, *Apos, *mupos, *muneg;
    uint8_t *useFD;
    int stdp_signed; /* 0: host build's arithmetic, 1: device build's (signed spike times) */
    int stdp_override;
    float stdp_p[11]; /* Apos, Aneg, STDPgap, tauspost, tauspre, taupos, tauneg, WexE, WexI, mupos, muneg */
    /* SynapseIndexMap (Core/SynapseIndexMap.h:38-104) */
    uint32_t *inMap, *inBegin, *inCount, *outMap, *outBegin, *outCount;
    int64_t total;
    /* ConnGrowth (Connections/ConnGrowth.h) */
    float *radii, *rates;
    float epsilon, beta, rho, target_rate, min_radius, start_radius, max_rate;
    /* recorder histories (Recorders/XmlRecorder.cpp, XmlGrowthRecorder.cpp) */
    float *burstinessHist, *spikesHistory, *ratesHistory, *radiiHistory;
    /* inputs: 0 none, 1 regular, 2 poisson */
    int input_kind;
    int reg_dur, reg_cycle, reg_in_cycle;
    float *reg_values;
    int *reg_shift;
    float pois_lambda;
    uint8_t *pois_mask;
    int *pois_nisi;
    /* the Poisson input synapses: one DS synapse per neuron (SInputPoisson::init) */
    float *in_W, *in_psr, *in_decay, *in_U, *in_D, *in_F, *in_u, *in_r;
    int *in_delay, *in_delayIdx;
    uint32_t *in_queue;
    uint64_t *in_last;
};

#define ALLOC(p, cnt) ((p) = calloc((size_t)(cnt) ? (size_t)(cnt) : 1, sizeof(*(p))))

bgo_net *bgo_create(int N, int max_syn, int width, int height, float epoch_duration, float delta_t,
                    int max_firing_rate, int max_epochs, int neuron_kind, int synapse_kind)
{
    bgo_net *n = calloc(1, sizeof(*n));
    n->N = N; n->max_syn = max_syn; n->width = width; n->height = height;
    n->epoch_duration = epoch_duration; n->delta_t = delta_t; n->max_firing_rate = max_firing_rate;
    n->max_epochs = max_epochs; n->neuron_kind = neuron_kind; n->syn_kind = synapse_kind;
    /* int max_spikes = (int)(epochDuration * maxFiringRate) (Neurons/AllSpikingNeurons.cpp:81) */
    n->max_spikes = (int)(epoch_duration * (float)max_firing_rate);
    bgo_mt_seed(&n->rng, 1);
    bgo_norm_init(&n->noise, 0.0f, 1.0f, 0);
    size_t S = (size_t)N * max_syn;
    ALLOC(n->xloc, N); ALLOC(n->yloc, N); ALLOC(n->ntype, N); ALLOC(n->starter, N);
    ALLOC(n->Vm, N); ALLOC(n->Vthresh, N); ALLOC(n->Vreset, N); ALLOC(n->Vrest, N);
    ALLOC(n->Vinit, N); ALLOC(n->I0, N); ALLOC(n->Inoise, N); ALLOC(n->Iinject, N);
    ALLOC(n->C1, N); ALLOC(n->C2, N); ALLOC(n->Trefract, N); ALLOC(n->Rm, N); ALLOC(n->Cm, N);
    ALLOC(n->Tau, N); ALLOC(n->sp, N); ALLOC(n->refr, N); ALLOC(n->spikeCount, N);
    ALLOC(n->spikeCountOffset, N); ALLOC(n->hasFired, N);
    ALLOC(n->Aconst, N); ALLOC(n->Bconst, N); ALLOC(n->Cconst, N); ALLOC(n->Dconst, N);
    ALLOC(n->u_izh, N); ALLOC(n->C3, N);
    ALLOC(n->history, (size_t)N * n->max_spikes);
    for (size_t i = 0; i < (size_t)N * n->max_spikes; i++) n->history[i] = ULONG_MAX_U64;
    ALLOC(n->in_use, S); ALLOC(n->src, S); ALLOC(n->dest, S); ALLOC(n->type, S);
    ALLOC(n->total_delay, S); ALLOC(n->delayIdx, S); ALLOC(n->ldelayQueue, S);
    ALLOC(n->W, S); ALLOC(n->psr, S); ALLOC(n->decay, S); ALLOC(n->tau, S); ALLOC(n->r, S);
    ALLOC(n->u, S); ALLOC(n->D, S); ALLOC(n->U, S); ALLOC(n->F, S); ALLOC(n->queue, S);
    ALLOC(n->lastSpike, S); ALLOC(n->counts, N);
    for (size_t i = 0; i < S; i++) n->type[i] = -1;
    if (synapse_kind == BGO_SYN_STDP || synapse_kind == BGO_SYN_DSTDP) {
        ALLOC(n->total_delayPost, S); ALLOC(n->delayIdxPost, S); ALLOC(n->ldelayQueuePost, S);
        ALLOC(n->queuePost, S); ALLOC(n->tauspost, S); ALLOC(n->tauspre, S); ALLOC(n->taupos, S);
        ALLOC(n->tauneg, S); ALLOC(n->STDPgap, S); ALLOC(n->Wex, S); ALLOC(n->Aneg, S);
        ALLOC(n->Apos, S); ALLOC(n->mupos, S); ALLOC(n->muneg, S); ALLOC(n->useFD, S);
    }
    ALLOC(n->inMap, S); ALLOC(n->outMap, S);
    ALLOC(n->inBegin, N); ALLOC(n->inCount, N); ALLOC(n->outBegin, N); ALLOC(n->outCount, N);
    ALLOC(n->radii, N); ALLOC(n->rates, N);
    int nb = (int)(max_epochs * epoch_duration);
    ALLOC(n->burstinessHist, nb);
    ALLOC(n->spikesHistory, (size_t)nb * 100);
    ALLOC(n->ratesHistory, (size_t)(max_epochs + 1) * N);
    ALLOC(n->radiiHistory, (size_t)(max_epochs + 1) * N);
    return n;
}

void bgo_destroy(bgo_net *n)
{
    if (!n) return;
    void *ptrs[] = {n->xloc, n->yloc, n->ntype, n->starter, n->Vm, n->Vthresh, n->Vreset, n->Vrest,
                    n->Vinit, n->I0, n->Inoise, n->Iinject, n->C1, n->C2, n->Trefract, n->Rm, n->Cm,
                    n->Tau, n->sp, n->refr, n->spikeCount, n->spikeCountOffset, n->hasFired,
                    n->history, n->in_use, n->src, n->dest, n->type, n->total_delay, n->delayIdx,
                    n->ldelayQueue, n->W, n->psr, n->decay, n->tau, n->r, n->u, n->D, n->U, n->F,
                    n->queue, n->lastSpike, n->counts, n->inMap, n->outMap, n->inBegin, n->inCount,
                    n->outBegin, n->outCount, n->radii, n->rates, n->burstinessHist,
                    n->spikesHistory, n->ratesHistory, n->radiiHistory, n->noise_rec};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
    void *izh[] = {n->Aconst, n->Bconst, n->Cconst, n->Dconst, n->u_izh, n->C3};
    for (size_t i = 0; i < sizeof(izh) / sizeof(izh[0]); i++) free(izh[i]);
    void *inp[] = {n->reg_values, n->reg_shift, n->pois_mask, n->pois_nisi, n->in_W, n->in_psr,
                   n->in_decay, n->in_U, n->in_D, n->in_F, n->in_u, n->in_r, n->in_delay,
                   n->in_delayIdx, n->in_queue, n->in_last};
    for (size_t i = 0; i < sizeof(inp) / sizeof(inp[0]); i++) free(inp[i]);
    void *stdp[] = {n->total_delayPost, n->delayIdxPost, n->ldelayQueuePost, n->queuePost,
                    n->tauspost, n->tauspre, n->taupos, n->tauneg, n->STDPgap, n->Wex, n->Aneg,
                    n->Apos, n->mupos, n->muneg, n->useFD};
    for (size_t i = 0; i < sizeof(stdp) / sizeof(stdp[0]); i++) free(stdp[i]);
    free(n);
}

void *bgo_array(bgo_net *n, const char *name, int64_t *count, int *esz)
{
    int64_t N = n->N, S = (int64_t)n->N * n->max_syn;
    int nb = (int)(n->max_epochs * n->epoch_duration);
#define A(nm, ptr, cnt) if (!strcmp(name, nm)) { *count = (cnt); *esz = (int)sizeof(*(ptr)); return (ptr); }
    A("xloc", n->xloc, N) A("yloc", n->yloc, N) A("ntype", n->ntype, N) A("starter", n->starter, N)
    A("Vm", n->Vm, N) A("Vthresh", n->Vthresh, N) A("Vreset", n->Vreset, N) A("Vrest", n->Vrest, N)
    A("Vinit", n->Vinit, N) A("I0", n->I0, N) A("Inoise", n->Inoise, N) A("Iinject", n->Iinject, N)
    A("C1", n->C1, N) A("C2", n->C2, N) A("Trefract", n->Trefract, N) A("Rm", n->Rm, N)
    A("Cm", n->Cm, N) A("Tau", n->Tau, N) A("sp", n->sp, N) A("refr", n->refr, N)
    A("spikeCount", n->spikeCount, N) A("spikeCountOffset", n->spikeCountOffset, N)
    A("hasFired", n->hasFired, N) A("history", n->history, N * n->max_spikes)
    A("in_use", n->in_use, S) A("src", n->src, S) A("dest", n->dest, S) A("type", n->type, S)
    A("total_delay", n->total_delay, S) A("delayIdx", n->delayIdx, S)
    A("ldelayQueue", n->ldelayQueue, S) A("W", n->W, S) A("psr", n->psr, S)
    A("decay", n->decay, S) A("tau", n->tau, S) A("r", n->r, S) A("u", n->u, S) A("D", n->D, S)
    A("U", n->U, S) A("F", n->F, S) A("queue", n->queue, S) A("lastSpike", n->lastSpike, S)
    A("counts", n->counts, N) A("inMap", n->inMap, n->total) A("outMap", n->outMap, n->total)
    A("inBegin", n->inBegin, N) A("inCount", n->inCount, N) A("outBegin", n->outBegin, N)
    A("outCount", n->outCount, N) A("radii", n->radii, N) A("rates", n->rates, N)
    A("burstinessHist", n->burstinessHist, nb) A("spikesHistory", n->spikesHistory, (int64_t)nb * 100)
    A("ratesHistory", n->ratesHistory, (int64_t)(n->max_epochs + 1) * N)
    A("radiiHistory", n->radiiHistory, (int64_t)(n->max_epochs + 1) * N)
    A("noise", n->noise_rec, n->noise_n)
    A("Aconst", n->Aconst, N) A("Bconst", n->Bconst, N) A("Cconst", n->Cconst, N)
    A("Dconst", n->Dconst, N) A("u_izh", n->u_izh, N) A("C3", n->C3, N)
    A("reg_values", n->reg_values, n->reg_values ? N : 0) A("reg_shift", n->reg_shift, n->reg_shift ? N : 0)
    A("pois_nisi", n->pois_nisi, n->pois_nisi ? N : 0) A("pois_mask", n->pois_mask, n->pois_mask ? N : 0)
    A("in_psr", n->in_psr, n->in_psr ? N : 0) A("in_u", n->in_u, n->in_u ? N : 0)
    A("in_r", n->in_r, n->in_r ? N : 0) A("in_last", n->in_last, n->in_last ? N : 0)
    A("in_queue", n->in_queue, n->in_queue ? N : 0) A("in_delayIdx", n->in_delayIdx, n->in_delayIdx ? N : 0)
    A("in_W", n->in_W, n->in_W ? N : 0) A("in_decay", n->in_decay, n->in_decay ? N : 0)
    A("in_delay", n->in_delay, n->in_delay ? N : 0) A("in_U", n->in_U, n->in_U ? N : 0)
    A("in_D", n->in_D, n->in_D ? N : 0) A("in_F", n->in_F, n->in_F ? N : 0)
    {
        int64_t P = n->queuePost ? S : 0;
        A("queuePost", n->queuePost, P) A("delayIdxPost", n->delayIdxPost, P)
        A("total_delayPost", n->total_delayPost, P) A("ldelayQueuePost", n->ldelayQueuePost, P)
        A("tauspost", n->tauspost, P) A("tauspre", n->tauspre, P) A("taupos", n->taupos, P)
        A("tauneg", n->tauneg, P) A("STDPgap", n->STDPgap, P) A("Wex", n->Wex, P)
        A("Aneg", n->Aneg, P) A("Apos", n->Apos, P) A("mupos", n->mupos, P)
        A("muneg", n->muneg, P) A("useFD", n->useFD, P)
    }
#undef A
    *count = 0; *esz = 0;
    return NULL;
}

uint64_t bgo_get_step(const bgo_net *n) { return n->step; }
void bgo_set_step(bgo_net *n, uint64_t s) { n->step = s; }
int64_t bgo_total_synapses(const bgo_net *n) { return n->total; }
int bgo_flags(const bgo_net *n) { return n->flags; }
void bgo_stdp_signed(bgo_net *n, int on) { n->stdp_signed = on ? 1 : 0; }
void bgo_rng_skip(bgo_net *n, int64_t draws)
{
    for (int64_t k = 0; k < draws; k++) (void)bgo_mt_inrange(&n->rng, 0.0f, 1.0f);
}
void bgo_stdp_params(bgo_net *n, const float *p11)
{
    n->stdp_override = 1;
    memcpy(n->stdp_p, p11, sizeof(n->stdp_p));
}

void bgo_record_noise(bgo_net *n, int64_t cap)
{
    free(n->noise_rec);
    n->noise_rec = malloc((size_t)(cap > 0 ? cap : 1) * sizeof(float));
    n->noise_cap = cap;
    n->noise_n = 0;
}
int64_t bgo_noise_recorded(const bgo_net *n) { return n->noise_n; }

/* ============================== setup ============================== */
/* Layout::initNeuronsLocs, grid branch (Layouts/Layout.cpp:148-158). */
void bgo_layout_grid(bgo_net *n)
{
    for (int i = 0; i < n->N; i++) {
        n->xloc[i] = (float)(i % n->width);
        n->yloc[i] = (float)(i / n->width);
    }
}
/* FixedLayout::generateNeuronTypeMap / initStarterMap (Layouts/FixedLayout.cpp:247-279). */
void bgo_set_types(bgo_net *n, const int *inh, int n_inh, const int *st, int n_st)
{
    for (int i = 0; i < n->N; i++) { n->ntype[i] = BGO_EXC; n->starter[i] = 0; }
    for (int i = 0; i < n_inh; i++) n->ntype[inh[i]] = BGO_INH;
    for (int i = 0; i < n_st; i++) n->starter[st[i]] = 1;
}
/* AllIFNeurons::createAllNeurons / setNeuronDefaults / createNeuron /
 * initNeuronConstsFromParamValues (Neurons/AllIFNeurons.cpp:380-503).  The draws come from the
 * global rng in neuron order: Iinject, Inoise, Vthresh, Vrest, Vreset, Vinit, then for starters
 * Vthresh and Vreset again. */
static void create_if_neuron(bgo_net *n, const float *g, int i);
void bgo_create_lif(bgo_net *n, const float *g)
{
    for (int i = 0; i < n->N; i++) create_if_neuron(n, g, i);
}

/* AllIZHNeurons::setNeuronDefaults / createNeuron / initNeuronConstsFromParamValues: the IF
 * draws first (AllIFNeurons::createNeuron), then a, b, c, d by neuron type, u = 0,
 * C3 = deltaT * 1000. */
void bgo_create_izh(bgo_net *n, const float *g, const float *z)
{
    for (int i = 0; i < n->N; i++) {
        create_if_neuron(n, g, i);
        n->C3[i] = n->delta_t * 1000.0f;
        int inh = n->ntype[i] != BGO_EXC;
        n->Aconst[i] = bgo_mt_inrange(&n->rng, z[0 + 2 * inh], z[1 + 2 * inh]);
        n->Bconst[i] = bgo_mt_inrange(&n->rng, z[4 + 2 * inh], z[5 + 2 * inh]);
        n->Cconst[i] = bgo_mt_inrange(&n->rng, z[8 + 2 * inh], z[9 + 2 * inh]);
        n->Dconst[i] = bgo_mt_inrange(&n->rng, z[12 + 2 * inh], z[13 + 2 * inh]);
        n->u_izh[i] = 0.0f;
    }
}

static void create_if_neuron(bgo_net *n, const float *g, int i)
{
    {
        n->Cm[i] = (float)3e-8;     /* DEFAULT_Cm (Utils/Global.h:103) */
        n->Rm[i] = (float)1e6;      /* DEFAULT_Rm */
        n->Tau[i] = (float)(3e-8 * 1e6);
        n->Iinject[i] = bgo_mt_inrange(&n->rng, g[0], g[1]);
        n->Inoise[i] = bgo_mt_inrange(&n->rng, g[2], g[3]);
        n->Vthresh[i] = bgo_mt_inrange(&n->rng, g[4], g[5]);
        n->Vrest[i] = bgo_mt_inrange(&n->rng, g[6], g[7]);
        n->Vreset[i] = bgo_mt_inrange(&n->rng, g[8], g[9]);
        n->Vinit[i] = bgo_mt_inrange(&n->rng, g[10], g[11]);
        n->Vm[i] = n->Vinit[i];
        float tau = n->Tau[i];
        if (tau > 0) {
            n->C1[i] = expf(-n->delta_t / tau);
            n->C2[i] = n->Rm[i] * (1.0f - n->C1[i]);
        } else {
            n->C1[i] = 0.0f;
            n->C2[i] = n->Rm[i];
        }
        n->I0[i] = n->Iinject[i] + n->Vrest[i] / n->Rm[i];
        /* DEFAULT_InhibTrefract 2.0e-3 / DEFAULT_ExcitTrefract 3.0e-3 (Utils/Global.h:121-123) */
        n->Trefract[i] = (n->ntype[i] == BGO_INH) ? (float)2.0e-3 : (float)3.0e-3;
        if (n->starter[i]) {
            n->Vthresh[i] = bgo_mt_inrange(&n->rng, g[12], g[13]);
            n->Vreset[i] = bgo_mt_inrange(&n->rng, g[14], g[15]);
            n->Trefract[i] = (float)3.0e-3;
        }
    }
}
void bgo_growth_init(bgo_net *n, float eps, float beta, float rho, float tr, float minr, float startr)
{
    n->epsilon = eps; n->beta = beta; n->rho = rho; n->target_rate = tr;
    n->min_radius = minr; n->start_radius = startr;
    n->max_rate = tr / eps; /* Connections/ConnGrowth.cpp:201-203 */
    for (int i = 0; i < n->N; i++) { n->radii[i] = startr; n->rates[i] = 0.0f; }
    /* XmlGrowthRecorder::initDefaultValues: history row 0 holds the start values. */
    for (int i = 0; i < n->N; i++) {
        n->radiiHistory[i] = startr;
        n->ratesHistory[i] = 0.0f;
    }
}
void bgo_seed_noise(bgo_net *n, uint32_t seed) { bgo_norm_init(&n->noise, 0.0f, 1.0f, seed); }

/* AllSpikingSynapses::createSynapse + AllDSSynapses::createSynapse + resets
 * (Synapses/AllSpikingSynapses.cpp:192-240, AllDSSynapses.cpp:160-218). */
static void create_synapse_slot(bgo_net *n, size_t iSyn, int src, int dest, int type)
{
    float tau, delay;
    n->in_use[iSyn] = 1;
    n->dest[iSyn] = dest;
    n->src[iSyn] = src;
    n->W[iSyn] = (float)((double)((type == BGO_II || type == BGO_IE) ? -1 : 1) * 10.0e-9);
    n->type[iSyn] = type;
    switch (type) {
    case BGO_II: tau = (float)6e-3; delay = (float)0.8e-3; break;
    case BGO_IE: tau = (float)6e-3; delay = (float)0.8e-3; break;
    case BGO_EI: tau = (float)3e-3; delay = (float)0.8e-3; break;
    default:     tau = (float)3e-3; delay = (float)1.5e-3; break;
    }
    n->tau[iSyn] = tau;
    n->total_delay[iSyn] = (int)(delay / n->delta_t) + 1;
    n->queue[iSyn] = 0;
    n->delayIdx[iSyn] = 0;
    n->ldelayQueue[iSyn] = LDELAYQUEUE;
    n->psr[iSyn] = 0.0f;
    n->decay[iSyn] = expf(-n->delta_t / tau);
    if (n->syn_kind == BGO_SYN_DS || n->syn_kind == BGO_SYN_DSTDP) {
        n->u[iSyn] = (float)0.4; /* DEFAULT_U */
        n->r[iSyn] = 1.0f;
        n->lastSpike[iSyn] = ULONG_MAX_U64;
        float U, D, F;
        switch (type) {
        case BGO_II: U = (float)0.32; D = (float)0.144; F = (float)0.06; break;
        case BGO_IE: U = (float)0.25; D = (float)0.7; F = (float)0.02; break;
        case BGO_EI: U = (float)0.05; D = (float)0.125; F = (float)1.2; break;
        default:     U = (float)0.5; D = (float)1.1; F = (float)0.05; break;
        }
        n->U[iSyn] = U; n->D[iSyn] = D; n->F[iSyn] = F;
    }
    if (n->queuePost) {
        /* AllSTDPSynapses::initSpikeQueue (:125-138) and createSynapse (:252-273) */
        n->queuePost[iSyn] = 0;
        n->delayIdxPost[iSyn] = 0;
        n->ldelayQueuePost[iSyn] = LDELAYQUEUE;
        n->Apos[iSyn] = (float)0.5;
        n->Aneg[iSyn] = (float)-0.5;
        n->STDPgap[iSyn] = (float)2e-3;
        n->total_delayPost[iSyn] = 0;
        n->tauspost[iSyn] = (float)75e-3;
        n->tauspre[iSyn] = (float)34e-3;
        n->taupos[iSyn] = (float)15e-3;
        n->tauneg[iSyn] = (float)35e-3;
        n->Wex[iSyn] = (float)1.0;
        n->mupos[iSyn] = 0.0f;
        n->muneg[iSyn] = 0.0f;
        n->useFD[iSyn] = 1;
        if (n->stdp_override) {
            const float *p = n->stdp_p;
            n->Apos[iSyn] = p[0]; n->Aneg[iSyn] = p[1]; n->STDPgap[iSyn] = p[2];
            n->tauspost[iSyn] = p[3]; n->tauspre[iSyn] = p[4]; n->taupos[iSyn] = p[5];
            n->tauneg[iSyn] = p[6];
            n->Wex[iSyn] = (type == BGO_II || type == BGO_IE) ? p[8] : p[7];
            n->mupos[iSyn] = p[9]; n->muneg[iSyn] = p[10];
        }
    }
}

/* AllSynapses::addSynapse (Synapses/AllSynapses.cpp:357-377): first free slot of the dest row. */
static long add_synapse(bgo_net *n, int type, int src, int dest)
{
    if (n->counts[dest] >= (uint32_t)n->max_syn) { n->flags |= 1; return -1; }
    size_t iSyn = 0;
    for (int k = 0; k < n->max_syn; k++) {
        iSyn = (size_t)n->max_syn * dest + k;
        if (!n->in_use[iSyn]) break;
    }
    n->counts[dest]++;
    create_synapse_slot(n, iSyn, src, dest, type);
    return (long)iSyn;
}
void bgo_create_synapse(bgo_net *n, int dest, int src, int type, float W)
{
    long iSyn = add_synapse(n, type, src, dest);
    if (iSyn >= 0) n->W[iSyn] = W;
}

/* AllSynapses::createSynapseImap (Synapses/AllSynapses.cpp:223-293).  The reference leaves the
 * previous map in place when there are no synapses; an empty map is equivalent. */
int bgo_rebuild_maps(bgo_net *n)
{
    int N = n->N, M = n->max_syn;
    int64_t total = 0;
    for (int i = 0; i < N; i++) total += n->counts[i];
    int64_t nin = 0;
    for (int i = 0; i < N; i++) n->outCount[i] = 0;
    for (int i = 0; i < N; i++) {
        n->inBegin[i] = (uint32_t)nin;
        uint32_t c = 0;
        for (int j = 0; j < M; j++) {
            size_t s = (size_t)i * M + j;
            if (n->in_use[s]) { n->inMap[nin++] = (uint32_t)s; c++; n->outCount[n->src[s]]++; }
        }
        n->inCount[i] = c;
    }
    /* outgoing: grouped by source, ascending slot order within a source */
    uint32_t acc = 0;
    for (int i = 0; i < N; i++) { n->outBegin[i] = acc; acc += n->outCount[i]; }
    uint32_t *fill = calloc(N > 0 ? (size_t)N : 1u, sizeof(uint32_t));
    for (int64_t q = 0; q < nin; q++) {
        uint32_t s = n->inMap[q];
        int sr = n->src[s];
        n->outMap[n->outBegin[sr] + fill[sr]++] = s;
    }
    free(fill);
    n->total = nin;
    return (nin == total) ? 0 : -1;
}

/* ============================== inputs ============================== */
/* SInputRegular::SInputRegular (Inputs/SInputRegular.cpp:20-112): step counts, the 10x10 value
 * pattern tiled over the grid, and per-neuron phase shifts. */
int bgo_input_regular(bgo_net *n, float duration, float interval, int sync, const float *v100)
{
    n->input_kind = 1;
    n->reg_dur = (int)((double)(duration / n->delta_t) + 0.5);
    int nint = (int)((double)(interval / n->delta_t) + 0.5);
    n->reg_cycle = n->reg_dur + nint;
    n->reg_in_cycle = 0;
    ALLOC(n->reg_values, n->N);
    ALLOC(n->reg_shift, n->N);
    for (int i = 0; i < n->height; i++)
        for (int j = 0; j < n->width; j++)
            n->reg_values[i * n->width + j] = v100[(i % 10) * 10 + j % 10];
    if (sync == 1) {
        for (int i = 0; i < n->height; i++)
            for (int j = 0; j < n->width; j++)
                n->reg_shift[i * n->width + j] =
                    (int)bgo_mt_inrange(&n->rng, 0.0f, (float)(n->reg_cycle - 1));
    } else if (sync == 2) {
        for (int i = 0; i < n->height; i++)
            for (int j = 0; j < n->width; j++)
                n->reg_shift[i * n->width + j] = (n->reg_cycle / n->width) * j;
    }
    return 0;
}

/* SInputPoisson::SInputPoisson / init (Inputs/SInputPoisson.cpp:19-146): lambda, masks, and one
 * DS input synapse per neuron (type EI onto inhibitory, EE onto excitatory neurons), created at
 * the current step with W = weight x 1e-8.  The reference indexes its one-slot-per-neuron
 * synapse object with maxSynapsesPerNeuron * neuron (SInputPoisson.cpp:141,
 * HostSInputPoisson.cpp:77), out of bounds whenever maxSynapsesPerNeuron > 1; slot = neuron here
 * (and in the reference harness that pins this code). */
int bgo_input_poisson(bgo_net *n, float fr_mean, float weight, const uint8_t *masks)
{
    int N = n->N;
    n->input_kind = 2;
    fr_mean = fr_mean / 1000.0f;
    n->pois_lambda = 1.0f / fr_mean;
    ALLOC(n->pois_mask, N); ALLOC(n->pois_nisi, N);
    ALLOC(n->in_W, N); ALLOC(n->in_psr, N); ALLOC(n->in_decay, N); ALLOC(n->in_U, N);
    ALLOC(n->in_D, N); ALLOC(n->in_F, N); ALLOC(n->in_u, N); ALLOC(n->in_r, N);
    ALLOC(n->in_delay, N); ALLOC(n->in_delayIdx, N); ALLOC(n->in_queue, N); ALLOC(n->in_last, N);
    for (int i = 0; i < N; i++) {
        n->pois_mask[i] = masks ? masks[i] : 1;
        int type = (n->ntype[i] == BGO_INH) ? BGO_EI : BGO_EE;
        float tau = (float)3e-3, delay = (type == BGO_EE) ? (float)1.5e-3 : (float)0.8e-3;
        n->in_delay[i] = (int)(delay / n->delta_t) + 1;
        n->in_queue[i] = 0;
        n->in_delayIdx[i] = 0;
        n->in_psr[i] = 0.0f;
        n->in_decay[i] = expf(-n->delta_t / tau);
        n->in_u[i] = (float)0.4;
        n->in_r[i] = 1.0f;
        n->in_last[i] = ULONG_MAX_U64;
        n->in_U[i] = (type == BGO_EE) ? (float)0.5 : (float)0.05;
        n->in_D[i] = (type == BGO_EE) ? (float)1.1 : (float)0.125;
        n->in_F[i] = (type == BGO_EE) ? (float)0.05 : (float)1.2;
        n->in_W[i] = weight * (float)1.0e-8;
    }
    return 0;
}

/* One ISI draw (HostSInputPoisson.cpp:81-84): exponential with mean lambda ms, rejection
 * U <= exp(-isi^2 / 32), converted to steps. */
static int poisson_draw(bgo_mt *rng, float lambda, float dt)
{
    float isi = -lambda * logf(bgo_mt_inrange(rng, 0.0f, 1.0f));
    while (bgo_mt_inrange(rng, 0.0f, 1.0f) <= expf(-(isi * isi) / 32.0f))
        isi = -lambda * logf(bgo_mt_inrange(rng, 0.0f, 1.0f));
    return (int)((double)((isi / 1000.0f) / dt) + 0.5);
}

/* HostSInputRegular::inputStimulus (Inputs/HostSInputRegular.cpp:59-80). */
static void input_regular(bgo_net *n)
{
    for (int i = n->N - 1; i >= 0; --i)
        if (n->reg_in_cycle >= n->reg_shift[i] &&
            n->reg_in_cycle < (n->reg_shift[i] + n->reg_dur) % n->reg_cycle)
            n->sp[i] += n->reg_values[i];
    n->reg_in_cycle = (n->reg_in_cycle + 1) % n->reg_cycle;
}

/* HostSInputPoisson::inputStimulus (Inputs/HostSInputPoisson.cpp:60-94): counter expiry fires
 * the input synapse and draws the next ISI; the synapse then advances like any DS synapse. */
static void input_poisson(bgo_net *n)
{
    for (int i = 0; i < n->N; i++) {
        if (!n->pois_mask[i]) continue;
        if (--n->pois_nisi[i] <= 0) {
            int idx = n->in_delayIdx[i] + n->in_delay[i];
            if (idx >= LDELAYQUEUE) idx -= LDELAYQUEUE;
            n->in_queue[i] |= (1u << idx);
            n->pois_nisi[i] = poisson_draw(&n->rng, n->pois_lambda, n->delta_t);
        }
        uint32_t bit = 1u << n->in_delayIdx[i];
        int hit = (n->in_queue[i] & bit) != 0;
        n->in_queue[i] &= ~bit;
        if (++n->in_delayIdx[i] >= LDELAYQUEUE) n->in_delayIdx[i] = 0;
        if (hit) {
            if (n->in_last[i] != ULONG_MAX_U64) {
                float isi = (float)(n->step - n->in_last[i]) * n->delta_t;
                n->in_r[i] = 1.0f + (n->in_r[i] * (1.0f - n->in_u[i]) - 1.0f) * expf(-isi / n->in_D[i]);
                n->in_u[i] = n->in_U[i] + n->in_u[i] * (1.0f - n->in_U[i]) * expf(-isi / n->in_F[i]);
            }
            n->in_psr[i] += ((n->in_W[i] / n->in_decay[i]) * n->in_u[i] * n->in_r[i]);
            n->in_last[i] = n->step;
        }
        n->in_psr[i] *= n->in_decay[i];
        n->sp[i] += n->in_psr[i];
    }
}

int64_t bgo_poisson_isi_draws(bgo_net *n, int nsteps, int32_t *begin, int32_t *out, int64_t cap)
{
    if (n->input_kind != 2) return -1;
    /* replay the counters on copies: per neuron, draws happen in step order, neurons ascending
     * within a step; the rng is copied so the real run is unaffected */
    bgo_mt rng = n->rng;
    int N = n->N;
    int *cnt = calloc((size_t)N, sizeof(int));
    int *nisi = malloc((size_t)N * sizeof(int));
    memcpy(nisi, n->pois_nisi, (size_t)N * sizeof(int));
    /* first pass: count draws per neuron, recording them in step order into a temp buffer */
    int64_t total = 0, tcap = 1024;
    int32_t *tn = malloc((size_t)tcap * sizeof(int32_t)), *tv = malloc((size_t)tcap * sizeof(int32_t));
    for (int t = 0; t < nsteps; t++)
        for (int i = 0; i < N; i++) {
            if (!n->pois_mask[i]) continue;
            if (--nisi[i] <= 0) {
                int v = poisson_draw(&rng, n->pois_lambda, n->delta_t);
                nisi[i] = v;
                if (total == tcap) {
                    tcap *= 2;
                    tn = realloc(tn, (size_t)tcap * sizeof(int32_t));
                    tv = realloc(tv, (size_t)tcap * sizeof(int32_t));
                }
                tn[total] = i;
                tv[total] = v;
                total++;
                cnt[i]++;
            }
        }
    int64_t rc = total;
    if (total > cap) rc = -1;
    else {
        begin[0] = 0;
        for (int i = 0; i < N; i++) begin[i + 1] = begin[i] + cnt[i];
        memset(cnt, 0, (size_t)N * sizeof(int));
        for (int64_t k = 0; k < total; k++) out[begin[tn[k]] + cnt[tn[k]]++] = tv[k];
    }
    free(cnt); free(nisi); free(tn); free(tv);
    return rc;
}

/* ============================== step ============================== */
/* AllSpikingNeurons::fire (Neurons/AllSpikingNeurons.cpp:155-172) + AllLIFNeurons::fire
 * (Neurons/AllLIFNeurons.cpp:67-77). */
static void lif_fire(bgo_net *n, int i)
{
    n->hasFired[i] = 1;
    int idxSp = (n->spikeCount[i] + n->spikeCountOffset[i]) % n->max_spikes;
    n->history[(size_t)i * n->max_spikes + idxSp] = n->step;
    n->spikeCount[i]++;
    n->refr[i] = (int)((double)(n->Trefract[i] / n->delta_t) + 0.5);
    n->Vm[i] = n->Vreset[i];
}

/* AllLIFNeurons::advanceNeuron (Neurons/AllLIFNeurons.cpp:20-59). */
static void lif_advance(bgo_net *n, int i)
{
    if (n->refr[i] > 0) {
        --n->refr[i];
    } else if (n->Vm[i] >= n->Vthresh[i]) {
        lif_fire(n, i);
    } else {
        n->sp[i] += n->I0[i];
        float noise = bgo_norm_next(&n->noise);
        if (n->noise_rec && n->noise_n < n->noise_cap) n->noise_rec[n->noise_n++] = noise;
        n->sp[i] += noise * n->Inoise[i];
        n->Vm[i] = n->C1[i] * n->Vm[i] + n->C2[i] * n->sp[i];
    }
    n->sp[i] = 0.0f;
}

/* AllSpikingSynapses::preSpikeHit (Synapses/AllSpikingSynapses.cpp:261-279). */
static void post_spike_hit(bgo_net *n, size_t s);
static void pre_spike_hit(bgo_net *n, uint32_t s)
{
    int idx = n->delayIdx[s] + n->total_delay[s];
    if (idx >= n->ldelayQueue[s]) idx -= n->ldelayQueue[s];
    n->queue[s] |= (1u << idx);
}

/* AllIZHNeurons::advanceNeuron / fire (Neurons/AllIZHNeurons.cpp:570-655): the Euler step in
 * mV with the reference's double literals (0.04, 0.001) promoting parts of it to double. */
static void izh_advance(bgo_net *n, int i)
{
    if (n->refr[i] > 0) {
        --n->refr[i];
    } else if (n->Vm[i] >= n->Vthresh[i]) {
        n->hasFired[i] = 1;
        int idxSp = (n->spikeCount[i] + n->spikeCountOffset[i]) % n->max_spikes;
        n->history[(size_t)i * n->max_spikes + idxSp] = n->step;
        n->spikeCount[i]++;
        n->refr[i] = (int)((double)(n->Trefract[i] / n->delta_t) + 0.5);
        n->Vm[i] = (float)((double)n->Cconst[i] * 0.001);
        n->u_izh[i] = n->u_izh[i] + n->Dconst[i];
    } else {
        n->sp[i] += n->I0[i];
        float noise = bgo_norm_next(&n->noise);
        if (n->noise_rec && n->noise_n < n->noise_cap) n->noise_rec[n->noise_n++] = noise;
        n->sp[i] += noise * n->Inoise[i];
        float Vint = n->Vm[i] * 1000.0f;
        float u = n->u_izh[i], C3 = n->C3[i];
        float Vb = (float)((double)Vint +
                           (double)C3 * (0.04 * (double)Vint * (double)Vint + (double)(5.0f * Vint) +
                                         140.0 - (double)u));
        n->u_izh[i] = u + C3 * n->Aconst[i] * (n->Bconst[i] * Vint - u);
        n->Vm[i] = (float)((double)Vb * 0.001 + (double)(n->C2[i] * n->sp[i]));
    }
    n->sp[i] = 0.0f;
}

/* AllSpikingNeurons::advanceNeurons (Neurons/AllSpikingNeurons.cpp:98-147): descending index. */
static void advance_neurons(bgo_net *n)
{
    for (int i = n->N - 1; i >= 0; --i) {
        if (n->neuron_kind == BGO_IZH) izh_advance(n, i);
        else lif_advance(n, i);
        if (n->hasFired[i]) {
            if (n->total > 0) {
                uint32_t c = n->outCount[i], b = n->outBegin[i];
                for (uint32_t k = 0; k < c; k++) pre_spike_hit(n, n->outMap[b + k]);
            }
            if (n->queuePost) {
                /* back propagation to the in-use incoming synapses (:128-138) */
                uint32_t notified = 0;
                for (int z = 0; notified < n->counts[i]; z++) {
                    size_t s = (size_t)n->max_syn * i + z;
                    if (n->in_use[s]) { post_spike_hit(n, s); notified++; }
                }
            }
            n->hasFired[i] = 0;
        }
    }
}

/* AllDSSynapses::changePSR (Synapses/AllDSSynapses.cpp:227-247). */
static void ds_change_psr(bgo_net *n, size_t s)
{
    if (n->lastSpike[s] != ULONG_MAX_U64) {
        float isi = (float)(n->step - n->lastSpike[s]) * n->delta_t;
        n->r[s] = 1.0f + (n->r[s] * (1.0f - n->u[s]) - 1.0f) * expf(-isi / n->D[s]);
        n->u[s] = n->U[s] + n->u[s] * (1.0f - n->U[s]) * expf(-isi / n->F[s]);
    }
    n->psr[s] += ((n->W[s] / n->decay[s]) * n->u[s] * n->r[s]);
    n->lastSpike[s] = n->step;
}

/* ---- STDP (Synapses/AllSTDPSynapses.cpp:283-517, device form AllSynapsesDeviceFuncs_d.cu:100-380).
 * The host build keeps spike times as uint64_t, so (spikeHistory - step) in the pre-spike walk
 * wraps to a huge positive interval and that walk only applies the sign and |Wex| clamps; the
 * device build holds them in int64_t and depresses.  stdp_signed selects the device form.  A
 * history walk that would pass the oldest entry of a full ring (where the host build reads
 * outside the ring) stops there and raises flag 4. */

/* AllSpikingNeurons::getSpikeHistory (Neurons/AllSpikingNeurons.cpp:182-188); returns 0 when the
 * ring index would be negative. */
static int spike_history(const bgo_net *n, int idx, int off, uint64_t *out)
{
    int x = n->spikeCount[idx] + n->spikeCountOffset[idx] + n->max_spikes + off;
    if (x < 0) return 0;
    *out = n->history[(size_t)idx * n->max_spikes + x % n->max_spikes];
    return 1;
}

/* AllSTDPSynapses::stdpLearning (:432-472) */
static void stdp_learning(bgo_net *n, size_t s, double delta, double epost, double epre)
{
    float gap = n->STDPgap[s], Wex = n->Wex[s];
    float W = n->W[s];
    float dw;
    if (delta < -gap)
        dw = (float)((double)(powf(W, n->muneg[s]) * n->Aneg[s]) * exp(delta / n->tauneg[s]));
    else if (delta > gap)
        dw = (float)((double)(powf(Wex - W, n->mupos[s]) * n->Apos[s]) * exp(-delta / n->taupos[s]));
    else
        return;
    W = (float)((double)W + epost * epre * dw);
    if ((Wex < 0 && W > 0) || (Wex > 0 && W < 0)) W = 0;
    if (fabsf(W) > fabsf(Wex)) W = Wex;
    n->W[s] = W;
}

/* Interval in seconds between spike times a - b as the chosen build computes it. */
static float stdp_interval(const bgo_net *n, uint64_t a, uint64_t b)
{
    if (n->stdp_signed) return (float)(int64_t)(a - b) * n->delta_t;
    return (float)(a - b) * n->delta_t;
}

static void stdp_pre(bgo_net *n, size_t s)
{
    int pre = n->src[s], post = n->dest[s];
    uint64_t sh, sh2;
    float delta, epre, epost;
    int have = spike_history(n, pre, -2, &sh);
    int ok = have && (n->stdp_signed ? ((int64_t)sh > 0) : (sh != ULONG_MAX_U64));
    if (ok && n->useFD[s]) {
        delta = stdp_interval(n, n->step, sh);
        epre = (float)(1.0 - (double)expf(-delta / n->tauspre[s]));
    } else {
        epre = 1.0f;
    }
    for (int off = -1;; --off) {
        if (off < -n->max_spikes || !spike_history(n, post, off, &sh)) { n->flags |= 4; break; }
        if (sh == ULONG_MAX_U64) break;
        delta = stdp_interval(n, sh, n->step);
        if ((double)delta <= -3.0 * (double)n->tauneg[s]) break;
        if (n->useFD[s]) {
            if (off - 1 < -n->max_spikes || !spike_history(n, post, off - 1, &sh2)) {
                n->flags |= 4;
                break;
            }
            if (sh2 == ULONG_MAX_U64) break;
            epost = (float)(1.0 - (double)expf(-stdp_interval(n, sh, sh2) / n->tauspost[s]));
        } else {
            epost = 1.0f;
        }
        stdp_learning(n, s, delta, epost, epre);
    }
}

static void stdp_post(bgo_net *n, size_t s)
{
    int pre = n->src[s], post = n->dest[s];
    uint64_t sh, sh2;
    float delta, epre, epost;
    int have = spike_history(n, post, -2, &sh);
    int ok = have && (n->stdp_signed ? ((int64_t)sh > 0) : (sh != ULONG_MAX_U64));
    if (ok && n->useFD[s]) {
        delta = stdp_interval(n, n->step, sh);
        epost = (float)(1.0 - (double)expf(-delta / n->tauspost[s]));
    } else {
        epost = 1.0f;
    }
    for (int off = -1;; --off) {
        if (off < -n->max_spikes || !spike_history(n, pre, off, &sh)) { n->flags |= 4; break; }
        if (sh == ULONG_MAX_U64) break;
        /* ((int64_t)step - spikeHistory - total_delay) */
        delta = stdp_interval(n, n->step - (uint64_t)(int64_t)n->total_delay[s], sh);
        if (delta <= 0 || (double)delta >= 3.0 * (double)n->taupos[s]) break;
        if (n->useFD[s]) {
            if (off - 1 < -n->max_spikes || !spike_history(n, pre, off - 1, &sh2)) {
                n->flags |= 4;
                break;
            }
            if (sh2 == ULONG_MAX_U64) break;
            epre = (float)(1.0 - (double)expf(-stdp_interval(n, sh, sh2) / n->tauspre[s]));
        } else {
            epre = 1.0f;
        }
        stdp_learning(n, s, delta, epost, epre);
    }
}

/* AllSTDPSynapses::postSpikeHit (:499-517) */
static void post_spike_hit(bgo_net *n, size_t s)
{
    int idx = n->delayIdxPost[s] + n->total_delayPost[s];
    if (idx >= n->ldelayQueuePost[s]) idx -= n->ldelayQueuePost[s];
    if (n->queuePost[s] & (1u << idx)) n->flags |= 8;
    n->queuePost[s] |= (1u << idx);
}

/* AllSynapses::advanceSynapses (Synapses/AllSynapses.cpp:325-331) over the incoming map, with
 * AllSpikingSynapses::advanceSynapse / isSpikeQueue (AllSpikingSynapses.cpp:242-319) and, for
 * the STDP kinds, AllSTDPSynapses::advanceSynapse / isSpikeQueuePost (:283-421, :480-492). */
static void advance_synapses(bgo_net *n)
{
    const int stdp = n->queuePost != NULL;
    const int ds = n->syn_kind == BGO_SYN_DS || n->syn_kind == BGO_SYN_DSTDP;
    for (int64_t q = 0; q < n->total; q++) {
        uint32_t s = n->inMap[q];
        uint32_t bit = 1u << n->delayIdx[s];
        int hit = (n->queue[s] & bit) != 0;
        n->queue[s] &= ~bit;
        if (++n->delayIdx[s] >= n->ldelayQueue[s]) n->delayIdx[s] = 0;
        int post = 0;
        if (stdp) {
            uint32_t pb = 1u << n->delayIdxPost[s];
            post = (n->queuePost[s] & pb) != 0;
            n->queuePost[s] &= ~pb;
            if (++n->delayIdxPost[s] >= n->ldelayQueuePost[s]) n->delayIdxPost[s] = 0;
        }
        if (hit) {
            if (stdp) stdp_pre(n, s);
            if (ds)
                ds_change_psr(n, s);
            else
                n->psr[s] += (n->W[s] / n->decay[s]); /* AllSpikingSynapses::changePSR :327-334 */
        }
        if (post) stdp_post(n, s);
        n->psr[s] *= n->decay[s];
        n->sp[n->dest[s]] += n->psr[s];
    }
}

void bgo_step(bgo_net *n, int nsteps)
{
    for (int t = 0; t < nsteps; t++) {
        /* Simulator::advanceUntilGrowth: inputStimulus, then advance (Core/Simulator.cpp:178-182) */
        if (n->input_kind == 1) input_regular(n);
        else if (n->input_kind == 2) input_poisson(n);
        advance_neurons(n);
        advance_synapses(n);
        n->step++;
    }
}

/* ============================== growth ============================== */
/* ConnGrowth::updateConns (Connections/ConnGrowth.cpp:295-311). */
static void update_conns(bgo_net *n)
{
    float T = n->epoch_duration;
    float trho = n->epoch_duration * n->rho;
    for (int i = 0; i < n->N; i++) {
        n->rates[i] = (float)n->spikeCount[i] / T;
        float e = expf((n->epsilon - n->rates[i] / n->max_rate) / n->beta);
        float og = 1.0f - 2.0f / (e + 1.0f);
        n->radii[i] += trho * og;
    }
}

/* Per-pair frontier distance and overlap area (ConnGrowth.cpp:319-376) for (i = src, j = dest). */
static float pair_area(const bgo_net *n, int i, int j)
{
    if (i == j) return 0.0f;
    float dx = n->xloc[i] - n->xloc[j], dy = n->yloc[i] - n->yloc[j];
    float lenAB2 = dx * dx + dy * dy;
    float lenAB = sqrtf(lenAB2);
    float r1 = n->radii[i], r2 = n->radii[j];
    float delta = lenAB - (r1 + r2);
    if (!(delta < 0)) return 0.0f;
    float rmin = r1 < r2 ? r1 : r2, rmax = r1 < r2 ? r2 : r1;
    if (lenAB + rmin <= rmax) {
        const float pi = (float)3.1415926536; /* Utils/Global.cpp:90 */
        return pi * rmin * rmin;
    }
    float r12 = r1 * r1, r22 = r2 * r2;
    float cosCBA = (float)((double)(r22 + lenAB2 - r12) / (2.0 * (double)r2 * (double)lenAB));
    float angCBA = acosf(cosCBA);
    float angCBD = (float)(2.0 * (double)angCBA);
    float cosCAB = (float)((double)(r12 + lenAB2 - r22) / (2.0 * (double)r1 * (double)lenAB));
    float angCAB = acosf(cosCAB);
    float angCAD = (float)(2.0 * (double)angCAB);
    return (float)(0.5 * (double)(r22 * (angCBD - sinf(angCBD)) + r12 * (angCAD - sinf(angCAD))));
}

static int syn_type(const bgo_net *n, int src, int dest)
{
    int si = n->ntype[src] == BGO_INH, di = n->ntype[dest] == BGO_INH;
    return si ? (di ? BGO_II : BGO_IE) : (di ? BGO_EI : BGO_EE);
}

/* ConnGrowth::updateSynapsesWeights, CPU variant (Connections/ConnGrowth.cpp:388-463).
 * The reference walks src (outer) x dest (inner) and, for each pair, scans the dest row for a
 * synapse from src.  Every action on a pair touches only the dest row, so walking dest (outer) x
 * src (inner, ascending) performs the same actions in the same per-row order; a src -> slot table
 * of the row replaces the row scan (rows hold at most one synapse per source). */
static void update_weights(bgo_net *n)
{
    const float adj = (float)1.0e-8; /* AllSynapses::SYNAPSE_STRENGTH_ADJUSTMENT */
    long *slot_of = malloc((size_t)(n->N > 0 ? n->N : 1) * sizeof(long));
    for (int s = 0; s < n->N; s++) slot_of[s] = -1;
    for (int d = 0; d < n->N; d++) {
        uint32_t cnt = n->counts[d], seen = 0;
        for (size_t iSyn = (size_t)n->max_syn * d; seen < cnt; iSyn++)
            if (n->in_use[iSyn]) { slot_of[n->src[iSyn]] = (long)iSyn; seen++; }
        for (int s = 0; s < n->N; s++) {
            float w = pair_area(n, s, d);
            int type = syn_type(n, s, d);
            int sign = (type == BGO_II || type == BGO_IE) ? -1 : 1;
            long iSyn = slot_of[s];
            if (iSyn >= 0) {
                if (w < 0) {
                    n->counts[d]--;
                    n->in_use[iSyn] = 0;
                } else {
                    n->W[iSyn] = w * (float)sign * adj;
                }
            } else if (w > 0) {
                long k = add_synapse(n, type, s, d);
                if (k >= 0) n->W[k] = w * (float)sign * adj;
            }
        }
        for (size_t iSyn = (size_t)n->max_syn * d; iSyn < (size_t)n->max_syn * (d + 1); iSyn++)
            if (n->src[iSyn] >= 0 && n->src[iSyn] < n->N) slot_of[n->src[iSyn]] = -1;
    }
    free(slot_of);
}

void bgo_growth(bgo_net *n)
{
    update_conns(n);
    update_weights(n);
    bgo_rebuild_maps(n);
}

/* XmlRecorder::compileHistories (Recorders/XmlRecorder.cpp:71-104) followed by the growth part
 * (Recorders/XmlGrowthRecorder.cpp:72-97: rates/radii history, radius clamp) and
 * AllSpikingNeurons::clearSpikeCounts (Neurons/AllSpikingNeurons.cpp:77-86). */
static void record_spikes(bgo_net *n);
void bgo_record_epoch(bgo_net *n, int epoch)
{
    record_spikes(n);
    for (int i = 0; i < n->N; i++) {
        n->ratesHistory[(size_t)epoch * n->N + i] = n->rates[i];
        if (n->radii[i] < n->min_radius) n->radii[i] = n->min_radius;
        n->radiiHistory[(size_t)epoch * n->N + i] = n->radii[i];
    }
    for (int i = 0; i < n->N; i++) {
        n->spikeCountOffset[i] = (n->spikeCount[i] + n->spikeCountOffset[i]) % n->max_spikes;
        n->spikeCount[i] = 0;
    }
}

/* XmlRecorder::compileHistories alone (Recorders/XmlRecorder.cpp:71-104): the recorder of a
 * network without growth (ConnStatic). */
void bgo_record_static(bgo_net *n)
{
    record_spikes(n);
    for (int i = 0; i < n->N; i++) {
        n->spikeCountOffset[i] = (n->spikeCount[i] + n->spikeCountOffset[i]) % n->max_spikes;
        n->spikeCount[i] = 0;
    }
}

static void record_spikes(bgo_net *n)
{
    int ms = n->max_spikes;
    for (int i = 0; i < n->N; i++) {
        const uint64_t *h = n->history + (size_t)i * ms;
        for (int k = 0, idx = n->spikeCountOffset[i]; k < n->spikeCount[i]; k++, idx++) {
            if (idx >= ms) idx = 0;
            int b1 = (int)((double)h[idx] * (double)n->delta_t);
            n->burstinessHist[b1] = n->burstinessHist[b1] + 1.0f;
            int b2 = (int)((double)h[idx] * (double)n->delta_t * 100);
            n->spikesHistory[b2] = n->spikesHistory[b2] + 1.0f;
        }
    }
}

/* ---- checkpoint stream ----------------------------------------------------------------------
 * Model::serialize (Core/Model.cpp:85-98) prints each value with std::ostream's defaults (a float
 * is printed as the double it converts to, "%.6g"; integers in decimal; bool as 0/1; the synapse
 * type enum as its int value) and ends it with `ends` (a NUL). */
typedef struct {
    char *buf;
    int64_t cap, len;
} ser_out;

static void ser_put(ser_out *o, const char *txt)
{
    const int64_t k = (int64_t)strlen(txt) + 1; /* with the NUL */
    if (o->buf && o->len + k <= o->cap) memcpy(o->buf + o->len, txt, (size_t)k);
    o->len += k;
}
static void ser_f(ser_out *o, float v)
{
    char t[64];
    snprintf(t, sizeof t, "%.*g", 6, (double)v);
    ser_put(o, t);
}
static void ser_i(ser_out *o, long long v)
{
    char t[32];
    snprintf(t, sizeof t, "%lld", v);
    ser_put(o, t);
}
static void ser_u(ser_out *o, unsigned long long v)
{
    char t[32];
    snprintf(t, sizeof t, "%llu", v);
    ser_put(o, t);
}

int64_t bgo_serialize(const bgo_net *n, int conn_growth, char *buf, int64_t cap)
{
    ser_out o = {buf, cap, 0};
    const int N = n->N;
    ser_i(&o, N); /* Model::serialize: totalNeurons */
    for (int i = 0; i < N; i++) {
        /* AllIFNeurons::writeNeuron (Neurons/AllIFNeurons.cpp:594-613) */
        ser_f(&o, n->Cm[i]); ser_f(&o, n->Rm[i]); ser_f(&o, n->Vthresh[i]); ser_f(&o, n->Vrest[i]);
        ser_f(&o, n->Vreset[i]); ser_f(&o, n->Vinit[i]); ser_f(&o, n->Trefract[i]);
        ser_f(&o, n->Inoise[i]); ser_f(&o, n->Iinject[i]); ser_f(&o, 0.0f /* Isyn */);
        ser_i(&o, n->refr[i]); ser_f(&o, n->C1[i]); ser_f(&o, n->C2[i]); ser_f(&o, n->I0[i]);
        ser_f(&o, n->Vm[i]); ser_i(&o, n->hasFired[i] ? 1 : 0); ser_f(&o, n->Tau[i]);
        if (n->neuron_kind == 1) {
            /* AllIZHNeurons::writeNeuron (Neurons/AllIZHNeurons.cpp:551-561) */
            ser_f(&o, n->Aconst[i]); ser_f(&o, n->Bconst[i]); ser_f(&o, n->Cconst[i]);
            ser_f(&o, n->Dconst[i]); ser_f(&o, n->u_izh[i]); ser_f(&o, n->C3[i]);
        }
    }
    /* AllSynapses::serialize (Synapses/AllSynapses.cpp:163-177): dest rows in order, the first
     * synapse_counts[dest] slots of each */
    long long total = 0;
    for (int d = 0; d < N; d++) total += n->counts[d];
    ser_i(&o, total);
    const int dyn = n->syn_kind == 1 || n->syn_kind == 3, stdp = n->syn_kind >= 2;
    for (int d = 0; d < N; d++)
        for (uint32_t k = 0; k < n->counts[d]; k++) {
            const size_t s = (size_t)d * (size_t)n->max_syn + k;
            /* AllSynapses::writeSynapse (:207-215) */
            ser_i(&o, n->src[s]); ser_i(&o, n->dest[s]); ser_f(&o, n->W[s]); ser_f(&o, n->psr[s]);
            ser_i(&o, n->type[s]); ser_i(&o, n->in_use[s] ? 1 : 0);
            /* AllSpikingSynapses::writeSynapse (Synapses/AllSpikingSynapses.cpp:168-178) */
            ser_f(&o, n->decay[s]); ser_i(&o, n->total_delay[s]); ser_u(&o, n->queue[s]);
            ser_i(&o, n->delayIdx[s]); ser_i(&o, n->ldelayQueue[s]); ser_f(&o, n->tau[s]);
            if (stdp) {
                /* AllSTDPSynapses::writeSynapse (Synapses/AllSTDPSynapses.cpp:209-228) */
                ser_i(&o, n->total_delayPost[s]); ser_u(&o, n->queuePost[s]);
                ser_i(&o, n->delayIdxPost[s]); ser_i(&o, n->ldelayQueuePost[s]);
                ser_f(&o, n->tauspost[s]); ser_f(&o, n->tauspre[s]); ser_f(&o, n->taupos[s]);
                ser_f(&o, n->tauneg[s]); ser_f(&o, n->STDPgap[s]); ser_f(&o, n->Wex[s]);
                ser_f(&o, n->Aneg[s]); ser_f(&o, n->Apos[s]); ser_f(&o, n->mupos[s]);
                ser_f(&o, n->muneg[s]); ser_i(&o, n->useFD[s] ? 1 : 0);
            }
            if (dyn) {
                /* AllDSSynapses::writeSynapse (Synapses/AllDSSynapses.cpp:142-152),
                 * AllDynamicSTDPSynapses::writeSynapse (AllDynamicSTDPSynapses.cpp:142-152) */
                ser_u(&o, n->lastSpike[s]); ser_f(&o, n->r[s]); ser_f(&o, n->u[s]);
                ser_f(&o, n->D[s]); ser_f(&o, n->U[s]); ser_f(&o, n->F[s]);
            }
        }
    if (conn_growth) {
        /* ConnGrowth::serialize (Connections/ConnGrowth.cpp:254-265) */
        for (int i = 0; i < N; i++) ser_f(&o, n->radii[i]);
        for (int i = 0; i < N; i++) ser_f(&o, n->rates[i]);
    }
    return o.len;
}
