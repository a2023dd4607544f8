/* CPU oracle for the BrainGrid per-step spiking hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's single-threaded
 * simulator (Core/SingleThreadedSpikingModel.cpp and the Neurons/Synapses/Connections/Recorders
 * classes it drives), used as the checker for the CUDA path.  Only tests/, the smoke check and
 * the CPU-baseline leg of bench.py load it; the product library never does.
 *
 * Parity pin: the restatement is checked bit-for-bit against the compiled reference (built from
 * the reference sources by oracle/ref.mk and dumped step by step by oracle/ref_harness.cpp) through
 * the fixtures in tests/golden/, which were generated by tests/golden/make_golden.py.
 *
 * Build (x86 or Arm):  cc -O2 -ffp-contract=off -fPIC -shared bg_oracle.c -lm
 * -ffp-contract=off is required: the reference is compiled by g++ -O2 on x86-64, which never
 * fuses a*b+c, while gcc on aarch64 fuses by default.
 */
#ifndef BG_ORACLE_H
#define BG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RNG: MT19937 as in RNG/MersenneTwister.{h,cpp}; Marsaglia polar normal as RNG/Norm.cpp ---- */
typedef struct { uint32_t s[624]; int left; int next; } bgo_mt;
void bgo_mt_seed(bgo_mt *m, uint32_t seed);
uint32_t bgo_mt_randint(bgo_mt *m);
float bgo_mt_rand(bgo_mt *m);                       /* MTRand::rand, [0,1]   */
float bgo_mt_inrange(bgo_mt *m, float lo, float hi); /* MTRand::inRange       */
typedef struct { bgo_mt mt; int odd; float mu, sigma, x2; } bgo_norm;
void bgo_norm_init(bgo_norm *n, float mu, float sigma, uint32_t seed);
float bgo_norm_next(bgo_norm *n);
/* Fill out[0..n) with the next n values of a fresh Norm(0,1,seed) stream. */
void bgo_norm_fill(uint32_t seed, float *out, int64_t n);

/* ---- network ---- */
enum { BGO_LIF = 0, BGO_IZH = 1 };
enum { BGO_SYN_SPIKING = 0, BGO_SYN_DS = 1, BGO_SYN_STDP = 2, BGO_SYN_DSTDP = 3 };
enum { BGO_INH = 1, BGO_EXC = 2 };                    /* Utils/Global.h:93 */
enum { BGO_II = 0, BGO_IE = 1, BGO_EI = 2, BGO_EE = 3 };/* Utils/Global.h:100 */

typedef struct bgo_net bgo_net;

bgo_net *bgo_create(int N, int max_syn, int width, int height, float epoch_duration,
                    float delta_t, int max_firing_rate, int max_epochs, int neuron_kind,
                    int synapse_kind);
void bgo_destroy(bgo_net *n);

/* Named array access (pointer to the live array, element count in *count). */
void *bgo_array(bgo_net *n, const char *name, int64_t *count, int *elem_size);
/* Scalars: step, total synapse count, epochs done. */
uint64_t bgo_get_step(const bgo_net *n);
void bgo_set_step(bgo_net *n, uint64_t step);
int64_t bgo_total_synapses(const bgo_net *n);

/* Setup (Model::setupSim order, Core/Model.cpp:136-160). */
void bgo_layout_grid(bgo_net *n);
void bgo_set_types(bgo_net *n, const int *inh, int n_inh, const int *starters, int n_starters);
/* LIF ranges, in order: Iinject, Inoise, Vthresh, Vresting, Vreset, Vinit, starter_Vthresh,
 * starter_Vreset — each as (min, max): 16 floats.  Draws from the global rng seeded 1. */
void bgo_create_lif(bgo_net *n, const float *ranges16);
/* Izhikevich neurons (Neurons/AllIZHNeurons.cpp:405-476): the 16 IF ranges as for LIF, then
 * for each of a, b, c, d: (minExc, maxExc, minInh, maxInh) — 16 floats. */
void bgo_create_izh(bgo_net *n, const float *ranges16, const float *izh16);
void bgo_growth_init(bgo_net *n, float epsilon, float beta, float rho, float target_rate,
                     float min_radius, float start_radius);
void bgo_seed_noise(bgo_net *n, uint32_t seed);
/* Rebuild incoming/outgoing maps from the slot arrays (AllSynapses::createSynapseImap). */
int bgo_rebuild_maps(bgo_net *n);
/* Fill per-type synapse constants of an in-use slot as createSynapse does. */
void bgo_create_synapse(bgo_net *n, int dest, int src, int type, float W);

/* External inputs (Inputs/).  Regular: values100 is the 10x10 pattern of <Values><I>, sync 0 =
 * "yes", 1 = "no" (random shifts from the global rng), 2 = "wave".  Poisson: fr_mean (Hz),
 * weight (x 1e-8 A), masks (N bytes, NULL = all).  Returns 0 on success. */
int bgo_input_regular(bgo_net *n, float duration, float interval, int sync, const float *values100);
int bgo_input_poisson(bgo_net *n, float fr_mean, float weight, const uint8_t *masks);
/* Poisson input spike schedule as the reference would draw it over the next nsteps steps, without
 * running the network (the draws depend only on the counters): per neuron, the ISI values (steps)
 * in draw order.  isi_out must hold max_isis entries; returns the number written, or -1. */
int64_t bgo_poisson_isi_draws(bgo_net *n, int nsteps, int32_t *isi_begin /* N+1 */,
                              int32_t *isi_out, int64_t max_isis);

/* Record every consumed noise value (bounded buffer) for inspection. */
void bgo_record_noise(bgo_net *n, int64_t capacity);
int64_t bgo_noise_recorded(const bgo_net *n);

/* Hot path. */
void bgo_step(bgo_net *n, int nsteps);        /* advanceNeurons + advanceSynapses, nsteps times */
void bgo_growth(bgo_net *n);                  /* updateConnections (ConnGrowth) + maps rebuild  */
void bgo_record_epoch(bgo_net *n, int epoch); /* XmlGrowthRecorder::compileHistories            */
/* XmlRecorder::compileHistories alone (Recorders/XmlRecorder.cpp:71-104), for ConnStatic. */
void bgo_record_static(bgo_net *n);
int bgo_flags(const bgo_net *n);
/* STDP arithmetic: 0 = the reference's host build (uint64_t spike times), 1 = its device build
 * (int64_t spike times, AllSynapsesDeviceFuncs_d.cu:239-380). */
void bgo_stdp_signed(bgo_net *n, int on);
/* Advance the global rng by the given number of rand() draws (e.g. the weight draws of
 * ConnStatic::setupConnections, Connections/ConnStatic.cpp:74-79, when its synapses are loaded
 * from a reference dump). */
void bgo_rng_skip(bgo_net *n, int64_t draws);
/* STDP constants of synapses created from now on (the reference hard-codes them in
 * AllSTDPSynapses::createSynapse): Apos, Aneg, STDPgap, tauspost, tauspre, taupos, tauneg,
 * WexE (excitatory source), WexI (inhibitory source), mupos, muneg. */
void bgo_stdp_params(bgo_net *n, const float *p11);
/* The reference's checkpoint stream (Model::serialize, Core/Model.cpp:85-98): totalNeurons, the
 * neurons, the in-use synapses, and with conn_growth the ConnGrowth radii and rates; every value
 * printed as std::ostream prints it and followed by a NUL.  Isyn, which the reference allocates
 * and never sets, is written as 0.  Returns the stream's length; writes it when cap suffices. */
int64_t bgo_serialize(const bgo_net *n, int conn_growth, char *buf, int64_t cap);              /* bit0: a row hit maxSynapsesPerNeuron          */

#ifdef __cplusplus
}
#endif
#endif
