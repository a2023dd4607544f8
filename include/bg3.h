/* bg3 — GB300-native BrainGrid spiking-network hot path: the C-ABI boundary (libbg3.so).
 *
 * Every entry point takes plain pointers and sizes.  Arrays passed in or out are HOST arrays in
 * the reference's own layouts (neuron-indexed SoA; synapse slots iSyn = dest * maxSyn + k as in
 * Synapses/AllSynapses.cpp:367), so a reference-side shim can hand its host objects over without
 * reshaping them.  Device layouts are private to the library.
 *
 * The reference calls these through its model and class interfaces; each declaration names the
 * reference interface it replaces (paths relative to the reference project root).
 *
 * Status convention: every function returns an int; 0 is success, negative values are the
 * BG3_E* codes below (the reference instead exit()s through HANDLE_ERROR).  bg3_status_string()
 * turns a code into text.  A sticky device error word (bg3_error_word) reports conditions the
 * reference would assert on (a spike-history ring overflow, a double spike in one delay-queue
 * slot, a synapse row that would exceed maxSynapsesPerNeuron).
 *
 * Threading: calls on one handle must not overlap; different handles are independent.  Each
 * handle owns one CUDA stream; every call is ordered on it and returns without a device sync
 * unless it copies data back to the host.
 */
#ifndef BG3_H
#define BG3_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    BG3_OK = 0,
    BG3_EINVAL = -1,      /* bad argument or state                                        */
    BG3_ENOMEM = -2,      /* device allocation failed                                     */
    BG3_ECUDA = -3,       /* a CUDA call failed                                           */
    BG3_ENOISE = -4,      /* injected noise stream ran out                                */
    BG3_EDEVICE = -5,     /* the device error word is set (see bg3_error_word)            */
    BG3_EUNSUPPORTED = -6, /* model combination not built                                 */
    BG3_ECANCELED = -7     /* a served job was cancelled (bg3_serve_cancel)                */
};

/* device error word bits */
enum {
    BG3_ERR_HISTORY_OVERFLOW = 1u << 0, /* spikeCount reached maxSpikes (AllSpikingNeurons.cpp:114) */
    BG3_ERR_QUEUE_DOUBLE = 1u << 1,     /* preSpikeHit on a set bit (AllSpikingSynapses.cpp:277)    */
    BG3_ERR_ROW_FULL = 1u << 2,         /* growth wanted a synapse in a full row (AllSynapses.cpp:360) */
    BG3_ERR_NOISE_EXHAUSTED = 1u << 3,  /* injected noise stream shorter than needed                */
    BG3_ERR_NEGATIVE_AREA = 1u << 4,    /* growth saw a negative weight (the reference would erase) */
    BG3_ERR_SPIKE_LIST = 1u << 5,       /* more spikes in one step than neurons (internal check)    */
    BG3_ERR_TIMEOUT = 1u << 6,          /* a bounded device wait expired (the kernel drained)       */
    BG3_ERR_STEP_RANGE = 1u << 7,       /* step counter beyond 2^32 - 256 (32-bit spike times)      */
    BG3_ERR_ISI_EXHAUSTED = 1u << 8,    /* injected Poisson ISI draws ran out                        */
    BG3_ERR_STDP_RING = 1u << 9,        /* an STDP walk reached the oldest entry of a full spike ring
                                           (the reference reads outside the ring there)              */
    BG3_ERR_STEP_SYNC = 1u << 10        /* internal check: the delivery and sweep step counters
                                           disagreed (that step's arrivals were not applied)         */
};

enum { BG3_NEURON_LIF = 0, BG3_NEURON_IZH = 1 };
enum { BG3_SYN_SPIKING = 0, BG3_SYN_DS = 1, BG3_SYN_STDP = 2, BG3_SYN_DYNSTDP = 3 };
/* Noise source.  DEVICE: a counter-based generator keyed by (seed, step, neuron), one draw per
 * neuron per step like the reference GPU path (Core/GPUSpikingModel.cu:194).  INJECT: values
 * pushed by the host with bg3_push_noise, consumed in the reference CPU order (one value per
 * integrating neuron, descending neuron index; Neurons/AllSpikingNeurons.cpp:104 and
 * Neurons/AllLIFNeurons.cpp:40). */
enum { BG3_NOISE_DEVICE = 0, BG3_NOISE_INJECT = 1 };

typedef struct bg3_net bg3_net;

/* Network shape; fields mirror SimulationInfo (Core/SimulationInfo.h:92-116). */
typedef struct {
    int32_t n_neurons;            /* totalNeurons                                      */
    int32_t max_syn_per_neuron;   /* maxSynapsesPerNeuron                              */
    int32_t width, height;        /* PoolSize x, y                                     */
    float epoch_duration;         /* Tsim (s)                                          */
    float delta_t;                /* deltaT (s)                                        */
    int32_t max_firing_rate;      /* maxFiringRate (Hz); ring = epoch * rate            */
    int32_t max_epochs;           /* numSims; sizes the recorder histories             */
    int32_t neuron_kind;          /* BG3_NEURON_*                                      */
    int32_t synapse_kind;         /* BG3_SYN_*                                         */
    int32_t noise_mode;           /* BG3_NOISE_*                                       */
    uint32_t noise_seed;          /* seed of the device generator                      */
} bg3_net_desc;

/* LIF neuron arrays, each n_neurons long (Neurons/AllIFNeurons.h:279-362,
 * Neurons/AllSpikingNeurons.h:181-204).  history: n_neurons x max_spikes uint64, row-major;
 * it may be NULL on upload (all ULONG_MAX). */
typedef struct {
    float *Vm, *Vthresh, *Vreset, *I0, *Inoise, *C1, *C2, *Trefract, *summation;
    int32_t *nStepsInRefr, *spikeCount, *spikeCountOffset;
    uint64_t *history;
} bg3_lif_arrays;

/* Izhikevich arrays, each n_neurons long (Neurons/AllIZHNeurons.h:439-471): a, b, c, d, the
 * recovery variable u and C3 = deltaT * 1000.  The IF fields (Vm, Vthresh, I0, Inoise, C2,
 * Trefract, ...) travel in bg3_lif_arrays; C1 and Vreset are unused by this model. */
typedef struct {
    float *Aconst, *Bconst, *Cconst, *Dconst, *u, *C3;
} bg3_izh_arrays;

/* Synapse slot arrays in the reference layout, n_neurons * max_syn_per_neuron long
 * (Synapses/AllSynapses.h:188-232, AllSpikingSynapses.h:342-355, AllDSSynapses.h:269-336).
 * in_use uses one byte per slot; counts is n_neurons long (synapse_counts).  On upload the
 * in-use slots of every row must form a prefix (what AllSynapses::addSynapse produces when no
 * synapse was ever erased).  DS fields may be NULL for BG3_SYN_SPIKING; a network holds at most
 * 16 distinct (U, D, F) triples (createSynapse makes four, one per synapse type), more is
 * BG3_EUNSUPPORTED. */
typedef struct {
    uint8_t *in_use;
    int32_t *src, *type, *delayIdx, *total_delay;
    float *W, *psr, *decay, *tau;
    uint32_t *delayQueue, *counts;
    float *U, *D, *F, *u, *r;
    uint64_t *lastSpike;
} bg3_synapse_arrays;

/* STDP slot arrays (Synapses/AllSTDPSynapses.h:330-420), n_neurons * max_syn_per_neuron long,
 * used with BG3_SYN_STDP and BG3_SYN_DYNSTDP. */
typedef struct {
    uint32_t *delayQueuePost;
    int32_t *delayIdxPost, *total_delayPost;
    float *tauspost, *tauspre, *taupos, *tauneg, *STDPgap, *Wex, *Aneg, *Apos, *mupos, *muneg;
    uint8_t *useFroemkeDanSTDP;
} bg3_stdp_arrays;

/* STDP constants per synapse type II, IE, EI, EE.  AllSTDPSynapses::createSynapse gives every
 * synapse the same values (Synapses/AllSTDPSynapses.cpp:252-273: Apos 0.5, Aneg -0.5, STDPgap
 * 2 ms, tauspost 75 ms, tauspre 34 ms, taupos 15 ms, tauneg 35 ms, Wex 1, mu 0, Froemke-Dan on),
 * which are the defaults of a new network. */
typedef struct {
    float Apos[4], Aneg[4], STDPgap[4], tauspost[4], tauspre[4], taupos[4], tauneg[4], Wex[4];
    float mupos[4], muneg[4];
    int32_t useFroemkeDanSTDP[4];
} bg3_stdp_constants;

/* Spike-time arithmetic of the STDP walks.  HOST: the reference's host build
 * (Synapses/AllSTDPSynapses.cpp:283-421, uint64_t spike times: the pre-spike walk's interval
 * wraps, so pre-after-post pairs only apply the weight clamps).  DEVICE: its device build
 * (Synapses/AllSynapsesDeviceFuncs_d.cu:239-380, int64_t spike times: depression applies). */
enum { BG3_STDP_HOST = 0, BG3_STDP_DEVICE = 1 };

/* Synapse constants per synapse type II, IE, EI, EE (Utils/Global.h:100), as the reference's
 * createSynapse computes them on the host (Synapses/AllSpikingSynapses.cpp:192-240,
 * AllDSSynapses.cpp:180-218).  Used for synapses the device growth pass creates. */
typedef struct {
    float tau[4], decay[4];
    int32_t total_delay[4];
    float U[4], D[4], F[4];
    float u0, r0;
} bg3_type_constants;

/* ConnGrowth parameters (Connections/ConnGrowth.h, m_growth) and the layout it needs. */
typedef struct {
    float epsilon, beta, rho, target_rate, min_radius, start_radius, max_rate;
} bg3_growth_params;

/* Outgoing / incoming maps in the reference order (Core/SynapseIndexMap.h:38-104); each
 * *_map holds total entries (bg3_total_synapses), the others n_neurons. */
typedef struct {
    uint32_t *outgoingSynapseIndexMap, *outgoingSynapseBegin, *outgoingSynapseCount;
    uint32_t *incomingSynapseIndexMap, *incomingSynapseBegin, *incomingSynapseCount;
} bg3_index_maps;

/* ---- lifetime -------------------------------------------------------------------------- */
/* Replaces GPUSpikingModel::setupSim's device allocation (Core/GPUSpikingModel.cu:106-160,
 * IAllNeurons::allocNeuronDeviceStruct Neurons/IAllNeurons.h:98, IAllSynapses::
 * allocSynapseDeviceStruct Synapses/IAllSynapses.h:134). */
int bg3_create(const bg3_net_desc *desc, bg3_net **out);
/* Replaces GPUSpikingModel::cleanupSim / delete*DeviceStruct (Core/GPUSpikingModel.cu:82-99). */
int bg3_destroy(bg3_net *net);
/* Device bytes a network of this shape holds (bg3_create plus an external input); no GPU work.
 * Negative status for an invalid desc.  No counterpart in the reference (admission control). */
int64_t bg3_net_footprint(const bg3_net_desc *desc);
/* Device bytes this network has allocated so far. */
uint64_t bg3_net_bytes(bg3_net *net);
/* The shape the network was created with. */
int bg3_get_desc(bg3_net *net, bg3_net_desc *desc);

/* ---- host -> device ------------------------------------------------------------------- */
/* IAllNeurons::copyNeuronHostToDevice (Neurons/IAllNeurons.h:114). */
int bg3_upload_lif(bg3_net *net, const bg3_lif_arrays *a);
/* AllIZHNeurons::copyNeuronHostToDevice (Neurons/AllIZHNeurons_d.cu:91-121): the Izhikevich
 * arrays of a BG3_NEURON_IZH network (the IF arrays go through bg3_upload_lif). */
int bg3_upload_izh(bg3_net *net, const bg3_izh_arrays *a);
/* Layout arrays (Layouts/Layout.h: xloc, yloc, neuron_type_map as INH=1 / EXC=2). */
int bg3_upload_layout(bg3_net *net, const float *xloc, const float *yloc, const int32_t *ntype);
/* IAllSynapses::copySynapseHostToDevice (Synapses/IAllSynapses.h:160) plus the index-map copy of
 * GPUSpikingModel::copySynapseIndexMapHostToDevice (Core/GPUSpikingModel.cu:326); the maps are
 * rebuilt on the device.  current_step is g_simulationStep (Utils/Global.h:85). */
int bg3_upload_synapses(bg3_net *net, const bg3_synapse_arrays *a, uint64_t current_step);
int bg3_set_type_constants(bg3_net *net, const bg3_type_constants *c);
/* ConnGrowth state (radii, rates) and parameters (Connections/ConnGrowth.h:219+).  p NULL keeps
 * the parameters; radii and rates also become row 0 of the recorder's histories
 * (XmlGrowthRecorder::initValues); NULL arrays are left as they are. */
int bg3_upload_growth(bg3_net *net, const bg3_growth_params *p, const float *radii,
                      const float *rates);
/* Sets W of every in-use slot from a reference-layout array (n_neurons * max_syn_per_neuron),
 * the weight upload of the reference's GPU growth path (Connections/ConnGrowth_d.cu:37-45). */
int bg3_upload_weights(bg3_net *net, const float *W);
/* Multiplies the weight of every in-use synapse by factor, on the device (W = W * factor in
 * float, the same bits as a host loop over the downloaded weights).  No counterpart in the
 * reference: it builds benchmark networks from grown ones without moving the synapse arrays. */
int bg3_scale_weights(bg3_net *net, float factor);
/* Switches the noise source between steps (BG3_NOISE_DEVICE keyed by seed, or BG3_NOISE_INJECT
 * starting from an empty stream), as the reference's model chooses its generator at setup
 * (initMTGPU / normalMTGPU, Core/GPUSpikingModel.h:220-223).  Not for a network inside a batch
 * (batches run device noise). */
int bg3_set_noise_mode(bg3_net *net, int32_t mode, uint32_t seed);
/* The CUDA device that networks created afterwards on this host thread use (the reference
 * driver's -d, g_deviceId, Core/BGDriver.cpp:323-326); device 0 if never called.  A network does
 * not switch devices by itself: every later call on it must be made with the device it was
 * created on current (as the reference, which sets the device once in setupSim). */
int bg3_set_device(int32_t device);
/* Appends n values to the injected noise stream (BG3_NOISE_INJECT), in Norm draw order. */
int bg3_push_noise(bg3_net *net, const float *values, int64_t n);
/* Injected noise values pushed and not yet consumed (0 in device-noise mode); waits for the
 * network's queued steps.  A host that draws the stream ahead uses it to keep at least one value
 * per neuron per queued step on the device without piling up the rest.  No counterpart in the
 * reference (its host model draws each value where it consumes it). */
int bg3_noise_pending(bg3_net *net, int64_t *pending);

/* The reference's own noise stream on the host, for bg3_push_noise: Norm(mu, sigma, seed)
 * (RNG/Norm.cpp:59-86, the Marsaglia polar method in float over MTRand,
 * RNG/MersenneTwister.cpp), the generator the reference's single-threaded model creates from
 * the parameter file's seed (Core/SingleThreadedSpikingModel.cpp:30).  bg3_norm_fill writes the
 * next n values; consecutive fills continue one stream.  Fills of 131,072 values or more run the
 * polar method's arithmetic on up to 16 host threads (the same values).  Host only (no device,
 * no stream); one generator is not to be filled from two threads at once.  BG3_ENOMEM when a
 * thread or memory cannot be had, after which the stream is lost. */
typedef struct bg3_norm bg3_norm;
int bg3_norm_create(uint32_t seed, float mu, float sigma, bg3_norm **out);
int bg3_norm_fill(bg3_norm *gen, float *values, int64_t n);
void bg3_norm_destroy(bg3_norm *gen);

/* ---- external input (one per network, as ISInput) --------------------------------------- */
/* Regular pulses (Inputs/SInputRegular.cpp:20-112, HostSInputRegular.cpp:59-80): per-neuron
 * values and phase shifts as the reference's constructor computed them, the pulse and cycle
 * lengths in steps, and the cycle position (nStepsInCycle) at the current step. */
int bg3_input_regular(bg3_net *net, const float *values, const int32_t *shifts,
                      int32_t n_steps_duration, int32_t n_steps_cycle, int32_t steps_in_cycle);
/* Poisson drive (Inputs/SInputPoisson.cpp:19-146, HostSInputPoisson.cpp:60-94): one DS input
 * synapse per neuron (arrays of n_neurons, reference semantics), the ISI counters nISIs, masks,
 * lambda (ms).  ISIs come from bg3_push_poisson_isis when given, else from a device generator
 * keyed by seed.  current_step is g_simulationStep. */
typedef struct {
    uint8_t *masks;
    int32_t *nISIs, *total_delay, *delayIdx;
    uint32_t *delayQueue;
    float *W, *psr, *decay, *U, *D, *F, *u, *r;
    uint64_t *lastSpike;
} bg3_poisson_arrays;
int bg3_input_poisson(bg3_net *net, const bg3_poisson_arrays *a, float lambda, uint32_t seed,
                      uint64_t current_step);
/* The reference's own ISI draws per neuron in draw order (begin: n_neurons + 1 offsets), e.g.
 * replayed from its MTRand stream; consumed from the next expiry of each neuron's counter. */
int bg3_push_poisson_isis(bg3_net *net, const int32_t *begin, const int32_t *isis);
int bg3_download_poisson(bg3_net *net, bg3_poisson_arrays *a);

/* ---- hot path ------------------------------------------------------------------------- */
/* nsteps of GPUSpikingModel::advance (Core/GPUSpikingModel.cu:188-230): neuron integration,
 * spike propagation into the delay queues, synapse sweep with summation; g_simulationStep
 * advances by nsteps. */
int bg3_step(bg3_net *net, int64_t nsteps);
/* GPUSpikingModel::updateConnections (Core/GPUSpikingModel.cu:246-258: ConnGrowth::
 * updateConns / updateFrontiers / updateOverlap, ConnGrowth_d.cu:18-61 weights and rewiring,
 * createSynapseImap) followed by updateHistory (:266, XmlGrowthRecorder::compileHistories:
 * histograms, rates/radii history, radius clamp, spike-count roll).  epoch is the 1-based
 * epoch number (SimulationInfo::currentStep). */
int bg3_epoch_growth(bg3_net *net, int32_t epoch);
/* updateHistory of a network without growth (ConnStatic: Connections/ConnStatic.h has no
 * updateConnections work): XmlRecorder::compileHistories (Recorders/XmlRecorder.cpp:71-104),
 * burstiness and 10 ms spike histograms plus the spike-count roll. */
int bg3_epoch_record(bg3_net *net);

/* AllSTDPSynapses::copySynapseHostToDevice (Synapses/AllSTDPSynapses_d.cu:125-195): the STDP
 * fields of the slots given by syn (in_use, type, delayIdx).  Constants must be uniform per
 * synapse type; post queues must be empty with total_delayPost 0; the weight-dependence
 * exponents mupos and muneg must be 0, the reference's values (it raises W to them with the
 * host's pow, which the device cannot reproduce bit for bit).  BG3_EUNSUPPORTED otherwise. */
int bg3_upload_stdp(bg3_net *net, const bg3_synapse_arrays *syn, const bg3_stdp_arrays *a);
/* Constants for synapses created by the device growth pass from now on (mupos and muneg 0,
 * BG3_EUNSUPPORTED otherwise, as for bg3_upload_stdp). */
int bg3_set_stdp_constants(bg3_net *net, const bg3_stdp_constants *c);
/* BG3_STDP_HOST (default) or BG3_STDP_DEVICE. */
int bg3_set_stdp_arithmetic(bg3_net *net, int mode);

/* ---- device -> host ------------------------------------------------------------------- */
int bg3_sync(bg3_net *net);
int bg3_get_step(bg3_net *net, uint64_t *step);
int bg3_error_word(bg3_net *net, uint32_t *err);
/* IAllNeurons::copyNeuronDeviceToHost (Neurons/IAllNeurons.h:122); history included. */
int bg3_download_lif(bg3_net *net, bg3_lif_arrays *a);
/* AllIZHNeurons::copyNeuronDeviceToHost (Neurons/AllIZHNeurons_d.cu:125-150). */
int bg3_download_izh(bg3_net *net, bg3_izh_arrays *a);
/* AllSTDPSynapses::copySynapseDeviceToHost (Synapses/AllSTDPSynapses_d.cu:198-250): STDP fields
 * of the in-use slots in the reference layout. */
int bg3_download_stdp(bg3_net *net, bg3_stdp_arrays *a);
/* IAllSynapses::copySynapseDeviceToHost (Synapses/IAllSynapses.h:177), reference layout, with
 * delayIdx and delayQueue in the reference's per-synapse phase. */
int bg3_download_synapses(bg3_net *net, bg3_synapse_arrays *a);
int64_t bg3_total_synapses(bg3_net *net);
int bg3_download_maps(bg3_net *net, bg3_index_maps *m);
int bg3_download_growth(bg3_net *net, float *radii, float *rates);
/* XmlRecorder / XmlGrowthRecorder histories (Recorders/XmlRecorder.cpp:71-104,
 * XmlGrowthRecorder.cpp:72-97): burstiness (epochs*Tsim bins), spikes (100 per second),
 * rates and radii ((max_epochs+1) x n_neurons). */
int bg3_download_histories(bg3_net *net, float *burstiness, float *spikes, float *rates_hist,
                           float *radii_hist);
/* The whole observable state in one call (what the reference's model copies back at the end of
 * a run, Core/GPUSpikingModel.cu:82-99, and its recorders read): each non-NULL member is filled
 * as the single-purpose download above fills it; NULL members are skipped. */
typedef struct {
    bg3_lif_arrays *neurons;          /* Vm, spike counts, refractory counters, spike history */
    bg3_izh_arrays *izh;              /* BG3_NEURON_IZH only                                  */
    bg3_synapse_arrays *synapses;     /* slot arrays incl. delay queues, counts               */
    bg3_stdp_arrays *stdp;            /* BG3_SYN_STDP / BG3_SYN_DYNSTDP only                  */
    bg3_index_maps *maps;             /* incoming / outgoing index maps                       */
    float *radii, *rates;             /* ConnGrowth state, n_neurons each (both or neither)   */
} bg3_state_view;
int bg3_download_state(bg3_net *net, const bg3_state_view *view);

/* ---- allocation-free variant -------------------------------------------------------------- */
/* No counterpart in the reference: an extra entry point for callers that cannot allocate device
 * memory when they need the map (host runtimes that own every device allocation through their
 * own pool; real-time loops that must not enter the allocator).  Builds the outgoing synapse map
 * in the reference's
 * order (Core/SynapseIndexMap.h: per source neuron, the slot ids d * max_syn + k in ascending
 * order) from caller-owned DEVICE buffers and allocates nothing:
 *   src_dev     [n_neurons * max_syn] int32, reference slot layout (sourceNeuronIndex)
 *   counts_dev  [n_neurons] uint32, in-use prefix length of each row (synapse_counts)
 *   begin_dev, count_dev  [n_neurons] uint32 out;  map_dev [sum of counts] uint32 out
 *   status_dev  one uint32 out: bit 0 a source index out of range, bit 1 a source with more than
 *               BG3_NOALLOC_MAX_FANOUT synapses (its run is left unsorted)
 *   stream      cudaStream_t (NULL: the legacy default stream); the call only enqueues work.
 * Its scratch (one counter per neuron) is a fixed array inside the library, shared by all calls
 * on a device and kept until the process exits: calls that overlap on the GPU race on it.  More
 * than BG3_NOALLOC_MAX_NEURONS neurons, or n_neurons * max_syn above 2^32 (32-bit slot ids), is
 * rejected with BG3_EINVAL.  The first call on each device resolves the array's address with
 * that device current and keeps it; make it before any stream capture.  After a cudaDeviceReset
 * the kept address is stale: do not call this entry point on a device the process has reset.
 * A CUDA error left pending by earlier calls is cleared on entry. */
#define BG3_NOALLOC_MAX_NEURONS 65536
#define BG3_NOALLOC_MAX_FANOUT 4096
int bg3_outgoing_map_noalloc(const int32_t *src_dev, const uint32_t *counts_dev,
                             int32_t n_neurons, int32_t max_syn, uint32_t *begin_dev,
                             uint32_t *count_dev, uint32_t *map_dev, uint32_t *status_dev,
                             void *stream);

/* ---- diagnostics ---------------------------------------------------------------------- */
const char *bg3_status_string(int status);
/* Per-launch timing of the last bg3_step call's kernels: fills up to n entries of
 * (kernel id, milliseconds) measured with CUDA events on the handle's stream when enabled. */
int bg3_enable_timing(bg3_net *net, int on);
int bg3_kernel_times(bg3_net *net, float *ms_neurons, float *ms_fanout, float *ms_sweep,
                     int64_t *launches);

/* ---- batched form ---------------------------------------------------------------------- */
/* Many networks of uneven size advanced together: each step is one spike-delivery launch and
 * one sweep launch over every network (per-network descriptor and tensor-map tables, tiles
 * ordered heaviest first), with runs of steps replayed from a CUDA graph.  The reference has no
 * counterpart (it runs one network per process, Core/BGDriver.cpp:49-158); each member network
 * is a bg3_net created and loaded as usual, which stays usable on its own.  Members must share
 * the synapse kind and use BG3_NOISE_DEVICE; results are identical to running each member with
 * bg3_step.  After bg3_epoch_growth on a member, call bg3_batch_refresh. */
typedef struct bg3_batch bg3_batch;
int bg3_batch_create(bg3_net *const *nets, int32_t count, bg3_batch **out);
int bg3_batch_destroy(bg3_batch *batch);
int bg3_batch_refresh(bg3_batch *batch);
int bg3_batch_step(bg3_batch *batch, int64_t nsteps);
int bg3_batch_sync(bg3_batch *batch);
int64_t bg3_batch_launches(bg3_batch *batch);
/* Same as bg3_bench_steps for a batch (step_ms[nsteps], CUDA events on the batch stream). */
int bg3_batch_bench_steps(bg3_batch *batch, int64_t nsteps, int64_t flush_bytes, float *step_ms);

/* Benchmark helper: runs nsteps steps on the handle's stream.  Before each step, when
 * flush_bytes > 0, a scratch buffer of that size is overwritten so that the step starts with a
 * cold L2.  The device time of each step (CUDA events on the handle's stream, flush excluded) is
 * written to step_ms[nsteps].  In device-noise mode a timed step is, as bg3_step runs them, the
 * sweep of step s followed by the spike delivery of step s + 1, which overlaps that sweep (the
 * first timed step also holds step 0's delivery, the last none: nsteps of each in total).  When
 * kernel_ms is not NULL the phases run one after the other instead, with an event between them:
 * kernel_ms[3 * s .. 3 * s + 2] = 0, spike delivery (plus the neuron pass in injected-noise mode),
 * and the sweep (whose epilogue runs the next step's neuron pass in device-noise mode).  The
 * standalone neuron pass before step 0 is not timed. */
int bg3_bench_steps(bg3_net *net, int64_t nsteps, int64_t flush_bytes, float *step_ms,
                    float *kernel_ms);

/* Self-test of the library's integer-pipe binary64 add / multiply / conversion (used by the
 * Izhikevich update) against the hardware on `samples` random operand pairs: counts[0..3] =
 * add mismatches, multiply mismatches, conversion mismatches, cases outside the restated range
 * (which the update recomputes in hardware).  No counterpart in the reference. */
int bg3_selftest_binary64(uint64_t samples, uint64_t seed, uint64_t *counts);
/* Self-test of the three evaluations of the Izhikevich update's double expression (the FP64
 * pipe, its integer-pipe restatement, and float-float arithmetic that hands uncertain roundings to
 * the FP64 pipe) on `samples` random operand sets: counts[0..3] = integer-pipe mismatches against
 * the FP64 pipe, float-float mismatches, float-float values handed to the FP64 pipe, operand sets
 * outside the integer pipe's restated range.  No counterpart in the reference. */
int bg3_selftest_izhikevich(uint64_t samples, uint64_t seed, uint64_t *counts);
/* Failure-detection self-test: one warp waits, with the bounded mbarrier wait the step kernels
 * use, on a barrier that nothing completes, for at most limit_ns (1 .. 2e9).  The wait gives up,
 * the kernel returns normally and the context stays usable: *status = BG3_ERR_TIMEOUT, and
 * *waited_ns the time it waited.  (In the step kernels the same expiry sets BG3_ERR_TIMEOUT in the
 * network's error word after about 1 s, and the CTA drains its copies in flight.) */
int bg3_selftest_timeout(uint64_t limit_ns, uint32_t *status, uint64_t *waited_ns);

/* ---- launch configuration and autotuning (no counterpart in the reference) ----------------- */
typedef struct {
    int32_t sweep_stages;     /* chunks in flight per TMA sweep tile: 4, 6 or 8 (default 6)          */
    int32_t thin_max_quads;   /* networks with at most 4 x this many slots per neuron take the thin
                                 sweep, one warp per 32 dests: 1 .. 4096 (default 16)               */
    int32_t thin_warps;       /* warps per block of the thin sweep: 1 .. 32 (default 8)              */
    int32_t deliver_blocks;   /* blocks of the spike-delivery grid: 1 .. 65535 (default 304); a
                                 batch shares four such grids out over its networks                 */
    int32_t growth_threads;   /* threads per block of the overlap pass: 128, 256 or 512 (256)       */
    int32_t sweep_dests;      /* dests per TMA sweep tile of a single network: 16 or 32 (32); more,
                                 smaller tiles spread a network over the SMs more evenly (a batch
                                 always uses 32)                                                    */
    int32_t deliver_early;    /* 1 (default): the spike delivery of spiking and DS synapses starts
                                 while the previous sweep runs and prepares its arrivals (slot
                                 positions, event state), applying only the psr increments after it;
                                 0: it starts after the sweep.  Same results either way.            */
    int32_t izh_hw_every;     /* Izhikevich networks: every k-th group of 32 neurons evaluates the
                                 update's double-precision expression on the FP64 pipe, the others
                                 on the integer pipe (an exact restatement): 0 .. 8, 0 = none,
                                 1 = all; -1 (default): every neuron in float-float arithmetic,
                                 with the FP64 pipe only for values whose float rounding the
                                 float-float result leaves uncertain (~0.2 %).  Same results every
                                 way.                                                                 */
    int32_t small_max_slots;  /* a network of at most 2,048 neurons whose synapse planes hold at most
                                 this many slots (neurons rounded up to 32 x max synapses rounded up
                                 to 4) runs up to 4,096 whole steps per launch on one CTA, with no
                                 launch between its passes (default 65,536; 0: never).  Same
                                 results either way.                                                */
} bg3_launch_cfg;
int bg3_get_launch(bg3_net *net, bg3_launch_cfg *cfg);
int bg3_set_launch(bg3_net *net, const bg3_launch_cfg *cfg);
int bg3_batch_get_launch(bg3_batch *batch, bg3_launch_cfg *cfg);
int bg3_batch_set_launch(bg3_batch *batch, const bg3_launch_cfg *cfg);
/* Chooses the launch configuration by timing candidates on the handle's own state: the device
 * state is copied aside, each candidate runs from that copy (warm-up steps, then
 * steps_per_trial timed steps; with tune_growth also one growth pass for the overlap block
 * size), one parameter at a time, and the state is put back, so the network is afterwards
 * exactly as before.  The fastest configuration is kept and returned with its time per step.
 * (Each trial first runs 35 untimed steps, so that its CUDA graph is captured before timing.)
 * Needs free device memory for one copy of the state (BG3_ENOMEM otherwise). */
int bg3_autotune(bg3_net *net, int32_t steps_per_trial, int32_t tune_growth, bg3_launch_cfg *best,
                 float *best_ms_per_step);
int bg3_batch_autotune(bg3_batch *batch, int32_t steps_per_trial, bg3_launch_cfg *best,
                       float *best_ms_per_step);

/* ---- checkpoints (bit-exact resume; no counterpart in the reference) --------------------------
 * The reference's own checkpoint (Model::serialize, Core/Model.cpp:85-98) prints six significant
 * digits per value and holds neither the step counter, the noise generator nor the spike
 * history, so a run restarted from it does not continue the original one.  These two calls save
 * and restore a network's entire state instead: every device array, the step counter, the
 * injected noise still to be consumed, the Poisson and regular input state, the tables and the
 * launch configuration.  A network loaded from a checkpoint continues exactly as the saved one
 * would have (same spikes, same float bits); device noise is keyed by (seed, step, neuron), so
 * restoring the step restores the generator.
 *
 * bg3_checkpoint_save: with buf == NULL only *len is set (the bytes needed); with cap < *len it
 * returns BG3_EINVAL and writes nothing.  The format is this library build's own (host byte order,
 * checked by a header); it is not meant for other programs.
 * bg3_checkpoint_load: into a network made by bg3_create with the same bg3_net_desc.  Everything
 * is checked before anything changes, and any mismatch is BG3_EINVAL with the network untouched:
 * the header and a checksum of the bytes, every shape scalar, the size of every array (only the
 * arrays of an external input may differ from the network's: the input set up before the save is
 * allocated, one set up since is freed) and every value a kernel addresses memory with (source
 * and neuron ids, row counts, class codes, map runs, cursors).  A network that is a member of a
 * batch needs bg3_batch_refresh afterwards.  If the load fails after those checks (a CUDA or
 * allocation error), destroy the network. */
int bg3_checkpoint_save(bg3_net *net, void *buf, uint64_t cap, uint64_t *len);
int bg3_checkpoint_load(bg3_net *net, const void *buf, uint64_t len);

/* ---- the reference's checkpoint stream ---------------------------------------------------- */
enum { BG3_CONN_STATIC = 0, BG3_CONN_GROWTH = 1 };  /* ConnStatic / ConnGrowth */
/* IF-neuron fields that only the reference's host objects hold: set by AllIFNeurons::
 * createNeuron and never read by the step (Neurons/AllIFNeurons.h:279-362), so the library does
 * not keep them.  Each array n_neurons long; NULL arrays are written as 0 and skipped on reading. */
typedef struct {
    float *Cm, *Rm, *Vrest, *Vinit, *Iinject, *Isyn, *Tau;
} bg3_if_fields;
/* The bytes Model::serialize writes (Core/Model.cpp:85-98; the -w file of Core/BGDriver.cpp:
 * 110-116): totalNeurons; per neuron the AllIFNeurons::writeNeuron fields (plus the six of
 * AllIZHNeurons); the synapse count and every in-use synapse, dest row by dest row, with the
 * writeSynapse fields of the network's synapse class; with BG3_CONN_GROWTH the radii and rates
 * (ConnGrowth::serialize; ConnStatic writes nothing).  Every value is printed as std::ostream
 * prints it (floats with six significant digits) and followed by a NUL.  hasFired is written as 0:
 * the step that sets it also clears it (Neurons/AllSpikingNeurons.cpp:144).  With buf NULL only
 * *len is set; with cap < *len nothing is written and BG3_EINVAL returned. */
int bg3_serialize(bg3_net *net, const bg3_if_fields *setup, int32_t conn, char *buf, uint64_t cap,
                  uint64_t *len);
/* Loads such a stream into the network (Model::deserialize, Core/Model.cpp:62-76, then the
 * recorder's initValues as Core/Simulator.cpp:206-214 does: radii and rates become row 0 of the
 * histories).  The reference's own reader cannot read its writer's layout: AllSynapses::
 * deserialize (Synapses/AllSynapses.cpp:123-155) reads a neuron index before every synapse that
 * writeSynapse never writes.  This reader follows the writer: each synapse goes to the next slot of
 * its dest row, which reproduces the written slots.  current_step is the g_simulationStep the state
 * belongs to (delay queues, delayIdx and lastSpike are relative to it; the reference's driver
 * restarts at 0).  Values the library keeps per synapse type or as classes (tau, U/D/F, the STDP
 * constants) must be representable: BG3_EUNSUPPORTED otherwise, and so for a hasFired of 1 or a
 * queue length other than 32.  A malformed stream is BG3_EINVAL.  setup_out, when given, receives
 * the fields of bg3_if_fields. */
int bg3_deserialize(bg3_net *net, const char *buf, uint64_t len, int32_t conn,
                    uint64_t current_step, bg3_if_fields *setup_out);

#ifdef __cplusplus
}
#endif
#endif
