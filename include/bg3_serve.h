/* libbg3 served form: a job server that keeps many independent simulations resident on one GPU
 * and advances them together (continuous batching).
 *
 * No counterpart in the reference: BrainGrid runs one simulation per process (Core/BGDriver.cpp).
 * A job here is one such simulation — a network built by the caller's setup callback through the
 * bg3_* C-ABI, run for a number of epochs that each end in ConnGrowth (bg3_epoch_growth) or in the
 * plain recorder (bg3_epoch_record), with its recorder histories copied out at the end.
 *
 * Scheduling, one bg3_serve_pump call per round:
 *   1. the resident jobs advance by one chunk: the smallest number of steps to any resident job's
 *      next epoch end, capped by chunk_steps; jobs are grouped by synapse kind and every group
 *      advances with one batched launch per kernel per step (bg3_batch_*), groups on their own
 *      streams;
 *   2. while that runs, queued jobs are admitted in arrival order as long as the device bytes of
 *      the resident jobs plus the job's bg3_net_footprint stay within hbm_budget_bytes, its
 *      synapse slots within max_resident_slots and fewer than max_resident jobs are resident;
 *      a job that does not fit may be passed by later ones that do, max_bypass times at most;
 *      admission creates the network and calls the job's setup callback; the job joins the
 *      batch in the next round;
 *   3. after the chunk, jobs at an epoch end run their epoch pass; finished jobs copy their
 *      results out (and their whole state, when asked: bg3_job_result.checkpoint), free their
 *      device memory and are reported by bg3_serve_take.
 * A job may start from an exported state (bg3_job_desc.resume): it continues bit for bit as the
 * job it came from would have, so long jobs can be split, moved between servers or GPUs, or
 * preempted and requeued.
 * Every job's arithmetic is independent of the others (device noise is keyed by the job's own
 * seed and step), so a job's results are the same alone and in any mix.
 */
#ifndef BG3_SERVE_H
#define BG3_SERVE_H

#include <stdint.h>

#include "bg3.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bg3_server bg3_server;

typedef struct {
    uint64_t hbm_budget_bytes;   /* admission budget: sum of resident bg3_net_footprint       */
    int32_t max_resident;        /* jobs on the GPU at once                                    */
    int32_t chunk_steps;         /* cap on the steps of one scheduling round                   */
    /* work budget: sum of the resident jobs' synapse slots (n_neurons x max_syn_per_neuron);
     * 0 = none.  Past the point where one step's sweep saturates HBM, more resident work only
     * stretches every job's latency, so jobs wait instead. */
    uint64_t max_resident_slots;
    /* a job that does not fit may be passed by later jobs that do (backfill) at most this many
     * times; then admission waits for it */
    int32_t max_bypass;
    /* which fitting queued job is admitted first: BG3_ORDER_ARRIVAL (0) the earliest,
     * BG3_ORDER_LEAST_WORK (1) the one with the least work (synapse slots x steps); either way a
     * job passed max_bypass times is admitted next (it ages into the head of the queue) */
    int32_t order;
} bg3_serve_desc;

enum { BG3_ORDER_ARRIVAL = 0, BG3_ORDER_LEAST_WORK = 1 };

/* Where a finished job's results go (host memory owned by the caller, valid until the job has
 * been returned by bg3_serve_take).  NULL pointers are skipped.  The histories are those of
 * bg3_download_histories; Vm is the final membrane potential (n_neurons). */
typedef struct {
    float *burstiness, *spikes_hist, *rates_hist, *radii_hist, *Vm;
    /* export of the finished job's state (bg3_checkpoint_save) into checkpoint[checkpoint_cap];
     * NULL: none.  checkpoint_len gets the bytes needed; too small a buffer fails the job with
     * BG3_EINVAL. */
    void *checkpoint;
    uint64_t checkpoint_cap, checkpoint_len;
    /* filled by the server */
    int64_t synapse_steps;       /* sum over the job's steps of its synapse count             */
    int64_t neuron_steps;
    int32_t status;              /* BG3_OK, or the status of the failed setup / step          */
    uint32_t error_word;         /* bg3_error_word at the end                                  */
} bg3_job_result;

/* Called once at admission with the freshly created network; uploads the job's state. */
typedef int (*bg3_job_setup_fn)(bg3_net *net, void *user);

typedef struct {
    bg3_net_desc desc;           /* noise_mode must be BG3_NOISE_DEVICE                       */
    int32_t epochs;              /* epochs to run, 1 .. desc.max_epochs                        */
    int32_t growth;              /* 1: epochs end in bg3_epoch_growth, 0: bg3_epoch_record     */
    bg3_job_setup_fn setup;
    void *user;
    bg3_job_result *result;
    /* import: a checkpoint (bg3_checkpoint_save of a network with this desc) loaded after setup;
     * the job continues from its step, its epochs counted from step 0 (a job exported after k
     * epochs and resumed with `epochs` = n runs n - k more).  NULL: start from setup's state. */
    const void *resume;
    uint64_t resume_len;
} bg3_job_desc;

typedef struct {
    int64_t queued, resident, done, failed, cancelled;
    uint64_t bytes_resident;     /* sum of the resident jobs' footprints                       */
    int64_t rounds;              /* pump rounds that advanced at least one job                 */
    int64_t synapse_steps, neuron_steps;
    int64_t peak_resident;
    /* host wall-clock seconds spent in: admission (create + setup), waiting for chunks,
     * epoch passes and completions, batch rebuilds */
    double admit_s, wait_s, epoch_s, rebuild_s;
} bg3_serve_stats;

int bg3_serve_create(const bg3_serve_desc *desc, bg3_server **out);
/* Frees every job still queued or resident (their results are not filled). */
int bg3_serve_destroy(bg3_server *srv);
/* Queues a job (host only; no device memory is taken until admission).  BG3_EINVAL for a job
 * whose footprint alone exceeds the budget. */
int bg3_serve_submit(bg3_server *srv, const bg3_job_desc *job, int64_t *job_id);
/* One scheduling round (above).  Returns after the round's chunk has finished on the GPU. */
int bg3_serve_pump(bg3_server *srv);
/* Cancels a job between rounds: a queued job leaves the queue, a resident one frees its device
 * memory at once (its group's batch is rebuilt in the next round); the other jobs go on as if it
 * had never been there.  Its result gets status BG3_ECANCELED (histories not filled) and
 * bg3_serve_take reports it.  BG3_EINVAL for an id that is not queued or resident. */
int bg3_serve_cancel(bg3_server *srv, int64_t job_id);
/* Ids of jobs finished since the last call (results filled), up to cap; *n gets the count. */
int bg3_serve_take(bg3_server *srv, int64_t *job_ids, int32_t cap, int32_t *n);
int bg3_serve_stats_get(bg3_server *srv, bg3_serve_stats *stats);

#ifdef __cplusplus
}
#endif
#endif
