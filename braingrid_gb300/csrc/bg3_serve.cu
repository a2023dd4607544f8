// Served form of libbg3 (include/bg3_serve.h): admission by device footprint (in arrival order
// or least work first, with a bound on how often a job is passed over), continuous
// batching of the resident jobs through the batched step (bg3_batch_*), per-job epoch ends.
// Host code only; it drives the GPU through the public C-ABI.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bg3.h"
#include "../../include/bg3_serve.h"

namespace {

struct Job {
    int64_t id = 0;
    bg3_job_desc d;
    int64_t footprint = 0;
    bg3_net *net = nullptr;
    int64_t spe = 0;          // steps per epoch
    int64_t to_boundary = 0;  // steps left in the current epoch
    int32_t epoch = 0;        // epochs finished
    int64_t syn = 0;          // current synapse count
    uint64_t slots = 0;       // n_neurons x max_syn_per_neuron (work estimate)
    int32_t bypassed = 0;     // times a later job was admitted ahead of it
};

const int KINDS = 4;  // one batch group per synapse kind

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct bg3_server {
    bg3_serve_desc cfg;
    std::deque<Job *> queue;
    std::vector<Job *> resident, joining;
    std::vector<int64_t> finished;
    bg3_batch *group[KINDS] = {nullptr, nullptr, nullptr, nullptr};
    bool dirty[KINDS] = {false, false, false, false};
    uint64_t bytes = 0, slots = 0;
    int64_t next_id = 1;
    bg3_serve_stats st;
};

static int64_t steps_per_epoch(const bg3_net_desc &d)
{
    // static_cast<uint64_t>(epochDuration / deltaT) in float (Core/Simulator.cpp:159-160)
    return (int64_t)(d.epoch_duration / d.delta_t);
}

static void finish(bg3_server *s, Job *j, int status)
{
    bg3_job_result *r = j->d.result;
    if (r) {
        r->status = status;
        if (j->net) {
            uint32_t err = 0;
            bg3_error_word(j->net, &err);
            r->error_word = err;
            if (status == BG3_OK) {
                int rc = bg3_download_histories(j->net, r->burstiness, r->spikes_hist, r->rates_hist,
                                                r->radii_hist);
                if (rc == BG3_OK && r->Vm) {
                    bg3_lif_arrays a;
                    memset(&a, 0, sizeof(a));
                    a.Vm = r->Vm;
                    rc = bg3_download_lif(j->net, &a);
                }
                if (rc == BG3_OK && r->checkpoint)
                    rc = bg3_checkpoint_save(j->net, r->checkpoint, r->checkpoint_cap,
                                             &r->checkpoint_len);
                r->status = rc;
            }
        }
    }
    if (j->net) {
        bg3_destroy(j->net);
        s->bytes -= (uint64_t)j->footprint;
        s->slots -= j->slots;
    }
    j->net = nullptr;
    if (status == BG3_OK) s->st.done++;
    else if (status == BG3_ECANCELED) s->st.cancelled++;
    else s->st.failed++;
    s->finished.push_back(j->id);
    delete j;
}

// Rebuilds the batch of every group whose membership or synapse counts changed.
static int rebuild_groups(bg3_server *s)
{
    for (int k = 0; k < KINDS; k++) {
        if (!s->dirty[k]) continue;
        s->dirty[k] = false;
        if (s->group[k]) bg3_batch_destroy(s->group[k]);
        s->group[k] = nullptr;
        std::vector<bg3_net *> nets;
        for (Job *j : s->resident)
            if (j->d.desc.synapse_kind == k) nets.push_back(j->net);
        if (nets.empty()) continue;
        int rc = bg3_batch_create(nets.data(), (int32_t)nets.size(), &s->group[k]);
        if (rc) return rc;
    }
    return BG3_OK;
}

static bool fits(const bg3_server *s, const Job *j)
{
    if (s->bytes + (uint64_t)j->footprint > s->cfg.hbm_budget_bytes) return false;
    if (s->cfg.max_resident_slots && s->slots > 0 &&
        s->slots + j->slots > s->cfg.max_resident_slots)
        return false;
    return true;
}

// A queued job's work: synapse slots x the steps of its epochs still to run.
static double work_left(const Job *j)
{
    const int64_t spe = std::max<int64_t>(1, steps_per_epoch(j->d.desc));
    // in double: only compared, and no product of the three overflows there
    return (double)j->slots * (double)std::max(0, j->d.epochs) * (double)spe;
}

// The queue index of the next job to admit, or -1: the oldest job once it has been passed
// max_bypass times (or nothing while it does not fit), else the first fitting job in arrival
// order, or the fitting job with the least work (ties to the earlier arrival).
static long pick(const bg3_server *s)
{
    if (s->queue.empty()) return -1;
    if (s->queue[0]->bypassed >= s->cfg.max_bypass) return fits(s, s->queue[0]) ? 0 : -1;
    long best = -1;
    for (size_t qi = 0; qi < s->queue.size(); qi++) {
        const Job *j = s->queue[qi];
        if (!fits(s, j)) continue;
        if (s->cfg.order != BG3_ORDER_LEAST_WORK) return (long)qi;
        if (best < 0 || work_left(j) < work_left(s->queue[(size_t)best])) best = (long)qi;
    }
    return best;
}

// Admits queued jobs (pick) while the budgets and the job count allow; every older job passed
// over counts a bypass.
static void admit(bg3_server *s)
{
    for (;;) {
        if ((int64_t)(s->resident.size() + s->joining.size()) >= s->cfg.max_resident) break;
        const long p = pick(s);
        if (p < 0) break;
        const size_t qi = (size_t)p;
        Job *j = s->queue[qi];
        for (size_t k = 0; k < qi; k++) s->queue[k]->bypassed++;
        s->queue.erase(s->queue.begin() + qi);
        s->bytes += (uint64_t)j->footprint;
        s->slots += j->slots;
        int rc = bg3_create(&j->d.desc, &j->net);
        if (rc == BG3_OK && j->d.setup) rc = j->d.setup(j->net, j->d.user);
        if (rc == BG3_OK && j->d.resume) rc = bg3_checkpoint_load(j->net, j->d.resume, j->d.resume_len);
        if (rc == BG3_OK) rc = bg3_sync(j->net);
        uint64_t step = 0;
        if (rc == BG3_OK) rc = bg3_get_step(j->net, &step);
        if (rc == BG3_OK) {
            int64_t t = bg3_total_synapses(j->net);
            if (t < 0) rc = (int)t;
            else j->syn = t;
        }
        if (rc != BG3_OK) {
            if (!j->net) {
                s->bytes -= (uint64_t)j->footprint;
                s->slots -= j->slots;
            }
            finish(s, j, rc);
            continue;
        }
        j->spe = steps_per_epoch(j->d.desc);
        // a resumed job continues its epoch count from its step counter
        j->epoch = (int32_t)(step / (uint64_t)j->spe);
        j->to_boundary = j->spe - (int64_t)(step % (uint64_t)j->spe);
        if (j->epoch >= j->d.epochs) {
            finish(s, j, BG3_EINVAL);  // nothing left to run
            continue;
        }
        s->joining.push_back(j);
    }
}

extern "C" {

int bg3_serve_create(const bg3_serve_desc *desc, bg3_server **out)
{
    if (!desc || !out || desc->max_resident <= 0 || desc->chunk_steps <= 0 || desc->max_bypass < 0 ||
        (desc->order != BG3_ORDER_ARRIVAL && desc->order != BG3_ORDER_LEAST_WORK))
        return BG3_EINVAL;
    bg3_server *s = new (std::nothrow) bg3_server();
    if (!s) return BG3_ENOMEM;
    s->cfg = *desc;
    memset(&s->st, 0, sizeof(s->st));
    *out = s;
    return BG3_OK;
}

int bg3_serve_destroy(bg3_server *s)
{
    if (!s) return BG3_EINVAL;
    for (int k = 0; k < KINDS; k++)
        if (s->group[k]) bg3_batch_destroy(s->group[k]);
    for (Job *j : s->resident) { if (j->net) bg3_destroy(j->net); delete j; }
    for (Job *j : s->joining) { if (j->net) bg3_destroy(j->net); delete j; }
    for (Job *j : s->queue) delete j;
    delete s;
    return BG3_OK;
}

int bg3_serve_submit(bg3_server *s, const bg3_job_desc *job, int64_t *job_id)
{
    if (!s || !job || job->epochs <= 0 || job->epochs > job->desc.max_epochs ||
        (job->resume && !job->resume_len) ||
        job->desc.noise_mode != BG3_NOISE_DEVICE || job->desc.synapse_kind < 0 ||
        job->desc.synapse_kind >= KINDS)
        return BG3_EINVAL;
    int64_t fp = bg3_net_footprint(&job->desc);
    if (fp < 0) return (int)fp;
    if ((uint64_t)fp > s->cfg.hbm_budget_bytes) return BG3_EINVAL;
    Job *j = new (std::nothrow) Job();
    if (!j) return BG3_ENOMEM;
    j->id = s->next_id++;
    j->d = *job;
    j->footprint = fp;
    j->slots = (uint64_t)job->desc.n_neurons * (uint64_t)job->desc.max_syn_per_neuron;
    if (j->d.result) {
        j->d.result->status = BG3_OK;
        j->d.result->synapse_steps = 0;
        j->d.result->neuron_steps = 0;
        j->d.result->error_word = 0;
        j->d.result->checkpoint_len = 0;
    }
    s->queue.push_back(j);
    if (job_id) *job_id = j->id;
    return BG3_OK;
}

int bg3_serve_pump(bg3_server *s)
{
    if (!s) return BG3_EINVAL;
    double t0 = now_s();
    int rc = rebuild_groups(s);
    double t1 = now_s();
    s->st.rebuild_s += t1 - t0;
    if (rc) return rc;
    // 1. launch one chunk for the resident jobs
    int64_t chunk = 0;
    if (!s->resident.empty()) {
        chunk = s->cfg.chunk_steps;
        for (Job *j : s->resident) chunk = std::min(chunk, j->to_boundary);
        for (int k = 0; k < KINDS; k++)
            if (s->group[k] && (rc = bg3_batch_step(s->group[k], chunk))) return rc;
        s->st.rounds++;
    }
    // 2. admit arrivals while the chunk runs
    t0 = now_s();
    admit(s);
    t1 = now_s();
    s->st.admit_s += t1 - t0;
    // 3. wait for the chunk, then epoch ends and completions
    for (int k = 0; k < KINDS; k++)
        if (s->group[k] && (rc = bg3_batch_sync(s->group[k]))) return rc;
    t0 = now_s();
    s->st.wait_s += t0 - t1;
    std::vector<Job *> keep;
    for (Job *j : s->resident) {
        const int64_t ss = j->syn * chunk, ns = (int64_t)j->d.desc.n_neurons * chunk;
        s->st.synapse_steps += ss;
        s->st.neuron_steps += ns;
        if (j->d.result) {
            j->d.result->synapse_steps += ss;
            j->d.result->neuron_steps += ns;
        }
        j->to_boundary -= chunk;
        if (j->to_boundary > 0) {
            keep.push_back(j);
            continue;
        }
        const int kind = j->d.desc.synapse_kind;
        j->epoch++;
        if (j->d.growth) {
            rc = bg3_epoch_growth(j->net, j->epoch);
            if (rc == BG3_OK) rc = bg3_sync(j->net);
            if (rc == BG3_OK) {
                int64_t t = bg3_total_synapses(j->net);
                if (t < 0) rc = (int)t;
                else j->syn = t;
            }
        } else {
            rc = bg3_epoch_record(j->net);
            if (rc == BG3_OK) rc = bg3_sync(j->net);
        }
        s->dirty[kind] = true;
        if (rc != BG3_OK || j->epoch >= j->d.epochs) {
            finish(s, j, rc);
            continue;
        }
        j->to_boundary = j->spe;
        keep.push_back(j);
    }
    s->resident.swap(keep);
    s->st.epoch_s += now_s() - t0;
    for (Job *j : s->joining) {
        s->resident.push_back(j);
        s->dirty[j->d.desc.synapse_kind] = true;
    }
    s->joining.clear();
    s->st.peak_resident = std::max<int64_t>(s->st.peak_resident, (int64_t)s->resident.size());
    return BG3_OK;
}

int bg3_serve_cancel(bg3_server *s, int64_t job_id)
{
    if (!s) return BG3_EINVAL;
    // between pump calls no chunk is in flight: the job can go at once
    for (size_t i = 0; i < s->queue.size(); i++)
        if (s->queue[i]->id == job_id) {
            Job *j = s->queue[i];
            s->queue.erase(s->queue.begin() + i);
            finish(s, j, BG3_ECANCELED);
            return BG3_OK;
        }
    for (std::vector<Job *> *v : {&s->resident, &s->joining})
        for (size_t i = 0; i < v->size(); i++)
            if ((*v)[i]->id == job_id) {
                Job *j = (*v)[i];
                v->erase(v->begin() + i);
                if (v == &s->resident) s->dirty[j->d.desc.synapse_kind] = true;
                finish(s, j, BG3_ECANCELED);
                return BG3_OK;
            }
    return BG3_EINVAL;
}

int bg3_serve_take(bg3_server *s, int64_t *ids, int32_t cap, int32_t *n)
{
    if (!s || !n || cap < 0 || (cap > 0 && !ids)) return BG3_EINVAL;
    const int32_t m = (int32_t)std::min<size_t>((size_t)cap, s->finished.size());
    for (int32_t i = 0; i < m; i++) ids[i] = s->finished[i];
    s->finished.erase(s->finished.begin(), s->finished.begin() + m);
    *n = m;
    return BG3_OK;
}

int bg3_serve_stats_get(bg3_server *s, bg3_serve_stats *out)
{
    if (!s || !out) return BG3_EINVAL;
    bg3_serve_stats st = s->st;
    st.queued = (int64_t)s->queue.size();
    st.resident = (int64_t)(s->resident.size() + s->joining.size());
    st.bytes_resident = s->bytes;
    *out = st;
    return BG3_OK;
}

}  // extern "C"
