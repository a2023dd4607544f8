"""Served form (bg3_serve_*): continuous batching must not change any job's results.

Each job's arithmetic is independent of the others (its own noise seed, its own step counter),
and the batched kernels are bit-exact with the single-network ones, so a job's recorder
histories and final state are identical whether it runs alone, in a mix that joins and leaves
around it, or through the plain single-network API."""
import ctypes

import numpy as np
import pytest

from braingrid_gb300 import lib as bg
from braingrid_gb300 import serve
from tests.netcases import assert_same

pytestmark = pytest.mark.gpu

T = 0.2  # epoch duration of the test jobs (2000 steps)


def make_jobs():
    return [serve.lif_growth_job(12, 2, seed=1, radius=2.0, epoch_duration=T),
            serve.izh_static_job(20, 15, 2, seed=2, epoch_duration=T),
            serve.lif_growth_job(20, 3, seed=3, radius=2.5, epoch_duration=T),
            serve.izh_static_job(10, 10, 1, seed=4, epoch_duration=T),
            serve.lif_growth_job(16, 1, seed=5, radius=1.6, epoch_duration=T)]


def run_alone(job):
    srv = serve.Server(max_resident=1, chunk_steps=700)
    srv.submit(job)
    done = srv.run_all()
    srv.close()
    assert done[0] is job and job.result.status == 0, job.error
    return job.outputs()


def check_same(a, b, name):
    for k in a:
        assert_same("%s %s" % (name, k), b[k], a[k])


def test_served_results_identical_alone_and_in_mix():
    alone = [run_alone(j) for j in make_jobs()]
    jobs = make_jobs()
    srv = serve.Server(max_resident=3, chunk_steps=300)
    for j in jobs[:2]:
        srv.submit(j)
    srv.pump()
    srv.pump()
    st = srv.stats()
    assert st["resident"] == 2 and st["rounds"] >= 1
    for j in jobs[2:]:          # arrive while the first two are on the GPU
        srv.submit(j)
    done = srv.run_all()
    st = srv.stats()
    srv.close()
    assert len(done) == len(jobs) and st["done"] == len(jobs) and st["failed"] == 0
    assert st["peak_resident"] == 3
    for j, a in zip(jobs, alone):
        assert j.result.status == 0 and j.result.error_word == 0, (j.name, j.error)
        assert j.result.synapse_steps > 0 or j.growth
        check_same(a, j.outputs(), j.name)
    assert sum(float(j.spikes_hist.sum()) for j in jobs) > 0


def test_admission_respects_the_device_budget():
    jobs = make_jobs()
    budget = max(j.footprint for j in jobs)
    srv = serve.Server(hbm_budget_bytes=budget, max_resident=8, chunk_steps=500)
    for j in jobs:
        srv.submit(j)
    done, waited = [], 0
    while len(done) < len(jobs):
        srv.pump()
        done += srv.take()
        st = srv.stats()
        assert st["bytes_resident"] <= budget
        waited = max(waited, st["queued"])
    srv.close()
    assert waited > 0 and st["peak_resident"] < len(jobs)
    assert all(j.result.status == 0 for j in jobs)


def test_job_larger_than_budget_is_rejected():
    j = make_jobs()[0]
    srv = serve.Server(hbm_budget_bytes=j.footprint - 1, max_resident=4)
    with pytest.raises(RuntimeError):
        srv.submit(j)
    srv.close()


def test_served_job_matches_plain_network():
    """The served job against the same network stepped epoch by epoch with bg3_step."""
    job = serve.lif_growth_job(20, 3, seed=3, radius=2.5, epoch_duration=T)
    served = run_alone(job)
    ref = serve.lif_growth_job(20, 3, seed=3, radius=2.5, epoch_duration=T)
    d = ref.desc
    net = bg.Network(d.n_neurons, d.max_syn_per_neuron, d.width, d.height, d.epoch_duration,
                     d.delta_t, d.max_firing_rate, d.max_epochs, d.synapse_kind, d.noise_mode,
                     d.noise_seed, neuron_kind=d.neuron_kind)
    ref.setup(net)
    assert net.device_bytes <= ref.footprint
    spe = int(np.float32(d.epoch_duration) / np.float32(d.delta_t))
    for e in range(ref.epochs):
        net.step(spe)
        net.growth(e + 1)
    b, s, rh, ra = net.download_histories()
    plain = dict(burstiness=b, spikes_hist=s, rates_hist=rh, radii_hist=ra,
                 Vm=net.download_lif(fields=("Vm",))["Vm"])
    for k in served:
        assert_same("plain vs served " + k, served[k][:len(plain[k])], plain[k])
    assert net.error_word == 0


def test_work_budget_backfills_small_jobs_past_a_large_one():
    """With a synapse-slot budget, a job that does not fit waits while later small jobs pass it,
    up to max_bypass times; every result is still the job's own."""
    big = [serve.lif_growth_job(20, 2, seed=11, radius=2.5, epoch_duration=T),
           serve.lif_growth_job(22, 2, seed=12, radius=2.5, epoch_duration=T)]
    small = [serve.izh_static_job(10, 10, 1, seed=13 + k, epoch_duration=T) for k in range(3)]
    alone = [run_alone(j) for j in (serve.lif_growth_job(20, 2, seed=11, radius=2.5, epoch_duration=T),
                                    serve.lif_growth_job(22, 2, seed=12, radius=2.5, epoch_duration=T))]
    cap = big[0].desc.n_neurons * big[0].desc.max_syn_per_neuron + 10000
    srv = serve.Server(max_resident=8, chunk_steps=400, max_resident_slots=cap, max_bypass=2)
    for j in big + small:
        srv.submit(j)
    srv.pump()
    st = srv.stats()
    # big[0] admitted; big[1] does not fit, the small jobs pass it (at most twice)
    assert st["resident"] == 3 and st["queued"] == 2
    done = srv.run_all()
    srv.close()
    assert len(done) == 5 and all(j.result.status == 0 for j in big + small)
    for j, a in zip(big, alone):
        check_same(a, j.outputs(), j.name)


def test_least_work_first_admission_with_aging():
    """ORDER_LEAST_WORK: with one job resident at a time the queued jobs are admitted least work
    (synapse slots x steps) first, except that a job passed over max_bypass times goes next; the
    results are the jobs' own either way."""
    def jobs():
        return [serve.lif_growth_job(20, 2, seed=21, radius=2.5, epoch_duration=T, name="big"),
                serve.izh_static_job(10, 10, 2, seed=22, epoch_duration=T, name="two"),
                serve.izh_static_job(10, 10, 1, seed=23, epoch_duration=T, name="one")]
    alone = [run_alone(j) for j in jobs()]
    for bypass, expect in ((8, ["one", "two", "big"]), (1, ["one", "big", "two"])):
        js = jobs()
        srv = serve.Server(max_resident=1, chunk_steps=400, max_bypass=bypass,
                           order=serve.ORDER_LEAST_WORK)
        for j in js:
            srv.submit(j)
        done = srv.run_all()
        srv.close()
        assert [j.name for j in done] == expect
        for j, a in zip(js, alone):
            assert j.result.status == 0
            check_same(a, j.outputs(), j.name)


@pytest.mark.parametrize("family", ["lif", "izh"])
def test_exported_job_resumes_bit_exact(family):
    """A job exported after 2 of 4 epochs and resumed as a new job, in another server and among
    other jobs, ends with the results of the same job run for 4 epochs in one go."""
    def job(epochs, **kw):
        if family == "lif":
            return serve.lif_growth_job(14, epochs, seed=7, radius=2.0, epoch_duration=T,
                                        max_epochs=4, **kw)
        return serve.izh_static_job(16, 12, epochs, seed=8, epoch_duration=T, max_epochs=4, **kw)
    want = run_alone(job(4))
    first = job(2, export=True)
    run_alone(first)
    ck = first.checkpoint()
    assert ck is not None and ck.size > 0
    second = job(4, resume=ck)
    srv = serve.Server(max_resident=3, chunk_steps=300)
    srv.submit(second)
    for j in make_jobs()[:2]:
        srv.submit(j)
    srv.run_all()
    srv.close()
    assert second.result.status == 0, second.error
    check_same(want, second.outputs(), "resumed " + family)
    # a checkpoint already at its last epoch leaves nothing to run: the job fails, no GPU work
    done = job(2, resume=ck)
    srv = serve.Server(max_resident=1, chunk_steps=300)
    srv.submit(done)
    srv.run_all()
    srv.close()
    assert done.result.status == bg.BG3_EINVAL


def test_sharded_trace_serves_every_job_once_with_unchanged_results():
    """The served stream split over two ranks (run here one after the other on one GPU): every
    job is served by exactly one rank and its results equal the job run alone."""
    alone = [run_alone(j) for j in make_jobs()]
    trace = [(0.02 * i, j) for i, j in enumerate(make_jobs())]
    index = {id(j): i for i, (_, j) in enumerate(trace)}
    seen = []
    for rank in range(2):
        part = serve.sharded_trace(trace, rank, 2)
        assert part, "both ranks get work"
        srv = serve.Server(max_resident=3, chunk_steps=300)
        times = serve.run_trace(srv, part)
        srv.close()
        for a, j in part:
            assert j.result.status == 0, (j.name, j.error)
            arrival, finish = times[j.id]
            assert arrival == a and finish >= a
            i = index[id(j)]
            check_same(alone[i], j.outputs(), "rank %d %s" % (rank, j.name))
            seen.append(i)
    assert sorted(seen) == list(range(len(trace)))


def test_cancelled_jobs_leave_the_others_unchanged():
    """A resident and a queued job cancelled between rounds: both come back with BG3_ECANCELED,
    their memory is freed, and the remaining jobs end exactly as they do alone."""
    alone = [run_alone(j) for j in make_jobs()]
    jobs = make_jobs()
    srv = serve.Server(max_resident=2, chunk_steps=300)
    for j in jobs:
        srv.submit(j)
    srv.pump()
    srv.pump()
    st = srv.stats()
    assert st["resident"] == 2 and st["queued"] == 3 and st["rounds"] == 1
    before = st["bytes_resident"]
    srv.cancel(jobs[1])  # resident, one chunk in
    srv.cancel(jobs[3])  # still queued
    assert srv.stats()["bytes_resident"] == before - bg.footprint(jobs[1].desc)
    with pytest.raises(bg.Bg3Error):
        srv.cancel(jobs[3])  # already gone
    done = srv.run_all()
    st = srv.stats()
    srv.close()
    assert len(done) == len(jobs) and st["cancelled"] == 2 and st["failed"] == 0
    for k, (j, a) in enumerate(zip(jobs, alone)):
        if k in (1, 3):
            assert j.result.status == bg.BG3_ECANCELED
        else:
            assert j.result.status == 0, (j.name, j.error)
            check_same(a, j.outputs(), j.name)


def test_bounded_device_wait_expires_with_a_status_and_the_context_survives():
    """The step kernels' bounded mbarrier wait, run on a barrier that nothing completes: it gives
    up after its limit, the kernel returns BG3_ERR_TIMEOUT, and the GPU keeps working."""
    L = bg.load()
    L.bg3_selftest_timeout.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32),
                                       ctypes.POINTER(ctypes.c_uint64)]
    for limit in (1_000_000, 50_000_000):
        status, waited = ctypes.c_uint32(), ctypes.c_uint64()
        assert L.bg3_selftest_timeout(limit, ctypes.byref(status), ctypes.byref(waited)) == 0
        assert status.value == bg.BG3_ERR_TIMEOUT
        assert limit <= waited.value < limit + 200_000_000
    status, waited = ctypes.c_uint32(), ctypes.c_uint64()
    assert L.bg3_selftest_timeout(0, ctypes.byref(status), ctypes.byref(waited)) == bg.BG3_EINVAL
    # the context is usable: a job runs as usual afterwards
    job = make_jobs()[0]
    out = run_alone(job)
    assert job.result.error_word == 0 and np.isfinite(out["Vm"]).all()
