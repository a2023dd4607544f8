"""Served form: the job server of libbg3 (include/bg3_serve.h) from Python.

A Job carries a network shape (bg3_net_desc), an epoch count, whether epochs end in growth, and a
setup function that fills the freshly created network through the usual Network methods.  The
server admits jobs by device footprint, keeps them resident across epochs and advances all of
them together with the batched kernels; results land in the job's numpy arrays.
"""
import ctypes

import numpy as np

from . import lib as bg
from . import netgen

SETUP_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p)


class ServeDesc(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_resident", ctypes.c_int32),
                ("chunk_steps", ctypes.c_int32), ("max_resident_slots", ctypes.c_uint64),
                ("max_bypass", ctypes.c_int32), ("order", ctypes.c_int32)]


ORDER_ARRIVAL, ORDER_LEAST_WORK = 0, 1  # bg3_serve_desc.order


class JobResult(ctypes.Structure):
    _fields_ = [(k, ctypes.POINTER(ctypes.c_float)) for k in
                ("burstiness", "spikes_hist", "rates_hist", "radii_hist", "Vm")] + \
               [("checkpoint", ctypes.c_void_p), ("checkpoint_cap", ctypes.c_uint64),
                ("checkpoint_len", ctypes.c_uint64),
                ("synapse_steps", ctypes.c_int64), ("neuron_steps", ctypes.c_int64),
                ("status", ctypes.c_int32), ("error_word", ctypes.c_uint32)]


class JobDesc(ctypes.Structure):
    _fields_ = [("desc", bg.NetDesc), ("epochs", ctypes.c_int32), ("growth", ctypes.c_int32),
                ("setup", SETUP_FN), ("user", ctypes.c_void_p),
                ("result", ctypes.POINTER(JobResult)),
                ("resume", ctypes.c_void_p), ("resume_len", ctypes.c_uint64)]


class ServeStats(ctypes.Structure):
    _fields_ = [("queued", ctypes.c_int64), ("resident", ctypes.c_int64), ("done", ctypes.c_int64),
                ("failed", ctypes.c_int64), ("cancelled", ctypes.c_int64),
                ("bytes_resident", ctypes.c_uint64),
                ("rounds", ctypes.c_int64), ("synapse_steps", ctypes.c_int64),
                ("neuron_steps", ctypes.c_int64), ("peak_resident", ctypes.c_int64),
                ("admit_s", ctypes.c_double), ("wait_s", ctypes.c_double),
                ("epoch_s", ctypes.c_double), ("rebuild_s", ctypes.c_double)]


_BOUND = False


def _bind():
    global _BOUND
    L = bg.load()
    if _BOUND:
        return L
    vp = ctypes.c_void_p
    sig = {
        "bg3_serve_create": ([ctypes.POINTER(ServeDesc), ctypes.POINTER(vp)], ctypes.c_int),
        "bg3_serve_destroy": ([vp], ctypes.c_int),
        "bg3_serve_submit": ([vp, ctypes.POINTER(JobDesc), ctypes.POINTER(ctypes.c_int64)],
                             ctypes.c_int),
        "bg3_serve_pump": ([vp], ctypes.c_int),
        "bg3_serve_cancel": ([vp, ctypes.c_int64], ctypes.c_int),
        "bg3_serve_take": ([vp, ctypes.POINTER(ctypes.c_int64), ctypes.c_int32,
                            ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
        "bg3_serve_stats_get": ([vp, ctypes.POINTER(ServeStats)], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    _BOUND = True
    return L


class Job:
    """One simulation: desc (bg.NetDesc), epochs, growth flag and setup(net) filling it.
    export=True keeps the finished job's whole state (checkpoint()); resume=<checkpoint> starts
    the job from an exported state (after setup), continuing its epoch count."""

    def __init__(self, desc, epochs, growth, setup, name="", export=False, resume=None):
        self.desc, self.epochs, self.growth, self.setup, self.name = desc, epochs, growth, setup, name
        N, E, T = desc.n_neurons, desc.max_epochs, desc.epoch_duration
        nb = int(np.float32(E) * np.float32(T))
        ns = int(np.float32(E) * np.float32(T) * np.float32(100))
        self.burstiness = np.zeros(max(nb, 1), np.float32)
        self.spikes_hist = np.zeros(max(ns, 1), np.float32)
        self.rates_hist = np.zeros((E + 1) * N, np.float32)
        self.radii_hist = np.zeros((E + 1) * N, np.float32)
        self.Vm = np.zeros(N, np.float32)
        self.result = JobResult(*[bg._p(a) for a in (self.burstiness, self.spikes_hist,
                                                      self.rates_hist, self.radii_hist, self.Vm)])
        self._ckpt = None
        if export:
            # the state is the job's device arrays plus a small header
            self._ckpt = np.empty(bg.footprint(desc) + (1 << 20), np.uint8)
            self.result.checkpoint = self._ckpt.ctypes.data
            self.result.checkpoint_cap = self._ckpt.size
        self._resume = None if resume is None else np.ascontiguousarray(
            np.frombuffer(resume, np.uint8))
        self.id = None
        self.error = None

    def checkpoint(self):
        """The exported state of a finished job (export=True)."""
        if self._ckpt is None:
            return None
        return self._ckpt[:self.result.checkpoint_len].copy()

    @property
    def footprint(self):
        return bg.footprint(self.desc)

    def outputs(self):
        return dict(burstiness=self.burstiness, spikes_hist=self.spikes_hist,
                    rates_hist=self.rates_hist, radii_hist=self.radii_hist, Vm=self.Vm)


class Server:
    def __init__(self, hbm_budget_bytes=150 << 30, max_resident=64, chunk_steps=2000,
                 max_resident_slots=0, max_bypass=8, order=ORDER_ARRIVAL):
        self.L = _bind()
        d = ServeDesc(int(hbm_budget_bytes), int(max_resident), int(chunk_steps),
                      int(max_resident_slots), int(max_bypass), int(order))
        h = ctypes.c_void_p()
        bg.check(self.L.bg3_serve_create(ctypes.byref(d), ctypes.byref(h)), "bg3_serve_create")
        self.h = h
        self.jobs = {}
        self._keep = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.bg3_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, job):
        def cb(handle, user, job=job):
            try:
                job.setup(bg.Network.borrow(handle, job.desc))
                return 0
            except Exception as e:  # reported through the job's status
                job.error = e
                return bg.BG3_EINVAL
        fn = SETUP_FN(cb)
        jd = JobDesc(job.desc, job.epochs, 1 if job.growth else 0, fn, None,
                     ctypes.pointer(job.result))
        if job._resume is not None:
            jd.resume = job._resume.ctypes.data
            jd.resume_len = job._resume.size
        jid = ctypes.c_int64()
        bg.check(self.L.bg3_serve_submit(self.h, ctypes.byref(jd), ctypes.byref(jid)),
                 "bg3_serve_submit")
        job.id = jid.value
        self.jobs[job.id] = job
        self._keep[job.id] = (fn, jd)
        return job.id

    def pump(self):
        bg.check(self.L.bg3_serve_pump(self.h), "bg3_serve_pump")

    def cancel(self, job):
        """Cancels a queued or resident job (bg3_serve_cancel); take() then returns it with
        status BG3_ECANCELED."""
        bg.check(self.L.bg3_serve_cancel(self.h, int(job.id)), "bg3_serve_cancel")

    def take(self):
        ids = (ctypes.c_int64 * 256)()
        n = ctypes.c_int32()
        out = []
        while True:
            bg.check(self.L.bg3_serve_take(self.h, ids, 256, ctypes.byref(n)), "bg3_serve_take")
            for k in range(n.value):
                jid = ids[k]
                self._keep.pop(jid, None)
                out.append(self.jobs.pop(jid))
            if n.value < 256:
                return out

    def stats(self):
        s = ServeStats()
        bg.check(self.L.bg3_serve_stats_get(self.h, ctypes.byref(s)), "bg3_serve_stats_get")
        return {k: getattr(s, k) for k, _ in ServeStats._fields_}

    def run_all(self):
        """Pumps until every submitted job has finished; returns them in completion order."""
        done = []
        while self.jobs:
            self.pump()
            done += self.take()
        return done


# ---- arrival traces ---------------------------------------------------------------------------
def run_trace(srv, trace, clock=None, sleep=None):
    """Serves an open-loop arrival trace [(arrival_s, job)] (ascending arrivals) on srv in real
    time: each job is submitted once the clock passes its arrival.  Returns {job.id: (arrival_s,
    finish_s)} on the trace's clock (finish = when bg3_serve_take reported it)."""
    import time
    clock = clock or time.perf_counter
    sleep = sleep or time.sleep
    pending = list(trace)
    arrival, out = {}, {}
    t0 = clock()
    while pending or srv.jobs:
        now = clock() - t0
        while pending and pending[0][0] <= now:
            a, job = pending.pop(0)
            srv.submit(job)
            arrival[job.id] = a
        if not srv.jobs:
            sleep(max(0.0, pending[0][0] - (clock() - t0)))
            continue
        srv.pump()
        now = clock() - t0
        for job in srv.take():
            out[job.id] = (arrival[job.id], now)
    return out


def sharded_trace(trace, rank, world):
    """The part of a trace that rank `rank` of `world` serves: jobs bin packed by work (synapse
    slots x simulated seconds), arrival times kept.  Every rank computes the same split."""
    from . import shard
    w = [shard.job_weight(job.desc, job.epochs) for _, job in trace]
    return [trace[i] for i in shard.partition(w, world)[rank]]


# ---- job families of the served stream -------------------------------------------------------
def lif_growth_job(side, epochs, seed, radius=None, weight_scale=0.003, target_rate=1.0,
                   frac_inh=0.10, max_syn=None, epoch_duration=1.0, max_epochs=None, name="",
                   max_firing_rate=1000, **job_kw):
    """The LIF growth family: LIF + DS + ConnGrowth on a side x side grid, pre-grown to
    radius (mean in-degree ~ pi (2 radius)^2, capped by max_syn), growth at every epoch end.
    The first growth pass sets the weights from the overlap areas unscaled, after which the
    larger networks fire at ~300 Hz: the spike-history ring is sized for max_firing_rate."""
    spec_args = dict(frac_inh=frac_inh, seed=seed)
    N = side * side
    if radius is None:
        radius = min(8.4, 0.45 * side)
    if max_syn is None:
        # in-degree ~ pi (2 radius)^2; the slack keeps growth from filling a row
        max_syn = int(min(1000, N, np.ceil(np.pi * (2 * radius + 2.0) ** 2 / 4) * 4))
        max_syn = max(4, (max_syn + 3) // 4 * 4)
    desc = bg.NetDesc(N, max_syn, side, side, epoch_duration, 1e-4, max_firing_rate,
                      max_epochs or epochs, bg.BG3_NEURON_LIF, bg.BG3_SYN_DS, bg.BG3_NOISE_DEVICE,
                      seed + 101)

    def setup(net):
        spec = netgen.lif_network(side, side, **spec_args)
        netgen.configure_lif(net, spec, dict(target_rate=target_rate))
        netgen.pregrow(net, spec, radius, weight_scale=weight_scale, seed=seed + 11)
    return Job(desc, epochs, True, setup, name or "lif%dx%d" % (side, side), **job_kw)


def config_job(config, stim=None, root=None, epochs=None, name="", **job_kw):
    """A job from a BrainGrid parameter file (and stimulus file): the network the reference's
    setup makes from it (braingrid_gb300.config), its numSims epochs (or epochs) of Tsim seconds,
    growth at each epoch end for ConnGrowth, the plain recorder otherwise; device noise keyed by
    the file's seed.  config may also be an already read config.Params."""
    from . import config as cf
    p = config if isinstance(config, cf.Params) else cf.read(config, stim, root)
    a = cf.setup(p)
    desc = cf.desc(p)

    def setup(net):
        cf.configure(net, p, a)
    return Job(desc, epochs or p.epochs, p.conn_class == "ConnGrowth", setup,
               name or "config%dx%d" % (p.width, p.height), **job_kw)


def izh_static_job(width, height, epochs, seed, epoch_duration=1.0, max_epochs=None, name="",
                   **job_kw):
    """The Izhikevich + STDP family: Izhikevich neurons, static wiring (10 nearest within radius 5,
    10 % rewired), dynamic STDP, Poisson drive at 10 Hz / 5 nA; epochs end in the recorder."""
    spec, syn, counts, M = netgen.izh_static_spec(width, height, seed)
    desc = bg.NetDesc(spec["N"], M, width, height, epoch_duration, 1e-4, 1000,
                      max_epochs or epochs, bg.BG3_NEURON_IZH, bg.BG3_SYN_DYNSTDP,
                      bg.BG3_NOISE_DEVICE, seed)

    def setup(net):
        netgen.configure_izh_static(net, spec, syn, counts, input_seed=seed)
    return Job(desc, epochs, False, setup, name or "izh%dx%d" % (width, height), **job_kw)
