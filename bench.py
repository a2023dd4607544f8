"""Benchmark of the spiking hot path on one GB300: synapse-updates/s (and neuron-steps/s).

Workload (the headline): the plain single-network step of a 100x100 = 10,000 neuron LIF +
AllDSSynapses + ConnGrowth network, max 1,000 synapses per neuron, dt 0.1 ms, excitatory fraction
0.90, targetRate 1.0 Hz, seed 7, synthetic parameters with the stated value distributions
(braingrid_gb300.netgen).  Connectivity is pre-grown (at the stated 0.4 start
radius no pair overlaps, so no synapse would ever form): radii ~ U[8.35, 8.45] and one device
growth pass wire every overlapping pair (~7.6 M synapses, up to ~884 per neuron); weights =
overlap area x 1e-8 x 0.0003, and every neuron gets a Poisson drive (the reference's
SInputPoisson, 10 Hz, weight 9.5), which holds the network at about the growth rule's 1 Hz target
rate (~1,000 spike arrivals per step).  A "step" is one simulation time step of the whole network:
one neuron pass, one spike-delivery pass and one synapse sweep with summation (the neuron pass
of step t + 1 runs in the epilogue of sweep t; the first step's runs standalone).  L2 is flushed (256 MiB write)
before every timed step; device time per step comes from CUDA events on the library's stream.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl bg3|reference]
                    [--serve-jobs J] [--serve-slots S] [--only izh512|serve|growth]

Beside the headline the line carries the batched forms of the 36-network growth sweep (36 LIF
networks) and of the 512-network Izhikevich + STDP batch, the served stream (a J-job trace through
the job server, against the same jobs one at a time) and the growth pass.

--impl reference times the reference algorithm's CPU path (the C restatement in oracle/, the
reference's own sources are not on the GPU host) on the same network, single-threaded as the
reference is.  Under torchrun every rank runs an independent replica of the headline (the path
does not shard within a network) and a share of the batched and served work (shard.py); value is
the sum over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from braingrid_gb300.workloads import PLAIN  # noqa: E402

WIDTH, HEIGHT, MAX_SYN = PLAIN["width"], PLAIN["height"], PLAIN["max_syn"]
RADIUS, WEIGHT_SCALE, SEED = PLAIN["radius"], PLAIN["weight_scale"], PLAIN["seed"]
POISSON = PLAIN["poisson"]
WORKLOAD = ("plain single-network step: 100x100 LIF + DS + ConnGrowth, max 1000 synapses/neuron, "
            "pre-grown radius U[8.35,8.45], weight scale %g, Poisson drive %g Hz x weight %g"
            % (WEIGHT_SCALE, POISSON["fr_mean"], POISSON["weight"]))
FLUSH_BYTES = 256 << 20
METRIC = "synapse-updates/s"
# Algorithmic bytes of the dominant kernel (k_sweep, with the next step's neuron pass fused in):
# every in-use synapse's psr is read and written and its decay class (4 bits) read; every neuron
# reads Vm, Vthresh, I0, Inoise, C1, C2, Trefract, refr and writes Vm, refr, sp (44 B, rounded
# to 48 with the spike-ring entry), and its Poisson input synapse reads mask, interval counter,
# queue word, psr, decay and delay and writes counter, queue word and psr (30 B).  The reference
# layout's per-synapse figure (psr, decay, queue word, delay index read; psr, queue, delay index
# written: 28 B) is reported beside it.
SWEEP_BYTES_PER_SYN = 8.5
SWEEP_BYTES_PER_NEURON = 48 + 30
# the batched workloads' neuron passes: LIF without input (the growth sweep) 48 B; Izhikevich
# (reads Vm, Vthresh, refr, Trefract, I0, Inoise, C2, a, b, c, d, u, C3 and writes Vm, u: 60 B)
# with its Poisson input synapse (30 B) and the tile's row counts (4 B): 94 B
SWEEP36_BYTES_PER_NEURON = 48
IZH_BYTES_PER_NEURON = 60 + 30 + 4
REF_LAYOUT_BYTES_PER_SYN = 28
# served form: resident work cap, about one and a half of the largest jobs' synapse slots
SERVE_SLOTS = 60e6
SERVED_LONG_JOBS = 64  # the second served trace: 64 jobs at epochs of 0.1 s
SERVE_ORDER = 0  # admission in arrival order with backfill (bg3_serve_desc.order)
# steps of a call long enough to capture and instantiate the library's 32-step graph, so that
# the timed calls only replay it
GRAPH_WARMUP = 40
# the izh512 networks' firing rate rises from ~1 Hz to a steady ~15 Hz over their first ~1,200
# steps as STDP strengthens their synapses: they run this many steps before they are tuned and
# timed, so that the figures are the steady state's
IZH_SETTLE = 2000


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile(prefix="bg3clk", suffix=".csv", delete=False)
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.close()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def build_network():
    from braingrid_gb300 import workloads
    return workloads.build(workloads.PLAIN)


def traffic_per_launch(S):
    """DRAM bytes per sweep launch from the committed ncu capture, scaled by synapse count."""
    p = os.path.join(ROOT, "profiles", "sweep_traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return float(d["dram_bytes_per_launch"]) * S / float(d["synapses"])


def cpu_baseline_port(net, spec, budget_s=12.0):
    """Time the oracle (reference algorithm, C, one core) on the same network state."""
    from oracle import pyoracle as po
    from braingrid_gb300 import lib as bg
    N = spec["N"]
    o = po.OracleNet(N, MAX_SYN, WIDTH, HEIGHT, 1.0, 1e-4, 200, 10)
    g = net.download_lif()
    s = net.download_synapses()
    for k, v in (("Vm", "Vm"), ("Vthresh", "Vthresh"), ("Vreset", "Vreset"), ("I0", "I0"),
                 ("Inoise", "Inoise"), ("C1", "C1"), ("C2", "C2"), ("Trefract", "Trefract"),
                 ("sp", "summation"), ("refr", "nStepsInRefr"), ("spikeCount", "spikeCount"),
                 ("spikeCountOffset", "spikeCountOffset")):
        o.arr(k)[:] = g[v]
    o.arr("history")[:] = g["history"]
    for k, v in (("in_use", "in_use"), ("src", "src"), ("type", "type"), ("W", "W"),
                 ("psr", "psr"), ("decay", "decay"), ("total_delay", "total_delay"),
                 ("queue", "delayQueue"), ("delayIdx", "delayIdx"), ("U", "U"), ("D", "D"),
                 ("F", "F"), ("u", "u"), ("r", "r"), ("lastSpike", "lastSpike")):
        o.arr(k)[:] = s[v]
    o.arr("ldelayQueue")[:] = 32
    o.arr("counts")[:] = s["counts"]
    o.arr("ntype")[:] = spec["ntype"]
    o.step = net.sim_step
    o.rebuild_maps()
    o.input_poisson(POISSON["fr_mean"], POISSON["weight"])  # same drive, the oracle's own draws
    S = o.total
    t0 = time.perf_counter()
    o.step_n(1)
    one = time.perf_counter() - t0
    n = max(1, min(400, int(budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    o.step_n(n)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": S * n / dt, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": "%d steps of the same %d-neuron / %d-synapse network (oracle C port, one "
                      "thread; host has %d cores)" % (n, N, S, os.cpu_count() or 0),
            "neuron_steps_per_s": N * n / dt}


def run_bg3(args):
    rank, world, local = dist_env()
    import torch  # plumbing: device selection, pinned host buffers, barrier for N>1
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from braingrid_gb300 import lib as bg
    from braingrid_gb300 import shard
    spec, net = build_network()
    N = spec["N"]
    S = net.total_synapses()
    maps = net.download_maps()
    fan = maps["outgoingSynapseCount"].astype(np.int64)
    # clocks sampled from here to the end of the headline's GPU work (the timed steps alone
    # last well under the sampler's 200 ms period)
    clk = ClockSampler(local) if rank == 0 else None
    # 0.5 s of simulated time for the driven network to settle, then the rate over the next
    # 0.5 s (the timed window itself is too short to estimate a 1 Hz rate)
    net.step(5000)
    s0 = net.download_lif(fields=("spikeCount",))["spikeCount"].astype(np.int64)
    net.step(5000)
    s1 = net.download_lif(fields=("spikeCount",))["spikeCount"].astype(np.int64)
    rate_hz = float((s1 - s0).mean()) / 0.5
    deliveries = float(((s1 - s0) * fan).sum()) / 5000
    # launch configuration chosen by the autotuner on this network's state (left unchanged)
    launch, _ = net.autotune(steps_per_trial=200)
    # warm-up: W benchmark steps (the state keeps running, so the rate holds)
    net.bench_steps(args.warmup, FLUSH_BYTES)
    c0 = net.download_lif(fields=("spikeCount",))["spikeCount"].astype(np.int64)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ms = net.bench_steps(args.steps, FLUSH_BYTES)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    c1 = net.download_lif(fields=("spikeCount",))["spikeCount"].astype(np.int64)
    t_total = float(np.sum(ms)) / 1e3
    # whole job: units of every replica over the slowest replica's time (no-op at N = 1)
    _, t_total = shard.reduce_timing(S * args.steps, t_total, device="cuda")
    timed_deliveries = float(((c1 - c0) * fan).sum()) / args.steps
    value = S * args.steps * world / t_total
    # roofline of the dominant kernel (the sweep): a second timed pass right after the first,
    # with an extra CUDA event between spike delivery and the sweep of every step
    _, km = net.bench_steps(min(args.steps, 2000), FLUSH_BYTES, per_kernel=True)
    sweep_ms = float(np.mean(km[:, 2]))
    shares = np.sum(km, axis=0) / np.sum(km)
    peak, peak_kind = peaks()
    alg_bytes = SWEEP_BYTES_PER_SYN * S + SWEEP_BYTES_PER_NEURON * N
    achieved = alg_bytes / (sweep_ms * 1e-3) / 1e9
    ref_layout_achieved = (REF_LAYOUT_BYTES_PER_SYN * S + 4 * N) / (sweep_ms * 1e-3) / 1e9
    size_matched = size_matched_copy(alg_bytes)
    # end to end through the C-ABI with pinned host buffers: every iteration uploads the neuron
    # state (H2D), advances E2E_STEPS steps and reads back the spike counts and history (D2H)
    E2E_STEPS = 500
    e2e_iters = max(2, min(10, args.steps // 100))
    pin = {}
    st = net.download_lif()
    for k in ("Vm", "Vthresh", "Vreset", "I0", "Inoise", "C1", "C2", "Trefract", "summation",
              "nStepsInRefr", "spikeCount", "spikeCountOffset"):
        t = torch.empty(N, dtype=torch.float32 if st[k].dtype == np.float32 else torch.int32,
                        pin_memory=True)
        t.numpy()[:] = st[k]
        pin[k] = t
    out_counts = torch.empty(N, dtype=torch.int32, pin_memory=True).numpy()
    h2d = sum(v.numel() * v.element_size() for v in pin.values())
    d2h = N * 4
    net.sync()
    t0 = time.perf_counter()
    for _ in range(e2e_iters):
        net.upload_lif(**{k: v.numpy() for k, v in pin.items()})
        net.step(E2E_STEPS)
        net.download_lif(fields=("spikeCount",), out={"spikeCount": out_counts})
    net.sync()
    e2e_s = time.perf_counter() - t0
    _, e2e_s = shard.reduce_timing(0, e2e_s, device="cuda")
    clocks = clk.stop() if clk else None
    if clocks is not None:
        clocks["span"] = "settle, autotune, timed steps, roofline pass and e2e of the headline"
    e2e = {"value": S * E2E_STEPS * e2e_iters * world / e2e_s, "unit": METRIC,
           "h2d_bytes_per_step": h2d / E2E_STEPS, "d2h_bytes_per_step": d2h / E2E_STEPS,
           "l2": "not evicted between steps: consecutive steps of one run, whose per-step state "
                 "(%.0f MB) fits the 129 MB L2" % (alg_bytes / 1e6)}
    err = net.error_word
    batched = izh_stdp = served = served64 = growth = small = None
    if world == 1:
        growth = run_growth()
        small = run_small()
        batched = run_batched(min(args.steps, 500), max(args.warmup, 20))
        izh_stdp = run_izh512(min(args.steps, 1000), max(args.warmup, 20))
        if args.serve_jobs > 0:
            served = run_served(args.serve_jobs, int(args.serve_slots), order=SERVE_ORDER)
            # a longer trace within the run's time: 64 jobs of the same families and epoch
            # counts, at epochs of 0.1 s
            served64 = run_served(SERVED_LONG_JOBS, int(args.serve_slots), epoch_duration=0.1,
                                  order=SERVE_ORDER)
    else:
        # the batched and served forms spread over the ranks by instance (bin packed, no
        # collective); whole-job figures over the slowest rank
        batched = run_batch_sharded("sweep36", rank, world, min(args.steps, 500),
                                    max(args.warmup, 20))
        izh_stdp = run_batch_sharded("izh512", rank, world, min(args.steps, 1000),
                                     max(args.warmup, 20))
        if args.serve_jobs > 0:
            served = run_served_sharded(args.serve_jobs, int(args.serve_slots), rank, world)
    if rank == 0:
        cpu = cpu_baseline_port(net, spec)
        tr = traffic_per_launch(S)
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_total * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "neurons": N, "synapses": S, "dt_s": 1e-4, "noise": "device",
                       "input": "Poisson %g Hz, weight %g, every neuron" % (POISSON["fr_mean"],
                                                                           POISSON["weight"]),
                       "l2": "flushed (256 MiB write) before every timed step",
                       "mean_rate_hz": rate_hz, "deliveries_per_step": deliveries,
                       "rate_window": "5,000 steps after a 5,000-step settle",
                       "timed_deliveries_per_step": timed_deliveries,
                       "launch": launch,
                       "parallelism": "replicas" if world > 1 else "single"},
            "neuron_steps_per_s": N * args.steps * world / t_total,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": tr,
                         "traffic_kind": "DRAM bytes read per launch from the committed ncu "
                                         "capture (profiles/sweep_traffic.json), scaled by "
                                         "synapses; the psr writes stay in L2 and leave at the "
                                         "next eviction, outside the launch",
                         "kernel": "k_sweep",
                         "peak_kind": peak_kind, "launch_ms": sweep_ms,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "bytes_per_synapse": SWEEP_BYTES_PER_SYN,
                         "reference_layout_bytes_per_synapse": REF_LAYOUT_BYTES_PER_SYN,
                         "reference_layout_equivalent_gbs": ref_layout_achieved,
                         "size_matched_copy": dict(size_matched,
                                                   frac=achieved / size_matched["gbs"]),
                         "kernel_shares": {"neurons": float(shares[0]), "deliver": float(shares[1]),
                                           "sweep": float(shares[2])}},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "growth": growth,
            "small_network": small,
            "batched": batched,
            "batched_izh_stdp": izh_stdp,
            "served": served,
            "served_64_jobs": served64,
            "gpu_launches": 2 * args.steps + 1,
            "clocks": clocks,
            "error_word": err,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def _alg_gbs(S, N, bytes_per_neuron, seconds_per_step):
    """Algorithmic GB/s of a batched step: 8.5 B per synapse and the neuron pass's bytes."""
    return (SWEEP_BYTES_PER_SYN * S + bytes_per_neuron * N) / seconds_per_step / 1e9


def _batch_graph_seconds(batch, steps):
    """Host wall clock around batch.step(steps): the path a caller runs (CUDA graphs of 32 fused
    steps, each step's sweep overlapping the kernels before it), synchronised on both sides,
    after a call that builds the batch's step graph."""
    import time as _t
    batch.step(GRAPH_WARMUP)
    batch.sync()
    t0 = _t.perf_counter()
    batch.step(steps)
    batch.sync()
    return _t.perf_counter() - t0


def run_batched(steps, warmup):
    """The 36-network growth sweep as one batch (one launch per kernel per step) against the
    same networks run one network at a time with bg3_step (each on its own CUDA graph)."""
    import time as _t
    from braingrid_gb300 import lib as bg
    from braingrid_gb300 import workloads
    members = workloads.sweep36_members()
    nets = [workloads.build_member(w)[1] for w in members]
    S = sum(n.total_synapses() for n in nets)
    N = sum(n.N for n in nets)
    batch = bg.Batch(nets)
    launch, _ = batch.autotune(steps_per_trial=100)
    batch.step(warmup)
    batch.sync()
    # batched: device time per step with CUDA events (the working set, ~1 GB, exceeds L2)
    ms = batch.bench_steps(steps)
    t_batch = float(np.sum(ms)) / 1e3
    t_graph = _batch_graph_seconds(batch, steps)
    # plain: every network advanced on its own for the same number of steps, back to back
    for n in nets:
        n.step(max(warmup, GRAPH_WARMUP))  # builds each network's step graph before timing
    for n in nets:
        n.sync()
    t0 = _t.perf_counter()
    for n in nets:
        n.step(steps)
    for n in nets:
        n.sync()
    t_plain = _t.perf_counter() - t0
    # plain lock-step: every step, each network advanced by its own bg3_step(1) call
    lock = min(steps, 100)
    t0 = _t.perf_counter()
    for _ in range(lock):
        for n in nets:
            n.step(1)
    for n in nets:
        n.sync()
    t_lock = (_t.perf_counter() - t0) / lock
    err = max(n.error_word for n in nets)
    out = {"workload": "36-network growth sweep: 9 each of 30x30, 50x50, 70x70, 100x100 "
                       "(targetRate x excitatory fraction x 4 seeds), pre-grown as the headline "
                       "network",
           "networks": len(nets), "neurons": N, "synapses": S, "steps": steps,
           "settle_steps": IZH_SETTLE,
           "batched_synapse_updates_per_s": S * steps / t_batch,
           "batched_neuron_steps_per_s": N * steps / t_batch,
           "batched_ms_per_step": t_batch * 1e3 / steps,
           "batched_sweep_gbs": _alg_gbs(S, N, SWEEP36_BYTES_PER_NEURON, t_batch / steps),
           "batched_frac_of_peak": _alg_gbs(S, N, SWEEP36_BYTES_PER_NEURON, t_batch / steps) /
                                   peaks()[0],
           "algorithmic_bytes_per_step": SWEEP_BYTES_PER_SYN * S + SWEEP36_BYTES_PER_NEURON * N,
           "bytes_per_synapse": SWEEP_BYTES_PER_SYN, "bytes_per_neuron": SWEEP36_BYTES_PER_NEURON,
           "plain_synapse_updates_per_s": S * steps / t_plain,
           "plain_neuron_steps_per_s": N * steps / t_plain,
           "plain_ms_per_step": t_plain * 1e3 / steps,
           "plain_timing": "host wall clock around 36 sequential bg3_step runs (each a CUDA graph)",
           "plain_lockstep_synapse_updates_per_s": S / t_lock,
           "plain_lockstep_ms_per_step": t_lock * 1e3,
           "plain_lockstep_timing": "host wall clock, %d steps of 36 bg3_step(1) calls" % lock,
           "batched_over_plain": t_plain / t_batch,
           "batched_over_plain_lockstep": t_lock * steps / t_batch,
           "batched_timing": "CUDA events around each step (the step's kernels launched one by "
                             "one, the next step's sweep not overlapping them)",
           "batched_graph_ms_per_step": t_graph * 1e3 / steps,
           "batched_graph_synapse_updates_per_s": S * steps / t_graph,
           "batched_graph_timing": "host wall clock around one bg3_batch_step call (CUDA graphs "
                                   "of 32 steps), as the plain form",
           "batched_graph_over_plain": t_plain / t_graph, "error_word": int(err),
           "launch": launch}
    batch.close()
    for n in nets:
        n.close()
    return out


def size_matched_copy(traffic_bytes, reps=25):
    """A plain device copy moving the same bytes as one sweep launch (half read, half written),
    L2 evicted before each copy like the timed steps; median of reps, CUDA events.  The measured
    peak comes from a copy of gigabytes; at tens of megabytes a copy's own start and tail show."""
    import torch
    n = max(1, int(traffic_bytes) // 8)  # float32 elements each way
    a = torch.ones(n, device="cuda")
    b = torch.empty_like(a)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    scrub = torch.zeros(FLUSH_BYTES // 4, device="cuda")
    ts = []
    for r in range(reps):
        flush.fill_(r & 0xff)
        scrub.sum()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.copy_(a)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    ms = float(np.median(ts))
    del a, b, flush, scrub
    return {"bytes": 8 * n, "ms": ms, "gbs": 8 * n / (ms * 1e-3) / 1e9,
            "how": "torch copy_ of %d MB into %d MB, L2 evicted before each, median of %d"
                   % (4 * n >> 20, 4 * n >> 20, reps)}


def run_batch_sharded(which, rank, world, steps, warmup):
    """The 36-network sweep ("sweep36") or the 512-network Izhikevich batch ("izh512") over N GPUs: each rank builds and batches its share of the networks
    (bin packed by synapse slots, the same split on every rank) and times its own batch; the
    whole-job rate is every rank's synapse-steps over the slowest rank's time."""
    from braingrid_gb300 import lib as bg
    from braingrid_gb300 import netgen, shard, workloads
    if which == "sweep36":
        members = workloads.sweep36_members()
        weights = [m["width"] * m["height"] * m["max_syn"] for m in members]
        mine = shard.share(list(range(len(members))), weights, rank, world)
        nets = [workloads.build_member(members[i])[1] for i in mine]
    else:
        shapes = workloads.izh512_shapes()
        weights = [w * h for w, h in shapes]
        mine = shard.share(list(range(len(shapes))), weights, rank, world)
        nets = [netgen.make_izh_static(shapes[k][0], shapes[k][1], seed=1000 + k,
                                       max_epochs=10)[1] for k in mine]
    S = sum(n.total_synapses() for n in nets)
    N = sum(n.N for n in nets)
    t = 0.0
    if nets:
        batch = bg.Batch(nets)
        batch.autotune(steps_per_trial=100)
        batch.step(warmup)
        batch.sync()
        t = float(np.sum(batch.bench_steps(steps))) / 1e3
        batch.close()
    for n in nets:
        n.close()
    units, t_max = shard.reduce_timing(S * steps, t, device="cuda")
    neuron_units, _ = shard.reduce_timing(N * steps, t, device="cuda")
    return {"workload": "%s sharded over %d GPUs by instance (%d networks on rank %d)"
                        % (which, world, len(mine), rank),
            "batched_synapse_updates_per_s": units / t_max if t_max > 0 else None,
            "batched_neuron_steps_per_s": neuron_units / t_max if t_max > 0 else None,
            "batched_ms_per_step": t_max * 1e3 / steps, "steps": steps}


def run_served_sharded(n_jobs, slots_cap, rank, world, chunk_steps=2000):
    """The served stream over N GPUs: every rank serves its share of the same trace (jobs bin packed by
    work, arrival times kept) with its own job server; latencies are gathered on rank 0."""
    from braingrid_gb300 import serve, shard, workloads
    trace = serve.sharded_trace(workloads.served_trace(n_jobs), rank, world)
    srv = serve.Server(hbm_budget_bytes=workloads.SERVED_BUDGET, max_resident=64,
                       chunk_steps=chunk_steps, max_resident_slots=slots_cap, order=SERVE_ORDER)
    shard.barrier()  # one trace clock for all ranks
    times = serve.run_trace(srv, trace) if trace else {}
    srv.close()
    mine = [(job.name, times[job.id][0], times[job.id][1], int(job.result.synapse_steps),
             int(job.result.status), int(job.result.error_word)) for _, job in trace]
    every = shard.gather(mine)
    if every is None:
        return None
    rows = [r for part in every for r in part]
    lat = [r[2] - r[1] for r in rows]
    span = max(r[2] for r in rows) - min(r[1] for r in rows)
    pct = shard.latency_percentiles(lat)
    syn = sum(r[3] for r in rows)
    return {"workload": "served stream: %d-job trace sharded over %d GPUs by job work" % (n_jobs, world),
            "jobs": len(rows), "all_ok": all(r[4] == 0 and r[5] == 0 for r in rows),
            "served_p50_s": pct["p50"], "served_p95_s": pct["p95"], "served_p99_s": pct["p99"],
            "served_makespan_s": span, "served_synapse_updates_per_s": syn / span,
            "jobs_per_rank": [len(part) for part in every]}


def _sm_max_mhz():
    """Maximum SM clock from MEASURED_PEAKS.json (2070 MHz on GB300 if absent)."""
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["sm_max_mhz"])
    except (OSError, KeyError, ValueError):
        return 2070.0


def _growth_passes(width, height, radius):
    """Pass times (s) of one network: at the stated start radius 0.4 (every pair rejected), at
    pre-grown radii U[radius - 0.05, radius + 0.05] creating the synapses, and once more at those
    radii updating them.  Host wall clock around a synchronised pass."""
    import time as _t
    from braingrid_gb300 import netgen
    spec = netgen.lif_network(width, height, frac_inh=0.10, seed=SEED)
    net = netgen.make_gpu_network(spec, MAX_SYN, noise_seed=SEED)
    N = spec["N"]

    def timed(epoch):
        net.sync()
        t0 = _t.perf_counter()
        net.growth(epoch)
        net.sync()
        return _t.perf_counter() - t0
    timed(1)  # first pass loads the module's kernels
    t_reject = timed(2)
    rs = np.random.RandomState(11)
    r = rs.uniform(radius - 0.05, radius + 0.05, N).astype(np.float32)
    g = netgen.GROWTH
    net.upload_growth(g["epsilon"], g["beta"], g["rho"], g["target_rate"], g["min_radius"],
                      g["start_radius"], r)
    t_create = timed(3)
    S = net.total_synapses()
    t_update = timed(4)
    err = net.error_word
    net.close()
    return N, t_reject, t_create, t_update, S, err


def run_growth():
    """ConnGrowth epoch pass (radii update, O(N^2) overlap scan, weight update / synapse
    creation, map rebuild, recorder) on the headline network (10^8 pairs) and on the served
    stream's largest job, 200x200 (1.6e9 pairs): at the stated start radius 0.4 (every pair
    rejected), at the pre-grown radii U[8.35, 8.45] creating the synapses, and once more at those
    radii updating them."""
    N, t_reject, t_create, t_update, S, err = _growth_passes(WIDTH, HEIGHT, RADIUS)
    # FP32 roofline of the rejecting pass: 8 FP32 operations per pair (dx, dy, d^2, the radius
    # sum and the comparison) against the FP32 pipe's peak, 128 lanes x 152 SMs x the SM clock
    # (no FMA: the library is compiled without contraction); the pass also holds the radii
    # update, the map rebuild and the recorder, so this understates the overlap kernel alone
    clk = _sm_max_mhz() * 1e6
    fp32_peak = 128 * 152 * clk
    out = {"pairs": N * N, "radius_0.4_s": t_reject, "radius_0.4_pairs_per_s": N * N / t_reject,
           "radius_0.4_fp32_ops_per_s": 8 * N * N / t_reject,
           "fp32_pipe_peak_ops_per_s": fp32_peak,
           "radius_0.4_fp32_frac": 8 * N * N / t_reject / fp32_peak,
           "grown_create_s": t_create, "grown_update_s": t_update,
           "grown_pairs_per_s": N * N / t_update, "synapses": S,
           # every overlapping pair (one per synapse here: no radius contains another)
           # evaluates the lens area with 2 acos and 2 sin
           "grown_transcendental_calls": 4 * S,
           "grown_transcendentals_per_s": 4 * S / t_update,
           "grown_bound": "fp64 (acos and sin of the overlap area evaluated in double; "
                          "86 % FP64-pipe busy, profiles/k_growth_plain.md)",
           "error_word": err}
    N2, r2, c2, u2, S2, e2 = _growth_passes(200, 200, RADIUS)
    out["served_largest_200x200"] = {
        "pairs": N2 * N2, "radius_0.4_s": r2, "radius_0.4_pairs_per_s": N2 * N2 / r2,
        "grown_create_s": c2, "grown_update_s": u2, "grown_pairs_per_s": N2 * N2 / u2,
        "synapses": S2, "grown_transcendentals_per_s": 4 * S2 / u2, "error_word": e2}
    return out


def run_small(steps=20000, warmup=2000):
    """The 100-neuron network (10x10 LIF + DS + ConnGrowth, 10 %
    inhibitory, 10 starters, max 100 synapses per neuron; at its stated 0.4 start radius it has no
    synapses) stepped on the one-CTA path (many whole steps per launch) and on the multi-kernel
    path, with the library's device noise and with the reference's Norm stream pushed ahead
    (injected noise); host wall clock around synchronised bg3_step calls, beside the oracle C
    port of the reference on one core of this host (the CPU baseline leg)."""
    import time as _t
    from braingrid_gb300 import lib as bg
    from braingrid_gb300 import netgen
    spec = netgen.lif_network(10, 10, frac_inh=0.10, seed=1)
    N = spec["N"]
    out = {"workload": "10x10 LIF + DS + ConnGrowth, start radius 0.4, %d steps" % steps}
    for mode, name in ((bg.BG3_NOISE_DEVICE, "device_noise"), (bg.BG3_NOISE_INJECT, "injected_noise")):
        for small, tag in ((65536, "one_cta"), (0, "multi_kernel")):
            net = netgen.make_gpu_network(spec, 100, noise_mode=mode, noise_seed=1)
            net.set_launch(small_max_slots=small)
            if mode == bg.BG3_NOISE_INJECT:
                gen = bg.NormStream(1)
                net.push_noise(gen.take(N * (steps + warmup)))
                gen.close()
            net.step(warmup)
            net.sync()
            l0 = net.launches
            t0 = _t.perf_counter()
            net.step(steps)
            net.sync()
            dt = _t.perf_counter() - t0
            out["%s_%s_us_per_step" % (name, tag)] = dt * 1e6 / steps
            out["%s_%s_launches" % (name, tag)] = net.launches - l0
            out["%s_%s_error_word" % (name, tag)] = net.error_word
            net.close()
    out["cpu_baseline"] = small_cpu_baseline(spec, steps)
    out["cpu_over_gpu_one_cta"] = (out["cpu_baseline"]["us_per_step"] /
                                   out["device_noise_one_cta_us_per_step"])
    return out


def small_cpu_baseline(spec, steps):
    """The oracle (the reference algorithm in C, one thread) on the same 100-neuron network."""
    from oracle import pyoracle as po
    N = spec["N"]
    o = po.OracleNet(N, 100, 10, 10, 1.0, 1e-4, 200, 10)
    for k in ("xloc", "yloc", "ntype", "Vm", "Vthresh", "Vreset", "I0", "Inoise", "C1", "C2",
              "Trefract"):
        o.arr(k)[:] = spec[k]
    o.growth_init(0.60, 0.10, 1e-4, 1.0, 0.1, 0.4)
    o.seed_noise(1)
    o.step_n(1000)
    t0 = time.perf_counter()
    o.step_n(steps)
    dt = time.perf_counter() - t0
    o.close()
    return {"us_per_step": dt * 1e6 / steps, "cores": 1, "kind": "port",
            "sample": "%d steps of the same network (oracle C port, one thread)" % steps}


def run_izh512(steps, warmup):
    """The 512-network batch: Izhikevich + dynamic STDP networks (static wiring, Poisson drive) advanced
    as one batch against the same networks run one at a time with bg3_step."""
    import time as _t
    from braingrid_gb300 import lib as bg
    from braingrid_gb300 import workloads
    t0 = _t.perf_counter()
    nets = workloads.build_izh512()
    t_build = _t.perf_counter() - t0
    S = sum(n.total_synapses() for n in nets)
    N = sum(n.N for n in nets)
    batch = bg.Batch(nets)

    def spikes():
        return sum(int(n.download_lif(fields=("spikeCount",))["spikeCount"].sum()) for n in nets)

    batch.step(IZH_SETTLE)
    launch, _ = batch.autotune(steps_per_trial=100)
    batch.step(warmup)
    batch.sync()
    s0 = spikes()
    ms = batch.bench_steps(steps)
    rate = (spikes() - s0) / float(N) / (steps * 1e-4)
    t_batch = float(np.sum(ms)) / 1e3
    t_graph = _batch_graph_seconds(batch, steps)
    for n in nets:
        n.step(max(warmup, GRAPH_WARMUP))  # builds each network's step graph before timing
    for n in nets:
        n.sync()
    t0 = _t.perf_counter()
    for n in nets:
        n.step(steps)
    for n in nets:
        n.sync()
    t_plain = _t.perf_counter() - t0
    err = max(n.error_word for n in nets)
    out = {"workload": "%d Izhikevich + dynamic STDP networks, N ~ U[500, 8000] "
                       "(grids), static wiring 10 nearest within radius 5 + 10%% rewired, "
                       "Poisson 10 Hz x 5 nA" % len(nets),
           "networks": len(nets), "neurons": N, "synapses": S, "steps": steps,
           "settle_steps": IZH_SETTLE,
           "build_s": t_build,
           "batched_synapse_updates_per_s": S * steps / t_batch,
           "batched_neuron_steps_per_s": N * steps / t_batch,
           "batched_ms_per_step": t_batch * 1e3 / steps,
           "plain_synapse_updates_per_s": S * steps / t_plain,
           "plain_neuron_steps_per_s": N * steps / t_plain,
           "plain_ms_per_step": t_plain * 1e3 / steps,
           "plain_timing": "host wall clock around %d sequential bg3_step runs" % len(nets),
           "batched_over_plain": t_plain / t_batch,
           "batched_gbs": _alg_gbs(S, N, IZH_BYTES_PER_NEURON, t_batch / steps),
           "batched_frac_of_peak": _alg_gbs(S, N, IZH_BYTES_PER_NEURON, t_batch / steps) /
                                   peaks()[0],
           "algorithmic_bytes_per_step": SWEEP_BYTES_PER_SYN * S + IZH_BYTES_PER_NEURON * N,
           "bytes_per_synapse": SWEEP_BYTES_PER_SYN, "bytes_per_neuron": IZH_BYTES_PER_NEURON,
           "batched_timing": "CUDA events around each step (the step's kernels launched one by "
                             "one, the next step's sweep not overlapping them)",
           "batched_graph_ms_per_step": t_graph * 1e3 / steps,
           "batched_graph_synapse_updates_per_s": S * steps / t_graph,
           "batched_graph_neuron_steps_per_s": N * steps / t_graph,
           "batched_graph_timing": "host wall clock around one bg3_batch_step call (CUDA graphs "
                                   "of 32 steps), as the plain form",
           "batched_graph_over_plain": t_plain / t_graph,
           # over the timed batched steps, after IZH_SETTLE + warmup steps
           "mean_rate_hz": rate,
           "error_word": int(err), "launch": launch}
    batch.close()
    for n in nets:
        n.close()
    return out


def run_served(n_jobs, slots_cap=0, chunk_steps=2000, epoch_duration=1.0, order=0, max_bypass=8):
    """The served stream: a seeded open-loop Poisson trace (20 jobs/s) through the job server
    (continuous batching, footprint admission, 150 GB budget), then the same jobs one at a
    time through the plain API.  Latency = completion - arrival, host wall clock."""
    import time as _t
    from braingrid_gb300 import lib as bg
    from braingrid_gb300 import serve, workloads
    trace = workloads.served_trace(n_jobs, epoch_duration=epoch_duration)
    srv = serve.Server(hbm_budget_bytes=workloads.SERVED_BUDGET, max_resident=64,
                       chunk_steps=chunk_steps, max_resident_slots=slots_cap, order=order,
                       max_bypass=max_bypass)
    times = serve.run_trace(srv, trace)
    lat = {k: f - a for k, (a, f) in times.items()}
    finish = {k: f for k, (_, f) in times.items()}
    st = srv.stats()
    srv.close()
    jobs = [j for _, j in trace]
    ok = all(j.result.status == 0 and j.result.error_word == 0 for j in jobs)
    syn_steps = sum(int(j.result.synapse_steps) for j in jobs)
    span = max(finish.values()) - trace[0][0]
    L = np.array([lat[j.id] for j in jobs])
    # plain: the same jobs, one at a time, each on its own network with bg3_step + epoch passes
    durations, setups = [], []
    for _, job in workloads.served_trace(n_jobs, epoch_duration=epoch_duration):
        d = job.desc
        t1 = _t.perf_counter()
        net = bg.Network(d.n_neurons, d.max_syn_per_neuron, d.width, d.height, d.epoch_duration,
                         d.delta_t, d.max_firing_rate, d.max_epochs, d.synapse_kind,
                         d.noise_mode, d.noise_seed, neuron_kind=d.neuron_kind)
        job.setup(net)
        net.sync()
        setups.append(_t.perf_counter() - t1)
        spe = int(np.float32(d.epoch_duration) / np.float32(d.delta_t))
        for e in range(job.epochs):
            net.step(spe)
            if job.growth:
                net.growth(e + 1)
            else:
                net.record()
        net.download_histories()
        net.close()
        durations.append(_t.perf_counter() - t1)
    t_free, plat = 0.0, []
    for (a, _), dur in zip(trace, durations):
        start = max(a, t_free)
        t_free = start + dur
        plat.append(t_free - a)
    plat = np.array(plat)
    pct = lambda x, q: float(np.percentile(x, q))
    return {"workload": "served stream: %d-job seeded Poisson trace at 20 jobs/s from the three "
                        "families (LIF sides U[10,200] pre-grown, Izhikevich N U[500,8000]), 1-20 "
                        "epochs of %g s, 150 GB admission budget" % (n_jobs, epoch_duration),
            "jobs": n_jobs, "all_ok": ok, "synapse_steps": syn_steps,
            "admission_order": ["arrival", "least work first"][order],
            "max_bypass": max_bypass,
            "max_resident_slots": int(slots_cap), "chunk_steps": chunk_steps,
            "served_p50_s": pct(L, 50), "served_p95_s": pct(L, 95), "served_p99_s": pct(L, 99),
            "served_makespan_s": span, "served_synapse_updates_per_s": syn_steps / span,
            "peak_resident": int(st["peak_resident"]), "rounds": int(st["rounds"]),
            "server_host_s": {k: round(float(st[k]), 3) for k in ("admit_s", "wait_s", "epoch_s",
                                                                   "rebuild_s")},
            "per_job": [{"name": j.name, "neurons": int(j.desc.n_neurons), "epochs": int(j.epochs),
                         "synapse_steps": int(j.result.synapse_steps),
                         "error_word": int(j.result.error_word),
                         "served_latency_s": round(float(lat[j.id]), 3),
                         "plain_duration_s": round(float(dur), 3),
                         "plain_setup_s": round(float(su), 3)}
                        for j, dur, su in zip(jobs, durations, setups)],
            "plain_p50_s": pct(plat, 50), "plain_p95_s": pct(plat, 95),
            "plain_p99_s": pct(plat, 99), "plain_makespan_s": float(t_free - trace[0][0]),
            "plain_synapse_updates_per_s": syn_steps / float(t_free - trace[0][0]),
            "plain_timing": "jobs run back to back (each with its own setup); latencies from the "
                            "measured durations and the same arrival times",
            "served_over_plain_throughput": float(t_free - trace[0][0]) / span}


def run_reference(args):
    """The reference algorithm's CPU path (oracle C port), single-threaded like the reference."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from braingrid_gb300 import netgen
    from oracle import pyoracle as po
    spec = netgen.lif_network(WIDTH, HEIGHT, frac_inh=0.10, seed=SEED)
    N = spec["N"]
    o = po.OracleNet(N, MAX_SYN, WIDTH, HEIGHT, 1.0, 1e-4, 200, 10)
    for k in ("xloc", "yloc", "ntype", "Vm", "Vthresh", "Vreset", "I0", "Inoise", "C1", "C2",
              "Trefract"):
        o.arr(k)[:] = spec[k]
    o.growth_init(0.60, 0.10, 1e-4, 1.0, 0.1, 0.4)
    rs = np.random.RandomState(11)
    o.arr("radii")[:] = rs.uniform(RADIUS - 0.05, RADIUS + 0.05, N).astype(np.float32)
    o.seed_noise(SEED)
    o.growth()
    o.arr("W")[:] = o.arr("W") * np.float32(WEIGHT_SCALE)
    o.input_poisson(POISSON["fr_mean"], POISSON["weight"])
    S = o.total
    o.step_n(max(1, min(args.warmup, 3)))
    # each timed "step" is one full simulation step; the sample is capped at ~60 s of CPU time
    t0 = time.perf_counter()
    o.step_n(1)
    one = time.perf_counter() - t0
    k = max(1, min(args.steps, int(60.0 / max(one, 1e-6))))
    t0 = time.perf_counter()
    o.step_n(k)
    dt = time.perf_counter() - t0
    value = S * k / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
            "n_gpus": world, "steps": k, "warmup": args.warmup, "ms_per_step": dt * 1e3 / k,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "neurons": N, "synapses": S},
            "neuron_steps_per_s": N * k / dt,
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": 1, "kind": "port",
                             "sample": "%d of %d requested steps (capped at ~60 s), one thread; "
                                       "host has %d cores" % (k, args.steps, os.cpu_count() or 0)},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    o.close()
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="bg3", choices=["bg3", "reference"])
    ap.add_argument("--serve-jobs", type=int, default=8,
                    help="jobs of the served-stream trace")
    ap.add_argument("--serve-slots", type=float, default=SERVE_SLOTS,
                    help="served form: cap on the resident jobs' synapse slots (0 = none)")
    ap.add_argument("--only", choices=["izh512", "serve", "growth", "small"], default=None,
                    help="run one secondary workload alone and print its JSON")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.only == "izh512":
        print(json.dumps(run_izh512(min(args.steps, 1000), max(args.warmup, 20))), flush=True)
        return
    if args.only == "growth":
        print(json.dumps(run_growth()), flush=True)
        return
    if args.only == "small":
        print(json.dumps(run_small()), flush=True)
        return
    if args.only == "serve":
        print(json.dumps(run_served(args.serve_jobs, int(args.serve_slots), order=SERVE_ORDER)),
              flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_bg3(args)


if __name__ == "__main__":
    main()
