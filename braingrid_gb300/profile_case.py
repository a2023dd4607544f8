"""Run a benchmark workload for a few steps, for profilers (ncu) to capture its kernels.

    python -m braingrid_gb300.profile_case [--workload plain|sweep36|izh512|big|growth|growth200|heavy|small] [--steps 20] [--flush]

plain is the 100x100 network of the headline, sweep36 the 36-network growth sweep, izh512 the
Izhikevich + STDP batch (--count networks, 512 by default); big is three pre-grown LIF
networks of the served stream's largest sizes (166x166, 176x176, 180x180) after one epoch and a
growth pass (which restores the unscaled growth weights: the networks then fire at ~300 Hz),
batched together.  heavy is one of those jobs (180x180) alone: 10,000 steps, a growth pass, 1,000
steps (it then fires at ~300 Hz), then --steps steps timed kernel by kernel; its delivery passes
after launch 11,000 are heavy ones.  growth200 is the growth pass of the served stream's largest
job (200x200, pre-grown); small the 10x10 LIF + DS + ConnGrowth network (100 neurons) on the one-CTA path
(k_small_run, 4,096 steps per launch).  --settle runs a batched workload for that many steps
first (the izh512 networks' firing rate rises from ~1 Hz to a steady ~15 Hz over the first
~1,200 steps as STDP strengthens their synapses).
"""
import argparse

from . import workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--flush", action="store_true", help="evict L2 before every step")
    ap.add_argument("--workload", default="plain",
                    choices=["plain", "sweep36", "izh512", "big", "growth", "growth200",
                             "heavy", "small"])
    ap.add_argument("--count", type=int, default=512, help="networks of the izh512 workload")
    ap.add_argument("--settle", type=int, default=0,
                    help="batched workloads: steps run (as one call) before the profiled steps")
    a = ap.parse_args()
    flush = (256 << 20) if a.flush else 0
    if a.workload in ("growth", "growth200"):
        # the growth pass at the pre-grown radii: creation, then an updating pass; growth is
        # the 10,000-neuron network, growth200 the served stream's largest job (200x200)
        from . import netgen
        if a.workload == "growth":
            spec, net = workloads.build()
        else:
            spec = netgen.lif_network(200, 200, frac_inh=0.10, seed=workloads.PLAIN["seed"])
            net = netgen.make_gpu_network(spec, workloads.PLAIN["max_syn"],
                                          noise_seed=workloads.PLAIN["seed"])
            netgen.pregrow(net, spec, workloads.PLAIN["radius"])
        net.growth(2)
        net.sync()
        print("synapses", net.total_synapses(), "error_word", net.error_word)
        return
    if a.workload == "small":
        # the 10x10 LIF + DS + ConnGrowth network (no synapse at its 0.4 start radius) on the
        # one-CTA path: --steps whole steps, 4,096 per launch
        from . import netgen
        spec = netgen.lif_network(10, 10, frac_inh=0.10, seed=1)
        net = netgen.make_gpu_network(spec, 100, noise_seed=1)
        net.step(a.steps)
        net.sync()
        print("steps", a.steps, "launches", net.launches, "error_word", net.error_word)
        return
    if a.workload == "heavy":
        import numpy as np
        from . import lib as bg
        from . import serve
        job = serve.lif_growth_job(180, 3, seed=77)
        d = job.desc
        net = bg.Network(d.n_neurons, d.max_syn_per_neuron, d.width, d.height, d.epoch_duration,
                         d.delta_t, d.max_firing_rate, d.max_epochs, d.synapse_kind, d.noise_mode,
                         d.noise_seed)
        job.setup(net)
        net.step(10000)
        net.growth(1)
        net.step(1000)
        _, km = net.bench_steps(a.steps, flush, per_kernel=True)
        print("steps", a.steps, "deliver_us %.1f sweep_us %.1f" % (np.mean(km[:, 1]) * 1e3,
                                                                 np.mean(km[:, 2]) * 1e3),
              "synapses", net.total_synapses(), "error_word", net.error_word)
        return
    if a.workload == "plain":
        spec, net = workloads.build()
        net.bench_steps(a.steps, flush)
        print("steps", a.steps, "synapses", net.total_synapses(), "error_word", net.error_word)
        assert net.error_word == 0
    else:
        from . import lib as bg
        if a.workload == "sweep36":
            nets = [workloads.build_member(w)[1] for w in workloads.sweep36_members()]
        elif a.workload == "izh512":
            nets = workloads.build_izh512(count=a.count)
        else:
            from . import serve
            nets = []
            for k, side in enumerate((166, 176, 180)):
                job = serve.lif_growth_job(side, 2, seed=60 + k)
                d = job.desc
                net = bg.Network(d.n_neurons, d.max_syn_per_neuron, d.width, d.height,
                                 d.epoch_duration, d.delta_t, d.max_firing_rate, d.max_epochs,
                                 d.synapse_kind, d.noise_mode, d.noise_seed)
                job.setup(net)
                net.step(10000)
                net.growth(1)
                net.step(1000)
                c = net.download_lif(fields=("spikeCount",))["spikeCount"]
                print("net", side, "synapses", net.total_synapses(), "rate_hz",
                      float(c.sum()) / c.size / 0.1)
                nets.append(net)
        batch = bg.Batch(nets)
        if a.settle:
            batch.step(a.settle)
        batch.bench_steps(a.steps, flush)
        S = sum(n.total_synapses() for n in nets)
        print("steps", a.steps, "networks", len(nets), "synapses", S)
        assert max(n.error_word for n in nets) == 0


if __name__ == "__main__":
    main()
