"""Benchmark workloads (synthetic networks with the stated configs' shapes and distributions)."""
import numpy as np

from . import netgen

# The plain single network: 100x100 LIF + DS + ConnGrowth, max 1000 synapses per neuron.
# At the stated start radius (0.4) no pair overlaps, so throughput is measured on a pre-grown
# state: radii ~ U[8.35, 8.45] wired by one device growth pass (~7.6 M synapses), weights scaled.
# Without input this network either stays near silent (0.03 Hz at weight scale 0.003) or, with
# stronger weights, bursts to saturation; a Poisson drive of every neuron (the reference's
# SInputPoisson: 10 Hz, weight 9.5, i.e. 95 nA per input synapse) with recurrent weights scaled
# by 0.0003 holds it at about the growth rule's 1 Hz target rate (~1,000 spike arrivals per step).
PLAIN = dict(width=100, height=100, max_syn=1000, radius=8.4, weight_scale=0.0003, seed=7,
             frac_inh=0.10, epoch_duration=1.0, max_firing_rate=200, max_epochs=10,
             poisson=dict(fr_mean=10.0, weight=9.5))


def build(w=PLAIN):
    spec = netgen.lif_network(w["width"], w["height"], frac_inh=w["frac_inh"], seed=w["seed"])
    net = netgen.make_gpu_network(spec, w["max_syn"], epoch_duration=w["epoch_duration"],
                                  max_firing_rate=w["max_firing_rate"],
                                  max_epochs=w["max_epochs"], noise_seed=w["seed"])
    netgen.pregrow(net, spec, w["radius"], weight_scale=w["weight_scale"])
    if w.get("poisson"):
        arr, lam = netgen.poisson_arrays(spec, w["poisson"]["fr_mean"], w["poisson"]["weight"])
        net.input_poisson(lam, seed=w["seed"], step=net.sim_step, **arr)
    return spec, net


# The 36-network growth sweep: targetRate {0.1, 1.0, 1.9} Hz x excitatory fraction {0.80, 0.90,
# 0.98} x 4 seeds, sizes cycling 30x30, 50x50, 70x70, 100x100; the plain network's model
# otherwise, with the same pre-grown radius, weights scaled by 0.003 and no external input.
SWEEP36_SIZES = [30, 50, 70, 100]
SWEEP36_BASE = dict(PLAIN, weight_scale=0.003, poisson=None)


def sweep36_members():
    out = []
    k = 0
    for tr in (0.1, 1.0, 1.9):
        for fe in (0.80, 0.90, 0.98):
            for seed in range(4):
                side = SWEEP36_SIZES[k % 4]
                out.append(dict(SWEEP36_BASE, width=side, height=side,
                                frac_inh=round(1.0 - fe, 2), seed=seed, target_rate=tr))
                k += 1
    return out


def build_member(w):
    spec = netgen.lif_network(w["width"], w["height"], frac_inh=w["frac_inh"], seed=w["seed"])
    net = netgen.make_gpu_network(spec, w["max_syn"], epoch_duration=w["epoch_duration"],
                                  max_firing_rate=w["max_firing_rate"],
                                  max_epochs=w["max_epochs"], noise_seed=w["seed"] + 101,
                                  growth=dict(target_rate=w.get("target_rate", 1.0)))
    netgen.pregrow(net, spec, w["radius"], weight_scale=w["weight_scale"], seed=w["seed"] + 11)
    return spec, net


# The 512-network batch: independent Izhikevich + dynamic STDP networks, sizes ~ U[500, 8000] neurons on
# near-square grids, 20 % inhibitory, static wiring (10 nearest within radius 5, 10 % rewired),
# weights U[10, 20] nA / U[-40, -20] nA, additive STDP (Apos 0.005, Aneg -0.00525 of the 30 nA
# bound, tau 20 ms), Poisson drive 10 Hz x 5 nA, dt 0.1 ms.
IZH512_NETWORKS = 512


def izh512_shapes(count=IZH512_NETWORKS, seed=3):
    rs = np.random.RandomState(seed)
    out = []
    for n in rs.randint(500, 8001, size=count):
        w = int(round(np.sqrt(n)))
        out.append((w, max(1, int(round(n / w)))))
    return out


def build_izh512(count=IZH512_NETWORKS, seed=3, max_epochs=10):
    nets = []
    for k, (w, h) in enumerate(izh512_shapes(count, seed)):
        nets.append(netgen.make_izh_static(w, h, seed=1000 + k, max_epochs=max_epochs)[1])
    return nets


# The served stream.  Open-loop Poisson arrivals at 20 jobs/s (seeded trace); each job
# drawn from the three families above: LIF + DS + ConnGrowth pre-grown like the plain network
# (side ~ U[10, 200], radius min(8.4, 0.45 side)), the growth-sweep parameters (targetRate,
# excitatory fraction), or the Izhikevich + STDP network (N ~ U[500, 8000]);
# 1-20 epochs of 1 s; admission against a 150 GB footprint budget.
SERVED_RATE = 20.0
SERVED_BUDGET = 150 << 30


def served_trace(n_jobs, seed=4, rate=SERVED_RATE, epoch_duration=1.0):
    """[(arrival_s, job)] for n_jobs jobs of the served stream."""
    from . import serve
    rs = np.random.RandomState(seed)
    t = 0.0
    out = []
    for k in range(n_jobs):
        t += rs.exponential(1.0 / rate)
        fam = rs.randint(3)
        epochs = int(rs.randint(1, 21))
        js = 50 + k
        if fam == 0:
            side = int(rs.randint(10, 201))
            job = serve.lif_growth_job(side, epochs, seed=js, epoch_duration=epoch_duration)
        elif fam == 1:
            side = int(rs.randint(10, 201))
            tr = float(rs.choice([0.1, 1.0, 1.9]))
            fe = float(rs.choice([0.80, 0.90, 0.98]))
            job = serve.lif_growth_job(side, epochs, seed=js, target_rate=tr,
                                       frac_inh=round(1.0 - fe, 2), epoch_duration=epoch_duration)
        else:
            n = int(rs.randint(500, 8001))
            w = int(round(np.sqrt(n)))
            job = serve.izh_static_job(w, max(1, int(round(n / w))), epochs, seed=js,
                                       epoch_duration=epoch_duration)
        out.append((t, job))
    return out
