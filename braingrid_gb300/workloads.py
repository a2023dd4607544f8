"""Benchmark workloads (synthetic networks with the stated configs' shapes and distributions)."""
from . import netgen

# config[1]: plain single network, 100x100 LIF + DS + ConnGrowth, max 1000 synapses per neuron.
# At the stated start radius (0.4) no pair overlaps, so throughput is measured on a pre-grown
# state: radii ~ U[8.35, 8.45] wired by one device growth pass (~7.6 M synapses), weights scaled.
C1 = dict(width=100, height=100, max_syn=1000, radius=8.4, weight_scale=0.003, seed=7,
          frac_inh=0.10, epoch_duration=1.0, max_firing_rate=200, max_epochs=10)


def build(w=C1):
    spec = netgen.lif_network(w["width"], w["height"], frac_inh=w["frac_inh"], seed=w["seed"])
    net = netgen.make_gpu_network(spec, w["max_syn"], epoch_duration=w["epoch_duration"],
                                  max_firing_rate=w["max_firing_rate"],
                                  max_epochs=w["max_epochs"], noise_seed=w["seed"])
    netgen.pregrow(net, spec, w["radius"], weight_scale=w["weight_scale"])
    return spec, net


# config[2]: 36 networks, targetRate {0.1, 1.0, 1.9} Hz x excitatory fraction {0.80, 0.90, 0.98}
# x 4 seeds, sizes cycling 30x30, 50x50, 70x70, 100x100; the config[1] model otherwise, with the
# same pre-grown radius and weight scale.
C2_SIZES = [30, 50, 70, 100]


def c2_members():
    out = []
    k = 0
    for tr in (0.1, 1.0, 1.9):
        for fe in (0.80, 0.90, 0.98):
            for seed in range(4):
                side = C2_SIZES[k % 4]
                out.append(dict(C1, width=side, height=side, frac_inh=round(1.0 - fe, 2),
                                seed=seed, target_rate=tr))
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
