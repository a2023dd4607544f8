"""Synthetic BrainGrid-style networks for the benchmarks (product side, numpy only).

Builds what the reference's host setup would (Layouts/Layout.cpp:41-73 grid positions,
FixedLayout E/I and starter sites, AllIFNeurons::createNeuron parameter ranges and constants,
Neurons/AllIFNeurons.cpp:398-503) from a seeded numpy generator, so that benchmark networks of
any size can be made without the reference's MTRand draws.  The value distributions are the
config[0] ones: Iinject 13.5 nA, Inoise U[1.0, 1.5] nA, Vthresh 15 mV (starters U[13.565,
13.655] mV), Vreset 13.5 mV (starters 13.0 mV), Vrest 0, Vinit 13.0 mV, Cm 30 nF, Rm 1 MOhm,
Trefract 3 ms (2 ms inhibitory), dt 0.1 ms.
"""
import numpy as np

from . import lib as bg


def lif_network(width, height, frac_inh=0.10, n_starters=None, seed=7, delta_t=1e-4):
    N = width * height
    rs = np.random.RandomState(seed)
    perm = rs.permutation(N)
    n_inh = int(round(frac_inh * N))
    if n_starters is None:
        n_starters = max(1, N // 10 if N <= 100 else N // 100)
    ntype = np.full(N, 2, np.int32)
    ntype[perm[:n_inh]] = 1
    starter = np.zeros(N, bool)
    starter[perm[n_inh:n_inh + n_starters]] = True
    f32 = np.float32
    Iinject = np.full(N, 13.5e-9, f32)
    Inoise = rs.uniform(1.0e-9, 1.5e-9, N).astype(f32)
    Vthresh = np.full(N, 15.0e-3, f32)
    Vreset = np.full(N, 13.5e-3, f32)
    Vrest = np.zeros(N, f32)
    Vm = np.full(N, 13.0e-3, f32)
    Vthresh[starter] = rs.uniform(13.565e-3, 13.655e-3, int(starter.sum())).astype(f32)
    Vreset[starter] = f32(13.0e-3)
    Rm = f32(1e6)
    tau = f32(3e-8) * Rm
    C1 = np.full(N, np.exp(-f32(delta_t) / tau, dtype=f32), f32)
    C2 = (Rm * (f32(1) - C1)).astype(f32)
    I0 = (Iinject + Vrest / Rm).astype(f32)
    Trefract = np.where(ntype == 1, f32(2.0e-3), f32(3.0e-3)).astype(f32)
    Trefract[starter] = f32(3.0e-3)
    idx = np.arange(N)
    return dict(N=N, width=width, height=height,
                xloc=(idx % width).astype(f32), yloc=(idx // width).astype(f32), ntype=ntype,
                starter=starter, Vm=Vm, Vthresh=Vthresh, Vreset=Vreset, I0=I0, Inoise=Inoise,
                C1=C1, C2=C2, Trefract=Trefract)


GROWTH = dict(epsilon=0.60, beta=0.10, rho=1e-4, target_rate=1.0, min_radius=0.1,
              start_radius=0.4)


def make_gpu_network(spec, max_syn, epoch_duration=1.0, max_firing_rate=200, max_epochs=10,
                     noise_seed=7, growth=None, noise_mode=bg.BG3_NOISE_DEVICE):
    g = dict(GROWTH, **(growth or {}))
    net = bg.Network(spec["N"], max_syn, spec["width"], spec["height"], epoch_duration, 1e-4,
                     max_firing_rate, max_epochs, bg.BG3_SYN_DS, noise_mode, noise_seed)
    net.upload_layout(spec["xloc"], spec["yloc"], spec["ntype"])
    net.upload_lif(Vm=spec["Vm"], Vthresh=spec["Vthresh"], Vreset=spec["Vreset"], I0=spec["I0"],
                   Inoise=spec["Inoise"], C1=spec["C1"], C2=spec["C2"], Trefract=spec["Trefract"])
    radii = np.full(spec["N"], g["start_radius"], np.float32)
    net.upload_growth(g["epsilon"], g["beta"], g["rho"], g["target_rate"], g["min_radius"],
                      g["start_radius"], radii)
    return net


def pregrow(net, spec, radius, spread=0.05, weight_scale=1.0, seed=11):
    """Pre-grown connectivity: radii ~ U[radius - spread, radius + spread], one device growth
    pass wires every overlapping pair (weights = overlap area x 1e-8 as in ConnGrowth), then the
    weights are scaled by weight_scale.  Returns the radii used."""
    rs = np.random.RandomState(seed)
    r = rs.uniform(radius - spread, radius + spread, spec["N"]).astype(np.float32)
    g = GROWTH
    net.upload_growth(g["epsilon"], g["beta"], g["rho"], g["target_rate"], g["min_radius"],
                      g["start_radius"], r)
    net.growth(0)
    net.sync()
    if weight_scale != 1.0:
        s = net.download_synapses()
        net.upload_weights((s["W"] * np.float32(weight_scale)).astype(np.float32))
    return r
