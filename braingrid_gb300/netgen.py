"""Synthetic BrainGrid-style networks for the benchmarks (product side, numpy only).

Builds what the reference's host setup would (Layouts/Layout.cpp:41-73 grid positions,
FixedLayout E/I and starter sites, AllIFNeurons::createNeuron parameter ranges and constants,
Neurons/AllIFNeurons.cpp:398-503) from a seeded numpy generator, so that benchmark networks of
any size can be made without the reference's MTRand draws.  The value distributions are the
10x10 benchmark network's: Iinject 13.5 nA, Inoise U[1.0, 1.5] nA, Vthresh 15 mV (starters U[13.565,
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
    net = bg.Network(spec["N"], max_syn, spec["width"], spec["height"], epoch_duration, 1e-4,
                     max_firing_rate, max_epochs, bg.BG3_SYN_DS, noise_mode, noise_seed)
    configure_lif(net, spec, growth)
    return net


def configure_lif(net, spec, growth=None):
    """Uploads a lif_network spec and the ConnGrowth parameters into a created network."""
    g = dict(GROWTH, **(growth or {}))
    net.upload_layout(spec["xloc"], spec["yloc"], spec["ntype"])
    net.upload_lif(Vm=spec["Vm"], Vthresh=spec["Vthresh"], Vreset=spec["Vreset"], I0=spec["I0"],
                   Inoise=spec["Inoise"], C1=spec["C1"], C2=spec["C2"], Trefract=spec["Trefract"])
    radii = np.full(spec["N"], g["start_radius"], np.float32)
    net.upload_growth(g["epsilon"], g["beta"], g["rho"], g["target_rate"], g["min_radius"],
                      g["start_radius"], radii)


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
    if weight_scale != 1.0:
        net.scale_weights(np.float32(weight_scale))
    net.sync()
    return r


# ---- Izhikevich networks with static connectivity, dynamic STDP and Poisson drive ------------
# Synapse types II, IE, EI, EE (Utils/Global.h:100); per-type constants of the reference's
# createSynapse (Synapses/AllSpikingSynapses.cpp:192-240, AllDSSynapses.cpp:180-218).
TYPE_TAU = np.array([6e-3, 6e-3, 3e-3, 3e-3], np.float32)
TYPE_U = np.array([0.32, 0.25, 0.05, 0.5], np.float32)
TYPE_D = np.array([0.144, 0.7, 0.125, 1.1], np.float32)
TYPE_F = np.array([0.06, 0.02, 1.2, 0.05], np.float32)


def syn_type(src_inh, dst_inh):
    """Layout::synType: II 0, IE 1 (inhibitory source), EI 2, EE 3."""
    return np.where(src_inh, np.where(dst_inh, 0, 1), np.where(dst_inh, 2, 3)).astype(np.int32)


def izh_network(width, height, frac_inh=0.20, seed=1, delta_t=1e-4):
    """Izhikevich neurons with r ~ U[0, 1] per neuron: excitatory a = 0.02, b = 0.2,
    c = -65 + 15 r^2 mV, d = 8 - 6 r^2; inhibitory a = 0.02 + 0.08 r, b = 0.25 - 0.05 r,
    c = -65 mV, d = 2.  IF fields as configfiles/static_izh_1000.xml: Iinject 13.5 nA,
    Inoise U[0.5, 0.7329] uA, Vthresh 30 mV, Vinit -65 mV; Trefract 3 ms (2 ms inhibitory)."""
    N = width * height
    rs = np.random.RandomState(seed)
    perm = rs.permutation(N)
    ntype = np.full(N, 2, np.int32)
    ntype[perm[:int(round(frac_inh * N))]] = 1
    inh = ntype == 1
    f32 = np.float32
    r = rs.uniform(0.0, 1.0, N).astype(f32)
    a = np.where(inh, f32(0.02) + f32(0.08) * r, f32(0.02)).astype(f32)
    b = np.where(inh, f32(0.25) - f32(0.05) * r, f32(0.2)).astype(f32)
    c = np.where(inh, f32(-65.0), f32(-65.0) + f32(15.0) * r * r).astype(f32)
    d = np.where(inh, f32(2.0), f32(8.0) - f32(6.0) * r * r).astype(f32)
    Rm = f32(1e6)
    tau = f32(3e-8) * Rm
    C1 = np.full(N, np.exp(-f32(delta_t) / tau, dtype=f32), f32)
    idx = np.arange(N)
    return dict(N=N, width=width, height=height, kind="izh",
                xloc=(idx % width).astype(f32), yloc=(idx // width).astype(f32), ntype=ntype,
                Vm=np.full(N, -0.065, f32), Vthresh=np.full(N, 30e-3, f32),
                Vreset=np.full(N, -0.065, f32), I0=np.full(N, 13.5e-9, f32),
                Inoise=rs.uniform(0.5e-6, 0.7329e-6, N).astype(f32), C1=C1,
                C2=(Rm * (f32(1) - C1)).astype(f32),
                Trefract=np.where(inh, f32(2e-3), f32(3e-3)).astype(f32),
                Aconst=a, Bconst=b, Cconst=c, Dconst=d, u=np.zeros(N, f32),
                C3=np.full(N, f32(delta_t) * f32(1000.0), f32))


def static_synapses(spec, n_conn=10, radius=5.0, p_rewire=0.10, exc=(10e-9, 20e-9),
                    inh=(-40e-9, -20e-9), delay=1.0e-3, seed=1, delta_t=1e-4, max_syn=None):
    """ConnStatic-style wiring (Connections/ConnStatic.cpp:33-88): every source connects to its
    n_conn nearest neurons within radius (distance ties broken by neuron index); then a fraction
    p_rewire of the synapses move to uniformly drawn targets (the reference computes that count
    but never rewires).  Weights U[exc] / U[inh] by source type; one delay for every type.
    Returns the reference-layout slot arrays (rows filled in source order, as addSynapse does)."""
    N, w, h = spec["N"], spec["width"], spec["height"]
    rs = np.random.RandomState(seed)
    xi, yi = spec["xloc"].astype(np.int64), spec["yloc"].astype(np.int64)
    inh_n = spec["ntype"] == 1
    R = int(np.ceil(radius))
    # grid offsets within the radius, nearest first; equal distances in row-major order, which
    # is neuron-index order for every source
    offs = sorted((dx * dx + dy * dy, dy, dx) for dy in range(-R, R + 1) for dx in range(-R, R + 1)
                  if (dx or dy) and dx * dx + dy * dy <= radius * radius)
    taken = np.zeros(N, np.int64)
    srcs, dsts = [], []
    idx = np.arange(N, dtype=np.int64)
    for _, dy, dx in offs:
        ok = (xi + dx >= 0) & (xi + dx < w) & (yi + dy >= 0) & (yi + dy < h) & (taken < n_conn)
        srcs.append(idx[ok])
        dsts.append((yi[ok] + dy) * w + xi[ok] + dx)
        taken += ok
    srcs, dsts = np.concatenate(srcs), np.concatenate(dsts)
    nre = int(len(srcs) * p_rewire)
    if nre:
        pick = rs.choice(len(srcs), nre, replace=False)
        new = rs.randint(N, size=nre)
        bad = new == srcs[pick]
        while bad.any():
            new[bad] = rs.randint(N, size=int(bad.sum()))
            bad = new == srcs[pick]
        dsts[pick] = new
        # a source keeps at most one synapse per target
        key = srcs * N + dsts
        _, first = np.unique(key, return_index=True)
        keep = np.zeros(len(key), bool)
        keep[first] = True
        srcs, dsts = srcs[keep], dsts[keep]
    order = np.lexsort((srcs, dsts))       # dest-major, sources ascending within a row
    srcs, dsts = srcs[order], dsts[order]
    indeg = np.bincount(dsts, minlength=N)
    M = max_syn or int(max(4, (indeg.max() + 3) // 4 * 4))
    assert indeg.max() <= M
    start = np.concatenate([[0], np.cumsum(indeg)[:-1]])
    k = np.arange(len(dsts)) - start[dsts]
    slot = dsts * M + k
    S = N * M
    f32 = np.float32
    typ = syn_type(inh_n[srcs], inh_n[dsts])
    W = np.where(inh_n[srcs], rs.uniform(inh[0], inh[1], len(srcs)),
                 rs.uniform(exc[0], exc[1], len(srcs))).astype(f32)
    arr = dict(in_use=np.zeros(S, np.uint8), src=np.zeros(S, np.int32),
               type=np.full(S, -1, np.int32), W=np.zeros(S, f32), psr=np.zeros(S, f32),
               decay=np.zeros(S, f32), tau=np.zeros(S, f32), total_delay=np.zeros(S, np.int32),
               delayIdx=np.zeros(S, np.int32), delayQueue=np.zeros(S, np.uint32),
               U=np.zeros(S, f32), D=np.zeros(S, f32), F=np.zeros(S, f32),
               u=np.zeros(S, f32), r=np.zeros(S, f32),
               lastSpike=np.full(S, np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64))
    arr["in_use"][slot] = 1
    arr["src"][slot] = srcs
    arr["type"][slot] = typ
    arr["W"][slot] = W
    tau = TYPE_TAU[typ]
    arr["tau"][slot] = tau
    arr["decay"][slot] = np.exp(-f32(delta_t) / tau).astype(f32)
    arr["total_delay"][slot] = int(f32(delay) / f32(delta_t)) + 1
    arr["U"][slot], arr["D"][slot], arr["F"][slot] = TYPE_U[typ], TYPE_D[typ], TYPE_F[typ]
    arr["u"][slot] = f32(0.4)
    arr["r"][slot] = f32(1.0)
    return arr, indeg.astype(np.uint32), M


# Additive STDP after Song, Miller and Abbott (2000): steps of 0.005 / -0.00525 of the 30 nA
# bound, tau+ = tau- = 20 ms; Wex +30 nA for excitatory sources, -40 nA for inhibitory ones.
STDP_ADDITIVE = dict(Apos=0.005 * 30e-9, Aneg=-0.00525 * 30e-9, STDPgap=2e-3, tauspost=75e-3,
                     tauspre=34e-3, taupos=20e-3, tauneg=20e-3,
                     Wex=[-40e-9, -40e-9, 30e-9, 30e-9], mupos=0.0, muneg=0.0,
                     useFroemkeDanSTDP=1)


def stdp_arrays(syn, c=STDP_ADDITIVE):
    """Reference-layout STDP slot arrays carrying the per-type constants c."""
    S = len(syn["in_use"])
    used = syn["in_use"].astype(bool)
    t = np.clip(syn["type"], 0, 3)
    out = dict(delayQueuePost=np.zeros(S, np.uint32), delayIdxPost=syn["delayIdx"].copy(),
               total_delayPost=np.zeros(S, np.int32),
               useFroemkeDanSTDP=np.where(used, int(c["useFroemkeDanSTDP"]), 0).astype(np.uint8))
    for k in ("tauspost", "tauspre", "taupos", "tauneg", "STDPgap", "Wex", "Aneg", "Apos",
              "mupos", "muneg"):
        v = np.broadcast_to(np.asarray(c[k], np.float32), (4,))
        out[k] = np.where(used, v[t], 0).astype(np.float32)
    return out


def poisson_arrays(spec, fr_mean=10.0, weight=0.5, delta_t=1e-4):
    """SInputPoisson::init (Inputs/SInputPoisson.cpp:19-146): one DS input synapse per neuron
    (EI onto inhibitory, EE onto excitatory), W = weight x 1e-8, nISIs 0 so every neuron draws its
    first interval on the first step.  Returns (arrays, lambda in ms)."""
    N = spec["N"]
    f32 = np.float32
    typ = np.where(spec["ntype"] == 1, 2, 3)
    tau = TYPE_TAU[typ]
    delay_s = np.where(typ == 3, f32(1.5e-3), f32(0.8e-3)).astype(f32)
    arr = dict(masks=np.ones(N, np.uint8), nISIs=np.zeros(N, np.int32),
               total_delay=((delay_s / f32(delta_t)).astype(np.int32) + 1),
               delayIdx=np.zeros(N, np.int32), delayQueue=np.zeros(N, np.uint32),
               W=np.full(N, f32(weight) * f32(1e-8), f32), psr=np.zeros(N, f32),
               decay=np.exp(-f32(delta_t) / tau).astype(f32), U=TYPE_U[typ], D=TYPE_D[typ],
               F=TYPE_F[typ], u=np.full(N, 0.4, f32), r=np.ones(N, f32),
               lastSpike=np.full(N, np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64))
    lam = f32(1.0) / (f32(fr_mean) / f32(1000.0))
    return arr, float(lam)


def izh_static_spec(width, height, seed, n_conn=10, radius=5.0, p_rewire=0.10):
    spec = izh_network(width, height, seed=seed)
    syn, counts, M = static_synapses(spec, n_conn=n_conn, radius=radius, p_rewire=p_rewire,
                                     seed=seed + 1000)
    return spec, syn, counts, M


def configure_izh_static(net, spec, syn, counts, stdp=STDP_ADDITIVE, fr_mean=10.0, weight=0.5,
                         input_seed=0):
    """Uploads an izh_static_spec network (static wiring, dynamic STDP, Poisson drive)."""
    net.upload_layout(spec["xloc"], spec["yloc"], spec["ntype"])
    net.upload_lif(Vm=spec["Vm"], Vthresh=spec["Vthresh"], Vreset=spec["Vreset"], I0=spec["I0"],
                   Inoise=spec["Inoise"], C1=spec["C1"], C2=spec["C2"], Trefract=spec["Trefract"])
    net.upload_izh(**{k: spec[k] for k in ("Aconst", "Bconst", "Cconst", "Dconst", "u", "C3")})
    net.upload_synapses(0, counts=counts, **syn)
    net.set_stdp_constants(**stdp)
    net.upload_stdp(syn["in_use"], syn["type"], syn["delayIdx"], **stdp_arrays(syn, stdp))
    arr, lam = poisson_arrays(spec, fr_mean, weight)
    net.input_poisson(lam, seed=input_seed, step=0, **arr)


def make_izh_static(width, height, seed, max_epochs=10, epoch_duration=1.0,
                    max_firing_rate=1000):
    spec, syn, counts, M = izh_static_spec(width, height, seed)
    net = bg.Network(spec["N"], M, width, height, epoch_duration, 1e-4, max_firing_rate,
                     max_epochs, bg.BG3_SYN_DYNSTDP, bg.BG3_NOISE_DEVICE, seed,
                     neuron_kind=bg.BG3_NEURON_IZH)
    configure_izh_static(net, spec, syn, counts, input_seed=seed)
    return spec, net
