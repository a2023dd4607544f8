"""Copy an oracle network onto the GPU through the C-ABI and compare the two states."""
import numpy as np

from braingrid_gb300 import lib as bg
from oracle import pyoracle as po
from tests.golden.configs import case
from tests.netcases import assert_same, oracle_from_case, steps_per_epoch

LIF_MAP = [("Vm", "Vm"), ("Vthresh", "Vthresh"), ("Vreset", "Vreset"), ("I0", "I0"),
           ("Inoise", "Inoise"), ("C1", "C1"), ("C2", "C2"), ("Trefract", "Trefract"),
           ("summation", "sp"), ("nStepsInRefr", "refr"), ("spikeCount", "spikeCount"),
           ("spikeCountOffset", "spikeCountOffset")]
SYN_MAP = [("in_use", "in_use"), ("src", "src"), ("type", "type"), ("delayIdx", "delayIdx"),
           ("total_delay", "total_delay"), ("W", "W"), ("psr", "psr"), ("decay", "decay"),
           ("delayQueue", "queue"), ("U", "U"), ("D", "D"), ("F", "F"), ("u", "u"), ("r", "r"),
           ("lastSpike", "lastSpike")]


IZH_MAP = [("Aconst", "Aconst"), ("Bconst", "Bconst"), ("Cconst", "Cconst"),
           ("Dconst", "Dconst"), ("u", "u_izh"), ("C3", "C3")]
POIS_MAP = [("masks", "pois_mask"), ("nISIs", "pois_nisi"), ("total_delay", "in_delay"),
            ("delayIdx", "in_delayIdx"), ("delayQueue", "in_queue"), ("W", "in_W"),
            ("psr", "in_psr"), ("decay", "in_decay"), ("U", "in_U"), ("D", "in_D"),
            ("F", "in_F"), ("u", "in_u"), ("r", "in_r"), ("lastSpike", "in_last")]


def f32_steps(seconds, dt=1e-4):
    """static_cast<int>(seconds / deltaT + 0.5) with the float division of the reference."""
    return int(float(np.float32(seconds) / np.float32(dt)) + 0.5)


def setup_input(net, o, c, isi_steps=0):
    stim = c.get("stim")
    if not stim:
        return
    if stim["kind"] == "regular":
        dur = f32_steps(stim["duration"])
        cyc = dur + f32_steps(stim["interval"])
        net.input_regular(o.arr("reg_values"), o.arr("reg_shift"), dur, cyc, 0)
    else:
        lam = np.float32(1.0) / (np.float32(stim["fr_mean"]) / np.float32(1000.0))
        net.input_poisson(float(lam), seed=7, step=o.step,
                          **{k: o.arr(v) for k, v in POIS_MAP})
        if isi_steps:
            begin, isis = o.poisson_isi_draws(isi_steps)
            net.push_poisson_isis(begin, isis)


STDP_MAP = [("delayQueuePost", "queuePost"), ("delayIdxPost", "delayIdxPost"),
            ("total_delayPost", "total_delayPost"), ("tauspost", "tauspost"),
            ("tauspre", "tauspre"), ("taupos", "taupos"), ("tauneg", "tauneg"),
            ("STDPgap", "STDPgap"), ("Wex", "Wex"), ("Aneg", "Aneg"), ("Apos", "Apos"),
            ("mupos", "mupos"), ("muneg", "muneg"), ("useFroemkeDanSTDP", "useFD")]


def stdp_constants(c):
    """Per-type constants of the synapses growth creates (the case's override, or the
    reference's createSynapse values)."""
    p = c.get("stdp")
    if p is None:
        p = [0.5, -0.5, 2e-3, 75e-3, 34e-3, 15e-3, 35e-3, 1.0, 1.0, 0.0, 0.0]
    wex = [p[8], p[8], p[7], p[7]]  # II, IE (inhibitory source), EI, EE
    return dict(Apos=p[0], Aneg=p[1], STDPgap=p[2], tauspost=p[3], tauspre=p[4], taupos=p[5],
                tauneg=p[6], Wex=wex, mupos=p[9], muneg=p[10], useFroemkeDanSTDP=1)


def setup_stdp(net, o, c):
    net.set_stdp_constants(**stdp_constants(c))
    if getattr(o, "_signed", False):
        net.set_stdp_arithmetic(bg.BG3_STDP_DEVICE)
    if o.total:
        net.upload_stdp(o.arr("in_use"), o.arr("type"), o.arr("delayIdx"),
                        **{k: o.arr(v) for k, v in STDP_MAP})


def compare_input(net, o, where):
    if o.arr("pois_nisi").size == 0:
        return
    g = net.download_poisson()
    for k, v in POIS_MAP[1:]:
        assert_same("%s input %s" % (where, k), g[k], o.arr(v))


def gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_INJECT, n_noise=0, noise_seed=None, isi_steps=0):
    izh = c.get("neuron") == "izh"
    net = bg.Network(c["N"], c["max_syn"], c["width"], c["height"], c["tsim"], 1e-4,
                     c["max_firing_rate"], c["epochs"], c.get("synapse", bg.BG3_SYN_DS),
                     noise_mode, noise_seed if noise_seed is not None else c["seed"],
                     neuron_kind=bg.BG3_NEURON_IZH if izh else bg.BG3_NEURON_LIF)
    net.upload_layout(o.arr("xloc"), o.arr("yloc"), o.arr("ntype"))
    kw = {k: o.arr(v) for k, v in LIF_MAP}
    kw["history"] = o.arr("history")
    net.upload_lif(**kw)
    if izh:
        net.upload_izh(**{k: o.arr(v) for k, v in IZH_MAP})
    skw = {k: o.arr(v) for k, v in SYN_MAP}
    net.upload_synapses(o.step, counts=o.arr("counts"), **skw)
    if c.get("synapse", 1) >= 2:
        setup_stdp(net, o, c)
    g = c["growth"]
    net.upload_growth(g["epsilon"], g["beta"], g["rho"], g["target_rate"], g["min_radius"],
                      g["start_radius"], o.arr("radii"), o.arr("rates"))
    if noise_mode == bg.BG3_NOISE_INJECT and n_noise:
        net.push_noise(po.norm_stream(c["seed"], n_noise))
    setup_input(net, o, c, isi_steps)
    return net


def compare_neurons(net, o, where, fields=("Vm", "summation", "nStepsInRefr", "spikeCount",
                                           "spikeCountOffset")):
    g = net.download_lif()
    m = dict(LIF_MAP)
    for f in fields:
        assert_same("%s %s" % (where, f), g[f], o.arr(m[f]))
    if o.neuron_kind == 1:
        assert_same(where + " u", net.download_izh()["u"], o.arr("u_izh"))
    return g


def compare_history(net, o, where):
    g = net.download_lif()
    assert_same(where + " history", g["history"], o.arr("history"))


DS_ONLY = {"U", "D", "F", "u", "r", "lastSpike"}


def compare_synapses(net, o, where, tol_fields=()):
    g = net.download_synapses()
    used = o.arr("in_use").astype(bool)
    ds = o.synapse_kind in (1, 3)
    assert_same(where + " in_use", g["in_use"], o.arr("in_use"))
    assert_same(where + " counts", g["counts"], o.arr("counts"))
    for k, v in SYN_MAP[1:]:
        if k in DS_ONLY and not ds:
            continue
        a, b = g[k][used], o.arr(v)[used]
        if k in tol_fields:
            np.testing.assert_allclose(a, b, rtol=1e-5, atol=0, err_msg=where + " " + k)
        else:
            assert_same("%s %s" % (where, k), a, b)
    if o.synapse_kind >= 2:
        st = net.download_stdp()
        for k, v in STDP_MAP:
            assert_same("%s %s" % (where, k), st[k][used], o.arr(v)[used])
    return g


def compare_maps(net, o, where):
    m = net.download_maps()
    assert_same(where + " outMap", m["outgoingSynapseIndexMap"], o.arr("outMap"))
    assert_same(where + " outBegin", m["outgoingSynapseBegin"], o.arr("outBegin"))
    assert_same(where + " outCount", m["outgoingSynapseCount"], o.arr("outCount"))
    assert_same(where + " inMap", m["incomingSynapseIndexMap"], o.arr("inMap"))
    assert_same(where + " inCount", m["incomingSynapseCount"], o.arr("inCount"))


def _growth_both(o, net, e, resync=True):
    o.growth()
    o.record_epoch(e)
    net.growth(e)
    r, q = net.download_growth()
    assert_same("radii after growth %d" % e, r, o.arr("radii"))
    assert_same("rates after growth %d" % e, q, o.arr("rates"))
    compare_synapses(net, o, "growth %d" % e, tol_fields=("W",))
    compare_maps(net, o, "growth %d" % e)
    if resync:
        net.upload_weights(o.arr("W"))


def run_locked(name, epochs=None, check_every=1, syn_every=None, stdp_signed=False):
    c = case(name)
    E = epochs or c["epochs"]
    spe = steps_per_epoch(c)
    o = oracle_from_case(c)
    if stdp_signed:
        o.stdp_signed(True)
    net = gpu_from_oracle(o, c, n_noise=c["N"] * spe * E + 64, isi_steps=spe * E + 2)
    t = 0
    for e in range(E):
        for _ in range(spe):
            o.step_n(1)
            net.step(1)
            t += 1
            if t % check_every == 0:
                compare_neurons(net, o, "step %d" % t)
                compare_input(net, o, "step %d" % t)
            if syn_every and t % syn_every == 0 and o.total:
                compare_synapses(net, o, "step %d" % t)
        compare_neurons(net, o, "epoch %d end" % e)
        compare_history(net, o, "epoch %d" % e)
        if o.total:
            compare_synapses(net, o, "epoch %d end" % e)
        if c.get("static"):
            o.record_static()
            net.record()
            compare_neurons(net, o, "record %d" % e)
        else:
            _growth_both(o, net, e + 1)
    assert net.error_word == 0
    return o, net
