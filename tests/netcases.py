"""Helpers that build the same network in the oracle and compare states against fixtures."""
import os

import numpy as np

from oracle import pyoracle as po
from tests.golden.configs import IZH_IF_RANGES, IZH_RANGES, LIF_RANGES, TEST_SMALL, case  # noqa: F401

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fixture(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def oracle_from_case(c, record_noise=0):
    """Set up an oracle network exactly as Model::setupSim does for this case."""
    izh = c.get("neuron") == "izh"
    o = po.OracleNet(c["N"], c["max_syn"], c["width"], c["height"], c["tsim"], 1e-4,
                     c["max_firing_rate"], c["epochs"], neuron_kind=1 if izh else 0,
                     synapse_kind=c.get("synapse", 1))
    o.layout_grid()
    o.set_types(c["inh"], c["starters"])
    stim = c.get("stim")
    # FSInput::CreateInstance runs before setupSim (Core/BGDriver.cpp:72-74), so a regular
    # input's random phases are drawn from the global rng before the neuron parameters
    if stim and stim["kind"] == "regular":
        o.input_regular(stim["duration"], stim["interval"], stim["sync"], stim["values"])
    if izh:
        o.create_izh(IZH_IF_RANGES, IZH_RANGES)
    else:
        o.create_lif(LIF_RANGES)
    if c.get("stdp") is not None:
        o.stdp_params(c["stdp"])
    if c.get("static"):
        load_static_synapses(o, c)
    if stim and stim["kind"] == "poisson":
        o.input_poisson(stim["fr_mean"], stim["weight"], stim.get("masks"))
    g = c["growth"]
    o.growth_init(g["epsilon"], g["beta"], g["rho"], g["target_rate"], g["min_radius"],
                  g["start_radius"])
    o.seed_noise(c["seed"])
    if record_noise:
        o.record_noise(record_noise)
    if c.get("radii") is not None:
        o.arr("radii")[:] = np.float32(c["radii"])
    return o


def load_static_synapses(o, c):
    """ConnStatic::setupConnections' synapses (Connections/ConnStatic.cpp:33-88) taken from the
    reference's own dump of the case (its neighbour sort breaks distance ties in libstdc++'s
    order), added in slot order so every row fills as in the reference; the global rng then
    skips the one weight draw per synapse."""
    fx = load_fixture(c["name"])
    slots = fx["i.slots"].astype(np.int64)
    for k, s in enumerate(slots):
        o.create_synapse(int(s // c["max_syn"]), int(fx["i.src"][k]), int(fx["i.type"][k]),
                         float(fx["i.W"][k]))
    assert o.rebuild_maps() == 0
    o.rng_skip(len(slots))


def steps_per_epoch(c):
    # static_cast<uint64_t>(epochDuration / deltaT) in float (Core/Simulator.cpp:159-160)
    return int(np.float32(c["tsim"]) / np.float32(1e-4))


def bits(a):
    a = np.asarray(a)
    if a.dtype == np.float32:
        return a.view(np.uint32)
    if a.dtype == np.float64:
        return a.view(np.uint64)
    return a


def assert_same(name, got, want):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, "%s: shape %s vs %s" % (name, got.shape, want.shape)
    if got.dtype.kind == "f":
        want = want.astype(got.dtype)
    gb, wb = bits(got), bits(want.astype(got.dtype) if got.dtype != want.dtype else want)
    if not np.array_equal(gb, wb):
        bad = np.nonzero(gb != wb)[0]
        raise AssertionError("%s: %d of %d differ, first at %d: %r vs %r"
                             % (name, len(bad), got.size, bad[0], got.flat[bad[0]],
                                want.flat[bad[0]]))


def raster_from_history(history, counts, offsets, N, ms):
    h = history.reshape(N, ms)
    steps, nrn = [], []
    for i in range(N):
        for j in range(int(counts[i])):
            steps.append(int(h[i, (int(offsets[i]) + j) % ms]))
            nrn.append(i)
    if not steps:
        return np.zeros((2, 0), np.int64)
    s, n = np.array(steps, np.int64), np.array(nrn, np.int64)
    order = np.lexsort((n, s))
    return np.stack([s[order], n[order]])


SYN_FIELDS = ("W", "src", "dest", "type", "psr", "decay", "tau", "total_delay", "queue",
              "delayIdx", "ldelayQueue", "lastSpike", "r", "u", "D", "U", "F", "queuePost",
              "delayIdxPost", "total_delayPost", "tauspost", "tauspre", "taupos", "tauneg",
              "STDPgap", "Wex", "Aneg", "Apos", "mupos", "muneg")
