"""bg3_serialize / bg3_deserialize: the reference's checkpoint stream (Model::serialize).

A GPU run locked to the oracle writes, at the end of each case, the same bytes as the compiled
reference did (tests/golden/serialize.npz; the oracle is pinned to those bytes in
test_oracle_serialize), and reading the reference's bytes into a fresh network and writing them
out again gives them back unchanged."""
import numpy as np
import pytest

from braingrid_gb300 import lib as bg
from tests.golden.configs import case
from tests.gpu_helpers import run_locked
from tests.netcases import steps_per_epoch
from tests.test_oracle_serialize import SER_CASES, comparable, tokens

pytestmark = pytest.mark.gpu


def reference_stream(name):
    return np.load("tests/golden/serialize.npz")[name].tobytes()


def same_stream(name, got, want, c=None):
    """Byte-identical streams; with the case c, every neuron's Isyn token is left out (the
    reference's uninitialised field, see comparable)."""
    tg, tw = (comparable(got, c), comparable(want, c)) if c else (tokens(got), tokens(want))
    if tg != tw:
        bad = [i for i, (a, b) in enumerate(zip(tg, tw)) if a != b]
        raise AssertionError("%s: %d vs %d tokens, first differences %r" % (
            name, len(tg), len(tw), [(i, tg[i], tw[i]) for i in bad[:5]]))


@pytest.mark.parametrize("name", SER_CASES)
def test_gpu_stream_matches_reference(name):
    c = case(name)
    o, net = run_locked(name, check_every=10 ** 9)
    extra = {k: o.arr(k) for k in ("Cm", "Rm", "Vrest", "Vinit", "Iinject", "Tau")}
    got = net.serialize(growth=not c.get("static"), **extra)
    same_stream(name, got, reference_stream(name), c)
    net.close()


@pytest.mark.parametrize("name", SER_CASES)
def test_reference_stream_round_trip(name):
    c = case(name)
    want = reference_stream(name)
    growth = not c.get("static")
    izh = c.get("neuron") == "izh"
    net = bg.Network(c["N"], c["max_syn"], c["width"], c["height"], c["tsim"], 1e-4,
                     c["max_firing_rate"], c["epochs"], c.get("synapse", bg.BG3_SYN_DS),
                     bg.BG3_NOISE_DEVICE, c["seed"],
                     neuron_kind=bg.BG3_NEURON_IZH if izh else bg.BG3_NEURON_LIF)
    step = steps_per_epoch(c) * c["epochs"]
    extra = net.deserialize(want, growth=growth, step=step)
    assert net.sim_step == step
    same_stream(name, net.serialize(growth=growth, **extra), want)
    # the loaded network runs
    net.step(100)
    net.sync()
    assert net.error_word == 0
    net.close()


def test_malformed_streams_are_refused():
    c = case("c0_grown")
    want = reference_stream("c0_grown")
    net = bg.Network(c["N"], c["max_syn"], c["width"], c["height"], c["tsim"], 1e-4,
                     c["max_firing_rate"], c["epochs"], bg.BG3_SYN_DS, bg.BG3_NOISE_DEVICE, 1)
    step = steps_per_epoch(c) * c["epochs"]
    t = tokens(want)
    bad_count = b"\0".join([b"99"] + t[1:])          # another neuron count
    bad_value = b"\0".join(t[:5] + [b"x1"] + t[6:])  # not a number
    for data in (want[:-7], want + b"1\0", bad_count, bad_value):
        with pytest.raises(bg.Bg3Error):
            net.deserialize(data, growth=True, step=step)
    # a stream read into a network without ConnGrowth state ends early
    with pytest.raises(bg.Bg3Error):
        net.deserialize(want, growth=False, step=step)
    net.close()
