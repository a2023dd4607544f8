"""Small networks run many steps per launch in one CTA (k_small_run): the same results as the
multi-kernel step path, bit for bit, and as the oracle.

Networks of at most 2,048 neurons and small_max_slots synapse slots take the one-CTA path by
default, so every step-locked test of the 100-neuron cases already compares it with the oracle
one step per call.  Here whole epochs go through one bg3_step call each (thousands of steps per
launch) on both paths, in both noise modes, for every synapse kind, both neuron models and both
inputs, and the oracle checks the one-CTA path at every epoch end."""
import pytest

from braingrid_gb300 import lib as bg
from tests.golden.configs import case
from tests.gpu_helpers import (compare_history, compare_maps, compare_neurons, compare_synapses,
                               gpu_from_oracle)
from tests.netcases import assert_same, oracle_from_case, steps_per_epoch

pytestmark = pytest.mark.gpu

CASES = ["c0_grown", "c0_spiking", "c0_stdp", "c0_dstdp", "izh_dstdp", "c0_regular",
         "c0_poisson", "ragged", "ragged_izh", "izh_static"]


def _state(net, c):
    g = net.download_lif()
    out = {"lif." + k: v for k, v in g.items()}
    if net.total_synapses():
        out.update({"syn." + k: v for k, v in net.download_synapses().items()})
        out.update({"map." + k: v for k, v in net.download_maps().items()})
    if c.get("neuron") == "izh":
        out.update({"izh." + k: v for k, v in net.download_izh().items()})
    if c.get("synapse", 1) >= 2 and net.total_synapses():
        out.update({"stdp." + k: v for k, v in net.download_stdp().items()})
    if c.get("stim") and c["stim"]["kind"] == "poisson":
        out.update({"in." + k: v for k, v in net.download_poisson().items()})
    r, q = net.download_growth()
    out["radii"], out["rates"] = r, q
    return out


@pytest.mark.parametrize("mode", [bg.BG3_NOISE_INJECT, bg.BG3_NOISE_DEVICE])
@pytest.mark.parametrize("name", CASES)
def test_small_path_equals_launch_path(name, mode):
    c = case(name)
    spe = steps_per_epoch(c)
    E = c["epochs"]
    nets = []
    for small in (65536, 0):
        o = oracle_from_case(c)
        net = gpu_from_oracle(o, c, noise_mode=mode, n_noise=c["N"] * spe * E + 64,
                              isi_steps=spe * E + 2)
        net.set_launch(small_max_slots=small)
        nets.append((o, net))
    (o, small), (_, plain) = nets
    for e in range(E):
        l0, p0 = small.launches, plain.launches
        small.step(spe)
        plain.step(spe)
        assert small.launches - l0 == (spe + 4095) // 4096  # whole epoch in one or two launches
        assert plain.launches - p0 > spe
        if mode == bg.BG3_NOISE_INJECT:
            o.step_n(spe)
            compare_neurons(small, o, "epoch %d end" % e)
            compare_history(small, o, "epoch %d" % e)
            if o.total:
                compare_synapses(small, o, "epoch %d end" % e)
        a, b = _state(small, c), _state(plain, c)
        for k in a:
            assert_same("%s epoch %d %s" % (name, e, k), a[k], b[k])
        if c.get("static"):
            small.record()
            plain.record()
            if mode == bg.BG3_NOISE_INJECT:
                o.record_static()
        else:
            small.growth(e + 1)
            plain.growth(e + 1)
            if mode == bg.BG3_NOISE_INJECT:
                o.growth()
                o.record_epoch(e + 1)
                compare_maps(small, o, "growth %d" % (e + 1))
                small.upload_weights(o.arr("W"))
                plain.upload_weights(o.arr("W"))
    assert small.error_word == 0 and plain.error_word == 0
    for o_, n_ in nets:
        n_.close()
        o_.close()


def test_small_path_many_steps_per_call_c0():
    """The 100-neuron benchmark network (10 x 1 s, 100,000 steps), one bg3_step call per epoch
    (three launches of up to 4,096 steps each): the recorder histories equal the oracle's."""
    c = case("c0")
    spe = steps_per_epoch(c)
    o = oracle_from_case(c)
    net = gpu_from_oracle(o, c, n_noise=c["N"] * spe * c["epochs"] + 64)
    for e in range(c["epochs"]):
        net.step(spe)
        o.step_n(spe)
        compare_history(net, o, "epoch %d" % e)
        o.growth()
        o.record_epoch(e + 1)
        net.growth(e + 1)
    b, s, rh, ra = net.download_histories()
    assert_same("burstiness", b, o.arr("burstinessHist"))
    assert_same("spikes history", s, o.arr("spikesHistory"))
    assert_same("radii history", ra, o.arr("radiiHistory"))
    assert_same("rates history", rh, o.arr("ratesHistory"))
    assert net.error_word == 0
