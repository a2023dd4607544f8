"""Launch configurations and the autotuner.

Every launch configuration computes the same thing: the configuration only changes grids, block
sizes and pipeline depths, never the order of any floating-point operation.  The autotuner times
candidates from a copy of the network's state and puts the state back."""
import numpy as np
import pytest

from braingrid_gb300 import lib as bg
from tests.golden.configs import case
from tests.gpu_helpers import gpu_from_oracle
from tests.netcases import assert_same, oracle_from_case

pytestmark = pytest.mark.gpu

CONFIGS = [dict(sweep_stages=4, thin_warps=4, deliver_blocks=152, growth_threads=128,
                izh_hw_every=0, small_max_slots=0),
           dict(sweep_stages=8, thin_warps=16, deliver_blocks=608, growth_threads=512,
                deliver_early=0),
           dict(sweep_dests=16, sweep_stages=6, izh_hw_every=1, small_max_slots=0),
           dict(sweep_dests=16, sweep_stages=4, izh_hw_every=3),
           dict(thin_max_quads=64, thin_warps=2, deliver_blocks=17),
           dict(thin_max_quads=1, sweep_stages=6, deliver_blocks=1, deliver_early=0)]


def make(name, seed=3):
    c = case(name)
    o = oracle_from_case(c)
    net = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE, noise_seed=seed)
    net.static = bool(c.get("static"))
    if not net.static:
        net.growth(1)
    return net


def epoch_end(net, e):
    if net.static:
        net.record()
    else:
        net.growth(e)


def state(net):
    g = net.download_lif()
    s = net.download_synapses()
    used = s["in_use"].astype(bool)
    out = {k: g[k] for k in ("Vm", "spikeCount", "history", "nStepsInRefr")}
    out.update({k: s[k][used] for k in ("W", "psr", "u", "r", "lastSpike", "delayQueue")})
    return out


@pytest.mark.parametrize("name", ["c0_grown", "izh_static", "izh_dstdp"])
def test_every_launch_configuration_gives_the_same_state(name):
    ref = make(name)
    ref.step(1500)
    epoch_end(ref, 2)
    ref.step(300)
    want = state(ref)
    for cfg in CONFIGS:
        net = make(name)
        net.set_launch(**cfg)
        net.step(1500)
        epoch_end(net, 2)
        net.step(300)
        got = state(net)
        for k in want:
            assert_same("%s %s %s" % (name, cfg, k), got[k], want[k])
        assert net.error_word == 0


def test_autotune_leaves_the_state_unchanged():
    tuned = make("c0_grown")
    plain = make("c0_grown")
    tuned.step(700)
    plain.step(700)
    before = state(tuned)
    cfg, ms = tuned.autotune(steps_per_trial=100, growth=True)
    assert ms > 0 and cfg == tuned.launch
    after = state(tuned)
    for k in before:
        assert_same("after tuning " + k, after[k], before[k])
    tuned.step(500)
    plain.step(500)
    a, b = state(tuned), state(plain)
    for k in a:
        assert_same("tuned vs untuned " + k, a[k], b[k])


def test_batch_autotune_keeps_results():
    # one TMA-swept and one thin network of the same synapse kind
    nets = [make("izh_dstdp", 5), make("izh_static", 6)]
    twins = [make("izh_dstdp", 5), make("izh_static", 6)]
    b = bg.Batch(nets)
    cfg, ms = b.autotune(steps_per_trial=50)
    assert ms > 0
    b.step(400)
    b.sync()
    for n in twins:
        n.step(400)
    for k, (p, q) in enumerate(zip(twins, nets)):
        sp, sq = state(p), state(q)
        for f in sp:
            assert_same("net %d %s" % (k, f), sq[f], sp[f])


def test_invalid_launch_configurations_are_rejected():
    net = make("c0_grown")
    for bad in (dict(sweep_stages=5), dict(thin_warps=0), dict(growth_threads=64),
                dict(deliver_blocks=0), dict(sweep_dests=8), dict(deliver_early=2),
                dict(izh_hw_every=9), dict(izh_hw_every=-2), dict(small_max_slots=-1)):
        with pytest.raises(RuntimeError):
            net.set_launch(**bad)
