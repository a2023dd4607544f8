"""CUDA path vs the oracle, step-locked, through the C-ABI (libbg3).

Injected-noise mode: the GPU consumes the reference noise stream in the reference's CPU order,
so spike rasters, refractory counters, spike counts, delay-queue bitmasks, index maps and
per-pair synapse counts must be bit-exact, and so must Vm, psr and the summation points (the
library rounds every float operation as the reference's x86-64 build does).

Growth weights go through acos/sin; the device evaluates them in double and rounds once, while
the reference uses glibc's float acosf/sinf, which are not correctly rounded for some arguments.
Weights are therefore compared within 1e-5 relative, and the strict tests then load the oracle's
weights (bg3_upload_weights) so that the following epochs stay bit-comparable.
test_free_running_on_own_growth_weights runs on the GPU's own growth weights instead: rasters
bit-exact up to the first growth, then Vm and psr within 1e-5 relative for as long as the two
rasters agree, and it reports the first step at which they part (if any).
"""
import numpy as np
import pytest

from braingrid_gb300 import lib as bg
from tests.golden.configs import case
from tests.gpu_helpers import (_growth_both, compare_history, compare_maps,
                               compare_neurons, compare_synapses, gpu_from_oracle, run_locked)
from tests.netcases import (assert_same, load_fixture, oracle_from_case, raster_from_history,
                            steps_per_epoch)

pytestmark = pytest.mark.gpu


def test_c0_first_epoch_bit_exact():
    """The 10x10 network (no synapses yet): every step of the first 1 s epoch."""
    run_locked("c0", epochs=1, check_every=1)


def test_c0_ten_epochs_epoch_ends_bit_exact():
    """The 10x10 network in full (10 x 1 s, 100,000 steps): radii, rates, spike histories and recorder
    histograms equal the oracle's at every epoch end, hence the FP32 reference's (whose gap to the
    FP64 build is pinned in test_oracle_golden)."""
    c = case("c0")
    spe = steps_per_epoch(c)
    o = oracle_from_case(c)
    net = gpu_from_oracle(o, c, n_noise=c["N"] * spe * c["epochs"] + 64)
    for e in range(c["epochs"]):
        o.step_n(spe)
        net.step(spe)
        compare_history(net, o, "epoch %d" % e)
        _growth_both(o, net, e + 1)
    b, s, rh, ra = net.download_histories()
    assert_same("burstiness", b, o.arr("burstinessHist"))
    assert_same("spikes history", s, o.arr("spikesHistory"))
    assert_same("radii history", ra, o.arr("radiiHistory"))
    assert_same("rates history", rh, o.arr("ratesHistory"))
    assert net.error_word == 0


def test_ref_tiny_bit_exact_vs_reference_fixture():
    o, net = run_locked("ref_tiny", check_every=1)
    fx = load_fixture("ref_tiny")
    b, s, rh, ra = net.download_histories()
    # the GPU histories vs the reference run itself
    assert_same("radii", ra.reshape(2, 4)[1], fx["post.radii"])


def test_c0_grown_bit_exact_with_synapses():
    """Pre-grown 10x10: growth wires it after epoch 1; DS dynamics for 4 more epochs."""
    o, net = run_locked("c0_grown", check_every=10, syn_every=500)
    assert o.total > 0


def test_c0_grown_gpu_raster_matches_reference_dump():
    """GPU vs the compiled reference directly (the fixture), not only vs the oracle."""
    c = case("c0_grown")
    fx = load_fixture("c0_grown")
    spe = steps_per_epoch(c)
    o = oracle_from_case(c)
    net = gpu_from_oracle(o, c, n_noise=c["N"] * spe * c["epochs"] + 64)
    for e in range(c["epochs"]):
        net.step(spe)
        g = net.download_lif()
        raster = raster_from_history(g["history"], g["spikeCount"], g["spikeCountOffset"],
                                     c["N"], net.max_spikes)
        assert_same("raster#%d" % e, raster, fx["raster#%d" % e])
        o.step_n(spe)
        o.growth()
        o.record_epoch(e + 1)
        net.growth(e + 1)
        net.upload_weights(o.arr("W"))
    assert net.error_word == 0


def test_regular_input_bit_exact():
    """Regular pulses with random per-neuron phases (10x10 network, 2 x 0.5 s)."""
    o, net = run_locked("c0_regular", check_every=50)
    assert int(o.arr("spikeCount").sum()) >= 0


@pytest.mark.parametrize("name", ["c0_poisson", "c0_poisson25"])
def test_poisson_input_bit_exact(name):
    """Poisson drive with the reference's own ISI draws (masked / all neurons, growth wiring)."""
    o, net = run_locked(name, check_every=20, syn_every=500)


def test_izhikevich_bit_exact():
    """Izhikevich neurons (AllIZHNeurons) on a pre-grown 12x12 DS network: Vm, u, spikes and
    synapses step-locked with the oracle over 5 epochs with growth."""
    o, net = run_locked("izh_grown", check_every=10, syn_every=500)
    fired = int((o.arr("history") != np.uint64(0xFFFFFFFFFFFFFFFF)).sum())
    assert o.total > 0 and fired > 0


def test_spiking_synapses_bit_exact():
    """Plain AllSpikingSynapses (no facilitation / depression) on a pre-grown 10x10 network."""
    o, net = run_locked("c0_spiking", check_every=10, syn_every=500)
    assert o.total > 0


@pytest.mark.parametrize("name", ["c0_stdp", "c0_dstdp"])
def test_stdp_bit_exact(name):
    """STDP / dynamic STDP with the reference's createSynapse constants (host-build arithmetic):
    weights, PSRs and the reconstructed post queues step-locked with the oracle."""
    o, net = run_locked(name, check_every=10, syn_every=250)
    assert o.total > 0


def test_izhikevich_dynamic_stdp_poisson_bit_exact():
    """Izhikevich neurons, dynamic STDP with bounded additive constants, Poisson drive."""
    o, net = run_locked("izh_dstdp", check_every=10, syn_every=250)
    assert o.total > 0


def test_static_connections_izhikevich_stdp_bit_exact():
    """ConnStatic network (the reference's own setupConnections output) with Izhikevich
    neurons, dynamic STDP and Poisson drive; the epoch end runs the plain recorder."""
    o, net = run_locked("izh_static", check_every=10, syn_every=250)
    assert o.total > 1000
    b, s, rh, ra = net.download_histories()
    assert_same("burstiness", b, o.arr("burstinessHist"))
    assert_same("spikes history", s, o.arr("spikesHistory"))


def test_stdp_device_arithmetic_bit_exact():
    """The reference device build's signed spike-time arithmetic (depression applies)."""
    o, net = run_locked("izh_dstdp", check_every=10, syn_every=250, stdp_signed=True)
    assert o.total > 0


@pytest.mark.slow
def test_m30_grown_bit_exact():
    run_locked("m30_grown", check_every=100, syn_every=1000)


def test_large_pregrown_network_bit_exact():
    """100x100 network wired by one growth pass at radius 6 (~110 synapses per neuron),
    then 300 steps step-locked."""
    c = dict(case("c0"), name="big", width=100, height=100, N=10000, max_syn=200, tsim=0.1,
             epochs=1, max_firing_rate=1000, radii=6.0)
    from tests.golden.configs import site_lists
    c["inh"], c["starters"] = site_lists(100, 100, 0.10, 100, seed=7)
    o = oracle_from_case(c)
    o.growth()
    o.record_epoch(1)
    assert o.total > 500000
    net = gpu_from_oracle(o, c, n_noise=c["N"] * 400)
    compare_maps(net, o, "upload")
    for t in range(300):
        o.step_n(1)
        net.step(1)
        if (t + 1) % 25 == 0:
            compare_neurons(net, o, "step %d" % (t + 1))
    compare_synapses(net, o, "after 300 steps")
    assert net.error_word == 0


def test_high_fanout_bursts_bit_exact():
    """60x60 network wired at radius 8 (~700 synapses per neuron, unscaled growth weights): the
    network bursts, so steps carry many spiking sources whose fan-out spans several delivery
    chunks; 400 steps step-locked."""
    c = dict(case("c0"), name="burst", width=60, height=60, N=3600, max_syn=1000, tsim=0.1,
             epochs=1, max_firing_rate=1000, radii=8.0)
    from tests.golden.configs import site_lists
    c["inh"], c["starters"] = site_lists(60, 60, 0.10, 60, seed=9)
    o = oracle_from_case(c)
    o.growth()
    o.record_epoch(1)
    assert o.total > 2000000
    # start every membrane near threshold so that the network bursts at once
    rs = np.random.RandomState(5)
    o.arr("Vm")[:] = rs.uniform(13.0e-3, 15.5e-3, c["N"]).astype(np.float32)
    net = gpu_from_oracle(o, c, n_noise=c["N"] * 500)
    for t in range(400):
        o.step_n(1)
        net.step(1)
        if (t + 1) % 25 == 0:
            compare_neurons(net, o, "step %d" % (t + 1))
    fired = int(o.arr("spikeCount").sum())
    assert fired > 20000, fired
    compare_synapses(net, o, "after 400 steps")
    assert net.error_word == 0


def test_device_noise_mode_runs_and_is_deterministic():
    c = case("c0_grown")
    outs = []
    for _ in range(2):
        o = oracle_from_case(c)
        net = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE, noise_seed=11)
        net.step(2000)
        net.growth(1)
        net.step(2000)
        g = net.download_lif()
        outs.append((g["Vm"].copy(), g["spikeCount"].copy(), net.total_synapses()))
        assert net.error_word == 0
    assert_same("Vm", outs[0][0], outs[1][0])
    assert_same("spikes", outs[0][1], outs[1][1])
    assert outs[0][2] == outs[1][2] > 0


@pytest.mark.parametrize("name", ["ragged", "ragged_izh"])
def test_ragged_shapes_bit_exact(name):
    """Neuron counts that leave a partial 32-dest tile (63, 65 neurons) and rows that end inside a
    row quad (30, 18 slots), DS and Izhikevich + dynamic STDP + Poisson."""
    o, net = run_locked(name, check_every=5, syn_every=50)
    assert o.total > 0


def test_device_weight_scaling_matches_host_scaling():
    """bg3_scale_weights gives the same bits as scaling the downloaded weights on the host."""
    c = case("c0_grown")
    o = oracle_from_case(c)
    a = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE)
    b = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE)
    a.growth(1)
    b.growth(1)
    f = np.float32(0.003)
    a.scale_weights(f)
    s = b.download_synapses()
    b.upload_weights((s["W"] * f).astype(np.float32))
    sa, sb = a.download_synapses(), b.download_synapses()
    assert int(sa["in_use"].sum()) > 0
    assert_same("W", sa["W"], sb["W"])
    a.close()
    b.close()


@pytest.mark.parametrize("name,epochs", [("c0_grown", 5), ("m30_grown", 5)])
def test_free_running_on_own_growth_weights(name, epochs):
    """No weight resync: the GPU keeps the weights its own growth passes computed (within 1e-5 of
    the reference's) and the oracle keeps its own.  Every 50 steps: spike rasters (counts and
    history) compared exactly; while they agree, Vm within 1e-5 relative and the psr of every
    in-use synapse within 1e-5 relative; the index maps and per-pair synapse counts after every
    growth exactly.  Before the first growth there are no synapses and everything is bit-exact.
    The first step at which the rasters part, if any, is printed (pytest -s)."""
    c = case(name)
    spe = steps_per_epoch(c)
    o = oracle_from_case(c)
    net = gpu_from_oracle(o, c, n_noise=c["N"] * spe * epochs + 64)
    every, first, worst_vm, worst_psr = 50, None, 0.0, 0.0
    for e in range(epochs):
        for k in range(spe // every):
            o.step_n(every)
            net.step(every)
            t = e * spe + (k + 1) * every
            g = net.download_lif()
            same = (np.array_equal(g["spikeCount"], o.arr("spikeCount")) and
                    np.array_equal(g["spikeCountOffset"], o.arr("spikeCountOffset")) and
                    np.array_equal(g["history"], o.arr("history")))
            if e == 0:
                assert same, "rasters differ before the first growth (step %d)" % t
                compare_neurons(net, o, "step %d" % t)
            if not same:
                if first is None:
                    first = t
                continue
            if first is not None:
                continue
            vm, ovm = g["Vm"].astype(np.float64), o.arr("Vm").astype(np.float64)
            rel = np.abs(vm - ovm) / np.maximum(np.abs(ovm), 1e-30)
            worst_vm = max(worst_vm, float(rel.max()))
            assert rel.max() <= 1e-5, "step %d: Vm relative difference %g" % (t, rel.max())
            if o.total and t % 500 == 0:
                used = o.arr("in_use").astype(bool)
                ps = net.download_synapses()["psr"][used].astype(np.float64)
                ops = o.arr("psr")[used].astype(np.float64)
                rel = np.abs(ps - ops) / np.maximum(np.abs(ops), 1e-30)
                rel[(ps == 0) & (ops == 0)] = 0.0
                worst_psr = max(worst_psr, float(rel.max()))
                assert rel.max() <= 1e-5, "step %d: psr relative difference %g" % (t, rel.max())
        o.growth()
        o.record_epoch(e + 1)
        net.growth(e + 1)
        if first is None:
            r, q = net.download_growth()
            assert_same("radii after growth %d" % (e + 1), r, o.arr("radii"))
            compare_maps(net, o, "growth %d" % (e + 1))
            sy = net.download_synapses()
            assert_same("counts after growth %d" % (e + 1), sy["counts"], o.arr("counts"))
            used = o.arr("in_use").astype(bool)
            np.testing.assert_allclose(sy["W"][used], o.arr("W")[used], rtol=1e-5, atol=0)
    assert o.total > 0 and net.error_word == 0
    print("%s free running on the GPU's own growth weights, %d steps: rasters %s; worst Vm "
          "relative difference %.3g, worst psr %.3g while they agreed"
          % (name, epochs * spe, "identical throughout" if first is None else
             "part at step %d" % first, worst_vm, worst_psr))


def test_benchmark_shape_step_locked():
    """The benchmark network's shape: 100x100 LIF + DS, 1,000 slots per neuron, one growth pass
    at radius U[8.35, 8.45] wiring ~7.6 M synapses on the 32-dest TMA sweep path; maps and
    per-pair counts bit-exact after the GPU's own growth pass, weights within 1e-5 relative or
    1e-7 of the largest weight (see below), then both
    sides take the oracle's weights times the benchmark's 0.003 (float products, the same bits on
    both) and every membrane starts just below threshold, so the first steps deliver heavy
    bursts; 2,000 steps step-locked with injected noise, neuron state checked every 250 steps and
    every synapse's state at 1,000 and 2,000."""
    from tests.golden.configs import site_lists
    N = 10000
    c = dict(case("c0"), name="plain100", width=100, height=100, N=N, max_syn=1000, tsim=1.0,
             epochs=1, max_firing_rate=200, radii=None, seed=7)
    c["inh"], c["starters"] = site_lists(100, 100, 0.10, 100, seed=7)
    o = oracle_from_case(c)
    rs = np.random.RandomState(11)
    o.arr("radii")[:] = rs.uniform(8.35, 8.45, N).astype(np.float32)
    net = gpu_from_oracle(o, c, n_noise=N * 2100)
    o.growth()
    o.record_epoch(1)
    net.growth(1)
    assert o.total > 7000000, o.total
    compare_maps(net, o, "growth")
    sy = net.download_synapses()
    assert_same("counts", sy["counts"], o.arr("counts"))
    used = o.arr("in_use").astype(bool)
    # A pair whose lenses barely overlap has angles near 0, where the reference's
    # 2 theta - sin 2 theta cancels: a one-ulp difference between glibc's acosf and the
    # correctly rounded acos grows there by ~6 / (2 theta)^2 (measured: 972 of 7.6 M weights
    # differ by up to 2.2e-4 relative, all below 2e-9 against a largest weight of 2e-6, absolute
    # differences at most 2.1e-14).  Such weights are compared against the network's scale.
    wg, wo = sy["W"][used].astype(np.float64), o.arr("W")[used].astype(np.float64)
    tol = 1e-5 * np.abs(wo) + 1e-7 * float(np.abs(wo).max())
    assert np.all(np.abs(wg - wo) <= tol), float(np.max(np.abs(wg - wo) - tol))
    o.arr("W")[:] = o.arr("W") * np.float32(0.003)
    net.upload_weights(o.arr("W"))
    o.arr("Vm")[:] = rs.uniform(13.0e-3, 15.2e-3, N).astype(np.float32)
    net.upload_lif(Vm=o.arr("Vm"))
    for t in range(250, 2001, 250):
        o.step_n(250)
        net.step(250)
        compare_neurons(net, o, "step %d" % t)
        compare_history(net, o, "step %d" % t)
        if t % 1000 == 0:
            compare_synapses(net, o, "step %d" % t)
    fired = int(o.arr("spikeCount").sum())
    assert fired > 1000, fired
    assert net.error_word == 0
    print("benchmark shape: %d synapses, %d spikes in 2,000 steps" % (o.total, fired))
