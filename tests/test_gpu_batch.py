"""Batched form (bg3_batch_*): one launch per kernel per step over many networks must give the
same state, bit for bit, as stepping every network on its own with bg3_step."""
import numpy as np
import pytest

from braingrid_gb300 import lib as bg
from braingrid_gb300 import netgen
from tests.netcases import assert_same

pytestmark = pytest.mark.gpu

SIZES = [(10, 10, 1.5, 3), (20, 20, 2.0, 4), (30, 30, 2.6, 5), (7, 13, 1.8, 6)]


def make_set():
    nets = []
    for w, h, r, seed in SIZES:
        spec = netgen.lif_network(w, h, seed=seed)
        # rows stay below max_syn (the reference aborts on a full row): (2r)^2 pi < 120
        net = netgen.make_gpu_network(spec, 120, epoch_duration=0.5, max_firing_rate=400,
                                      noise_seed=seed)
        netgen.pregrow(net, spec, r, weight_scale=0.2, seed=seed)
        nets.append(net)
    return nets


def state(net):
    g = net.download_lif()
    s = net.download_synapses()
    return g, s


def test_batch_matches_plain_networks_bit_exact():
    plain = make_set()
    batched = make_set()
    assert all(n.total_synapses() > 0 for n in plain)
    b = bg.Batch(batched)
    for chunk in (1, 37, 1500, 3, 800):
        for n in plain:
            n.step(chunk)
        b.step(chunk)
        b.sync()
        for k, (p, q) in enumerate(zip(plain, batched)):
            gp, sp = state(p)
            gq, sq = state(q)
            for f in ("Vm", "summation", "nStepsInRefr", "spikeCount", "history"):
                assert_same("net %d %s" % (k, f), gq[f], gp[f])
            used = sp["in_use"].astype(bool)
            for f in ("psr", "u", "r", "lastSpike", "delayQueue", "delayIdx"):
                assert_same("net %d %s" % (k, f), sq[f][used], sp[f][used])
    assert sum(int(n.download_lif()["spikeCount"].sum()) for n in plain) > 0
    errs = [n.error_word for n in plain + batched]
    assert all(e == 0 for e in errs), errs


def test_batch_then_member_step_and_growth():
    """A member stays usable on its own between batch steps (stream ordering both ways)."""
    plain = make_set()
    batched = make_set()
    b = bg.Batch(batched)
    b.step(50)
    batched[1].step(10)
    batched[1].growth(1)
    b.refresh()
    b.step(40)
    for n in plain:
        n.step(50)
    plain[1].step(10)
    plain[1].growth(1)
    for n in plain:
        n.step(40)
    b.sync()
    for k, (p, q) in enumerate(zip(plain, batched)):
        assert_same("net %d Vm" % k, q.download_lif()["Vm"], p.download_lif()["Vm"])
        assert p.sim_step == q.sim_step


def make_mixed_stdp():
    """An Izhikevich network with Poisson drive and a LIF network (device-build STDP
    arithmetic), both dynamic STDP and wired by one device growth pass, and a statically wired
    Izhikevich network of at most 32 synapses per neuron (thin sweep tiles in the same batch)."""
    from tests.golden.configs import case
    from tests.gpu_helpers import gpu_from_oracle
    from tests.netcases import oracle_from_case
    nets = []
    for name, seed, signed in (("izh_dstdp", 3, False), ("c0_dstdp", 5, True),
                               ("izh_static", 7, False)):
        c = case(name)
        o = oracle_from_case(c)
        if signed:
            o.stdp_signed(True)
        net = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE, noise_seed=seed)
        if not c.get("static"):
            net.growth(1)
        nets.append(net)
    return nets


def test_batch_izhikevich_stdp_matches_plain_bit_exact():
    plain = make_mixed_stdp()
    batched = make_mixed_stdp()
    assert all(n.total_synapses() > 0 for n in plain)
    b = bg.Batch(batched)
    for chunk in (1, 250, 2000):
        for n in plain:
            n.step(chunk)
        b.step(chunk)
        b.sync()
        for k, (p, q) in enumerate(zip(plain, batched)):
            gp, sp = state(p)
            gq, sq = state(q)
            for f in ("Vm", "nStepsInRefr", "spikeCount", "history"):
                assert_same("net %d %s" % (k, f), gq[f], gp[f])
            used = sp["in_use"].astype(bool)
            for f in ("W", "psr", "u", "r", "lastSpike"):
                assert_same("net %d %s" % (k, f), sq[f][used], sp[f][used])
        assert_same("izh u", batched[0].download_izh()["u"], plain[0].download_izh()["u"])
    assert all(int(n.download_lif()["spikeCount"].sum()) > 0 for n in plain)
    errs = [n.error_word for n in plain + batched]
    assert all(e == 0 for e in errs), errs


def make_thin_lif():
    """Four LIF networks of 45 k-75 k neurons with at most 40 synapses per neuron (thin tiles,
    last tile partial in three of them) and regular input: ~7,500 thin tiles, so that every warp
    of the pipelined thin sweep runs several tiles in a row."""
    nets = []
    for w, h, seed in ((260, 260, 21), (301, 151, 22), (199, 257, 23), (283, 263, 24)):
        spec = netgen.lif_network(w, h, seed=seed)
        net = netgen.make_gpu_network(spec, 40, epoch_duration=0.5, max_firing_rate=400,
                                      noise_seed=seed)
        netgen.pregrow(net, spec, 1.6, weight_scale=0.5, seed=seed)
        rs = np.random.RandomState(seed)
        net.input_regular(rs.uniform(0.5e-9, 2e-9, spec["N"]), rs.randint(0, 100, spec["N"]),
                          20, 100)
        nets.append(net)
    return nets


def _compare(plain, batched, fields):
    for k, (p, q) in enumerate(zip(plain, batched)):
        gp, sp = state(p)
        gq, sq = state(q)
        for f in ("Vm", "nStepsInRefr", "spikeCount", "history"):
            assert_same("net %d %s" % (k, f), gq[f], gp[f])
        used = sp["in_use"].astype(bool)
        for f in fields:
            assert_same("net %d %s" % (k, f), sq[f][used], sp[f][used])


def test_thin_lif_batch_with_regular_input_matches_plain_bit_exact():
    plain = make_thin_lif()
    batched = make_thin_lif()
    assert all(n.total_synapses() > 0 for n in plain)
    b = bg.Batch(batched)
    for chunk in (1, 300, 45):
        for n in plain:
            n.step(chunk)
        b.step(chunk)
        b.sync()
        _compare(plain, batched, ("psr", "u", "r", "lastSpike"))
    assert sum(int(n.download_lif()["spikeCount"].sum()) for n in plain) > 0
    errs = [n.error_word for n in plain + batched]
    assert all(e == 0 for e in errs), errs


def test_thin_izhikevich_batch_matches_plain_bit_exact():
    """40 networks of the 512-network Izhikevich + dynamic STDP workload (N ~ U[500, 8000],
    Poisson drive): ~5,300 thin tiles over 40 networks, so that warps' runs of tiles cross from
    one network into the next."""
    from braingrid_gb300 import workloads
    plain = workloads.build_izh512(count=40, seed=5)
    batched = workloads.build_izh512(count=40, seed=5)
    b = bg.Batch(batched)
    for chunk in (1, 400, 33):
        for n in plain:
            n.step(chunk)
        b.step(chunk)
        b.sync()
        _compare(plain, batched, ("W", "psr", "u", "r", "lastSpike"))
        for k, (p, q) in enumerate(zip(plain, batched)):
            assert_same("net %d izh u" % k, q.download_izh()["u"], p.download_izh()["u"])
    assert sum(int(n.download_lif()["spikeCount"].sum()) for n in plain) > 0
    errs = [n.error_word for n in plain + batched]
    assert all(e == 0 for e in errs), errs
    b.close()
    for n in plain + batched:
        n.close()


@pytest.mark.parametrize("warps", [1, 32])
def test_thin_tile_table_padding_at_any_block_size(warps):
    """The thin tile table pads each network's tiles to whole blocks of the configured warps: one
    warp a block (no padding) and 32 (a network of up to 32 tiles in one block, the rest idle
    entries) give the plain networks' results bit for bit."""
    plain = make_mixed_stdp()
    batched = make_mixed_stdp()
    b = bg.Batch(batched)
    b.set_launch(thin_warps=warps)
    for chunk in (1, 300):
        for n in plain:
            n.step(chunk)
        b.step(chunk)
        b.sync()
        _compare(plain, batched, ("W", "psr", "u", "r", "lastSpike"))
    errs = [n.error_word for n in plain + batched]
    assert all(e == 0 for e in errs), errs
    b.close()
