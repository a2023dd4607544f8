"""bg3_checkpoint_save / bg3_checkpoint_load: a network restored from a checkpoint continues
exactly as the saved one would have, bit for bit, across epoch ends (growth or the plain
recorder), STDP, Izhikevich neurons, Poisson and regular input, injected and device noise.
Malformed checkpoints and checkpoints of another network shape are refused."""
import ctypes

import numpy as np
import pytest

from braingrid_gb300 import lib as bg
from tests.golden.configs import case
from tests.gpu_helpers import gpu_from_oracle
from tests.netcases import assert_same, oracle_from_case, steps_per_epoch

pytestmark = pytest.mark.gpu


def advance(net, c, t_from, t_to):
    """Steps from t_from to t_to, running the epoch pass whenever an epoch ends."""
    spe = steps_per_epoch(c)
    t = t_from
    while t < t_to:
        k = min(t_to, (t // spe + 1) * spe) - t
        net.step(k)
        t += k
        if t % spe == 0:
            if c.get("static"):
                net.record()
            else:
                net.growth(t // spe)
    net.sync()


def snapshot(net, c):
    s = {"lif." + k: v for k, v in net.download_lif().items()}
    s.update({"syn." + k: v for k, v in net.download_synapses().items()})
    s.update({"map." + k: v for k, v in net.download_maps().items()})
    for k, v in zip(("burstiness", "spikes", "rates_hist", "radii_hist"), net.download_histories()):
        s["hist." + k] = v
    s["radii"], s["rates"] = net.download_growth()
    if c.get("neuron") == "izh":
        s.update({"izh." + k: v for k, v in net.download_izh().items()})
    if c.get("synapse", 1) >= 2:
        s.update({"stdp." + k: v for k, v in net.download_stdp().items()})
    if c.get("stim") and c["stim"]["kind"] == "poisson":
        s.update({"in." + k: v for k, v in net.download_poisson().items()})
    s["step"] = np.array([net.sim_step], np.uint64)
    s["err"] = np.array([net.error_word], np.uint32)
    return s


def assert_snapshots_equal(a, b, where):
    assert set(a) == set(b)
    for k in sorted(a):
        assert_same("%s %s" % (where, k), b[k], a[k])


CASES = [("c0_grown", "inject"), ("c0_grown", "device"), ("izh_dstdp", "inject"),
         ("izh_dstdp", "device"), ("c0_regular", "inject"), ("c0_stdp", "inject"),
         ("izh_static", "device")]


@pytest.mark.parametrize("name,noise", CASES)
def test_resume_continues_bit_exact(name, noise):
    c = case(name)
    E, spe = c["epochs"], steps_per_epoch(c)
    o = oracle_from_case(c)
    inject = noise == "inject"
    net = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_INJECT if inject else bg.BG3_NOISE_DEVICE,
                          n_noise=c["N"] * spe * E + 64, isi_steps=spe * E + 2 if inject else 0)
    t0 = spe + spe // 3  # inside the second epoch, after one epoch pass
    advance(net, c, 0, t0)
    ck = net.checkpoint()
    advance(net, c, t0, spe * E)
    want = snapshot(net, c)
    assert want["step"][0] == spe * E

    # a fresh network of the same shape
    net2 = bg.Network.from_desc(net.desc)
    net2.load_checkpoint(ck)
    assert net2.sim_step == t0
    advance(net2, c, t0, spe * E)
    assert_snapshots_equal(want, snapshot(net2, c), "fresh")

    # the saved network itself, rewound
    net.load_checkpoint(ck)
    advance(net, c, t0, spe * E)
    assert_snapshots_equal(want, snapshot(net, c), "rewound")
    net.close()
    net2.close()


# Checkpoint layout (this library's own format): a 144-byte header whose last 8 bytes are an
# FNV-1a 64 checksum of everything after it, the saved descriptor (netdev_bytes), the decay and
# delay tables, the injected noise, then every device array as [uint64 bytes][bytes] in a fixed
# order: 'count' is the 34th array, 'ring_n' the 27th.
HDR = 144
ARR_COUNT, ARR_RING_N = 33, 26


def array_offset(ck, index):
    netdev = int(ck[12:16].view(np.uint32)[0])
    noise = int(ck[112:120].view(np.int64)[0])
    n_dtab, n_ltab = (int(v) for v in ck[120:128].view(np.uint32))
    p = HDR + netdev + 4 * n_dtab + 4 * n_ltab + 4 * noise
    for _ in range(index):
        p += 8 + int(ck[p:p + 8].view(np.uint64)[0])
    return p + 8


def reseal(ck):
    h = 0xcbf29ce484222325
    for b in ck[HDR:].tobytes():
        h = ((h ^ b) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    ck[HDR - 8:HDR] = np.frombuffer(np.uint64(h).tobytes(), np.uint8)


def test_checkpoint_is_refused_when_malformed_or_of_another_shape():
    c = case("c0_grown")
    o = oracle_from_case(c)
    net = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE)
    net.step(50)
    before = snapshot(net, c)
    ck = net.checkpoint()
    # too small a buffer: nothing written, size reported
    n = ctypes.c_uint64()
    small = np.zeros(16, np.uint8)
    assert net.L.bg3_checkpoint_save(net.h, small.ctypes.data, small.size,
                                     ctypes.byref(n)) == bg.BG3_EINVAL
    assert n.value == ck.size and not small.any()
    for bad in (ck[:-1], np.concatenate([ck, np.zeros(8, np.uint8)])):
        with pytest.raises(RuntimeError):
            net.load_checkpoint(bad)
    corrupt = ck.copy()
    corrupt[0] ^= 0xFF
    with pytest.raises(RuntimeError):
        net.load_checkpoint(corrupt)
    # a flipped byte deep inside the arrays: the checksum refuses it
    corrupt = ck.copy()
    corrupt[ck.size // 2] ^= 0x10
    with pytest.raises(RuntimeError):
        net.load_checkpoint(corrupt)
    # well-formed bytes (checksum recomputed) whose row count or spike-ring count would address
    # memory outside the network: refused by the content checks
    for array, value in ((ARR_COUNT, c["max_syn"] + 1), (ARR_RING_N, c["N"] + 1)):
        forged = ck.copy()
        off = array_offset(forged, array)
        forged[off:off + 4] = np.frombuffer(np.int32(value).tobytes(), np.uint8)
        reseal(forged)
        with pytest.raises(RuntimeError):
            net.load_checkpoint(forged)
    # another shape (one more neuron row)
    d = net.desc
    other = bg.Network(d.n_neurons + d.width, d.max_syn_per_neuron, d.width, d.height + 1,
                       d.epoch_duration, d.delta_t, d.max_firing_rate, d.max_epochs,
                       d.synapse_kind, d.noise_mode, d.noise_seed)
    with pytest.raises(RuntimeError):
        other.load_checkpoint(ck)
    # the refused loads changed nothing
    assert_snapshots_equal(before, snapshot(net, c), "after refusals")
    other.close()
    net.close()
