"""bg3_set_noise_mode: the noise source switched between steps.  A network created with device
noise and switched to the injected stream runs in lock step with the oracle; one switched to
device noise matches a network created with it."""
import pytest

from braingrid_gb300 import lib as bg
from tests.golden.configs import case
from tests.gpu_helpers import compare_neurons, gpu_from_oracle
from tests.netcases import assert_same, oracle_from_case

pytestmark = pytest.mark.gpu


def test_switch_to_injected_stream_stays_bit_exact():
    c = case("c0")
    o = oracle_from_case(c)
    net = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE)
    net.set_noise_mode(bg.BG3_NOISE_INJECT, c["seed"])
    net.push_noise(bg.NormStream(c["seed"]).take(c["N"] * 600))
    for t in range(1, 601):
        o.step_n(1)
        net.step(1)
        if t % 100 == 0:
            compare_neurons(net, o, "step %d" % t)
    assert net.error_word == 0
    # a bad mode is refused and changes nothing
    with pytest.raises(bg.Bg3Error):
        net.set_noise_mode(7, 1)
    net.close()
    o.close()


def test_switch_to_device_noise_matches_a_device_network():
    c = case("c0_grown")
    o = oracle_from_case(c)
    a = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE, noise_seed=5)
    b = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_INJECT)
    b.set_noise_mode(bg.BG3_NOISE_DEVICE, 5)
    a.step(700)
    b.step(700)
    la, lb = a.download_lif(), b.download_lif()
    for k in la:
        assert_same("device-switched " + k, lb[k], la[k])
    assert a.error_word == 0 and b.error_word == 0
    a.close()
    b.close()
    o.close()
