"""bg3_download_state: the whole observable state in one call equals the single-purpose
downloads (neurons, Izhikevich, synapses, STDP, index maps, growth radii and rates)."""
import pytest

from tests.golden.configs import case
from tests.gpu_helpers import gpu_from_oracle
from tests.netcases import assert_same, oracle_from_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["izh_dstdp", "c0_grown"])
def test_download_state_equals_single_downloads(name):
    c = case(name)
    o = oracle_from_case(c)
    from braingrid_gb300 import lib as bg
    net = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE)
    net.step(1500)
    izh, stdp = c.get("neuron") == "izh", c.get("synapse", 1) >= 2
    st = net.download_state(izh=izh, stdp=stdp)
    for k, v in net.download_lif().items():
        assert_same("neurons " + k, st["neurons"][k], v)
    for k, v in net.download_synapses().items():
        assert_same("synapses " + k, st["synapses"][k], v)
    for k, v in net.download_maps().items():
        assert_same("maps " + k, st["maps"][k], v)
    r, q = net.download_growth()
    assert_same("radii", st["radii"], r)
    assert_same("rates", st["rates"], q)
    if izh:
        for k, v in net.download_izh().items():
            assert_same("izh " + k, st["izh"][k], v)
    if stdp:
        for k, v in net.download_stdp().items():
            assert_same("stdp " + k, st["stdp"][k], v)
    if not izh:
        with pytest.raises(bg.Bg3Error):
            net.download_state(izh=True)
    net.close()
    o.close()


def test_stdp_weight_exponent_other_than_zero_is_refused():
    """The reference raises W to mupos / muneg with the host's pow (both 0 in its createSynapse);
    the library accepts only 0 and refuses other exponents instead of rounding them differently."""
    from braingrid_gb300 import lib as bg
    from tests.gpu_helpers import stdp_constants
    c = case("c0_stdp")
    o = oracle_from_case(c)
    net = gpu_from_oracle(o, c, noise_mode=bg.BG3_NOISE_DEVICE)
    k = stdp_constants(c)
    net.set_stdp_constants(**k)
    for field in ("mupos", "muneg"):
        bad = dict(k, **{field: 0.5})
        with pytest.raises(bg.Bg3Error) as e:
            net.set_stdp_constants(**bad)
        assert "(-6)" in str(e.value)  # BG3_EUNSUPPORTED
    net.step(100)
    assert net.error_word == 0
    net.close()
    o.close()
