"""Networks built from BrainGrid parameter files alone (braingrid_gb300.config / .sim) on the GPU.

(1) A whole run from the parameter file, with the reference's noise stream made by the library
(bg3_norm_*), writes the reference driver's result file byte for byte (tests/golden/outputs.npz,
written by the compiled reference from the same files).  (2) A ConnStatic + dynamic STDP +
Poisson network built by config.network runs in lock step with the oracle holding the same
wiring (config's neighbour order), bit for bit.  (3) With a Poisson stimulus (which the
reference's driver cannot run) the run from the parameter files gives the oracle's result file."""
import numpy as np
import pytest

from braingrid_gb300 import config as cf
from braingrid_gb300 import lib as bg
from braingrid_gb300 import sim
from tests.golden import configs
from tests.gpu_helpers import compare_input, compare_neurons, compare_synapses
from tests.netcases import assert_same, oracle_from_case, steps_per_epoch

pytestmark = pytest.mark.gpu


def read_output_case(name, tmp_path):
    c, text, stim = configs.output_case(name)
    configs.write_case(c, str(tmp_path / "configfiles"))
    return cf.read(text, stim, root=str(tmp_path))


@pytest.mark.parametrize("name", configs.OUTPUT_CASES)
def test_run_from_parameter_file_writes_reference_result(name, tmp_path):
    p = read_output_case(name, tmp_path)
    r = sim.simulate(p, noise="reference")
    assert r["error_word"] == 0
    assert r["steps"] == p.steps_per_epoch * p.epochs
    want = np.load("tests/golden/outputs.npz")[name].tobytes().decode()
    if r["text"] != want:
        got_l, want_l = r["text"].splitlines(), want.splitlines()
        bad = [i for i, (a, b) in enumerate(zip(got_l, want_l)) if a != b]
        raise AssertionError("%s: %d lines differ, first %r" % (
            name, len(bad), [(got_l[i][:120], want_l[i][:120]) for i in bad[:2]]))


@pytest.mark.parametrize("name", ["c0_poisson25"])
def test_run_with_poisson_stimulus_matches_oracle_result(name, tmp_path):
    """A Poisson stimulus (the reference's driver faults on one, so the oracle, pinned to the
    reference harness, writes the expected result file): the run from the parameter files with
    the reference's noise and interval draws gives the oracle's result file byte for byte."""
    from tests.test_config import oracle_output
    c, text, stim = configs.output_case(name)
    configs.write_case(c, str(tmp_path / "configfiles"))
    p = cf.read(text, stim, root=str(tmp_path))
    r = sim.simulate(p, noise="reference")
    assert r["error_word"] == 0
    assert r["text"] == oracle_output(name)


def test_cli_writes_result_file(tmp_path):
    c, text, stim = configs.output_case("ref_tiny")
    configs.write_case(c, str(tmp_path / "configfiles"))
    cfg = tmp_path / "tiny.xml"
    cfg.write_text(text)
    out = tmp_path / "out.xml"
    import os
    cwd = os.getcwd()
    os.chdir(str(tmp_path))
    try:
        assert sim.main(["-t", str(cfg), "-o", str(out), "-d", "0"]) == 0
        with pytest.raises(bg.Bg3Error):
            bg.set_device(4096)
    finally:
        os.chdir(cwd)
    assert out.read_text() == np.load("tests/golden/outputs.npz")["ref_tiny"].tobytes().decode()


def test_static_stdp_poisson_network_from_parameter_file(tmp_path):
    c = configs.case("izh_static")
    configs.write_case(c, str(tmp_path / "configfiles"), stdp_params=True)
    base = str(tmp_path / "configfiles" / "bg3" / c["name"])
    p = cf.read(base + ".xml", base + "-stim.xml", root=str(tmp_path))
    a = cf.setup(p)
    net = cf.network(p, a, noise_mode=bg.BG3_NOISE_INJECT)
    # the uploads round-trip
    g = net.download_synapses()
    s = a["synapses"]
    used = s["in_use"].astype(bool)
    assert_same("in_use", g["in_use"], s["in_use"])
    for k in ("src", "type", "W", "decay", "total_delay", "U", "D", "F", "u", "r"):
        assert_same(k, g[k][used], s[k][used])
    st = net.download_stdp()
    want = cf.stdp_arrays(s, cf.stdp_constants(p))
    for k in ("Apos", "Aneg", "Wex", "tauspost", "taupos", "tauneg"):
        assert_same(k, st[k][used], want[k][used])
    izh = net.download_izh()
    for k in ("Aconst", "Bconst", "Cconst", "Dconst", "C3"):
        assert_same(k, izh[k], a[k])

    # the oracle with the same wiring: the case minus the reference's dump, then the synapses in
    # creation order, then the weight draws skipped on its global generator
    o = oracle_from_case(dict(c, static=None))
    slots = a["creation_slots"]
    M = p.max_syn
    for sl in slots:
        o.create_synapse(int(sl // M), int(s["src"][sl]), int(s["type"][sl]), float(s["W"][sl]))
    assert o.rebuild_maps() == 0
    o.rng_skip(len(slots))
    spe = steps_per_epoch(c)
    steps = spe
    # the product's own interval draws (equal to the oracle's, test_config)
    begin, isis = cf.poisson_intervals(a, steps + 2)
    net.push_poisson_isis(begin, isis)
    net.push_noise(bg.NormStream(p.seed).take(c["N"] * steps + 64))
    for t in range(1, steps + 1):
        o.step_n(1)
        net.step(1)
        if t % 50 == 0:
            compare_neurons(net, o, "step %d" % t)
            compare_input(net, o, "step %d" % t)
    compare_synapses(net, o, "end")
    assert net.error_word == 0
    net.close()
    o.close()


def test_parameter_file_job_served_like_a_plain_network(tmp_path):
    """serve.config_job: a parameter file submitted to the job server (device noise) gives the
    histories of the same file run as a plain network."""
    from braingrid_gb300 import serve
    jobs = []
    for name in ("c0_regular", "izh_static"):
        c = configs.case(name)
        configs.write_case(c, str(tmp_path / "configfiles"), stdp_params=True)
        base = str(tmp_path / "configfiles" / "bg3" / name)
        stim = base + "-stim.xml" if c.get("stim") else None
        jobs.append((cf.read(base + ".xml", stim, root=str(tmp_path)), name))
    srv = serve.Server(max_resident=2, chunk_steps=400)
    served = [serve.config_job(p, name=name) for p, name in jobs]
    for j in served:
        srv.submit(j)
    done = srv.run_all()
    srv.close()
    assert len(done) == 2
    for (p, name), job in zip(jobs, served):
        assert job.result.status == 0 and job.result.error_word == 0, (name, job.error)
        net = cf.network(p)
        for e in range(p.epochs):
            net.step(p.steps_per_epoch)
            if p.conn_class == "ConnGrowth":
                net.growth(e + 1)
            else:
                net.record()
        b, s_, rh, ra = net.download_histories()
        plain = dict(burstiness=b, spikes_hist=s_, rates_hist=rh, radii_hist=ra,
                     Vm=net.download_lif(fields=("Vm",))["Vm"])
        out = job.outputs()
        for k in plain:
            assert_same("%s served vs plain %s" % (name, k), out[k][:len(plain[k])], plain[k])
        assert net.error_word == 0
        net.close()


def test_driver_state_flags_match_reference(tmp_path):
    """sim's -w and -r against the reference driver's: the end-of-run checkpoint stream of the
    c0 run, and a second run started from that stream (its result file byte for byte, its own
    end-of-run stream), every neuron's uninitialised Isyn token aside."""
    from tests.test_oracle_serialize import comparable
    out = np.load("tests/golden/outputs.npz")
    c, text, stim = configs.output_case("c0")
    configs.write_case(c, str(tmp_path / "configfiles"))
    p = cf.read(text, stim, root=str(tmp_path))
    r = sim.simulate(p, "reference", save=True)
    assert comparable(r["stream"], c) == comparable(out["c0.ser"].tobytes(), c)
    r2 = sim.simulate(p, "reference", restore=out["c0.ser"].tobytes(), save=True)
    assert r2["error_word"] == 0
    assert r2["text"] == out["c0_resumed"].tobytes().decode()
    assert comparable(r2["stream"], c) == comparable(out["c0_resumed.ser"].tobytes(), c)
