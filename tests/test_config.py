"""braingrid_gb300.config: BrainGrid parameter files read and set up as the reference does.

Every case's parameter file (tests/golden/configs.py writes the same files the reference harness
ran) is read back and set up; the arrays are compared with what the compiled reference built
from the same file (the fixtures' setup arrays), bit for bit, and with the oracle where the
fixtures hold no setup copy (input arrays).  ConnStatic's wiring is compared up to the order of
equal distances (see config's docstring).  No GPU: the network itself is built in
test_gpu_config.py."""
import os

import numpy as np
import pytest

from braingrid_gb300 import config as cf
from tests.golden import configs
from tests.golden.configs import CASES, case
from tests.netcases import assert_same, load_fixture, oracle_from_case

SETUP = ("Vm", "Vthresh", "Vreset", "Vrest", "Vinit", "I0", "Inoise", "Iinject", "C1", "C2",
         "Trefract", "Rm", "Cm", "Tau")
IZH = ("Aconst", "Bconst", "Cconst", "Dconst", "u", "C3")


def read_case(c, tmp_path, stdp_params=True):
    configs.write_case(c, str(tmp_path / "configfiles"), stdp_params)
    base = tmp_path / "configfiles" / "bg3" / c["name"]
    stim = str(base) + "-stim.xml" if c.get("stim") else None
    return cf.read(str(base) + ".xml", stim, root=str(tmp_path))


def test_mtrand_matches_the_oracle_generator():
    import ctypes
    from oracle import pyoracle as po
    L = po.lib()
    L.bgo_mt_randint.restype = ctypes.c_uint32
    state = ctypes.create_string_buffer(8192)      # holds the oracle's bgo_mt
    L.bgo_mt_seed(state, ctypes.c_uint32(1))
    want = np.array([L.bgo_mt_randint(state) for _ in range(2000)], np.uint32)
    m = cf.MTRand(1)
    got = np.concatenate([m.randint(1), m.randint(700), m.randint(0), m.randint(1299)])
    assert_same("randint", got, want)
    # rand() and inRange() as MTRand computes them
    m, u = cf.MTRand(1), want[:5].astype(np.float32).astype(np.float64) / 4294967295.0
    assert_same("rand", m.rand(5), u.astype(np.float32))
    m = cf.MTRand(1)
    v = m.in_range(np.float32(2), np.float32(7), 5)
    assert_same("inRange", v, (u.astype(np.float32) * np.float32(5)) + np.float32(2))


# the FP64 reference runs are long-run comparison bases with no setup arrays kept
NAMES = [c["name"] for c in CASES if not c.get("fp64")]


@pytest.mark.parametrize("name", NAMES)
def test_setup_matches_reference(name, tmp_path):
    c = case(name)
    fx = load_fixture(name)
    p = read_case(c, tmp_path)
    assert (p.width, p.height, p.epochs, p.max_syn, p.seed) == \
        (c["width"], c["height"], c["epochs"], c["max_syn"], c["seed"])
    assert p.max_firing_rate == c["max_firing_rate"]
    assert p.tsim == np.float32(c["tsim"])
    a = cf.setup(p)
    for k in SETUP:
        assert_same(k, a[k], fx[k])
    if c.get("neuron") == "izh":
        for k in IZH:
            assert_same(k, a[k], fx[k])
    assert_same("ntype", a["ntype"], fx["ntype"])
    assert_same("starter", a["starter"].astype(fx["starter"].dtype), fx["starter"])
    assert_same("xloc", a["xloc"], fx["xloc"])
    assert_same("yloc", a["yloc"], fx["yloc"])
    stim = c.get("stim")
    if stim:
        o = oracle_from_case(c)
        if stim["kind"] == "regular":
            assert_same("reg_values", a["regular"]["values"], o.arr("reg_values"))
            assert_same("reg_shift", a["regular"]["shifts"], o.arr("reg_shift"))
        else:
            pa = a["poisson"]["arrays"]
            for k, v in (("masks", "pois_mask"), ("nISIs", "pois_nisi"), ("total_delay", "in_delay"),
                         ("W", "in_W"), ("decay", "in_decay"), ("U", "in_U"), ("D", "in_D"),
                         ("F", "in_F"), ("u", "in_u"), ("r", "in_r"), ("lastSpike", "in_last")):
                assert_same("input " + k, pa[k], o.arr(v))
            fr = np.float32(stim["fr_mean"]) / np.float32(1000)
            assert np.float32(a["poisson"]["lam"]) == np.float32(1) / fr
        o.close()
    if c.get("static"):
        check_static(c, fx, p, a)


def check_static(c, fx, p, a):
    """ConnStatic wiring against the reference's: the same count per source and per (source,
    distance); the same destinations below each source's last distance kept; the same weights
    within each (source, distance) group; per-type constants equal.  Destination in-degrees
    differ where the tie choices differ (the reference's std::sort order)."""
    N, W, M = c["N"], c["width"], c["max_syn"]
    s = a["synapses"]
    used = np.nonzero(s["in_use"])[0]
    # per source (per destination the counts follow the tie choices)
    assert_same("out-degree", np.bincount(s["src"][used], minlength=N),
                np.bincount(fx["i.src"], minlength=N))
    assert a["counts"].sum() == fx["i.counts"].sum()

    def groups(slots, src, w):
        dest = slots // M
        dx = (src % W) - (dest % W)
        dy = (src // W) - (dest // W)
        d2 = dx * dx + dy * dy
        out = {}
        for k in range(len(slots)):
            out.setdefault((int(src[k]), int(d2[k])), []).append((int(dest[k]), float(w[k])))
        return out

    mine = groups(used, s["src"][used], s["W"][used])
    ref = groups(fx["i.slots"].astype(np.int64), fx["i.src"], fx["i.W"])
    assert set(mine) == set(ref)
    last = {}
    for (src, d2) in ref:
        last[src] = max(last.get(src, -1), d2)
    for key in ref:
        a_, b_ = sorted(mine[key]), sorted(ref[key])
        assert len(a_) == len(b_), key
        assert sorted(w for _, w in a_) == sorted(w for _, w in b_), key
        if key[1] < last[key[0]]:
            assert [d for d, _ in a_] == [d for d, _ in b_], key
    # per-type synapse constants
    for k in ("tau", "decay", "total_delay", "U", "D", "F", "u", "r", "psr", "lastSpike"):
        fk = {"lastSpike": "i.lastSpike"}.get(k, "i." + k)
        for t in range(4):
            mt, rt = s["type"][used] == t, fx["i.type"] == t
            if rt.any():
                assert set(np.unique(s[k][used][mt]).tolist()) == \
                    set(np.unique(fx[fk][rt]).tolist()), (k, t)
    if c.get("synapse", 1) >= 2:
        st = cf.stdp_arrays(s, cf.stdp_constants(p))
        for k in ("Apos", "Aneg", "STDPgap", "tauspost", "tauspre", "taupos", "tauneg", "Wex",
                  "mupos", "muneg"):
            for t in range(4):
                mt, rt = s["type"][used] == t, fx["i.type"] == t
                if rt.any():
                    assert set(np.unique(st[k][used][mt]).tolist()) == \
                        set(np.unique(fx["i." + k][rt]).tolist()), (k, t)


def test_stdp_params_match_the_harness_override(tmp_path):
    c = case("izh_dstdp")
    p = read_case(c, tmp_path)
    k = cf.stdp_constants(p)
    s = c["stdp"]
    assert [np.float32(k[n]) for n in ("Apos", "Aneg", "STDPgap", "tauspost", "tauspre",
                                       "taupos", "tauneg")] == [np.float32(v) for v in s[:7]]
    assert [np.float32(v) for v in k["Wex"]] == [np.float32(v) for v in (s[8], s[8], s[7], s[7])]
    # without the element: the reference's built-in constants
    p0 = read_case(c, tmp_path, stdp_params=False)
    assert p0.stdp is None and cf.stdp_constants(p0)["Apos"] == 0.5


def test_dynamic_layout_draws(tmp_path):
    """DynamicLayout (Layouts/DynamicLayout.cpp:97-162): the inhibitory reservoir sample and
    the starter rejection loop on the global generator, restated draw by draw here."""
    c = case("c0")
    text = configs.dynamic_layout_text(configs.config_text(c), 0.8, 0.1)
    p = cf.read(text, root=str(tmp_path))
    assert p.layout_class == "DynamicLayout"
    a = cf.setup(p)
    N = 100
    rng = cf.MTRand(1)
    n_inh = N - int(float(np.float32(0.8) * np.float32(N)) + 0.5)
    lay = list(range(n_inh))
    for i in range(n_inh, N):
        j = int(np.float32(rng.rand(1)[0] * np.float32(N)))
        if j < n_inh:
            lay[j] = i
    inh = np.zeros(N, bool)
    inh[lay] = True
    assert_same("ntype", a["ntype"], np.where(inh, 1, 2).astype(np.int32))
    want, st = 10, np.zeros(N, bool)
    while st.sum() < want:
        i = int(rng.in_range(np.float32(0), np.float32(N), 1)[0])
        if not inh[i] and not st[i]:
            st[i] = True
    assert_same("starter", a["starter"], st)
    assert a["starter"].sum() == 10 and not (a["starter"] & inh).any()


def test_izh_r_squared_draws(tmp_path):
    c = case("izh_grown")
    text = configs.config_text(c).replace(
        '<NeuronsParams class="AllIZHNeurons" name="NeuronsParams">',
        '<NeuronsParams class="AllIZHNeurons" name="NeuronsParams">'
        '<ParameterDraw>r_squared</ParameterDraw>')
    configs.write_case(c, str(tmp_path / "configfiles"))
    p = cf.read(text, root=str(tmp_path))
    assert p.izh_draw == "r_squared"
    a = cf.setup(p)
    # the draw keeps the flat ranges' four draws per neuron, so every other value the setup draws
    # is that of the flat-range file, for every neuron
    fx = load_fixture("izh_grown")
    for k in ("Iinject", "Inoise", "Vthresh", "Vrest", "Vreset", "Vinit"):
        assert_same(k, a[k], fx[k])
    inh = a["ntype"] == 1
    f32 = np.float32
    r_inh = (a["Aconst"][inh] - f32(0.02)) / f32(0.08)
    assert np.all((r_inh >= 0) & (r_inh <= 1.0001))
    assert np.all(a["Cconst"][inh] == f32(-65)) and np.all(a["Dconst"][inh] == f32(2))
    e = ~inh
    assert np.all(a["Aconst"][e] == f32(0.02)) and np.all(a["Bconst"][e] == f32(0.2))
    assert np.all((a["Cconst"][e] >= f32(-65)) & (a["Cconst"][e] <= f32(-50)))
    assert np.all((a["Dconst"][e] >= f32(2)) & (a["Dconst"][e] <= f32(8)))
    # c and d of one excitatory neuron come from the same r
    r2 = (a["Cconst"][e] + f32(65)) / f32(15)
    np.testing.assert_allclose((f32(8) - a["Dconst"][e]) / f32(6), r2, atol=1e-5)


def test_refused_files(tmp_path):
    c = case("c0")
    good = configs.config_text(c)
    configs.write_case(c, str(tmp_path / "configfiles"))
    cf.read(good, root=str(tmp_path))
    bad = [good.replace("AllLIFNeurons", "AllBogusNeurons"),
           good.replace("AllDSSynapses", "AllBogusSynapses"),
           good.replace("ConnGrowth", "ConnBogus"),
           good.replace("<maxFiringRate name=\"maxFiringRate\">200", "<maxFiringRate name=\"maxFiringRate\">-2"),
           good.replace("<min name=\"min\">1e-09</min><max name=\"max\">1.5e-09</max>",
                        "<min name=\"min\">2e-09</min><max name=\"max\">1.5e-09</max>"),
           good.replace("<Tsim name=\"Tsim\">1.0</Tsim>", "")]
    for b in bad:
        assert b != good
        with pytest.raises(cf.ConfigError):
            cf.read(b, root=str(tmp_path))
    # STDP constants for a synapse class without STDP
    with pytest.raises(cf.ConfigError):
        cf.read(good.replace('name="SynapsesParams"></SynapsesParams>',
                             'name="SynapsesParams"><STDPParams><Apos>1</Apos></STDPParams>'
                             '</SynapsesParams>'), root=str(tmp_path))


def test_extensions_in_bg3params(tmp_path):
    """<STDPParams> / <ParameterDraw> in a root-level <BG3Params> (which the reference's readers
    do not visit) read as they do inside the model's sections; config.write puts them there."""
    c = case("izh_static")
    configs.write_case(c, str(tmp_path / "configfiles"))
    inside = cf.read(configs.config_text(c, stdp_params=True), root=str(tmp_path))
    root_text = configs.config_text(c, stdp_params="root")
    outside = cf.read(root_text, root=str(tmp_path))
    assert outside.stdp is not None and outside.stdp == inside.stdp
    assert "<BG3Params>" in root_text and "<STDPParams>" not in root_text.split("</ModelParams>")[0]
    text, files = cf.write(outside)
    assert "<BG3Params><STDPParams>" in text and "<STDPParams>" not in text.split("</ModelParams>")[0]
    for rel, body in files.items():
        os.makedirs(os.path.dirname(str(tmp_path / rel)), exist_ok=True)
        with open(str(tmp_path / rel), "w") as f:
            f.write(body)
    assert cf.read(text, root=str(tmp_path)).stdp == outside.stdp
    bad = [
        # the same element twice
        configs.config_text(c, stdp_params=True).replace(
            "</BGSimParams>", "<BG3Params><STDPParams><Apos>1</Apos></STDPParams></BG3Params>"
            "</BGSimParams>"),
        # an element this reader does not know
        root_text.replace("<BG3Params>", "<BG3Params><Bogus>1</Bogus>"),
        # STDP constants for a synapse class without STDP
        root_text.replace("AllDynamicSTDPSynapses", "AllDSSynapses"),
    ]
    for b in bad:
        assert b != root_text
        with pytest.raises(cf.ConfigError):
            cf.read(b, root=str(tmp_path))
    # the r^2 draw in BG3Params, for Izhikevich neurons and (refused) for LIF ones
    izh = cf.read(root_text.replace("<BG3Params>",
                                    "<BG3Params><ParameterDraw>r_squared</ParameterDraw>"),
                  root=str(tmp_path))
    assert izh.izh_draw == "r_squared"
    lif = case("c0")
    configs.write_case(lif, str(tmp_path / "configfiles"))
    for b in (configs.config_text(lif).replace(
            "</BGSimParams>", "<BG3Params><ParameterDraw>r_squared</ParameterDraw></BG3Params>"
            "</BGSimParams>"),):
        with pytest.raises(cf.ConfigError):
            cf.read(b, root=str(tmp_path))


def test_norm_stream_matches_the_oracle():
    """bg3_norm_fill gives the oracle's stream however it is split into calls: single values,
    odd and even counts, and fills large enough to run the polar method on several threads
    (starting with and without a pending second value of a pair)."""
    from braingrid_gb300 import lib as bg
    from oracle import pyoracle as po
    want = po.norm_stream(5, 2600003)
    g = bg.NormStream(5)
    got = np.concatenate([g.take(1), g.take(0), g.take(30000), g.take(970000), g.take(300001),
                          g.take(1000000), g.take(300001)])
    assert_same("norm", got, want)
    g.close()


def reference_output(name):
    return np.load("tests/golden/outputs.npz")[name].tobytes().decode()


def oracle_output(name):
    """The oracle runs the case as the reference's driver does; results.state_xml writes it."""
    from braingrid_gb300 import results
    from tests.netcases import steps_per_epoch
    c, _, _ = configs.output_case(name)
    o = oracle_from_case(c)
    spe = steps_per_epoch(c)
    for e in range(c["epochs"]):
        o.step_n(spe)
        o.growth()
        o.record_epoch(e + 1)
    starter = np.zeros(c["N"], bool)
    starter[c["starters"]] = True
    text = results.state_xml(True, c["N"], c["epochs"], np.float32(c["tsim"]), cf.DELTA_T, o.step,
                             (o.arr("burstinessHist"), o.arr("spikesHistory"),
                              o.arr("ratesHistory"), o.arr("radiiHistory")),
                             o.arr("xloc"), o.arr("yloc"), o.arr("ntype"), starter,
                             o.arr("Vthresh"))
    o.close()
    return text


@pytest.mark.parametrize("name", [n for n in configs.OUTPUT_CASES if n != "ref_small"])
def test_result_file_matches_reference_driver(name):
    """The reference driver's result file (XmlGrowthRecorder::saveSimData), byte for byte, from
    the same run (the oracle, pinned to the reference step by step)."""
    assert oracle_output(name) == reference_output(name)


@pytest.mark.slow
def test_result_file_matches_reference_driver_small():
    assert oracle_output("ref_small") == reference_output("ref_small")


def test_result_file_format():
    from braingrid_gb300 import results
    assert results.vector_xml("v", np.array([0.5, 1e-5, -0.0, 3], np.float32)) == \
        '<Matrix name="v" type="complete" rows="1" columns="4" multiplier="1.0">\n' \
        '   0.5 1e-05 -0 3 \n</Matrix>'
    assert results.complete_xml("m", np.array([[1, 2], [0.25, 0.1]], np.float32)) == \
        '<Matrix name="m" type="complete" rows="2" columns="2" multiplier="1.0">\n' \
        '   1 2 \n0.25 0.1 \n\n</Matrix>'


@pytest.mark.parametrize("name", ["c0_poisson", "c0_poisson25", "izh_dstdp", "izh_static"])
def test_poisson_intervals_match_the_oracle(name, tmp_path):
    """The Poisson stimulus's intervals drawn ahead on the global generator after setup
    (config.poisson_intervals) equal the oracle's, which replays HostSInputPoisson step by step
    and is pinned to the reference harness's input state."""
    from tests.netcases import steps_per_epoch
    c = case(name)
    p = read_case(c, tmp_path)
    a = cf.setup(p)
    n = steps_per_epoch(c) * c["epochs"] + 2
    begin, steps = cf.poisson_intervals(a, n)
    o = oracle_from_case(c)
    ob, ov = o.poisson_isi_draws(n)
    assert_same("begin", begin, ob)
    assert_same("intervals", steps, ov)
    o.close()


def test_tinyxml_style_declarations_are_read(tmp_path):
    """The reference's stimulus files declare standalone=no without quotes (TinyXML takes it);
    they read here too."""
    c = case("c0_regular")
    text = configs.stim_xml(c["stim"]).replace('<?xml version="1.0" standalone="no"?>',
                                               '<?xml version="1.0" standalone=no?>')
    configs.write_case(c, str(tmp_path / "configfiles"))
    p = cf.read(configs.config_text(c), text, root=str(tmp_path))
    assert p.stim["kind"] == "regular" and p.stim["sync"] == "no"
    with pytest.raises(cf.ConfigError):
        cf.read(configs.config_text(c).replace("</BGSimParams>", ""), root=str(tmp_path))


def test_run_driver_imports_and_parses_arguments_without_a_gpu():
    from braingrid_gb300 import sim
    with pytest.raises(SystemExit) as e:
        sim.main(["-h"])
    assert e.value.code == 0
    with pytest.raises(SystemExit):
        sim.main(["-t", "x.xml", "--noise", "bogus"])


def test_missing_or_bad_neuron_lists_are_refused(tmp_path):
    c = case("c0")
    text = configs.config_text(c)
    with pytest.raises(cf.ConfigError):            # the list files were never written
        cf.read(text, root=str(tmp_path))
    configs.write_case(c, str(tmp_path / "configfiles"))
    inh = tmp_path / "configfiles" / "bg3" / "c0-inh.xml"
    inh.write_text('<?xml version="1.0"?>\n<I>3 100</I>\n')     # 100 is past the 10x10 grid
    with pytest.raises(cf.ConfigError):
        cf.read(text, root=str(tmp_path))
    inh.write_text('<?xml version="1.0"?>\n<A>3</A>\n')         # wrong root element
    with pytest.raises(cf.ConfigError):
        cf.read(text, root=str(tmp_path))
    inh.write_text('<?xml version="1.0"?>\n<I>3 17</I>\n')
    p = cf.read(text, root=str(tmp_path))
    a = cf.setup(p)
    assert list(np.nonzero(a["ntype"] == cf.INH)[0]) == [3, 17]


def test_poisson_mask_list_file(tmp_path):
    c = case("c0_poisson")
    configs.write_case(c, str(tmp_path / "configfiles"))
    (tmp_path / "masks.xml").write_text('<?xml version="1.0"?>\n<M>0 5 9</M>\n')
    stim = ('<?xml version="1.0" standalone=no?>\n<InputParams><IMethod name="SInputPoisson"/>'
            '<IntParams fr_mean="10" weight="0.5"/><Masks><LayoutFiles '
            'maskNListFileName="masks.xml"/></Masks></InputParams>')
    p = cf.read(configs.config_text(c), stim, root=str(tmp_path))
    assert list(np.nonzero(p.stim["masks"])[0]) == [0, 5, 9]


def test_oracle_end_of_run_stream_matches_reference_driver():
    """The driver's -w stream of the c0 run (tests/golden/outputs.npz) from the oracle's run,
    Isyn tokens aside."""
    from tests.netcases import steps_per_epoch
    from tests.test_oracle_serialize import comparable
    c, _, _ = configs.output_case("c0")
    o = oracle_from_case(c)
    for e in range(c["epochs"]):
        o.step_n(steps_per_epoch(c))
        o.growth()
        o.record_epoch(e + 1)
    want = np.load("tests/golden/outputs.npz")["c0.ser"].tobytes()
    assert comparable(o.serialize(conn_growth=True), c) == comparable(want, c)
    o.close()


def test_dense_static_wiring(tmp_path):
    """ConnStatic with more connections per neuron than neighbours in reach (static_izh_1000's
    shape: nConnsPerNeuron 999, radius 50 on a 40 x 25 grid): every source reaches every other
    neuron, so no tie choice is left and the wiring is complete; one weight draw per synapse, from
    the range of the source's type, in creation order (source, then nearness)."""
    c = dict(case("izh_static"), name="dense", width=40, height=25, N=1000, max_syn=1000,
             synapse=0, stdp=None, stim=None, inh=list(range(0, 1000, 5)), starters=[],
             static=dict(n=999, radius=50.0, rewire=0.0, exc=(0.0, 0.5e-7), inh=(-0.5e-7, 0.0)))
    configs.write_case(c, str(tmp_path / "configfiles"))
    p = cf.read(configs.config_text(c), root=str(tmp_path))
    assert p.synapse_class == "AllSpikingSynapses" and p.static["n"] == 999
    a = cf.setup(p)
    s = a["synapses"]
    assert a["counts"].tolist() == [999] * 1000
    used = s["in_use"].astype(bool)
    assert used.sum() == 999000
    src = s["src"][used]
    assert np.bincount(src, minlength=1000).tolist() == [999] * 1000
    inh = a["ntype"] == cf.INH
    w = s["W"][used]
    assert np.all(w[inh[src]] <= 0) and np.all(w[~inh[src]] >= 0)
    # the draws: the generator after the neuron draws, one per synapse in creation order
    b = cf.setup(p)
    slots = b["creation_slots"]
    rng = cf.MTRand(1)
    rng.rand(int(6 * 1000 + 4 * 1000))             # IF draws, then a, b, c, d (no starters)
    lo = np.where(inh[b["synapses"]["src"][slots]], np.float32(-0.5e-7), np.float32(0.0))
    hi = np.where(inh[b["synapses"]["src"][slots]], np.float32(0.0), np.float32(0.5e-7))
    assert_same("W in creation order", b["synapses"]["W"][slots], rng.in_range(lo, hi))


@pytest.mark.parametrize("name", ["c0", "izh_static", "izh_dstdp", "c0_spiking"])
def test_write_reads_back_to_the_same_parameters(name, tmp_path):
    c = case(name)
    p = read_case(c, tmp_path)
    text, files = cf.write(p, name=name)
    for rel, t in files.items():
        f = tmp_path / "out" / rel
        f.parent.mkdir(parents=True, exist_ok=True)
        f.write_text(t)
    q = cf.read(text, root=str(tmp_path / "out"))
    for k in ("width", "height", "tsim", "epochs", "max_firing_rate", "max_syn", "seed",
              "neuron_class", "synapse_class", "conn_class", "layout_class", "izh_draw",
              "inh_list", "active_list", "stdp"):
        assert getattr(q, k) == getattr(p, k), k
    for k in p.if_ranges:
        assert q.if_ranges[k] == p.if_ranges[k], k
    assert q.izh_ranges == p.izh_ranges and q.growth == p.growth
    assert {k: (v if not isinstance(v, tuple) else tuple(v)) for k, v in q.static.items()} == \
        {k: (v if not isinstance(v, tuple) else tuple(v)) for k, v in p.static.items()}
    a, b = cf.setup(p), cf.setup(q)
    for k in ("Vthresh", "Inoise", "C1", "I0", "ntype"):
        assert_same(k, b[k], a[k])


def test_written_file_runs_in_the_reference_driver(tmp_path):
    """A parameter file written by config.write (no extension elements) is read by the compiled
    reference's own driver, which then writes the same result file as from the original."""
    import os
    import subprocess
    growth = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle",
                          "_ref", "growth")
    if not os.path.exists(growth):
        pytest.skip("the compiled reference is built only where its sources are")
    c, text, _ = configs.output_case("c0")
    configs.write_case(c, str(tmp_path / "configfiles"))
    p = cf.read(text, root=str(tmp_path))
    out_text, files = cf.write(p, name="w")
    for rel, t in files.items():
        f = tmp_path / rel
        f.parent.mkdir(parents=True, exist_ok=True)
        f.write_text(t)
    (tmp_path / "results").mkdir(exist_ok=True)
    (tmp_path / "w.xml").write_text(out_text.replace(p.output, "results/w-out.xml"))
    subprocess.check_call([growth, "-t", "w.xml"], cwd=str(tmp_path), stdout=subprocess.DEVNULL,
                          stderr=subprocess.DEVNULL, timeout=300)
    got = (tmp_path / "results" / "w-out.xml").read_bytes()
    assert got == np.load("tests/golden/outputs.npz")["c0"].tobytes()
