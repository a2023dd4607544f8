"""Network configurations shared by the fixture generator and the tests.

Each case is described twice, consistently: as a BrainGrid XML config (written by
write_config_tree for the reference harness) and as plain parameters (read by the tests to set up
the oracle and the CUDA path without the reference tree).

The 10x10-style networks follow the stated model: LIF neurons, AllDSSynapses, ConnGrowth,
FixedLayout with 10 % inhibitory and 10 endogenously active (starter) sites chosen by a seeded
shuffle; Iinject 13.5 nA, Inoise U[1.0, 1.5] nA, Vthresh 15 mV (starters U[13.565, 13.655] mV),
Vreset 13.5 mV (starters 13.0 mV), Vrest 0, Vinit 13.0 mV, dt 0.1 ms.
"""
import os

import numpy as np

LIF_RANGES = [13.5e-9, 13.5e-9, 1.0e-9, 1.5e-9, 15.0e-3, 15.0e-3, 0.0, 0.0,
              13.5e-3, 13.5e-3, 13.0e-3, 13.0e-3, 13.565e-3, 13.655e-3, 13.0e-3, 13.0e-3]


def site_lists(width, height, frac_inh=0.10, n_starters=10, seed=1):
    """Seeded choice of inhibitory and starter sites (starters are excitatory)."""
    N = width * height
    rs = np.random.RandomState(seed)
    perm = rs.permutation(N)
    n_inh = int(round(frac_inh * N))
    inh = np.sort(perm[:n_inh])
    starters = np.sort(perm[n_inh:n_inh + n_starters])
    return [int(x) for x in inh], [int(x) for x in starters]


# static_izh_1000-style Izhikevich parameters: IF ranges, then a, b, c, d (minExc, maxExc,
# minInh, maxInh)
IZH_IF_RANGES = [13.5e-9, 13.5e-9, 0.5e-6, 0.7329e-6, 30.0e-3, 30.0e-3, 0.0, 0.0,
                 -0.065, -0.065, -0.065, -0.065, 13.565e-3, 13.655e-3, 13.0e-3, 13.0e-3]
IZH_RANGES = [0.02, 0.02, 0.02, 0.1, 0.2, 0.2, 0.2, 0.25, -65.0, -50.0, -65.0, -65.0,
              2.0, 8.0, 2.0, 2.0]
SYN_CLASS = {0: "AllSpikingSynapses", 1: "AllDSSynapses", 2: "AllSTDPSynapses",
             3: "AllDynamicSTDPSynapses"}

# Additive STDP after Song, Miller and Abbott (2000): increments of 0.005 / -0.00525 of the 30 nA
# weight bound, tau+ = tau- = 20 ms; Wex +30 nA for excitatory sources, -40 nA for inhibitory
# ones.  Order: Apos, Aneg, STDPgap, tauspost, tauspre, taupos, tauneg, WexE, WexI, mupos, muneg.
STDP_SOFT = [0.005 * 30e-9, -0.00525 * 30e-9, 2e-3, 75e-3, 34e-3, 20e-3, 20e-3, 30e-9, -40e-9,
             0.0, 0.0]

REG_VALUES = [1.5e-8 if ((i // 10) + (i % 10)) % 3 == 0 else 0.0 for i in range(100)]


def _case(name, width, height, tsim, epochs, max_syn, seed=1, target_rate=1.0, radii=None,
          max_firing_rate=200, frac_inh=0.10, n_starters=10, site_seed=1, keep_steps_every=None,
          fp64=False, config=None, inh=None, starters=None, syn_keep=None, stim=None,
          neuron="lif", synapse=1, stdp=None, static=None):
    if inh is None:
        inh, starters = site_lists(width, height, frac_inh, n_starters, site_seed)
    c = dict(name=name, width=width, height=height, N=width * height, tsim=tsim, epochs=epochs,
             max_syn=max_syn, seed=seed, max_firing_rate=max_firing_rate, inh=inh,
             starters=starters, growth=dict(epsilon=0.60, beta=0.10, rho=1e-4,
                                            target_rate=target_rate, min_radius=0.1,
                                            start_radius=0.4),
             radii=radii, keep_steps_every=keep_steps_every, fp64=fp64, syn_keep=syn_keep,
             stim=stim, neuron=neuron, synapse=synapse, stdp=stdp, static=static)
    c["config"] = config or "configfiles/bg3/%s.xml" % name
    args = []
    if stim is not None:
        args += ["-s", "configfiles/bg3/%s-stim.xml" % name]
    if radii is not None:
        args += ["--radii", repr(radii)]
    if keep_steps_every:
        args += ["--dump-every", str(keep_steps_every)]
    if stdp is not None:
        args += ["--stdp", ",".join(repr(float(v)) for v in stdp)]
    c["args"] = args
    return c


CASES = [
    # the reference's own tiny test (2x2, 1 epoch of 1 s), with its own NLists
    _case("ref_tiny", 2, 2, 1.0, 1, 200, target_rate=1.9, config="configfiles/test-tiny.xml",
          inh=[1], starters=[0], keep_steps_every=500),
    # the 100-neuron benchmark network: 10x10, 10 epochs x 1 s, max 100 synapses per neuron, seed 1
    _case("c0", 10, 10, 1.0, 10, 100, keep_steps_every=5000),
    # the same network with a pre-grown radius so that growth wires it after epoch 1
    # (the reference recorder needs epoch duration x epochs >= 1 s)
    _case("c0_grown", 10, 10, 0.2, 5, 100, radii=1.2, max_firing_rate=1000,
          keep_steps_every=100),
    # 30x30 pre-grown network, larger fan-in and fan-out
    _case("m30_grown", 30, 30, 0.1, 10, 200, radii=2.0, max_firing_rate=1000, site_seed=3,
          keep_steps_every=1000, syn_keep=(9,)),
    # FP64 reference on the 10x10 network (long-run comparison base)
    _case("c0_fp64", 10, 10, 1.0, 10, 100, fp64=True),
    # FP64 reference on the 100x100 benchmark network's model (10,000 neurons, 100 starters,
    # max 1000 synapses per neuron, seed 7), 2 x 1 s
    _case("c1_fp64", 100, 100, 1.0, 2, 1000, seed=7, n_starters=100, site_seed=7, fp64=True),
    # FP64 reference on the Izhikevich + dynamic STDP + Poisson network (izh_dstdp)
    _case("izh_dstdp_fp64", 12, 12, 0.5, 2, 100, radii=1.3, max_firing_rate=1000, site_seed=4,
          neuron="izh", synapse=3, stdp=STDP_SOFT, fp64=True,
          stim=dict(kind="poisson", fr_mean=10.0, weight=0.5, masks=None)),
    # Regular pulse input, random per-neuron phase (sync="no": shifts drawn before the neurons)
    _case("c0_regular", 10, 10, 0.5, 2, 100, keep_steps_every=250,
          stim=dict(kind="regular", duration=0.005, interval=0.045, sync="no", values=REG_VALUES)),
    # Poisson input on the pre-grown network (10 Hz, weight 0.5 -> 5 nA), masked subset
    _case("c0_poisson", 10, 10, 0.2, 5, 100, radii=1.2, max_firing_rate=1000, keep_steps_every=100,
          stim=dict(kind="poisson", fr_mean=10.0, weight=0.5, masks=list(range(0, 100, 3)))),
    # Poisson input at the reference files' strength (10 Hz, weight 25), all neurons
    _case("c0_poisson25", 10, 10, 0.2, 5, 100, max_firing_rate=1000, keep_steps_every=100,
          stim=dict(kind="poisson", fr_mean=10.0, weight=25.0, masks=None)),
    # Izhikevich neurons, DS synapses, pre-grown 12x12 network
    _case("izh_grown", 12, 12, 0.2, 5, 100, radii=1.3, max_firing_rate=1000, site_seed=4,
          keep_steps_every=100, neuron="izh"),
    # STDP with the reference's built-in constants (Apos 0.5 A: one potentiation saturates the
    # network), two epochs so that the spike rings never fill
    _case("c0_stdp", 10, 10, 0.5, 2, 100, radii=1.2, max_firing_rate=1000, keep_steps_every=50,
          synapse=2),
    _case("c0_dstdp", 10, 10, 0.5, 2, 100, radii=1.2, max_firing_rate=1000, keep_steps_every=50,
          synapse=3),
    # Izhikevich neurons, dynamic STDP synapses with bounded additive constants and Poisson
    # drive (10 Hz, 5 nA), as in the 512-network Izhikevich + STDP sweep
    _case("izh_dstdp", 12, 12, 0.5, 2, 100, radii=1.3, max_firing_rate=1000, site_seed=4,
          keep_steps_every=50, neuron="izh", synapse=3, stdp=STDP_SOFT,
          stim=dict(kind="poisson", fr_mean=10.0, weight=0.5, masks=None)),
    # ConnStatic: 10 nearest neighbours within radius 5, weights U[10, 20] nA / U[-40, -20] nA
    # (pRewiring 0.1 is read but never applied by the reference); Izhikevich neurons, dynamic
    # STDP and Poisson drive as in the 512-network sweep
    # (max 32 synapses per neuron: the thin sweep path)
    _case("izh_static", 12, 12, 0.5, 2, 32, max_firing_rate=1000, site_seed=5,
          keep_steps_every=50, neuron="izh", synapse=3, stdp=STDP_SOFT,
          stim=dict(kind="poisson", fr_mean=10.0, weight=0.5, masks=None),
          static=dict(n=10, radius=5.0, rewire=0.1, exc=(10e-9, 20e-9), inh=(-40e-9, -20e-9))),
    # LIF neurons with plain spiking synapses (AllSpikingSynapses), pre-grown
    _case("c0_spiking", 10, 10, 0.2, 5, 100, radii=1.2, max_firing_rate=1000, keep_steps_every=100,
          synapse=0),
    # ragged shapes: 63 neurons (a full 32-dest tile and one of 31), 30 slots per row (the last
    # row quad half used), pre-grown DS network
    _case("ragged", 7, 9, 0.25, 4, 30, radii=1.2, max_firing_rate=1000, site_seed=6,
          keep_steps_every=100),
    # 65 neurons (the last tile holds one), 18 slots per row, Izhikevich + dynamic STDP + Poisson
    _case("ragged_izh", 5, 13, 0.5, 2, 18, radii=1.1, max_firing_rate=1000, site_seed=7,
          keep_steps_every=50, neuron="izh", synapse=3, stdp=STDP_SOFT,
          stim=dict(kind="poisson", fr_mean=10.0, weight=0.5, masks=None)),
]


def stim_xml(stim):
    if stim["kind"] == "regular":
        vals = " ".join(repr(v) for v in stim["values"])
        return ('<?xml version="1.0" standalone="no"?>\n<InputParams>\n'
                '  <IMethod name="SInputRegular"/>\n'
                '  <IntParams duration="%r" interval="%r" sync="%s"/>\n'
                '  <Values><I>%s</I></Values>\n</InputParams>\n'
                % (stim["duration"], stim["interval"], stim["sync"], vals))
    masks = ""
    if stim.get("masks") is not None:
        masks = "  <Masks><M>%s</M></Masks>\n" % " ".join(str(i) for i in stim["masks"])
    return ('<?xml version="1.0" standalone="no"?>\n<InputParams>\n'
            '  <IMethod name="SInputPoisson"/>\n'
            '  <IntParams fr_mean="%r" weight="%r"/>\n%s</InputParams>\n'
            % (stim["fr_mean"], stim["weight"], masks))


def case(name):
    for c in CASES:
        if c["name"] == name:
            return c
    raise KeyError(name)


_XML = """<?xml version="1.0" encoding="UTF-8" standalone="no"?>
<BGSimParams>
  <SimInfoParams name="SimInfoParams">
    <PoolSize name="PoolSize"><x name="x">{width}</x><y name="y">{height}</y><z name="z">1</z></PoolSize>
    <SimParams name="SimParams"><Tsim name="Tsim">{tsim}</Tsim><numSims name="numSims">{epochs}</numSims></SimParams>
    <SimConfig name="SimConfig">
      <maxFiringRate name="maxFiringRate">{max_firing_rate}</maxFiringRate>
      <maxSynapsesPerNeuron name="maxSynapsesPerNeuron">{max_syn}</maxSynapsesPerNeuron>
    </SimConfig>
    <Seed name="Seed"><value name="value">{seed}</value></Seed>
    <OutputParams name="OutputParams"><stateOutputFileName name="stateOutputFileName">results/{name}-out.xml</stateOutputFileName></OutputParams>
  </SimInfoParams>
  <ModelParams>
    <NeuronsParams class="{neuron_class}" name="NeuronsParams">
{neuron_params}
    </NeuronsParams>
    <SynapsesParams class="{synapse_class}" name="SynapsesParams"></SynapsesParams>
{connections}
    <LayoutParams class="FixedLayout" name="LayoutParams">
      <LayoutFiles name="LayoutFiles">
        <activeNListFileName name="activeNListFileName" type="InputFile">configfiles/bg3/{name}-active.xml</activeNListFileName>
        <inhNListFileName name="inhNListFileName" type="InputFile">configfiles/bg3/{name}-inh.xml</inhNListFileName>
        <probedNListFileName name="prbNListFileName" type="InputFile"/>
      </LayoutFiles>
    </LayoutParams>
  </ModelParams>
</BGSimParams>
"""


GROWTH_XML = """    <ConnectionsParams class="ConnGrowth" name="ConnectionsParams">
      <GrowthParams name="GrowthParams">
        <epsilon name="epsilon">{epsilon}</epsilon><beta name="beta">{beta}</beta><rho name="rho">{rho}</rho>
        <targetRate name="targetRate">{target_rate}</targetRate><minRadius name="minRadius">{min_radius}</minRadius>
        <startRadius name="startRadius">{start_radius}</startRadius>
      </GrowthParams>
    </ConnectionsParams>"""

STATIC_XML = """    <ConnectionsParams class="ConnStatic" name="ConnectionsParams">
      <StaticConnectionsParams name="StaticConnectionsParams">
        <nConnsPerNeuron name="nConnsPerNeuron">{n}</nConnsPerNeuron>
        <threshConnsRadius name="threshConnsRadius">{radius!r}</threshConnsRadius>
        <pRewiring name="pRewiring">{rewire!r}</pRewiring>
      </StaticConnectionsParams>
      <StaticConnectionsWeight name="StaticConnectionsWeight">
        <minExc name="minExc">{exc[0]!r}</minExc><maxExc name="maxExc">{exc[1]!r}</maxExc>
        <minInh name="minInh">{inh[0]!r}</minInh><maxInh name="maxInh">{inh[1]!r}</maxInh>
      </StaticConnectionsWeight>
    </ConnectionsParams>"""


def _range_xml(ranges):
    names = ["Iinject", "Inoise", "Vthresh", "Vresting", "Vreset", "Vinit", "starter_vthresh",
             "starter_vreset"]
    return "\n".join('      <%s name="%s"><min name="min">%r</min><max name="max">%r</max></%s>'
                     % (nm, nm, ranges[2 * k], ranges[2 * k + 1], nm)
                     for k, nm in enumerate(names))


def _izh_xml(z):
    return "\n".join('      <%s name="%s"><minExc name="minExc">%r</minExc><maxExc name="maxExc">%r'
                     '</maxExc><minInh name="minInh">%r</minInh><maxInh name="maxInh">%r</maxInh>'
                     '</%s>' % (nm, nm, z[4 * k], z[4 * k + 1], z[4 * k + 2], z[4 * k + 3], nm)
                     for k, nm in enumerate(["Aconst", "Bconst", "Cconst", "Dconst"]))


def neuron_ranges(c):
    return IZH_IF_RANGES if c.get("neuron") == "izh" else LIF_RANGES


STDP_NAMES = ("Apos", "Aneg", "STDPgap", "tauspost", "tauspre", "taupos", "tauneg", "WexExc",
              "WexInh", "mupos", "muneg")


def config_text(c, stdp_params=False):
    """The case's BrainGrid parameter file.  stdp_params=True adds the case's STDP constants as
    an <STDPParams> element inside <SynapsesParams>, stdp_params="root" inside a root-level
    <BG3Params> (both read by braingrid_gb300.config, the second also by the drop-in driver; the
    reference harness takes them with --stdp instead)."""
    p = dict(c)
    p.update(c["growth"])
    p["synapse_class"] = SYN_CLASS[c.get("synapse", 1)]
    if c.get("static"):
        p["connections"] = STATIC_XML.format(**c["static"])
    else:
        p["connections"] = GROWTH_XML.format(**c["growth"])
    if c.get("neuron") == "izh":
        p["neuron_class"] = "AllIZHNeurons"
        p["neuron_params"] = _range_xml(IZH_IF_RANGES) + "\n" + _izh_xml(IZH_RANGES)
    else:
        p["neuron_class"] = "AllLIFNeurons"
        p["neuron_params"] = _range_xml(LIF_RANGES)
    text = _XML.format(**p)
    if stdp_params and c.get("stdp") is not None:
        st = "".join("<%s>%r</%s>" % (k, float(v), k) for k, v in zip(STDP_NAMES, c["stdp"]))
        if stdp_params == "root":
            text = text.replace("</BGSimParams>",
                                "<BG3Params><STDPParams>%s</STDPParams></BG3Params>\n"
                                "</BGSimParams>" % st)
        else:
            text = text.replace('name="SynapsesParams"></SynapsesParams>',
                                'name="SynapsesParams"><STDPParams>%s</STDPParams>'
                                '</SynapsesParams>' % st)
    return text


def list_texts(c):
    """The case's active (starter) and inhibitory neuron-list files."""
    return ('<?xml version="1.0" encoding="UTF-8"?>\n<A>%s</A>\n'
            % " ".join(str(i) for i in c["starters"]),
            '<?xml version="1.0" encoding="UTF-8"?>\n<I>%s</I>\n'
            % " ".join(str(i) for i in c["inh"]))


def write_case(c, cfgdir, stdp_params=False):
    """Write configfiles/bg3/<case>.xml, its neuron lists and its stimulus file under cfgdir
    (the configfiles directory)."""
    d = os.path.join(cfgdir, "bg3")
    os.makedirs(d, exist_ok=True)
    name = c["name"]
    with open(os.path.join(d, name + ".xml"), "w") as f:
        f.write(config_text(c, stdp_params))
    active, inh = list_texts(c)
    with open(os.path.join(d, name + "-active.xml"), "w") as f:
        f.write(active)
    with open(os.path.join(d, name + "-inh.xml"), "w") as f:
        f.write(inh)
    if c.get("stim") is not None:
        with open(os.path.join(d, name + "-stim.xml"), "w") as f:
            f.write(stim_xml(c["stim"]))


# The reference's own test-small (configfiles/test-small.xml with its 10x10 NLists)
TEST_SMALL = dict(name="ref_small", width=10, height=10, N=100, tsim=100.0, epochs=2, max_syn=200,
                  seed=1, max_firing_rate=200, inh=[33, 66],
                  starters=[7, 11, 14, 37, 41, 44, 67, 71, 74, 97],
                  growth=dict(epsilon=0.60, beta=0.10, rho=1e-4, target_rate=1.9, min_radius=0.1,
                              start_radius=0.4), radii=None)

# Whole runs whose result file (Recorders/XmlGrowthRecorder.cpp:104-153) the compiled reference's
# own driver wrote from the same parameter files: tests/golden/outputs.npz.  Every one keeps its
# start radii below the grid spacing, so no synapse forms and a GPU run stays bit-exact.
# No DynamicLayout run: the reference refuses every DynamicLayout file, its
# DynamicLayout::readParameters returning false after reading frac_EXC
# (Layouts/DynamicLayout.cpp:60-78).  No Poisson run: the driver indexes its one-slot input
# synapse object by maxSynapsesPerNeuron * neuron (Inputs/HostSInputPoisson.cpp:77) and faults.
OUTPUT_CASES = ("ref_tiny", "ref_small", "c0", "c0_regular", "c100")

# 100x100 LIF + DS + ConnGrowth, one epoch of 1 s at the stated start radius (10 % inhibitory, 1 %
# starters on fixed strides): the injected-noise neuron pass of networks above 2,048 neurons
C100 = dict(name="c100", width=100, height=100, N=10000, tsim=1.0, epochs=1, max_syn=100, seed=1,
            max_firing_rate=200, inh=list(range(3, 10000, 10)), starters=list(range(7, 10000, 100)),
            growth=dict(epsilon=0.60, beta=0.10, rho=1e-4, target_rate=1.0, min_radius=0.1,
                        start_radius=0.4), radii=None)


def dynamic_layout_text(text, frac_exc, frac_starter):
    """A parameter file with its FixedLayout replaced by DynamicLayout."""
    return text.replace(
        '<LayoutParams class="FixedLayout" name="LayoutParams">',
        '<LayoutParams class="DynamicLayout" name="LayoutParams">'
        '<frac_EXC name="frac_EXC">%r</frac_EXC><starter_neurons name="starter_neurons">%r'
        '</starter_neurons>' % (frac_exc, frac_starter))


def output_case(name):
    """(case, parameter-file text, stimulus text or None) of an OUTPUT_CASES entry."""
    c = {"ref_small": TEST_SMALL, "c100": C100}.get(name) or case(name)
    return c, config_text(c), (stim_xml(c["stim"]) if c.get("stim") else None)


def write_config_tree(cfgdir):
    """Write configfiles/bg3/<case>.xml and its NLists for every generated case."""
    for c in CASES:
        if c["config"].startswith("configfiles/bg3/"):
            write_case(c, cfgdir)
