"""BrainGrid parameter files: the reference's XML configuration read into a network on the GPU.

Reading follows the reference's parameter visitors, each class taking the elements it knows by
tag name under its own section: SimulationInfo::readParameters (Core/SimulationInfo.cpp:55-175)
for the pool size, epoch length and count, firing-rate bound, synapse slots per neuron and seed;
AllIFNeurons / AllIZHNeurons::readParameters (Neurons/) for the neuron parameter ranges;
ConnGrowth / ConnStatic::readParameters (Connections/); FixedLayout / DynamicLayout::
readParameters (Layouts/) with the neuron-list files they name; FSInput, SInputRegular and
SInputPoisson (Inputs/) for a stimulus file.

Setup follows Model::setupSim (Core/Model.cpp:136-158) and the driver before it.  Every random
value comes from the reference's global generator, MTRand seeded with 1 (Utils/Global.cpp:79),
drawn in the reference's order: a regular input's per-neuron phases (the stimulus is created
before the model is set up, Core/BGDriver.cpp:72-74), DynamicLayout's type and starter maps
(Layouts/DynamicLayout.cpp:97-162), each neuron's parameters (Neurons/AllIFNeurons.cpp:398-443,
AllIZHNeurons.cpp:413-432), then ConnStatic's weights (Connections/ConnStatic.cpp:33-80).  The
arrays are the reference's, bit for bit.  The noise generator is keyed by the file's seed
(Core/SingleThreadedSpikingModel.cpp:30): the device generator, or the reference's own Norm
stream pushed into BG3_NOISE_INJECT (lib.NormStream).

Two element groups that the reference's files cannot express are read as well, so that the
Izhikevich + STDP benchmark networks need no other override.  They sit in <BG3Params>, a child of
the root element that the reference's readers never visit (so its driver reads such a file, and
the drop-in driver of braingrid_gb300/dropin applies the STDP constants), or, as this reader
also accepts, inside <SynapsesParams> / <NeuronsParams> (where the reference's reader rejects
them):

  <STDPParams> (synapse classes AllSTDPSynapses, AllDynamicSTDPSynapses) holding any of
      Apos, Aneg, STDPgap, tauspost, tauspre, taupos, tauneg, WexExc, WexInh, mupos, muneg,
      useFroemkeDanSTDP: the constants of every synapse made (by ConnStatic or by growth), in
      place of AllSTDPSynapses::createSynapse's built-in ones (Synapses/AllSTDPSynapses.cpp:
      252-273); Wex is WexInh for synapses from inhibitory neurons, WexExc otherwise;
  <ParameterDraw>r_squared</ParameterDraw> (AllIZHNeurons): Izhikevich's (2003) spread instead
      of four flat ranges.  The neuron's four range draws are made as before (so the generator's
      stream, and everything drawn after the neurons, is that of the flat-range file) and the
      first of them, as r = inRange(0, 1), gives all four: excitatory a = 0.02, b = 0.2,
      c = -65 + 15 r r, d = 8 - 6 r r; inhibitory a = 0.02 + 0.08 r, b = 0.25 - 0.05 r, c = -65,
      d = 2 (float arithmetic, left to right).  The drop-in driver replays the same draws from
      the generator's state before the neurons drew.

One difference from the reference: ConnStatic keeps each source's nConnsPerNeuron nearest
neurons with equal distances in neuron-index order.  The reference sorts with std::sort, which
leaves the order of equal distances to the C++ library, so where the last distance kept is shared
by more neurons than are kept, the two can keep different ones.  Everything else is the same: the
count per source, the distances kept, and the weights, drawn one per synapse in creation order.
"""
import ctypes
import ctypes.util
import os
import re
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import lib as bg

f32 = np.float32
DELTA_T = f32(1e-4)                       # DEFAULT_dt (Utils/Global.h)
EXC, INH = 2, 1                           # neuronType (Utils/Global.h)
II, IE, EI, EE = 0, 1, 2, 3               # synapseType (Utils/Global.h:100)
SYNAPSE_STRENGTH_ADJUSTMENT = f32(1.0e-8)

NEURON_CLASSES = {"AllLIFNeurons": bg.BG3_NEURON_LIF, "AllIZHNeurons": bg.BG3_NEURON_IZH}
SYNAPSE_CLASSES = {"AllSpikingSynapses": bg.BG3_SYN_SPIKING, "AllDSSynapses": bg.BG3_SYN_DS,
                   "AllSTDPSynapses": bg.BG3_SYN_STDP,
                   "AllDynamicSTDPSynapses": bg.BG3_SYN_DYNSTDP}
IF_RANGES = ("Iinject", "Inoise", "Vthresh", "Vresting", "Vreset", "Vinit", "starter_vthresh",
             "starter_vreset")
IZH_RANGES = ("Aconst", "Bconst", "Cconst", "Dconst")
# AllSTDPSynapses::createSynapse's constants (Synapses/AllSTDPSynapses.cpp:252-273)
STDP_DEFAULTS = dict(Apos=0.5, Aneg=-0.5, STDPgap=2e-3, tauspost=75e-3, tauspre=34e-3,
                     taupos=15e-3, tauneg=35e-3, WexExc=1.0, WexInh=1.0, mupos=0.0, muneg=0.0,
                     useFroemkeDanSTDP=1)
# per synapse type II, IE, EI, EE: AllSpikingSynapses / AllDSSynapses::createSynapse
# (Synapses/AllSpikingSynapses.cpp:192-240, AllDSSynapses.cpp:180-218)
TYPE_TAU = (f32(6e-3), f32(6e-3), f32(3e-3), f32(3e-3))
TYPE_DELAY = (f32(0.8e-3), f32(0.8e-3), f32(0.8e-3), f32(1.5e-3))
TYPE_UDF = ((f32(0.32), f32(0.144), f32(0.06)), (f32(0.25), f32(0.7), f32(0.02)),
            (f32(0.05), f32(0.125), f32(1.2)), (f32(0.5), f32(1.1), f32(0.05)))


class ConfigError(ValueError):
    """A parameter file the reference would refuse (ParseParamError, or a missing element)."""


# ---- the reference's global generator ---------------------------------------------------------
class MTRand:
    """MTRand (RNG/MersenneTwister.cpp): MT19937 of Matsumoto and Nishimura (1998) with Knuth's
    seeding, tempered 32-bit outputs.  rand() is float(x) / (2^32 - 1) computed in double and
    rounded to float; inRange(lo, hi) is rand() * (hi - lo) + lo in float.  Outputs are made 624
    at a time with numpy (the three independent stretches of the state update)."""

    def __init__(self, seed=1):
        s = [0] * 624
        s[0] = seed & 0xFFFFFFFF
        for i in range(1, 624):
            s[i] = (1812433253 * (s[i - 1] ^ (s[i - 1] >> 30)) + i) & 0xFFFFFFFF
        self._s = np.array(s, np.uint32)
        self._out = np.empty(0, np.uint32)
        self._pos = 0
        self._reload()

    @staticmethod
    def _twist(m, u, v):
        y = (u & np.uint32(0x80000000)) | (v & np.uint32(0x7FFFFFFF))
        odd = (v & np.uint32(1)).astype(bool)
        return m ^ (y >> np.uint32(1)) ^ np.where(odd, np.uint32(0x9908B0DF), np.uint32(0))

    def _reload(self):
        s, t = self._s, self._twist
        s[0:227] = t(s[397:624], s[0:227], s[1:228])
        s[227:454] = t(s[0:227], s[227:454], s[228:455])
        s[454:623] = t(s[227:396], s[454:623], s[455:624])
        s[623] = t(s[396], s[623], s[0])
        y = s.copy()
        y ^= y >> np.uint32(11)
        y ^= (y << np.uint32(7)) & np.uint32(0x9D2C5680)
        y ^= (y << np.uint32(15)) & np.uint32(0xEFC60000)
        y ^= y >> np.uint32(18)
        self._out, self._pos = y, 0

    def randint(self, n):
        """The next n 32-bit outputs."""
        parts, n = [], int(n)
        while n > 0:
            if self._pos == 624:
                self._reload()
            k = min(n, 624 - self._pos)
            parts.append(self._out[self._pos:self._pos + k])
            self._pos += k
            n -= k
        return np.concatenate(parts) if parts else np.empty(0, np.uint32)

    def rand(self, n):
        x = self.randint(n).astype(f32).astype(np.float64) * (1.0 / 4294967295.0)
        return x.astype(f32)

    def rand1(self):
        """One rand() as a float32 scalar (for sequential draws)."""
        if self._pos == 624:
            self._reload()
        x = int(self._out[self._pos])
        self._pos += 1
        return f32(float(f32(x)) * (1.0 / 4294967295.0))

    def in_range(self, lo, hi, n=None):
        """inRange with scalar or per-draw bounds; n defaults to the bounds' length."""
        lo, hi = np.asarray(lo, f32), np.asarray(hi, f32)
        if n is None:
            n = np.broadcast(lo, hi).size
        v = self.rand(n)
        return (v * (hi - lo)).astype(f32) + lo


_libm = None


def _m():
    global _libm
    if _libm is None:
        _libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
        for fn in ("expf", "logf"):
            getattr(_libm, fn).restype = ctypes.c_float
            getattr(_libm, fn).argtypes = [ctypes.c_float]
    return _libm


def expf(x):
    """The C library's expf, which the reference's exp(float) calls (the host library, not
    numpy's own exp, decides the last bit)."""
    return f32(_m().expf(float(f32(x))))


def logf(x):
    """The C library's logf (the reference's log(float))."""
    return f32(_m().logf(float(f32(x))))


# ---- parameters --------------------------------------------------------------------------------
@dataclass
class Params:
    """What a BrainGrid parameter file (plus an optional stimulus file) says."""
    width: int = 0
    height: int = 0
    tsim: np.float32 = f32(0)
    epochs: int = 0
    max_firing_rate: int = 0
    max_syn: int = 0
    seed: int = 0
    output: str = ""
    neuron_class: str = ""
    if_ranges: dict = field(default_factory=dict)     # name -> (min, max) float32
    izh_ranges: dict = field(default_factory=dict)    # name -> (minExc, maxExc, minInh, maxInh)
    izh_draw: str = "ranges"
    synapse_class: str = ""
    stdp: dict = None                                 # STDPParams override, or None
    conn_class: str = ""
    growth: dict = field(default_factory=dict)
    static: dict = field(default_factory=dict)
    layout_class: str = ""
    inh_list: list = field(default_factory=list)
    active_list: list = field(default_factory=list)
    probed_list: list = field(default_factory=list)
    frac_exc: np.float32 = f32(0)
    frac_starter: np.float32 = f32(0)
    stim: dict = None

    @property
    def n_neurons(self):
        return self.width * self.height

    @property
    def neuron_kind(self):
        return NEURON_CLASSES[self.neuron_class]

    @property
    def synapse_kind(self):
        return SYNAPSE_CLASSES[self.synapse_class]

    @property
    def steps_per_epoch(self):
        # static_cast<uint64_t>(epochDuration / deltaT) in float (Core/Simulator.cpp:159-160)
        return int(f32(self.tsim) / DELTA_T)


def _text(el, what):
    if el is None or el.text is None or not el.text.strip():
        raise ConfigError("missing value: " + what)
    return el.text.strip()


def _atof(s):
    """atof: the longest numeric prefix (0.0 if none)."""
    s = s.strip()
    for k in range(len(s), 0, -1):
        try:
            return float(s[:k])
        except ValueError:
            pass
    return 0.0


def _atoi(s):
    s = s.strip()
    k = 1 if s[:1] in "+-" else 0
    while k < len(s) and s[k].isdigit():
        k += 1
    try:
        return int(s[:k])
    except ValueError:
        return 0


def _child(sec, tag):
    """First element with this tag under sec (the visitors match by tag at any depth)."""
    return None if sec is None else next(sec.iter(tag), None)


def _value_list(text):
    """getValueList: whitespace-separated integers (Utils/Util.cpp)."""
    return [_atoi(t) for t in (text or "").split()]


def _parse(source):
    """The root element of an XML file or text.  The XML declaration is dropped first: the
    reference's files are read by TinyXML, which accepts declarations such as
    standalone=no that a strict parser refuses."""
    if not source.lstrip().startswith("<"):
        try:
            with open(source, encoding="utf-8", errors="replace") as f:
                source = f.read()
        except OSError as e:
            raise ConfigError("cannot read %s: %s" % (source, e.strerror))
    source = re.sub(r"^\s*<\?xml[^>]*\?>", "", source, count=1)
    try:
        return ET.fromstring(source)
    except ET.ParseError as e:
        raise ConfigError("malformed XML: %s" % e)


def _read_list_file(path, root_tag):
    doc = _parse(path)
    if doc.tag != root_tag:
        raise ConfigError("could not find <%s> in %s" % (root_tag, path))
    return _value_list(doc.text)


def read(config, stim=None, root=None):
    """Reads a parameter file (path, or the XML text itself when it starts with '<') and an
    optional stimulus file (the reference's -s).  File names inside the files are resolved
    against root (the reference resolves them against its working directory; default: the
    current directory)."""
    root = root or os.getcwd()

    def path(p):
        return p if os.path.isabs(p) else os.path.join(root, p)

    doc = _parse(config)
    p = Params()
    si = doc.find("SimInfoParams")
    if si is None:
        raise ConfigError("missing SimInfoParams")
    pool = _child(si, "PoolSize")
    p.width = _atoi(_text(_child(pool, "x"), "PoolSize x"))
    p.height = _atoi(_text(_child(pool, "y"), "PoolSize y"))
    sp = _child(si, "SimParams")
    p.tsim = f32(_atof(_text(_child(sp, "Tsim"), "Tsim")))
    p.epochs = int(_atof(_text(_child(sp, "numSims"), "numSims")))
    sc = _child(si, "SimConfig")
    p.max_firing_rate = _atoi(_text(_child(sc, "maxFiringRate"), "maxFiringRate"))
    p.max_syn = _atoi(_text(_child(sc, "maxSynapsesPerNeuron"), "maxSynapsesPerNeuron"))
    p.seed = _atoi(_text(_child(_child(si, "Seed"), "value"), "Seed value"))
    out = _child(si, "stateOutputFileName")
    p.output = out.text.strip() if out is not None and out.text else ""
    if p.width <= 0 or p.height <= 0 or p.tsim < 0 or p.epochs < 0 or p.max_firing_rate < 0 \
            or p.max_syn < 0:
        raise ConfigError("invalid SimInfoParams")

    model = doc.find("ModelParams")
    if model is None:
        raise ConfigError("missing ModelParams")
    ext = doc.find("BG3Params")
    if ext is not None:
        unknown = [e.tag for e in ext if e.tag not in ("STDPParams", "ParameterDraw")]
        if unknown:
            raise ConfigError("unknown BG3Params element %r" % unknown[0])
    _read_neurons(p, model.find("NeuronsParams"), ext)
    syn = model.find("SynapsesParams")
    p.synapse_class = syn.get("class", "") if syn is not None else ""
    if p.synapse_class not in SYNAPSE_CLASSES:
        raise ConfigError("unsupported synapse class %r" % p.synapse_class)
    st = _extension(syn, ext, "STDPParams")
    if st is not None:
        if p.synapse_kind < bg.BG3_SYN_STDP:
            raise ConfigError("STDPParams given for %s" % p.synapse_class)
        p.stdp = dict(STDP_DEFAULTS)
        for k in STDP_DEFAULTS:
            e = _child(st, k)
            if e is not None:
                p.stdp[k] = _atoi(_text(e, k)) if k == "useFroemkeDanSTDP" else \
                    float(f32(_atof(_text(e, k))))
    _read_connections(p, model.find("ConnectionsParams"))
    _read_layout(p, model.find("LayoutParams"), path)
    if stim is not None:
        p.stim = _read_stim(stim, path, p)
    return p


def _extension(sec, ext, tag):
    """The element tag of this reader's extensions: in <BG3Params> (ext) or inside sec, not both."""
    a, b = _child(sec, tag), _child(ext, tag)
    if a is not None and b is not None:
        raise ConfigError("%s given twice" % tag)
    return a if a is not None else b


def _read_neurons(p, sec, ext=None):
    if sec is None or sec.get("class") not in NEURON_CLASSES:
        raise ConfigError("unsupported neuron class %r" % (sec.get("class") if sec is not None
                                                            else None))
    p.neuron_class = sec.get("class")
    for name in IF_RANGES:
        e = _child(sec, name)
        lo = f32(_atof(_text(_child(e, "min"), name + " min")))
        hi = f32(_atof(_text(_child(e, "max"), name + " max")))
        if lo > hi:
            raise ConfigError("%s: min above max" % name)
        p.if_ranges[name] = (lo, hi)
    d = _extension(sec, ext, "ParameterDraw")
    if d is not None and p.neuron_class != "AllIZHNeurons":
        raise ConfigError("ParameterDraw given for %s" % p.neuron_class)
    if p.neuron_class == "AllIZHNeurons":
        p.izh_draw = _text(d, "ParameterDraw") if d is not None else "ranges"
        if p.izh_draw not in ("ranges", "r_squared"):
            raise ConfigError("ParameterDraw must be ranges or r_squared")
        if p.izh_draw == "ranges":
            for name in IZH_RANGES:
                e = _child(sec, name)
                v = tuple(f32(_atof(_text(_child(e, k), name + " " + k)))
                          for k in ("minExc", "maxExc", "minInh", "maxInh"))
                p.izh_ranges[name] = v


def _read_connections(p, sec):
    p.conn_class = sec.get("class", "") if sec is not None else ""
    if p.conn_class == "ConnGrowth":
        g = _child(sec, "GrowthParams")
        keys = (("epsilon", "epsilon"), ("beta", "beta"), ("rho", "rho"),
                ("targetRate", "target_rate"), ("minRadius", "min_radius"),
                ("startRadius", "start_radius"))
        p.growth = {k: f32(_atof(_text(_child(g, x), x))) for x, k in keys}
    elif p.conn_class == "ConnStatic":
        s = _child(sec, "StaticConnectionsParams")
        w = _child(sec, "StaticConnectionsWeight")
        p.static = dict(
            n=_atoi(_text(_child(s, "nConnsPerNeuron"), "nConnsPerNeuron")),
            radius=f32(_atof(_text(_child(s, "threshConnsRadius"), "threshConnsRadius"))),
            rewire=f32(_atof(_text(_child(s, "pRewiring"), "pRewiring"))),
            exc=tuple(f32(_atof(_text(_child(w, k), k))) for k in ("minExc", "maxExc")),
            inh=tuple(f32(_atof(_text(_child(w, k), k))) for k in ("minInh", "maxInh")))
    else:
        raise ConfigError("unsupported connections class %r" % p.conn_class)


def _read_layout(p, sec, path):
    p.layout_class = sec.get("class", "") if sec is not None else ""
    if p.layout_class == "FixedLayout":
        files = _child(sec, "LayoutFiles")
        for tag, root_tag, attr in (("activeNListFileName", "A", "active_list"),
                                    ("inhNListFileName", "I", "inh_list"),
                                    ("probedNListFileName", "P", "probed_list")):
            e = _child(files, tag)
            if e is not None and e.text and e.text.strip():
                setattr(p, attr, _read_list_file(path(e.text.strip()), root_tag))
        N = p.n_neurons
        if any(not 0 <= i < N for i in p.inh_list + p.active_list):
            raise ConfigError("neuron list index out of range")
    elif p.layout_class == "DynamicLayout":
        p.frac_exc = f32(_atof(_text(_child(sec, "frac_EXC"), "frac_EXC")))
        p.frac_starter = f32(_atof(_text(_child(sec, "starter_neurons"), "starter_neurons")))
        if not (0 <= p.frac_exc <= 1 and 0 <= p.frac_starter <= 1):
            raise ConfigError("invalid range for a fraction")
    else:
        raise ConfigError("unsupported layout class %r" % p.layout_class)


def _read_stim(stim, path, p):
    doc = _parse(stim)
    if doc.tag != "InputParams":
        raise ConfigError("missing InputParams")
    m = doc.find("IMethod")
    name = m.get("name") if m is not None else None
    ip = doc.find("IntParams")
    if ip is None:
        raise ConfigError("missing IntParams")
    if name == "SInputRegular":
        vals = []
        v = doc.find("Values")
        if v is None:
            raise ConfigError("missing Values")
        for e in v:
            if e.tag != "I":
                raise ConfigError("error I")
            vals += [f32(_atof(t)) for t in (e.text or "").split()]
        if len(vals) != 100:
            raise ConfigError("SInputRegular wants a 10x10 value pattern")
        return dict(kind="regular", duration=f32(_atof(ip.get("duration", ""))),
                    interval=f32(_atof(ip.get("interval", ""))), sync=ip.get("sync", ""),
                    values=np.array(vals, f32))
    if name == "SInputPoisson":
        masks = None
        mk = doc.find("Masks")
        if mk is not None:
            idx = []
            for e in mk:
                if e.tag == "M":
                    idx += _value_list(e.text)
                elif e.tag == "LayoutFiles":
                    f = e.get("maskNListFileName") or _text(_child(e, "maskNListFileName"),
                                                            "maskNListFileName")
                    idx += _read_list_file(path(f), "M")
            masks = np.zeros(p.n_neurons, np.uint8)
            masks[np.asarray(idx, np.int64)] = 1
        return dict(kind="poisson", fr_mean=f32(_atof(ip.get("fr_mean", ""))),
                    weight=f32(_atof(ip.get("weight", ""))), masks=masks)
    raise ConfigError("unsupported input method %r" % name)


def write(p, lists_dir="configfiles/bg3", name="network"):
    """p as a parameter file in the reference's element layout (the reverse of read), plus the
    neuron-list files it names: returns (text, {relative path: list-file text}).  Values are
    written with Python's shortest round-trip repr, so reading the text back gives p's float32
    values exactly.  STDP constants and the r_squared draw go into <BG3Params> (see the module
    docstring), which the reference's driver reads past."""
    def v(x):
        return repr(float(x)) if not isinstance(x, (int, np.integer)) else str(int(x))

    def rng(tag, lo, hi):
        return '<%s name="%s"><min name="min">%s</min><max name="max">%s</max></%s>' % (
            tag, tag, v(lo), v(hi), tag)

    files = {}
    ext = []
    neu = [rng(k, *p.if_ranges[k]) for k in IF_RANGES]
    if p.neuron_class == "AllIZHNeurons":
        if p.izh_draw == "r_squared":
            ext.append("<ParameterDraw>r_squared</ParameterDraw>")
        else:
            for k in IZH_RANGES:
                z = p.izh_ranges[k]
                neu.append('<%s name="%s">%s</%s>' % (k, k, "".join(
                    '<%s name="%s">%s</%s>' % (t, t, v(x), t)
                    for t, x in zip(("minExc", "maxExc", "minInh", "maxInh"), z)), k))
    syn = ""
    if p.stdp is not None:
        ext.append("<STDPParams>%s</STDPParams>" % "".join(
            "<%s>%s</%s>" % (k, v(p.stdp[k]), k) for k in STDP_DEFAULTS))
    if p.conn_class == "ConnGrowth":
        g = p.growth
        conn = '<GrowthParams name="GrowthParams">%s</GrowthParams>' % "".join(
            '<%s name="%s">%s</%s>' % (x, x, v(g[k]), x) for x, k in (
                ("epsilon", "epsilon"), ("beta", "beta"), ("rho", "rho"),
                ("targetRate", "target_rate"), ("minRadius", "min_radius"),
                ("startRadius", "start_radius")))
    else:
        st = p.static
        conn = ('<StaticConnectionsParams name="StaticConnectionsParams">'
                '<nConnsPerNeuron name="nConnsPerNeuron">%d</nConnsPerNeuron>'
                '<threshConnsRadius name="threshConnsRadius">%s</threshConnsRadius>'
                '<pRewiring name="pRewiring">%s</pRewiring></StaticConnectionsParams>'
                '<StaticConnectionsWeight name="StaticConnectionsWeight">'
                '<minExc name="minExc">%s</minExc><maxExc name="maxExc">%s</maxExc>'
                '<minInh name="minInh">%s</minInh><maxInh name="maxInh">%s</maxInh>'
                '</StaticConnectionsWeight>' % (st["n"], v(st["radius"]), v(st["rewire"]),
                                                v(st["exc"][0]), v(st["exc"][1]),
                                                v(st["inh"][0]), v(st["inh"][1])))
    if p.layout_class == "FixedLayout":
        lay = []
        for tag, root_tag, lst in (("activeNListFileName", "A", p.active_list),
                                   ("inhNListFileName", "I", p.inh_list),
                                   ("probedNListFileName", "P", p.probed_list)):
            if not lst:
                # an empty element, as the reference's files have it (an empty list file makes
                # its reader fail)
                lay.append('<%s name="%s" type="InputFile"/>' % (tag, tag))
                continue
            rel = "%s/%s-%s.xml" % (lists_dir, name, root_tag)
            files[rel] = '<?xml version="1.0" encoding="UTF-8"?>\n<%s>%s</%s>\n' % (
                root_tag, " ".join(str(int(i)) for i in lst), root_tag)
            lay.append('<%s name="%s" type="InputFile">%s</%s>' % (tag, tag, rel, tag))
        layout = '<LayoutFiles name="LayoutFiles">%s</LayoutFiles>' % "".join(lay)
    else:
        layout = ('<frac_EXC name="frac_EXC">%s</frac_EXC><starter_neurons '
                  'name="starter_neurons">%s</starter_neurons>' % (v(p.frac_exc),
                                                                   v(p.frac_starter)))
    text = (
        '<?xml version="1.0" encoding="UTF-8" standalone="no"?>\n<BGSimParams>\n'
        '  <SimInfoParams name="SimInfoParams">'
        '<PoolSize name="PoolSize"><x name="x">%d</x><y name="y">%d</y><z name="z">1</z></PoolSize>'
        '<SimParams name="SimParams"><Tsim name="Tsim">%s</Tsim><numSims name="numSims">%d'
        '</numSims></SimParams><SimConfig name="SimConfig"><maxFiringRate name="maxFiringRate">%d'
        '</maxFiringRate><maxSynapsesPerNeuron name="maxSynapsesPerNeuron">%d'
        '</maxSynapsesPerNeuron></SimConfig><Seed name="Seed"><value name="value">%d</value>'
        '</Seed><OutputParams name="OutputParams"><stateOutputFileName '
        'name="stateOutputFileName">%s</stateOutputFileName></OutputParams></SimInfoParams>\n'
        '  <ModelParams>\n'
        '    <NeuronsParams class="%s" name="NeuronsParams">%s</NeuronsParams>\n'
        '    <SynapsesParams class="%s" name="SynapsesParams">%s</SynapsesParams>\n'
        '    <ConnectionsParams class="%s" name="ConnectionsParams">%s</ConnectionsParams>\n'
        '    <LayoutParams class="%s" name="LayoutParams">%s</LayoutParams>\n'
        '  </ModelParams>\n%s</BGSimParams>\n' % (
            p.width, p.height, v(p.tsim), p.epochs, p.max_firing_rate, p.max_syn, p.seed,
            p.output or "results/%s-out.xml" % name, p.neuron_class, "".join(neu),
            p.synapse_class, syn, p.conn_class, conn, p.layout_class, layout,
            "  <BG3Params>%s</BG3Params>\n" % "".join(ext) if ext else ""))
    return text, files


# ---- setup ------------------------------------------------------------------------------------
def _steps(seconds):
    """static_cast<int>(seconds / deltaT + 0.5): float quotient, double sum."""
    return int(float(f32(seconds) / DELTA_T) + 0.5)


def setup(p):
    """The host arrays of Model::setupSim for p, in the reference's layouts (dict of numpy
    arrays, see the module docstring for the draw order)."""
    N, W, H = p.n_neurons, p.width, p.height
    rng = MTRand(1)
    out = dict(N=N)
    stim = p.stim
    if stim is not None and stim["kind"] == "regular":
        dur = _steps(stim["duration"])
        cyc = dur + _steps(stim["interval"])
        values = np.array([stim["values"][(i % 10) * 10 + j % 10]
                           for i in range(H) for j in range(W)], f32)
        if stim["sync"] == "no":
            shifts = rng.in_range(f32(0), f32(cyc - 1), N).astype(np.int32)
        elif stim["sync"] == "wave":
            shifts = np.tile((cyc // W) * np.arange(W, dtype=np.int64), H).astype(np.int32)
        else:
            shifts = np.zeros(N, np.int32)
        out["regular"] = dict(values=values, shifts=shifts, n_steps_duration=dur,
                              n_steps_cycle=cyc)

    # Layout::setupLayout / initNeuronsLocs (grid), type and starter maps
    idx = np.arange(N)
    out["xloc"], out["yloc"] = (idx % W).astype(f32), (idx // W).astype(f32)
    ntype = np.full(N, EXC, np.int32)
    starter = np.zeros(N, bool)
    if p.layout_class == "FixedLayout":
        ntype[np.asarray(p.inh_list, np.int64)] = INH
        starter[np.asarray(p.active_list, np.int64)] = True
    else:
        n_exc = int(float(p.frac_exc * f32(N)) + 0.5)
        n_inh = N - n_exc
        layout = np.arange(max(n_inh, 0))
        if N > n_inh:
            u = rng.rand(N - n_inh)
            j = (u * f32(N)).astype(f32).astype(np.int64)
            for i, jj in zip(range(n_inh, N), j):
                if jj < n_inh:
                    layout[jj] = i
        ntype[layout] = INH
        want = int(float(p.frac_starter * f32(N)) + 0.5)
        got = 0
        while got < want:
            # rng.inRange(0, N) can return N itself (probability 2^-32), an index the reference
            # reads past its map; such a draw is passed over here
            i = int(rng.in_range(f32(0), f32(N), 1)[0])
            if i < N and ntype[i] == EXC and not starter[i]:
                starter[i] = True
                got += 1
    out["ntype"], out["starter"] = ntype, starter

    _create_neurons(p, rng, out)
    if p.conn_class == "ConnStatic":
        _connect_static(p, rng, out)
    if stim is not None and stim["kind"] == "poisson":
        out["poisson"] = _poisson_input(p, out)
    out["rng"] = rng                 # the global generator as setup leaves it
    return out


def poisson_intervals(a, nsteps):
    """The Poisson stimulus's interval draws for steps [0, nsteps) as the reference makes them
    on the global generator after setup (HostSInputPoisson::inputStimulus, Inputs/
    HostSInputPoisson.cpp:60-94): every step, neurons ascending, each masked neuron whose
    counter runs out draws isi = -lambda log U ms until a second draw U' > exp(-isi^2 / 32) keeps
    it, and waits (int)(isi / 1000 / deltaT + 0.5) steps.  The draws depend on the masks and
    the counters only, so they are made ahead, event by event.  Returns (begin[N + 1], steps)
    for bg3_push_poisson_isis (neuron i's intervals in steps[begin[i]:begin[i + 1]]); advances
    a["rng"]."""
    import heapq
    pa = a["poisson"]["arrays"]
    lam, rng, N = f32(a["poisson"]["lam"]), a["rng"], a["N"]
    mlam = f32(-lam)
    heap = [(max(int(c), 1) - 1, i) for i, c in enumerate(pa["nISIs"]) if pa["masks"][i]]
    heapq.heapify(heap)
    seqs = [[] for _ in range(N)]
    while heap and heap[0][0] < nsteps:
        t, i = heapq.heappop(heap)
        isi = f32(mlam * logf(rng.rand1()))
        while rng.rand1() <= expf(-(isi * isi) / f32(32)):
            isi = f32(mlam * logf(rng.rand1()))
        v = int(float((isi / f32(1000)) / DELTA_T) + 0.5)
        seqs[i].append(v)
        heapq.heappush(heap, (t + max(v, 1), i))
    begin = np.zeros(N + 1, np.int32)
    begin[1:] = np.cumsum([len(q) for q in seqs])
    steps = np.array([v for q in seqs for v in q], np.int32)
    return begin, steps


def _create_neurons(p, rng, out):
    """AllIFNeurons::createAllNeurons / createNeuron / initNeuronConstsFromParamValues and the
    Izhikevich additions.  Per neuron: Iinject, Inoise, Vthresh, Vrest, Vreset, Vinit; two more
    (Vthresh, Vreset) for a starter; then a, b, c, d for an Izhikevich neuron (with the r^2
    draw the first of these is r and the other three are unused)."""
    N = out["N"]
    ntype, starter = out["ntype"], out["starter"]
    izh = p.neuron_class == "AllIZHNeurons"
    extra = 4 if izh else 0
    per = 6 + 2 * starter.astype(np.int64) + extra
    first = np.concatenate([[0], np.cumsum(per)[:-1]])
    u = rng.rand(int(per.sum()))

    def draw(off, lo, hi):
        """inRange(lo, hi) with each neuron's draw number off: v * (hi - lo) + lo in float."""
        return (u[first + off] * (f32(hi) - f32(lo))).astype(f32) + f32(lo)

    r = p.if_ranges
    Iinject = draw(0, *r["Iinject"])
    Inoise = draw(1, *r["Inoise"])
    Vthresh = draw(2, *r["Vthresh"])
    Vrest = draw(3, *r["Vresting"])
    Vreset = draw(4, *r["Vreset"])
    Vinit = draw(5, *r["Vinit"])
    Cm = np.full(N, f32(3e-8), f32)                 # DEFAULT_Cm, DEFAULT_Rm (Utils/Global.h)
    Rm = np.full(N, f32(1e6), f32)
    Tau = np.full(N, f32(3e-8 * 1e6), f32)
    c1 = expf(-DELTA_T / f32(3e-8 * 1e6))
    C1 = np.full(N, c1, f32)
    C2 = (Rm * (f32(1) - C1)).astype(f32)
    I0 = (Iinject + (Vrest / Rm).astype(f32)).astype(f32)
    Trefract = np.where(ntype == INH, f32(2.0e-3), f32(3.0e-3)).astype(f32)
    st = np.nonzero(starter)[0]
    sv = r["starter_vthresh"]
    sr = r["starter_vreset"]
    Vthresh[st] = (u[first[st] + 6] * (sv[1] - sv[0])).astype(f32) + sv[0]
    Vreset[st] = (u[first[st] + 7] * (sr[1] - sr[0])).astype(f32) + sr[0]
    Trefract[st] = f32(3.0e-3)
    out.update(Iinject=Iinject, Inoise=Inoise, Vthresh=Vthresh, Vrest=Vrest, Vreset=Vreset,
               Vinit=Vinit, Vm=Vinit.copy(), Cm=Cm, Rm=Rm, Tau=Tau, C1=C1, C2=C2, I0=I0,
               Trefract=Trefract)
    if not izh:
        return
    off = 6 + 2 * starter.astype(np.int64)
    inh = ntype != EXC
    if p.izh_draw == "r_squared":
        rr = u[first + off]
        a = np.where(inh, f32(0.02) + f32(0.08) * rr, f32(0.02)).astype(f32)
        b = np.where(inh, f32(0.25) - f32(0.05) * rr, f32(0.2)).astype(f32)
        c = np.where(inh, f32(-65.0), f32(-65.0) + f32(15.0) * rr * rr).astype(f32)
        d = np.where(inh, f32(2.0), f32(8.0) - f32(6.0) * rr * rr).astype(f32)
    else:
        vals = []
        for k, name in enumerate(IZH_RANGES):
            z = p.izh_ranges[name]
            lo = np.where(inh, z[2], z[0]).astype(f32)
            hi = np.where(inh, z[3], z[1]).astype(f32)
            vals.append(((u[first + off + k] * (hi - lo)).astype(f32) + lo).astype(f32))
        a, b, c, d = vals
    out.update(Aconst=a, Bconst=b, Cconst=c, Dconst=d, u=np.zeros(N, f32),
               C3=np.full(N, DELTA_T * f32(1000), f32))


def syn_type(src_inh, dst_inh):
    """Layout::synType: II 0, IE 1 (inhibitory source), EI 2, EE 3."""
    return np.where(src_inh, np.where(dst_inh, II, IE), np.where(dst_inh, EI, EE)).astype(np.int32)


def empty_slots(N, M):
    S = N * M
    return dict(in_use=np.zeros(S, np.uint8), src=np.zeros(S, np.int32),
                type=np.full(S, -1, np.int32), W=np.zeros(S, f32), psr=np.zeros(S, f32),
                decay=np.zeros(S, f32), tau=np.zeros(S, f32), total_delay=np.zeros(S, np.int32),
                delayIdx=np.zeros(S, np.int32), delayQueue=np.zeros(S, np.uint32),
                U=np.zeros(S, f32), D=np.zeros(S, f32), F=np.zeros(S, f32), u=np.zeros(S, f32),
                r=np.zeros(S, f32),
                lastSpike=np.full(S, np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64))


def _connect_static(p, rng, out):
    """ConnStatic::setupConnections (Connections/ConnStatic.cpp:33-80): each source, in index
    order, connects to its nConnsPerNeuron nearest neurons within threshConnsRadius (distances
    sqrt(dx^2 + dy^2) in float; equal distances in neuron-index order); each synapse goes to the
    first free slot of its destination's row (AllSynapses::addSynapse) and takes one weight draw,
    from the excitatory or the inhibitory range by its source's type.  pRewiring is read and, as
    in the reference, not applied."""
    N, W, H, M = out["N"], p.width, p.height, p.max_syn
    s = p.static
    radius = f32(s["radius"])
    xi, yi = np.arange(N) % W, np.arange(N) // W
    # grid offsets within the radius, nearest first; equal distances in row-major order, which
    # is neuron-index order for every source
    R = int(np.ceil(float(radius))) + 1
    offs = []
    for dy in range(-R, R + 1):
        for dx in range(-R, R + 1):
            if dx or dy:
                d = np.sqrt(f32(dx * dx + dy * dy), dtype=f32)
                if d <= radius:
                    offs.append((float(d), dy, dx))
    offs.sort()
    taken = np.zeros(N, np.int64)
    srcs, dsts, rank = [], [], []
    for k, (_, dy, dx) in enumerate(offs):
        ok = (xi + dx >= 0) & (xi + dx < W) & (yi + dy >= 0) & (yi + dy < H) & (taken < s["n"])
        srcs.append(np.nonzero(ok)[0])
        dsts.append((yi[ok] + dy) * W + xi[ok] + dx)
        rank.append(taken[ok])
        taken += ok
    srcs = np.concatenate(srcs) if srcs else np.zeros(0, np.int64)
    dsts = np.concatenate(dsts) if dsts else np.zeros(0, np.int64)
    rank = np.concatenate(rank) if rank else np.zeros(0, np.int64)
    order = np.lexsort((rank, srcs))                 # creation order: source, then nearness
    srcs, dsts = srcs[order], dsts[order]
    inh_n = out["ntype"] == INH
    lo = np.where(inh_n[srcs], s["inh"][0], s["exc"][0]).astype(f32)
    hi = np.where(inh_n[srcs], s["inh"][1], s["exc"][1]).astype(f32)
    Wd = rng.in_range(lo, hi, len(srcs))
    # slot: the destination row's next free slot, in creation order
    by_dest = np.argsort(dsts, kind="stable")
    counts = np.bincount(dsts, minlength=N)
    if counts.max(initial=0) > M:
        raise ConfigError("maxSynapsesPerNeuron %d is below the in-degree %d" %
                          (M, counts.max()))
    start = np.concatenate([[0], np.cumsum(counts)[:-1]])
    pos = np.empty(len(dsts), np.int64)
    pos[by_dest] = np.arange(len(dsts)) - start[dsts[by_dest]]
    slot = dsts * M + pos
    syn = empty_slots(N, M)
    typ = syn_type(inh_n[srcs], inh_n[dsts])
    syn["in_use"][slot] = 1
    syn["src"][slot] = srcs
    syn["type"][slot] = typ
    syn["W"][slot] = Wd
    _fill_types(syn, slot, typ, p.synapse_kind)
    out["synapses"], out["counts"] = syn, counts.astype(np.uint32)
    out["creation_slots"] = slot


def _fill_types(syn, slot, typ, kind):
    tau = np.array(TYPE_TAU, f32)[typ]
    delay = np.array(TYPE_DELAY, f32)[typ]
    dec = {t: expf(-DELTA_T / TYPE_TAU[t]) for t in range(4)}
    syn["tau"][slot] = tau
    syn["decay"][slot] = np.array([dec[t] for t in range(4)], f32)[typ]
    syn["total_delay"][slot] = (delay / DELTA_T).astype(f32).astype(np.int32) + 1
    if kind in (bg.BG3_SYN_DS, bg.BG3_SYN_DYNSTDP):
        udf = np.array(TYPE_UDF, f32)[typ]
        syn["U"][slot], syn["D"][slot], syn["F"][slot] = udf[:, 0], udf[:, 1], udf[:, 2]
        syn["u"][slot] = f32(0.4)                      # DEFAULT_U
        syn["r"][slot] = f32(1.0)


def stdp_constants(p):
    """Per-type (II, IE, EI, EE) STDP constants of the synapses made: the file's STDPParams, or
    AllSTDPSynapses::createSynapse's values."""
    c = dict(STDP_DEFAULTS, **(p.stdp or {}))
    out = {k: c[k] for k in ("Apos", "Aneg", "STDPgap", "tauspost", "tauspre", "taupos",
                             "tauneg", "mupos", "muneg", "useFroemkeDanSTDP")}
    out["Wex"] = [c["WexInh"], c["WexInh"], c["WexExc"], c["WexExc"]]
    return out


def stdp_arrays(syn, consts):
    """Reference-layout STDP slot fields carrying the per-type constants (AllSTDPSynapses::
    createSynapse and initSpikeQueue, Synapses/AllSTDPSynapses.cpp:125-138,252-273)."""
    S = len(syn["in_use"])
    used = syn["in_use"].astype(bool)
    t = np.clip(syn["type"], 0, 3)
    out = dict(delayQueuePost=np.zeros(S, np.uint32), delayIdxPost=np.zeros(S, np.int32),
               total_delayPost=np.zeros(S, np.int32),
               useFroemkeDanSTDP=np.where(used, int(consts["useFroemkeDanSTDP"]), 0)
               .astype(np.uint8))
    for k in ("tauspost", "tauspre", "taupos", "tauneg", "STDPgap", "Wex", "Aneg", "Apos",
              "mupos", "muneg"):
        v = np.broadcast_to(np.asarray(consts[k], f32), (4,))
        out[k] = np.where(used, v[t], 0).astype(f32)
    return out


def _poisson_input(p, out):
    """SInputPoisson::SInputPoisson / init (Inputs/SInputPoisson.cpp:19-146): lambda in ms, the
    masks, and one DS input synapse per neuron (EI onto inhibitory, EE onto excitatory neurons)
    with W = weight x 1e-8 and every interval counter at 0."""
    stim, N = p.stim, out["N"]
    typ = np.where(out["ntype"] == INH, EI, EE)
    tau = f32(3e-3)
    delay = np.where(typ == EE, f32(1.5e-3), f32(0.8e-3)).astype(f32)
    udf = np.array(TYPE_UDF, f32)[typ]
    fr = stim["fr_mean"] / f32(1000)
    arr = dict(masks=stim["masks"] if stim["masks"] is not None else np.ones(N, np.uint8),
               nISIs=np.zeros(N, np.int32),
               total_delay=(delay / DELTA_T).astype(f32).astype(np.int32) + 1,
               delayIdx=np.zeros(N, np.int32), delayQueue=np.zeros(N, np.uint32),
               W=np.full(N, stim["weight"] * SYNAPSE_STRENGTH_ADJUSTMENT, f32),
               psr=np.zeros(N, f32), decay=np.full(N, expf(-DELTA_T / tau), f32),
               U=udf[:, 0].copy(), D=udf[:, 1].copy(), F=udf[:, 2].copy(),
               u=np.full(N, f32(0.4), f32), r=np.ones(N, f32),
               lastSpike=np.full(N, np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64))
    return dict(arrays=arr, lam=float(f32(1) / fr))


# ---- the network on the device -----------------------------------------------------------------
def desc(p, noise_mode=bg.BG3_NOISE_DEVICE):
    """The network shape (bg3_net_desc) of p; the noise keyed by the file's seed."""
    if p.max_syn <= 0:
        raise ConfigError("maxSynapsesPerNeuron must be positive")
    return bg.NetDesc(p.n_neurons, p.max_syn, p.width, p.height, float(p.tsim), float(DELTA_T),
                      p.max_firing_rate, max(p.epochs, 1), p.neuron_kind, p.synapse_kind,
                      noise_mode, p.seed)


def network(p, arrays=None, noise_mode=bg.BG3_NOISE_DEVICE, poisson_seed=None):
    """A bg3 network holding what setup(p) built: layout, neurons, synapses (ConnStatic), the
    ConnGrowth parameters, STDP constants and the stimulus.  Noise is keyed by the file's seed;
    with BG3_NOISE_INJECT push the reference's stream (NormStream(p.seed)) before stepping.
    Poisson intervals are drawn on the device keyed by poisson_seed (default the file's seed),
    or pushed (poisson_intervals)."""
    a = arrays if arrays is not None else setup(p)
    net = bg.Network.from_desc(desc(p, noise_mode))
    try:
        configure(net, p, a, poisson_seed)
    except Exception:
        net.close()
        raise
    return net


def configure(net, p, a, poisson_seed=None):
    """Uploads setup(p)'s arrays a into a created network of p's shape (the served form's setup
    callback calls this on the network the server made)."""
    N = a["N"]
    net.upload_layout(a["xloc"], a["yloc"], a["ntype"])
    net.upload_lif(Vm=a["Vm"], Vthresh=a["Vthresh"], Vreset=a["Vreset"], I0=a["I0"],
                   Inoise=a["Inoise"], C1=a["C1"], C2=a["C2"], Trefract=a["Trefract"])
    if p.neuron_kind == bg.BG3_NEURON_IZH:
        net.upload_izh(**{k: a[k] for k in ("Aconst", "Bconst", "Cconst", "Dconst", "u", "C3")})
    if "synapses" in a:
        net.upload_synapses(0, counts=a["counts"], **a["synapses"])
    if p.synapse_kind >= bg.BG3_SYN_STDP:
        consts = stdp_constants(p)
        net.set_stdp_constants(**consts)
        if "synapses" in a:
            s = a["synapses"]
            net.upload_stdp(s["in_use"], s["type"], s["delayIdx"], **stdp_arrays(s, consts))
    g = p.growth if p.conn_class == "ConnGrowth" else dict(
        epsilon=0.6, beta=0.1, rho=1e-4, target_rate=1.0, min_radius=0.1, start_radius=0.4)
    net.upload_growth(g["epsilon"], g["beta"], g["rho"], g["target_rate"], g["min_radius"],
                      g["start_radius"], np.full(N, g["start_radius"], f32))
    if "regular" in a:
        r = a["regular"]
        net.input_regular(r["values"], r["shifts"], r["n_steps_duration"],
                          r["n_steps_cycle"], 0)
    if "poisson" in a:
        net.input_poisson(a["poisson"]["lam"],
                          seed=p.seed if poisson_seed is None else poisson_seed, step=0,
                          **a["poisson"]["arrays"])
