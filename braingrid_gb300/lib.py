"""ctypes binding of libbg3 (include/bg3.h) and a thin host-side network handle.

The product path is the CUDA library; this module only marshals numpy arrays across the C-ABI.
There is no CPU fallback: importing works without a GPU, but creating a network raises if the
library or a CUDA device is missing.
"""
import ctypes
import os

import numpy as np

from . import build as _build

c_f32p = ctypes.POINTER(ctypes.c_float)
c_i32p = ctypes.POINTER(ctypes.c_int32)
c_u32p = ctypes.POINTER(ctypes.c_uint32)
c_u64p = ctypes.POINTER(ctypes.c_uint64)
c_u8p = ctypes.POINTER(ctypes.c_uint8)

BG3_NEURON_LIF, BG3_NEURON_IZH = 0, 1
BG3_SYN_SPIKING, BG3_SYN_DS, BG3_SYN_STDP, BG3_SYN_DYNSTDP = 0, 1, 2, 3
BG3_NOISE_DEVICE, BG3_NOISE_INJECT = 0, 1
BG3_STDP_HOST, BG3_STDP_DEVICE = 0, 1
(BG3_OK, BG3_EINVAL, BG3_ENOMEM, BG3_ECUDA, BG3_ENOISE, BG3_EDEVICE,
 BG3_EUNSUPPORTED, BG3_ECANCELED) = 0, -1, -2, -3, -4, -5, -6, -7
BG3_ERR_TIMEOUT = 1 << 6
ERR_BITS = {1: "history overflow", 2: "double spike in a queue slot", 4: "synapse row full",
            8: "injected noise exhausted", 16: "negative growth weight"}


class NetDesc(ctypes.Structure):
    _fields_ = [("n_neurons", ctypes.c_int32), ("max_syn_per_neuron", ctypes.c_int32),
                ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("epoch_duration", ctypes.c_float), ("delta_t", ctypes.c_float),
                ("max_firing_rate", ctypes.c_int32), ("max_epochs", ctypes.c_int32),
                ("neuron_kind", ctypes.c_int32), ("synapse_kind", ctypes.c_int32),
                ("noise_mode", ctypes.c_int32), ("noise_seed", ctypes.c_uint32)]


class LifArrays(ctypes.Structure):
    _fields_ = [(k, c_f32p) for k in ("Vm", "Vthresh", "Vreset", "I0", "Inoise", "C1", "C2",
                                      "Trefract", "summation")] + \
               [(k, c_i32p) for k in ("nStepsInRefr", "spikeCount", "spikeCountOffset")] + \
               [("history", c_u64p)]


class IzhArrays(ctypes.Structure):
    _fields_ = [(k, c_f32p) for k in ("Aconst", "Bconst", "Cconst", "Dconst", "u", "C3")]


STDP_FLOATS = ("tauspost", "tauspre", "taupos", "tauneg", "STDPgap", "Wex", "Aneg", "Apos",
               "mupos", "muneg")


class StdpArrays(ctypes.Structure):
    _fields_ = [("delayQueuePost", c_u32p), ("delayIdxPost", c_i32p), ("total_delayPost", c_i32p)] + \
               [(k, c_f32p) for k in STDP_FLOATS] + [("useFroemkeDanSTDP", c_u8p)]


class StdpConstants(ctypes.Structure):
    _fields_ = [(k, ctypes.c_float * 4) for k in ("Apos", "Aneg", "STDPgap", "tauspost", "tauspre",
                                                  "taupos", "tauneg", "Wex", "mupos", "muneg")] + \
               [("useFroemkeDanSTDP", ctypes.c_int32 * 4)]


class LaunchCfg(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int32) for k in ("sweep_stages", "thin_max_quads", "thin_warps",
                                              "deliver_blocks", "growth_threads", "sweep_dests",
                                              "deliver_early", "izh_hw_every",
                                              "small_max_slots")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SynArrays(ctypes.Structure):
    _fields_ = [("in_use", c_u8p)] + \
               [(k, c_i32p) for k in ("src", "type", "delayIdx", "total_delay")] + \
               [(k, c_f32p) for k in ("W", "psr", "decay", "tau")] + \
               [(k, c_u32p) for k in ("delayQueue", "counts")] + \
               [(k, c_f32p) for k in ("U", "D", "F", "u", "r")] + \
               [("lastSpike", c_u64p)]


class PoissonArrays(ctypes.Structure):
    _fields_ = [("masks", c_u8p)] + \
               [(k, c_i32p) for k in ("nISIs", "total_delay", "delayIdx")] + \
               [("delayQueue", c_u32p)] + \
               [(k, c_f32p) for k in ("W", "psr", "decay", "U", "D", "F", "u", "r")] + \
               [("lastSpike", c_u64p)]


POISSON_FIELDS = [("masks", np.uint8), ("nISIs", np.int32), ("total_delay", np.int32),
                  ("delayIdx", np.int32), ("delayQueue", np.uint32), ("W", np.float32),
                  ("psr", np.float32), ("decay", np.float32), ("U", np.float32),
                  ("D", np.float32), ("F", np.float32), ("u", np.float32), ("r", np.float32),
                  ("lastSpike", np.uint64)]


class TypeConstants(ctypes.Structure):
    _fields_ = [("tau", ctypes.c_float * 4), ("decay", ctypes.c_float * 4),
                ("total_delay", ctypes.c_int32 * 4), ("U", ctypes.c_float * 4),
                ("D", ctypes.c_float * 4), ("F", ctypes.c_float * 4),
                ("u0", ctypes.c_float), ("r0", ctypes.c_float)]


class GrowthParams(ctypes.Structure):
    _fields_ = [(k, ctypes.c_float) for k in ("epsilon", "beta", "rho", "target_rate",
                                              "min_radius", "start_radius", "max_rate")]


class IndexMaps(ctypes.Structure):
    _fields_ = [(k, c_u32p) for k in ("outgoingSynapseIndexMap", "outgoingSynapseBegin",
                                      "outgoingSynapseCount", "incomingSynapseIndexMap",
                                      "incomingSynapseBegin", "incomingSynapseCount")]


class StateView(ctypes.Structure):
    _fields_ = [("neurons", ctypes.POINTER(LifArrays)), ("izh", ctypes.POINTER(IzhArrays)),
                ("synapses", ctypes.POINTER(SynArrays)), ("stdp", ctypes.POINTER(StdpArrays)),
                ("maps", ctypes.POINTER(IndexMaps)), ("radii", c_f32p), ("rates", c_f32p)]


_LIB = None


IF_FIELDS = ("Cm", "Rm", "Vrest", "Vinit", "Iinject", "Isyn", "Tau")


class IfFields(ctypes.Structure):
    _fields_ = [(k, ctypes.POINTER(ctypes.c_float)) for k in IF_FIELDS]


BG3_CONN_STATIC, BG3_CONN_GROWTH = 0, 1


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libbg3.so (building it first if absent).  Raises if it cannot be loaded."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("libbg3.so is not built; run braingrid_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    sig = {
        "bg3_create": ([ctypes.POINTER(NetDesc), ctypes.POINTER(vp)], ctypes.c_int),
        "bg3_destroy": ([vp], ctypes.c_int),
        "bg3_upload_lif": ([vp, ctypes.POINTER(LifArrays)], ctypes.c_int),
        "bg3_upload_izh": ([vp, ctypes.POINTER(IzhArrays)], ctypes.c_int),
        "bg3_download_izh": ([vp, ctypes.POINTER(IzhArrays)], ctypes.c_int),
        "bg3_upload_stdp": ([vp, ctypes.POINTER(SynArrays), ctypes.POINTER(StdpArrays)], ctypes.c_int),
        "bg3_download_stdp": ([vp, ctypes.POINTER(StdpArrays)], ctypes.c_int),
        "bg3_set_stdp_constants": ([vp, ctypes.POINTER(StdpConstants)], ctypes.c_int),
        "bg3_set_stdp_arithmetic": ([vp, ctypes.c_int], ctypes.c_int),
        "bg3_epoch_record": ([vp], ctypes.c_int),
        "bg3_selftest_izhikevich": ([ctypes.c_uint64, ctypes.c_uint64,
                                     ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
        "bg3_selftest_binary64": ([ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)],
                                  ctypes.c_int),
        "bg3_get_launch": ([vp, ctypes.POINTER(LaunchCfg)], ctypes.c_int),
        "bg3_set_launch": ([vp, ctypes.POINTER(LaunchCfg)], ctypes.c_int),
        "bg3_batch_get_launch": ([vp, ctypes.POINTER(LaunchCfg)], ctypes.c_int),
        "bg3_batch_set_launch": ([vp, ctypes.POINTER(LaunchCfg)], ctypes.c_int),
        "bg3_autotune": ([vp, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(LaunchCfg),
                          ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
        "bg3_batch_autotune": ([vp, ctypes.c_int32, ctypes.POINTER(LaunchCfg),
                                ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
        "bg3_serialize": ([vp, ctypes.POINTER(IfFields), ctypes.c_int32, ctypes.c_char_p,
                           ctypes.c_uint64, c_u64p], ctypes.c_int),
        "bg3_deserialize": ([vp, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_uint64,
                             ctypes.POINTER(IfFields)], ctypes.c_int),
        "bg3_get_desc": ([vp, ctypes.POINTER(NetDesc)], ctypes.c_int),
        "bg3_checkpoint_save": ([vp, ctypes.c_void_p, ctypes.c_uint64, c_u64p], ctypes.c_int),
        "bg3_checkpoint_load": ([vp, ctypes.c_void_p, ctypes.c_uint64], ctypes.c_int),
        "bg3_net_footprint": ([ctypes.POINTER(NetDesc)], ctypes.c_int64),
        "bg3_net_bytes": ([vp], ctypes.c_uint64),
        "bg3_upload_layout": ([vp, c_f32p, c_f32p, c_i32p], ctypes.c_int),
        "bg3_upload_synapses": ([vp, ctypes.POINTER(SynArrays), ctypes.c_uint64], ctypes.c_int),
        "bg3_set_type_constants": ([vp, ctypes.POINTER(TypeConstants)], ctypes.c_int),
        "bg3_upload_growth": ([vp, ctypes.POINTER(GrowthParams), c_f32p, c_f32p], ctypes.c_int),
        "bg3_push_noise": ([vp, c_f32p, ctypes.c_int64], ctypes.c_int),
        "bg3_noise_pending": ([vp, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "bg3_set_noise_mode": ([vp, ctypes.c_int32, ctypes.c_uint32], ctypes.c_int),
        "bg3_set_device": ([ctypes.c_int32], ctypes.c_int),
        "bg3_norm_create": ([ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.POINTER(vp)],
                            ctypes.c_int),
        "bg3_norm_fill": ([vp, c_f32p, ctypes.c_int64], ctypes.c_int),
        "bg3_norm_destroy": ([vp], None),
        "bg3_upload_weights": ([vp, c_f32p], ctypes.c_int),
        "bg3_scale_weights": ([vp, ctypes.c_float], ctypes.c_int),
        "bg3_input_regular": ([vp, c_f32p, c_i32p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32],
                              ctypes.c_int),
        "bg3_input_poisson": ([vp, ctypes.POINTER(PoissonArrays), ctypes.c_float, ctypes.c_uint32,
                               ctypes.c_uint64], ctypes.c_int),
        "bg3_push_poisson_isis": ([vp, c_i32p, c_i32p], ctypes.c_int),
        "bg3_download_poisson": ([vp, ctypes.POINTER(PoissonArrays)], ctypes.c_int),
        "bg3_step": ([vp, ctypes.c_int64], ctypes.c_int),
        "bg3_epoch_growth": ([vp, ctypes.c_int32], ctypes.c_int),
        "bg3_sync": ([vp], ctypes.c_int),
        "bg3_get_step": ([vp, c_u64p], ctypes.c_int),
        "bg3_error_word": ([vp, c_u32p], ctypes.c_int),
        "bg3_download_lif": ([vp, ctypes.POINTER(LifArrays)], ctypes.c_int),
        "bg3_download_synapses": ([vp, ctypes.POINTER(SynArrays)], ctypes.c_int),
        "bg3_total_synapses": ([vp], ctypes.c_int64),
        "bg3_download_maps": ([vp, ctypes.POINTER(IndexMaps)], ctypes.c_int),
        "bg3_download_growth": ([vp, c_f32p, c_f32p], ctypes.c_int),
        "bg3_download_state": ([vp, ctypes.POINTER(StateView)], ctypes.c_int),
        "bg3_download_histories": ([vp, c_f32p, c_f32p, c_f32p, c_f32p], ctypes.c_int),
        "bg3_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "bg3_enable_timing": ([vp, ctypes.c_int], ctypes.c_int),
        "bg3_bench_steps": ([vp, ctypes.c_int64, ctypes.c_int64, c_f32p, c_f32p], ctypes.c_int),
        "bg3_batch_create": ([ctypes.POINTER(vp), ctypes.c_int32, ctypes.POINTER(vp)], ctypes.c_int),
        "bg3_batch_destroy": ([vp], ctypes.c_int),
        "bg3_batch_refresh": ([vp], ctypes.c_int),
        "bg3_batch_step": ([vp, ctypes.c_int64], ctypes.c_int),
        "bg3_batch_sync": ([vp], ctypes.c_int),
        "bg3_batch_launches": ([vp], ctypes.c_int64),
        "bg3_batch_bench_steps": ([vp, ctypes.c_int64, ctypes.c_int64, c_f32p], ctypes.c_int),
        "bg3_kernel_times": ([vp, c_f32p, c_f32p, c_f32p, ctypes.POINTER(ctypes.c_int64)],
                             ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _LIB = L
    return L


class Bg3Error(RuntimeError):
    pass


def check(rc, what=""):
    if rc != 0:
        msg = load().bg3_status_string(rc).decode()
        raise Bg3Error("%s failed: %s (%d)" % (what, msg, rc))


def ptr(a, ctype):
    if a is None:
        return ctypes.cast(None, ctypes.POINTER(ctype))
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctype))


_CT = {np.float32: ctypes.c_float, np.int32: ctypes.c_int32, np.uint32: ctypes.c_uint32,
       np.uint64: ctypes.c_uint64, np.uint8: ctypes.c_uint8}


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(_CT[a.dtype.type]))


LIF_FIELDS = [("Vm", np.float32), ("Vthresh", np.float32), ("Vreset", np.float32),
              ("I0", np.float32), ("Inoise", np.float32), ("C1", np.float32), ("C2", np.float32),
              ("Trefract", np.float32), ("summation", np.float32), ("nStepsInRefr", np.int32),
              ("spikeCount", np.int32), ("spikeCountOffset", np.int32)]
STDP_FIELDS = [("delayQueuePost", np.uint32), ("delayIdxPost", np.int32),
               ("total_delayPost", np.int32)] + [(k, np.float32) for k in STDP_FLOATS] + \
              [("useFroemkeDanSTDP", np.uint8)]
IZH_FIELDS = ("Aconst", "Bconst", "Cconst", "Dconst", "u", "C3")
SYN_FIELDS = [("in_use", np.uint8), ("src", np.int32), ("type", np.int32),
              ("delayIdx", np.int32), ("total_delay", np.int32), ("W", np.float32),
              ("psr", np.float32), ("decay", np.float32), ("tau", np.float32),
              ("delayQueue", np.uint32), ("U", np.float32), ("D", np.float32),
              ("F", np.float32), ("u", np.float32), ("r", np.float32), ("lastSpike", np.uint64)]


def footprint(desc):
    """Device bytes a network of this NetDesc holds (bg3_net_footprint; no GPU needed)."""
    v = int(load().bg3_net_footprint(ctypes.byref(desc)))
    if v < 0:
        check(v, "bg3_net_footprint")
    return v


def set_device(device):
    """bg3_set_device: the CUDA device of the networks created afterwards on this thread."""
    check(load().bg3_set_device(int(device)), "bg3_set_device")


class NormStream:
    """The reference's noise stream, Norm(mu, sigma, seed) (bg3_norm_*): take(n) returns the next
    n values; consecutive takes continue one stream.  Host only."""

    def __init__(self, seed, mu=0.0, sigma=1.0):
        self.L = load()
        h = ctypes.c_void_p()
        check(self.L.bg3_norm_create(int(seed) & 0xFFFFFFFF, mu, sigma, ctypes.byref(h)),
              "bg3_norm_create")
        self.h = h

    def take(self, n):
        out = np.empty(int(n), np.float32)
        check(self.L.bg3_norm_fill(self.h, _p(out) if n else None, int(n)), "bg3_norm_fill")
        return out

    def close(self):
        if getattr(self, "h", None):
            self.L.bg3_norm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Network:
    """One network on the GPU, driven through the C-ABI."""

    def __init__(self, n_neurons, max_syn, width, height, epoch_duration, delta_t=1e-4,
                 max_firing_rate=200, max_epochs=1, synapse_kind=BG3_SYN_DS,
                 noise_mode=BG3_NOISE_DEVICE, noise_seed=1, neuron_kind=BG3_NEURON_LIF):
        self.L = load()
        self.desc = NetDesc(n_neurons, max_syn, width, height, epoch_duration, delta_t,
                            max_firing_rate, max_epochs, neuron_kind, synapse_kind, noise_mode,
                            noise_seed)
        self.N, self.max_syn = n_neurons, max_syn
        self.max_spikes = int(np.float32(epoch_duration) * np.float32(max_firing_rate))
        self.max_epochs = max_epochs
        self.epoch_duration = epoch_duration
        h = ctypes.c_void_p()
        check(self.L.bg3_create(ctypes.byref(self.desc), ctypes.byref(h)), "bg3_create")
        self.h = h
        self._owned = True

    @classmethod
    def from_desc(cls, desc):
        """A new network of the same shape as desc (a NetDesc)."""
        d = desc
        return cls(d.n_neurons, d.max_syn_per_neuron, d.width, d.height, d.epoch_duration,
                   d.delta_t, d.max_firing_rate, d.max_epochs, d.synapse_kind, d.noise_mode,
                   d.noise_seed, neuron_kind=d.neuron_kind)

    @classmethod
    def borrow(cls, handle, desc):
        """Wraps a bg3_net* created elsewhere (e.g. by the job server); close() leaves it."""
        self = cls.__new__(cls)
        self.L = load()
        self.desc = desc
        self.N, self.max_syn = desc.n_neurons, desc.max_syn_per_neuron
        self.max_spikes = int(np.float32(desc.epoch_duration) * np.float32(desc.max_firing_rate))
        self.max_epochs = desc.max_epochs
        self.epoch_duration = desc.epoch_duration
        self.h = ctypes.c_void_p(handle)
        self._owned = False
        return self

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                self.L.bg3_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # uploads
    def upload_lif(self, **arrs):
        keep = {}
        s = LifArrays()
        for k, dt in LIF_FIELDS:
            if k in arrs and arrs[k] is not None:
                keep[k] = np.ascontiguousarray(arrs[k], dtype=dt)
                setattr(s, k, _p(keep[k]))
        if arrs.get("history") is not None:
            keep["history"] = np.ascontiguousarray(arrs["history"], dtype=np.uint64)
            s.history = _p(keep["history"])
        check(self.L.bg3_upload_lif(self.h, ctypes.byref(s)), "bg3_upload_lif")

    def upload_izh(self, **arrs):
        """Izhikevich arrays Aconst, Bconst, Cconst, Dconst, u, C3 (all required)."""
        keep = {k: np.ascontiguousarray(arrs[k], dtype=np.float32) for k in IZH_FIELDS}
        s = IzhArrays(*[_p(keep[k]) for k in IZH_FIELDS])
        check(self.L.bg3_upload_izh(self.h, ctypes.byref(s)), "bg3_upload_izh")

    def download_izh(self):
        out = {k: np.zeros(self.N, np.float32) for k in IZH_FIELDS}
        s = IzhArrays(*[_p(out[k]) for k in IZH_FIELDS])
        check(self.L.bg3_download_izh(self.h, ctypes.byref(s)), "bg3_download_izh")
        return out

    def upload_stdp(self, in_use, type, delayIdx, **arrs):
        """STDP fields of the slots (reference layout); in_use, type and delayIdx as uploaded."""
        keep = {"in_use": np.ascontiguousarray(in_use, np.uint8),
                "type": np.ascontiguousarray(type, np.int32),
                "delayIdx": np.ascontiguousarray(delayIdx, np.int32)}
        syn = SynArrays()
        for k in keep:
            setattr(syn, k, _p(keep[k]))
        st = StdpArrays()
        for k, dt in STDP_FIELDS:
            keep["s_" + k] = np.ascontiguousarray(arrs[k], dt)
            setattr(st, k, _p(keep["s_" + k]))
        check(self.L.bg3_upload_stdp(self.h, ctypes.byref(syn), ctypes.byref(st)), "bg3_upload_stdp")

    def download_stdp(self):
        S = self.N * self.max_syn
        out = {k: np.zeros(S, dt) for k, dt in STDP_FIELDS}
        st = StdpArrays()
        for k, _ in STDP_FIELDS:
            setattr(st, k, _p(out[k]))
        check(self.L.bg3_download_stdp(self.h, ctypes.byref(st)), "bg3_download_stdp")
        return out

    def set_stdp_constants(self, **per_type):
        """Per-type (II, IE, EI, EE) constants: each keyword a scalar or 4 values."""
        c = StdpConstants()
        for k, _ in StdpConstants._fields_:
            v = np.broadcast_to(np.asarray(per_type[k]), (4,))
            getattr(c, k)[:] = [float(x) if k != "useFroemkeDanSTDP" else int(x) for x in v]
        check(self.L.bg3_set_stdp_constants(self.h, ctypes.byref(c)), "bg3_set_stdp_constants")

    def set_stdp_arithmetic(self, mode):
        check(self.L.bg3_set_stdp_arithmetic(self.h, int(mode)), "bg3_set_stdp_arithmetic")

    def upload_layout(self, xloc, yloc, ntype):
        x = np.ascontiguousarray(xloc, np.float32)
        y = np.ascontiguousarray(yloc, np.float32)
        t = np.ascontiguousarray(ntype, np.int32)
        check(self.L.bg3_upload_layout(self.h, _p(x), _p(y), _p(t)), "bg3_upload_layout")

    def upload_synapses(self, step, counts=None, **arrs):
        keep = {}
        s = SynArrays()
        for k, dt in SYN_FIELDS:
            if k in arrs and arrs[k] is not None:
                keep[k] = np.ascontiguousarray(arrs[k], dtype=dt)
                setattr(s, k, _p(keep[k]))
        if counts is not None:
            keep["counts"] = np.ascontiguousarray(counts, np.uint32)
            s.counts = _p(keep["counts"])
        check(self.L.bg3_upload_synapses(self.h, ctypes.byref(s), int(step)),
              "bg3_upload_synapses")

    def upload_growth(self, epsilon, beta, rho, target_rate, min_radius, start_radius, radii,
                      rates=None):
        g = GrowthParams(epsilon, beta, rho, target_rate, min_radius, start_radius,
                         np.float32(target_rate) / np.float32(epsilon))
        r = np.ascontiguousarray(radii, np.float32)
        q = np.ascontiguousarray(rates if rates is not None else np.zeros(self.N), np.float32)
        check(self.L.bg3_upload_growth(self.h, ctypes.byref(g), _p(r), _p(q)), "bg3_upload_growth")

    def upload_weights(self, W):
        w = np.ascontiguousarray(W, np.float32)
        assert w.size == self.N * self.max_syn
        check(self.L.bg3_upload_weights(self.h, _p(w)), "bg3_upload_weights")

    def input_regular(self, values, shifts, n_steps_duration, n_steps_cycle, steps_in_cycle=0):
        v = np.ascontiguousarray(values, np.float32)
        sh = np.ascontiguousarray(shifts, np.int32)
        check(self.L.bg3_input_regular(self.h, _p(v), _p(sh), int(n_steps_duration),
                                       int(n_steps_cycle), int(steps_in_cycle)),
              "bg3_input_regular")

    def input_poisson(self, lam, seed=0, step=0, **arrs):
        keep = {}
        s = PoissonArrays()
        for k, dt in POISSON_FIELDS:
            if arrs.get(k) is not None:
                keep[k] = np.ascontiguousarray(arrs[k], dtype=dt)
                setattr(s, k, _p(keep[k]))
        check(self.L.bg3_input_poisson(self.h, ctypes.byref(s), float(lam), int(seed), int(step)),
              "bg3_input_poisson")

    def push_poisson_isis(self, begin, isis):
        b = np.ascontiguousarray(begin, np.int32)
        v = np.ascontiguousarray(isis if len(isis) else np.zeros(1), np.int32)
        check(self.L.bg3_push_poisson_isis(self.h, _p(b), _p(v)), "bg3_push_poisson_isis")

    def download_poisson(self):
        out = {k: np.zeros(self.N, dt) for k, dt in POISSON_FIELDS}
        s = PoissonArrays(*[_p(out[k]) for k, _ in POISSON_FIELDS])
        check(self.L.bg3_download_poisson(self.h, ctypes.byref(s)), "bg3_download_poisson")
        return out

    def scale_weights(self, factor):
        """W *= factor for every in-use synapse, on the device (bg3_scale_weights)."""
        check(self.L.bg3_scale_weights(self.h, float(factor)), "bg3_scale_weights")

    def set_noise_mode(self, mode, seed):
        check(self.L.bg3_set_noise_mode(self.h, int(mode), int(seed) & 0xFFFFFFFF),
              "bg3_set_noise_mode")
        self.desc.noise_mode, self.desc.noise_seed = int(mode), int(seed) & 0xFFFFFFFF

    def push_noise(self, values):
        v = np.ascontiguousarray(values, np.float32)
        check(self.L.bg3_push_noise(self.h, _p(v), len(v)), "bg3_push_noise")

    def noise_pending(self):
        """Injected noise values pushed and not yet consumed."""
        v = ctypes.c_int64()
        check(self.L.bg3_noise_pending(self.h, ctypes.byref(v)), "bg3_noise_pending")
        return v.value

    # hot path
    def step(self, n=1):
        check(self.L.bg3_step(self.h, int(n)), "bg3_step")

    def growth(self, epoch):
        check(self.L.bg3_epoch_growth(self.h, int(epoch)), "bg3_epoch_growth")

    # launch configuration
    @property
    def launch(self):
        c = LaunchCfg()
        check(self.L.bg3_get_launch(self.h, ctypes.byref(c)), "bg3_get_launch")
        return c.as_dict()

    def set_launch(self, **kw):
        c = LaunchCfg(**dict(self.launch, **kw))
        check(self.L.bg3_set_launch(self.h, ctypes.byref(c)), "bg3_set_launch")

    def autotune(self, steps_per_trial=200, growth=False):
        """Times launch configurations on this network's state (left unchanged) and keeps the
        fastest; returns (config dict, ms per step)."""
        c, ms = LaunchCfg(), ctypes.c_float()
        check(self.L.bg3_autotune(self.h, int(steps_per_trial), 1 if growth else 0,
                                  ctypes.byref(c), ctypes.byref(ms)), "bg3_autotune")
        return c.as_dict(), ms.value

    @property
    def device_bytes(self):
        return int(self.L.bg3_net_bytes(self.h))

    def checkpoint(self):
        """The network's whole state (bg3_checkpoint_save) as a numpy uint8 array."""
        n = ctypes.c_uint64()
        check(self.L.bg3_checkpoint_save(self.h, None, 0, ctypes.byref(n)), "bg3_checkpoint_save")
        buf = np.empty(n.value, np.uint8)
        check(self.L.bg3_checkpoint_save(self.h, buf.ctypes.data, buf.size, ctypes.byref(n)),
              "bg3_checkpoint_save")
        return buf

    def load_checkpoint(self, buf):
        b = np.ascontiguousarray(np.frombuffer(buf, np.uint8))
        check(self.L.bg3_checkpoint_load(self.h, b.ctypes.data, b.size), "bg3_checkpoint_load")

    def serialize(self, growth=True, **if_fields):
        """The reference's checkpoint stream (bg3_serialize) as bytes; if_fields gives the IF
        neuron arrays the library does not keep (Cm, Rm, Vrest, Vinit, Iinject, Isyn, Tau)."""
        keep = {k: np.ascontiguousarray(v, np.float32) for k, v in if_fields.items()}
        f = IfFields(*[_p(keep[k]) if k in keep else None for k in IF_FIELDS])
        conn = BG3_CONN_GROWTH if growth else BG3_CONN_STATIC
        n = ctypes.c_uint64()
        check(self.L.bg3_serialize(self.h, ctypes.byref(f), conn, None, 0, ctypes.byref(n)),
              "bg3_serialize")
        buf = ctypes.create_string_buffer(max(n.value, 1))
        check(self.L.bg3_serialize(self.h, ctypes.byref(f), conn, buf, n.value, ctypes.byref(n)),
              "bg3_serialize")
        return buf.raw[:n.value]

    def deserialize(self, data, growth=True, step=0):
        """Loads a reference checkpoint stream (bg3_deserialize); returns the IF arrays it held
        that the library does not keep."""
        out = {k: np.zeros(self.N, np.float32) for k in IF_FIELDS}
        f = IfFields(*[_p(out[k]) for k in IF_FIELDS])
        conn = BG3_CONN_GROWTH if growth else BG3_CONN_STATIC
        check(self.L.bg3_deserialize(self.h, bytes(data), len(data), conn, int(step),
                                     ctypes.byref(f)), "bg3_deserialize")
        return out

    def record(self):
        """Epoch end of a network without growth (recorder histograms, spike-count roll)."""
        check(self.L.bg3_epoch_record(self.h), "bg3_epoch_record")

    def sync(self):
        check(self.L.bg3_sync(self.h), "bg3_sync")

    # downloads
    @property
    def sim_step(self):
        v = ctypes.c_uint64()
        check(self.L.bg3_get_step(self.h, ctypes.byref(v)), "bg3_get_step")
        return v.value

    @property
    def error_word(self):
        v = ctypes.c_uint32()
        check(self.L.bg3_error_word(self.h, ctypes.byref(v)), "bg3_error_word")
        return v.value

    def download_lif(self, fields=None, out=None):
        """Neuron state; fields limits the copy to the named arrays (plus 'history'), out may
        supply destination arrays (e.g. pinned host buffers)."""
        want = [k for k, _ in LIF_FIELDS] + ["history"] if fields is None else list(fields)
        res = dict(out or {})
        for k, dt in LIF_FIELDS:
            if k in want and k not in res:
                res[k] = np.zeros(self.N, dt)
        if "history" in want and "history" not in res:
            res["history"] = np.zeros(self.N * self.max_spikes, np.uint64)
        out = res
        s = LifArrays()
        for k, _ in LIF_FIELDS:
            if k in out:
                setattr(s, k, _p(out[k]))
        if "history" in out:
            s.history = _p(out["history"])
        check(self.L.bg3_download_lif(self.h, ctypes.byref(s)), "bg3_download_lif")
        return out

    def download_synapses(self):
        S = self.N * self.max_syn
        out = {k: np.zeros(S, dt) for k, dt in SYN_FIELDS}
        out["counts"] = np.zeros(self.N, np.uint32)
        s = SynArrays()
        for k, _ in SYN_FIELDS:
            setattr(s, k, _p(out[k]))
        s.counts = _p(out["counts"])
        check(self.L.bg3_download_synapses(self.h, ctypes.byref(s)), "bg3_download_synapses")
        return out

    def total_synapses(self):
        v = self.L.bg3_total_synapses(self.h)
        if v < 0:
            check(int(v), "bg3_total_synapses")
        return int(v)

    def download_maps(self):
        T = self.total_synapses()
        out = {k: np.zeros(max(T, 1) if k.endswith("IndexMap") else self.N, np.uint32)
               for k, _ in IndexMaps._fields_}
        m = IndexMaps(*[_p(out[k]) for k, _ in IndexMaps._fields_])
        check(self.L.bg3_download_maps(self.h, ctypes.byref(m)), "bg3_download_maps")
        for k in out:
            if k.endswith("IndexMap"):
                out[k] = out[k][:T]
        return out

    def download_state(self, izh=False, stdp=False):
        """Everything bg3_download_state returns, in one call: dict with 'neurons', 'synapses',
        'maps', 'radii', 'rates' (and 'izh', 'stdp' when asked)."""
        S, T = self.N * self.max_syn, self.total_synapses()
        out = {"neurons": {k: np.zeros(self.N, dt) for k, dt in LIF_FIELDS},
               "synapses": {k: np.zeros(S, dt) for k, dt in SYN_FIELDS},
               "maps": {k: np.zeros(max(T, 1) if k.endswith("IndexMap") else self.N, np.uint32)
                        for k, _ in IndexMaps._fields_},
               "radii": np.zeros(self.N, np.float32), "rates": np.zeros(self.N, np.float32)}
        out["neurons"]["history"] = np.zeros(self.N * self.max_spikes, np.uint64)
        out["synapses"]["counts"] = np.zeros(self.N, np.uint32)
        la = LifArrays(*[_p(out["neurons"][k]) for k, _ in LIF_FIELDS] +
                       [_p(out["neurons"]["history"])])
        sa = SynArrays()
        for k in out["synapses"]:
            setattr(sa, k, _p(out["synapses"][k]))
        ma = IndexMaps(*[_p(out["maps"][k]) for k, _ in IndexMaps._fields_])
        v = StateView(ctypes.pointer(la), None, ctypes.pointer(sa), None, ctypes.pointer(ma),
                      _p(out["radii"]), _p(out["rates"]))
        if izh:
            out["izh"] = {k: np.zeros(self.N, np.float32) for k in IZH_FIELDS}
            ia = IzhArrays(*[_p(out["izh"][k]) for k in IZH_FIELDS])
            v.izh = ctypes.pointer(ia)
        if stdp:
            out["stdp"] = {k: np.zeros(S, dt) for k, dt in STDP_FIELDS}
            st = StdpArrays()
            for k, _ in STDP_FIELDS:
                setattr(st, k, _p(out["stdp"][k]))
            v.stdp = ctypes.pointer(st)
        check(self.L.bg3_download_state(self.h, ctypes.byref(v)), "bg3_download_state")
        for k in out["maps"]:
            if k.endswith("IndexMap"):
                out["maps"][k] = out["maps"][k][:T]
        return out

    def download_growth(self):
        r = np.zeros(self.N, np.float32)
        q = np.zeros(self.N, np.float32)
        check(self.L.bg3_download_growth(self.h, _p(r), _p(q)), "bg3_download_growth")
        return r, q

    def download_histories(self):
        nb = int(np.float32(self.max_epochs) * np.float32(self.epoch_duration))
        ns = int(np.float32(self.max_epochs) * np.float32(self.epoch_duration) * np.float32(100))
        b = np.zeros(max(nb, 1), np.float32)
        s = np.zeros(max(ns, 1), np.float32)
        rh = np.zeros((self.max_epochs + 1) * self.N, np.float32)
        ra = np.zeros((self.max_epochs + 1) * self.N, np.float32)
        check(self.L.bg3_download_histories(self.h, _p(b), _p(s), _p(rh), _p(ra)),
              "bg3_download_histories")
        return b[:nb], s[:ns], rh, ra

    def bench_steps(self, nsteps, flush_bytes=0, per_kernel=False):
        """Device time (ms) of each of nsteps steps; with per_kernel also (nsteps, 3) kernel
        times (neurons, fan-out, sweep)."""
        ms = np.zeros(max(int(nsteps), 1), np.float32)
        km = np.zeros(3 * max(int(nsteps), 1), np.float32) if per_kernel else None
        check(self.L.bg3_bench_steps(self.h, int(nsteps), int(flush_bytes), _p(ms), _p(km)),
              "bg3_bench_steps")
        return (ms[:nsteps], km[:3 * nsteps].reshape(-1, 3)) if per_kernel else ms[:nsteps]

    def enable_timing(self, on=True):
        check(self.L.bg3_enable_timing(self.h, 1 if on else 0), "bg3_enable_timing")

    @property
    def launches(self):
        """Kernels this network has launched so far (bg3_kernel_times)."""
        return self.kernel_times()[3]

    def kernel_times(self):
        a, b, c = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        n = ctypes.c_int64()
        check(self.L.bg3_kernel_times(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                      ctypes.byref(n)), "bg3_kernel_times")
        return a.value, b.value, c.value, n.value


class Batch:
    """Several Networks advanced together, one launch per kernel per step (bg3_batch_*)."""

    def __init__(self, nets):
        self.L = load()
        self.nets = list(nets)
        arr = (ctypes.c_void_p * len(self.nets))(*[n.h.value for n in self.nets])
        h = ctypes.c_void_p()
        check(self.L.bg3_batch_create(arr, len(self.nets), ctypes.byref(h)), "bg3_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.bg3_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def refresh(self):
        check(self.L.bg3_batch_refresh(self.h), "bg3_batch_refresh")

    def step(self, n=1):
        check(self.L.bg3_batch_step(self.h, int(n)), "bg3_batch_step")

    def sync(self):
        check(self.L.bg3_batch_sync(self.h), "bg3_batch_sync")

    @property
    def launches(self):
        return int(self.L.bg3_batch_launches(self.h))

    @property
    def launch(self):
        c = LaunchCfg()
        check(self.L.bg3_batch_get_launch(self.h, ctypes.byref(c)), "bg3_batch_get_launch")
        return c.as_dict()

    def set_launch(self, **kw):
        c = LaunchCfg(**dict(self.launch, **kw))
        check(self.L.bg3_batch_set_launch(self.h, ctypes.byref(c)), "bg3_batch_set_launch")

    def autotune(self, steps_per_trial=100):
        """Times launch configurations on the members' state (left unchanged); keeps the fastest."""
        c, ms = LaunchCfg(), ctypes.c_float()
        check(self.L.bg3_batch_autotune(self.h, int(steps_per_trial), ctypes.byref(c),
                                        ctypes.byref(ms)), "bg3_batch_autotune")
        return c.as_dict(), ms.value

    def bench_steps(self, nsteps, flush_bytes=0):
        ms = np.zeros(max(int(nsteps), 1), np.float32)
        check(self.L.bg3_batch_bench_steps(self.h, int(nsteps), int(flush_bytes), _p(ms)),
              "bg3_batch_bench_steps")
        return ms[:nsteps]


def selftest_binary64(samples=1 << 26, seed=1):
    """(add, multiply, conversion mismatches, out-of-range cases) of the integer-pipe binary64
    arithmetic against the hardware."""
    c = (ctypes.c_uint64 * 4)()
    check(load().bg3_selftest_binary64(int(samples), int(seed), c), "bg3_selftest_binary64")
    return tuple(int(x) for x in c)


def selftest_izhikevich(samples=1 << 26, seed=1):
    """(integer-pipe mismatches, float-float mismatches, float-float values handed to the FP64
    pipe, operand sets outside the integer pipe's range) of the Izhikevich update's double
    expression against the FP64 pipe."""
    c = (ctypes.c_uint64 * 4)()
    check(load().bg3_selftest_izhikevich(int(samples), int(seed), c), "bg3_selftest_izhikevich")
    return tuple(int(x) for x in c)
