"""ctypes wrapper around the C oracle (oracle/bg_oracle.c) — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may import this module.
The product library (braingrid_gb300) never loads it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbgoracle.so")

_NP = {1: np.uint8, 4: None, 8: None}
# element type per array name (ambiguous sizes resolved by name)
_INT32 = {"ntype", "starter", "refr", "spikeCount", "spikeCountOffset", "src", "dest", "type",
          "total_delay", "delayIdx", "ldelayQueue", "reg_shift", "pois_nisi", "in_delay",
          "in_delayIdx", "delayIdxPost", "total_delayPost", "ldelayQueuePost"}
_UINT32 = {"queue", "counts", "inMap", "outMap", "inBegin", "inCount", "outBegin", "outCount",
           "in_queue", "queuePost"}
_UINT64 = {"history", "lastSpike", "in_last"}
_UINT8 = {"hasFired", "in_use", "pois_mask", "useFD"}

LIF_CONFIG0_RANGES = [13.5e-9, 13.5e-9, 1.0e-9, 1.5e-9, 15.0e-3, 15.0e-3, 0.0, 0.0,
                      13.5e-3, 13.5e-3, 13.0e-3, 13.0e-3, 13.565e-3, 13.655e-3, 13.0e-3, 13.0e-3]


def reference_tree():
    """The reference source tree the recipe oracle/ref.mk resolves (its REF, from the
    BRAINGRID_REF environment variable or the recipe's default), or None where it is absent (as on
    a machine that only runs the tests)."""
    r = subprocess.run(["make", "-s", "-f", os.path.join(HERE, "ref.mk"), "where"],
                       capture_output=True, text=True)
    path = r.stdout.strip()
    return path if r.returncode == 0 and path else None


def build(force=False):
    """Compile the oracle into oracle/_build/libbgoracle.so (host CPU, any architecture)."""
    src = os.path.join(HERE, "bg_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "bg_oracle.h"))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["cc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                           "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        vp, i, f, u32, u64, i64 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint32,
                                   ctypes.c_uint64, ctypes.c_int64)
        L.bgo_create.restype = vp
        L.bgo_create.argtypes = [i, i, i, i, f, f, i, i, i, i]
        L.bgo_destroy.argtypes = [vp]
        L.bgo_array.restype = vp
        L.bgo_array.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(i64), ctypes.POINTER(i)]
        L.bgo_get_step.restype = u64
        L.bgo_get_step.argtypes = [vp]
        L.bgo_set_step.argtypes = [vp, u64]
        L.bgo_total_synapses.restype = i64
        L.bgo_total_synapses.argtypes = [vp]
        L.bgo_layout_grid.argtypes = [vp]
        L.bgo_set_types.argtypes = [vp, ctypes.POINTER(i), i, ctypes.POINTER(i), i]
        L.bgo_create_lif.argtypes = [vp, ctypes.POINTER(f)]
        L.bgo_create_izh.argtypes = [vp, ctypes.POINTER(f), ctypes.POINTER(f)]
        L.bgo_growth_init.argtypes = [vp, f, f, f, f, f, f]
        L.bgo_seed_noise.argtypes = [vp, u32]
        L.bgo_rebuild_maps.restype = i
        L.bgo_rebuild_maps.argtypes = [vp]
        L.bgo_create_synapse.argtypes = [vp, i, i, i, f]
        L.bgo_record_noise.argtypes = [vp, i64]
        L.bgo_noise_recorded.restype = i64
        L.bgo_noise_recorded.argtypes = [vp]
        L.bgo_step.argtypes = [vp, i]
        L.bgo_growth.argtypes = [vp]
        L.bgo_record_epoch.argtypes = [vp, i]
        L.bgo_record_static.argtypes = [vp]
        L.bgo_flags.restype = i
        L.bgo_flags.argtypes = [vp]
        L.bgo_stdp_signed.argtypes = [vp, i]
        L.bgo_rng_skip.argtypes = [vp, i64]
        L.bgo_stdp_params.argtypes = [vp, ctypes.POINTER(f)]
        L.bgo_serialize.restype = i64
        L.bgo_serialize.argtypes = [vp, i, ctypes.c_char_p, i64]
        L.bgo_norm_fill.argtypes = [u32, ctypes.POINTER(f), i64]
        L.bgo_input_regular.argtypes = [vp, f, f, i, ctypes.POINTER(f)]
        L.bgo_input_regular.restype = i
        L.bgo_input_poisson.argtypes = [vp, f, f, ctypes.c_void_p]
        L.bgo_input_poisson.restype = i
        L.bgo_poisson_isi_draws.argtypes = [vp, i, ctypes.POINTER(ctypes.c_int32),
                                            ctypes.POINTER(ctypes.c_int32), i64]
        L.bgo_poisson_isi_draws.restype = i64
        _lib = L
    return _lib


def norm_stream(seed, n):
    """The first n values of the reference noise stream Norm(0, 1, seed) (RNG/Norm.cpp:59-86)."""
    out = np.empty(int(n), dtype=np.float32)
    lib().bgo_norm_fill(seed, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), int(n))
    return out


def _iarr(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class OracleNet:
    """One network in the C oracle; arrays are live numpy views of the C state."""

    def __init__(self, N, max_syn, width, height, epoch_duration, delta_t=1e-4,
                 max_firing_rate=200, max_epochs=1, neuron_kind=0, synapse_kind=1):
        self.L = lib()
        self.h = self.L.bgo_create(N, max_syn, width, height, epoch_duration, delta_t,
                                   max_firing_rate, max_epochs, neuron_kind, synapse_kind)
        self.N, self.max_syn = N, max_syn
        self.epoch_duration, self.delta_t = epoch_duration, delta_t
        self.max_epochs = max_epochs
        self.neuron_kind, self.synapse_kind = neuron_kind, synapse_kind

    def close(self):
        if self.h:
            self.L.bgo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def arr(self, name):
        cnt = ctypes.c_int64()
        esz = ctypes.c_int()
        p = self.L.bgo_array(self.h, name.encode(), ctypes.byref(cnt), ctypes.byref(esz))
        if not p or cnt.value == 0:
            return np.zeros(0, dtype=np.float32)
        if name in _INT32:
            dt = np.int32
        elif name in _UINT32:
            dt = np.uint32
        elif name in _UINT64:
            dt = np.uint64
        elif name in _UINT8:
            dt = np.uint8
        else:
            dt = np.float32
        assert np.dtype(dt).itemsize == esz.value, name
        buf = (ctypes.c_char * (cnt.value * esz.value)).from_address(p)
        return np.frombuffer(buf, dtype=dt)

    @property
    def step(self):
        return int(self.L.bgo_get_step(self.h))

    @step.setter
    def step(self, v):
        self.L.bgo_set_step(self.h, int(v))

    @property
    def total(self):
        return int(self.L.bgo_total_synapses(self.h))

    # setup
    def layout_grid(self):
        self.L.bgo_layout_grid(self.h)

    def set_types(self, inh, starters):
        a, pa = _iarr(inh)
        b, pb = _iarr(starters)
        self.L.bgo_set_types(self.h, pa, len(a), pb, len(b))

    def create_lif(self, ranges16=LIF_CONFIG0_RANGES):
        g = np.asarray(ranges16, dtype=np.float32)
        self.L.bgo_create_lif(self.h, g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    def create_izh(self, ranges16, izh16):
        g = np.asarray(ranges16, dtype=np.float32)
        z = np.asarray(izh16, dtype=np.float32)
        self.L.bgo_create_izh(self.h, g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                              z.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    def growth_init(self, epsilon, beta, rho, target_rate, min_radius, start_radius):
        self.L.bgo_growth_init(self.h, epsilon, beta, rho, target_rate, min_radius, start_radius)

    def seed_noise(self, seed):
        self.L.bgo_seed_noise(self.h, seed)

    def record_noise(self, cap):
        self.L.bgo_record_noise(self.h, int(cap))

    def rebuild_maps(self):
        return self.L.bgo_rebuild_maps(self.h)

    def create_synapse(self, dest, src, type_, W):
        self.L.bgo_create_synapse(self.h, dest, src, type_, W)

    # inputs (call input_regular before create_lif: with sync="no" it draws from the same rng)
    def input_regular(self, duration, interval, sync, values100):
        v = np.ascontiguousarray(values100, dtype=np.float32)
        mode = {"yes": 0, "no": 1, "wave": 2}[sync]
        assert self.L.bgo_input_regular(self.h, duration, interval, mode,
                                        v.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0

    def input_poisson(self, fr_mean, weight, masks=None):
        m = None
        if masks is not None:
            self._mask = np.zeros(self.N, np.uint8)
            self._mask[np.asarray(masks, dtype=np.int64)] = 1
            m = self._mask.ctypes.data
        assert self.L.bgo_input_poisson(self.h, fr_mean, weight, m) == 0

    def poisson_isi_draws(self, nsteps, cap=None):
        cap = cap or self.N * (nsteps // 5 + 4)
        begin = np.zeros(self.N + 1, np.int32)
        out = np.zeros(cap, np.int32)
        k = self.L.bgo_poisson_isi_draws(self.h, int(nsteps),
                                         begin.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), cap)
        assert k >= 0
        return begin, out[:k]

    # hot path
    def step_n(self, n):
        self.L.bgo_step(self.h, int(n))

    def growth(self):
        self.L.bgo_growth(self.h)

    def record_epoch(self, epoch):
        self.L.bgo_record_epoch(self.h, int(epoch))

    def record_static(self):
        """The recorder of a network without growth (XmlRecorder::compileHistories)."""
        self.L.bgo_record_static(self.h)

    def stdp_signed(self, on=True):
        """STDP arithmetic of the reference's device build (signed spike-time differences)."""
        self._signed = bool(on)
        self.L.bgo_stdp_signed(self.h, 1 if on else 0)

    def rng_skip(self, draws):
        self.L.bgo_rng_skip(self.h, int(draws))

    def serialize(self, conn_growth=True):
        """The reference's checkpoint stream (Model::serialize) of the current state, as bytes."""
        n = self.L.bgo_serialize(self.h, 1 if conn_growth else 0, None, 0)
        buf = ctypes.create_string_buffer(int(n))
        assert self.L.bgo_serialize(self.h, 1 if conn_growth else 0, buf, n) == n
        return buf.raw

    def stdp_params(self, p11):
        self._stdp = np.asarray(p11, dtype=np.float32)
        self.L.bgo_stdp_params(self.h, self._stdp.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    @property
    def flags(self):
        return int(self.L.bgo_flags(self.h))
