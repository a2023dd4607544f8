"""The C-ABI library builds, loads without a GPU and exports every symbol include/bg3.h declares."""
import ctypes
import os
import re
import subprocess

from braingrid_gb300 import build as bgbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(bg3_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_loads_and_exports_all_declared_symbols():
    path = bgbuild.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (bg3_[a-z0-9_]+)$", out, flags=re.M))
    assert names <= exported


def test_status_strings_without_gpu():
    lib = ctypes.CDLL(bgbuild.build())
    lib.bg3_status_string.restype = ctypes.c_char_p
    assert lib.bg3_status_string(0) == b"ok"
    assert b"invalid" in lib.bg3_status_string(-1)


def test_hot_kernels_do_not_spill():
    """The per-step kernels of the default configuration keep everything in registers (a spill in
    the fused 32-dest sweep once cost the 10,000-neuron network 10 % of its step time): ptxas's report of the last
    build for the single-network TMA sweep with the fused neuron pass (32-dest tiles, every
    pipeline depth), the thin sweeps and the spiking / DS delivery.  (The 16-dest and unfused
    sweep variants, and the batched STDP passes, spill a few bytes and are not held to this.)"""
    bgbuild.build()
    rep = bgbuild.ptxas_report("bg3_step.cu")
    hot = {k: v for k, v in rep.items()
           if k.startswith(("_ZN3bg37k_sweepILi1ELb1ELi4ELi32E", "_ZN3bg37k_sweepILi1ELb1ELi6ELi32E",
                            "_ZN3bg37k_sweepILi1ELb1ELi8ELi32E", "_ZN3bg312k_sweep_thin",
                            "_ZN3bg39k_deliverILi0E", "_ZN3bg39k_deliverILi1E",
                            "_ZN3bg315k_deliver_batchILi0E", "_ZN3bg315k_deliver_batchILi1E"))}
    assert len(hot) == 9, sorted(rep)
    spilling = {k: v for k, v in hot.items() if v[1] or v[2]}
    assert not spilling, spilling


def test_serve_desc_validation_without_a_gpu():
    """bg3_serve_create checks its descriptor on the host (no device call): an admission order
    other than arrival (0) or least work (1), a negative bypass bound and a zero chunk are refused;
    a valid descriptor makes a server that an empty destroy frees."""
    from braingrid_gb300 import serve
    lib = serve._bind()
    ok = dict(hbm_budget_bytes=1 << 30, max_resident=4, chunk_steps=100, max_resident_slots=0,
              max_bypass=8, order=serve.ORDER_LEAST_WORK)
    h = ctypes.c_void_p()
    assert lib.bg3_serve_create(ctypes.byref(serve.ServeDesc(**ok)), ctypes.byref(h)) == 0
    assert lib.bg3_serve_destroy(h) == 0
    for bad in (dict(order=2), dict(order=-1), dict(max_bypass=-1), dict(chunk_steps=0),
                dict(max_resident=0)):
        d = serve.ServeDesc(**dict(ok, **bad))
        h = ctypes.c_void_p()
        assert lib.bg3_serve_create(ctypes.byref(d), ctypes.byref(h)) != 0, bad
