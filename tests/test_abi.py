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
