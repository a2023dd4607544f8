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
