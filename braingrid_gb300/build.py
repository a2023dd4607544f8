"""In-tree build of libbg3.so (CUDA, sm_103a only) with nvcc.

    python -m braingrid_gb300.build          # or __graft_entry__.build()

Translation units compile in parallel; the shared library lands in braingrid_gb300/_build/.
The library is built with -fmad=false so that every a*b+c rounds twice, like the reference's
x86-64 float arithmetic; that is what makes the injected-noise mode bit-exact.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbg3.so")
ROOT = os.path.dirname(HERE)

SOURCES = ["bg3_step.cu", "bg3_growth.cu", "bg3_api.cu", "bg3_noalloc.cu", "bg3_serve.cu",
           "bg3_selftest.cu", "bg3_serialize.cu", "bg3_hostrng.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in ("bg3.h", "bg3_serve.h")]
    objs = []
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if _stale(obj, [src] + headers):
            # -Xptxas -v: ptxas's per-kernel registers and spills, kept beside the object
            # (ptxas_report) for the no-spill check of the hot kernels
            # the host noise generator's loops are vectorised at -O3 (host code only)
            host = ["-Xcompiler", "-O3"] if s == "bg3_hostrng.cu" else []
            jobs.append(([nvcc()] + ARCH + FLAGS + host + list(extra) +
                         ["-Xptxas", "-v", "-c", src, "-o", obj], obj + ".ptxas.txt"))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    def compile_one(job):
        cmd, report = job
        err = run(cmd)
        with open(report, "w") as f:
            f.write(err)
        return err

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for err in ex.map(compile_one, jobs):
            if verbose and err:
                print(err)
    if jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    return LIB


def ptxas_report(source="bg3_step.cu"):
    """{kernel (mangled name): (registers, spill store bytes, spill load bytes)} from the last
    compile of a source (build() keeps ptxas's -v output beside the object)."""
    import re
    path = os.path.join(BUILD, source.replace(".cu", ".o") + ".ptxas.txt")
    out, name = {}, None
    for line in open(path):
        m = re.search(r"Compiling entry function '([^']+)'", line)
        if m:
            name = m.group(1)
            continue
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", line)
        if m and name:
            out.setdefault(name, [0, 0, 0])[1:] = [int(m.group(1)), int(m.group(2))]
        m = re.search(r"Used (\d+) registers", line)
        if m and name:
            out.setdefault(name, [0, 0, 0])[0] = int(m.group(1))
    return {k: tuple(v) for k, v in out.items()}


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
