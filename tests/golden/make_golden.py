"""Generate the committed parity fixtures in tests/golden/ from the compiled reference.

Run in a checkout that has the reference sources (the tree oracle/ref.mk resolves, or --ref):

    python tests/golden/make_golden.py [--ref PATH]

It (1) writes the network configs and NLists under tests/golden/configs/, (2) builds the
reference single-threaded simulator and oracle/ref_harness.cpp with oracle/ref.mk, (3) runs the
harness on each case, and (4) keeps a compact subset of each dump as tests/golden/<case>.npz.
The reference's own CPU golden outputs for test-tiny and test-small
(old/validation/4-2016/growth/test-{tiny,small}-out.xml) are parsed into ref_goldens.npz, and the
reference's checkpoint stream at the end of a few cases (Simulator::serialize) goes to
serialize.npz (--only-serialize rewrites that file alone), and the reference driver's result
files of whole runs (OUTPUT_CASES in configs.py) go to outputs.npz (--only-outputs).

Nothing at test time reads the reference tree: the tests only read the .npz files written here.
"""
import argparse
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.refdump import read_dump  # noqa: E402
from tests.golden.configs import (CASES, OUTPUT_CASES, list_texts, output_case,  # noqa: E402
                                  write_config_tree)


def build_reference(ref, fp64=False):
    target = ["fp64"] if fp64 else []
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref.mk"),
                           "REF=" + ref, "-j8"] + target, cwd=ROOT)
    return os.path.join(ROOT, "oracle", "_ref64" if fp64 else "_ref", "bg_ref_harness")


def run_harness(harness, workdir, cfg, args, out, serialize=None):
    cmd = [harness, "-t", cfg, "-o", out] + args
    if serialize:
        cmd += ["--serialize", serialize]
    subprocess.check_call(cmd, cwd=workdir, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return read_dump(out)


# cases whose end-of-run checkpoint stream (Simulator::serialize) is kept in serialize.npz
SERIALIZE_CASES = ("c0_grown", "c0_spiking", "c0_stdp", "izh_dstdp", "izh_static", "ragged", "ragged_izh")


def run_outputs(growth, work, ref):
    """The reference driver's result file for each OUTPUT_CASES entry, run from the same
    parameter files the product reads (the reference's own test-tiny and test-small results must
    come out equal to its committed goldens)."""
    out = {}
    d = os.path.join(work, "configfiles", "bg3")
    os.makedirs(d, exist_ok=True)
    os.makedirs(os.path.join(work, "results"), exist_ok=True)
    for name in OUTPUT_CASES:
        c, text, stim = output_case(name)
        cfg = os.path.join(d, "out_%s.xml" % name)
        with open(cfg, "w") as f:
            f.write(text.replace("results/%s-out.xml" % c["name"], "results/out_%s.xml" % name))
        active, inh = list_texts(c)
        for suffix, t in (("-active.xml", active), ("-inh.xml", inh)):
            with open(os.path.join(d, c["name"] + suffix), "w") as f:
                f.write(t)
        cmd = [growth, "-t", cfg]
        if stim:
            sp = os.path.join(d, "out_%s-stim.xml" % name)
            with open(sp, "w") as f:
                f.write(stim)
            cmd += ["-s", sp]
        subprocess.check_call(cmd, cwd=work, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        res = open(os.path.join(work, "results", "out_%s.xml" % name), "rb").read()
        out[name] = np.frombuffer(res, np.uint8)
        gold = {"ref_tiny": "test-tiny", "ref_small": "test-small"}.get(name)
        if gold:
            want = open(os.path.join(ref, "old/validation/4-2016/growth/%s-out.xml" % gold),
                        "rb").read()
            assert res == want, "%s: the driver's result differs from its golden" % name
    # the driver's -w and -r on c0: the end-of-run checkpoint stream, and a second run that
    # starts from it (its result file and its own end-of-run stream)
    res_dir = os.path.join(work, "results")
    cfg = os.path.join(d, "out_c0.xml")
    subprocess.check_call([growth, "-t", cfg, "-w", os.path.join(res_dir, "c0.ser")], cwd=work,
                          stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    cfg2 = os.path.join(d, "out_c0_resumed.xml")
    with open(cfg) as f, open(cfg2, "w") as g:
        g.write(f.read().replace("results/out_c0.xml", "results/out_c0_resumed.xml"))
    subprocess.check_call([growth, "-t", cfg2, "-r", os.path.join(res_dir, "c0.ser"), "-w",
                           os.path.join(res_dir, "c0_resumed.ser")], cwd=work,
                          stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    for key, fn in (("c0.ser", "c0.ser"), ("c0_resumed", "out_c0_resumed.xml"),
                    ("c0_resumed.ser", "c0_resumed.ser")):
        out[key] = np.frombuffer(open(os.path.join(res_dir, fn), "rb").read(), np.uint8)
    return out


def compact(d, keep_steps_every=None, syn_keep=None):
    """Select the records the tests use; spike rasters become (step, neuron) pairs."""
    out = {}
    for name, recs in d.items():
        if name.startswith(("n.",)):
            continue
        if name.startswith(("s.", "in.")):
            for step, a in recs:
                if keep_steps_every and step % keep_steps_every == 0:
                    out["%s@%d" % (name, step)] = a
            continue
        if name.endswith(("history",)) and name.split(".")[0] in ("pre",):
            # spike raster of each epoch from the history ring + counts
            pass
        for k, (step, a) in enumerate(recs):
            key = name if len(recs) == 1 else "%s#%d" % (name, k)
            out[key] = a
    # rasters per epoch from the pre-growth snapshots
    cnts = d.get("pre.spikeCount", [])
    offs = d.get("pre.spikeCountOffset", [])
    hist = d.get("pre.history", [])
    ms = int(d["hdr"][0][1][4])
    N = int(d["hdr"][0][1][0])
    for k, ((_, c), (_, o), (_, h)) in enumerate(zip(cnts, offs, hist)):
        h = h.reshape(N, ms)
        steps, nrn = [], []
        for i in range(N):
            for j in range(int(c[i])):
                steps.append(int(h[i, (int(o[i]) + j) % ms]))
                nrn.append(i)
        order = np.lexsort((np.array(nrn), np.array(steps))) if steps else np.zeros(0, np.int64)
        out["raster#%d" % k] = np.stack([np.array(steps, np.int64)[order],
                                         np.array(nrn, np.int64)[order]]) if steps else \
            np.zeros((2, 0), np.int64)
    # drop the bulky per-epoch history rings; keep slot arrays only at in-use slots (their
    # indices are stored as <prefix>slots), and skip the post-growth synapse copy, which the
    # recorder step does not change
    S = N * int(d["hdr"][0][1][1])
    for key in list(out):
        if ".history" in key or (key.startswith("grow.") and out[key].size == S):
            del out[key]
        elif key.startswith("post.") and out[key].size == S and key.split("#")[0] not in (
                "post.in_use", "post.W", "post.src"):
            del out[key]
        elif syn_keep is not None and out[key].size != N and "#" in key \
                and key.startswith(("pre.", "grow.", "post.")) \
                and int(key.split("#")[1]) not in syn_keep:
            del out[key]
    for key in list(out):
        if key.endswith("in_use") or key.split("#")[0].endswith(".in_use"):
            pfx, _, idx = key.partition("in_use")
            mask = out.pop(key, None)
            if mask is None:
                continue
            mask = mask.astype(bool)
            out[pfx + "slots" + idx] = np.nonzero(mask)[0].astype(np.int64)
            for k2 in list(out):
                base, _, i2 = k2.partition("#")
                if k2 != key and base.startswith(pfx) and (("#" + i2) if i2 else "") == idx \
                        and out[k2].size == S and base.count(".") == pfx.count("."):
                    out[k2] = out[k2][mask]
    return out


def parse_xml_matrix(text, name):
    m = re.search(r'<Matrix name="%s"[^>]*rows="(\d+)" columns="(\d+)"[^>]*>(.*?)</Matrix>' % name,
                  text, re.S)
    rows, cols = int(m.group(1)), int(m.group(2))
    vals = np.array([float(v) for v in m.group(3).split()], dtype=np.float64)
    return vals.reshape(rows, cols)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None,
                    help="reference source tree (default: the one oracle/ref.mk resolves)")
    ap.add_argument("--cases", default="")
    ap.add_argument("--only-serialize", action="store_true",
                    help="write serialize.npz only (the other fixtures stay as they are)")
    ap.add_argument("--only-outputs", action="store_true",
                    help="write outputs.npz only (the reference driver's result files)")
    a = ap.parse_args()
    if a.ref is None:
        from oracle import pyoracle
        a.ref = pyoracle.reference_tree()
        if a.ref is None:
            sys.exit("no reference source tree: set BRAINGRID_REF or pass --ref")
    harness = build_reference(a.ref)
    if a.only_outputs:
        work = tempfile.mkdtemp(prefix="bg_golden_")
        try:
            out = run_outputs(os.path.join(os.path.dirname(harness), "growth"), work, a.ref)
            np.savez_compressed(os.path.join(HERE, "outputs.npz"), **out)
            print("wrote outputs", sorted(out))
        finally:
            shutil.rmtree(work, ignore_errors=True)
        return
    harness64 = build_reference(a.ref, fp64=True)
    work = tempfile.mkdtemp(prefix="bg_golden_")
    try:
        cfgdir = os.path.join(work, "configfiles")
        shutil.copytree(os.path.join(a.ref, "configfiles"), cfgdir)
        write_config_tree(cfgdir)
        os.makedirs(os.path.join(work, "results"), exist_ok=True)
        ser = {}
        for case in ([] if a.cases else CASES):  # --cases: those fixtures alone
            if case["name"] in SERIALIZE_CASES:
                path = os.path.join(work, case["name"] + ".ser")
                run_harness(harness, work, case["config"], case["args"],
                            os.path.join(work, case["name"] + ".sbin"), serialize=path)
                ser[case["name"]] = np.frombuffer(open(path, "rb").read(), np.uint8)
        if ser:
            np.savez_compressed(os.path.join(HERE, "serialize.npz"), **ser)
            print("wrote serialize", sorted(ser))
        if a.only_serialize:
            return
        selected = [c for c in CASES if not a.cases or c["name"] in a.cases.split(",")]
        for case in selected:
            h = harness64 if case.get("fp64") else harness
            d = run_harness(h, work, case["config"], case["args"],
                            os.path.join(work, case["name"] + ".bin"))
            out = compact(d, case.get("keep_steps_every"), case.get("syn_keep"))
            if case.get("fp64") and case["name"] != "c0_fp64":
                # long-run comparison bases: the growth state after every epoch and the rasters
                out = {k: v for k, v in out.items()
                       if k.startswith(("post.rates", "post.radii", "raster#"))}
            np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
            print("wrote", case["name"], len(out), "arrays")
        if a.cases:
            return
        # the reference's own CPU goldens
        g = {}
        for nm in ("test-tiny", "test-small"):
            txt = open(os.path.join(a.ref, "old/validation/4-2016/growth/%s-out.xml" % nm)).read()
            for mat in ("radiiHistory", "ratesHistory", "burstinessHist", "spikesHistory"):
                g["%s.%s" % (nm, mat)] = parse_xml_matrix(txt, mat)
        np.savez_compressed(os.path.join(HERE, "ref_goldens.npz"), **g)
        print("wrote ref_goldens")
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
