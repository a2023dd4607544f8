"""The reference-side drop-in (braingrid_gb300/dropin/): the reference's own driver, compiled
unmodified with -DUSE_GPU, links against the drop-in and libbg3.so with no unresolved symbol and
none of the reference's CUDA code, and a run reaches the model's first C-ABI call.

Needs the reference's sources (the tree oracle/ref.mk resolves); skipped where they are absent.
Without a GPU the run stops at that first call (bg3_set_device), which is what this test checks:
the unchanged BGDriver parses the parameter file, creates the model through its USE_GPU branch
(Core/BGDriver.cpp:204-208) and hands control to the drop-in."""
import os
import re
import shutil
import subprocess

import pytest

from braingrid_gb300 import build as bgbuild
from oracle import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MK = os.path.join(ROOT, "braingrid_gb300", "dropin", "dropin.mk")
OUT = os.path.join(ROOT, "braingrid_gb300", "_build", "dropin")
EXE = os.path.join(OUT, "growth_bg3")


@pytest.fixture(scope="module")
def driver():
    ref = pyoracle.reference_tree()
    if ref is None:
        pytest.skip("the reference's sources are not on this machine")
    bgbuild.build()
    subprocess.check_call(["make", "-s", "-f", MK, "-j8"], cwd=ROOT)
    return ref


def test_unchanged_driver_links_with_no_unresolved_symbol(driver):
    assert os.path.exists(EXE)
    r = subprocess.run(["ldd", "-r", EXE], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "undefined symbol" not in r.stdout + r.stderr
    assert re.search(r"libbg3\.so => \S*_build/dropin/\.\./libbg3\.so", r.stdout), r.stdout


def test_no_reference_cuda_or_sample_code_is_linked(driver):
    objs = []
    for d, _, files in os.walk(os.path.join(OUT, "ref")):
        objs += [os.path.relpath(os.path.join(d, f), os.path.join(OUT, "ref")) for f in files]
    assert "Core/BGDriver.o" in objs and "Core/Model.o" in objs
    assert not [o for o in objs if o.endswith("_d.o") or "GPUSpikingModel" in o or
                "GpuSInput" in o or "MersenneTwister_d" in o or "HostSInput" in o], objs
    syms = subprocess.run(["nm", "-C", EXE], capture_output=True, text=True).stdout
    for name in ("normalMTGPU", "initMTGPU", "calcSummationMapDevice", "cudaMalloc"):
        assert name not in syms, name
    # the model and the device members of the classes come from the drop-in
    for name in ("GPUSpikingModel::advance", "AllLIFNeurons::advanceNeurons",
                 "AllDSSynapses::copySynapseHostToDevice", "ConnGrowth::updateSynapsesWeights",
                 "GpuSInputPoisson::init"):
        assert re.search(r" T %s\(" % re.escape(name), syms), name


def test_driver_reaches_the_drop_in(driver, tmp_path):
    shutil.copytree(os.path.join(driver, "configfiles"), str(tmp_path / "configfiles"))
    (tmp_path / "results").mkdir()
    r = subprocess.run([EXE, "-t", "configfiles/test-tiny.xml"], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=120)
    out = r.stdout + r.stderr
    assert "Setup simulation." in out
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        assert r.returncode == 0, out
    else:
        # no device: the model's first C-ABI call reports it and the driver exits as the
        # reference's HANDLE_ERROR does
        assert r.returncode != 0 and "bg3_set_device" in out, out


def _run_driver(tmp_path, text, name):
    cfg = tmp_path / "configfiles" / "bg3" / (name + ".xml")
    cfg.write_text(text)
    (tmp_path / "results").mkdir(exist_ok=True)
    r = subprocess.run([EXE, "-t", str(cfg.relative_to(tmp_path))], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=120)
    return r.returncode, r.stdout + r.stderr


def test_bg3params_stdp_constants_reach_the_drop_in(driver, tmp_path):
    """A parameter file carrying STDP constants in a root-level <BG3Params> (the Izhikevich +
    dynamic STDP + ConnStatic case): the reference's readers take the file, the drop-in reads the
    eleven constants before its first C-ABI call; STDP constants for a class without STDP, and a
    <ParameterDraw> other than ranges or r_squared, are refused with a message."""
    from tests.golden import configs
    from tests.golden.configs import case
    c = case("izh_static")
    configs.write_case(c, str(tmp_path / "configfiles"))
    text = configs.config_text(c, stdp_params="root")
    rc, out = _run_driver(tmp_path, text, "izh_static_bg3")
    assert "BG3Params: 11 STDP constants from configfiles/bg3/izh_static_bg3.xml" in out, out
    assert "Unrecognized" not in out
    rc, out = _run_driver(tmp_path, text.replace("<BG3Params>", "<BG3Params><ParameterDraw>"
                                                 "squared</ParameterDraw>"), "izh_draw")
    assert rc != 0 and "<ParameterDraw> must be ranges or r_squared" in out, out
    rc, out = _run_driver(tmp_path, text.replace("AllDynamicSTDPSynapses", "AllDSSynapses"),
                          "izh_ds")
    assert rc != 0 and "STDPParams given for a synapse class without STDP" in out, out


def _fnv1a64(data):
    h = 1469598103934665603
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_r_squared_draw_in_the_drop_in_equals_the_config_reader(driver, tmp_path):
    """<BG3Params><ParameterDraw>r_squared</ParameterDraw> on the Izhikevich + dynamic STDP +
    ConnStatic case: the drop-in replays the draw from the reference's generator after the
    reference's own host setup; its a, b, c, d are those braingrid_gb300.config draws from the
    same file, byte for byte (the FNV-1a hash the driver logs, before its first C-ABI call).  A
    Lif network asking for the draw is refused."""
    from braingrid_gb300 import config as cf
    from tests.golden import configs
    from tests.golden.configs import case
    c = case("izh_static")
    configs.write_case(c, str(tmp_path / "configfiles"))
    text = configs.config_text(c, stdp_params="root").replace(
        "<BG3Params>", "<BG3Params><ParameterDraw>r_squared</ParameterDraw>")
    rc, out = _run_driver(tmp_path, text, "izh_r2")
    line = [l for l in out.splitlines() if "Izhikevich r^2 draw" in l]
    assert line, out
    p = cf.read(text, root=str(tmp_path))
    assert p.izh_draw == "r_squared"
    a = cf.setup(p)
    want = _fnv1a64(b"".join(a[k].astype("<f4").tobytes()
                             for k in ("Aconst", "Bconst", "Cconst", "Dconst")))
    assert "for %d neurons" % len(a["Aconst"]) in line[0], line[0]
    assert "FNV-1a %016x" % want in line[0], (line[0], "%016x" % want)
    configs.write_case(case("c0_stdp"), str(tmp_path / "configfiles"))
    lif = configs.config_text(case("c0_stdp")).replace(
        "</BGSimParams>", "<BG3Params><ParameterDraw>r_squared</ParameterDraw></BG3Params>"
        "</BGSimParams>")
    rc, out = _run_driver(tmp_path, lif, "lif_r2")
    assert rc != 0 and "ParameterDraw given for a neuron class other than AllIZHNeurons" in out, out
