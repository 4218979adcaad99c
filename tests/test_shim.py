"""The reference-side binding (semantic_icpslam_gb300/shim/sfusion_shim.cpp)
compiles against the reference's own declarations and links to this
library.

g++ compiles the shim with the reference's Tracking/Reduction.h and
Mapping/RenderScene.h (and the 2-line <opencv.hpp> stand-in the recipes
use) and -Werror=missing-declarations, so every launcher the shim defines
has exactly the signature the reference declares (a mismatch would be a new
overload, which the flag rejects).  The launchers of the drop-in boundary
are all defined, and every C-ABI symbol the object needs is exported by
libsfusion.so.  Needs the reference sources (skipped where they are absent).
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SHIM = os.path.join(ROOT, "semantic_icpslam_gb300", "shim", "sfusion_shim.cpp")

# the launchers the drop-in boundary replaces (Tracking/Reduction.h,
# Mapping/RenderScene.h)
LAUNCHERS = ["FilterDepth", "ComputeVMap", "ComputeNMap", "PyrDownGauss", "ResizeMap", "ICPStep", "RGBStep",
             "ImageToIntensity", "ComputeDerivativeImage", "ResetMap", "Raycast", "CreateRenderingBlocks",
             "CheckBlockVisibility", "FuseMapColor", "AnalyzeMapSemantics"]


def _ref_dir():
    from oracle.ref_shim.build_ref import REF
    return REF


@pytest.fixture(scope="module")
def shim_obj(tmp_path_factory):
    ref = _ref_dir()
    if not os.path.isdir(os.path.join(ref, "Tracking")):
        pytest.skip("reference sources not present")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    d = tmp_path_factory.mktemp("shim")
    stub = d / "stub"
    stub.mkdir()
    shutil.copy(os.path.join(ROOT, "oracle", "ref_shim", "include", "opencv.hpp"), stub / "opencv.hpp")
    obj = d / "sfusion_shim.o"
    cmd = ["g++", "-std=c++17", "-c", "-Wno-deprecated-declarations", "-Werror=missing-declarations",
           "-I", os.path.join(ref, "Tracking"), "-I", os.path.join(ref, "Mapping"), "-I", os.path.join(ref, "Utility"),
           "-I", os.path.join(ROOT, "include"), "-I", str(stub), "-I", cuda_inc, SHIM, "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return str(obj)


def _nm(args, path):
    r = subprocess.run(["nm"] + args + [path], capture_output=True, text=True, check=True)
    return r.stdout.splitlines()


def test_shim_defines_every_launcher(shim_obj):
    defined = [ln.split(" ", 2)[2] for ln in _nm(["-C", "--defined-only"], shim_obj) if " T " in ln]
    names = {d.split("(")[0] for d in defined}
    missing = [n for n in LAUNCHERS if n not in names]
    assert not missing, missing


def test_shim_needs_only_exported_symbols(shim_obj):
    from semantic_icpslam_gb300 import build
    lib = build.build()
    need = {ln.split()[-1] for ln in _nm(["-u"], shim_obj) if ln.split()[-1].startswith("sf_")}
    have = {ln.split()[-1] for ln in _nm(["-D", "--defined-only"], lib)}
    assert need and need <= have, sorted(need - have)
