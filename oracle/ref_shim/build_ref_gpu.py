"""Recipe: the reference's own CUDA build, for timing on the GPU next to this
loop (test and benchmark infrastructure only).

prepare() (in the container that holds the reference sources) copies
Mapping/, Tracking/ and Utility/ sources from /root/reference into
oracle/_ref/gpu_c2/src (git-ignored) with two edits:

  * DeviceMap's static constexpr constants take the 640x480 benchmark map's
    values (5 mm voxels, 4 cm truncation, 2^20 buckets, 2^18 excess,
    2^19 heap blocks), as the reference's own constants are edited for a
    map size (Mapping/DeviceMap.h:166-189);
  * the raycast's per-ray cache `HashEntry b;` (RenderScene.cu) starts at
    an unused block position.  Its default {(0,0,0), ptr -1} would make a
    ray whose first lookup is block (0,0,0) read voxelBlocks[-1 + idx],
    out of bounds.  The change alters no lookup result.

build() (on any machine with nvcc, the GPU machine included) compiles those
copies for sm_103a with oracle/ref_shim/ref_gpu_driver.cu (the loop of
ref_loop.h) into oracle/_ref/gpu_c2/librefgpu.so.  Nothing here is shipped or imported by
the product.
"""
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref", "gpu_c2")
SRC = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "librefgpu.so")
# The same sources built with FMA contraction off (-fmad=false): every float
# operation rounds once, as the CPU oracle computes it
OUT_NOFMA = os.path.join(ORACLE, "_ref", "gpu_c2_nofma")
LIB_NOFMA = os.path.join(OUT_NOFMA, "librefgpu.so")
REF = os.environ.get("SF_REFERENCE_DIR", "/root/reference")

SOURCES = ["Mapping/DeviceMap.cu", "Mapping/FuseMap.cu", "Mapping/RenderScene.cu", "Tracking/Pyrdown.cu",
           "Tracking/Reduction.cu"]
HEADER_DIRS = ["Mapping", "Tracking", "Utility"]
C2 = dict(VoxelSize="0.005f", TruncateDist="VoxelSize * 8", NumBuckets="1048576", NumExcess="262144",
          NumSdfBlocks="524288", DepthMin="0.1f", DepthMax="3.0f")


def _patch(name, text):
    if name == "DeviceMap.h":
        for field, value in C2.items():
            pat = re.compile(r"^(\s*static constexpr \w+ %s = )[^;]+;" % field, re.M)
            assert pat.search(text), field
            text = pat.sub(lambda m: m.group(1) + value + ";", text, count=1)
    if name == "RenderScene.cu":
        decl = "HashEntry b;"
        assert text.count(decl) == 1
        text = text.replace(decl, decl + " b.pos = make_int3(0x7fffffff);  /* recipe: unused block position */")
    return text


def prepare():
    """Copies and edits the reference sources (needs the reference tree)."""
    if not os.path.isdir(REF):
        raise FileNotFoundError("reference sources not found at %s" % REF)
    os.makedirs(SRC, exist_ok=True)
    names = list(SOURCES)
    for d in HEADER_DIRS:
        names += [os.path.join(d, f) for f in sorted(os.listdir(os.path.join(REF, d))) if f.endswith(".h")]
    for rel in names:
        with open(os.path.join(REF, rel), encoding="utf-8", errors="replace") as f:
            text = f.read()
        name = os.path.basename(rel)
        with open(os.path.join(SRC, name), "w") as f:
            f.write(_patch(name, text))
    shutil.copy(os.path.join(HERE, "include", "opencv.hpp"), os.path.join(SRC, "opencv.hpp"))


def build(force=False, verbose=False):
    """Compiles the prepared copies and the driver into librefgpu.so, as
    the reference builds them (FMA contraction on) and with contraction
    off (gpu_c2_nofma), both variants in parallel."""
    if not os.path.isdir(SRC):
        if os.path.isdir(REF):
            prepare()
        else:
            return None
    driver = os.path.join(HERE, "ref_gpu_driver.cu")
    srcs = [os.path.join(SRC, os.path.basename(s)) for s in SOURCES] + [driver]
    deps = srcs + [os.path.join(HERE, "ref_loop.h"), os.path.join(ROOT, "semantic_icpslam_gb300", "csrc", "sf_solve.h")]
    newest = max(os.path.getmtime(s) for s in deps)
    todo = [(out, lib, extra) for out, lib, extra in ((OUT, LIB, []), (OUT_NOFMA, LIB_NOFMA, ["-fmad=false"]))
            if force or not os.path.exists(lib) or os.path.getmtime(lib) <= newest]
    if not todo:
        return LIB
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    nvcc = nvcc if os.path.exists(nvcc) else "nvcc"
    flags = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-rdc=true", "-Xcompiler", "-fPIC", "-w",
             "-I", SRC, "-I", os.path.join(ROOT, "semantic_icpslam_gb300", "csrc")]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference CUDA build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))

    cmds, links = [], []
    for out, lib, extra in todo:
        os.makedirs(out, exist_ok=True)
        objs = [os.path.join(out, os.path.basename(s) + ".o") for s in srcs]
        cmds += [[nvcc] + flags + extra + ["-c", s, "-o", o] for s, o in zip(srcs, objs)]
        links.append((lib, [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-rdc=true", "-shared", "-o",
                            lib + ".tmp"] + objs))
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(run, cmds))
    for lib, cmd in links:
        run(cmd)
        os.replace(lib + ".tmp", lib)
    return LIB


if __name__ == "__main__":
    if "--prepare" in sys.argv or os.path.isdir(REF):
        prepare()
    print(build(force=True, verbose=True))
