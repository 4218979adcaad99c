"""Builds libsfusion.so in-tree: hand-written sm_103a CUDA kernels + the C ABI.

Every .cu is compiled with -fmad=false so each float operation rounds once,
as the reference's source states it (bit-exact integer outputs against the
CPU oracle).  Translation units compile in parallel; the result is
semantic_icpslam_gb300/libsfusion.so (git-ignored).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsfusion.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                     "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(h) > t for h in headers)


LIB_CHECKED = os.path.join(HERE, "libsfusion_checked.so")


def build(force=False, verbose=False, jobs=None, debug_bounds=False):
    """The release library, or with debug_bounds the bounds-checked one
    (-DSF_BOUNDS_CHECK, libsfusion_checked.so, objects in _build/checked):
    the same kernels with every hash-chain link and block pointer checked
    before use, for tests against corrupted maps."""
    bdir = os.path.join(BUILD, "checked") if debug_bounds else BUILD
    lib = LIB_CHECKED if debug_bounds else LIB
    extra = ["-DSF_BOUNDS_CHECK"] if debug_bounds else []
    os.makedirs(bdir, exist_ok=True)
    cu, cpp = sources()
    headers = _headers()
    nvcc = _nvcc()
    cmds = []
    objs = []
    for f in cu:
        src, obj = os.path.join(CSRC, f), os.path.join(bdir, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            cmds.append([nvcc] + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    for f in cpp:
        src, obj = os.path.join(CSRC, f), os.path.join(bdir, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            cmds.append(["g++"] + CXX_FLAGS + extra + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for err in ex.map(run, cmds):
            if verbose and err.strip():
                print(err)
    if cmds or not os.path.exists(lib) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in objs):
        run([nvcc] + ARCH + ["-shared", "-o", lib + ".tmp"] + objs)
        os.replace(lib + ".tmp", lib)
    return lib


# The libtorch C++ autograd function (torch_ext/raycast_autograd.cpp): a
# Python extension module linked against libtorch and libsfusion.so.
TORCH_EXT_SRC = os.path.join(HERE, "torch_ext", "raycast_autograd.cpp")
TORCH_EXT = os.path.join(HERE, "sf_torch.so")


def _torch_ext_cmds():
    import sysconfig
    import torch
    import torch.utils.cpp_extension as ce
    inc = ce.include_paths() + [sysconfig.get_paths()["include"], INCLUDE]
    obj = os.path.join(BUILD, "raycast_autograd.o")
    cc = ["g++", "-O2", "-std=c++17", "-fPIC", "-D_GLIBCXX_USE_CXX11_ABI=%d" % int(torch._C._GLIBCXX_USE_CXX11_ABI),
          "-DTORCH_EXTENSION_NAME=sf_torch", "-DTORCH_API_INCLUDE_EXTENSION_H"] + sum([["-I", i] for i in inc], [])
    compile_cmd = cc + ["-c", TORCH_EXT_SRC, "-o", obj]
    link_cmd = ["g++", "-shared", obj, "-o", TORCH_EXT + ".tmp", "-L", ce.library_paths()[0], "-lc10", "-ltorch",
                "-ltorch_cpu", "-ltorch_python", "-L", HERE, "-lsfusion", "-Wl,-rpath,$ORIGIN",
                "-Wl,-rpath," + ce.library_paths()[0]]
    return obj, compile_cmd, link_cmd


def build_all(force=False, verbose=False):
    """libsfusion.so, then the torch extension (compiled alongside, linked
    after).  A torch extension that cannot build is reported and skipped:
    the library and its Python torch.autograd form do not need it."""
    ext = None
    try:
        obj, compile_cmd, link_cmd = _torch_ext_cmds()
        os.makedirs(BUILD, exist_ok=True)
        if force or not os.path.exists(obj) or os.path.getmtime(TORCH_EXT_SRC) > os.path.getmtime(obj) or \
                os.path.getmtime(os.path.join(INCLUDE, "sfusion.h")) > os.path.getmtime(obj):
            ext = subprocess.Popen(compile_cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    except Exception as e:  # no torch headers
        print("torch extension skipped: %s" % e, file=sys.stderr)
        link_cmd = None
    lib = build(force=force, verbose=verbose)
    if link_cmd is None:
        return lib
    if ext is not None:
        out, err = ext.communicate()
        if ext.returncode != 0:
            print("torch extension skipped: compile failed\n%s" % err[-2000:], file=sys.stderr)
            return lib
    if force or not os.path.exists(TORCH_EXT) or os.path.getmtime(obj) > os.path.getmtime(TORCH_EXT) or \
            os.path.getmtime(lib) > os.path.getmtime(TORCH_EXT):
        r = subprocess.run(link_cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print("torch extension skipped: link failed\n%s" % r.stderr[-2000:], file=sys.stderr)
            return lib
        os.replace(TORCH_EXT + ".tmp", TORCH_EXT)
    return lib


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
