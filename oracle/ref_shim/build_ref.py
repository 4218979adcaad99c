"""Recipe: compile the reference's own device code for the CPU (test
infrastructure only; run in the container that holds the reference sources).

Reads Mapping/, Tracking/ and Utility/ sources where they lie under
/root/reference, writes rewritten scratch copies into oracle/_ref/<cfg>/src
(git-ignored) and links them with ref_driver.cpp into oracle/_ref/<cfg>/libref.so.
The rewrites only make the CUDA sources compile as serial host C++:

  * kernel launches `K<<<grid, block>>>(args)` become serial loops over the
    grid (cuda_runtime.h in oracle/ref_shim/include);
  * `static __shared__` becomes `__shared__` (emulated as static);
  * Utility/ParallelScan.h is replaced by a serial prefix offset;
  * DeviceMap's static constexpr constants take the golden configuration's
    values (voxel size, truncation, table sizes, mesh triangle cap);
  * FuseMapColor's SemanticAnalysisKernel and UnifyNeighborKernel launches
    use the (8, 8) thread block that AnalyzeMapSemantics uses (the (8, 8, 8)
    launch applies one update per z-thread, a race on the GPU);
  * UnifyNeighbor's in-place write of each voxel's label fields goes to a
    copy of the voxel array taken at the launch, which replaces the array
    after it, so every voxel updates from the pass-start state (on the GPU
    neighbours read voxels other threads are rewriting, a race);
  * FuseMapColor's GarbageCollectKernel is left out: it only overwrites the
    visible-list copy's ptr with EntryToDelete, after which the label pass
    would index voxelBlocks[EntryToDelete + locId] (FuseMap.cu:176-207,
    518-582) instead of the block's own voxels;
  * functions computing ICPReduce::getRow and RGBReduction's FindCorresp /
    GetRow per pixel are appended to Reduction.cu's copy (the reference
    reduces rows with warp shuffles, which the serial emulation does not
    model), and one launching UnifyNeighborKernel alone over a given grid
    to FuseMap.cu's copy.

Nothing here is shipped or imported by the product.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref")
REF = os.environ.get("SF_REFERENCE_DIR", "/root/reference")

SOURCES = ["Mapping/DeviceMap.cu", "Mapping/FuseMap.cu", "Mapping/RenderScene.cu", "Mapping/MeshScene.cu",
           "Tracking/Pyrdown.cu", "Tracking/Reduction.cu"]
HEADERS = ["Mapping/DeviceMap.h", "Mapping/RenderScene.h", "Mapping/Constant.h", "Tracking/Reduction.h",
           "Utility/DeviceArray.h", "Utility/VectorMath.h", "Utility/SafeCall.h", "Utility/Intrinsics.h"]

# Configurations: DeviceMap constants (Mapping/DeviceMap.h:166-189).
#  * g1: the golden fixtures' 128x96 / 10 mm map, serial launches;
#  * c2: the benchmark's 640x480 map (5 mm voxels, 4 cm truncation, 2^20
#    buckets, 2^18 excess entries, 2^19 heap blocks), OpenMP over each
#    launch's blocks, linked with the loop driver ref_cpu_driver.cpp: the
#    reference's own loop on the host cores (the CPU baseline).
CONFIGS = {
    "g1": dict(VoxelSize="0.01f", TruncateMul=3, NumBuckets=4096, NumExcess=8192, NumSdfBlocks=16384,
               DepthMin="0.1f", DepthMax="3.0f", MaxTriangles=1000000),
    "c2": dict(VoxelSize="0.005f", TruncateMul=8, NumBuckets=1048576, NumExcess=262144, NumSdfBlocks=524288,
               DepthMin="0.1f", DepthMax="3.0f", MaxTriangles=1000000, omp=True, driver="ref_cpu_driver.cpp"),
}

ICP_APPENDIX = r'''
// ---- appended by oracle/ref_shim/build_ref.py: per-pixel ICP rows ----
extern "C" void ref_icp_rows_impl(const float *vc, const float *vl, const float *nc, const float *nl,
                                  int cols, int rows, const float *Rc, const float *tc, const float *Rl,
                                  const float *RlInv, const float *tl, float fx, float fy, float cx,
                                  float cy, float *out29) {
  ICPReduce icp;
  auto m3 = [](const float *R) {
    Matrix3f M;
    M.rowx = make_float3(R[0], R[1], R[2]);
    M.rowy = make_float3(R[3], R[4], R[5]);
    M.rowz = make_float3(R[6], R[7], R[8]);
    return M;
  };
  icp.Rcurr = m3(Rc); icp.Rlast = m3(Rl); icp.RlastInv = m3(RlInv);
  icp.tcurr = make_float3(tc[0], tc[1], tc[2]);
  icp.tlast = make_float3(tl[0], tl[1], tl[2]);
  icp.VMapCurr.data = (float4 *)vc; icp.VMapCurr.step = sizeof(float4) * cols;
  icp.VMapLast.data = (float4 *)vl; icp.VMapLast.step = sizeof(float4) * cols;
  icp.NMapCurr.data = (float4 *)nc; icp.NMapCurr.step = sizeof(float4) * cols;
  icp.NMapLast.data = (float4 *)nl; icp.NMapLast.step = sizeof(float4) * cols;
  icp.cols = cols; icp.rows = rows; icp.N = cols * rows;
  icp.fx = fx; icp.fy = fy; icp.cx = cx; icp.cy = cy;
  icp.angleThresh = 0.6; icp.distThresh = 0.1;  // as ICPStep sets them
  for (int i = 0; i < cols * rows; ++i) icp.getRow(i, out29 + 29 * (size_t)i);
}

// ---- appended by oracle/ref_shim/build_ref.py: ICP sums over every pixel ----
// ICPStep's 29 sums: ICPReduce::getRow for every pixel, summed in FP64 per
// host thread and then over the threads (the reference reduces the rows
// with warp shuffles and a block tree, which have no serial form).
extern "C" void ref_icp_sums_impl(const float *vc, const float *vl, const float *nc, const float *nl,
                                  int cols, int rows, const float *Rc, const float *tc, const float *Rl,
                                  const float *RlInv, const float *tl, float fx, float fy, float cx,
                                  float cy, double *sums29) {
  ICPReduce icp;
  auto m3 = [](const float *R) {
    Matrix3f M;
    M.rowx = make_float3(R[0], R[1], R[2]);
    M.rowy = make_float3(R[3], R[4], R[5]);
    M.rowz = make_float3(R[6], R[7], R[8]);
    return M;
  };
  icp.Rcurr = m3(Rc); icp.Rlast = m3(Rl); icp.RlastInv = m3(RlInv);
  icp.tcurr = make_float3(tc[0], tc[1], tc[2]);
  icp.tlast = make_float3(tl[0], tl[1], tl[2]);
  icp.VMapCurr.data = (float4 *)vc; icp.VMapCurr.step = sizeof(float4) * cols;
  icp.VMapLast.data = (float4 *)vl; icp.VMapLast.step = sizeof(float4) * cols;
  icp.NMapCurr.data = (float4 *)nc; icp.NMapCurr.step = sizeof(float4) * cols;
  icp.NMapLast.data = (float4 *)nl; icp.NMapLast.step = sizeof(float4) * cols;
  icp.cols = cols; icp.rows = rows; icp.N = cols * rows;
  icp.fx = fx; icp.fy = fy; icp.cx = cx; icp.cy = cy;
  icp.angleThresh = 0.6; icp.distThresh = 0.1;  // as ICPStep sets them
  double tot[29] = {0};
#pragma omp parallel
  {
    double part[29] = {0};
    float row[29];
#pragma omp for schedule(static)
    for (int i = 0; i < cols * rows; ++i) {
      icp.getRow(i, row);
      for (int k = 0; k < 29; ++k) part[k] += row[k];
    }
#pragma omp critical
    for (int k = 0; k < 29; ++k) tot[k] += part[k];
  }
  for (int k = 0; k < 29; ++k) sums29[k] = tot[k];
}

// ---- appended by oracle/ref_shim/build_ref.py: per-pixel RGB rows ----
// RGBStep's two passes over every pixel (FindCorresp, then GetRow), with the
// integer sums and sigma computed as RGBStep computes them between the two.
extern "C" void ref_rgb_rows_impl(const unsigned char *inext, const unsigned char *ilast, const float *vn,
                                  const float *vl, const short *dx, const short *dy, int cols, int rows,
                                  const float *Rc, const float *RcI, const float *Rl, const float *RlI,
                                  const float *tc, const float *tl, float fx, float fy, float cx, float cy,
                                  int *res2, float *sigma, float *out29) {
  RGBReduction rgb;
  auto m3 = [](const float *R) {
    Matrix3f M;
    M.rowx = make_float3(R[0], R[1], R[2]);
    M.rowy = make_float3(R[3], R[4], R[5]);
    M.rowz = make_float3(R[6], R[7], R[8]);
    return M;
  };
  std::vector<Residual> resid((size_t)cols * rows);
  rgb.cols = cols; rgb.rows = rows; rgb.N = cols * rows;
  rgb.nextImage.data = (unsigned char *)inext; rgb.nextImage.step = cols;
  rgb.lastImage.data = (unsigned char *)ilast; rgb.lastImage.step = cols;
  rgb.nextVMap.data = (float4 *)vn; rgb.nextVMap.step = sizeof(float4) * cols;
  rgb.lastVMap.data = (float4 *)vl; rgb.lastVMap.step = sizeof(float4) * cols;
  rgb.dIdx.data = (short *)dx; rgb.dIdx.step = sizeof(short) * cols;
  rgb.dIdy.data = (short *)dy; rgb.dIdy.step = sizeof(short) * cols;
  rgb.Rcurr = m3(Rc); rgb.RcurrInv = m3(RcI); rgb.Rlast = m3(Rl); rgb.RlastInv = m3(RlI);
  rgb.tcurr = make_float3(tc[0], tc[1], tc[2]);
  rgb.tlast = make_float3(tl[0], tl[1], tl[2]);
  rgb.RGBResidual.data = resid.data(); rgb.RGBResidual.size = resid.size();
  rgb.fx = fx; rgb.fy = fy; rgb.cx = cx; rgb.cy = cy;
  int s0 = 0, s1 = 0;
  for (int k = 0; k < cols * rows; ++k) {
    int2 v = rgb.FindCorresp(k);
    s0 += v.x;
    s1 += v.y;
  }
  rgb.sigma = sqrt((float) s1 / (s0 == 0 ? 1 : s0));
  for (int k = 0; k < cols * rows; ++k) rgb.GetRow(k, out29 + 29 * (size_t)k);
  res2[0] = s0;
  res2[1] = s1;
  *sigma = rgb.sigma;
}
'''


FUSE_APPENDIX = r'''
// ---- appended by oracle/ref_shim/build_ref.py: UnifyNeighborKernel alone ----
extern "C" void ref_unify_neighbor_impl(DeviceMap map, unsigned nvis) {
  Fusion fuse;
  fuse.map = map;
  shim_unify_begin(map.voxelBlocks.data, map.voxelBlocks.size * sizeof(Voxel));
  shim_launch_any(dim3(nvis), dim3(8, 8), [&] { UnifyNeighborKernel(fuse); });
  shim_unify_end();
}
'''


def _match_back(s, i, open_c, close_c):
    depth = 0
    while i >= 0:
        if s[i] == close_c:
            depth += 1
        elif s[i] == open_c:
            depth -= 1
            if depth == 0:
                return i
        i -= 1
    raise ValueError("unbalanced")


def _match_fwd(s, i, open_c, close_c):
    depth = 0
    while i < len(s):
        if s[i] == open_c:
            depth += 1
        elif s[i] == close_c:
            depth -= 1
            if depth == 0:
                return i
        i += 1
    raise ValueError("unbalanced")


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{<":
            depth += 1
        elif ch in ")]}>":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def rewrite_launches(src):
    out = src
    while True:
        i = out.find("<<<")
        if i < 0:
            return out
        j = out.index(">>>", i)
        cfg = _split_top(out[i + 3:j])
        # kernel expression before <<<
        k = i - 1
        while out[k].isspace():
            k -= 1
        if out[k] == ">":
            k = _match_back(out, k, "<", ">") - 1
        while out[k].isspace():
            k -= 1
        e = k
        while out[k].isalnum() or out[k] == "_":
            k -= 1
        kstart = k + 1
        kernel = out[kstart:i].strip()
        p = j + 3
        while out[p].isspace():
            p += 1
        assert out[p] == "(", out[p:p + 40]
        q = _match_fwd(out, p, "(", ")")
        args = out[p + 1:q]
        semi = out.index(";", q)
        repl = "shim_launch_any(%s, %s, [&] { %s(%s); })" % (cfg[0], cfg[1], kernel, args)
        out = out[:kstart] + repl + out[semi:]


def patch_sources(name, text, cfg):
    text = text.replace("static __shared__", "__shared__")
    if name == "DeviceMap.h":
        def sub(field, value):
            nonlocal text
            pat = re.compile(r"^(\s*static constexpr \w+ %s = )[^;]+;" % field, re.M)
            assert pat.search(text), field
            text = pat.sub(lambda m: m.group(1) + str(value) + ";", text, count=1)
        sub("VoxelSize", cfg["VoxelSize"])
        sub("TruncateDist", "VoxelSize * %d" % cfg["TruncateMul"])
        sub("NumBuckets", cfg["NumBuckets"])
        sub("NumExcess", cfg["NumExcess"])
        sub("NumSdfBlocks", cfg["NumSdfBlocks"])
        sub("DepthMin", cfg["DepthMin"])
        sub("DepthMax", cfg["DepthMax"])
        sub("MaxTriangles", cfg["MaxTriangles"])
    if name == "FuseMap.cu":
        # GarbageCollectKernel only rewrites the visible-list copy's ptr to
        # EntryToDelete; SemanticAnalysisKernel then indexes
        # voxelBlocks[EntryToDelete + locId].  Left out so the label pass
        # updates each block's own voxels.
        gc = "GarbageCollectKernel<<<block, thread>>>(fuse);"
        assert text.count(gc) == 1
        text = text.replace(gc, "/* GarbageCollect left out by the recipe */")
        launch = "SemanticAnalysisKernel<<<block, thread>>>(fuse);"
        first = text.index(launch)
        text = text[:first] + "thread = dim3(8, 8);\n\t\t" + text[first:]
        # UnifyNeighbor writes `cur` in place while other threads read it as
        # a neighbour; the write goes to the launch's copy of the voxel array
        # instead (shim_unify_begin/end in include/cuda_runtime.h).
        cur = "Voxel &cur = map.voxelBlocks[entry.ptr + locId];"
        assert text.count(cur) == 1
        text = text.replace(cur, "Voxel &cur = ((Voxel *)shim_unify_dst)[entry.ptr + locId];")
        un = "UnifyNeighborKernel<<<block, thread>>>(fuse);"
        assert text.count(un) == 2, text.count(un)
        text = text.replace(un, "shim_unify_begin(fuse.map.voxelBlocks.data, fuse.map.voxelBlocks.size * "
                                "sizeof(Voxel));\n\t\t" + un + "\n\t\tshim_unify_end();")
    if name.endswith(".cu"):
        text = rewrite_launches(text)
    if name == "Reduction.cu":
        text += ICP_APPENDIX
    if name == "FuseMap.cu":
        text += FUSE_APPENDIX
    return text


def prepare(cfg_name="g1"):
    """Writes the rewritten copies of the reference sources into
    oracle/_ref/<cfg>/src (needs the reference tree)."""
    if not os.path.isdir(REF):
        raise FileNotFoundError("reference sources not found at %s" % REF)
    cfg = CONFIGS[cfg_name]
    src_dir = os.path.join(OUT, cfg_name, "src")
    os.makedirs(src_dir, exist_ok=True)
    for rel in HEADERS + SOURCES:
        name = os.path.basename(rel)
        text = open(os.path.join(REF, rel)).read()
        text = patch_sources(name, text, cfg)
        out_name = name[:-3] + ".cpp" if name.endswith(".cu") else name
        with open(os.path.join(src_dir, out_name), "w") as f:
            f.write(text)
    with open(os.path.join(src_dir, ".prepared"), "w") as f:
        f.write(_recipe_stamp())
    return src_dir


def _recipe_stamp():
    return "%.6f" % os.path.getmtime(__file__)


def build(cfg_name="g1", force=False, verbose=False):
    """Compiles oracle/_ref/<cfg>/libref.so from the prepared copies,
    preparing them first where the reference tree is present.  On a machine
    without the reference tree (the GPU machine) it compiles copies prepared
    elsewhere, and raises FileNotFoundError when there are none."""
    cfg = CONFIGS[cfg_name]
    dst = os.path.join(OUT, cfg_name)
    src_dir = os.path.join(dst, "src")
    lib = os.path.join(dst, "libref.so")
    driver = os.path.join(HERE, cfg.get("driver", "ref_driver.cpp"))
    deps = [driver, os.path.join(HERE, "include", "cuda_runtime.h"), os.path.join(HERE, "include", "ParallelScan.h"),
            os.path.join(HERE, "ref_loop.h"), os.path.join(ROOT, "semantic_icpslam_gb300", "csrc", "sf_solve.h")]
    stamp = os.path.join(src_dir, ".prepared")
    if os.path.isdir(REF):
        if force or not os.path.exists(stamp) or open(stamp).read() != _recipe_stamp():
            prepare(cfg_name)
    elif not os.path.exists(stamp):
        raise FileNotFoundError("reference sources not found at %s and no prepared copies" % REF)
    deps.append(stamp)
    if not force and os.path.exists(lib) and os.path.getmtime(lib) > max(os.path.getmtime(d) for d in deps):
        return lib
    objs = []
    flags = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-w",
             "-I", os.path.join(HERE, "include"), "-I", src_dir]
    if cfg.get("omp"):
        flags += ["-fopenmp", "-DSHIM_OMP", "-I", HERE, "-I", os.path.join(ROOT, "semantic_icpslam_gb300", "csrc")]
    units = [os.path.join(src_dir, os.path.basename(r)[:-3] + ".cpp") for r in SOURCES] + [driver]
    procs = []
    for u in units:
        o = os.path.join(dst, os.path.basename(u) + ".o")
        objs.append(o)
        cmd = ["g++"] + flags + ["-c", u, "-o", o]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), out[-4000:]))
    subprocess.check_call(["g++", "-shared", "-o", lib + ".tmp"] + objs + (["-fopenmp"] if cfg.get("omp") else []))
    os.replace(lib + ".tmp", lib)
    return lib


def build_all(force=False, verbose=False):
    """Every configuration that can be built here; returns {name: path or
    the reason it was skipped}."""
    out = {}
    for name in CONFIGS:
        try:
            out[name] = build(name, force=force, verbose=verbose)
        except (FileNotFoundError, RuntimeError, subprocess.CalledProcessError) as e:
            out[name] = "skipped: %s" % str(e).splitlines()[0]
    return out


if __name__ == "__main__":
    for k, v in build_all(force="--force" in sys.argv, verbose="-v" in sys.argv).items():
        print(k, v)
