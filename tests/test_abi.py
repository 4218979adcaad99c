"""The C ABI library loads and exports every entry point include/*.h
declares; POD layouts match the reference's (HashEntry 32 B, Voxel 16 B,
RenderingBlock 16 B).  No compute call is made (no GPU needed)."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"^\s*int\s+(sf_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_symbols()
    for must in ["sf_FilterDepth", "sf_ComputeVMap", "sf_ComputeNMap", "sf_PyrDownGauss", "sf_ResizeMap",
                 "sf_ICPStep", "sf_ResetMap", "sf_Raycast", "sf_CreateRenderingBlocks",
                 "sf_CheckBlockVisibility", "sf_FuseMapColor", "sf_AnalyzeMapSemantics", "sf_UnifyNeighbor",
                 "sf_ComputeSE3", "sf_system_grab"]:
        assert must in names


def test_library_exports_every_declared_symbol(built):
    from semantic_icpslam_gb300 import _lib
    L = _lib.load()
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (sf_\w+)$", out, flags=re.M))
    assert set(declared_symbols()) <= exported


def test_bindings_cover_declarations(built):
    from semantic_icpslam_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_pod_layouts():
    from oracle.oracle import ENTRY_DTYPE, RBLOCK_DTYPE, VOXEL_DTYPE
    from semantic_icpslam_gb300 import _lib
    assert ENTRY_DTYPE.itemsize == 32 and ENTRY_DTYPE.fields["ptr"][1] == 12 and ENTRY_DTYPE.fields["offset"][1] == 16
    assert VOXEL_DTYPE.itemsize == 16
    assert [VOXEL_DTYPE.fields[k][1] for k in ("sdf", "weight", "color", "label", "count", "label_2", "count_2",
                                                "color_2", "obj_idx")] == [0, 4, 5, 8, 9, 10, 11, 12, 15]
    assert RBLOCK_DTYPE.itemsize == 16 and RBLOCK_DTYPE.fields["zmin"][1] == 8
    assert C.sizeof(_lib.Mat3) == 36 and C.sizeof(_lib.Image) == 24


def test_no_device_fails_loudly(built):
    """Without a GPU the library reports SF_ERR_NO_DEVICE instead of falling back."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import semantic_icpslam_gb300 as sf
    with pytest.raises(sf.SfError) as e:
        sf.Context()
    assert e.value.status == sf._lib.SF_ERR_NO_DEVICE
