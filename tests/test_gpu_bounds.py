"""The bounds-checked build of the library (-DSF_BOUNDS_CHECK,
libsfusion_checked.so): every hash-chain link and every block pointer taken
from the hash table or the block window is checked before use, and a bad
one sets a bit in the map's status word instead of being followed.

* On a healthy sequence the checked build computes what the release build
  computes (poses and statistics bit for bit) and records nothing.
* A hash entry whose block pointer is moved off its block boundary (still
  inside the voxel array, so even an unchecked read would stay in bounds)
  is caught by the ray lookups: SF_BOUND_PTR is set and the block reads as
  missing.

Each build runs in its own process (the library is chosen when it loads).
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tests.helpers import C1, MAP_C1, sequence

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import ctypes as C, json, sys
import numpy as np
sys.path.insert(0, %(root)r)
import semantic_icpslam_gb300 as sf
from semantic_icpslam_gb300 import _lib
from tests.helpers import C1, MAP_C1, sequence, cuda, empty, host
flags = C.c_uint32()
sf.call("sf_build_flags", C.byref(flags))
ctx = sf.Context()
seq = sequence(C1["cols"], C1["rows"], C1["K"], 6, trajectory=1, dropout=0.02)
cfg = sf.system_config(cols=C1["cols"], rows=C1["rows"], K=C1["K"], use_graph=1, **MAP_C1)
s = sf.System(ctx, cfg, init_pose=seq[0][3])
poses, stats = [], []
for d, rgb, _, _ in seq:
    st = s.grab(d, rgb)
    poses.append(list(st.pose[:]))
    stats.append([st.tracked, st.iterations, st.icp_count, st.visible, st.allocated])
status = C.c_uint32()
sf.call("sf_map_bounds_status", ctx.h, s.map().h, C.byref(status))
out = {"flags": flags.value, "poses": poses, "stats": stats, "status": status.value}
if %(corrupt)r:
    # move one visible block's pointer off its block boundary (one voxel:
    # still inside the voxel array) and render through the map again
    import torch
    from oracle.oracle import ENTRY_DTYPE
    m = s.map()
    a = m.arrays()
    ent = ctx.download(a.hash_entries, ENTRY_DTYPE, m.num_entries)
    vis = ctx.download(a.visible_entries, ENTRY_DTYPE, m.num_entries)[:m.counters(ctx)[2]]
    pos = vis[len(vis) // 2]
    k = int(np.flatnonzero((ent["x"] == pos["x"]) & (ent["y"] == pos["y"]) & (ent["z"] == pos["z"]) &
                           (ent["ptr"] >= 0))[0])
    bad = np.array([int(ent["ptr"][k]) + 1], np.int32)
    ctx.memcpy(a.hash_entries + 32 * k + 12, bad.ctypes.data, 4)
    P = np.array(poses[-1]).reshape(4, 4)
    R, RI, t = sf.pose_to_gpu(P)
    K = C1["K"]
    nv = C.c_uint32()
    sf.call("sf_CheckBlockVisibility", ctx.h, m.h, R, RI, t, C1["cols"], C1["rows"], *K, 3.0, 0.1, C.byref(nv))
    zc, zr = (C1["cols"] + 7) // 8, (C1["rows"] + 7) // 8
    zmin, zmax = empty((zr, zc), torch.float32), empty((zr, zc), torch.float32)
    blocks = torch.zeros((260000, 4), dtype=torch.int32, device="cuda")
    nrb = torch.zeros(1, dtype=torch.int32, device="cuda")
    ok = C.c_int()
    sf.call("sf_CreateRenderingBlocks", ctx.h, m.h, sf.image(zmin), sf.image(zmax), 3.0, 0.1, blocks.data_ptr(),
            nrb.data_ptr(), RI, t, nv.value, *K, C.byref(ok))
    vm, nm = empty((C1["rows"], C1["cols"], 4), torch.float32), empty((C1["rows"], C1["cols"], 4), torch.float32)
    sf.call("sf_Raycast", ctx.h, m.h, sf.image(vm), sf.image(nm), sf.image(zmin), sf.image(zmax), R, RI, t,
            float(np.float32(1.0 / np.float32(K[0]))), float(np.float32(1.0 / np.float32(K[1]))), K[2], K[3])
    ctx.sync()
    sf.call("sf_map_bounds_status", ctx.h, m.h, C.byref(status))
    out["status_after"] = status.value
s.close()
ctx.close()
print("RESULT " + json.dumps(out))
'''


def _run(lib, corrupt=False):
    env = dict(os.environ)
    if lib:
        env["SF_LIBRARY"] = lib
    else:
        env.pop("SF_LIBRARY", None)
    r = subprocess.run([sys.executable, "-c", CHILD % {"root": ROOT, "corrupt": corrupt}], capture_output=True,
                       text=True, env=env, cwd=ROOT, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    return json.loads(line[7:])


@pytest.fixture(scope="module")
def checked_lib(built):
    from semantic_icpslam_gb300 import build
    return build.build(debug_bounds=True)


def test_checked_build_matches_release_and_records_nothing(checked_lib):
    rel = _run(None)
    chk = _run(checked_lib)
    assert rel["flags"] == 0 and chk["flags"] == 1
    assert chk["poses"] == rel["poses"] and chk["stats"] == rel["stats"]
    assert rel["status"] == 0 and chk["status"] == 0


def test_checked_build_catches_a_misaligned_block_pointer(checked_lib):
    chk = _run(checked_lib, corrupt=True)
    assert chk["status"] == 0
    assert chk["status_after"] & 2  # SF_BOUND_PTR
