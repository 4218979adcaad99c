"""sf_MeshScene (MeshScene, Mapping/MeshScene.cu) on the GPU: on the fused
golden map, the reference kernel's triangle count and vertex records
(tests/golden/g1.npz); on every map, the oracle's triangles exactly (as a
set: the GPU appends cubes in no fixed order); the triangle cap; the PLY
file of System::WriteMeshToDisk."""
import ctypes as C
import hashlib
import os

import numpy as np
import pytest

from tests.helpers import C1, MAP_C1, empty, host, map_to_host, sequence

pytestmark = pytest.mark.gpu

G1 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "g1.npz")


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _records(v, n, c):
    k = v.reshape(-1, 3).shape[0]
    rec = np.zeros((k, 28), np.uint8)
    rec[:, :12] = np.ascontiguousarray(v.reshape(-1, 3)).view(np.uint8).reshape(k, 12)
    rec[:, 12:24] = np.ascontiguousarray(n.reshape(-1, 3)).view(np.uint8).reshape(k, 12)
    rec[:, 24:27] = c.reshape(-1, 3)
    return np.unique(rec, axis=0)


def _triangle_set(v, n, c):
    t = np.concatenate([np.ascontiguousarray(v).view(np.uint8).reshape(len(v), 36),
                        np.ascontiguousarray(n).view(np.uint8).reshape(len(n), 36),
                        np.ascontiguousarray(c).reshape(len(c), 9)], 1)
    return np.unique(t, axis=0)


def _gpu_mesh(sf, ctx, gmap, max_tri):
    import torch
    v = empty((max_tri, 3, 3), torch.float32)
    n = empty((max_tri, 3, 3), torch.float32)
    c = empty((max_tri, 3, 3), torch.uint8)
    k = C.c_uint32()
    sf.call("sf_MeshScene", ctx.h, gmap.h, v.data_ptr(), n.data_ptr(), c.data_ptr(), max_tri, C.byref(k))
    k = k.value
    return host(v)[:k], host(n)[:k], host(c)[:k], (v, n, c)


def _load(sf, ctx, gmap, entries, voxels):
    a = gmap.arrays()
    entries = np.ascontiguousarray(entries)
    voxels = np.ascontiguousarray(voxels)
    ctx.memcpy(a.hash_entries, entries.ctypes.data, entries.nbytes)
    ctx.memcpy(a.voxel_blocks, voxels.ctypes.data, voxels.nbytes)
    sf.call("sf_map_rebuild_index", ctx.h, gmap.h)


def test_mesh_golden_map(lib):
    """The golden map (five fused frames, made again by the oracle, which
    equals the reference's map there byte for byte)."""
    from oracle import oracle as O
    from tests.test_oracle_golden import _frame, _K, _oracle_map
    sf, ctx = lib
    g = dict(np.load(G1))
    om = _oracle_map(g)
    for i in range(5):
        raw, _, nm = _frame(g, i)
        om.fuse(raw, g["rgb%d" % i], nm, g["mask%d" % i], 10 if i >= 2 else 0, g["pose%d" % i], _K(g))
    c = g["consts"]
    gmap = sf.Map(voxel_size=float(np.float32(c[0])), trunc_dist=float(np.float32(c[1])), num_buckets=int(c[2]),
                  num_excess=int(c[3]), num_sdf_blocks=int(c[4]))
    e = om.entries.copy()
    nvox = int(e["ptr"].max()) + 512
    _load(sf, ctx, gmap, e, om.voxels[:nvox].copy())
    v, n, col, _ = _gpu_mesh(sf, ctx, gmap, 400000)
    assert len(v) == int(g["mesh_ntri"])
    recs = _records(v, n, col)
    assert len(recs) == int(g["mesh_nrec"])
    assert np.array_equal(np.frombuffer(hashlib.sha1(recs.tobytes()).digest(), np.uint8), g["mesh_rec_sha1"])
    ov, on, oc = om.mesh(400000)
    assert np.array_equal(_triangle_set(v, n, col), _triangle_set(ov, on, oc))
    gmap.close()


def test_mesh_fused_map_cap_and_ply(lib, tmp_path):
    """A map fused on the GPU (320x240, 4 frames): its mesh equals the
    oracle's on the same map state; a cap below the total keeps exactly
    the cap; the PLY file has the reference's header and counts."""
    from oracle import oracle as O
    import torch
    sf, ctx = lib
    K = C1["K"]
    seq = sequence(C1["cols"], C1["rows"], K, 4, trajectory=0)
    cfg = sf.system_config(cols=C1["cols"], rows=C1["rows"], K=K, **MAP_C1)
    s = sf.System(ctx, cfg, init_pose=seq[0][3])
    for d, rgb, _, _ in seq:
        s.grab(d, rgb)
    m = s.map()
    v, n, c, dev = _gpu_mesh(sf, ctx, m, 1000000)
    assert len(v) > 10000
    e, vox, _ = map_to_host(ctx, m)
    om = O.Map(**MAP_C1)
    om.entries[:] = e
    om.voxels[:] = vox
    ov, on, oc = om.mesh(1000000)
    assert np.array_equal(_triangle_set(v, n, c), _triangle_set(ov, on, oc))
    assert np.isfinite(v).all() and np.allclose(np.linalg.norm(n, axis=-1), 1.0, atol=1e-5)
    cap = len(v) // 3
    v2, _, _, _ = _gpu_mesh(sf, ctx, m, cap)
    assert len(v2) == cap
    path = str(tmp_path / "scene.ply")
    dv, dn, dc = dev
    sf.call("sf_mesh_write_ply", ctx.h, path.encode(), dv.data_ptr(), dn.data_ptr(), dc.data_ptr(), len(v))
    lines = open(path).read().splitlines()
    assert lines[0] == "ply" and lines[2] == "element vertex %d" % (3 * len(v))
    assert lines[12] == "element face %d" % len(v) and lines[14] == "end_header"
    first = lines[15].split()
    assert np.allclose([float(x) for x in first[:6]], np.concatenate([v[0, 0], n[0, 0]]), rtol=1e-5, atol=1e-6)
    assert [int(x) for x in first[6:]] == list(c[0, 0])
    assert lines[15 + 3 * len(v)] == "3 0 1 2" and len(lines) == 15 + 4 * len(v)
    s.close()
