"""sf_UnifyNeighbor (UnifyNeighborKernel, Mapping/FuseMap.cu:757-896) on the
GPU: bit-exact against the reference's own kernel on the seeded state of
tests/golden/g1.npz, and against the oracle on fused label states loaded
into both maps with the same hash-slot layout; the pass inside
FuseMapColor and the frame graph with detections."""
import ctypes as C
import os

import numpy as np
import pytest

from tests.helpers import C1, map_to_host, sequence

pytestmark = pytest.mark.gpu

G1 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "g1.npz")
# 4096 buckets: hash slots [0, visible count) then hold a third of a room's
# blocks (with 2^18 buckets they hold a handful).
MAP_SMALL = dict(voxel_size=0.01, trunc_dist=0.03, num_buckets=1 << 12, num_excess=1 << 15,
                 num_sdf_blocks=1 << 15)


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _g1_cfg(g):
    c = g["consts"]
    return dict(voxel_size=float(np.float32(c[0])), trunc_dist=float(np.float32(c[1])), num_buckets=int(c[2]),
                num_excess=int(c[3]), num_sdf_blocks=int(c[4]), depth_min=float(np.float32(c[5])),
                depth_max=float(np.float32(c[6])))


def _load(ctx, gmap, entries, voxels, nvis):
    """Writes a hash table, the first len(voxels) voxels and the visible
    count into a device map."""
    a = gmap.arrays()
    entries = np.ascontiguousarray(entries)
    voxels = np.ascontiguousarray(voxels)
    ctx.memcpy(a.hash_entries, entries.ctypes.data, entries.nbytes)
    ctx.memcpy(a.voxel_blocks, voxels.ctypes.data, voxels.nbytes)
    n = np.array([nvis], np.uint32)
    ctx.memcpy(a.no_visible_blocks, n.ctypes.data, 4)


def _voxel_bytes(ctx, gmap, n):
    return ctx.download(gmap.arrays().voxel_blocks, np.uint8, n * 16).reshape(n, 16)


def test_unify_golden(lib):
    """The reference kernel's output on the seeded state: excess-list
    chains, full neighbour tables, zero counts, the count_2 + 5 wrap."""
    sf, ctx = lib
    g = dict(np.load(G1))
    vox = g["uni_vox"]
    for k, nvis in enumerate(g["uni_nvis"]):
        gmap = sf.Map(**_g1_cfg(g))
        _load(ctx, gmap, g["uni_entries"], vox, int(nvis))
        sf.call("sf_UnifyNeighbor", ctx.h, gmap.h)
        got = _voxel_bytes(ctx, gmap, len(vox))
        assert np.array_equal(got[:, 8:12], g["uni_out%d" % k]), "nvis %d" % nvis
        assert np.array_equal(np.delete(got, [8, 9, 10, 11], 1), np.delete(vox, [8, 9, 10, 11], 1))
        gmap.close()


def _fused_oracle_state(K, n, seed):
    """An oracle map after n FuseMapColor frames with labels, then the
    visibility pass of the next pose."""
    from oracle import oracle as O
    cfg = C1
    seq = sequence(cfg["cols"], cfg["rows"], K, n + 1, trajectory=0, label_flip=0.05, n_objects=10, seed=seed)
    om = O.Map(**MAP_SMALL)
    for i in range(n):
        d, rgb, mask, P = seq[i]
        raw, filt = O.filter_depth(d, 1000.0, 3.0)
        nm = O.nmap(O.vmap(filt, *K, 3.0))
        om.fuse(raw, rgb, nm, mask, 10, P, K)
    om.visibility(seq[n][3], K, cfg["cols"], cfg["rows"])
    return om


def test_unify_matches_oracle_on_fused_state(lib):
    """Two passes in a row from a fused label state (320x240, 4 frames)."""
    sf, ctx = lib
    K = C1["K"]
    om = _fused_oracle_state(K, 4, seed=5)
    nvis = int(om.counters()[2])
    e = om.entries.copy()
    nvox = int(e["ptr"].max()) + 512
    gmap = sf.Map(**MAP_SMALL)
    _load(ctx, gmap, e, om.voxels[:nvox].copy(), nvis)
    for rep in range(2):
        before = om.voxels[:nvox].copy()
        sf.call("sf_UnifyNeighbor", ctx.h, gmap.h)
        om.unify_neighbor()
        got = _voxel_bytes(ctx, gmap, nvox)
        want = om.voxels[:nvox].view(np.uint8).reshape(nvox, 16)
        assert np.array_equal(got, want), "pass %d" % rep
        changed = (want[:, 8:12] != before.view(np.uint8).reshape(nvox, 16)[:, 8:12]).any(1).sum()
        if rep == 0:
            assert changed > 500
    gmap.close()


def test_unify_visible_count_edges(lib):
    """A visible count of 0 changes nothing; one beyond the table is the
    whole table (the kernel's hashEntries.size bound)."""
    sf, ctx = lib
    g = dict(np.load(G1))
    vox = g["uni_vox"]
    gmap = sf.Map(**_g1_cfg(g))
    _load(ctx, gmap, g["uni_entries"], vox, 0)
    sf.call("sf_UnifyNeighbor", ctx.h, gmap.h)
    assert np.array_equal(_voxel_bytes(ctx, gmap, len(vox)), vox)
    _load(ctx, gmap, g["uni_entries"], vox, 0xffffffff)
    sf.call("sf_UnifyNeighbor", ctx.h, gmap.h)
    assert int(g["uni_nvis"][1]) == gmap.num_entries
    assert np.array_equal(_voxel_bytes(ctx, gmap, len(vox))[:, 8:12], g["uni_out1"])
    gmap.close()


def test_frame_graph_runs_unify(lib):
    """The system loop with detections runs the pass (inside the second,
    labelled FuseColor of the semantic mode), in graph and plain form; the
    label state it leaves is a fixed input the oracle's pass reproduces on
    the same layout."""
    from oracle import oracle as O
    sf, ctx = lib
    K = C1["K"]
    seq = sequence(C1["cols"], C1["rows"], K, 4, trajectory=0, label_flip=0.05, n_objects=10, seed=9)
    per_frame = {}
    for mode in (1, 0):
        for ndet in (0, 10):
            cfg = sf.system_config(cols=C1["cols"], rows=C1["rows"], K=K, use_graph=mode, **MAP_SMALL)
            s = sf.System(ctx, cfg, init_pose=seq[0][3])
            counts = []
            for d, rgb, mask, _ in seq:
                n0 = C.c_uint64()
                sf.call("sf_kernel_launches", C.byref(n0))
                st = s.grab(d, rgb, mask, ndet)
                n1 = C.c_uint64()
                sf.call("sf_kernel_launches", C.byref(n1))
                counts.append(n1.value - n0.value)
                assert st.flags == 0
            per_frame[(mode, ndet)] = counts[-1]
            if ndet:
                m = s.map()
                e, v, _ = map_to_host(ctx, m)
                assert (v["label"][v["weight"] > 0] > 0).sum() > 100
                # one more pass from this state, on the device and the oracle
                om = O.Map(**MAP_SMALL)
                nvox = int(e["ptr"].max()) + 512
                om.entries[:] = e
                om.voxels[:nvox] = v[:nvox]
                nvis = int(m.counters(ctx)[2])
                sf.call("sf_UnifyNeighbor", ctx.h, m.h)
                om.unify_neighbor(nvis)
                got = _voxel_bytes(ctx, m, nvox)
                assert np.array_equal(got, om.voxels[:nvox].view(np.uint8).reshape(nvox, 16))
            s.close()
    # with detections the frame graph runs FuseColor again with the labels
    # (allocation 3 launches, the insert launch also starting the visibility
    # pass, visibility 1, integration 1, UnifyNeighbor 3) and RayTrace (1),
    # System.cc:184-205.  (The plain form's count also follows the ICP
    # iterations, which differ between the two maps.)
    assert per_frame[(1, 10)] == per_frame[(1, 0)] + 9
