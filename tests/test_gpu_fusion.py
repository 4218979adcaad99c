"""GPU parity of allocation, visibility, TSDF/colour integration and label
fusion (Mapping/DeviceMap.cu, Mapping/FuseMap.cu) against the oracle.

Compared as sets keyed by block position (heap pointers and list orders are
not deterministic in the reference either): allocated blocks, the visible
set, heapCounter / entryPtr, and every voxel's bytes (sdf, weight, colour,
label, count, label_2, count_2, colour_2) - all bit-exact.
"""
import numpy as np
import pytest

from tests.helpers import C1, C2, MAP_C1, MAP_C2, adopt_layout, cuda, empty, host, map_to_host, positions, sequence, \
    voxels_by_pos

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _frame_inputs(sf, ctx, d, rgb, mask, K):
    """Raw depth and level-0 normal map computed on the GPU (FillImages)."""
    import torch
    from oracle import oracle as O
    dd = cuda(d)
    raw = empty(d.shape, torch.float32)
    filt = empty(d.shape, torch.float32)
    vm = empty(d.shape + (4,), torch.float32)
    nm = empty(d.shape + (4,), torch.float32)
    sf.call("sf_FilterDepth", ctx.h, sf.image(dd), sf.image(raw), sf.image(filt), 1000.0, 3.0)
    sf.call("sf_ComputeVMap", ctx.h, sf.image(filt), sf.image(vm), *K, 3.0)
    sf.call("sf_ComputeNMap", ctx.h, sf.image(vm), sf.image(nm))
    ctx.sync()
    return dict(raw=raw, rgb=cuda(rgb), nmap=nm, mask=cuda(mask), raw_h=host(raw), nmap_h=host(nm))


def _compare_maps(ctx, gmap, omap, check_visible=True):
    e, v, vis = map_to_host(ctx, gmap)
    oe, ov = omap.entries.copy(), omap.voxels.copy()
    gc = gmap.counters(ctx)
    oc = omap.counters()
    # allocated block positions, heap and excess counters
    assert positions(e[e["ptr"] >= 0]) == positions(oe[oe["ptr"] >= 0])
    assert gc[0] == oc[0], "heapCounter"
    assert gc[1] == oc[1], "entryPtr"
    assert gc[3] == oc[3], "allocated count"
    if check_visible:
        assert gc[2] == oc[2], "visible count"
        assert positions(vis[:gc[2]]) == positions(omap.visible[:oc[2]])
    # voxel bytes per block position
    kg, vg = voxels_by_pos(e, v)
    ko, vo = voxels_by_pos(oe, ov)
    assert kg == ko
    assert np.array_equal(vg.view(np.uint8), vo.view(np.uint8))
    return len(kg)


@pytest.mark.parametrize("cfg,mcfg,dropout,nframes", [(C1, MAP_C1, 0.0, 4), (C2, MAP_C2, 0.02, 3)])
def test_fuse_sequence_bit_exact(lib, cfg, mcfg, dropout, nframes):
    """FuseMapColor over several frames at ground-truth poses."""
    from oracle import oracle as O
    sf, ctx = lib
    K = cfg["K"]
    seq = sequence(cfg["cols"], cfg["rows"], K, nframes, trajectory=1, dropout=dropout)
    gmap = sf.Map(**mcfg)
    omap = O.Map(**mcfg)
    import ctypes as C
    for i in range(nframes):
        d, rgb, mask, P = seq[i]
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        R, RI, t = sf.pose_to_gpu(P)
        nvis = C.c_uint32()
        empty_img = sf.image(f["mask"])
        sf.call("sf_FuseMapColor", ctx.h, gmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
                empty_img, 0, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
        onv = omap.fuse(f["raw_h"], rgb, f["nmap_h"], None, 0, P, K)
        assert nvis.value == onv
        nblocks = _compare_maps(ctx, gmap, omap)
        assert nblocks > 100
    gmap.close()


@pytest.mark.parametrize("cfg,mcfg,nframes", [(C1, MAP_C1, 5), (C2, MAP_C2, 3)])
def test_label_fusion_bit_exact(lib, cfg, mcfg, nframes):
    """FuseMapColor with instance masks: label / count / label_2 / count_2.
    The 640x480 case is the label-fusion workload: class ids 0-80, ten
    projected primitives per frame, 5% random label flips."""
    from oracle import oracle as O
    import ctypes as C
    sf, ctx = lib
    K = cfg["K"]
    seq = sequence(cfg["cols"], cfg["rows"], K, nframes, trajectory=0, label_flip=0.05, n_objects=10, seed=5)
    gmap = sf.Map(**mcfg)
    omap = O.Map(**mcfg)
    labels = set()
    for i in range(nframes):
        d, rgb, mask, P = seq[i]
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        R, RI, t = sf.pose_to_gpu(P)
        nvis = C.c_uint32()
        sf.call("sf_FuseMapColor", ctx.h, gmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
                sf.image(f["mask"]), 10, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
        # UnifyNeighbor visits hash slots [0, visible count): on the device layout
        omap.fuse(f["raw_h"], rgb, f["nmap_h"], mask, 10, P, K, unify=False)
        adopt_layout(omap, map_to_host(ctx, gmap)[0])
        omap.unify_neighbor()
        _compare_maps(ctx, gmap, omap)
        labels |= set(np.unique(mask).tolist())
    e, v, _ = map_to_host(ctx, gmap)
    assert (v["count"] > 0).sum() > 1000 and (v["label"] > 0).sum() > 100
    assert max(labels) <= 80 and len(labels) > 40  # flipped labels span the 0-80 ids
    gmap.close()


def test_analyze_semantics_and_visibility(lib):
    from oracle import oracle as O
    import ctypes as C
    sf, ctx = lib
    cfg = C1
    K = cfg["K"]
    seq = sequence(cfg["cols"], cfg["rows"], K, 3, trajectory=0, label_flip=0.05, n_objects=10, seed=5)
    gmap = sf.Map(**MAP_C1)
    omap = O.Map(**MAP_C1)
    for i in range(2):
        d, rgb, mask, P = seq[i]
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        R, RI, t = sf.pose_to_gpu(P)
        nvis = C.c_uint32()
        sf.call("sf_FuseMapColor", ctx.h, gmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
                sf.image(f["mask"]), 0, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
        omap.fuse(f["raw_h"], rgb, f["nmap_h"], None, 0, P, K)
    d, rgb, mask, P = seq[2]
    f = _frame_inputs(sf, ctx, d, rgb, mask, K)
    R, RI, t = sf.pose_to_gpu(P)
    # CheckBlockVisibility alone
    nvis = C.c_uint32()
    sf.call("sf_CheckBlockVisibility", ctx.h, gmap.h, R, RI, t, cfg["cols"], cfg["rows"], *K, 3.0, 0.1,
            C.byref(nvis))
    onv = omap.visibility(P, K, cfg["cols"], cfg["rows"])
    assert nvis.value == onv
    _compare_maps(ctx, gmap, omap)
    # AnalyzeMapSemantics: visibility + label pass, num_detection 10
    sf.call("sf_AnalyzeMapSemantics", ctx.h, gmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
            sf.image(f["mask"]), 10, R, RI, t, *K, 3.0, 0.1)
    omap.visibility(P, K, cfg["cols"], cfg["rows"])
    omap.semantics(f["raw_h"], rgb, f["nmap_h"], mask, 10, P, K)
    adopt_layout(omap, map_to_host(ctx, gmap)[0])
    omap.unify_neighbor()
    _compare_maps(ctx, gmap, omap)
    gmap.close()


def test_small_heap_and_excess_overflow(lib):
    """Heap of 64 blocks and 16 excess slots: counters follow the reference
    (one heap pop per distinct requested block), nothing faults."""
    from oracle import oracle as O
    import ctypes as C
    sf, ctx = lib
    cfg = C1
    K = cfg["K"]
    small = dict(voxel_size=0.01, trunc_dist=0.03, num_buckets=64, num_excess=16, num_sdf_blocks=64)
    seq = sequence(cfg["cols"], cfg["rows"], K, 1)
    d, rgb, mask, P = seq[0]
    f = _frame_inputs(sf, ctx, d, rgb, mask, K)
    gmap = sf.Map(**small)
    R, RI, t = sf.pose_to_gpu(P)
    nvis = C.c_uint32()
    sf.call("sf_FuseMapColor", ctx.h, gmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
            sf.image(f["mask"]), 0, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
    gc = gmap.counters(ctx)
    flags = ctx.flags()
    assert gc[3] <= 64 and gc[0] < 0  # heap exhausted
    assert flags & (1 << 2)           # SF_FLAG_HEAP_EMPTY recorded
    e, v, _ = map_to_host(ctx, gmap)
    assert (e["ptr"] >= 0).sum() == gc[3]
    assert len(set(e[e["ptr"] >= 0]["ptr"].tolist())) == gc[3]  # no heap block handed out twice
    gmap.close()


def test_reset_map(lib):
    import ctypes as C
    sf, ctx = lib
    gmap = sf.Map(**MAP_C1)
    sf.call("sf_ResetMap", ctx.h, gmap.h)
    ctx.sync()
    gc = gmap.counters(ctx)
    assert gc == [MAP_C1["num_sdf_blocks"] - 1, 1, 0, 0]
    a = gmap.arrays()
    heap = ctx.download(a.heap_mem, np.int32, MAP_C1["num_sdf_blocks"])
    assert np.array_equal(heap, np.arange(MAP_C1["num_sdf_blocks"] - 1, -1, -1, dtype=np.int32))
    gmap.close()
