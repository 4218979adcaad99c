"""GPU kernels against the reference's own outputs (tests/golden/g1.npz,
produced by the reference's device code; see tests/golden/make_golden.py).

Same checks as tests/test_oracle_golden.py, with the CUDA path in place of
the oracle: bit-exact except the bilateral filter (CUDA expf vs the host
libm expf the fixture was made with; FILTER_RTOL).
"""
import ctypes as C
import hashlib
import os

import numpy as np
import pytest

from tests.helpers import adopt_layout, cuda, empty, host, map_to_host, same_nan

pytestmark = pytest.mark.gpu

G1 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "g1.npz")
FILTER_RTOL = 2e-6


@pytest.fixture(scope="module")
def env(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    g = dict(np.load(G1))
    yield sf, ctx, g
    ctx.close()


def _K(g, level=0):
    div = float(1 << level)
    return tuple(float(k) / div for k in g["K"])


def test_pyramid_vs_reference(env):
    import torch
    sf, ctx, g = env
    for i in range(2):
        d = g["depth%d" % i]
        dd = cuda(d)
        raw = empty(d.shape, torch.float32)
        filt = empty(d.shape, torch.float32)
        sf.call("sf_FilterDepth", ctx.h, sf.image(dd), sf.image(raw), sf.image(filt), 1000.0, 3.0)
        ctx.sync()
        assert same_nan(host(raw), g["raw%d" % i])
        f = host(filt)
        ok = ~np.isnan(g["filt%d" % i])
        assert np.array_equal(ok, ~np.isnan(f))
        np.testing.assert_allclose(f[ok], g["filt%d" % i][ok], rtol=FILTER_RTOL)
        for l in range(3):
            src = cuda(g["f%d_depth%d" % (i, l)])
            rows, cols = src.shape
            vm = empty((rows, cols, 4), torch.float32)
            nm = empty((rows, cols, 4), torch.float32)
            sf.call("sf_ComputeVMap", ctx.h, sf.image(src), sf.image(vm), *_K(g, l), 3.0)
            sf.call("sf_ComputeNMap", ctx.h, sf.image(vm), sf.image(nm))
            ctx.sync()
            rv = g["f%d_vmap%d" % (i, l)]
            valid = ~np.isnan(rv[..., 0])
            gv = host(vm)
            assert np.array_equal(valid, ~np.isnan(gv[..., 0]))
            assert np.array_equal(gv[valid], rv[valid])
            assert same_nan(host(nm), g["f%d_nmap%d" % (i, l)])
            if l < 2:
                dst = empty((rows // 2, cols // 2), torch.float32)
                sf.call("sf_PyrDownGauss", ctx.h, sf.image(src), sf.image(dst))
                ctx.sync()
                assert same_nan(host(dst), g["f%d_depth%d" % (i, l + 1)])


def test_resize_vs_reference(env):
    import torch
    sf, ctx, g = env
    vs, ns = cuda(g["resize_vsrc"]), cuda(g["resize_nsrc"])
    r, c = g["resize_vdst"].shape[:2]
    vd = empty((r, c, 4), torch.float32)
    nd = empty((r, c, 4), torch.float32)
    sf.call("sf_ResizeMap", ctx.h, sf.image(vs), sf.image(ns), sf.image(vd), sf.image(nd))
    ctx.sync()
    assert same_nan(host(vd), g["resize_vdst"])
    assert same_nan(host(nd), g["resize_ndst"])


def test_icp_vs_reference(env):
    sf, ctx, g = env
    Rc, _, tc = sf.pose_to_gpu(g["icp_pose_curr"])
    Rl, RlI, tl = sf.pose_to_gpu(g["pose0"])
    for l in range(3):
        v1, v0 = cuda(g["f1_vmap%d" % l]), cuda(g["f0_vmap%d" % l])
        n1, n0 = cuda(g["f1_nmap%d" % l]), cuda(g["f0_nmap%d" % l])
        res = (C.c_float * 2)()
        A = (C.c_double * 36)()
        b = (C.c_double * 6)()
        sf.call("sf_ICPStep", ctx.h, sf.image(v1), sf.image(v0), sf.image(n1), sf.image(n0), Rc, tc, Rl, RlI, tl,
                sf.Intrinsics(*_K(g, l)), res, A, b)
        s = g["icp_sums%d" % l]
        assert res[1] == s[28]
        assert abs(res[0] - s[27]) <= 2e-6 * abs(s[27])
        diag = np.abs(s[[0, 7, 13, 18, 22, 25]]).max()
        k = 0
        for i in range(6):
            for j in range(i, 7):
                got = b[i] if j == 6 else A[i * 6 + j]
                tol = 2e-6 * (np.sqrt(diag * s[27]) if j == 6 else diag)
                assert abs(got - s[k]) <= tol + 2e-6 * abs(s[k])
                k += 1


def _gpu_frame(sf, ctx, g, i):
    import torch
    d = g["depth%d" % i]
    dd = cuda(d)
    raw = empty(d.shape, torch.float32)
    filt = empty(d.shape, torch.float32)
    vm = empty(d.shape + (4,), torch.float32)
    nm = empty(d.shape + (4,), torch.float32)
    sf.call("sf_FilterDepth", ctx.h, sf.image(dd), sf.image(raw), sf.image(filt), 1000.0, 3.0)
    sf.call("sf_ComputeVMap", ctx.h, sf.image(filt), sf.image(vm), *_K(g), 3.0)
    sf.call("sf_ComputeNMap", ctx.h, sf.image(vm), sf.image(nm))
    ctx.sync()
    return raw, vm, nm


def _digests(e, v):
    sel = e[e["ptr"] >= 0]
    order = np.lexsort((sel["z"], sel["y"], sel["x"]))
    sel = sel[order]
    pos = np.stack([sel["x"], sel["y"], sel["z"]], 1).astype(np.int32)
    vox = v.view(np.uint8)
    dig = np.stack([np.frombuffer(hashlib.sha1(vox[p * 16:(p + 512) * 16].tobytes()).digest(), np.uint8)
                    for p in sel["ptr"]])
    return pos, dig


def _gpu_map(sf, g):
    c = g["consts"]
    return sf.Map(voxel_size=float(np.float32(c[0])), trunc_dist=float(np.float32(c[1])), num_buckets=int(c[2]),
                  num_excess=int(c[3]), num_sdf_blocks=int(c[4]), depth_min=float(np.float32(c[5])),
                  depth_max=float(np.float32(c[6])))


def _oracle_map(g):
    from oracle import oracle as O
    c = g["consts"]
    return O.Map(voxel_size=float(np.float32(c[0])), trunc_dist=float(np.float32(c[1])), num_buckets=int(c[2]),
                 num_excess=int(c[3]), num_sdf_blocks=int(c[4]), depth_min=float(np.float32(c[5])),
                 depth_max=float(np.float32(c[6])))


def test_map_and_raytrace_vs_reference(env):
    """FuseMapColor x5 (labels from frame 2), then z-range + raycast from two
    poses: filtered depth differs by ulps, so the GPU fuses from its own raw
    depth (bit-exact) and the reference's normal maps.

    The UnifyNeighbor pass of the labelled frames visits hash slots
    [0, visible count), whose holders follow allocation order (a race on the
    GPU), so the voxel bytes are checked against the oracle (pinned to these
    fixtures by tests/test_oracle_golden.py) on the device map's slot layout;
    the block set, counters and visible sets against the fixtures directly."""
    import torch
    sf, ctx, g = env
    m = _gpu_map(sf, g)
    om = _oracle_map(g)
    cols, rows = g["depth0"].shape[1], g["depth0"].shape[0]
    from oracle import oracle as O
    for i in range(5):
        raw, _, _ = _gpu_frame(sf, ctx, g, i)
        oraw, filt = O.filter_depth(g["depth%d" % i], 1000.0, 3.0)
        nm_h = O.nmap(O.vmap(filt, *_K(g), 3.0))  # oracle == reference here (pinned)
        nm = cuda(nm_h)
        R, RI, t = sf.pose_to_gpu(g["pose%d" % i])
        nvis = C.c_uint32()
        ndet = 10 if i >= 2 else 0
        rgb, mask = cuda(g["rgb%d" % i]), cuda(g["mask%d" % i])  # keep the device buffers alive
        sf.call("sf_FuseMapColor", ctx.h, m.h, sf.image(raw), sf.image(rgb), sf.image(nm),
                sf.image(mask), ndet, R, RI, t, *_K(g), 3.0, 0.1, C.byref(nvis))
        cnt = m.counters(ctx)
        ref = g["counters"][i]
        assert cnt[0] == ref[0] and cnt[1] == ref[1] and cnt[3] == ref[3], "frame %d" % i
        assert nvis.value == ref[2]
        e, v, vis = map_to_host(ctx, m)
        got = np.sort(np.stack([vis["x"][:nvis.value], vis["y"][:nvis.value], vis["z"][:nvis.value]], 1)
                      .astype(np.int32).view([("x", "<i4"), ("y", "<i4"), ("z", "<i4")]).ravel())
        assert np.array_equal(got, g["visible%d" % i])
        om.fuse(host(raw), g["rgb%d" % i], nm_h, g["mask%d" % i], ndet, g["pose%d" % i], _K(g), unify=False)
        if ndet > 0:
            adopt_layout(om, e)
            om.unify_neighbor()
    e, v, _ = map_to_host(ctx, m)
    pos, dig = _digests(e, v)
    assert np.array_equal(pos, g["map_pos"])
    opos, odig = _digests(om.entries, om.voxels)
    assert np.array_equal(pos, opos)
    assert np.array_equal(dig, odig)
    for k, fi in enumerate((4, 5)):
        R, RI, t = sf.pose_to_gpu(g["pose%d" % fi])
        nvis = C.c_uint32()
        sf.call("sf_CheckBlockVisibility", ctx.h, m.h, R, RI, t, cols, rows, *_K(g), 3.0, 0.1, C.byref(nvis))
        assert nvis.value == int(g["ray%d_nvis" % k])
        zmin = empty((60, 80), torch.float32)
        zmax = empty((60, 80), torch.float32)
        blocks = empty((260000, 16), torch.uint8)
        nblk = empty((1,), torch.int32)
        ok = C.c_int()
        sf.call("sf_CreateRenderingBlocks", ctx.h, m.h, sf.image(zmin), sf.image(zmax), 3.0, 0.1,
                blocks.data_ptr(), nblk.data_ptr(), RI, t, nvis.value, *_K(g), C.byref(ok))
        assert ok.value == int(g["ray%d_ok" % k])
        assert int(host(nblk)[0]) == int(g["ray%d_nblocks" % k])
        assert same_nan(host(zmin), g["ray%d_zmin" % k])
        assert same_nan(host(zmax), g["ray%d_zmax" % k])
        vm = empty((rows, cols, 4), torch.float32)
        nmo = empty((rows, cols, 4), torch.float32)
        K = _K(g)
        invfx = float(np.float32(1.0 / np.float64(np.float32(K[0]))))
        invfy = float(np.float32(1.0 / np.float64(np.float32(K[1]))))
        sf.call("sf_Raycast", ctx.h, m.h, sf.image(vm), sf.image(nmo), sf.image(zmin), sf.image(zmax), R, RI, t,
                invfx, invfy, K[2], K[3])
        ctx.sync()
        assert ok.value == 1  # the reference raycasts only then (Mapping.cc:152-160)
        assert same_nan(host(vm), g["ray%d_vmap" % k])
        assert same_nan(host(nmo), g["ray%d_nmap" % k])
    m.close()
