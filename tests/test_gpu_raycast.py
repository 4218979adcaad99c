"""GPU parity of the rendering-block z-range and the block-skipping raycast
(Mapping/RenderScene.cu) against the oracle, on maps fused identically.

z-range images and vertex / normal maps are compared bit-exact (NaN-aware).
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, C2, MAP_C1, MAP_C2, cuda, empty, host, same_nan, sequence
from tests.test_gpu_fusion import _frame_inputs

pytestmark = pytest.mark.gpu

RAYCAST_DEPTH_TOL = 1e-4  # metres (the bar for rendered depth); the test also asserts bit-exactness


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


@pytest.mark.parametrize("cfg,mcfg,nframes", [(C1, MAP_C1, 5), (C2, MAP_C2, 3)])
def test_zrange_and_raycast_bit_exact(lib, cfg, mcfg, nframes):
    import torch
    from oracle import oracle as O
    sf, ctx = lib
    K = cfg["K"]
    cols, rows = cfg["cols"], cfg["rows"]
    seq = sequence(cols, rows, K, nframes + 1, trajectory=1, dropout=0.02)
    gmap = sf.Map(**mcfg)
    omap = O.Map(**mcfg)
    for i in range(nframes):
        d, rgb, mask, P = seq[i]
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        R, RI, t = sf.pose_to_gpu(P)
        nvis = C.c_uint32()
        sf.call("sf_FuseMapColor", ctx.h, gmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
                sf.image(f["mask"]), 0, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
        omap.fuse(f["raw_h"], rgb, f["nmap_h"], None, 0, P, K)
    # render from the last fused pose and from the next (unfused) pose
    for P in (seq[nframes - 1][3], seq[nframes][3]):
        R, RI, t = sf.pose_to_gpu(P)
        nvis = C.c_uint32()
        sf.call("sf_CheckBlockVisibility", ctx.h, gmap.h, R, RI, t, cols, rows, *K, 3.0, 0.1, C.byref(nvis))
        onv = omap.visibility(P, K, cols, rows)
        assert nvis.value == onv > 0
        zc, zr = (cols + 7) // 8, (rows + 7) // 8
        zmin = empty((zr, zc), torch.float32)
        zmax = empty((zr, zc), torch.float32)
        blocks = empty((mcfg.get("max_rendering_blocks", 260000), 16), torch.uint8)
        nblk = empty((1,), torch.int32)
        ok = C.c_int()
        sf.call("sf_CreateRenderingBlocks", ctx.h, gmap.h, sf.image(zmin), sf.image(zmax), 3.0, 0.1,
                blocks.data_ptr(), nblk.data_ptr(), RI, t, nvis.value, *K, C.byref(ok))
        ook, ozmin, ozmax, oblocks, on = omap.zrange(P, K, zc, zr, max_blocks=1)
        assert bool(ok.value) == ook
        assert int(host(nblk)[0]) == on
        assert same_nan(host(zmin), ozmin)
        assert same_nan(host(zmax), ozmax)
        vm = empty((rows, cols, 4), torch.float32)
        nm = empty((rows, cols, 4), torch.float32)
        invfx = float(np.float32(1.0 / np.float64(np.float32(K[0]))))
        invfy = float(np.float32(1.0 / np.float64(np.float32(K[1]))))
        sf.call("sf_Raycast", ctx.h, gmap.h, sf.image(vm), sf.image(nm), sf.image(zmin), sf.image(zmax), R, RI, t,
                invfx, invfy, K[2], K[3])
        ctx.sync()
        ovm, onm = O.Map.raycast(omap, P, K, cols, rows, ozmin, ozmax)
        gv, gn = host(vm), host(nm)
        valid = np.isfinite(ovm[..., 0])
        assert valid.mean() > 0.5
        assert same_nan(gv, ovm)
        assert same_nan(gn, onm)
        both = valid & np.isfinite(gv[..., 0])
        assert np.abs(gv[both][:, 2] - ovm[both][:, 2]).max() <= RAYCAST_DEPTH_TOL
    gmap.close()
