"""GPU parity of the depth pyramid against the oracle (Tracking/Pyrdown.cu).

Bit-exact except the bilateral filter, whose 25 exp() per pixel use CUDA's
expf on the GPU and glibc's on the CPU (both within 2 ulp); its tolerance is
stated below.  Every later stage is checked bit-exact from identical inputs.
"""
import numpy as np
import pytest

from tests.helpers import C1, C2, cuda, empty, host, same_nan, sequence

pytestmark = pytest.mark.gpu

# bilateral filter: relative tolerance for CUDA expf vs glibc expf
FILTER_RTOL = 2e-6


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


@pytest.mark.parametrize("cfg,dropout", [(C1, 0.0), (C2, 0.02)])
def test_filter_depth(lib, cfg, dropout):
    import torch
    from oracle import oracle as O
    sf, ctx = lib
    d, _, _, _ = sequence(cfg["cols"], cfg["rows"], cfg["K"], 1, dropout=dropout)[0]
    dd = cuda(d.astype(np.uint16))
    raw = empty(d.shape, torch.float32)
    filt = empty(d.shape, torch.float32)
    sf.call("sf_FilterDepth", ctx.h, sf.image(dd), sf.image(raw), sf.image(filt), 1000.0, 3.0)
    ctx.sync()
    o_raw, o_filt = O.filter_depth(d, 1000.0, 3.0)
    assert same_nan(host(raw), o_raw)
    g = host(filt)
    assert np.array_equal(np.isnan(g), np.isnan(o_filt))
    ok = ~np.isnan(g)
    np.testing.assert_allclose(g[ok], o_filt[ok], rtol=FILTER_RTOL, atol=0)


@pytest.mark.parametrize("cfg", [C1, C2])
def test_pyramid_levels_bit_exact(lib, cfg):
    """PyrDownGauss, ComputeVMap, ComputeNMap from identical filtered depth."""
    import torch
    from oracle import oracle as O
    sf, ctx = lib
    d, _, _, _ = sequence(cfg["cols"], cfg["rows"], cfg["K"], 1, dropout=0.02)[0]
    _, f0 = O.filter_depth(d, 1000.0, 3.0)
    K = cfg["K"]
    src = cuda(f0)
    for level in range(3):
        rows, cols = src.shape
        div = float(1 << level)
        vm = empty((rows, cols, 4), torch.float32)
        nm = empty((rows, cols, 4), torch.float32)
        sf.call("sf_ComputeVMap", ctx.h, sf.image(src), sf.image(vm), K[0] / div, K[1] / div, K[2] / div,
                K[3] / div, 3.0)
        sf.call("sf_ComputeNMap", ctx.h, sf.image(vm), sf.image(nm))
        ctx.sync()
        s_host = host(src)
        o_vm = O.vmap(s_host, K[0] / div, K[1] / div, K[2] / div, K[3] / div, 3.0)
        o_nm = O.nmap(o_vm)
        assert same_nan(host(vm), o_vm), "vmap level %d" % level
        assert same_nan(host(nm), o_nm), "nmap level %d" % level
        if level < 2:
            dst = empty((rows // 2, cols // 2), torch.float32)
            sf.call("sf_PyrDownGauss", ctx.h, sf.image(src), sf.image(dst))
            ctx.sync()
            assert same_nan(host(dst), O.pyrdown(s_host)), "pyrdown level %d" % (level + 1)
            src = dst


@pytest.mark.parametrize("cols,rows,levels", [(640, 480, 3), (320, 240, 2), (1280, 720, 4), (100, 75, 3),
                                              (37, 29, 3), (64, 48, 1)])
def test_build_pyramid_fused_matches_oracle(lib, cols, rows, levels):
    """sf_BuildPyramid (bilateral filter, then one launch for the coarser
    levels and every level's vertex and normal maps) against the oracle's
    PyrDownGauss / ComputeVMap / ComputeNMap chain, bit-exact, on full and
    ragged sizes (tiles cut by the image edge, odd level sizes)."""
    import torch
    from oracle import oracle as O
    sf, ctx = lib
    f = cols / 640.0
    K = (525.0 * f, 525.0 * f, cols / 2 - 0.5, rows / 2 - 0.5)
    d, _, _, _ = sequence(cols, rows, K, 1, dropout=0.02)[0]
    dd = cuda(d)
    raw = empty(d.shape, torch.float32)
    depths = [empty((d.shape[0] >> l, d.shape[1] >> l), torch.float32) for l in range(levels)]
    vms = [empty((d.shape[0] >> l, d.shape[1] >> l, 4), torch.float32) for l in range(levels)]
    nms = [empty((d.shape[0] >> l, d.shape[1] >> l, 4), torch.float32) for l in range(levels)]
    arr = lambda ts: (sf.Image * levels)(*[sf.image(t) for t in ts])
    sf.call("sf_BuildPyramid", ctx.h, sf.image(dd), sf.image(raw), arr(depths), arr(vms), arr(nms), levels,
            sf.Intrinsics(*K), 1000.0, 3.0)
    ctx.sync()
    assert np.isfinite(host(depths[0])).mean() > 0.5
    for l in range(levels):
        div = float(1 << l)
        dh = host(depths[l])
        o_vm = O.vmap(dh, K[0] / div, K[1] / div, K[2] / div, K[3] / div, 3.0)
        assert same_nan(host(vms[l]), o_vm), "vmap level %d" % l
        assert same_nan(host(nms[l]), O.nmap(o_vm)), "nmap level %d" % l
        if l > 0:
            assert same_nan(dh, O.pyrdown(host(depths[l - 1]))), "pyrdown level %d" % l


def test_resize_map_bit_exact(lib):
    """ResizeMap on raycast-like maps, float4 normal norm including w."""
    import torch
    from oracle import oracle as O
    sf, ctx = lib
    rng = np.random.default_rng(3)
    rows, cols = 240, 320
    v = rng.normal(size=(rows, cols, 4)).astype(np.float32)
    v[..., 3] = 1.0
    n = rng.normal(size=(rows, cols, 4)).astype(np.float32)
    n[..., :3] /= np.linalg.norm(n[..., :3], axis=-1, keepdims=True)
    n[..., 3] = 1.0
    holes = rng.random((rows, cols)) < 0.05
    v[holes] = np.nan
    n[rng.random((rows, cols)) < 0.05] = np.nan
    vs, ns = cuda(v), cuda(n)
    vd = empty((rows // 2, cols // 2, 4), torch.float32)
    nd = empty((rows // 2, cols // 2, 4), torch.float32)
    sf.call("sf_ResizeMap", ctx.h, sf.image(vs), sf.image(ns), sf.image(vd), sf.image(nd))
    ctx.sync()
    ov, on = O.resize(v, n)
    assert same_nan(host(vd), ov)
    assert same_nan(host(nd), on)


def test_invalid_arguments_rejected(lib):
    import torch
    sf, ctx = lib
    a = empty((8, 8), torch.float32)
    b = empty((4, 4), torch.float32)
    with pytest.raises(sf.SfError):
        sf.call("sf_FilterDepth", ctx.h, sf.image(empty((8, 8), torch.int16)), sf.image(a), sf.image(b), 1000.0, 3.0)
    with pytest.raises(sf.SfError):
        sf.call("sf_PyrDownGauss", ctx.h, sf.image(b), sf.image(a))
