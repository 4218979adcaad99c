"""GPU parity of the photometric (RGB) term: the intensity pyramid and
derivative images (Tracking/Pyrdown.cu:201-316), RGBStep
(Tracking/Reduction.cu:387-642) and ComputeSE3 with icpOnly = false
(Tracking/Tracking.cc:369-517), against the reference's own kernels
(tests/golden/g1.npz) and the oracle.

Images are bit-exact.  The correspondence count is exact; the 29 sums agree
to SUMS_RTOL (FP32 rows, compensated sums on the GPU, FP64 in the oracle);
the pose of the whole loop to POSE_TOL.
"""
import ctypes as C
import os

import numpy as np
import pytest

from tests.helpers import C2, cuda, empty, host, sequence

pytestmark = pytest.mark.gpu

G1 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "g1.npz")
SUMS_RTOL = 2e-6
POSE_TOL = 1e-6


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _gpu_intensity(sf, ctx, rgb, levels=3):
    """Intensity pyramid and derivative images through the C ABI."""
    import torch
    c = cuda(rgb)
    rows, cols = rgb.shape[:2]
    imgs = [empty((rows >> l, cols >> l), torch.uint8) for l in range(levels)]
    dxs = [empty((rows >> l, cols >> l), torch.int16) for l in range(levels)]
    dys = [empty((rows >> l, cols >> l), torch.int16) for l in range(levels)]
    sf.call("sf_ImageToIntensity", ctx.h, sf.image(c, 3), sf.image(imgs[0]))
    for l in range(1, levels):
        sf.call("sf_PyrDownGauss_u8", ctx.h, sf.image(imgs[l - 1]), sf.image(imgs[l]))
    for l in range(levels):
        sf.call("sf_ComputeDerivativeImage", ctx.h, sf.image(imgs[l]), sf.image(dxs[l]), sf.image(dys[l]))
    ctx.sync()
    return imgs, dxs, dys


def test_intensity_pyramid_golden(lib):
    sf, ctx = lib
    g = dict(np.load(G1))
    for i in range(2):
        imgs, dxs, dys = _gpu_intensity(sf, ctx, g["rgb%d" % i])
        for l in range(3):
            assert np.array_equal(host(imgs[l]), g["f%d_int%d" % (i, l)]), "frame %d level %d" % (i, l)
            assert np.array_equal(host(dxs[l]), g["f%d_dx%d" % (i, l)])
            assert np.array_equal(host(dys[l]), g["f%d_dy%d" % (i, l)])


@pytest.mark.parametrize("cols,rows", [(640, 480), (97, 73), (1280, 720)])
def test_intensity_pyramid_vs_oracle(lib, cols, rows):
    from oracle import oracle as O
    sf, ctx = lib
    rgb = np.random.default_rng(cols).integers(0, 256, (rows, cols, 3), dtype=np.uint8)
    rgb[: rows // 3, : cols // 3] = 0  # dark corner: zero intensity and flat gradients
    imgs, dxs, dys = _gpu_intensity(sf, ctx, rgb)
    img = O.intensity(rgb)
    for l in range(3):
        if l > 0:
            img = O.pyrdown_u8(img)
        assert np.array_equal(host(imgs[l]), img), "level %d" % l
        dx, dy = O.sobel(img)
        assert np.array_equal(host(dxs[l]), dx)
        assert np.array_equal(host(dys[l]), dy)


def test_intensity_every_colour(lib):
    """Every one of the 2^24 colours, including the 1,722 whose weighted sum
    is an exact integer and the double expression decides."""
    from oracle import oracle as O
    import torch
    sf, ctx = lib
    v = np.arange(1 << 24, dtype=np.uint32)
    rgb = np.stack([(v >> 16) & 255, (v >> 8) & 255, v & 255], -1).astype(np.uint8).reshape(4096, 4096, 3)
    out = empty((4096, 4096), torch.uint8)
    dc = cuda(rgb)  # alive through the call
    sf.call("sf_ImageToIntensity", ctx.h, sf.image(dc, 3), sf.image(out))
    ctx.sync()
    assert np.array_equal(host(out), O.intensity(rgb))


def _rgb_step(sf, ctx, inext, ilast, vnext, vlast, dx, dy, Pc, Pl, K):
    Rc, RcI, tc = sf.pose_to_gpu(Pc)
    Rl, RlI, tl = sf.pose_to_gpu(Pl)
    res = (C.c_float * 2)()
    A = (C.c_double * 36)()
    b = (C.c_double * 6)()
    sf.call("sf_RGBStep", ctx.h, sf.image(inext), sf.image(ilast), sf.image(vnext), sf.image(vlast), sf.image(dx),
            sf.image(dy), Rc, RcI, Rl, RlI, tc, tl, sf.Intrinsics(*K), res, A, b)
    return np.float32(res[0]), np.float32(res[1]), np.array(A[:]).reshape(6, 6), np.array(b[:])


def _check_sums(res0, res1, A, b, s):
    from oracle import oracle as O
    Ao, bo = O.create_matrix(s)
    assert res1 == np.float32(s[28]) and s[28] > 100
    assert abs(float(res0) - float(np.float32(s[27]))) <= SUMS_RTOL * float(s[27])
    np.testing.assert_allclose(A, Ao, rtol=SUMS_RTOL, atol=SUMS_RTOL * np.abs(np.diag(Ao)).max())
    np.testing.assert_allclose(b, bo, rtol=SUMS_RTOL, atol=SUMS_RTOL * np.sqrt(np.abs(np.diag(Ao)).max() * s[27]))


def test_rgb_step_golden(lib):
    """RGBStep on the reference kernels' inputs (frame 1 against frame 0 at
    the halfway pose): count exact, sums against the reference's rows."""
    sf, ctx = lib
    g = dict(np.load(G1))
    K = [float(k) for k in g["K"]]
    for l in range(3):
        div = float(1 << l)
        Kl = [k / div for k in K]
        r0, r1, A, b = _rgb_step(sf, ctx, cuda(g["f1_int%d" % l]), cuda(g["f0_int%d" % l]), cuda(g["f1_vmap%d" % l]),
                                 cuda(g["f0_vmap%d" % l]), cuda(g["f1_dx%d" % l]), cuda(g["f1_dy%d" % l]),
                                 g["icp_pose_curr"], g["pose0"], Kl)
        assert int(r1) == int(g["rgb_res%d" % l][0]), "level %d" % l
        _check_sums(r0, r1, A, b, g["rgb_sums%d" % l])


def _frames_c2(sf, ctx, n=3):
    """Oracle depth and intensity pyramids of a 640x480 sequence."""
    from oracle import oracle as O
    K = C2["K"]
    seq = sequence(C2["cols"], C2["rows"], K, n, trajectory=1, dropout=0.02)
    out = []
    for d, rgb, _, P in seq:
        _, filt = O.filter_depth(d, 1000.0, 3.0)
        deps = [filt]
        for l in range(1, 3):
            deps.append(O.pyrdown(deps[-1]))
        vms = [O.vmap(deps[l], *[k / (1 << l) for k in K], 3.0) for l in range(3)]
        nms = [O.nmap(v) for v in vms]
        imgs = [O.intensity(rgb)]
        for l in range(1, 3):
            imgs.append(O.pyrdown_u8(imgs[-1]))
        ders = [O.sobel(i) for i in imgs]
        out.append(dict(P=P, v=vms, n=nms, i=imgs, dx=[a for a, _ in ders], dy=[b for _, b in ders]))
    return seq, out


def test_rgb_step_vs_oracle(lib):
    from oracle import oracle as O
    sf, ctx = lib
    _, f = _frames_c2(sf, ctx)
    K = C2["K"]
    P0, P1 = f[0]["P"], f[2]["P"]
    Pc = P0.copy()
    Pc[:3, 3] = 0.5 * (P0[:3, 3] + P1[:3, 3])
    for l in range(3):
        Kl = [k / (1 << l) for k in K]
        r0, r1, A, b = _rgb_step(sf, ctx, cuda(f[2]["i"][l]), cuda(f[0]["i"][l]), cuda(f[2]["v"][l]),
                                 cuda(f[0]["v"][l]), cuda(f[2]["dx"][l]), cuda(f[2]["dy"][l]), Pc, P0, Kl)
        s, res, sigma = O.rgb_step(f[2]["i"][l], f[0]["i"][l], f[2]["v"][l], f[0]["v"][l], f[2]["dx"][l],
                                   f[2]["dy"][l], Pc, P0, Kl)
        assert int(r1) == res[0]
        _check_sums(r0, r1, A, b, s)


@pytest.mark.parametrize("step", [1, 2])
def test_compute_se3_rgbd(lib, step):
    """ComputeSE3(icpOnly = false) in one persistent launch vs the oracle."""
    from oracle import oracle as O
    sf, ctx = lib
    seq, f = _frames_c2(sf, ctx)
    K = C2["K"]
    a, n = f[0], f[step]
    dev = {k: [cuda(x) for x in n[k]] for k in ("v", "n", "i", "dx", "dy")}
    last = {k: [cuda(x) for x in a[k]] for k in ("v", "n", "i")}
    arr = lambda ts: (sf.Image * 3)(*[sf.image(t) for t in ts])
    iters = (C.c_int * 3)(10, 5, 4)
    mins = (C.c_int * 3)(2000, 1000, 100)
    lp = np.ascontiguousarray(a["P"], np.float64)
    out = np.zeros(16, np.float64)
    stats = (C.c_int * 6)()
    errs = (C.c_float * 2)()
    sf.call("sf_ComputeSE3_rgbd", ctx.h, 3, arr(dev["v"]), arr(dev["n"]), arr(last["v"]), arr(last["n"]),
            arr(dev["i"]), arr(last["i"]), arr(dev["dx"]), arr(dev["dy"]), sf.Intrinsics(*K), iters, mins, 1e-4,
            lp.ctypes.data_as(sf._lib.F64P), out.ctypes.data_as(sf._lib.F64P), stats, errs)
    ok, Po, st = O.compute_se3(n["v"], n["n"], a["v"], a["n"], K, (10, 5, 4), (2000, 1000, 100), 1e-4, a["P"],
                               a["P"], rgb=(n["i"], a["i"], n["dx"], n["dy"]))
    Pg = out.reshape(4, 4)
    assert bool(stats[0]) == ok
    assert stats[2] == int(st[2]), "iterations run"
    assert stats[4] == int(st[5]) and stats[4] > 1000, "photometric correspondences of the last iteration"
    assert np.abs(Pg - Po).max() < POSE_TOL
    assert ok and np.linalg.norm(Pg[:3, 3] - seq[step][3][:3, 3]) < 0.01
