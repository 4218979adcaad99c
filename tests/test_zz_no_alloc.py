"""sf_ICPStep_static: the projective ICP step for callers that cannot
allocate device memory.

Some hosts own every byte of device memory through their own allocator and
forbid outside cudaMalloc.  Others run a real-time loop where cudaMalloc's
implicit device synchronisation is not acceptable.  Neither can create an
sf_context, because creating one allocates its workspace.
sf_ICPStep_static takes a stream plus the same inputs and host outputs as
sf_ICPStep, and keeps its scratch in a fixed array inside the library's
device image.

Its results must match sf_ICPStep on the same inputs, for three calls in a
row.  Each later call reuses the array the call before left behind.  The
match count must be exact.  The sums may differ only by summation order:
the two calls split the pixels over different numbers of CTAs.  The
tolerance is the one the ICP parity tests use.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, cuda, empty, sequence

pytestmark = pytest.mark.gpu

SUMS_RTOL = 2e-6


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _pyramid(sf, ctx, d, K, levels=3):
    dd = cuda(d)
    import torch
    raw = empty(d.shape, torch.float32)
    shp = lambda l: (d.shape[0] >> l, d.shape[1] >> l)
    depths = [empty(shp(l), torch.float32) for l in range(levels)]
    vms = [empty(shp(l) + (4,), torch.float32) for l in range(levels)]
    nms = [empty(shp(l) + (4,), torch.float32) for l in range(levels)]
    arr = lambda ts: (sf.Image * levels)(*[sf.image(t) for t in ts])
    sf.call("sf_BuildPyramid", ctx.h, sf.image(dd), sf.image(raw), arr(depths), arr(vms), arr(nms), levels,
            sf.Intrinsics(*K), 1000.0, 3.0)
    ctx.sync()
    return vms, nms, (dd, raw, depths)


def _step(sf, fn, first, ims, Pc, P0, K):
    Rc, _, tc = sf.pose_to_gpu(Pc)
    Rl, RlI, tl = sf.pose_to_gpu(P0)
    res = (C.c_float * 2)()
    A = (C.c_double * 36)()
    b = (C.c_double * 6)()
    sf.call(fn, first, *[sf.image(t) for t in ims], Rc, tc, Rl, RlI, tl, sf.Intrinsics(*K), res, A, b)
    return np.array(res[:], np.float64), np.array(A[:]).reshape(6, 6), np.array(b[:])


def _same(got, want):
    (rg, Ag, bg), (rw, Aw, bw) = got, want
    assert rg[1] == rw[1] and rw[1] > 100
    assert abs(rg[0] - rw[0]) <= SUMS_RTOL * abs(rw[0])
    scale = np.abs(np.diag(Aw)).max()
    np.testing.assert_allclose(Ag, Aw, rtol=SUMS_RTOL, atol=SUMS_RTOL * scale)
    np.testing.assert_allclose(bg, bw, rtol=SUMS_RTOL, atol=SUMS_RTOL * np.sqrt(scale * rw[0]))


def test_static_icp_step_matches_context_step(lib):
    import torch
    sf, ctx = lib
    seq = sequence(C1["cols"], C1["rows"], C1["K"], 3, dropout=0.02)
    d0, _, _, P0 = seq[0]
    d1, _, _, P1 = seq[2]
    v0, n0, keep0 = _pyramid(sf, ctx, d0, C1["K"])
    v1, n1, keep1 = _pyramid(sf, ctx, d1, C1["K"])
    Pc = P0.copy()
    Pc[:3, 3] = 0.5 * (P0[:3, 3] + P1[:3, 3])
    stream = torch.cuda.Stream()
    K = C1["K"]
    calls = [(0, Pc), (1, P1), (0, P1)]  # calls in a row, different sizes and poses
    free = []
    for level, P in calls:
        div = float(1 << level)
        Kl = tuple(k / div for k in K)
        ims = (v1[level], v0[level], n1[level], n0[level])
        want = _step(sf, "sf_ICPStep", ctx.h, ims, P, P0, Kl)
        got = _step(sf, "sf_ICPStep_static", C.c_void_p(stream.cuda_stream), ims, P, P0, Kl)
        _same(got, want)
        free.append(torch.cuda.mem_get_info()[0])
    # the calls after the first allocated nothing on the device (the first
    # may load the library's device image under lazy module loading)
    assert free[1] >= free[0] and free[2] >= free[0]
    del keep0, keep1


def test_static_icp_step_rejects_oversize(lib):
    import torch
    from semantic_icpslam_gb300 import _lib
    sf, ctx = lib
    # real buffers large enough for the claimed size, so a missing check
    # could not read out of bounds
    cols, rows = 2049, 2048
    assert cols * rows > _lib.ICP_STATIC_MAX_PIXELS
    buf = torch.zeros((rows, cols, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(_lib.SfError) as e:
        _step(sf, "sf_ICPStep_static", None, (buf, buf, buf, buf), np.eye(4), np.eye(4), C1["K"])
    assert e.value.status == _lib.SF_ERR_TOO_LARGE
