"""GPU parity of projective point-to-plane ICP (Tracking/Reduction.cu,
Tracker::ComputeSE3 in Tracking/Tracking.cc:369-517) against the oracle.

The per-pixel rows are FP32 in both; the GPU sums them with compensated
FP32 warp trees and FP64 block/cross-block totals, the oracle in FP64.  The
match count is exact; the 29 sums agree to SUMS_RTOL; the final pose of the
whole ComputeSE3 loop agrees to POSE_TOL (metres / radians).
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, C2, cuda, empty, host, sequence

pytestmark = pytest.mark.gpu

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


def _pyramid(sf, ctx, d, K, levels=3):
    import torch
    dd = cuda(d)
    raw = empty(d.shape, torch.float32)
    depths = [empty((d.shape[0] >> l, d.shape[1] >> l), torch.float32) for l in range(levels)]
    vms = [empty((d.shape[0] >> l, d.shape[1] >> l, 4), torch.float32) for l in range(levels)]
    nms = [empty((d.shape[0] >> l, d.shape[1] >> l, 4), torch.float32) for l in range(levels)]
    arr = lambda ts: (sf.Image * levels)(*[sf.image(t) for t in ts])
    sf.call("sf_BuildPyramid", ctx.h, sf.image(dd), sf.image(raw), arr(depths), arr(vms), arr(nms), levels,
            sf.Intrinsics(*K), 1000.0, 3.0)
    ctx.sync()
    return vms, nms


def _rel_err(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)


@pytest.mark.parametrize("cfg,step", [(C1, 1), (C2, 2)])
def test_icp_step_sums(lib, cfg, step):
    from oracle import oracle as O
    sf, ctx = lib
    seq = sequence(cfg["cols"], cfg["rows"], cfg["K"], 3, dropout=0.02)
    d0, _, _, P0 = seq[0]
    d1, _, _, P1 = seq[step]
    v0, n0 = _pyramid(sf, ctx, d0, cfg["K"])
    v1, n1 = _pyramid(sf, ctx, d1, cfg["K"])
    # the current estimate: halfway between the two true poses
    Pc = P0.copy()
    Pc[:3, 3] = 0.5 * (P0[:3, 3] + P1[:3, 3])
    K = cfg["K"]
    for level in range(3):
        div = float(1 << level)
        Kl = (K[0] / div, K[1] / div, K[2] / div, K[3] / div)
        Rc, _, tc = sf.pose_to_gpu(Pc)
        Rl, RlI, tl = sf.pose_to_gpu(P0)
        res = (C.c_float * 2)()
        A = (C.c_double * 36)()
        b = (C.c_double * 6)()
        sf.call("sf_ICPStep", ctx.h, sf.image(v1[level]), sf.image(v0[level]), sf.image(n1[level]),
                sf.image(n0[level]), Rc, tc, Rl, RlI, tl, sf.Intrinsics(*Kl), res, A, b)
        s = O.icp_sums(host(v1[level]), host(v0[level]), host(n1[level]), host(n0[level]), Pc, P0, Kl)
        Ao, bo = O.create_matrix(s)
        assert res[1] == s[28] and s[28] > 100
        assert _rel_err(np.float64(res[0]), np.float64(np.float32(s[27]))) < SUMS_RTOL
        # entries with cancellation are bounded on the scale of the
        # largest diagonal (A) and by Cauchy-Schwarz sqrt(max A_ii * sum r^2) (b)
        np.testing.assert_allclose(np.array(A[:]).reshape(6, 6), Ao, rtol=SUMS_RTOL,
                                   atol=SUMS_RTOL * np.abs(np.diag(Ao)).max())
        np.testing.assert_allclose(np.array(b[:]), bo, rtol=SUMS_RTOL,
                                   atol=SUMS_RTOL * np.sqrt(np.abs(np.diag(Ao)).max() * s[27]))


def test_icp_rows_bit_exact_count(lib):
    """Rows found on the GPU == rows found by the oracle (count is exact)."""
    from oracle import oracle as O
    sf, ctx = lib
    cfg = C1
    seq = sequence(cfg["cols"], cfg["rows"], cfg["K"], 2)
    v0, n0 = _pyramid(sf, ctx, seq[0][0], cfg["K"])
    v1, n1 = _pyramid(sf, ctx, seq[1][0], cfg["K"])
    P0 = seq[0][3]
    rows = O.icp_rows(host(v1[0]), host(v0[0]), host(n1[0]), host(n0[0]), P0, P0, cfg["K"])
    res = (C.c_float * 2)()
    A = (C.c_double * 36)()
    b = (C.c_double * 6)()
    Rc, RcI, tc = sf.pose_to_gpu(P0)
    sf.call("sf_ICPStep", ctx.h, sf.image(v1[0]), sf.image(v0[0]), sf.image(n1[0]), sf.image(n0[0]), Rc, tc,
            Rc, RcI, tc, sf.Intrinsics(*cfg["K"]), res, A, b)
    assert int(res[1]) == int(rows[:, 28].sum())


@pytest.mark.parametrize("cfg,step", [(C1, 1), (C1, 3), (C2, 2)])
def test_compute_se3_persistent(lib, cfg, step):
    """Whole ComputeSE3 loop in one persistent launch vs the oracle loop."""
    from oracle import oracle as O
    sf, ctx = lib
    seq = sequence(cfg["cols"], cfg["rows"], cfg["K"], 4, dropout=0.02)
    d0, _, _, P0 = seq[0]
    d1, _, _, P1 = seq[step]
    v0, n0 = _pyramid(sf, ctx, d0, cfg["K"])
    v1, n1 = _pyramid(sf, ctx, d1, cfg["K"])
    iters = (C.c_int * 3)(10, 5, 4)
    mins = (C.c_int * 3)(2000, 1000, 100)
    arr = lambda ts: (sf.Image * 3)(*[sf.image(t) for t in ts])
    lp = np.ascontiguousarray(P0, np.float64)
    out = np.zeros(16, np.float64)
    stats = (C.c_int * 4)()
    err = C.c_float()
    sf.call("sf_ComputeSE3", ctx.h, 3, arr(v1), arr(n1), arr(v0), arr(n0), sf.Intrinsics(*cfg["K"]), iters, mins,
            1e-4, lp.ctypes.data_as(sf._lib.F64P), out.ctypes.data_as(sf._lib.F64P), stats, C.byref(err))
    ok, Po, st = O.compute_se3([host(t) for t in v1], [host(t) for t in n1], [host(t) for t in v0],
                               [host(t) for t in n0], cfg["K"], (10, 5, 4), (2000, 1000, 100), 1e-4, P0, P0)
    Pg = out.reshape(4, 4)
    assert bool(stats[0]) == ok
    assert stats[2] == int(st[2]), "iterations run"
    assert np.abs(Pg - Po).max() < POSE_TOL
    if ok:  # converged near the truth
        assert np.linalg.norm(Pg[:3, 3] - P1[:3, 3]) < 0.01


def test_compute_se3_failure_rolls_back(lib):
    """Too few matches (min_count above the pixel count): pose rolls back."""
    sf, ctx = lib
    cfg = C1
    seq = sequence(cfg["cols"], cfg["rows"], cfg["K"], 2)
    v0, n0 = _pyramid(sf, ctx, seq[0][0], cfg["K"])
    v1, n1 = _pyramid(sf, ctx, seq[1][0], cfg["K"])
    iters = (C.c_int * 3)(10, 5, 4)
    mins = (C.c_int * 3)(2000, 1000, 10 ** 7)
    arr = lambda ts: (sf.Image * 3)(*[sf.image(t) for t in ts])
    P0 = np.ascontiguousarray(seq[0][3], np.float64)
    out = np.zeros(16, np.float64)
    stats = (C.c_int * 4)()
    sf.call("sf_ComputeSE3", ctx.h, 3, arr(v1), arr(n1), arr(v0), arr(n0), sf.Intrinsics(*cfg["K"]), iters, mins,
            1e-4, P0.ctypes.data_as(sf._lib.F64P), out.ctypes.data_as(sf._lib.F64P), stats, None)
    assert stats[0] == 0 and stats[1] == 1 and stats[2] == 1
    assert np.array_equal(out.reshape(4, 4), P0)
