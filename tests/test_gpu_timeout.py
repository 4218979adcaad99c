"""Failure detection on the device without a fault: the persistent ICP
kernel's grid barriers are bounded waits.  A test-only bound makes every
wait unreachable (the barrier waits for one arrival more than the grid has)
and short, so each barrier gives up: the kernel records
SF_FLAG_BARRIER_TIMEOUT, leaves its iterations with the tracking failed,
and sf_ComputeSE3 returns SF_ERR_TIMEOUT instead of hanging.  With the
default bounds restored, the same context computes the same pose as a
fresh one, so the context stays usable.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, sequence
from tests.test_gpu_validate import _pyramid

pytestmark = pytest.mark.gpu


def _compute_se3(sf, ctx, cur, last, P0):
    vms, nms = cur
    lvm, lnm = last
    arr = lambda ts: (sf.Image * 3)(*[sf.image(t) for t in ts])
    out = np.zeros(16, np.float64)
    stats = (C.c_int * 4)()
    err = C.c_float()
    P = np.ascontiguousarray(P0, np.float64)
    st = sf.load().sf_ComputeSE3(ctx.h, 3, arr(vms), arr(nms), arr(lvm), arr(lnm), sf.Intrinsics(*C1["K"]),
                                 (C.c_int * 3)(10, 5, 4), (C.c_int * 3)(2000, 1000, 100), C.c_float(1e-4),
                                 P.ctypes.data_as(C.POINTER(C.c_double)), out.ctypes.data_as(C.POINTER(C.c_double)),
                                 stats, C.byref(err))
    return st, out.reshape(4, 4), list(stats)


def test_barrier_wait_runs_out_and_context_recovers(built):
    import torch
    import semantic_icpslam_gb300 as sf
    from semantic_icpslam_gb300 import _lib
    assert torch.cuda.is_available()
    seq = sequence(C1["cols"], C1["rows"], C1["K"], 2, trajectory=1, dropout=0.02)
    ctx = sf.Context()
    ref = sf.Context()
    try:
        v0, n0, k0 = _pyramid(sf, ctx, seq[0][0], C1["K"])
        v1, n1, k1 = _pyramid(sf, ctx, seq[1][0], C1["K"])
        P0 = seq[0][3]
        want_st, want, _ = _compute_se3(sf, ref, (v1, n1), (v0, n0), P0)
        assert want_st == _lib.SF_OK
        # every barrier waits for one arrival more than the grid can give,
        # for at most 2000 polls
        sf.call("sf_icp_barrier_limits", ctx.h, 2000, 1)
        st, pose, stats = _compute_se3(sf, ctx, (v1, n1), (v0, n0), P0)
        assert st == _lib.SF_ERR_TIMEOUT
        assert ctx.flags() & (1 << 6)  # SF_FLAG_BARRIER_TIMEOUT
        assert stats[0] == 0 and stats[1] == 1  # not accepted, failed
        assert np.array_equal(pose, P0)  # rolled back to the last pose
        # default bounds: the same context tracks as a fresh one
        sf.call("sf_icp_barrier_limits", ctx.h, 0, 0)
        st, pose, _ = _compute_se3(sf, ctx, (v1, n1), (v0, n0), P0)
        assert st == _lib.SF_OK
        assert np.array_equal(pose, want)
        with pytest.raises(sf.SfError):
            sf.call("sf_icp_barrier_limits", ctx.h, 0, 1 << 20)
    finally:
        ctx.close()
        ref.close()
