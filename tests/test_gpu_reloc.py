"""GPU parity of the batched relocalisation scorer (sf_RelocScoreBatch)
against the oracle's restatement (oracle/sfo.cpp sfo_reloc_score).

Both maps are fused identically from the same frames (bit-exact, as
test_gpu_fusion checks), the candidates are the true pose and seeded
perturbations (sigma 5 cm / 5 deg, the relocalisation workload), and the
samples are read with the raycast's trilinear interpolation.  Counts must
be equal and the fixed-order sums bit-equal; the true pose must score
among the best.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, MAP_C1, cuda, host, sequence
from tests.test_gpu_fusion import _frame_inputs

pytestmark = pytest.mark.gpu


def _rot(axis_angle):
    th = np.linalg.norm(axis_angle)
    if th == 0:
        return np.eye(3)
    k = axis_angle / th
    Kx = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx


def candidates(P, n, seed, sigma_t=0.05, sigma_r=np.deg2rad(5.0)):
    """The true pose first, then n - 1 seeded perturbations of it."""
    rng = np.random.default_rng(seed)
    out = [P.copy()]
    for _ in range(n - 1):
        Q = P.copy()
        Q[:3, :3] = _rot(rng.normal(0, sigma_r, 3)) @ P[:3, :3]
        Q[:3, 3] = P[:3, 3] + rng.normal(0, sigma_t, 3)
        out.append(Q)
    return np.array(out)


@pytest.fixture(scope="module")
def fused(built):
    import torch
    import semantic_icpslam_gb300 as sf
    from oracle import oracle as O
    assert torch.cuda.is_available()
    ctx = sf.Context()
    K = C1["K"]
    seq = sequence(C1["cols"], C1["rows"], K, 5, trajectory=1, dropout=0.02)
    gmap, omap = sf.Map(**MAP_C1), O.Map(**MAP_C1)
    for d, rgb, mask, P in seq[:4]:
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        R, RI, t = sf.pose_to_gpu(P)
        nvis = C.c_uint32()
        sf.call("sf_FuseMapColor", ctx.h, gmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
                sf.image(f["mask"]), 0, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
        omap.fuse(f["raw_h"], rgb, f["nmap_h"], None, 0, P, K)
    # the next frame's vertex map (camera frame) is what gets relocalised
    d, rgb, mask, P = seq[4]
    f = _frame_inputs(sf, ctx, d, rgb, mask, K)
    import torch
    dd = cuda(d)
    raw = torch.empty(d.shape, dtype=torch.float32, device="cuda")
    filt = torch.empty(d.shape, dtype=torch.float32, device="cuda")
    vm = torch.empty(d.shape + (4,), dtype=torch.float32, device="cuda")
    sf.call("sf_FilterDepth", ctx.h, sf.image(dd), sf.image(raw), sf.image(filt), 1000.0, 3.0)
    sf.call("sf_ComputeVMap", ctx.h, sf.image(filt), sf.image(vm), *K, 3.0)
    ctx.sync()
    yield sf, ctx, gmap, omap, vm, P
    ctx.close()


@pytest.mark.parametrize("stride,n", [(2, 256), (1, 7)])
def test_reloc_scores_match_oracle(fused, stride, n):
    sf, ctx, gmap, omap, vm, P = fused
    cand = candidates(P, n, seed=11 + n)
    out = (sf._lib.RelocScore * n)()
    sf.call("sf_RelocScoreBatch", ctx.h, gmap.h, sf.image(vm), stride,
            np.ascontiguousarray(cand, np.float64).ctypes.data_as(C.POINTER(C.c_double)), n, 0.5, out)
    g = np.array([(o.valid, o.inliers, o.sum_abs_sdf, o.mean_abs_sdf) for o in out],
                 dtype=[("valid", "<u4"), ("inliers", "<u4"), ("sum", "<f4"), ("mean", "<f4")])
    o = omap.reloc_score(host(vm), stride, cand, 0.5)
    assert np.array_equal(g["valid"], o["valid"])
    assert np.array_equal(g["inliers"], o["inliers"])
    assert np.array_equal(g["sum"].view(np.uint32), o["sum_abs_sdf"].view(np.uint32))
    assert np.array_equal(g["mean"].view(np.uint32), o["mean_abs_sdf"].view(np.uint32))
    assert g["valid"][0] > 1000 // stride ** 2
    # the true pose is among the best-scoring candidates
    assert g["inliers"][0] >= np.sort(g["inliers"])[-max(2, n // 50)]


def test_reloc_rejects_bad_arguments(fused):
    sf, ctx, gmap, omap, vm, P = fused
    out = (sf._lib.RelocScore * 1)()
    poses = np.ascontiguousarray(P[None], np.float64).ctypes.data_as(C.POINTER(C.c_double))
    for stride, n in [(0, 1), (1, 0), (1, 65537)]:
        with pytest.raises(sf.SfError):
            sf.call("sf_RelocScoreBatch", ctx.h, gmap.h, sf.image(vm), stride, poses, n, 0.5, out)
