"""The autograd raycast (semantic_icpslam_gb300.autograd) and the keyframe
TSDF refinement it drives.

* Its backward equals direct sf_RaycastAdjoint calls (pose exactly, TSDF up
  to the order of float atomics).
* 50 Adam steps on the TSDF against 8 seeded keyframes with noisy depth
  (the differentiable-raycast workload, at 320x240 / 10 mm and at
  640x480 / 5 mm) lower the depth loss.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, C2, MAP_C1, MAP_C2, cuda, sequence
from tests.test_gpu_fusion import _frame_inputs

pytestmark = pytest.mark.gpu


# c1: 320x240 / 10 mm; c4: the differentiable-raycast workload at 640x480
# and 5 mm (50 Adam steps against 8 seeded keyframes with noisy depth)
SCENES = {"c1": (C1, MAP_C1), "c4": (C2, MAP_C2)}


@pytest.fixture(scope="module", params=sorted(SCENES))
def fused(built, request):
    import torch
    import semantic_icpslam_gb300 as sf
    from semantic_icpslam_gb300 import autograd as ag
    assert torch.cuda.is_available()
    ctx = sf.Context()
    cfg, mapkw = SCENES[request.param]
    K = cfg["K"]
    seq = sequence(cfg["cols"], cfg["rows"], K, 9, trajectory=0, dropout=0.02)
    tmap = ag.TorchMap(ctx, **mapkw)
    for d, rgb, mask, P in seq[:8]:
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        R, RI, t = sf.pose_to_gpu(P)
        nvis = C.c_uint32()
        sf.call("sf_FuseMapColor", ctx.h, tmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
                sf.image(f["mask"]), 0, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
    ctx.sync()
    r = ag.Renderer(ctx, tmap, cfg["cols"], cfg["rows"], K)
    yield sf, ag, ctx, tmap, r, seq
    tmap.close()
    ctx.close()


def test_autograd_backward_equals_the_adjoint(fused):
    import torch
    sf, ag, ctx, tmap, r, seq = fused
    P = seq[8][3]
    xi = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    sdf = tmap.sdf().detach().requires_grad_(True)
    vm, nm = ag.raycast(xi, sdf, r, P)
    g = torch.Generator(device="cuda").manual_seed(7)
    wv = torch.randn(vm.shape, device="cuda", generator=g)
    wn = torch.randn(nm.shape, device="cuda", generator=g)
    loss = (torch.nan_to_num(vm) * wv).sum() + (torch.nan_to_num(nm) * wn).sum()
    loss.backward()
    ok = torch.isfinite(vm[..., :1]) & torch.isfinite(nm[..., :1])
    gv = torch.where(ok, wv, torch.zeros_like(wv))
    gn = torch.where(ok, wn, torch.zeros_like(wn))
    _, _, zmin, zmax = r.render(P)
    gs = torch.zeros(tmap.num_voxels, dtype=torch.float32, device="cuda")
    gp = r.adjoint(P, zmin, zmax, gv, gn, gs)
    np.testing.assert_allclose(xi.grad.numpy(), gp, rtol=1e-9, atol=1e-9 * np.abs(gp).max())
    a, b = sdf.grad.cpu().numpy(), gs.cpu().numpy()
    assert np.count_nonzero(b) > 1000
    np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-6 * np.abs(b).max())


def test_refine_tsdf_lowers_keyframe_depth_loss(fused):
    import torch
    sf, ag, ctx, tmap, r, seq = fused
    keyframes = []
    for d, _, _, P in seq[:8]:
        dm = cuda(d.astype(np.float32) / 1000.0)
        keyframes.append((P, torch.where(dm > 0, dm, torch.full_like(dm, float("nan")))))
    before = tmap.sdf().clone()
    losses = ag.refine_tsdf(r, tmap, keyframes, steps=50, lr=0.01)
    assert len(losses) == 50 and all(np.isfinite(losses))
    assert losses[-1] < 0.97 * losses[0], losses[::10]
    after = tmap.sdf()
    observed = tmap.weight() > 0
    assert torch.equal(torch.isnan(after), torch.isnan(before))            # unobserved voxels untouched
    assert float((after[observed] - before[observed]).abs().max()) > 0      # observed voxels moved
    assert float(after[observed].abs().max()) <= 1.0


def test_cpp_autograd_function_matches_python(fused):
    """The libtorch C++ torch::autograd::Function (sf_torch.raycast) renders
    the same maps and backpropagates the same gradients as the Python form:
    pose gradient exactly (a fixed-order reduction), TSDF gradient up to the
    order of float atomics."""
    import torch
    sf, ag, ctx, tmap, r, seq = fused
    P = seq[8][3]
    g = torch.Generator(device="cuda").manual_seed(11)
    outs = []
    for fn in (ag.raycast, ag.raycast_cpp):
        xi = torch.zeros(6, dtype=torch.float64, requires_grad=True)
        sdf = tmap.sdf().detach().requires_grad_(True)
        vm, nm = fn(xi, sdf, r, P)
        assert vm.grad_fn is not None
        if not outs:
            wv = torch.randn(vm.shape, device="cuda", generator=g)
            wn = torch.randn(nm.shape, device="cuda", generator=g)
        loss = (torch.nan_to_num(vm) * wv).sum() + (torch.nan_to_num(nm) * wn).sum()
        loss.backward()
        outs.append((vm.detach(), nm.detach(), xi.grad.detach().clone(), sdf.grad.detach().clone()))
    (v1, n1, x1, s1), (v2, n2, x2, s2) = outs
    assert torch.equal(torch.nan_to_num(v1, 7.0), torch.nan_to_num(v2, 7.0))
    assert torch.equal(torch.nan_to_num(n1, 7.0), torch.nan_to_num(n2, 7.0))
    assert torch.equal(x1, x2) and x1.abs().max() > 0
    scale = s1.abs().max()
    assert scale > 0 and (s1 - s2).abs().max() <= 1e-5 * scale
