"""GPU RaycastAdjoint (sf_RaycastAdjoint) against central finite differences
of the oracle's FP64 reference (oracle/sfo.cpp sfo_raycast_smooth_f64).

The loss is L = sum gv . v + gn . n over the rendered pixels, with seeded
upstream gradients gv, gn.  The reference holds the float march's discrete
outcome and the interpolation cells fixed (as the adjoint does) and
evaluates the rest of the raycast in double.  Its central differences with
step 1e-4 (the differentiable-raycast workload's step), along the six se(3)
axes of exp(xi) T and for single voxels' TSDF values, must agree with the
GPU gradient.  The pose check extrapolates the step-h and step-h/2
differences (Richardson, error O(h^4)).  With the normal term, h is 1e-5:
the normal curves strongly in the rotation axes, and at 5 mm voxels its
central differences at 1e-4 are still 10% from their limit (at 1e-5 they
are within 0.1% and settle; the 640x480 / 5 mm scene measured on a GB300).
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, C2, MAP_C1, MAP_C2, empty, host, map_to_host, sequence
from tests.test_gpu_fusion import _frame_inputs

pytestmark = pytest.mark.gpu

H = 1e-4
H_NORMAL = 1e-5    # pose step with the normal term (module docstring)
POSE_RTOL = 2e-3   # of the pose gradient's norm (float adjoint vs FP64 differences)
SDF_RTOL = 5e-3    # per voxel, of the largest voxel gradient checked


# c1: 320x240 / 10 mm; c4: the differentiable-raycast workload, a 640x480
# view at 5 mm of the region four frames have fused (over 5e5 voxels
# receive a TSDF gradient)
SCENES = {"c1": (C1, MAP_C1), "c4": (C2, MAP_C2)}


@pytest.fixture(scope="module", params=sorted(SCENES))
def scene(built, request):
    import torch
    import semantic_icpslam_gb300 as sf
    from oracle import oracle as O
    assert torch.cuda.is_available()
    ctx = sf.Context()
    cfg, mapkw = SCENES[request.param]
    K = cfg["K"]
    cols, rows = cfg["cols"], cfg["rows"]
    seq = sequence(cols, rows, K, 5, trajectory=1, dropout=0.02)
    gmap, omap = sf.Map(**mapkw), O.Map(**mapkw)
    for d, rgb, mask, P in seq[:4]:
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        R, RI, t = sf.pose_to_gpu(P)
        nvis = C.c_uint32()
        sf.call("sf_FuseMapColor", ctx.h, gmap.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
                sf.image(f["mask"]), 0, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
        omap.fuse(f["raw_h"], rgb, f["nmap_h"], None, 0, P, K)
    P = seq[4][3]   # render from the next (unfused) pose
    R, RI, t = sf.pose_to_gpu(P)
    nvis = C.c_uint32()
    sf.call("sf_CheckBlockVisibility", ctx.h, gmap.h, R, RI, t, cols, rows, *K, 3.0, 0.1, C.byref(nvis))
    zc, zr = (cols + 7) // 8, (rows + 7) // 8
    zmin = empty((zr, zc), torch.float32)
    zmax = empty((zr, zc), torch.float32)
    blocks = empty((260000, 16), torch.uint8)
    nblk = empty((1,), torch.int32)
    ok = C.c_int()
    sf.call("sf_CreateRenderingBlocks", ctx.h, gmap.h, sf.image(zmin), sf.image(zmax), 3.0, 0.1,
            blocks.data_ptr(), nblk.data_ptr(), RI, t, nvis.value, *K, C.byref(ok))
    vm = empty((rows, cols, 4), torch.float32)
    nm = empty((rows, cols, 4), torch.float32)
    invfx = float(np.float32(1.0 / np.float64(np.float32(K[0]))))
    invfy = float(np.float32(1.0 / np.float64(np.float32(K[1]))))
    sf.call("sf_Raycast", ctx.h, gmap.h, sf.image(vm), sf.image(nm), sf.image(zmin), sf.image(zmax), R, RI, t,
            invfx, invfy, K[2], K[3])
    ctx.sync()
    rng = np.random.default_rng(3)
    valid = np.isfinite(host(vm)[..., 0])
    gv = np.where(valid[..., None], rng.normal(0, 1, (rows, cols, 4)), 0).astype(np.float32)
    gn = np.where(valid[..., None], rng.normal(0, 1, (rows, cols, 4)), 0).astype(np.float32)
    yield dict(sf=sf, ctx=ctx, gmap=gmap, omap=omap, P=P, R=R, RI=RI, t=t, K=K, zmin=zmin, zmax=zmax,
               zmin_h=host(zmin), zmax_h=host(zmax), invfx=invfx, invfy=invfy, gv=gv, gn=gn, valid=valid,
               mapkw=mapkw, name=request.param)
    ctx.close()


def _gpu_adjoint(s, gv, gn):
    import torch
    sf = s["sf"]
    n = s["mapkw"]["num_sdf_blocks"] * 512
    gsdf = torch.zeros(n, dtype=torch.float32, device="cuda")
    gpose = (C.c_double * 6)()
    gvt, gnt = torch.from_numpy(gv).cuda(), torch.from_numpy(gn).cuda() if gn is not None else None
    sf.call("sf_RaycastAdjoint", s["ctx"].h, s["gmap"].h, sf.image(s["zmin"]), sf.image(s["zmax"]), s["R"], s["RI"],
            s["t"], s["invfx"], s["invfy"], s["K"][2], s["K"][3], sf.image(gvt),
            sf.image(gnt) if gnt is not None else sf.Image(), gsdf.data_ptr(), gpose)
    s["ctx"].sync()
    return np.array(gpose[:]), gsdf.cpu().numpy()


def _L(s, gv, gn, xi=(0, 0, 0, 0, 0, 0), vox=-1, delta=0.0):
    return s["omap"].raycast_smooth_f64(s["P"], s["K"], s["zmin_h"], s["zmax_h"], gv, gn, xi, vox, delta)


@pytest.mark.parametrize("with_normals", [False, True])
def test_pose_gradient_matches_fp64_differences(scene, with_normals):
    s = scene
    assert s["valid"].mean() > 0.5
    gn = s["gn"] if with_normals else None
    g, _ = _gpu_adjoint(s, s["gv"], gn)

    def central(h):
        d = np.zeros(6)
        for k in range(6):
            e = np.zeros(6)
            e[k] = h
            d[k] = (_L(s, s["gv"], gn, e) - _L(s, s["gv"], gn, -e)) / (2 * h)
        return d

    h = H_NORMAL if with_normals else H
    fd = (4 * central(h / 2) - central(h)) / 3
    assert np.linalg.norm(g - fd) <= POSE_RTOL * np.linalg.norm(fd), (g, fd)


def _oracle_index(s, v):
    """The oracle's voxel index of GPU voxel index v: same block position and
    local index (the two maps number their heap blocks differently)."""
    from oracle.oracle import ENTRY_DTYPE
    if "entries" not in s:
        s["entries"] = s["ctx"].download(s["gmap"].arrays().hash_entries, ENTRY_DTYPE, s["gmap"].num_entries)
    e = s["entries"]
    oe = s["omap"].entries
    blk = (v // 512) * 512
    g = e[e["ptr"] == blk][0]
    o = oe[(oe["x"] == g["x"]) & (oe["y"] == g["y"]) & (oe["z"] == g["z"]) & (oe["ptr"] >= 0)][0]
    return int(o["ptr"]) + int(v % 512)


def test_sdf_gradient_matches_fp64_differences(scene):
    s = scene
    _, gs = _gpu_adjoint(s, s["gv"], s["gn"])
    nz = np.flatnonzero(gs)
    assert nz.size > (500000 if s["name"] == "c4" else 1000)
    rng = np.random.default_rng(5)
    pick = np.concatenate([nz[np.argsort(-np.abs(gs[nz]))[:8]], rng.choice(nz, 8, replace=False)])
    scale = np.abs(gs[pick]).max()
    for v in pick:
        ov = _oracle_index(s, int(v))
        fd = (_L(s, s["gv"], s["gn"], vox=ov, delta=H) - _L(s, s["gv"], s["gn"], vox=ov, delta=-H)) / (2 * H)
        assert abs(gs[v] - fd) <= SDF_RTOL * scale, (int(v), gs[v], fd)


def test_adjoint_is_linear_in_the_upstream_gradient(scene):
    s = scene
    g1, s1 = _gpu_adjoint(s, s["gv"], None)
    g2, s2 = _gpu_adjoint(s, 2 * s["gv"], None)
    np.testing.assert_allclose(g2, 2 * g1, rtol=1e-5, atol=1e-9 * np.abs(g1).max())
    np.testing.assert_allclose(s2, 2 * s1, rtol=1e-5, atol=1e-6 * np.abs(s1).max())
