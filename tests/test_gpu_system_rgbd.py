"""The per-frame loop with the photometric term (ComputeSE3 with icpOnly =
false, the reference's default tracking, Tracking/Tracking.cc:170) in its
three forms, 640x480.

Per frame, the GPU's tracking result is checked against the oracle's
ComputeSE3 on the same inputs (this frame's measured pyramid and intensity
pyramid, the model maps the GPU raycast for the previous frame, the last
tracked frame's intensity pyramid, the previous pose): pose within
POSE_TOL, same acceptance and iterations, the photometric correspondence
count of the last iteration within 1e-4 (it is taken at a pose that agrees
to rounding; at equal poses the count is exact, tests/test_gpu_rgb.py).
Over the sequence the trajectory stays within TRAJ_TOL of the oracle's
whole loop and within 5 cm of ground truth; the graph and eager forms agree
bit for bit.
"""
import numpy as np
import pytest

from tests.helpers import C2, MAP_C2, sequence

pytestmark = pytest.mark.gpu

POSE_TOL = 1e-6
TRAJ_TOL = 2e-4
N = 6


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


@pytest.fixture(scope="module")
def seq():
    return sequence(C2["cols"], C2["rows"], C2["K"], N, trajectory=1, dropout=0.02)


def _maps(ctx, imgs):
    return [ctx.download(im.data, np.float32, im.rows * im.cols * 4).reshape(im.rows, im.cols, 4) for im in imgs]


def _inputs(d, rgb, K):
    """Measured pyramid and intensity pyramid of a frame (oracle, pinned to
    the reference's kernels)."""
    from oracle import oracle as O
    _, filt = O.filter_depth(d, 1000.0, 3.0)
    deps = [filt]
    for _ in range(2):
        deps.append(O.pyrdown(deps[-1]))
    vms = [O.vmap(deps[l], *[k / (1 << l) for k in K], 3.0) for l in range(3)]
    imgs = [O.intensity(rgb)]
    for _ in range(2):
        imgs.append(O.pyrdown_u8(imgs[-1]))
    ders = [O.sobel(i) for i in imgs]
    return vms, [O.nmap(v) for v in vms], imgs, [a for a, _ in ders], [b for _, b in ders]


def _run(sf, ctx, seq, mode, check=True):
    from oracle import oracle as O
    K = C2["K"]
    cfg = sf.system_config(cols=C2["cols"], rows=C2["rows"], K=K, use_graph=mode, rgb_term=1, **MAP_C2)
    s = sf.System(ctx, cfg, init_pose=seq[0][3])
    out, prev_pose, last_imgs = [], None, None
    for i, (d, rgb, _, _) in enumerate(seq):
        if check and i > 0:
            model = [s.model_maps(l) for l in range(3)]
            mv = _maps(ctx, [m[0] for m in model])
            mn = _maps(ctx, [m[1] for m in model])
        st = s.grab(d, rgb)
        pose = np.array(st.pose[:]).reshape(4, 4)
        if check:
            vms, nms, imgs, dxs, dys = _inputs(d, rgb, K)
            if i > 0:
                ok, Po, ost = O.compute_se3(vms, nms, mv, mn, K, (10, 5, 4), (2000, 1000, 100), 1e-4, prev_pose,
                                            prev_pose, rgb=(imgs, last_imgs, dxs, dys))
                assert ok == bool(st.accepted), "frame %d acceptance" % i
                assert int(ost[2]) == st.iterations, "frame %d iterations" % i
                # counted at the last iteration's pose, which agrees to rounding:
                # a correspondence test can flip at the 1e-7 level
                assert abs(int(ost[5]) - st.rgb_count) <= 1e-4 * ost[5], "frame %d photometric count" % i
                assert np.abs(Po - pose).max() < POSE_TOL, "frame %d pose" % i
            if st.tracked:
                last_imgs = imgs
        prev_pose = pose
        out.append((st.tracked, pose, st.iterations, st.visible, st.allocated, st.flags, st.rgb_count))
    s.close()
    return out


@pytest.mark.parametrize("mode", [0, 2, 1])
def test_system_rgbd_per_frame_and_trajectory(lib, seq, mode):
    from oracle import oracle as O
    sf, ctx = lib
    gpu = _run(sf, ctx, seq, mode)
    osys = O.System(MAP_C2, C2["cols"], C2["rows"], C2["K"], init_pose=seq[0][3], rgb_term=True)
    for i, (d, rgb, _, Pgt) in enumerate(seq):
        ok, P, st = osys.grab(d, rgb)
        g = gpu[i]
        assert bool(g[0]) == ok, "frame %d" % i
        assert g[5] == 0
        assert np.abs(g[1] - P).max() < TRAJ_TOL, "frame %d" % i
        assert np.linalg.norm(g[1][:3, 3] - Pgt[:3, 3]) < 0.05
        if i > 0:
            assert g[6] > 10000  # the photometric term ran


def test_system_rgbd_graph_equals_eager(lib, seq):
    sf, ctx = lib
    a = _run(sf, ctx, seq, 1, check=False)
    b = _run(sf, ctx, seq, 2, check=False)
    for x, y in zip(a, b):
        assert x[0] == y[0] and np.array_equal(x[1], y[1]) and x[2:] == y[2:]
