"""The 1280x720 corridor stress configuration (4-level pyramid, 3 mm voxels,
2^22 buckets, forward trajectory at 1.5 cm per frame; see tests.helpers.C3)
through the whole loop
in its graph form.  Per frame, the GPU's ComputeSE3 result equals the
oracle's on the same inputs (the frame's measured 4-level pyramid and the
model maps the GPU raycast for the previous frame) within ICP_POSE_TOL, with
the same acceptance and iteration count; over the run the trajectory stays
within TRAJ_TOL of the oracle's whole loop and the allocated block sets
agree."""
import numpy as np
import pytest

from tests.helpers import C3, C3_ICP, C3_SEQ, MAP_C3, cuda, empty, host, map_to_host, positions, sequence

pytestmark = pytest.mark.gpu

ICP_POSE_TOL = 1e-6
TRAJ_TOL = 2e-4
N = 5


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _pyramid(sf, ctx, d, K, levels):
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
    return [host(v) for v in vms], [host(n) for n in nms]


def _maps(ctx, imgs):
    return [ctx.download(im.data, np.float32, im.rows * im.cols * 4).reshape(im.rows, im.cols, 4) for im in imgs]


def test_corridor_loop_matches_oracle(lib):
    from oracle import oracle as O
    sf, ctx = lib
    K, L = C3["K"], C3_ICP["levels"]
    seq = sequence(C3["cols"], C3["rows"], K, N, **C3_SEQ)
    cfg = sf.system_config(cols=C3["cols"], rows=C3["rows"], K=K, use_graph=1, **C3_ICP, **MAP_C3)
    s = sf.System(ctx, cfg, init_pose=seq[0][3])
    osys = O.System(MAP_C3, C3["cols"], C3["rows"], K, init_pose=seq[0][3], **C3_ICP)
    prev = None
    try:
        for i in range(N):
            d, rgb, _, Pgt = seq[i]
            if i > 0:
                model = [s.model_maps(l) for l in range(L)]
                mv, mn = _maps(ctx, [m[0] for m in model]), _maps(ctx, [m[1] for m in model])
            st = s.grab(d, rgb)
            pose = np.array(st.pose[:]).reshape(4, 4)
            assert st.flags == 0
            if i > 0:
                vms, nms = _pyramid(sf, ctx, d, K, L)
                ok, Po, ost = O.compute_se3(vms, nms, mv, mn, K, C3_ICP["iters"], C3_ICP["min_count"], 1e-4,
                                            prev, prev)
                assert ok == bool(st.accepted), "frame %d acceptance" % i
                assert int(ost[2]) == st.iterations, "frame %d iterations" % i
                assert np.abs(Po - pose).max() < ICP_POSE_TOL, "frame %d ICP pose" % i
            ok, P, _ = osys.grab(d, rgb)
            assert bool(st.tracked) == ok, "frame %d" % i
            assert np.abs(pose - P).max() < TRAJ_TOL, "frame %d" % i
            assert np.linalg.norm(pose[:3, 3] - Pgt[:3, 3]) < 0.05
            prev = pose
        assert st.visible > 1000
        e, _, _ = map_to_host(ctx, s.map())
        oe = osys.entries()
        a, b = positions(e[e["ptr"] >= 0]), positions(oe[oe["ptr"] >= 0])
        assert len(b) > 5000 and len(a ^ b) <= 0.01 * len(b)
    finally:
        s.close()
