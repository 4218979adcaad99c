"""sf_system_autotune (the Autotune entry point, no counterpart in the
reference): it times the last frame's raycast under each launch shape and
keeps the fastest.  Every shape computes the same maps, so a system that
autotunes mid-sequence must produce the same poses, statistics and model
maps, bit for bit, as one that does not."""
import numpy as np
import pytest

from tests.helpers import C1, MAP_C1, sequence

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _model(ctx, s, levels=3):
    out = []
    for l in range(levels):
        for im in s.model_maps(l):
            a = ctx.download(im.data, np.float32, im.rows * im.cols * 4)
            out.append(a.reshape(im.rows, im.cols, 4).view(np.uint32))
    return out


@pytest.mark.parametrize("mode", [1, 0])
def test_autotune_changes_no_result(lib, mode):
    sf, ctx = lib
    seq = sequence(C1["cols"], C1["rows"], C1["K"], 7, trajectory=1, dropout=0.02)
    cfg = sf.system_config(cols=C1["cols"], rows=C1["rows"], K=C1["K"], use_graph=mode, **MAP_C1)
    a = sf.System(ctx, cfg, init_pose=seq[0][3])
    b = sf.System(ctx, cfg, init_pose=seq[0][3])
    try:
        _compare(sf, ctx, seq, a, b)
    finally:
        a.close()
        b.close()


def _compare(sf, ctx, seq, a, b):
    with pytest.raises(sf.SfError):
        b.autotune(reps=2)  # no frame grabbed yet
    for d, rgb, _, _ in seq[:3]:
        a.grab(d, rgb)
        b.grab(d, rgb)
    cands, chosen = b.autotune(reps=3)
    assert len(cands) == 6 and 0 <= chosen < 6
    assert all(ms > 0 for _, _, _, ms in cands)
    assert {(m, x, y) for m, x, y, _ in cands} == {(m, x, y) for m in (8, 6) for x, y in ((8, 16), (16, 8), (32, 4))}
    for x, y in zip(_model(ctx, a), _model(ctx, b)):  # the timing runs left the model maps as they were
        np.testing.assert_array_equal(x, y)
    for d, rgb, _, _ in seq[3:]:
        sa = a.grab(d, rgb)
        sb = b.grab(d, rgb)
        assert np.array_equal(np.array(sa.pose[:]), np.array(sb.pose[:]))
        assert (sa.tracked, sa.iterations, sa.icp_count, sa.visible) == (sb.tracked, sb.iterations, sb.icp_count,
                                                                       sb.visible)
    for x, y in zip(_model(ctx, a), _model(ctx, b)):
        np.testing.assert_array_equal(x, y)
    with pytest.raises(sf.SfError):
        b.autotune(reps=0)
