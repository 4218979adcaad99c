"""Next-pose prediction of the persistent ICP kernel (sf_icp_predict).

While the FP64 solve of an iteration runs, one warp predicts the float pose
it will give and the pixel warps accumulate the next iteration's rows on
the prediction; the rows are kept only when the prediction equals the FP64
path's float pose in every bit.  So the loop's results must not depend on
the prediction: the same sequence with the prediction on and off gives the
same stats and poses bit for bit, in the ICP-only and the photometric
(RGB-D) forms, eager and graph.  The phase-clock slot that records whether
an iteration's rows came from a prediction shows that predictions were
made and held (the test is not vacuous).
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, C2, MAP_C1, MAP_C2, sequence

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sf(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    return sf


def _run(sf, cfgd, mcfg, seq, predict, use_graph, rgb):
    ctx = sf.Context()
    sf.call("sf_icp_predict", ctx.h, int(predict))
    if use_graph == 2:
        sf.call("sf_icp_profile", ctx.h, 1, None)
    cfg = sf.system_config(cols=cfgd["cols"], rows=cfgd["rows"], K=cfgd["K"], use_graph=use_graph, rgb_term=int(rgb),
                           **mcfg)
    s = sf.System(ctx, cfg, init_pose=seq[0][3])
    prof = (C.c_uint64 * (64 * 16))()
    out, predicted = [], 0
    for d, rgbi, _, _ in seq:
        st = s.grab(d, rgbi)
        out.append((np.array(st.pose[:]), st.iterations, st.icp_count, st.icp_error, st.rgb_count, st.rgb_error,
                    st.tracked, st.accepted, st.fail, st.visible))
        if use_graph == 2:
            sf.call("sf_icp_profile", ctx.h, 1, prof)
            p = np.array(prof[:], np.uint64).reshape(64, 16)
            predicted += int((p[:st.iterations, 7] != 0).sum())
    s.close()
    ctx.close()
    return out, predicted


@pytest.mark.parametrize("rgb", [False, True])
@pytest.mark.parametrize("use_graph", [2, 1])
def test_prediction_changes_nothing(sf, use_graph, rgb):
    seq = sequence(C1["cols"], C1["rows"], C1["K"], 12, dropout=0.02)
    on, npred = _run(sf, C1, MAP_C1, seq, True, use_graph, rgb)
    off, _ = _run(sf, C1, MAP_C1, seq, False, use_graph, rgb)
    for i, (a, b) in enumerate(zip(on, off)):
        assert np.array_equal(a[0], b[0]), "frame %d pose" % i
        assert a[1:] == b[1:], "frame %d stats" % i
    if use_graph == 2:
        iters = sum(o[1] for o in on)
        # every iteration but the first of a frame can take predicted rows
        assert npred > 0.8 * (iters - len(on)), (npred, iters)


def test_prediction_changes_nothing_640x480(sf):
    seq = sequence(C2["cols"], C2["rows"], C2["K"], 8, trajectory=1, seed=2, dropout=0.02)
    on, npred = _run(sf, C2, MAP_C2, seq, True, 2, False)
    off, _ = _run(sf, C2, MAP_C2, seq, False, 2, False)
    for i, (a, b) in enumerate(zip(on, off)):
        assert np.array_equal(a[0], b[0]) and a[1:] == b[1:], "frame %d" % i
    iters = sum(o[1] for o in on)
    assert npred > 0.8 * (iters - len(on)), (npred, iters)
