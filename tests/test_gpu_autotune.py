"""sf_system_autotune (the Autotune entry point, no counterpart in the
reference): it times the last frame's raycast under each launch shape, the
integration under each grid size and the allocation walk's probe under each
pixel tile, in the state the frame left, and keeps the fastest.  Every shape computes the same maps, so a system that
autotunes mid-sequence, or takes any shape by sf_system_set_tune, must
produce the same poses, statistics, model maps and map, bit for bit, as one
that does not; and the timing runs must leave the map and model maps as
they were.  semantic_icpslam_gb300.tune caches the choice per
configuration as JSON."""
import numpy as np
import pytest

from tests.helpers import C1, MAP_C1, map_to_host, sequence, voxels_by_pos

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
    import ctypes as C
    rep = sf._lib.AutotuneReport()
    sf.call("sf_system_autotune", b.h, 3, C.byref(rep))
    cands = [(rep.minb[i], rep.tile_x[i], rep.tile_y[i], rep.ms[i]) for i in range(rep.candidates)]
    assert len(cands) == 6 and 0 <= rep.chosen < 6
    assert all(ms > 0 for _, _, _, ms in cands)
    assert {(m, x, y) for m, x, y, _ in cands} == {(m, x, y) for m in (8, 6) for x, y in ((8, 16), (16, 8), (32, 4))}
    assert rep.integrate_candidates == 4 and 0 <= rep.integrate_chosen < 4
    assert [rep.integrate_ctas[i] for i in range(4)] == [2, 4, 8, 16] and min(rep.integrate_ms[:4]) > 0
    assert rep.alloc_candidates == 4 and 0 <= rep.alloc_chosen < 4 and min(rep.alloc_ms[:4]) > 0
    assert [(rep.alloc_tile_x[i], rep.alloc_tile_y[i]) for i in range(4)] == [(32, 8), (64, 4), (16, 16), (128, 2)]
    t = sf._lib.FrameTune()
    sf.call("sf_system_get_tune", b.h, C.byref(t))
    assert t.raycast == rep.chosen and t.integrate_ctas_per_sm == rep.integrate_ctas[rep.integrate_chosen]
    assert t.alloc_tile == rep.alloc_chosen
    for x, y in zip(_model(ctx, a), _model(ctx, b)):  # the timing runs left the model maps as they were
        np.testing.assert_array_equal(x, y)
    ea, va, _ = map_to_host(ctx, a.map())  # and the voxels the integration runs touched (per block
    eb, vb, _ = map_to_host(ctx, b.map())  # position: which heap block a block takes varies between runs)
    ka, xa = voxels_by_pos(ea, va)
    kb, xb = voxels_by_pos(eb, vb)
    assert ka == kb and np.array_equal(xa.view(np.uint8), xb.view(np.uint8))
    # the least likely shapes: the results still do not change
    far = sf._lib.FrameTune(5, 2, 2)
    sf.call("sf_system_set_tune", b.h, C.byref(far))
    with pytest.raises(sf.SfError):
        sf.call("sf_system_set_tune", b.h, C.byref(sf._lib.FrameTune(6, 8, 0)))
    with pytest.raises(sf.SfError):
        sf.call("sf_system_set_tune", b.h, C.byref(sf._lib.FrameTune(0, 8, 4)))
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


def test_every_raycast_shape_same_maps(lib):
    """Each raycast launch shape gives the default shape's poses,
    statistics and model maps, bit for bit."""
    sf, ctx = lib
    seq = sequence(C1["cols"], C1["rows"], C1["K"], 4, trajectory=1, dropout=0.02)
    cfg = sf.system_config(cols=C1["cols"], rows=C1["rows"], K=C1["K"], use_graph=1, **MAP_C1)
    import ctypes as C

    def run(shape):
        s = sf.System(ctx, cfg, init_pose=seq[0][3])
        try:
            if shape is not None:
                sf.call("sf_system_set_tune", s.h, C.byref(sf._lib.FrameTune(shape, 8, 0)))
            out = []
            for d, rgb, _, _ in seq:
                st = s.grab(d, rgb)
                out.append((np.array(st.pose[:]), st.iterations, st.icp_count, st.visible, _model(ctx, s)))
            return out
        finally:
            s.close()

    ref = run(None)
    for shape in range(6):
        for i, (x, y) in enumerate(zip(ref, run(shape))):
            assert np.array_equal(x[0], y[0]) and x[1:4] == y[1:4], (shape, i)
            for u, v in zip(x[4], y[4]):
                np.testing.assert_array_equal(u, v, err_msg="shape %d frame %d" % (shape, i))


def test_tune_cache_per_configuration(lib, tmp_path):
    """The first system of a configuration times and caches; the next takes
    the cached shapes without timing."""
    import ctypes as C
    from semantic_icpslam_gb300 import tune as T
    sf, ctx = lib
    seq = sequence(C1["cols"], C1["rows"], C1["K"], 2, trajectory=1, dropout=0.02)
    cfg = sf.system_config(cols=C1["cols"], rows=C1["rows"], K=C1["K"], use_graph=1, **MAP_C1)
    path = str(tmp_path / "tune.json")
    s1 = sf.System(ctx, cfg, init_pose=seq[0][3])
    s1.grab(seq[0][0], seq[0][1])
    e1, cached1 = T.tuned(s1, reps=2, path=path)
    s2 = sf.System(ctx, cfg, init_pose=seq[0][3])
    e2, cached2 = T.tuned(s2, reps=2, path=path)  # before any frame: only the cache can serve it
    assert not cached1 and cached2 and e1 == e2
    t = sf._lib.FrameTune()
    sf.call("sf_system_get_tune", s2.h, C.byref(t))
    assert (t.raycast, t.integrate_ctas_per_sm, t.alloc_tile) == (e1["raycast"], e1["integrate_ctas_per_sm"],
                                                                  e1["alloc_tile"])
    s1.close()
    s2.close()
