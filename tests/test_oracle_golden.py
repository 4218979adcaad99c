"""Pins the oracle to the reference's own device code.

tests/golden/g1.npz holds outputs of the reference's Tracking/ and Mapping/
kernels (compiled for the CPU by oracle/ref_shim/build_ref.py, generated by
tests/golden/make_golden.py) on seeded 128x96 inputs.  The oracle must
reproduce them bit-for-bit: filtered depth, pyramid levels, vertex and
normal maps, ResizeMap, per-pixel ICP rows, and after five FuseMapColor
frames the allocated block set, heapCounter / entryPtr, the visible sets and
every voxel byte of every block; then the z-range and the raycast from two
poses, and AnalyzeMapSemantics.
"""
import hashlib
import os

import numpy as np
import pytest

from tests.helpers import same_nan

G1 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "g1.npz")


@pytest.fixture(scope="module")
def g(built):
    return dict(np.load(G1))


def _K(g, level=0):
    div = float(1 << level)
    return tuple(float(k) / div for k in g["K"])


def test_filter_depth(g):
    from oracle import oracle as O
    for i in range(2):
        raw, filt = O.filter_depth(g["depth%d" % i], 1000.0, 3.0)
        assert same_nan(raw, g["raw%d" % i])
        assert same_nan(filt, g["filt%d" % i])


def test_pyramid(g):
    from oracle import oracle as O
    for i in range(2):
        for l in range(3):
            d = g["f%d_depth%d" % (i, l)]
            if l > 0:
                assert same_nan(O.pyrdown(g["f%d_depth%d" % (i, l - 1)]), d)
            vm = O.vmap(d, *_K(g, l), 3.0)
            assert same_nan(vm[..., 0], g["f%d_vmap%d" % (i, l)][..., 0])
            valid = ~np.isnan(vm[..., 0])
            assert np.array_equal(vm[valid], g["f%d_vmap%d" % (i, l)][valid])
            assert same_nan(O.nmap(vm), g["f%d_nmap%d" % (i, l)])


def test_resize(g):
    from oracle import oracle as O
    vd, nd = O.resize(g["resize_vsrc"], g["resize_nsrc"])
    assert same_nan(vd, g["resize_vdst"])
    assert same_nan(nd, g["resize_ndst"])


def test_icp_rows(g):
    from oracle import oracle as O
    for l in range(3):
        rows = O.icp_rows(g["f1_vmap%d" % l], g["f0_vmap%d" % l], g["f1_nmap%d" % l], g["f0_nmap%d" % l],
                          g["icp_pose_curr"], g["pose0"], _K(g, l))
        assert np.array_equal(np.frombuffer(hashlib.sha1(rows.tobytes()).digest(), np.uint8),
                              g["icp_rows_sha1_%d" % l]), "level %d" % l
        np.testing.assert_allclose(rows.astype(np.float64).sum(0), g["icp_sums%d" % l], rtol=1e-12)
    assert rows[:, 28].sum() > 50


def _oracle_map(g):
    from oracle import oracle as O
    c = g["consts"]
    return O.Map(voxel_size=float(np.float32(c[0])), trunc_dist=float(np.float32(c[1])), num_buckets=int(c[2]),
                 num_excess=int(c[3]), num_sdf_blocks=int(c[4]), depth_min=float(np.float32(c[5])),
                 depth_max=float(np.float32(c[6])))


def _frame(g, i):
    from oracle import oracle as O
    raw, filt = O.filter_depth(g["depth%d" % i], 1000.0, 3.0)
    nm = O.nmap(O.vmap(filt, *_K(g), 3.0))
    return raw, filt, nm


def _digests(m):
    e = m.entries
    sel = e[e["ptr"] >= 0]
    order = np.lexsort((sel["z"], sel["y"], sel["x"]))
    sel = sel[order]
    pos = np.stack([sel["x"], sel["y"], sel["z"]], 1).astype(np.int32)
    vox = m.voxels.view(np.uint8)
    dig = np.stack([np.frombuffer(hashlib.sha1(vox[p * 16:(p + 512) * 16].tobytes()).digest(), np.uint8)
                    for p in sel["ptr"]])
    return pos, dig


def _pos_sorted(e):
    return np.sort(np.stack([e["x"], e["y"], e["z"]], 1).astype(np.int32).view(
        [("x", "<i4"), ("y", "<i4"), ("z", "<i4")]).ravel())


@pytest.fixture(scope="module")
def fused(g):
    m = _oracle_map(g)
    counters = []
    for i in range(5):
        raw, _, nm = _frame(g, i)
        n = m.fuse(raw, g["rgb%d" % i], nm, g["mask%d" % i], 10 if i >= 2 else 0, g["pose%d" % i], _K(g))
        counters.append((m.counters(), n))
    return m, counters


def test_fuse_map(g, fused):
    m, counters = fused
    for i, (c, n) in enumerate(counters):
        ref = g["counters"][i]
        assert c[0] == ref[0] and c[1] == ref[1], "frame %d heapCounter/entryPtr" % i
        assert n == ref[2] == len(g["visible%d" % i]), "frame %d visible count" % i
    assert g["counters"][-1][3] > 500  # blocks allocated
    pos, dig = _digests(m)
    assert np.array_equal(pos, g["map_pos"])
    assert np.array_equal(dig, g["map_sha1"])


def test_visible_sets(g):
    m = _oracle_map(g)
    for i in range(5):
        raw, _, nm = _frame(g, i)
        n = m.fuse(raw, g["rgb%d" % i], nm, g["mask%d" % i], 10 if i >= 2 else 0, g["pose%d" % i], _K(g))
        assert np.array_equal(_pos_sorted(m.visible[:n]), g["visible%d" % i])


def test_raytrace(g, fused):
    from oracle import oracle as O
    m, _ = fused
    cols, rows = g["depth0"].shape[1], g["depth0"].shape[0]
    for k, fi in enumerate((4, 5)):
        P = g["pose%d" % fi]
        n = m.visibility(P, _K(g), cols, rows)
        assert n == int(g["ray%d_nvis" % k])
        ok, zmin, zmax, _, nb = m.zrange(P, _K(g), 80, 60)
        assert ok == bool(g["ray%d_ok" % k]) and nb == int(g["ray%d_nblocks" % k])
        assert same_nan(zmin, g["ray%d_zmin" % k])
        assert same_nan(zmax, g["ray%d_zmax" % k])
        vm, nm = m.raycast(P, _K(g), cols, rows, zmin, zmax)
        assert same_nan(vm, g["ray%d_vmap" % k])
        assert same_nan(nm, g["ray%d_nmap" % k])
        assert np.isfinite(vm[..., 0]).mean() > 0.5


def test_analyze_semantics(g):
    m = _oracle_map(g)
    for i in range(5):
        raw, _, nm = _frame(g, i)
        m.fuse(raw, g["rgb%d" % i], nm, g["mask%d" % i], 10 if i >= 2 else 0, g["pose%d" % i], _K(g))
    cols, rows = g["depth0"].shape[1], g["depth0"].shape[0]
    # the two raytrace visibility passes, then AnalyzeMapSemantics from frame 4
    m.visibility(g["pose4"], _K(g), cols, rows)
    m.visibility(g["pose5"], _K(g), cols, rows)
    raw, _, nm = _frame(g, 4)
    m.visibility(g["pose4"], _K(g), cols, rows)
    m.analyze_semantics(raw, g["rgb4"], nm, g["mask4"], 10, g["pose4"], _K(g))
    pos, dig = _digests(m)
    assert np.array_equal(pos, g["sem_pos"])
    assert np.array_equal(dig, g["sem_sha1"])


def load_unify_state(m, g):
    """The seeded UnifyNeighbor state of the fixtures into an oracle map."""
    from oracle.oracle import ENTRY_DTYPE
    m.entries[:] = np.ascontiguousarray(g["uni_entries"]).view(ENTRY_DTYPE).ravel()
    vox = g["uni_vox"]
    m.voxels.view(np.uint8).reshape(-1, 16)[:len(vox)] = vox
    return len(vox)


def test_unify_neighbor(g):
    """UnifyNeighborKernel alone on the seeded state (chains through the
    excess list, full neighbour tables, zero counts, the count_2 + 5 wrap),
    over half the bucket slots and over every slot."""
    for k, nvis in enumerate(g["uni_nvis"]):
        m = _oracle_map(g)
        n = load_unify_state(m, g)
        m.unify_neighbor(int(nvis))
        got = m.voxels.view(np.uint8).reshape(-1, 16)[:n]
        assert np.array_equal(got[:, 8:12], g["uni_out%d" % k]), "nvis %d" % nvis
        assert np.array_equal(np.delete(got, [8, 9, 10, 11], 1), np.delete(g["uni_vox"], [8, 9, 10, 11], 1))
    # the pass is not the identity on this state
    assert (g["uni_out0"] != g["uni_vox"][:, 8:12]).any(1).sum() > 1000


def test_intensity_pyramid(g):
    """ImageToIntensity, PyrDownGauss(unsigned char), ComputeDerivativeImage."""
    from oracle import oracle as O
    for i in range(2):
        img = O.intensity(g["rgb%d" % i])
        for l in range(3):
            if l > 0:
                img = O.pyrdown_u8(img)
            assert np.array_equal(img, g["f%d_int%d" % (i, l)]), "frame %d level %d" % (i, l)
            dx, dy = O.sobel(img)
            assert np.array_equal(dx, g["f%d_dx%d" % (i, l)])
            assert np.array_equal(dy, g["f%d_dy%d" % (i, l)])


def test_rgb_rows(g):
    """RGBStep's correspondences, integer sums, sigma and per-pixel rows."""
    from oracle import oracle as O
    for l in range(3):
        sums, res, sigma, rows = O.rgb_step(g["f1_int%d" % l], g["f0_int%d" % l], g["f1_vmap%d" % l],
                                            g["f0_vmap%d" % l], g["f1_dx%d" % l], g["f1_dy%d" % l],
                                            g["icp_pose_curr"], g["pose0"], _K(g, l), rows=True)
        assert res == tuple(int(v) for v in g["rgb_res%d" % l]), "level %d" % l
        assert np.float32(sigma) == g["rgb_sigma%d" % l][0]
        assert np.array_equal(np.frombuffer(hashlib.sha1(rows.tobytes()).digest(), np.uint8),
                              g["rgb_rows_sha1_%d" % l]), "level %d" % l
        np.testing.assert_allclose(sums, g["rgb_sums%d" % l], rtol=1e-12)
    assert g["rgb_res0"][0] > 5000


def mesh_records(v, n, c):
    """Sorted distinct vertex records (position, normal, colour, 28 bytes),
    as tests/golden/make_golden.py makes them."""
    k = v.reshape(-1, 3).shape[0]
    rec = np.zeros((k, 28), np.uint8)
    rec[:, :12] = np.ascontiguousarray(v.reshape(-1, 3)).view(np.uint8).reshape(k, 12)
    rec[:, 12:24] = np.ascontiguousarray(n.reshape(-1, 3)).view(np.uint8).reshape(k, 12)
    rec[:, 24:27] = c.reshape(-1, 3)
    return np.unique(rec, axis=0)


def test_mesh(g, fused):
    """MeshScene on the five fused frames' map: the same triangle count and
    the same set of vertex records (every active edge of every cube: its
    interpolated position, normal and colour) as the reference's kernel.
    Each cube's polygons are the reference table's (tests/test_oracle_mesh.py);
    only their split into triangles differs, which neither measure sees."""
    m, _ = fused
    v, n, c = m.mesh(1000000)
    assert len(v) == int(g["mesh_ntri"])
    recs = mesh_records(v, n, c)
    assert len(recs) == int(g["mesh_nrec"])
    assert np.array_equal(np.frombuffer(hashlib.sha1(recs.tobytes()).digest(), np.uint8), g["mesh_rec_sha1"])
