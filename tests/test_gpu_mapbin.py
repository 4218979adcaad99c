"""map.bin checkpoints (System::WriteMapToDisk / ReadMapFromDisk,
Core/System.cc:327-403; arrays of Mapping::DownloadToRAM / UploadFromRAM,
Mapping/Mapping.cc:205-250).

The layout is restated here from the reference's writer (read_map_bin /
write_map_bin) and checked against the library both ways:
  * a map the GPU loop built is written by sf_map_write and parsed here:
    every field equals the device arrays;
  * the file read back by sf_map_read into a fresh map gives the same
    arrays and the same raycast, bit for bit;
  * an oracle map written here in the reference's layout and read by
    sf_map_read renders exactly as the oracle renders it;
  * wrong sizes, a missing file and a truncated file are rejected.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, MAP_C1, cuda, empty, host, same_nan, sequence
from tests.test_gpu_fusion import _frame_inputs

pytestmark = pytest.mark.gpu

MAX_KEYS = 100000              # KeyMap::MaxKeys (Mapping/DeviceMap.h:207)
KEY_ENTRIES = MAX_KEYS * 5     # KeyMap::maxEntries
SURF_BYTES = 288               # sizeof(SURF): bool valid, float3 pos, float4 normal, float[64]


def _dtypes():
    from oracle import oracle as O
    return O.ENTRY_DTYPE, O.VOXEL_DTYPE


def read_map_bin(path):
    """The fields of a map.bin in the reference writer's order."""
    entry, voxel = _dtypes()
    buf = open(path, "rb").read()
    nsdf, nb, nvox, ne = np.frombuffer(buf, "<i4", 4, 0)
    off = 16
    out = {"header": (int(nsdf), int(nb), int(nvox), int(ne))}
    out["heap_counter"], out["entry_ptr"], out["no_visible"] = (int(v) for v in np.frombuffer(buf, "<i4", 3, off))
    off += 12
    for name, dt, n in (("heap", np.dtype("<i4"), nsdf), ("bucket_mutex", np.dtype("<i4"), nb),
                        ("voxels", voxel, nvox), ("entries", entry, ne), ("visible", entry, ne),
                        ("key_mutex", np.dtype("<i4"), MAX_KEYS), ("keys", np.dtype("u1"), KEY_ENTRIES * SURF_BYTES)):
        out[name] = np.frombuffer(buf, dt, int(n), off)
        off += dt.itemsize * int(n)
    out["size_ok"] = off == len(buf)
    return out


def write_map_bin(path, nsdf, nb, ne, counters, heap, mutex, voxels, entries, visible):
    """A map.bin in the reference writer's order (a reset key map at the end)."""
    with open(path, "wb") as f:
        f.write(np.array([nsdf, nb, nsdf * 512, ne], "<i4").tobytes())
        f.write(np.array(counters[:3], "<i4").tobytes())
        for a in (heap, mutex, voxels, entries, visible):
            f.write(np.ascontiguousarray(a).tobytes())
        f.write(np.full(MAX_KEYS, -1, "<i4").tobytes())
        f.write(bytes(KEY_ENTRIES * SURF_BYTES))


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _device_arrays(sf, ctx, m):
    entry, voxel = _dtypes()
    a = m.arrays()
    nsdf, ne, nb = MAP_C1["num_sdf_blocks"], m.num_entries, MAP_C1["num_buckets"]
    return {
        "heap": ctx.download(a.heap_mem, np.int32, nsdf),
        "bucket_mutex": ctx.download(a.bucket_mutex, np.int32, nb),
        "voxels": ctx.download(a.voxel_blocks, np.uint8, nsdf * 512 * 16).view(voxel),
        "entries": ctx.download(a.hash_entries, np.uint8, ne * 32).view(entry),
        "visible": ctx.download(a.visible_entries, np.uint8, ne * 32).view(entry),
    }


def _render(sf, ctx, gmap, P, K, cols, rows):
    import torch
    R, RI, t = sf.pose_to_gpu(P)
    nvis = C.c_uint32()
    sf.call("sf_CheckBlockVisibility", ctx.h, gmap.h, R, RI, t, cols, rows, *K, 3.0, 0.1, C.byref(nvis))
    zc, zr = (cols + 7) // 8, (rows + 7) // 8
    zmin, zmax = empty((zr, zc), torch.float32), empty((zr, zc), torch.float32)
    blocks = empty((260000, 16), torch.uint8)
    nblk = empty((1,), torch.int32)
    ok = C.c_int()
    sf.call("sf_CreateRenderingBlocks", ctx.h, gmap.h, sf.image(zmin), sf.image(zmax), 3.0, 0.1,
            blocks.data_ptr(), nblk.data_ptr(), RI, t, nvis.value, *K, C.byref(ok))
    vm, nm = empty((rows, cols, 4), torch.float32), empty((rows, cols, 4), torch.float32)
    invfx = float(np.float32(1.0 / np.float64(np.float32(K[0]))))
    invfy = float(np.float32(1.0 / np.float64(np.float32(K[1]))))
    sf.call("sf_Raycast", ctx.h, gmap.h, sf.image(vm), sf.image(nm), sf.image(zmin), sf.image(zmax), R, RI, t,
            invfx, invfy, K[2], K[3])
    ctx.sync()
    return nvis.value, host(zmin), host(zmax), host(vm), host(nm)


def test_write_then_read_round_trip(lib, tmp_path):
    sf, ctx = lib
    K, cols, rows = C1["K"], C1["cols"], C1["rows"]
    seq = sequence(cols, rows, K, 5, trajectory=1, dropout=0.02)
    cfg = sf.system_config(cols=cols, rows=rows, K=K, use_graph=1, **MAP_C1)
    s = sf.System(ctx, cfg, init_pose=seq[0][3])
    try:
        for d, rgb, _, _ in seq[:4]:
            s.grab(d, rgb)
        m = s.map()
        path = str(tmp_path / "map.bin")
        m.write(ctx, path)
        f = read_map_bin(path)
        assert f["size_ok"]
        assert f["header"] == (MAP_C1["num_sdf_blocks"], MAP_C1["num_buckets"], MAP_C1["num_sdf_blocks"] * 512,
                               m.num_entries)
        ctr = m.counters(ctx)
        assert (f["heap_counter"], f["entry_ptr"], f["no_visible"]) == tuple(ctr[:3])
        dev = _device_arrays(sf, ctx, m)
        for k in ("heap", "bucket_mutex", "voxels", "entries", "visible"):
            assert np.array_equal(f[k].view(np.uint8), dev[k].view(np.uint8)), k
        assert (f["entries"]["ptr"] >= 0).sum() == ctr[3] > 100
        assert np.all(f["key_mutex"] == -1) and not f["keys"].any()
        # read back into a fresh map of the same sizes
        g = sf.Map(**MAP_C1)
        g.read(ctx, path)
        dev2 = _device_arrays(sf, ctx, g)
        for k in dev:
            assert np.array_equal(dev2[k].view(np.uint8), dev[k].view(np.uint8)), k
        assert g.counters(ctx) == ctr
        P = seq[4][3]
        r1 = _render(sf, ctx, m, P, K, cols, rows)
        r2 = _render(sf, ctx, g, P, K, cols, rows)
        assert r1[0] == r2[0] > 0
        for a, b in zip(r1[1:], r2[1:]):
            assert same_nan(a, b)
        g.close()
    finally:
        s.close()


def test_reference_layout_file_renders_as_the_oracle(lib, tmp_path):
    from oracle import oracle as O
    sf, ctx = lib
    K, cols, rows = C1["K"], C1["cols"], C1["rows"]
    seq = sequence(cols, rows, K, 4, trajectory=1, dropout=0.02)
    omap = O.Map(**MAP_C1)
    for d, rgb, mask, P in seq[:3]:
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        omap.fuse(f["raw_h"], rgb, f["nmap_h"], None, 0, P, K)
    nsdf, nb = MAP_C1["num_sdf_blocks"], MAP_C1["num_buckets"]
    path = str(tmp_path / "oracle_map.bin")
    write_map_bin(path, nsdf, nb, omap.num_entries, omap.counters(), omap.heap, np.full(nb, -1, "<i4"),
                  omap.voxels, omap.entries, omap.visible)
    g = sf.Map(**MAP_C1)
    g.read(ctx, path)
    dev = _device_arrays(sf, ctx, g)
    assert np.array_equal(dev["voxels"].view(np.uint8), omap.voxels.view(np.uint8))
    assert np.array_equal(dev["entries"].view(np.uint8), omap.entries.view(np.uint8))
    assert g.counters(ctx)[:3] == list(omap.counters()[:3])
    P = seq[3][3]
    nvis, zmin, zmax, vm, nm = _render(sf, ctx, g, P, K, cols, rows)
    assert nvis == omap.visibility(P, K, cols, rows) > 0
    zc, zr = (cols + 7) // 8, (rows + 7) // 8
    _, ozmin, ozmax, _, _ = omap.zrange(P, K, zc, zr, max_blocks=1)
    assert same_nan(zmin, ozmin) and same_nan(zmax, ozmax)
    ovm, onm = O.Map.raycast(omap, P, K, cols, rows, ozmin, ozmax)
    assert np.isfinite(ovm[..., 0]).mean() > 0.5
    assert same_nan(vm, ovm)
    assert same_nan(nm, onm)
    g.close()


def test_bad_files_rejected(lib, tmp_path):
    sf, ctx = lib
    g = sf.Map(**MAP_C1)
    with pytest.raises(sf.SfError) as e:
        g.read(ctx, str(tmp_path / "missing.bin"))
    assert e.value.status == sf._lib.SF_ERR_IO
    path = str(tmp_path / "small.bin")
    small = dict(MAP_C1)
    small["num_sdf_blocks"] = 1 << 10
    h = sf.Map(**small)
    h.write(ctx, path)
    with pytest.raises(sf.SfError) as e:
        g.read(ctx, path)  # sizes differ from this map's
    assert e.value.status == sf._lib.SF_ERR_INVALID
    data = open(path, "rb").read()
    cut = str(tmp_path / "cut.bin")
    open(cut, "wb").write(data[: 28 + 4 * (1 << 10) + 100])
    with pytest.raises(sf.SfError) as e:
        h.read(ctx, cut)
    assert e.value.status == sf._lib.SF_ERR_IO
    h.close()
    g.close()
