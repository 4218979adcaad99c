"""The drop-in path for the reference's own map arrays: a caller allocates
them as Mapping::Create does (Mapping/Mapping.cc:11-51: heap, heapCounter,
hashCounter, bucketMutex, sdfBlock, noVisibleEntries, hashEntries,
visibleEntries, sized by DeviceMap's constants), hands them to sf_map_wrap,
resets them with sf_ResetMap (Mapping::Reset), and runs FuseMapColor and
the raycast (CheckBlockVisibility, CreateRenderingBlocks, Raycast) on them.
Every array, the rendering blocks and the ray traced maps must equal the
same calls on a map that sf_map_create allocated, bit for bit, and the
wrapped map must leave the caller's arrays where they are.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import C1, MAP_C1, cuda, empty, host, map_to_host, positions, sequence, voxels_by_pos
from tests.test_gpu_fusion import _frame_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(built):
    import torch
    import semantic_icpslam_gb300 as sf
    assert torch.cuda.is_available()
    ctx = sf.Context()
    yield sf, ctx
    ctx.close()


def _mapping_create(sf, mc):
    """The reference Mapping's device arrays, owned by the caller."""
    import torch
    nb, ne, ns = mc["num_buckets"], mc["num_excess"], mc["num_sdf_blocks"]
    i32 = lambda n: torch.zeros(n, dtype=torch.int32, device="cuda")
    arrays = dict(heap=i32(ns), entry_ptr=i32(1), heap_counter=i32(1), bucket_mutex=i32(nb),
                  voxels=torch.zeros(ns * 512 * 16, dtype=torch.uint8, device="cuda"), no_visible=i32(1),
                  entries=torch.zeros((nb + ne) * 32, dtype=torch.uint8, device="cuda"),
                  visible=torch.zeros((nb + ne) * 32, dtype=torch.uint8, device="cuda"))
    a = sf._lib.DeviceMap(arrays["heap"].data_ptr(), arrays["entry_ptr"].data_ptr(),
                          arrays["heap_counter"].data_ptr(), arrays["bucket_mutex"].data_ptr(),
                          arrays["voxels"].data_ptr(), arrays["no_visible"].data_ptr(),
                          arrays["entries"].data_ptr(), arrays["visible"].data_ptr())
    cfg = sf._lib.MapConfig(mc["voxel_size"], mc["trunc_dist"], 0.1, 3.0, nb, ne, ns, 260000)
    h = C.c_void_p()
    sf.call("sf_map_wrap", C.byref(cfg), C.byref(a), C.byref(h))
    return sf.Map(**mc, _handle=h), arrays, h


def _render(sf, ctx, m, P, K, cols, rows):
    """CheckBlockVisibility + CreateRenderingBlocks + Raycast (Mapping::UpdateVisibility,
    Mapping::RayTrace)."""
    import torch
    R, RI, t = sf.pose_to_gpu(P)
    nv = C.c_uint32()
    sf.call("sf_CheckBlockVisibility", ctx.h, m.h, R, RI, t, cols, rows, *K, 3.0, 0.1, C.byref(nv))
    zc, zr = (cols + 7) // 8, (rows + 7) // 8
    zmin, zmax = empty((zr, zc), torch.float32), empty((zr, zc), torch.float32)
    blocks = torch.zeros((260000, 4), dtype=torch.int32, device="cuda")
    nrb = torch.zeros(1, dtype=torch.int32, device="cuda")
    ok = C.c_int()
    sf.call("sf_CreateRenderingBlocks", ctx.h, m.h, sf.image(zmin), sf.image(zmax), 3.0, 0.1, blocks.data_ptr(),
            nrb.data_ptr(), RI, t, nv.value, *K, C.byref(ok))
    vm, nm = empty((rows, cols, 4), torch.float32), empty((rows, cols, 4), torch.float32)
    if ok.value:
        sf.call("sf_Raycast", ctx.h, m.h, sf.image(vm), sf.image(nm), sf.image(zmin), sf.image(zmax), R, RI, t,
                float(np.float32(1.0 / np.float32(K[0]))), float(np.float32(1.0 / np.float32(K[1]))), K[2], K[3])
    ctx.sync()
    return nv.value, ok.value, host(zmin), host(zmax), host(vm), host(nm)


def test_wrapped_reference_arrays_equal_created_map(lib):
    sf, ctx = lib
    K = C1["K"]
    cols, rows = C1["cols"], C1["rows"]
    seq = sequence(cols, rows, K, 4, trajectory=1, dropout=0.02)
    made = sf.Map(**MAP_C1)
    wrapped, arrays, h = _mapping_create(sf, MAP_C1)
    sf.call("sf_ResetMap", ctx.h, wrapped.h)  # Mapping::Reset
    ptrs = {k: v.data_ptr() for k, v in arrays.items()}
    for d, rgb, mask, P in seq:
        f = _frame_inputs(sf, ctx, d, rgb, mask, K)
        R, RI, t = sf.pose_to_gpu(P)
        counts = []
        for m in (made, wrapped):
            nvis = C.c_uint32()
            sf.call("sf_FuseMapColor", ctx.h, m.h, sf.image(f["raw"]), sf.image(f["rgb"]), sf.image(f["nmap"]),
                    sf.image(f["mask"]), 0, R, RI, t, *K, 3.0, 0.1, C.byref(nvis))
            counts.append(nvis.value)
        assert counts[0] == counts[1] and counts[0] > 0
        r0 = _render(sf, ctx, made, P, K, cols, rows)
        r1 = _render(sf, ctx, wrapped, P, K, cols, rows)
        assert r0[:2] == r1[:2] and r0[1] == 1
        for a, b in zip(r0[2:], r1[2:]):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    # the map: the same blocks with the same voxels at every position, the
    # same counters (which heap block a new block takes follows the order
    # the insert pass pops the heap in, which varies between runs, in the
    # reference as here)
    ea, va, sa = map_to_host(ctx, made)
    eb, vb, sb = map_to_host(ctx, wrapped)
    assert positions(ea[ea["ptr"] >= 0]) == positions(eb[eb["ptr"] >= 0])
    ka, xa = voxels_by_pos(ea, va)
    kb, xb = voxels_by_pos(eb, vb)
    assert ka == kb and np.array_equal(xa.view(np.uint8), xb.view(np.uint8))
    assert positions(sa[:counts[0]]) == positions(sb[:counts[1]])
    assert made.counters(ctx) == wrapped.counters(ctx)
    got = wrapped.arrays()
    assert (got.heap_mem, got.voxel_blocks, got.hash_entries) == (ptrs["heap"], ptrs["voxels"], ptrs["entries"])
    # the caller's arrays hold the map (the library wrote into them)
    assert np.array_equal(arrays["entries"].cpu().numpy(), eb.view(np.uint8).reshape(-1))
    wrapped.close()
    sf.call("sf_map_destroy", h)
    made.close()
    del arrays
