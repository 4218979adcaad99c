"""Generates tests/golden/*.npz from the reference's own device code.

The reference (YuhangMing/semantic_icpSLAM) ships no tests or golden vectors,
so the fixtures are its own kernels' outputs: oracle/ref_shim/build_ref.py
compiles the reference's Mapping/ and Tracking/ CUDA sources for the CPU
(serial emulation of each launch) and this script runs them on seeded
synthetic inputs.  Run in the container that holds the reference sources:

    python tests/golden/make_golden.py

Fixture g1 (128x96 frames, fx = fy = 105, 10 mm voxels, 3 cm truncation,
4096 buckets, 8192 excess, 16384 heap blocks): FilterDepth, PyrDownGauss,
ComputeVMap, ComputeNMap, ResizeMap, per-pixel ICP rows, the intensity pyramid
(ImageToIntensity, PyrDownGauss(uchar), ComputeDerivativeImage), per-pixel
RGB rows (RGBStep's FindCorresp and GetRow), FuseMapColor over
five frames (labels from frame 2 on), CheckBlockVisibility, AnalyzeMapSemantics,
CreateRenderingBlocks + Raycast from two poses, MeshScene on the fused map,
and UnifyNeighborKernel alone
on a seeded label state (unify_state below).
"""
import ctypes as C
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

COLS, ROWS = 128, 96
K = (105.0, 105.0, 63.5, 47.5)
NFRAMES = 5
ENTRY = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("ptr", "<i4"), ("offset", "<i4"), ("pad", "<i4", 3)])
VOXEL_BYTES = 16


def load_ref():
    from oracle.ref_shim import build_ref
    L = C.CDLL(build_ref.build("g1"))
    vp = C.c_void_p
    L.ref_map_create.restype = vp
    L.ref_map_entries.restype = vp
    L.ref_map_visible.restype = vp
    L.ref_map_voxels.restype = vp
    L.ref_map_fuse.restype = C.c_uint
    L.ref_map_visibility.restype = C.c_uint
    L.ref_map_raytrace.restype = C.c_int
    L.ref_map_mesh.restype = C.c_uint
    for n in ("ref_map_fuse", "ref_map_visibility", "ref_map_semantics", "ref_map_raytrace", "ref_map_counters",
              "ref_map_unify", "ref_map_entries", "ref_map_visible", "ref_map_voxels", "ref_map_destroy",
              "ref_intensity", "ref_pyrdown_u8", "ref_sobel", "ref_rgb_rows", "ref_map_mesh"):
        getattr(L, n).argtypes = None
    return L


def fptr(a):
    return a.ctypes.data_as(C.c_void_p)


def pose_parts(P):
    R = np.ascontiguousarray(P[:3, :3], np.float32)
    Ri = np.ascontiguousarray(P[:3, :3].T, np.float32)
    t = np.ascontiguousarray(P[:3, 3], np.float32)
    return R, Ri, t


def mesh_records(v, n, c):
    """The sorted distinct vertex records of a mesh: 3 floats position, 3
    floats normal, 3 bytes colour and a zero byte, 28 bytes each."""
    k = v.reshape(-1, 3).shape[0]
    rec = np.zeros((k, 28), np.uint8)
    rec[:, :12] = np.ascontiguousarray(v.reshape(-1, 3)).view(np.uint8).reshape(k, 12)
    rec[:, 12:24] = np.ascontiguousarray(n.reshape(-1, 3)).view(np.uint8).reshape(k, 12)
    rec[:, 24:27] = c.reshape(-1, 3)
    return np.unique(rec, axis=0)


def block_digests(entries, voxels_ptr, n_sdf):
    vox = np.frombuffer((C.c_char * (n_sdf * 512 * VOXEL_BYTES)).from_address(voxels_ptr), dtype=np.uint8)
    sel = entries[entries["ptr"] >= 0]
    order = np.lexsort((sel["z"], sel["y"], sel["x"]))
    sel = sel[order]
    pos = np.stack([sel["x"], sel["y"], sel["z"]], 1).astype(np.int32)
    dig = np.zeros((len(sel), 20), np.uint8)
    for i, p in enumerate(sel["ptr"]):
        b = vox[p * VOXEL_BYTES:(p + 512) * VOXEL_BYTES].tobytes()
        dig[i] = np.frombuffer(hashlib.sha1(b).digest(), np.uint8)
    sample = np.stack([vox[p * VOXEL_BYTES:(p + 512) * VOXEL_BYTES] for p in sel["ptr"][:32]]) if len(sel) else \
        np.zeros((0, 512 * VOXEL_BYTES), np.uint8)
    return pos, dig, sample


def block_hash(p, nb):
    x, y, z = (np.uint32(np.int64(c) & 0xffffffff) for c in p)
    with np.errstate(over="ignore"):
        h = (x * np.uint32(73856093)) ^ (y * np.uint32(19349669)) ^ (z * np.uint32(83492791))
    return int(h) % nb


def unify_state(n_buckets, n_entries, seed=3):
    """A seeded map state for UnifyNeighbor: a 4x3x3 cluster of blocks
    around the origin (negative coordinates included), three of its blocks
    pushed to the excess list by far blocks entered first in their buckets,
    and isolated blocks; labels from a small set so the 4-slot neighbour
    tables fill and overflow; counts 0 (skipped neighbours) to 255 (the
    count_2 + 5 wrap); a fifth of the voxels at weight 0.  Returns (entries,
    voxels)."""
    rng = np.random.default_rng(seed)
    cluster = [(x, y, z) for x in range(-2, 2) for y in range(-1, 2) for z in range(-2, 1)]
    far = []
    for b in (cluster[4], cluster[17], cluster[30]):
        want, k = block_hash(b, n_buckets), 0
        while block_hash((100 + k, 50, 20), n_buckets) != want:
            k += 1
        far.append((100 + k, 50, 20))
    blocks = far + cluster + [(40, -7, 3), (-33, 12, -9), (5, 5, 60), (-1, -60, 2)]
    ent = np.zeros(n_entries, ENTRY)
    ent["ptr"] = -1
    next_off = 1
    for k, p in enumerate(blocks):
        b = block_hash(p, n_buckets)
        if ent["ptr"][b] == -1:
            ent["x"][b], ent["y"][b], ent["z"][b], ent["ptr"][b] = p[0], p[1], p[2], k * 512
            continue
        e = b
        while ent["offset"][e] > 0:
            e = n_buckets + ent["offset"][e] - 1
        slot = n_buckets + next_off - 1
        ent["x"][slot], ent["y"][slot], ent["z"][slot], ent["ptr"][slot] = p[0], p[1], p[2], k * 512
        ent["offset"][e] = next_off
        next_off += 1
    nvox = len(blocks) * 512
    vox = np.zeros((nvox, VOXEL_BYTES), np.uint8)
    weight = rng.integers(1, 256, nvox)
    weight[rng.random(nvox) < 0.2] = 0
    labels = np.array([0, 3, 7, 9, 12, 40], np.uint8)
    count = rng.integers(0, 12, nvox)
    hi = rng.random(nvox) < 0.1
    count[hi] = rng.integers(240, 256, int(hi.sum()))
    count_2 = rng.integers(0, 12, nvox)
    hi2 = rng.random(nvox) < 0.15
    count_2[hi2] = rng.integers(248, 256, int(hi2.sum()))
    vox[:, 4] = weight
    vox[:, 8] = labels[rng.integers(0, len(labels), nvox)]
    vox[:, 9] = count
    vox[:, 10] = labels[rng.integers(0, len(labels), nvox)]
    vox[:, 11] = count_2
    same = rng.random(nvox) < 0.2  # label_2 == label on a fifth of the voxels
    vox[same, 10] = vox[same, 8]
    return ent, vox


UNIFY_NVIS = (2048, 4096 + 8192)  # half the bucket slots; every slot


def main():
    from synth import Synth
    L = load_ref()
    consts = np.zeros(8, np.float64)
    L.ref_constants(fptr(consts))
    n_sdf = int(consts[4])
    n_entries = int(consts[2] + consts[3])
    syn = Synth(COLS, ROWS, K, scene=0, trajectory=1, seed=7, dropout=0.02, label_flip=0.05, n_objects=10)
    frames = [syn.frame(i) for i in range(NFRAMES + 1)]
    out = {"K": np.array(K, np.float32), "consts": consts}
    for i, (d, rgb, mask, P) in enumerate(frames):
        out["depth%d" % i] = d
        out["rgb%d" % i] = rgb
        out["mask%d" % i] = mask
        out["pose%d" % i] = P

    # pyramid of every frame through the reference launchers
    pyr = []
    for i, (d, _, _, _) in enumerate(frames):
        raw = np.zeros((ROWS, COLS), np.float32)
        filt = np.zeros((ROWS, COLS), np.float32)
        L.ref_filter_depth(fptr(d), COLS, ROWS, C.c_float(1000.0), C.c_float(3.0), fptr(raw), fptr(filt))
        depths, vms, nms = [filt], [], []
        for l in range(3):
            c, r = COLS >> l, ROWS >> l
            if l > 0:
                dd = np.zeros((r, c), np.float32)
                L.ref_pyrdown(fptr(depths[-1]), c * 2, r * 2, fptr(dd))
                depths.append(dd)
            div = float(1 << l)
            vm = np.zeros((r, c, 4), np.float32)
            nm = np.zeros((r, c, 4), np.float32)
            L.ref_vmap(fptr(depths[l]), c, r, *[C.c_float(k / div) for k in K], C.c_float(3.0), fptr(vm))
            L.ref_nmap(fptr(vm), c, r, fptr(nm))
            vms.append(vm)
            nms.append(nm)
        pyr.append((raw, depths, vms, nms))
        if i < 2:
            out["raw%d" % i] = raw
            out["filt%d" % i] = filt
            for l in range(3):
                out["f%d_depth%d" % (i, l)] = depths[l]
                out["f%d_vmap%d" % (i, l)] = vms[l]
                out["f%d_nmap%d" % (i, l)] = nms[l]

    # ResizeMap on seeded maps with holes
    rng = np.random.default_rng(11)
    v = rng.normal(size=(ROWS, COLS, 4)).astype(np.float32)
    v[..., 3] = 1
    n = rng.normal(size=(ROWS, COLS, 4)).astype(np.float32)
    n[..., :3] /= np.linalg.norm(n[..., :3], axis=-1, keepdims=True)
    n[..., 3] = 1
    v[rng.random((ROWS, COLS)) < 0.03] = np.nan
    n[rng.random((ROWS, COLS)) < 0.03] = np.nan
    vd = np.zeros((ROWS // 2, COLS // 2, 4), np.float32)
    nd = np.zeros((ROWS // 2, COLS // 2, 4), np.float32)
    L.ref_resize(fptr(v), fptr(n), COLS, ROWS, fptr(vd), fptr(nd))
    out.update(resize_vsrc=v, resize_nsrc=n, resize_vdst=vd, resize_ndst=nd)

    # ICP rows: frame 1 against frame 0, current pose halfway
    P0, P1 = frames[0][3], frames[1][3]
    Pc = P0.copy()
    Pc[:3, 3] = 0.5 * (P0[:3, 3] + P1[:3, 3])
    out["icp_pose_curr"] = Pc
    Rc, _, tc = pose_parts(Pc)
    Rl, RlI, tl = pose_parts(P0)
    for l in range(3):
        c, r = COLS >> l, ROWS >> l
        rows29 = np.zeros((r * c, 29), np.float32)
        div = float(1 << l)
        L.ref_icp_rows(fptr(pyr[1][2][l]), fptr(pyr[0][2][l]), fptr(pyr[1][3][l]), fptr(pyr[0][3][l]), c, r,
                       fptr(Rc), fptr(tc), fptr(Rl), fptr(RlI), fptr(tl), *[C.c_float(k / div) for k in K],
                       fptr(rows29))
        out["icp_sums%d" % l] = rows29.astype(np.float64).sum(0)
        out["icp_rows_sha1_%d" % l] = np.frombuffer(hashlib.sha1(rows29.tobytes()).digest(), np.uint8)
        if l == 2:
            out["icp_rows2"] = rows29

    # intensity pyramid and derivative images of frames 0 and 1, then the
    # per-pixel RGB rows (FindCorresp + GetRow) of frame 1 against frame 0 at
    # the same halfway pose as the ICP rows
    ipyr = []
    for i in range(2):
        rgb = frames[i][1]
        imgs = [np.zeros((ROWS, COLS), np.uint8)]
        L.ref_intensity(fptr(rgb), COLS, ROWS, fptr(imgs[0]))
        for l in range(1, 3):
            c, r = COLS >> l, ROWS >> l
            imgs.append(np.zeros((r, c), np.uint8))
            L.ref_pyrdown_u8(fptr(imgs[l - 1]), c * 2, r * 2, fptr(imgs[l]))
        ders = []
        for l in range(3):
            c, r = COLS >> l, ROWS >> l
            dx = np.zeros((r, c), np.int16)
            dy = np.zeros((r, c), np.int16)
            L.ref_sobel(fptr(imgs[l]), c, r, fptr(dx), fptr(dy))
            ders.append((dx, dy))
            out["f%d_int%d" % (i, l)] = imgs[l]
            out["f%d_dx%d" % (i, l)] = dx
            out["f%d_dy%d" % (i, l)] = dy
        ipyr.append((imgs, ders))
    Rc, RcI, tc = pose_parts(Pc)
    for l in range(3):
        c, r = COLS >> l, ROWS >> l
        rows29 = np.zeros((r * c, 29), np.float32)
        res2 = np.zeros(2, np.int32)
        sigma = np.zeros(1, np.float32)
        div = float(1 << l)
        L.ref_rgb_rows(fptr(ipyr[1][0][l]), fptr(ipyr[0][0][l]), fptr(pyr[1][2][l]), fptr(pyr[0][2][l]),
                       fptr(ipyr[1][1][l][0]), fptr(ipyr[1][1][l][1]), c, r, fptr(Rc), fptr(RcI), fptr(Rl),
                       fptr(RlI), fptr(tc), fptr(tl), *[C.c_float(k / div) for k in K], fptr(res2), fptr(sigma),
                       fptr(rows29))
        out["rgb_res%d" % l] = res2
        out["rgb_sigma%d" % l] = sigma
        out["rgb_sums%d" % l] = rows29.astype(np.float64).sum(0)
        out["rgb_rows_sha1_%d" % l] = np.frombuffer(hashlib.sha1(rows29.tobytes()).digest(), np.uint8)
        print("rgb level %d: %d correspondences, sigma %.3f" % (l, res2[0], sigma[0]))

    # the map: FuseMapColor at ground-truth poses, labels from frame 2 on
    m = L.ref_map_create()
    counters = []
    for i in range(NFRAMES):
        d, rgb, mask, P = frames[i]
        raw, _, _, nms = pyr[i]
        R, Ri, t = pose_parts(P)
        ndet = 10 if i >= 2 else 0
        nvis = L.ref_map_fuse(C.c_void_p(m), fptr(raw), fptr(rgb), fptr(nms[0]), fptr(mask), C.c_int(ndet),
                              C.c_int(COLS), C.c_int(ROWS), fptr(R), fptr(Ri), fptr(t),
                              *[C.c_float(k) for k in K])
        cnt = np.zeros(4, np.int32)
        L.ref_map_counters(C.c_void_p(m), fptr(cnt))
        counters.append(cnt)
        vis = np.frombuffer((C.c_char * (n_entries * 32)).from_address(L.ref_map_visible(C.c_void_p(m))), ENTRY)
        vis = vis[:nvis]
        out["visible%d" % i] = np.sort(np.stack([vis["x"], vis["y"], vis["z"]], 1).view(
            [("x", "<i4"), ("y", "<i4"), ("z", "<i4")]).ravel())
    out["counters"] = np.stack(counters)
    ent = np.frombuffer((C.c_char * (n_entries * 32)).from_address(L.ref_map_entries(C.c_void_p(m))), ENTRY).copy()
    pos, dig, sample = block_digests(ent, L.ref_map_voxels(C.c_void_p(m)), n_sdf)
    out.update(map_pos=pos, map_sha1=dig, map_sample=sample)

    # MeshScene on that map (Mapping::CreateModel): the triangle count and a
    # digest of the set of distinct vertex records (position, normal, colour)
    max_tri = 1000000
    v = np.zeros((max_tri, 3, 3), np.float32)
    nrm = np.zeros((max_tri, 3, 3), np.float32)
    col = np.zeros((max_tri, 3, 3), np.uint8)
    ntri = L.ref_map_mesh(C.c_void_p(m), C.c_uint(max_tri), fptr(v), fptr(nrm), fptr(col))
    recs = mesh_records(v[:ntri], nrm[:ntri], col[:ntri])
    out.update(mesh_ntri=np.int64(ntri), mesh_nrec=np.int64(len(recs)),
               mesh_rec_sha1=np.frombuffer(hashlib.sha1(recs.tobytes()).digest(), np.uint8))
    print("mesh: %d triangles, %d distinct vertex records" % (ntri, len(recs)))

    # raytrace from the last fused pose and the next pose (Mapping::RayTrace)
    for k, fi in enumerate((NFRAMES - 1, NFRAMES)):
        P = frames[fi][3]
        R, Ri, t = pose_parts(P)
        nvis = L.ref_map_visibility(C.c_void_p(m), fptr(R), fptr(Ri), fptr(t), C.c_int(COLS), C.c_int(ROWS),
                                    *[C.c_float(x) for x in K])
        zmin = np.zeros((60, 80), np.float32)
        zmax = np.zeros((60, 80), np.float32)
        nblk = C.c_uint(0)
        vm = pyr[fi][2][0].copy()
        nm = pyr[fi][3][0].copy()
        ok = L.ref_map_raytrace(C.c_void_p(m), C.c_int(COLS), C.c_int(ROWS), fptr(R), fptr(Ri), fptr(t),
                                *[C.c_float(x) for x in K], fptr(zmin), fptr(zmax), C.byref(nblk), fptr(vm),
                                fptr(nm))
        out.update({"ray%d_nvis" % k: np.int64(nvis), "ray%d_ok" % k: np.int64(ok), "ray%d_nblocks" % k:
                    np.int64(nblk.value), "ray%d_zmin" % k: zmin, "ray%d_zmax" % k: zmax,
                    "ray%d_vmap" % k: vm, "ray%d_nmap" % k: nm})

    # AnalyzeMapSemantics from the last pose with that frame's mask
    d, rgb, mask, P = frames[NFRAMES - 1]
    R, Ri, t = pose_parts(P)
    L.ref_map_semantics(C.c_void_p(m), fptr(pyr[NFRAMES - 1][0]), fptr(rgb), fptr(pyr[NFRAMES - 1][3][0]),
                        fptr(mask), C.c_int(10), C.c_int(COLS), C.c_int(ROWS), fptr(R), fptr(Ri), fptr(t),
                        *[C.c_float(x) for x in K])
    ent = np.frombuffer((C.c_char * (n_entries * 32)).from_address(L.ref_map_entries(C.c_void_p(m))), ENTRY).copy()
    pos2, dig2, _ = block_digests(ent, L.ref_map_voxels(C.c_void_p(m)), n_sdf)
    out.update(sem_pos=pos2, sem_sha1=dig2)
    L.ref_map_destroy(C.c_void_p(m))

    # UnifyNeighborKernel alone on a seeded state, per visible count
    ent, vox = unify_state(int(consts[2]), n_entries)
    out.update(uni_entries=ent.view(np.int32).reshape(n_entries, 8), uni_vox=vox,
               uni_nvis=np.array(UNIFY_NVIS, np.int64))
    for k, nvis in enumerate(UNIFY_NVIS):
        m = L.ref_map_create()
        C.memmove(L.ref_map_entries(C.c_void_p(m)), ent.ctypes.data, ent.nbytes)
        C.memmove(L.ref_map_voxels(C.c_void_p(m)), vox.ctypes.data, vox.nbytes)
        L.ref_map_unify(C.c_void_p(m), C.c_uint(nvis))
        after = np.frombuffer((C.c_char * vox.nbytes).from_address(L.ref_map_voxels(C.c_void_p(m))),
                              np.uint8).reshape(vox.shape).copy()
        L.ref_map_destroy(C.c_void_p(m))
        assert np.array_equal(np.delete(after, [8, 9, 10, 11], 1), np.delete(vox, [8, 9, 10, 11], 1))
        out["uni_out%d" % k] = after[:, 8:12].copy()
        print("unify nvis=%d: %d of %d voxels changed" % (nvis, int((after[:, 8:12] != vox[:, 8:12]).any(1).sum()),
                                                          len(vox)))

    path = os.path.join(HERE, "g1.npz")
    np.savez_compressed(path, **out)
    print("wrote %s (%.1f KB)" % (path, os.path.getsize(path) / 1024))


if __name__ == "__main__":
    main()
