"""ctypes front end of the oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product never does.  Arrays are numpy, C-contiguous.
"""
import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

_lib = None
_lock = threading.Lock()

F32P = C.POINTER(C.c_float)
F64P = C.POINTER(C.c_double)
U16P = C.POINTER(C.c_uint16)
U8P = C.POINTER(C.c_uint8)
I32P = C.POINTER(C.c_int)
I16P = C.POINTER(C.c_int16)

ENTRY_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("ptr", "<i4"),
                        ("offset", "<i4"), ("pad", "<i4", 3)])
VOXEL_DTYPE = np.dtype([("sdf", "<f4"), ("weight", "u1"), ("color", "u1", 3),
                        ("label", "u1"), ("count", "u1"), ("label_2", "u1"),
                        ("count_2", "u1"), ("color_2", "u1", 3), ("obj_idx", "u1")])
RBLOCK_DTYPE = np.dtype([("ulx", "<i2"), ("uly", "<i2"), ("lrx", "<i2"), ("lry", "<i2"),
                         ("zmin", "<f4"), ("zmax", "<f4")])
RELOC_DTYPE = np.dtype([("valid", "<u4"), ("inliers", "<u4"), ("sum_abs_sdf", "<f4"), ("mean_abs_sdf", "<f4")])
assert ENTRY_DTYPE.itemsize == 32 and VOXEL_DTYPE.itemsize == 16 and RBLOCK_DTYPE.itemsize == 16


class Config(C.Structure):
    _fields_ = [("voxel_size", C.c_float), ("trunc_dist", C.c_float),
                ("depth_min", C.c_float), ("depth_max", C.c_float),
                ("num_buckets", C.c_uint32), ("num_excess", C.c_uint32),
                ("num_sdf_blocks", C.c_uint32), ("max_rendering_blocks", C.c_uint32)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = C.CDLL(path)
            vp = C.c_void_p
            sig = {
                "sfo_filter_depth": (None, [U16P, C.c_int, C.c_int, C.c_float, C.c_float, F32P, F32P]),
                "sfo_pyrdown": (None, [F32P, C.c_int, C.c_int, F32P, C.c_int, C.c_int]),
                "sfo_vmap": (None, [F32P, C.c_int, C.c_int] + [C.c_float] * 5 + [F32P]),
                "sfo_nmap": (None, [F32P, C.c_int, C.c_int, F32P]),
                "sfo_resize": (None, [F32P, F32P, C.c_int, C.c_int, F32P, F32P, C.c_int, C.c_int]),
                "sfo_icp_sums": (None, [F32P] * 4 + [C.c_int, C.c_int] + [F32P] * 5 + [C.c_float] * 4 + [C.c_int, F64P]),
                "sfo_icp_rows": (None, [F32P] * 4 + [C.c_int, C.c_int] + [F32P] * 5 + [C.c_float] * 4 + [F32P]),
                "sfo_create_matrix": (None, [F64P, F64P, F64P]),
                "sfo_ldlt_solve6": (None, [F64P, F64P, F64P]),
                "sfo_se3_exp": (None, [F64P, F64P]),
                "sfo_compute_se3": (C.c_int, [C.c_int, I32P, I32P, vp, vp, vp, vp, F32P, I32P, I32P,
                                              C.c_float, F64P, F64P, C.c_int, F64P]),
                "sfo_compute_se3_ex": (C.c_int, [C.c_int, I32P, I32P] + [vp] * 8 + [F32P, I32P, I32P,
                                                 C.c_float, F64P, F64P, C.c_int, F64P]),
                "sfo_intensity": (None, [U8P, C.c_int, C.c_int, U8P]),
                "sfo_pyrdown_u8": (None, [U8P, C.c_int, C.c_int, U8P, C.c_int, C.c_int]),
                "sfo_sobel": (None, [U8P, C.c_int, C.c_int, I16P, I16P]),
                "sfo_rgb_step": (None, [U8P, U8P, F32P, F32P, I16P, I16P, C.c_int, C.c_int, F64P, F64P]
                                 + [C.c_float] * 4 + [C.c_int, F64P, I32P, F32P, F32P]),
                "sfo_map_create": (vp, [C.POINTER(Config)]),
                "sfo_map_destroy": (None, [vp]),
                "sfo_map_reset": (None, [vp]),
                "sfo_map_entries": (vp, [vp]),
                "sfo_map_voxels": (vp, [vp]),
                "sfo_map_visible": (vp, [vp]),
                "sfo_map_heap": (vp, [vp]),
                "sfo_map_counters": (None, [vp, I32P]),
                "sfo_alloc": (None, [vp, F32P, C.c_int, C.c_int, F32P, F32P] + [C.c_float] * 4),
                "sfo_visibility": (C.c_uint, [vp, F32P, F32P, F32P, C.c_int, C.c_int] + [C.c_float] * 6),
                "sfo_integrate": (None, [vp, F32P, U8P, C.c_int, C.c_int, F32P, F32P] + [C.c_float] * 6),
                "sfo_validate_pose_batch": (C.c_int, [vp, C.c_int, C.c_int, C.c_int] + [vp] * 4
                                            + [F32P, F64P, C.c_int, I32P, I32P, C.c_float, C.c_uint, F64P]),
                "sfo_system_set_reloc": (None, [vp, F64P, C.c_int]),
                "sfo_integrate_f64": (None, [vp, F32P, C.c_int, C.c_int, F32P, F32P, F64P] + [C.c_float] * 6),
                "sfo_tsdf_f64_error": (None, [vp, F64P]),
                "sfo_semantics": (None, [vp, F32P, U8P, F32P, U8P, C.c_int, C.c_int, C.c_int, F32P, F32P] + [C.c_float] * 6),
                "sfo_unify_neighbor": (None, [vp]),
                "sfo_map_set_no_visible": (None, [vp, C.c_uint]),
                "sfo_fuse": (C.c_uint, [vp, F32P, U8P, F32P, U8P, C.c_int, C.c_int, C.c_int, F32P, F32P, F32P] + [C.c_float] * 4
                             + [C.c_int]),
                "sfo_zrange": (C.c_int, [vp, F32P, F32P, C.c_int, C.c_int, C.c_float, C.c_float, F32P, F32P]
                               + [C.c_float] * 4 + [vp, C.c_int, C.POINTER(C.c_uint)]),
                "sfo_reloc_score": (None, [vp, F32P, C.c_int, C.c_int, C.c_int, F32P, C.c_int, C.c_float, vp]),
                "sfo_raycast_smooth_f64": (C.c_double, [vp, F32P, F32P, C.c_int, C.c_int, F32P, F32P, C.c_int,
                                                        C.c_int, F64P, C.c_float, C.c_float, C.c_float, C.c_float,
                                                        F64P, C.c_longlong, C.c_double]),
                "sfo_raycast": (None, [vp, F32P, F32P, C.c_int, C.c_int, F32P, F32P, C.c_int, C.c_int,
                                       F32P, F32P, F32P] + [C.c_float] * 4),
                "sfo_system_create": (vp, [C.POINTER(Config), C.c_int, C.c_int, C.c_int, F32P, C.c_float,
                                           C.c_float, I32P, I32P, C.c_float, F64P]),
                "sfo_system_destroy": (None, [vp]),
                "sfo_system_grab": (C.c_int, [vp, U16P, U8P, U8P, C.c_int, F64P, F64P]),
                "sfo_system_set_rgb": (None, [vp, C.c_int]),
                "sfo_system_set_mapping": (None, [vp, C.c_int]),
                "sfo_mc_tables": (None, [I32P, I32P, I32P]),
                "sfo_mesh": (C.c_uint, [vp, C.c_uint, F32P, F32P, U8P]),
                "sfo_system_map": (vp, [vp]),
                "sfo_system_vmap": (vp, [vp, C.c_int]),
                "sfo_system_nmap": (vp, [vp, C.c_int]),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def filter_depth(depth_u16, depth_scale, cutoff):
    d = np.ascontiguousarray(depth_u16, dtype=np.uint16)
    rows, cols = d.shape
    raw = np.empty((rows, cols), np.float32)
    filt = np.empty((rows, cols), np.float32)
    lib().sfo_filter_depth(_p(d, U16P), cols, rows, depth_scale, cutoff, _p(raw, F32P), _p(filt, F32P))
    return raw, filt


def pyrdown(src):
    src = _f32(src)
    sr, sc = src.shape
    dst = np.empty((sr // 2, sc // 2), np.float32)
    lib().sfo_pyrdown(_p(src, F32P), sc, sr, _p(dst, F32P), sc // 2, sr // 2)
    return dst


def vmap(depth, fx, fy, cx, cy, cutoff):
    depth = _f32(depth)
    rows, cols = depth.shape
    out = np.empty((rows, cols, 4), np.float32)
    lib().sfo_vmap(_p(depth, F32P), cols, rows, fx, fy, cx, cy, cutoff, _p(out, F32P))
    return out


def nmap(vm):
    vm = _f32(vm)
    rows, cols = vm.shape[:2]
    out = np.empty((rows, cols, 4), np.float32)
    lib().sfo_nmap(_p(vm, F32P), cols, rows, _p(out, F32P))
    return out


def resize(vsrc, nsrc):
    vsrc, nsrc = _f32(vsrc), _f32(nsrc)
    sr, sc = vsrc.shape[:2]
    vd = np.empty((sr // 2, sc // 2, 4), np.float32)
    nd = np.empty((sr // 2, sc // 2, 4), np.float32)
    lib().sfo_resize(_p(vsrc, F32P), _p(nsrc, F32P), sc, sr, _p(vd, F32P), _p(nd, F32P), sc // 2, sr // 2)
    return vd, nd


def pose_to_gpu(P):
    """Frame::GpuRotation / GpuInvRotation / GpuTranslation (Frame.cc:626-645)."""
    P = np.asarray(P, np.float64)
    R = P[:3, :3].astype(np.float32)
    Rinv = P[:3, :3].T.astype(np.float32)
    t = P[:3, 3].astype(np.float32)
    return np.ascontiguousarray(R), np.ascontiguousarray(Rinv), np.ascontiguousarray(t)


def icp_sums(vcurr, vlast, ncurr, nlast, Pcurr, Plast, K, fp64=False):
    vcurr, vlast, ncurr, nlast = map(_f32, (vcurr, vlast, ncurr, nlast))
    rows, cols = vcurr.shape[:2]
    Rc, _, tc = pose_to_gpu(Pcurr)
    Rl, RlI, tl = pose_to_gpu(Plast)
    out = np.zeros(29, np.float64)
    lib().sfo_icp_sums(_p(vcurr, F32P), _p(vlast, F32P), _p(ncurr, F32P), _p(nlast, F32P), cols, rows,
                       _p(Rc, F32P), _p(tc, F32P), _p(Rl, F32P), _p(RlI, F32P), _p(tl, F32P),
                       *map(float, K), int(fp64), _p(out, F64P))
    return out


def icp_rows(vcurr, vlast, ncurr, nlast, Pcurr, Plast, K):
    vcurr, vlast, ncurr, nlast = map(_f32, (vcurr, vlast, ncurr, nlast))
    rows, cols = vcurr.shape[:2]
    Rc, _, tc = pose_to_gpu(Pcurr)
    Rl, RlI, tl = pose_to_gpu(Plast)
    out = np.zeros((rows * cols, 29), np.float32)
    lib().sfo_icp_rows(_p(vcurr, F32P), _p(vlast, F32P), _p(ncurr, F32P), _p(nlast, F32P), cols, rows,
                       _p(Rc, F32P), _p(tc, F32P), _p(Rl, F32P), _p(RlI, F32P), _p(tl, F32P),
                       *map(float, K), _p(out, F32P))
    return out


def create_matrix(s29):
    s = np.ascontiguousarray(s29, np.float64)
    A = np.zeros(36, np.float64)
    b = np.zeros(6, np.float64)
    lib().sfo_create_matrix(_p(s, F64P), _p(A, F64P), _p(b, F64P))
    return A.reshape(6, 6), b


def ldlt_solve6(A, b):
    A = np.ascontiguousarray(A, np.float64).reshape(36)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(6, np.float64)
    lib().sfo_ldlt_solve6(_p(A, F64P), _p(b, F64P), _p(x, F64P))
    return x


def se3_exp(xi):
    xi = np.ascontiguousarray(xi, np.float64)
    T = np.zeros(16, np.float64)
    lib().sfo_se3_exp(_p(xi, F64P), _p(T, F64P))
    return T.reshape(4, 4)


def compute_se3(vnext, nnext, vlast, nlast, K, iters, min_count, thresh, last_pose, next_pose,
                fp64=False, rgb=None):
    """Tracker::ComputeSE3.  rgb = (inext, ilast, dIdx, dIdy) per level adds
    the photometric term (icpOnly = false); stats then has six entries."""
    L = len(vnext)
    keep = [_f32(a) for a in list(vnext) + list(nnext) + list(vlast) + list(nlast)]
    if rgb is not None:
        inext, ilast, dx, dy = rgb
        keep += [np.ascontiguousarray(a, np.uint8) for a in list(inext) + list(ilast)]
        keep += [np.ascontiguousarray(a, np.int16) for a in list(dx) + list(dy)]
    ptrs = [a.ctypes.data for a in keep]
    arr = lambda k: (C.c_void_p * L)(*ptrs[k * L:(k + 1) * L]) if k * L < len(ptrs) else None
    cols = (C.c_int * L)(*[a.shape[1] for a in keep[:L]])
    rows = (C.c_int * L)(*[a.shape[0] for a in keep[:L]])
    Kf = np.asarray(K, np.float32)
    it = np.asarray(iters, np.int32)
    mc = np.asarray(min_count, np.int32)
    lp = np.ascontiguousarray(last_pose, np.float64)
    npose = np.ascontiguousarray(next_pose, np.float64).copy()
    stats = np.zeros(6, np.float64)
    ok = lib().sfo_compute_se3_ex(L, cols, rows, arr(0), arr(1), arr(2), arr(3), arr(4), arr(5), arr(6), arr(7),
                                  _p(Kf, F32P), _p(it, I32P), _p(mc, I32P), thresh, _p(lp, F64P),
                                  _p(npose, F64P), int(fp64), _p(stats, F64P))
    return bool(ok), npose, (stats if rgb is not None else stats[:4])


def validate_pose_batch(m, vnext, nnext, vlast, nlast, K, poses, iters=(3, 3, 2), min_count=(2000, 1000, 100),
                        thresh=1e-3, min_visible=512):
    """Tracker::ValidatePose over n candidates (sfo_validate_pose_batch).
    Returns (n x 24 array of per-candidate results, chosen index or -1)."""
    L = len(vnext)
    keep = [_f32(a) for a in list(vnext) + list(nnext) + list(vlast) + list(nlast)]
    arr = lambda k: (C.c_void_p * L)(*[a.ctypes.data for a in keep[k * L:(k + 1) * L]])
    rows, cols = keep[0].shape[:2]
    P = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 16))
    n = P.shape[0]
    Kf = np.asarray(K, np.float32)
    it = np.asarray([iters[l] if l < len(iters) else 0 for l in range(L)], np.int32)
    mc = np.asarray([min_count[l] if l < len(min_count) else 0 for l in range(L)], np.int32)
    out = np.zeros((n, 24), np.float64)
    chosen = lib().sfo_validate_pose_batch(m.h, L, cols, rows, arr(0), arr(1), arr(2), arr(3), _p(Kf, F32P),
                                           _p(P, F64P), n, _p(it, I32P), _p(mc, I32P), float(thresh),
                                           int(min_visible), _p(out, F64P))
    return out, int(chosen)


def mc_tables():
    """(triangle table [256,16], vertex counts [256], edge masks [256])."""
    t = np.zeros((256, 16), np.int32)
    nv = np.zeros(256, np.int32)
    ed = np.zeros(256, np.int32)
    lib().sfo_mc_tables(_p(t, I32P), _p(nv, I32P), _p(ed, I32P))
    return t, nv, ed


def intensity(rgb):
    """ImageToIntensity: uchar3 rows x cols x 3 -> uint8."""
    rgb = np.ascontiguousarray(rgb, np.uint8)
    rows, cols = rgb.shape[:2]
    out = np.empty((rows, cols), np.uint8)
    lib().sfo_intensity(_p(rgb, U8P), cols, rows, _p(out, U8P))
    return out


def pyrdown_u8(src):
    """PyrDownGauss(unsigned char)."""
    src = np.ascontiguousarray(src, np.uint8)
    sr, sc = src.shape
    dst = np.empty((sr // 2, sc // 2), np.uint8)
    lib().sfo_pyrdown_u8(_p(src, U8P), sc, sr, _p(dst, U8P), sc // 2, sr // 2)
    return dst


def sobel(img):
    """ComputeDerivativeImage: (dIdx, dIdy) int16."""
    img = np.ascontiguousarray(img, np.uint8)
    rows, cols = img.shape
    dx = np.empty((rows, cols), np.int16)
    dy = np.empty((rows, cols), np.int16)
    lib().sfo_sobel(_p(img, U8P), cols, rows, _p(dx, I16P), _p(dy, I16P))
    return dx, dy


def rgb_step(inext, ilast, vnext, vlast, dIdx, dIdy, Pcurr, Plast, K, fp64=False, rows=False):
    """RGBStep at the 4x4 poses: (sums29, (count, sum diff^2), sigma[, per-pixel rows])."""
    inext, ilast = (np.ascontiguousarray(a, np.uint8) for a in (inext, ilast))
    vnext, vlast = _f32(vnext), _f32(vlast)
    dIdx, dIdy = (np.ascontiguousarray(a, np.int16) for a in (dIdx, dIdy))
    r, c = inext.shape
    Pc = np.ascontiguousarray(Pcurr, np.float64)
    Pl = np.ascontiguousarray(Plast, np.float64)
    out = np.zeros(29, np.float64)
    res = np.zeros(2, np.int32)
    sigma = np.zeros(1, np.float32)
    per = np.zeros((r * c, 29), np.float32) if rows else None
    lib().sfo_rgb_step(_p(inext, U8P), _p(ilast, U8P), _p(vnext, F32P), _p(vlast, F32P), _p(dIdx, I16P),
                       _p(dIdy, I16P), c, r, _p(Pc, F64P), _p(Pl, F64P), *map(float, K), int(fp64), _p(out, F64P),
                       _p(res, I32P), _p(sigma, F32P), _p(per, F32P) if rows else None)
    return (out, (int(res[0]), int(res[1])), float(sigma[0])) + ((per,) if rows else ())


def _view(ptr, dtype, n):
    buf = (C.c_char * (n * dtype.itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype, count=n)


class Map:
    """Oracle voxel-block hash map (Mapping::Create, Mapping.cc:11-51)."""

    def __init__(self, voxel_size, trunc_dist, num_buckets, num_excess, num_sdf_blocks,
                 depth_min=0.1, depth_max=3.0, max_rendering_blocks=260000):
        self.cfg = Config(voxel_size, trunc_dist, depth_min, depth_max, num_buckets, num_excess,
                          num_sdf_blocks, max_rendering_blocks)
        self.h = lib().sfo_map_create(C.byref(self.cfg))
        self.num_entries = num_buckets + num_excess

    def __del__(self):
        if getattr(self, "h", None):
            lib().sfo_map_destroy(self.h)
            self.h = None

    def reset(self):
        lib().sfo_map_reset(self.h)

    @property
    def entries(self):
        return _view(lib().sfo_map_entries(self.h), ENTRY_DTYPE, self.num_entries)

    @property
    def voxels(self):
        return _view(lib().sfo_map_voxels(self.h), VOXEL_DTYPE, self.cfg.num_sdf_blocks * 512)

    @property
    def visible(self):
        return _view(lib().sfo_map_visible(self.h), ENTRY_DTYPE, self.num_entries)

    @property
    def heap(self):
        return _view(lib().sfo_map_heap(self.h), np.dtype("<i4"), self.cfg.num_sdf_blocks)

    def counters(self):
        out = np.zeros(4, np.int32)
        lib().sfo_map_counters(self.h, _p(out, I32P))
        return out

    def alloc(self, depth, P, K):
        depth = _f32(depth)
        rows, cols = depth.shape
        R, _, t = pose_to_gpu(P)
        lib().sfo_alloc(self.h, _p(depth, F32P), cols, rows, _p(R, F32P), _p(t, F32P), *map(float, K))

    def visibility(self, P, K, cols, rows, depth_max=None, depth_min=None):
        R, RI, t = pose_to_gpu(P)
        dmax = self.cfg.depth_max if depth_max is None else depth_max
        dmin = self.cfg.depth_min if depth_min is None else depth_min
        return lib().sfo_visibility(self.h, _p(R, F32P), _p(RI, F32P), _p(t, F32P), cols, rows,
                                    *map(float, K), dmax, dmin)

    def integrate(self, depth, rgb, P, K):
        depth = _f32(depth)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        rows, cols = depth.shape
        _, RI, t = pose_to_gpu(P)
        lib().sfo_integrate(self.h, _p(depth, F32P), _p(rgb, U8P), cols, rows, _p(RI, F32P), _p(t, F32P),
                            *map(float, K), self.cfg.depth_max, self.cfg.depth_min)

    def integrate_f64(self, depth, P, K):
        """The FP64 shadow of this frame's TSDF update (measurement only):
        call after visibility() and before integrate() of the same frame.
        P: the FP64 camera->world pose the FP32 rotation is taken from."""
        depth = _f32(depth)
        rows, cols = depth.shape
        _, RI, t = pose_to_gpu(P)
        P64 = np.ascontiguousarray(P, np.float64)
        lib().sfo_integrate_f64(self.h, _p(depth, F32P), cols, rows, _p(RI, F32P), _p(t, F32P), _p(P64, F64P),
                                *map(float, K), self.cfg.depth_max, self.cfg.depth_min)

    def tsdf_f64_error(self):
        """(max |tsdf32 - tsdf64|, RMS, voxels) over the voxels the FP64
        shadow covers."""
        out = np.zeros(3, np.float64)
        lib().sfo_tsdf_f64_error(self.h, _p(out, F64P))
        return float(out[0]), float(out[1]), int(out[2])

    def semantics(self, depth, rgb, nmap_, mask, num_detection, P, K):
        depth, nmap_ = _f32(depth), _f32(nmap_)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        mask = np.ascontiguousarray(mask, np.uint8)
        rows, cols = depth.shape
        _, RI, t = pose_to_gpu(P)
        lib().sfo_semantics(self.h, _p(depth, F32P), _p(rgb, U8P), _p(nmap_, F32P), _p(mask, U8P),
                            num_detection, cols, rows, _p(RI, F32P), _p(t, F32P), *map(float, K),
                            self.cfg.depth_max, self.cfg.depth_min)

    def unify_neighbor(self, nvis=None):
        """Fusion::UnifyNeighbor over hash entries [0, noVisible); `nvis`
        first sets noVisible."""
        if nvis is not None:
            lib().sfo_map_set_no_visible(self.h, int(nvis))
        lib().sfo_unify_neighbor(self.h)

    def analyze_semantics(self, depth, rgb, nmap_, mask, num_detection, P, K):
        """AnalyzeMapSemantics (FuseMap.cu:1164-1247) after its visibility
        pass: the label pass, then UnifyNeighbor."""
        self.semantics(depth, rgb, nmap_, mask, num_detection, P, K)
        self.unify_neighbor()

    def mesh(self, max_tri=2000000):
        """MeshScene: (vertices [n,3,3], normals [n,3,3], colours [n,3,3] uint8)."""
        v = np.zeros((max_tri, 3, 3), np.float32)
        n = np.zeros((max_tri, 3, 3), np.float32)
        c = np.zeros((max_tri, 3, 3), np.uint8)
        k = lib().sfo_mesh(self.h, max_tri, _p(v, F32P), _p(n, F32P), _p(c, U8P))
        return v[:k], n[:k], c[:k]

    def fuse(self, depth, rgb, nmap_, mask, num_detection, P, K, unify=True):
        """FuseMapColor.  unify=False stops before the UnifyNeighbor pass
        (which then runs as unify_neighbor())."""
        depth, nmap_ = _f32(depth), _f32(nmap_)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        rows, cols = depth.shape
        mask = np.zeros((rows, cols), np.uint8) if mask is None else np.ascontiguousarray(mask, np.uint8)
        R, RI, t = pose_to_gpu(P)
        return lib().sfo_fuse(self.h, _p(depth, F32P), _p(rgb, U8P), _p(nmap_, F32P), _p(mask, U8P),
                              num_detection, cols, rows, _p(R, F32P), _p(RI, F32P), _p(t, F32P),
                              *map(float, K), 1 if unify else 0)

    def zrange(self, P, K, zc, zr, max_blocks=0):
        _, RI, t = pose_to_gpu(P)
        zmin = np.zeros((zr, zc), np.float32)
        zmax = np.zeros((zr, zc), np.float32)
        blocks = np.zeros(max(max_blocks, 1), RBLOCK_DTYPE)
        n = C.c_uint(0)
        ok = lib().sfo_zrange(self.h, _p(zmin, F32P), _p(zmax, F32P), zc, zr, self.cfg.depth_max,
                              self.cfg.depth_min, _p(RI, F32P), _p(t, F32P), *map(float, K),
                              blocks.ctypes.data_as(C.c_void_p), max_blocks, C.byref(n))
        return bool(ok), zmin, zmax, blocks[:min(n.value, max_blocks)], n.value

    def reloc_score(self, vmap, stride, poses, inlier_sdf):
        """RelocScoreBatch: scores of candidate poses (n x 4 x 4, camera -> world)."""
        vm = _f32(vmap)
        rows, cols = vm.shape[:2]
        poses = np.asarray(poses, np.float64).reshape(-1, 4, 4)
        pf = np.concatenate([poses[:, :3, :3].reshape(-1, 9), poses[:, :3, 3]], axis=1).astype(np.float32)
        out = np.zeros(len(poses), RELOC_DTYPE)
        lib().sfo_reloc_score(self.h, _p(vm, F32P), cols, rows, int(stride), _p(np.ascontiguousarray(pf), F32P),
                              len(poses), float(inlier_sdf), out.ctypes.data_as(C.c_void_p))
        return out

    def raycast_smooth_f64(self, P, K, zmin, zmax, gv, gn, xi=(0, 0, 0, 0, 0, 0), vox=-1, delta=0.0):
        """FP64 reference of RaycastAdjoint: sum(gv . v + gn . n) at exp(xi) P with voxel `vox` moved by delta,
        the march's decisions fixed by the float march at P."""
        zmin, zmax = _f32(zmin), _f32(zmax)
        zr, zc = zmin.shape
        gv = _f32(gv)
        rows, cols = gv.shape[:2]
        fx, fy, cx, cy = map(float, K)
        invfx = np.float32(1.0 / np.float64(np.float32(fx)))
        invfy = np.float32(1.0 / np.float64(np.float32(fy)))
        T = np.ascontiguousarray(P, np.float64)
        x = np.ascontiguousarray(xi, np.float64)
        gnp = _p(_f32(gn), F32P) if gn is not None else None
        return lib().sfo_raycast_smooth_f64(self.h, _p(gv, F32P), gnp, cols, rows, _p(zmin, F32P), _p(zmax, F32P),
                                            zc, zr, _p(T, F64P), float(invfx), float(invfy), cx, cy, _p(x, F64P),
                                            int(vox), float(delta))

    def raycast(self, P, K, cols, rows, zmin, zmax):
        zmin, zmax = _f32(zmin), _f32(zmax)
        zr, zc = zmin.shape
        R, RI, t = pose_to_gpu(P)
        vm = np.empty((rows, cols, 4), np.float32)
        nm = np.empty((rows, cols, 4), np.float32)
        fx, fy, cx, cy = map(float, K)
        invfx = np.float32(1.0 / np.float64(np.float32(fx)))
        invfy = np.float32(1.0 / np.float64(np.float32(fy)))
        lib().sfo_raycast(self.h, _p(vm, F32P), _p(nm, F32P), cols, rows, _p(zmin, F32P), _p(zmax, F32P),
                          zc, zr, _p(R, F32P), _p(RI, F32P), _p(t, F32P), float(invfx), float(invfy), cx, cy)
        return vm, nm


class System:
    """Oracle of the whole per-frame loop (System::GrabImage, System.cc:131-270)."""

    def __init__(self, map_kw, cols, rows, K, levels=3, iters=(10, 5, 4), min_count=(2000, 1000, 100),
                 depth_scale=1000.0, depth_cutoff=3.0, icp_thresh=1e-4, init_pose=None, rgb_term=False):
        self.cfg = Config(map_kw["voxel_size"], map_kw["trunc_dist"], map_kw.get("depth_min", 0.1),
                          map_kw.get("depth_max", 3.0), map_kw["num_buckets"], map_kw["num_excess"],
                          map_kw["num_sdf_blocks"], map_kw.get("max_rendering_blocks", 260000))
        Kf = np.asarray(K, np.float32)
        it = np.asarray(iters, np.int32)
        mc = np.asarray(min_count, np.int32)
        ip = np.eye(4) if init_pose is None else np.ascontiguousarray(init_pose, np.float64)
        ip = np.ascontiguousarray(ip, np.float64)
        self.cols, self.rows, self.levels = cols, rows, levels
        self.h = lib().sfo_system_create(C.byref(self.cfg), cols, rows, levels, _p(Kf, F32P), depth_scale,
                                         depth_cutoff, _p(it, I32P), _p(mc, I32P), icp_thresh, _p(ip, F64P))
        self.num_entries = self.cfg.num_buckets + self.cfg.num_excess
        self.rgb_term = bool(rgb_term)
        lib().sfo_system_set_rgb(self.h, int(self.rgb_term))

    def __del__(self):
        if getattr(self, "h", None):
            lib().sfo_system_destroy(self.h)
            self.h = None

    def set_reloc(self, poses):
        """Relocalisation candidates (n x 4 x 4 camera->world) for lost frames."""
        P = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 16))
        self._reloc = P
        lib().sfo_system_set_reloc(self.h, _p(P, F64P), int(P.shape[0]))

    def set_mapping(self, enabled):
        """Tracker::mappingDisabled = not enabled (localisation mode)."""
        lib().sfo_system_set_mapping(self.h, int(bool(enabled)))

    def grab(self, depth_u16, rgb, mask=None, num_detection=0):
        d = np.ascontiguousarray(depth_u16, np.uint16)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        m = np.zeros(d.shape, np.uint8) if mask is None else np.ascontiguousarray(mask, np.uint8)
        pose = np.zeros(16, np.float64)
        stats = np.zeros(13, np.float64)
        ok = lib().sfo_system_grab(self.h, _p(d, U16P), _p(rgb, U8P), _p(m, U8P), num_detection,
                                   _p(pose, F64P), _p(stats, F64P))
        return bool(ok), pose.reshape(4, 4), stats

    def entries(self):
        return _view(lib().sfo_map_entries(lib().sfo_system_map(self.h)), ENTRY_DTYPE, self.num_entries).copy()

    def voxels(self):
        return _view(lib().sfo_map_voxels(lib().sfo_system_map(self.h)), VOXEL_DTYPE,
                     self.cfg.num_sdf_blocks * 512).copy()

    def vmap(self, level=0):
        n = (self.cols >> level) * (self.rows >> level) * 4
        return _view(lib().sfo_system_vmap(self.h, level), np.dtype("<f4"), n).reshape(
            self.rows >> level, self.cols >> level, 4).copy()

    def nmap(self, level=0):
        n = (self.cols >> level) * (self.rows >> level) * 4
        return _view(lib().sfo_system_nmap(self.h, level), np.dtype("<f4"), n).reshape(
            self.rows >> level, self.cols >> level, 4).copy()
