"""GB300-native dense tracking-and-fusion loop (sm_103a CUDA behind a C ABI).

Python host layer over include/sfusion.h, shaped like the reference's
Tracker / Mapping / System host code.  Device memory for the reference-shaped
launchers is plain CUDA memory; helpers accept torch CUDA tensors.  There is
no CPU path: everything here calls libsfusion.so.
"""
import ctypes as C
import os
import weakref

import numpy as np

from . import _lib
from ._lib import (FrameStats, Image, Intrinsics, MapConfig, Mat3, Float3, SfError,
                   SystemConfig, call, load)

__all__ = ["Context", "Map", "System", "image", "pose_to_gpu", "mat3", "float3",
           "SfError", "load", "DEFAULT_C1", "DEFAULT_C2"]


# ----------------------------------------------------------------- helpers
def image(t, elem_bytes=None):
    """sf_image view of a 2-D (rows, cols[, channels]) CUDA tensor."""
    rows, cols = int(t.shape[0]), int(t.shape[1])
    if elem_bytes is None:
        elem_bytes = t.element_size() * (int(np.prod(t.shape[2:])) if t.dim() > 2 else 1)
    assert t.is_contiguous(), "image tensors must be contiguous"
    return Image(t.data_ptr(), cols * elem_bytes, cols, rows)


def mat3(R):
    R = np.asarray(R, np.float32)
    return Mat3(Float3(*R[0]), Float3(*R[1]), Float3(*R[2]))


def float3(t):
    t = np.asarray(t, np.float32)
    return Float3(float(t[0]), float(t[1]), float(t[2]))


def pose_to_gpu(P):
    """Frame::GpuRotation / GpuInvRotation / GpuTranslation (Core/Frame.cc:626-645):
    (Matrix3f R, Matrix3f R^T, float3 t) from a double 4x4 camera->world pose."""
    P = np.asarray(P, np.float64)
    return mat3(P[:3, :3].astype(np.float32)), mat3(P[:3, :3].T.astype(np.float32)), \
        float3(P[:3, 3].astype(np.float32))


class Context:
    """sf_context: one CUDA stream + ICP scratch on the current device."""

    def __init__(self):
        h = C.c_void_p()
        call("sf_context_create", C.byref(h))
        self.h = h
        self._systems = weakref.WeakSet()  # closed before the context

    def close(self):
        if getattr(self, "log", None) is not None:
            self.log.close()
            self.log = None
        if getattr(self, "h", None):
            for s in list(getattr(self, "_systems", ())):
                s.close()
            load().sf_context_destroy(self.h)
            self.h = None

    __del__ = close

    @property
    def stream(self):
        s = C.c_void_p()
        call("sf_context_stream", self.h, C.byref(s))
        return s.value

    def sync(self):
        call("sf_context_sync", self.h)

    def flags(self):
        f = C.c_uint32()
        call("sf_context_flags", self.h, C.byref(f))
        return f.value

    def memcpy(self, dst, src, nbytes):
        """Copy between host/device addresses (ints) and wait."""
        call("sf_memcpy", self.h, dst, src, nbytes)

    def download(self, ptr, dtype, count):
        out = np.empty(count, dtype)
        self.memcpy(out.ctypes.data, ptr, out.nbytes)
        return out


class Map:
    """sf_map: the voxel-block hash map (Mapping::Create, Mapping.cc:11-51)."""

    def __init__(self, voxel_size, trunc_dist, num_buckets, num_excess, num_sdf_blocks,
                 depth_min=0.1, depth_max=3.0, max_rendering_blocks=260000, _handle=None):
        self.cfg = MapConfig(voxel_size, trunc_dist, depth_min, depth_max, num_buckets, num_excess,
                             num_sdf_blocks, max_rendering_blocks)
        self.num_entries = num_buckets + num_excess
        self._owned = _handle is None
        if _handle is None:
            h = C.c_void_p()
            call("sf_map_create", C.byref(self.cfg), C.byref(h))
            self.h = h
        else:
            self.h = _handle

    def close(self):
        if getattr(self, "h", None) and self._owned:
            load().sf_map_destroy(self.h)
        self.h = None

    __del__ = close

    def arrays(self):
        d = _lib.DeviceMap()
        call("sf_map_arrays", self.h, C.byref(d))
        return d

    def counters(self, ctx):
        out = (C.c_int * 4)()
        call("sf_map_counters", ctx.h, self.h, out)
        return list(out)

    def unify_neighbor(self, ctx):
        """sf_UnifyNeighbor: the neighbour-label pass over hash slots
        [0, visible count) (UnifyNeighborKernel)."""
        call("sf_UnifyNeighbor", ctx.h, self.h)

    def write(self, ctx, path):
        """map.bin in the reference's byte layout (System::WriteMapToDisk)."""
        call("sf_map_write", ctx.h, self.h, os.fsencode(path))

    def read(self, ctx, path):
        """Loads a map.bin of this map's sizes (System::ReadMapFromDisk)."""
        call("sf_map_read", ctx.h, self.h, os.fsencode(path))


class System:
    """sf_system: the whole per-frame loop (System::GrabImage)."""

    def __init__(self, ctx, cfg, init_pose=None, log=None):
        """log: a metrics.FrameLog, or a path for one (one JSON line per
        grabbed frame)."""
        self.ctx = ctx
        self.cfg = cfg
        if isinstance(log, str):
            from .metrics import FrameLog
            log = FrameLog(log, cfg.map.num_sdf_blocks)
        self.log = log
        h = C.c_void_p()
        P = np.eye(4) if init_pose is None else np.asarray(init_pose, np.float64)
        P = np.ascontiguousarray(P, np.float64)
        call("sf_system_create", ctx.h, C.byref(cfg), P.ctypes.data_as(_lib.F64P), C.byref(h))
        self.h = h
        ctx._systems.add(self)

    def close(self):
        if getattr(self, "log", None) is not None:
            self.log.close()
            self.log = None
        if getattr(self, "h", None):
            load().sf_system_destroy(self.h)
            self.h = None

    __del__ = close

    def grab(self, depth, rgb, mask=None, num_detection=0):
        d = np.ascontiguousarray(depth, np.uint16)
        c = np.ascontiguousarray(rgb, np.uint8)
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        st = FrameStats()
        call("sf_system_grab", self.h, d.ctypes.data, c.ctypes.data, None if m is None else m.ctypes.data,
             num_detection, C.byref(st))
        if self.log is not None:
            self.log.write(st)
        return st

    def set_reloc_candidates(self, poses):
        """sf_system_set_reloc_candidates: candidate camera->world poses
        (n x 4 x 4) tried by every frame that starts lost."""
        P = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 16))
        call("sf_system_set_reloc_candidates", self.h, P.ctypes.data_as(_lib.F64P), int(P.shape[0]))

    def grab_device(self, depth_ptr, rgb_ptr, mask_ptr=None, num_detection=0):
        call("sf_system_grab_device", self.h, depth_ptr, rgb_ptr, mask_ptr, num_detection)

    def autotune(self, reps=20):
        """sf_system_autotune: times the last frame's raycast under each
        launch shape and keeps the fastest.  Returns a list of
        (minb, tile_x, tile_y, ms) per candidate and the chosen index."""
        rep = _lib.AutotuneReport()
        call("sf_system_autotune", self.h, int(reps), C.byref(rep))
        cands = [(rep.minb[i], rep.tile_x[i], rep.tile_y[i], rep.ms[i]) for i in range(rep.candidates)]
        return cands, rep.chosen

    def set_mapping(self, enabled):
        """sf_system_set_mapping: False switches to localisation
        (Tracker::mappingDisabled), True back to mapping."""
        call("sf_system_set_mapping", self.h, int(bool(enabled)))

    def stats(self):
        st = FrameStats()
        call("sf_system_stats", self.h, C.byref(st))
        return st

    def model_maps(self, level=0):
        v, n = Image(), Image()
        call("sf_system_model_maps", self.h, level, C.byref(v), C.byref(n))
        return v, n

    def frame_maps(self, level=0):
        v, n, d = Image(), Image(), Image()
        call("sf_system_frame_maps", self.h, level, C.byref(v), C.byref(n), C.byref(d))
        return v, n, d

    def map(self):
        h = C.c_void_p()
        call("sf_system_get_map", self.h, C.byref(h))
        m = self.cfg.map
        return Map(m.voxel_size, m.trunc_dist, m.num_buckets, m.num_excess, m.num_sdf_blocks,
                   m.depth_min, m.depth_max, m.max_rendering_blocks, _handle=h)


def system_config(cols, rows, K, voxel_size, trunc_dist, num_buckets, num_excess, num_sdf_blocks,
                  levels=3, iters=(10, 5, 4), min_count=(2000, 1000, 100), depth_scale=1000.0,
                  depth_cutoff=3.0, icp_thresh=1e-4, use_graph=1, depth_min=0.1, depth_max=3.0,
                  zrange=(0, 0), max_rendering_blocks=260000, rgb_term=0):
    cfg = SystemConfig()
    cfg.map = MapConfig(voxel_size, trunc_dist, depth_min, depth_max, num_buckets, num_excess, num_sdf_blocks,
                        max_rendering_blocks)
    cfg.cols, cfg.rows, cfg.levels = cols, rows, levels
    cfg.K = Intrinsics(*K)
    cfg.depth_scale, cfg.depth_cutoff = depth_scale, depth_cutoff
    for l in range(4):
        cfg.iters[l] = iters[l] if l < len(iters) else 0
        cfg.min_count[l] = min_count[l] if l < len(min_count) else 0
    cfg.icp_thresh = icp_thresh
    cfg.zrange_cols, cfg.zrange_rows = zrange
    cfg.use_graph = use_graph
    cfg.rgb_term = int(rgb_term)
    return cfg


def validate_pose_batch(ctx, m, next_vmaps, next_nmaps, last_vmaps, last_nmaps, K, poses, iters=(3, 3, 2),
                        min_count=(2000, 1000, 100), thresh=1e-3, min_visible=512):
    """sf_ValidatePoseBatch (Tracker::ValidatePose over n candidates).
    Image lists are sf_image per level (level 0 first); poses n x 4 x 4.
    Returns (list of RelocCandidate, chosen index or -1)."""
    L = len(next_vmaps)
    P = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 16))
    n = P.shape[0]
    arr = lambda ims: (Image * L)(*ims)
    it = (C.c_int * L)(*[int(iters[l]) if l < len(iters) else 0 for l in range(L)])
    mc = (C.c_int * L)(*[int(min_count[l]) if l < len(min_count) else 0 for l in range(L)])
    out = (_lib.RelocCandidate * n)()
    chosen = C.c_int(-1)
    call("sf_ValidatePoseBatch", ctx.h, m.h, L, arr(next_vmaps), arr(next_nmaps), arr(last_vmaps), arr(last_nmaps),
         Intrinsics(*K), P.ctypes.data_as(_lib.F64P), n, it, mc, float(thresh), int(min_visible), out,
         C.byref(chosen))
    return list(out), chosen.value


# Workloads: a 320x240 / 10 mm room sequence and a 640x480 / 5 mm room
# sequence (2% dropout, spline trajectory).
DEFAULT_C1 = dict(cols=320, rows=240, K=(262.5, 262.5, 159.5, 119.5), voxel_size=0.01, trunc_dist=0.03,
                  num_buckets=1 << 18, num_excess=1 << 16, num_sdf_blocks=1 << 16, iters=(10, 5, 4))
DEFAULT_C2 = dict(cols=640, rows=480, K=(525.0, 525.0, 319.5, 239.5), voxel_size=0.005, trunc_dist=0.04,
                  num_buckets=1 << 20, num_excess=1 << 18, num_sdf_blocks=1 << 18, iters=(10, 5, 4))
