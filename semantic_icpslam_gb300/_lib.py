"""ctypes binding of libsfusion.so (the C ABI declared in include/sfusion.h).

There is no CPU fallback: importing the bindings without the built library
raises, and every entry point reports a non-zero status as an exception.
"""
import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
# SF_LIBRARY selects another build of the library (the bounds-checked
# libsfusion_checked.so); the default is the release build
LIB_PATH = os.environ.get("SF_LIBRARY") or os.path.join(_HERE, "libsfusion.so")

(SF_OK, SF_ERR_INVALID, SF_ERR_CUDA, SF_ERR_OVERFLOW, SF_ERR_TIMEOUT, SF_ERR_NO_DEVICE, SF_ERR_STATE,
 SF_ERR_TOO_LARGE, SF_ERR_IO) = range(9)
STATUS_NAMES = {0: "SF_OK", 1: "SF_ERR_INVALID", 2: "SF_ERR_CUDA", 3: "SF_ERR_OVERFLOW",
                4: "SF_ERR_TIMEOUT", 5: "SF_ERR_NO_DEVICE", 6: "SF_ERR_STATE", 7: "SF_ERR_TOO_LARGE",
                8: "SF_ERR_IO"}
ICP_STATIC_MAX_PIXELS = 4194304  # SF_ICP_STATIC_MAX_PIXELS

FLAG_NAMES = {1 << 0: "DEDUP_FULL", 1 << 1: "PENDING_FULL", 1 << 2: "HEAP_EMPTY", 1 << 3: "EXCESS_FULL",
              1 << 4: "VISIBLE_FULL", 1 << 5: "RENDER_FULL", 1 << 6: "BARRIER_TIMEOUT",
              1 << 7: "COORD_RANGE"}


class SfError(RuntimeError):
    def __init__(self, fn, status):
        super().__init__("%s returned %s" % (fn, STATUS_NAMES.get(status, status)))
        self.status = status


class Float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Mat3(C.Structure):
    _fields_ = [("rowx", Float3), ("rowy", Float3), ("rowz", Float3)]


class Intrinsics(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float)]


class Image(C.Structure):
    _fields_ = [("data", C.c_void_p), ("step", C.c_size_t), ("cols", C.c_int), ("rows", C.c_int)]


class RelocScore(C.Structure):
    _fields_ = [("valid", C.c_uint32), ("inliers", C.c_uint32), ("sum_abs_sdf", C.c_float),
                ("mean_abs_sdf", C.c_float)]


class MapConfig(C.Structure):
    _fields_ = [("voxel_size", C.c_float), ("trunc_dist", C.c_float), ("depth_min", C.c_float),
                ("depth_max", C.c_float), ("num_buckets", C.c_uint32), ("num_excess", C.c_uint32),
                ("num_sdf_blocks", C.c_uint32), ("max_rendering_blocks", C.c_uint32)]


class DeviceMap(C.Structure):
    _fields_ = [("heap_mem", C.c_void_p), ("entry_ptr", C.c_void_p), ("heap_counter", C.c_void_p),
                ("bucket_mutex", C.c_void_p), ("voxel_blocks", C.c_void_p),
                ("no_visible_blocks", C.c_void_p), ("hash_entries", C.c_void_p),
                ("visible_entries", C.c_void_p)]


class SystemConfig(C.Structure):
    _fields_ = [("map", MapConfig), ("cols", C.c_int), ("rows", C.c_int), ("levels", C.c_int),
                ("K", Intrinsics), ("depth_scale", C.c_float), ("depth_cutoff", C.c_float),
                ("iters", C.c_int * 4), ("min_count", C.c_int * 4), ("icp_thresh", C.c_float),
                ("zrange_cols", C.c_int), ("zrange_rows", C.c_int), ("use_graph", C.c_int), ("rgb_term", C.c_int)]


class FrameStats(C.Structure):
    _fields_ = [("tracked", C.c_int), ("accepted", C.c_int), ("fail", C.c_int), ("iterations", C.c_int),
                ("icp_error", C.c_float), ("icp_count", C.c_int), ("visible", C.c_uint32),
                ("heap_counter", C.c_int), ("entry_ptr", C.c_int), ("allocated", C.c_int),
                ("flags", C.c_uint32), ("pose", C.c_double * 16), ("rgb_error", C.c_float),
                ("rgb_count", C.c_int), ("state", C.c_int), ("missed", C.c_int), ("relocalised", C.c_int)]


class RelocCandidate(C.Structure):
    _fields_ = [("visible", C.c_uint32), ("rendered", C.c_int), ("evaluated", C.c_int), ("accepted", C.c_int),
                ("fail", C.c_int), ("iterations", C.c_int), ("icp_error", C.c_float), ("icp_count", C.c_int),
                ("pose", C.c_double * 16)]


class AutotuneReport(C.Structure):
    _fields_ = [("candidates", C.c_int), ("chosen", C.c_int), ("ms", C.c_float * 16), ("minb", C.c_int * 16),
                ("tile_x", C.c_int * 16), ("tile_y", C.c_int * 16), ("integrate_candidates", C.c_int),
                ("integrate_chosen", C.c_int), ("integrate_ms", C.c_float * 8), ("integrate_ctas", C.c_int * 8),
                ("alloc_candidates", C.c_int), ("alloc_chosen", C.c_int), ("alloc_ms", C.c_float * 8),
                ("alloc_tile_x", C.c_int * 8), ("alloc_tile_y", C.c_int * 8)]


class FrameTune(C.Structure):
    _fields_ = [("raycast", C.c_int), ("integrate_ctas_per_sm", C.c_int), ("alloc_tile", C.c_int)]


vp = C.c_void_p
pvp = C.POINTER(C.c_void_p)
U32P = C.POINTER(C.c_uint32)
I32P = C.POINTER(C.c_int)
F32P = C.POINTER(C.c_float)
F64P = C.POINTER(C.c_double)

# name -> argtypes (restype is int status for every entry point)
SIGNATURES = {
    "sf_context_create": [pvp],
    "sf_context_destroy": [vp],
    "sf_context_stream": [vp, pvp],
    "sf_context_sync": [vp],
    "sf_context_flags": [vp, U32P],
    "sf_memcpy": [vp, vp, vp, C.c_size_t],
    "sf_kernel_launches": [C.POINTER(C.c_uint64)],
    "sf_icp_profile": [vp, C.c_int, C.POINTER(C.c_uint64)],
    "sf_icp_barrier_limits": [vp, C.c_uint32, C.c_uint32],
    "sf_icp_predict": [vp, C.c_int],
    "sf_map_create": [C.POINTER(MapConfig), pvp],
    "sf_map_wrap": [C.POINTER(MapConfig), C.POINTER(DeviceMap), pvp],
    "sf_map_destroy": [vp],
    "sf_map_arrays": [vp, C.POINTER(DeviceMap)],
    "sf_map_bounds_status": [vp, vp, U32P],
    "sf_build_flags": [U32P],
    "sf_map_rebuild_index": [vp, vp],
    "sf_map_counters": [vp, vp, I32P],
    "sf_map_write": [vp, vp, C.c_char_p],
    "sf_map_read": [vp, vp, C.c_char_p],
    "sf_ResetMap": [vp, vp],
    "sf_FilterDepth": [vp, Image, Image, Image, C.c_float, C.c_float],
    "sf_ComputeVMap": [vp, Image, Image, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float],
    "sf_ComputeNMap": [vp, Image, Image],
    "sf_PyrDownGauss": [vp, Image, Image],
    "sf_ResizeMap": [vp, Image, Image, Image, Image],
    "sf_BuildPyramid": [vp, Image, Image, C.POINTER(Image), C.POINTER(Image), C.POINTER(Image), C.c_int,
                        Intrinsics, C.c_float, C.c_float],
    "sf_ICPStep": [vp, Image, Image, Image, Image, Mat3, Float3, Mat3, Mat3, Float3, Intrinsics, F32P,
                   F64P, F64P],
    "sf_ICPStep_static": [vp, Image, Image, Image, Image, Mat3, Float3, Mat3, Mat3, Float3, Intrinsics,
                          F32P, F64P, F64P],
    "sf_ImageToIntensity": [vp, Image, Image],
    "sf_PyrDownGauss_u8": [vp, Image, Image],
    "sf_ComputeDerivativeImage": [vp, Image, Image, Image],
    "sf_RGBStep": [vp] + [Image] * 6 + [Mat3] * 4 + [Float3, Float3, Intrinsics, F32P, F64P, F64P],
    "sf_ComputeSE3_rgbd": [vp, C.c_int] + [C.POINTER(Image)] * 8 + [Intrinsics, I32P, I32P, C.c_float, F64P, F64P,
                                                                    I32P, F32P],
    "sf_RaycastAdjoint": [vp, vp, Image, Image, Mat3, Mat3, Float3] + [C.c_float] * 4 + [Image, Image, vp, F64P],
    "sf_RelocScoreBatch": [vp, vp, Image, C.c_int, F64P, C.c_int, C.c_float, C.POINTER(RelocScore)],
    "sf_ValidatePoseBatch": [vp, vp, C.c_int] + [C.POINTER(Image)] * 4 + [Intrinsics, F64P, C.c_int, I32P, I32P,
                                                                         C.c_float, C.c_uint32,
                                                                         C.POINTER(RelocCandidate), I32P],
    "sf_system_set_reloc_candidates": [vp, F64P, C.c_int],
    "sf_ComputeSE3": [vp, C.c_int, C.POINTER(Image), C.POINTER(Image), C.POINTER(Image), C.POINTER(Image),
                      Intrinsics, I32P, I32P, C.c_float, F64P, F64P, I32P, F32P],
    "sf_CheckBlockVisibility": [vp, vp, Mat3, Mat3, Float3, C.c_int, C.c_int] + [C.c_float] * 6 + [U32P],
    "sf_FuseMapColor": [vp, vp, Image, Image, Image, Image, C.c_int, Mat3, Mat3, Float3] + [C.c_float] * 6
                       + [U32P],
    "sf_AnalyzeMapSemantics": [vp, vp, Image, Image, Image, Image, C.c_int, Mat3, Mat3, Float3]
                              + [C.c_float] * 6,
    "sf_UnifyNeighbor": [vp, vp],
    "sf_MeshScene": [vp, vp, vp, vp, vp, C.c_uint32, U32P],
    "sf_mesh_write_ply": [vp, C.c_char_p, vp, vp, vp, C.c_uint32],
    "sf_SemanticAnalysis": [vp, vp, Image, Image, Image, Image, C.c_int, Mat3, Mat3, Float3] + [C.c_float] * 4,
    "sf_CreateRenderingBlocks": [vp, vp, Image, Image, C.c_float, C.c_float, vp, vp, Mat3, Float3, C.c_uint32]
                                + [C.c_float] * 4 + [I32P],
    "sf_Raycast": [vp, vp, Image, Image, Image, Image, Mat3, Mat3, Float3] + [C.c_float] * 4,
    "sf_system_create": [vp, C.POINTER(SystemConfig), F64P, pvp],
    "sf_system_destroy": [vp],
    "sf_system_grab": [vp, vp, vp, vp, C.c_int, C.POINTER(FrameStats)],
    "sf_system_grab_device": [vp, vp, vp, vp, C.c_int],
    "sf_system_stats": [vp, C.POINTER(FrameStats)],
    "sf_system_model_maps": [vp, C.c_int, C.POINTER(Image), C.POINTER(Image)],
    "sf_system_frame_maps": [vp, C.c_int, C.POINTER(Image), C.POINTER(Image), C.POINTER(Image)],
    "sf_system_get_map": [vp, pvp],
    "sf_system_set_timing": [vp, C.c_int],
    "sf_system_autotune": [vp, C.c_int, C.POINTER(AutotuneReport)],
    "sf_system_get_tune": [vp, C.POINTER(FrameTune)],
    "sf_system_set_tune": [vp, C.POINTER(FrameTune)],
    "sf_system_set_mapping": [vp, C.c_int],
    "sf_system_stage_ms": [vp, F32P],
    "sf_system_pose_device": [vp, C.POINTER(C.POINTER(C.c_double))],
}

_lib = None
_lock = threading.Lock()


def load():
    """Loads libsfusion.so; raises ImportError if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError("libsfusion.so is not built (run __graft_entry__.build() or "
                                  "python -m semantic_icpslam_gb300.build): %s" % LIB_PATH)
            L = C.CDLL(LIB_PATH)
            for name, args in SIGNATURES.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = C.c_int
            _lib = L
    return _lib


def call(name, *args):
    st = getattr(load(), name)(*args)
    if st != SF_OK:
        raise SfError(name, st)
    return st
