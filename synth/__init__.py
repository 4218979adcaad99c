"""Seeded synthetic RGB-D sequences: the workload generator of the tests and
the benchmark (sf_synth.h, synth.cpp).

The reference runs on TUM RGB-D sequences (640x480 uint16 depth, uchar3
colour), which are not available here.  This generator renders analytic
scenes of the same shapes: a room of boxes and spheres or a corridor of
boxes and pillars, along a seeded circle, spline or forward trajectory, with
depth noise sigma = 0.0012 + 0.0019 (z - 0.4)^2 m, random dropout, seeded
Perlin colour and optional instance masks with random label flips.

It is host C++ in its own library, libsfsynth.so, apart from the CUDA
library, so a process that only needs frames (the CPU baseline arm of the
benchmark) loads none of the product's code.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libsfsynth.so")
SRC = os.path.join(HERE, "synth.cpp")
HDR = os.path.join(HERE, "sf_synth.h")

_lib = None


def build(force=False):
    """Compiles libsfsynth.so in-tree (g++, no CUDA)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > max(os.path.getmtime(SRC),
                                                                           os.path.getmtime(HDR)):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", HERE, SRC, "-o", LIB + ".tmp", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("synth build failed: %s\n%s" % (" ".join(cmd), r.stderr[-3000:]))
    os.replace(LIB + ".tmp", LIB)
    return LIB


class SynthConfig(C.Structure):
    _fields_ = [("scene", C.c_int), ("trajectory", C.c_int), ("cols", C.c_int), ("rows", C.c_int),
                ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("depth_scale", C.c_float), ("dropout", C.c_float), ("label_flip", C.c_float),
                ("n_objects", C.c_int), ("noise", C.c_float), ("seed", C.c_uint64)]


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        F64P = C.POINTER(C.c_double)
        L.sf_synth_create.argtypes = [C.POINTER(SynthConfig), C.POINTER(C.c_void_p)]
        L.sf_synth_destroy.argtypes = [C.c_void_p]
        L.sf_synth_pose.argtypes = [C.c_void_p, C.c_int, F64P]
        L.sf_synth_frame.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, F64P]
        for f in (L.sf_synth_create, L.sf_synth_destroy, L.sf_synth_pose, L.sf_synth_frame):
            f.restype = C.c_int
        _lib = L
    return _lib


def _check(status, what):
    if status != 0:
        raise RuntimeError("%s failed with status %d" % (what, status))


class Synth:
    """Seeded synthetic RGB-D sequence (sf_synth.h)."""

    ROOM, CORRIDOR = 0, 1
    CIRCLE, SPLINE, FORWARD = 0, 1, 2

    def __init__(self, cols, rows, K, scene=0, trajectory=0, seed=1, dropout=0.0, label_flip=0.0,
                 n_objects=0, noise=1.0, depth_scale=1000.0):
        self.cfg = SynthConfig(scene, trajectory, cols, rows, K[0], K[1], K[2], K[3], depth_scale, dropout,
                               label_flip, n_objects, noise, seed)
        h = C.c_void_p()
        _check(load().sf_synth_create(C.byref(self.cfg), C.byref(h)), "sf_synth_create")
        self.h = h
        self.cols, self.rows = cols, rows

    def close(self):
        if getattr(self, "h", None):
            load().sf_synth_destroy(self.h)
            self.h = None

    __del__ = close

    def frame(self, i):
        """(depth uint16 HxW in depth units, rgb uint8 HxWx3, mask uint8 HxW,
        ground-truth camera->world pose 4x4) of frame i."""
        d = np.zeros((self.rows, self.cols), np.uint16)
        rgb = np.zeros((self.rows, self.cols, 3), np.uint8)
        m = np.zeros((self.rows, self.cols), np.uint8)
        P = np.zeros(16, np.float64)
        _check(load().sf_synth_frame(self.h, i, d.ctypes.data, rgb.ctypes.data, m.ctypes.data,
                                     P.ctypes.data_as(C.POINTER(C.c_double))), "sf_synth_frame")
        return d, rgb, m, P.reshape(4, 4)

    def pose(self, i):
        P = np.zeros(16, np.float64)
        _check(load().sf_synth_pose(self.h, i, P.ctypes.data_as(C.POINTER(C.c_double))), "sf_synth_pose")
        return P.reshape(4, 4)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
