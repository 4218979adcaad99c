"""Launch-shape tuning of the frame loop with a per-configuration cache.

sf_system_autotune times the raycast's launch shapes, the integration's
grid and the allocation walk's pixel tile on the device at hand, in the state the frame left (every shape
computes the same maps), and keeps the fastest.  tuned() runs it once per
configuration and device and keeps the choice in a JSON file, so later
systems of the same configuration take it with sf_system_set_tune instead
of timing again.

The cache lives at $SF_TUNE_CACHE, else in the user's cache directory.
"""
import ctypes as C
import json
import os
import tempfile

from . import _lib


def cache_path():
    p = os.environ.get("SF_TUNE_CACHE")
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "semantic_icpslam_gb300", "tune.json")


def config_key(cfg, device):
    """The configuration a choice belongs to: device, image size, pyramid,
    voxel size, map sizes and tracking mode."""
    m = cfg.map
    return "|".join(str(x) for x in (device, cfg.cols, cfg.rows, cfg.levels, round(m.voxel_size, 6),
                                     round(m.trunc_dist, 6), m.num_buckets, m.num_excess, m.num_sdf_blocks,
                                     cfg.rgb_term))


def _device_name():
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return "cuda"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    d = os.path.dirname(path)
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=d, suffix=".tmp")
    with os.fdopen(fd, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tuned(system, reps=10, path=None):
    """Applies the cached launch shapes of this system's configuration, or
    times them (sf_system_autotune, after at least one grabbed frame) and
    caches the choice.  Returns (entry, cached)."""
    path = path or cache_path()
    key = config_key(system.cfg, _device_name())
    data = _load(path)
    if key in data:
        e = data[key]
        t = _lib.FrameTune(int(e["raycast"]), int(e["integrate_ctas_per_sm"]), int(e.get("alloc_tile", 0)))
        _lib.call("sf_system_set_tune", system.h, C.byref(t))
        return e, True
    rep = _lib.AutotuneReport()
    _lib.call("sf_system_autotune", system.h, int(reps), C.byref(rep))
    t = _lib.FrameTune()
    _lib.call("sf_system_get_tune", system.h, C.byref(t))
    entry = {"raycast": t.raycast, "integrate_ctas_per_sm": t.integrate_ctas_per_sm, "alloc_tile": t.alloc_tile,
             "raycast_ms": {"%dx%d/%d" % (rep.tile_x[i], rep.tile_y[i], rep.minb[i]): round(rep.ms[i], 5)
                            for i in range(rep.candidates)},
             "integrate_ms": {str(rep.integrate_ctas[i]): round(rep.integrate_ms[i], 5)
                              for i in range(rep.integrate_candidates)},
             "alloc_ms": {"%dx%d" % (rep.alloc_tile_x[i], rep.alloc_tile_y[i]): round(rep.alloc_ms[i], 5)
                          for i in range(rep.alloc_candidates)}}
    data[key] = entry
    _store(path, data)
    return entry, False
