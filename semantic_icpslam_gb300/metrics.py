"""Per-frame metrics log of the frame loop: one JSON object per line.

The reference reports per frame on stdout: "track icp failed" when a level's
ICP count falls short or the error is NaN (Tracking/Tracking.cc:451-455),
"bad : <icp>/<rgb> <|sin euler|> <|t|>" when the frame-end gate rejects the
motion (Tracking.cc:508-515), and Mapping::CheckVisPercent's visible share
of the used blocks (Mapping/Mapping.cc:383-401).  FrameLog writes those
quantities, with the rest of sf_frame_stats, as JSON lines, and with
echo=True also prints the reference's two tracking messages.
"""
import json
import sys
import time

import numpy as np

_FAIL = {0: "ok", 1: "icp_count_or_nan", 2: "rejected", 3: "timeout"}


def visible_percent(stats, num_sdf_blocks):
    """Mapping::CheckVisPercent: visible blocks over the blocks taken from
    the heap (heapCounter counts the free blocks down)."""
    used = num_sdf_blocks - max(int(stats.heap_counter), 0)
    return float(stats.visible) / float(used) if used > 0 else 0.0


def frame_record(index, stats, num_sdf_blocks, host_ms=None):
    """The JSON object of one frame."""
    pose = np.array(stats.pose[:], np.float64).reshape(4, 4)
    rec = {
        "frame": int(index),
        "tracked": int(stats.tracked),
        "accepted": int(stats.accepted),
        "fail": _FAIL.get(int(stats.fail), int(stats.fail)),
        "state": int(stats.state),
        "missed": int(stats.missed),
        "relocalised": int(stats.relocalised),
        "iterations": int(stats.iterations),
        "icp_error": float(stats.icp_error),
        "icp_count": int(stats.icp_count),
        "rgb_error": float(stats.rgb_error),
        "rgb_count": int(stats.rgb_count),
        "visible_blocks": int(stats.visible),
        "allocated_entries": int(stats.allocated),
        "heap_counter": int(stats.heap_counter),
        "visible_percent": visible_percent(stats, num_sdf_blocks),
        "flags": int(stats.flags),
        "t": pose[:3, 3].tolist(),
    }
    if host_ms is not None:
        rec["host_ms"] = float(host_ms)
    return rec


class FrameLog:
    """Appends one JSON line per frame to `path` (or a file object).

    `echo` prints the reference's tracking messages to stdout for frames it
    would print them for.  Use as System(..., log=FrameLog(path)) or call
    write(stats) after each grab."""

    def __init__(self, path, num_sdf_blocks, echo=False):
        self._own = isinstance(path, str)
        self.f = open(path, "a") if self._own else path
        self.num_sdf_blocks = int(num_sdf_blocks)
        self.echo = echo
        self.index = 0

    def write(self, stats, host_ms=None):
        rec = frame_record(self.index, stats, self.num_sdf_blocks, host_ms)
        self.f.write(json.dumps(rec) + "\n")
        self.index += 1
        if self.echo and not stats.accepted:
            if stats.fail == 1:
                print("track icp failed", file=sys.stdout)
            elif stats.fail == 2:
                print("bad : %g/%g" % (stats.icp_error, stats.rgb_error), file=sys.stdout)
        return rec

    def timed_grab(self, system, *args, **kw):
        """system.grab(*args) with its host wall time in the record (for a
        System created without a log of its own)."""
        t0 = time.perf_counter()
        st = system.grab(*args, **kw)
        self.write(st, (time.perf_counter() - t0) * 1e3)
        return st

    def flush(self):
        self.f.flush()

    def close(self):
        if self._own and not self.f.closed:
            self.f.close()
