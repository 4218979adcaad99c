#!/usr/bin/env python
"""Frames/s of the dense tracking-and-fusion loop on GB300.

Workload: 640x480 seeded room sequence (spline trajectory, 2 % depth dropout,
Perlin RGB, depth noise 0.0012 + 0.0019 (z - 0.4)^2 m), 5 mm voxels, 2^20
buckets, 4 cm truncation, 3-level ICP with 10/5/4 iterations.  One step is
one frame through System::GrabImage's order: pyramid -> ICP (all levels and
iterations) -> allocation -> visibility -> integration -> raycast -> resize.
Frames 0..W-1 warm the loop up; frames W..W+K-1 are timed.

`value`: CUDA-graph form, inputs resident in HBM, one CUDA-event pair per
step on the system's stream; L2 is flushed (a 256 MiB write) before every
timed step, outside the timed intervals.
`plain`: the same kernels launched one by one, host-driven (ICP sums
downloaded and solved on the host every iteration, as the reference does).
`e2e`: CUDA-graph form through the public host-buffer API (sf_system_grab:
pinned host -> device copies and the stats read-back inside the timed
region; each step timed on the host clock up to the context's
synchronisation, L2 flushed between steps).
`errors`: per timed frame, the loop's pose against the FP64 oracle's
ComputeSE3 on the same inputs, sf_ICPStep's J^T J / J^T r against FP64 sums,
and, over the whole sequence, the TSDF against an FP64 shadow of the
integration and the device map against the FP32 oracle map.
`--impl reference`: the reference's own device code compiled as host
C++/OpenMP at these constants (oracle/_ref/c2), driven in GrabImage's order,
timed on the host cores over the same frames; beside it the reference's CUDA
build on the GPU.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s ICP+fuse+raycast 640x480 at ≤1e-5 pose err: graph vs plain; %HBM peak"
COLS, ROWS = 640, 480
K = (525.0, 525.0, 319.5, 239.5)
MAP = dict(voxel_size=0.005, trunc_dist=0.04, num_buckets=1 << 20, num_excess=1 << 18, num_sdf_blocks=1 << 19)
ITERS = (10, 5, 4)
LEVELS, MIN_COUNT = 3, (2000, 1000, 100)
SEQ = dict(trajectory=1, seed=2, dropout=0.02)
WORKLOAD = ("640x480 room sequence (seeded spline trajectory, 2% dropout, Perlin RGB), 5 mm voxels, "
            "2^20 buckets, 4 cm truncation, 3-level ICP 10/5/4")
STAGES = ["pyramid", "icp", "alloc", "visibility_zrange", "integrate", "raycast", "resize_stats"]


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.p = None
        self.lines = []
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-i", str(gpu_index), "-lms", "20"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x):
    """The largest x over the ranks of the default process group (x itself
    when there is none, or one rank): the job's time is its slowest rank's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_fps(ws, steps, elapsed):
    """Whole-job frames/s: every rank runs `steps` frames of its own copy of
    the sequence (weak scaling), the job takes the slowest rank's time."""
    return ws * steps / elapsed


def make_frames(n, rank=0):
    """The sequence a rank runs: every replica runs the same frames (the
    same work per GPU), independently."""
    from synth import Synth  # host-only generator library: loads none of the product's code
    syn = Synth(COLS, ROWS, K, **SEQ)
    return [syn.frame(i) for i in range(n)]


def bench_config():
    """The `config` of both arms' lines (the same dict, so the two arms'
    configurations compare equal)."""
    return {"workload": WORKLOAD, "global_batch": "1 frame per GPU per step",
            "parallelism": "replicas (every GPU runs its own copy of the sequence; no data exchanged)",
            "l2": "flushed before every timed step (a %d MiB write on the timed stream, outside the timed "
                  "intervals); each step reads a new frame" % (FLUSH_BYTES >> 20)}


FLUSH_BYTES = 256 << 20
AUTOTUNE = True  # every timed form takes the tuned launch shapes of its configuration (--no-autotune: defaults)


class L2Flush:
    """Writes a buffer larger than L2 on a stream (between timed steps)."""

    def __init__(self):
        import torch
        self.buf = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def __call__(self, stream):
        import torch
        with torch.cuda.stream(stream):
            self.buf.fill_(1)


def sys_cfg(sf, mode, rgb=0):
    return sf.system_config(cols=COLS, rows=ROWS, K=K, levels=LEVELS, iters=ITERS, min_count=MIN_COUNT,
                            use_graph=mode, rgb_term=rgb, **MAP)


def use_corridor_config():
    """The 1280x720 corridor stress configuration (`--config c3`): 4-level
    pyramid, 3 mm voxels, 2^22 buckets, 2.4 cm truncation, seeded corridor of
    boxes and pillars walked forward at 1.5 cm per frame."""
    global METRIC, COLS, ROWS, K, MAP, ITERS, LEVELS, MIN_COUNT, SEQ, WORKLOAD
    METRIC = "frames/s ICP+fuse+raycast 1280x720 corridor stress (4 levels, 3 mm, 2^22 buckets)"
    COLS, ROWS = 1280, 720
    K = (1050.0, 1050.0, 639.5, 359.5)
    MAP = dict(voxel_size=0.003, trunc_dist=0.024, num_buckets=1 << 22, num_excess=1 << 20,
               num_sdf_blocks=1 << 21)
    # the 160x90 level runs no ICP iteration (with the reference's
    # NaN-propagating ResizeMap the coarsest model level is too sparse in the
    # corridor); 72 boxes and pillars, so that surfaces facing along the
    # corridor stay in view and the tracker keeps its position along it;
    # depth noise a quarter of the room's
    ITERS, LEVELS, MIN_COUNT = (10, 5, 4, 0), 4, (2000, 1000, 100, 0)
    SEQ = dict(scene=1, trajectory=2, seed=2, dropout=0.02, noise=0.25, n_objects=72)
    WORKLOAD = ("1280x720 corridor sequence (20 m corridor of 72 seeded boxes and pillars, forward at 1.5 cm per "
                "frame, 2% dropout, noise x0.25, Perlin RGB), 3 mm voxels, 2^22 buckets, 2.4 cm truncation, "
                "4-level pyramid, ICP 10/5/4/0")


def launches(sf):
    import ctypes as C
    v = C.c_uint64()
    sf.call("sf_kernel_launches", C.byref(v))
    return v.value


def label_frames(n):
    """The room with ten labelled objects and 5% label flips (the semantic
    mode's workload)."""
    from synth import Synth
    syn = Synth(COLS, ROWS, K, **dict(SEQ, n_objects=10, label_flip=0.05))
    return [syn.frame(i) for i in range(n)]


def time_device_resident(sf, ctx, frames, steps, warmup, mode, barrier, timing=False, autotune=None, rgb=0,
                         ndet=0, flush=None):
    """Frames/s with inputs already in HBM: one CUDA-event pair per timed
    step on the system stream, L2 flushed before each step outside the
    pair.  With autotune, sf_system_autotune runs half-way through the
    warm-up (its choice is recaptured in the graph before the timed
    frames)."""
    import ctypes as C
    import torch
    dev = [(torch.from_numpy(d).cuda(), torch.from_numpy(c).cuda(), torch.from_numpy(m).cuda())
           for d, c, m, _ in frames[:steps + warmup]]
    torch.cuda.synchronize()
    s = sf.System(ctx, sys_cfg(sf, mode, rgb), init_pose=frames[0][3])
    stage_ms = np.zeros(len(STAGES))
    stats = []
    if timing:
        sf.call("sf_system_set_timing", s.h, 1)
    tune = None
    autotune = AUTOTUNE if autotune is None else autotune
    for i in range(warmup):
        s.grab_device(dev[i][0].data_ptr(), dev[i][1].data_ptr(), dev[i][2].data_ptr() if ndet else None, ndet)
        if autotune and i == warmup // 2:
            from semantic_icpslam_gb300 import tune as T
            entry, cached = T.tuned(s, reps=10)
            tune = dict(entry, cached=cached, cache=T.cache_path())
    ctx.sync()
    stream = torch.cuda.ExternalStream(ctx.stream)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    barrier()
    torch.cuda.synchronize()
    l0 = launches(sf)
    sampler = ClockSampler(torch.cuda.current_device()) if not timing else None
    ms = (C.c_float * 7)()
    for k, i in enumerate(range(warmup, warmup + steps)):
        if flush is not None:
            flush(stream)
        ev[k][0].record(stream)
        s.grab_device(dev[i][0].data_ptr(), dev[i][1].data_ptr(), dev[i][2].data_ptr() if ndet else None, ndet)
        ev[k][1].record(stream)
        if timing:
            sf.call("sf_system_stage_ms", s.h, ms)
            stage_ms += np.array(ms[:])
            stats.append(s.stats())
    ev[-1][1].synchronize()
    clocks = sampler.stop() if sampler else None
    torch.cuda.synchronize()
    barrier()
    elapsed = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    n_launch = launches(sf) - l0
    last = s.stats()
    s.close()
    del dev
    return dict(elapsed=elapsed, launches=n_launch, clocks=clocks, stage_ms=stage_ms / max(steps, 1),
                stats=stats, last=last, autotune=tune)


def time_mesh(sf, ctx, frames, n, reps=3):
    """sf_MeshScene over the map of the whole sequence (Mapping::CreateModel):
    milliseconds per call (CUDA events on the context stream, mean of reps
    after one warm-up) and triangles."""
    import ctypes as C
    import torch
    s = sf.System(ctx, sys_cfg(sf, 1), init_pose=frames[0][3])
    for i in range(n):
        s.grab(frames[i][0], frames[i][1])
    m = s.map()
    cap = 8000000
    v = torch.empty((cap, 9), dtype=torch.float32, device="cuda")
    nn = torch.empty((cap, 9), dtype=torch.float32, device="cuda")
    c = torch.empty((cap, 9), dtype=torch.uint8, device="cuda")
    k = C.c_uint32()
    sf.call("sf_MeshScene", ctx.h, m.h, v.data_ptr(), nn.data_ptr(), c.data_ptr(), cap, C.byref(k))
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        sf.call("sf_MeshScene", ctx.h, m.h, v.data_ptr(), nn.data_ptr(), c.data_ptr(), cap, C.byref(k))
    e1.record(stream)
    e1.synchronize()
    blocks = int(m.counters(ctx)[3])
    s.close()
    return {"ms": round(e0.elapsed_time(e1) / reps, 3), "triangles": int(k.value), "blocks": blocks}


def pinned(a):
    """A copy of numpy array a in page-locked host memory."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()


def time_e2e(sf, ctx, frames, steps, warmup, mode, rgb=0, flush=None):
    """Frames/s through sf_system_grab with host buffers in pinned memory:
    each step from the call to the context's synchronisation (the H2D
    copies of the frame, the whole frame, the D2H of its stats), on the
    host clock; L2 flushed between steps outside the timed intervals."""
    import torch
    s = sf.System(ctx, sys_cfg(sf, mode, rgb), init_pose=frames[0][3])
    host = [(pinned(d), pinned(c)) for d, c, _, _ in frames[:warmup + steps]]
    for i in range(warmup):
        s.grab(*host[i])
        if AUTOTUNE and i == warmup // 2:
            from semantic_icpslam_gb300 import tune as T
            T.tuned(s, reps=10)
    ctx.sync()
    stream = torch.cuda.ExternalStream(ctx.stream)
    total = 0.0
    tracked = 0
    for i in range(warmup, warmup + steps):
        if flush is not None:
            flush(stream)
            ctx.sync()
        t0 = time.perf_counter()
        st = s.grab(*host[i])
        ctx.sync()
        total += time.perf_counter() - t0
        tracked += st.tracked
    s.close()
    return total, tracked


class _DevBuf:
    """A device allocation of this library seen as a torch tensor (bytes)."""

    def __init__(self, ptr, nbytes):
        self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False),
                                         "version": 3, "strides": None}


def _dev_bytes(ptr, nbytes):
    import torch
    return torch.as_tensor(_DevBuf(ptr, nbytes), device="cuda")


def _icp_bytes(iterations):
    """ICP algorithmic bytes of one frame: 64 B per pixel per iteration
    (current vertex + normal, gathered model vertex + normal), iterations
    split over the levels coarse to fine as ComputeSE3 runs them (a stop
    ends every level)."""
    left, b = int(iterations), 0
    for l in range(LEVELS - 1, -1, -1):
        k = min(left, ITERS[l])
        b += 64 * (COLS >> l) * (ROWS >> l) * k
        left -= k
    return b


def stage_bytes(stats_list):
    """Mean algorithmic bytes per frame of the stages with a byte model
    (per-unit figures: pyramid 2WH + 4WH + 4P + 32P; ICP 64 B per pixel per
    iteration; integration V*512*32 + 8WH; raycast 32V + V*512*8 + 32WH;
    resize 32*(L1+L2 pixels)*5)."""
    V = np.array([st.visible for st in stats_list], np.float64)
    it = np.array([st.iterations for st in stats_list], np.float64)
    wh = COLS * ROWS
    P = sum((COLS >> l) * (ROWS >> l) for l in range(LEVELS))
    return {"pyramid": 6 * wh + 36 * P,
            "icp": float(np.mean([_icp_bytes(i) for i in it])),
            "integrate": float((V * 512 * 32 + 8 * wh).mean()),
            "raycast": float((32 * V + V * 512 * 8 + 32 * wh).mean()),
            "resize_stats": 32 * 5 * sum((COLS >> l) * (ROWS >> l) for l in range(1, LEVELS))}, V


def l2_copy_peak():
    """L2-resident copy bandwidth (GB/s, read + write bytes): a 24 MiB
    buffer copied back and forth 400 times after a warm-up; CUDA events."""
    import torch
    n = 24 << 20
    a = torch.empty(n, dtype=torch.uint8, device="cuda")
    b = torch.empty(n, dtype=torch.uint8, device="cuda")
    a.fill_(1)
    for _ in range(20):
        b.copy_(a)
        a.copy_(b)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(200):
        b.copy_(a)
        a.copy_(b)
    e1.record()
    e1.synchronize()
    return 2 * n * 400 / (e0.elapsed_time(e1) * 1e-3) / 1e9


def error_pass(sf, ctx, frames, steps, warmup):
    """Accuracy of the loop against the FP64 oracle, over frames 0..W+K-1 in
    the eager form (equal to the graph form bit for bit):
      * pose: for every timed frame, the loop's ComputeSE3 pose against the
        FP64 oracle's ComputeSE3 on the same inputs (the frame's measured
        pyramid, the model maps the loop raycast for the previous frame,
        the previous pose), max abs element of the 4x4 difference; beside
        it the FP32 oracle's (the reference's arithmetic) on the same
        inputs, against the loop and against FP64, and the largest error
        over the frames where FP64 runs as many iterations as the loop
        (ComputeSE3's divergence guard is discontinuous in the error, so a
        rounding-level difference can end a level one iteration earlier);
      * J^T J / J^T r: for every timed frame, sf_ICPStep at the frame's
        final pose (level 0) against the oracle's FP64 rows and sums,
        relative to the largest diagonal entry / the largest |b|;
      * TSDF: the oracle replays the mapping of every tracked frame with the
        loop's poses, with an FP64 shadow of each TSDF update (same voxels,
        distance and running average in double); max and RMS of
        |tsdf32 - tsdf64| at the end, and whether the device map equals the
        oracle's FP32 map voxel for voxel (per block position)."""
    import ctypes as C
    import torch
    from oracle import oracle as O
    s = sf.System(ctx, sys_cfg(sf, 2), init_pose=frames[0][3])
    om = O.Map(**MAP)
    pose_err, jtj_err, jtr_err, mism = [], [], [], 0
    e32, ref32, worst, same_it = [], [], None, []
    prev = None
    dl = lambda im: ctx.download(im.data, np.float32, im.rows * im.cols * 4).reshape(im.rows, im.cols, 4)
    Kf = lambda l: tuple(k / float(1 << l) for k in K)
    for i in range(warmup + steps):
        d, rgb, _, _ = frames[i]
        timed = i >= warmup and i > 0
        if timed:
            mv, mn = zip(*[tuple(map(dl, s.model_maps(l))) for l in range(LEVELS)])
        st = s.grab(d, rgb)
        P = np.array(st.pose[:]).reshape(4, 4)
        if timed:
            fm = [s.frame_maps(l) for l in range(LEVELS)]
            vs, ns = [dl(f[0]) for f in fm], [dl(f[1]) for f in fm]
            ok, P64, s64st = O.compute_se3(vs, ns, list(mv), list(mn), K, ITERS, MIN_COUNT, 1e-4, prev, prev,
                                           fp64=True)
            ok32, P32, s32st = O.compute_se3(vs, ns, list(mv), list(mn), K, ITERS, MIN_COUNT, 1e-4, prev, prev,
                                             fp64=False)
            if ok == bool(st.accepted):
                e = float(np.abs(P64 - P).max())
                pose_err.append(e)
                if int(s64st[2]) == int(st.iterations):
                    same_it.append(e)
                e32.append(float(np.abs(P32 - P).max()))
                ref32.append(float(np.abs(P32 - P64).max()))
                if e >= max(pose_err):
                    worst = {"frame": i, "err": e, "iterations": int(st.iterations),
                             "iterations_fp64": int(s64st[2]), "iterations_fp32_oracle": int(s32st[2]),
                             "fp32_oracle_vs_fp64": ref32[-1]}
            else:
                mism += 1
            # J^T J / J^T r at the final pose, level 0
            mv0, mn0 = torch.from_numpy(mv[0]).cuda(), torch.from_numpy(mn[0]).cuda()
            Rc, _, tc = sf.pose_to_gpu(P)
            Rl, RlI, tl = sf.pose_to_gpu(prev)
            res, A, b = (C.c_float * 2)(), (C.c_double * 36)(), (C.c_double * 6)()
            sf.call("sf_ICPStep", ctx.h, fm[0][0], sf.image(mv0), fm[0][1], sf.image(mn0), Rc, tc, Rl, RlI, tl,
                    sf.Intrinsics(*Kf(0)), res, A, b)
            s64 = O.icp_sums(vs[0], mv[0], ns[0], mn[0], P, prev, Kf(0), fp64=True)
            A64, b64 = O.create_matrix(s64)
            A32, b32 = np.array(A[:]).reshape(6, 6), np.array(b[:])
            # J^T J relative to its largest diagonal entry; J^T r relative to
            # its natural scale sqrt(max diag(J^T J) * sum r^2) (J^T r itself
            # is near zero at a converged pose)
            dmax = np.abs(np.diag(A64)).max()
            jtj_err.append(float(np.abs(A32 - A64).max() / dmax))
            jtr_err.append(float(np.abs(b32 - b64).max() / np.sqrt(dmax * max(s64[27], 1e-30))))
            del mv0, mn0
        if st.tracked:  # the oracle maps the frame as the loop did, with an FP64 shadow
            raw, _ = O.filter_depth(d, 1000.0, 3.0)
            om.alloc(raw, P, K)
            if om.visibility(P, K, COLS, ROWS):
                om.integrate_f64(raw, P, K)
                om.integrate(raw, rgb, P, K)
        prev = P
    tsdf_max, tsdf_rms, nvox = om.tsdf_f64_error()
    # the device map against the oracle's FP32 map, per block position
    from oracle.oracle import ENTRY_DTYPE, VOXEL_DTYPE
    m = s.map()
    a = m.arrays()
    ne = MAP["num_buckets"] + MAP["num_excess"]
    ge = ctx.download(a.hash_entries, ENTRY_DTYPE, ne)
    oe = np.array(om.entries)
    gsel, osel = ge[ge["ptr"] >= 0], oe[oe["ptr"] >= 0]
    key = lambda e: (e["x"].astype(np.int64) << 42) ^ ((e["y"].astype(np.int64) & 0x1fffff) << 21) ^ \
        (e["z"].astype(np.int64) & 0x1fffff)
    gk, ok_ = key(gsel), key(osel)
    same_set = np.array_equal(np.sort(gk), np.sort(ok_))
    map_equal = False
    if same_set:
        gsel, osel = gsel[np.argsort(gk)], osel[np.argsort(ok_)]
        vox = _dev_bytes(a.voxel_blocks, MAP["num_sdf_blocks"] * 512 * 16).view(-1, 512 * 16)
        gblk = vox[torch.from_numpy((gsel["ptr"] // 512).astype(np.int64)).cuda()].cpu().numpy()
        ov = om.voxels.view(np.uint8).reshape(-1, 512 * 16)
        oblk = ov[(osel["ptr"] // 512).astype(np.int64)]
        map_equal = bool(np.array_equal(gblk, oblk))
        del vox
    s.close()
    n_t = len(pose_err) + mism
    return {"frames": "timed frames %d..%d (pose, J^T J: %d compared); TSDF over frames 0..%d"
                      % (warmup, warmup + steps - 1, n_t, warmup + steps - 1),
            "pose_max": max(pose_err) if pose_err else None, "pose_mean": float(np.mean(pose_err)) if pose_err else None,
            "pose_median": float(np.median(pose_err)) if pose_err else None,
            "pose_frac_le_1e-5": float(np.mean(np.array(pose_err) <= 1e-5)) if pose_err else None,
            "fp32_oracle_frac_le_1e-5": float(np.mean(np.array(ref32) <= 1e-5)) if ref32 else None,
            "pose_worst": worst,
            "pose_max_same_iterations": max(same_it) if same_it else None,
            "frames_same_iterations": len(same_it),
            "pose_vs_fp32_oracle_max": max(e32) if e32 else None,
            "fp32_oracle_vs_fp64_max": max(ref32) if ref32 else None,
            "acceptance_mismatch": mism,
            "jtj_rel_max": max(jtj_err) if jtj_err else None, "jtr_rel_max": max(jtr_err) if jtr_err else None,
            "tsdf_max": tsdf_max, "tsdf_rms": tsdf_rms, "tsdf_voxels": nvox,
            "map_blocks": int(len(gsel)), "map_block_set_equal_fp32_oracle": bool(same_set),
            "map_voxels_equal_fp32_oracle": map_equal}


def _ref_cpu_lib():
    import ctypes as C
    path = os.path.join(ROOT, "oracle", "_ref", "c2", "libref.so")
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    L.refcpu_create.restype = C.c_void_p
    L.refcpu_create.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), C.c_float, C.c_float,
                                C.POINTER(C.c_double)]
    L.refcpu_grab.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    L.refcpu_destroy.argtypes = [C.c_void_p]
    L.refcpu_threads.restype = C.c_int
    return L


def time_reference_cpu(frames, steps, warmup, budget_s=None):
    """The reference's CPU implementation of the loop over frames
    0..warmup+steps-1, frames warmup.. timed (host clock per frame).  The
    reference's own device code compiled as host C++/OpenMP at the 640x480
    constants (oracle/_ref/c2/libref.so) when present and the workload is
    the 640x480 room; else the oracle port of the loop (C++/OpenMP).
    budget_s bounds the timed frames' total time (at least two frames)."""
    import ctypes as C
    L = _ref_cpu_lib() if (COLS, ROWS) == (640, 480) else None
    pose = np.zeros(16, np.float64)
    if L is not None:
        init = np.ascontiguousarray(frames[0][3], np.float64)
        h = L.refcpu_create(COLS, ROWS, (C.c_float * 4)(*K), 1000.0, 3.0, init.ctypes.data_as(C.POINTER(C.c_double)))
        grab = lambda d, c: L.refcpu_grab(h, np.ascontiguousarray(d).ctypes.data, np.ascontiguousarray(c).ctypes.data,
                                          pose.ctypes.data_as(C.POINTER(C.c_double)))
        kind, cores = "reference", int(L.refcpu_threads())
        what = ("the reference's Tracking/*.cu and Mapping/*.cu compiled as host C++ (CUDA emulation header, "
                "OpenMP over each launch's blocks) at the 640x480 constants, driven in GrabImage's order, "
                "ICP-only ComputeSE3 (getRow per pixel, FP64 sums per thread)")
    else:
        from oracle import oracle as O
        so = O.System(dict(MAP), COLS, ROWS, K, levels=LEVELS, iters=ITERS, min_count=MIN_COUNT,
                      init_pose=frames[0][3])
        grab = lambda d, c: so.grab(d, c)[0]
        kind, cores = "port", omp_threads()
        what = "the oracle loop (the reference's algorithm restated in C++/OpenMP, pinned to its kernels)"
    for i in range(warmup):
        grab(frames[i][0], frames[i][1])
    total, n, tracked = 0.0, 0, 0
    for i in range(warmup, warmup + steps):
        t0 = time.perf_counter()
        tracked += int(bool(grab(frames[i][0], frames[i][1])))
        total += time.perf_counter() - t0
        n += 1
        if budget_s is not None and n >= 2 and total >= budget_s:
            break
    if L is not None:
        L.refcpu_destroy(h)
    return {"fps": n / total, "frames": n, "kind": kind, "cores": cores, "what": what, "tracked": tracked}


def omp_threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def time_validate(sf, ctx, frames, n=256, reps=3, seed=5):
    """Tracker::ValidatePose over n candidate poses (the true pose and seeded
    5 cm / 5 deg perturbations) against one 640x480 frame
    (sf_ValidatePoseBatch: visibility, raycast, resize and ComputeSE3 with
    ITERATIONS_RELOC {3, 3, 2} for every candidate), after the sequence's
    first frames are fused.  Milliseconds per call through the C ABI (host
    poses in, host results out), mean of reps after one warm-up."""
    s = sf.System(ctx, sys_cfg(sf, 2), init_pose=frames[0][3])
    k = min(8, len(frames) - 2)
    for i in range(k):
        s.grab(frames[i][0], frames[i][1])
    m = s.map()
    s.grab(frames[k][0], frames[k][1])  # frame k's pyramid: the frame to relocalise
    nxt = [s.frame_maps(l)[:2] for l in range(LEVELS)]
    P = np.array(s.stats().pose[:], np.float64).reshape(4, 4)
    rng = np.random.default_rng(seed)
    cand = [P]
    for _ in range(n - 1):
        w = rng.normal(0, np.deg2rad(5.0), 3)
        th = np.linalg.norm(w)
        Kx = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]]) / max(th, 1e-12)
        Q = P.copy()
        Q[:3, :3] = (np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx) @ P[:3, :3]
        Q[:3, 3] += rng.normal(0, 0.05, 3)
        cand.append(Q)
    cand = np.array(cand)
    # LastFrame's maps: the model maps the loop ray traced for frame k - 1
    # (now overwritten by frame k's); frame k's raycast stands in for them
    lv = [v for v, _ in [s.model_maps(l) for l in range(LEVELS)]]
    ln = [n_ for _, n_ in [s.model_maps(l) for l in range(LEVELS)]]
    args = (ctx, m, [v for v, _ in nxt], [n_ for _, n_ in nxt], lv, ln, K, cand, (3, 3, 2)[:LEVELS],
            MIN_COUNT[:LEVELS], 1e-3, 512)
    out, chosen = sf.validate_pose_batch(*args)
    t0 = time.perf_counter()
    for _ in range(reps):
        out, chosen = sf.validate_pose_batch(*args)
    ms = (time.perf_counter() - t0) * 1e3 / reps
    s.close()
    return {"candidates": n, "pixels": int(COLS * ROWS), "ms_per_call": round(ms, 3),
            "evaluated": int(sum(c.evaluated for c in out)), "accepted": int(sum(c.accepted for c in out)),
            "chosen": int(chosen), "true_pose_accepted": bool(out[0].accepted),
            "note": "Tracker::ValidatePose per candidate (UpdateVisibility, RayTrace, ResizeImages, ComputeSE3 "
                    "{3, 3, 2}) for all candidates in one call; sigma 5 cm / 5 deg around the tracked pose of "
                    "frame %d" % k}


def time_reloc(sf, ctx, frames, n=256, reps=10, seed=5):
    """RelocScoreBatch on the workload: n candidate poses (the true pose and
    seeded 5 cm / 5 deg perturbations) scored against one 640x480 frame in one
    launch, after the sequence's first frames are fused.  Time per call through
    the C ABI (host poses in, host scores out)."""
    import ctypes as C
    s = sf.System(ctx, sys_cfg(sf, 2), init_pose=frames[0][3])
    for i in range(min(8, len(frames) - 1)):
        s.grab(frames[i][0], frames[i][1])
    k = min(8, len(frames) - 1)
    s.grab(frames[k][0], frames[k][1])
    vmap, _, _ = s.frame_maps(0)
    P = np.array(s.stats().pose[:], np.float64).reshape(4, 4)
    rng = np.random.default_rng(seed)
    cand = [P]
    for _ in range(n - 1):
        w = rng.normal(0, np.deg2rad(5.0), 3)
        th = np.linalg.norm(w)
        Kx = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]]) / max(th, 1e-12)
        Q = P.copy()
        Q[:3, :3] = (np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx) @ P[:3, :3]
        Q[:3, 3] += rng.normal(0, 0.05, 3)
        cand.append(Q)
    poses = np.ascontiguousarray(np.array(cand), np.float64)
    out = (sf._lib.RelocScore * n)()
    m = s.map()
    pp = poses.ctypes.data_as(C.POINTER(C.c_double))
    sf.call("sf_RelocScoreBatch", ctx.h, m.h, vmap, 1, pp, n, 0.5, out)
    t0 = time.perf_counter()
    for _ in range(reps):
        sf.call("sf_RelocScoreBatch", ctx.h, m.h, vmap, 1, pp, n, 0.5, out)
    ms = (time.perf_counter() - t0) * 1e3 / reps
    inl = np.array([o.inliers for o in out])
    s.close()
    return {"candidates": n, "pixels": int(COLS * ROWS), "ms_per_call": round(ms, 3),
            "candidate_pixels_per_s": round(n * COLS * ROWS / (ms * 1e-3), 1),
            "true_pose_rank": int((inl > inl[0]).sum()),
            "note": "two launches per call (8 CTAs per candidate, then the fixed-order sum of their partials); "
                    "sigma 5 cm / 5 deg candidates around the tracked pose of frame %d" % k}


def load_traffic(kernel, first, count):
    """Mean dram__bytes_read.sum + dram__bytes_write.sum per launch of the
    kernel over frames first..first+count-1 of this workload, from the
    committed ncu capture of the same frames (None when the capture does not
    cover them)."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic_640x480.json")
    try:
        with open(path) as f:
            per = json.load(f)["kernels"][kernel]["per_frame_dram_bytes"]  # entry i: frame i
        if first + count > len(per):
            return None
        vals = per[first:first + count]
        return float(np.mean(vals))
    except (OSError, KeyError, ValueError, TypeError):
        return None


STAGE_KERNEL = {"pyramid": "k_pyramid_levels_3", "icp": "k_icp_persistent", "integrate": "k_integrate",
                "raycast": "k_raycast", "resize_stats": "k_resize"}


def time_reference_cuda(frames, steps, warmup, rgb_term=False, flush=None):
    """The reference's own CUDA launchers (oracle/_ref/gpu_c2/librefgpu.so,
    built by oracle/ref_shim/build_ref_gpu.py) in System::GrabImage's order,
    ICP-only (or with the photometric term, the reference's default, when
    rgb_term), host buffers in: frames/s over `steps` frames after `warmup`,
    each frame timed on the host clock up to the device's synchronisation,
    L2 flushed between frames outside the timed intervals."""
    import ctypes as C
    lib_path = os.path.join(ROOT, "oracle", "_ref", "gpu_c2", "librefgpu.so")
    if not os.path.exists(lib_path):
        return {"unavailable": "the reference's CUDA build is not present (oracle/_ref/gpu_c2 not prepared)"}
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no GPU"}
    except ImportError:
        return {"unavailable": "no torch"}
    L = C.CDLL(lib_path)
    L.refgpu_create.restype = C.c_void_p
    L.refgpu_create.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), C.c_float, C.c_float, C.POINTER(C.c_double)]
    L.refgpu_grab.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    L.refgpu_destroy.argtypes = [C.c_void_p]
    K4 = (C.c_float * 4)(*K)
    init = np.ascontiguousarray(frames[0][3], np.float64)
    h = L.refgpu_create(COLS, ROWS, K4, 1000.0, 3.0, init.ctypes.data_as(C.POINTER(C.c_double)))
    if not h:
        return {"unavailable": "refgpu_create failed"}
    if rgb_term:
        if not hasattr(L, "refgpu_set_rgb"):
            L.refgpu_destroy(h)
            return {"unavailable": "the reference's CUDA build predates its photometric mode"}
        L.refgpu_set_rgb.argtypes = [C.c_void_p, C.c_int]
        L.refgpu_set_rgb(h, 1)
    pose = np.zeros(16, np.float64)
    n = min(len(frames), steps + warmup)
    host = [(pinned(frames[i][0]), pinned(frames[i][1])) for i in range(n)]
    stream = torch.cuda.current_stream()
    tracked, err, dt = 0, 0.0, 0.0
    for i in range(n):
        if i >= warmup and flush is not None:
            flush(stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d, rgb = host[i]
        tr = L.refgpu_grab(h, d.ctypes.data, rgb.ctypes.data, pose.ctypes.data_as(C.POINTER(C.c_double)))
        torch.cuda.synchronize()
        if i >= warmup:
            dt += time.perf_counter() - t0
            tracked += tr
            err = max(err, float(np.abs(pose.reshape(4, 4)[:3, 3] - frames[i][3][:3, 3]).max()))
    L.refgpu_destroy(h)
    timed = n - warmup
    return {"value": round(timed / dt, 3), "unit": "frames/s", "steps": timed, "warmup": warmup,
            "tracked_frames": int(tracked), "max_translation_error_vs_ground_truth_m": round(err, 5),
            "kind": "reference CUDA build (Tracking/*.cu, Mapping/*.cu for sm_103a), %s ComputeSE3, "
                    "pinned host buffers in, the reference's per-launch synchronisation; the same timed frames and "
                    "L2 flush as e2e" % ("RGB-D (icpOnly = false: RGBStep + ICPStep)" if rgb_term else "ICP-only")}


def run_reference(args):
    """The reference arm: the reference's CPU implementation of the loop on
    the host cores, over the same frames, steps and warm-up as the GPU arm
    (rank 0 only); its CUDA build beside it."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    n = args.steps + args.warmup
    frames = make_frames(n)
    r = time_reference_cpu(frames, args.steps, args.warmup)
    fps = r["fps"]
    line = {"impl": "reference", "metric": METRIC, "value": round(fps, 4), "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000.0 / fps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 6x6 solve)",
            "data": "synthetic: " + WORKLOAD, "config": bench_config(),
            "cpu_baseline": {"value": round(fps, 4), "unit": "frames/s", "cores": r["cores"], "kind": r["kind"],
                             "sample": "frames %d..%d of the sequence after %d warm-up frames: %s"
                                       % (args.warmup, args.warmup + r["frames"] - 1, args.warmup, r["what"])},
            "tracked_frames": r["tracked"],
            "e2e": {"value": round(fps, 4), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    try:
        flush = L2Flush()
    except Exception:
        flush = None
    line["reference_cuda"] = time_reference_cuda(frames, args.steps, args.warmup, flush=flush)
    if args.config == "c2":
        line["reference_cuda_rgbd"] = time_reference_cuda(frames, args.steps, args.warmup, rgb_term=True,
                                                          flush=flush)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=280)  # 300 frames with the warm-up, as the workload names
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-errors", action="store_true", help="skip the accuracy pass against the FP64 oracle")
    ap.add_argument("--no-modes", action="store_true",
                    help="skip the RGB-D, semantic, mesh, ValidatePose and reloc-score measurements")
    ap.add_argument("--map-blocks", type=int, default=19,
                    help="log2 of the voxel-block heap (2^19 blocks = 4 GB of voxels)")
    ap.add_argument("--config", default="c2", choices=["c2", "c3"],
                    help="c2: the 640x480 room sequence (the headline); c3: the 1280x720 corridor stress run")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch shapes (by default the headline form takes the tuned shapes of "
                         "its configuration during the warm-up: cached, else timed by sf_system_autotune)")
    ap.add_argument("--quick", action="store_true",
                    help="only the CUDA-graph timing (for profiler runs)")
    ap.add_argument("--rgbd", action="store_true",
                    help="with --quick: time the RGB-D tracking mode (ComputeSE3 with icpOnly = false) instead")
    ap.add_argument("--labels", action="store_true",
                    help="with --quick: time the semantic mode (detections every frame) instead")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.config == "c3":
        use_corridor_config()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        barrier = lambda: dist.barrier()
    else:
        barrier = lambda: None
    import semantic_icpslam_gb300 as sf
    sf.load()
    ctx = sf.Context()
    flush = L2Flush()
    n = args.steps + args.warmup
    MAP["num_sdf_blocks"] = 1 << args.map_blocks
    frames = make_frames(n, rank)
    if args.quick and args.labels:  # for profiler runs of the semantic mode's kernels
        g = time_device_resident(sf, ctx, label_frames(n), args.steps, args.warmup, 1, barrier, ndet=10, flush=flush)
        ctx.close()
        if rank == 0:
            print(json.dumps({"labels": round(args.steps / g["elapsed"], 3), "unit": "frames/s"}), flush=True)
        return

    # headline: CUDA graph, inputs in HBM
    global AUTOTUNE
    AUTOTUNE = not args.no_autotune
    g = time_device_resident(sf, ctx, frames, args.steps, args.warmup, 1, barrier,
                             rgb=1 if (args.quick and args.rgbd) else 0, flush=flush)
    elapsed = max_over_ranks(g["elapsed"])
    fps = job_fps(ws, args.steps, elapsed)
    out = {"metric": METRIC, "value": round(fps, 3), "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(1000.0 * elapsed / args.steps, 4), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 6x6 solve)",
           "data": "synthetic: " + WORKLOAD, "config": bench_config(),
           "gpu_launches": int(g["launches"]), "clocks": g["clocks"]}
    if g["autotune"]:
        out["autotune"] = g["autotune"]

    if args.quick:
        ctx.close()
        if rank == 0:
            print(json.dumps(out), flush=True)
        return
    # per-stage timing pass (eager device-driven form, same kernels, same frames)
    tp = time_device_resident(sf, ctx, frames, args.steps, args.warmup, 2, barrier, timing=True, flush=flush)
    sbytes, V = stage_bytes(tp["stats"])
    peak, peak_kind = load_peaks()
    l2_peak = l2_copy_peak()
    st_ms = dict(zip(STAGES, [round(float(x), 5) for x in tp["stage_ms"]]))
    kern = {}
    for name, b in sbytes.items():
        gbs = b / (st_ms[name] * 1e-3) / 1e9
        kern[name] = {"kernel": STAGE_KERNEL[name], "ms": st_ms[name], "algorithmic_bytes": int(b),
                      "achieved_gbs": round(gbs, 1), "frac_of_%s_hbm" % peak_kind: round(gbs / peak, 4)}
    dom = max(sbytes, key=lambda k: st_ms[k])  # the frame's dominant kernel
    out["stages_ms"] = st_ms
    out["frames"] = {"tracked": int(sum(st.tracked for st in tp["stats"])),
                     "lost": int(sum(st.state == -1 for st in tp["stats"])), "timed": len(tp["stats"]),
                     "note": "a lost frame (state -1, no relocalisation candidates) runs no ICP and no mapping"}
    out["kernels"] = kern
    out["visible_blocks_mean"] = round(float(V.mean()), 1)
    d = kern[dom]
    traffic = load_traffic(STAGE_KERNEL[dom], args.warmup, args.steps) if args.config == "c2" else None
    out["roofline"] = {"kernel": STAGE_KERNEL[dom], "bound": "hbm", "achieved": d["achieved_gbs"], "peak": peak,
                       "unit": "GB/s", "frac": d["frac_of_%s_hbm" % peak_kind], "peak_source": peak_kind,
                       "traffic": traffic, "algorithmic_bytes": d["algorithmic_bytes"],
                       "traffic_source": ("profiles/roofline_traffic_640x480.json: ncu dram bytes per launch, mean "
                                          "over the same frames %d..%d" % (args.warmup, n - 1)) if traffic else
                       "no ncu capture of these frames",
                       "l2": {"peak_gbs": round(l2_peak, 1), "frac": round(d["achieved_gbs"] / l2_peak, 4),
                              "peak_source": "measured live: L2-resident 24 MiB copies (read + write bytes)"}}

    if not args.no_plain:
        p = time_device_resident(sf, ctx, frames, args.steps, args.warmup, 0, barrier, flush=flush)
        out["plain"] = {"value": round(args.steps / p["elapsed"], 3),
                        "ms_per_step": round(1000.0 * p["elapsed"] / args.steps, 4),
                        "gpu_launches": int(p["launches"]), "frames": "the same frames as value"}
        out["graph_over_plain"] = round(out["value"] / out["plain"]["value"], 3)

    e2e_t, tracked = time_e2e(sf, ctx, frames, args.steps, args.warmup, 1, flush=flush)
    out["e2e"] = {"value": round(args.steps / e2e_t, 3), "unit": "frames/s",
                  "h2d_bytes_per_step": COLS * ROWS * (2 + 3),
                  "d2h_bytes_per_step": C.sizeof(sf._lib.FrameStats),
                  "tracked_frames": int(tracked)}
    if args.config == "c2" and not args.no_modes:
        # the reference's default tracking mode: ComputeSE3(icpOnly = false)
        r = time_device_resident(sf, ctx, frames, args.steps, args.warmup, 1, barrier, rgb=1, flush=flush)
        re2e, rtracked = time_e2e(sf, ctx, frames, args.steps, args.warmup, 1, rgb=1, flush=flush)
        rt = time_device_resident(sf, ctx, frames, args.steps, args.warmup, 2, barrier, timing=True, rgb=1,
                                  flush=flush)
        out["rgbd"] = {"value": round(args.steps / r["elapsed"], 3), "unit": "frames/s",
                       "stages_ms": dict(zip(STAGES, [round(float(x), 5) for x in rt["stage_ms"]])),
                       "e2e": round(args.steps / re2e, 3), "tracked_frames": int(rtracked),
                       "gpu_launches": int(r["launches"]),
                       "mode": "ComputeSE3 with icpOnly = false (the reference's default): RGBStep beside ICPStep "
                               "in every iteration, same frames"}
        if not args.no_plain:
            rp = time_device_resident(sf, ctx, frames, args.steps, args.warmup, 0, barrier, rgb=1, flush=flush)
            out["rgbd"]["plain"] = round(args.steps / rp["elapsed"], 3)
        # the semantic mode (System.cc:184-205): the same room with ten
        # labelled objects and 5% label flips, detections every frame
        lab = time_device_resident(sf, ctx, label_frames(n), args.steps, args.warmup, 1, barrier, ndet=10,
                                   flush=flush)
        out["labels"] = {"value": round(args.steps / lab["elapsed"], 3), "unit": "frames/s",
                         "gpu_launches": int(lab["launches"]),
                         "mode": "detections every frame (10 objects, 5% label flips): FuseColor, RayTrace, "
                                 "FuseColor with the labels (label pass + UnifyNeighbor), RayTrace"}
        out["mesh"] = time_mesh(sf, ctx, frames, args.steps + args.warmup)
    if not args.no_errors:
        out["errors"] = error_pass(sf, ctx, frames, args.steps, args.warmup)
    if args.config == "c2" and not args.no_modes:
        out["validate_pose"] = time_validate(sf, ctx, frames)
        out["reloc_score"] = time_reloc(sf, ctx, frames)
    if rank == 0 and not args.no_cpu:
        r = time_reference_cpu(frames, args.steps, args.warmup, budget_s=10.0)
        out["cpu_baseline"] = {"value": round(r["fps"], 4), "unit": "frames/s", "cores": r["cores"],
                               "kind": r["kind"],
                               "sample": "frames %d..%d after %d warm-up frames (bounded to ~10 s): %s"
                                         % (args.warmup, args.warmup + r["frames"] - 1, args.warmup, r["what"])}
    ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
