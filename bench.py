#!/usr/bin/env python
"""Benchmark of the GB300 Reconflow solver: 720p frame pairs per second.

Default workload ``720p-learned`` (the headline: batched + learned warm start
against the plain solver at equal endpoint error): 64 1280x720 float32 gray
frame pairs from the seeded synthetic scene generator (8 planes, depth 2-10
m, blob + 1/f texture, pose <= 2 deg / 0.1 m, N(0, 0.01) noise), lambda = 50,
theta = 0.33 (alpha_tv = 1/theta), tau = 0.25, with the reference demo's
projection weights (alpha_proj = 60, lambdaf = 0.1, lambdams = 100) and the
K-pyramid fix.  One step = the whole batch through the learned path:
plane-sweep features, the network, the warm-start state at pyramid level 2,
the refinement from there, the energies, and a plain re-solve of every pair
whose energy exceeds its plain solve's by more than 2%.  The line also
carries the plain solver's single-pair and batched throughput (6 levels,
5 warps x 100 iterations) and both solvers' endpoint errors on the same
pairs.  Workload ``720p`` is the plain drop-in solve of one pair.

``value``: pairs/s with the frames already in HBM (CUDA events on the solve
stream, L2 flushed between steps).  ``e2e``: the same through the C ABI with
host buffers: pinned upload of both frames, solve, download of flow, inverse
depth and 3D points, every step; for the learned workloads as a serving loop
whose copies overlap the previous / next step's solve (pipelined transfers
of the batch API), with the blocking per-step figure beside it
(``serial_value``).  ``roofline``: the dominant kernel at level
0, timed live with CUDA events on its stream.  ``cpu_baseline``: the oracle's
FP32 reference-semantics path on this host's cores, on a bounded sample.

``--impl reference`` times the reference semantics of the plain solve of one
pair of the workload's size on the host CPU (the FP32 oracle; the reference
itself cannot be built: it needs OpenCV and the texture reference API that
CUDA 12 removed, and it has no batched or learned path).  Several GPUs run
independent replicas.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # 1280x720, 6 levels, 5 warps, 100 iterations: the headline workload
    "720p": dict(width=1280, height=720, levels=6, warps=5, iters=100, seed=0),
    # 640x480, 5 levels, 3 warps, 50 iterations
    "480p": dict(width=640, height=480, levels=5, warps=3, iters=50, seed=0),
    # profiling case: the 720p pair at its finest level only, 1 warp, 4 iterations
    # (a dozen launches, so a profiler capture ends in seconds)
    "720p-l0": dict(width=1280, height=720, levels=1, warps=1, iters=4, seed=0),
    # batched: 64 pairs of sizes drawn uniformly from four resolutions, independent
    # seeded scenes and poses, one launch per schedule step for all pairs
    "batch64": dict(pairs=64, sizes=[(320, 240), (640, 480), (1280, 720), (1920, 1080)],
                    levels=6, warps=5, iters=100, seed=0),
    # batched + learned warm start: 64 pairs of 1280x720; the network predicts
    # inverse depth at 1/8, the solve refines from pyramid level 2 with the
    # per-level schedule below (index = level, 0 = finest: 1 x 4, 1 x 40,
    # 1 x 50); plain 5 x 100
    "720p-learned": dict(width=1280, height=720, pairs=64, levels=6, seed=2000, plain_warps=5,
                         plain_iters=100, warm_level=1, warm_warps=[1, 1],
                         warm_iters=[3, 50], fallback_margin=0.02,
                         checkpoint="reconflow_gb300/weights/warmstart_f125.bin",
                         tiles="reconflow_gb300/tuning/gb300_720p_x64.json"),
    # batched + learned on mixed sizes (the 4K / 1080p stream at a reduced
    # count: 16 pairs of 3840x2160 and 16 of 1920x1080, independent scenes);
    # 4K starts the refinement at pyramid level 3 (its network grid is 1/32)
    "mixed-4k-1080p-learned": dict(
        levels=6, plain_warps=5, plain_iters=100, fallback_margin=0.02,
        checkpoint="reconflow_gb300/weights/warmstart_f125.bin",
        groups=[dict(width=3840, height=2160, pairs=16, seed=6000, warm_level=3,
                     warm_warps=[1, 1, 1, 1], warm_iters=[4, 30, 60, 80]),
                dict(width=1920, height=1080, pairs=16, seed=6500, warm_level=2,
                     warm_warps=[1, 1, 1], warm_iters=[4, 60, 80])]),
    # batched: 64 pairs of 1280x720 (per-pair throughput of the batched path)
    "batch64-720p": dict(pairs=64, sizes=[(1280, 720)], levels=6, warps=5, iters=100, seed=0),
    # profiling case of the batched kernels: 4 pairs of 1280x720 at their finest
    # level only, 1 warp, 4 iterations, the 64-pair tile table (a dozen launches;
    # 3.7 M pixels per launch, above the L2 size)
    "720p-x4-l0": dict(pairs=4, sizes=[(1280, 720)], levels=1, warps=1, iters=4, seed=2000,
                       tiles="reconflow_gb300/tuning/gb300_720p_x64.json"),
    # pose front end (CameraPose): 64 pairs of 1280x720, features, matching,
    # LMedS and pose recovery per pair, 8 handles on 8 host threads / streams;
    # Hessian threshold 20 for the generator's texture (the reference's 2000
    # is for camera images)
    "pose-720p": dict(width=1280, height=720, pairs=64, seed=2000, threads=8, threshold=20.0,
                      pose=True),
    # the C5 stream: 8 seeded moving-camera sequences of 33 frames (0.05 m per
    # frame), 4 at 3840x2160 and 4 at 1920x1080: 256 consecutive pairs, solved
    # in 32 waves of one pair per sequence.  Wave 0 starts from the network;
    # every later wave starts from the previous wave's solved depth carried
    # into the new frame (rf_ws_propagate); a pair whose energy fails the
    # fallback test is solved again with the full plain schedule.
    "c5-stream": dict(
        levels=6, plain_warps=5, plain_iters=100, frames=33, fallback_margin=0.02,
        checkpoint="reconflow_gb300/weights/warmstart_f125.bin",
        groups=[dict(width=3840, height=2160, sequences=4, seed=7000, warm_level=3,
                     warm_warps=[1, 1, 1, 1], warm_iters=[4, 30, 60, 80],
                     temporal_warps=[1, 1, 1, 1], temporal_iters=[4, 30, 60, 80]),
                dict(width=1920, height=1080, sequences=4, seed=7500, warm_level=2,
                     warm_warps=[1, 1, 1], warm_iters=[4, 60, 80],
                     temporal_warps=[1, 1, 1], temporal_iters=[4, 60, 80])]),
    # the warm-start network alone: one forward pass over the 1/8-grid inputs
    # of 64 720p pairs (64 x 90 x 160 x 16), the committed checkpoint
    "warmstart-net-720p": dict(pairs=64, height=90, width=160,
                               checkpoint="reconflow_gb300/weights/warmstart_f125.bin", net=True),
}
SOLVER = dict(method=14, lam=50.0, theta=0.33, tau=0.25, alpha_proj=60.0, lambdaf=0.1,
              lambdams=100.0, fix_quirks=1)
# algorithmic bytes per pixel per launch of the two inner-iteration kernels:
# A reads u,v,duhat(2),p(4),uproj(2),sk(2),Ix,Iy,Iz,X,Y,Z = 18 floats, writes
# duhat(2),uproj(2),X1,Y1,Z1 = 7; B reads duhat(2),p(4),X1(3),sk(2),u,v,uproj(2)
# = 15, writes p(4),X,Y,Z,sk(2) = 9.
ALG_BYTES = {"recon_a": 25 * 4, "recon_b": 24 * 4}
# compulsory bytes of one inner iteration per pixel (both kernels together)
ITER_BYTES = 31 * 4
L2_FLUSH_BYTES = 512 << 20
E2E_MODE = ("pipelined: the frames of step k+1 go up and the results of step k come down on "
            "copy streams while step k solves (rf_batch_stage_upload / "
            "rf_batch_stage_download, pinned host memory); every step's copies lie inside the "
            "timed wall time; serial_value: blocking upload_all + step + download_all per step")
E2E_MODE_LAGGED = (
    "pipelined serving loop with the fallback test one step behind: step k+1's frames are taken "
    "and its solve and energies (rf_batch_energies_async) queued, after step k's results were "
    "staged for download, before the host reads step k's energies; a pair that falls back is "
    "solved again by the plain solver from its pinned host frames and its results downloaded; "
    "frames go up and results come down on copy streams (rf_batch_stage_upload / "
    "rf_batch_stage_download, pinned host memory); every step's copies, the L2 flush and the "
    "fallback test lie inside the timed wall time; in_step_fallback_value: the loop with the "
    "test inside each step (the host waits for each step's energies before queueing the next); "
    "serial_value: blocking upload_all + step + download_all per step; value and "
    "in_step_fallback_value: the median of three timed runs of `steps` steps each (all three in "
    "*_runs), because the host link is shared with the other GPUs' jobs on the machine")
E2E_RUNS = 3
LEARNED_METRIC = ("720p frame pairs/s, batched + learned warm start (vs the plain solver at "
                  "equal EPE)")
PLAIN_METRIC = "720p frame pairs/s (ReconFlow flow + depth)"


# tile table of the single-pair (drop-in) solver at 1280x720 on GB300
SINGLE_TILES = "reconflow_gb300/tuning/gb300_720p_single.json"


def load_tiles(rel):
    """A committed autotuner table (reconflow_gb300/autotune.py), or None."""
    if not rel:
        return None
    path = os.path.join(ROOT, rel)
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        return json.load(fh)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def serve_pipelined(items, step, steps, flush=None):
    """`steps` solves as a serving loop through the batch API's pipelined
    transfers: batch k+1's frames go up (rf_batch_stage_upload) and batch
    k's results come down (rf_batch_stage_download) on their own copy
    streams while a solve runs; every step's upload and download lie inside
    the returned wall time.  items: [(batch, host pointer columns [I0, I1,
    u, v, inverse depth, X, Y, Z], pitch)]."""
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for b, c, p in items:
        b.stageUpload(c[0], c[1], p)
    for k in range(steps):
        for b, c, p in items:
            b.takeUpload()
            if k + 1 < steps:
                b.stageUpload(c[0], c[1], p)
        if flush is not None:
            flush.zero_()
        step()
        for b, c, p in items:
            b.stageDownload(p, u=c[2], v=c[3], inv_depth=c[4], X=c[5], Y=c[6], Z=c[7])
    for b, _, _ in items:
        b.waitDownload()
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def serve_learned_lagged(b, ls, f, stream, scenes, size, n, col, s0, flush, steps, test,
                         fell_back):
    """The learned serving loop with the fallback test one step behind.
    Step k+1 is queued (frames taken from staging, the learned solve, the
    energies into pinned memory, the results staged for download) before the
    host reads step k's energies, so the GPU has the next step while the host
    tests this one.  A pair that falls back is solved again by the plain
    single-pair solver `f` from its pinned host frames, and its results are
    downloaded (a deployment rotating its output arrays writes them into step
    k's).  Returns the wall time of `steps` steps."""
    import torch

    import reconflow_gb300 as R

    mode, ceil, margin, e_plain = test
    W, H = size
    Ks = [sc["K"] for sc in scenes]
    Rs = [sc["R"] for sc in scenes]
    ts = [sc["t"] for sc in scenes]
    lib = R.load()
    pinned = []
    e_np = []
    for _ in range(2):
        p_ = ctypes.c_void_p()
        R._native.check(lib.rf_host_alloc(8 * n, ctypes.byref(p_)))
        pinned.append(p_)
        e_np.append(np.ctypeslib.as_array(ctypes.cast(p_, ctypes.POINTER(ctypes.c_double)),
                                          shape=(n,)))
    evs = [torch.cuda.Event(), torch.cuda.Event()]

    def view(ptr):
        return np.ctypeslib.as_array(ctypes.cast(ctypes.c_void_p(ptr),
                                                 ctypes.POINTER(ctypes.c_float)), shape=(H, s0))

    def queue(k):
        b.takeUpload()
        if k + 1 < steps:
            b.stageUpload(col[0], col[1], s0)
        with torch.cuda.stream(stream):
            flush.zero_()
        ls.solve(Ks, Rs, ts)
        b.energiesAsync(pinned[k % 2].value)
        evs[k % 2].record(stream)
        b.stageDownload(s0, u=col[2], v=col[3], inv_depth=col[4], X=col[5], Y=col[6], Z=col[7])

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.stageUpload(col[0], col[1], s0)
    queue(0)
    for k in range(steps):
        if k + 1 < steps:
            queue(k + 1)
        evs[k % 2].synchronize()
        e = e_np[k % 2]
        bad = [i for i in range(n) if fallback_test(mode, e[i], e_plain[i], W * H, ceil, margin)]
        for i in bad:
            f.setCameraMatrices(Ks[i], Ks[i])
            f.copyImagesToDevice(view(col[0][i]), view(col[1][i]))
            f.solveR(Rs[i], ts[i], 5.0)
            f.copyOpticalFlowToHost()
            f.copy3dToHost()
            f.copyInverseDepthToHost()
        fell_back.append(len(bad))
    b.waitDownload()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    for p_ in pinned:
        lib.rf_host_free(p_)
    return wall


def make_inputs(wl):
    from reconflow_gb300.scene import make_scene

    sc = make_scene(wl["width"], wl["height"], seed=wl["seed"])
    s = (wl["width"] + 31) // 32 * 32
    pad = lambda a: np.pad(a, ((0, 0), (0, s - a.shape[1]))).astype(np.float32)  # noqa: E731
    return sc, pad(sc["I0"]), pad(sc["I1"]), s


def cpu_sample(wl, sc, I0, I1, threads=None):
    """FP32 reference-semantics oracle on this host: ``run(iters)`` times one
    plain solve of the pair with the workload's levels and warps and `iters`
    inner iterations."""
    from oracle import oracle as O

    O.build()
    if threads:
        O.set_num_threads(threads)

    def run(iters):
        p = O.make_params(wl["width"], wl["height"], wl["levels"], method=SOLVER["method"],
                          lam=SOLVER["lam"], lambdaf=SOLVER["lambdaf"],
                          lambdams=SOLVER["lambdams"], alpha_tv=1.0 / SOLVER["theta"],
                          alpha_proj=SOLVER["alpha_proj"], tau=SOLVER["tau"],
                          n_warp_iters=wl["warps"], n_solver_iters=iters,
                          fix_quirks=SOLVER["fix_quirks"])
        t0 = time.perf_counter()
        O.solve(p, I0, I1, K0=sc["K"], K1=sc["K"], R1=sc["R"], t1=sc["t"], dtype=np.float32)
        return time.perf_counter() - t0

    return run, O.num_threads()


def run_reference(args, wl, world, rank):
    """The reference semantics on the host CPU: every timed step is one full
    plain solve of one pair of the workload's size (all levels, warps and
    inner iterations), timed on its own; the warm-up steps are the same
    solve at one inner iteration (they only page the buffers in and start
    the thread pool)."""
    if rank != 0:
        return
    sc, I0, I1, s = make_inputs(wl)
    run, cores = cpu_sample(wl, sc, I0, I1)
    for _ in range(args.warmup):
        run(1)
    per_pair = [run(wl["iters"]) for _ in range(args.steps)]
    total = sum(per_pair)
    value = args.steps / total
    sample = (f"one {wl['width']}x{wl['height']} pair per step, the full {wl['levels']}-level x "
              f"{wl['warps']}-warp x {wl['iters']}-iteration plain schedule, measured "
              f"(median {statistics.median(per_pair):.2f} s per pair on {cores} threads); "
              f"warm-up steps at 1 inner iteration")
    cfg = config_of(wl)
    cfg["l2"] = "not applicable (host CPU)"
    if "workload" in wl:
        cfg["workload"] = wl["workload"]
        cfg["reference_path"] = ("the plain solve of one pair: the reference has no batched "
                                 "or learned path, so this arm times its counterpart")
    line = {
        "impl": "reference", "metric": wl.get("metric", PLAIN_METRIC),
        "value": value, "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generator)", "config": cfg,
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_pose(args, wl, world, rank):
    """Reference arm of the pose workload: the oracle's feature stages and
    the host LMedS / pose recovery (the reference's own CameraPose needs
    OpenCV with CUDA), one pair per step, on the workload's pairs."""
    if rank != 0:
        return
    from reconflow_gb300.scene import make_scene

    n = max(1, args.steps)
    scenes = [make_scene(wl["width"], wl["height"], seed=wl["seed"] + i) for i in range(n)]
    pose_cpu_sample(scenes[:1], wl["threshold"])  # warm-up (builds the oracle)
    t0 = time.perf_counter()
    cpu = pose_cpu_sample(scenes, wl["threshold"])
    total = time.perf_counter() - t0
    value = n / total
    cpu["value"] = value
    line = {
        "impl": "reference", "metric": POSE_METRIC, "value": value, "unit": "pairs/s",
        "n_gpus": args.gpus, "steps": n, "warmup": args.warmup, "ms_per_step": 1000.0 * total / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (features), f64 (geometry)", "data": "synthetic (seeded scene generator)",
        "config": {"workload": args.workload, "width": wl["width"], "height": wl["height"],
                   "pairs_per_step": 1, "hessian_threshold": wl["threshold"],
                   "parallelism": "replicas"},
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batch_sizes(wl):
    rng = np.random.default_rng(wl["seed"])
    idx = rng.integers(0, len(wl["sizes"]), wl["pairs"])
    return [wl["sizes"][i] for i in idx]


def run_batch(args, wl, world, rank, local):
    """Batched workloads: one step = one batched solve of all pairs."""
    import torch

    import reconflow_gb300 as R
    from reconflow_gb300.scene import make_scene

    torch.cuda.set_device(local)
    lib = R.load()
    sizes = batch_sizes(wl)
    t0 = time.perf_counter()
    scenes = [make_scene(w, h, seed=wl["seed"] + 1000 * rank + i, device="cuda")
              for i, (w, h) in enumerate(sizes)]
    gen_s = time.perf_counter() - t0
    b = R.ReconFlowBatch(sizes, wl["levels"], method=SOLVER["method"], lambda_=SOLVER["lam"],
                         lambdaf=SOLVER["lambdaf"], lambdams=SOLVER["lambdams"],
                         alphaTv=1.0 / SOLVER["theta"], alphaProj=SOLVER["alpha_proj"],
                         tau=SOLVER["tau"], nWarpIters=wl["warps"], nSolverIters=wl["iters"],
                         fix_quirks=SOLVER["fix_quirks"])
    stream = torch.cuda.Stream()
    b.setStream(stream.cuda_stream)
    padded = []
    for i, sc in enumerate(scenes):
        s_ = b.strides[i]
        I0 = np.pad(sc["I0"], ((0, 0), (0, s_ - sc["I0"].shape[1]))).astype(np.float32)
        I1 = np.pad(sc["I1"], ((0, 0), (0, s_ - sc["I1"].shape[1]))).astype(np.float32)
        padded.append((I0, I1))
        b.setCameraMatrices(i, sc["K"], sc["K"])
        b.copyImagesToDevice(i, I0, I1)
    tiles = load_tiles(wl.get("tiles"))
    if tiles is not None:
        from reconflow_gb300 import autotune

        autotune.apply(b, tiles["levels"])
    Rs = [sc["R"] for sc in scenes]
    ts = [sc["t"] for sc in scenes]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            b.solveR(Rs, ts)
        torch.cuda.synchronize()
        barrier(world)
        l0 = b.kernelLaunches()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            for a, e in evs:
                flush.zero_()
                a.record(stream)
                b.solveR(Rs, ts)
                e.record(stream)
            torch.cuda.synchronize()
        launches = b.kernelLaunches() - l0
        step_ms = [a.elapsed_time(e) for a, e in evs]
    total_s = max_over_ranks(sum(step_ms) / 1000.0, world)
    npairs = wl["pairs"]
    value = world * npairs * args.steps / total_s
    if args.solve_only:
        if rank == 0:
            print(json.dumps({"metric": "frame pairs/s, batched ReconFlow solve", "value": value,
                              "unit": "pairs/s", "note": "solve-only run"}), flush=True)
        b.close()
        return
    # accuracy over the batch
    epes = []
    for i, sc in enumerate(scenes):
        w, h = sizes[i]
        u, v = b.copyOpticalFlowToHost(i)
        e = np.sqrt((u[:, :w] - sc["flow"][..., 0]) ** 2 + (v[:, :w] - sc["flow"][..., 1]) ** 2)
        e = e[sc["valid"]]
        epes.append(float(np.median(np.where(np.isfinite(e), e, np.float32(1e4)))))
    e2e = None
    if not args.no_e2e:
        nb = [sizes[i][1] * b.strides[i] * 4 for i in range(npairs)]
        hosts = []
        for i in range(npairs):
            ptrs = []
            for _ in range(8):
                p_ = ctypes.c_void_p()
                R._native.check(lib.rf_host_alloc(nb[i], ctypes.byref(p_)))
                ptrs.append(p_)
            h_ = sizes[i][1]
            a0 = np.ctypeslib.as_array(ctypes.cast(ptrs[0], ctypes.POINTER(ctypes.c_float)),
                                       shape=(h_, b.strides[i]))
            a1 = np.ctypeslib.as_array(ctypes.cast(ptrs[1], ctypes.POINTER(ctypes.c_float)),
                                       shape=(h_, b.strides[i]))
            a0[:] = padded[i][0]
            a1[:] = padded[i][1]
            hosts.append(ptrs)
        hb = b._h
        uniform = len(set(b.strides)) == 1
        col = [[hosts[i][k].value for i in range(npairs)] for k in range(8)]

        def step():
            if uniform:  # one pitch: whole-batch transfers, one sync each way
                b.uploadAll(col[0], col[1], b.strides[0])
                b.solveR(Rs, ts)
                b.downloadAll(b.strides[0], u=col[2], v=col[3], inv_depth=col[4], X=col[5],
                              Y=col[6], Z=col[7])
                return
            for i in range(npairs):
                R._native.check(lib.rf_batch_upload_images(hb, i, hosts[i][0], hosts[i][1],
                                                           b.strides[i]))
            b.solveR(Rs, ts)
            for i in range(npairs):
                s_ = b.strides[i]
                R._native.check(lib.rf_batch_download_flow(hb, i, hosts[i][2], hosts[i][3], s_))
                R._native.check(lib.rf_batch_download_inv_depth(hb, i, hosts[i][4], s_))
                R._native.check(lib.rf_batch_download_points(hb, i, hosts[i][5], hosts[i][6],
                                                             hosts[i][7], s_))

        step()
        times = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            step()
            times.append(time.perf_counter() - t1)
        e2e = {"value": world * npairs * args.steps / max_over_ranks(sum(times), world),
               "unit": "pairs/s",
               "h2d_bytes_per_step": sum(2 * w * h * 4 for w, h in sizes),
               "d2h_bytes_per_step": sum(6 * w * h * 4 for w, h in sizes)}
        for ptrs in hosts:
            for p_ in ptrs:
                lib.rf_host_free(p_)
    if rank == 0:
        counts = {}
        for w, h in sizes:
            counts[f"{w}x{h}"] = counts.get(f"{w}x{h}", 0) + 1
        print(json.dumps({
            "metric": "frame pairs/s, batched ReconFlow solve", "value": value, "unit": "pairs/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene generator)",
            "config": {"workload": args.workload, "pairs_per_step": npairs, "sizes": counts,
                       "pyramid_levels": wl["levels"], "warps": wl["warps"],
                       "iters": wl["iters"], "l2": "flushed between steps",
                       "parallelism": "replicas"},
            "e2e": e2e, "clocks": clk.summary(), "gpu_launches": int(launches),
            "accuracy": {"epe_median_px_mean_over_pairs": float(np.mean(epes)),
                         "note": "non-finite flow counts as 1e4 px"},
            "scene_gen_s": gen_s,
        }), flush=True)
    b.close()


def run_learned(args, wl, world, rank, local):
    """Batched + learned warm start against the plain solver, on 720p pairs.

    Untimed: the plain batched solve of the same pairs (its endpoint errors
    and energies) and the plain single-pair solve of one pair (the drop-in
    path's throughput).  Timed, one step = the whole batch through the
    learned path: input features, network, warm-start state, refinement
    from the warm level, energies, and a plain re-solve of every pair whose
    energy exceeds its plain solve's by more than the fallback margin."""
    import torch

    import reconflow_gb300 as R
    from reconflow_gb300.scene import make_scene
    from reconflow_gb300.warmstart import LearnedBatchSolver, WarmStartNet

    torch.cuda.set_device(local)
    lib = R.load()
    W, H, n = wl["width"], wl["height"], args.pairs or wl["pairs"]
    t0 = time.perf_counter()
    scenes = [make_scene(W, H, seed=wl["seed"] + 1000 * rank + i, device="cuda") for i in range(n)]
    gen_s = time.perf_counter() - t0
    Ks = [sc["K"] for sc in scenes]
    Rs = [sc["R"] for sc in scenes]
    ts = [sc["t"] for sc in scenes]
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    from reconflow_gb300 import autotune

    tiles = load_tiles(wl.get("tiles"))

    def new_batch(warps, iters):
        b = R.ReconFlowBatch([(W, H)] * n, wl["levels"], method=SOLVER["method"],
                             lambda_=SOLVER["lam"], lambdaf=SOLVER["lambdaf"],
                             lambdams=SOLVER["lambdams"], alphaTv=1.0 / SOLVER["theta"],
                             alphaProj=SOLVER["alpha_proj"], tau=SOLVER["tau"], nWarpIters=warps,
                             nSolverIters=iters, fix_quirks=SOLVER["fix_quirks"])
        b.setStream(stream.cuda_stream)
        for i, sc in enumerate(scenes):
            b.setCameraMatrices(i, sc["K"], sc["K"])
            b.copyImagesToDevice(i, sc["I0"], sc["I1"])
        if tiles is not None:
            autotune.apply(b, tiles["levels"])
        return b

    def epe_stats(b):
        means, meds, allv = [], [], []
        for i, sc in enumerate(scenes):
            u, v = b.copyOpticalFlowToHost(i)
            e = np.sqrt((u[:, :W] - sc["flow"][..., 0]) ** 2 + (v[:, :W] - sc["flow"][..., 1]) ** 2)
            e = e[sc["valid"]]
            e = np.where(np.isfinite(e), e, np.float32(1e4))
            means.append(float(e.mean()))
            meds.append(float(np.median(e)))
            allv.append(e)
        a = np.concatenate(allv)
        return {"epe_mean_px": float(np.mean(means)), "epe_median_px": float(np.mean(meds)),
                "frac_epe_gt_3px": float((a > 3).mean())}

    def timed(fn, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        for a, e in evs:
            flush.zero_()
            a.record(stream)
            fn()
            e.record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(e) for a, e in evs]

    # plain, batched: reference accuracy and energies (a solve-only run, for
    # profiler launch lists, skips it and so never falls back)
    if args.solve_only:
        e_plain = np.full(n, np.inf)
    else:
        plain = new_batch(wl["plain_warps"], wl["plain_iters"])
        with torch.cuda.stream(stream):
            plain.solveR(Rs, ts)
            torch.cuda.synchronize()
            plain_acc = epe_stats(plain)
            e_plain = plain.energies()
            plain_batch_ms = timed(lambda: plain.solveR(Rs, ts), 2)
        plain.close()
    # plain, one pair through the drop-in path
    f = R.ReconFlow()
    f.initializeR(W, H, 1, wl["levels"], 2.0, SOLVER["method"], SOLVER["lam"], 0.0,
                  SOLVER["lambdaf"], SOLVER["lambdams"], 1.0 / SOLVER["theta"],
                  SOLVER["alpha_proj"], 0.5, SOLVER["tau"], wl["plain_warps"], wl["plain_iters"],
                  cvType=5, fix_quirks=SOLVER["fix_quirks"])
    f.setStream(stream.cuda_stream)
    single_tiles = load_tiles(SINGLE_TILES)
    if single_tiles is not None:
        autotune.apply_single(f, single_tiles["levels"], wl["levels"])
        autotune.apply_iterations_per_launch(lib, single_tiles)
    f.setCameraMatrices(scenes[0]["K"], scenes[0]["K"])
    f.copyImagesToDevice(scenes[0]["I0"], scenes[0]["I1"])
    if not args.solve_only:
        with torch.cuda.stream(stream):
            for _ in range(2):
                f.solveR(Rs[0], ts[0], 5.0)
            single_ms = timed(lambda: f.solveR(Rs[0], ts[0], 5.0), 5)

    # learned
    net = WarmStartNet(n, (H // 8) + 1, (W // 8) + 1, seed=0)
    net.load(os.path.join(ROOT, wl["checkpoint"]))
    b = new_batch(wl["plain_warps"], wl["plain_iters"])
    ls = LearnedBatchSolver(net, b, (W, H), Ks[0], warm_level=wl["warm_level"],
                            warps=wl["warm_warps"], iters=wl["warm_iters"])
    ls.set_stream(stream.cuda_stream)
    margin = wl["fallback_margin"]
    fallbacks = []
    mode, ceil = fallback_setup(args, W, H, "network")

    def step():
        ls.solve(Ks, Rs, ts)
        e = b.energies()
        bad = [i for i in range(n) if fallback_test(mode, e[i], e_plain[i], W * H, ceil, margin)]
        for i in bad:  # fall back to the plain solve, one pair at a time
            f.setCameraMatrices(Ks[i], Ks[i])
            f.copyImagesToDeviceFromDevice(*b.imagePlanes(i, 0), b.strides[i])
            f.solveR(Rs[i], ts[i], 5.0)
            b.importResults(i, f.deviceResults(), f.stride)  # the accepted solution
        fallbacks.append(len(bad))

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if not args.solve_only:
            learned_acc = epe_stats(b)
            e_learned = b.energies()
        barrier(world)
        l0 = b.kernelLaunches() + net.kernel_launches() + f.kernelLaunches()
        fallbacks.clear()
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            step_ms = timed(step, args.steps)
        launches = b.kernelLaunches() + net.kernel_launches() + f.kernelLaunches() - l0
    # the network's tensor-core launches flag a bounded wait that gave up
    try:
        tc_gave_up = net.wait_gave_up()
    except Exception as exc:  # report a failed read instead of hiding it
        tc_gave_up = f"status read failed: {exc}"
    if tc_gave_up is not False:
        print(f"bench.py: tensor-core wait status: {tc_gave_up}", file=sys.stderr)
    timed_fallbacks = list(fallbacks)
    total_s = max_over_ranks(sum(step_ms) / 1000.0, world)
    value = world * n * args.steps / total_s
    if args.solve_only:
        if rank == 0:
            print(json.dumps({"metric": LEARNED_METRIC, "value": value, "unit": "pairs/s",
                              "pairs_per_step": n, "note": "solve-only run (no plain reference "
                              "solve, no fallbacks)"}), flush=True)
        return

    # end to end: frames from pinned host memory in, flow / inverse depth /
    # points out, every step
    e2e = None
    if not args.no_e2e:
        s0 = b.strides[0]
        nb = H * s0 * 4
        hosts = []
        for i in range(n):
            ptrs = []
            for _ in range(8):
                p_ = ctypes.c_void_p()
                R._native.check(lib.rf_host_alloc(nb, ctypes.byref(p_)))
                ptrs.append(p_)
            for k, img in ((0, scenes[i]["I0"]), (1, scenes[i]["I1"])):
                a_ = np.ctypeslib.as_array(ctypes.cast(ptrs[k], ctypes.POINTER(ctypes.c_float)),
                                           shape=(H, s0))
                a_[:, :W] = img
            hosts.append(ptrs)
        col = [[hosts[i][k].value for i in range(n)] for k in range(8)]

        def e2e_step():
            b.uploadAll(col[0], col[1], s0)  # rf_batch_upload_all
            step()
            b.downloadAll(s0, u=col[2], v=col[3], inv_depth=col[4], X=col[5], Y=col[6],
                          Z=col[7])  # rf_batch_download_all

        with torch.cuda.stream(stream):
            e2e_step()
            times = []
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                e2e_step()
                torch.cuda.synchronize()
                times.append(time.perf_counter() - t1)
            piped_runs = [serve_pipelined([(b, col, s0)], step, args.steps, flush)
                          for _ in range(E2E_RUNS)]
            lag_fb = []
            serve_learned_lagged(b, ls, f, stream, scenes, (W, H), n, col, s0, flush, 2,
                                 (mode, ceil, margin, e_plain), lag_fb)
            lag_fb.clear()
            lagged_runs = []
            for _ in range(E2E_RUNS):
                run_fb = []
                lagged_runs.append(serve_learned_lagged(
                    b, ls, f, stream, scenes, (W, H), n, col, s0, flush, args.steps,
                    (mode, ceil, margin, e_plain), run_fb))
                lag_fb.extend(run_fb)

        def rate(t):  # pairs/s of `args.steps` steps in t seconds, slowest rank
            return world * n * args.steps / max_over_ranks(t, world)

        lag_values = [rate(t) for t in lagged_runs]
        piped_values = [rate(t) for t in piped_runs]
        e2e = {"value": float(np.median(lag_values)),
               "unit": "pairs/s", "h2d_bytes_per_step": 2 * n * W * H * 4,
               "d2h_bytes_per_step": 6 * n * W * H * 4, "mode": E2E_MODE_LAGGED,
               "value_runs": lag_values,
               "fallbacks_per_step": lag_fb,
               "in_step_fallback_value": float(np.median(piped_values)),
               "in_step_fallback_runs": piped_values,
               "serial_value": rate(sum(times))}
        for ptrs in hosts:
            for p_ in ptrs:
                lib.rf_host_free(p_)

    # roofline: the dominant kernel of the step, the batched level-0 data /
    # triangulation kernel over all pairs (rf_batch_profile_level); the
    # single-pair kernels of the drop-in path beside it
    with torch.cuda.stream(stream):
        ms_b = b.profileLevel(0, 20)
    roofline = roofline_of(ms_b, W * H * n, batched=True)
    ms = (ctypes.c_float * 2)()
    with torch.cuda.stream(stream):
        f.setCameraMatrices(Ks[0], Ks[0])
        f.copyImagesToDevice(scenes[0]["I0"], scenes[0]["I1"])
        f.solveR(Rs[0], ts[0], 5.0)
        R._native.check(lib.rf_profile_iterations(f._handle(), 0, 50, ms))
    roofline["single_pair"] = roofline_of(ms, W * H)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        wl1 = dict(width=W, height=H, levels=wl["levels"], warps=wl["plain_warps"],
                   iters=wl["plain_iters"], seed=wl["seed"])
        sc0 = scenes[0]
        s_ = (W + 31) // 32 * 32
        pad = lambda a: np.pad(a, ((0, 0), (0, s_ - W))).astype(np.float32)  # noqa: E731
        run, cores = cpu_sample(wl1, sc0, pad(sc0["I0"]), pad(sc0["I1"]))
        run(1)
        per_pair = run(wl["plain_iters"])
        cpu = {"value": 1.0 / per_pair, "unit": "pairs/s", "cores": cores, "kind": "port",
               "sample": f"one plain solve of one {W}x{H} pair, the full {wl['levels']}-level x "
                         f"{wl['plain_warps']}-warp x {wl['plain_iters']}-iteration schedule, "
                         f"measured ({per_pair:.2f} s)"}
    if rank == 0:
        single_pps = 1000.0 / statistics.median(single_ms)
        tol = 0.05
        line = {
            "metric": LEARNED_METRIC,
            "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene generator)",
            "config": {"workload": args.workload, "width": W, "height": H, "pairs_per_step": n,
                       "pyramid_levels": wl["levels"], "plain_schedule": [wl["plain_warps"],
                                                                          wl["plain_iters"]],
                       "warm_level": wl["warm_level"], "warm_warps_per_level": wl["warm_warps"],
                       "warm_iters_per_level": wl["warm_iters"],
                       "fallback": fallback_desc(mode, ceil, margin),
                       "checkpoint": wl["checkpoint"],
                       "tiles": wl.get("tiles") if tiles is not None else "default 32x8",
                       "single_pair_tiles": SINGLE_TILES if single_tiles is not None
                       else "default 32x8",
                       "method": "METHODR_TVL1_MS",
                       "lambda": SOLVER["lam"], "theta": SOLVER["theta"], "tau": SOLVER["tau"],
                       "alpha_proj": SOLVER["alpha_proj"], "lambdaf": SOLVER["lambdaf"],
                       "lambdams": SOLVER["lambdams"], "fix_quirks": SOLVER["fix_quirks"],
                       "scene_seeds": [wl["seed"], wl["seed"] + n - 1],
                       "l2": "flushed between steps (512 MiB write)", "parallelism": "replicas"},
            "plain": {"single_pair_pairs_per_s": single_pps,
                      "batched_pairs_per_s": 1000.0 * n / statistics.median(plain_batch_ms),
                      "accuracy": plain_acc},
            "learned": {"accuracy": learned_acc, "fallbacks_per_step": timed_fallbacks,
                        "tc_wait_gave_up": tc_gave_up,
                        "energy_ratio_median": float(np.median(e_learned / e_plain)),
                        "energy_per_px_max": float(np.max(e_learned) / (W * H)),
                        "plain_energy_test_flags": int(sum(
                            over_margin(a, c, margin) for a, c in zip(e_learned, e_plain)))},
            "speedup_vs_plain_single_pair": value / single_pps,
            "equal_epe": {"mean": learned_acc["epe_mean_px"] <= plain_acc["epe_mean_px"] + tol,
                          "median": learned_acc["epe_median_px"] <= plain_acc["epe_median_px"] + tol,
                          "tolerance_px": tol},
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary(),
            "gpu_launches": int(launches), "scene_gen_s": gen_s,
        }
        print(json.dumps(line), flush=True)
    b.close()
    f.close()
    net.close()


POSE_METRIC = "720p pose estimates/s (CameraPose: features, matching, LMedS, pose recovery)"
NET_METRIC = "720p pairs/s through the warm-start network's forward pass (64 per pass)"

# (cin, cout, stride) of the network's six convolutions; 3 and 4 run at half
# resolution, 5 takes the upsampled 96 channels concatenated with layer 1's 32
NET_LAYERS = [(16, 32, 1, 1), (32, 96, 2, 2), (96, 96, 1, 2), (96, 8, 1, 2), (128, 64, 1, 1),
              (64, 8, 1, 1)]


def run_net(args, wl, world, rank, local):
    """The warm-start network's forward pass (six tcgen05 implicit-GEMM
    convolutions, BF16 operands, FP32 accumulation) on seeded inputs of the
    learned workload's shape; roofline against the measured BF16 GEMM peak."""
    import torch

    from reconflow_gb300.warmstart import WarmStartNet

    torch.cuda.set_device(local)
    B, H, W = wl["pairs"], wl["height"], wl["width"]
    net = WarmStartNet(B, H + 1, W + 1, seed=0)
    net.load(os.path.join(ROOT, wl["checkpoint"]))
    stream = torch.cuda.Stream()
    net.set_stream(stream.cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(1000 + rank)
    x = (torch.randn(B, H, W, 16, device="cuda", generator=g) * 0.3).contiguous()
    o16 = torch.empty(B, (H + 1) // 2, (W + 1) // 2, 8, device="cuda")
    o8 = torch.empty(B, H, W, 8, device="cuda")
    flops = 0
    for cin, cout, stride, res in NET_LAYERS:
        m = B * H * W if res == 1 else B * ((H + 1) // 2) * ((W + 1) // 2)
        flops += 2 * m * cout * 9 * cin
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            net.forward(x, o16, o8)
        torch.cuda.synchronize()
        barrier(world)
        l0 = net.kernel_launches()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(local) as clk:
            for a, e in evs:
                a.record(stream)
                net.forward(x, o16, o8)
                e.record(stream)
            torch.cuda.synchronize()
        launches = net.kernel_launches() - l0
        ms = [a.elapsed_time(e) for a, e in evs]
        # end to end: inputs from pinned host memory in, both outputs back
        xh = x.cpu().pin_memory()
        h16 = torch.empty(o16.shape, pin_memory=True)
        h8 = torch.empty(o8.shape, pin_memory=True)
        et = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            x.copy_(xh, non_blocking=True)
            net.forward(x, o16, o8)
            h16.copy_(o16, non_blocking=True)
            h8.copy_(o8, non_blocking=True)
            torch.cuda.synchronize()
            et.append(time.perf_counter() - t1)
    total_s = max_over_ranks(sum(ms) / 1000.0, world)
    per_pass = total_s / args.steps
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, kind = 1900.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as fh:
            peak, kind = float(json.load(fh)["bf16_tflops"]), "measured"
    achieved = flops / per_pass / 1e12
    if rank == 0:
        print(json.dumps({
            "metric": NET_METRIC, "value": world * B / per_pass, "unit": "pairs/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * per_pass, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 (FP32 accumulate)", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "batch": B, "grid": [H, W], "channels_in": 16,
                       "layers": NET_LAYERS, "checkpoint": wl["checkpoint"],
                       "parallelism": "replicas"},
            "e2e": {"value": world * B * len(et) / max_over_ranks(sum(et), world),
                    "unit": "pairs/s", "h2d_bytes_per_step": x.numel() * 4,
                    "d2h_bytes_per_step": (o16.numel() + o8.numel()) * 4},
            "roofline": {"bound": "tensor", "kernel": "k_tc_gemm (six convolutions)",
                         "achieved": achieved, "peak": peak, "peak_kind": kind,
                         "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                         "flops_per_pass": flops},
            "clocks": clk.summary(), "gpu_launches": int(launches),
        }), flush=True)
    net.close()


def run_pose(args, wl, world, rank, local):
    """Pose front end: one step = the relative pose of every pair through the
    C ABI (rf_pose_solve_f32), `threads` handles each on its own host thread
    and CUDA stream (the API is synchronous per handle).  `value`: frames
    resident in HBM; `e2e`: frames in pinned host memory, copied by the call."""
    import threading

    import torch

    import reconflow_gb300 as R
    from reconflow_gb300 import _native as N
    from reconflow_gb300.scene import make_scene

    torch.cuda.set_device(local)
    lib = R.load()
    W, H, n = wl["width"], wl["height"], args.pairs or wl["pairs"]
    T = min(wl["threads"], n)
    t0 = time.perf_counter()
    scenes = [make_scene(W, H, seed=wl["seed"] + 1000 * rank + i, device="cuda") for i in range(n)]
    gen_s = time.perf_counter() - t0
    dev = [tuple(torch.as_tensor(np.ascontiguousarray(sc[k], np.float32), device="cuda")
                 for k in ("I0", "I1")) for sc in scenes]
    Ks = [np.ascontiguousarray(sc["K"], np.float64) for sc in scenes]
    streams = [torch.cuda.Stream() for _ in range(T)]
    poses = []
    for k in range(T):
        cp = R.CameraPose()
        cp.initialize(Ks[0], wl["threshold"])
        cp.set_stream(streams[k].cuda_stream)
        cp._handle(W, H)
        poses.append(cp)
    out_R = np.zeros((n, 9))
    out_t = np.zeros((n, 3))
    fails = []

    def worker(k, frames):
        h = poses[k]._h
        for i in range(k, n, T):
            a, b = frames[i]
            st = lib.rf_pose_solve_f32(h, ctypes.c_void_p(a), ctypes.c_void_p(b), W,
                                       Ks[i].ctypes.data_as(ctypes.c_void_p),
                                       out_R[i].ctypes.data_as(ctypes.c_void_p),
                                       out_t[i].ctypes.data_as(ctypes.c_void_p))
            if st != 0:
                fails.append(i)

    def step(frames):
        ths = [threading.Thread(target=worker, args=(k, frames)) for k in range(T)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()

    dptr = [(a.data_ptr(), b.data_ptr()) for a, b in dev]
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        step(dptr)
    torch.cuda.synchronize()
    barrier(world)
    fails.clear()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            step(dptr)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t1)
    total_s = max_over_ranks(sum(times), world)
    value = world * n * args.steps / total_s
    if args.solve_only:
        if rank == 0:
            print(json.dumps({"metric": POSE_METRIC, "value": value, "unit": "pairs/s",
                              "note": "solve-only run"}), flush=True)
        return
    timed_fails = len(fails)

    def errors():
        rot, tra = [], []
        for i, sc in enumerate(scenes):
            if i in fails:
                continue
            Rm = out_R[i].reshape(3, 3)
            rot.append(np.degrees(np.arccos(np.clip((np.trace(Rm.T @ sc["R"]) - 1) / 2, -1, 1))))
            tg = sc["t"] / np.linalg.norm(sc["t"])
            tra.append(np.degrees(np.arccos(np.clip(out_t[i] @ tg, -1, 1))))
        return {"rot_err_deg_median": float(np.median(rot)), "rot_err_deg_max": float(np.max(rot)),
                "t_dir_err_deg_median": float(np.median(tra)), "t_dir_err_deg_max": float(np.max(tra))}

    acc = errors()
    counts = [poses[0].counts()]
    # refined poses (rf_pose_params.refine = 1) on the same frames, untimed
    for cp in poses:
        cp.params.refine = 1
        cp._release()
        cp._handle(W, H)
        cp.set_stream(None)
    fails.clear()
    step(dptr)
    torch.cuda.synchronize()
    acc_refined = errors()
    for cp in poses:
        cp.params.refine = 0
        cp._release()
        cp._handle(W, H)

    # end to end: frames in pinned host memory
    e2e = None
    if not args.no_e2e:
        hosts = []
        for i in range(n):
            pr = []
            for k in ("I0", "I1"):
                p_ = ctypes.c_void_p()
                R._native.check(lib.rf_host_alloc(W * H * 4, ctypes.byref(p_)))
                arr = np.ctypeslib.as_array(ctypes.cast(p_, ctypes.POINTER(ctypes.c_float)),
                                            shape=(H, W))
                arr[:] = scenes[i][k]
                pr.append(p_)
            hosts.append(pr)
        hptr = [(a.value, b.value) for a, b in hosts]
        step(hptr)
        et = []
        for _ in range(args.steps):
            t1 = time.perf_counter()
            step(hptr)
            et.append(time.perf_counter() - t1)
        e2e = {"value": world * n * args.steps / max_over_ranks(sum(et), world), "unit": "pairs/s",
               "h2d_bytes_per_step": 2 * n * W * H * 4, "d2h_bytes_per_step": n * 12 * 8}
        for pr in hosts:
            for p_ in pr:
                lib.rf_host_free(p_)

    # roofline: the dominant GPU stage of one solve, kernels timed with CUDA
    # events on the handle's stream (rf_pose_profile)
    ms = (ctypes.c_float * 8)()
    a, b = dptr[0]
    R._native.check(lib.rf_pose_profile(poses[0]._h, ctypes.c_void_p(a), ctypes.c_void_p(b), W,
                                        Ks[0].ctypes.data_as(ctypes.c_void_p), 20, ms))
    roofline = pose_roofline(list(ms), W, H, poses[0])
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = pose_cpu_sample(scenes[:2], wl["threshold"])
    if rank == 0:
        line = {
            "metric": POSE_METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (features), f64 (geometry)",
            "data": "synthetic (seeded scene generator)",
            "config": {"workload": args.workload, "width": W, "height": H, "pairs_per_step": n,
                       "handles_threads_streams": T, "hessian_threshold": wl["threshold"],
                       "n_octaves": 4, "n_octave_layers": 2, "ratio": 0.6,
                       "lmeds_confidence": 0.999, "scene_seeds": [wl["seed"], wl["seed"] + n - 1],
                       "timing": "host clock around each step, device synchronized on both "
                                 "sides (the call returns the pose)",
                       "parallelism": "replicas"},
            "accuracy": acc, "accuracy_refined": acc_refined, "failures": timed_fails,
            "counts_first_handle": counts[0],
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clk.summary(), "gpu_launches": int(sum(cp.kernel_launches() for cp in poses)),
            "scene_gen_s": gen_s,
        }
        print(json.dumps(line), flush=True)
    for cp in poses:
        cp.close()


def pose_roofline(ms, W, H, cp):
    """Roofline entry of the feature detector's Hessian-response kernel (every
    octave of one frame) and the per-launch times of every GPU stage: ms =
    [integral image, Hessian responses, keypoint selection, orientation,
    descriptors, matching, LMedS scoring] of frame 0 / the pair, then the
    keypoint count."""
    names = ["integral", "hessian", "extrema", "orientation", "descriptor", "match", "lmeds"]
    dom = max(range(len(names)), key=lambda k: ms[k])
    peak, peak_kind = load_peaks()
    layers = 4
    # algorithmic bytes of the response kernels: the integral image read once
    # per octave, every response written
    cells = sum((W >> o) * (H >> o) for o in range(4))
    a_bytes = 4 * (W + 1) * (H + 1) * 4 + layers * cells * 4
    achieved = a_bytes / (ms[1] * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": "k_hessian (4 octaves)", "achieved": achieved, "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
            "alg_bytes_per_launch": a_bytes, "dominant_stage": names[dom],
            "launch_ms": dict(zip(names, ms[:len(names)])), "keypoints": int(ms[7]),
            "timing": "each stage's launches back to back, CUDA events on the handle's stream"}


def pose_cpu_sample(scenes, threshold):
    """The oracle's feature stages (one core) and the library's host LMedS on
    a bounded sample of the workload's pairs."""
    from oracle import oracle as O
    from reconflow_gb300 import pose as P

    O.build()
    to8 = lambda a: np.clip(np.floor(a * 255 + 0.5), 0, 255).astype(np.uint8)  # noqa: E731
    t0 = time.perf_counter()
    for sc in scenes:
        k0, d0 = O.surf_detect(to8(sc["I0"]), threshold=threshold)
        k1, d1 = O.surf_detect(to8(sc["I1"]), threshold=threshold)
        best, a, b = O.surf_match(d0, d1)
        q = np.nonzero(np.sqrt(a).astype(np.float64) < 0.6 * np.sqrt(b).astype(np.float64))[0]
        Ki = np.linalg.inv(sc["K"])
        nrm = lambda p: (np.c_[p, np.ones(len(p))] @ Ki.T)[:, :2]  # noqa: E731
        x0, x1 = nrm(k0[q, :2].astype(np.float64)), nrm(k1[best[q], :2].astype(np.float64))
        E, m = P.essential_lmeds(x0, x1)
        P.recover_pose(E, x0, x1, m)
    dt = time.perf_counter() - t0
    return {"value": len(scenes) / dt, "unit": "pairs/s", "cores": 1, "kind": "port",
            "sample": f"{len(scenes)} pairs of the workload: oracle features and matching (one "
                      f"core), the library's host LMedS and pose recovery; {dt:.1f} s"}


def run_learned_mixed(args, wl, world, rank, local):
    """Batched + learned warm start on a mix of frame sizes (one batch, one
    network pass and one refinement per size group; the 4K / 1080p stream at
    a reduced count, with independent seeded scenes instead of sequences).
    One step = every group through the learned path with its fallback; the
    plain solver's batched and single-pair times are measured per group."""
    import torch

    import reconflow_gb300 as R
    from reconflow_gb300.scene import make_scene
    from reconflow_gb300.warmstart import LearnedBatchSolver, WarmStartNet, net_factor

    torch.cuda.set_device(local)
    lib = R.load()
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    groups = []
    t0 = time.perf_counter()
    for gi, g in enumerate(wl["groups"]):
        W, H, n = g["width"], g["height"], g["pairs"]
        scenes = [make_scene(W, H, seed=g["seed"] + 1000 * rank + i, device="cuda")
                  for i in range(n)]
        groups.append(dict(g=g, W=W, H=H, n=n, scenes=scenes, Ks=[s_["K"] for s_ in scenes],
                           Rs=[s_["R"] for s_ in scenes], ts=[s_["t"] for s_ in scenes]))
    gen_s = time.perf_counter() - t0

    def new_batch(G):
        b = R.ReconFlowBatch([(G["W"], G["H"])] * G["n"], wl["levels"], method=SOLVER["method"],
                             lambda_=SOLVER["lam"], lambdaf=SOLVER["lambdaf"],
                             lambdams=SOLVER["lambdams"], alphaTv=1.0 / SOLVER["theta"],
                             alphaProj=SOLVER["alpha_proj"], tau=SOLVER["tau"],
                             nWarpIters=wl["plain_warps"], nSolverIters=wl["plain_iters"],
                             fix_quirks=SOLVER["fix_quirks"])
        b.setStream(stream.cuda_stream)
        for i, sc in enumerate(G["scenes"]):
            b.setCameraMatrices(i, sc["K"], sc["K"])
            b.copyImagesToDevice(i, sc["I0"], sc["I1"])
        return b

    def epe_stats(G, b):
        means, meds = [], []
        for i, sc in enumerate(G["scenes"]):
            u, v = b.copyOpticalFlowToHost(i)
            W = G["W"]
            e = np.sqrt((u[:, :W] - sc["flow"][..., 0]) ** 2 + (v[:, :W] - sc["flow"][..., 1]) ** 2)
            e = e[sc["valid"]]
            e = np.where(np.isfinite(e), e, np.float32(1e4))
            means.append(float(e.mean()))
            meds.append(float(np.median(e)))
        return {"epe_mean_px": float(np.mean(means)), "epe_median_px": float(np.mean(meds))}

    def timed(fn, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        for a, e in evs:
            flush.zero_()
            a.record(stream)
            fn()
            e.record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(e) for a, e in evs]

    with torch.cuda.stream(stream):
        for G in groups:
            plain = new_batch(G)
            plain.solveR(G["Rs"], G["ts"])
            torch.cuda.synchronize()
            G["plain_acc"] = epe_stats(G, plain)
            G["e_plain"] = plain.energies()
            G["plain_batch_ms"] = statistics.median(timed(lambda: plain.solveR(G["Rs"], G["ts"]), 1))
            plain.close()
            f = R.ReconFlow()
            f.initializeR(G["W"], G["H"], 1, wl["levels"], 2.0, SOLVER["method"], SOLVER["lam"],
                          0.0, SOLVER["lambdaf"], SOLVER["lambdams"], 1.0 / SOLVER["theta"],
                          SOLVER["alpha_proj"], 0.5, SOLVER["tau"], wl["plain_warps"],
                          wl["plain_iters"], cvType=5, fix_quirks=SOLVER["fix_quirks"])
            f.setStream(stream.cuda_stream)
            f.setCameraMatrices(G["Ks"][0], G["Ks"][0])
            f.copyImagesToDevice(G["scenes"][0]["I0"], G["scenes"][0]["I1"])
            f.solveR(G["Rs"][0], G["ts"][0], 5.0)
            G["single_ms"] = statistics.median(timed(lambda: f.solveR(G["Rs"][0], G["ts"][0], 5.0), 2))
            # the learned step runs each size group on its own stream
            G["st"] = torch.cuda.Stream()
            torch.cuda.synchronize()
            f.setStream(G["st"].cuda_stream)
            G["f"] = f
            fct = net_factor(G["Ks"][0])
            net = WarmStartNet(G["n"], G["H"] // fct + 1, G["W"] // fct + 1, seed=0)
            net.load(os.path.join(ROOT, wl["checkpoint"]))
            b = new_batch(G)
            G["net"], G["b"] = net, b
            G["ls"] = LearnedBatchSolver(net, b, (G["W"], G["H"]), G["Ks"][0],
                                         warm_level=G["g"]["warm_level"],
                                         warps=G["g"]["warm_warps"], iters=G["g"]["warm_iters"])
            G["ls"].set_stream(G["st"].cuda_stream)
    margin = wl["fallback_margin"]
    fallbacks = []
    for G in groups:
        G["mode"], G["ceil"] = fallback_setup(args, G["W"], G["H"], "network")

    def step():
        # both groups' solves are queued before the first group's energies
        # are read: one group's solve runs while the host tests the other
        nbad = 0
        for G in groups:
            G["st"].wait_stream(stream)
            G["ls"].solve(G["Ks"], G["Rs"], G["ts"])
        for G in groups:
            e = G["b"].energies()
            bad = [i for i in range(G["n"])
                   if fallback_test(G["mode"], e[i], G["e_plain"][i], G["W"] * G["H"], G["ceil"],
                                    margin)]
            for i in bad:
                f = G["f"]
                f.setCameraMatrices(G["Ks"][i], G["Ks"][i])
                f.copyImagesToDeviceFromDevice(*G["b"].imagePlanes(i, 0), G["b"].strides[i])
                f.solveR(G["Rs"][i], G["ts"][i], 5.0)
                G["b"].importResults(i, f.deviceResults(), f.stride)
            nbad += len(bad)
        for G in groups:
            stream.wait_stream(G["st"])
        fallbacks.append(nbad)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        for G in groups:
            G["learned_acc"] = epe_stats(G, G["b"])
        barrier(world)
        fallbacks.clear()
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            step_ms = timed(step, args.steps)
    timed_fallbacks = list(fallbacks)
    npairs = sum(G["n"] for G in groups)
    total_s = max_over_ranks(sum(step_ms) / 1000.0, world)
    value = world * npairs * args.steps / total_s
    single_step_ms = sum(G["single_ms"] * G["n"] for G in groups)
    e2e = None
    if not args.no_e2e:
        hosts = []
        for G in groups:
            s0, H = G["b"].strides[0], G["H"]
            for i in range(G["n"]):
                ptrs = []
                for _ in range(8):
                    p_ = ctypes.c_void_p()
                    R._native.check(lib.rf_host_alloc(H * s0 * 4, ctypes.byref(p_)))
                    ptrs.append(p_)
                for k, img in ((0, G["scenes"][i]["I0"]), (1, G["scenes"][i]["I1"])):
                    a_ = np.ctypeslib.as_array(ctypes.cast(ptrs[k], ctypes.POINTER(ctypes.c_float)),
                                               shape=(H, s0))
                    a_[:, :G["W"]] = img
                hosts.append((G, i, ptrs))

        cols = {}
        for G, i, ptrs in hosts:
            cols.setdefault(id(G), (G, [[] for _ in range(8)]))
            for k in range(8):
                cols[id(G)][1][k].append(ptrs[k].value)

        def e2e_step():
            for G, c in cols.values():
                G["b"].uploadAll(c[0], c[1], G["b"].strides[0])
            step()
            for G, c in cols.values():
                G["b"].downloadAll(G["b"].strides[0], u=c[2], v=c[3], inv_depth=c[4], X=c[5],
                                   Y=c[6], Z=c[7])

        with torch.cuda.stream(stream):
            e2e_step()
            times = []
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                e2e_step()
                torch.cuda.synchronize()
                times.append(time.perf_counter() - t1)
            piped = serve_pipelined([(G["b"], c, G["b"].strides[0]) for G, c in cols.values()],
                                    step, args.steps, flush)
        px = sum(G["n"] * G["W"] * G["H"] for G in groups)
        e2e = {"value": world * npairs * args.steps / max_over_ranks(piped, world),
               "unit": "pairs/s", "h2d_bytes_per_step": 2 * px * 4, "d2h_bytes_per_step": 6 * px * 4,
               "mode": E2E_MODE,
               "serial_value": world * npairs * args.steps / max_over_ranks(sum(times), world)}
        for _, _, ptrs in hosts:
            for p_ in ptrs:
                lib.rf_host_free(p_)
    if rank == 0:
        tol = 0.05
        per = {}
        for G in groups:
            key = f"{G['W']}x{G['H']}"
            per[key] = {"pairs": G["n"], "warm_level": G["g"]["warm_level"],
                        "warm_warps_per_level": G["g"]["warm_warps"],
                        "warm_iters_per_level": G["g"]["warm_iters"],
                        "plain_accuracy": G["plain_acc"], "learned_accuracy": G["learned_acc"],
                        "plain_single_pair_ms": G["single_ms"],
                        "plain_batched_ms_per_pair": G["plain_batch_ms"] / G["n"],
                        "equal_epe_median": G["learned_acc"]["epe_median_px"]
                        <= G["plain_acc"]["epe_median_px"] + tol,
                        "equal_epe_mean": G["learned_acc"]["epe_mean_px"]
                        <= G["plain_acc"]["epe_mean_px"] + tol}
        print(json.dumps({
            "metric": "frame pairs/s, batched + learned warm start on mixed 4K / 1080p pairs",
            "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene generator, independent scenes, not sequences)",
            "config": {"workload": args.workload, "groups": per, "pyramid_levels": wl["levels"],
                       "plain_schedule": [wl["plain_warps"], wl["plain_iters"]],
                       "fallback": {f"{G['W']}x{G['H']}": fallback_desc(G["mode"], G["ceil"],
                                                                         margin)
                                    for G in groups},
                       "checkpoint": wl["checkpoint"], "l2": "flushed between steps",
                       "parallelism": "replicas"},
            "speedup_vs_plain_single_pair": single_step_ms / (1000.0 * total_s / args.steps),
            "fallbacks_per_step": timed_fallbacks, "e2e": e2e, "clocks": clk.summary(),
            "scene_gen_s": gen_s,
        }), flush=True)
    for G in groups:
        G["b"].close()
        G["net"].close()
        G["f"].close()


def fallback_setup(args, W, H, source):
    """The fallback test of the learned workloads: "calibrated" (default,
    deployable: the learned energy per pixel against the ceiling measured on
    calibration scenes, reconflow_gb300/tuning/fallback_energy.json),
    "plain" (the pair's own plain-solve energy, computed untimed beforehand)
    or "none".  Returns (mode, ceiling)."""
    from reconflow_gb300 import fallback as FB

    mode = args.fallback or "calibrated"
    ceil = None
    if mode == "calibrated":
        try:
            ceil = FB.ceiling(FB.load(), W, H, source)
        except OSError:
            ceil = None
    return mode, ceil


def fallback_test(mode, e, e_plain, pixels, ceil, margin):
    from reconflow_gb300 import fallback as FB

    if mode == "none":
        return False
    if mode == "plain":
        return over_margin(e, e_plain, margin)
    return FB.over(e, pixels, ceil)


def fallback_desc(mode, ceil, margin):
    if mode == "calibrated":
        return (f"calibrated: plain re-solve when the learned energy per pixel > {ceil} "
                f"((1 + {margin}) x the calibration scenes' largest) or not finite")
    if mode == "plain":
        return f"plain re-solve when energy > (1 + {margin}) x the pair's plain-solve energy"
    return "none"


def over_margin(e, ref, margin):
    """The fallback test: a solution whose energy is not finite always falls
    back; one whose reference energy is not finite never has to."""
    if not np.isfinite(e):
        return True
    return bool(np.isfinite(ref) and e > (1.0 + margin) * ref)


def c5_fallback_desc(G, warm_mode, margin):
    from reconflow_gb300 import fallback as FB

    if G["mode"] == "calibrated" and warm_mode == "temporal":
        return (f"calibrated: wave 0 (network start) plain re-solve when the learned energy per "
                f"pixel > {G['ceil_net']} ((1 + {margin}) x the calibration scenes' largest); "
                f"later waves when it exceeds {FB.HISTORY_FACTOR} x the median of the "
                f"sequence's last {FB.HISTORY} pairs; always when not finite")
    return fallback_desc(G["mode"], G["ceil_net"], margin)


C5_METRIC = ("frame pairs/s, C5 stream: 256 pairs of 3840x2160 / 1920x1080 from 32-frame "
             "sequences, batched + learned / temporal warm start")


def run_c5_stream(args, wl, world, rank, local):
    """The C5 stream.  One step = the whole stream: 32 waves; in each wave
    every sequence's next pair is solved, the pairs of a size together in
    one batch.  Wave 0 warm-starts from the network; wave k > 0 from wave
    k-1's solved depth of the same sequence carried into frame k
    (rf_ws_propagate -> rf_ws_state), refined from the same pyramid level.
    After each wave the pairs' energies are compared with the fallback
    reference; a pair over the margin is solved again with the full plain
    schedule (single-pair drop-in solver, from the batch's frames).  The
    accuracy pass (untimed) also solves every pair with the plain batched
    solver for its energy and endpoint error."""
    import torch

    import reconflow_gb300 as R
    from reconflow_gb300 import fallback as FB
    from reconflow_gb300.scene import make_sequence
    from reconflow_gb300.warmstart import TemporalBatchSolver, WarmStartNet, net_factor

    torch.cuda.set_device(local)
    lib = R.load()
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    nf = wl["frames"]
    nw = nf - 1  # waves (pairs per sequence)
    warm_mode = args.warm or "temporal"
    groups = []
    t0 = time.perf_counter()
    for g in wl["groups"]:
        W, H, n = g["width"], g["height"], g["sequences"]
        s = (W + 31) // 32 * 32
        seqs = [make_sequence(W, H, nf, seed=g["seed"] + 1000 * rank + j, device="cuda")
                for j in range(n)]
        frames = [[torch.nn.functional.pad(torch.as_tensor(f_, device="cuda"), (0, s - W))
                   .contiguous() for f_ in q["frames"]] for q in seqs]
        # one stream per size group: the host reads one group's energies
        # while the other group's wave runs
        groups.append(dict(g=g, W=W, H=H, n=n, s=s, seqs=seqs, frames=frames,
                           Ks=[q["K"] for q in seqs], st=torch.cuda.Stream()))
    torch.cuda.synchronize()  # the frames (default stream) before the groups' streams use them
    gen_s = time.perf_counter() - t0

    def new_batch(G, warps, iters):
        b = R.ReconFlowBatch([(G["W"], G["H"])] * G["n"], wl["levels"], method=SOLVER["method"],
                             lambda_=SOLVER["lam"], lambdaf=SOLVER["lambdaf"],
                             lambdams=SOLVER["lambdams"], alphaTv=1.0 / SOLVER["theta"],
                             alphaProj=SOLVER["alpha_proj"], tau=SOLVER["tau"],
                             nWarpIters=warps, nSolverIters=iters,
                             fix_quirks=SOLVER["fix_quirks"])
        b.setStream(G["st"].cuda_stream)
        for i, K in enumerate(G["Ks"]):
            b.setCameraMatrices(i, K, K)
        return b

    def load_wave(G, b, k):
        for i in range(G["n"]):
            b.copyImagesToDeviceFromDevice(i, G["frames"][i][k].data_ptr(),
                                           G["frames"][i][k + 1].data_ptr(), G["s"])

    def pose(G, k):
        return ([q["pairs"][k]["R"] for q in G["seqs"]], [q["pairs"][k]["t"] for q in G["seqs"]])

    def epe(G, b, i, k):
        u, v = b.copyOpticalFlowToHost(i)
        pr = G["seqs"][i]["pairs"][k]
        W = G["W"]
        e = np.sqrt((u[:, :W] - pr["flow"][..., 0]) ** 2 + (v[:, :W] - pr["flow"][..., 1]) ** 2)
        e = e[pr["valid"]]
        e = np.where(np.isfinite(e), e, np.float32(1e4))
        return float(e.mean()), float(np.median(e))

    with torch.cuda.stream(stream):
        for G in groups:
            g = G["g"]
            fct = net_factor(G["Ks"][0])
            G["factor"] = fct
            G["hn"], G["wn"] = G["H"] // fct, G["W"] // fct
            net = WarmStartNet(G["n"], G["hn"] + 1, G["wn"] + 1, seed=0)
            net.load(os.path.join(ROOT, wl["checkpoint"]))
            b = new_batch(G, wl["plain_warps"], wl["plain_iters"])
            tsol = TemporalBatchSolver(net, b, (G["W"], G["H"]), G["Ks"][0],
                                       warm_level=g["warm_level"], warps=g["warm_warps"],
                                       iters=g["warm_iters"], temporal_warps=g["temporal_warps"],
                                       temporal_iters=g["temporal_iters"])
            tsol.set_stream(G["st"].cuda_stream)
            G.update(net=net, b=b, tsol=tsol)
            G["mode"], G["ceil_net"] = fallback_setup(args, G["W"], G["H"], "network")
            G["guard"] = FB.SequenceGuard(G["n"])
            f = R.ReconFlow()
            f.initializeR(G["W"], G["H"], 1, wl["levels"], 2.0, SOLVER["method"], SOLVER["lam"],
                          0.0, SOLVER["lambdaf"], SOLVER["lambdams"], 1.0 / SOLVER["theta"],
                          SOLVER["alpha_proj"], 0.5, SOLVER["tau"], wl["plain_warps"],
                          wl["plain_iters"], cvType=5, fix_quirks=SOLVER["fix_quirks"])
            f.setStream(G["st"].cuda_stream)
            G["f"] = f

    def solve_wave(G, k):
        """Warm-started solve of wave k for group G (no fallback)."""
        Rs, ts = pose(G, k)
        load_wave(G, G["b"], k)
        if k == 0 or warm_mode == "network":
            G["tsol"].first(G["Ks"], Rs, ts)
        else:
            G["tsol"].next(G["Ks"], *pose(G, k - 1), Rs, ts)

    def must_fall_back(G, gi, i, k, e):
        """The fallback test of pair i of wave k (call in wave order: the
        calibrated temporal test keeps each sequence's energy history)."""
        if G["mode"] == "calibrated" and warm_mode == "temporal":
            if k == 0 and i == 0:
                G["guard"].reset()
            return G["guard"].over(i, e, G["W"] * G["H"], G["ceil_net"])
        return fallback_test(G["mode"], e, refs[(gi, i, k)], G["W"] * G["H"], G["ceil_net"],
                             margin)

    margin = wl["fallback_margin"]
    refs = {}  # (group, pair, wave) -> reference energy for the fallback test
    fallbacks = []
    record = []

    def stream_once(collect=False):
        nbad = 0
        for k in range(nw):
            for G in groups:
                solve_wave(G, k)
            for gi, G in enumerate(groups):
                e = G["b"].energies()
                bad = [i for i in range(G["n"]) if must_fall_back(G, gi, i, k, e[i])]
                if collect:
                    for i in range(G["n"]):
                        record.append(dict(group=gi, seq=i, wave=k, e_learned=float(e[i]),
                                           epe_learned=epe(G, G["b"], i, k),
                                           fell_back=i in bad))
                for i in bad:
                    # the full plain solve of the pair, in place of the learned result
                    f = G["f"]
                    Rs, ts = pose(G, k)
                    f.setCameraMatrices(G["Ks"][i], G["Ks"][i])
                    f.copyImagesToDeviceFromDevice(G["frames"][i][k].data_ptr(),
                                                   G["frames"][i][k + 1].data_ptr(), G["s"])
                    f.solveR(Rs[i], ts[i], 5.0)
                    G["b"].importResults(i, f.deviceResults(), f.stride)
                nbad += len(bad)
        fallbacks.append(nbad)

    # the plain solve of every pair (untimed): its energy is the fallback
    # reference ("plain") and its endpoint error the accuracy reference
    plain_rec = {}
    with torch.cuda.stream(stream):
        for gi, G in enumerate(groups):
            pb = new_batch(G, wl["plain_warps"], wl["plain_iters"])
            for k in range(nw):
                load_wave(G, pb, k)
                Rs, ts = pose(G, k)
                pb.solveR(Rs, ts)
                e = pb.energies()
                for i in range(G["n"]):
                    refs[(gi, i, k)] = float(e[i])
                    plain_rec[(gi, i, k)] = (float(e[i]), epe(G, pb, i, k))
            pb.close()
        torch.cuda.synchronize()
        plain_gen_s = time.perf_counter() - t0 - gen_s
        stream_once(collect=True)
        for _ in range(max(0, args.warmup - 1)):
            stream_once()
        torch.cuda.synchronize()
        barrier(world)
        fallbacks.clear()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            for a, e_ in evs:
                flush.zero_()
                a.record(stream)
                for G in groups:  # each size group works on its own stream
                    G["st"].wait_stream(stream)
                stream_once()
                for G in groups:
                    stream.wait_stream(G["st"])
                e_.record(stream)
            torch.cuda.synchronize()
        step_ms = [a.elapsed_time(e_) for a, e_ in evs]
    timed_fallbacks = list(fallbacks)
    npairs = nw * sum(G["n"] for G in groups)
    total_s = max_over_ranks(sum(step_ms) / 1000.0, world)
    value = world * npairs * args.steps / total_s

    e2e = None
    if not args.no_e2e:
        # every wave's frames from pinned host memory and every pair's
        # results back to it, inside the timed wall time
        host_frames = {}
        outs = {}
        for gi, G in enumerate(groups):
            nb = G["H"] * G["s"] * 4
            for i in range(G["n"]):
                for k in range(nf):
                    p_ = ctypes.c_void_p()
                    R._native.check(lib.rf_host_alloc(nb, ctypes.byref(p_)))
                    a_ = np.ctypeslib.as_array(ctypes.cast(p_, ctypes.POINTER(ctypes.c_float)),
                                               shape=(G["H"], G["s"]))
                    a_[:] = 0.0
                    a_[:, :G["W"]] = G["seqs"][i]["frames"][k]
                    host_frames[(gi, i, k)] = p_
                ptrs = []
                for _ in range(6):
                    p_ = ctypes.c_void_p()
                    R._native.check(lib.rf_host_alloc(nb, ctypes.byref(p_)))
                    ptrs.append(p_)
                outs[(gi, i)] = ptrs

        def e2e_stream():
            for k in range(nw):
                for gi, G in enumerate(groups):
                    n = G["n"]
                    G["b"].uploadAll([host_frames[(gi, i, k)].value for i in range(n)],
                                     [host_frames[(gi, i, k + 1)].value for i in range(n)],
                                     G["s"])
                    b = G["b"]
                    Rs, ts = pose(G, k)
                    if k == 0 or warm_mode == "network":
                        G["tsol"].first(G["Ks"], Rs, ts)
                    else:
                        G["tsol"].next(G["Ks"], *pose(G, k - 1), Rs, ts)
                    e = b.energies()
                    for i in range(n):
                        if must_fall_back(G, gi, i, k, e[i]):
                            f = G["f"]
                            f.setCameraMatrices(G["Ks"][i], G["Ks"][i])
                            f.copyImagesToDeviceFromDevice(*b.imagePlanes(i, 0), G["s"])
                            f.solveR(Rs[i], ts[i], 5.0)
                            b.importResults(i, f.deviceResults(), f.stride)
                    o = [outs[(gi, i)] for i in range(n)]
                    b.downloadAll(G["s"], *[[o[i][c].value for i in range(n)] for c in range(6)])

        with torch.cuda.stream(stream):
            e2e_stream()
            torch.cuda.synchronize()
            times = []
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                e2e_stream()
                torch.cuda.synchronize()
                times.append(time.perf_counter() - t1)
        px = nw * sum(G["n"] * G["W"] * G["H"] for G in groups)
        e2e = {"value": world * npairs * args.steps / max_over_ranks(sum(times), world),
               "unit": "pairs/s", "h2d_bytes_per_step": 2 * px * 4,
               "d2h_bytes_per_step": 6 * px * 4,
               "mode": "blocking: each wave's frames uploaded from pinned host memory and its "
                       "results (flow, inverse depth, points) downloaded to it, every wave"}
        for p_ in list(host_frames.values()) + [q for v in outs.values() for q in v]:
            lib.rf_host_free(p_)

    if rank == 0:
        per = {}
        for gi, G in enumerate(groups):
            rec = [r for r in record if r["group"] == gi]
            plain = [plain_rec[(gi, r["seq"], r["wave"])] for r in rec]
            lm = [r["epe_learned"][0] for r in rec]
            lmed = [r["epe_learned"][1] for r in rec]
            pm = [p_[1][0] for p_ in plain]
            pmed = [p_[1][1] for p_ in plain]
            ratio = [r["e_learned"] / p_[0] for r, p_ in zip(rec, plain)]
            per[f"{G['W']}x{G['H']}"] = {
                "sequences": G["n"], "pairs": G["n"] * nw, "warm_level": G["g"]["warm_level"],
                "network_iters_per_level": G["g"]["warm_iters"],
                "temporal_iters_per_level": G["g"]["temporal_iters"],
                "learned_epe_mean_px": float(np.mean(lm)),
                "learned_epe_median_px": float(np.mean(lmed)),
                "plain_epe_mean_px": float(np.mean(pm)),
                "plain_epe_median_px": float(np.mean(pmed)),
                "energy_ratio_median": float(np.median(ratio)),
                "energy_ratio_max": float(np.max(ratio)),
                "over_margin": int(sum(x > 1.0 + margin for x in ratio)),
                "fell_back": int(sum(r["fell_back"] for r in rec)),
                "fell_back_and_over_margin": int(sum(r["fell_back"] and x > 1.0 + margin
                                                     for r, x in zip(rec, ratio)))}
        if args.dump:
            np.savez(args.dump, group=[r["group"] for r in record],
                     seq=[r["seq"] for r in record], wave=[r["wave"] for r in record],
                     e_learned=[r["e_learned"] for r in record],
                     epe_learned=[r["epe_learned"] for r in record],
                     fell_back=[r["fell_back"] for r in record],
                     e_plain=[plain_rec[(r["group"], r["seq"], r["wave"])][0] for r in record],
                     epe_plain=[plain_rec[(r["group"], r["seq"], r["wave"])][1] for r in record])
        print(json.dumps({
            "metric": C5_METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded moving-camera sequences of the scene generator)",
            "config": {"workload": args.workload, "frames_per_sequence": nf,
                       "pairs_per_step": npairs, "groups": per, "pyramid_levels": wl["levels"],
                       "plain_schedule": [wl["plain_warps"], wl["plain_iters"]],
                       "warm_start": "network at wave 0, then the previous wave's depth "
                                     "carried into the new frame (rf_ws_propagate)"
                                     if warm_mode == "temporal" else "network for every pair",
                       "fallback": {f"{G['W']}x{G['H']}": c5_fallback_desc(G, warm_mode, margin)
                                    for G in groups},
                       "checkpoint": wl["checkpoint"], "l2": "flushed between steps",
                       "parallelism": "replicas"},
            "fallbacks_per_step": timed_fallbacks, "e2e": e2e, "clocks": clk.summary(),
            "scene_gen_s": gen_s, "plain_reference_s": plain_gen_s,
        }), flush=True)
    for G in groups:
        G["b"].close()
        G["net"].close()
        G["f"].close()


def roofline_of(ms, px, batched=False):
    """Roofline entry of the dominant level-0 kernel from per-launch times
    (`px` pixels per launch; `batched`: the batched solver's kernels)."""
    names = ["recon_a", "recon_b"]
    dom = 0 if ms[0] >= ms[1] else 1
    achieved = ALG_BYTES[names[dom]] * px / (ms[dom] * 1e-3) / 1e9
    peak, peak_kind = load_peaks()
    traffic = None
    tpath = os.path.join(ROOT, "profiles",
                         "traffic_720p_batch.json" if batched else "traffic_720p.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            tr = json.load(fh)
        per = tr.get(names[dom])
        # the capture's DRAM bytes per launch scaled by pixels (traffic grows
        # with the pixel count: one pass over every field per launch)
        traffic = None if per is None else per * px / tr["pixels"]
    return {"bound": "hbm", "kernel": ("k_batch<OpReconA>" if dom == 0 else "k_batch<OpReconB>")
            if batched else ("k_recon_a" if dom == 0 else "k_recon_b"),
            "achieved": achieved, "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "alg_bytes_per_launch": ALG_BYTES[names[dom]] * px,
            "launch_ms": {names[0]: ms[0], names[1]: ms[1]},
            "frac_each": {names[k]: ALG_BYTES[names[k]] * px / (ms[k] * 1e-3) / 1e9 / peak
                          for k in range(2)},
            "iteration": iteration_roofline(ms, px, peak),
            "issue": issue_roofline(ms, px, tr.get("warp_instructions_per_32px")
                                    if os.path.exists(tpath) else None),
            "timing": "launches of one kernel back to back in a CUDA graph, CUDA events"}


def issue_roofline(ms, px, inst):
    """The data step against the SMs' instruction-issue rate (it is bound by
    issue, not by DRAM): warp instructions per 32 pixels from the committed
    ncu capture x pixels / launch time, against 152 SMs x 4 schedulers x
    one warp instruction per cycle at the maximum SM clock."""
    if not inst:
        return None
    peak = 152 * 4 * measured_sm_mhz() * 1e6
    out = {}
    for k, name in enumerate(("recon_a", "recon_b")):
        if name in inst:
            rate = inst[name] * px / 32.0 / (ms[k] * 1e-3)
            out[name] = {"warp_inst_per_32px": inst[name], "achieved_ginst_s": rate / 1e9,
                         "peak_ginst_s": peak / 1e9, "frac": rate / peak}
    return out


def measured_sm_mhz():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh).get("sm_max_mhz", 2070.0))
    except (OSError, ValueError):
        return 2070.0


def iteration_roofline(ms, px, peak):
    """The whole inner iteration against its compulsory traffic: 13 state
    floats read and written plus 5 per-warp constants read = 124 B per
    pixel-iteration, over the time of both inner-iteration kernels."""
    t = (ms[0] + ms[1]) * 1e-3
    achieved = ITER_BYTES * px / t / 1e9
    return {"alg_bytes_per_pixel": ITER_BYTES, "ms": ms[0] + ms[1], "achieved": achieved,
            "frac": achieved / peak}


def config_of(wl):
    return {"workload": f"reconflow_{wl['width']}x{wl['height']}_L{wl['levels']}_w{wl['warps']}"
                        f"_i{wl['iters']}",
            "width": wl["width"], "height": wl["height"], "pyramid_levels": wl["levels"],
            "warps": wl["warps"], "iters": wl["iters"], "pairs_per_step": 1,
            "method": "METHODR_TVL1_MS", "lambda": SOLVER["lam"], "theta": SOLVER["theta"],
            "tau": SOLVER["tau"], "alpha_proj": SOLVER["alpha_proj"], "lambdaf": SOLVER["lambdaf"],
            "lambdams": SOLVER["lambdams"], "fix_quirks": SOLVER["fix_quirks"],
            "scene_seed": wl["seed"], "l2": "flushed between steps (512 MiB write)",
            "parallelism": "replicas"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="720p-learned", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--solve-only", action="store_true",
                    help="only warm-up + timed solves (for profiler launch lists)")
    ap.add_argument("--fallback", default=None, choices=["plain", "none"],
                    help="learned workloads: compare with the pair's own plain-solve energy "
                         "(computed untimed) or take no fallback (default: the calibrated, "
                         "deployable test)")
    ap.add_argument("--checkpoint", default=None,
                    help="learned workloads: the network weights (default: the committed "
                         "checkpoint)")
    ap.add_argument("--warm", default=None, choices=["temporal", "network"],
                    help="c5-stream: warm start of waves after the first (default temporal)")
    ap.add_argument("--dump", default=None,
                    help="c5-stream: write per-pair energies and endpoint errors to this .npz")
    ap.add_argument("--pairs", type=int, default=0,
                    help="pairs per step of the 720p learned or pose workload (profiling; "
                         "default: the workload's)")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.checkpoint and "checkpoint" in wl:
        wl = dict(wl, checkpoint=args.checkpoint)
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        if "net" in wl:
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no "
                                  "learned warm start (no network to time)"}), flush=True)
            return
        if "pose" in wl:
            run_reference_pose(args, wl, world, rank)
            return
        if "groups" in wl or "frames" in wl or ("pairs" in wl and "checkpoint" not in wl):
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference solves "
                                  "one pair at a time and has no batched path; its per-pair "
                                  "rate is the reference arm of --workload 720p / 480p"}),
                      flush=True)
            return
        if "checkpoint" in wl:
            # the reference's counterpart of a learned batch: its plain solve, one pair
            wl = dict(width=wl["width"], height=wl["height"], levels=wl["levels"],
                      warps=wl["plain_warps"], iters=wl["plain_iters"], seed=wl["seed"],
                      metric=LEARNED_METRIC, workload=args.workload)
        run_reference(args, wl, world, rank)
        return
    if "pose" in wl:
        run_pose(args, wl, world, rank, local)
        return
    if "net" in wl:
        run_net(args, wl, world, rank, local)
        return
    if "frames" in wl:
        run_c5_stream(args, wl, world, rank, local)
        return
    if "groups" in wl:
        run_learned_mixed(args, wl, world, rank, local)
        return
    if "checkpoint" in wl:
        run_learned(args, wl, world, rank, local)
        return
    if "pairs" in wl:
        run_batch(args, wl, world, rank, local)
        return

    import torch

    import reconflow_gb300 as R

    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (the solver has no CPU path)")
    torch.cuda.set_device(local)
    lib = R.load()
    sc, I0, I1, s = make_inputs(wl)
    f = R.ReconFlow()
    f.initializeR(wl["width"], wl["height"], 1, wl["levels"], 2.0, SOLVER["method"], SOLVER["lam"],
                  0.0, SOLVER["lambdaf"], SOLVER["lambdams"], 1.0 / SOLVER["theta"],
                  SOLVER["alpha_proj"], 0.5, SOLVER["tau"], wl["warps"], wl["iters"], cvType=5,
                  fix_quirks=SOLVER["fix_quirks"])
    stream = torch.cuda.Stream()
    f.setStream(stream.cuda_stream)
    single_tiles = load_tiles(SINGLE_TILES) if (wl["width"], wl["height"]) == (1280, 720) else None
    if single_tiles is not None:
        from reconflow_gb300 import autotune

        autotune.apply_single(f, single_tiles["levels"], wl["levels"])
        autotune.apply_iterations_per_launch(lib, single_tiles)
    f.setCameraMatrices(sc["K"], sc["K"])
    f.copyImagesToDevice(I0, I1)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def solve():
        f.solveR(sc["R"], sc["t"], 5.0)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            solve()
        torch.cuda.synchronize()
        barrier(world)
        launches0 = f.kernelLaunches()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            wall0 = time.perf_counter()
            for a, b in evs:
                flush.zero_()
                a.record(stream)
                solve()
                b.record(stream)
            torch.cuda.synchronize()
            wall = time.perf_counter() - wall0
        launches = f.kernelLaunches() - launches0
        step_ms = [a.elapsed_time(b) for a, b in evs]
        total_s = max_over_ranks(sum(step_ms) / 1000.0, world)
        barrier(world)
    value = world * args.steps / total_s
    if args.solve_only:
        if rank == 0:
            print(json.dumps({"metric": "720p frame pairs/s", "value": value, "unit": "pairs/s",
                              "note": "solve-only run"}), flush=True)
        return

    # accuracy of the last solve against the generator's ground truth
    u, v = f.copyOpticalFlowToHost()
    X, Y, Z = f.copy3dToHost()
    w, h = wl["width"], wl["height"]
    val = sc["valid"]
    epe = np.sqrt((u[:, :w] - sc["flow"][..., 0]) ** 2 + (v[:, :w] - sc["flow"][..., 1]) ** 2)[val]
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / Z[:, :w]
        rel = np.abs(inv - sc["inv_depth"]) / sc["inv_depth"]
    accuracy = {"epe_mean_px": float(epe.mean()), "epe_median_px": float(np.median(epe)),
                "inv_depth_rel_err_median": float(np.nanmedian(rel[val]))}

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        nbytes_plane = h * s * 4
        hosts = []
        for _ in range(8):
            p = ctypes.c_void_p()
            R._native.check(lib.rf_host_alloc(nbytes_plane, ctypes.byref(p)))
            hosts.append(p)
        np_h = [np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_float)),
                                      shape=(h, s)) for p in hosts]
        np_h[0][:] = I0
        np_h[1][:] = I1
        hnd = f._handle()

        def e2e_step():
            R._native.check(lib.rf_upload_images(hnd, hosts[0], hosts[1], s))
            f.solveR(sc["R"], sc["t"], 5.0)
            R._native.check(lib.rf_download_flow(hnd, hosts[2], hosts[3], s))
            R._native.check(lib.rf_download_inv_depth(hnd, hosts[4], s))
            R._native.check(lib.rf_download_points(hnd, hosts[5], hosts[6], hosts[7], s))

        for _ in range(max(1, args.warmup)):
            e2e_step()
        barrier(world)
        times = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e2e_step()
            times.append(time.perf_counter() - t0)
        e2e_total = max_over_ranks(sum(times), world)
        e2e = {"value": world * args.steps / e2e_total, "unit": "pairs/s",
               "h2d_bytes_per_step": 2 * w * h * 4, "d2h_bytes_per_step": 6 * w * h * 4}
        for p in hosts:
            lib.rf_host_free(p)

    # roofline of the dominant kernel: level-0 inner iterations, CUDA events
    ms = (ctypes.c_float * 2)()
    f.solveR(sc["R"], sc["t"], 5.0)
    R._native.check(lib.rf_profile_iterations(f._handle(), 0, 50, ms))
    roofline = roofline_of(ms, w * h)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        run, cores = cpu_sample(wl, sc, I0, I1)
        run(1)
        per_pair = run(wl["iters"])
        cpu = {"value": 1.0 / per_pair, "unit": "pairs/s", "cores": cores, "kind": "port",
               "sample": f"one plain solve of one {w}x{h} pair, the full {wl['levels']}-level x "
                         f"{wl['warps']}-warp x {wl['iters']}-iteration schedule, measured "
                         f"({per_pair:.2f} s)"}

    if rank == 0:
        line = {
            "metric": PLAIN_METRIC if (w, h) == (1280, 720) else
                      f"{w}x{h} frame pairs/s (ReconFlow flow + depth)", "value": value,
            "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene generator)",
            "config": dict(config_of(wl), tiles=SINGLE_TILES if single_tiles is not None
                           else "default 32x8",
                           cluster_px=(single_tiles or {}).get("iterations_per_launch",
                                                               {}).get("cluster_px", 0)),
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clk.summary(), "gpu_launches": int(launches),
            "wall_s_timed": wall, "accuracy": accuracy,
            "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms),
                        "max": max(step_ms)},
        }
        print(json.dumps(line), flush=True)
    f.close()


if __name__ == "__main__":
    main()
