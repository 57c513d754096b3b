"""Autotuner for the batched and single-pair solvers.

Every step of a batched solve is one launch over the tiles of every pair at
one pyramid level (``rf_batch.cu``); the tile shape decides how pixels map
to blocks (and so the wave count, the tail of the last wave and how well
neighbouring pixels share cache lines), never the arithmetic, so results are
identical for every shape.  ``autotune`` times the two inner-iteration
kernels of each level (``rf_batch_profile_level``: launches back to back in a
CUDA graph, CUDA events) for every candidate shape and keeps the fastest per
level.  ``tiles_for`` turns a saved table into per-level shapes for a batch
of any size by the pixel count of the level (summed over pairs).

    python -m reconflow_gb300.autotune --size 1280x720 --pairs 64 --out table.json

The tile candidates span 2 to 8 warps per block (32 x 2 .. 16 x 16), so the
shape search also picks the warps per block.  For one ReconFlow handle a
second dimension is searched: iterations per launch.  The two-launch loop
runs one inner iteration per pair of launches (a CUDA graph); the
thread-block-cluster kernel runs all of a warp's iterations at a level in
one launch (rf_set_cluster_pixels: every level of at most n pixels).
`autotune_iterations_per_launch` times whole solves for each threshold and
keeps the fastest; the table records it under "iterations_per_launch".

    python -m reconflow_gb300.autotune --single --size 1280x720 --out table.json
"""
from __future__ import annotations

import json
import os

CANDIDATES = [(32, 8), (64, 4), (128, 2), (32, 4), (64, 2), (16, 16), (32, 2), (16, 8)]


def autotune(batch, R1s, t1s, candidates=CANDIDATES, iters=20, log=None):
    """Pick the fastest tile per level of `batch` (images and cameras set).
    Returns [{"level", "pixels", "tile", "ms": {shape: ms}}] and leaves the
    batch set to the chosen tiles."""
    L = int(batch.params.n_levels)
    best = [(32, 8)] * L
    table = []
    for level in range(L):
        px = sum(batch.levelDims(i, level)[0] * batch.levelDims(i, level)[1]
                 for i in range(batch.n))
        times = {}
        for shape in candidates:
            trial = list(best)
            trial[level] = shape
            batch.setTiles([s[0] for s in trial], [s[1] for s in trial])
            batch.solveR(R1s, t1s)
            a, b = batch.profileLevel(level, iters)
            times[f"{shape[0]}x{shape[1]}"] = a + b
        pick = min(times, key=times.get)
        best[level] = tuple(int(x) for x in pick.split("x"))
        table.append({"level": level, "pixels": px, "tile": list(best[level]), "ms": times})
        if log:
            log(f"level {level} ({px} px): {pick}  " +
                " ".join(f"{k} {v * 1e3:.1f}us" for k, v in sorted(times.items(), key=lambda x: x[1])))
    batch.setTiles([s[0] for s in best], [s[1] for s in best])
    return table


def autotune_single(flow, R1, t1, n_levels, candidates=CANDIDATES, iters=20, log=None):
    """The same search for one ReconFlow handle (rf_set_tiles,
    rf_profile_iterations); images and cameras must be set."""
    best = [(32, 8)] * n_levels
    table = []
    for level in range(n_levels):
        times = {}
        for shape in candidates:
            trial = list(best)
            trial[level] = shape
            flow.setTiles([x[0] for x in trial], [x[1] for x in trial])
            flow.solveR(R1, t1, 5.0)
            a, b = flow.profileLevel(level, iters)
            times[f"{shape[0]}x{shape[1]}"] = a + b
        pick = min(times, key=times.get)
        best[level] = tuple(int(x) for x in pick.split("x"))
        table.append({"level": level, "tile": list(best[level]), "ms": times})
        if log:
            log(f"level {level}: {pick}  " +
                " ".join(f"{k} {v * 1e3:.1f}us" for k, v in sorted(times.items(), key=lambda x: x[1])))
    flow.setTiles([x[0] for x in best], [x[1] for x in best])
    return table


# rf_set_cluster_pixels thresholds: 0 = one iteration per launch everywhere;
# at 1280x720, 1000 = level 5, 4000 = levels 4-5, 16384 = levels 3-5,
# 60000 = levels 2-5 run a warp's iterations in one cluster launch
CLUSTER_CANDIDATES = [0, 1000, 4000, 16384, 60000]


def autotune_iterations_per_launch(flow, R1, t1, candidates=CLUSTER_CANDIDATES, solves=5,
                                   log=None):
    """Time `solves` whole solves of one ReconFlow handle (images and cameras
    set) for each cluster threshold; set and return the fastest as
    {"cluster_px": n, "ms": {n: ms per solve}}."""
    import time

    lib = flow._lib
    times = {}
    for px in candidates:
        lib.rf_set_cluster_pixels(px)
        for _ in range(2):  # the first solve captures the graph
            flow.solveR(R1, t1, 5.0)
        flow.synchronize()
        t0 = time.perf_counter()
        for _ in range(solves):
            flow.solveR(R1, t1, 5.0)
        flow.synchronize()
        times[px] = (time.perf_counter() - t0) * 1000.0 / solves
        if log:
            log(f"cluster levels up to {px} px: {times[px]:.3f} ms per solve")
    best = min(times, key=times.get)
    lib.rf_set_cluster_pixels(best)
    return {"cluster_px": best, "ms": {str(k): v for k, v in times.items()}}


def apply_iterations_per_launch(lib, table):
    """The single-pair table's iterations-per-launch choice (process-wide:
    rf_set_cluster_pixels); tables without one leave the default."""
    ent = table.get("iterations_per_launch") if isinstance(table, dict) else None
    if ent is not None:
        lib.rf_set_cluster_pixels(int(ent["cluster_px"]))


def tiles_for(batch, table):
    """Per-level shapes for `batch` from a saved table: each level takes the
    tile of the table entry whose pixel count is closest (in ratio)."""
    import math

    L = int(batch.params.n_levels)
    tw, th = [], []
    for level in range(L):
        px = sum(batch.levelDims(i, level)[0] * batch.levelDims(i, level)[1]
                 for i in range(batch.n))
        e = min(table, key=lambda r: abs(math.log(max(px, 1) / max(r["pixels"], 1))))
        tw.append(e["tile"][0])
        th.append(e["tile"][1])
    return tw, th


def apply(batch, table):
    tw, th = tiles_for(batch, table)
    batch.setTiles(tw, th)


def apply_single(flow, table, n_levels):
    """Per-level shapes of a single-pair table (by level index; levels past
    the table take its last entry) on a ReconFlow handle."""
    ent = [table[min(l, len(table) - 1)]["tile"] for l in range(n_levels)]
    flow.setTiles([e[0] for e in ent], [e[1] for e in ent])


def main(argv=None):
    import argparse

    from .reconflow import ReconFlowBatch
    from .scene import make_scene
    from .warmstart import SOLVER_WEIGHTS

    ap = argparse.ArgumentParser(description="tile-shape autotuner for the batched solver")
    ap.add_argument("--size", default="1280x720")
    ap.add_argument("--pairs", type=int, default=64)
    ap.add_argument("--levels", type=int, default=6)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--out", required=True)
    ap.add_argument("--single", action="store_true",
                    help="tune one ReconFlow handle (the drop-in path) instead of a batch")
    a = ap.parse_args(argv)
    w, h = (int(x) for x in a.size.split("x"))
    if a.single:
        from .reconflow import ReconFlow

        sc = make_scene(w, h, seed=7000, device="cuda")
        f = ReconFlow()
        sw = SOLVER_WEIGHTS
        f.initializeR(w, h, 1, a.levels, 2.0, 14, sw["lambda_"], 0.0, sw["lambdaf"], sw["lambdams"],
                      sw["alphaTv"], sw["alphaProj"], 0.5, sw["tau"], 1, 5, cvType=5,
                      fix_quirks=sw["fix_quirks"])
        f.setCameraMatrices(sc["K"], sc["K"])
        f.copyImagesToDevice(sc["I0"], sc["I1"])
        table = autotune_single(f, sc["R"], sc["t"], a.levels, iters=a.iters, log=print)
        # iterations per launch, on the schedule the drop-in path runs (the
        # tile search uses a short one)
        g = ReconFlow()
        g.initializeR(w, h, 1, a.levels, 2.0, 14, sw["lambda_"], 0.0, sw["lambdaf"],
                      sw["lambdams"], sw["alphaTv"], sw["alphaProj"], 0.5, sw["tau"], 5, 100,
                      cvType=5, fix_quirks=sw["fix_quirks"])
        g.setCameraMatrices(sc["K"], sc["K"])
        g.copyImagesToDevice(sc["I0"], sc["I1"])
        apply_single(g, table, a.levels)
        ipl = autotune_iterations_per_launch(g, sc["R"], sc["t"], log=print)
        g.close()
        with open(a.out, "w") as fh:
            json.dump({"device": "GB300", "size": a.size, "pairs": 1, "levels": table,
                       "iterations_per_launch": ipl,
                       "command": f"python -m reconflow_gb300.autotune --single --size {a.size}"
                                  f" --out {os.path.basename(a.out)}"}, fh, indent=1)
        f.close()
        return
    scs = [make_scene(w, h, seed=7000 + i, device="cuda") for i in range(a.pairs)]
    b = ReconFlowBatch([(w, h)] * a.pairs, a.levels, method=14, nWarpIters=1, nSolverIters=5,
                       **SOLVER_WEIGHTS)
    for i, sc in enumerate(scs):
        b.setCameraMatrices(i, sc["K"], sc["K"])
        b.copyImagesToDevice(i, sc["I0"], sc["I1"])
    table = autotune(b, [s["R"] for s in scs], [s["t"] for s in scs], iters=a.iters, log=print)
    with open(a.out, "w") as f:
        json.dump({"device": "GB300", "size": a.size, "pairs": a.pairs, "levels": table}, f,
                  indent=1)
    b.close()


if __name__ == "__main__":
    main()
