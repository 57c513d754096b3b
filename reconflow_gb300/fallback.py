"""The learned path's fallback test, in a form a deployment can run.

A warm-started solve is replaced by the full plain solve when its energy
(``rf_batch_energies``: brightness residual + flow TV + truncated
reprojection residual, non-finite pixels at the terms' caps) is too high.
Comparing it with the same pair's plain-solve energy would need the plain
solve that the warm start exists to avoid, so the reference energy is a
per-pixel ceiling measured beforehand: the largest energy per pixel of the
learned solutions of calibration scenes (seeds no bench or test uses) of the
same frame size and warm-start source, raised by the margin.  A solution
above it (or with a non-finite energy) falls back.

Measured on the calibration and held-out sets (see ``calibrate``): at 720p
the learned energy per pixel spans 1.0 .. 3.2 while the plain solve's spans
0.7 .. 30, so the pair's own plain energy mostly says how badly the plain
solve diverged, not how good the learned solution is; the ceiling flags the
learned solutions that are outliers among learned solutions.

Along a sequence (the temporal warm start) the energy per pixel drifts with
the scene: over 32 frames of a moving camera both the learned and the plain
solutions' energies per pixel grow about threefold, so a fixed ceiling
measured on short sequences flags correct solutions late in a stream.  There
the reference is the sequence's own recent history: a pair falls back when
its energy per pixel exceeds ``HISTORY_FACTOR`` times the median of the
sequence's last ``HISTORY`` pairs (``SequenceGuard``); the first pair of a
sequence, warm-started by the network, uses the network ceiling.  The
history holds every pair's learned energy, accepted or not, so a lasting
change of the scene is accepted after two pairs while a single outlier is
not.  The calibration records the distribution of that ratio on its
sequences.

The table is ``tuning/fallback_energy.json``, written by
``python -m reconflow_gb300.fallback --calibrate``.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning", "fallback_energy.json")
MARGIN = 0.02
HISTORY = 3
HISTORY_FACTOR = 2.0

# calibration sets: (width, height, source, count, first seed); sequences
# give count - 1 pairs per sequence of `frames` frames
CALIBRATION = [
    (1280, 720, "network", 128, 8000, None),
    (1920, 1080, "network", 16, 8500, None),
    (3840, 2160, "network", 16, 8700, None),
    (1920, 1080, "temporal", 2, 8800, 33),
    (3840, 2160, "temporal", 2, 8900, 33),
]


def key(width: int, height: int, source: str) -> str:
    return f"{width}x{height}/{source}"


def load(path: str = TABLE) -> dict:
    with open(path) as fh:
        return json.load(fh)


def ceiling(table: dict, width: int, height: int, source: str = "network"):
    """Energy-per-pixel ceiling for this frame size and warm-start source,
    or None when the table has no ceiling for it (temporal sources are
    tested against their sequence's history instead)."""
    ent = table.get("entries", {}).get(key(width, height, source))
    return None if ent is None or "ceiling" not in ent else float(ent["ceiling"])


def over(energy: float, pixels: int, ceil) -> bool:
    """True: fall back to the plain solve.  A non-finite energy always
    falls back; without a ceiling only that does."""
    if not np.isfinite(energy):
        return True
    return ceil is not None and energy / pixels > ceil


class SequenceGuard:
    """The fallback test along sequences: one history per sequence."""

    def __init__(self, n: int, factor: float = HISTORY_FACTOR, length: int = HISTORY):
        self.factor = factor
        self.length = length
        self.hist = [[] for _ in range(n)]

    def reset(self) -> None:
        for h in self.hist:
            h.clear()

    def ratio(self, i: int, energy_per_px: float):
        """Energy per pixel over the median of sequence i's history (None
        while the history is empty)."""
        h = self.hist[i]
        return None if not h else energy_per_px / float(np.median(h))

    def over(self, i: int, energy: float, pixels: int, first_ceil) -> bool:
        """True: fall back.  Non-finite energies always fall back (and are
        kept out of the history); the first pair of a sequence is tested
        against `first_ceil` (the network ceiling, None: no test), later
        pairs against the factor x the history median."""
        if not np.isfinite(energy):
            return True
        e = energy / pixels
        q = self.ratio(i, e)
        bad = (first_ceil is not None and e > first_ceil) if q is None else q > self.factor
        self.hist[i].append(e)
        del self.hist[i][:-self.length]
        return bool(bad)


def calibrate(out: str = TABLE, log=print) -> dict:
    """Solve the calibration sets with the learned path on the GPU and write
    the table.  Network: independent scenes (scene.make_scene); temporal:
    sequences (scene.make_sequence) through TemporalBatchSolver, with a
    flagged pair re-solved by the plain single-pair solver and its result
    imported before the next frame, as a deployment does.  For validation
    every pair is also solved with the plain batched schedule (outside the
    test itself): the table records how many pairs the test flags, how many
    have an energy over (1 + margin) x their plain solve's, and how many
    both."""
    import torch

    import reconflow_gb300 as R

    from .scene import make_scene, make_sequence
    from .warmstart import (SCHEDULES, SOLVER_WEIGHTS, LearnedBatchSolver, TemporalBatchSolver,
                            WarmStartNet, net_factor)

    R.load()
    ckpt = os.path.join(HERE, "weights", "warmstart_f125.bin")
    levels, plain_warps, plain_iters = 6, 5, 100
    entries = {}
    table0 = {}
    for W, H, source, count, seed0, frames in CALIBRATION:
        sch = SCHEDULES[(W, H)]
        n = count
        npx = W * H

        def batch(warps, iters):
            return R.ReconFlowBatch([(W, H)] * n, levels, method=14, nWarpIters=warps,
                                    nSolverIters=iters, **SOLVER_WEIGHTS)

        per_px, flags, over_plain = [], [], []
        ratios = []
        if source == "network":
            scenes = [make_scene(W, H, seed=seed0 + i, device="cuda") for i in range(n)]
            Ks = [sc["K"] for sc in scenes]
            Rs, ts = [sc["R"] for sc in scenes], [sc["t"] for sc in scenes]
            fct = net_factor(Ks[0])
            net = WarmStartNet(n, H // fct + 1, W // fct + 1, seed=0)
            net.load(ckpt)
            b, pb = batch(plain_warps, plain_iters), batch(plain_warps, plain_iters)
            for i, sc in enumerate(scenes):
                for x in (b, pb):
                    x.setCameraMatrices(i, sc["K"], sc["K"])
                    x.copyImagesToDevice(i, sc["I0"], sc["I1"])
            ls = LearnedBatchSolver(net, b, (W, H), Ks[0], sch["warm_level"], sch["warps"],
                                    sch["iters"])
            ls.solve(Ks, Rs, ts)
            e = b.energies()
            pb.solveR(Rs, ts)
            ep = pb.energies()
            per_px += list(e / npx)
            over_plain += [bool(np.isfinite(a) and (not np.isfinite(c) or a > (1 + MARGIN) * c))
                           for a, c in zip(e, ep)]
            for x in (b, pb, net):
                x.close()
            seeds = [seed0, seed0 + n - 1]
        else:
            seqs = [make_sequence(W, H, frames, seed=seed0 + j, device="cuda") for j in range(n)]
            Ks = [q["K"] for q in seqs]
            fct = net_factor(Ks[0])
            net = WarmStartNet(n, H // fct + 1, W // fct + 1, seed=0)
            net.load(ckpt)
            b, pb = batch(plain_warps, plain_iters), batch(plain_warps, plain_iters)
            for i, K in enumerate(Ks):
                b.setCameraMatrices(i, K, K)
                pb.setCameraMatrices(i, K, K)
            f = R.ReconFlow()
            wt = SOLVER_WEIGHTS
            f.initializeR(W, H, 1, levels, 2.0, 14, wt["lambda_"], 0.0, wt["lambdaf"],
                          wt["lambdams"], wt["alphaTv"], wt["alphaProj"], 0.5, wt["tau"],
                          plain_warps, plain_iters, cvType=5, fix_quirks=wt["fix_quirks"])
            s = b.strides[0]
            pad = lambda a: np.pad(a, ((0, 0), (0, s - W))).astype(np.float32)  # noqa: E731
            ts_ = TemporalBatchSolver(net, b, (W, H), Ks[0], sch["warm_level"], sch["warps"],
                                      sch["iters"])
            guard = SequenceGuard(n)
            ceil_net = table0.get(key(W, H, "network"), {}).get("ceiling")
            for k in range(frames - 1):
                for i, q in enumerate(seqs):
                    for x in (b, pb):
                        x.copyImagesToDevice(i, pad(q["frames"][k]), pad(q["frames"][k + 1]))
                Rs = [q["pairs"][k]["R"] for q in seqs]
                tt = [q["pairs"][k]["t"] for q in seqs]
                if k == 0:
                    ts_.first(Ks, Rs, tt)
                else:
                    ts_.next(Ks, [q["pairs"][k - 1]["R"] for q in seqs],
                             [q["pairs"][k - 1]["t"] for q in seqs], Rs, tt)
                e = b.energies()
                pb.solveR(Rs, tt)
                ep = pb.energies()
                for i in range(n):
                    q = guard.ratio(i, e[i] / npx)
                    if q is not None and np.isfinite(q):
                        ratios.append(q)
                    bad = guard.over(i, e[i], npx, ceil_net)
                    flags.append(bad)
                    over_plain.append(bool(np.isfinite(e[i]) and (
                        not np.isfinite(ep[i]) or e[i] > (1 + MARGIN) * ep[i])))
                    if bad:
                        f.setCameraMatrices(Ks[i], Ks[i])
                        f.copyImagesToDeviceFromDevice(*b.imagePlanes(i, 0), s)
                        f.solveR(Rs[i], tt[i], 5.0)
                        b.importResults(i, f.deviceResults(), f.stride)
                per_px += list(e / npx)
            for x in (b, pb, net, f):
                x.close()
            seeds = [seed0, seed0 + n - 1]
        torch.cuda.synchronize()
        e = np.array(per_px)
        finite = e[np.isfinite(e)]
        top = float(finite.max()) if finite.size else float("nan")
        ent = {"pairs": int(e.size), "seeds": seeds, "frames": frames,
               "energy_per_px_median": float(np.median(finite)) if finite.size else None,
               "energy_per_px_max": top}
        if source == "network":
            ent["ceiling"] = top * (1.0 + MARGIN)
            flags = [False] * len(per_px)  # the ceiling is their maximum: nothing is over
        else:
            r = np.array(ratios)
            ent.update(history=HISTORY, history_factor=HISTORY_FACTOR,
                       history_ratio_median=float(np.median(r)),
                       history_ratio_p99=float(np.percentile(r, 99)),
                       history_ratio_max=float(r.max()))
        ent.update(flagged=int(sum(flags)), over_plain_margin=int(sum(over_plain)),
                   flagged_and_over=int(sum(a and c for a, c in zip(flags, over_plain))))
        entries[key(W, H, source)] = ent
        table0 = entries
        log(f"{key(W, H, source)}: {e.size} pairs, energy per pixel median "
            f"{ent['energy_per_px_median']:.3f}, max {top:.3f}; flagged {ent['flagged']}, over "
            f"the plain solve's energy {ent['over_plain_margin']}, both "
            f"{ent['flagged_and_over']}"
            + ("" if source == "network" else
               f"; history ratio median {ent['history_ratio_median']:.3f}, "
               f"max {ent['history_ratio_max']:.3f}"))
    table = {"margin": MARGIN, "entries": entries,
             "command": "python -m reconflow_gb300.fallback --calibrate",
             "what": "network: ceiling = (1 + margin) x the largest learned-solution energy "
                     "per pixel of the calibration set; temporal: a pair falls back when its "
                     "energy per pixel exceeds history_factor x the median of its sequence's "
                     "last `history` pairs (the first pair: the network ceiling); flagged / "
                     "over_plain_margin / flagged_and_over: pairs the test flags, pairs whose "
                     "energy exceeds (1 + margin) x their plain solve's, and both"}
    with open(out, "w") as fh:
        json.dump(table, fh, indent=1)
    return table


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if "--calibrate" in argv:
        out = argv[argv.index("--out") + 1] if "--out" in argv else TABLE
        calibrate(out)
    else:
        print(json.dumps(load(), indent=1))


if __name__ == "__main__":
    main()
