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
    the ceilings.  Network: independent scenes (scene.make_scene); temporal:
    sequences (scene.make_sequence) through TemporalBatchSolver."""
    import torch

    import reconflow_gb300 as R

    from .scene import make_scene, make_sequence
    from .warmstart import (SCHEDULES, SOLVER_WEIGHTS, LearnedBatchSolver, TemporalBatchSolver,
                            WarmStartNet, net_factor)

    R.load()
    ckpt = os.path.join(HERE, "weights", "warmstart_f125.bin")
    entries = {}
    for W, H, source, count, seed0, frames in CALIBRATION:
        sch = SCHEDULES[(W, H)]
        levels = 6
        n = count
        per_px = []
        if source == "network":
            scenes = [make_scene(W, H, seed=seed0 + i, device="cuda") for i in range(n)]
            Ks = [sc["K"] for sc in scenes]
            fct = net_factor(Ks[0])
            net = WarmStartNet(n, H // fct + 1, W // fct + 1, seed=0)
            net.load(ckpt)
            b = R.ReconFlowBatch([(W, H)] * n, levels, method=14, nWarpIters=5,
                                 nSolverIters=100, **SOLVER_WEIGHTS)
            for i, sc in enumerate(scenes):
                b.setCameraMatrices(i, sc["K"], sc["K"])
                b.copyImagesToDevice(i, sc["I0"], sc["I1"])
            ls = LearnedBatchSolver(net, b, (W, H), Ks[0], sch["warm_level"], sch["warps"],
                                    sch["iters"])
            ls.solve(Ks, [sc["R"] for sc in scenes], [sc["t"] for sc in scenes])
            per_px += list(b.energies() / (W * H))
            b.close()
            net.close()
            seeds = [seed0, seed0 + n - 1]
        else:
            seqs = [make_sequence(W, H, frames, seed=seed0 + j, device="cuda") for j in range(n)]
            Ks = [q["K"] for q in seqs]
            fct = net_factor(Ks[0])
            net = WarmStartNet(n, H // fct + 1, W // fct + 1, seed=0)
            net.load(ckpt)
            b = R.ReconFlowBatch([(W, H)] * n, levels, method=14, nWarpIters=5,
                                 nSolverIters=100, **SOLVER_WEIGHTS)
            for i, K in enumerate(Ks):
                b.setCameraMatrices(i, K, K)
            s = b.strides[0]
            pad = lambda a: np.pad(a, ((0, 0), (0, s - W))).astype(np.float32)  # noqa: E731
            ts_ = TemporalBatchSolver(net, b, (W, H), Ks[0], sch["warm_level"], sch["warps"],
                                      sch["iters"])
            guard = SequenceGuard(n)
            ratios = []
            for k in range(frames - 1):
                for i, q in enumerate(seqs):
                    b.copyImagesToDevice(i, pad(q["frames"][k]), pad(q["frames"][k + 1]))
                Rs = [q["pairs"][k]["R"] for q in seqs]
                tt = [q["pairs"][k]["t"] for q in seqs]
                if k == 0:
                    ts_.first(Ks, Rs, tt)
                else:
                    ts_.next(Ks, [q["pairs"][k - 1]["R"] for q in seqs],
                             [q["pairs"][k - 1]["t"] for q in seqs], Rs, tt)
                e_k = b.energies()
                for i in range(n):
                    q = guard.ratio(i, e_k[i] / (W * H))
                    if q is not None and np.isfinite(q):
                        ratios.append(q)
                    guard.over(i, e_k[i], W * H, None)
                per_px += list(e_k / (W * H))
            b.close()
            net.close()
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
            tail = ""
        else:
            r = np.array(ratios)
            ent.update(history=HISTORY, history_factor=HISTORY_FACTOR,
                       history_ratio_median=float(np.median(r)),
                       history_ratio_p99=float(np.percentile(r, 99)),
                       history_ratio_max=float(r.max()),
                       history_flags=int((r > HISTORY_FACTOR).sum()))
            tail = (f"; history ratio median {ent['history_ratio_median']:.3f}, max "
                    f"{ent['history_ratio_max']:.3f}, flags {ent['history_flags']}")
        entries[key(W, H, source)] = ent
        log(f"{key(W, H, source)}: {e.size} pairs, energy per pixel median "
            f"{ent['energy_per_px_median']:.3f}, max {top:.3f}" + tail)
    table = {"margin": MARGIN, "entries": entries,
             "command": "python -m reconflow_gb300.fallback --calibrate",
             "what": "network: ceiling = (1 + margin) x the largest learned-solution energy "
                     "per pixel of the calibration set; temporal: a pair falls back when its "
                     "energy per pixel exceeds history_factor x the median of its sequence's "
                     "last `history` pairs (the ratio's distribution on the calibration "
                     "sequences recorded)"}
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
