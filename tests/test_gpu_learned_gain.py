"""What the trained warm-start network gains (tests the committed checkpoint).

On seeded 640x480 pairs the solve is refined from pyramid level 2 with one
cheap schedule, starting either from the network's inverse depth or from the
same pipeline fed a constant inverse depth (a fronto-parallel plane at 5 m:
the method without the network).  The network's start must end far more
accurate, and close to the full plain coarse-to-fine solve."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CKPT = os.path.join(ROOT, "reconflow_gb300", "weights", "warmstart_f125.bin")


def _epe(b, scs, w):
    meds, means = [], []
    for i, sc in enumerate(scs):
        u, v = b.copyOpticalFlowToHost(i)
        e = np.sqrt((u[:, :w] - sc["flow"][..., 0]) ** 2 + (v[:, :w] - sc["flow"][..., 1]) ** 2)
        e = e[sc["valid"]]
        e = np.where(np.isfinite(e), e, 1e4)
        meds.append(np.median(e))
        means.append(e.mean())
    return float(np.mean(meds)), float(np.mean(means))


def test_network_warm_start_beats_the_same_schedule_without_it(rf):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from reconflow_gb300.reconflow import ReconFlowBatch
    from reconflow_gb300.scene import make_scene
    from reconflow_gb300.warmstart import (SOLVER_WEIGHTS, LearnedBatchSolver, WarmStartNet,
                                           level_intrinsics, state)

    W, H, n = 640, 480, 4
    scs = [make_scene(W, H, seed=5000 + i, device="cuda") for i in range(n)]
    Ks, Rs, ts = [s["K"] for s in scs], [s["R"] for s in scs], [s["t"] for s in scs]
    b = ReconFlowBatch([(W, H)] * n, 5, method=14, nWarpIters=3, nSolverIters=50,
                       **SOLVER_WEIGHTS)
    for i, sc in enumerate(scs):
        b.setCameraMatrices(i, sc["K"], sc["K"])
        b.copyImagesToDevice(i, sc["I0"], sc["I1"])
    b.solveR(Rs, ts)
    plain_med, plain_mean = _epe(b, scs, W)

    net = WarmStartNet(n, 120, 160, seed=0)
    net.load(CKPT)
    sched = dict(warps=[1, 1, 2], iters=[10, 10, 20])
    ls = LearnedBatchSolver(net, b, (W, H), Ks[0], warm_level=2, **sched)
    ls.solve(Ks, Rs, ts)
    learned_med, learned_mean = _epe(b, scs, W)

    # the same refinement from a constant inverse depth (no network)
    flat = torch.zeros_like(ls.o8)
    flat[..., 2] = 0.2
    lw, lh, lsd = b.levelDims(0, 2)
    state(flat, lw, lh, lsd, ls.up, [level_intrinsics(K, 2) for K in Ks], Rs, ts, ls.planes)
    b.solveWarm(2, Rs, ts, sched["warps"], sched["iters"])
    flat_med, flat_mean = _epe(b, scs, W)
    b.close()
    net.close()
    print(f"median / mean EPE: plain {plain_med:.3f} / {plain_mean:.3f}, learned "
          f"{learned_med:.3f} / {learned_mean:.3f}, flat start {flat_med:.3f} / {flat_mean:.3f}")
    assert learned_med < 0.5 * flat_med
    assert learned_mean < 0.5 * flat_mean
    assert learned_med < plain_med + 0.15
