"""The temporal warm start of frame sequences on the GPU (rf_ws_propagate):
frame k-1's solved depth carried into frame k's coarse inverse-depth grid.
The device grid equals the float32 restatement in oracle/temporal_oracle.py
bit for bit; chained through the warm-start state into a batched refinement
it gives exactly the single-pair warm solve from the same state."""
import numpy as np
import pytest

from helpers import pad_rows

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _depth_plane(inv, valid, s, rng, holes=0.05):
    """A solved-depth plane: 1 / inverse depth where valid, with NaN, 0 and
    negative holes, (h + 1) x s floats."""
    h, w = inv.shape
    with np.errstate(divide="ignore"):
        Z = np.where(valid & (inv > 0), 1.0 / np.maximum(inv, 1e-12), np.nan).astype(np.float32)
    Z = Z * (1 + rng.normal(0, 0.01, Z.shape)).astype(np.float32)
    r = rng.random(Z.shape)
    Z[r < holes / 3] = 0.0
    Z[(r >= holes / 3) & (r < 2 * holes / 3)] = -1.0
    Z[(r >= 2 * holes / 3) & (r < holes)] = np.nan
    out = np.zeros((h + 1, s), np.float32)
    out[:h, :w] = Z
    return out


def test_propagation_matches_float32_oracle(torch_cuda):
    from oracle import temporal_oracle as TO
    from reconflow_gb300 import scene as S
    from reconflow_gb300.warmstart import propagate

    T = torch_cuda
    w, h, s, f = 200, 120, 224, 8
    q = S.make_sequence(w, h, 3, seed=6)
    rng = np.random.default_rng(1)
    planes = [_depth_plane(q["pairs"][k]["inv_depth"], q["pairs"][k]["valid"], s, rng)
              for k in range(2)]
    # a third pair whose points all move behind the camera, a fourth all unknown
    planes.append(np.full((h + 1, s), 2.0, np.float32))
    planes.append(np.full((h + 1, s), np.nan, np.float32))
    Rs = [q["pairs"][0]["R"], q["pairs"][1]["R"], np.eye(3), np.eye(3)]
    ts = [q["pairs"][0]["t"], q["pairs"][1]["t"], np.array([0.0, 0.0, -5.0]), np.zeros(3)]
    Ks = [q["K"]] * 4
    dev = [T.as_tensor(p, device="cuda") for p in planes]
    hn, wn = -(-h // f), -(-w // f)
    for C, ch in ((3, 2), (1, 0)):
        grid = T.full((4, hn, wn, C), 7.0, device="cuda")
        propagate([d.data_ptr() for d in dev], w, h, s, Ks, Rs, ts, f, grid, channel=ch)
        got = grid.cpu().numpy()
        for k in range(4):
            want = TO.propagate_depth_f32(planes[k][:h, :w], Ks[k], Rs[k], ts[k], f, (hn, wn))
            g = np.ascontiguousarray(got[k, ..., ch])
            assert np.array_equal(g.view(np.uint32), want.view(np.uint32)), (C, k)
            if C == 3:  # the other channels are left as they were
                assert np.all(got[k, ..., :2] == 7.0)
        assert np.all(got[2, ..., ch] == 0.0) and np.all(got[3, ..., ch] == 0.0)


def test_sequence_chain_equals_single_pair_warm_solve(torch_cuda, rf):
    """Pair 0 of a sequence solved by the batch; its depth carried into
    frame 1 (rf_ws_propagate), turned into the warm state at pyramid level 2
    (rf_ws_state) and refined for pair 1 in the batch: the result equals the
    single-pair warm solve (rf_solve_warm) from the same warm state bit for
    bit, and the carried grid is close to frame 1's true inverse depth."""
    from oracle import temporal_oracle as TO
    from reconflow_gb300 import scene as S
    from reconflow_gb300.reconflow import ReconFlowBatch
    from reconflow_gb300.warmstart import SOLVER_WEIGHTS, level_intrinsics, propagate, state

    T = torch_cuda
    w, h, L, f, wl = 320, 240, 4, 4, 2
    q = S.make_sequence(w, h, 3, seed=21, device="cuda")
    K = q["K"]
    s = (w + 31) // 32 * 32
    b = ReconFlowBatch([(w, h)], L, method=14, nWarpIters=3, nSolverIters=50, **SOLVER_WEIGHTS)
    b.setCameraMatrices(0, K, K)
    p0, p1 = q["pairs"][0], q["pairs"][1]
    b.copyImagesToDevice(0, pad_rows(q["frames"][0], s), pad_rows(q["frames"][1], s))
    b.solveR([p0["R"]], [p0["t"]])
    # the batch solves on its own stream, the kernels below run on the
    # default stream: order them by synchronising the device in between
    b.synchronize()
    hn, wn = h // f, w // f
    grid = T.zeros((1, hn, wn, 3), device="cuda")
    propagate([b.deviceResults(0)[4]], w, h, s, [K], [p0["R"]], [p0["t"]], f, grid)
    T.cuda.synchronize()
    # the carried grid equals the float32 restatement on the solved depth
    Z0 = b.copy3dToHost(0)[2][:h, :w]
    want = TO.propagate_depth_f32(Z0, K, p0["R"], p0["t"], f, (hn, wn))
    g = grid.cpu().numpy()[0, ..., 2]
    assert np.array_equal(g.view(np.uint32), want.view(np.uint32))
    # and is as close to frame 1's true inverse depth (cell means) as the
    # solve's own depth is to frame 0's: carrying adds no error of its own
    t0 = np.where(p0["valid"], p0["inv_depth"], np.nan)
    with np.errstate(invalid="ignore", divide="ignore"):
        inv0 = 1.0 / Z0
        ok0 = np.isfinite(t0) & np.isfinite(inv0)
        e_solve = float(np.median(np.abs(inv0[ok0] - t0[ok0]) / t0[ok0]))
        truth = np.where(p1["valid"], p1["inv_depth"], np.nan)
        tc = np.nanmean(truth[:hn * f, :wn * f].reshape(hn, f, wn, f), axis=(1, 3))
    ok = np.isfinite(tc) & (g > 0)
    e_carry = float(np.median(np.abs(g[ok] - tc[ok]) / tc[ok]))
    assert ok.sum() > 0.5 * hn * wn
    assert e_carry < 1.5 * e_solve + 0.02, (e_carry, e_solve)
    # warm state for pair 1 at level 2, into the batch's warm planes and into
    # tensors of our own for the single-pair solve (the same kernel, the same
    # inputs: the same bits)
    lw, lh, lsd = b.levelDims(0, wl)
    Kl = level_intrinsics(K, wl)
    up = float(f) / float(2 ** wl)
    b.copyImagesToDevice(0, pad_rows(q["frames"][1], s), pad_rows(q["frames"][2], s))
    state(grid, lw, lh, lsd, up, [Kl], [p1["R"]], [p1["t"]], [b.warmPlanes(0)])
    own = [T.zeros((lh + 1) * lsd, device="cuda") for _ in range(5)]
    state(grid, lw, lh, lsd, up, [Kl], [p1["R"]], [p1["t"]], [[t.data_ptr() for t in own]])
    planes = [t.cpu().numpy().reshape(lh + 1, lsd)[:lh] for t in own]
    T.cuda.synchronize()
    b.solveWarm(wl, [p1["R"]], [p1["t"]], 1, 10)
    u_b, v_b = b.copyOpticalFlowToHost(0)
    b.close()
    wt = SOLVER_WEIGHTS
    single = rf.ReconFlow()
    single.initializeR(w, h, 1, L, 2.0, 14, wt["lambda_"], 0.0, wt["lambdaf"], wt["lambdams"],
                       wt["alphaTv"], wt["alphaProj"], 0.5, wt["tau"], 1, 10, cvType=5,
                       fix_quirks=1)
    single.setCameraMatrices(K, K)
    single.copyImagesToDevice(pad_rows(q["frames"][1], s), pad_rows(q["frames"][2], s))
    single.solveWarm(wl, *planes, p1["R"], p1["t"], 1, 10)
    u_s, v_s = single.copyOpticalFlowToHost()
    single.close()
    for a, c in ((u_b, u_s), (v_b, v_s)):
        a, c = a[:, :w], c[:, :w]
        same = (a.view(np.uint32) == c.view(np.uint32)) | (np.isnan(a) & np.isnan(c))
        assert same.all()
    epe = np.hypot(u_b[:, :w] - p1["flow"][..., 0], v_b[:, :w] - p1["flow"][..., 1])
    assert np.median(epe[p1["valid"]]) < 0.5
