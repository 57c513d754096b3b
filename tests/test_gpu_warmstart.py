"""The learned warm start on the GPU: its tensor-core forward and backward
kernels against the FP64 oracle of the network (gradient check), training
that reduces the loss, and the warm-started solve it feeds."""
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


def _rand_case(rng, B, H, W):
    x = rng.normal(0, 0.5, (B, H, W, 16)).astype(np.float32)
    H2, W2 = (H + 1) // 2, (W + 1) // 2
    t16 = rng.normal(0, 1, (B, H2, W2, 8)).astype(np.float32)
    t8 = rng.normal(0, 1, (B, H, W, 8)).astype(np.float32)
    m16 = (rng.random((B, H2, W2)) < 0.8).astype(np.float32)
    m8 = (rng.random((B, H, W)) < 0.8).astype(np.float32)
    return x, t16, m16, t8, m8


def test_gradients_match_fp64_oracle(torch_cuda):
    from oracle import cnn_oracle as CO
    from reconflow_gb300.warmstart import WarmStartNet

    rng = np.random.default_rng(0)
    B, H, W = 2, 12, 10
    net = WarmStartNet(B, H, W, seed=3)
    params = net.params()
    x, t16, m16, t8, m8 = _rand_case(rng, B, H, W)
    T = lambda a: torch_cuda.as_tensor(a, device="cuda")  # noqa: E731
    w = (1.0, 1.0, 10.0)
    loss = net.backward(T(x), T(t16), T(m16), T(t8), T(m8), w)
    g = net.grads()
    o16, o8 = net.forward(T(x))
    gref, lref, f = CO.backward(params.astype(np.float64), x, t16, m16, t8, m8, w)
    # forward outputs (FP32 accumulation of BF16 products vs FP64)
    np.testing.assert_allclose(o8.cpu().numpy(), f["o8"], rtol=0, atol=2e-2 * np.abs(f["o8"]).max())
    np.testing.assert_allclose(o16.cpu().numpy(), f["o16"], rtol=0,
                               atol=2e-2 * np.abs(f["o16"]).max())
    assert loss == pytest.approx(lref, rel=2e-2)
    # per-layer gradient tensors
    off = 0
    for cin, cout, _, _ in CO.LAYERS:
        for n in (cout * 9 * cin, cout):
            a, b = g[off:off + n], gref[off:off + n]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            assert rel < 3e-2, (cin, cout, n, rel)
            off += n
    assert off == net.n_params
    # no tensor-core launch gave up on its bounded mbarrier waits
    assert net.wait_gave_up() is False


def test_wait_give_up_is_reported_and_recovers(torch_cuda):
    """The bounded ring-slot wait of the tensor-core GEMM: with the test hook
    its first wait gives up at once (the MMAs it waited for still complete,
    so nothing hangs); the launch reports it through rf_cnn_status, and a
    normal forward pass afterwards is bit-identical to one before."""
    from reconflow_gb300.warmstart import WarmStartNet

    rng = np.random.default_rng(5)
    B, H, W = 2, 40, 48
    net = WarmStartNet(B, H, W, seed=7)
    x = torch_cuda.as_tensor(rng.normal(0, 0.5, (B, H, W, 16)).astype(np.float32),
                             device="cuda")
    ref16, ref8 = (t.clone() for t in net.forward(x))
    assert net.wait_gave_up() is False
    net.set_test_wait_limit(0)
    net.forward(x)
    assert net.wait_gave_up() is True
    net.set_test_wait_limit(-1)
    o16, o8 = net.forward(x)
    assert net.wait_gave_up() is False
    assert torch_cuda.equal(o16, ref16) and torch_cuda.equal(o8, ref8)
    net.close()


def test_training_reduces_loss_and_is_deterministic(torch_cuda):
    from reconflow_gb300.warmstart import WarmStartNet, train

    rng = np.random.default_rng(1)
    B, H, W = 8, 16, 20
    x = rng.normal(0, 0.5, (32, H, W, 16)).astype(np.float32)
    # a learnable target: a fixed linear map of the input channels
    A = rng.normal(0, 0.3, (16, 8)).astype(np.float32)
    t8 = x @ A
    t16 = t8[:, ::2, ::2]
    m8 = np.ones((32, H, W), np.float32)
    m16 = np.ones((32, H // 2, W // 2), np.float32)
    losses, params = [], []
    for _ in range(2):
        net = WarmStartNet(B, H, W, seed=5)
        hist = train(net, (x, t16, m16, t8, m8), epochs=15, batch=B, lr=2e-3, seed=0)
        losses.append(hist)
        params.append(net.params())
        net.close()
    assert losses[0][-1] < 0.5 * losses[0][0]
    # same seed, same data: identical weights (the reported loss is summed with
    # atomics, so only it may differ in the last bits)
    np.testing.assert_array_equal(params[0].view(np.uint32), params[1].view(np.uint32))
    np.testing.assert_allclose(losses[0], losses[1], rtol=1e-12)


def _features_ref(I0, I1, K, R, t, factor):
    """numpy restatement of rf_ws_features (float64)."""
    from reconflow_gb300.warmstart import box_down

    c0, c1 = box_down(I0.astype(np.float64), factor), box_down(I1.astype(np.float64), factor)
    hn, wn = c0.shape
    fx, fy, cx, cy = K[0, 0] / factor, K[1, 1] / factor, K[0, 2] / factor, K[1, 2] / factor
    Kc = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1.0]])
    ys, xs = np.mgrid[0:hn, 0:wn].astype(np.float64)
    a = np.stack([xs, ys, np.ones_like(xs)], -1) @ (Kc @ R @ np.linalg.inv(Kc)).T
    b = Kc @ t

    def samp(x, y):
        x = np.clip(x, 0, wn - 1)
        y = np.clip(y, 0, hn - 1)
        x0 = np.minimum(x.astype(int), max(wn - 2, 0))
        y0 = np.minimum(y.astype(int), max(hn - 2, 0))
        x1, y1 = np.minimum(x0 + 1, wn - 1), np.minimum(y0 + 1, hn - 1)
        ax, ay = x - x0, y - y0
        return ((1 - ay) * ((1 - ax) * c1[y0, x0] + ax * c1[y0, x1]) +
                ay * ((1 - ax) * c1[y1, x0] + ax * c1[y1, x1]))

    out = np.zeros((hn, wn, 16))
    out[..., 0], out[..., 1] = c0 - 0.5, c1 - 0.5
    for k in range(12):
        rho = 0.05 * k
        den = a[..., 2] + rho * b[2]
        c = np.abs(samp((a[..., 0] + rho * b[0]) / den, (a[..., 1] + rho * b[1]) / den) - c0) * 10
        out[..., 2 + k] = np.where(den > 1e-6, c, 1.0)
    rm = 0.25
    den = a[..., 2] + rm * b[2]
    out[..., 14] = (b[0] * den - (a[..., 0] + rm * b[0]) * b[2]) / den ** 2 * 0.1
    out[..., 15] = (b[1] * den - (a[..., 1] + rm * b[1]) * b[2]) / den ** 2 * 0.1
    return out


def test_features_match_numpy(torch_cuda, rf):
    from reconflow_gb300.scene import make_scene
    from reconflow_gb300.warmstart import features

    T = torch_cuda
    w, h, s, f = 200, 120, 224, 4
    scs = [make_scene(w, h, seed=31 + i) for i in range(3)]
    dev = [(T.as_tensor(pad_rows(sc["I0"], s), device="cuda"),
            T.as_tensor(pad_rows(sc["I1"], s), device="cuda")) for sc in scs]
    out = T.empty((3, h // f, w // f, 16), device="cuda")
    features([d[0].data_ptr() for d in dev], [d[1].data_ptr() for d in dev], w, h, s, f,
             [sc["K"] for sc in scs], [sc["R"] for sc in scs], [sc["t"] for sc in scs], out)
    got = out.cpu().numpy()
    for i, sc in enumerate(scs):
        ref = _features_ref(sc["I0"], sc["I1"], sc["K"], sc["R"], sc["t"], f)
        # FP32 on the GPU against FP64: costs are differences of samples
        np.testing.assert_allclose(got[i], ref, rtol=1e-4, atol=2e-4)


def test_state_matches_numpy(torch_cuda, rf):
    from reconflow_gb300.warmstart import level_intrinsics, state

    T = torch_cuda
    rng = np.random.default_rng(4)
    n, hn, wn, C = 2, 9, 13, 8
    net = rng.uniform(0.1, 0.5, (n, hn, wn, C)).astype(np.float32)
    net[1, 2, 3, 2] = -1.0  # clamped to 0.02
    w, h, s, up = 26, 18, 32, 2.0
    K = np.array([[100.0, 0, 52], [0, 100.0, 36], [0, 0, 1]])
    Kl = level_intrinsics(K, 2)
    Rs = [np.eye(3), np.array([[0.9998, -0.02, 0], [0.02, 0.9998, 0], [0, 0, 1.0]])]
    ts = [np.array([0.1, 0, 0]), np.array([0, 0.05, 0.08])]
    planes = [[T.zeros((h + 1) * s, device="cuda") for _ in range(5)] for _ in range(n)]
    state(T.as_tensor(net, device="cuda"), w, h, s, up, [Kl, Kl], Rs, ts,
          [[p.data_ptr() for p in pl] for pl in planes])
    fx, cx, cy = Kl[0, 0], Kl[0, 2], Kl[1, 2]
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    for i in range(n):
        sx = np.clip((xs + 0.5) / up - 0.5, 0, wn - 1)
        sy = np.clip((ys + 0.5) / up - 0.5, 0, hn - 1)
        x0, y0 = sx.astype(int), sy.astype(int)
        x1, y1 = np.minimum(x0 + 1, wn - 1), np.minimum(y0 + 1, hn - 1)
        ax, ay = sx - x0, sy - y0
        r = net[i, ..., 2].astype(np.float64)
        rho = (1 - ay) * ((1 - ax) * r[y0, x0] + ax * r[y0, x1]) + ay * ((1 - ax) * r[y1, x0] + ax * r[y1, x1])
        rho = np.clip(rho, 0.02, 2.0)
        Z = 1 / rho
        P = np.stack([Z * (xs - cx) / fx, Z * (ys - cy) / Kl[1, 1], Z], -1)
        P2 = P @ Rs[i].T + ts[i]
        want = [fx * P2[..., 0] / P2[..., 2] + cx - xs, fx * P2[..., 1] / P2[..., 2] + cy - ys,
                P[..., 0], P[..., 1], P[..., 2]]
        for k in range(5):
            got = planes[i][k].cpu().numpy().reshape(h + 1, s)[:h, :w]
            np.testing.assert_allclose(got, want[k], rtol=2e-5, atol=2e-5)


def test_learned_batch_pipeline_runs(torch_cuda, rf):
    """Features -> network -> warm state -> warm-started batched solve on two
    640x480 pairs with an untrained network: finite results, and the warm
    solve of a pair equals the single-pair warm solve from the same state."""
    from reconflow_gb300.reconflow import ReconFlowBatch
    from reconflow_gb300.scene import make_scene
    from reconflow_gb300.warmstart import (SOLVER_WEIGHTS, LearnedBatchSolver, WarmStartNet,
                                           level_intrinsics)

    scs = [make_scene(640, 480, seed=77 + i, device="cuda") for i in range(2)]
    net = WarmStartNet(2, 120, 160, seed=0)
    bt = ReconFlowBatch([(640, 480)] * 2, 5, method=14, nWarpIters=3, nSolverIters=50,
                        **SOLVER_WEIGHTS)
    for i, sc in enumerate(scs):
        bt.setCameraMatrices(i, sc["K"], sc["K"])
        bt.copyImagesToDevice(i, pad_rows(sc["I0"], 640), pad_rows(sc["I1"], 640))
    ls = LearnedBatchSolver(net, bt, (640, 480), scs[0]["K"], warm_level=2, warps=1, iters=10)
    assert ls.factor == 4 and (ls.hn, ls.wn) == (120, 160)
    # without set_stream every kernel of the pipeline goes on the batch's own
    # (non-blocking) stream, ordered with the solve
    assert ls.stream == bt.stream() != 0
    Ks, Rs, ts = [sc["K"] for sc in scs], [sc["R"] for sc in scs], [sc["t"] for sc in scs]
    ls.solve(Ks, Rs, ts)
    u, v = bt.copyOpticalFlowToHost(1)
    assert np.isfinite(u[:, :640]).mean() > 0.99
    # the same warm state through the single-pair path
    from reconflow_gb300.warmstart import state

    T = torch_cuda
    lw, lh, lsd = bt.levelDims(1, 2)
    Kl = level_intrinsics(scs[1]["K"], 2)
    tens = [T.zeros((lh + 1) * lsd, device="cuda") for _ in range(5)]
    state(ls.o8[1:2], lw, lh, lsd, ls.up, [Kl], [Rs[1]], [ts[1]], [[t.data_ptr() for t in tens]])
    planes = [t.cpu().numpy().reshape(lh + 1, lsd)[:lh] for t in tens]
    f = rf.ReconFlow()
    f.initializeR(640, 480, 1, 5, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25, 3,
                  50, cvType=5, fix_quirks=1)
    f.setCameraMatrices(scs[1]["K"], scs[1]["K"])
    f.copyImagesToDevice(pad_rows(scs[1]["I0"], 640), pad_rows(scs[1]["I1"], 640))
    f.solveWarm(2, *planes, Rs[1], ts[1], 1, 10)
    u1, _ = f.copyOpticalFlowToHost()
    f.close()
    same = (u1[:, :640].view(np.uint32) == u[:, :640].view(np.uint32)) | (
        np.isnan(u1[:, :640]) & np.isnan(u[:, :640]))
    assert same.all()


def test_direct_convolutions_match_the_gemm_path(torch_cuda, monkeypatch):
    """Inference runs the stride-1 layers as direct 3x3 convolutions on
    padded activations (TMA-staged slabs, nine shifted-view MMAs per 16
    input channels); RF_CNN_DIRECT=0 runs every layer as the im2col GEMM.
    Both accumulate BF16 products in FP32, in different orders, so the
    outputs agree to the BF16 rounding of the activations.  One network
    serves calls of several sizes up to its allocation, in turn (the padded
    layout follows the call's frame size), with fewer images than allocated
    too."""
    import os

    from reconflow_gb300.warmstart import WarmStartNet

    ckpt = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "reconflow_gb300", "weights", "warmstart_f125.bin")
    rng = np.random.default_rng(11)
    alloc = (4, 91, 161)
    calls = [(3, 90, 160), (4, 91, 161), (2, 12, 10), (1, 37, 45), (3, 90, 160)]
    xs = [torch_cuda.as_tensor(rng.normal(0, 0.5, (B, H, W, 16)).astype(np.float32),
                               device="cuda") for B, H, W in calls]
    xs[4] = xs[0]
    outs = {}
    for flag in ("0", "1"):
        monkeypatch.setenv("RF_CNN_DIRECT", flag)
        net = WarmStartNet(*alloc, seed=5)
        net.load(ckpt)
        outs[flag] = []
        for x in xs:
            o16, o8 = net.forward(x)
            outs[flag].append((o16.cpu().numpy(), o8.cpu().numpy()))
        assert net.wait_gave_up() is False
        net.close()
    for (B, H, W), ref, got in zip(calls, outs["0"], outs["1"]):
        for a, b in zip(ref, got):
            scale = float(np.abs(a).max())
            assert np.isfinite(b).all()
            assert np.abs(a - b).max() <= 3e-2 * scale, (B, H, W, np.abs(a - b).max(), scale)
            assert np.abs(a - b).mean() <= 3e-3 * scale, (B, H, W, np.abs(a - b).mean(), scale)
        if H * W > 1000:  # a different accumulation order ran
            assert not np.array_equal(ref[1], got[1])
    # the same call before and after other sizes: identical results
    for a, b in zip(outs["1"][0], outs["1"][4]):
        assert np.array_equal(a, b)
