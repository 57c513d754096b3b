"""Full-schedule parity on the GPU through the reference-facing API.

The CUDA solver (C ABI, via the ReconFlow / CudaFlow mirror) must reproduce
the FP32 reference-semantics oracle bit for bit after the whole
coarse-to-fine schedule, for every method, input type and reference quirk
switch; against the FP64 oracle it must reach the same accuracy on scenes
with known ground truth.
"""
import numpy as np
import pytest

from helpers import align_up, assert_bitexact, pad_rows, textured_pair

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _K(w, h):
    f = 500.0 * w / 640.0
    return np.array([[f, 0, w / 2.0], [0, f, h / 2.0], [0, 0, 1.0]])


def _pose(seed):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=3)
    a /= np.linalg.norm(a)
    ang = np.radians(rng.uniform(0.5, 2.0))
    Kx = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = np.eye(3) + np.sin(ang) * Kx + (1 - np.cos(ang)) * Kx @ Kx
    t = rng.normal(size=3)
    t = 0.1 * t / np.linalg.norm(t)
    return R, t


def run_gpu(rf, w, h, L, method, I0, I1, K, R, t, input_type=0, prior=None, **kw):
    from reconflow_gb300.reconflow import CV_8U, CV_16U, CV_32F, CV_8UC3

    cv = {0: CV_32F, 1: CV_8UC3, 2: CV_8U, 3: CV_16U}[input_type]
    if method == 0:
        f = rf.CudaFlow()
        f.initialize(w, h, 1, cv, L, 2.0, 0, kw.get("lam", 50.0), 0.0, kw.get("theta", 0.33),
                     kw.get("tau", 0.25), kw["warps"], kw["iters"])
        f.copyImagesToDevice(I0, I1)
        f.solveOpticalFlow()
        u, v = f.copyOpticalFlowToHost()
        return {"u": u, "v": v}, f
    f = rf.ReconFlow()
    f.initializeR(w, h, 1, L, 2.0, method, kw.get("lam", 50.0), 0.0, kw.get("lambdaf", 0.1),
                  kw.get("lambdams", 100.0), kw.get("alpha_tv", 1 / 0.33), kw.get("alpha_proj", 60.0),
                  kw.get("alpha_fn", 0.5), kw.get("tau", 0.25), kw["warps"], kw["iters"], cvType=cv,
                  fix_quirks=kw.get("fix", 0))
    f.setCameraMatrices(K, K)
    f.copyImagesToDevice(I0, I1)
    if prior is not None:
        f.copySparseOpticalFlowToDevice(*prior)
    f.solveR(R, t, 5.0)
    u, v = f.copyOpticalFlowToHost()
    X, Y, Z = f.copy3dToHost()
    return {"u": u, "v": v, "X": X, "Y": Y, "Z": Z}, f


def run_oracle(oracle, w, h, L, method, I0, I1, K, R, t, input_type=0, prior=None,
               dtype=np.float32, **kw):
    p = oracle.make_params(w, h, L, method=method, input_type=input_type, lam=kw.get("lam", 50.0),
                           lambdaf=kw.get("lambdaf", 0.1), lambdams=kw.get("lambdams", 100.0),
                           alpha_tv=kw.get("alpha_tv", 1 / 0.33),
                           alpha_proj=kw.get("alpha_proj", 60.0), alpha_fn=kw.get("alpha_fn", 0.5),
                           tau=kw.get("tau", 0.25), theta=kw.get("theta", 0.33),
                           n_warp_iters=kw["warps"], n_solver_iters=kw["iters"],
                           fix_quirks=kw.get("fix", 0))
    ufn = vfn = mask = None
    if prior is not None:
        ufn, vfn = prior[0], prior[1]
        mask = prior[2] if len(prior) > 2 else None
    return oracle.solve(p, I0, I1, K0=K, K1=K, R1=R, t1=t, ufn=ufn, vfn=vfn, mask=mask, dtype=dtype)


def compare(got, want, w, h):
    for k in want:
        assert_bitexact(got[k], want[k], k, region=(h, w))


CASES = [
    # (w, h, L, warps, iters)
    (37, 23, 2, 2, 3),
    (64, 48, 3, 2, 5),
    (96, 64, 3, 2, 4),   # stride == width at every level: row-wrap reads
    (45, 90, 2, 1, 6),
    (130, 70, 4, 2, 3),
]


@pytest.mark.parametrize("w,h,L,warps,iters", CASES)
@pytest.mark.parametrize("fix", [0, 1, 3])
def test_recon_bitexact(oracle, rf, w, h, L, warps, iters, fix):
    rng = np.random.default_rng(w + h + fix)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    I0, I1 = pad_rows(I0, s), pad_rows(I1, s)
    K = _K(w, h)
    R, t = _pose(w)
    kw = dict(warps=warps, iters=iters, fix=fix)
    got, _ = run_gpu(rf, w, h, L, 14, I0, I1, K, R, t, **kw)
    want = run_oracle(oracle, w, h, L, 14, I0, I1, K, R, t, **kw)
    compare(got, want, w, h)


@pytest.mark.parametrize("method", [17, 20])
def test_prior_methods_bitexact(oracle, rf, method):
    w, h, L = 70, 50, 3
    rng = np.random.default_rng(method)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    I0, I1 = pad_rows(I0, s), pad_rows(I1, s)
    ufn = pad_rows(rng.normal(1.5, 0.3, (h, w)).astype(np.float32), s)
    vfn = pad_rows(rng.normal(-0.7, 0.3, (h, w)).astype(np.float32), s)
    mask = pad_rows((rng.random((h, w)) < 0.3).astype(np.float32), s)
    prior = (ufn, vfn, mask) if method == 20 else (ufn, vfn)
    K = _K(w, h)
    R, t = _pose(3)
    kw = dict(warps=2, iters=4, fix=1, alpha_fn=100.0)
    got, _ = run_gpu(rf, w, h, L, method, I0, I1, K, R, t, prior=prior, **kw)
    want = run_oracle(oracle, w, h, L, method, I0, I1, K, R, t, prior=prior, **kw)
    compare(got, want, w, h)


@pytest.mark.parametrize("w,h,L,warps,iters", CASES[:3])
def test_plain_tvl1_bitexact(oracle, rf, w, h, L, warps, iters):
    rng = np.random.default_rng(w)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    I0, I1 = pad_rows(I0, s), pad_rows(I1, s)
    kw = dict(warps=warps, iters=iters)
    got, _ = run_gpu(rf, w, h, L, 0, I0, I1, None, None, None, **kw)
    want = run_oracle(oracle, w, h, L, 0, I0, I1, None, None, None, **kw)
    compare(got, want, w, h)


@pytest.mark.parametrize("input_type", [1, 2, 3])
def test_input_types_bitexact(oracle, rf, input_type):
    w, h, L = 50, 40, 2
    rng = np.random.default_rng(input_type)
    s = align_up(w)
    if input_type == 1:
        I0 = rng.integers(0, 256, (h, s, 3)).astype(np.uint8)
        I1 = np.roll(I0, 1, axis=1)
    elif input_type == 2:
        I0 = rng.integers(0, 256, (h, s)).astype(np.uint8)
        I1 = np.roll(I0, 1, axis=1)
    else:
        I0 = rng.integers(0, 65536, (h, s)).astype(np.uint16)
        I1 = np.roll(I0, -1, axis=0)
    K = _K(w, h)
    R, t = _pose(5)
    kw = dict(warps=1, iters=3, fix=1)
    got, _ = run_gpu(rf, w, h, L, 14, I0, I1, K, R, t, input_type=input_type, **kw)
    want = run_oracle(oracle, w, h, L, 14, I0, I1, K, R, t, input_type=input_type, **kw)
    compare(got, want, w, h)


def test_repeated_solves_are_identical(rf):
    """The captured schedule replays deterministically, and a new pose is
    picked up without re-capture."""
    w, h = 80, 60
    rng = np.random.default_rng(11)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    I0, I1 = pad_rows(I0, s), pad_rows(I1, s)
    K = _K(w, h)
    R, t = _pose(1)
    f = rf.ReconFlow()
    f.initializeR(w, h, 1, 3, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25, 2, 5,
                  cvType=5, fix_quirks=1)
    f.setCameraMatrices(K, K)
    f.copyImagesToDevice(I0, I1)
    f.solveR(R, t, 5.0)
    a = f.copy3dToHost()
    f.solveR(R, t, 5.0)
    b = f.copy3dToHost()
    for x, y in zip(a, b):
        assert_bitexact(x, y, "repeat")
    R2, t2 = _pose(2)
    f.solveR(R2, t2, 5.0)
    c = f.copy3dToHost()
    assert not np.array_equal(a[2], c[2])
    launches = f.kernelLaunches()
    assert launches > 3 * 2 * 5 * 2


def test_scene_640x480_matches_fp32_oracle_and_ground_truth(oracle, rf):
    """The 640x480 workload (5 levels, 3 warps, 50 iterations): bit-exact with
    the FP32 oracle, and the same median endpoint error as the FP64 oracle."""
    from reconflow_gb300.scene import make_scene

    sc = make_scene(640, 480, seed=0)
    w, h, L = 640, 480, 5
    s = align_up(w)
    I0, I1 = pad_rows(sc["I0"], s), pad_rows(sc["I1"], s)
    kw = dict(warps=3, iters=50, fix=1)
    got, _ = run_gpu(rf, w, h, L, 14, I0, I1, sc["K"], sc["R"], sc["t"], **kw)
    want = run_oracle(oracle, w, h, L, 14, I0, I1, sc["K"], sc["R"], sc["t"], **kw)
    compare(got, want, w, h)
    ref64 = run_oracle(oracle, w, h, L, 14, I0, I1, sc["K"], sc["R"], sc["t"], dtype=np.float64,
                       **kw)
    val = sc["valid"]

    def epe(o):
        return np.sqrt((o["u"][:, :w] - sc["flow"][..., 0]) ** 2 +
                       (o["v"][:, :w] - sc["flow"][..., 1]) ** 2)[val]

    e32, e64 = np.median(epe(got)), np.median(epe(ref64))
    assert e32 < 0.5 and abs(e32 - e64) < 0.05, (e32, e64)


@pytest.mark.slow
def test_scene_720p_headline_workload_matches_fp32_oracle(oracle, rf):
    """The benchmark's 1280x720 workload (6 levels, 5 warps, 100 iterations,
    the bench's weights and tuned tiles): bit-exact with the FP32 oracle at
    full size, and inverse depth = 1 / Z exactly."""
    import json
    import os

    from reconflow_gb300 import autotune
    from reconflow_gb300.scene import make_scene

    sc = make_scene(1280, 720, seed=0)
    w, h, L = 1280, 720, 6
    s = align_up(w)
    I0, I1 = pad_rows(sc["I0"], s), pad_rows(sc["I1"], s)
    f = rf.ReconFlow()
    f.initializeR(w, h, 1, L, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25, 5, 100,
                  cvType=5, fix_quirks=1)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(root, "reconflow_gb300", "tuning", "gb300_720p_single.json")) as fh:
        autotune.apply_single(f, json.load(fh)["levels"], L)
    f.setCameraMatrices(sc["K"], sc["K"])
    f.copyImagesToDevice(I0, I1)
    f.solveR(sc["R"], sc["t"], 5.0)
    u, v = f.copyOpticalFlowToHost()
    X, Y, Z = f.copy3dToHost()
    inv = f.copyInverseDepthToHost()
    f.close()
    want = run_oracle(oracle, w, h, L, 14, I0, I1, sc["K"], sc["R"], sc["t"], warps=5, iters=100,
                      fix=1)
    compare({"u": u, "v": v, "X": X, "Y": Y, "Z": Z}, want, w, h)
    with np.errstate(divide="ignore"):
        assert_bitexact(inv, np.float32(1) / Z, "inverse depth", region=(h, w))


def test_device_results_and_inverse_depth(rf):
    w, h = 64, 48
    rng = np.random.default_rng(4)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    K = _K(w, h)
    R, t = _pose(4)
    f = rf.ReconFlow()
    f.initializeR(w, h, 1, 2, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 3.0, 60.0, 0.5, 0.25, 1, 3, cvType=5)
    f.setCameraMatrices(K, K)
    f.copyImagesToDevice(pad_rows(I0, s), pad_rows(I1, s))
    f.solveR(R, t, 5.0)
    X, Y, Z = f.copy3dToHost()
    inv = f.copyInverseDepthToHost()
    np.testing.assert_array_equal(inv[:, :w], (np.float32(1) / Z[:, :w]))
    ptrs = f.deviceResults()
    assert all(p != 0 for p in ptrs)


def test_degenerate_baseline_nan_parity(oracle, rf):
    """Pure sideways baseline (t_z = 0, R = I): the reference's projection
    divides 0/0 wherever a point is reset to the origin, so NaNs appear; the
    GPU must still match the oracle everywhere (NaN for NaN)."""
    w, h, L = 96, 72, 3
    rng = np.random.default_rng(0)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    I0 = (0.5 + 0.2 * np.sin(0.31 * x + 0.17 * y) + rng.normal(0, 0.01, (h, w))).astype(np.float32)
    I1 = np.roll(I0, 1, axis=1)
    K = _K(w, h)
    kw = dict(warps=2, iters=5, fix=1)
    got, _ = run_gpu(rf, w, h, L, 14, I0, I1, K, np.eye(3), np.array([-0.1, 0.0, 0.0]), **kw)
    want = run_oracle(oracle, w, h, L, 14, I0, I1, K, np.eye(3), np.array([-0.1, 0.0, 0.0]), **kw)
    compare(got, want, w, h)


@pytest.mark.parametrize("level", [0, 1, 2])
def test_warm_start_bitexact(oracle, rf, level):
    """A solve started at `level` from a given flow and 3D state matches the
    oracle's warm-started schedule bit for bit."""
    w, h, L = 96, 72, 3
    rng = np.random.default_rng(level)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    I0, I1 = pad_rows(I0, s), pad_rows(I1, s)
    K = _K(w, h)
    R, t = _pose(7)
    W, H, S = oracle.pyramid_dims(w, h, L)
    hl, sl = H[level], S[level]
    u0 = rng.normal(1.0, 0.2, (hl, sl)).astype(np.float32)
    v0 = rng.normal(-0.5, 0.2, (hl, sl)).astype(np.float32)
    Z0 = rng.uniform(2, 6, (hl, sl)).astype(np.float32)
    X0 = (Z0 * rng.normal(0, 0.3, (hl, sl))).astype(np.float32)
    Y0 = (Z0 * rng.normal(0, 0.3, (hl, sl))).astype(np.float32)
    f = rf.ReconFlow()
    f.initializeR(w, h, 1, L, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25, 3, 10,
                  cvType=5, fix_quirks=1)
    f.setCameraMatrices(K, K)
    f.copyImagesToDevice(I0, I1)
    f.solveWarm(level, u0, v0, X0, Y0, Z0, R, t, 2, 4)
    u, v = f.copyOpticalFlowToHost()
    X, Y, Z = f.copy3dToHost()
    p = oracle.make_params(w, h, L, lam=50.0, lambdaf=0.1, lambdams=100.0, alpha_tv=1 / 0.33,
                           alpha_proj=60.0, tau=0.25, n_warp_iters=3, n_solver_iters=10,
                           fix_quirks=1)
    pad = lambda a: np.pad(a, ((0, 1), (0, 0))).ravel()  # noqa: E731  (guard row)
    want = oracle.solve_warm(p, I0, I1, level, pad(u0), pad(v0), pad(X0), pad(Y0), pad(Z0), 2, 4,
                             K0=K, K1=K, R1=R, t1=t)
    compare({"u": u, "v": v, "X": X, "Y": Y, "Z": Z}, want, w, h)
    # a full solve afterwards re-captures the normal schedule
    f.solveR(R, t, 5.0)
    full = run_oracle(oracle, w, h, L, 14, I0, I1, K, R, t, warps=3, iters=10, fix=1)
    assert_bitexact(f.copyOpticalFlowToHost()[0], full["u"], "u after warm", region=(h, w))


def test_plain_warm_start_bitexact(oracle, rf):
    w, h, L, level = 80, 60, 3, 1
    rng = np.random.default_rng(3)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    I0, I1 = pad_rows(I0, s), pad_rows(I1, s)
    W, H, S = oracle.pyramid_dims(w, h, L)
    u0 = rng.normal(0.8, 0.1, (H[level], S[level])).astype(np.float32)
    v0 = rng.normal(-0.4, 0.1, (H[level], S[level])).astype(np.float32)
    f = rf.CudaFlow()
    f.initialize(w, h, 1, 5, L, 2.0, 0, 50.0, 0.0, 0.33, 0.25, 2, 6)
    f.copyImagesToDevice(I0, I1)
    f.solveOpticalFlowWarm(level, u0, v0, 1, 5)
    u, v = f.copyOpticalFlowToHost()
    p = oracle.make_params(w, h, L, method=0, lam=50.0, theta=0.33, tau=0.25, n_warp_iters=2,
                           n_solver_iters=6)
    z = np.zeros((H[level] + 1) * S[level], np.float32)
    pad = lambda a: np.pad(a, ((0, 1), (0, 0))).ravel()  # noqa: E731
    want = oracle.solve_warm(p, I0, I1, level, pad(u0), pad(v0), z, z, z, 1, 5)
    assert_bitexact(u, want["u"], "u", region=(h, w))
    assert_bitexact(v, want["v"], "v", region=(h, w))


@pytest.mark.parametrize("method", [14, 0])
def test_energy_matches_oracle(oracle, rf, method):
    w, h, L = 96, 64, 3
    rng = np.random.default_rng(9)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    I0, I1 = pad_rows(I0, s), pad_rows(I1, s)
    K = _K(w, h)
    R, t = _pose(8)
    res, f = run_gpu(rf, w, h, L, method, I0, I1, K, R, t, warps=2, iters=5, fix=1)
    e_gpu = f.energy()
    if method == 0:
        z = np.zeros_like(res["u"])
        e_ref = oracle.energy(I0, I1, res["u"], res["v"], z, z, z, w, h, s, 50.0, 60.0, np.eye(3),
                              np.zeros(3), np.eye(3), recon=False)
    else:
        e_ref = oracle.energy(I0, I1, res["u"], res["v"], res["X"], res["Y"], res["Z"], w, h, s,
                              50.0, 60.0, R, t, K)
    # per-pixel terms and each thread's few pixels in FP32 on the GPU, FP64 in
    # the oracle; the GPU adds the thread sums in double
    assert e_gpu == pytest.approx(e_ref, rel=1e-5)


def test_tiles_do_not_change_single_pair_results(rf):
    """rf_set_tiles changes only the launch shape of the inner iterations."""
    from reconflow_gb300._native import RfError

    w, h, L = 150, 100, 3
    rng = np.random.default_rng(12)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    I0, I1 = pad_rows(I0, s), pad_rows(I1, s)
    K, (R, t) = _K(w, h), _pose(3)
    f = rf.ReconFlow()
    f.initializeR(w, h, 1, L, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25, 2, 6,
                  cvType=5, fix_quirks=1)
    f.setCameraMatrices(K, K)
    f.copyImagesToDevice(I0, I1)
    f.solveR(R, t, 5.0)
    ref = f.copyOpticalFlowToHost() + f.copy3dToHost()
    for tw, th in (([32, 16, 64], [2, 8, 4]), ([128, 32, 16], [2, 4, 16])):
        f.setTiles(tw, th)
        f.solveR(R, t, 5.0)
        got = f.copyOpticalFlowToHost() + f.copy3dToHost()
        for a, b, nm in zip(got, ref, "uvXYZ"):
            assert_bitexact(a, b, f"{nm} tiles {tw}x{th}")
    with pytest.raises(RfError):
        f.setTiles([32, 32, 32], [8, 8, 9])
    f.close()


@pytest.mark.parametrize("w,h,L,method", [(160, 90, 2, 14), (96, 72, 3, 17), (37, 23, 2, 14),
                                          (330, 200, 3, 20)])
def test_cluster_levels_equal_two_launch_loop(oracle, rf, w, h, L, method):
    """A warp's inner iterations as one thread-block-cluster launch (cluster
    barriers between the half-steps) give exactly the two-launches-per-
    iteration loop's results, at every level (forced on) and never (off),
    and the oracle's."""
    lib = rf.load()
    s = align_up(w)
    rng = np.random.default_rng(w + h)
    I0, I1 = textured_pair(rng, h, s, shift=(1.3, -0.6))
    K = np.array([[0.8 * w, 0, w / 2], [0, 0.8 * w, h / 2], [0, 0, 1.0]])
    c, sn = np.cos(0.01), np.sin(0.01)
    R = np.array([[c, 0, sn], [0, 1, 0], [-sn, 0, c]])
    t = np.array([-0.1, 0.01, 0.02])
    ufn = (rng.normal(size=(h, s)) * 0.5 + 1.0).astype(np.float32)
    vfn = (rng.normal(size=(h, s)) * 0.5).astype(np.float32)
    mask = (rng.random((h, s)) < 0.3).astype(np.float32)
    outs = []
    try:
        for px in (0, 1 << 40):
            lib.rf_set_cluster_pixels(px)
            f = rf.ReconFlow()
            f.initializeR(w, h, 1, L, 2.0, method, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5,
                          0.25, 2, 7, cvType=5, fix_quirks=1)
            f.setCameraMatrices(K, K)
            f.copyImagesToDevice(I0, I1)
            if method in (17, 20):
                f.copySparseOpticalFlowToDevice(ufn, vfn, mask if method == 20 else None)
            f.solveR(R, t, 5.0)
            u, v = f.copyOpticalFlowToHost()
            X, Y, Z = f.copy3dToHost()
            f.close()
            outs.append((u, v, X, Y, Z))
    finally:
        lib.rf_set_cluster_pixels(-1)
    for a, b, nm in zip(outs[0], outs[1], "uvXYZ"):
        assert_bitexact(b, a, f"{nm}: cluster vs two-launch", region=(h, w))
    p = oracle.make_params(w, h, L, method=method, lam=50.0, lambdaf=0.1, lambdams=100.0,
                           alpha_tv=1 / 0.33, alpha_proj=60.0, tau=0.25, n_warp_iters=2,
                           n_solver_iters=7, fix_quirks=1)
    kw = {}
    if method in (17, 20):
        kw = dict(ufn=ufn, vfn=vfn, mask=mask if method == 20 else None)
    want = oracle.solve(p, I0, I1, K0=K, K1=K, R1=R, t1=t, dtype=np.float32, **kw)
    for k, got in zip("uvXYZ", outs[1]):
        assert_bitexact(got, want[k], f"{k}: cluster vs oracle", region=(h, w))
