"""Pose front end on the GPU (CameraPose, reconflow/CameraPose.cpp:47-118):
every feature stage through the C ABI equals the CPU oracle bit for bit
(Hessian responses of every octave, keypoints with their orientation and
scale, descriptors, ratio-tested matches), and the estimated pose of rendered
scenes agrees with the generator's ground truth."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THRESHOLD = 20.0


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _to8(a):
    return np.clip(np.floor(a * 255 + 0.5), 0, 255).astype(np.uint8)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _scene(w, h, seed):
    from reconflow_gb300.scene import make_scene

    return make_scene(w, h, seed=seed)


def _pose(rf, K, thr=THRESHOLD):
    cp = rf.CameraPose()
    cp.initialize(K, thr)
    return cp


@pytest.mark.parametrize("w,h,seed", [(640, 480, 0), (333, 211, 5)])
def test_features_bitexact(oracle, rf, w, h, seed):
    sc = _scene(w, h, seed)
    a, b = _to8(sc["I0"]), _to8(sc["I1"])
    cp = _pose(rf, sc["K"])
    ret, R, t = cp.solvePose_8uc1(a, b)
    assert ret == 0
    for f, img in ((0, a), (1, b)):
        for o in range(4):
            got = cp.responses(f, o)
            want = oracle.surf_responses(img, o, 4)
            assert np.array_equal(_bits(got), _bits(want)), (f, o)
        kp, desc = cp.keypoints(f)
        kp_ref, desc_ref = oracle.surf_detect(img, threshold=THRESHOLD)
        assert len(kp) == len(kp_ref) > 20
        assert np.array_equal(_bits(kp), _bits(kp_ref)), f
        assert np.array_equal(_bits(desc), _bits(desc_ref)), f
    # matches: the oracle's nearest neighbours through the same ratio test
    _, d0 = oracle.surf_detect(a, threshold=THRESHOLD)
    _, d1 = oracle.surf_detect(b, threshold=THRESHOLD)
    best, e1, e2 = oracle.surf_match(d0, d1)
    q = np.nonzero(np.sqrt(e1).astype(np.float64) < 0.6 * np.sqrt(e2).astype(np.float64))[0]
    i0, i1, dist, inl = cp.matches()
    assert np.array_equal(i0, q)
    assert np.array_equal(i1, best[q])
    assert np.array_equal(_bits(dist), _bits(np.sqrt(e1[q])))
    assert inl.sum() == cp.counts()[3] > 0.8 * len(q)


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("refine", [0, 1])
def test_pose_matches_ground_truth_720p(rf, seed, refine):
    """The reference's LMedS model (refine = 0) and the inlier refinement
    (refine = 1) against the generator's pose (0.1 m baseline)."""
    sc = _scene(1280, 720, 2000 + seed)
    cp = _pose(rf, sc["K"])
    cp.params.refine = refine
    ret, R, t = cp.solvePose_f32(sc["I0"], sc["I1"])
    assert ret == 0
    ang = np.degrees(np.arccos(np.clip((np.trace(R.T @ sc["R"]) - 1) / 2, -1, 1)))
    tg = sc["t"] / np.linalg.norm(sc["t"])
    tang = np.degrees(np.arccos(np.clip(t @ tg, -1, 1)))
    assert ang < (0.3 if not refine else 0.1), ang
    assert tang < (5.0 if not refine else 1.0), tang
    assert abs(np.linalg.norm(t) - 1) < 1e-9
    assert abs(np.linalg.det(R) - 1) < 1e-9


def test_float_input_equals_8bit_input(rf):
    sc = _scene(640, 480, 7)
    cp = _pose(rf, sc["K"])
    r1 = cp.solvePose_f32(sc["I0"], sc["I1"])
    k1 = cp.keypoints(0)
    r2 = cp.solvePose_8uc1(_to8(sc["I0"]), _to8(sc["I1"]))
    k2 = cp.keypoints(0)
    assert r1[0] == r2[0] == 0
    assert np.array_equal(r1[1], r2[1]) and np.array_equal(r1[2], r2[2])
    assert np.array_equal(_bits(k1[0]), _bits(k2[0]))


def test_device_frames_equal_host_frames(rf):
    import torch

    sc = _scene(640, 480, 8)
    cp = _pose(rf, sc["K"])
    _, Rh, th = cp.solvePose_f32(sc["I0"], sc["I1"])
    a = torch.from_numpy(np.ascontiguousarray(sc["I0"], np.float32)).cuda()
    b = torch.from_numpy(np.ascontiguousarray(sc["I1"], np.float32)).cuda()
    torch.cuda.synchronize()
    import ctypes

    from reconflow_gb300 import _native as N

    R = np.zeros(9)
    t = np.zeros(3)
    K = np.ascontiguousarray(sc["K"], np.float64)
    N.check(N.load().rf_pose_solve_f32(cp._handle(640, 480), ctypes.c_void_p(a.data_ptr()),
                                       ctypes.c_void_p(b.data_ptr()), 640,
                                       K.ctypes.data_as(ctypes.c_void_p),
                                       R.ctypes.data_as(ctypes.c_void_p),
                                       t.ctypes.data_as(ctypes.c_void_p)))
    assert np.array_equal(R.reshape(3, 3), Rh) and np.array_equal(t, th)


def test_blank_frames_give_no_pose(rf):
    cp = _pose(rf, np.array([[500.0, 0, 160], [0, 500.0, 120], [0, 0, 1]]))
    blank = np.full((240, 320), 128, np.uint8)
    assert cp.solvePose_8uc1(blank, blank) == (1, None, None)
    assert cp.counts()[0] == 0


def test_bgr_frames(rf):
    """solvePose_8uc3 converts BGR to gray first (CameraPose.cpp:120-128)."""
    sc = _scene(640, 480, 9)
    g0, g1 = _to8(sc["I0"]), _to8(sc["I1"])
    bgr0, bgr1 = (np.repeat(g[..., None], 3, axis=2) for g in (g0, g1))
    cp = _pose(rf, sc["K"])
    r_gray = cp.solvePose_8uc1(g0, g1)
    r_bgr = cp.solvePose_8uc3(bgr0, bgr1)
    assert np.array_equal(r_gray[1], r_bgr[1]) and np.array_equal(r_gray[2], r_bgr[2])


def test_keypoint_cap_keeps_the_strongest(oracle, rf):
    """max_keypoints keeps the strongest keypoints (ties by octave, layer,
    cell), exactly as the oracle's list cut at the same length."""
    sc = _scene(640, 480, 11)
    a, b = _to8(sc["I0"]), _to8(sc["I1"])
    cp = _pose(rf, sc["K"])
    cp.params.max_keypoints = 300
    cp.solvePose_8uc1(a, b)
    kp, desc = cp.keypoints(0)
    kp_ref, desc_ref = oracle.surf_detect(a, threshold=THRESHOLD, max_kp=300)
    assert len(kp) == 300
    assert np.array_equal(_bits(kp), _bits(kp_ref))
    assert np.array_equal(_bits(desc), _bits(desc_ref))
    assert np.all(np.diff(kp[:, 4]) <= 0)  # strongest first


def test_small_and_degenerate_frames(rf):
    """Frames too small for the coarser octaves, and noise at threshold 0
    (tens of thousands of candidates, possibly more than their buffer holds),
    end in a pose or in 1 (no pose), never in an error."""
    K = np.array([[100.0, 0, 24], [0, 100.0, 20], [0, 0, 1]])
    rng = np.random.default_rng(0)
    tiny = rng.integers(0, 256, (40, 48)).astype(np.uint8)
    cp = _pose(rf, K)
    ret, R, t = cp.solvePose_8uc1(tiny, tiny)
    assert ret in (0, 1)
    n0 = rng.integers(0, 256, (720, 1280)).astype(np.uint8)
    n1 = rng.integers(0, 256, (720, 1280)).astype(np.uint8)
    cp2 = _pose(rf, K, thr=0.0)
    cp2.params.max_keypoints = 64
    assert cp2.solvePose_8uc1(n0, n1)[0] in (0, 1)


def test_gpu_matches_committed_fixtures(rf):
    """The GPU's keypoints, descriptors and matches on the committed frames
    equal the committed oracle fixtures bit for bit."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "pose_cases.npz"))
    cp = _pose(rf, np.array([[150.0, 0, 80], [0, 150.0, 60], [0, 0, 1]]), thr=10.0)
    cp.solvePose_8uc1(g["frame0"], g["frame1"])
    for f in (0, 1):
        kp, desc = cp.keypoints(f)
        assert np.array_equal(_bits(kp), _bits(g[f"kp{f}"])), f
        assert np.array_equal(_bits(desc), _bits(g[f"desc{f}"])), f
    q = np.nonzero(np.sqrt(g["d1"]).astype(np.float64) < 0.6 * np.sqrt(g["d2"]).astype(np.float64))[0]
    i0, i1, dist, _ = cp.matches()
    assert np.array_equal(i0, q) and np.array_equal(i1, g["best"][q])


def test_gpu_lmeds_equals_host_lmeds(rf):
    """The GPU's five-point solutions and medians pick the same model as the
    host API on the same matches and seed: R and t bit for bit."""
    from reconflow_gb300 import pose as P

    sc = _scene(640, 480, 12)
    cp = _pose(rf, sc["K"])
    ret, R, t = cp.solvePose_8uc1(_to8(sc["I0"]), _to8(sc["I1"]))
    assert ret == 0
    k0, _ = cp.keypoints(0)
    k1, _ = cp.keypoints(1)
    i0, i1, _, inl = cp.matches()
    K = sc["K"]
    fx, sk, cx, fy, cy = K[0, 0], K[0, 1], K[0, 2], K[1, 1], K[1, 2]

    def norm(k):
        y = (k[:, 1].astype(np.float64) - cy) / fy
        x = ((k[:, 0].astype(np.float64) - cx) - sk * y) / fx
        return np.ascontiguousarray(np.stack([x, y], 1))

    x0, x1 = norm(k0[i0]), norm(k1[i1])
    E, mask = P.essential_lmeds(x0, x1, confidence=cp.params.confidence, seed=cp.params.seed)
    assert np.array_equal(mask, inl)
    Rh, th, _ = P.recover_pose(E, x0, x1, mask)
    assert np.array_equal(Rh, R) and np.array_equal(th, t)
