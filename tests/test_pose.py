"""Pose front end on the CPU: the host-side relative pose of the C ABI
(five-point solver, LMedS, pose recovery; CameraPose.cpp:79-104) on exact and
noisy synthetic matches, and the feature oracle's properties (integral image,
responses of a blob, rotation behaviour, the oracle's own pose on a rendered
scene).  No GPU: the library's host functions run without a device."""
import numpy as np
import pytest

from reconflow_gb300 import pose as P


def _rot(rng, deg):
    a = rng.normal(size=3)
    a /= np.linalg.norm(a)
    ang = np.radians(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K


def _skew(t):
    return np.array([[0, -t[2], t[1]], [t[2], 0, -t[0]], [-t[1], t[0], 0]])


def _project(X, R, t):
    X1 = X @ R.T + t
    return X[:, :2] / X[:, 2:], X1[:, :2] / X1[:, 2:]


def _angle(Ra, Rb):
    return np.degrees(np.arccos(np.clip((np.trace(Ra.T @ Rb) - 1) / 2, -1, 1)))


@pytest.mark.parametrize("seed", range(40))
def test_five_point_recovers_E(seed):
    """One of the (up to 10) solutions through five exact matches is
    [t]x R up to sign."""
    rng = np.random.default_rng(seed)
    R = _rot(rng, rng.uniform(0.5, 25))
    t = rng.normal(size=3)
    t /= np.linalg.norm(t)
    X = np.c_[rng.uniform(-2, 2, (5, 2)), rng.uniform(2, 12, 5)]
    x0, x1 = _project(X, R, t)
    Es = P.essential_5pt(x0, x1)
    assert 1 <= len(Es) <= 10
    E = _skew(t) @ R
    E /= np.linalg.norm(E)
    err = min(min(np.linalg.norm(e - E), np.linalg.norm(e + E)) for e in Es)
    assert err < 1e-5, err
    for e in Es:  # every solution satisfies the five epipolar constraints and det = 0
        r = [np.r_[b, 1] @ e @ np.r_[a, 1] for a, b in zip(x0, x1)]
        assert np.max(np.abs(r)) < 1e-8
        assert abs(np.linalg.det(e)) < 1e-8


@pytest.mark.parametrize("seed", range(6))
def test_lmeds_and_recover_pose_with_outliers(seed):
    rng = np.random.default_rng(100 + seed)
    R = _rot(rng, rng.uniform(1, 5))
    t = rng.normal(size=3)
    t /= np.linalg.norm(t)
    n = 400
    X = np.c_[rng.uniform(-3, 3, (n, 2)), rng.uniform(3, 10, n)]
    x0, x1 = _project(X, R, t)
    out = rng.random(n) < 0.3
    x1[out] = rng.uniform(-0.6, 0.6, (out.sum(), 2))
    E, mask = P.essential_lmeds(x0, x1, seed=seed)
    assert (mask == ~out).mean() > 0.98
    Rg, tg, good = P.recover_pose(E, x0, x1, mask)
    assert _angle(Rg, R) < 1e-4
    # least squares over the mask (which admits the few outliers that lie on
    # their epipolar lines) stays within a hundredth of a degree
    Rr, tr = P.refine_pose(Rg, tg, x0, x1, mask)
    assert _angle(Rr, R) < 0.01 and np.degrees(np.arccos(np.clip(tr @ t, -1, 1))) < 0.05
    assert np.degrees(np.arccos(np.clip(tg @ t, -1, 1))) < 1e-3
    assert good >= 0.95 * (~out).sum()
    # deterministic for a seed
    E2, mask2 = P.essential_lmeds(x0, x1, seed=seed)
    assert np.array_equal(E, E2) and np.array_equal(mask, mask2)


def test_lmeds_rejects_too_few_matches():
    from reconflow_gb300._native import RfError

    with pytest.raises(RfError):
        P.essential_lmeds(np.zeros((4, 2)), np.zeros((4, 2)))


def test_bgr_to_gray_fixed_point():
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (7, 9, 3)).astype(np.uint8)
    g = P.bgr_to_gray(img)
    want = np.floor(0.299 * img[..., 2] + 0.587 * img[..., 1] + 0.114 * img[..., 0] + 0.5)
    assert np.max(np.abs(g.astype(float) - want)) <= 1


# ---- the feature oracle ----------------------------------------------------

def _to8(a):
    return np.clip(np.floor(a * 255 + 0.5), 0, 255).astype(np.uint8)


def test_oracle_integral_image(oracle):
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (37, 53)).astype(np.uint8)
    S = oracle.surf_integral(img)
    want = np.zeros((38, 54), np.uint64)
    want[1:, 1:] = img.astype(np.uint64).cumsum(0).cumsum(1)
    assert np.array_equal(S.astype(np.uint64), want)


@pytest.mark.parametrize("sigma,layer", [(3.0, 1), (4.0, 2), (5.0, 3)])
def test_oracle_blob_response_peaks_at_its_centre(oracle, sigma, layer):
    """A dark Gaussian blob on a flat background: the strongest response of
    octave 0 is at the blob centre, in a layer that grows with the blob
    (filter sizes 15, 21, 27 for sigma 3, 4, 5), and it is a keypoint."""
    h, w = 128, 160
    y, x = np.mgrid[0:h, 0:w]
    img = _to8(0.8 - 0.6 * np.exp(-((x - 80) ** 2 + (y - 64) ** 2) / (2 * sigma ** 2)))
    R = oracle.surf_responses(img, 0, 4)
    k, j, i = np.unravel_index(np.argmax(R), R.shape)
    assert (i, j, k) == (80, 64, layer)
    kp, _ = oracle.surf_detect(img, threshold=5.0)
    assert len(kp) >= 1
    assert abs(kp[0, 0] - 80) < 0.5 and abs(kp[0, 1] - 64) < 0.5


def test_oracle_features_follow_a_rotation(oracle):
    """Keypoints of a frame rotated by 90 degrees are the rotated keypoints,
    and the descriptors match across the rotation."""
    from reconflow_gb300.scene import make_scene

    sc = make_scene(320, 240, seed=3)
    a = _to8(sc["I0"])
    b = np.ascontiguousarray(np.rot90(a))  # (x, y) -> (y, w - 1 - x)
    ka, da = oracle.surf_detect(a, threshold=10.0)
    kb, db = oracle.surf_detect(b, threshold=10.0)
    assert len(ka) > 50 and abs(len(ka) - len(kb)) < 0.25 * len(ka)
    best, d1, d2 = oracle.surf_match(da, db)
    ok = np.sqrt(d1) < 0.6 * np.sqrt(d2)
    assert ok.mean() > 0.3
    pa = ka[ok, :2]
    pb = kb[best[ok], :2]
    want = np.c_[pa[:, 1], 320 - 1 - pa[:, 0]]
    assert np.median(np.linalg.norm(pb - want, axis=1)) < 1.0


def test_oracle_pose_on_a_rendered_scene(oracle):
    """Oracle features + the library's host pose recover the generator's pose."""
    from reconflow_gb300.scene import make_scene

    sc = make_scene(640, 480, seed=0)
    k0, d0 = oracle.surf_detect(_to8(sc["I0"]), threshold=20.0)
    k1, d1_ = oracle.surf_detect(_to8(sc["I1"]), threshold=20.0)
    best, a, b = oracle.surf_match(d0, d1_)
    q = np.nonzero(np.sqrt(a).astype(np.float64) < 0.6 * np.sqrt(b).astype(np.float64))[0]
    Ki = np.linalg.inv(sc["K"])
    norm = lambda p: (np.c_[p, np.ones(len(p))] @ Ki.T)[:, :2]  # noqa: E731
    x0, x1 = norm(k0[q, :2].astype(np.float64)), norm(k1[best[q], :2].astype(np.float64))
    E, mask = P.essential_lmeds(x0, x1)
    R, t, _ = P.recover_pose(E, x0, x1, mask)
    tg = sc["t"] / np.linalg.norm(sc["t"])
    assert _angle(R, sc["R"]) < 0.3
    assert np.degrees(np.arccos(np.clip(t @ tg, -1, 1))) < 5.0
    # refinement on the inliers brings both within a tenth of that
    R2, t2 = P.refine_pose(R, t, x0, x1, mask)
    assert _angle(R2, sc["R"]) < 0.05
    assert np.degrees(np.arccos(np.clip(t2 @ tg, -1, 1))) < 0.5


def test_oracle_matches_committed_fixtures(oracle):
    """The pose oracle's feature stages on the committed frames equal the
    committed fixtures bit for bit (tests/golden/make_pose_golden.py)."""
    import os

    path = os.path.join(os.path.dirname(__file__), "golden", "pose_cases.npz")
    g = np.load(path)
    k0, d0 = oracle.surf_detect(g["frame0"], threshold=10.0)
    k1, d1 = oracle.surf_detect(g["frame1"], threshold=10.0)
    best, e1, e2 = oracle.surf_match(d0, d1)
    for got, key in ((k0, "kp0"), (d0, "desc0"), (k1, "kp1"), (d1, "desc1"), (e1, "d1"),
                     (e2, "d2")):
        assert np.array_equal(got.view(np.uint32), g[key].view(np.uint32)), key
    assert np.array_equal(best, g["best"])
    # the frames differ by a 2.3 / -1.7 px shift and a 0.05 rad rotation about
    # the centre: every ratio-tested match follows that motion
    ok = np.sqrt(e1) < 0.6 * np.sqrt(e2)
    assert ok.sum() >= 10
    c, s = np.cos(0.05), np.sin(0.05)
    R = np.array([[c, s], [-s, c]])
    ctr = np.array([80.0, 60.0])
    want = (k0[ok, :2].astype(np.float64) + np.array([2.3, -1.7]) - ctr) @ R + ctr
    err = np.linalg.norm(k1[best[ok], :2] - want, axis=1)
    assert np.max(err) < 0.5 and np.median(err) < 0.1, err


def _roots_tool(tmp_path):
    import os
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = tmp_path / "fivept_roots"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I",
                    os.path.join(root, "reconflow_gb300", "csrc"),
                    os.path.join(root, "tests", "cpp", "fivept_roots.cpp"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)

    def run(polys):
        txt = "".join(f"{len(c)} " + " ".join(repr(float(x)) for x in c) + "\n" for c in polys)
        out = subprocess.run([str(exe)], input=txt, capture_output=True, text=True, check=True)
        res = []
        for line in out.stdout.splitlines():
            v = line.split()
            res.append(np.array([float(x) for x in v[1:1 + int(v[0])]]))
        return res
    return run


def test_five_point_real_roots_against_numpy(tmp_path):
    """The five-point solver's real-root finder (derivative bracketing,
    safeguarded Newton) on polynomials of degree <= 10: Wilkinson-type
    products, random real-rooted ones with clusters, random ones with
    complex pairs, a double root and a vanishing leading coefficient."""
    run = _roots_tool(tmp_path)
    rng = np.random.default_rng(7)
    cases, want = [], []

    def from_roots(rs, scale=1.0, extra=()):
        c = np.poly(list(rs) + list(extra))[::-1] * scale  # ascending
        return c

    cases.append(from_roots(range(1, 11)))  # (z-1)...(z-10)
    want.append(np.arange(1.0, 11.0))
    for _ in range(40):  # real-rooted, degree 3..10, some clustered pairs
        d = int(rng.integers(3, 11))
        rs = np.sort(rng.uniform(-5, 5, d))
        if d > 3:
            rs[1] = rs[0] + rng.uniform(1e-3, 1e-2)
        rs = np.sort(rs)
        cases.append(from_roots(rs, scale=rng.uniform(-100, 100)))
        want.append(rs)
    for _ in range(40):  # real roots plus complex pairs
        nr = int(rng.integers(0, 7))
        rs = np.sort(rng.uniform(-3, 3, nr))
        quad = []
        for _ in range((10 - nr) // 2):
            a, b = rng.uniform(-3, 3), rng.uniform(0.3, 2)
            quad += [a + 1j * b, a - 1j * b]
        cases.append(np.real(from_roots(rs, extra=quad)))
        want.append(rs)
    got = run(cases)
    for k, (g, w) in enumerate(zip(got, want)):
        assert len(g) == len(w), (k, g, w)
        assert np.all(np.diff(g) >= 0), k
        assert np.allclose(g, w, rtol=1e-6, atol=1e-6), (k, g, w)

    # a double root: found (once or twice) within the square root of the
    # rounding error, the simple roots exactly
    g = run([from_roots([-2.0, 1.0, 1.0, 3.0])])[0]
    assert np.isclose(g[0], -2.0) and np.isclose(g[-1], 3.0)
    assert np.all(np.abs(g[1:-1] - 1.0) < 1e-6) and 1 <= len(g) - 2 <= 2
    # a leading coefficient at rounding level of the others: treated as
    # degree 2
    c = list(from_roots([0.5, 2.0])) + [1e-20]
    g = run([c])[0]
    assert np.allclose(g, [0.5, 2.0])


def test_five_point_near_tangent_complex_pair(tmp_path):
    """A complex pair close to the real axis.  At 1e-4 from it the
    polynomial's minimum between the pair (1e-8 relative) is far above the
    rounding level, and no real root comes back there.  At 1e-9 the minimum
    (1e-18) is below the rounding error of evaluating the polynomial in
    double precision, so it cannot be told from a real double root: the
    finder reports one or two roots there, and the essential-matrix LMedS
    scores that extra candidate like any other (it is kept only if its
    median residual wins)."""
    run = _roots_tool(tmp_path)
    real = [-2.5, -1.0, 1.5, 3.0]
    for dist, expect_root in ((1e-4, False), (1e-9, True)):
        c = np.real(np.poly(real + [0.7 + 1j * dist, 0.7 - 1j * dist]))[::-1]
        g = run([c])[0]
        near = np.abs(g - 0.7) < 1e-3
        others = g[~near]
        assert np.allclose(others, real, atol=1e-9), (dist, g)
        if expect_root:
            assert 1 <= near.sum() <= 2 and np.all(np.abs(g[near] - 0.7) < 1e-6), (dist, g)
        else:
            assert near.sum() == 0, (dist, g)
