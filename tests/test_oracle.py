"""CPU tests of the oracle: known answers, properties and an independent
pure-Python restatement of the reference's median selection loops.

The reference ships no tests or golden outputs (its only test is the demo
``test_reconflow/main.cpp``), so the oracle is pinned here by analytic
known answers and by properties of the update equations.
"""
import numpy as np
import pytest

from helpers import align_up, pad_rows, textured_pair


# Cudaflow.cu:146-171 pyramid sizes for the benchmark workloads
@pytest.mark.parametrize("w,h,L,want", [
    (640, 480, 5, ([640, 320, 160, 80, 40], [480, 240, 120, 60, 30], [640, 320, 160, 96, 64])),
    (1280, 720, 6, ([1280, 640, 320, 160, 80, 40], [720, 360, 180, 90, 45, 22],
                    [1280, 640, 320, 160, 96, 64])),
    (1920, 1080, 6, ([1920, 960, 480, 240, 120, 60], [1080, 540, 270, 135, 67, 33],
                     [1920, 960, 480, 256, 128, 64])),
    (320, 240, 6, ([320, 160, 80, 40, 20, 10], [240, 120, 60, 30, 15, 7], [320, 160, 96, 64, 32, 32])),
    (768, 320, 1, ([768], [320], [768])),
])
def test_pyramid_dims(oracle, w, h, L, want):
    assert tuple(oracle.pyramid_dims(w, h, L)) == want


def test_pyramid_total_pixels(oracle):
    # 720p, 6 levels: 1 228 480 pixels per sweep of the pyramid
    W, H, _ = oracle.pyramid_dims(1280, 720, 6)
    assert sum(a * b for a, b in zip(W, H)) == 1228480


def test_k_pyramid_quirk(oracle):
    K = np.array([[500.0, 0, 320], [0, 510.0, 240], [0, 0, 1]])
    pK = oracle.k_pyramid(K, 3)
    assert np.array_equal(pK[0], K)
    for l in (1, 2):
        f = 2.0 ** l
        assert pK[l][0, 0] == 500 / f and pK[l][0, 2] == 320 / f
        assert pK[l][1, 1] == 510 / f and pK[l][1, 2] == 240 / f
        assert pK[l][2, 2] == 0.0  # Reconflow.cu:98-110 starts from zeros


def _median_ref_5(u, w, h, s):
    """Pure-Python restatement of MedianFilterKernel5 (medianFilter.cu:3-75)."""
    out = np.zeros_like(u)
    for iy in range(h):
        for ix in range(w):
            m = [0.0] * 25
            for j in range(5):
                for i in range(5):
                    col, row = ix + i - 2, iy + j - 2
                    if 0 <= col < w and 0 <= row < h:
                        m[j * 5 + i] = u[col + s * row]
                    elif col < 0 and 0 <= row < h:
                        m[j * 5 + i] = u[s * row]
                    elif col >= w and 0 <= row < h:
                        m[j * 5 + i] = u[w - 1 + s * row]
                    elif 0 <= col < w and row < 0:
                        m[j * 5 + i] = u[col]
                    elif 0 <= col < w and row >= h:
                        m[j * 5 + i] = u[col + s * (h - 1)]
            m = [np.float32(x) for x in m]
            for j in range(13):
                for i in range(j + 1, 25):
                    if m[j] > m[i]:
                        m[j], m[i] = m[i], m[j]
            out[ix + iy * s] = m[12]
    return out


def _median_ref_3(u, w, h, s):
    """Pure-Python restatement of MedianFilter3DKernel3 (medianFilter.cu:166-243)."""
    out = np.zeros_like(u)
    for iy in range(h):
        for ix in range(w):
            m = [0.0] * 9
            for j in range(3):
                for i in range(3):
                    col, row = ix + i - 1, iy + j - 1
                    k = j * 3 + i
                    if 0 <= col < w and 0 <= row < h:
                        m[k] = u[col + s * row]
                    elif col < 0 and 0 <= row < h:
                        m[k] = u[s * row]
                    elif col > w and 0 <= row < h:
                        m[k] = u[w - 1 + s * row]
                    elif 0 <= col < w and row < 0:
                        m[k] = u[col]
                    elif 0 <= col < w and row > h:
                        m[k] = u[col + s * (h - 1)]
            m = [np.float32(x) for x in m]
            for j in range(5):
                for i in range(j + 1, 9):
                    if m[j] > m[i]:
                        m[j], m[i] = m[i], m[j]
            out[ix + iy * s] = m[4]
    return out


@pytest.mark.parametrize("w,h", [(9, 7), (5, 5), (1, 4), (6, 1)])
def test_median_matches_python_restatement(oracle, w, h):
    rng = np.random.default_rng(w * 100 + h)
    s = align_up(w, 8)
    u = rng.integers(-3, 4, (h + 1) * s).astype(np.float32)  # many ties
    u[rng.random(u.shape) < 0.2] = -0.0
    v = rng.normal(size=(h + 1) * s).astype(np.float32)
    ou, ov = oracle.median5(u, v, w, h, s)
    for a, o in ((u, ou), (v, ov)):
        ref = _median_ref_5(a, w, h, s)
        for iy in range(h):
            np.testing.assert_array_equal(o[iy * s: iy * s + w].view(np.uint32),
                                          ref[iy * s: iy * s + w].view(np.uint32))
    X, Y, Z = oracle.median3d(u, v, -u, w, h, s)
    for a, o in ((u, X), (v, Y), (-u, Z)):
        ref = _median_ref_3(a, w, h, s)
        for iy in range(h):
            np.testing.assert_array_equal(o[iy * s: iy * s + w].view(np.uint32),
                                          ref[iy * s: iy * s + w].view(np.uint32))


def test_median_corner_zero_taps(oracle):
    # corners of the 5x5 window out of range on both axes stay 0 (medianFilter.cu:14-53)
    w, h, s = 3, 3, 8
    u = np.full((h + 1) * s, 7.0, np.float32)
    ou, _ = oracle.median5(u, u, w, h, s)
    # (0,0): 4 corner taps are 0, 21 taps are 7 -> median 7
    assert ou[0] == 7.0
    # 3D median: right column / bottom row taps are 0 (col > width never holds)
    X, _, _ = oracle.median3d(u, u, u, w, h, s)
    assert X[1 * s + (w - 1)] == 7.0  # right edge: 3 of 9 taps are 0 -> median 7
    assert X[(h - 1) * s + (w - 1)] == 0.0  # far corner: 5 of 9 taps are 0 -> median 0
    u1 = np.full((2 * s,), 5.0, np.float32)
    X, _, _ = oracle.median3d(u1, u1, u1, 1, 1, s)
    # 1x1 image: taps (left, up clamp) = 5 x 4 (incl. centre), others 0 -> median 0
    assert X[0] == 0.0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_texture_constants(oracle, dtype):
    w, h, s = 45, 22, 64
    c = np.full((h + 1) * s, 0.375, dtype)
    d = oracle.downscale(c, w, h, s, 22, 11, 32)
    assert np.all(d[: 11 * 32].reshape(11, 32)[:, :22] == 0.375)
    up = oracle.upscale(c, w, h, s, 90, 44, 96, 2.0)
    assert np.all(up[: 44 * 96].reshape(44, 96)[:, :90] == 0.75)


def test_downscale_is_box_filter_for_even_sizes(oracle):
    rng = np.random.default_rng(3)
    w, h, s = 40, 30, 64
    a = rng.random((h + 1) * s)
    d = oracle.downscale(a, w, h, s, 20, 15, 32)
    A = a[: h * s].reshape(h, s)[:, :w]
    box = 0.25 * (A[0::2, 0::2] + A[1::2, 0::2] + A[0::2, 1::2] + A[1::2, 1::2])
    np.testing.assert_allclose(d[: 15 * 32].reshape(15, 32)[:, :20], box, rtol=0, atol=1e-12)


def test_warp_integer_shift_and_mirror(oracle):
    rng = np.random.default_rng(4)
    w, h, s = 20, 12, 32
    I = rng.random((h + 1) * s)
    u = np.full_like(I, 2.0)
    v = np.full_like(I, -1.0)
    out = oracle.warp(I, w, h, s, u, v).reshape(h + 1, s)
    Im = I.reshape(h + 1, s)
    np.testing.assert_allclose(out[1:h, : w - 2], Im[0: h - 1, 2:w], atol=1e-12)
    # past the right edge the texture mirrors: x = w-1+2 -> w-2 (half-sample symmetric)
    np.testing.assert_allclose(out[5, w - 1], Im[4, w - 2], atol=1e-12)
    # zero flow is the identity
    z = np.zeros_like(I)
    np.testing.assert_allclose(oracle.warp(I, w, h, s, z, z).reshape(h + 1, s)[:h, :w],
                               Im[:h, :w], atol=1e-12)


def test_derivatives_of_ramp(oracle):
    w, h, s = 16, 11, 32
    y, x = np.mgrid[0:h + 1, 0:s].astype(np.float64)
    I = (0.3 * x - 0.2 * y).ravel()
    Ix, Iy, Iz = oracle.derivatives(I, I, w, h, s)
    Ix = Ix.reshape(h + 1, s)
    Iy = Iy.reshape(h + 1, s)
    np.testing.assert_allclose(Ix[:h, 2: w - 2], 0.3, atol=1e-12)
    np.testing.assert_allclose(Iy[2: h - 2, :w], -0.2, atol=1e-12)
    assert np.all(Iz.reshape(h + 1, s)[:h, :w] == 0)
    # at x = 0 the taps mirror (-1 -> 0, -2 -> 1): (I1 - 8 I0 + 8 I1 - I2)/12
    row = 0.3 * np.arange(4)
    want = (row[1] - 8 * row[0] + 8 * row[1] - row[2]) / 12
    np.testing.assert_allclose(Ix[3, 0], want, atol=1e-12)


def test_data_term_branches(oracle):
    # one pixel per branch of solveReconDataL1.cu:44-63
    w, h, s = 4, 1, 4
    n = (h + 1) * s
    z = np.zeros(n)
    Ix = np.array([1.0, 0.5, -1.0, 0.0] + [0] * 4)
    Iy = np.array([0.0, 0.5, 0.0, 0.0] + [0] * 4)
    Iz = np.array([0.001, 10.0, 20.0, 3.0] + [0] * 4)
    lam, atv, ap = 50.0, 3.0, 1.0
    A = atv + ap
    du, dv = oracle.recon_data_l1(z, z, z, z, z, z, z, z, z, z, z, z, Ix, Iy, Iz, w, h, s,
                                  lam, atv, ap)
    # pixel 0: |rho| small -> du = -rho*Ix/|I|^2
    assert du[0] == pytest.approx(-0.001)
    # pixel 1: rho > lambda*g/A -> du = -lambda*Ix/A
    assert du[1] == pytest.approx(-lam * 0.5 / A) and dv[1] == pytest.approx(-lam * 0.5 / A)
    # pixel 2: Ix = -1, rho = 20 > upper = 12.5 -> du = +lambda/A
    assert du[2] == pytest.approx(lam / A)
    # pixel 3: zero gradient -> inside the band only if rho == 0, else rho > upper = 0
    assert du[3] == 0.0


def test_solve3d_triangulates_exact_point(oracle):
    # lambdams = 0 removes the smoothing: the 3x3 normal equations give the point
    K = np.array([[500.0, 0, 20], [0, 500.0, 15], [0, 0, 1]])
    ang = 0.02
    R = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]])
    t = np.array([-0.1, 0.02, 0.01])
    P = oracle.camera_matrix(K, np.eye(3), np.zeros(3))
    Q = oracle.camera_matrix(K, R, t)
    w, h, s = 6, 4, 8
    n = (h + 1) * s
    Zt = 3.0 + 0.1 * np.arange(n)
    uproj = np.zeros(n)
    vproj = np.zeros(n)
    Xt = np.zeros(n)
    Yt = np.zeros(n)
    for iy in range(h):
        for ix in range(w):
            p = ix + iy * s
            Xw = np.linalg.inv(K) @ np.array([ix, iy, 1.0]) * Zt[p]
            X1 = R @ Xw + t
            q = K @ X1
            uproj[p] = q[0] / q[2] - ix
            vproj[p] = q[1] / q[2] - iy
            Xt[p], Yt[p] = Xw[0], Xw[1]
    X0 = np.zeros(n)
    X, Y, Z = oracle.solve3d(uproj, vproj, X0, X0, X0, P, Q, 1.0, 0.0, w, h, s)
    for iy in range(h):
        sl = slice(iy * s, iy * s + w)
        np.testing.assert_allclose(X[sl], Xt[sl], rtol=1e-7, atol=1e-9)
        np.testing.assert_allclose(Y[sl], Yt[sl], rtol=1e-7, atol=1e-9)
        np.testing.assert_allclose(Z[sl], Zt[sl], rtol=1e-7)


def test_solve_uc_projection(oracle):
    w, h, s = 3, 2, 4
    n = (h + 1) * s
    X = np.full(n, 0.5)
    Y = np.full(n, -0.25)
    Z = np.full(n, 4.0)
    R = np.eye(3)
    t = np.array([0.1, 0.0, 0.0])
    uc, vc = oracle.solve_uc(X, Y, Z, R, t, 400.0, 1.5, 1.0, w, h, s)
    assert uc[1 + s] == pytest.approx(400 * 0.6 / 4 + 1.5 - 1)
    assert vc[1 + s] == pytest.approx(400 * -0.25 / 4 + 1.0 - 1)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_plain_zero_motion_is_exactly_zero(oracle, dtype):
    rng = np.random.default_rng(0)
    w, h = 48, 36
    s = align_up(w)
    I0, _ = textured_pair(rng, h, w)
    p = oracle.make_params(w, h, 3, method=oracle.METHOD_TVL1, n_warp_iters=2, n_solver_iters=10,
                           lam=50.0, theta=0.33)
    out = oracle.solve(p, pad_rows(I0, s), pad_rows(I0, s), dtype=dtype)
    assert np.all(out["u"][:, :w] == 0) and np.all(out["v"][:, :w] == 0)


def test_plain_recovers_subpixel_shift(oracle):
    rng = np.random.default_rng(1)
    w, h = 96, 64
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w, shift=(1.6, -0.7))
    p = oracle.make_params(w, h, 3, method=oracle.METHOD_TVL1, n_warp_iters=3, n_solver_iters=50,
                           lam=50.0, theta=0.33)
    out = oracle.solve(p, pad_rows(I0, s), pad_rows(I1, s))
    u = out["u"][8:-8, 8:w - 8]
    v = out["v"][8:-8, 8:w - 8]
    assert abs(np.median(u) - 1.6) < 0.05 and abs(np.median(v) + 0.7) < 0.05


def test_fp32_fp64_single_steps_agree(oracle):
    rng = np.random.default_rng(5)
    w, h, s = 37, 23, 64
    n = (h + 1) * s
    f = [rng.normal(size=n) * sc for sc in (1, 1, 0.1, 0.1, 1, 1, 0.2, 0.2, 0.3, 0.3, 0.3, 0.3,
                                            0.5, 0.5, 0.1)]
    out64 = oracle.recon_data_l1(*f, w, h, s, 50.0, 3.0303, 60.0)
    out32 = oracle.recon_data_l1(*[a.astype(np.float32) for a in f], w, h, s, 50.0, 3.0303, 60.0)
    for a, b in zip(out64, out32):
        np.testing.assert_allclose(b[: h * s], a[: h * s], rtol=1e-4, atol=1e-5)
    d64 = oracle.dual_tv(*f[:6], w, h, s, 0.25, 0.33)
    d32 = oracle.dual_tv(*[a.astype(np.float32) for a in f[:6]], w, h, s, 0.25, 0.33)
    for a, b in zip(d64, d32):
        np.testing.assert_allclose(b[: h * s], a[: h * s], rtol=1e-5, atol=1e-6)


def test_recon_zero_iterations_keep_zero_flow(oracle):
    # with no inner iterations duhat stays at its memset value 0 (Reconflow.cu:245-258)
    rng = np.random.default_rng(2)
    w, h = 40, 30
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, w)
    K = np.array([[50.0, 0, 20], [0, 50.0, 15], [0, 0, 1]])
    p = oracle.make_params(w, h, 2, n_warp_iters=2, n_solver_iters=0)
    out = oracle.solve(p, pad_rows(I0, s), pad_rows(I1, s), K0=K, K1=K, t1=np.array([0.1, 0, 0]))
    assert np.all(out["u"] == 0) and np.all(out["X"] == 0)
