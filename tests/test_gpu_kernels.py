"""Kernel-level parity on the GPU: each CUDA kernel, called through the C ABI
kernel entry points, must reproduce the FP32 oracle bit for bit on the same
inputs, at odd sizes that exercise every border branch and both stride
cases (stride > width: padding cells; stride == width: row wrap)."""
import ctypes

import numpy as np
import pytest

from helpers import assert_bitexact

pytestmark = pytest.mark.gpu

SIZES = [(37, 23, 64), (40, 22, 64), (45, 90, 64), (32, 16, 32), (5, 3, 32), (1, 1, 32)]


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy()


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def ok(rf, status):
    from reconflow_gb300 import _native

    _native.check(status)


@pytest.mark.parametrize("w,h,s", SIZES)
def test_median5_bitexact(oracle, rf, torch_cuda, w, h, s):
    rng = np.random.default_rng(w * 7 + h)
    n = (h + 1) * s
    u = rng.integers(-4, 5, n).astype(np.float32)
    u[rng.random(n) < 0.15] = -0.0
    v = rng.normal(size=n).astype(np.float32)
    lib = rf.load()
    du, dv = dev(torch_cuda, u), dev(torch_cuda, v)
    ou, ov = torch_cuda.zeros_like(du), torch_cuda.zeros_like(dv)
    ok(rf, lib.rfk_median5(P(du), P(dv), w, h, s, P(ou), P(ov), None))
    wu, wv = oracle.median5(u, v, w, h, s)
    for got, want, nm in ((host(ou), wu, "u"), (host(ov), wv, "v")):
        assert_bitexact(got.reshape(h + 1, s), want.reshape(h + 1, s), nm, region=(h, w))


@pytest.mark.parametrize("case", ["pos_zero", "neg_zero", "mixed_zero", "nan"])
def test_median5_zero_nan_bitexact(oracle, rf, torch_cuda, case):
    """Windows whose median is a zero of one sign, of both signs, and windows
    holding NaN (the exchange order decides those results), in the interior
    and at the borders."""
    w, h, s = 70, 45, 96
    rng = np.random.default_rng(len(case))
    n = (h + 1) * s
    u = rng.integers(-2, 3, n).astype(np.float32)
    v = rng.normal(size=n).astype(np.float32)
    zero = u == 0
    if case == "neg_zero":
        u[zero] = -0.0
    elif case == "mixed_zero":
        u[zero & (rng.random(n) < 0.5)] = -0.0
    elif case == "nan":
        u[rng.random(n) < 0.04] = np.nan
        v[rng.random(n) < 0.04] = np.nan
    lib = rf.load()
    du, dv = dev(torch_cuda, u), dev(torch_cuda, v)
    ou, ov = torch_cuda.zeros_like(du), torch_cuda.zeros_like(dv)
    ok(rf, lib.rfk_median5(P(du), P(dv), w, h, s, P(ou), P(ov), None))
    wu, wv = oracle.median5(u, v, w, h, s)
    for got, want, nm in ((host(ou), wu, "u"), (host(ov), wv, "v")):
        assert_bitexact(got.reshape(h + 1, s), want.reshape(h + 1, s), nm, region=(h, w))


@pytest.mark.parametrize("w,h,s", SIZES)
def test_median3d_bitexact(oracle, rf, torch_cuda, w, h, s):
    rng = np.random.default_rng(w * 11 + h)
    n = (h + 1) * s
    X = rng.integers(-3, 4, n).astype(np.float32)
    X[rng.random(n) < 0.2] = -0.0
    Y = rng.normal(size=n).astype(np.float32)
    Z = (rng.random(n) * 8).astype(np.float32)
    lib = rf.load()
    d = [dev(torch_cuda, a) for a in (X, Y, Z)]
    o = [torch_cuda.zeros_like(d[0]) for _ in range(3)]
    ok(rf, lib.rfk_median3d(*[P(t) for t in d], w, h, s, *[P(t) for t in o], None))
    want = oracle.median3d(X, Y, Z, w, h, s)
    for got, wt, nm in zip(o, want, "XYZ"):
        assert_bitexact(host(got).reshape(h + 1, s), wt.reshape(h + 1, s), nm, region=(h, w))


@pytest.mark.parametrize("w,h,s,nw,nh,ns", [(40, 30, 64, 20, 15, 32), (45, 22, 64, 22, 11, 32),
                                            (1280, 720, 1280, 640, 360, 640), (7, 5, 32, 3, 2, 32)])
@pytest.mark.parametrize("scaled", [0, 1])
def test_downscale_bitexact(oracle, rf, torch_cuda, w, h, s, nw, nh, ns, scaled):
    rng = np.random.default_rng(w + nh)
    src = rng.random((h + 1) * s).astype(np.float32)
    lib = rf.load()
    d = dev(torch_cuda, src)
    out = torch_cuda.zeros((nh + 1) * ns, dtype=torch_cuda.float32, device="cuda")
    sc = 0.5 if scaled else 1.0
    ok(rf, lib.rfk_downscale(P(d), w, h, s, nw, nh, ns, ctypes.c_float(sc), scaled, P(out), None))
    want = oracle.downscale(src, w, h, s, nw, nh, ns, sc, bool(scaled))
    assert_bitexact(host(out).reshape(nh + 1, ns), want.reshape(nh + 1, ns), "downscale",
                    region=(nh, nw))


@pytest.mark.parametrize("w,h,s,nw,nh,ns", [(20, 15, 32, 40, 30, 64), (22, 11, 32, 45, 22, 64),
                                            (40, 22, 64, 80, 45, 96), (3, 2, 32, 7, 5, 32)])
def test_upscale_bitexact(oracle, rf, torch_cuda, w, h, s, nw, nh, ns):
    rng = np.random.default_rng(nw)
    src = rng.normal(size=(h + 1) * s).astype(np.float32)
    lib = rf.load()
    d = dev(torch_cuda, src)
    out = torch_cuda.zeros((nh + 1) * ns, dtype=torch_cuda.float32, device="cuda")
    ok(rf, lib.rfk_upscale(P(d), w, h, s, nw, nh, ns, ctypes.c_float(2.0), P(out), None))
    want = oracle.upscale(src, w, h, s, nw, nh, ns, 2.0)
    assert_bitexact(host(out).reshape(nh + 1, ns), want.reshape(nh + 1, ns), "upscale",
                    region=(nh, nw))


@pytest.mark.parametrize("w,h,s", SIZES)
def test_warp_bitexact(oracle, rf, torch_cuda, w, h, s):
    rng = np.random.default_rng(w * 3 + h)
    n = (h + 1) * s
    I = rng.random(n).astype(np.float32)
    u = (rng.normal(size=n) * 3).astype(np.float32)
    v = (rng.normal(size=n) * 3).astype(np.float32)
    u[::7] = 2.5 * w  # far outside: exercises the periodic mirror
    v[::11] = -1.7 * h
    u[5] = np.nan
    lib = rf.load()
    dI, du, dv = dev(torch_cuda, I), dev(torch_cuda, u), dev(torch_cuda, v)
    out = torch_cuda.zeros_like(dI)
    ok(rf, lib.rfk_warp(P(dI), w, h, s, P(du), P(dv), P(out), None))
    want = oracle.warp(I, w, h, s, u, v)
    assert_bitexact(host(out).reshape(h + 1, s), want.reshape(h + 1, s), "warp", region=(h, w))


@pytest.mark.parametrize("w,h,s", SIZES)
def test_derivatives_bitexact(oracle, rf, torch_cuda, w, h, s):
    rng = np.random.default_rng(w * 5 + h)
    n = (h + 1) * s
    I0 = rng.random(n).astype(np.float32)
    I1 = rng.random(n).astype(np.float32)
    lib = rf.load()
    a, b = dev(torch_cuda, I0), dev(torch_cuda, I1)
    o = [torch_cuda.zeros_like(a) for _ in range(3)]
    ok(rf, lib.rfk_derivatives(P(a), P(b), w, h, s, *[P(t) for t in o], None))
    want = oracle.derivatives(I0, I1, w, h, s)
    for got, wt, nm in zip(o, want, ("Ix", "Iy", "Iz")):
        assert_bitexact(host(got).reshape(h + 1, s), wt.reshape(h + 1, s), nm, region=(h, w))


@pytest.mark.parametrize("w,h,s", SIZES + [(70, 45, 96), (2, 2, 32)])
def test_fused_warp_derivatives_bitexact(oracle, rf, torch_cuda, w, h, s):
    """The solver's fused warp + derivatives kernel (shared-memory tile with
    a mirrored 2-pixel halo) against the oracle's warp followed by its
    derivatives, including tiles whose halo wraps several times (w, h < 5)."""
    rng = np.random.default_rng(w * 13 + h)
    n = (h + 1) * s
    I0 = rng.random(n).astype(np.float32)
    I1 = rng.random(n).astype(np.float32)
    u = (rng.normal(size=n) * 3).astype(np.float32)
    v = (rng.normal(size=n) * 3).astype(np.float32)
    u[::7] = 2.5 * w
    v[::11] = -1.7 * h
    lib = rf.load()
    d = [dev(torch_cuda, a) for a in (I0, I1, u, v)]
    o = [torch_cuda.zeros_like(d[0]) for _ in range(3)]
    ok(rf, lib.rfk_warp_derivatives(*[P(t) for t in d], w, h, s, *[P(t) for t in o], None))
    i1w = oracle.warp(I1, w, h, s, u, v)
    want = oracle.derivatives(I0, i1w, w, h, s)
    for got, wt, nm in zip(o, want, ("Ix", "Iy", "Iz")):
        assert_bitexact(host(got).reshape(h + 1, s), wt.reshape(h + 1, s), nm, region=(h, w))


def test_rgb_to_gray_bitexact(oracle, rf, torch_cuda):
    rng = np.random.default_rng(9)
    w, h, s = 37, 23, 64
    rgb = rng.integers(0, 256, (h, s, 3)).astype(np.uint8)
    lib = rf.load()
    d = dev(torch_cuda, rgb)
    out = torch_cuda.zeros(h * s, dtype=torch_cuda.float32, device="cuda")
    ok(rf, lib.rfk_rgb_to_gray(P(d), w, h, s, P(out), None))
    want = np.zeros(h * s, np.float32)
    oracle.lib().rfo_rgb_to_gray_f32(rgb.ctypes.data_as(ctypes.c_void_p), w, h, s,
                                      want.ctypes.data_as(ctypes.c_void_p))
    assert_bitexact(host(out).reshape(h, s), want.reshape(h, s), "gray", region=(h, w))


@pytest.mark.parametrize("rng_w", [1, 3])
def test_remove_edge_artifacts_bitexact(oracle, rf, torch_cuda, rng_w):
    rng = np.random.default_rng(rng_w)
    w, h, s = 37, 23, 64
    n = (h + 1) * s
    X, Y, Z = (rng.normal(size=n).astype(np.float32) for _ in range(3))
    lib = rf.load()
    d = [dev(torch_cuda, a) for a in (X, Y, Z)]
    o = [torch_cuda.zeros_like(d[0]) for _ in range(3)]
    ok(rf, lib.rfk_remove_edge_artifacts(*[P(t) for t in d], rng_w, ctypes.c_float(0.8), w, h, s,
                                         *[P(t) for t in o], None))
    want = oracle.remove_edge_artifacts(X, Y, Z, rng_w, 0.8, w, h, s)
    for got, wt, nm in zip(o, want, "XYZ"):
        assert_bitexact(host(got).reshape(h + 1, s), wt.reshape(h + 1, s), nm, region=(h, w))


def test_flow_color_matches_formula(rf, torch_cuda):
    w, h, s = 33, 9, 64
    rng = np.random.default_rng(2)
    u = (rng.normal(size=h * s) * 4).astype(np.float32)
    v = (rng.normal(size=h * s) * 4).astype(np.float32)
    lib = rf.load()
    du, dv = dev(torch_cuda, u), dev(torch_cuda, v)
    out = torch_cuda.zeros(h * s * 3, dtype=torch_cuda.float32, device="cuda")
    ok(rf, lib.rfk_flow_to_color(P(du), P(dv), w, h, s, ctypes.c_float(5.0), P(out), None))
    got = host(out).reshape(h, s, 3)[:, :w]
    # float64 restatement of ComputeColorKernel (flowToHSV.cu:194-302)
    R = [255] * 16 + [213, 170, 128, 85, 43] + [0] * 16 + [19, 39, 58, 78, 98, 117, 137, 156, 176,
                                                          196, 215, 235] + [255] * 6
    G = [0, 17, 34, 51, 68, 85, 102, 119, 136, 153, 170, 187, 204, 221, 238] + [255] * 11 + \
        [232, 209, 186, 163, 140, 116, 93, 70, 47, 24] + [0] * 19
    B = [0] * 22 + [63, 127, 191] + [255] * 25 + [213, 170, 128, 85, 43]
    wheel = np.array([R, G, B], np.float64) / 255.0
    U = u.reshape(h, s)[:, :w] / 5.0
    V = v.reshape(h, s)[:, :w] / 5.0
    rad = np.sqrt(U * U + V * V)
    a = np.arctan2(-V, -U) / 3.14159
    fk = (a + 1) / 2 * 54 + 1
    k0 = np.floor(fk).astype(int)
    k1 = k0 + 1
    k1[k1 == 56] = 1
    f = fk - k0
    col = (1 - f) * wheel[:, k0 % 55] + f * wheel[:, k1 % 55]
    col = np.where(rad <= 1, 1 - rad * (1 - col), col * 0.75)
    np.testing.assert_allclose(got[..., 2], col[0], atol=2e-5)
    np.testing.assert_allclose(got[..., 1], col[1], atol=2e-5)
    np.testing.assert_allclose(got[..., 0], col[2], atol=2e-5)


@pytest.mark.parametrize("w,h,s", SIZES)
def test_warp_update_bitexact(oracle, rf, torch_cuda, w, h, s):
    """median5(duhat) -> u += it -> median5(u) (Reconflow.cu:410-420)."""
    rng = np.random.default_rng(w * 13 + h)
    n = (h + 1) * s
    du, dv = (rng.normal(size=n).astype(np.float32) for _ in range(2))
    u, v = ((rng.normal(size=n) * 3).astype(np.float32) for _ in range(2))
    lib = rf.load()
    d = [dev(torch_cuda, a) for a in (du, dv, u, v)]
    tmp = [torch_cuda.zeros_like(d[0]) for _ in range(2)]
    out = [torch_cuda.zeros_like(d[0]) for _ in range(2)]
    ok(rf, lib.rfk_warp_update(*[P(t) for t in d], w, h, s, *[P(t) for t in tmp],
                               *[P(t) for t in out], None))
    mu, mv = oracle.median5(du, dv, w, h, s)
    tu, tv = u + mu, v + mv
    wu, wv = oracle.median5(tu, tv, w, h, s)
    for got, want, nm in ((out[0], wu, "u"), (out[1], wv, "v")):
        assert_bitexact(host(got).reshape(h + 1, s), want.reshape(h + 1, s), nm, region=(h, w))
