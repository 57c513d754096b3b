"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates the reference's update equations and schedule on the CPU
(``rf_oracle.cpp``): ``*_f64`` entry points are the FP64 oracle that parity is
measured against, ``*_f32`` the reference-semantics FP32 path that is also the
timed CPU baseline.  Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "librforacle.so")
_lib = None

METHOD_TVL1 = 0
METHODR_TVL1_MS = 14
METHODR_TVL1_MS_FN = 17
METHODR_TVL1_MS_FNSPARSE = 20

INPUT_F32, INPUT_RGB8, INPUT_U8, INPUT_U16 = 0, 1, 2, 3


class RfoParams(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int), ("input_type", ctypes.c_int),
        ("n_levels", ctypes.c_int), ("scale", ctypes.c_float), ("method", ctypes.c_int),
        ("lambda_", ctypes.c_float), ("lambdaf", ctypes.c_float), ("lambdams", ctypes.c_float),
        ("alpha_tv", ctypes.c_float), ("alpha_proj", ctypes.c_float), ("alpha_fn", ctypes.c_float),
        ("tau", ctypes.c_float), ("theta", ctypes.c_float),
        ("n_warp_iters", ctypes.c_int), ("n_solver_iters", ctypes.c_int),
        ("stride_alignment", ctypes.c_int), ("fix_quirks", ctypes.c_int),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle library with its Makefile (g++, OpenMP)."""
    srcs = [os.path.join(_HERE, f) for f in ("rf_oracle.cpp", "pose_oracle.cpp", "Makefile")]
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(f) for f in srcs)
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
    return _lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def _real(dtype):
    return ctypes.c_double if np.dtype(dtype) == np.float64 else ctypes.c_float


def _sfx(dtype):
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def set_num_threads(n: int) -> None:
    lib().rfo_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().rfo_num_threads())


def pyramid_dims(w, h, levels, scale=2.0, align=32):
    W = (ctypes.c_int * levels)()
    H = (ctypes.c_int * levels)()
    S = (ctypes.c_int * levels)()
    lib().rfo_pyramid_dims(int(w), int(h), int(levels), ctypes.c_float(scale), int(align), W, H, S)
    return list(W), list(H), list(S)


def k_pyramid(K, levels, scale=2.0):
    K = np.ascontiguousarray(K, dtype=np.float64).reshape(9)
    out = np.zeros((levels, 9), np.float64)
    lib().rfo_k_pyramid(_ptr(K), int(levels), ctypes.c_float(scale), _ptr(out))
    return out.reshape(levels, 3, 3)


def camera_matrix(K, R, t):
    K = np.ascontiguousarray(K, np.float64).reshape(9)
    R = np.ascontiguousarray(R, np.float64).reshape(9)
    t = np.ascontiguousarray(t, np.float64).reshape(3)
    P = np.zeros(12, np.float64)
    lib().rfo_camera_matrix(_ptr(K), _ptr(R), _ptr(t), _ptr(P))
    return P.reshape(3, 4)


def _call(name, dtype, *args):
    fn = getattr(lib(), f"rfo_{name}_{_sfx(dtype)}")
    real = _real(dtype)
    cargs = []
    for a in args:
        if isinstance(a, np.ndarray):
            cargs.append(_ptr(a))
        elif a is None:
            cargs.append(None)
        elif isinstance(a, float):
            cargs.append(real(a))
        else:
            cargs.append(int(a))
    fn.restype = ctypes.c_int
    return fn(*cargs)


def _field(h, s, dtype):
    # level buffers carry one zero guard row past the image (row `h`)
    return np.zeros(((h + 1) * s,), dtype=dtype)


# --- per-kernel entry points (arrays are flat, `stride` elements per row) ---

def downscale(src, w, h, s, nw, nh, ns, scale=1.0, scaled=False):
    out = np.zeros(nh * ns + ns, src.dtype)
    _call("downscale", src.dtype, src, w, h, s, nw, nh, ns, float(scale), int(scaled), out)
    return out


def upscale(src, w, h, s, nw, nh, ns, scale):
    out = np.zeros(nh * ns + ns, src.dtype)
    _call("upscale", src.dtype, src, w, h, s, nw, nh, ns, float(scale), out)
    return out


def warp(src, w, h, s, u, v):
    out = np.zeros_like(src)
    _call("warp", src.dtype, src, w, h, s, u, v, out)
    return out


def derivatives(I0, I1, w, h, s):
    Ix, Iy, Iz = (np.zeros_like(I0) for _ in range(3))
    _call("derivatives", I0.dtype, I0, I1, w, h, s, Ix, Iy, Iz)
    return Ix, Iy, Iz


def median5(u, v, w, h, s):
    ou, ov = np.zeros_like(u), np.zeros_like(v)
    _call("median5", u.dtype, u, v, w, h, s, ou, ov)
    return ou, ov


def median3d(X, Y, Z, w, h, s):
    o = [np.zeros_like(X) for _ in range(3)]
    _call("median3d", X.dtype, X, Y, Z, w, h, s, *o)
    return tuple(o)


def recon_data_l1(u, v, duhat, dvhat, uproj, vproj, sku, skv, pu1, pu2, pv1, pv2, Ix, Iy, Iz,
                  w, h, s, lam, alpha_tv, alpha_proj, alpha_fn=0.0, prior=0, ufn=None, vfn=None,
                  mask=None):
    o1, o2 = np.zeros_like(u), np.zeros_like(u)
    _call("recon_data_l1", u.dtype, u, v, duhat, dvhat, uproj, vproj, ufn, vfn, mask, sku, skv,
          pu1, pu2, pv1, pv2, Ix, Iy, Iz, w, h, s, float(lam), float(alpha_tv), float(alpha_proj),
          float(alpha_fn), int(prior), o1, o2)
    return o1, o2


def data_l1(duhat, dvhat, pu1, pu2, pv1, pv2, Ix, Iy, Iz, w, h, s, lam, theta):
    o1, o2 = np.zeros_like(duhat), np.zeros_like(duhat)
    _call("data_l1", duhat.dtype, duhat, dvhat, pu1, pu2, pv1, pv2, Ix, Iy, Iz, w, h, s,
          float(lam), float(theta), o1, o2)
    return o1, o2


def dual_tv(duhat, dvhat, pu1, pu2, pv1, pv2, w, h, s, tau, theta):
    o = [np.zeros_like(duhat) for _ in range(4)]
    _call("dual_tv", duhat.dtype, duhat, dvhat, pu1, pu2, pv1, pv2, w, h, s, float(tau),
          float(theta), *o)
    return tuple(o)


def uv_proj(u, v, du, dv, uc, vc, sku, skv, w, h, s, lambdaf, alpha_proj):
    o1, o2 = np.zeros_like(u), np.zeros_like(u)
    _call("uv_proj", u.dtype, u, v, du, dv, uc, vc, sku, skv, w, h, s, float(lambdaf),
          float(alpha_proj), o1, o2)
    return o1, o2


def solve3d(uproj, vproj, X0, Y0, Z0, P, Q, lambdaf, lambdams, w, h, s):
    o = [np.zeros_like(X0) for _ in range(3)]
    P = np.ascontiguousarray(P, X0.dtype).reshape(12)
    Q = np.ascontiguousarray(Q, X0.dtype).reshape(12)
    _call("solve3d", X0.dtype, uproj, vproj, X0, Y0, Z0, P, Q, float(lambdaf), float(lambdams),
          w, h, s, *o)
    return tuple(o)


def cleanup3d(X, Y, Z, Xm, Ym, Zm, w, h, s):
    o = [np.zeros_like(X) for _ in range(3)]
    _call("cleanup3d", X.dtype, X, Y, Z, Xm, Ym, Zm, w, h, s, *o)
    return tuple(o)


def solve_uc(X, Y, Z, R, t, f, cx, cy, w, h, s):
    o1, o2 = np.zeros_like(X), np.zeros_like(X)
    R = np.ascontiguousarray(R, X.dtype).reshape(9)
    t = np.ascontiguousarray(t, X.dtype).reshape(3)
    _call("solve_uc", X.dtype, X, Y, Z, R, t, float(f), float(cx), float(cy), w, h, s, o1, o2)
    return o1, o2


def update_sk(sku, skv, u, v, du, dv, uproj, vproj, w, h, s):
    o1, o2 = np.zeros_like(sku), np.zeros_like(sku)
    _call("update_sk", sku.dtype, sku, skv, u, v, du, dv, uproj, vproj, w, h, s, o1, o2)
    return o1, o2


def remove_edge_artifacts(X, Y, Z, rng, max_area, w, h, s):
    o = [np.zeros_like(X) for _ in range(3)]
    _call("remove_edge_artifacts", X.dtype, X, Y, Z, int(rng), float(max_area), w, h, s, *o)
    return tuple(o)


def make_params(width, height, n_levels, method=METHODR_TVL1_MS, input_type=INPUT_F32, scale=2.0,
                lam=50.0, lambdaf=100.0, lambdams=100.0, alpha_tv=1.0 / 0.33, alpha_proj=1.0,
                alpha_fn=0.5, tau=0.25, theta=0.33, n_warp_iters=1, n_solver_iters=100,
                stride_alignment=32, fix_quirks=0):
    return RfoParams(width, height, input_type, n_levels, scale, method, lam, lambdaf, lambdams,
                     alpha_tv, alpha_proj, alpha_fn, tau, theta, n_warp_iters, n_solver_iters,
                     stride_alignment, fix_quirks)


def solve(params: RfoParams, I0, I1, K0=None, K1=None, R0=None, t0=None, R1=None, t1=None,
          ufn=None, vfn=None, mask=None, dtype=np.float64):
    """Full reference schedule.  Images are (height, stride) arrays of the input
    type; returns dict of (height, stride) arrays u, v (and X, Y, Z)."""
    W, H, S = pyramid_dims(params.width, params.height, params.n_levels, params.scale,
                           params.stride_alignment)
    s, h = S[0], H[0]
    I0 = np.ascontiguousarray(I0)
    I1 = np.ascontiguousarray(I1)
    in_stride = s
    eye = np.eye(3)
    z3 = np.zeros(3)
    K0 = np.ascontiguousarray(eye if K0 is None else K0, np.float64)
    K1 = np.ascontiguousarray(K0 if K1 is None else K1, np.float64)
    R0 = np.ascontiguousarray(eye if R0 is None else R0, np.float64)
    t0 = np.ascontiguousarray(z3 if t0 is None else t0, np.float64)
    R1 = np.ascontiguousarray(eye if R1 is None else R1, np.float64)
    t1 = np.ascontiguousarray(z3 if t1 is None else t1, np.float64)
    prior = params.method in (METHODR_TVL1_MS_FN, METHODR_TVL1_MS_FNSPARSE)
    if prior:
        ufn = np.ascontiguousarray(ufn, np.float32)
        vfn = np.ascontiguousarray(vfn, np.float32)
        if mask is not None:
            mask = np.ascontiguousarray(mask, np.float32)
    out = {k: np.zeros((h, s), dtype) for k in ("u", "v", "X", "Y", "Z")}
    fn = getattr(lib(), f"rfo_solve_{_sfx(dtype)}")
    rc = fn(ctypes.byref(params), _ptr(I0), _ptr(I1), int(in_stride), _ptr(K0), _ptr(K1),
            _ptr(R0), _ptr(t0), _ptr(R1), _ptr(t1), _ptr(ufn) if prior else None,
            _ptr(vfn) if prior else None, _ptr(mask) if prior else None, _ptr(out["u"]),
            _ptr(out["v"]), _ptr(out["X"]), _ptr(out["Y"]), _ptr(out["Z"]))
    if rc != 0:
        raise RuntimeError(f"oracle solve failed: {rc}")
    if params.method == METHOD_TVL1:
        for k in ("X", "Y", "Z"):
            out.pop(k)
    return out


def solve_warm(params: RfoParams, I0, I1, level, u0, v0, X0, Y0, Z0, warps, iters, K0=None,
               K1=None, R0=None, t0=None, R1=None, t1=None, dtype=np.float32):
    """Schedule started at pyramid `level` from the given flow and points
    (float planes with that level's stride), in FP32 or FP64.  Returns dict of
    (height, stride) arrays."""
    W, H, S = pyramid_dims(params.width, params.height, params.n_levels, params.scale,
                           params.stride_alignment)
    s, h = S[0], H[0]
    eye, z3 = np.eye(3), np.zeros(3)
    K0 = np.ascontiguousarray(eye if K0 is None else K0, np.float64)
    K1 = np.ascontiguousarray(K0 if K1 is None else K1, np.float64)
    R0 = np.ascontiguousarray(eye if R0 is None else R0, np.float64)
    t0 = np.ascontiguousarray(z3 if t0 is None else t0, np.float64)
    R1 = np.ascontiguousarray(eye if R1 is None else R1, np.float64)
    t1 = np.ascontiguousarray(z3 if t1 is None else t1, np.float64)
    ws = [np.ascontiguousarray(a, np.float32) for a in (u0, v0, X0, Y0, Z0)]
    out = {k: np.zeros((h, s), dtype) for k in ("u", "v", "X", "Y", "Z")}
    I0 = np.ascontiguousarray(I0, np.float32)
    I1 = np.ascontiguousarray(I1, np.float32)
    fn = getattr(lib(), f"rfo_solve_warm_{_sfx(dtype)}")
    rc = fn(ctypes.byref(params), _ptr(I0), _ptr(I1), int(s), _ptr(K0), _ptr(K1), _ptr(R0),
            _ptr(t0), _ptr(R1), _ptr(t1), int(level), *[_ptr(a) for a in ws], int(warps),
            int(iters), *[_ptr(out[k]) for k in ("u", "v", "X", "Y", "Z")])
    if rc != 0:
        raise RuntimeError(f"oracle warm solve failed: {rc}")
    return out


def energy(I0, I1, u, v, X, Y, Z, w, h, s, lam, alpha_proj, R1, t1, K1, recon=True):
    """Solution energy on level 0 (data + TV + reprojection), in double."""
    fn = lib().rfo_energy
    fn.restype = ctypes.c_double
    arrs = [np.ascontiguousarray(a, np.float32) for a in (I0, I1, u, v, X, Y, Z)]
    R1 = np.ascontiguousarray(R1, np.float64)
    t1 = np.ascontiguousarray(t1, np.float64)
    K1 = np.ascontiguousarray(K1, np.float64)
    return float(fn(*[_ptr(a) for a in arrs], int(w), int(h), int(s), ctypes.c_float(lam),
                    ctypes.c_float(alpha_proj), _ptr(R1), _ptr(t1), _ptr(K1), int(recon)))


# ---------------------------------------------------------------------------
# Pose front end (pose_oracle.cpp): the feature stages the GPU runs
# ---------------------------------------------------------------------------

def surf_integral(img):
    """Integral image of an 8-bit frame, (h + 1) x (w + 1) uint32."""
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape
    out = np.zeros((h + 1, w + 1), np.uint32)
    lib().rfo_surf_integral(img.ctypes.data_as(ctypes.c_void_p), w, h,
                            out.ctypes.data_as(ctypes.c_void_p))
    return out


def surf_responses(img, octave, layers):
    """Determinant-of-Hessian responses of one octave: layers x (h >> o) x (w >> o)."""
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape
    out = np.zeros((layers, h >> octave, w >> octave), np.float32)
    lib().rfo_surf_responses(img.ctypes.data_as(ctypes.c_void_p), w, h, octave, layers,
                             out.ctypes.data_as(ctypes.c_void_p))
    return out


def surf_detect(img, threshold=2000.0, n_octaves=4, n_layers=2, max_kp=None, cand_cap=None):
    """Keypoints [n][6] (x, y, scale, angle, response, octave) strongest first,
    and descriptors [n][64]; None when the candidates exceed cand_cap."""
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape
    max_kp = max_kp or max(16, w * h // 100)
    cand_cap = cand_cap or max(4 * max_kp, 65536)
    kp = np.zeros((max_kp, 6), np.float32)
    desc = np.zeros((max_kp, 64), np.float32)
    f = lib().rfo_surf_detect
    f.restype = ctypes.c_int
    n = f(img.ctypes.data_as(ctypes.c_void_p), w, h, ctypes.c_double(threshold), n_octaves,
          n_layers, max_kp, cand_cap, kp.ctypes.data_as(ctypes.c_void_p),
          desc.ctypes.data_as(ctypes.c_void_p))
    if n < 0:
        return None
    return kp[:n].copy(), desc[:n].copy()


def surf_match(d0, d1):
    """Nearest and second-nearest descriptor of frame 1 for each of frame 0:
    (index, squared distance 1, squared distance 2)."""
    d0 = np.ascontiguousarray(d0, np.float32)
    d1 = np.ascontiguousarray(d1, np.float32)
    n0, n1 = len(d0), len(d1)
    best = np.zeros(n0, np.int32)
    b1 = np.zeros(n0, np.float32)
    b2 = np.zeros(n0, np.float32)
    lib().rfo_surf_match(d0.ctypes.data_as(ctypes.c_void_p), n0,
                         d1.ctypes.data_as(ctypes.c_void_p), n1,
                         best.ctypes.data_as(ctypes.c_void_p), b1.ctypes.data_as(ctypes.c_void_p),
                         b2.ctypes.data_as(ctypes.c_void_p))
    return best, b1, b2
