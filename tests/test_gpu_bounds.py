"""Bounds-checked debug build (RF_BOUNDS_CHECK, ``lib/librfgb300_check.so``).

Every field access of the inner iteration (the data, dual, projection and
3D steps of ``recon_a_px`` / ``recon_b_px``) goes through a checked
accessor: an index outside its plane is counted and redirected to a sink
cell, never followed.  A child process loads the checked library, makes one
deliberate out-of-range access through ``rf_debug_bounds_selftest`` (the
count must be exactly 1, at index 1 of a one-float field), then runs single
pair solves at ragged sizes (both the two-launch loop and the cluster
kernel), every prior method, and a ragged batch: the count must be 0.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, ROOT)
sys.path.insert(0, ROOT + "/tests")
import reconflow_gb300 as rf
from reconflow_gb300 import _native as N
from helpers import align_up, pad_rows, textured_pair

lib = rf.load()
assert lib._name.endswith("librfgb300_check.so"), lib._name


def take():
    c = ctypes.c_ulonglong(0)
    first = ctypes.c_longlong(-1)
    N.check(lib.rf_debug_bounds(ctypes.byref(c), ctypes.byref(first)))
    return c.value, first.value


N.check(lib.rf_debug_bounds_selftest())
c, first = take()
assert (c, first) == (1, 1), (c, first)
assert take() == (0, -1)


def scene(w, h, seed):
    rng = np.random.default_rng(seed)
    s = align_up(w)
    I0, I1 = textured_pair(rng, h, s, shift=(1.3, -0.6))
    K = np.array([[0.8 * w, 0, w / 2], [0, 0.8 * w, h / 2], [0, 0, 1.0]])
    c, sn = np.cos(0.01), np.sin(0.01)
    R = np.array([[c, 0, sn], [0, 1, 0], [-sn, 0, c]])
    t = np.array([-0.1, 0.01, 0.02])
    ufn = (rng.normal(size=(h, s)) * 0.5 + 1.0).astype(np.float32)
    vfn = (rng.normal(size=(h, s)) * 0.5).astype(np.float32)
    mask = (rng.random((h, s)) < 0.3).astype(np.float32)
    return I0, I1, K, R, t, ufn, vfn, mask


for (w, h, L, method, cluster_px) in [(37, 23, 2, 14, 0), (37, 23, 2, 14, 1 << 40),
                                      (161, 91, 3, 14, 0), (161, 91, 3, 14, 1 << 40),
                                      (96, 72, 3, 17, -1), (130, 70, 3, 20, -1),
                                      (5, 3, 1, 14, -1), (64, 48, 3, 0, -1)]:
    lib.rf_set_cluster_pixels(cluster_px)
    I0, I1, K, R, t, ufn, vfn, mask = scene(w, h, w * h + method)
    if method == 0:
        f = rf.CudaFlow()
        f.initialize(w, h, 1, 5, L, 2.0, 0, 50.0, 0.0, 0.33, 0.25, 2, 6)
        f.copyImagesToDevice(I0, I1)
        f.solveOpticalFlow()
    else:
        f = rf.ReconFlow()
        f.initializeR(w, h, 1, L, 2.0, method, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25,
                      2, 6, cvType=5, fix_quirks=1)
        f.setCameraMatrices(K, K)
        f.copyImagesToDevice(I0, I1)
        if method in (17, 20):
            f.copySparseOpticalFlowToDevice(ufn, vfn, mask if method == 20 else None)
        f.solveR(R, t, 5.0)
    u, v = f.copyOpticalFlowToHost()
    f.close()
    assert np.isfinite(u[:, :w]).all()
    got = take()
    assert got == (0, -1), ((w, h, L, method, cluster_px), got)
lib.rf_set_cluster_pixels(-1)

sizes = [(64, 48), (37, 23), (130, 70), (45, 90)]
b = rf.ReconFlowBatch(sizes, 2, method=14, lambda_=50.0, lambdaf=0.1, lambdams=100.0,
                      alphaTv=1 / 0.33, alphaProj=60.0, tau=0.25, nWarpIters=2, nSolverIters=5,
                      fix_quirks=1)
Rs, ts = [], []
for i, (w, h) in enumerate(sizes):
    I0, I1, K, R, t, *_ = scene(w, h, 300 + i)
    s = b.strides[i]
    b.setCameraMatrices(i, K, K)
    b.copyImagesToDevice(i, pad_rows(I0[:, :w], s), pad_rows(I1[:, :w], s))
    Rs.append(R)
    ts.append(t)
b.solveR(Rs, ts)
b.synchronize()
b.close()
got = take()
assert got == (0, -1), ("batch", got)
print("BOUNDS OK")
"""


def test_checked_build_counts_only_the_planted_access():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from reconflow_gb300 import build

    build.build(bounds_check=True)
    env = dict(os.environ, RF_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + CHILD], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "BOUNDS OK" in r.stdout, r.stdout + r.stderr
