"""Committed regression fixtures of the oracle (tests/golden/oracle_cases.npz,
made by tests/golden/make_golden.py).

CPU: the oracle reproduces the fixtures bit for bit (FP32 and FP64).  GPU:
the CUDA path, through the C ABI, reproduces the FP32 fixtures bit for bit
(a fixed-vector check that does not depend on building the oracle)."""
import os
import sys

import numpy as np
import pytest

from helpers import assert_bitexact

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as G  # noqa: E402

FIX = np.load(os.path.join(HERE, "golden", "oracle_cases.npz"))


def test_inputs_regenerate():
    c = G.cases()
    for k in ("I0", "I1", "K", "R", "t", "med_u", "med_v"):
        np.testing.assert_array_equal(c[k], FIX[k])


def test_oracle_reproduces_fixtures(oracle):
    out = G.run(oracle, G.cases())
    for k, v in out.items():
        got, want = np.asarray(v), FIX[k]
        if got.dtype == np.float64:
            same = (got == want) | (np.isnan(got) & np.isnan(want))
            assert same.all(), k
        else:
            assert_bitexact(got, want, k)


@pytest.mark.gpu
def test_gpu_reproduces_fp32_fixtures(rf):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = G.cases()
    w, h = c["w"], c["h"]
    r = G.RECON
    f = rf.ReconFlow()
    f.initializeR(w, h, 1, 2, 2.0, 14, r["lam"], 0.0, r["lambdaf"], r["lambdams"], r["alpha_tv"],
                  r["alpha_proj"], 0.5, r["tau"], r["n_warp_iters"], r["n_solver_iters"], cvType=5,
                  fix_quirks=r["fix_quirks"])
    f.setCameraMatrices(c["K"], c["K"])
    f.copyImagesToDevice(c["I0"], c["I1"])
    f.solveR(c["R"], c["t"], 5.0)
    u, v = f.copyOpticalFlowToHost()
    X, Y, Z = f.copy3dToHost()
    f.close()
    for k, a in zip("uvXYZ", (u, v, X, Y, Z)):
        assert_bitexact(a, FIX[f"recon_{k}_f32"], f"recon {k}", region=(h, w))
    p = G.PLAIN
    g = rf.CudaFlow()
    g.initialize(w, h, 1, 5, 2, 2.0, 0, p["lam"], 0.0, p["theta"], p["tau"], p["n_warp_iters"],
                 p["n_solver_iters"])
    g.copyImagesToDevice(c["I0"], c["I1"])
    g.solveOpticalFlow()
    u, v = g.copyOpticalFlowToHost()
    g.close()
    assert_bitexact(u, FIX["plain_u_f32"], "plain u", region=(h, w))
    assert_bitexact(v, FIX["plain_v_f32"], "plain v", region=(h, w))
    # 5x5 median with ties, signed zeros and a NaN (rfk_median5)
    import ctypes

    from reconflow_gb300 import _native

    lib = _native.load()
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float32).ravel(), device="cuda")  # noqa: E731
    a, b = T(c["med_u"]), T(c["med_v"])
    oa, ob = torch.zeros_like(a), torch.zeros_like(b)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    _native.check(lib.rfk_median5(P(a), P(b), 27, 20, 32, P(oa), P(ob), None))
    torch.cuda.synchronize()
    assert_bitexact(oa.cpu().numpy().reshape(21, 32), FIX["median5_u"], "median5 u", region=(20, 27))
    assert_bitexact(ob.cpu().numpy().reshape(21, 32), FIX["median5_v"], "median5 v", region=(20, 27))
