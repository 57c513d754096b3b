"""Allocation failures injected on the host (rf_test_fail_alloc): for every
create call of the library, the k-th device or pinned allocation fails for
k = 1, 2, ... until the call needs fewer allocations than k.  Each failing
call must return RF_ERR_OOM without a crash, and device memory must be back
where it started once the failed and the final successful objects are gone
(nothing leaked on any failure path).  No GPU fault is involved: the failing
allocation never reaches the driver."""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OOM = 4  # RF_ERR_OOM


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.zeros(1, device="cuda")
    return torch


def _free(torch):
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _sweep(rf, torch, make, close, max_k=80):
    from reconflow_gb300 import _native as N

    lib = rf.load()
    gc.collect()
    before = _free(torch)
    failed = 0
    try:
        for k in range(1, max_k + 1):
            lib.rf_test_fail_alloc(k)
            try:
                obj = make()
            except N.RfError as e:
                assert e.status == OOM, str(e)
                failed += 1
                continue
            lib.rf_test_fail_alloc(0)
            close(obj)
            break
        else:
            pytest.fail("the create call still failed with every allocation allowed")
    finally:
        lib.rf_test_fail_alloc(0)
    gc.collect()
    after = _free(torch)
    return failed, before - after


def test_solver_create_failures_leak_nothing(rf, torch_cuda):
    def make():
        f = rf.ReconFlow()
        f.initializeR(640, 480, 1, 5, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25,
                      1, 5, cvType=16)  # RGB8 input: two staging buffers too
        return f

    failed, leaked = _sweep(rf, torch_cuda, make, lambda f: f.close())
    assert failed >= 5
    assert abs(leaked) < (8 << 20), leaked


def test_batch_create_failures_leak_nothing(rf, torch_cuda):
    def make():
        return rf.ReconFlowBatch([(320, 240), (200, 120)], 4, method=14, nWarpIters=1,
                                 nSolverIters=5)

    failed, leaked = _sweep(rf, torch_cuda, make, lambda b: b.close())
    assert failed >= 5
    assert abs(leaked) < (8 << 20), leaked


def test_network_create_failures_leak_nothing(rf, torch_cuda):
    from reconflow_gb300.warmstart import WarmStartNet

    failed, leaked = _sweep(rf, torch_cuda, lambda: WarmStartNet(4, 60, 80, seed=0),
                            lambda n: n.close())
    assert failed >= 5
    assert abs(leaked) < (8 << 20), leaked


def test_pose_create_failures_leak_nothing(rf, torch_cuda):
    # CameraPose creates its device handle for the frame size of its first
    # solve (rf_pose_create)
    frame = (np.arange(240 * 320, dtype=np.int64).reshape(240, 320) * 37 % 251).astype(np.uint8)

    def make():
        cp = rf.CameraPose()
        cp.initialize(np.array([[300.0, 0, 160], [0, 300.0, 120], [0, 0, 1]]), 20.0)
        try:
            cp.solvePose_8uc1(frame, frame)
        except Exception:
            cp.close()
            raise
        return cp

    failed, leaked = _sweep(rf, torch_cuda, make, lambda cp: cp.close())
    assert failed >= 5
    assert abs(leaked) < (8 << 20), leaked


def _small_solve(rf):
    y, x = np.mgrid[0:48, 0:64].astype(np.float64)
    I0 = (0.5 + 0.2 * np.sin(0.3 * x + 0.2 * y)).astype(np.float32)
    I1 = np.roll(I0, 1, axis=1)
    f = rf.ReconFlow()
    f.initializeR(64, 48, 1, 2, 2.0, 14, 50.0, 0.0, 0.1, 100.0, 1 / 0.33, 60.0, 0.5, 0.25, 1, 5,
                  cvType=5, fix_quirks=1)
    K = np.array([[50.0, 0, 32], [0, 50.0, 24], [0, 0, 1]])
    f.setCameraMatrices(K, K)
    f.copyImagesToDevice(I0, I1)
    f.solveR(np.eye(3), np.array([0.1, 0.0, 0.0]), 5.0)
    u, v = f.copyOpticalFlowToHost()
    f.close()
    return u, v


def test_failed_create_then_normal_use(rf, torch_cuda):
    """After an injected failure the library works normally: a solve on a
    fresh handle gives bit for bit the results of the same solve before."""
    from reconflow_gb300 import _native as N

    lib = rf.load()
    before = _small_solve(rf)
    lib.rf_test_fail_alloc(1)
    try:
        with pytest.raises(N.RfError):
            rf.ReconFlowBatch([(64, 48)], 2, method=14, nWarpIters=1, nSolverIters=2)
    finally:
        lib.rf_test_fail_alloc(0)
    after = _small_solve(rf)
    for a, b in zip(before, after):
        assert a.tobytes() == b.tobytes()
