"""CPU checks of the C-ABI library: it loads, exports every entry point the
public header declares, and validates arguments before touching a device."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(hdr).read()
        names += re.findall(r"RF_API\s+[\w\s\*]+?\b(rfk?_\w+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("rf_create", "rf_destroy", "rf_set_cameras", "rf_upload_images", "rf_solve",
                 "rf_solve_flow", "rf_download_flow", "rf_download_points",
                 "rf_download_inv_depth", "rf_last_error_string"):
        assert must in names


def test_library_exports_every_declared_symbol(rf):
    lib = rf.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(rf):
    from reconflow_gb300 import _native

    assert sorted(_native.EXPORTED) == declared_symbols()


def test_params_defaults_match_reference(rf):
    from reconflow_gb300 import _native as N

    lib = rf.load()
    p = N.RfParams()
    assert lib.rf_params_default(ctypes.byref(p), 14) == 0
    # ReconFlow::initializeR defaults (Reconflow.cu:15-18)
    assert (p.lambda_, p.lambdagrad, p.lambdaf, p.lambdams) == (100.0, 400.0, 100.0, 100.0)
    assert (p.alpha_tv, p.alpha_proj, p.alpha_fn, p.tau) == (3.0, 1.0, 0.5, 0.25)
    assert (p.n_warp_iters, p.n_solver_iters, p.stride_alignment) == (1, 100, 32)
    assert lib.rf_params_default(ctypes.byref(p), 0) == 0
    # CudaFlow::initialize defaults (Cudaflow.cu:16-18)
    assert p.theta == pytest.approx(0.33) and p.lambda_ == 100.0


def _create(rf, **over):
    from reconflow_gb300 import _native as N

    lib = rf.load()
    p = N.RfParams()
    lib.rf_params_default(ctypes.byref(p), over.pop("method", 14))
    p.width, p.height, p.n_levels = 64, 48, 3
    for k, v in over.items():
        setattr(p, k, v)
    h = ctypes.c_void_p()
    st = lib.rf_create(ctypes.byref(p), ctypes.byref(h))
    if st == 0:
        lib.rf_destroy(h)
    return st, lib.rf_last_error_string().decode()


@pytest.mark.parametrize("over,status", [
    (dict(method=3), 2),          # METHOD_TVL1PATCH is not on the implemented path
    (dict(width=0), 1),
    (dict(n_levels=0), 1),
    (dict(n_levels=12), 1),       # 48 rows cannot make 12 levels
    (dict(scale=1.0), 1),
    (dict(input_type=9), 2),
    (dict(alpha_tv=0.0), 1),
])
def test_create_rejects_bad_params(rf, over, status):
    st, msg = _create(rf, **over)
    assert st == status, msg
    assert msg


def test_null_handle_calls_fail_cleanly(rf):
    lib = rf.load()
    assert lib.rf_solve(None, None, None, None, None) == 1
    assert lib.rf_download_flow(None, None, None, 0) == 1
    assert lib.rf_destroy(None) == 0
    assert "null" in lib.rf_last_error_string().decode()


def test_batch_null_handle_calls_fail_cleanly(rf):
    """The batch entry points (and the network's status read) check their
    handle before any CUDA call, so they fail with RF_ERR_INVALID_ARG (1)
    and a message on any host."""
    lib = rf.load()
    calls = [
        ("rf_batch_upload_all", (None, None, None, 0)),
        ("rf_batch_download_all", (None, None, None, None, None, None, None, 0)),
        ("rf_batch_stage_upload", (None, None, None, 0)),
        ("rf_batch_take_upload", (None,)),
        ("rf_batch_stage_download", (None, None, None, None, None, None, None, 0)),
        ("rf_batch_wait_download", (None,)),
        ("rf_batch_synchronize", (None,)),
        ("rf_batch_energies", (None, None)),
    ]
    calls.append(("rf_cnn_status", (None, None)))
    for name, args in calls:
        assert getattr(lib, name)(*args) == 1, name
        assert "null" in lib.rf_last_error_string().decode(), name
    assert lib.rf_batch_destroy(None) == 0


def test_class_surface_keeps_reference_member_names():
    """The Python classes carry the reference's public members on this path
    (Reconflow.h:67-83, Cudaflow.h:36-63), aliases included; calls before
    initialisation fail with the library's error, not an AttributeError."""
    import numpy as np

    import reconflow_gb300 as R
    from reconflow_gb300._native import RfError

    names = ["initialize", "copyImagesToDevice", "copyOpticalFlowToHost", "solveOpticalFlow",
             "initializeColorWheel", "copyToDevice", "copyToHost", "close", "initializeR",
             "setCameraMatrices", "copySparseOpticalFlowToDevice",
             "copyInitialOpticalFlowToDevice", "solveR", "solveReconFlow", "copy3dToHost",
             "removeEdgeArtifacts3D"]
    f = R.ReconFlow()
    for nm in names:
        assert callable(getattr(f, nm, None)), nm
    assert f.initializeColorWheel() == 0
    with pytest.raises(RfError):
        f.solveReconFlow(np.eye(3), np.zeros(3), 5.0)
    assert f.close() == 0
