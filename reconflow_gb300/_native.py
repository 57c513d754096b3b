"""ctypes binding of the C ABI (``include/reconflow_gb300.h``).

The CUDA library is built in-tree (``reconflow_gb300/lib/librfgb300.so``).  If
it is missing or cannot be loaded, every call raises: there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "librfgb300.so")
# RF_BOUNDS_CHECK=1 in the environment loads the bounds-checked debug build
CHECK_LIB_PATH = os.path.join(_HERE, "lib", "librfgb300_check.so")

RF_OK = 0
STATUS_NAMES = {0: "RF_OK", 1: "RF_ERR_INVALID_ARG", 2: "RF_ERR_UNSUPPORTED", 3: "RF_ERR_CUDA",
                4: "RF_ERR_OOM", 5: "RF_ERR_STATE", 6: "RF_ERR_NO_DEVICE"}

METHOD_TVL1 = 0
METHODR_TVL1_MS = 14
METHODR_TVL1_MS_FN = 17
METHODR_TVL1_MS_FNSPARSE = 20

INPUT_F32, INPUT_RGB8, INPUT_U8, INPUT_U16 = 0, 1, 2, 3
FIX_K_PYRAMID, FIX_XYZ_UPSCALE = 1, 2


class RfError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class RfParams(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int), ("channels", ctypes.c_int),
        ("input_type", ctypes.c_int), ("n_levels", ctypes.c_int), ("scale", ctypes.c_float),
        ("method", ctypes.c_int), ("lambda_", ctypes.c_float), ("lambdagrad", ctypes.c_float),
        ("lambdaf", ctypes.c_float), ("lambdams", ctypes.c_float), ("alpha_tv", ctypes.c_float),
        ("alpha_proj", ctypes.c_float), ("alpha_fn", ctypes.c_float), ("tau", ctypes.c_float),
        ("theta", ctypes.c_float), ("n_warp_iters", ctypes.c_int), ("n_solver_iters", ctypes.c_int),
        ("stride_alignment", ctypes.c_int), ("block_width", ctypes.c_int),
        ("block_height", ctypes.c_int), ("fix_quirks", ctypes.c_int),
    ]


class RfPoseParams(ctypes.Structure):
    _fields_ = [
        ("hessian_threshold", ctypes.c_double), ("n_octaves", ctypes.c_int),
        ("n_octave_layers", ctypes.c_int), ("max_keypoints", ctypes.c_int),
        ("ratio", ctypes.c_double), ("confidence", ctypes.c_double), ("seed", ctypes.c_ulonglong),
        ("refine", ctypes.c_int),
    ]


class RfKeypoint(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("scale", ctypes.c_float),
                ("angle", ctypes.c_float), ("response", ctypes.c_float), ("octave", ctypes.c_int)]


# (name, restype, argtypes) of every exported entry point
_VP, _I, _F, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_void_p
_SIGS = [
    ("rf_params_default", _I, [ctypes.POINTER(RfParams), _I]),
    ("rf_create", _I, [ctypes.POINTER(RfParams), ctypes.POINTER(_VP)]),
    ("rf_destroy", _I, [_VP]),
    ("rf_stride", _I, [_VP]),
    ("rf_pyramid_dims", _I, [_VP, _VP, _VP, _VP]),
    ("rf_set_cameras", _I, [_VP, _D, _D]),
    ("rf_upload_images", _I, [_VP, _VP, _VP, _I]),
    ("rf_upload_images_device", _I, [_VP, _VP, _VP, _I]),
    ("rf_set_prior_flow", _I, [_VP, _VP, _VP, _VP, _I]),
    ("rf_solve", _I, [_VP, _D, _D, _D, _D]),
    ("rf_solve_flow", _I, [_VP]),
    ("rf_solve_warm", _I, [_VP, _D, _D, _D, _D, _I, _VP, _VP, _VP, _VP, _VP, _I, _I, _I, _I]),
    ("rf_solve_flow_warm", _I, [_VP, _I, _VP, _VP, _I, _I, _I, _I]),
    ("rf_energy", _I, [_VP, ctypes.POINTER(ctypes.c_double)]),
    ("rf_download_flow", _I, [_VP, _VP, _VP, _I]),
    ("rf_download_points", _I, [_VP, _VP, _VP, _VP, _I]),
    ("rf_download_inv_depth", _I, [_VP, _VP, _I]),
    ("rf_download_flow_color", _I, [_VP, _F, _VP, _I]),
    ("rf_remove_edge_artifacts", _I, [_VP, _I, _F]),
    ("rf_device_results", _I, [_VP, _VP, _VP, _VP, _VP, _VP]),
    ("rf_debug_bounds", _I, [ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_longlong)]),
    ("rf_debug_bounds_selftest", _I, []),
    ("rf_set_cluster_pixels", _I, [ctypes.c_longlong]),
    ("rf_set_tiles", _I, [_VP, _VP, _VP]),
    ("rf_set_stream", _I, [_VP, _VP]),
    ("rf_synchronize", _I, [_VP]),
    ("rf_host_alloc", _I, [ctypes.c_size_t, ctypes.POINTER(_VP)]),
    ("rf_host_free", _I, [_VP]),
    ("rf_profile_iterations", _I, [_VP, _I, _I, _VP]),
    ("rf_kernel_launches", ctypes.c_uint64, [_VP]),
    ("rf_last_error_string", ctypes.c_char_p, []),
    ("rf_version", ctypes.c_char_p, []),
    ("rf_batch_create", _I, [ctypes.POINTER(RfParams), _I, _VP, _VP, ctypes.POINTER(_VP)]),
    ("rf_batch_destroy", _I, [_VP]),
    ("rf_batch_stride", _I, [_VP, _I]),
    ("rf_batch_set_cameras", _I, [_VP, _I, _D, _D]),
    ("rf_batch_upload_images", _I, [_VP, _I, _VP, _VP, _I]),
    ("rf_batch_upload_images_device", _I, [_VP, _I, _VP, _VP, _I]),
    ("rf_batch_solve", _I, [_VP, _D, _D, _D, _D]),
    ("rf_batch_solve_flow", _I, [_VP]),
    ("rf_batch_solve_warm", _I, [_VP, _D, _D, _D, _D, _I, _I, _I]),
    ("rf_batch_energies", _I, [_VP, _VP]),
    ("rf_batch_energies_async", _I, [_VP, _VP]),
    ("rf_batch_solve_warm_levels", _I, [_VP, _D, _D, _D, _D, _I, _VP, _VP]),
    ("rf_batch_warm_planes", _I, [_VP, _I, _VP, _VP, _VP, _VP, _VP]),
    ("rf_batch_image_planes", _I, [_VP, _I, _I, _VP, _VP]),
    ("rf_batch_set_tiles", _I, [_VP, _VP, _VP]),
    ("rf_batch_profile_level", _I, [_VP, _I, _I, _VP]),
    ("rf_batch_download_flow", _I, [_VP, _I, _VP, _VP, _I]),
    ("rf_batch_download_points", _I, [_VP, _I, _VP, _VP, _VP, _I]),
    ("rf_batch_download_inv_depth", _I, [_VP, _I, _VP, _I]),
    ("rf_batch_upload_all", _I, [_VP, _VP, _VP, _I]),
    ("rf_batch_download_all", _I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _I]),
    ("rf_batch_stage_upload", _I, [_VP, _VP, _VP, _I]),
    ("rf_batch_take_upload", _I, [_VP]),
    ("rf_batch_stage_download", _I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _I]),
    ("rf_batch_wait_download", _I, [_VP]),
    ("rf_batch_device_results", _I, [_VP, _I, _VP, _VP, _VP, _VP, _VP]),
    ("rf_batch_import_results", _I, [_VP, _I, _VP, _VP, _VP, _VP, _VP, _I]),
    ("rf_batch_set_stream", _I, [_VP, _VP]),
    ("rf_batch_get_stream", _I, [_VP, ctypes.POINTER(ctypes.c_void_p)]),
    ("rf_batch_synchronize", _I, [_VP]),
    ("rf_batch_kernel_launches", ctypes.c_uint64, [_VP]),
    ("rf_cnn_create", _I, [_I, _I, _I, ctypes.c_ulonglong, ctypes.POINTER(_VP)]),
    ("rf_cnn_destroy", _I, [_VP]),
    ("rf_cnn_num_params", _I, [_VP]),
    ("rf_cnn_set_stream", _I, [_VP, _VP]),
    ("rf_cnn_get_params", _I, [_VP, _VP]),
    ("rf_cnn_set_params", _I, [_VP, _VP]),
    ("rf_cnn_get_grads", _I, [_VP, _VP]),
    ("rf_cnn_forward", _I, [_VP, _VP, _I, _I, _I, _VP, _VP]),
    ("rf_cnn_backward", _I, [_VP, _VP, _VP, _VP, _VP, _VP, _I, _I, _I, _VP,
                             ctypes.POINTER(ctypes.c_double)]),
    ("rf_cnn_adam_step", _I, [_VP, _F, _F, _F, _F]),
    ("rf_cnn_kernel_launches", ctypes.c_uint64, [_VP]),
    ("rf_cnn_status", _I, [_VP, ctypes.POINTER(ctypes.c_int)]),
    ("rf_cnn_set_test_wait_limit", _I, [_VP, ctypes.c_int]),
    ("rf_ws_features", _I, [_I, _VP, _VP, _I, _I, _I, _I, _D, _D, _D, _VP, _VP]),
    ("rf_ws_state", _I, [_I, _VP, _I, _I, _I, _I, _I, _I, _F, _D, _D, _D, _VP, _VP, _VP, _VP,
                         _VP, _VP]),
    ("rf_test_fail_alloc", None, [ctypes.c_longlong]),
    ("rf_ws_propagate", _I, [_I, _VP, _I, _I, _I, _D, _D, _D, _I, _I, _I, _I, _I, _VP, _VP,
                             _VP]),
    ("rfk_downscale", _I, [_VP, _I, _I, _I, _I, _I, _I, _F, _I, _VP, _VP]),
    ("rfk_upscale", _I, [_VP, _I, _I, _I, _I, _I, _I, _F, _VP, _VP]),
    ("rfk_warp", _I, [_VP, _I, _I, _I, _VP, _VP, _VP, _VP]),
    ("rfk_derivatives", _I, [_VP, _VP, _I, _I, _I, _VP, _VP, _VP, _VP]),
    ("rfk_warp_derivatives", _I, [_VP, _VP, _VP, _VP, _I, _I, _I, _VP, _VP, _VP, _VP]),
    ("rfk_median5", _I, [_VP, _VP, _I, _I, _I, _VP, _VP, _VP]),
    ("rfk_median3d", _I, [_VP, _VP, _VP, _I, _I, _I, _VP, _VP, _VP, _VP]),
    ("rfk_warp_update", _I, [_VP, _VP, _VP, _VP, _I, _I, _I, _VP, _VP, _VP, _VP, _VP]),
    ("rfk_warp_update_noalloc", _I, [_VP, _VP, _VP, _VP, _I, _I, _I, _VP, _VP, _VP]),
    ("rfk_rgb_to_gray", _I, [_VP, _I, _I, _I, _VP, _VP]),
    ("rfk_remove_edge_artifacts", _I, [_VP, _VP, _VP, _I, _F, _I, _I, _I, _VP, _VP, _VP, _VP]),
    ("rfk_flow_to_color", _I, [_VP, _VP, _I, _I, _I, _F, _VP, _VP]),
    # pose front end
    ("rf_pose_params_default", _I, [ctypes.POINTER(RfPoseParams)]),
    ("rf_pose_create", _I, [ctypes.POINTER(RfPoseParams), _I, _I, ctypes.POINTER(_VP)]),
    ("rf_pose_destroy", _I, [_VP]),
    ("rf_pose_set_stream", _I, [_VP, _VP]),
    ("rf_pose_solve_u8", _I, [_VP, _VP, _VP, _I, _VP, _VP, _VP]),
    ("rf_pose_solve_f32", _I, [_VP, _VP, _VP, _I, _VP, _VP, _VP]),
    ("rf_pose_counts", _I, [_VP, _VP, _VP, _VP, _VP]),
    ("rf_pose_keypoints", _I, [_VP, _I, _VP, _VP, _I]),
    ("rf_pose_matches", _I, [_VP, _VP, _VP, _VP, _VP, _I]),
    ("rf_pose_responses", _I, [_VP, _I, _I, _VP, ctypes.c_size_t]),
    ("rf_pose_kernel_launches", ctypes.c_uint64, [_VP]),
    ("rf_pose_profile", _I, [_VP, _VP, _VP, _I, _VP, _I, _VP]),
    ("rf_essential_5pt", _I, [_VP, _VP, _VP]),
    ("rf_essential_lmeds", _I, [_VP, _VP, _I, ctypes.c_double, ctypes.c_ulonglong, _VP, _VP]),
    ("rf_recover_pose", _I, [_VP, _VP, _VP, _I, _VP, _VP, _VP, _VP]),
    ("rf_refine_pose", _I, [_VP, _VP, _I, _VP, _VP, _VP]),
]

EXPORTED = [s[0] for s in _SIGS]

_lib = None


def load(path: str | None = None):
    """Load the CUDA library (building it first if absent); raises if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    checked = path is None and os.environ.get("RF_BOUNDS_CHECK", "0") not in ("", "0")
    path = path or (CHECK_LIB_PATH if checked else LIB_PATH)
    if not os.path.exists(path):
        from . import build as _build

        _build.build(bounds_check=checked)
    lib = ctypes.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != RF_OK:
        msg = load().rf_last_error_string().decode(errors="replace")
        raise RfError(status, msg)
