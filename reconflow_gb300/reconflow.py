"""Python mirror of the reference's ``CudaFlow`` / ``ReconFlow`` classes.

Same method names, argument meaning and call order as
``reconflow/Cudaflow.h:17-362`` and ``reconflow/Reconflow.h:9-160``
(``test_reconflow/main.cpp:24-106`` shows the order): construct, initialize,
set cameras, copy images (and prior flow) to the device, solve, copy results
to the host.  Host images are numpy arrays of shape (height, pitch[, 3]); a
result is written into a caller's array when one is passed (the reference's
pre-allocated ``cv::Mat``) or returned as a new (height, stride) array.

Every call goes through the C ABI of the CUDA library; a failure raises
``RfError`` (the reference aborts the process inside ``checkCudaErrors``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from ._native import RfError

__all__ = ["CudaFlow", "ReconFlow", "ReconFlowBatch", "RfError"]

# OpenCV type codes accepted by initialize(cvType=...) (Cudaflow.cu:288-311)
CV_8U, CV_16U, CV_32F, CV_8UC3 = 0, 2, 5, 16
_CV_TO_INPUT = {CV_8UC3: N.INPUT_RGB8, CV_8U: N.INPUT_U8, CV_16U: N.INPUT_U16, CV_32F: N.INPUT_F32}
_INPUT_DTYPE = {N.INPUT_F32: np.float32, N.INPUT_RGB8: np.uint8, N.INPUT_U8: np.uint8,
                N.INPUT_U16: np.uint16}


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _dbl(a, n):
    a = np.ascontiguousarray(np.asarray(a, np.float64).reshape(n))
    return a, _ptr(a)


class CudaFlow:
    """Plain TV-L1 optical flow (Cudaflow.h:17-362)."""

    METHOD_TVL1 = N.METHOD_TVL1

    def __init__(self, BlockWidth: int = 32, BlockHeight: int = 12, StrideAlignment: int = 32):
        self._lib = N.load()
        self.BlockWidth, self.BlockHeight, self.StrideAlignment = BlockWidth, BlockHeight, StrideAlignment
        self._h = None
        self.params = None

    # -- lifecycle ---------------------------------------------------------
    def _create(self, params: N.RfParams) -> int:
        self.close()
        h = ctypes.c_void_p()
        N.check(self._lib.rf_create(ctypes.byref(params), ctypes.byref(h)))
        self._h = h
        self.params = params
        self.width, self.height = params.width, params.height
        self.stride = self._lib.rf_stride(h)
        self.nLevels = params.n_levels
        return 0

    def close(self) -> int:
        if self._h is not None:
            self._lib.rf_destroy(self._h)
            self._h = None
        return 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _handle(self):
        if self._h is None:
            raise RfError(5, "not initialized")
        return self._h

    def iAlignUp(self, n: int) -> int:
        m = self.StrideAlignment
        return n + m - n % m if n % m else n

    def pyramid(self):
        """(pW, pH, pS) level sizes (Cudaflow.cu:146-171)."""
        L = self.nLevels
        W, H, S = (ctypes.c_int * L)(), (ctypes.c_int * L)(), (ctypes.c_int * L)()
        N.check(self._lib.rf_pyramid_dims(self._handle(), W, H, S))
        return list(W), list(H), list(S)

    def initialize(self, width, height, channels, cvType=CV_8UC3, nLevels=1, scale=2.0,
                   method=METHOD_TVL1, lambda_=100.0, lambdagrad=400.0, theta=0.33, tau=0.25,
                   nWarpIters=1, nSolverIters=100, withVisualization=True):
        """CudaFlow::initialize (Cudaflow.cu:99-269)."""
        if cvType not in _CV_TO_INPUT:
            raise RfError(2, f"unsupported cvType {cvType}")
        p = N.RfParams()
        N.check(self._lib.rf_params_default(ctypes.byref(p), int(method)))
        p.width, p.height, p.channels = int(width), int(height), int(channels)
        p.input_type = _CV_TO_INPUT[cvType]
        p.n_levels, p.scale, p.method = int(nLevels), float(scale), int(method)
        p.lambda_, p.lambdagrad, p.theta, p.tau = lambda_, lambdagrad, theta, tau
        p.n_warp_iters, p.n_solver_iters = int(nWarpIters), int(nSolverIters)
        p.stride_alignment = self.StrideAlignment
        p.block_width, p.block_height = self.BlockWidth, self.BlockHeight
        self.withVisualization = withVisualization
        return self._create(p)

    # -- copies ------------------------------------------------------------
    def _input(self, img):
        dt = _INPUT_DTYPE[self.params.input_type]
        a = np.ascontiguousarray(img, dtype=dt)
        if a.shape[0] != self.height or a.shape[1] < self.width:
            raise RfError(1, f"image shape {a.shape} does not match {self.height}x{self.width}")
        return a

    def copyImagesToDevice(self, i0, i1) -> int:
        """CudaFlow::copyImagesToDevice (Cudaflow.cu:288-311)."""
        a, b = self._input(i0), self._input(i1)
        N.check(self._lib.rf_upload_images(self._handle(), _ptr(a), _ptr(b), a.shape[1]))
        return 0

    def copyImagesToDeviceFromDevice(self, ptr0: int, ptr1: int, pitch: int) -> int:
        """Images already in device memory (e.g. torch tensors' data_ptr())."""
        N.check(self._lib.rf_upload_images_device(self._handle(), ctypes.c_void_p(ptr0),
                                                  ctypes.c_void_p(ptr1), int(pitch)))
        return 0

    def _out(self, out, ch=1):
        shape = (self.height, self.stride) if ch == 1 else (self.height, self.stride, ch)
        if out is None:
            return np.zeros(shape, np.float32)
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.shape[0] != self.height:
            raise RfError(1, "output must be a C-contiguous float32 array of `height` rows")
        return out

    def copyOpticalFlowToHost(self, u=None, v=None, uvrgb=None):
        """CudaFlow::copyOpticalFlowToHost (Cudaflow.cu:313-325); returns (u, v[, uvrgb])."""
        u, v = self._out(u), self._out(v)
        N.check(self._lib.rf_download_flow(self._handle(), _ptr(u), _ptr(v), u.shape[1]))
        if uvrgb is not None:
            N.check(self._lib.rf_download_flow_color(self._handle(), ctypes.c_float(self.flowScale),
                                                     _ptr(uvrgb), uvrgb.shape[1]))
            return u, v, uvrgb
        return u, v

    def copyFlowColorToHost(self, flowScale: float = 5.0, uvrgb=None):
        uvrgb = self._out(uvrgb, 3)
        N.check(self._lib.rf_download_flow_color(self._handle(), ctypes.c_float(flowScale),
                                                 _ptr(uvrgb), uvrgb.shape[1]))
        return uvrgb

    def initializeColorWheel(self) -> int:
        """CudaFlow::initializeColorWheel (Cudaflow.h:47): the colour wheel
        is a constant table of the colour kernel, nothing to set up."""
        return 0

    # the reference's older names (Cudaflow.h:52-53)
    def copyToDevice(self, i0, i1) -> int:
        return self.copyImagesToDevice(i0, i1)

    def copyToHost(self, u=None, v=None, uvrgb=None):
        if uvrgb is None:
            uvrgb = self._out(None, 3)
        return self.copyOpticalFlowToHost(u, v, uvrgb)

    # -- solve -------------------------------------------------------------
    def solveOpticalFlow(self, flowScale: float = 5.0) -> int:
        """CudaFlow::solveOpticalFlow (Cudaflow.cu:394-621)."""
        self.flowScale = flowScale
        N.check(self._lib.rf_solve_flow(self._handle()))
        return 0

    def synchronize(self) -> int:
        N.check(self._lib.rf_synchronize(self._handle()))
        return 0

    def energy(self) -> float:
        """Energy of the last solution (rf_energy)."""
        e = ctypes.c_double()
        N.check(self._lib.rf_energy(self._handle(), ctypes.byref(e)))
        return float(e.value)

    def solveOpticalFlowWarm(self, level, u, v, nWarpIters=-1, nSolverIters=-1) -> int:
        """Plain TV-L1 started at pyramid `level` from flow (u, v) on that level."""
        a = np.ascontiguousarray(u, np.float32)
        b = np.ascontiguousarray(v, np.float32)
        N.check(self._lib.rf_solve_flow_warm(self._handle(), int(level), _ptr(a), _ptr(b),
                                             a.shape[1], 0, int(nWarpIters), int(nSolverIters)))
        return 0

    def kernelLaunches(self) -> int:
        return int(self._lib.rf_kernel_launches(self._handle()))

    def deviceResults(self):
        """Device pointers (u, v, X, Y, Z) of the last solve (0 when absent)."""
        ptrs = [ctypes.c_void_p() for _ in range(5)]
        N.check(self._lib.rf_device_results(self._handle(), *[ctypes.byref(p) for p in ptrs]))
        return [p.value or 0 for p in ptrs]

    def setTiles(self, tile_w, tile_h) -> int:
        """Tile shape of the inner-iteration kernels per pyramid level
        (rf_set_tiles); results do not depend on it."""
        n = len(tile_w)
        N.check(self._lib.rf_set_tiles(self._handle(), (ctypes.c_int * n)(*map(int, tile_w)),
                                       (ctypes.c_int * n)(*map(int, tile_h))))
        return 0

    def profileLevel(self, level, nIters=20):
        """Mean ms per launch of the two inner-iteration kernels at `level`
        (rf_profile_iterations); needs a prior solve and invalidates it."""
        ms = (ctypes.c_float * 2)()
        N.check(self._lib.rf_profile_iterations(self._handle(), int(level), int(nIters), ms))
        return float(ms[0]), float(ms[1])

    def setStream(self, stream_ptr: int | None) -> int:
        N.check(self._lib.rf_set_stream(self._handle(), ctypes.c_void_p(stream_ptr or 0)))
        return 0


class ReconFlow(CudaFlow):
    """Simultaneous flow + 3D reconstruction (Reconflow.h:9-160)."""

    METHODR_TVL1_MS = N.METHODR_TVL1_MS
    METHODR_TVL1_MS_FN = N.METHODR_TVL1_MS_FN
    METHODR_TVL1_MS_FNSPARSE = N.METHODR_TVL1_MS_FNSPARSE

    def initializeR(self, width, height, channels, nLevels, scale, method, lambda_=100.0,
                    lambdagrad=400.0, lambdaf=100.0, lambdams=100.0, alphaTv=3.0, alphaProj=1.0,
                    alphaFn=0.5, tau=0.25, nWarpIters=1, nSolverIters=100, cvType=None,
                    fix_quirks=0):
        """ReconFlow::initializeR (Reconflow.cu:15-63).  The reference forces
        CV_8UC3 input (Cudaflow.cu:16-25); cvType=CV_32F selects float gray."""
        p = N.RfParams()
        N.check(self._lib.rf_params_default(ctypes.byref(p), int(method)))
        cvType = CV_8UC3 if cvType is None else cvType
        if cvType not in _CV_TO_INPUT:
            raise RfError(2, f"unsupported cvType {cvType}")
        p.width, p.height, p.channels = int(width), int(height), int(channels)
        p.input_type = _CV_TO_INPUT[cvType]
        p.n_levels, p.scale, p.method = int(nLevels), float(scale), int(method)
        p.lambda_, p.lambdagrad, p.lambdaf, p.lambdams = lambda_, lambdagrad, lambdaf, lambdams
        p.alpha_tv, p.alpha_proj, p.alpha_fn, p.tau = alphaTv, alphaProj, alphaFn, tau
        p.theta = 1.0 / alphaTv
        p.n_warp_iters, p.n_solver_iters = int(nWarpIters), int(nSolverIters)
        p.stride_alignment = self.StrideAlignment
        p.block_width, p.block_height = self.BlockWidth, self.BlockHeight
        p.fix_quirks = int(fix_quirks)
        return self._create(p)

    def setCameraMatrices(self, intrinsic0, intrinsic1=None) -> int:
        """ReconFlow::setCameraMatrices (Reconflow.cu:78-116)."""
        intrinsic1 = intrinsic0 if intrinsic1 is None else intrinsic1
        k0, p0 = _dbl(intrinsic0, 9)
        k1, p1 = _dbl(intrinsic1, 9)
        N.check(self._lib.rf_set_cameras(self._handle(), p0, p1))
        return 0

    def copySparseOpticalFlowToDevice(self, u, v, mask=None) -> int:
        """CudaFlow::copySparseOpticalFlowToDevice (Cudaflow.cu:327-343)."""
        u = np.ascontiguousarray(u, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        m = None if mask is None else np.ascontiguousarray(mask, np.float32)
        N.check(self._lib.rf_set_prior_flow(self._handle(), _ptr(u), _ptr(v),
                                            None if m is None else _ptr(m), u.shape[1]))
        return 0

    copyInitialOpticalFlowToDevice = copySparseOpticalFlowToDevice

    def solveR(self, *args) -> int:
        """solveR(R1, t1, flowScale) or solveR(R0, t0, R1, t1, flowScale)
        (Reconflow.cu:130-144)."""
        if len(args) in (2, 3):
            R0 = t0 = None
            R1, t1 = args[0], args[1]
            fs = args[2] if len(args) == 3 else 5.0
        elif len(args) in (4, 5):
            R0, t0, R1, t1 = args[:4]
            fs = args[4] if len(args) == 5 else 5.0
        else:
            raise RfError(1, "solveR(R1, t1[, flowScale]) or solveR(R0, t0, R1, t1[, flowScale])")
        self.flowScale = fs
        keep = []
        ptrs = []
        for a, n in ((R0, 9), (t0, 3), (R1, 9), (t1, 3)):
            if a is None:
                ptrs.append(None)
            else:
                arr, p = _dbl(a, n)
                keep.append(arr)
                ptrs.append(p)
        N.check(self._lib.rf_solve(self._handle(), *ptrs))
        return 0

    solveReconFlow = solveR

    def solveWarm(self, level, u, v, X, Y, Z, R1, t1, nWarpIters=-1, nSolverIters=-1, R0=None,
                  t0=None, on_device=False) -> int:
        """ReconFlow started at pyramid `level` from flow and 3D points given on
        that level (host arrays of shape (h_level, pitch), or device pointers
        with on_device=True and an explicit pitch via arrays' shape)."""
        planes = [np.ascontiguousarray(a, np.float32) for a in (u, v, X, Y, Z)]
        keep = []
        pose = []
        for a, n in ((R0, 9), (t0, 3), (R1, 9), (t1, 3)):
            if a is None:
                pose.append(None)
            else:
                arr, p_ = _dbl(a, n)
                keep.append(arr)
                pose.append(p_)
        N.check(self._lib.rf_solve_warm(self._handle(), *pose, int(level),
                                        *[_ptr(a) for a in planes], planes[0].shape[1], 0,
                                        int(nWarpIters), int(nSolverIters)))
        return 0

    def copy3dToHost(self, X=None, Y=None, Z=None):
        """ReconFlow::copy3dToHost (Reconflow.cu:65-70); returns (X, Y, Z)."""
        X, Y, Z = self._out(X), self._out(Y), self._out(Z)
        N.check(self._lib.rf_download_points(self._handle(), _ptr(X), _ptr(Y), _ptr(Z), X.shape[1]))
        return X, Y, Z

    def copyInverseDepthToHost(self, out=None):
        out = self._out(out)
        N.check(self._lib.rf_download_inv_depth(self._handle(), _ptr(out), out.shape[1]))
        return out

    def removeEdgeArtifacts3D(self, surfaceWidth: int, maxSurfaceArea: float) -> int:
        """ReconFlow::removeEdgeArtifacts3D (Reconflow.cu:468-477)."""
        N.check(self._lib.rf_remove_edge_artifacts(self._handle(), int(surfaceWidth),
                                                   ctypes.c_float(maxSurfaceArea)))
        return 0


class ReconFlowBatch:
    """Many frame pairs solved together (rf_batch_* C ABI): one launch per
    schedule step covers every pair.  Pairs may differ in size, cameras and
    pose; they share the solver parameters.  Float32 gray input; methods
    METHODR_TVL1_MS (14) and METHOD_TVL1 (0)."""

    def __init__(self, sizes, nLevels, scale=2.0, method=N.METHODR_TVL1_MS, lambda_=100.0,
                 lambdaf=100.0, lambdams=100.0, alphaTv=3.0, alphaProj=1.0, tau=0.25,
                 theta=0.33, nWarpIters=1, nSolverIters=100, fix_quirks=0, StrideAlignment=32):
        self._lib = N.load()
        p = N.RfParams()
        N.check(self._lib.rf_params_default(ctypes.byref(p), int(method)))
        p.width, p.height = sizes[0]
        p.input_type = N.INPUT_F32
        p.n_levels, p.scale, p.method = int(nLevels), float(scale), int(method)
        p.lambda_, p.lambdaf, p.lambdams = lambda_, lambdaf, lambdams
        p.alpha_tv, p.alpha_proj, p.tau = alphaTv, alphaProj, tau
        p.theta = theta if method == N.METHOD_TVL1 else 1.0 / alphaTv
        p.n_warp_iters, p.n_solver_iters = int(nWarpIters), int(nSolverIters)
        p.stride_alignment, p.fix_quirks = StrideAlignment, int(fix_quirks)
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        n = len(self.sizes)
        ws = (ctypes.c_int * n)(*[w for w, _ in self.sizes])
        hs = (ctypes.c_int * n)(*[h for _, h in self.sizes])
        self._h = None
        h = ctypes.c_void_p()
        N.check(self._lib.rf_batch_create(ctypes.byref(p), n, ws, hs, ctypes.byref(h)))
        self._h = h
        self.n = n
        self.params = p
        self.strides = [self._lib.rf_batch_stride(h, i) for i in range(n)]

    def close(self):
        if self._h is not None:
            self._lib.rf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setCameraMatrices(self, pair, K0, K1=None):
        K1 = K0 if K1 is None else K1
        a, pa = _dbl(K0, 9)
        b, pb = _dbl(K1, 9)
        N.check(self._lib.rf_batch_set_cameras(self._h, int(pair), pa, pb))

    def copyImagesToDevice(self, pair, i0, i1):
        a = np.ascontiguousarray(i0, np.float32)
        b = np.ascontiguousarray(i1, np.float32)
        N.check(self._lib.rf_batch_upload_images(self._h, int(pair), _ptr(a), _ptr(b), a.shape[1]))

    def solveR(self, R1s, t1s, R0s=None, t0s=None):
        R1 = np.ascontiguousarray(np.asarray(R1s, np.float64).reshape(self.n, 9))
        t1 = np.ascontiguousarray(np.asarray(t1s, np.float64).reshape(self.n, 3))
        R0 = None if R0s is None else np.ascontiguousarray(np.asarray(R0s, np.float64).reshape(self.n, 9))
        t0 = None if t0s is None else np.ascontiguousarray(np.asarray(t0s, np.float64).reshape(self.n, 3))
        N.check(self._lib.rf_batch_solve(self._h, None if R0 is None else _ptr(R0),
                                         None if t0 is None else _ptr(t0), _ptr(R1), _ptr(t1)))

    def solveOpticalFlow(self):
        N.check(self._lib.rf_batch_solve_flow(self._h))

    def _poses(self, R1s, t1s, R0s, t0s):
        R1 = np.ascontiguousarray(np.asarray(R1s, np.float64).reshape(self.n, 9))
        t1 = np.ascontiguousarray(np.asarray(t1s, np.float64).reshape(self.n, 3))
        R0 = None if R0s is None else np.ascontiguousarray(np.asarray(R0s, np.float64).reshape(self.n, 9))
        t0 = None if t0s is None else np.ascontiguousarray(np.asarray(t0s, np.float64).reshape(self.n, 3))
        return R0, t0, R1, t1

    def solveWarm(self, level, R1s, t1s, nWarpIters, nSolverIters, R0s=None, t0s=None):
        """Warm-started solve (rf_batch_solve_warm_levels): every pair starts at
        `level` from the planes of warmPlanes(pair).  nWarpIters and
        nSolverIters are ints (every level) or sequences indexed by level
        (0 = finest, level + 1 entries)."""
        R0, t0, R1, t1 = self._poses(R1s, t1s, R0s, t0s)
        n = int(level) + 1
        w = [int(nWarpIters)] * n if np.isscalar(nWarpIters) else [int(x) for x in nWarpIters]
        it = [int(nSolverIters)] * n if np.isscalar(nSolverIters) else [int(x) for x in nSolverIters]
        if len(w) != n or len(it) != n:
            raise ValueError("per-level schedules need level + 1 entries")
        wa, ia = (ctypes.c_int * n)(*w), (ctypes.c_int * n)(*it)
        N.check(self._lib.rf_batch_solve_warm_levels(self._h, None if R0 is None else _ptr(R0),
                                                     None if t0 is None else _ptr(t0), _ptr(R1),
                                                     _ptr(t1), int(level), wa, ia))

    def uploadAll(self, ptrs0, ptrs1, pitch):
        """rf_batch_upload_all: every pair's frames from host pointers."""
        a = (ctypes.c_void_p * self.n)(*[ctypes.c_void_p(int(p)) for p in ptrs0])
        b = (ctypes.c_void_p * self.n)(*[ctypes.c_void_p(int(p)) for p in ptrs1])
        N.check(self._lib.rf_batch_upload_all(self._h, a, b, int(pitch)))

    def downloadAll(self, pitch, u=None, v=None, inv_depth=None, X=None, Y=None, Z=None):
        """rf_batch_download_all: each argument a list of n host pointers (or
        None to skip that output); blocking."""
        def arr(lst):
            if lst is None:
                return None
            return (ctypes.c_void_p * self.n)(*[ctypes.c_void_p(int(p)) for p in lst])
        N.check(self._lib.rf_batch_download_all(self._h, arr(u), arr(v), arr(inv_depth), arr(X),
                                                arr(Y), arr(Z), int(pitch)))

    def stageUpload(self, ptrs0, ptrs1, pitch):
        """rf_batch_stage_upload: queue every pair's frames (host pointers,
        unchanged until the solve that uses them has finished) on the upload
        copy stream; returns at once."""
        a = (ctypes.c_void_p * self.n)(*[ctypes.c_void_p(int(p)) for p in ptrs0])
        b = (ctypes.c_void_p * self.n)(*[ctypes.c_void_p(int(p)) for p in ptrs1])
        N.check(self._lib.rf_batch_stage_upload(self._h, a, b, int(pitch)))

    def takeUpload(self):
        """rf_batch_take_upload: the staged frames become the pairs' frames
        for the next solve (ordered on the batch's stream)."""
        N.check(self._lib.rf_batch_take_upload(self._h))

    def stageDownload(self, pitch, u=None, v=None, inv_depth=None, X=None, Y=None, Z=None):
        """rf_batch_stage_download: like downloadAll, but returns at once;
        the host arrays are complete after waitDownload()."""
        def arr(lst):
            if lst is None:
                return None
            return (ctypes.c_void_p * self.n)(*[ctypes.c_void_p(int(p)) for p in lst])
        N.check(self._lib.rf_batch_stage_download(self._h, arr(u), arr(v), arr(inv_depth),
                                                  arr(X), arr(Y), arr(Z), int(pitch)))

    def waitDownload(self):
        """rf_batch_wait_download: block until the last staged download
        has reached the host."""
        N.check(self._lib.rf_batch_wait_download(self._h))

    def energies(self):
        """Energy of every pair's last solution (rf_batch_energies)."""
        out = np.zeros(self.n, np.float64)
        N.check(self._lib.rf_batch_energies(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def energiesAsync(self, out_ptr: int):
        """rf_batch_energies_async: queue the evaluation; the n doubles at
        out_ptr (pinned host memory) are valid once the batch's stream has
        reached them."""
        N.check(self._lib.rf_batch_energies_async(self._h, ctypes.c_void_p(int(out_ptr))))

    def warmPlanes(self, pair):
        """Device pointers (u, v, X, Y, Z) of pair's warm-start input planes."""
        ps = [ctypes.c_void_p() for _ in range(5)]
        N.check(self._lib.rf_batch_warm_planes(self._h, int(pair), *[ctypes.byref(p) for p in ps]))
        return [p.value for p in ps]

    def imagePlanes(self, pair, level=0):
        a, b = ctypes.c_void_p(), ctypes.c_void_p()
        N.check(self._lib.rf_batch_image_planes(self._h, int(pair), int(level), ctypes.byref(a),
                                                ctypes.byref(b)))
        return a.value, b.value

    def copyImagesToDeviceFromDevice(self, pair, ptr0, ptr1, pitch):
        N.check(self._lib.rf_batch_upload_images_device(self._h, int(pair), ctypes.c_void_p(ptr0),
                                                        ctypes.c_void_p(ptr1), int(pitch)))

    def setTiles(self, tile_w, tile_h):
        """Tile shape per pyramid level (rf_batch_set_tiles)."""
        n = int(self.params.n_levels)
        if len(tile_w) != n or len(tile_h) != n:
            raise ValueError("one tile shape per level")
        N.check(self._lib.rf_batch_set_tiles(self._h, (ctypes.c_int * n)(*map(int, tile_w)),
                                             (ctypes.c_int * n)(*map(int, tile_h))))

    def profileLevel(self, level, nIters=20):
        """Mean ms per launch of the two inner-iteration kernels at `level`
        (rf_batch_profile_level); needs a prior solve and invalidates it."""
        ms = (ctypes.c_float * 2)()
        N.check(self._lib.rf_batch_profile_level(self._h, int(level), int(nIters), ms))
        return float(ms[0]), float(ms[1])

    def levelDims(self, pair, level):
        """(w, h, stride) of pair's pyramid level (Cudaflow.cu:146-171 rule)."""
        w, h = self.sizes[pair]
        s = self.strides[pair]
        sc = float(self.params.scale)
        al = int(self.params.stride_alignment)
        for _ in range(level):
            h = int(float(h) / sc)
            w = int(float(w) / sc)
            s = (w + al - 1) // al * al
        return w, h, s

    def deviceResults(self, pair):
        ps = [ctypes.c_void_p() for _ in range(5)]
        N.check(self._lib.rf_batch_device_results(self._h, int(pair), *[ctypes.byref(p) for p in ps]))
        return [p.value for p in ps]

    def _out(self, pair):
        w, h = self.sizes[pair]
        return np.zeros((h, self.strides[pair]), np.float32)

    def copyOpticalFlowToHost(self, pair):
        u, v = self._out(pair), self._out(pair)
        N.check(self._lib.rf_batch_download_flow(self._h, int(pair), _ptr(u), _ptr(v), u.shape[1]))
        return u, v

    def copy3dToHost(self, pair):
        X, Y, Z = self._out(pair), self._out(pair), self._out(pair)
        N.check(self._lib.rf_batch_download_points(self._h, int(pair), _ptr(X), _ptr(Y), _ptr(Z),
                                                   X.shape[1]))
        return X, Y, Z

    def copyInverseDepthToHost(self, pair):
        o = self._out(pair)
        N.check(self._lib.rf_batch_download_inv_depth(self._h, int(pair), _ptr(o), o.shape[1]))
        return o

    def importResults(self, pair, ptrs, pitch):
        """rf_batch_import_results: pair's solution replaced by device planes
        (u, v, X, Y, Z pointers, e.g. another solver's deviceResults())."""
        N.check(self._lib.rf_batch_import_results(self._h, int(pair),
                                                  *[ctypes.c_void_p(p or 0) for p in ptrs],
                                                  int(pitch)))

    def setStream(self, stream_ptr):
        N.check(self._lib.rf_batch_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def stream(self) -> int:
        """The CUDA stream the batch enqueues on (rf_batch_get_stream)."""
        st = ctypes.c_void_p()
        N.check(self._lib.rf_batch_get_stream(self._h, ctypes.byref(st)))
        return st.value or 0

    def synchronize(self):
        N.check(self._lib.rf_batch_synchronize(self._h))

    def kernelLaunches(self):
        return int(self._lib.rf_batch_kernel_launches(self._h))
