"""CameraPose: relative pose of two frames (reconflow/CameraPose.h:11-64).

The reference's class detects SURF keypoints with OpenCV's CUDA SURF, matches
them by brute force with a 0.6 ratio test, and estimates the pose with
findEssentialMat (LMEDS) and recoverPose (CameraPose.cpp:47-118).  This class
keeps its method names and return convention (0 = pose found, 1 = not) over
the C ABI ``rf_pose_*``: GPU feature detection, description and matching, and
the five-point LMedS and pose recovery on the host.  R and t satisfy
x1 = R x0 + t with |t| = 1, the pose ``ReconFlow.solveR`` takes.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N


def _dbl(a, n):
    a = np.ascontiguousarray(np.asarray(a, np.float64).reshape(n))
    return a, a.ctypes.data_as(ctypes.c_void_p)


def bgr_to_gray(img):
    """cv::cvtColor(..., CV_BGR2GRAY) for 8-bit frames (CameraPose.cpp:121-122):
    Y = 0.299 R + 0.587 G + 0.114 B in 14-bit fixed point, rounded."""
    img = np.asarray(img, np.uint8)
    b, g, r = (img[..., k].astype(np.int64) for k in range(3))
    return ((r * 4899 + g * 9617 + b * 1868 + (1 << 13)) >> 14).astype(np.uint8)


class CameraPose:
    def __init__(self):
        self._lib = N.load()
        self._h = None
        self._size = None
        self.params = N.RfPoseParams()
        N.check(self._lib.rf_pose_params_default(ctypes.byref(self.params)))
        self.intrinsic = None
        self.K = None
        self.R = None
        self.t = None
        self.stream = None

    # -- CameraPose::initialize overloads (CameraPose.cpp:11-45) ------------
    def initialize(self, *args):
        """initialize(K), initialize(K, minHessian), initialize(focal, pp),
        initialize(focal, pp, minHessian), initialize(focalx, focaly, pp,
        minHessian); minHessian defaults to 2000."""
        min_hessian = 2000.0
        if np.ndim(args[0]) == 2:
            K = np.asarray(args[0], np.float64).reshape(3, 3)
            if len(args) > 1:
                min_hessian = float(args[1])
        elif len(args) == 4:
            fx, fy, pp, min_hessian = float(args[0]), float(args[1]), args[2], float(args[3])
            K = np.array([[fx, 0.0, pp[0]], [0.0, fy, pp[1]], [0.0, 0.0, 1.0]])
        else:
            f, pp = float(args[0]), args[1]
            if len(args) > 2:
                min_hessian = float(args[2])
            K = np.array([[f, 0.0, pp[0]], [0.0, f, pp[1]], [0.0, 0.0, 1.0]])
        self.intrinsic = K.copy()
        self.K = self.intrinsic
        self.params.hessian_threshold = min_hessian
        self._release()
        return 0

    def set_stream(self, stream_ptr):
        self.stream = stream_ptr
        if self._h is not None:
            N.check(self._lib.rf_pose_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def _handle(self, w, h):
        if self._h is not None and self._size == (w, h):
            return self._h
        self._release()
        hp = ctypes.c_void_p()
        N.check(self._lib.rf_pose_create(ctypes.byref(self.params), int(w), int(h),
                                         ctypes.byref(hp)))
        self._h, self._size = hp, (w, h)
        if self.stream:
            N.check(self._lib.rf_pose_set_stream(self._h, ctypes.c_void_p(self.stream)))
        return self._h

    def _release(self):
        if self._h is not None:
            self._lib.rf_pose_destroy(self._h)
            self._h = None
            self._size = None

    def close(self):
        self._release()

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass

    # -- solve -----------------------------------------------------------------
    def _solve(self, fn, im1, im2, dtype):
        if self.K is None:
            raise RuntimeError("CameraPose.initialize first")
        a = np.ascontiguousarray(im1, dtype)
        b = np.ascontiguousarray(im2, dtype)
        if a.shape != b.shape or a.ndim != 2:
            raise ValueError("two gray frames of one size")
        h, w = a.shape
        hd = self._handle(w, h)
        _, pK = _dbl(self.K, 9)
        R = np.zeros(9)
        t = np.zeros(3)
        st = fn(hd, a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p), w, pK,
                R.ctypes.data_as(ctypes.c_void_p), t.ctypes.data_as(ctypes.c_void_p))
        if st != N.RF_OK:
            if st == 5:  # RF_ERR_STATE: no keypoints / too few matches / no model
                return 1, None, None
            N.check(st)
        self.R, self.t = R.reshape(3, 3), t
        return 0, self.R, self.t

    def solvePose_8uc1(self, im1, im2):
        """(0, R, t) for 8-bit gray frames, or (1, None, None) when no pose is
        found (CameraPose.cpp:47-118)."""
        return self._solve(self._lib.rf_pose_solve_u8, im1, im2, np.uint8)

    def solvePose_8uc3(self, im1, im2):
        """BGR frames: gray conversion, then solvePose_8uc1 (CameraPose.cpp:120-128)."""
        return self.solvePose_8uc1(bgr_to_gray(im1), bgr_to_gray(im2))

    def solvePose_f32(self, im1, im2):
        """Float gray frames in [0, 1] (converted to 8 bits on the GPU as
        round(255 v))."""
        return self._solve(self._lib.rf_pose_solve_f32, im1, im2, np.float32)

    # -- results of the last solve ---------------------------------------------
    def counts(self):
        """(keypoints in frame 0, in frame 1, matches, inliers)."""
        v = [ctypes.c_int() for _ in range(4)]
        N.check(self._lib.rf_pose_counts(self._h, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def keypoints(self, frame):
        """([n][6] array of x, y, scale, angle, response, octave; [n][64] descriptors)."""
        n = self.counts()[frame]
        kp = (N.RfKeypoint * max(n, 1))()
        desc = np.zeros((n, 64), np.float32)
        N.check(self._lib.rf_pose_keypoints(self._h, int(frame), kp,
                                            desc.ctypes.data_as(ctypes.c_void_p), n))
        arr = np.array([[k.x, k.y, k.scale, k.angle, k.response, k.octave] for k in kp[:n]],
                       np.float32).reshape(n, 6)
        return arr, desc

    def matches(self):
        """(idx0, idx1, distance, inlier) of the matches that passed the ratio test."""
        n = self.counts()[2]
        i0 = np.zeros(n, np.int32)
        i1 = np.zeros(n, np.int32)
        d = np.zeros(n, np.float32)
        inl = np.zeros(n, np.uint8)
        N.check(self._lib.rf_pose_matches(self._h, i0.ctypes.data_as(ctypes.c_void_p),
                                          i1.ctypes.data_as(ctypes.c_void_p),
                                          d.ctypes.data_as(ctypes.c_void_p),
                                          inl.ctypes.data_as(ctypes.c_void_p), n))
        return i0, i1, d, inl.astype(bool)

    def kernel_launches(self):
        return int(self._lib.rf_pose_kernel_launches(self._h)) if self._h is not None else 0

    def responses(self, frame, octave):
        w, h = self._size
        layers = self.params.n_octave_layers + 2
        out = np.zeros((layers, h >> octave, w >> octave), np.float32)
        N.check(self._lib.rf_pose_responses(self._h, int(frame), int(octave),
                                            out.ctypes.data_as(ctypes.c_void_p), out.size))
        return out


def essential_5pt(x0, x1):
    """Up to 10 essential matrices through five normalized matches ([5][2] each)."""
    lib = N.load()
    a = np.ascontiguousarray(np.asarray(x0, np.float64).reshape(5, 2))
    b = np.ascontiguousarray(np.asarray(x1, np.float64).reshape(5, 2))
    out = np.zeros((10, 3, 3))
    n = lib.rf_essential_5pt(a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p),
                             out.ctypes.data_as(ctypes.c_void_p))
    return out[:max(n, 0)].copy()


def essential_lmeds(x0, x1, confidence=0.999, seed=0x5EED):
    """(E, inlier mask) by least median of squares over normalized matches."""
    lib = N.load()
    a = np.ascontiguousarray(np.asarray(x0, np.float64).reshape(-1, 2))
    b = np.ascontiguousarray(np.asarray(x1, np.float64).reshape(-1, 2))
    n = len(a)
    E = np.zeros(9)
    mask = np.zeros(n, np.uint8)
    N.check(lib.rf_essential_lmeds(a.ctypes.data_as(ctypes.c_void_p),
                                   b.ctypes.data_as(ctypes.c_void_p), n, float(confidence),
                                   int(seed), E.ctypes.data_as(ctypes.c_void_p),
                                   mask.ctypes.data_as(ctypes.c_void_p)))
    return E.reshape(3, 3), mask.astype(bool)


def recover_pose(E, x0, x1, mask=None):
    """(R, t, number of points in front of both cameras)."""
    lib = N.load()
    a = np.ascontiguousarray(np.asarray(x0, np.float64).reshape(-1, 2))
    b = np.ascontiguousarray(np.asarray(x1, np.float64).reshape(-1, 2))
    n = len(a)
    _, pE = _dbl(E, 9)
    m = None if mask is None else np.ascontiguousarray(np.asarray(mask, np.uint8))
    R = np.zeros(9)
    t = np.zeros(3)
    good = ctypes.c_int()
    N.check(lib.rf_recover_pose(pE, a.ctypes.data_as(ctypes.c_void_p),
                                b.ctypes.data_as(ctypes.c_void_p), n,
                                None if m is None else m.ctypes.data_as(ctypes.c_void_p),
                                R.ctypes.data_as(ctypes.c_void_p),
                                t.ctypes.data_as(ctypes.c_void_p), ctypes.byref(good)))
    return R.reshape(3, 3), t, good.value


def refine_pose(R, t, x0, x1, mask=None):
    """(R, t) refined on the inliers' Sampson distances (rf_refine_pose)."""
    lib = N.load()
    a = np.ascontiguousarray(np.asarray(x0, np.float64).reshape(-1, 2))
    b = np.ascontiguousarray(np.asarray(x1, np.float64).reshape(-1, 2))
    m = None if mask is None else np.ascontiguousarray(np.asarray(mask, np.uint8))
    Rr = np.ascontiguousarray(np.asarray(R, np.float64).reshape(9)).copy()
    tr = np.ascontiguousarray(np.asarray(t, np.float64).reshape(3)).copy()
    N.check(lib.rf_refine_pose(a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p),
                               len(a), None if m is None else m.ctypes.data_as(ctypes.c_void_p),
                               Rr.ctypes.data_as(ctypes.c_void_p), tr.ctypes.data_as(ctypes.c_void_p)))
    return Rr.reshape(3, 3), tr
