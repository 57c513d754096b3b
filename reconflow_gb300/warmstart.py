"""Learned warm start for the ReconFlow solve.

A small BF16 convolutional encoder-decoder (``rf_cnn_*`` in the C ABI; all of
its forward, backward and optimizer work runs in this library's own CUDA
kernels) maps a coarse image pair plus the camera pose to flow and inverse
depth.  It is trained on flow and depth fields produced by the plain solver
itself on seeded synthetic scenes, then used to start the solve at a finer
pyramid level (``ReconFlow.solveWarm``) with fewer iterations.  The solution
energy (``ReconFlow.energy``) decides whether the warm-started result is kept
or the plain solve is used instead.

Scale convention: the network sees images sampled at the same angular
resolution in training and use: 640x480 pairs (f = 500) at 1/8 scale (80x60)
in training, 1280x720 pairs (f = 1000) at 1/16 (80x45) in use.  Its finer
output is at the input resolution, its coarser output at half of it; flow is
in pixels of the output's own grid, inverse depth in 1/m.
"""
from __future__ import annotations

import ctypes
import math
import struct
import zlib

import numpy as np

from . import _native as N

IN_CH = 16
OUT_CH = 8
LOSS_WEIGHTS = (1.0, 1.0, 10.0)  # u, v, inverse depth


def rotation_vector(R) -> np.ndarray:
    R = np.asarray(R, np.float64)
    c = (np.trace(R) - 1.0) / 2.0
    ang = math.acos(max(-1.0, min(1.0, c)))
    if ang < 1e-12:
        return np.zeros(3)
    v = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    return v * (ang / (2.0 * math.sin(ang)))


def make_input(I0c, I1c, R, t) -> np.ndarray:
    """(H, W) coarse frames + pose -> (H, W, 16) float32 network input."""
    H, W = I0c.shape
    x = np.zeros((H, W, IN_CH), np.float32)
    x[..., 0] = I0c
    x[..., 1] = I1c
    x[..., 2] = (np.arange(W)[None, :] + 0.5) / W - 0.5
    x[..., 3] = (np.arange(H)[:, None] + 0.5) / H - 0.5
    rv = rotation_vector(R) * 30.0
    tt = np.asarray(t, np.float64) * 10.0
    for k in range(3):
        x[..., 4 + k] = rv[k]
        x[..., 7 + k] = tt[k]
    return x


def box_down(a: np.ndarray, f: int) -> np.ndarray:
    """Mean over f x f blocks (the solver's 2x downscale applied log2(f)
    times, for sizes divisible by f); trailing rows / columns are dropped."""
    H, W = a.shape[0] // f * f, a.shape[1] // f * f
    a = a[:H, :W]
    return a.reshape(H // f, f, W // f, f, *a.shape[2:]).mean(axis=(1, 3))


class WarmStartNet:
    """The network and its Adam state on the GPU."""

    def __init__(self, max_batch: int, height: int, width: int, seed: int = 0):
        self._lib = N.load()
        h = ctypes.c_void_p()
        N.check(self._lib.rf_cnn_create(int(max_batch), int(height), int(width),
                                        ctypes.c_ulonglong(seed), ctypes.byref(h)))
        self._h = h
        self.max_batch, self.height, self.width = max_batch, height, width
        self.n_params = self._lib.rf_cnn_num_params(h)

    def close(self):
        if self._h is not None:
            self._lib.rf_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        N.check(self._lib.rf_cnn_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        N.check(self._lib.rf_cnn_get_params(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        N.check(self._lib.rf_cnn_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))

    def grads(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        N.check(self._lib.rf_cnn_get_grads(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def forward(self, x, out16=None, out8=None):
        """x: torch CUDA tensor (B, H, W, 16) float32 -> (out16, out8) tensors."""
        import torch

        B, H, W, _ = x.shape
        x = x.contiguous()
        if out16 is None:
            out16 = torch.empty((B, (H + 1) // 2, (W + 1) // 2, OUT_CH), device=x.device)
        if out8 is None:
            out8 = torch.empty((B, H, W, OUT_CH), device=x.device)
        N.check(self._lib.rf_cnn_forward(self._h, ctypes.c_void_p(x.data_ptr()), B, H, W,
                                         ctypes.c_void_p(out16.data_ptr()),
                                         ctypes.c_void_p(out8.data_ptr())))
        return out16, out8

    def backward(self, x, t16, m16, t8, m8, weights=LOSS_WEIGHTS) -> float:
        B, H, W, _ = x.shape
        w = (ctypes.c_float * 3)(*weights)
        loss = ctypes.c_double()
        args = [ctypes.c_void_p(a.contiguous().data_ptr()) for a in (x, t16, m16, t8, m8)]
        N.check(self._lib.rf_cnn_backward(self._h, *args, B, H, W, w, ctypes.byref(loss)))
        return float(loss.value)

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        N.check(self._lib.rf_cnn_adam_step(self._h, ctypes.c_float(lr), ctypes.c_float(beta1),
                                           ctypes.c_float(beta2), ctypes.c_float(eps)))

    # checkpoint: magic, version, parameter count, CRC32 of the FP32 weights
    def save(self, path: str):
        p = self.params()
        blob = p.tobytes()
        with open(path, "wb") as f:
            f.write(struct.pack("<8sIIQI", b"RFWSNET1", 1, 0, p.size, zlib.crc32(blob)))
            f.write(blob)

    def load(self, path: str):
        with open(path, "rb") as f:
            magic, ver, _, n, crc = struct.unpack("<8sIIQI", f.read(28))
            blob = f.read()
        if magic != b"RFWSNET1" or n != self.n_params or zlib.crc32(blob) != crc:
            raise N.RfError(1, f"warm-start checkpoint {path} does not match this network")
        self.set_params(np.frombuffer(blob, np.float32))


# ---------------------------------------------------------------------------
# Training data from the plain solver
# ---------------------------------------------------------------------------

SOLVER_640 = dict(levels=5, warps=3, iters=50)  # the 640x480 workload's schedule


def training_set(n_scenes: int, seed0: int = 10_000, width: int = 640, height: int = 480,
                 batch: int = 64, solver_params=None, device="cuda"):
    """Render n seeded scenes, solve them with the plain (batched) solver and
    return network inputs at 1/8 and targets at 1/8 and 1/16 (numpy)."""
    from .reconflow import ReconFlowBatch
    from .scene import make_scene

    sp = dict(lambda_=50.0, lambdaf=0.1, lambdams=100.0, alphaTv=1 / 0.33, alphaProj=60.0,
              tau=0.25, fix_quirks=1)
    sp.update(solver_params or {})
    xs, t8s, m8s, t16s, m16s = [], [], [], [], []
    for b0 in range(0, n_scenes, batch):
        n = min(batch, n_scenes - b0)
        scenes = [make_scene(width, height, seed=seed0 + b0 + i, device=device) for i in range(n)]
        bt = ReconFlowBatch([(width, height)] * n, SOLVER_640["levels"], method=14,
                            nWarpIters=SOLVER_640["warps"], nSolverIters=SOLVER_640["iters"], **sp)
        for i, sc in enumerate(scenes):
            s = bt.strides[i]
            pad = lambda a: np.pad(a, ((0, 0), (0, s - width))).astype(np.float32)  # noqa: E731
            bt.setCameraMatrices(i, sc["K"], sc["K"])
            bt.copyImagesToDevice(i, pad(sc["I0"]), pad(sc["I1"]))
        bt.solveR([sc["R"] for sc in scenes], [sc["t"] for sc in scenes])
        for i, sc in enumerate(scenes):
            u, v = bt.copyOpticalFlowToHost(i)
            _, _, Z = bt.copy3dToHost(i)
            u, v, Z = u[:, :width], v[:, :width], Z[:, :width]
            with np.errstate(divide="ignore", invalid="ignore"):
                inv = np.where((Z > 0.5) & (Z < 50.0) & np.isfinite(Z), 1.0 / Z, 0.0)
            ok = (inv > 0).astype(np.float32)
            for f, (tl, ml) in ((8, (t8s, m8s)), (16, (t16s, m16s))):
                t = np.zeros((height // f, width // f, OUT_CH), np.float32)
                t[..., 0] = box_down(u, f) / f
                t[..., 1] = box_down(v, f) / f
                okf = box_down(ok, f)
                with np.errstate(invalid="ignore"):
                    t[..., 2] = np.where(okf > 0, box_down(inv, f) / np.maximum(okf, 1e-6), 0.0)
                tl.append(t)
                ml.append((okf > 0.99).astype(np.float32))
            xs.append(make_input(box_down(sc["I0"], 8), box_down(sc["I1"], 8), sc["R"], sc["t"]))
        bt.close()
    return (np.stack(xs), np.stack(t16s), np.stack(m16s), np.stack(t8s), np.stack(m8s))


def train(net: WarmStartNet, data, epochs: int = 20, batch: int = 64, lr: float = 1e-3,
          seed: int = 0, log=None):
    """Adam on shuffled mini-batches; returns the loss per epoch."""
    import torch

    x, t16, m16, t8, m8 = (torch.as_tensor(a, device="cuda") for a in data)
    n = x.shape[0]
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        perm = rng.permutation(n)
        tot, cnt = 0.0, 0
        for b0 in range(0, n - batch + 1 if n >= batch else 1, batch):
            idx = torch.as_tensor(perm[b0:b0 + batch], device="cuda")
            loss = net.backward(x[idx], t16[idx], m16[idx], t8[idx], m8[idx])
            net.adam_step(lr)
            tot += loss
            cnt += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4f}")
    return hist


# ---------------------------------------------------------------------------
# Warm-started solve of a 1280x720 pair
# ---------------------------------------------------------------------------

def predict(net: WarmStartNet, I0, I1, R, t, factor: int):
    """Network prediction for one pair at 1/factor scale: (u, v, inv_depth)
    on the input grid of the network (flow in its pixels)."""
    import torch

    x = make_input(box_down(I0, factor), box_down(I1, factor), R, t)
    _, o8 = net.forward(torch.as_tensor(x[None], device="cuda"))
    o = o8[0].cpu().numpy()
    return o[..., 0], o[..., 1], o[..., 2]


def warm_state(pred, K, level_shape, level_stride, scale_up: int, level_K):
    """Upsample a prediction to the warm-start level: flow scaled by
    scale_up, inverse depth turned into 3D points with that level's K."""
    import torch
    import torch.nn.functional as F

    u, v, inv = pred
    h, w = level_shape
    t = torch.as_tensor(np.stack([u * scale_up, v * scale_up, inv])[None], dtype=torch.float32)
    up = F.interpolate(t, size=(h, w), mode="bilinear", align_corners=False)[0].numpy()
    uu, vv = up[0], up[1]
    inv = np.clip(up[2], 0.02, 2.0)
    Z = 1.0 / inv
    fx, fy, cx, cy = level_K[0, 0], level_K[1, 1], level_K[0, 2], level_K[1, 2]
    xs = np.arange(w)[None, :]
    ys = np.arange(h)[:, None]
    X = Z * (xs - cx) / fx
    Y = Z * (ys - cy) / fy
    pad = lambda a: np.pad(a, ((0, 0), (0, level_stride - w))).astype(np.float32)  # noqa: E731
    return pad(uu), pad(vv), pad(X), pad(Y), pad(Z)


def level_intrinsics(K, level, scale=2.0):
    """K at a pyramid level with K[2][2] = 1 (the K-pyramid fix)."""
    Kl = np.array(K, np.float64).copy()
    for _ in range(level):
        Kl[0, 0] /= scale
        Kl[0, 2] /= scale
        Kl[1, 1] /= scale
        Kl[1, 2] /= scale
    Kl[2, 2] = 1.0
    return Kl
