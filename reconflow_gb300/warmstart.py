"""Learned warm start for the ReconFlow solve.

A small BF16 convolutional encoder-decoder (``rf_cnn_*`` in the C ABI; all of
its forward, backward and optimizer work runs in this library's own CUDA
kernels) maps a coarse frame pair plus the camera pose to flow and inverse
depth.  Its input is built on the GPU by ``rf_ws_features``: the two coarse
frames and a plane sweep of photometric costs over inverse depth along each
pixel's epipolar line (the pose and intrinsics enter through the sweep), so
the network regresses inverse depth from matching evidence rather than
learning the camera geometry.  ``rf_ws_state`` turns its inverse depth into
the solver's state at a pyramid level (3D points and their flow, exactly as
the solver's projection forms it), and ``ReconFlowBatch.solveWarm`` refines
from there with fewer levels, warps and iterations than the plain solve.
The network is trained on flow and depth fields produced by the plain
solver itself on seeded synthetic scenes.

Scale convention: the network sees frames at the same angular resolution in
training and use (focal length 125 px on its input grid): 640x480 pairs
(f = 500) at 1/4 scale (160x120) in training, 1280x720 pairs (f = 1000) at
1/8 (160x90) in use.  Its finer output is on its input grid (1/8 of a 720p
frame), its coarser output at half of it (1/16); flow is in pixels of the
output's own grid, inverse depth in 1/m.
"""
from __future__ import annotations

import ctypes
import struct
import zlib

import numpy as np

from . import _native as N

IN_CH = 16
OUT_CH = 8
# u, v, inverse depth: the warm start uses the inverse depth; the flow heads
# are an auxiliary task
LOSS_WEIGHTS = (0.1, 0.1, 10.0)
F_NET = 125.0  # focal length (pixels) of the network's input grid

# Refinement schedules of the learned path by frame size (warps and
# iterations per pyramid level, index 0 = finest), chosen on held-out
# scenes: few level-0 iterations, more at the coarser levels.  The temporal
# warm start of sequences refines with the same schedules.
SCHEDULES = {
    (1280, 720): dict(warm_level=1, warps=[1, 1], iters=[3, 50]),
    (1920, 1080): dict(warm_level=2, warps=[1, 1, 1], iters=[4, 60, 80]),
    (3840, 2160): dict(warm_level=3, warps=[1, 1, 1, 1], iters=[4, 30, 60, 80]),
}


def box_down(a: np.ndarray, f: int) -> np.ndarray:
    """Mean over f x f blocks (the solver's 2x downscale applied log2(f)
    times, for sizes divisible by f); trailing rows / columns are dropped."""
    H, W = a.shape[0] // f * f, a.shape[1] // f * f
    a = a[:H, :W]
    return a.reshape(H // f, f, W // f, f, *a.shape[2:]).mean(axis=(1, 3))


def _dptr_array(ptrs):
    return (ctypes.c_void_p * len(ptrs))(*[ctypes.c_void_p(int(p)) for p in ptrs])


def _dbl_rows(rows, k):
    a = np.ascontiguousarray(np.asarray(rows, np.float64).reshape(-1, k))
    return a, a.ctypes.data_as(ctypes.c_void_p)


def features(I0_ptrs, I1_ptrs, w0, h0, s0, factor, Ks, Rs, ts, out, stream=0):
    """rf_ws_features: network input for n pairs of device frames into the
    (n, h0 // factor, w0 // factor, 16) float32 CUDA tensor `out`."""
    lib = N.load()
    n = len(I0_ptrs)
    assert out.shape == (n, h0 // factor, w0 // factor, IN_CH) and out.is_contiguous()
    K, pK = _dbl_rows(Ks, 9)
    R, pR = _dbl_rows(Rs, 9)
    t, pt = _dbl_rows(ts, 3)
    N.check(lib.rf_ws_features(n, _dptr_array(I0_ptrs), _dptr_array(I1_ptrs), int(w0), int(h0),
                               int(s0), int(factor), pK, pR, pt, ctypes.c_void_p(out.data_ptr()),
                               ctypes.c_void_p(stream or 0)))
    return out


def state(net_out, w, h, s, up, K_level, Rs, ts, planes, stream=0):
    """rf_ws_state: warm-start planes (u, v, X, Y, Z device pointers per
    pair) at a w x h level from the network output tensor (n, hn, wn, C)."""
    lib = N.load()
    n, hn, wn, C = net_out.shape
    K, pK = _dbl_rows(K_level, 9)
    R, pR = _dbl_rows(Rs, 9)
    t, pt = _dbl_rows(ts, 3)
    cols = list(zip(*planes))
    N.check(lib.rf_ws_state(n, ctypes.c_void_p(net_out.data_ptr()), int(C), int(wn), int(hn),
                            int(w), int(h), int(s), ctypes.c_float(up), pK, pR, pt,
                            *[_dptr_array(c) for c in cols], ctypes.c_void_p(stream or 0)))


def propagate(Z_ptrs, w, h, s, Ks, Rs, ts, factor, out, channel=2, stream=0, scratch=None):
    """rf_ws_propagate: frame k's inverse-depth grid from frame k-1's solved
    depth planes (device pointers, one per pair) into channel `channel` of
    the (n, hn, wn, C) float32 CUDA tensor `out` (R, t: camera k-1 -> k);
    `scratch`: an int32 CUDA tensor of 2 n hn wn elements (made if None)."""
    import torch

    lib = N.load()
    n, hn, wn, C = out.shape
    assert len(Z_ptrs) == n and out.is_contiguous()
    if scratch is None:
        scratch = torch.empty(2 * n * hn * wn, dtype=torch.int32, device=out.device)
    assert scratch.numel() >= 2 * n * hn * wn
    K, pK = _dbl_rows(Ks, 9)
    R, pR = _dbl_rows(Rs, 9)
    t, pt = _dbl_rows(ts, 3)
    N.check(lib.rf_ws_propagate(n, _dptr_array(Z_ptrs), int(w), int(h), int(s), pK, pR, pt,
                                int(factor), int(wn), int(hn), int(C), int(channel),
                                ctypes.c_void_p(out.data_ptr()),
                                ctypes.c_void_p(scratch.data_ptr()), ctypes.c_void_p(stream or 0)))
    return out


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

    def kernel_launches(self) -> int:
        return int(self._lib.rf_cnn_kernel_launches(self._h))

    def wait_gave_up(self) -> bool:
        """rf_cnn_status: whether a tensor-core launch gave up on a bounded
        wait since the last call (clears the flag; synchronizes)."""
        v = ctypes.c_int(0)
        N.check(self._lib.rf_cnn_status(self._h, ctypes.byref(v)))
        return bool(v.value)

    def set_test_wait_limit(self, polls: int):
        """rf_cnn_set_test_wait_limit: cap the first ring-slot wait of every
        tensor-core CTA at `polls` polls (0: give up at once); -1 restores
        the normal limit.  For tests of the give-up path."""
        N.check(self._lib.rf_cnn_set_test_wait_limit(self._h, int(polls)))

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

# the 640x480 workload's schedule and the solver weights of the benchmarks
SOLVER_640 = dict(levels=5, warps=3, iters=50)
SOLVER_WEIGHTS = dict(lambda_=50.0, lambdaf=0.1, lambdams=100.0, alphaTv=1 / 0.33, alphaProj=60.0,
                      tau=0.25, fix_quirks=1)


def _targets(u, v, Z, f):
    """(H/f, W/f, 8) target and (H/f, W/f) mask from a level-0 solution:
    flow / f and inverse depth box-averaged; the mask keeps blocks whose every
    pixel has a finite flow and a depth in (0.5, 50) m."""
    with np.errstate(divide="ignore", invalid="ignore"):
        ok = np.isfinite(u) & np.isfinite(v) & np.isfinite(Z) & (Z > 0.5) & (Z < 50.0)
        inv = np.where(ok, 1.0 / Z, 0.0)
    u0 = np.where(ok, u, 0.0)
    v0 = np.where(ok, v, 0.0)
    okf = box_down(ok.astype(np.float32), f)
    H, W = okf.shape
    t = np.zeros((H, W, OUT_CH), np.float32)
    den = np.maximum(okf, 1e-6)
    t[..., 0] = box_down(u0, f) / den / f
    t[..., 1] = box_down(v0, f) / den / f
    t[..., 2] = box_down(inv, f) / den
    m = (okf > 0.99).astype(np.float32)
    t[m == 0] = 0.0
    return t, m


def training_set(n_scenes: int, seed0: int = 10_000, width: int = 640, height: int = 480,
                 factor: int = 4, batch: int = 64, solver_params=None, log=None):
    """Render n seeded scenes on the GPU, solve them with the plain batched
    solver (the 640x480 schedule) and return numpy arrays: network inputs at
    1/factor, targets and masks at 1/(2 factor) and 1/factor, and the
    ground-truth inverse depth at 1/factor (for reporting only)."""
    import time

    import torch

    from .reconflow import ReconFlowBatch
    from .scene import make_scene

    sp = dict(SOLVER_WEIGHTS)
    sp.update(solver_params or {})
    hn, wn = height // factor, width // factor
    xs, t8s, m8s, t16s, m16s, gts = [], [], [], [], [], []
    t_render = t_solve = 0.0
    for b0 in range(0, n_scenes, batch):
        n = min(batch, n_scenes - b0)
        ta = time.perf_counter()
        scenes = [make_scene(width, height, seed=seed0 + b0 + i, device="cuda") for i in range(n)]
        tb = time.perf_counter()
        bt = ReconFlowBatch([(width, height)] * n, SOLVER_640["levels"], method=14,
                            nWarpIters=SOLVER_640["warps"], nSolverIters=SOLVER_640["iters"], **sp)
        for i, sc in enumerate(scenes):
            s = bt.strides[i]
            pad = lambda a: np.pad(a, ((0, 0), (0, s - width))).astype(np.float32)  # noqa: E731
            bt.setCameraMatrices(i, sc["K"], sc["K"])
            bt.copyImagesToDevice(i, pad(sc["I0"]), pad(sc["I1"]))
        bt.solveR([sc["R"] for sc in scenes], [sc["t"] for sc in scenes])
        x = torch.empty((n, hn, wn, IN_CH), device="cuda")
        planes = [bt.imagePlanes(i, 0) for i in range(n)]
        features([p[0] for p in planes], [p[1] for p in planes], width, height, bt.strides[0],
                 factor, [sc["K"] for sc in scenes], [sc["R"] for sc in scenes],
                 [sc["t"] for sc in scenes], x)
        xs.append(x.cpu().numpy())
        for i, sc in enumerate(scenes):
            u, v = bt.copyOpticalFlowToHost(i)
            _, _, Z = bt.copy3dToHost(i)
            u, v, Z = u[:, :width], v[:, :width], Z[:, :width]
            for f, (tl, ml) in ((factor, (t8s, m8s)), (2 * factor, (t16s, m16s))):
                t, m = _targets(u, v, Z, f)
                tl.append(t)
                ml.append(m)
            gts.append(box_down(sc["inv_depth"], factor))
        bt.close()
        t_solve += time.perf_counter() - tb
        t_render += tb - ta
        if log:
            log(f"training set: {b0 + n} / {n_scenes} scenes (render {t_render:.0f} s, "
                f"solve + features {t_solve:.0f} s)")
    return (np.concatenate(xs), np.stack(t16s), np.stack(m16s), np.stack(t8s), np.stack(m8s),
            np.stack(gts))


def train(net: WarmStartNet, data, epochs: int = 20, batch: int = 64, lr: float = 1e-3,
          seed: int = 0, log=None, lr_decay_at=None, weights=LOSS_WEIGHTS):
    """Adam on shuffled mini-batches; returns the loss per epoch.  `data` =
    (x, t16, m16, t8, m8[, ...]) numpy arrays or CUDA tensors."""
    import torch

    x, t16, m16, t8, m8 = (torch.as_tensor(a, device="cuda") for a in data[:5])
    n = x.shape[0]
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        cur = lr * (0.1 if lr_decay_at is not None and ep >= lr_decay_at else 1.0)
        perm = rng.permutation(n)
        tot, cnt = 0.0, 0
        for b0 in range(0, n - batch + 1 if n >= batch else 1, batch):
            idx = torch.as_tensor(perm[b0:b0 + batch], device="cuda")
            loss = net.backward(x[idx], t16[idx], m16[idx], t8[idx], m8[idx], weights)
            net.adam_step(cur)
            tot += loss
            cnt += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4f}")
    return hist


# ---------------------------------------------------------------------------
# Warm-started batched solve
# ---------------------------------------------------------------------------

def net_factor(K, f_net: float = F_NET) -> int:
    """Power-of-two downscale that brings a camera's focal length closest to
    the network's (8 for 1280x720 at f = 1000, 4 for 640x480 at f = 500)."""
    f = float(np.asarray(K)[0, 0])
    k = max(0, int(round(np.log2(max(f / f_net, 1.0)))))
    return 1 << k


class LearnedBatchSolver:
    """Batched ReconFlow solve started from the network's prediction.

    All pairs share one size.  solve() runs, on one CUDA stream: the input
    features at 1/factor (rf_ws_features), the network forward pass
    (rf_cnn_forward), the warm-start state at pyramid level `warm_level`
    from the network's finer output (rf_ws_state, written into the batch's
    warm planes) and the refinement from that level (rf_batch_solve_warm)
    with `warps` x `iters` per level."""

    def __init__(self, net: WarmStartNet, batch, size, K, warm_level=2, warps=2, iters=20):
        import torch

        self.net, self.batch = net, batch
        self.w, self.h = size
        self.factor = net_factor(K)
        self.hn, self.wn = self.h // self.factor, self.w // self.factor
        n = batch.n
        if n > net.max_batch or self.hn > net.height or self.wn > net.width:
            raise ValueError("network buffers are smaller than the batch")
        self.x = torch.empty((n, self.hn, self.wn, IN_CH), device="cuda")
        self.o16 = torch.empty((n, (self.hn + 1) // 2, (self.wn + 1) // 2, OUT_CH), device="cuda")
        self.o8 = torch.empty((n, self.hn, self.wn, OUT_CH), device="cuda")
        self.warm_level, self.warps, self.iters = warm_level, warps, iters
        lw, lh, ls = batch.levelDims(0, warm_level)
        self.level_dims = (lw, lh, ls)
        self.up = float(self.factor) / float(2 ** warm_level)
        self.planes = [batch.warmPlanes(i) for i in range(n)]
        self.images = [batch.imagePlanes(i, 0) for i in range(n)]
        # the buffers above were made on torch's stream; every later kernel
        # runs on the batch's stream
        torch.cuda.synchronize()

    @property
    def stream(self) -> int:
        """The stream everything runs on: the batch's (ReconFlowBatch.stream)."""
        return self.batch.stream()

    def set_stream(self, stream_ptr):
        """Run the features, the network, the state and the solve on this
        stream (0 / None: the batch's own)."""
        self.batch.setStream(stream_ptr)

    def predict(self, Ks, Rs, ts):
        st = self.stream
        self.net.set_stream(st)
        features([p[0] for p in self.images], [p[1] for p in self.images], self.w, self.h,
                 self.batch.strides[0], self.factor, Ks, Rs, ts, self.x, st)
        self.net.forward(self.x, self.o16, self.o8)
        return self.o16, self.o8

    def solve(self, Ks, Rs, ts):
        self.predict(Ks, Rs, ts)
        lw, lh, ls = self.level_dims
        Kl = [level_intrinsics(K, self.warm_level) for K in Ks]
        state(self.o8, lw, lh, ls, self.up, Kl, Rs, ts, self.planes, self.stream)
        self.batch.solveWarm(self.warm_level, Rs, ts, self.warps, self.iters)


class TemporalBatchSolver:
    """Batched ReconFlow solve of frame sequences: slot i of the batch
    follows sequence i, one pair (frame k, frame k + 1) per wave.  Wave 0
    starts from the network (LearnedBatchSolver); every later wave starts
    from the previous wave's solved depth carried into the new frame
    (rf_ws_propagate, the previous pair's pose) and turned into the warm
    planes (rf_ws_state), then refines from `warm_level` with the temporal
    schedule.  The caller uploads each wave's frames into the batch before
    calling first() / next()."""

    def __init__(self, net: WarmStartNet, batch, size, K, warm_level=2, warps=1, iters=20,
                 temporal_warps=None, temporal_iters=None):
        import torch

        self.learned = LearnedBatchSolver(net, batch, size, K, warm_level, warps, iters)
        self.batch = batch
        self.w, self.h = size
        ls = self.learned
        self.factor, self.hn, self.wn = ls.factor, ls.hn, ls.wn
        n = batch.n
        self.grid = torch.zeros((n, self.hn, self.wn, 3), device="cuda")
        self.scratch = torch.zeros(2 * n * self.hn * self.wn, dtype=torch.int32, device="cuda")
        self.warm_level = warm_level
        self.t_warps = warps if temporal_warps is None else temporal_warps
        self.t_iters = iters if temporal_iters is None else temporal_iters
        torch.cuda.synchronize()

    @property
    def stream(self) -> int:
        return self.batch.stream()

    def set_stream(self, stream_ptr):
        self.learned.set_stream(stream_ptr)

    def first(self, Ks, Rs, ts):
        """Wave 0: the network's warm start."""
        self.learned.solve(Ks, Rs, ts)

    def next(self, Ks, R_prev, t_prev, Rs, ts):
        """Wave k > 0 from wave k - 1's solutions still in the batch (its
        pairs' poses R_prev, t_prev carry them into the new frames)."""
        b = self.batch
        zs = [b.deviceResults(i)[4] for i in range(b.n)]
        propagate(zs, self.w, self.h, b.strides[0], Ks, R_prev, t_prev, self.factor, self.grid,
                  stream=self.stream, scratch=self.scratch)
        lw, lh, lsd = self.learned.level_dims
        Kl = [level_intrinsics(K, self.warm_level) for K in Ks]
        state(self.grid, lw, lh, lsd, self.learned.up, Kl, Rs, ts, self.learned.planes,
              self.stream)
        b.solveWarm(self.warm_level, Rs, ts, self.t_warps, self.t_iters)


# ---------------------------------------------------------------------------
# Command line: train the network and write a checkpoint
# ---------------------------------------------------------------------------

def main(argv=None):
    """python -m reconflow_gb300.warmstart --scenes N --epochs E --out PATH

    Renders N seeded 640x480 scenes (seeds 10000 ...), solves them with the
    plain batched solver, trains the network on its results (the last
    N // 8 scenes held out) and writes the checkpoint."""
    import argparse
    import time

    ap = argparse.ArgumentParser(description=main.__doc__.split("\n\n")[0])
    ap.add_argument("--scenes", type=int, default=20480)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    t0 = time.time()
    log = lambda m: print(f"[{time.time() - t0:7.1f} s] {m}", flush=True)  # noqa: E731
    data = training_set(a.scenes, log=log)
    nh = max(1, a.scenes // 8)
    tr = tuple(d[:-nh] for d in data[:5])
    te = tuple(d[-nh:] for d in data)
    net = WarmStartNet(64, 120, 160, seed=a.seed)
    train(net, tr, epochs=a.epochs, batch=64, lr=a.lr, seed=a.seed, log=log,
          lr_decay_at=int(a.epochs * 0.75))
    net.save(a.out)
    import torch

    xt = torch.as_tensor(te[0], device="cuda")
    p8 = np.concatenate([net.forward(xt[b0:b0 + 64])[1].cpu().numpy() for b0 in range(0, nh, 64)])
    m = te[4] > 0
    rel = (np.abs(p8[..., 2] - te[3][..., 2]) / np.maximum(te[3][..., 2], 1e-3))[m]
    relgt = (np.abs(p8[..., 2] - te[5]) / te[5])[m]
    log(f"held out ({nh} scenes): inverse depth relative error, median {np.median(rel):.4f} "
        f"against the plain solver, {np.median(relgt):.4f} against ground truth; wrote {a.out}")


if __name__ == "__main__":
    main()
