"""Seeded synthetic stereo scenes with analytic ground truth.

A scene is a piecewise-planar surface seen by camera 0 (at the origin) and a
second camera moved rigidly (X1 = R X + t, the convention of the reference's
SolveUc, ``reconflow/solveUcSk.cu:25-33``):

* depth: 8 planes over a Voronoi partition of camera 0's image, each plane's
  inverse depth linear in pixel coordinates with depth inside [2, 10] m over
  the image;
* texture: 200 Gaussian blobs plus 1/f noise, an analytic function of camera-0
  pixel coordinates, normalised to [0, 1];
* frame 2: every camera-1 pixel is ray-cast against the planes (nearest hit
  whose camera-0 projection lies in that plane's cell) and takes the texture
  there;
* pose: rotation <= 2 degrees about a random axis, |t| = 0.1 m;
* N(0, 0.01) pixel noise on both frames.

K defaults to fx = fy = 500 * w / 640, cx = w / 2, cy = h / 2 (500, 320, 240
at 640x480).  Ground truth: flow of every camera-0 pixel, inverse depth, and
a validity mask (in view and not occluded in camera 1).
"""
from __future__ import annotations

import math

import numpy as np

__all__ = ["make_scene", "make_sequence", "smooth_path", "intrinsics_for", "random_pose",
           "render_pair"]


def intrinsics_for(width: int, height: int) -> np.ndarray:
    f = 500.0 * width / 640.0
    return np.array([[f, 0.0, width / 2.0], [0.0, f, height / 2.0], [0.0, 0.0, 1.0]])


def _rodrigues(axis: np.ndarray, angle: float) -> np.ndarray:
    a = axis / np.linalg.norm(axis)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * (K @ K)


def random_pose(rng: np.random.Generator, max_rot_deg: float = 2.0, trans: float = 0.1):
    axis = rng.normal(size=3)
    ang = math.radians(rng.uniform(0.0, max_rot_deg))
    R = _rodrigues(axis, ang)
    d = rng.normal(size=3)
    t = trans * d / np.linalg.norm(d)
    return R, t


class _Texture:
    """Gaussian blobs + 1/f noise, analytic in camera-0 pixel coordinates."""

    def __init__(self, rng, width, height, n_blobs=200, n_waves=48):
        w, h = float(width), float(height)
        m = 0.15  # blobs also cover a margin around the image
        self.cx = rng.uniform(-m * w, (1 + m) * w, n_blobs)
        self.cy = rng.uniform(-m * h, (1 + m) * h, n_blobs)
        self.sig = np.exp(rng.uniform(math.log(0.004 * w), math.log(0.05 * w), n_blobs))
        self.amp = rng.uniform(-1.0, 1.0, n_blobs)
        fmin, fmax = 1.0 / w, 0.2
        self.freq = np.exp(rng.uniform(math.log(fmin), math.log(fmax), n_waves))
        th = rng.uniform(0, 2 * math.pi, n_waves)
        self.kx = 2 * math.pi * self.freq * np.cos(th)
        self.ky = 2 * math.pi * self.freq * np.sin(th)
        self.ph = rng.uniform(0, 2 * math.pi, n_waves)
        self.wamp = 0.6 * (fmin / self.freq) ** 0.5
        self.lo, self.hi = 0.0, 1.0

    def raw(self, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        x = x.astype(np.float64).ravel()
        y = y.astype(np.float64).ravel()
        out = np.zeros_like(x)
        for i in range(len(self.amp)):
            r = 4.0 * self.sig[i]
            sel = np.nonzero((np.abs(x - self.cx[i]) < r) & (np.abs(y - self.cy[i]) < r))[0]
            if sel.size == 0:
                continue
            dx = x[sel] - self.cx[i]
            dy = y[sel] - self.cy[i]
            out[sel] += self.amp[i] * np.exp(-(dx * dx + dy * dy) / (2 * self.sig[i] ** 2))
        for i in range(len(self.freq)):
            out += self.wamp[i] * np.cos(self.kx[i] * x + self.ky[i] * y + self.ph[i])
        return out

    def __call__(self, x, y):
        shape = np.shape(x)
        v = (self.raw(x, y) - self.lo) / (self.hi - self.lo)
        return np.clip(v, 0.0, 1.0).reshape(shape)


class _Planes:
    """Inverse depth a + b x + c y over Voronoi cells of camera 0's image."""

    def __init__(self, rng, width, height, K, n_planes=8, zmin=2.0, zmax=10.0):
        w, h = float(width), float(height)
        self.seeds = np.stack([rng.uniform(0, w, n_planes), rng.uniform(0, h, n_planes)], 1)
        lo, hi = 1.0 / zmax, 1.0 / zmin
        abc = []
        for _ in range(n_planes):
            while True:
                d00, d10, d01 = rng.uniform(lo, hi, 3)
                d11 = d10 + d01 - d00
                if lo <= d11 <= hi:
                    break
            b = (d10 - d00) / w
            c = (d01 - d00) / h
            abc.append((d00, b, c))
        self.abc = np.array(abc)
        fx, fy, cx, cy = K[0, 0], K[1, 1], K[0, 2], K[1, 2]
        a, b, c = self.abc.T
        # inverse depth plane -> 3D plane n . X = 1 in camera-0 coordinates
        self.n = np.stack([b * fx, c * fy, a + b * cx + c * cy], 1)

    def label(self, x, y):
        d = (x[..., None] - self.seeds[:, 0]) ** 2 + (y[..., None] - self.seeds[:, 1]) ** 2
        return np.argmin(d, axis=-1)

    def inv_depth(self, x, y):
        k = self.label(x, y)
        a, b, c = self.abc[k, 0], self.abc[k, 1], self.abc[k, 2]
        return a + b * x + c * y


def _raycast(planes: _Planes, K, Kinv, R, t, xs, ys):
    """Nearest valid plane hit for camera-1 pixels; returns (X in camera 0, ok)."""
    C = -R.T @ t
    rays = np.stack([xs.ravel(), ys.ravel(), np.ones(xs.size)], 0)
    d = R.T @ (Kinv @ rays)  # directions in camera-0 coordinates, (3, N)
    best = np.full(xs.size, np.inf)
    hit = np.zeros((3, xs.size))
    nC = planes.n @ C
    nd = planes.n @ d  # (P, N)
    for k in range(planes.n.shape[0]):
        with np.errstate(divide="ignore", invalid="ignore"):
            lam = (1.0 - nC[k]) / nd[k]
        X = C[:, None] + lam[None, :] * d
        z = X[2]
        ok = (lam > 0) & (z > 1e-6) & np.isfinite(lam)
        with np.errstate(divide="ignore", invalid="ignore"):
            px = K[0, 0] * X[0] / z + K[0, 2]
            py = K[1, 1] * X[1] / z + K[1, 2]
        ok &= planes.label(np.where(ok, px, 0.0), np.where(ok, py, 0.0)) == k
        better = ok & (lam < best)
        best = np.where(better, lam, best)
        hit[:, better] = X[:, better]
    found = np.isfinite(best)
    return hit, found


def render_pair(width, height, K, R, t, planes, tex, rng, noise=0.01):
    """Render both frames and the ground truth of one pose."""
    Kinv = np.linalg.inv(K)
    ys, xs = np.mgrid[0:height, 0:width].astype(np.float64)
    inv_depth = planes.inv_depth(xs, ys)
    Z = 1.0 / inv_depth
    I0 = tex(xs, ys)
    # camera 1: ray-cast every pixel
    X, found = _raycast(planes, K, Kinv, R, t, xs, ys)
    with np.errstate(divide="ignore", invalid="ignore"):
        px = K[0, 0] * X[0] / X[2] + K[0, 2]
        py = K[1, 1] * X[1] / X[2] + K[1, 2]
    px = np.where(found, px, xs.ravel())
    py = np.where(found, py, ys.ravel())
    I1 = tex(px, py).reshape(height, width)
    # ground-truth flow of camera-0 pixels
    P0 = np.stack([xs.ravel() * Z.ravel(), ys.ravel() * Z.ravel(), Z.ravel()], 0)
    X0 = Kinv @ P0
    X1 = R @ X0 + t[:, None]
    u1 = K[0, 0] * X1[0] / X1[2] + K[0, 2]
    v1 = K[1, 1] * X1[1] / X1[2] + K[1, 2]
    flow = np.stack([(u1 - xs.ravel()).reshape(height, width),
                     (v1 - ys.ravel()).reshape(height, width)], -1)
    # validity: lands inside camera 1 and is the surface camera 1 sees there
    inb = (u1 >= 0) & (u1 <= width - 1) & (v1 >= 0) & (v1 <= height - 1)
    Xv, fv = _raycast(planes, K, Kinv, R, t, u1, v1)
    same = fv & (np.linalg.norm(Xv - X0, axis=0) < 1e-3 * np.maximum(X0[2], 1.0))
    valid = (inb & same).reshape(height, width)
    I0 = I0 + rng.normal(0.0, noise, I0.shape)
    I1 = I1 + rng.normal(0.0, noise, I1.shape)
    return {
        "I0": I0.astype(np.float32), "I1": I1.astype(np.float32),
        "flow": flow.astype(np.float32), "inv_depth": inv_depth.astype(np.float32),
        "depth": Z.astype(np.float32), "valid": valid,
    }


def make_scene(width: int, height: int, seed: int = 0, K=None, n_planes: int = 8,
               n_blobs: int = 200, max_rot_deg: float = 2.0, trans: float = 0.1,
               noise: float = 0.01, device=None) -> dict:
    """One seeded frame pair with ground truth (see module docstring).

    device=None renders with numpy; a torch CUDA device renders the same
    scene (same seeded parameters, same formulas) on the GPU, which is much
    faster for large or many scenes.  Returned arrays are numpy either way.
    """
    rng = np.random.default_rng(seed)
    K = intrinsics_for(width, height) if K is None else np.asarray(K, np.float64)
    planes = _Planes(rng, width, height, K, n_planes)
    tex = _Texture(rng, width, height, n_blobs)
    # normalise the texture once, from a coarse sample of camera 0's view
    gy, gx = np.mgrid[0:height:4, 0:width:4].astype(np.float64)
    raw = tex.raw(gx, gy) if device is None else _raw_torch(tex, gx, gy, device)
    tex.lo, tex.hi = float(np.percentile(raw, 0.5)), float(np.percentile(raw, 99.5))
    R, t = random_pose(rng, max_rot_deg, trans)
    if device is None:
        out = render_pair(width, height, K, R, t, planes, tex, rng, noise)
    else:
        out = _render_pair_torch(width, height, K, R, t, planes, tex, rng, noise, device)
    out.update({"K": K, "R": R, "t": t, "seed": seed})
    return out


# ---------------------------------------------------------------------------
# Sequences: one scene seen along a smooth camera path
# ---------------------------------------------------------------------------

def smooth_path(rng: np.random.Generator, n_frames: int, step: float = 0.05,
                max_turn_deg: float = 0.3):
    """Poses (R_k, t_k), X_k = R_k X + t_k, of a camera moving `step` metres
    per frame from the origin: mostly forward (the heading starts within
    ~17 degrees of the optical axis and drifts by a small random amount per
    frame), the orientation turning by at most `max_turn_deg` per frame
    about a slowly varying axis.  Frame 0 is the identity."""
    heading = np.array([rng.uniform(-0.3, 0.3), rng.uniform(-0.3, 0.3), 1.0])
    heading /= np.linalg.norm(heading)
    axis = rng.normal(size=3)
    C = np.zeros(3)
    R = np.eye(3)
    poses = [(R.copy(), np.zeros(3))]
    for _ in range(1, n_frames):
        heading = heading + rng.normal(0.0, 0.02, 3)
        heading /= np.linalg.norm(heading)
        C = C + step * heading
        axis = axis + rng.normal(0.0, 0.2, 3)
        R = _rodrigues(axis, math.radians(rng.uniform(0.0, max_turn_deg))) @ R
        poses.append((R.copy(), -R @ C))
    return poses


def _render_view(width, height, K, R, t, planes, tex):
    """Frame of the camera X' = R X + t (noise-free) and the scene point of
    every pixel in camera-0 coordinates (3, N) with its found mask."""
    Kinv = np.linalg.inv(K)
    ys, xs = np.mgrid[0:height, 0:width].astype(np.float64)
    X, found = _raycast(planes, K, Kinv, R, t, xs, ys)
    with np.errstate(divide="ignore", invalid="ignore"):
        px = K[0, 0] * X[0] / X[2] + K[0, 2]
        py = K[1, 1] * X[1] / X[2] + K[1, 2]
    px = np.where(found, px, xs.ravel())
    py = np.where(found, py, ys.ravel())
    return tex(px, py).reshape(height, width), X, found


def make_sequence(width: int, height: int, n_frames: int = 32, seed: int = 0, K=None,
                  n_planes: int = 8, n_blobs: int = 200, step: float = 0.05,
                  max_turn_deg: float = 0.3, noise: float = 0.01, device=None) -> dict:
    """One seeded scene (planes and texture as in make_scene) seen from
    `n_frames` cameras along smooth_path, rendered with numpy, or with torch
    (float64) on `device` (the same seeded parameters and formulas).

    Returns frames (float32, N(0, noise) added), poses [(R_k, t_k)] and, for
    each consecutive pair (k, k + 1), the ground truth in frame k's pixels:
    flow, inverse depth in camera k, a validity mask (the point is seen by
    camera k + 1: inside its image and not occluded), and the relative pose
    (R, t) mapping camera-k coordinates to camera k + 1's, which is what a
    solve with camera k at the identity takes.
    """
    rng = np.random.default_rng(seed)
    K = intrinsics_for(width, height) if K is None else np.asarray(K, np.float64)
    Kinv = np.linalg.inv(K)
    planes = _Planes(rng, width, height, K, n_planes)
    tex = _Texture(rng, width, height, n_blobs)
    gy, gx = np.mgrid[0:height:4, 0:width:4].astype(np.float64)
    raw = tex.raw(gx, gy)
    tex.lo, tex.hi = float(np.percentile(raw, 0.5)), float(np.percentile(raw, 99.5))
    poses = smooth_path(rng, n_frames, step, max_turn_deg)
    if device is not None:
        images, pairs = _sequence_torch(width, height, K, poses, planes, tex, device)
        frames = [(I + rng.normal(0.0, noise, I.shape)).astype(np.float32) for I in images]
        return {"frames": frames, "poses": poses, "pairs": pairs, "K": K, "seed": seed}
    views = [_render_view(width, height, K, R, t, planes, tex) for R, t in poses]
    frames = [(I + rng.normal(0.0, noise, I.shape)).astype(np.float32) for I, _, _ in views]
    ys, xs = np.mgrid[0:height, 0:width].astype(np.float64)
    pairs = []
    for k in range(n_frames - 1):
        (Ra, ta), (Rb, tb) = poses[k], poses[k + 1]
        _, X, found = views[k]
        Xa = Ra @ X + ta[:, None]
        Xb = Rb @ X + tb[:, None]
        with np.errstate(divide="ignore", invalid="ignore"):
            u1 = K[0, 0] * Xb[0] / Xb[2] + K[0, 2]
            v1 = K[1, 1] * Xb[1] / Xb[2] + K[1, 2]
            inv = np.where(found, 1.0 / Xa[2], 0.0)
        inb = found & (Xb[2] > 1e-6) & (u1 >= 0) & (u1 <= width - 1) & (v1 >= 0) & (v1 <= height - 1)
        Xv, fv = _raycast(planes, K, Kinv, Rb, tb, np.where(inb, u1, 0.0), np.where(inb, v1, 0.0))
        same = fv & (np.linalg.norm(Xv - X, axis=0) < 1e-3 * np.maximum(np.abs(Xa[2]), 1.0))
        flow = np.stack([np.where(found, u1 - xs.ravel(), 0.0).reshape(height, width),
                         np.where(found, v1 - ys.ravel(), 0.0).reshape(height, width)], -1)
        Rr = Rb @ Ra.T
        pairs.append({"flow": flow.astype(np.float32),
                      "inv_depth": inv.reshape(height, width).astype(np.float32),
                      "valid": (inb & same).reshape(height, width),
                      "R": Rr, "t": tb - Rr @ ta})
    return {"frames": frames, "poses": poses, "pairs": pairs, "K": K, "seed": seed}


# ---------------------------------------------------------------------------
# The same renderer on the GPU with torch (float64), for fast input generation
# ---------------------------------------------------------------------------

def _raw_torch(tex, x, y, device, chunk=16):
    import torch

    X = torch.as_tensor(np.asarray(x, np.float64).ravel(), device=device)
    Y = torch.as_tensor(np.asarray(y, np.float64).ravel(), device=device)
    out = torch.zeros_like(X)
    cx = torch.as_tensor(tex.cx, device=device)
    cy = torch.as_tensor(tex.cy, device=device)
    sig = torch.as_tensor(tex.sig, device=device)
    amp = torch.as_tensor(tex.amp, device=device)
    for i in range(0, len(tex.amp), chunk):
        dx = X[:, None] - cx[None, i:i + chunk]
        dy = Y[:, None] - cy[None, i:i + chunk]
        r = 4.0 * sig[None, i:i + chunk]
        inside = (dx.abs() < r) & (dy.abs() < r)
        val = amp[None, i:i + chunk] * torch.exp(-(dx * dx + dy * dy) / (2 * sig[None, i:i + chunk] ** 2))
        out += torch.where(inside, val, torch.zeros_like(val)).sum(1)
    kx = torch.as_tensor(tex.kx, device=device)
    ky = torch.as_tensor(tex.ky, device=device)
    ph = torch.as_tensor(tex.ph, device=device)
    wa = torch.as_tensor(tex.wamp, device=device)
    for i in range(len(tex.freq)):
        out += wa[i] * torch.cos(kx[i] * X + ky[i] * Y + ph[i])
    return out.cpu().numpy()


def _render_pair_torch(width, height, K, R, t, planes, tex, rng, noise, device):
    import torch

    dev = torch.device(device)
    T = lambda a: torch.as_tensor(np.asarray(a, np.float64), device=dev)  # noqa: E731
    Kt, Rt, tt = T(K), T(R), T(t)
    Kinv = T(np.linalg.inv(np.asarray(K, np.float64)))  # host inverse: no GPU LAPACK needed
    ys, xs = torch.meshgrid(torch.arange(height, device=dev, dtype=torch.float64),
                            torch.arange(width, device=dev, dtype=torch.float64), indexing="ij")
    xs, ys = xs.reshape(-1), ys.reshape(-1)
    seeds = T(planes.seeds)
    abc = T(planes.abc)
    nrm = T(planes.n)

    def label(x, y):
        d = (x[:, None] - seeds[None, :, 0]) ** 2 + (y[:, None] - seeds[None, :, 1]) ** 2
        return torch.argmin(d, dim=1)

    def texture(x, y):
        v = (torch.as_tensor(_raw_torch(tex, x.cpu().numpy(), y.cpu().numpy(), dev), device=dev)
             - tex.lo) / (tex.hi - tex.lo)
        return v.clamp(0.0, 1.0)

    def raycast(px, py):
        C = -Rt.T @ tt
        rays = torch.stack([px, py, torch.ones_like(px)], 0)
        d = Rt.T @ (Kinv @ rays)
        best = torch.full_like(px, float("inf"))
        hit = torch.zeros((3, px.numel()), dtype=torch.float64, device=dev)
        nC = nrm @ C
        nd = nrm @ d
        for k in range(nrm.shape[0]):
            lam = (1.0 - nC[k]) / nd[k]
            X = C[:, None] + lam[None, :] * d
            z = X[2]
            ok = (lam > 0) & (z > 1e-6) & torch.isfinite(lam)
            qx = torch.where(ok, Kt[0, 0] * X[0] / z + Kt[0, 2], torch.zeros_like(z))
            qy = torch.where(ok, Kt[1, 1] * X[1] / z + Kt[1, 2], torch.zeros_like(z))
            ok &= label(qx, qy) == k
            better = ok & (lam < best)
            best = torch.where(better, lam, best)
            hit[:, better] = X[:, better]
        return hit, torch.isfinite(best)

    k = label(xs, ys)
    inv_depth = abc[k, 0] + abc[k, 1] * xs + abc[k, 2] * ys
    Z = 1.0 / inv_depth
    I0 = texture(xs, ys)
    X, found = raycast(xs, ys)
    px = torch.where(found, Kt[0, 0] * X[0] / X[2] + Kt[0, 2], xs)
    py = torch.where(found, Kt[1, 1] * X[1] / X[2] + Kt[1, 2], ys)
    I1 = texture(px, py)
    P0 = torch.stack([xs * Z, ys * Z, Z], 0)
    X0 = Kinv @ P0
    X1 = Rt @ X0 + tt[:, None]
    u1 = Kt[0, 0] * X1[0] / X1[2] + Kt[0, 2]
    v1 = Kt[1, 1] * X1[1] / X1[2] + Kt[1, 2]
    inb = (u1 >= 0) & (u1 <= width - 1) & (v1 >= 0) & (v1 <= height - 1)
    Xv, fv = raycast(u1, v1)
    same = fv & (torch.sqrt(((Xv - X0) ** 2).sum(0)) < 1e-3 * torch.clamp(X0[2], min=1.0))
    valid = (inb & same).reshape(height, width)
    sh = (height, width)
    I0 = I0.reshape(sh).cpu().numpy() + rng.normal(0.0, noise, sh)
    I1 = I1.reshape(sh).cpu().numpy() + rng.normal(0.0, noise, sh)
    flow = torch.stack([(u1 - xs).reshape(sh), (v1 - ys).reshape(sh)], -1)
    return {
        "I0": I0.astype(np.float32), "I1": I1.astype(np.float32),
        "flow": flow.cpu().numpy().astype(np.float32),
        "inv_depth": inv_depth.reshape(sh).cpu().numpy().astype(np.float32),
        "depth": Z.reshape(sh).cpu().numpy().astype(np.float32), "valid": valid.cpu().numpy(),
    }


def _sequence_torch(width, height, K, poses, planes, tex, device):
    """The views and per-pair ground truth of make_sequence with torch
    (float64) on `device`: the same ray casts and projections as the numpy
    path, frame after frame."""
    import torch

    dev = torch.device(device)
    T = lambda a: torch.as_tensor(np.asarray(a, np.float64), device=dev)  # noqa: E731
    Kt = T(K)
    Kinv = T(np.linalg.inv(np.asarray(K, np.float64)))
    fx, fy, cx, cy = float(K[0, 0]), float(K[1, 1]), float(K[0, 2]), float(K[1, 2])
    ys, xs = torch.meshgrid(torch.arange(height, device=dev, dtype=torch.float64),
                            torch.arange(width, device=dev, dtype=torch.float64), indexing="ij")
    xs, ys = xs.reshape(-1), ys.reshape(-1)
    seeds = T(planes.seeds)
    nrm = T(planes.n)

    def label(x, y):
        d = (x[:, None] - seeds[None, :, 0]) ** 2 + (y[:, None] - seeds[None, :, 1]) ** 2
        return torch.argmin(d, dim=1)

    def texture(x, y):
        v = (torch.as_tensor(_raw_torch(tex, x.cpu().numpy(), y.cpu().numpy(), dev), device=dev)
             - tex.lo) / (tex.hi - tex.lo)
        return v.clamp(0.0, 1.0)

    def raycast(Rt, tt, px, py):
        C = -Rt.T @ tt
        d = Rt.T @ (Kinv @ torch.stack([px, py, torch.ones_like(px)], 0))
        best = torch.full_like(px, float("inf"))
        hit = torch.zeros((3, px.numel()), dtype=torch.float64, device=dev)
        nC = nrm @ C
        nd = nrm @ d
        for k in range(nrm.shape[0]):
            lam = (1.0 - nC[k]) / nd[k]
            X = C[:, None] + lam[None, :] * d
            z = X[2]
            ok = (lam > 0) & (z > 1e-6) & torch.isfinite(lam)
            qx = torch.where(ok, fx * X[0] / z + cx, torch.zeros_like(z))
            qy = torch.where(ok, fy * X[1] / z + cy, torch.zeros_like(z))
            ok &= label(qx, qy) == k
            better = ok & (lam < best)
            best = torch.where(better, lam, best)
            hit[:, better] = X[:, better]
        return hit, torch.isfinite(best)

    sh = (height, width)
    views = []
    for R, t in poses:
        X, found = raycast(T(R), T(t), xs, ys)
        px = torch.where(found, fx * X[0] / X[2] + cx, xs)
        py = torch.where(found, fy * X[1] / X[2] + cy, ys)
        views.append((texture(px, py).reshape(sh).cpu().numpy(), X, found))
    pairs = []
    for k in range(len(poses) - 1):
        (Ra, ta), (Rb, tb) = poses[k], poses[k + 1]
        _, X, found = views[k]
        Xa = T(Ra) @ X + T(ta)[:, None]
        Xb = T(Rb) @ X + T(tb)[:, None]
        u1 = fx * Xb[0] / Xb[2] + cx
        v1 = fy * Xb[1] / Xb[2] + cy
        inv = torch.where(found, 1.0 / Xa[2], torch.zeros_like(Xa[2]))
        inb = (found & (Xb[2] > 1e-6) & (u1 >= 0) & (u1 <= width - 1) & (v1 >= 0)
               & (v1 <= height - 1))
        zero = torch.zeros_like(u1)
        Xv, fv = raycast(T(Rb), T(tb), torch.where(inb, u1, zero), torch.where(inb, v1, zero))
        same = fv & (torch.sqrt(((Xv - X) ** 2).sum(0))
                     < 1e-3 * torch.clamp(Xa[2].abs(), min=1.0))
        flow = torch.stack([torch.where(found, u1 - xs, zero).reshape(sh),
                            torch.where(found, v1 - ys, zero).reshape(sh)], -1)
        Rr = Rb @ Ra.T
        pairs.append({"flow": flow.cpu().numpy().astype(np.float32),
                      "inv_depth": inv.reshape(sh).cpu().numpy().astype(np.float32),
                      "valid": (inb & same).reshape(sh).cpu().numpy(),
                      "R": Rr, "t": tb - Rr @ ta})
    return [v[0] for v in views], pairs
