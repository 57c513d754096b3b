"""Numpy restatement of the temporal warm start for frame sequences (test
infrastructure only: the reference for a device kernel, never called by the
product path).

Frame k's coarse inverse-depth grid from frame k-1's solution: every pixel
of frame k-1 with a finite positive inverse depth is lifted to 3D (camera
k-1 coordinates, X = z K^-1 [x, y, 1]), moved by the relative pose
(X' = R X + t, camera k-1 -> camera k), projected into frame k and binned
into the cell of the `factor`-times-coarser grid it lands in; each cell
keeps the nearest point (largest inverse depth), as a z-buffer does.  Cells
no point reaches take the median of the filled cells (the network's
fallback value for an empty view).
"""
from __future__ import annotations

import numpy as np


def propagate_inv_depth(inv_depth, K, R, t, factor, out_shape=None):
    """inv_depth: (h, w) of frame k-1 (0 or non-finite = unknown); K: 3x3;
    R, t: camera k-1 -> camera k; returns (grid (hc, wc) float64, filled
    mask) for frame k, hc = ceil(h / factor), wc = ceil(w / factor) unless
    out_shape is given."""
    h, w = inv_depth.shape
    hc, wc = out_shape if out_shape is not None else (-(-h // factor), -(-w // factor))
    rho = np.asarray(inv_depth, np.float64)
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    ok = np.isfinite(rho) & (rho > 0)
    z = 1.0 / rho[ok]
    Kinv = np.linalg.inv(K)
    P = Kinv @ np.stack([xs[ok] * z, ys[ok] * z, z])
    Q = np.asarray(R, np.float64) @ P + np.asarray(t, np.float64)[:, None]
    front = Q[2] > 1e-6
    Q = Q[:, front]
    u = K[0, 0] * Q[0] / Q[2] + K[0, 2]
    v = K[1, 1] * Q[1] / Q[2] + K[1, 2]
    cx = np.floor(u / factor).astype(np.int64)
    cy = np.floor(v / factor).astype(np.int64)
    inside = (cx >= 0) & (cx < wc) & (cy >= 0) & (cy < hc)
    cell = cy[inside] * wc + cx[inside]
    val = 1.0 / Q[2][inside]
    grid = np.full(hc * wc, -np.inf)
    np.maximum.at(grid, cell, val)
    filled = np.isfinite(grid)
    if filled.any():
        grid[~filled] = np.median(grid[filled])
    else:
        grid[:] = 0.0
    return grid.reshape(hc, wc), filled.reshape(hc, wc)


def propagate_depth_f32(Z, K, R, t, factor, out_shape):
    """Float32 restatement of ``rf_ws_propagate``: Z (h, w) float32 depth of
    frame k-1 (non-finite or <= 0 = unknown); K, R, t as above (cast to
    float32); returns the (hc, wc) float32 grid of per-cell mean inverse
    depths of the points landing at 0.5 .. 50 m, summed in fixed point
    (2^-16 1/m), empty cells at the median of the filled ones.  Every
    floating-point operation is one float32 rounding in the kernel's order."""
    f32 = np.float32
    Z = np.asarray(Z, f32)
    h, w = Z.shape
    hc, wc = out_shape
    fx, fy, cx, cy = (f32(K[0][0]), f32(K[1][1]), f32(K[0][2]), f32(K[1][2]))
    Rf = np.asarray(R, np.float64).astype(f32).ravel()
    tf = np.asarray(t, np.float64).astype(f32).ravel()
    ys, xs = np.mgrid[0:h, 0:w]
    with np.errstate(invalid="ignore"):
        ok = np.isfinite(Z) & (Z > 0)
    z = Z[ok]
    x = xs[ok].astype(f32)
    y = ys[ok].astype(f32)
    X = ((x - cx) * z) / fx
    Y = ((y - cy) * z) / fy
    Q = [((Rf[3 * r] * X + Rf[3 * r + 1] * Y) + Rf[3 * r + 2] * z) + tf[r] for r in range(3)]
    keep = (Q[2] >= f32(0.5)) & (Q[2] <= f32(50.0))
    Q0, Q1, Q2 = (q[keep] for q in Q)
    u = (fx * Q0) / Q2 + cx
    v = (fy * Q1) / Q2 + cy
    fu = np.floor(u / f32(factor))
    fv = np.floor(v / f32(factor))
    inside = (fu >= 0) & (fu < wc) & (fv >= 0) & (fv < hc)
    cell = fv[inside].astype(np.int64) * wc + fu[inside].astype(np.int64)
    q = np.rint((f32(1.0) / Q2[inside]) * f32(65536.0)).astype(np.int64)
    sums = np.zeros(hc * wc, np.int64)
    np.add.at(sums, cell, q)
    cnt = np.bincount(cell, minlength=hc * wc)
    filled = cnt > 0
    grid = np.zeros(hc * wc, f32)
    grid[filled] = (sums[filled].astype(np.float64) / cnt[filled].astype(np.float64)
                    / 65536.0).astype(f32)
    if filled.any():
        vals = np.sort(grid[filled])
        n = vals.size
        med = vals[(n - 1) // 2] if n % 2 else (vals[n // 2 - 1] + vals[n // 2]) * f32(0.5)
        grid[~filled] = med
    return grid.reshape(hc, wc)
