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
