"""The temporal warm start's numpy reference (oracle/temporal_oracle.py)
against the sequence generator's ground truth: frame k-1's true inverse
depth, carried into frame k by the true relative pose, reproduces frame k's
true inverse depth on its coarse grid."""
import numpy as np

from oracle import temporal_oracle as TO
from reconflow_gb300 import scene as S


def _coarse_truth(inv, valid, f):
    h, w = inv.shape
    hc, wc = -(-h // f), -(-w // f)
    out = np.full((hc, wc), np.nan)
    for cy in range(hc):
        for cx in range(wc):
            blk = inv[cy * f:(cy + 1) * f, cx * f:(cx + 1) * f]
            m = valid[cy * f:(cy + 1) * f, cx * f:(cx + 1) * f]
            if m.any():
                out[cy, cx] = blk[m].max()  # the nearest surface in the cell
    return out


def test_propagated_inverse_depth_matches_the_next_frame():
    q = S.make_sequence(160, 120, 4, seed=6)
    f = 8
    for k in range(1, 3):
        prev, cur = q["pairs"][k - 1], q["pairs"][k]
        rho_prev = np.where(prev["valid"], prev["inv_depth"], 0.0)
        grid, filled = TO.propagate_inv_depth(rho_prev, q["K"], prev["R"], prev["t"], f)
        truth = _coarse_truth(cur["inv_depth"], cur["valid"], f)
        both = filled & np.isfinite(truth)
        assert filled.mean() > 0.9 and both.mean() > 0.85
        rel = np.abs(grid[both] - truth[both]) / truth[both]
        # cells on a depth edge may mix surfaces; the rest agree closely
        assert np.median(rel) < 0.005 and np.mean(rel < 0.05) > 0.97


def test_empty_and_behind_camera_inputs():
    K = S.intrinsics_for(64, 48)
    g, m = TO.propagate_inv_depth(np.zeros((48, 64)), K, np.eye(3), np.zeros(3), 8)
    assert g.shape == (6, 8) and not m.any() and np.all(g == 0.0)
    # everything moved behind the camera: nothing lands
    g, m = TO.propagate_inv_depth(np.full((48, 64), 0.5), K, np.eye(3), np.array([0, 0, -5.0]), 8)
    assert not m.any()
    # a pure translation along the axis scales the inverse depth exactly
    g, m = TO.propagate_inv_depth(np.full((48, 64), 0.25), K, np.eye(3), np.array([0, 0, -1.0]), 8)
    assert m.any() and np.allclose(g[m], 1.0 / 3.0)


def test_float32_mean_carry_matches_the_next_frame():
    """propagate_depth_f32 (the device kernel's restatement: the mean
    inverse depth of the points landing in a cell) carries frame k-1's true
    depth into frame k's true box-mean inverse depth."""
    q = S.make_sequence(160, 120, 3, seed=9)
    f = 8
    prev, cur = q["pairs"][0], q["pairs"][1]
    with np.errstate(divide="ignore"):
        Z = np.where(prev["valid"], 1.0 / prev["inv_depth"], np.nan).astype(np.float32)
    hc, wc = 120 // f, 160 // f
    grid = TO.propagate_depth_f32(Z, q["K"], prev["R"], prev["t"], f, (hc, wc))
    assert grid.dtype == np.float32 and grid.shape == (hc, wc)
    inv = np.where(cur["valid"], cur["inv_depth"], np.nan)[:hc * f, :wc * f]
    with np.errstate(invalid="ignore"):
        truth = np.nanmean(inv.reshape(hc, f, wc, f), axis=(1, 3))
    ok = np.isfinite(truth)
    rel = np.abs(grid[ok] - truth[ok]) / truth[ok]
    assert np.median(rel) < 0.01 and np.mean(rel < 0.05) > 0.9
    # unknown depth everywhere: all zeros
    empty = TO.propagate_depth_f32(np.full((120, 160), np.nan, np.float32), q["K"], prev["R"],
                                   prev["t"], f, (hc, wc))
    assert np.all(empty == 0.0)
