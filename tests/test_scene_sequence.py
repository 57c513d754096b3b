"""The sequence generator (scene.make_sequence): one seeded scene along a
smooth camera path of 0.05 m per frame, with ground truth per consecutive
pair.  CPU only: the path's geometry, the ground truth's consistency with
the relative pose and inverse depth, and the photometric consistency of the
noise-free frames under the ground-truth flow."""
import math

import numpy as np

from reconflow_gb300 import scene as S


def _bilinear(I, x, y):
    h, w = I.shape
    x0 = np.clip(np.floor(x).astype(int), 0, w - 2)
    y0 = np.clip(np.floor(y).astype(int), 0, h - 2)
    fx, fy = x - x0, y - y0
    return ((1 - fy) * ((1 - fx) * I[y0, x0] + fx * I[y0, x0 + 1])
            + fy * ((1 - fx) * I[y0 + 1, x0] + fx * I[y0 + 1, x0 + 1]))


def test_smooth_path_steps_and_turns():
    poses = S.smooth_path(np.random.default_rng(1), 32, step=0.05, max_turn_deg=0.3)
    assert len(poses) == 32
    assert np.array_equal(poses[0][0], np.eye(3)) and np.array_equal(poses[0][1], np.zeros(3))
    centres = [-R.T @ t for R, t in poses]
    for k in range(31):
        (Ra, _), (Rb, _) = poses[k], poses[k + 1]
        assert math.isclose(np.linalg.norm(centres[k + 1] - centres[k]), 0.05, rel_tol=1e-9)
        turn = math.degrees(math.acos(min(1.0, (np.trace(Rb @ Ra.T) - 1) / 2)))
        assert turn <= 0.3 + 1e-9
        assert np.allclose(Rb @ Rb.T, np.eye(3), atol=1e-12)
    # mostly forward: every heading within 45 degrees of camera 0's axis
    for k in range(31):
        d = centres[k + 1] - centres[k]
        assert d[2] / np.linalg.norm(d) > math.cos(math.radians(45))


def test_sequence_ground_truth_matches_pose_and_depth():
    q = S.make_sequence(96, 72, 5, seed=3)
    K = q["K"]
    Kinv = np.linalg.inv(K)
    ys, xs = np.mgrid[0:72, 0:96].astype(np.float64)
    assert len(q["frames"]) == 5 and len(q["pairs"]) == 4
    for k, p in enumerate(q["pairs"]):
        v = p["valid"]
        assert v.mean() > 0.8
        # the relative pose is camera k -> camera k + 1
        (Ra, ta), (Rb, tb) = q["poses"][k], q["poses"][k + 1]
        assert np.allclose(p["R"] @ Ra, Rb) and np.allclose(p["R"] @ ta + p["t"], tb)
        # back-project with the inverse depth, move, project: the flow
        z = 1.0 / p["inv_depth"][v].astype(np.float64)
        P = Kinv @ np.stack([xs[v] * z, ys[v] * z, z])
        P1 = p["R"] @ P + p["t"][:, None]
        u = K[0, 0] * P1[0] / P1[2] + K[0, 2] - xs[v]
        w = K[1, 1] * P1[1] / P1[2] + K[1, 2] - ys[v]
        assert np.max(np.abs(u - p["flow"][..., 0][v])) < 1e-3
        assert np.max(np.abs(w - p["flow"][..., 1][v])) < 1e-3


def test_sequence_frames_agree_under_ground_truth_flow():
    q = S.make_sequence(160, 120, 4, seed=4, noise=0.0)
    ys, xs = np.mgrid[0:120, 0:160].astype(np.float64)
    for k, p in enumerate(q["pairs"]):
        v = p["valid"]
        warped = _bilinear(q["frames"][k + 1], xs + p["flow"][..., 0], ys + p["flow"][..., 1])
        err = np.abs(warped - q["frames"][k])[v]
        assert np.median(err) < 0.005 and np.percentile(err, 95) < 0.02


def test_sequence_is_seeded():
    a = S.make_sequence(64, 48, 3, seed=9)
    b = S.make_sequence(64, 48, 3, seed=9)
    c = S.make_sequence(64, 48, 3, seed=10)
    assert all(np.array_equal(x, y) for x, y in zip(a["frames"], b["frames"]))
    assert not np.array_equal(a["frames"][1], c["frames"][1])


def test_sequence_torch_renderer_matches_numpy():
    """The torch renderer (run here on the CPU; on a GPU it renders the
    full-size streams) gives the numpy path's frames and ground truth."""
    import pytest

    pytest.importorskip("torch")
    a = S.make_sequence(80, 60, 3, seed=5)
    b = S.make_sequence(80, 60, 3, seed=5, device="cpu")
    for x, y in zip(a["frames"], b["frames"]):
        assert np.allclose(x, y, atol=1e-6)
    for p, q in zip(a["pairs"], b["pairs"]):
        assert (p["valid"] == q["valid"]).mean() > 0.999
        both = p["valid"] & q["valid"]
        assert np.allclose(p["flow"][both], q["flow"][both], atol=1e-5)
        assert np.allclose(p["inv_depth"], q["inv_depth"], atol=1e-6)
        assert np.array_equal(p["R"], q["R"]) and np.array_equal(p["t"], q["t"])
