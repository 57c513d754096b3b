"""Regenerate the oracle's regression fixtures (tests/golden/oracle_cases.npz).

The reference ships no golden outputs and cannot be built here, so these
fixtures pin the oracle's own results: seeded inputs and the FP32 and FP64
oracle outputs of three small cases (a ReconFlow solve, a plain TV-L1 solve,
and the 5x5 median on values with ties, signed zeros and NaN).  A change to
the oracle's arithmetic shows up as a fixture mismatch; rerun this script
only for a deliberate change, and say why in the commit.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def cases():
    """Seeded inputs of every case (shared with tests/test_golden.py)."""
    rng = np.random.default_rng(2024)
    w, h, s = 45, 30, 64
    y, x = np.mgrid[0:h, 0:s].astype(np.float64)
    I0 = 0.5 + 0.2 * np.sin(0.37 * x + 0.11 * y) + 0.15 * np.cos(0.09 * x - 0.29 * y)
    I0 = (I0 + rng.normal(0, 0.01, I0.shape)).astype(np.float32)
    I1 = np.roll(I0, 1, axis=1) + rng.normal(0, 0.005, I0.shape).astype(np.float32)
    I0[:, w:] = 0
    I1[:, w:] = 0
    K = np.array([[40.0, 0, 22.0], [0, 40.0, 15.0], [0, 0, 1]])
    c, sn = np.cos(0.01), np.sin(0.01)
    R = np.array([[c, 0, sn], [0, 1, 0], [-sn, 0, c]])
    t = np.array([-0.1, 0.01, 0.02])
    med = rng.integers(-3, 4, (21, 32)).astype(np.float32) * 0.5
    med[rng.random(med.shape) < 0.1] = -0.0
    med[3, 5] = np.nan
    med2 = rng.normal(size=(21, 32)).astype(np.float32)
    return dict(w=w, h=h, s=s, I0=I0.astype(np.float32), I1=I1.astype(np.float32), K=K, R=R,
                t=t, med_u=med, med_v=med2)


RECON = dict(lam=50.0, lambdaf=0.1, lambdams=100.0, alpha_tv=1 / 0.33, alpha_proj=60.0, tau=0.25,
             n_warp_iters=2, n_solver_iters=6, fix_quirks=1)
PLAIN = dict(lam=50.0, theta=0.33, tau=0.25, n_warp_iters=2, n_solver_iters=8)


def run(O, c):
    out = {}
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        p = O.make_params(c["w"], c["h"], 2, **RECON)
        r = O.solve(p, c["I0"], c["I1"], K0=c["K"], K1=c["K"], R1=c["R"], t1=c["t"], dtype=dt)
        for k in ("u", "v", "X", "Y", "Z"):
            out[f"recon_{k}_{tag}"] = r[k]
        p = O.make_params(c["w"], c["h"], 2, method=O.METHOD_TVL1, **PLAIN)
        r = O.solve(p, c["I0"], c["I1"], dtype=dt)
        out[f"plain_u_{tag}"], out[f"plain_v_{tag}"] = r["u"], r["v"]
    mu, mv = O.median5(c["med_u"].ravel(), c["med_v"].ravel(), 27, 20, 32)
    out["median5_u"], out["median5_v"] = mu.reshape(21, 32), mv.reshape(21, 32)
    return out


def main():
    from oracle import oracle as O

    O.build()
    c = cases()
    out = run(O, c)
    path = os.path.join(HERE, "oracle_cases.npz")
    np.savez_compressed(path, **{k: v for k, v in c.items() if isinstance(v, np.ndarray)}, **out)
    print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
