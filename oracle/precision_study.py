"""FP32 against FP64: how far the reference's arithmetic in FP32 sits from the
same schedule in FP64, by schedule length (test infrastructure; CPU only).

The library's CUDA path equals the FP32 oracle bit for bit (the GPU tests),
and the FP32 oracle's kernels equal the reference's own kernels built
without contraction, so the FP32 column here is the library's deviation from
the FP64 oracle.  Workload: the 640x480 scene (seed 0) with the bench's
solver weights (lambda 50, alpha_tv 1/0.33, tau 0.25, alpha_proj 60,
lambdaf 0.1, lambdams 100, K-pyramid fix).  Valid pixels: the scene's
non-occluded pixels where both results are finite; depth is compared where
the FP64 depth lies in 0.5-50 m.

Sections:
1. cold start (the reference's schedule from zero flow and points), five
   levels, by iterations at one warp and by warps at 50 iterations;
2. cold start at one level, with the step where the gap opens: the points
   solved at near-zero disparity, and the pixels where the two precisions
   take different branches of the ``isfinite`` clean-up (a point set to the
   origin, whose projection uc then enters uproj);
3. warm start at level 0 from the ground truth (the learned path's regime);
4. the plain TV-L1 sub-mode (method 0, no 3D step), five levels.

Run: ``python oracle/precision_study.py`` (a few minutes on 8 cores); it
prints markdown tables.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a file, the script's own folder would shadow the ``oracle`` package
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402

W, H, LEVELS = 640, 480, 5
WEIGHTS = dict(lam=50.0, lambdaf=0.1, lambdams=100.0, alpha_tv=1 / 0.33, alpha_proj=60.0,
               tau=0.25, fix_quirks=1)


def scene():
    from reconflow_gb300.scene import make_scene

    return make_scene(W, H, seed=0)


def params(warps, iters, levels=LEVELS, method=14):
    return O.make_params(W, H, levels, method=method, n_warp_iters=warps, n_solver_iters=iters,
                         **WEIGHTS)


def deviation(a, b, valid):
    """Largest |flow32 - flow64| (px), the share above 1e-3 px, and the
    relative depth deviation (max, median, share above 1e-4)."""
    u32, v32 = (a[k][:, :W].astype(np.float64) for k in ("u", "v"))
    u64, v64 = (b[k][:, :W].astype(np.float64) for k in ("u", "v"))
    m = valid & np.isfinite(u32) & np.isfinite(v32) & np.isfinite(u64) & np.isfinite(v64)
    df = np.maximum(np.abs(u32 - u64), np.abs(v32 - v64))[m]
    out = dict(flow_max=float(df.max()), flow_frac=float((df > 1e-3).mean()))
    if "Z" in a:
        z32, z64 = a["Z"][:, :W].astype(np.float64), b["Z"][:, :W].astype(np.float64)
        mz = m & np.isfinite(z32) & np.isfinite(z64) & (z64 > 0.5) & (z64 < 50)
        dz = np.abs(z32 - z64)[mz] / z64[mz]
        out.update(depth_max=float(dz.max()), depth_med=float(np.median(dz)),
                   depth_frac=float((dz > 1e-4).mean()))
    return out


def row(label, d):
    s = f"| {label} | {d['flow_max']:.2e} | {100 * d['flow_frac']:.2f}% |"
    if "depth_max" in d:
        s += f" {d['depth_max']:.2e} | {d['depth_med']:.1e} | {100 * d['depth_frac']:.1f}% |"
    else:
        s += " - | - | - |"
    return s


HEADER = ("| schedule | flow max-abs (px) | flow > 1e-3 px | depth max rel | depth median rel "
          "| depth > 1e-4 |\n|---|---|---|---|---|---|")


def cold(sc, warps, iters, levels=LEVELS, method=14):
    p = params(warps, iters, levels, method)
    kw = {} if method == 0 else dict(K0=sc["K"], K1=sc["K"], R1=sc["R"], t1=sc["t"])
    return [O.solve(p, sc["I0"].astype(np.float32), sc["I1"].astype(np.float32), dtype=dt, **kw)
            for dt in (np.float32, np.float64)]


def warm_from_truth(sc, iters):
    K = sc["K"]
    Z = sc["depth"]
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    X = (x - K[0, 2]) * Z / K[0, 0]
    Y = (y - K[1, 2]) * Z / K[1, 1]
    planes = [sc["flow"][..., 0], sc["flow"][..., 1], X, Y, Z]
    p = params(1, iters)
    return [O.solve_warm(p, sc["I0"], sc["I1"], 0, *planes, 1, iters, K0=K, K1=K, R1=sc["R"],
                         t1=sc["t"], dtype=dt) for dt in (np.float32, np.float64)]


def first_iteration_branches(sc):
    """One inner iteration at level 0 from the cold start, kernel by kernel in
    both precisions: the disparity the point solve sees, and the pixels whose
    clean-up branch differs between FP32 and FP64."""
    s = W
    n = (H + 1) * s
    K, R1, t1 = sc["K"], sc["R"], sc["t"]
    Pd = O.camera_matrix(K, np.eye(3), np.zeros(3)).ravel()
    Qd = O.camera_matrix(K, R1, t1).ravel()
    i0 = np.zeros(n)
    i1 = np.zeros(n)
    i0[:H * s] = sc["I0"].ravel()
    i1[:H * s] = sc["I1"].ravel()
    res = {}
    for dt in (np.float32, np.float64):
        z = lambda: np.zeros(n, dt)  # noqa: E731
        u, v, up, vp, uc, vc, X, Y, Z, sku, skv, du, dv = (z() for _ in range(13))
        p = [z() for _ in range(4)]
        Ix, Iy, Iz = O.derivatives(i0.astype(dt), O.warp(i1.astype(dt), W, H, s, u, v), W, H, s)
        du, dv = O.recon_data_l1(u, v, du, dv, up, vp, sku, skv, *p, Ix, Iy, Iz, W, H, s,
                                 WEIGHTS["lam"], WEIGHTS["alpha_tv"], WEIGHTS["alpha_proj"])
        up, vp = O.uv_proj(u, v, du, dv, uc, vc, sku, skv, W, H, s, WEIGHTS["lambdaf"],
                           WEIGHTS["alpha_proj"])
        P = Pd.astype(np.float32).astype(dt)
        Q = Qd.astype(np.float32).astype(dt)
        Xs, Ys, Zs = O.solve3d(up, vp, X, Y, Z, P, Q, WEIGHTS["lambdaf"], WEIGHTS["lambdams"],
                               W, H, s)
        Xm, Ym, Zm = O.median3d(Xs, Ys, Zs, W, H, s)
        Xc, Yc, Zc = O.cleanup3d(Xs, Ys, Zs, Xm, Ym, Zm, W, H, s)
        res[dt] = dict(uproj=up, Z=Zs, zeroed=(Xc == 0) & (Yc == 0) & (Zc == 0))
    m = lambda a: a.reshape(H + 1, s)[:H, :W]  # noqa: E731
    disp = np.abs(m(res[np.float64]["uproj"]))
    z32, z64 = m(res[np.float32]["Z"]).astype(np.float64), m(res[np.float64]["Z"])
    fin = np.isfinite(z32) & np.isfinite(z64)
    zero_diff = m(res[np.float32]["zeroed"]) != m(res[np.float64]["zeroed"])
    return dict(disp_median=float(np.median(disp)),
                depth_rel_median=float(np.median(np.abs(z32 - z64)[fin] / np.abs(z64[fin]))),
                cleanup_branch_differs=int(zero_diff.sum()))


def main():
    sc = scene()
    valid = sc["valid"]
    print("### 1. Cold start (the reference's schedule), 5 levels\n")
    print(HEADER)
    for warps, iters in [(1, 1), (1, 2), (1, 5), (1, 10), (1, 20), (1, 50), (2, 50), (3, 50)]:
        print(row(f"{warps} warp x {iters}", deviation(*cold(sc, warps, iters), valid)),
              flush=True)
    print("\n### 2. Cold start, one level\n")
    print(HEADER)
    for iters in (1, 2, 5):
        print(row(f"level 0 only, 1 warp x {iters}", deviation(*cold(sc, 1, iters, 1), valid)),
              flush=True)
    b = first_iteration_branches(sc)
    print(f"\nfirst iteration at level 0: median |uproj| {b['disp_median']:.3g} px; median "
          f"relative gap of the solved depth {b['depth_rel_median']:.2g}; clean-up branch "
          f"differs at {b['cleanup_branch_differs']} pixels")
    print("\n### 3. Warm start at level 0 from the ground truth\n")
    print(HEADER)
    for iters in (1, 5, 20, 100):
        print(row(f"1 warp x {iters}", deviation(*warm_from_truth(sc, iters), valid)),
              flush=True)
    print("\n### 4. Plain TV-L1 (method 0), 5 levels\n")
    print(HEADER)
    for warps, iters in [(1, 5), (1, 20), (1, 50), (3, 50)]:
        print(row(f"{warps} warp x {iters}", deviation(*cold(sc, warps, iters, method=0),
                                                       valid)), flush=True)


if __name__ == "__main__":
    main()
