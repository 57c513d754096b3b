"""The reference's demo pipeline on this library.

``test_reconflow/main.cpp`` reads two RGB frames (PNG), a ``.flo`` prior flow
and a KITTI ``calib.txt``; picks the pyramid depth from a minimum size
(``:45-53``); runs ReconFlow with the sparse prior-flow data term
(``METHODR_TVL1_MS_FNSPARSE``, ``:72-76``) against R = I, t = (-1, 1e-5,
1e-5); and writes the 3D points as a coloured PLY (``:106-139``).  ``run``
does the same with this library's C ABI and the file formats of
``reconflow_gb300.io``, and also writes the flow (``.flo``) and its colour
coding (PNG).  It needs the CUDA library; there is no CPU path.

    python -m reconflow_gb300.demo --data DIR --out DIR [--iters N]
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from . import io as rio
from .reconflow import CV_8UC3, ReconFlow

# the demo's parameters (main.cpp:27-40)
DEMO = dict(lambda_=50.0, tau=0.125, alphaTv=33.3, alphaFn=100.0, alphaProj=60.0, lambdaf=0.1,
            lambdams=100.0, nWarpIters=1, iters=10000, scale=2.0, minWidth=400)


def pyramid_levels(height: int, scale: float, min_width: int) -> int:
    """main.cpp:47-53: add levels while the (float-divided, truncated)
    height stays above min_width."""
    n = 1
    ph = int(float(height) / scale)
    while ph > min_width:
        n += 1
        ph = int(float(ph) / scale)
    return n


def run(i0, i1, prior, K, R, t, iters=DEMO["iters"], n_warps=DEMO["nWarpIters"], n_levels=None,
        params=None, flow_scale=50.0):
    """Solve one RGB8 pair (H, W, 3) with the prior flow (H, W, 2).
    Returns dict(u, v, X, Y, Z, color) cropped to (H, W)."""
    p = dict(DEMO)
    p.update(params or {})
    h, w = i0.shape[:2]
    if n_levels is None:
        n_levels = pyramid_levels(h, p["scale"], p["minWidth"])
    f = ReconFlow(32, 12, 32)
    try:
        f.initializeR(w, h, 3, n_levels, p["scale"], ReconFlow.METHODR_TVL1_MS_FNSPARSE,
                      p["lambda_"], 0.0, p["lambdaf"], p["lambdams"], p["alphaTv"], p["alphaProj"],
                      p["alphaFn"], p["tau"], n_warps, iters, cvType=CV_8UC3)
        f.setCameraMatrices(K, K)
        s = f.iAlignUp(w)
        padc = lambda a: np.pad(a, ((0, 0), (0, s - w)) + ((0, 0),) * (a.ndim - 2))  # noqa: E731
        f.copyImagesToDevice(padc(np.ascontiguousarray(i0, np.uint8)),
                             padc(np.ascontiguousarray(i1, np.uint8)))
        f.copySparseOpticalFlowToDevice(padc(prior[..., 0].astype(np.float32)),
                                        padc(prior[..., 1].astype(np.float32)))
        f.solveR(R, t, flow_scale)
        u, v = f.copyOpticalFlowToHost()
        color = f.copyFlowColorToHost(flow_scale)
        X, Y, Z = f.copy3dToHost()
    finally:
        f.close()
    crop = lambda a: a[:, :w]  # noqa: E731
    return dict(u=crop(u), v=crop(v), X=crop(X), Y=crop(Y), Z=crop(Z), color=crop(color))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--data", required=True, help="folder with im319.png, im318.png, "
                    "flo319.flo and calib.txt (the reference demo's names)")
    ap.add_argument("--out", required=True)
    ap.add_argument("--iters", type=int, default=DEMO["iters"])
    ap.add_argument("--im0", default="im319.png")
    ap.add_argument("--im1", default="im318.png")
    ap.add_argument("--flo", default="flo319.flo")
    ap.add_argument("--calib", default="calib.txt")
    a = ap.parse_args(argv)
    i0 = rio.read_png(os.path.join(a.data, a.im0))
    i1 = rio.read_png(os.path.join(a.data, a.im1))
    prior = rio.read_flo(os.path.join(a.data, a.flo))
    K, R, t = rio.demo_camera(os.path.join(a.data, a.calib))
    res = run(i0, i1, prior, K, R, t, iters=a.iters)
    os.makedirs(a.out, exist_ok=True)
    pts, cols = rio.demo_cloud(res["X"], res["Y"], res["Z"], i0)
    rio.write_ply(os.path.join(a.out, "output3doursfn.ply"), pts, cols)
    rio.write_flo(os.path.join(a.out, "flow.flo"), np.stack([res["u"], res["v"]], -1))
    rgb = (np.clip(res["color"][..., ::-1], 0, 1) * 255 + 0.5).astype(np.uint8)
    rio.write_png(os.path.join(a.out, "flow_color.png"), rgb, filters=1)
    n_ok = int(np.isfinite(pts).all(axis=1).sum())
    print(f"wrote {a.out}: {n_ok} of {len(pts)} points kept")


if __name__ == "__main__":
    main()
