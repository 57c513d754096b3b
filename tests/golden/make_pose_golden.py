"""Regenerate the pose oracle's regression fixtures (tests/golden/pose_cases.npz).

The reference's pose front end is OpenCV code that is not part of its tree,
so these fixtures pin the oracle's own feature stages (pose_oracle.cpp): two
seeded 8-bit frames (Gaussian blobs on a ramp, the second moved by a
sub-pixel shift and a small rotation), their keypoints and descriptors, and
the nearest-neighbour matches between them.  A change to the oracle's
arithmetic shows up as a fixture mismatch; rerun this script only for a
deliberate change, and say why in the commit.

    python tests/golden/make_pose_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

THRESHOLD = 10.0


def frames():
    rng = np.random.default_rng(77)
    h, w = 120, 160
    cx, cy = rng.uniform(8, w - 8, 60), rng.uniform(8, h - 8, 60)
    sig = rng.uniform(1.5, 5.0, 60)
    amp = rng.uniform(-0.4, 0.4, 60)

    def render(dx, dy, ang):
        y, x = np.mgrid[0:h, 0:w].astype(np.float64)
        c, s = np.cos(ang), np.sin(ang)
        xs = c * (x - w / 2) + s * (y - h / 2) + w / 2 - dx
        ys = -s * (x - w / 2) + c * (y - h / 2) + h / 2 - dy
        img = 0.3 + 0.3 * xs / w
        for k in range(60):
            img = img + amp[k] * np.exp(-((xs - cx[k]) ** 2 + (ys - cy[k]) ** 2) / (2 * sig[k] ** 2))
        return np.clip(np.floor(img * 255 + 0.5), 0, 255).astype(np.uint8)

    return render(0.0, 0.0, 0.0), render(2.3, -1.7, 0.05)


def run(O, a, b):
    k0, d0 = O.surf_detect(a, threshold=THRESHOLD)
    k1, d1 = O.surf_detect(b, threshold=THRESHOLD)
    best, e1, e2 = O.surf_match(d0, d1)
    return dict(kp0=k0, desc0=d0, kp1=k1, desc1=d1, best=best, d1=e1, d2=e2)


def main():
    from oracle import oracle as O

    a, b = frames()
    out = run(O, a, b)
    np.savez_compressed(os.path.join(HERE, "pose_cases.npz"), frame0=a, frame1=b, **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
