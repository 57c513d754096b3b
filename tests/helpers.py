"""Shared test helpers: seeded inputs, padding to the reference stride, and
bitwise comparison of float arrays."""
from __future__ import annotations

import numpy as np


def align_up(n, m=32):
    return n + m - n % m if n % m else n


def pad_rows(a, stride, dtype=None):
    """(h, w[, c]) -> (h, stride[, c]) zero-padded, as the reference pads its images."""
    a = np.asarray(a)
    dtype = dtype or a.dtype
    shape = (a.shape[0], stride) + a.shape[2:]
    out = np.zeros(shape, dtype)
    out[:, : a.shape[1]] = a
    return out


def bits(a):
    a = np.ascontiguousarray(a, np.float32)
    return a.view(np.uint32)


def assert_bitexact(got, want, what="", region=None):
    """Bitwise equality of float32 arrays.  Any NaN equals any NaN: the
    payload of a NaN made by an invalid operation (0/0 in the reference's
    projection when Z2 = 0) is host-specific and carries no value."""
    got = np.asarray(got, np.float32)
    want = np.asarray(want, np.float32)
    if region is not None:
        h, w = region
        got, want = got[:h, :w], want[:h, :w]
    assert got.shape == want.shape, (what, got.shape, want.shape)
    diff = (bits(got) != bits(want)) & ~(np.isnan(got) & np.isnan(want))
    if diff.any():
        idx = np.argwhere(diff)
        i = tuple(idx[0])
        d = np.abs(got.astype(np.float64) - want.astype(np.float64))
        raise AssertionError(
            f"{what}: {diff.sum()} of {diff.size} values differ; first at {i}: "
            f"got {got[i]!r} want {want[i]!r}; max |diff| {np.nanmax(d):.3e}")


def smooth_field(rng, h, w, scale=1.0, freq=3):
    """Smooth random field (sum of a few sinusoids)."""
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    f = np.zeros((h, w))
    for _ in range(freq):
        kx, ky = rng.uniform(-0.3, 0.3, 2)
        f += rng.uniform(-1, 1) * np.sin(kx * x + ky * y + rng.uniform(0, 6.28))
    return (scale * f).astype(np.float32)


def textured_pair(rng, h, w, shift=(1.5, -0.75)):
    """A smooth random texture and a sub-pixel shifted copy."""
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)

    def tex(xx, yy):
        v = np.zeros_like(xx)
        r = np.random.default_rng(7)
        for _ in range(12):
            kx, ky = r.uniform(-0.6, 0.6, 2)
            v += r.uniform(0.2, 1) * np.sin(kx * xx + ky * yy + r.uniform(0, 6.28))
        return 0.5 + 0.1 * v

    I0 = tex(x, y)
    I1 = tex(x - shift[0], y - shift[1])
    I0 = I0 + rng.normal(0, 0.002, I0.shape)
    I1 = I1 + rng.normal(0, 0.002, I1.shape)
    return I0.astype(np.float32), I1.astype(np.float32)
