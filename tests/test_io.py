"""File formats around the solver (reconflow_gb300.io) and the demo pipeline.

CPU tests: .flo, PNG, PLY round trips, every PNG scanline filter, the KITTI
calibration parse and the demo's camera / point-list rules
(test_reconflow/main.cpp:45-53, 109-131, 143-157).  The GPU test writes a
small synthetic demo folder (two RGB PNGs, a .flo prior, calib.txt) and runs
``reconflow_gb300.demo`` on it through the C ABI.
"""
import os
import struct
import zlib

import numpy as np
import pytest

from reconflow_gb300 import io as rio
from reconflow_gb300.demo import pyramid_levels


def test_flo_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    flow = rng.normal(0, 5, (7, 11, 2)).astype(np.float32)
    flow[2, 3, 0] = np.nan
    p = str(tmp_path / "a.flo")
    rio.write_flo(p, flow)
    raw = open(p, "rb").read()
    assert raw[:4] == b"PIEH"  # 202021.25 as little-endian float32
    assert struct.unpack("<ii", raw[4:12]) == (11, 7)
    back = rio.read_flo(p)
    assert back.shape == (7, 11, 2) and back.dtype == np.float32
    np.testing.assert_array_equal(back.view(np.uint32), flow.view(np.uint32))


def test_flo_rejects_bad_files(tmp_path):
    p = str(tmp_path / "bad.flo")
    open(p, "wb").write(struct.pack("<fii", 1.0, 4, 4))
    with pytest.raises(ValueError, match="not a .flo"):
        rio.read_flo(p)
    open(p, "wb").write(struct.pack("<fii", rio.FLO_TAG, 4, 4) + b"\0" * 20)
    with pytest.raises(ValueError, match="payload"):
        rio.read_flo(p)


@pytest.mark.parametrize("shape,dtype", [((9, 13), np.uint8), ((9, 13, 3), np.uint8),
                                         ((5, 6, 4), np.uint8), ((6, 5), np.uint16),
                                         ((4, 7, 3), np.uint16), ((3, 3, 2), np.uint8)])
@pytest.mark.parametrize("filt", [0, 1, 2, 3, 4, "mixed"])
def test_png_round_trip_every_filter(tmp_path, shape, dtype, filt):
    rng = np.random.default_rng(1)
    img = rng.integers(0, np.iinfo(dtype).max + 1, shape, dtype=np.int64).astype(dtype)
    f = [int(i % 5) for i in range(shape[0])] if filt == "mixed" else filt
    p = str(tmp_path / "a.png")
    rio.write_png(p, img, filters=f)
    back = rio.read_png(p)
    assert back.dtype == dtype and back.shape == img.shape
    np.testing.assert_array_equal(back, img)


def _png_bytes(w, h, depth, ctype, rows, extra=b""):
    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data))
    raw = b"".join(b"\0" + r for r in rows)
    return (rio.PNG_SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
            + extra + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


def test_png_palette_and_errors(tmp_path):
    plte = bytes([10, 20, 30, 40, 50, 60])
    blob = _png_bytes(3, 1, 8, 3, [bytes([1, 0, 1])],
                      extra=struct.pack(">I", 6) + b"PLTE" + plte +
                      struct.pack(">I", zlib.crc32(b"PLTE" + plte)))
    p = str(tmp_path / "pal.png")
    open(p, "wb").write(blob)
    np.testing.assert_array_equal(rio.read_png(p), [[[40, 50, 60], [10, 20, 30], [40, 50, 60]]])
    bad = bytearray(blob)
    bad[20] ^= 0xFF  # inside IHDR: CRC mismatch
    open(p, "wb").write(bytes(bad))
    with pytest.raises(ValueError, match="CRC"):
        rio.read_png(p)
    open(p, "wb").write(b"GIF89a")
    with pytest.raises(ValueError, match="not a PNG"):
        rio.read_png(p)


def test_reference_demo_png_decodes():
    """The reference demo's frames decode (768x320 RGB) when its data folder
    (``test_reconflow/data`` of a reference checkout) is named by the
    RF_REFERENCE_DATA environment variable; skipped otherwise."""
    d = os.environ.get("RF_REFERENCE_DATA", "")
    if not d or not os.path.isdir(d):
        pytest.skip("RF_REFERENCE_DATA does not name the reference demo's data folder")
    img = rio.read_png(os.path.join(d, "im319.png"))
    assert img.dtype == np.uint8 and img.ndim == 3 and img.shape[2] == 3
    flo = rio.read_flo(os.path.join(d, "flo319.flo"))
    assert flo.shape[:2] == img.shape[:2]
    K, R, t = rio.demo_camera(os.path.join(d, "calib.txt"))
    assert K.shape == (3, 3) and K[0, 0] > 0 and K[2, 2] == 1.0


CALIB = ("P0: 7.0e+02 0.0 6.0e+02 0.0 0.0 7.0e+02 1.8e+02 0.0 0.0 0.0 1.0 0.0\n"
         "P1: 7.0e+02 0.0 6.0e+02 -3.8e+02 0.0 7.0e+02 1.8e+02 0.0 0.0 0.0 1.0 0.0\n")


def test_calib_and_demo_camera():
    cal = rio.read_calib(CALIB)
    assert sorted(cal) == ["P0", "P1"] and cal["P1"][0, 3] == -380.0
    K, R, t = rio.demo_camera(CALIB)
    np.testing.assert_array_equal(K, [[700, 0, 600], [0, 700, 180], [0, 0, 1]])
    np.testing.assert_array_equal(R, np.eye(3))
    np.testing.assert_array_equal(t, [-1.0, 1e-5, 1e-5])
    with pytest.raises(ValueError):
        rio.demo_camera("no numbers here\n")


def test_demo_cloud_rules():
    X = np.array([[0.0, 80.0, 0.0, 1.0]], np.float32)
    Y = np.array([[1.0, 0.0, -75.0, 2.0]], np.float32)
    Z = np.array([[20.0, 20.0, 20.0, 10.0]], np.float32)
    pts, cols = rio.demo_cloud(X, Y, Z)
    np.testing.assert_array_equal(pts[0], [0.0, -1.0, -20.0])
    assert np.isnan(pts[1:]).all()  # x > 75, y = -75, z = 10 are dropped
    assert cols is None


@pytest.mark.parametrize("binary", [True, False])
def test_ply_round_trip(tmp_path, binary):
    rng = np.random.default_rng(2)
    pts = rng.normal(size=(50, 3)).astype(np.float32)
    pts[3] = np.nan
    cols = rng.integers(0, 256, (50, 3)).astype(np.uint8)
    p = str(tmp_path / "c.ply")
    rio.write_ply(p, pts, cols, binary=binary)
    bp, bc = rio.read_ply(p)
    np.testing.assert_array_equal(bc, cols)
    np.testing.assert_allclose(bp, pts, rtol=1e-7, equal_nan=True)
    rio.write_ply(p, pts, None, binary=binary, drop_nan=True)
    bp, bc = rio.read_ply(p)
    assert bc is None and len(bp) == 49


def test_pyramid_levels_rule():
    # main.cpp:47-53 with scale 2 and minWidth 400 on the demo's 320-row frames
    assert pyramid_levels(320, 2.0, 400) == 1
    assert pyramid_levels(1080, 2.0, 400) == 2   # 540 > 400, 270 stops
    assert pyramid_levels(2160, 2.0, 400) == 3   # 1080, 540 > 400
    assert pyramid_levels(720, 2.0, 100) == 3    # 360, 180 > 100, 90 stops


@pytest.mark.gpu
def test_gpu_demo_pipeline(tmp_path):
    """The demo pipeline on a synthetic scene: PNG / .flo / calib in, PLY /
    .flo / colour PNG out, through the C ABI."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from reconflow_gb300 import demo

    h, w = 64, 96
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    rng = np.random.default_rng(3)
    tex = lambda x, y: 0.5 + 0.25 * np.sin(0.31 * x + 0.17 * y) * np.cos(0.23 * y - 0.11 * x)  # noqa: E731
    g0 = tex(xx, yy)
    g1 = tex(xx - 1.0, yy)  # frame 2 shifted by one pixel (a stereo pair)
    to_rgb = lambda g: np.clip(np.repeat(g[..., None], 3, 2) * 255 + rng.normal(0, 1, (h, w, 3)),  # noqa: E731
                               0, 255).astype(np.uint8)
    data = tmp_path / "data"
    data.mkdir()
    rio.write_png(str(data / "im319.png"), to_rgb(g0), filters=4)
    rio.write_png(str(data / "im318.png"), to_rgb(g1), filters=4)
    prior = np.zeros((h, w, 2), np.float32)
    prior[..., 0] = -1.0
    rio.write_flo(str(data / "flo319.flo"), prior)
    (data / "calib.txt").write_text("P0: 100.0 0.0 48.0 0.0 0.0 100.0 32.0 0.0 0.0 0.0 1.0 0.0\n")
    out = tmp_path / "out"
    demo.main(["--data", str(data), "--out", str(out), "--iters", "20"])
    pts, cols = rio.read_ply(str(out / "output3doursfn.ply"))
    assert pts.shape == (h * w, 3) and cols.shape == (h * w, 3)
    flow = rio.read_flo(str(out / "flow.flo"))
    assert flow.shape == (h, w, 2) and np.isfinite(flow).all()
    color = rio.read_png(str(out / "flow_color.png"))
    assert color.shape == (h, w, 3)
