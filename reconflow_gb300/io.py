"""File formats around the solver: Middlebury ``.flo`` flow files, PNG images,
KITTI-style calibration text and PLY point clouds.

These are the formats the reference's demo reads and writes
(``test_reconflow/main.cpp``): ``cv::imread`` of PNG frames (``:50,79-80``),
``cv::optflow::readOpticalFlow`` of a ``.flo`` prior (``:83``), the camera
matrix from the ``P0:`` line of a KITTI ``calib.txt`` (``getRtStereo``,
``:143-157``) and ``cv::viz::writeCloud`` of the 3D points as PLY
(``:109-139``).  OpenCV is not a dependency here: every format is decoded
and encoded by this module with numpy and the standard library's zlib.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

# ---------------------------------------------------------------------------
# Middlebury .flo: "PIEH" (float 202021.25), int32 width, int32 height, then
# height * width * 2 float32 (u, v interleaved), little endian.
# ---------------------------------------------------------------------------

FLO_TAG = 202021.25


def read_flo(path: str) -> np.ndarray:
    """(H, W, 2) float32 flow, as cv::optflow::readOpticalFlow returns it."""
    with open(path, "rb") as f:
        head = f.read(12)
        if len(head) < 12:
            raise ValueError(f"{path}: truncated .flo header")
        tag, w, h = struct.unpack("<fii", head)
        if tag != FLO_TAG:
            raise ValueError(f"{path}: not a .flo file (tag {tag!r})")
        if not (0 < w < 1 << 20 and 0 < h < 1 << 20):
            raise ValueError(f"{path}: implausible .flo size {w}x{h}")
        data = np.fromfile(f, dtype="<f4", count=w * h * 2)
    if data.size != w * h * 2:
        raise ValueError(f"{path}: .flo payload has {data.size} floats, expected {w * h * 2}")
    return data.reshape(h, w, 2).astype(np.float32)


def write_flo(path: str, flow) -> None:
    flow = np.asarray(flow, np.float32)
    if flow.ndim != 3 or flow.shape[2] != 2:
        raise ValueError("flow must be (H, W, 2)")
    h, w = flow.shape[:2]
    with open(path, "wb") as f:
        f.write(struct.pack("<fii", FLO_TAG, w, h))
        f.write(np.ascontiguousarray(flow, "<f4").tobytes())


# ---------------------------------------------------------------------------
# PNG (ISO/IEC 15948): chunk framing with CRC-32, zlib-compressed scanlines,
# one filter byte per scanline (None, Sub, Up, Average, Paeth).
# ---------------------------------------------------------------------------

PNG_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunks(blob: bytes):
    if blob[:8] != PNG_SIG:
        raise ValueError("not a PNG file")
    off = 8
    while off + 12 <= len(blob):
        n, = struct.unpack(">I", blob[off:off + 4])
        kind = blob[off + 4:off + 8]
        data = blob[off + 8:off + 8 + n]
        crc, = struct.unpack(">I", blob[off + 8 + n:off + 12 + n])
        if len(data) != n or zlib.crc32(kind + data) != crc:
            raise ValueError(f"PNG chunk {kind!r}: bad length or CRC")
        yield kind, data
        off += 12 + n
        if kind == b"IEND":
            return
    raise ValueError("PNG without IEND")


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(raw: bytes, height: int, rowbytes: int, bpp: int) -> np.ndarray:
    """Reverse the per-scanline filters; returns (height, rowbytes) uint8."""
    if len(raw) < height * (rowbytes + 1):
        raise ValueError("PNG image data too short")
    rows = np.frombuffer(raw, np.uint8, height * (rowbytes + 1)).reshape(height, rowbytes + 1)
    out = np.zeros((height, rowbytes), np.uint8)
    prior = np.zeros(rowbytes, np.uint8)
    for y in range(height):
        ft, line = int(rows[y, 0]), rows[y, 1:]
        if ft == 0:
            cur = line.copy()
        elif ft == 1:  # Sub: modular running sum along each byte lane of a pixel
            pad = (-rowbytes) % bpp
            lanes = np.concatenate([line, np.zeros(pad, np.uint8)]).reshape(-1, bpp)
            cur = (np.cumsum(lanes, axis=0, dtype=np.uint64) & 0xFF).astype(np.uint8).ravel()
            cur = cur[:rowbytes]
        elif ft == 2:  # Up
            cur = line + prior
        elif ft in (3, 4):  # Average / Paeth depend on the reconstructed left byte
            cur_l = bytearray(rowbytes)
            ln, pr = line.tobytes(), prior.tobytes()
            if ft == 3:
                for i in range(rowbytes):
                    left = cur_l[i - bpp] if i >= bpp else 0
                    cur_l[i] = (ln[i] + ((left + pr[i]) >> 1)) & 0xFF
            else:
                for i in range(rowbytes):
                    if i >= bpp:
                        cur_l[i] = (ln[i] + _paeth(cur_l[i - bpp], pr[i], pr[i - bpp])) & 0xFF
                    else:
                        cur_l[i] = (ln[i] + pr[i]) & 0xFF
            cur = np.frombuffer(bytes(cur_l), np.uint8)
        else:
            raise ValueError(f"PNG scanline {y}: unknown filter type {ft}")
        out[y] = cur
        prior = out[y]
    return out


def read_png(path: str) -> np.ndarray:
    """Decode a non-interlaced PNG with 8- or 16-bit samples (gray, gray+alpha,
    RGB, RGBA) or an 8-bit palette.  Returns uint8 or uint16 (big-endian
    samples converted to native), shape (H, W) for gray, else (H, W, C) with
    channels in file order (R, G, B[, A]); palette images expand to RGB."""
    with open(path, "rb") as f:
        blob = f.read()
    ihdr, idat, plte = None, [], None
    for kind, data in _chunks(blob):
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", data)
        elif kind == b"IDAT":
            idat.append(data)
        elif kind == b"PLTE":
            plte = np.frombuffer(data, np.uint8).reshape(-1, 3)
    if ihdr is None:
        raise ValueError(f"{path}: no IHDR")
    w, h, depth, ctype, comp, filt, interlace = ihdr
    if comp != 0 or filt != 0:
        raise ValueError(f"{path}: unknown compression/filter method")
    if interlace != 0:
        raise ValueError(f"{path}: interlaced PNG is not supported")
    if ctype not in _CHANNELS or depth not in ((8,) if ctype == 3 else (8, 16)):
        raise ValueError(f"{path}: colour type {ctype} with bit depth {depth} is not supported")
    ch = _CHANNELS[ctype]
    bpp = ch * depth // 8
    img = _unfilter(zlib.decompress(b"".join(idat)), h, w * bpp, bpp)
    if depth == 16:
        img = img.view(">u2").astype(np.uint16)
    img = img.reshape(h, w, ch)
    if ctype == 3:
        if plte is None:
            raise ValueError(f"{path}: palette image without PLTE")
        img = plte[img[..., 0]]
    return img[..., 0] if img.shape[2] == 1 else img


def _filter_row(line: np.ndarray, prior: np.ndarray, bpp: int, ft: int) -> np.ndarray:
    a = np.concatenate([np.zeros(bpp, np.int32), line[:-bpp].astype(np.int32)]) \
        if line.size > bpp else np.zeros(line.size, np.int32)
    a = a[:line.size]
    b = prior.astype(np.int32)
    c = np.concatenate([np.zeros(bpp, np.int32), b[:-bpp]])[:line.size]
    x = line.astype(np.int32)
    if ft == 0:
        r = x
    elif ft == 1:
        r = x - a
    elif ft == 2:
        r = x - b
    elif ft == 3:
        r = x - ((a + b) >> 1)
    else:
        p = a + b - c
        pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
        pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
        r = x - pred
    return (r & 0xFF).astype(np.uint8)


def write_png(path: str, img, filters=0, level: int = 6) -> None:
    """Encode uint8/uint16 (H, W), (H, W, 3) or (H, W, 4) as PNG.  `filters`
    is one filter type for every scanline or a sequence with one per row."""
    img = np.asarray(img)
    if img.dtype not in (np.uint8, np.uint16):
        raise ValueError("PNG samples must be uint8 or uint16")
    if img.ndim == 2:
        img = img[..., None]
    h, w, ch = img.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}.get(ch)
    if ctype is None:
        raise ValueError("PNG needs 1, 2, 3 or 4 channels")
    depth = 8 * img.dtype.itemsize
    bpp = ch * img.dtype.itemsize
    rows = np.ascontiguousarray(img.astype(">u2") if depth == 16 else img).view(np.uint8)
    rows = rows.reshape(h, w * bpp)
    ft = [filters] * h if np.isscalar(filters) else list(filters)
    raw = bytearray()
    prior = np.zeros(w * bpp, np.uint8)
    for y in range(h):
        raw.append(ft[y])
        raw += _filter_row(rows[y], prior, bpp, ft[y]).tobytes()
        prior = rows[y]

    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data))

    with open(path, "wb") as f:
        f.write(PNG_SIG)
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(bytes(raw), level)))
        f.write(chunk(b"IEND", b""))


# ---------------------------------------------------------------------------
# KITTI-style calibration: lines "Pn: p00 p01 ... p23" (3x4 row-major).
# ---------------------------------------------------------------------------

def read_calib(path_or_text: str) -> dict:
    """All 'name: 12 numbers' lines as 3x4 float64 matrices."""
    text = path_or_text
    if "\n" not in path_or_text and ":" not in path_or_text:
        with open(path_or_text) as f:
            text = f.read()
    out = {}
    for line in text.splitlines():
        if ":" not in line:
            continue
        name, rest = line.split(":", 1)
        vals = rest.split()
        if len(vals) == 12:
            out[name.strip()] = np.array([float(v) for v in vals], np.float64).reshape(3, 4)
    return out


def demo_camera(path_or_text: str):
    """(K, R, t) as the reference demo sets them (main.cpp:143-157): K is the
    left 3x3 block of the first calibration line, R = I and
    t = (-1, 1e-5, 1e-5), a unit stereo baseline to the left."""
    cal = read_calib(path_or_text)
    if not cal:
        raise ValueError("calibration has no 'Pn:' line with 12 numbers")
    P0 = next(iter(cal.values()))
    K = P0[:, :3].copy()
    return K, np.eye(3), np.array([-1.0, 1e-5, 1e-5])


# ---------------------------------------------------------------------------
# PLY point clouds
# ---------------------------------------------------------------------------

def demo_cloud(X, Y, Z, colors=None):
    """The demo's point list (main.cpp:109-131): one point per pixel in row
    order; points with 10 < z <= 75, x <= 75 and -75 < y <= 75 become
    (x, -y, -z), every other point NaN.  The reference's test puts no lower
    bound on x."""
    X, Y, Z = (np.asarray(a, np.float32) for a in (X, Y, Z))
    keep = (Z <= 75) & (Z > 10) & (X <= 75) & (Y > -75) & (Y <= 75)
    pts = np.stack([X, -Y, -Z], axis=-1).reshape(-1, 3)
    pts[~keep.reshape(-1)] = np.nan
    cols = None if colors is None else np.asarray(colors, np.uint8).reshape(-1, 3)
    return pts, cols


def write_ply(path: str, points, colors=None, binary: bool = True, drop_nan: bool = False):
    """Vertices x, y, z (float) and optionally red, green, blue (uchar)."""
    pts = np.asarray(points, np.float32).reshape(-1, 3)
    cols = None if colors is None else np.asarray(colors, np.uint8).reshape(-1, 3)
    if cols is not None and len(cols) != len(pts):
        raise ValueError("colors must have one row per point")
    if drop_nan:
        ok = np.isfinite(pts).all(axis=1)
        pts = pts[ok]
        cols = None if cols is None else cols[ok]
    fmt = "binary_little_endian" if binary else "ascii"
    head = [f"ply", f"format {fmt} 1.0", f"element vertex {len(pts)}",
            "property float x", "property float y", "property float z"]
    if cols is not None:
        head += ["property uchar red", "property uchar green", "property uchar blue"]
    head.append("end_header")
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode("ascii"))
        if binary:
            if cols is None:
                f.write(pts.astype("<f4").tobytes())
            else:
                rec = np.zeros(len(pts), dtype=[("x", "<f4"), ("y", "<f4"), ("z", "<f4"),
                                                ("r", "u1"), ("g", "u1"), ("b", "u1")])
                rec["x"], rec["y"], rec["z"] = pts[:, 0], pts[:, 1], pts[:, 2]
                rec["r"], rec["g"], rec["b"] = cols[:, 0], cols[:, 1], cols[:, 2]
                f.write(rec.tobytes())
        else:
            for i in range(len(pts)):
                line = "%.9g %.9g %.9g" % tuple(pts[i])
                if cols is not None:
                    line += " %d %d %d" % tuple(cols[i])
                f.write((line + "\n").encode("ascii"))


def read_ply(path: str):
    """Read back what write_ply writes: (points, colors or None)."""
    with open(path, "rb") as f:
        head = []
        while True:
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: PLY header without end_header")
            line = line.decode("ascii").strip()
            head.append(line)
            if line == "end_header":
                break
        body = f.read()
    if head[0] != "ply":
        raise ValueError(f"{path}: not a PLY file")
    fmt = head[1].split()[1]
    n = int(next(h for h in head if h.startswith("element vertex")).split()[2])
    has_col = any(h.endswith(" red") for h in head)
    if fmt == "binary_little_endian":
        dt = [("x", "<f4"), ("y", "<f4"), ("z", "<f4")] + \
            ([("r", "u1"), ("g", "u1"), ("b", "u1")] if has_col else [])
        rec = np.frombuffer(body, dtype=dt, count=n)
        pts = np.stack([rec["x"], rec["y"], rec["z"]], axis=1)
        cols = np.stack([rec["r"], rec["g"], rec["b"]], axis=1) if has_col else None
    elif fmt == "ascii":
        rows = [r.split() for r in body.decode("ascii").splitlines()[:n]]
        pts = np.array([[float(v) for v in r[:3]] for r in rows], np.float32).reshape(-1, 3)
        cols = np.array([[int(v) for v in r[3:6]] for r in rows], np.uint8) if has_col else None
    else:
        raise ValueError(f"{path}: PLY format {fmt} is not supported")
    return pts, cols
