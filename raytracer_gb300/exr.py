"""Headless OpenEXR output for rendered films.

The reference saves its film through OpenEXR's `RgbaOutputFile` (writeEXR,
core/main.cpp:292-318): one scanline image with half-float R, G, B and an
alpha of 1, the library's default ZIP compression, holding the film after
Screen::postProcessColor (colour / weight).  `write_exr` produces the same
kind of file from the device film without OpenEXR: the header attributes
OpenEXR writes for such a file, the chunk offset table, and the scanline
blocks, 16 lines each compressed with zlib after OpenEXR's byte split and
delta predictor (or stored uncompressed).  `read_exr` reads back the
scanline files this module writes (and other uncompressed or ZIP scanline
files with HALF or FLOAT channels).
"""
import struct
import zlib

import numpy as np

from .core import post_process

_HALF, _FLOAT = 1, 2
_NO_COMPRESSION, _ZIPS_COMPRESSION, _ZIP_COMPRESSION = 0, 2, 3
_LINES = {_NO_COMPRESSION: 1, _ZIPS_COMPRESSION: 1, _ZIP_COMPRESSION: 16}


def _attr(name, kind, data):
    return name.encode() + b"\0" + kind.encode() + b"\0" + struct.pack("<i", len(data)) + data


def _zip_pack(raw):
    # OpenEXR's zip filter: bytes split into even and odd positions, then a
    # delta predictor (difference to the previous byte, plus 128), then zlib
    b = np.frombuffer(raw, np.uint8)
    t = np.concatenate([b[0::2], b[1::2]]).astype(np.int16)
    d = t.astype(np.uint8)
    d[1:] = ((t[1:] - t[:-1] + 128) % 256).astype(np.uint8)
    return zlib.compress(d.tobytes())


def _zip_unpack(data, size):
    d = np.frombuffer(zlib.decompress(data), np.uint8).astype(np.int64)
    if len(d) != size:
        raise ValueError("EXR: corrupt zip block")
    # undo the predictor: t[i] = t[i-1] + d[i] - 128 (mod 256), t[0] = d[0]
    t = np.empty(size, np.uint8)
    t[0] = d[0]
    t[1:] = ((d[0] + np.cumsum(d[1:] - 128)) % 256).astype(np.uint8)
    half = (size + 1) // 2
    out = np.empty(size, np.uint8)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out.tobytes()


def write_exr(path, image, compression="zip"):
    """Write an H x W x 3 (or a raw H x W x 4 film, which is post-processed
    first) image as a half-float RGBA scanline EXR with alpha 1."""
    img = np.asarray(image, np.float32)
    if img.ndim != 3 or img.shape[2] not in (3, 4):
        raise ValueError("write_exr: expected an H x W x 3 image or an H x W x 4 film")
    if img.shape[2] == 4:
        img = post_process(img)
    comp = {"none": _NO_COMPRESSION, "zip": _ZIP_COMPRESSION}[compression]
    H, W = img.shape[:2]
    # channels in OpenEXR's (alphabetical) file order: A, B, G, R
    with np.errstate(over="ignore"):   # beyond the half range is infinity, as in half(float)
        planes = [np.ones((H, W), np.float16), img[..., 2].astype(np.float16), img[..., 1].astype(np.float16),
                  img[..., 0].astype(np.float16)]
    chl = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", _HALF, 0, 1, 1) for n in "ABGR") + b"\0"
    box = struct.pack("<iiii", 0, 0, W - 1, H - 1)
    header = (struct.pack("<ii", 20000630, 2)
              + _attr("channels", "chlist", chl)
              + _attr("compression", "compression", bytes([comp]))
              + _attr("dataWindow", "box2i", box)
              + _attr("displayWindow", "box2i", box)
              + _attr("lineOrder", "lineOrder", bytes([0]))
              + _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
              + _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
              + _attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
              + b"\0")
    lines = _LINES[comp]
    chunks = []
    for y0 in range(0, H, lines):
        y1 = min(H, y0 + lines)
        raw = b"".join(p[y].tobytes() for y in range(y0, y1) for p in planes)
        data = raw
        if comp == _ZIP_COMPRESSION:
            z = _zip_pack(raw)
            if len(z) < len(raw):
                data = z
        chunks.append(struct.pack("<ii", y0, len(data)) + data)
    offset = len(header) + 8 * len(chunks)
    table = []
    for c in chunks:
        table.append(struct.pack("<Q", offset))
        offset += len(c)
    with open(path, "wb") as f:
        f.write(header)
        f.write(b"".join(table))
        f.write(b"".join(chunks))


def read_exr(path):
    """Read a single-part scanline EXR (no compression, ZIPS or ZIP; HALF or
    FLOAT channels).  Returns {channel name: H x W float32 array}."""
    buf = open(path, "rb").read()
    magic, version = struct.unpack_from("<ii", buf, 0)
    if magic != 20000630:
        raise ValueError("not an OpenEXR file")
    if version & 0x200 or version & 0x1000:
        raise ValueError("EXR: tiled and multi-part files are not read")
    pos = 8
    attrs = {}
    while buf[pos] != 0:
        e = buf.index(b"\0", pos)
        name = buf[pos:e].decode()
        e2 = buf.index(b"\0", e + 1)
        kind = buf[e + 1:e2].decode()
        size = struct.unpack_from("<i", buf, e2 + 1)[0]
        attrs[name] = (kind, buf[e2 + 5:e2 + 5 + size])
        pos = e2 + 5 + size
    pos += 1
    channels = []
    chl = attrs["channels"][1]
    p = 0
    while chl[p] != 0:
        e = chl.index(b"\0", p)
        ptype, _, xs, ys = struct.unpack_from("<iB3xii", chl, e + 1)
        if (xs, ys) != (1, 1) or ptype not in (_HALF, _FLOAT):
            raise ValueError("EXR: subsampled or UINT channels are not read")
        channels.append((chl[p:e].decode(), ptype))
        p = e + 1 + 16
    comp = attrs["compression"][1][0]
    if comp not in _LINES:
        raise ValueError("EXR: compression %d is not read" % comp)
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    W, H = x1 - x0 + 1, y1 - y0 + 1
    out = {n: np.zeros((H, W), np.float32) for n, _ in channels}
    lines = _LINES[comp]
    nchunks = (H + lines - 1) // lines
    offsets = struct.unpack_from("<%dQ" % nchunks, buf, pos)
    for off in offsets:
        y, size = struct.unpack_from("<ii", buf, off)
        n = min(lines, y1 + 1 - y)
        data = buf[off + 8:off + 8 + size]
        full = sum(W * n * (2 if t == _HALF else 4) for _, t in channels)
        if size < full:
            data = _zip_unpack(data, full)
        q = 0
        for r in range(n):
            for name, t in channels:
                dt = np.float16 if t == _HALF else np.float32
                k = W * np.dtype(dt).itemsize
                out[name][y - y0 + r] = np.frombuffer(data[q:q + k], dt)
                q += k
    return out
