"""Image files for ImageTexture, read as io/ImageLoader.cpp:34-140 leaves them.

ImageLoader::load reads Radiance .hdr and OpenEXR files as linear values
(gamma 1 unless the texture's "gamma" says otherwise) and every other image
through SFML as 8-bit channels divided by 255, decoded from sRGB by default
(gammaFrom -1, Color3::fromSRGB, core/Color.h:330-342).  A "channel" of r, g,
b or a replicates that channel into all three (ImageLoader::setPixel).

Formats read here: Radiance .hdr (the library's RGBE reader), OpenEXR
scanline files (exr.read_exr), PNG (8- and 16-bit, every colour type,
non-interlaced; inflated with zlib), binary PPM/PGM and PFM.  Returns
(H, W, 3) float32 images, row 0 the top row, as Array2D(x, y) holds them.
"""
import os
import struct
import zlib

import numpy as np

_PNG_SIG = b"\x89PNG\r\n\x1a\n"


class ImageError(ValueError):
    pass


def _unfilter(raw, width, height, bpp, stride):
    """PNG scanline filters (None, Sub, Up, Average, Paeth), undone row by row."""
    out = np.zeros((height, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(height):
        ftype = raw[pos]
        line = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int32)
        pos += 1 + stride
        if ftype == 0:
            cur = line
        elif ftype == 1:   # Sub: running sum per byte lane of the pixel
            cur = np.cumsum(line.reshape(-1, bpp), axis=0).reshape(-1) & 0xFF
        elif ftype == 2:   # Up
            cur = (line + prev) & 0xFF
        elif ftype == 3:   # Average
            cur = np.zeros(stride, np.int32)
            for i in range(stride):
                left = cur[i - bpp] if i >= bpp else 0
                cur[i] = (line[i] + ((left + prev[i]) >> 1)) & 0xFF
        elif ftype == 4:   # Paeth
            cur = np.zeros(stride, np.int32)
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[i] = (line[i] + pred) & 0xFF
        else:
            raise ImageError("PNG: bad filter type %d" % ftype)
        out[y] = cur
        prev = cur
    return out


def read_png(path):
    """(H, W, C) channels scaled to [0, 1] (C = 1 grey, 2 grey+alpha, 3 RGB,
    4 RGBA; palettes expanded to RGB or RGBA)."""
    data = open(path, "rb").read()
    if not data.startswith(_PNG_SIG):
        raise ImageError("not a PNG file")
    pos = 8
    idat = []
    hdr = None
    plte = None
    trns = None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if hdr is None:
        raise ImageError("PNG: no IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    if interlace:
        raise ImageError("PNG: interlaced images are not read")
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}.get(ctype)
    if chans is None or depth not in ((8, 16) if ctype != 3 else (8,)):
        raise ImageError("PNG: colour type %d at %d bits is not read" % (ctype, depth))
    bpp = chans * depth // 8
    raw = zlib.decompress(b"".join(idat))
    if len(raw) != h * (1 + w * bpp):
        raise ImageError("PNG: truncated image data")
    px = _unfilter(raw, w, h, bpp, w * bpp)
    if depth == 16:
        img = px.reshape(h, w * chans, 2).astype(np.uint32)
        img = ((img[..., 0] << 8) | img[..., 1]).reshape(h, w, chans).astype(np.float32) / np.float32(65535.0)
    else:
        img = px.reshape(h, w, chans)
        if ctype == 3:
            if plte is None:
                raise ImageError("PNG: palette image without PLTE")
            idx = img[..., 0]
            rgb = plte[idx]
            if trns is not None:
                alpha = np.full(len(plte), 255, np.uint8)
                alpha[:len(trns)] = trns
                img = np.concatenate([rgb, alpha[idx][..., None]], axis=2)
            else:
                img = rgb
        img = img.astype(np.float32) / np.float32(255.0)
    return img


def read_pnm(path):
    """Binary PPM (P6) / PGM (P5), maxval up to 65535, scaled to [0, 1]."""
    data = open(path, "rb").read()
    tokens, pos = [], 0
    while len(tokens) < 4:
        while data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            pos = data.index(b"\n", pos) + 1
            continue
        end = pos
        while not data[end:end + 1].isspace():
            end += 1
        tokens.append(data[pos:end])
        pos = end
    pos += 1
    magic, w, h, mx = tokens[0], int(tokens[1]), int(tokens[2]), int(tokens[3])
    chans = {b"P6": 3, b"P5": 1}.get(magic)
    if chans is None:
        raise ImageError("PNM: only binary P5/P6 are read")
    dt = np.dtype(">u2") if mx > 255 else np.uint8
    px = np.frombuffer(data, dt, w * h * chans, pos).reshape(h, w, chans)
    return px.astype(np.float32) / np.float32(mx)


def read_pfm(path):
    """PFM (PF colour / Pf grey); rows stored bottom first."""
    f = open(path, "rb")
    kind = f.readline().strip()
    w, h = (int(x) for x in f.readline().split())
    scale = float(f.readline())
    chans = {b"PF": 3, b"Pf": 1}.get(kind)
    if chans is None:
        raise ImageError("not a PFM file")
    dt = "<f4" if scale < 0 else ">f4"
    px = np.frombuffer(f.read(w * h * chans * 4), dt).reshape(h, w, chans)
    return px[::-1].astype(np.float32)


def write_pfm(path, img):
    img = np.asarray(img, np.float32)
    if img.ndim == 2:
        img = img[..., None]
    kind = b"PF" if img.shape[2] == 3 else b"Pf"
    with open(path, "wb") as f:
        f.write(kind + b"\n%d %d\n-1\n" % (img.shape[1], img.shape[0]))
        f.write(np.ascontiguousarray(img[::-1], "<f4").tobytes())


def from_srgb(v):
    """Color3::fromSRGB per channel (core/Color.h:330-342), in binary32."""
    v = np.asarray(v, np.float32)
    lo = v * np.float32(1.0 / 12.92)
    hi = np.power((v + np.float32(0.055)) * np.float32(1.0 / 1.055), np.float32(2.4), dtype=np.float32)
    return np.where(v <= np.float32(0.04045), lo, hi).astype(np.float32)


def _is_hdr(path):
    head = open(path, "rb").read(10)
    return head[:4] == b"\x76\x2f\x31\x01" or head == b"#?RADIANCE"


def load_image(path, gamma=0.0, channel="all"):
    """ImageLoader::load (ImageLoader.cpp:34-140) with gammaDest 1: a linear
    (H, W, 3) float32 image."""
    hdr = _is_hdr(path)
    if hdr:
        head = open(path, "rb").read(4)
        if head == b"\x76\x2f\x31\x01":
            from .exr import read_exr
            ch = read_exr(path)
            if not all(k in ch for k in "RGB"):
                raise ImageError("EXR texture without R, G and B channels")
            a = ch.get("A", np.zeros_like(ch["R"]))
            img = np.stack([ch["R"], ch["G"], ch["B"], a], axis=2)
        else:
            from .core import load_hdr
            rgb = load_hdr(path)
            img = np.concatenate([rgb, np.zeros(rgb.shape[:2] + (1,), np.float32)], axis=2)
        gamma_from = 1.0 if gamma == 0 else gamma
    else:
        ext = os.path.splitext(path)[1].lower()
        if ext == ".png":
            img = read_png(path)
        elif ext in (".ppm", ".pgm", ".pnm"):
            img = read_pnm(path)
        elif ext == ".pfm":
            img = read_pfm(path)
        else:
            raise ImageError("texture image format %s is not read (PNG, PPM/PGM, PFM, .hdr and .exr are)" % ext)
        c = img.shape[2]
        if c == 1:
            img = np.concatenate([img, img, img, np.ones_like(img)], axis=2)
        elif c == 2:
            img = np.concatenate([img[..., :1], img[..., :1], img[..., :1], img[..., 1:]], axis=2)
        elif c == 3:
            img = np.concatenate([img, np.ones(img.shape[:2] + (1,), np.float32)], axis=2)
        gamma_from = -1.0 if gamma == 0 else gamma
    ch = channel.lower()
    pick = {"r": 0, "g": 1, "b": 2, "a": 3}.get(ch)
    rgb = img[..., :3] if pick is None else np.repeat(img[..., pick:pick + 1], 3, axis=2)
    rgb = rgb.astype(np.float32)
    if gamma_from == -1.0:
        rgb = from_srgb(rgb)
    elif gamma_from != 1.0:
        rgb = np.power(rgb, np.float32(gamma_from), dtype=np.float32)
    return np.ascontiguousarray(rgb, np.float32)
