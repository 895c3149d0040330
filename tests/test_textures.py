"""ImageTexture on the host (no GPU): image files read as ImageLoader leaves
them (PNG with every scanline filter and colour type, PPM/PGM, PFM, sRGB
decoding), the oracle's ImageTexture::eval against an independent binary32
restatement (wrap, invert, scale, one-texel edges), and textured scene files
(ImageTexture elements, OBJ texture coordinates) read back to the same
scene and the same oracle film."""
import struct
import zlib

import numpy as np
import pytest

import oracle_lib as O
from raytracer_gb300 import desc as D, scenes
from raytracer_gb300.images import from_srgb, load_image, read_png, read_pfm, read_pnm, write_pfm
from raytracer_gb300.scene_export import write_scene
from raytracer_gb300.xml_scene import UnsupportedScene, load_scene

F = np.float32


@pytest.fixture(scope="module")
def built():
    from raytracer_gb300 import build
    return build.build()


# ------------------------------------------------------------------ PNG writer (test side)
def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def _png(arr, ctype, depth=8, palette=None, trns=None):
    """PNG bytes of `arr` (H, W, C), cycling through the five filter types."""
    h, w = arr.shape[:2]
    if depth == 16:
        rows = arr.astype(">u2").reshape(h, -1).view(np.uint8).reshape(h, -1)
    else:
        rows = arr.astype(np.uint8).reshape(h, -1)
    bpp = max(1, (arr.shape[2] if arr.ndim == 3 else 1) * depth // 8)
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int64)
    for y in range(h):
        cur = rows[y].astype(np.int64)
        ft = y % 5
        f = np.zeros_like(cur)
        for i in range(len(cur)):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            f[i] = (cur[i] - pred) & 0xFF
        out += bytes([ft]) + f.astype(np.uint8).tobytes()
        prev = cur

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if palette is not None:
        png += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        png += chunk(b"tRNS", trns.astype(np.uint8).tobytes())
    return png + chunk(b"IDAT", zlib.compress(bytes(out))) + chunk(b"IEND", b"")


@pytest.mark.parametrize("ctype,chans,depth", [(2, 3, 8), (6, 4, 8), (0, 1, 8), (4, 2, 8), (2, 3, 16)])
def test_png_decoder_every_filter(tmp_path, ctype, chans, depth):
    rng = np.random.default_rng(ctype + depth)
    arr = rng.integers(0, 2 ** depth, (11, 7, chans))
    p = tmp_path / "a.png"
    p.write_bytes(_png(arr, ctype, depth))
    got = read_png(str(p))
    assert got.shape == (11, 7, chans)
    assert np.array_equal(got, (arr / (2 ** depth - 1)).astype(F))


def test_png_palette_with_transparency(tmp_path):
    rng = np.random.default_rng(3)
    pal = rng.integers(0, 256, (5, 3))
    idx = rng.integers(0, 5, (6, 9, 1))
    p = tmp_path / "p.png"
    p.write_bytes(_png(idx, 3, 8, palette=pal, trns=np.array([10, 20])))
    got = read_png(str(p))
    alpha = np.array([10, 20, 255, 255, 255])
    expect = np.concatenate([pal[idx[..., 0]], alpha[idx[..., 0]][..., None]], axis=2) / 255.0
    assert np.array_equal(got, expect.astype(F))


def test_pnm_pfm_and_srgb(tmp_path):
    rng = np.random.default_rng(5)
    a = rng.integers(0, 256, (4, 5, 3)).astype(np.uint8)
    (tmp_path / "a.ppm").write_bytes(b"P6\n# comment\n5 4\n255\n" + a.tobytes())
    assert np.array_equal(read_pnm(str(tmp_path / "a.ppm")), (a / 255.0).astype(F))
    f = rng.random((3, 6, 3)).astype(F)
    write_pfm(str(tmp_path / "a.pfm"), f)
    assert np.array_equal(read_pfm(str(tmp_path / "a.pfm")), f)
    # 8-bit images are decoded from sRGB unless a gamma is given
    v = np.linspace(0, 1, 257, dtype=F)
    ref = np.where(v <= 0.04045, v / 12.92, ((v + 0.055) / 1.055) ** 2.4)
    assert np.allclose(from_srgb(v), ref, rtol=2e-6, atol=1e-9)
    img = load_image(str(tmp_path / "a.ppm"))
    assert np.array_equal(img, from_srgb(a / np.float32(255.0)))
    g = load_image(str(tmp_path / "a.ppm"), gamma=2.2, channel="g")
    assert np.allclose(g[..., 0], (a[..., 1] / 255.0) ** 2.2, rtol=1e-5) and np.array_equal(g[..., 0], g[..., 2])
    (tmp_path / "a.jpg").write_bytes(b"\xff\xd8\xff\xe0" + bytes(16))
    with pytest.raises(ValueError):
        load_image(str(tmp_path / "a.jpg"))


# ------------------------------------------------------------------ ImageTexture::eval
def _interp2(img, x, y):
    h, w = img.shape[:2]
    ax, ay = F(x - F(int(x))), F(y - F(int(y)))
    clamp = lambda v, lo, hi: lo if v < lo else (hi if v > hi else v)
    x0 = 0 if w < 2 else clamp(int(x), 0, w - 2)
    y0 = 0 if h < 2 else clamp(int(y), 0, h - 2)
    x1 = clamp(x0 + 1 if x0 + 1 < w else x0, 0, w - 1)
    y1 = clamp(y0 + 1 if y0 + 1 < h else y0, 0, h - 1)
    one = F(1)
    r = img[y0, x0] * ((one - ax) * (one - ay))
    r = r + img[y1, x0] * ((one - ax) * ay)
    r = r + img[y0, x1] * (ax * (one - ay))
    return r + img[y1, x1] * (ax * ay)


def _eval(img, u, v, scale, ix, iy):
    """ImageTexture::eval (ImageTexture.cpp:28-70) restated in binary32."""
    h, w = img.shape[:2]
    W, H = F(w), F(h)
    u, v = F(u), F(v)
    sg = lambda t: F(1) if t >= 0 else F(-1)
    y = v * H if not iy else F(int(v)) + (sg(v) * F(1) - (v - F(int(v)))) * H
    x = u * (W - F(1)) if not ix else F(int(u)) + (sg(u) * F(1) - (u - F(int(u)))) * W
    x, y = F(x * F(scale)), F(y * F(scale))
    if x >= W:
        x = F(int(x) % w) + (x - F(int(x)))
    elif x < 0:
        x = F(w - abs(int(x)) % w) + (x - F(int(x)))
    if y >= H:
        y = F(int(y) % h) + (y - F(int(y)))
    elif y < 0:
        y = F(h - abs(int(y)) % h) + (y - F(int(y)))
    return _interp2(img, F(x), F(y))


@pytest.mark.parametrize("shape,scale,ix,iy", [((48, 64), 1.0, False, False), ((48, 64), 3.0, False, False),
                                               ((5, 7), 1.0, True, True), ((1, 1), 1.0, False, False),
                                               ((2, 2), 2.5, True, False), ((1, 9), 1.0, False, True)])
def test_texture_eval_matches_restatement(built, shape, scale, ix, iy):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    img = rng.random(shape + (3,)).astype(F)
    uv = np.concatenate([rng.random((300, 2)), rng.uniform(-3, 4, (300, 2)),
                         np.array([[0, 0], [1, 1], [0.5, 1], [1, 0.5], [-1, -1], [2, 2]])]).astype(F)
    got = O.tex_eval(img, uv, scale, ix, iy)
    expect = np.array([_eval(img, u, v, scale, ix, iy) for u, v in uv], F)
    assert np.array_equal(got, expect)
    # at texel corners (in range, no scale or flip) it is the texel itself
    if scale == 1.0 and not ix and not iy and shape[0] > 1 and shape[1] > 1:
        h, w = shape
        xs, ys = np.arange(w - 1), np.arange(h - 1)
        g = np.stack(np.meshgrid(xs / F(w - 1), ys / F(h), indexing="xy"), -1).reshape(-1, 2).astype(F)
        assert np.allclose(O.tex_eval(img, g), img[:h - 1, :w - 1].reshape(-1, 3), atol=1e-6)


# ------------------------------------------------------------------ scene files
def test_textured_scene_roundtrip(built, tmp_path):
    s = scenes.textured_room(24, 20)
    t = load_scene(write_scene(s, str(tmp_path)))
    assert len(t.textures) == len(s.textures)
    # the file lists textures where they are used: compare what each BSDF refers to
    for x, y in zip(s.meshes + s.spheres, t.meshes + t.spheres):
        bx, by = s.bsdfs[x["bsdf"]], t.bsdfs[y["bsdf"]]
        for k in D.TEX_PARAMS:
            assert (bx.get(k) is None) == (by.get(k) is None), k
            if bx.get(k) is not None:
                a, b = s.textures[bx[k]], t.textures[by[k]]
                assert np.array_equal(a["rgb"], b["rgb"])
                assert (a["scale"], a["invert_x"], a["invert_y"]) == (b["scale"], b["invert_x"], b["invert_y"])
    fa = O.OracleScene(s).render(4, seed=3, threads=4)
    fb = O.OracleScene(t).render(4, seed=3, threads=4)
    assert np.array_equal(fa, fb)
    # the textures change the film
    u = scenes.textured_room(24, 20)
    for b in u.bsdfs:
        for k in D.TEX_PARAMS:
            b.pop(k, None)
    assert not np.array_equal(O.OracleScene(u).render(4, seed=3, threads=4), fa)


def test_png_texture_in_a_scene_file(built, tmp_path):
    s = scenes.cornell_box(8, 8)
    xmlp = write_scene(s, str(tmp_path))
    text = open(xmlp).read()
    rng = np.random.default_rng(11)
    px = rng.integers(0, 256, (4, 6, 3))
    (tmp_path / "t.png").write_bytes(_png(px, 2))
    tex = ('<texture name="albedo" type="ImageTexture"><string name="path" value="t.png"/>'
           '<double name="scale" value="-2"/><bool name="invertY" value="true"/></texture>')
    first = text.index('<color name="albedo"')
    end = text.index("/>", first) + 2
    open(tmp_path / "p.xml", "w").write(text[:first] + tex + text[end:])
    t = load_scene(str(tmp_path / "p.xml"))
    b = t.bsdfs[t.meshes[0]["bsdf"]]
    T = t.textures[b["tex_albedo"]]
    assert np.array_equal(T["rgb"], from_srgb(px / np.float32(255.0)))
    assert T["scale"] == 2.0 and T["invert_y"] and not T["invert_x"]
    open(tmp_path / "j.xml", "w").write(text[:first] + tex.replace("t.png", "t.jpg") + text[end:])
    with pytest.raises(UnsupportedScene):
        load_scene(str(tmp_path / "j.xml"))
