"""EXR output (no GPU): the headless writer's files read back to the same
half-float pixels, with both compressions, the ZIP filter round trip, the
header attributes an OpenEXR reader requires, and the film post-processing
rule of Screen::postProcessColor."""
import struct

import numpy as np
import pytest

from raytracer_gb300 import post_process
from raytracer_gb300.exr import _zip_pack, _zip_unpack, read_exr, write_exr


def _image(h, w, seed):
    rng = np.random.default_rng(seed)
    img = rng.lognormal(0.0, 2.0, (h, w, 3)).astype(np.float32)
    img[0, 0] = (0.0, 1e-8, 7e4)    # zero, a half subnormal, above half max (inf)
    return img


@pytest.mark.parametrize("compression", ["zip", "none"])
@pytest.mark.parametrize("shape", [(1, 1), (17, 33), (40, 7)])
def test_exr_roundtrip_half_pixels(tmp_path, compression, shape):
    img = _image(*shape, seed=shape[0])
    p = str(tmp_path / "a.exr")
    write_exr(p, img, compression=compression)
    ch = read_exr(p)
    assert sorted(ch) == ["A", "B", "G", "R"]
    for i, n in enumerate("RGB"):
        with np.errstate(over="ignore"):
            expect = img[..., i].astype(np.float16).astype(np.float32)
        assert np.array_equal(ch[n], expect, equal_nan=True)
    assert np.all(ch["A"] == 1)


def test_exr_header_attributes(tmp_path):
    p = str(tmp_path / "h.exr")
    write_exr(p, _image(5, 9, 1))
    buf = open(p, "rb").read()
    assert struct.unpack_from("<ii", buf, 0) == (20000630, 2)
    for name in (b"channels\0chlist", b"compression\0compression", b"dataWindow\0box2i",
                 b"displayWindow\0box2i", b"lineOrder\0lineOrder", b"pixelAspectRatio\0float",
                 b"screenWindowCenter\0v2f", b"screenWindowWidth\0float"):
        assert name in buf
    i = buf.index(b"dataWindow\0box2i\0") + len(b"dataWindow\0box2i\0") + 4
    assert struct.unpack_from("<iiii", buf, i) == (0, 0, 8, 4)


def test_zip_filter_roundtrip():
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 1000, 4097):
        raw = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        assert _zip_unpack(_zip_pack(raw), n) == raw


def test_film_is_post_processed(tmp_path):
    film = np.zeros((2, 3, 4), np.float32)
    film[..., :3] = 2.0
    film[..., 3] = [[4.0, 0.0, -2.0], [1.0, 0.5, 0.0]]
    img = post_process(film)
    # colour / weight where the weight is not zero (negative included), the colour elsewhere
    assert np.allclose(img[..., 0], [[0.5, 2.0, -1.0], [2.0, 4.0, 2.0]])
    p = str(tmp_path / "f.exr")
    write_exr(p, film)
    assert np.allclose(read_exr(p)["G"], img[..., 1])


def test_write_exr_rejects_bad_shapes(tmp_path):
    with pytest.raises(ValueError):
        write_exr(str(tmp_path / "x.exr"), np.zeros((4, 4), np.float32))
