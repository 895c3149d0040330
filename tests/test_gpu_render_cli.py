"""The headless scene-file render (python -m raytracer_gb300.render) on the
GPU: the EXR it writes holds the device film of the same scene, post-
processed and rounded to half floats; rectangular tiles from the file's
blockSizeX/blockSizeY reach the device and match the oracle."""
import os

import numpy as np
import pytest

import oracle_lib as O
from raytracer_gb300 import desc as D, scenes
from raytracer_gb300.exr import read_exr
from raytracer_gb300.scene_export import write_scene

pytestmark = pytest.mark.gpu


def test_render_cli_writes_the_device_film(ctx, rtlib, tmp_path):
    from raytracer_gb300 import render
    s = scenes.cornell_smooth(40, 24)
    s.block = (16, 8)
    s.file_name = str(tmp_path / "out.png")
    xmlp = write_scene(s, str(tmp_path / "scene"), spp=3)
    rc = render.main([xmlp, "--seed", "4"])
    assert rc == 0 and os.path.exists(tmp_path / "out.exr")
    ch = read_exr(str(tmp_path / "out.exr"))
    g = rtlib.Scene(ctx, s)
    film = g.render(3, seed=4, block=(16, 8))
    g.close()
    img = rtlib.post_process(film)
    for i, n in enumerate("RGB"):
        assert np.array_equal(ch[n], img[..., i].astype(np.float16).astype(np.float32))
    # the file's tiles are 16 x 8: the oracle with the same tiles gives the same film
    fo = O.OracleScene(s).render(3, seed=4, block=(16, 8))
    assert np.array_equal(film[..., 3], fo[..., 3])
    a, b = film[..., :3].astype(np.float64), fo[..., :3].astype(np.float64)
    bad = np.mean((np.abs(a - b) / np.maximum(np.abs(b), 1e-3)).max(-1) > 1e-3)
    assert bad <= 0.03
    out2 = str(tmp_path / "o2.exr")
    img2, dst = render.render_file(xmlp, out=out2, seed=4, ctx=ctx, compression="none")
    assert dst == out2 and np.array_equal(img2, img)
