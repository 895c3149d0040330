"""ScaleTexture (texture/ScaleTexture.cpp): eval = texture.eval(uv) * scale,
read from scene files over a constant and over an ImageTexture."""
import numpy as np
import pytest

import oracle_lib as O
from raytracer_gb300 import scenes
from raytracer_gb300.scene_export import write_scene
from raytracer_gb300.xml_scene import UnsupportedScene, load_scene


@pytest.fixture(scope="module")
def built():
    from raytracer_gb300 import build
    return build.build()


def _with_scale(text, k):
    """Wrap the first albedo texture of a written scene in a ScaleTexture."""
    a = text.index('<texture name="albedo"')
    b = text.index("</texture>", a) + len("</texture>")
    inner = text[a:b].replace('name="albedo"', 'name="texture"', 1)
    return (text[:a] + '<texture name="albedo" type="ScaleTexture">' + inner +
            '<double name="scale" value="%r"/></texture>' % k + text[b:])


def test_scale_texture_over_image(built, tmp_path):
    s = scenes.plane_room(16, 12, textured=True)
    path = write_scene(s, str(tmp_path))
    text = open(path).read()
    base = load_scene(path)
    open(tmp_path / "scaled.xml", "w").write(_with_scale(text, 0.5))
    t = load_scene(str(tmp_path / "scaled.xml"))
    i = [b["tex_albedo"] for b in base.bsdfs if b.get("tex_albedo", -1) >= 0][0]
    j = [b["tex_albedo"] for b in t.bsdfs if b.get("tex_albedo", -1) >= 0][0]
    assert t.textures[j]["scale"] == base.textures[i]["scale"] * 0.5
    assert np.array_equal(t.textures[j]["rgb"], base.textures[i]["rgb"])
    fa = O.OracleScene(base).render(2, seed=5, threads=4)
    fb = O.OracleScene(t).render(2, seed=5, threads=4)
    assert fb[..., :3].sum() < fa[..., :3].sum()
    open(tmp_path / "neg.xml", "w").write(_with_scale(text, -1.0))
    with pytest.raises(UnsupportedScene):
        load_scene(str(tmp_path / "neg.xml"))


def test_scale_texture_over_constant(built, tmp_path):
    s = scenes.cornell_box(8, 8)
    text = open(write_scene(s, str(tmp_path))).read()
    a = text.index('<color name="albedo" value="')
    b = text.index("/>", a) + 2
    val = text[a:b].split('value="')[1].split('"')[0]
    wrapped = ('<texture name="albedo" type="ScaleTexture"><texture name="texture" type="ConstantTexture">'
               '<color name="albedo" value="%s"/></texture><double name="scale" value="0.25"/></texture>' % val)
    open(tmp_path / "c.xml", "w").write(text[:a] + wrapped + text[b:])
    t = load_scene(str(tmp_path / "c.xml"))
    want = tuple(float(x) * 0.25 for x in val.replace(",", " ").split())
    assert tuple(t.bsdfs[0]["albedo"]) == pytest.approx(want, rel=0, abs=0)
