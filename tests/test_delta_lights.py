"""PointLight and SpotLight (light/PointLight.cpp, light/SpotLight.cpp): the
oracle's restatement against the reference's formulas written out here in
float64, films lit by them alone under both integrators, and the scene-file
round trip.  The device side is held to the oracle in test_gpu_parity.py."""
import math

import numpy as np
import pytest

import oracle_lib as O
from raytracer_gb300 import desc as D, scenes
from raytracer_gb300.scene_export import write_scene
from raytracer_gb300.xml_scene import load_scene


@pytest.fixture(scope="module")
def built():
    from raytracer_gb300 import build
    return build.build()


def _points(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.random((n, 3)).astype(np.float32)
    u = rng.random((n, 2)).astype(np.float32)
    return p, u


def test_point_light_sample(built):
    """PointLight::sample: direction to the position, intensity / d^2, pdf 1
    whatever the 2-D sample; PointLight::pdf is 0."""
    s = scenes.cornell_delta_lights(8, 8)
    li = [i for i, L in enumerate(s.lights) if L["type"] == D.LIGHT_POINT][0]
    pos = np.array(s.lights[li]["position"], np.float64)
    I = np.array(s.lights[li]["intensity"], np.float64)
    p, u = _points(4000, 1)
    o = O.OracleScene(s)
    r = o.light_query(li, p, u)
    d = pos - p.astype(np.float64)
    dist = np.linalg.norm(d, axis=1)
    np.testing.assert_allclose(r["distance"], dist, rtol=1e-6)
    np.testing.assert_allclose(r["to_light"], d / dist[:, None], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(r["intensity"], I / dist[:, None] ** 2, rtol=1e-5)
    assert np.all(r["pdf"] == 1.0)
    assert np.all(r["pdf_eval"] == 0.0)
    np.testing.assert_array_equal(r["point"], np.broadcast_to(pos.astype(np.float32), (len(p), 3)))
    o.close()


@pytest.mark.parametrize("scale", [1.0, 1.05])
def test_spot_light_falloff(built, scale):
    """SpotLight::falloff: 1 inside falloffStart, 0 outside totalWidth, the
    fourth power of the normalised cosine between; the cosine is the z of the
    inverse-toWorld image of the direction, not renormalised, so a scaled
    toWorld narrows the cone."""
    s = scenes.cornell_delta_lights(8, 8, spot_scale=scale)
    li = [i for i, L in enumerate(s.lights) if L["type"] == D.LIGHT_SPOT][0]
    L = s.lights[li]
    M = L["to_world"]
    pos = (M @ np.array([0, 0, 0, 1.0]))[:3]
    inv = np.linalg.inv(M)
    cfs, ctw = math.cos(math.radians(L["falloff_start"])), math.cos(math.radians(L["total_width"]))
    # points on the floor and walls below the spot, inside and outside its cone
    rng = np.random.default_rng(2)
    p = np.column_stack([rng.random(6000), rng.random(6000) * 0.6, rng.random(6000)]).astype(np.float32)
    u = rng.random((6000, 2)).astype(np.float32)
    o = O.OracleScene(s)
    r = o.light_query(li, p, u)
    d = pos - p.astype(np.float64)
    dist = np.linalg.norm(d, axis=1)
    w = d / dist[:, None]
    ct = (inv[:3, :3] @ (-w).T)[2]
    f = np.where(ct < ctw, 0.0, np.where(ct > cfs, 1.0, ((ct - ctw) / (cfs - ctw)) ** 4))
    want = np.array(L["intensity"])[None, :] * f[:, None] / dist[:, None] ** 2
    # away from the two cone edges, where a last-ulp cosine flips the branch;
    # near the outer edge the fourth power magnifies the binary32 cosine's
    # error (relative error of f about 4 ulp(ct) / (ct - cosTotalWidth))
    edge = (np.abs(ct - ctw) < 1e-5) | (np.abs(ct - cfs) < 1e-5)
    dl = (ct - ctw) / (cfs - ctw)
    tight = ~edge & ((dl > 0.1) | (f == 0))
    np.testing.assert_allclose(r["intensity"][tight], want[tight], rtol=1e-4, atol=1e-12)
    np.testing.assert_allclose(r["intensity"][~edge], want[~edge], rtol=2e-3, atol=1e-12)
    assert (f == 0).mean() > 0.2 and (f == 1).mean() > 0.02 and ((f > 0) & (f < 1)).mean() > 0.02
    assert np.all(r["pdf"] == 1.0) and np.all(r["pdf_eval"] == 0.0)
    o.close()


def test_delta_light_films_are_lit(built):
    """Both integrators light the room from the delta lights alone: the film
    is finite, the spot adds light (most of it on the floor below it), and
    without media the two integrators agree in total."""
    sums = []
    for integ in (D.INTEGRATOR_PATH_MIS, D.INTEGRATOR_VOLPATH):
        s = scenes.cornell_delta_lights(24, 24, area_light=False)
        s.integrator = dict(s.integrator, integrator=integ)
        both = O.OracleScene(s).render(16, seed=3, threads=4)[..., :3]
        s.lights = s.lights[:1]   # the point light alone
        point = O.OracleScene(s).render(16, seed=3, threads=4)[..., :3]
        assert np.isfinite(both).all() and point.sum() > 0
        assert both.sum() > 1.05 * point.sum()
        # image rows run top to bottom; the spot lights the floor around x 0.7
        assert both[-6:, 12:20].mean() > 1.2 * point[-6:, 12:20].mean()
        sums.append(both.sum())
    assert abs(sums[0] - sums[1]) < 0.03 * sums[0]


def test_xml_roundtrip_delta_lights(built, tmp_path):
    """PointLight and SpotLight survive the scene-file round trip (lights
    block after the objects, as the area light comes first), film for film."""
    s = scenes.cornell_delta_lights(16, 12, spot_scale=1.05)
    t = load_scene(write_scene(s, str(tmp_path)))
    assert [L["type"] for L in t.lights] == [L["type"] for L in s.lights]
    fa = O.OracleScene(s).render(2, seed=5, threads=4)
    fb = O.OracleScene(t).render(2, seed=5, threads=4)
    assert np.array_equal(fa, fb)
    # defaults: falloffStart 30, totalWidth 60, intensity black
    text = open(write_scene(s, str(tmp_path / "b"))).read()
    text = text.replace('<double name="falloffStart"', '<double name="ignored1"')
    text = text.replace('<double name="totalWidth"', '<double name="ignored2"')
    open(tmp_path / "c.xml", "w").write(text)
    u = load_scene(str(tmp_path / "c.xml"))
    spot = [L for L in u.lights if L["type"] == D.LIGHT_SPOT][0]
    assert spot["falloff_start"] == 30.0 and spot["total_width"] == 60.0


def test_all_lights_with_one_light_equals_one_light_uniform(built):
    """With a single light, the all-lights loop (PathTracingMIS.cpp:80-117)
    draws the same 2-D sample and takes the same pdf as one-light-uniform
    selection (a one-entry light CDF maps u to itself with weight 1), so the
    oracle's films are identical; with several lights the two strategies
    differ but converge to the same image."""
    s = scenes.cornell_box(24, 20)
    assert len(s.lights) == 1
    o = O.OracleScene(s)
    a = o.render(4, seed=3, strategy=D.STRATEGY_ALL_LIGHTS)
    b = o.render(4, seed=3, strategy=D.STRATEGY_ONE_LIGHT_UNIFORM)
    o.close()
    assert np.array_equal(a, b)
    m = scenes.cornell_delta_lights(16, 16)
    assert len(m.lights) == 3
    o = O.OracleScene(m)
    a = o.render(64, seed=1, strategy=D.STRATEGY_ALL_LIGHTS)
    b = o.render(64, seed=1, strategy=D.STRATEGY_ONE_LIGHT_UNIFORM)
    o.close()
    assert not np.array_equal(a, b)
    ma, mb = a[..., :3].sum() / a[..., 3].sum(), b[..., :3].sum() / b[..., 3].sum()
    assert abs(ma / mb - 1) < 0.05
