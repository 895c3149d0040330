"""Plane (geometricShape/Plane.cpp): the oracle's restatement of the ray test,
the area-light sample and pdf against the reference's formulas written out
here in float64, and the scene-file round trip.  The device side is held to
the oracle in test_gpu_parity.py."""
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


def _planes(s):
    return [i for i, sp in enumerate(s.spheres) if sp.get("kind") == D.ANALYTIC_PLANE]


def test_plane_ray_test(built):
    """Plane::intersection: t = -o.z / d.z in object space (the direction is
    not renormalised, so t is the world distance parameter), inside the
    square [-1,1]^2; uv = ((x + 1) / 2, (y + 1) / 2)."""
    s = scenes.plane_room(8, 8)
    s.meshes, s.indices, s.vertices = [], np.zeros((0, 3), np.int32), np.zeros((0, 3), np.float32)
    floor = _planes(s)[0]
    s.spheres = [s.spheres[floor]]
    s.lights = []
    rng = np.random.default_rng(4)
    n = 20000
    o = np.column_stack([rng.uniform(-2, 3, n), rng.uniform(0.05, 2, n), rng.uniform(-2, 3, n)])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, D.RAY_DTYPE)
    rays["o"], rays["d"], rays["mint"], rays["maxt"] = o, d, 1e-4, 1e8
    M = np.asarray(s.spheres[0]["to_world"], np.float32).astype(np.float64)
    inv = np.linalg.inv(M)
    lo = (inv[:3, :3] @ o.T).T + inv[:3, 3]
    ld = (inv[:3, :3] @ d.T).T
    t = -lo[:, 2] / ld[:, 2]
    q = lo + t[:, None] * ld
    inside = (np.abs(q[:, 0]) <= 1) & (np.abs(q[:, 1]) <= 1)
    want = (t >= 1e-4) & inside
    margin = np.minimum(1 - np.abs(q[:, 0]), 1 - np.abs(q[:, 1]))
    clear = np.abs(margin) > 1e-5
    h = O.OracleScene(s).trace(rays)
    got = h["prim"] == -2
    assert np.array_equal(got[clear], want[clear])
    assert 0.05 < want.mean() < 0.8
    np.testing.assert_allclose(h["t"][got & want], t[got & want], rtol=1e-5)


def test_plane_light_sample_and_pdf(built):
    """A Plane under an AreaLight: Plane::sample maps (u, v) to toWorld
    (1 - 2u, 1 - 2v, 0); ISampledShape::pdf = d^2 / (area cos) with the area
    |toWorld edge 1| |toWorld edge 2|, and the back side gets nothing."""
    s = scenes.plane_room(8, 8)
    li = [i for i, L in enumerate(s.lights) if L["type"] == D.LIGHT_AREA][0]
    sp = s.spheres[s.lights[li]["shape"]]
    M = np.asarray(sp["to_world"], np.float32).astype(np.float64)
    rng = np.random.default_rng(5)
    n = 5000
    p = np.column_stack([rng.uniform(0, 1, n), rng.uniform(0, 1.3, n), rng.uniform(0, 1, n)]).astype(np.float32)
    u = rng.random((n, 2)).astype(np.float32)
    r = O.OracleScene(s).light_query(li, p, u)
    loc = np.column_stack([1 - 2 * u[:, 0].astype(np.float64), 1 - 2 * u[:, 1].astype(np.float64),
                           np.zeros(n), np.ones(n)])
    pt = (M @ loc.T).T[:, :3]
    nrm = np.linalg.inv(M)[:3, :3].T @ np.array([0.0, 0.0, 1.0])
    nrm /= np.linalg.norm(nrm)
    e1 = M[:3, :3] @ np.array([0.0, 2.0, 0.0])
    e2 = M[:3, :3] @ np.array([2.0, 0.0, 0.0])
    area = np.linalg.norm(e1) * np.linalg.norm(e2)
    dv = pt - p
    dist = np.linalg.norm(dv, axis=1)
    w = dv / dist[:, None]
    c = -(w @ nrm)
    front = c > 1e-4
    np.testing.assert_allclose(r["point"], pt, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(r["pdf"][front], (dist ** 2 / (area * c))[front], rtol=1e-4)
    assert np.all(r["pdf"][c < -1e-4] == 0) and np.all(r["intensity"][c < -1e-4] == 0)
    assert 0.2 < front.mean() < 0.9
    np.testing.assert_allclose(r["pdf_eval"][front], r["pdf"][front], rtol=1e-6)


@pytest.mark.parametrize("textured", [False, True])
def test_xml_roundtrip_planes(built, tmp_path, textured):
    """Planes (one of them an area light, one textured) survive the
    scene-file round trip, film for film."""
    s = scenes.plane_room(16, 12, textured=textured)
    t = load_scene(write_scene(s, str(tmp_path)))
    assert [sp.get("kind", 0) for sp in t.spheres] == [sp.get("kind", 0) for sp in s.spheres]
    fa = O.OracleScene(s).render(2, seed=5, threads=4)
    fb = O.OracleScene(t).render(2, seed=5, threads=4)
    assert np.array_equal(fa, fb)
    assert fa[..., :3].sum() > 0
