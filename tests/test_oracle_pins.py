"""Pin the CPU oracle to the reference's own code.

* PCG32 and CDF against tools/Rng.h and core/CDF.{h,cpp} (golden fixtures
  pcg32_ref.json, cdf_ref.json) and the published PCG32 known answer.
* The rest of the hot path against the reference's own sources compiled in
  place with a project-written Eigen-subset shim (oracle/build_oracle.py,
  oracle/ref_hot.cpp): Triangle::intersection, the Mapping warps, Fresnel,
  MicrofacetDistribution, Diffuse / RoughConductor / RoughDielectric /
  SmoothLayeredBSDF eval, pdf and sample, MeshLight, AreaLight on a Sphere,
  EnvironmentLight, HGPhaseFunction, Homogeneous and Heterogeneous (grid)
  sampleDistance / transmittance, on the queries of tests/pin_cases.py
  (golden fixture ref_hot.npz, written by tests/golden/make_golden.py).
  Stated tolerance: triangle hits bit-exact; every other value within 1e-5
  relative.  Measured: every value of every family bit-identical.
* Where the pin library was built on this machine, the same comparison runs
  live on fresh queries.
Plus determinism and physical sanity checks of the restatement."""
import json
import os

import numpy as np
import pytest

import oracle_lib as O
from raytracer_gb300 import desc as D, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _stream(st, sq, n):
    out = np.zeros(n, np.uint32)
    O.lib().oracle_pcg_stream(st, sq, n, O._p(out))
    return out


def test_pcg32_published_known_answer():
    # pcg32 reference demo: seed(42, 54) -> first six outputs
    assert [hex(x) for x in _stream(42, 54, 6)] == [
        "0xa15c02b7", "0x7b47f409", "0xba1d3330", "0x83d2f293", "0xbfa4784b", "0xcbed606e"]


def test_pcg32_matches_reference_rng_h():
    g = json.load(open(os.path.join(GOLDEN, "pcg32_ref.json")))
    assert len(g["streams"]) >= 10
    for s in g["streams"]:
        st, sq = int(s["initstate"]), int(s["initseq"])
        assert list(_stream(st, sq, 64)) == s["u32"]
        f = np.zeros(64, np.float32)
        O.lib().oracle_pcg_reals(st, sq, 64, O._p(f))
        assert list(f.view(np.uint32)) == s["real_bits"]


def test_cdf_matches_reference_cdf_h():
    g = json.load(open(os.path.join(GOLDEN, "cdf_ref.json")))
    for c in g["cases"]:
        pdfs = np.array(c["pdf_bits"], np.uint32).view(np.float32)
        u = np.array(c["u_bits"], np.uint32).view(np.float32)
        idx = np.zeros(len(u), np.int32)
        uo = np.zeros(len(u), np.float32)
        po = np.zeros(len(u), np.float32)
        sm = np.zeros(1, np.float32)
        O.lib().oracle_cdf_sample_reuse(O._p(pdfs), len(pdfs), O._p(u), len(u), O._p(idx), O._p(uo), O._p(po), O._p(sm))
        assert list(idx) == c["index"]
        assert list(uo.view(np.uint32)) == c["u_out_bits"]
        assert list(po.view(np.uint32)) == c["pdf_out_bits"]
        assert int(sm.view(np.uint32)[0]) == c["sum_bits"]
        idx2 = np.zeros(len(u), np.int32)
        po2 = np.zeros(len(u), np.float32)
        O.lib().oracle_cdf_sample(O._p(pdfs), len(pdfs), O._p(u), len(u), O._p(idx2), O._p(po2))
        assert list(idx2) == c["sample_index"]
        assert list(po2.view(np.uint32)) == c["sample_pdf_bits"]


def test_reference_pin_library_agrees_live():
    """Where the reference's Rng.h / CDF.h were compiled on this machine
    (oracle/_ref/libref_pin.so), re-run them live."""
    path = os.path.join(O.ROOT, "oracle", "_ref", "libref_pin.so")
    if not os.path.exists(path):
        pytest.skip("reference pin library not built on this machine")
    import ctypes as C
    L = C.CDLL(path)
    L.ref_pcg_stream.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]
    rng = np.random.default_rng(3)
    for _ in range(20):
        st, sq = int(rng.integers(0, 2 ** 63)), int(rng.integers(0, 2 ** 63))
        ref = np.zeros(100, np.uint32)
        L.ref_pcg_stream(st, sq, 100, ref.ctypes.data)
        assert np.array_equal(ref, _stream(st, sq, 100))


HOT = os.path.join(GOLDEN, "ref_hot.npz")


def _hot_fixture():
    g = np.load(HOT)
    inp = {k[3:]: g[k] for k in g.files if k.startswith("in_")}
    out = {k[4:]: g[k] for k in g.files if k.startswith("out_")}
    return inp, out


def _fields(a):
    if a.dtype.names:
        return [(f, np.asarray(a[f], np.float64)) for f in a.dtype.names if f != "pad"]
    return [("value", a.astype(np.float64))]


def _compare_family(key, ref, mine):
    """Per query: all fields within 1e-5 relative (triangle hits: bit-exact).
    Returns the fraction of bit-identical values."""
    exact = total = 0
    for (f, x), (_, y) in zip(_fields(ref), _fields(mine)):
        x = x.reshape(len(x), -1) if x.ndim > 1 else x.reshape(-1, 1)
        y = y.reshape(x.shape)
        same = (x == y) | (np.isnan(x) & np.isnan(y))
        exact += int(same.sum())
        total += same.size
        if key.startswith("tri"):
            assert same.all(), "%s.%s not bit-exact" % (key, f)
        else:
            tol = 1e-5 * np.maximum(np.abs(x), np.abs(y))
            ok = same | (np.abs(x - y) <= tol)
            assert ok.all(), "%s.%s: %d values beyond 1e-5 relative" % (key, f, int((~ok).sum()))
    return exact / max(total, 1)


@pytest.fixture(scope="module")
def hot():
    import pin_cases
    inp, ref = _hot_fixture()
    return ref, pin_cases.run("oracle", inp)


HOT_KEYS = sorted(k[4:] for k in np.load(HOT).files if k.startswith("out_"))


@pytest.mark.parametrize("key", HOT_KEYS)
def test_oracle_matches_reference_hot_path(hot, key):
    ref, mine = hot
    frac = _compare_family(key, ref[key], mine[key])
    print("%s: %.4f of values bit-identical" % (key, frac))


def test_reference_hot_path_agrees_live():
    """Where the reference's hot-path sources were compiled on this machine
    (oracle/_ref/libref_hot.so, built when the reference tree is given),
    compare on 4,096 fresh queries per family."""
    import ctypes as C
    import pin_cases
    path = os.path.join(O.ROOT, "oracle", "_ref", "libref_hot.so")
    if not os.path.exists(path):
        pytest.skip("reference pin library not built on this machine")
    inp = pin_cases.inputs(n=4096, seed=99)
    ref = pin_cases.run(C.CDLL(path), inp)
    mine = pin_cases.run("oracle", inp)
    for key in sorted(ref):
        _compare_family(key, ref[key], mine[key])


PATHS = os.path.join(GOLDEN, "ref_paths.npz")


@pytest.mark.parametrize("case", [0, 1, 2], ids=["cornell", "icosphere", "volume"])
def test_oracle_paths_match_reference_integrator(case):
    """Every path sample of small renders of the three configurations' scene
    families, against the reference's own PathTracingMIS::li /
    VolPathTracing::li over its own BVH (ref_paths.npz).  Stated tolerance:
    per-path radiance within 1e-5 relative for every path.  Measured:
    bit-identical."""
    import pin_cases
    name, scene, spp = pin_cases.film_scenes()[case]
    gold = np.load(PATHS)
    assert str(gold[name + "_digest"]) == pin_cases.scene_digest(scene), \
        "the scene generator changed: regenerate tests/golden/ref_paths.npz"
    pix, smp = pin_cases.all_paths(scene, spp)
    ref = gold[name + "_rad"]
    mine = O.OracleScene(scene).render_paths(pix, smp, seed=0)
    same = np.all(ref == mine, axis=1)
    rel = np.abs(ref - mine) / np.maximum(np.maximum(np.abs(ref), np.abs(mine)), 1e-30)
    print("%s: %d paths, %.4f bit-identical, max rel %.2e" % (name, len(pix), same.mean(), rel.max()))
    assert np.all(same[:, None] | (rel <= 1e-5))


def test_oracle_paths_match_reference_integrator_live():
    """Where the reference pin library was built on this machine: larger
    renders (the Cornell box at its full 256x256, a level-6 icosphere, a 64^3
    grid), path by path."""
    import ctypes as C
    import pin_cases
    path = os.path.join(O.ROOT, "oracle", "_ref", "libref_hot.so")
    if not os.path.exists(path):
        pytest.skip("reference pin library not built on this machine")
    L = C.CDLL(path)
    for scene, spp in [(scenes.cornell_box(256, 256), 1),
                       (scenes.displaced_icosphere(level=6, width=64, height=64, env_size=(256, 128)), 2),
                       (scenes.volume_grid(64, 48, res=64), 2)]:
        pix, smp = pin_cases.all_paths(scene, spp)
        ref = pin_cases.reference_paths(L, scene, pix, smp, seed=3)
        mine = O.OracleScene(scene).render_paths(pix, smp, seed=3)
        same = np.all(ref == mine, axis=1)
        rel = np.abs(ref - mine) / np.maximum(np.maximum(np.abs(ref), np.abs(mine)), 1e-30)
        print("%s: %d paths, %.4f bit-identical" % (scene.name, len(pix), same.mean()))
        assert np.all(same[:, None] | (rel <= 1e-5))


def test_oracle_render_is_thread_count_independent():
    s = scenes.cornell_box(40, 24)
    o = O.OracleScene(s)
    a = o.render(3, seed=5, threads=1, block=16)
    b = o.render(3, seed=5, threads=7, block=16)
    assert np.array_equal(a, b)
    assert a[..., 3].min() >= 2 and a[..., 3].max() <= 4   # box-filter weights


def _q(wi, wo=None, u=None):
    q = np.zeros(len(wi), O.BSDF_Q)
    q["wi"] = wi
    if wo is not None:
        q["wo"] = wo
    if u is not None:
        q["u"] = u
    return q


def _sphere_dirs(n, rng, upper=True):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    if upper:
        v[:, 2] = np.abs(v[:, 2])
    return v.astype(np.float32)


def test_diffuse_furnace_and_pdf():
    rng = np.random.default_rng(0)
    b = D.bsdf(D.BSDF_DIFFUSE, albedo=(0.3, 0.6, 0.9))
    wi = _sphere_dirs(4000, rng)
    r = O.bsdf_query(b, D.BSDF_OP_SAMPLE, _q(wi, u=rng.random((4000, 2))))
    assert np.allclose(r["value"], [0.3, 0.6, 0.9])
    assert np.allclose(r["pdf"], r["wo"][:, 2] / np.pi, rtol=1e-6)
    # eval * cos / pdf == albedo along sampled directions
    e = O.bsdf_query(b, D.BSDF_OP_EVAL, _q(wi, r["wo"]))
    ok = r["pdf"] > 1e-3
    assert np.allclose(e["value"][ok] * r["wo"][ok, 2:3] / r["pdf"][ok, None], [0.3, 0.6, 0.9], rtol=1e-5)


def test_rough_conductor_estimator_consistency():
    """sample() weight == eval * |cos| / pdf for the reference's RoughConductor."""
    rng = np.random.default_rng(1)
    for dist in (D.DIST_BECKMANN, D.DIST_GGX, D.DIST_PHONG):
        b = D.bsdf(D.BSDF_ROUGH_CONDUCTOR, distribution=dist, alpha=0.3 if dist != D.DIST_PHONG else 20.0,
                   eta=scenes.AU_ETA, k=scenes.AU_K)
        wi = _sphere_dirs(2000, rng)
        r = O.bsdf_query(b, D.BSDF_OP_SAMPLE, _q(wi, u=rng.random((2000, 2))))
        ok = (r["pdf"] > 1e-2) & (np.abs(r["value"]).sum(1) > 0)
        assert ok.sum() > 200
        e = O.bsdf_query(b, D.BSDF_OP_EVAL, _q(wi[ok], r["wo"][ok]))
        p = O.bsdf_query(b, D.BSDF_OP_PDF, _q(wi[ok], r["wo"][ok]))
        assert np.allclose(p["pdf"], r["pdf"][ok], rtol=1e-5)
        est = e["value"] * np.abs(r["wo"][ok, 2:3]) / p["pdf"][:, None]
        assert np.allclose(est, r["value"][ok], rtol=1e-4)


def test_fresnel_normal_incidence_of_smooth_coat():
    # SmoothLayered reflects with probability Fr(normal) = ((n-1)/(n+1))^2
    b = D.bsdf(D.BSDF_SMOOTH_LAYERED, eta_int=1.5, eta_ext=1.0)
    fr = ((1.5 - 1.0) / 2.5) ** 2
    r = O.bsdf_query(b, D.BSDF_OP_SAMPLE, _q(np.array([[0, 0, 1]] * 2, np.float32),
                                             u=np.array([[fr * 0.99, 0.3], [fr * 1.01, 0.3]], np.float32)))
    assert r["sampled_type"][0] == 2 and np.isclose(r["pdf"][0], fr, rtol=1e-6)   # delta reflection
    assert r["sampled_type"][1] == 0                                              # through the coat


def test_smooth_dielectric_fresnel_and_snell():
    """Dielectric.cpp:28-82: reflect with probability Fr, else refract by
    Snell's law with weight transmittance * eta^2; total internal reflection
    from inside past the critical angle."""
    n = 1.5
    b = D.bsdf(D.BSDF_DIELECTRIC, eta_int=n, eta_ext=1.0, transmittance=(0.9, 0.8, 0.7), reflectance=(0.5, 0.6, 0.7))
    fr = ((n - 1.0) / (n + 1.0)) ** 2
    up = np.array([[0, 0, 1]] * 2, np.float32)
    r = O.bsdf_query(b, D.BSDF_OP_SAMPLE, _q(up, u=np.array([[fr * 0.99, 0.5], [fr * 1.01, 0.5]], np.float32)))
    assert r["sampled_type"][0] == 2 and np.isclose(r["pdf"][0], fr, rtol=1e-5)
    assert np.allclose(r["value"][0], [0.5, 0.6, 0.7]) and np.allclose(r["wo"][0], [0, 0, 1])
    assert r["sampled_type"][1] == 8 and np.isclose(r["pdf"][1], 1 - fr, rtol=1e-5)
    assert np.allclose(r["value"][1], np.array([0.9, 0.8, 0.7]) / n / n, rtol=1e-6)
    assert np.allclose(r["wo"][1], [0, 0, -1]) and np.isclose(r["relative_eta"][1], 1 / n)
    rng = np.random.default_rng(3)
    wi = _sphere_dirs(4000, rng, upper=False)
    r = O.bsdf_query(b, D.BSDF_OP_SAMPLE, _q(wi, u=np.full((4000, 2), 0.999, np.float32)))
    inside = wi[:, 2] <= 0
    rel = np.where(inside, n, 1 / n)
    sin_t = rel * np.sqrt(np.maximum(0, 1 - wi[:, 2].astype(np.float64) ** 2))
    tir = sin_t >= 1
    assert np.all(r["sampled_type"][tir] == 2) and np.all(r["pdf"][tir] == 1)
    t = ~tir & (r["sampled_type"] == 8)
    assert t.sum() > 1000
    # Snell: tangential components scale by eta_i / eta_t, the side flips
    assert np.allclose(r["wo"][t, :2], -rel[t, None] * wi[t, :2], rtol=1e-5, atol=1e-6)
    assert np.all(np.sign(r["wo"][t, 2]) == -np.sign(wi[t, 2]))
    assert np.allclose(np.linalg.norm(r["wo"][t], axis=1), 1, atol=1e-5)
    for op in (D.BSDF_OP_EVAL, D.BSDF_OP_PDF):
        e = O.bsdf_query(b, op, _q(wi, -wi))
        assert not np.any(e["value"]) and not np.any(e["pdf"])


def test_smooth_conductor_and_mirror():
    """Conductor.cpp:39-53 (reflectance * per-channel Fresnel), Mirror.cpp:31-43."""
    rng = np.random.default_rng(4)
    wi = _sphere_dirs(1000, rng, upper=False)
    eta, k = np.array(scenes.AU_ETA), np.array(scenes.AU_K)
    c = D.bsdf(D.BSDF_CONDUCTOR, eta=tuple(eta), k=tuple(k), reflectance=(0.9, 1.0, 0.8))
    r = O.bsdf_query(c, D.BSDF_OP_SAMPLE, _q(wi, u=rng.random((1000, 2))))
    up = wi[:, 2] > 0
    ci = wi[up, 2:3].astype(np.float64)
    epa = eta * eta + k * k
    rpar = (epa * ci * ci - 2 * eta * ci + 1) / (epa * ci * ci + 2 * eta * ci + 1)
    rperp = (epa - 2 * eta * ci + ci * ci) / (epa + 2 * eta * ci + ci * ci)
    assert np.allclose(r["value"][up], np.array([0.9, 1.0, 0.8]) * (rpar ** 2 + rperp ** 2) / 2, rtol=1e-5)
    assert np.all(r["value"][~up] == 0)
    assert np.allclose(r["wo"][up], wi[up] * [-1, -1, 1]) and np.all(r["pdf"][up] == 1)
    m = O.bsdf_query(D.bsdf(D.BSDF_MIRROR), D.BSDF_OP_SAMPLE, _q(wi, u=rng.random((1000, 2))))
    assert np.all(m["value"][up] == 1) and np.all(m["value"][~up] == 0)
    assert np.all(m["sampled_type"][up] == 2)


@pytest.mark.parametrize("kind", [D.BSDF_DIFFUSE, D.BSDF_ROUGH_CONDUCTOR, D.BSDF_CONDUCTOR, D.BSDF_DIELECTRIC])
def test_two_sides_mirrors_the_lower_side(kind):
    """TwoSides.cpp:22-70: from below, the wrapped BSDF sees both directions
    with z negated, and a sampled direction comes back with z negated."""
    rng = np.random.default_rng(5 + kind)
    one = D.bsdf(kind, eta=scenes.AU_ETA, k=scenes.AU_K, distribution=D.DIST_GGX, alpha=0.3)
    two = dict(one, two_sided=True)
    wi = _sphere_dirs(3000, rng, upper=True)
    wo = _sphere_dirs(3000, rng, upper=False)
    u = rng.random((3000, 2)).astype(np.float32)
    flip = np.array([1, 1, -1], np.float32)
    for op, f in ((D.BSDF_OP_EVAL, "value"), (D.BSDF_OP_PDF, "pdf")):
        a = O.bsdf_query(two, op, _q(wi * flip, wo * flip, u))   # wi below
        b = O.bsdf_query(one, op, _q(wi, wo, u))
        assert np.array_equal(a[f], b[f])
    below = wi * flip
    a = O.bsdf_query(two, D.BSDF_OP_SAMPLE, _q(below, u=u))
    b = O.bsdf_query(one, D.BSDF_OP_SAMPLE, _q(wi, u=u))
    assert np.array_equal(a["value"], b["value"]) and np.array_equal(a["pdf"], b["pdf"])
    assert np.array_equal(a["wo"], b["wo"] * flip)
    # from above it is the wrapped BSDF itself
    c = O.bsdf_query(two, D.BSDF_OP_SAMPLE, _q(wi, u=u))
    assert np.array_equal(c["value"], b["value"]) and np.array_equal(c["wo"], b["wo"])


def test_triangle_hit_exactness_small_scene():
    s = scenes.cornell_box(16, 16)
    o = O.OracleScene(s)
    rays = np.zeros(3, D.RAY_DTYPE)
    rays["o"] = [(0.5, 0.5, 0.5), (0.8, 0.8, 0.5), (0.2, 0.9, 0.5)]
    rays["d"] = [(0, -1, 0), (0, 0, -1), (0, 1, 0)]
    rays["mint"] = 1e-4
    rays["maxt"] = 1e8
    h = o.trace(rays)
    assert np.allclose(h["t"], [0.5, 0.5, 0.1], atol=1e-6)
    assert (h["prim"] >= 0).all()
    a = o.trace(rays, anyhit=True)
    assert (a["prim"] == 0).all()


def test_microfacet_estimator_and_sheet_dielectric():
    """Microfacet.cpp:120-182: the sample weight is eval |cos| / pdf and the
    sample's pdf is pdf(); SheetDielectric.cpp:122-174: reflection with
    probability fr + T^2 fr / (1 - fr^2), else straight through, typed
    UNKNOWN (not delta)."""
    rng = np.random.default_rng(9)
    for dist in (D.DIST_GGX, D.DIST_BECKMANN):
        b = D.bsdf(D.BSDF_MICROFACET, albedo=(0.6, 0.4, 0.2), ks=0.4, alpha=0.3, distribution=dist)
        wi = _sphere_dirs(3000, rng)
        r = O.bsdf_query(b, D.BSDF_OP_SAMPLE, _q(wi, u=rng.random((3000, 2))))
        ok = (r["pdf"] > 1e-2) & (np.abs(r["value"]).sum(1) > 0)
        assert ok.sum() > 1000
        assert set(np.unique(r["sampled_type"][ok])) <= {4, 0x200}   # glossy or diffuse lobe
        e = O.bsdf_query(b, D.BSDF_OP_EVAL, _q(wi[ok], r["wo"][ok]))
        p = O.bsdf_query(b, D.BSDF_OP_PDF, _q(wi[ok], r["wo"][ok]))
        assert np.allclose(p["pdf"], r["pdf"][ok], rtol=1e-5)
        assert np.allclose(e["value"] * np.abs(r["wo"][ok, 2:3]) / p["pdf"][:, None], r["value"][ok], rtol=1e-4)
    n = 1.5
    s = D.bsdf(D.BSDF_SHEET_DIELECTRIC, eta_int=n, eta_ext=1.0, transmittance=(0.9, 0.8, 0.7))
    fr = ((n - 1) / (n + 1)) ** 2
    fr_sheet = fr + (1 - fr) ** 2 * fr / (1 - fr * fr)
    wi = np.array([[0, 0, 1]] * 2 + [[0.3, 0.1, -0.9]], np.float32)
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    r = O.bsdf_query(s, D.BSDF_OP_SAMPLE, _q(wi, u=np.array([[fr_sheet * 0.99, 0.5], [fr_sheet * 1.01, 0.5],
                                                               [0.99, 0.5]], np.float32)))
    assert r["sampled_type"][0] == 2 and np.isclose(r["pdf"][0], fr_sheet, rtol=1e-5)
    assert r["sampled_type"][1] == 0 and np.isclose(r["pdf"][1], 1 - fr_sheet, rtol=1e-5)
    assert np.allclose(r["wo"][1], -wi[1]) and np.allclose(r["wo"][2], -wi[2])
    assert np.allclose(r["value"][1], [0.9, 0.8, 0.7]) and np.all(r["relative_eta"] == 1)
