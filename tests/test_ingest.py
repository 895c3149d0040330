"""Scene ingestion on the host (no GPU): OBJ meshes read by the library's
C++ loader with the reference ObjLoader's rules, Radiance .hdr maps,
GridVolume files, and reference XML scene files written by scene_export and
read back by xml_scene, which must give the same SceneData and, through the
oracle, the same film."""
import os

import numpy as np
import pytest

import raytracer_gb300 as R
from raytracer_gb300 import desc as D
from raytracer_gb300 import scenes
from raytracer_gb300.scene_export import encode_rgbe, write_hdr, write_scene, write_vol
from raytracer_gb300.xml_scene import UnsupportedScene, load_scene, load_vol


@pytest.fixture(scope="module")
def built():
    from raytracer_gb300 import build
    return build.build()


OBJ = """# quads, triangles, negative indices, missing uv / normal indices
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0 0 1
vt 0.25 0.5
vt 0.75 0.5
vn 0 0 1
vn 0 1 0
f 1/1/1 2/2/1 3/1/1 4/2/1
f -1//2 1//2 2
  f 5 3 4
"""


def _ref_obj(text, M):
    """The reference ObjLoader's rules restated in numpy for the test."""
    P, N, T, corners, idx, cmap = [], [], [], [], [], {}
    M = np.asarray(M, np.float32)
    NI = np.linalg.inv(M[:3, :3].astype(np.float64)).T.astype(np.float32)
    for line in text.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            p = np.array([float(x) for x in t[1:4]], np.float32)
            q = [((M[r, 0] * p[0] + M[r, 1] * p[1]) + M[r, 2] * p[2]) + M[r, 3] for r in range(4)]
            w = q[3]
            P.append([q[0] / w, q[1] / w, q[2] / w] if w not in (0, 1) else q[:3])
        elif t[0] == "vn":
            n = np.array([float(x) for x in t[1:4]], np.float32)
            N.append([(NI[r, 0] * n[0] + NI[r, 1] * n[1]) + NI[r, 2] * n[2] for r in range(3)])
        elif t[0] == "vt":
            T.append([float(x) for x in t[1:3]])
        elif t[0] == "f":
            cs = []
            for tok in t[1:5]:
                parts = tok.split("/")
                c = [int(parts[0]), 1, 1]
                if len(parts) > 1 and parts[1]:
                    c[1] = int(parts[1])
                if len(parts) > 2 and parts[2]:
                    c[2] = int(parts[2])
                cs.append(tuple(c))
            tri = cs[:3] + ([cs[3], cs[0], cs[2]] if len(cs) > 3 else [])
            for c in tri:
                if c not in cmap:
                    cmap[c] = len(corners)
                    corners.append(c)
                idx.append(cmap[c])
    res = lambda i, n: n + i + 1 if i < 0 else i
    v = np.array([P[res(c[0], len(P)) - 1] for c in corners], np.float32)
    n = np.array([N[res(c[2], len(N)) - 1] for c in corners], np.float32) if N else None
    uv = np.array([T[res(c[1], len(T)) - 1] for c in corners], np.float32) if T else None
    return v, n, uv, np.array(idx, np.int32).reshape(-1, 3)


def test_obj_loader_follows_reference_rules(built, tmp_path):
    path = tmp_path / "m.obj"
    path.write_text(OBJ)
    M = np.array([[0, -2, 0, 1], [2, 0, 0, -3], [0, 0, 0.5, 0.25], [0, 0, 0, 1]], np.float32)
    for tw in (None, M):
        v, n, uv, t = R.load_obj(str(path), tw)
        ev, en, euv, et = _ref_obj(OBJ, np.eye(4) if tw is None else tw)
        assert np.array_equal(t, et)
        assert np.array_equal(v, ev)
        np.testing.assert_allclose(n, en, rtol=1e-6, atol=1e-7)
        assert np.array_equal(uv, euv)
    assert t.tolist()[:2] == [[0, 1, 2], [3, 0, 2]]          # quad split (a b c) (d a c)
    with pytest.raises(R.RtError):
        R.load_obj(str(tmp_path / "missing.obj"))
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2\n")
    with pytest.raises(R.RtError):
        R.load_obj(str(bad))


def _rle_scanlines(rgbe):
    """Adaptive run-length encoding of RGBE scanlines (runs for repeats)."""
    h, w = rgbe.shape[:2]
    out = bytearray()
    for y in range(h):
        out += bytes([2, 2, w >> 8, w & 255])
        for k in range(4):
            row = rgbe[y, :, k]
            x = 0
            while x < w:
                r = 1
                while x + r < w and r < 127 and row[x + r] == row[x]:
                    r += 1
                if r >= 3:
                    out += bytes([128 + r, row[x]])
                    x += r
                else:
                    lit = min(128, w - x)
                    out += bytes([lit]) + bytes(row[x:x + lit])
                    x += lit
    return bytes(out)


def test_hdr_loader_flat_and_rle(built, tmp_path):
    rng = np.random.default_rng(1)
    img = (rng.random((9, 40, 3)) ** 3 * 50).astype(np.float32)
    img[2, 5:30] = img[2, 5]                                     # runs
    img[4, :] = 0.0
    rgbe = encode_rgbe(img)
    e = rgbe[..., 3].astype(np.int64)
    expect = np.where(e[..., None] > 0, rgbe[..., :3] * np.ldexp(1.0, e - 136)[..., None], 0).astype(np.float32)
    write_hdr(str(tmp_path / "flat.hdr"), img)
    assert np.array_equal(R.load_hdr(str(tmp_path / "flat.hdr")), expect)
    with open(tmp_path / "rle.hdr", "wb") as f:
        f.write(b"#?RGBE\n# comment\nFORMAT=32-bit_rle_rgbe\n\n-Y 9 +X 40\n" + _rle_scanlines(rgbe))
    assert np.array_equal(R.load_hdr(str(tmp_path / "rle.hdr")), expect)
    # RGBE keeps 8 bits of the largest channel: error below one quantum of it
    assert np.all(np.abs(expect - img) <= img.max(-1, keepdims=True) * 2.0 ** -7)
    (tmp_path / "x.hdr").write_bytes(b"P6\n")
    with pytest.raises(R.RtError):
        R.load_hdr(str(tmp_path / "x.hdr"))


def test_vol_file_layout(tmp_path):
    d = np.random.default_rng(2).random((3, 4, 5)).astype(np.float32)
    write_vol(str(tmp_path / "g.vol"), d, (0, 1, 2), (3, 4, 5))
    got, lo, hi = load_vol(str(tmp_path / "g.vol"))
    assert np.array_equal(got, d) and lo == (0, 1, 2) and hi == (3, 4, 5)


def _same_scene(a, b):
    # the OBJ files renumber vertices in order of first use; triangles and
    # their corners keep their order
    assert np.array_equal(a.vertices[a.indices], b.vertices[b.indices])
    assert (a.normals is None) == (b.normals is None)
    if a.normals is not None:
        na, nb = a.normals[a.indices], b.normals[b.indices]
        assert np.array_equal(np.isnan(na), np.isnan(nb))
        m = ~np.isnan(na)
        np.testing.assert_allclose(na[m], nb[m], rtol=1e-6)
    assert len(a.meshes) == len(b.meshes) and len(a.lights) == len(b.lights)
    def same_bsdf(i, j):
        assert (i < 0) == (j < 0)
        if i >= 0:
            x, y = a.bsdfs[i], b.bsdfs[j]
            for k in x:
                np.testing.assert_allclose(np.asarray(x[k], np.float32), np.asarray(y[k], np.float32), rtol=1e-6)
    # the file gives every shape its own BSDF; compare the BSDF each refers to
    for x, y in zip(a.meshes, b.meshes):
        assert {k: v for k, v in x.items() if k != "bsdf"} == {k: v for k, v in y.items() if k != "bsdf"}
        same_bsdf(x["bsdf"], y["bsdf"])
    for x, y in zip(a.spheres, b.spheres):
        same_bsdf(x["bsdf"], y["bsdf"])
    for x, y in zip(a.lights, b.lights):
        assert x["type"] == y["type"]
    ca, cb = a.camera, b.camera
    assert ca["width"] == cb["width"] and ca["height"] == cb["height"]
    np.testing.assert_array_equal(np.asarray(ca["camera_to_world"], np.float32),
                                  np.asarray(cb["camera_to_world"], np.float32))
    assert a.integrator == b.integrator


def _films_equal(a, b, spp=2):
    import oracle_lib as O
    fa = O.OracleScene(a).render(spp, seed=5, threads=4)
    fb = O.OracleScene(b).render(spp, seed=5, threads=4)
    return fa, fb


def test_xml_roundtrip_cornell(built, tmp_path):
    s = scenes.cornell_box(24, 16)
    xmlp = write_scene(s, str(tmp_path), spp=4)
    t = load_scene(xmlp)
    assert t.spp == 4 and t.block == (32, 32)
    _same_scene(s, t)
    fa, fb = _films_equal(s, t)
    assert np.array_equal(fa, fb)


def test_xml_roundtrip_layered(built, tmp_path):
    s = scenes.cornell_box(16, 12)
    ly = s.add_bsdf(D.bsdf(D.BSDF_LAYERED, distribution=D.DIST_GGX, alpha=0.05, eta=scenes.AU_ETA, k=scenes.AU_K,
                           distribution_base=D.DIST_GGX, alpha_base=0.25, thickness=0.5, absorbance=(0.1, 0.2, 0.3)))
    s.meshes[3]["bsdf"] = ly
    t = load_scene(write_scene(s, str(tmp_path)))
    _same_scene(s, t)
    fa, fb = _films_equal(s, t)
    assert np.array_equal(fa, fb)


@pytest.mark.parametrize("flt", [D.gaussian_filter(1.5, 1.5), D.mitchell_filter(2.0, 1.0)], ids=["gauss", "mitchell"])
def test_xml_roundtrip_filter(built, tmp_path, flt):
    s = scenes.cornell_box(20, 14)
    s.camera["filter"] = flt
    t = load_scene(write_scene(s, str(tmp_path)))
    assert t.camera["filter"]["type"] == flt["type"]
    np.testing.assert_allclose(t.camera["filter"]["param"], flt["param"], rtol=1e-6)
    fa, fb = _films_equal(s, t)
    assert np.array_equal(fa, fb)


def test_xml_roundtrip_volume(built, tmp_path):
    s = scenes.volume_grid(20, 16, res=12)
    xmlp = write_scene(s, str(tmp_path))
    t = load_scene(xmlp)
    _same_scene(s, t)
    assert len(t.media) >= 2 and t.media[0]["type"] == D.MEDIUM_HETEROGENEOUS
    assert np.array_equal(t.media[0]["density"], s.media[0]["density"])
    fa, fb = _films_equal(s, t, spp=1)
    assert np.array_equal(fa, fb)


def test_xml_roundtrip_sky_quantised(built, tmp_path):
    s = scenes.displaced_icosphere(level=2, width=16, height=16, env_size=(64, 32))
    xmlp = write_scene(s, str(tmp_path))
    t = load_scene(xmlp)
    _same_scene(s, t)
    env = s.lights[s.env_light]["rgb"]
    rgbe = encode_rgbe(env)
    e = rgbe[..., 3].astype(np.int64)
    expect = np.where(e[..., None] > 0, rgbe[..., :3] * np.ldexp(1.0, e - 136)[..., None], 0).astype(np.float32)
    assert np.array_equal(t.lights[t.env_light]["rgb"], expect)


def test_xml_unsupported_and_quirks(built, tmp_path):
    s = scenes.cornell_box(8, 8)
    xmlp = write_scene(s, str(tmp_path))
    text = open(xmlp).read()
    open(tmp_path / "f.xml", "w").write(text.replace('<filter type="BoxFilter">', '<filter type="LanczosFilter">'))
    with pytest.raises(UnsupportedScene):
        load_scene(str(tmp_path / "f.xml"))
    open(tmp_path / "b.xml", "w").write(text.replace('type="Diffuse"', 'type="Phong"', 1))
    with pytest.raises(UnsupportedScene):
        load_scene(str(tmp_path / "b.xml"))
    # a 1-value colour is an error that the reference turns into black
    open(tmp_path / "c.xml", "w").write(text.replace('name="albedo" value="', 'name="albedo" value="0.5" x="', 1))
    with pytest.warns(UserWarning):
        t = load_scene(str(tmp_path / "c.xml"))
    assert tuple(t.bsdfs[0]["albedo"]) == (0.0, 0.0, 0.0)


def test_xml_roundtrip_smooth_bsdfs(built, tmp_path):
    """Dielectric, Conductor, Mirror and TwoSides-wrapped Diffuse and
    RoughConductor survive the file round trip, film for film."""
    s = scenes.cornell_smooth(16, 12)
    t = load_scene(write_scene(s, str(tmp_path)))
    _same_scene(s, t)
    kinds = {b["type"] for b in t.bsdfs}
    assert {D.BSDF_DIELECTRIC, D.BSDF_CONDUCTOR, D.BSDF_MIRROR} <= kinds
    assert any(b.get("two_sided") for b in t.bsdfs)
    fa, fb = _films_equal(s, t)
    assert np.array_equal(fa, fb)


def test_xml_two_sides_forms(built, tmp_path):
    """TwoSides over a nested or referenced BSDF (a referenced BSDF keeps the
    name of its top-level element, XMLLoader.cpp:762-775); a different bsdf2
    is not provided."""
    s = scenes.cornell_box(8, 8)
    text = open(write_scene(s, str(tmp_path))).read()
    first = text.index('<bsdf type="Diffuse">')
    end = text.index("</bsdf>", first) + len("</bsdf>")
    inner = text[first:end]
    nested = '<bsdf type="TwoSides">' + inner.replace('<bsdf type=', '<bsdf name="bsdf" type=') + "</bsdf>"
    open(tmp_path / "n.xml", "w").write(text[:first] + nested + text[end:])
    t = load_scene(str(tmp_path / "n.xml"))
    b = t.bsdfs[t.meshes[0]["bsdf"]]
    assert b["two_sided"] and b["type"] == D.BSDF_DIFFUSE and np.allclose(b["albedo"], s.bsdfs[0]["albedo"])
    top = inner.replace('<bsdf type=', '<bsdf id="wall" name="bsdf" type=')
    ref = '<bsdf type="TwoSides"><bsdf ref="wall"/></bsdf>'
    body = text[:first] + ref + text[end:]
    body = body.replace("<objects>", top + "\n<objects>", 1)
    open(tmp_path / "r.xml", "w").write(body)
    t = load_scene(str(tmp_path / "r.xml"))
    assert t.bsdfs[t.meshes[0]["bsdf"]]["two_sided"]
    two = nested.replace("</bsdf></bsdf>", '</bsdf><bsdf name="bsdf2" type="Mirror"/></bsdf>')
    open(tmp_path / "m.xml", "w").write(text[:first] + two + text[end:])
    with pytest.raises(UnsupportedScene):
        load_scene(str(tmp_path / "m.xml"))


def test_conductor_material_names(built, tmp_path):
    """material="gold" (and the other seven names of tools/Common.cpp:44-54)
    gives the RGB eta/k the reference converts from its data/IOR spectra;
    a caller's materials= mapping overrides; an unknown name falls back to
    the eta and absorption colors with a warning, as in the reference."""
    from raytracer_gb300.conductor_ior import MATERIALS
    assert set(MATERIALS) == {"gold", "silver", "aluminium", "copper", "chromium", "iron", "nickel", "tin"}
    s = scenes.cornell_box(8, 8)
    s.meshes[3]["bsdf"] = s.add_bsdf(D.bsdf(D.BSDF_ROUGH_CONDUCTOR, eta=(0.5, 0.5, 0.5), k=(1, 1, 1)))
    text = open(write_scene(s, str(tmp_path))).read()
    i = text.index('<bsdf type="RoughConductor">') + len('<bsdf type="RoughConductor">')
    named = text[:i] + '<string name="material" value="gold"/>' + text[i:]
    open(tmp_path / "g.xml", "w").write(named)
    t = load_scene(str(tmp_path / "g.xml"))
    b = t.bsdfs[t.meshes[3]["bsdf"]]
    assert np.allclose(b["eta"], MATERIALS["gold"][0]) and np.allclose(b["k"], MATERIALS["gold"][1])
    t = load_scene(str(tmp_path / "g.xml"), materials={"gold": ((1, 2, 3), (4, 5, 6))})
    assert tuple(t.bsdfs[t.meshes[3]["bsdf"]]["eta"]) == (1, 2, 3)
    open(tmp_path / "u.xml", "w").write(named.replace('value="gold"', 'value="unobtainium"'))
    with pytest.warns(UserWarning):
        t = load_scene(str(tmp_path / "u.xml"))
    assert np.allclose(t.bsdfs[t.meshes[3]["bsdf"]]["eta"], (0.5, 0.5, 0.5))


def test_conductor_table_matches_the_reference_data():
    """The committed table is what make_conductor_ior.py computes from the
    reference's spectra and CIE tables (where the reference tree exists)."""
    import os
    from raytracer_gb300 import make_conductor_ior as M
    from raytracer_gb300.conductor_ior import MATERIALS
    import __graft_entry__
    root = os.environ.get("RT_REFERENCE_ROOT") or os.path.dirname(__graft_entry__.REFERENCE_SRC)
    if not os.path.isdir(os.path.join(root, "data", "IOR")):
        pytest.skip("reference tree not present")
    assert M.compute(root) == MATERIALS
    # gold lands where published RGB fits of Au do (eta low in red, k ~ 4, 2.4, 1.6)
    eta, k = MATERIALS["gold"]
    assert 0.1 < eta[0] < 0.2 and 1.3 < eta[2] < 1.6 and 3.8 < k[0] < 4.1


def test_type_names_ignore_case(built, tmp_path):
    """The reference's factories match type names without regard to case
    (ObjectFactoryManager::formatType): a file written with lower-case type
    names loads to the same scene."""
    import re
    s = scenes.cornell_smooth(16, 12)
    text = open(write_scene(s, str(tmp_path))).read()
    lower = re.sub(r'type="([A-Za-z]+)"', lambda m: 'type="%s"' % m.group(1).lower(), text)
    assert lower != text
    open(tmp_path / "lower.xml", "w").write(lower)
    t = load_scene(str(tmp_path / "lower.xml"))
    _same_scene(s, t)
    fa, fb = _films_equal(s, t)
    assert np.array_equal(fa, fb)


def test_exr_environment_map_and_stratified_sampler(built, tmp_path):
    """EnvironmentLight reads its image through ImageLoader (EXR linear);
    a StratifiedSampler file loads with a warning, its sample count kept."""
    from raytracer_gb300.exr import write_exr
    s = scenes.displaced_icosphere(level=1, width=8, height=8, env_size=(32, 16))
    text = open(write_scene(s, str(tmp_path), spp=6)).read()
    env = s.lights[s.env_light]["rgb"]
    write_exr(str(tmp_path / "sky.exr"), env)
    i = text.index('.hdr"')
    j = text.rindex('"', 0, i)
    text = text[:j + 1] + "sky.exr" + text[i + 4:]
    open(tmp_path / "e.xml", "w").write(text.replace('type="RandomSampler"', 'type="StratifiedSampler"'))
    with pytest.warns(UserWarning):
        t = load_scene(str(tmp_path / "e.xml"))
    assert t.spp == 6
    with np.errstate(over="ignore"):
        expect = env.astype(np.float16).astype(np.float32)
    assert np.array_equal(t.lights[t.env_light]["rgb"], expect)


def test_xml_roundtrip_sheet_and_microfacet(built, tmp_path):
    s = scenes.cornell_smooth(16, 12)
    s.meshes[0]["bsdf"] = s.add_bsdf(D.bsdf(D.BSDF_MICROFACET, albedo=(0.6, 0.55, 0.5), ks=0.35, alpha=0.25))
    s.meshes[6]["bsdf"] = s.add_bsdf(D.bsdf(D.BSDF_SHEET_DIELECTRIC, eta_int=1.45, transmittance=(0.8, 0.9, 1.0)))
    t = load_scene(write_scene(s, str(tmp_path)))
    _same_scene(s, t)
    fa, fb = _films_equal(s, t)
    assert np.array_equal(fa, fb)
