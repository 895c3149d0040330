"""Seeded query sets that pin the CPU oracle to the reference's own code.

Each family exercises one function of the path on the configurations'
parameters, with the same inputs for both sides:

  tri        Triangle::intersection          geometricShape/Triangle.cpp:46-88
  mapping    squareTo* warps                 core/Mapping.h:62-164
  fresnel    fresnelConductor/Dielectric,    core/Fresnel.h:30-114
             estimateDielectric
  microfacet D, G, sampleNormal              bsdf/MicrofacetDistribution.cpp:29-158
  bsdf       eval/pdf/sample of Diffuse,     bsdf/Diffuse.cpp:28-106, RoughConductor.cpp:77-145,
             RoughConductor, RoughDielectric, RoughDielectric.cpp:83-329,
             SmoothLayeredBSDF               SmoothLayeredBSDF.cpp:139-403
  light      MeshLight, AreaLight on a       light/MeshLight.cpp:32-64, AreaLight.cpp:23-61,
             Sphere, EnvironmentLight        Sphere.cpp:146-201, EnvironmentLight.cpp:85-237
  phase      HGPhaseFunction eval/sample     medium/HGPhaseFunction.cpp:27-79
  medium     Homogeneous, Heterogeneous      medium/Homogeneous.cpp:30-78,
             (GridVolume) sampleDistance /   Heterogeneous.cpp:281-546, GridVolume.cpp:118-149
             transmittance

`inputs()` builds the queries; `run(side, inp)` answers them through the
oracle (side "oracle") or through the reference's own code compiled by
oracle/build_oracle.py (side = the loaded libref_hot.so).  The golden
fixture tests/golden/ref_hot.npz holds the inputs with the reference's
answers (tests/golden/make_golden.py); tests/test_oracle_pins.py compares.
"""
import ctypes as C

import numpy as np

import oracle_lib as O
from raytracer_gb300 import desc as D, scenes

BSDF_Q, BSDF_R = O.BSDF_Q, O.BSDF_R
LIGHT_Q = np.dtype([("p", np.float32, 3), ("u", np.float32, 2)])
LIGHT_R = np.dtype([("intensity", np.float32, 3), ("pdf", np.float32), ("to_light", np.float32, 3),
                    ("distance", np.float32), ("point", np.float32, 3), ("normal", np.float32, 3),
                    ("pdf_eval", np.float32), ("pad", np.float32)])

# the materials of the benchmark configurations, plus the other
# distributions of the same BSDFs
BSDFS = [
    ("diffuse_wall", D.bsdf(D.BSDF_DIFFUSE, albedo=(0.65, 0.05, 0.05))),
    ("conductor_ggx_au_a0.05", D.bsdf(D.BSDF_ROUGH_CONDUCTOR, distribution=D.DIST_GGX, alpha=0.05,
                                      eta=scenes.AU_ETA, k=scenes.AU_K)),
    ("conductor_ggx_au_a0.3", D.bsdf(D.BSDF_ROUGH_CONDUCTOR, distribution=D.DIST_GGX, alpha=0.3,
                                     eta=scenes.AU_ETA, k=scenes.AU_K)),
    ("conductor_beckmann_a0.2", D.bsdf(D.BSDF_ROUGH_CONDUCTOR, distribution=D.DIST_BECKMANN, alpha=0.2,
                                       eta=(0.2, 0.9, 1.1), k=(3.9, 2.4, 2.2))),
    ("conductor_phong_a20", D.bsdf(D.BSDF_ROUGH_CONDUCTOR, distribution=D.DIST_PHONG, alpha=20.0,
                                   eta=(1.6, 0.9, 0.5), k=(3.0, 2.9, 2.7))),
    ("dielectric_ggx_a0.1", D.bsdf(D.BSDF_ROUGH_DIELECTRIC, distribution=D.DIST_GGX, alpha=0.1, eta_int=1.5)),
    ("dielectric_beckmann_a0.3", D.bsdf(D.BSDF_ROUGH_DIELECTRIC, distribution=D.DIST_BECKMANN, alpha=0.3,
                                        eta_int=1.33, reflectance=(0.9, 0.8, 0.7), transmittance=(0.6, 0.9, 1.0))),
    ("smooth_layered", D.bsdf(D.BSDF_SMOOTH_LAYERED, albedo=(0.7, 0.25, 0.2), eta_int=1.5, thickness=0.1)),
    ("smooth_layered_absorbing", D.bsdf(D.BSDF_SMOOTH_LAYERED, albedo=(0.2, 0.6, 0.3), eta_int=1.8,
                                        thickness=0.5, absorbance=(0.4, 0.1, 0.7))),
]
MICROFACETS = [(D.DIST_BECKMANN, 0.2), (D.DIST_GGX, 0.05), (D.DIST_GGX, 0.45), (D.DIST_PHONG, 30.0)]
PHASE_G = [0.3, -0.5, 0.9, 0.0]


def _dirs(rng, n, zmin=-1.0):
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    if zmin >= 0:
        d[:, 2] = np.abs(d[:, 2])
    return d.astype(np.float32)


def _u(rng, n):
    u = rng.random((n, 2)).astype(np.float32)
    edge = np.array([[0, 0], [0, 0.5], [0.5, 0], [0.999999, 0.25], [0.25, 0.999999], [1e-7, 1e-7]], np.float32)
    u[:len(edge)] = edge
    return u


def inputs(n=4096, seed=2024):
    rng = np.random.default_rng(seed)
    inp = {}
    # --- triangles: random, thin, large-offset; rays aimed at them and grazing
    tris = [np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32),
            np.array([[0.2, 1.3, -0.4], [0.9, 1.1, 0.3], [0.1, 0.2, 0.8]], np.float32),
            np.array([[100.0, 100.0, 100.0], [100.01, 100.0, 100.0], [100.0, 100.002, 100.0]], np.float32),
            np.array([[-3, 0, -3], [3, 0, -3], [3, 0, 3]], np.float32)]
    tri_v, rays = [], []
    for t in tris:
        c = t.mean(0)
        o = c + rng.normal(size=(n, 3)) * np.abs(t - c).max() * 3
        bary = rng.dirichlet([1, 1, 1], size=n) * 1.2 - 0.07    # some aimed just outside the edges
        tgt = bary @ t
        d = tgt - o
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        r = np.zeros(n, D.RAY_DTYPE)
        r["o"], r["d"] = o, d
        r["mint"] = np.where(rng.random(n) < 0.8, 1e-4, 0.0)
        r["maxt"] = np.where(rng.random(n) < 0.9, 1e8, np.linalg.norm(tgt - o, axis=1) * 0.999)
        tri_v.append(np.ascontiguousarray(t.reshape(-1)))
        rays.append(r)
    inp["tri_v"] = np.stack(tri_v)
    inp["tri_rays"] = np.stack(rays)
    # --- warps
    inp["map_u"] = _u(rng, n)
    # --- Fresnel
    fr = np.zeros((3, n, 4), np.float32)
    fr[0, :, 0] = rng.uniform(0.05, 2.0, n); fr[0, :, 1] = rng.uniform(0.0, 4.0, n); fr[0, :, 2] = rng.uniform(-1, 1, n)
    fr[1, :, 0] = rng.uniform(1.0, 1.8, n); fr[1, :, 1] = rng.uniform(1.0, 1.8, n)
    fr[1, :, 2] = rng.uniform(0, 1, n); fr[1, :, 3] = rng.uniform(0, 1, n)
    fr[2, :, 0] = 1.000277; fr[2, :, 1] = rng.choice([1.5, 1.33, 1.5046, 2.4], n); fr[2, :, 2] = rng.uniform(-1, 1, n)
    fr[2, :8, 2] = [0, 1, -1, 1e-6, -1e-6, 0.5, -0.5, 0.05]
    inp["fresnel_in"] = fr
    # --- microfacet: D(wh), G(wi, wo, wh), sampleNormal(u)
    mf = np.zeros((3, n, 9), np.float32)
    mf[0, :, :3] = _dirs(rng, n)
    wi, wo = _dirs(rng, n), _dirs(rng, n)
    wh = wi + wo
    wh /= np.linalg.norm(wh, axis=1, keepdims=True)
    mf[1, :, :3], mf[1, :, 3:6], mf[1, :, 6:] = wi, wo, wh
    mf[2, :, :2] = _u(rng, n)
    inp["mf_in"] = mf
    # --- BSDFs: eval/pdf on mixed hemispheres, sample on both sides
    q = np.zeros(n, BSDF_Q)
    q["wi"], q["wo"], q["u"] = _dirs(rng, n), _dirs(rng, n), _u(rng, n)
    inp["bsdf_q"] = q
    # --- phase function
    ph = np.zeros((2, n, 6), np.float32)
    ph[0, :, :3], ph[0, :, 3:] = _dirs(rng, n), _dirs(rng, n)
    ph[1, :, :3], ph[1, :, 3:5] = _dirs(rng, n), _u(rng, n)
    inp["phase_in"] = ph
    # --- lights
    lq = np.zeros(n, LIGHT_Q)
    lq["p"] = rng.uniform(-1.5, 2.5, (n, 3))
    lq["u"] = _u(rng, n)
    inp["light_q"] = lq
    inp["mesh_light_v"] = np.array([[0.375, 0.999, 0.375], [0.625, 0.999, 0.375], [0.625, 0.999, 0.625],
                                    [0.375, 0.999, 0.625], [0.1, 1.2, 0.1], [0.4, 1.5, 0.3], [0.3, 1.1, 0.9]],
                                   np.float32)
    inp["mesh_light_i"] = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6]], np.int32)
    inp["mesh_light_radiance"] = np.array([17.0, 12.0, 4.0], np.float32)
    T = np.eye(4, dtype=np.float32)
    T[:3, 3] = (1.1, 1.7, 0.9)
    inp["sphere_light_T"] = T
    inp["sphere_light_radius"] = np.float32(0.2)
    inp["sphere_light_radiance"] = np.array([50.0, 50.0, 50.0], np.float32)
    env, _ = scenes.sky_env(64, 32, sun_radius_deg=4.0, sun_radiance=1e4)
    inp["env_rgb"] = np.ascontiguousarray(env, np.float32)
    inp["env_scale"] = np.float32(1.0)
    # --- media: homogeneous slab, fBm grid in the configuration's cube
    mq = np.zeros(n, scenes_medium_q())
    o = rng.uniform(-0.7, 0.7, (n, 3)).astype(np.float32) + np.array([0.0, 0.75, 0.0], np.float32)
    mq["o"], mq["d"] = o, _dirs(rng, n)
    mq["mint"] = np.where(rng.random(n) < 0.5, 0.0, 1e-4)
    mq["maxt"] = rng.uniform(0.05, 2.5, n)
    mq["seed"] = rng.integers(0, 2 ** 31, n)
    mq["pixel"] = rng.integers(0, 1 << 20, n)
    mq["sample"] = rng.integers(0, 256, n)
    inp["medium_q"] = mq
    inp["grid"] = scenes.density_grid(16, seed=5)
    return inp


def scenes_medium_q():
    from raytracer_gb300.core import MEDIUM_Q
    return MEDIUM_Q


def _medium_descs(inp):
    homog = dict(type=D.MEDIUM_HOMOGENEOUS, phase=D.PHASE_ISOTROPIC, sigma_a=(0.4, 0.4, 0.4),
                 sigma_s=(1.6, 1.6, 1.6), scale=1.0)
    hetero = dict(type=D.MEDIUM_HETEROGENEOUS, phase=D.PHASE_HG, g=0.3, scale=20.0, albedo=(0.9, 0.9, 0.9),
                  density=inp["grid"], grid_min=(0, 0, 0), grid_max=(1, 1, 1), centered=1)
    # owner: the configuration's unit cube centred at (0, 0.75, 0)
    return [("homogeneous", homog), ("heterogeneous", hetero)], ((-0.5, 0.25, -0.5), (0.5, 1.25, 0.5))


# ---------------------------------------------------------------- scenes for the oracle side
def _light_scenes(inp):
    out = {}
    s = D.SceneData()
    lm = s.add_mesh(inp["mesh_light_v"], inp["mesh_light_i"])
    li = s.add_area_light(tuple(inp["mesh_light_radiance"]), D.SHAPE_MESH, lm, mesh_light=True)
    s.meshes[lm]["light"] = li
    s.camera = D.camera(8, 8, 40.0, np.eye(4))
    out["mesh"] = (s, li)
    s = D.SceneData()
    sp = s.add_sphere(float(inp["sphere_light_radius"]), inp["sphere_light_T"].astype(np.float64))
    li = s.add_area_light(tuple(inp["sphere_light_radiance"]), D.SHAPE_SPHERE, sp, mesh_light=False)
    s.spheres[sp]["light"] = li
    s.camera = D.camera(8, 8, 40.0, np.eye(4))
    out["sphere"] = (s, li)
    s = D.SceneData()
    bv, bf = scenes._box((0.0, 1.0, 0.0), (2.0, 2.0, 2.0))
    s.add_mesh(bv, bf)
    li = s.add_env_light(inp["env_rgb"], scale=float(inp["env_scale"]))
    s.camera = D.camera(8, 8, 40.0, np.eye(4))
    out["env"] = (s, li)
    return out


def _medium_scene(inp):
    s = D.SceneData()
    (hn, homog), (en, hetero) = _medium_descs(inp)[0]
    lo, hi = _medium_descs(inp)[1]
    c = tuple((np.array(lo) + np.array(hi)) / 2)
    ids = [s.add_medium(dict(homog)), s.add_medium(dict(hetero))]
    bv, bf = scenes._box(c, tuple(np.array(hi) - np.array(lo)))
    s.add_mesh(bv, bf, interior=ids[1])
    s.camera = D.camera(8, 8, 40.0, np.eye(4))
    return s, ids


# ---------------------------------------------------------------- running
def _p(a):
    return C.c_void_p(a.ctypes.data)


def bind_reference(L):
    vp = C.c_void_p
    L.ref_tri_query.argtypes = [vp, vp, C.c_int32, vp]
    L.ref_bsdf_query.argtypes = [C.POINTER(D.BsdfDesc), C.c_int32, vp, C.c_int32, vp]
    L.ref_fresnel_query.argtypes = [C.c_int32, vp, C.c_int32, vp]
    L.ref_mapping_query.argtypes = [C.c_int32, vp, C.c_int32, vp]
    L.ref_microfacet_query.argtypes = [C.c_int32, C.c_int32, C.c_float, vp, C.c_int32, vp]
    L.ref_phase_query.argtypes = [C.c_float, C.c_int32, vp, C.c_int32, vp]
    L.ref_mesh_light_query.argtypes = [vp, C.c_int32, vp, C.c_int32, vp, vp, C.c_int32, vp]
    L.ref_sphere_light_query.argtypes = [vp, C.c_float, vp, vp, C.c_int32, vp]
    L.ref_env_light_query.argtypes = [vp, C.c_int32, C.c_int32, C.c_float, vp, vp, C.c_float, vp, C.c_int32, vp]
    L.ref_medium_query.argtypes = [C.POINTER(D.MediumDesc), vp, vp, C.c_int32, vp, C.c_int32, vp]
    for name in ("ref_tri_query", "ref_bsdf_query", "ref_fresnel_query", "ref_mapping_query", "ref_microfacet_query",
                 "ref_phase_query", "ref_mesh_light_query", "ref_sphere_light_query", "ref_env_light_query",
                 "ref_medium_query"):
        getattr(L, name).restype = C.c_int32
    return L


def _bind_oracle():
    L = O.lib()
    vp = C.c_void_p
    L.oracle_tri_query.argtypes = [vp, vp, C.c_int32, vp]
    L.oracle_fresnel_query.argtypes = [C.c_int32, vp, C.c_int32, vp]
    L.oracle_mapping_query.argtypes = [C.c_int32, vp, C.c_int32, vp]
    L.oracle_microfacet_query.argtypes = [C.c_int32, C.c_int32, C.c_float, vp, C.c_int32, vp]
    L.oracle_phase_query.argtypes = [C.c_float, C.c_int32, vp, C.c_int32, vp]
    L.oracle_env_sphere.argtypes = [vp, C.c_int32, vp]
    return L


def run(side, inp):
    """Answer every query family through `side`: "oracle" or the reference
    pin library (a ctypes CDLL of libref_hot.so)."""
    ref = side != "oracle"
    L = bind_reference(side) if ref else _bind_oracle()
    pre = "ref_" if ref else "oracle_"
    out = {}
    n = len(inp["map_u"])
    # triangles
    hits = []
    for tv, rays in zip(inp["tri_v"], inp["tri_rays"]):
        h = np.zeros(len(rays), D.HIT_DTYPE)
        rr = np.ascontiguousarray(rays)
        assert getattr(L, pre + "tri_query")(_p(np.ascontiguousarray(tv)), _p(rr), len(rr), _p(h)) == 0
        hits.append(h)
    out["tri_hits"] = np.stack(hits)
    # warps
    m = np.zeros((4, n, 3), np.float32)
    for op in range(4):
        res = np.zeros((n, 3), np.float32)
        assert getattr(L, pre + "mapping_query")(op, _p(inp["map_u"]), n, _p(res)) == 0
        m[op] = res
    out["mapping"] = m
    # Fresnel
    f = np.zeros((3, n, 5), np.float32)
    for op in range(3):
        res = np.zeros((n, 5), np.float32)
        assert getattr(L, pre + "fresnel_query")(op, _p(np.ascontiguousarray(inp["fresnel_in"][op])), n, _p(res)) == 0
        f[op] = res
    out["fresnel"] = f
    # microfacet
    mf = np.zeros((len(MICROFACETS), 3, n, 3), np.float32)
    for k, (dist, alpha) in enumerate(MICROFACETS):
        for op in range(3):
            res = np.zeros((n, 3), np.float32)
            assert getattr(L, pre + "microfacet_query")(dist, op, alpha, _p(np.ascontiguousarray(inp["mf_in"][op])),
                                                        n, _p(res)) == 0
            mf[k, op] = res
    out["microfacet"] = mf
    # BSDFs
    q = inp["bsdf_q"]
    for name, b in BSDFS:
        for op, tag in ((0, "eval"), (1, "pdf"), (2, "sample")):
            if ref:
                r = np.zeros(len(q), BSDF_R)
                bs = D.bsdf_struct(b)
                assert L.ref_bsdf_query(C.byref(bs), op, _p(q), len(q), _p(r)) == 0
            else:
                r = O.bsdf_query(b, op, q)
            out["bsdf_%s_%s" % (name, tag)] = r
    # phase function
    for g in PHASE_G:
        for op, tag in ((0, "eval"), (1, "sample")):
            res = np.zeros((n, 5), np.float32)
            assert getattr(L, pre + "phase_query")(g, op, _p(np.ascontiguousarray(inp["phase_in"][op])), n, _p(res)) == 0
            out["phase_g%g_%s" % (g, tag)] = res
    # lights
    lq = np.ascontiguousarray(inp["light_q"])
    if ref:
        oscene = _light_scenes(inp)
        r = np.zeros(len(lq), LIGHT_R)
        v, ix = np.ascontiguousarray(inp["mesh_light_v"]), np.ascontiguousarray(inp["mesh_light_i"])
        assert L.ref_mesh_light_query(_p(v), len(v), _p(ix), len(ix), _p(inp["mesh_light_radiance"]), _p(lq),
                                      len(lq), _p(r)) == 0
        out["light_mesh"] = r
        r = np.zeros(len(lq), LIGHT_R)
        T = np.ascontiguousarray(inp["sphere_light_T"], np.float32)
        assert L.ref_sphere_light_query(_p(T), float(inp["sphere_light_radius"]), _p(inp["sphere_light_radiance"]),
                                        _p(lq), len(lq), _p(r)) == 0
        out["light_sphere"] = r
        # the bounding sphere comes from the oracle's scene box, as
        # EnvironmentLight::initialize would take it from the scene
        s, li = oscene["env"]
        osc = O.OracleScene(s)
        sph = np.zeros(4, np.float32)
        assert O.lib().oracle_env_sphere(osc.h, li, _p(sph)) == 0
        osc.close()
        r = np.zeros(len(lq), LIGHT_R)
        rgb = np.ascontiguousarray(inp["env_rgb"], np.float32)
        I = np.eye(4, dtype=np.float32)
        assert L.ref_env_light_query(_p(rgb), rgb.shape[1], rgb.shape[0], float(inp["env_scale"]), _p(I),
                                     _p(sph[:3].copy()), float(sph[3]), _p(lq), len(lq), _p(r)) == 0
        out["light_env"] = r
        out["env_sphere"] = sph
    else:
        for key, (s, li) in _light_scenes(inp).items():
            osc = O.OracleScene(s)
            out["light_" + key] = osc.light_query(li, lq["p"], lq["u"])
            if key == "env":
                sph = np.zeros(4, np.float32)
                O.lib().oracle_env_sphere(osc.h, li, _p(sph))
                out["env_sphere"] = sph
            osc.close()
    # media
    mq = np.ascontiguousarray(inp["medium_q"])
    from raytracer_gb300.core import MEDIUM_R
    descs, (lo, hi) = _medium_descs(inp)
    if ref:
        lo32, hi32 = np.array(lo, np.float32), np.array(hi, np.float32)
        for k, (name, md) in enumerate(descs):
            keep = []
            st = D.medium_struct(md, keep)
            for op, tag in ((0, "sample"), (1, "tr")):
                r = np.zeros(len(mq), MEDIUM_R)
                assert L.ref_medium_query(C.byref(st), _p(lo32), _p(hi32), op, _p(mq), len(mq), _p(r)) == 0
                out["medium_%s_%s" % (name, tag)] = r
    else:
        s, ids = _medium_scene(inp)
        osc = O.OracleScene(s)
        for (name, _), mid in zip(descs, ids):
            for op, tag in ((0, "sample"), (1, "tr")):
                out["medium_%s_%s" % (name, tag)] = osc.medium_query(mid, op, mq)
        osc.close()
    return out


# ---------------------------------------------------------------- whole paths
def film_scenes():
    """Scenes whose every path sample the reference's own integrator renders
    for the film pins: the configurations' scene families at small sizes."""
    return [("cornell_64x64_4spp", scenes.cornell_box(64, 64), 4),
            ("icosphere_l5_48x48_2spp", scenes.displaced_icosphere(level=5, width=48, height=48, env_size=(128, 64)), 2),
            ("volume_res32_40x32_2spp", scenes.volume_grid(40, 32, res=32), 2)]


def scene_digest(s):
    """A checksum of a scene's geometry, maps and grids (the fixture records
    it, so a changed generator is reported as such)."""
    import hashlib
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(s.vertices, np.float32).tobytes())
    h.update(np.ascontiguousarray(s.indices, np.int32).tobytes())
    for l in s.lights:
        if "rgb" in l:
            h.update(np.ascontiguousarray(l["rgb"], np.float32).tobytes())
    for m in s.media:
        if m.get("density") is not None:
            h.update(np.ascontiguousarray(m["density"], np.float32).tobytes())
    return h.hexdigest()


def all_paths(s, spp):
    W, H = s.camera["width"], s.camera["height"]
    pix = np.repeat(np.arange(W * H, dtype=np.int32), spp)
    smp = np.tile(np.arange(spp, dtype=np.int32), W * H)
    return pix, smp


def reference_paths(L, s, pix, smp, seed=0):
    """Per-path radiance of the reference's own integrator (ref_render_paths)."""
    L.ref_scene_create.restype = C.c_void_p
    L.ref_scene_create.argtypes = [C.POINTER(D.SceneDesc), C.POINTER(D.RenderDesc)]
    L.ref_render_paths.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    L.ref_render_paths.restype = C.c_int32
    L.ref_scene_destroy.argtypes = [C.c_void_p]
    d = s.desc()
    rd = s.render_desc(1, seed=seed)
    h = L.ref_scene_create(C.byref(d), C.byref(rd))
    assert h, "scene has parts the reference pin build does not assemble"
    pix = np.ascontiguousarray(pix, np.int32)
    smp = np.ascontiguousarray(smp, np.int32)
    rad = np.zeros((len(pix), 3), np.float32)
    assert L.ref_render_paths(h, seed, _p(pix), _p(smp), len(pix), _p(rad), None) == 0
    L.ref_scene_destroy(h)
    return rad
