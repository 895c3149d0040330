"""ctypes mirror of include/rtgpu.h and a numpy-backed scene container.

`SceneData` holds the flattened arrays of one scene (the reference's Mesh /
Sphere / BSDF / Light / Medium objects after XML loading) and builds the
`rt_scene_desc` struct that both the CUDA library and the CPU oracle read.
The numpy arrays stay owned by the SceneData object; the struct only points
at them, so keep the SceneData alive while a desc is in use.
"""
import ctypes as C
import math
import numpy as np

f3 = C.c_float * 3
f16 = C.c_float * 16
i3 = C.c_int32 * 3

BSDF_DIFFUSE, BSDF_ROUGH_CONDUCTOR, BSDF_ROUGH_DIELECTRIC, BSDF_SMOOTH_LAYERED, BSDF_LAYERED = 0, 1, 2, 3, 4
BSDF_DIELECTRIC, BSDF_CONDUCTOR, BSDF_MIRROR = 5, 6, 7
BSDF_SHEET_DIELECTRIC, BSDF_MICROFACET = 8, 9
DIST_BECKMANN, DIST_PHONG, DIST_GGX = 0, 1, 2
LIGHT_AREA, LIGHT_ENV, LIGHT_POINT, LIGHT_SPOT = 0, 1, 2, 3
SHAPE_MESH, SHAPE_SPHERE = 0, 1
ANALYTIC_SPHERE, ANALYTIC_PLANE = 0, 1
MEDIUM_HOMOGENEOUS, MEDIUM_HETEROGENEOUS = 0, 1
PHASE_ISOTROPIC, PHASE_HG = 0, 1
INTEGRATOR_PATH_MIS, INTEGRATOR_VOLPATH = 0, 1
STRATEGY_ALL_LIGHTS, STRATEGY_ONE_LIGHT_UNIFORM, STRATEGY_ONE_LIGHT_WEIGHTED = 0, 1, 2
BSDF_OP_EVAL, BSDF_OP_PDF, BSDF_OP_SAMPLE = 0, 1, 2

# reference name -> enum (XML "type" attributes, bsdf/*.cpp RT_REGISTER_TYPE)
BSDF_TYPES = {"diffuse": BSDF_DIFFUSE, "roughconductor": BSDF_ROUGH_CONDUCTOR,
              "roughdielectric": BSDF_ROUGH_DIELECTRIC, "smoothlayeredbsdf": BSDF_SMOOTH_LAYERED,
              "layeredbsdf": BSDF_LAYERED, "dielectric": BSDF_DIELECTRIC,
              "conductor": BSDF_CONDUCTOR, "mirror": BSDF_MIRROR, "sheetdielectric": BSDF_SHEET_DIELECTRIC,
              "microfacet": BSDF_MICROFACET}
DIST_TYPES = {"beckmann": DIST_BECKMANN, "phong": DIST_PHONG, "ggx": DIST_GGX}


class BsdfDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("distribution", C.c_int32), ("albedo", f3),
                ("reflectance", f3), ("transmittance", f3), ("eta", f3), ("k", f3),
                ("alpha", C.c_float), ("eta_int", C.c_float), ("eta_ext", C.c_float),
                ("thickness", C.c_float), ("absorbance", f3),
                ("distribution_base", C.c_int32), ("alpha_base", C.c_float),
                ("two_sided", C.c_int32), ("tex_albedo", C.c_int32), ("tex_reflectance", C.c_int32),
                ("tex_transmittance", C.c_int32), ("tex_alpha", C.c_int32), ("ks", C.c_float)]


class TextureDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", C.POINTER(C.c_float)),
                ("scale", C.c_float), ("invert_x", C.c_int32), ("invert_y", C.c_int32)]


class MeshDesc(C.Structure):
    _fields_ = [("first_tri", C.c_int32), ("n_tris", C.c_int32), ("bsdf", C.c_int32),
                ("light", C.c_int32), ("interior", C.c_int32), ("exterior", C.c_int32)]


class SphereDesc(C.Structure):
    _fields_ = [("radius", C.c_float), ("to_world", f16), ("to_object", f16),
                ("bsdf", C.c_int32), ("light", C.c_int32), ("interior", C.c_int32),
                ("exterior", C.c_int32), ("kind", C.c_int32)]


class LightDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("mesh_light", C.c_int32), ("shape_kind", C.c_int32),
                ("shape", C.c_int32), ("radiance", f3), ("env_width", C.c_int32),
                ("env_height", C.c_int32), ("env_rgb", C.POINTER(C.c_float)),
                ("env_scale", C.c_float), ("env_to_world", f16), ("env_to_light", f16),
                ("position", f3), ("intensity", f3), ("spot_to_light", f16),
                ("cos_falloff_start", C.c_float), ("cos_total_width", C.c_float)]


class MediumDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("phase", C.c_int32), ("g", C.c_float),
                ("sigma_a", f3), ("sigma_s", f3), ("scale", C.c_float), ("albedo", f3),
                ("res", i3), ("density", C.POINTER(C.c_float)), ("grid_min", f3),
                ("grid_max", f3), ("to_world", f16), ("centered", C.c_int32)]


class CameraDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("sample_to_camera", f16),
                ("camera_to_world", f16), ("near_clip", C.c_float), ("far_clip", C.c_float),
                ("aperture_radius", C.c_float), ("focal_plane", C.c_float),
                ("medium", C.c_int32), ("filter", C.c_int32), ("filter_radius", C.c_float * 2),
                ("filter_param", C.c_float * 2)]


class SceneDesc(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("vertices", C.POINTER(C.c_float)),
                ("normals", C.POINTER(C.c_float)), ("n_triangles", C.c_int32),
                ("indices", C.POINTER(C.c_int32)), ("n_meshes", C.c_int32),
                ("meshes", C.POINTER(MeshDesc)), ("n_spheres", C.c_int32),
                ("spheres", C.POINTER(SphereDesc)), ("n_bsdfs", C.c_int32),
                ("bsdfs", C.POINTER(BsdfDesc)), ("n_lights", C.c_int32),
                ("lights", C.POINTER(LightDesc)), ("env_light", C.c_int32),
                ("n_media", C.c_int32), ("media", C.POINTER(MediumDesc)),
                ("camera", CameraDesc), ("n_textures", C.c_int32), ("textures", C.POINTER(TextureDesc)),
                ("uvs", C.POINTER(C.c_float))]


class RenderDesc(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("max_depth", C.c_int32), ("min_depth", C.c_int32),
                ("strategy", C.c_int32), ("spp", C.c_int32), ("sample_begin", C.c_int32),
                ("seed", C.c_uint64), ("block_x", C.c_int32), ("block_y", C.c_int32),
                ("flags", C.c_int32)]


class Ray(C.Structure):
    _fields_ = [("o", f3), ("mint", C.c_float), ("d", f3), ("maxt", C.c_float)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("prim", C.c_int32)]


class BsdfQ(C.Structure):
    _fields_ = [("wi", f3), ("wo", f3), ("u", C.c_float * 2)]


class BsdfR(C.Structure):
    _fields_ = [("value", f3), ("pdf", C.c_float), ("wo", f3), ("relative_eta", C.c_float),
                ("sampled_type", C.c_int32), ("pad", C.c_int32)]


class LightQ(C.Structure):
    _fields_ = [("p", f3), ("u", C.c_float * 2)]


class LightR(C.Structure):
    _fields_ = [("intensity", f3), ("pdf", C.c_float), ("to_light", f3), ("distance", C.c_float),
                ("point", f3), ("normal", f3), ("pdf_eval", C.c_float), ("pad", C.c_float)]


class RenderStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("camera_ms", C.c_double), ("trace_closest_ms", C.c_double),
                ("trace_any_ms", C.c_double), ("shade_ms", C.c_double), ("volpath_ms", C.c_double),
                ("film_ms", C.c_double), ("paths", C.c_int64), ("closest_rays", C.c_int64),
                ("shadow_rays", C.c_int64), ("launches", C.c_int64), ("trace_closest_launches", C.c_int64),
                ("trace_any_launches", C.c_int64), ("nodes_closest", C.c_int64), ("tris_closest", C.c_int64),
                ("nodes_any", C.c_int64), ("tris_any", C.c_int64), ("limit_hits", C.c_int64),
                ("nan_samples", C.c_int64), ("resolve_ms", C.c_double), ("sort_ms", C.c_double)]


RAY_DTYPE = np.dtype([("o", np.float32, 3), ("mint", np.float32), ("d", np.float32, 3),
                      ("maxt", np.float32)])
HIT_DTYPE = np.dtype([("t", np.float32), ("u", np.float32), ("v", np.float32), ("prim", np.int32)])
assert RAY_DTYPE.itemsize == C.sizeof(Ray) and HIT_DTYPE.itemsize == C.sizeof(Hit)


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def mat(m):
    a = f16()
    flat = np.asarray(m, dtype=np.float64).reshape(16)
    for i in range(16):
        a[i] = float(np.float32(flat[i]))
    return a


def inv4(m):
    return np.linalg.inv(np.asarray(m, dtype=np.float64).reshape(4, 4))


IDENTITY = np.eye(4)


def bsdf(kind, **kw):
    """BSDF parameters with the reference constructors' defaults
    (Diffuse.cpp:11-18, RoughConductor.cpp:13-30, RoughDielectric.cpp:13-32,
    SmoothLayeredBSDF.cpp:12-28, LayeredBSDF.cpp:17-36: coat distribution ggx,
    alphaTop 0.01, over a default RoughConductor: beckmann, alpha 0.2,
    eta = k = 0; Dielectric.cpp:10-17, Conductor.cpp:13-21, Mirror.cpp:7-15,
    SheetDielectric.cpp:10-17, Microfacet.cpp:11-25: kd black, alpha 0.2,
    etaInt 1.5946, ggx, probabilitySpecular (ks) 1).
    two_sided=True wraps it in a TwoSides (TwoSides.cpp:5-15) with the same
    BSDF on both sides.  tex_albedo, tex_reflectance, tex_transmittance and
    tex_alpha name a texture of the scene (SceneData.add_texture) that
    replaces that parameter (None: the constant)."""
    layered = kind == BSDF_LAYERED
    mf = kind == BSDF_MICROFACET
    d = dict(type=kind, distribution=kw.get("distribution", DIST_GGX if (layered or mf) else DIST_BECKMANN),
             albedo=kw.get("albedo", (0.0, 0.0, 0.0) if mf else (0.5, 0.5, 0.5)),
             reflectance=kw.get("reflectance", (1.0, 1.0, 1.0)),
             transmittance=kw.get("transmittance", (1.0, 1.0, 1.0)),
             eta=kw.get("eta", (0.0, 0.0, 0.0)), k=kw.get("k", (0.0, 0.0, 0.0)),
             alpha=kw.get("alpha", 0.01 if layered else 0.2), eta_int=kw.get("eta_int", 1.5946 if mf else 1.5046),
             eta_ext=kw.get("eta_ext", 1.000277), thickness=kw.get("thickness", 1.2),
             absorbance=kw.get("absorbance", (0.0, 0.0, 0.0)),
             distribution_base=kw.get("distribution_base", DIST_BECKMANN),
             alpha_base=kw.get("alpha_base", 0.2), two_sided=bool(kw.get("two_sided", False)),
             ks=float(kw.get("ks", 1.0)))
    for k in TEX_PARAMS:
        if kw.get(k) is not None:
            d[k] = int(kw[k])
    return d


TEX_PARAMS = ("tex_albedo", "tex_reflectance", "tex_transmittance", "tex_alpha")


def medium_struct(m, keep):
    """rt_medium_desc of a medium dict (its density grid, if any, appended to
    `keep`, which must outlive the struct)."""
    M = MediumDesc()
    M.type = m["type"]
    M.phase = m.get("phase", PHASE_ISOTROPIC)
    M.g = m.get("g", -0.8)
    M.sigma_a = f3(*m.get("sigma_a", (0.15, 0.15, 0.15)))
    M.sigma_s = f3(*m.get("sigma_s", (0.15, 0.15, 0.15)))
    M.scale = m.get("scale", 1.0)
    M.albedo = f3(*m.get("albedo", (0.0, 0.0, 0.0)))
    dens = m.get("density")
    if dens is not None:
        dens = np.ascontiguousarray(dens, np.float32)
        keep.append(dens)
        M.res = i3(dens.shape[2], dens.shape[1], dens.shape[0])
        M.density = _fp(dens)
        M.grid_min = f3(*m.get("grid_min", (0, 0, 0)))
        M.grid_max = f3(*m.get("grid_max", (1, 1, 1)))
    M.to_world = mat(m.get("to_world", IDENTITY))
    M.centered = int(m.get("centered", 1))
    return M


def bsdf_struct(b):
    """rt_bsdf_desc of a bsdf() dict."""
    return BsdfDesc(b["type"], b["distribution"], f3(*b["albedo"]), f3(*b["reflectance"]),
                    f3(*b["transmittance"]), f3(*b["eta"]), f3(*b["k"]), b["alpha"],
                    b["eta_int"], b["eta_ext"], b["thickness"], f3(*b["absorbance"]),
                    b.get("distribution_base", DIST_BECKMANN), b.get("alpha_base", 0.2),
                    int(bool(b.get("two_sided", False))),
                    *[0 if b.get(k) is None else int(b[k]) + 1 for k in TEX_PARAMS], b.get("ks", 1.0))


class SceneData:
    """Flattened scene: numpy geometry plus lists of component dicts."""

    def __init__(self):
        self.vertices = np.zeros((0, 3), np.float32)
        self.normals = None
        self.uvs = None      # per-vertex texture coordinates (NaN: mesh without)
        self.textures = []   # dict(rgb (H, W, 3), scale, invert_x, invert_y)
        self.indices = np.zeros((0, 3), np.int32)
        self.meshes = []     # dict(first_tri, n_tris, bsdf, light, interior, exterior)
        self.spheres = []    # dict(radius, to_world, bsdf, light, interior, exterior)
        self.bsdfs = []
        self.lights = []     # dict(type, ...)
        self.media = []
        self.env_light = -1
        self.camera = None   # dict(width, height, sample_to_camera, camera_to_world, ...)
        self.integrator = dict(integrator=INTEGRATOR_PATH_MIS, max_depth=1000, min_depth=3,
                               strategy=STRATEGY_ONE_LIGHT_UNIFORM)
        self.name = "scene"
        self._keep = []

    # ------------------------------------------------------------ building
    def add_bsdf(self, d):
        self.bsdfs.append(d)
        return len(self.bsdfs) - 1

    def add_texture(self, rgb, scale=1.0, invert_x=False, invert_y=False):
        """An ImageTexture: `rgb` an (H, W, 3) linear image; returns its index."""
        rgb = np.ascontiguousarray(rgb, np.float32)
        if rgb.ndim != 3 or rgb.shape[2] != 3 or rgb.shape[0] < 1 or rgb.shape[1] < 1:
            raise ValueError("texture: expected an (H, W, 3) image")
        self.textures.append(dict(rgb=rgb, scale=abs(float(scale)), invert_x=bool(invert_x),
                                  invert_y=bool(invert_y)))
        return len(self.textures) - 1

    def add_mesh(self, verts, tris, bsdf=-1, light=-1, interior=-1, exterior=-1, normals=None, uvs=None):
        verts = np.asarray(verts, np.float32).reshape(-1, 3)
        tris = np.asarray(tris, np.int32).reshape(-1, 3)
        base = len(self.vertices)
        first = len(self.indices)
        self.vertices = np.concatenate([self.vertices, verts]) if len(self.vertices) else verts.copy()
        self.indices = np.concatenate([self.indices, tris + base]) if len(self.indices) else (tris + base).astype(np.int32)
        # one normal array for all vertices: the vertices of meshes without
        # normals carry NaN, and their triangles shade with the geometric normal
        if normals is not None:
            if self.normals is None:
                self.normals = np.full((base, 3), np.nan, np.float32)
            self.normals = np.concatenate([self.normals, np.asarray(normals, np.float32).reshape(-1, 3)])
        elif self.normals is not None:
            self.normals = np.concatenate([self.normals, np.full((len(verts), 3), np.nan, np.float32)])
        # texture coordinates likewise: NaN for the vertices of meshes without
        if uvs is not None:
            if self.uvs is None:
                self.uvs = np.full((base, 2), np.nan, np.float32)
            self.uvs = np.concatenate([self.uvs, np.asarray(uvs, np.float32).reshape(-1, 2)])
        elif self.uvs is not None:
            self.uvs = np.concatenate([self.uvs, np.full((len(verts), 2), np.nan, np.float32)])
        self.meshes.append(dict(first_tri=first, n_tris=len(tris), bsdf=bsdf, light=light,
                                interior=interior, exterior=exterior))
        return len(self.meshes) - 1

    def add_sphere(self, radius, to_world, bsdf=-1, light=-1, interior=-1, exterior=-1):
        self.spheres.append(dict(radius=radius, to_world=np.asarray(to_world, np.float64),
                                 bsdf=bsdf, light=light, interior=interior, exterior=exterior))
        return len(self.spheres) - 1

    def add_plane(self, to_world, bsdf=-1, light=-1, interior=-1, exterior=-1):
        """Plane (geometricShape/Plane.cpp): the square [-1,1]^2 at z = 0 of
        its object space, normal +z, placed by "toWorld".  It joins the
        analytic shapes (an area light on it uses SHAPE_SPHERE and this index)."""
        self.spheres.append(dict(radius=0.0, to_world=np.asarray(to_world, np.float64), kind=ANALYTIC_PLANE,
                                 bsdf=bsdf, light=light, interior=interior, exterior=exterior))
        return len(self.spheres) - 1

    def add_area_light(self, radiance, shape_kind, shape, mesh_light=True):
        self.lights.append(dict(type=LIGHT_AREA, mesh_light=int(mesh_light), shape_kind=shape_kind,
                                shape=shape, radiance=tuple(radiance)))
        return len(self.lights) - 1

    def add_point_light(self, position, intensity):
        """PointLight (light/PointLight.cpp:7-11): "position", "intensity"."""
        self.lights.append(dict(type=LIGHT_POINT, position=tuple(float(x) for x in position),
                                intensity=tuple(float(x) for x in intensity)))
        return len(self.lights) - 1

    def add_spot_light(self, to_world, intensity, falloff_start=30.0, total_width=60.0):
        """SpotLight (light/SpotLight.cpp:8-15): "toWorld", "intensity", and the
        "falloffStart" / "totalWidth" angles in degrees; the light sits at
        toWorld (0,0,0) and shines along its +z."""
        M = np.asarray(to_world, np.float64)
        self.lights.append(dict(type=LIGHT_SPOT, to_world=M,
                                intensity=tuple(float(x) for x in intensity),
                                falloff_start=float(falloff_start), total_width=float(total_width)))
        return len(self.lights) - 1

    def add_env_light(self, rgb, scale=1.0, to_world=IDENTITY):
        rgb = np.ascontiguousarray(rgb, dtype=np.float32)
        self.lights.append(dict(type=LIGHT_ENV, rgb=rgb, scale=scale,
                                to_world=np.asarray(to_world, np.float64)))
        self.env_light = len(self.lights) - 1
        return self.env_light

    def add_medium(self, d):
        if d.get("density") is not None:
            d["density"] = np.ascontiguousarray(d["density"], dtype=np.float32)
        self.media.append(d)
        return len(self.media) - 1

    # ------------------------------------------------------------ ctypes
    @property
    def n_triangles(self):
        return len(self.indices)

    def desc(self):
        """Build the rt_scene_desc struct pointing at this object's arrays."""
        keep = []
        v = np.ascontiguousarray(self.vertices, np.float32)
        ix = np.ascontiguousarray(self.indices, np.int32)
        nrm = None if self.normals is None else np.ascontiguousarray(self.normals, np.float32)
        keep += [v, ix, nrm]
        D = SceneDesc()
        D.n_vertices = len(v)
        D.vertices = _fp(v)
        D.normals = _fp(nrm) if nrm is not None else None
        D.n_triangles = len(ix)
        D.indices = _ip(ix)

        meshes = (MeshDesc * max(1, len(self.meshes)))()
        for i, m in enumerate(self.meshes):
            meshes[i] = MeshDesc(m["first_tri"], m["n_tris"], m["bsdf"], m["light"],
                                 m["interior"], m["exterior"])
        D.n_meshes = len(self.meshes)
        D.meshes = C.cast(meshes, C.POINTER(MeshDesc))

        spheres = (SphereDesc * max(1, len(self.spheres)))()
        for i, s in enumerate(self.spheres):
            # the binary32 toWorld a scene file holds, inverted in float64
            tw = np.asarray(s["to_world"], np.float32).astype(np.float64)
            spheres[i] = SphereDesc(s["radius"], mat(tw), mat(inv4(tw)),
                                    s["bsdf"], s["light"], s["interior"], s["exterior"],
                                    s.get("kind", ANALYTIC_SPHERE))
        D.n_spheres = len(self.spheres)
        D.spheres = C.cast(spheres, C.POINTER(SphereDesc))

        bs = (BsdfDesc * max(1, len(self.bsdfs)))()
        for i, b in enumerate(self.bsdfs):
            bs[i] = bsdf_struct(b)
        D.n_bsdfs = len(self.bsdfs)
        D.bsdfs = C.cast(bs, C.POINTER(BsdfDesc))

        ls = (LightDesc * max(1, len(self.lights)))()
        for i, l in enumerate(self.lights):
            L = LightDesc()
            L.type = l["type"]
            if l["type"] == LIGHT_ENV:
                rgb = l["rgb"]
                keep.append(rgb)
                L.env_height, L.env_width = rgb.shape[0], rgb.shape[1]
                L.env_rgb = _fp(rgb)
                L.env_scale = l["scale"]
                L.env_to_world = mat(l["to_world"])
                L.env_to_light = mat(inv4(l["to_world"]))
                L.radiance = f3(0, 0, 0)
                L.shape = -1
            elif l["type"] in (LIGHT_POINT, LIGHT_SPOT):
                L.shape = -1
                L.radiance = f3(0, 0, 0)
                L.env_to_world = mat(IDENTITY)
                L.env_to_light = mat(IDENTITY)
                L.intensity = f3(*l["intensity"])
                if l["type"] == LIGHT_POINT:
                    L.position = f3(*l["position"])
                    L.spot_to_light = mat(IDENTITY)
                else:
                    # the binary32 toWorld a scene file holds, inverted in float64
                    M = np.asarray(l["to_world"], np.float32).astype(np.float64)
                    c = M @ np.array([0.0, 0.0, 0.0, 1.0])
                    L.position = f3(*(c[:3] / c[3]))
                    L.spot_to_light = mat(inv4(M))
                    L.cos_falloff_start = math.cos(math.radians(l["falloff_start"]))
                    L.cos_total_width = math.cos(math.radians(l["total_width"]))
            else:
                L.mesh_light = l["mesh_light"]
                L.shape_kind = l["shape_kind"]
                L.shape = l["shape"]
                L.radiance = f3(*l["radiance"])
                L.env_to_world = mat(IDENTITY)
                L.env_to_light = mat(IDENTITY)
            ls[i] = L
        D.n_lights = len(self.lights)
        D.lights = C.cast(ls, C.POINTER(LightDesc))
        D.env_light = self.env_light

        ms = (MediumDesc * max(1, len(self.media)))()
        for i, m in enumerate(self.media):
            ms[i] = medium_struct(m, keep)
        D.n_media = len(self.media)
        D.media = C.cast(ms, C.POINTER(MediumDesc))

        c = self.camera
        flt = c.get("filter", box_filter())
        D.camera = CameraDesc(c["width"], c["height"], mat(c["sample_to_camera"]),
                              mat(c["camera_to_world"]), c["near_clip"], c["far_clip"],
                              c.get("aperture_radius", 0.0), c.get("focal_plane", 1e8),
                              c.get("medium", -1), flt["type"], (C.c_float * 2)(*flt["radius"]),
                              (C.c_float * 2)(*flt["param"]))
        tx = (TextureDesc * max(1, len(self.textures)))()
        for i, t in enumerate(self.textures):
            keep.append(t["rgb"])
            tx[i] = TextureDesc(t["rgb"].shape[1], t["rgb"].shape[0], _fp(t["rgb"]), t.get("scale", 1.0),
                                int(t.get("invert_x", False)), int(t.get("invert_y", False)))
        D.n_textures = len(self.textures)
        D.textures = C.cast(tx, C.POINTER(TextureDesc))
        uv = None if self.uvs is None else np.ascontiguousarray(self.uvs, np.float32)
        D.uvs = _fp(uv) if uv is not None else None
        keep += [meshes, spheres, bs, ls, ms, tx, uv]
        self._keep = keep
        return D

    def render_desc(self, spp, seed=0, sample_begin=0, block=32, flags=0, **over):
        """`block`: the tile size (blockSizeX = blockSizeY), or a pair
        (blockSizeX, blockSizeY)."""
        it = dict(self.integrator)
        it.update(over)
        bx, by = (block, block) if np.isscalar(block) else block
        return RenderDesc(it["integrator"], it["max_depth"], it["min_depth"], it["strategy"],
                          spp, sample_begin, seed, int(bx), int(by), flags)

    def bounds(self):
        lo = self.vertices.min(0) if len(self.vertices) else np.full(3, np.inf)
        hi = self.vertices.max(0) if len(self.vertices) else np.full(3, -np.inf)
        return lo, hi


RENDER_ACCUMULATE = 1   # rt_render_desc.flags: add to the film instead of overwriting it

FILTER_BOX, FILTER_GAUSSIAN, FILTER_MITCHELL = 0, 1, 2


def box_filter(rx=0.5, ry=0.5):
    """BoxFilter (filter/BoxFilter.h), radii default 0.5 (ReconstructionFilter.cpp:15-16)."""
    return dict(type=FILTER_BOX, radius=(rx, ry), param=(0.0, 0.0))


def gaussian_filter(rx=0.5, ry=0.5, alpha=None, omega=None):
    """GaussianFilter: alpha default 1 / (2 * 0.5 * 0.5), omega default radiusX
    (GaussianFilter.cpp:14-19)."""
    return dict(type=FILTER_GAUSSIAN, radius=(rx, ry),
                param=(1 / (2.0 * 0.5 * 0.5) if alpha is None else alpha, rx if omega is None else omega))


def mitchell_filter(rx=0.5, ry=0.5, b=1.0 / 3, c=1.0 / 3):
    """MitchellNetravaliFilter: B and C default 1/3 (MitchellNetravaliFilter.cpp:14-19)."""
    return dict(type=FILTER_MITCHELL, radius=(rx, ry), param=(b, c))


# ---------------------------------------------------------------- cameras
def look_at(origin, target, up):
    """Transform::fromLookAt (core/Transform.cpp:199-227): columns
    left, newUp, dir, origin."""
    o = np.asarray(origin, np.float64)
    d = np.asarray(target, np.float64) - o
    d /= np.linalg.norm(d)
    u = np.asarray(up, np.float64)
    u = u / np.linalg.norm(u)
    left = np.cross(u, d)
    left /= np.linalg.norm(left)
    nu = np.cross(d, left)
    nu /= np.linalg.norm(nu)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = left, nu, d, o
    return m


def nori_perspective(width, height, fov=30.0, near=1e-4, far=1e4):
    """sampleToCamera of NoriPerspective (camera/NoriPerspective.cpp:10-37),
    formed in double precision."""
    aspect = width / float(height)
    recip = 1.0 / (far - near)
    cot = 1.0 / np.tan(np.radians(fov / 2.0))
    P = np.array([[cot, 0, 0, 0], [0, cot, 0, 0], [0, 0, far * recip, -near * far * recip],
                  [0, 0, 1, 0]], np.float64)
    D = np.diag([-0.5, -0.5 * aspect, 1.0, 1.0])
    T = np.eye(4)
    T[0, 3], T[1, 3] = -1.0, -1.0 / aspect
    return np.linalg.inv(D @ T @ P)


def camera(width, height, fov, to_world, near=1e-4, far=1e4, medium=-1):
    return dict(width=width, height=height, sample_to_camera=nori_perspective(width, height, fov, near, far),
                camera_to_world=np.asarray(to_world, np.float64), near_clip=near, far_clip=far,
                aperture_radius=0.0, focal_plane=1e8, medium=medium, fov=fov)
