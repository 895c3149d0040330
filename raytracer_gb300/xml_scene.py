"""Reference scene files (XML) into a SceneData the device renders.

Follows xml::XMLLoader (core/XMLLoader.cpp) element by element for the
types the GPU path renders; anything else raises UnsupportedScene naming
the element.  Paths in the file are resolved against the file's folder
(XMLLoader.cpp:36 adds it to the search path).

    integrator   PathTracingMIS | VolPathTracing: maxDepth, minDepth, strategy
                 (PathTracingMIS.cpp:15-19, VolPathTracing.cpp:13-17)
    camera       NoriPerspective: fov, nearClip, farClip (NoriPerspective.cpp:15-17),
                 sizeX, sizeY, apertureRadius, focalPlane (Camera.cpp:11-14),
                 <transform> = camera to world, <filter> BoxFilter, GaussianFilter,
                 MitchellNetravaliFilter (radiusX, radiusY, alpha/omega, B/C)
    sampler      RandomSampler, StratifiedSampler: sampleNumber -> `spp`
                 (RandomSampler.cpp:10, StratifiedSampler.cpp:23); every path draws
                 from its own stream
    parameters   blockSizeX, blockSizeY -> `block`, fileName -> `file_name`
                 (XMLLoader.cpp:217-259)
    medium       (top level) the camera medium (XMLLoader.cpp:96-101; the later
                 referable-medium branch of the reference is unreachable)
    lights       EnvironmentLight: path (.hdr, .exr, PNG...), toWorld, scale, gamma
                 (EnvironmentLight.cpp:8-19); PointLight (position, intensity);
                 SpotLight (toWorld, intensity, falloffStart, totalWidth)
    objects      shape Mesh (path .obj, toWorld; MeshFactory.h:39-139), Cube
                 (toWorld; Cube.cpp), Sphere (radius, toWorld; Sphere.cpp:14-15),
                 Plane (toWorld; Plane.cpp:7-18),
                 each with <bsdf>, <light type="AreaLight|MeshLight"> (radiance),
                 <medium name="interior|exterior">
    bsdf         Diffuse, RoughConductor, RoughDielectric, SmoothLayeredBSDF
                 (over Diffuse), LayeredBSDF (over RoughConductor), Dielectric,
                 Conductor, Mirror, SheetDielectric, Microfacet, TwoSides (one
                 "bsdf" for both sides);
                 top-level <bsdf id=..> and <transform id=..>
                 can be referenced with ref=".."
    media        Homogeneous (sigmaA, sigmaS, scale), Heterogeneous (albedo,
                 <volume type="GridVolume"> path .vol, centered, toWorld, scale),
                 <phase name="phaseFunction" type="HGPhaseFunction|IsotropicPhaseFunction">

`load_scene(path)` returns the SceneData with `spp` and `block` attributes.
"""
import math
import os
import warnings
import xml.etree.ElementTree as ET

import numpy as np

from . import desc as D

F32 = np.float32


# The reference's object factories match type names without regard to case
# (ObjectFactoryManager::formatType, factory/ObjectFactoryManager.h:81-89):
# "roughconductor" is RoughConductor.  _type gives the spelling used here.
_TYPE_NAMES = ["ConstantTexture", "ImageTexture", "ScaleTexture", "Diffuse", "RoughConductor", "RoughDielectric",
               "SmoothLayeredBSDF", "LayeredBSDF", "Dielectric", "Conductor", "Mirror", "TwoSides",
               "SheetDielectric", "Microfacet",
               "HGPhaseFunction", "IsotropicPhaseFunction", "Homogeneous", "Heterogeneous", "Mesh", "Cube", "Sphere",
               "Plane",
               "MeshLight", "AreaLight", "NoriPerspective", "BoxFilter", "GaussianFilter", "MitchellNetravaliFilter",
               "EnvironmentLight", "PointLight", "SpotLight", "RandomSampler", "StratifiedSampler",
               "PathTracingMIS", "VolPathTracing",
               "GridVolume"]
_CANON = {n.lower(): n for n in _TYPE_NAMES}


def _type(el):
    t = el.get("type") or ""
    return _CANON.get(t.lower(), t)


class UnsupportedScene(ValueError):
    """The scene uses a type or option the GPU path does not provide."""


# --------------------------------------------------------------- values
def _num(s, kind):
    s = s.strip()
    if kind == "bool":
        return s == "1" or s.lower() == "true"   # tools/Tools.h:119-126
    if kind == "int":
        return int(float(s)) if s else 0
    return float(s)


def _triple(s):
    v = [float(x) for x in s.replace(",", " ").split()]
    v = (v + [0.0, 0.0, 0.0])[:3]
    return tuple(v)


def _color(s, where):
    """tools::stringToColor(.., 1): exactly three rgb values, blank or comma
    separated; anything else is an error that yields black in the reference."""
    parts = [p for p in s.replace(",", " ").split() if p]
    if len(parts) != 3 or any(":" in p for p in parts):
        warnings.warn("%s: RGB string %r is of wrong size; black, as in the reference" % (where, s))
        return (0.0, 0.0, 0.0)
    return tuple(float(p) for p in parts)


# ------------------------------------------------------------ transforms
def _deg2rad(a):
    return F32(a) * F32(math.pi) / F32(180.0)


def _rot(axis, deg):
    r = _deg2rad(deg)
    c, s = F32(math.cos(r)), F32(math.sin(r))
    m = np.eye(4, dtype=F32)
    i, j = {"x": (1, 2), "y": (2, 0), "z": (0, 1)}[axis]
    m[i, i], m[i, j], m[j, i], m[j, j] = c, -s, s, c
    return m


def _xyz(el, default):
    v = list(default)
    for c in el:
        if c.tag in ("x", "y", "z"):
            v["xyz".index(c.tag)] = float(c.text)
        else:
            warnings.warn("unknown parameter %s" % c.tag)
    return v


def _transform(el):
    """XMLLoader::handleTransform (XMLLoader.cpp:857-905): each child is
    multiplied on the left of what came before."""
    T = np.eye(4, dtype=F32)
    for c in el:
        if c.tag == "rotation":
            r = _xyz(c, (0.0, 0.0, 0.0))
            M = _rot("x", r[0]) @ _rot("y", r[1]) @ _rot("z", r[2])
        elif c.tag == "translation":
            t = _xyz(c, (0.0, 0.0, 0.0))
            M = np.eye(4, dtype=F32)
            M[:3, 3] = t
        elif c.tag == "scale":
            M = np.diag(list(_xyz(c, (1.0, 1.0, 1.0))) + [1.0]).astype(F32)
        elif c.tag == "matrix":
            M = np.array([float(x) for x in c.get("value").split()], F32).reshape(4, 4)
        elif c.tag == "lookAt":
            o = t = u = (0.0, 0.0, 0.0)
            for k in c:
                if k.tag == "origin":
                    o = _triple(k.text)
                elif k.tag == "lookAt":
                    t = _triple(k.text)
                elif k.tag == "up":
                    u = _triple(k.text)
            M = np.asarray(D.look_at(o, t, u), F32)
        else:
            warnings.warn("unknown transform element %s" % c.tag)
            continue
        T = (M.astype(F32) @ T).astype(F32)
    return T


# ------------------------------------------------------------- the loader
class _Loader:
    def __init__(self, path, materials):
        self.path = os.path.abspath(path)
        self.dir = os.path.dirname(self.path)
        self.materials = dict(materials or {})
        self.s = D.SceneData()
        self.s.name = os.path.splitext(os.path.basename(path))[0]
        self.ref_bsdf = {}
        self.ref_bsdf_name = {}   # id -> the element's name attribute (XMLLoader.cpp:108-114)
        self.tex_cache = {}
        self.ref_transform = {}
        self.ref_medium = {}
        self.camera_params = None
        self.camera_transform = np.eye(4, dtype=F32)
        self.camera_medium = -1
        self.spp = 1
        self.block = (32, 32)
        self.file_name = ""
        self.filter = D.box_filter()

    def resolve(self, p):
        return p if os.path.isabs(p) else os.path.normpath(os.path.join(self.dir, p))

    # XMLLoader::handleProperty (XMLLoader.cpp:714-830)
    def props(self, el):
        params = {}
        for c in el:
            name = c.get("name")
            val = c.get("value")
            tag = c.tag
            if name is None and c.get("ref") is None:
                warnings.warn("no name attribute for %s property" % tag)
                continue
            if tag == "bool":
                params[name] = _num(val, "bool")
            elif tag == "integer":
                params[name] = _num(val, "int")
            elif tag in ("double", "real"):
                params[name] = _num(val, "float")
            elif tag == "string":
                params[name] = val
            elif tag in ("point", "vector"):
                params[name] = _triple(val)
            elif tag == "color":
                params[name] = _color(val, name)
            elif tag == "spectrum":
                raise UnsupportedScene("spectrum values (%s) are not provided" % name)
            elif tag == "transform":
                if c.get("ref"):
                    params[name or "toWorld"] = self.ref_transform[c.get("ref")]
                else:
                    params[name] = _transform(c)
            elif tag == "texture":
                kind = _type(c)
                tp = self.props(c)
                if kind == "ConstantTexture":
                    params[name] = ("texture", tp.get("albedo", (0.5, 0.5, 0.5)))   # ConstantTexture.cpp:6-10
                elif kind == "ImageTexture":
                    params[name] = ("image", self.image_texture(tp))
                elif kind == "ScaleTexture":
                    params[name] = self.scale_texture(tp)
                else:
                    raise UnsupportedScene("texture type %s is not provided" % kind)
            elif tag == "bsdf":
                # a referenced BSDF keeps the name its <bsdf id=..> element
                # gave it (XMLLoader.cpp:762-775)
                if c.get("ref"):
                    params[self.ref_bsdf_name[c.get("ref")]] = self.ref_bsdf[c.get("ref")]
                else:
                    params[name] = self.bsdf(c)
            elif tag == "medium":
                params[name] = self.ref_medium[c.get("ref")] if c.get("ref") else self.medium(c)
            elif tag == "phase":
                params[name] = ("phase", _type(c), self.props(c))
            elif tag == "volume":
                params[name] = ("volume", _type(c), self.props(c))
            else:
                warnings.warn("unknown property %s" % name)
        return params

    @staticmethod
    def _tex_or(params, name, default):
        v = params.get(name, default)
        if isinstance(v, tuple) and len(v) == 2 and v[0] == "texture":
            return tuple(v[1])
        if isinstance(v, tuple) and len(v) == 2 and v[0] == "image":
            return default
        return v

    @staticmethod
    def _image(params, name):
        """The scene texture index of an ImageTexture parameter, else None."""
        v = params.get(name)
        if isinstance(v, tuple) and len(v) == 2 and v[0] == "image":
            return v[1]
        return None

    def image_texture(self, tp):
        """ImageTexture (ImageTexture.cpp:8-21): path, invertX/Y, scale
        (absolute value), gamma, channel; boundaryCondition is parsed by the
        reference but not used by its eval."""
        from .images import ImageError, load_image
        path = tp.get("path", "")
        gamma, channel = float(tp.get("gamma", 0.0)), str(tp.get("channel", "all")).lower()
        scale = abs(float(tp.get("scale", 1.0)))
        ix, iy = bool(tp.get("invertX", False)), bool(tp.get("invertY", False))
        # one texture per distinct image and settings (ImageLoader caches the
        # image array by path and channel, ImageLoader.cpp:36-41)
        key = (self.resolve(path), gamma, channel, scale, ix, iy)
        if key in self.tex_cache:
            return self.tex_cache[key]
        try:
            rgb = load_image(key[0], gamma=gamma, channel=channel)
        except (ImageError, OSError) as e:
            raise UnsupportedScene("ImageTexture %s: %s" % (path, e))
        self.tex_cache[key] = self.s.add_texture(rgb, scale=scale, invert_x=ix, invert_y=iy)
        return self.tex_cache[key]

    def scale_texture(self, tp):
        """ScaleTexture (texture/ScaleTexture.cpp): eval = texture.eval(uv) *
        scale.  Over a constant it is the scaled constant; over an
        ImageTexture it becomes a copy of that texture whose scale is the
        product of the two (the texel is then multiplied once by the product,
        where the reference multiplies by each in turn: at most an ulp or so
        apart).  A negative scale is not provided: the device's textures
        carry a non-negative scale."""
        inner = tp.get("texture")
        k = float(tp.get("scale", 1.0))
        if not (isinstance(inner, tuple) and len(inner) == 2):
            raise UnsupportedScene("ScaleTexture without a texture")
        if k < 0:
            raise UnsupportedScene("ScaleTexture with a negative scale is not provided")
        if inner[0] == "texture":
            return ("texture", tuple(float(x) * k for x in inner[1]))
        T = self.s.textures[inner[1]]
        key = ("scaled", inner[1], k)
        if key not in self.tex_cache:
            self.tex_cache[key] = self.s.add_texture(T["rgb"], scale=T["scale"] * k, invert_x=T["invert_x"],
                                                     invert_y=T["invert_y"])
        return ("image", self.tex_cache[key])

    # BSDFs: returns the index in the scene's BSDF table
    def bsdf(self, el, params=None):
        kind = _type(el)
        p = self.props(el) if params is None else params
        if kind == "Diffuse":   # Diffuse.cpp:11-18
            b = D.bsdf(D.BSDF_DIFFUSE, albedo=self._tex_or(p, "albedo", (0.5, 0.5, 0.5)),
                       tex_albedo=self._image(p, "albedo"))
        elif kind == "RoughConductor":   # RoughConductor.cpp:13-30, tools/Common.cpp:56-81
            eta, k = self._conductor_ior(p)
            alpha = self._tex_or(p, "alpha", 0.2)
            if isinstance(alpha, tuple):
                alpha = (alpha[0] + alpha[0] + alpha[0]) / 3.0
            b = D.bsdf(D.BSDF_ROUGH_CONDUCTOR, distribution=_dist(p.get("distribution", "beckmann")),
                       alpha=alpha, eta=eta, k=k, reflectance=self._tex_or(p, "reflectanceTexture", (1.0, 1.0, 1.0)),
                       tex_reflectance=self._image(p, "reflectanceTexture"), tex_alpha=self._image(p, "alpha"))
        elif kind == "RoughDielectric":   # RoughDielectric.cpp:13-32
            alpha = self._tex_or(p, "alpha", 0.2)
            if isinstance(alpha, tuple):
                alpha = (alpha[0] + alpha[0] + alpha[0]) / 3.0
            b = D.bsdf(D.BSDF_ROUGH_DIELECTRIC, distribution=_dist(p.get("distribution", "beckmann")),
                       alpha=alpha, eta_int=p.get("etaInt", 1.5046), eta_ext=p.get("etaExt", 1.000277),
                       reflectance=self._tex_or(p, "reflectanceTexture", (1.0, 1.0, 1.0)),
                       transmittance=self._tex_or(p, "transmittedTexture", (1.0, 1.0, 1.0)),
                       tex_reflectance=self._image(p, "reflectanceTexture"),
                       tex_transmittance=self._image(p, "transmittedTexture"), tex_alpha=self._image(p, "alpha"))
        elif kind == "SmoothLayeredBSDF":   # SmoothLayeredBSDF.cpp:12-28
            base = p.get("baseBSDF")
            albedo = (0.5, 0.5, 0.5)
            if base is not None:
                bd = self.s.bsdfs[base]
                if bd["type"] != D.BSDF_DIFFUSE:
                    raise UnsupportedScene("SmoothLayeredBSDF over a non-Diffuse base is not provided")
                if any(bd.get(k) is not None for k in D.TEX_PARAMS):
                    raise UnsupportedScene("SmoothLayeredBSDF over a textured base is not provided")
                albedo = bd["albedo"]
            b = D.bsdf(D.BSDF_SMOOTH_LAYERED, albedo=albedo, eta_int=p.get("etaInt", 1.5046),
                       eta_ext=p.get("etaExt", 1.000277), thickness=p.get("thickness", 1.2),
                       absorbance=p.get("absorbance", (0.0, 0.0, 0.0)))
        elif kind == "LayeredBSDF":   # LayeredBSDF.cpp:17-36
            base = p.get("baseBSDF")
            bd = D.bsdf(D.BSDF_ROUGH_CONDUCTOR)   # RoughConductor(Parameters()): eta = k = 0
            if base is not None:
                bd = self.s.bsdfs[base]
                if bd["type"] != D.BSDF_ROUGH_CONDUCTOR:
                    raise UnsupportedScene("LayeredBSDF over a non-RoughConductor base is not provided")
                if any(bd.get(k) is not None for k in D.TEX_PARAMS):
                    raise UnsupportedScene("LayeredBSDF over a textured base is not provided")
            b = D.bsdf(D.BSDF_LAYERED, distribution=_dist(p.get("distribution", "ggx")),
                       alpha=p.get("alphaTop", 0.01), eta_int=p.get("etaInt", 1.5046),
                       eta_ext=p.get("etaExt", 1.000277), thickness=p.get("thickness", 1.2),
                       absorbance=p.get("absorbance", (0.0, 0.0, 0.0)), eta=bd["eta"], k=bd["k"],
                       reflectance=bd["reflectance"], distribution_base=bd["distribution"], alpha_base=bd["alpha"])
        elif kind == "Dielectric":   # Dielectric.cpp:10-17
            b = D.bsdf(D.BSDF_DIELECTRIC, eta_int=p.get("etaInt", 1.5046), eta_ext=p.get("etaExt", 1.000277),
                       reflectance=self._tex_or(p, "reflectanceTexture", (1.0, 1.0, 1.0)),
                       transmittance=self._tex_or(p, "transmittedTexture", (1.0, 1.0, 1.0)),
                       tex_reflectance=self._image(p, "reflectanceTexture"),
                       tex_transmittance=self._image(p, "transmittedTexture"))
        elif kind == "Conductor":   # Conductor.cpp:13-21, tools/Common.cpp:56-81
            eta, k = self._conductor_ior(p)
            b = D.bsdf(D.BSDF_CONDUCTOR, eta=eta, k=k,
                       reflectance=self._tex_or(p, "reflectanceTexture", (1.0, 1.0, 1.0)),
                       tex_reflectance=self._image(p, "reflectanceTexture"))
        elif kind == "Mirror":   # Mirror.cpp:7-15
            b = D.bsdf(D.BSDF_MIRROR)
        elif kind == "SheetDielectric":   # SheetDielectric.cpp:10-17
            b = D.bsdf(D.BSDF_SHEET_DIELECTRIC, eta_int=p.get("etaInt", 1.5046), eta_ext=p.get("etaExt", 1.000277),
                       reflectance=self._tex_or(p, "reflectanceTexture", (1.0, 1.0, 1.0)),
                       transmittance=self._tex_or(p, "transmittedTexture", (1.0, 1.0, 1.0)),
                       tex_reflectance=self._image(p, "reflectanceTexture"),
                       tex_transmittance=self._image(p, "transmittedTexture"))
        elif kind == "Microfacet":   # Microfacet.cpp:11-25: kd a color or a texture, alpha a real
            b = D.bsdf(D.BSDF_MICROFACET, albedo=self._tex_or(p, "kd", (0.0, 0.0, 0.0)),
                       tex_albedo=self._image(p, "kd"), alpha=float(p.get("alpha", 0.2)),
                       eta_int=p.get("etaInt", 1.5946), eta_ext=p.get("etaExt", 1.000277),
                       distribution=_dist(p.get("distribution", "ggx")), ks=float(p.get("probabilitySpecular", 1.0)))
        elif kind == "TwoSides":   # TwoSides.cpp:5-15
            front = p.get("bsdf")
            if front is None:
                raise UnsupportedScene("TwoSides without a bsdf")
            back = p.get("bsdf2", front)
            if back != front:
                raise UnsupportedScene("TwoSides with a different bsdf2 is not provided")
            b = dict(self.s.bsdfs[front], two_sided=True)
        else:
            raise UnsupportedScene("BSDF type %s is not provided" % kind)
        return self.s.add_bsdf(b)

    def _conductor_ior(self, p):
        """IORHelper::evalConductorIOR (tools/Common.cpp:56-81): a named
        material's RGB eta and k (the caller's `materials`, else the
        reference's eight names converted from its data/IOR spectra), else
        the eta and absorption colors; an unknown name is reported and falls
        back to the colors, as in the reference."""
        from .conductor_ior import MATERIALS
        mat = p.get("material", "")
        if mat:
            if mat in self.materials:
                return self.materials[mat]
            if mat in MATERIALS:
                return MATERIALS[mat]
            warnings.warn("material %s not found" % mat)
        return p.get("eta", (0.0, 0.0, 0.0)), p.get("absorption", (0.0, 0.0, 0.0))

    def phase(self, p):
        ph = p.get("phaseFunction")
        if ph is None:
            return dict(phase=D.PHASE_ISOTROPIC)   # Medium.cpp:9
        _, kind, pp = ph
        if kind == "HGPhaseFunction":
            return dict(phase=D.PHASE_HG, g=pp.get("g", -0.8))   # HGPhaseFunction.cpp:8
        if kind == "IsotropicPhaseFunction":
            return dict(phase=D.PHASE_ISOTROPIC)
        raise UnsupportedScene("phase function %s is not provided" % kind)

    def medium(self, el):
        kind = _type(el)
        p = self.props(el)
        if p.get("temperature", 0.0) or p.get("scaleEmissivity", 1.0) != 1.0:
            raise UnsupportedScene("emissive media are not provided")
        if kind == "Homogeneous":   # Homogeneous.cpp:9-14
            m = dict(type=D.MEDIUM_HOMOGENEOUS, sigma_a=p.get("sigmaA", (0.15, 0.15, 0.15)),
                     sigma_s=p.get("sigmaS", (0.15, 0.15, 0.15)), scale=p.get("scale", 1.0))
        elif kind == "Heterogeneous":   # Heterogeneous.cpp:21-37
            vol = p.get("volume")
            if vol is None or vol[1] != "GridVolume":
                raise UnsupportedScene("Heterogeneous media need a GridVolume")
            dens, lo, hi = load_vol(self.resolve(vol[2].get("path", "")))
            m = dict(type=D.MEDIUM_HETEROGENEOUS, albedo=p.get("albedo", (0.0, 0.0, 0.0)), density=dens,
                     grid_min=lo, grid_max=hi, centered=int(p.get("centered", True)),
                     to_world=np.asarray(p.get("toWorld", np.eye(4)), np.float64), scale=p.get("scale", 1.0))
        else:
            raise UnsupportedScene("medium type %s is not provided" % kind)
        m.update(self.phase(p))
        return self.s.add_medium(m)

    # XMLLoader::handleObject (XMLLoader.cpp:293-398)
    def shape(self, el):
        kind = _type(el)
        bsdf, light = -1, None
        rest = []
        for c in el:
            if c.tag == "bsdf":
                if bsdf >= 0:
                    warnings.warn("only 1 BSDF allowed for %s" % kind)
                    continue
                bsdf = self.ref_bsdf[c.get("ref")] if c.get("ref") else self.bsdf(c)
            elif c.tag == "light":
                if light is not None:
                    warnings.warn("only 1 light allowed for %s" % kind)
                    continue
                light = (_type(c), self.props(c))
            elif c.tag == "bssrdf":
                raise UnsupportedScene("BSSRDFs are not provided")
            else:
                rest.append(c)
        holder = ET.Element("shape")
        holder.extend(rest)
        p = self.props(holder)
        interior = p.get("interior", -1)
        exterior = p.get("exterior", -1)
        to_world = np.asarray(p.get("toWorld", np.eye(4, dtype=F32)), F32)
        if light is not None and light[0] not in ("AreaLight", "MeshLight"):
            raise UnsupportedScene("shape light type %s is not provided" % light[0])
        if kind in ("Mesh", "Cube"):
            if kind == "Mesh":
                if p.get("useMtl", False):
                    raise UnsupportedScene("useMtl (OBJ materials) is not provided")
                from .core import load_obj
                v, n, uv, t = load_obj(self.resolve(p.get("path", "")), to_world)
                if uv is not None and len(uv) < 3:   # Triangle.cpp:155 uses uvs from three on
                    uv = None
            else:
                v, n, uv, t = cube_mesh(to_world)
            mi = self.s.add_mesh(v, t, bsdf=bsdf, interior=interior, exterior=exterior, normals=n, uvs=uv)
            if light is not None:   # MeshFactory.h:88-114
                li = self.s.add_area_light(light[1].get("radiance", (0.0, 0.0, 0.0)), D.SHAPE_MESH, mi,
                                           mesh_light=light[0] == "MeshLight")
                self.s.meshes[mi]["light"] = li
        elif kind in ("Sphere", "Plane"):
            if kind == "Sphere":
                si = self.s.add_sphere(p.get("radius", 1.0), np.asarray(to_world, np.float64), bsdf=bsdf,
                                       interior=interior, exterior=exterior)
            else:   # Plane.cpp:7-18
                si = self.s.add_plane(np.asarray(to_world, np.float64), bsdf=bsdf, interior=interior,
                                      exterior=exterior)
            if light is not None:
                li = self.s.add_area_light(light[1].get("radiance", (0.0, 0.0, 0.0)), D.SHAPE_SPHERE, si,
                                           mesh_light=light[0] == "MeshLight")
                self.s.spheres[si]["light"] = li
        else:
            raise UnsupportedScene("shape type %s is not provided" % kind)

    def camera(self, el):
        kind = _type(el)
        if kind != "NoriPerspective":
            raise UnsupportedScene("camera type %s is not provided" % kind)
        rest = []
        for c in el:
            if c.tag == "transform":
                self.camera_transform = _transform(c)
            elif c.tag == "filter":   # ReconstructionFilter.cpp:12-18 and the filters' constructors
                fp = self.props(c)
                rx, ry = fp.get("radiusX", 0.5), fp.get("radiusY", 0.5)
                kind = _type(c)
                if kind == "BoxFilter":
                    self.filter = D.box_filter(rx, ry)
                elif kind == "GaussianFilter":
                    self.filter = D.gaussian_filter(rx, ry, fp.get("alpha"), fp.get("omega"))
                elif kind == "MitchellNetravaliFilter":
                    self.filter = D.mitchell_filter(rx, ry, fp.get("B", 1.0 / 3), fp.get("C", 1.0 / 3))
                else:
                    raise UnsupportedScene("filter %s is not provided" % kind)
            else:
                rest.append(c)
        holder = ET.Element("camera")
        holder.extend(rest)
        self.camera_params = self.props(holder)

    def lights(self, el):
        for c in el:
            kind = _type(c)
            p = self.props(c)
            if kind == "PointLight":   # PointLight.cpp:7-11
                self.s.add_point_light(p.get("position", (0.0, 0.0, 0.0)), p.get("intensity", (0.0, 0.0, 0.0)))
                continue
            if kind == "SpotLight":    # SpotLight.cpp:8-15
                self.s.add_spot_light(np.asarray(p.get("toWorld", np.eye(4)), np.float64),
                                      p.get("intensity", (0.0, 0.0, 0.0)),
                                      p.get("falloffStart", 30.0), p.get("totalWidth", 60.0))
                continue
            if kind != "EnvironmentLight":
                raise UnsupportedScene("light type %s is not provided" % kind)
            if p.get("isProbe", False) or p.get("offsetU", 0.0) or p.get("offsetV", 0.0):
                raise UnsupportedScene("EnvironmentLight isProbe / offsets are not provided")
            # ImageLoader::load(path, ALL, gamma) (EnvironmentLight.cpp:18):
            # .hdr and .exr linear, 8-bit images decoded from sRGB
            from .images import ImageError, load_image
            path = self.resolve(p.get("path", ""))
            try:
                rgb = load_image(path, gamma=float(p.get("gamma", 0.0)))
            except (ImageError, OSError) as e:
                raise UnsupportedScene("EnvironmentLight %s: %s" % (p.get("path", ""), e))
            self.s.add_env_light(rgb, scale=p.get("scale", 1.0),
                                 to_world=np.asarray(p.get("toWorld", np.eye(4)), np.float64))

    def load(self):
        root = ET.parse(self.path).getroot()
        for el in root:   # XMLLoader.cpp:56-133
            key = el.tag
            if key == "camera":
                self.camera(el)
            elif key == "lights":
                self.lights(el)
            elif key == "parameters":
                bx, by = 32, 32
                for c in el:
                    if c.tag == "blockSizeX":
                        bx = int(c.text)
                    elif c.tag == "blockSizeY":
                        by = int(c.text)
                    elif c.tag == "fileName":   # where main.cpp:560-563 saves the image
                        self.file_name = (c.text or "").strip()
                self.block = (bx, by)
            elif key == "sampler":
                # the device draws every path from its own stream (the
                # path-stream sampler); a StratifiedSampler's sample count is
                # kept, its stratification is not
                if _type(el) == "StratifiedSampler":
                    warnings.warn("StratifiedSampler: rendered with per-path random streams")
                elif _type(el) != "RandomSampler":
                    raise UnsupportedScene("sampler %s is not provided" % el.get("type"))
                self.spp = int(self.props(el).get("sampleNumber", 1))
            elif key == "integrator":
                kind = _type(el)
                p = self.props(el)
                ig = {"PathTracingMIS": D.INTEGRATOR_PATH_MIS, "VolPathTracing": D.INTEGRATOR_VOLPATH}.get(kind)
                if ig is None:
                    raise UnsupportedScene("integrator %s is not provided" % kind)
                strat = {"all_lights": D.STRATEGY_ALL_LIGHTS, "one_light_uniform": D.STRATEGY_ONE_LIGHT_UNIFORM,
                         "one_light_weighted": D.STRATEGY_ONE_LIGHT_WEIGHTED}[p.get("strategy", "one_light_uniform")]
                self.s.integrator = dict(integrator=ig, max_depth=p.get("maxDepth", 1000),
                                         min_depth=p.get("minDepth", 3), strategy=strat)
            elif key == "medium":
                self.camera_medium = self.medium(el)
                if el.get("id"):
                    self.ref_medium[el.get("id")] = self.camera_medium
            elif key == "objects":
                for c in el:
                    self.shape(c)
            elif key == "bsdf":
                self.ref_bsdf[el.get("id")] = self.bsdf(el)
                self.ref_bsdf_name[el.get("id")] = el.get("name") or ""
            elif key == "transform":
                self.ref_transform[el.get("id")] = _transform(el)
        if self.camera_params is None:
            raise UnsupportedScene("the scene has no camera")
        cp = self.camera_params
        cam = D.camera(int(cp.get("sizeX", 768)), int(cp.get("sizeY", 768)), cp.get("fov", 30.0),
                       np.asarray(self.camera_transform, np.float64), near=cp.get("nearClip", 1e-4),
                       far=cp.get("farClip", 1e4), medium=self.camera_medium)
        cam["aperture_radius"] = cp.get("apertureRadius", 0.0)
        cam["filter"] = self.filter
        cam["focal_plane"] = cp.get("focalPlane", 3.4028234663852886e38)
        self.s.camera = cam
        self.s.spp = self.spp
        self.s.block = self.block
        self.s.file_name = self.file_name
        return self.s


def _dist(name):
    # MicrofacetDistribution names (bsdf/MicrofacetDistribution.h:9-13)
    d = {"beckmann": D.DIST_BECKMANN, "phong": D.DIST_PHONG, "ggx": D.DIST_GGX}.get(name)
    if d is None:
        raise UnsupportedScene("microfacet distribution %s is not provided" % name)
    return d


def cube_mesh(to_world):
    """The Cube shape's mesh (geometricShape/Cube.cpp): the [-1, 1]^3 cube as
    six faces of four vertices with face normals and uvs (0,1) (1,1) (1,0)
    (0,0), two triangles per face, in the reference's face and vertex order,
    transformed to world.  Returns (vertices, normals, uvs, triangles)."""
    faces = [  # (normal axis, sign, four corners)
        ((0, -1, 0), [(1, -1, -1), (1, -1, 1), (-1, -1, 1), (-1, -1, -1)]),
        ((0, 1, 0), [(1, 1, -1), (-1, 1, -1), (-1, 1, 1), (1, 1, 1)]),
        ((1, 0, 0), [(1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)]),
        ((0, 0, 1), [(1, -1, 1), (1, 1, 1), (-1, 1, 1), (-1, -1, 1)]),
        ((-1, 0, 0), [(-1, -1, 1), (-1, 1, 1), (-1, 1, -1), (-1, -1, -1)]),
        ((0, 0, -1), [(1, 1, -1), (1, -1, -1), (-1, -1, -1), (-1, 1, -1)]),
    ]
    M = np.asarray(to_world, F32)
    NI = np.linalg.inv(M[:3, :3].astype(np.float64)).T.astype(F32)
    v, n, uv, t = [], [], [], []
    for f, (nrm, quad) in enumerate(faces):
        uv += [(0, 1), (1, 1), (1, 0), (0, 0)]
        for q in quad:
            p = np.asarray(q, F32)
            x = ((M[0, 0] * p[0] + M[0, 1] * p[1]) + M[0, 2] * p[2]) + M[0, 3]
            y = ((M[1, 0] * p[0] + M[1, 1] * p[1]) + M[1, 2] * p[2]) + M[1, 3]
            z = ((M[2, 0] * p[0] + M[2, 1] * p[1]) + M[2, 2] * p[2]) + M[2, 3]
            w = ((M[3, 0] * p[0] + M[3, 1] * p[1]) + M[3, 2] * p[2]) + M[3, 3]
            if w != 1 and w != 0:
                x, y, z = x / w, y / w, z / w
            v.append((x, y, z))
            n.append(NI @ np.asarray(nrm, F32))
        b = 4 * f
        t += [(b, b + 1, b + 2), (b + 3, b, b + 2)]
    return np.asarray(v, F32), np.asarray(n, F32), np.asarray(uv, F32), np.asarray(t, np.int32)


def load_vol(path):
    """GridVolume file (volume/GridVolume.cpp:7-59): "VOL", version 3, an
    encoding id, x/y/z resolution, a channel count and the float bounding
    box, then float data with x fastest.  The reference skips four bytes
    after the header before it reads the data (GridVolume.cpp:52-54), so
    voxel i holds the file's value i + 1 and the last voxel is left unread;
    the same offset is applied here, with 0 in the last voxel."""
    raw = open(path, "rb").read()
    if raw[:3] != b"VOL" or raw[3] != 3:
        raise ValueError("%s is not a valid volume data file" % path)
    rx, ry, rz, _ch = np.frombuffer(raw, "<i4", 4, 8)
    lo = tuple(float(x) for x in np.frombuffer(raw, "<f4", 3, 24))
    hi = tuple(float(x) for x in np.frombuffer(raw, "<f4", 3, 36))
    n = int(rx) * int(ry) * int(rz)
    data = np.frombuffer(raw, "<f4", min(n, max(0, (len(raw) - 52) // 4)), 52).astype(np.float32)
    dens = np.zeros(n, np.float32)
    dens[:len(data)] = data
    return dens.reshape(int(rz), int(ry), int(rx)), lo, hi


def load_scene(path, materials=None):
    """Read a reference scene file.  `materials` maps conductor material
    names (material="gold") to (eta rgb, k rgb), overriding the reference's
    eight names (conductor_ior.py); the reference derives them
    from spectral data files (tools/Common.cpp:56-81)."""
    return _Loader(path, materials).load()
