"""Write a SceneData as a reference scene file (XML + OBJ + .hdr + .vol).

The generated scenes (raytracer_gb300.scenes) can then be rendered by the
reference renderer itself, and read back by xml_scene.load_scene.  Files use
the element and parameter names xml_scene reads (core/XMLLoader.cpp):
meshes are written in world space with an identity toWorld, one OBJ per
mesh; spheres and the camera carry their matrices; the environment map is a
flat (not run-length encoded) Radiance RGBE file, so it is quantised to RGBE
precision; grids are GridVolume files laid out for the reference's reader,
which skips four bytes after the 48-byte header (GridVolume.cpp:52-54).
"""
import os
import struct

import numpy as np

from . import desc as D
from .exr import write_exr

_BSDF_NAMES = {D.BSDF_DIFFUSE: "Diffuse", D.BSDF_ROUGH_CONDUCTOR: "RoughConductor",
               D.BSDF_ROUGH_DIELECTRIC: "RoughDielectric", D.BSDF_SMOOTH_LAYERED: "SmoothLayeredBSDF",
               D.BSDF_LAYERED: "LayeredBSDF", D.BSDF_DIELECTRIC: "Dielectric", D.BSDF_CONDUCTOR: "Conductor",
               D.BSDF_MIRROR: "Mirror", D.BSDF_SHEET_DIELECTRIC: "SheetDielectric", D.BSDF_MICROFACET: "Microfacet"}
_DIST_NAMES = {D.DIST_BECKMANN: "beckmann", D.DIST_PHONG: "phong", D.DIST_GGX: "ggx"}
_STRATEGY_NAMES = {D.STRATEGY_ALL_LIGHTS: "all_lights", D.STRATEGY_ONE_LIGHT_UNIFORM: "one_light_uniform",
                   D.STRATEGY_ONE_LIGHT_WEIGHTED: "one_light_weighted"}


def _f(x):
    return repr(float(np.float32(x)))


def _c(v):
    return " ".join(_f(x) for x in v)


def _matrix(m):
    return " ".join(_f(x) for x in np.asarray(m, np.float64).reshape(16))


def encode_rgbe(rgb):
    """Float RGB (h, w, 3) -> RGBE bytes (h, w, 4): the largest channel's
    exponent, mantissas scaled so that c * 2^(e - 136) rounds down to them."""
    rgb = np.asarray(rgb, np.float64)
    m = rgb.max(-1)
    out = np.zeros(rgb.shape[:2] + (4,), np.uint8)
    ok = m >= 1e-32
    e = np.zeros(m.shape, np.int64)
    e[ok] = np.floor(np.log2(m[ok])).astype(np.int64) + 1
    scale = np.ldexp(1.0, (8 - e).astype(np.int64))
    mant = np.floor(rgb * scale[..., None])
    mant = np.clip(mant, 0, 255)
    out[..., :3] = np.where(ok[..., None], mant, 0).astype(np.uint8)
    out[..., 3] = np.where(ok, np.clip(e + 128, 0, 255), 0).astype(np.uint8)
    return out


def write_hdr(path, rgb):
    rgbe = encode_rgbe(rgb)
    h, w = rgbe.shape[:2]
    with open(path, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n" % (h, w))
        f.write(rgbe.tobytes())
    return rgbe


def write_vol(path, density, lo=(0, 0, 0), hi=(1, 1, 1)):
    d = np.ascontiguousarray(density, np.float32)
    rz, ry, rx = d.shape
    with open(path, "wb") as f:
        f.write(b"VOL" + bytes([3]) + struct.pack("<i", 1) + struct.pack("<3i", rx, ry, rz) + struct.pack("<i", 1))
        f.write(struct.pack("<6f", *lo, *hi))
        f.write(b"\0\0\0\0")   # the reference's reader skips these four bytes
        f.write(d.tobytes())


def _write_obj(path, v, n, t, uv=None):
    with open(path, "w") as f:
        for p in v:
            f.write("v %s\n" % _c(p))
        if uv is not None:
            for q in uv:
                f.write("vt %s %s\n" % (_f(q[0]), _f(q[1])))
        if n is not None:
            for q in n:
                f.write("vn %s\n" % _c(q))
        for a, b, c in t + 1:
            if n is not None and uv is not None:
                f.write("f %d/%d/%d %d/%d/%d %d/%d/%d\n" % (a, a, a, b, b, b, c, c, c))
            elif n is not None:
                f.write("f %d//%d %d//%d %d//%d\n" % (a, a, b, b, c, c))
            elif uv is not None:
                f.write("f %d/%d %d/%d %d/%d\n" % (a, a, b, b, c, c))
            else:
                f.write("f %d %d %d\n" % (a, b, c))


def _tex_xml(pad, name, c):
    return ('%s  <texture name="%s" type="ConstantTexture"><color name="albedo" value="%s"/></texture>'
            % (pad, name, _c(c)))


def _bsdf_xml(b, indent, tex=()):
    """`tex`: per scene texture, the inner XML of its ImageTexture element."""
    pad = " " * indent

    def image(name, key):
        return '%s  <texture name="%s" type="ImageTexture">%s</texture>' % (pad, name, tex[b[key]])

    def refl_trans(names):
        out = []
        for name, key, tkey in names:
            if b.get(tkey) is not None:
                out.append(image(name, tkey))
            elif tuple(b[key]) != (1.0, 1.0, 1.0):
                out.append(_tex_xml(pad, name, b[key]))
        return out

    def alpha_line():
        if b.get("tex_alpha") is not None:
            return image("alpha", "tex_alpha")
        return '%s  <double name="alpha" value="%s"/>' % (pad, _f(b["alpha"]))

    if b.get("two_sided"):
        inner = _bsdf_xml(dict(b, two_sided=False), indent + 2, tex)
        inner[0] = inner[0].replace('<bsdf type=', '<bsdf name="bsdf" type=')
        return ['%s<bsdf type="TwoSides">' % pad] + inner + ["%s</bsdf>" % pad]
    name = _BSDF_NAMES[b["type"]]
    lines = ['%s<bsdf type="%s">' % (pad, name)]
    refl = ("reflectanceTexture", "reflectance", "tex_reflectance")
    trans = ("transmittedTexture", "transmittance", "tex_transmittance")
    if b["type"] == D.BSDF_DIFFUSE:
        if b.get("tex_albedo") is not None:
            lines.append(image("albedo", "tex_albedo"))
        else:
            lines.append('%s  <color name="albedo" value="%s"/>' % (pad, _c(b["albedo"])))
    elif b["type"] == D.BSDF_ROUGH_CONDUCTOR:
        lines += ['%s  <color name="eta" value="%s"/>' % (pad, _c(b["eta"])),
                  '%s  <color name="absorption" value="%s"/>' % (pad, _c(b["k"])),
                  alpha_line(),
                  '%s  <string name="distribution" value="%s"/>' % (pad, _DIST_NAMES[b["distribution"]])]
        lines += refl_trans([refl])
    elif b["type"] == D.BSDF_ROUGH_DIELECTRIC:
        lines += [alpha_line(),
                  '%s  <double name="etaInt" value="%s"/>' % (pad, _f(b["eta_int"])),
                  '%s  <double name="etaExt" value="%s"/>' % (pad, _f(b["eta_ext"])),
                  '%s  <string name="distribution" value="%s"/>' % (pad, _DIST_NAMES[b["distribution"]])]
        lines += refl_trans([refl, trans])
    elif b["type"] == D.BSDF_DIELECTRIC:
        lines += ['%s  <double name="etaInt" value="%s"/>' % (pad, _f(b["eta_int"])),
                  '%s  <double name="etaExt" value="%s"/>' % (pad, _f(b["eta_ext"]))]
        lines += refl_trans([refl, trans])
    elif b["type"] == D.BSDF_CONDUCTOR:
        lines += ['%s  <color name="eta" value="%s"/>' % (pad, _c(b["eta"])),
                  '%s  <color name="absorption" value="%s"/>' % (pad, _c(b["k"]))]
        lines += refl_trans([refl])
    elif b["type"] == D.BSDF_MIRROR:
        pass
    elif b["type"] == D.BSDF_SHEET_DIELECTRIC:
        lines += ['%s  <double name="etaInt" value="%s"/>' % (pad, _f(b["eta_int"])),
                  '%s  <double name="etaExt" value="%s"/>' % (pad, _f(b["eta_ext"]))]
        lines += refl_trans([refl, trans])
    elif b["type"] == D.BSDF_MICROFACET:
        if b.get("tex_albedo") is not None:
            lines.append(image("kd", "tex_albedo"))
        else:
            lines.append('%s  <color name="kd" value="%s"/>' % (pad, _c(b["albedo"])))
        lines += ['%s  <double name="alpha" value="%s"/>' % (pad, _f(b["alpha"])),
                  '%s  <double name="etaInt" value="%s"/>' % (pad, _f(b["eta_int"])),
                  '%s  <double name="etaExt" value="%s"/>' % (pad, _f(b["eta_ext"])),
                  '%s  <string name="distribution" value="%s"/>' % (pad, _DIST_NAMES[b["distribution"]]),
                  '%s  <double name="probabilitySpecular" value="%s"/>' % (pad, _f(b.get("ks", 1.0)))]
    elif b["type"] == D.BSDF_SMOOTH_LAYERED:
        lines += ['%s  <double name="etaInt" value="%s"/>' % (pad, _f(b["eta_int"])),
                  '%s  <double name="etaExt" value="%s"/>' % (pad, _f(b["eta_ext"])),
                  '%s  <double name="thickness" value="%s"/>' % (pad, _f(b["thickness"])),
                  '%s  <color name="absorbance" value="%s"/>' % (pad, _c(b["absorbance"])),
                  '%s  <bsdf name="baseBSDF" type="Diffuse"><color name="albedo" value="%s"/></bsdf>'
                  % (pad, _c(b["albedo"]))]
    else:
        base = dict(b, type=D.BSDF_ROUGH_CONDUCTOR, distribution=b.get("distribution_base", D.DIST_BECKMANN),
                    alpha=b.get("alpha_base", 0.2))
        inner = _bsdf_xml(base, indent + 2, tex)
        inner[0] = inner[0].replace('<bsdf type=', '<bsdf name="baseBSDF" type=')
        lines += ['%s  <double name="etaInt" value="%s"/>' % (pad, _f(b["eta_int"])),
                  '%s  <double name="etaExt" value="%s"/>' % (pad, _f(b["eta_ext"])),
                  '%s  <double name="thickness" value="%s"/>' % (pad, _f(b["thickness"])),
                  '%s  <color name="absorbance" value="%s"/>' % (pad, _c(b["absorbance"])),
                  '%s  <double name="alphaTop" value="%s"/>' % (pad, _f(b["alpha"])),
                  '%s  <string name="distribution" value="%s"/>' % (pad, _DIST_NAMES[b["distribution"]])] + inner
    lines.append("%s</bsdf>" % pad)
    return lines


def _medium_xml(m, name, folder, stem, indent):
    pad = " " * indent
    if m["type"] == D.MEDIUM_HOMOGENEOUS:
        lines = ['%s<medium name="%s" type="Homogeneous">' % (pad, name),
                 '%s  <color name="sigmaA" value="%s"/>' % (pad, _c(m.get("sigma_a", (0.15,) * 3))),
                 '%s  <color name="sigmaS" value="%s"/>' % (pad, _c(m.get("sigma_s", (0.15,) * 3))),
                 '%s  <double name="scale" value="%s"/>' % (pad, _f(m.get("scale", 1.0)))]
    else:
        vol = stem + ".vol"
        write_vol(os.path.join(folder, vol), m["density"], m.get("grid_min", (0, 0, 0)), m.get("grid_max", (1, 1, 1)))
        lines = ['%s<medium name="%s" type="Heterogeneous">' % (pad, name),
                 '%s  <color name="albedo" value="%s"/>' % (pad, _c(m.get("albedo", (0, 0, 0)))),
                 '%s  <double name="scale" value="%s"/>' % (pad, _f(m.get("scale", 1.0))),
                 '%s  <bool name="centered" value="%s"/>' % (pad, "true" if m.get("centered", 1) else "false"),
                 '%s  <transform name="toWorld"><matrix value="%s"/></transform>'
                 % (pad, _matrix(m.get("to_world", np.eye(4)))),
                 '%s  <volume name="volume" type="GridVolume"><string name="path" value="%s"/></volume>' % (pad, vol)]
    if m.get("phase", D.PHASE_ISOTROPIC) == D.PHASE_HG:
        lines.append('%s  <phase name="phaseFunction" type="HGPhaseFunction"><double name="g" value="%s"/></phase>'
                     % (pad, _f(m.get("g", -0.8))))
    lines.append("%s</medium>" % pad)
    return lines


def _filter_xml(f):
    name = {D.FILTER_BOX: "BoxFilter", D.FILTER_GAUSSIAN: "GaussianFilter",
            D.FILTER_MITCHELL: "MitchellNetravaliFilter"}[f["type"]]
    body = '<double name="radiusX" value="%s"/><double name="radiusY" value="%s"/>' % (
        _f(f["radius"][0]), _f(f["radius"][1]))
    if f["type"] == D.FILTER_GAUSSIAN:
        body += '<double name="alpha" value="%s"/><double name="omega" value="%s"/>' % (
            _f(f["param"][0]), _f(f["param"][1]))
    elif f["type"] == D.FILTER_MITCHELL:
        body += '<double name="B" value="%s"/><double name="C" value="%s"/>' % (_f(f["param"][0]), _f(f["param"][1]))
    return '    <filter type="%s">%s</filter>' % (name, body)


def write_scene(scene, folder, spp=1, name="scene"):
    """Write `scene` as folder/name.xml plus its mesh, map and grid files.
    Returns the XML path."""
    os.makedirs(folder, exist_ok=True)
    s = scene
    cam = s.camera
    out = ["<?xml version='1.0' encoding='utf-8'?>", "<scene>"]
    it = s.integrator
    out += ['  <integrator type="%s">' % ("VolPathTracing" if it["integrator"] == D.INTEGRATOR_VOLPATH
                                         else "PathTracingMIS"),
            '    <integer name="maxDepth" value="%d"/>' % it["max_depth"],
            '    <integer name="minDepth" value="%d"/>' % it["min_depth"],
            '    <string name="strategy" value="%s"/>' % _STRATEGY_NAMES[it["strategy"]],
            "  </integrator>"]
    out += ['  <camera type="NoriPerspective">',
            '    <transform name="toWorld"><matrix value="%s"/></transform>' % _matrix(cam["camera_to_world"]),
            '    <double name="fov" value="%s"/>' % _f(cam["fov"]),
            '    <double name="nearClip" value="%s"/>' % _f(cam["near_clip"]),
            '    <double name="farClip" value="%s"/>' % _f(cam["far_clip"]),
            '    <integer name="sizeX" value="%d"/>' % cam["width"],
            '    <integer name="sizeY" value="%d"/>' % cam["height"],
            _filter_xml(cam.get("filter", D.box_filter())),
            "  </camera>"]
    block = getattr(s, "block", (32, 32))
    fname = getattr(s, "file_name", "")
    out += ["  <parameters>", "    <blockSizeX>%d</blockSizeX>" % block[0],
            "    <blockSizeY>%d</blockSizeY>" % block[1]]
    if fname:
        out.append("    <fileName>%s</fileName>" % fname)
    out += ["  </parameters>",
            '  <sampler type="RandomSampler"><integer name="sampleNumber" value="%d"/></sampler>' % spp]
    if cam.get("medium", -1) >= 0:
        out += _medium_xml(s.media[cam["medium"]], "camera", folder, "medium%d" % cam["medium"], 2)
    # lights are numbered in document order: shape lights with their shapes in
    # <objects>, the others (environment, point, spot) in a <lights> block that
    # goes before the objects when those lights come first, after them otherwise
    free = [li for li, L in enumerate(s.lights) if L["type"] != D.LIGHT_AREA]
    area = [li for li, L in enumerate(s.lights) if L["type"] == D.LIGHT_AREA]
    free_first = bool(free) and (not area or max(free) < min(area))
    if free and area and not free_first and min(free) < max(area):
        raise ValueError("the light order (environment/point/spot lights between shape lights) "
                         "cannot be written as one <lights> block")
    env_lines = []
    for li in free:
        L = s.lights[li]
        if L["type"] == D.LIGHT_ENV:
            hdr = "env%d.hdr" % li
            write_hdr(os.path.join(folder, hdr), L["rgb"])
            env_lines += ['    <light type="EnvironmentLight">',
                          '      <string name="path" value="%s"/>' % hdr,
                          '      <double name="scale" value="%s"/>' % _f(L.get("scale", 1.0)),
                          '      <transform name="toWorld"><matrix value="%s"/></transform>'
                          % _matrix(L.get("to_world", np.eye(4))),
                          "    </light>"]
        elif L["type"] == D.LIGHT_POINT:
            env_lines += ['    <light type="PointLight">',
                          '      <point name="position" value="%s"/>' % _c(L["position"]),
                          '      <color name="intensity" value="%s"/>' % _c(L["intensity"]),
                          "    </light>"]
        else:
            env_lines += ['    <light type="SpotLight">',
                          '      <transform name="toWorld"><matrix value="%s"/></transform>' % _matrix(L["to_world"]),
                          '      <color name="intensity" value="%s"/>' % _c(L["intensity"]),
                          '      <double name="falloffStart" value="%s"/>' % _f(L["falloff_start"]),
                          '      <double name="totalWidth" value="%s"/>' % _f(L["total_width"]),
                          "    </light>"]
    if env_lines:
        env_lines = ["  <lights>"] + env_lines + ["  </lights>"]
    env_first = free_first
    if env_first:
        out += env_lines
    # textures: half-float OpenEXR files, which the reference reads linearly
    # (ImageLoader.cpp:46-74), so their texels are quantised to half
    tex = []
    for ti, T in enumerate(getattr(s, "textures", [])):
        name = "tex%d.exr" % ti
        write_exr(os.path.join(folder, name), T["rgb"][::1])
        tex.append('<string name="path" value="%s"/><double name="scale" value="%s"/>'
                   '<bool name="invertX" value="%s"/><bool name="invertY" value="%s"/>'
                   % (name, _f(T.get("scale", 1.0)), "true" if T.get("invert_x") else "false",
                      "true" if T.get("invert_y") else "false"))
    out.append("  <objects>")
    for mi, m in enumerate(s.meshes):
        a, b = m["first_tri"], m["first_tri"] + m["n_tris"]
        tri = s.indices[a:b]
        used, remap = np.unique(tri.reshape(-1), return_inverse=True)
        v = s.vertices[used]
        n = None
        if s.normals is not None and not np.isnan(s.normals[used]).any():
            n = s.normals[used]
        uv = None
        uvs = getattr(s, "uvs", None)
        if uvs is not None and not np.isnan(uvs[used]).any():
            uv = uvs[used]
        obj = "mesh%d.obj" % mi
        _write_obj(os.path.join(folder, obj), v, n, remap.reshape(-1, 3).astype(np.int64), uv)
        out += ['    <shape type="Mesh">', '      <string name="path" value="%s"/>' % obj]
        if m["bsdf"] >= 0:
            out += _bsdf_xml(s.bsdfs[m["bsdf"]], 6, tex)
        if m["light"] >= 0:
            L = s.lights[m["light"]]
            out.append('      <light type="%s"><color name="radiance" value="%s"/></light>'
                       % ("MeshLight" if L.get("mesh_light", 1) else "AreaLight", _c(L["radiance"])))
        for key in ("interior", "exterior"):
            if m[key] >= 0:
                out += _medium_xml(s.media[m[key]], key, folder, "medium%d" % m[key], 6)
        out.append("    </shape>")
    for si, sp in enumerate(s.spheres):
        if sp.get("kind", D.ANALYTIC_SPHERE) == D.ANALYTIC_PLANE:
            out += ['    <shape type="Plane">',
                    '      <transform name="toWorld"><matrix value="%s"/></transform>' % _matrix(sp["to_world"])]
        else:
            out += ['    <shape type="Sphere">', '      <double name="radius" value="%s"/>' % _f(sp["radius"]),
                    '      <transform name="toWorld"><matrix value="%s"/></transform>' % _matrix(sp["to_world"])]
        if sp["bsdf"] >= 0:
            out += _bsdf_xml(s.bsdfs[sp["bsdf"]], 6, tex)
        if sp["light"] >= 0:
            L = s.lights[sp["light"]]
            out.append('      <light type="%s"><color name="radiance" value="%s"/></light>'
                       % ("MeshLight" if L.get("mesh_light", 1) else "AreaLight", _c(L["radiance"])))
        for key in ("interior", "exterior"):
            if sp[key] >= 0:
                out += _medium_xml(s.media[sp[key]], key, folder, "medium%d" % sp[key], 6)
        out.append("    </shape>")
    out.append("  </objects>")
    if not env_first:
        out += env_lines
    out.append("</scene>")
    path = os.path.join(folder, name + ".xml")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return path
