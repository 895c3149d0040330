"""Seeded synthetic scenes standing in for the benchmark configurations.

The reference ships no scene assets (its XML scenes point at OBJ/HDR/VOL
files that are not in the repository), so every workload is generated here,
deterministically from a seed, in the shapes and sizes the configurations
describe:

* cornell_box          -- Cornell-box room of 10 + 12 + 12 + 2 triangles,
                          Lambertian walls, quad area light (17,12,4),
                          256x256, PathTracingMIS, depth 8, RR from 3.
* displaced_icosphere  -- icosahedron subdivided 8x (1,310,720 triangles),
                          radially displaced by 5-octave fBm (amplitude 0.15),
                          on a 2-triangle ground; per-triangle categorical
                          material (40% GGX rough conductor with alpha in
                          [0.05,0.5] quantised to 32 meshes, 30% rough
                          dielectric IOR 1.5 alpha 0.1, 30% smooth-coated
                          diffuse); 1024x512 procedural sky with a 0.5 deg sun
                          disk of radiance 1e4; 1024x1024, depth 16.
* volume_grid          -- 128^3 fBm density (4 octaves) in a unit-cube null
                          boundary (sigma_t max 20, albedo 0.9, HG g=0.3),
                          homogeneous slab (sigma_t 2, albedo 0.8), sphere area
                          light r=0.2 radiance 50; VolPathTracing, depth 64.

Sizes can be scaled down for tests through the keyword arguments.
"""
import math

import numpy as np

from .desc import (SceneData, bsdf, camera, look_at, BSDF_DIFFUSE, BSDF_ROUGH_CONDUCTOR,
                   BSDF_ROUGH_DIELECTRIC, BSDF_SMOOTH_LAYERED, DIST_GGX, SHAPE_MESH, SHAPE_SPHERE,
                   MEDIUM_HOMOGENEOUS, MEDIUM_HETEROGENEOUS, PHASE_HG, PHASE_ISOTROPIC,
                   INTEGRATOR_PATH_MIS, INTEGRATOR_VOLPATH, STRATEGY_ONE_LIGHT_UNIFORM)

# Gold-like conductor constants (the reference's RoughConductor.cpp:27-28)
AU_ETA = (0.22273, 0.42791, 1.2597)
AU_K = (3.0325, 2.3345, 1.7531)


# ------------------------------------------------------------------ noise
def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841)) \
        ^ (iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32(seed * 0x9E3779B1 & 0xFFFFFFFF)
    h ^= h >> np.uint32(16)
    h *= np.uint32(0x7FEB352D)
    h ^= h >> np.uint32(15)
    h *= np.uint32(0x846CA68B)
    h ^= h >> np.uint32(16)
    return (h.astype(np.float64) / 4294967295.0) * 2.0 - 1.0


def value_noise(p, seed):
    """Trilinear value noise in [-1,1] with smoothstep fade (project-written)."""
    p = np.asarray(p, np.float64)
    f = np.floor(p)
    i = f.astype(np.int64)
    t = p - f
    w = t * t * (3.0 - 2.0 * t)
    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                c = _hash3(i[..., 0] + dx, i[..., 1] + dy, i[..., 2] + dz, seed)
                wx = w[..., 0] if dx else 1 - w[..., 0]
                wy = w[..., 1] if dy else 1 - w[..., 1]
                wz = w[..., 2] if dz else 1 - w[..., 2]
                out = out + c * wx * wy * wz
    return out


def fbm(p, octaves, seed, base_freq=1.0):
    total, amp, norm, freq = 0.0, 1.0, 0.0, base_freq
    for o in range(octaves):
        total = total + amp * value_noise(p * freq, seed + 101 * o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


# ------------------------------------------------------------------ geometry helpers
def _box(center, size, rot_y_deg=0.0):
    """12-triangle box (Cube tessellation, geometricShape/Cube.cpp:18-32),
    outward winding."""
    sx, sy, sz = np.asarray(size, np.float64) / 2
    c = np.array([[-sx, -sy, -sz], [sx, -sy, -sz], [sx, sy, -sz], [-sx, sy, -sz],
                  [-sx, -sy, sz], [sx, -sy, sz], [sx, sy, sz], [-sx, sy, sz]])
    a = np.radians(rot_y_deg)
    R = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
    v = c @ R.T + np.asarray(center, np.float64)
    f = np.array([[0, 2, 1], [0, 3, 2],   # -z
                  [4, 5, 6], [4, 6, 7],   # +z
                  [0, 1, 5], [0, 5, 4],   # -y
                  [3, 6, 2], [3, 7, 6],   # +y
                  [0, 4, 7], [0, 7, 3],   # -x
                  [1, 2, 6], [1, 6, 5]])  # +x
    return v.astype(np.float32), f


def _quad(p0, p1, p2, p3):
    v = np.array([p0, p1, p2, p3], np.float32)
    return v, np.array([[0, 1, 2], [0, 2, 3]])


def icosphere(level):
    """Subdivided icosahedron on the unit sphere: 20 * 4**level triangles."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                 np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                  [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                  [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                  [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        nv = len(v)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a, b = uk // nv, uk % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = (inv.reshape(3, -1) + nv)
        m01, m12, m20 = m[0], m[1], m[2]
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
        v = np.concatenate([v, mid])
    return v, f


def sky_env(width=1024, height=512, sun_elev_deg=35.0, sun_azim_deg=60.0, sun_radius_deg=0.5,
            sun_radiance=1e4):
    """Procedural lat-long sky in the reference's parameterisation
    (EnvironmentLight.cpp:113-121: theta = pi*row/H from +y, phi = 2pi*col/W,
    direction (sin phi sin theta, cos theta, -cos phi sin theta))."""
    rows = (np.arange(height) + 0.5) / height * np.pi
    cols = (np.arange(width) + 0.5) / width * 2 * np.pi
    th, ph = np.meshgrid(rows, cols, indexing="ij")
    d = np.stack([np.sin(ph) * np.sin(th), np.cos(th), -np.cos(ph) * np.sin(th)], -1)
    up = np.clip(d[..., 1], -1, 1)
    zen = np.array([0.25, 0.45, 1.0])
    hor = np.array([0.9, 0.9, 1.0])
    gnd = np.array([0.12, 0.1, 0.08])
    tsky = np.clip(up, 0, 1)[..., None] ** 0.5
    col = np.where(up[..., None] >= 0, hor * (1 - tsky) + zen * tsky, gnd + (hor - gnd) * np.exp(up[..., None] * 8))
    el, az = np.radians(sun_elev_deg), np.radians(sun_azim_deg)
    sth = np.pi / 2 - el
    sdir = np.array([np.sin(az) * np.sin(sth), np.cos(sth), -np.cos(az) * np.sin(sth)])
    cosang = d @ sdir
    sun = cosang >= np.cos(np.radians(sun_radius_deg))
    col = np.where(sun[..., None], np.array([1.0, 0.97, 0.92]) * sun_radiance, col)
    return np.ascontiguousarray(col.astype(np.float32)), int(sun.sum())


# ------------------------------------------------------------------ configurations
def cornell_box(width=256, height=256):
    """Config [0]: Cornell-box room built from triangles."""
    s = SceneData()
    s.name = "cornell_box_256"
    grey = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.73, 0.73, 0.73)))
    red = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.65, 0.05, 0.05)))
    green = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.12, 0.45, 0.15)))
    lightmat = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.78, 0.78, 0.78)))
    # room [0,1]^3, front face (z=1) open, inward-facing windings
    fl = _quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0))
    ce = _quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1))
    bk = _quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))
    lf = _quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1))
    rt = _quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0))
    wv = np.concatenate([fl[0], ce[0], bk[0]])
    wf = np.concatenate([fl[1], ce[1] + 4, bk[1] + 8])
    s.add_mesh(wv, wf, bsdf=grey)
    s.add_mesh(*lf, bsdf=red)
    s.add_mesh(*rt, bsdf=green)
    tv, tf = _box((0.33, 0.3, 0.37), (0.3, 0.6, 0.3), 15.0)
    s.add_mesh(tv, tf, bsdf=grey)
    sv, sf = _box((0.66, 0.15, 0.65), (0.3, 0.3, 0.3), -18.0)
    s.add_mesh(sv, sf, bsdf=grey)
    # 0.25 x 0.25 light just below the ceiling, facing down
    h = 0.999
    lv, lfc = _quad((0.375, h, 0.375), (0.625, h, 0.375), (0.625, h, 0.625), (0.375, h, 0.625))
    lm = s.add_mesh(lv, lfc, bsdf=lightmat)
    li = s.add_area_light((17.0, 12.0, 4.0), SHAPE_MESH, lm, mesh_light=True)
    s.meshes[lm]["light"] = li
    s.camera = camera(width, height, 40.0, look_at((0.5, 0.5, 2.4), (0.5, 0.5, 0.0), (0, 1, 0)))
    s.integrator = dict(integrator=INTEGRATOR_PATH_MIS, max_depth=8, min_depth=3,
                        strategy=STRATEGY_ONE_LIGHT_UNIFORM)
    return s


def cornell_smooth(width=128, height=128, max_depth=12):
    """The Cornell-box room furnished with the smooth BSDFs: a gold Conductor
    tall box, a glass (Dielectric) short box, a Mirror sphere, and two thin
    panels seen from both sides, one a TwoSides Diffuse and one a TwoSides
    RoughConductor."""
    s = cornell_box(width, height)
    s.name = "cornell_smooth_%d" % width
    from .desc import BSDF_CONDUCTOR, BSDF_DIELECTRIC, BSDF_MIRROR
    gold = s.add_bsdf(bsdf(BSDF_CONDUCTOR, eta=AU_ETA, k=AU_K))
    glass = s.add_bsdf(bsdf(BSDF_DIELECTRIC, eta_int=1.5, transmittance=(0.95, 0.97, 1.0)))
    mirror = s.add_bsdf(bsdf(BSDF_MIRROR))
    pan_d = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.2, 0.3, 0.7), two_sided=True))
    pan_c = s.add_bsdf(bsdf(BSDF_ROUGH_CONDUCTOR, distribution=DIST_GGX, alpha=0.25, eta=AU_ETA, k=AU_K,
                            two_sided=True))
    s.meshes[3]["bsdf"] = gold    # tall box
    s.meshes[4]["bsdf"] = glass   # short box
    T = np.eye(4)
    T[:3, 3] = (0.22, 0.1, 0.78)
    s.add_sphere(0.1, T, bsdf=mirror)
    # panels facing +z (toward the camera) in the upper corners, tilted so
    # that both of their sides see the light
    s.add_mesh(*_quad((0.05, 0.62, 0.55), (0.3, 0.62, 0.45), (0.3, 0.85, 0.6), (0.05, 0.85, 0.7)), bsdf=pan_d)
    s.add_mesh(*_quad((0.7, 0.62, 0.45), (0.95, 0.62, 0.55), (0.95, 0.85, 0.7), (0.7, 0.85, 0.6)), bsdf=pan_c)
    s.integrator = dict(s.integrator, max_depth=max_depth)
    return s


def cornell_delta_lights(width=96, height=96, area_light=True, spot_scale=1.0):
    """The Cornell-box room lit by a PointLight in the upper left and a
    SpotLight under the ceiling aimed straight down (falloff from 20 to 35
    degrees), beside the ceiling area light unless `area_light` is False.
    `spot_scale` scales the spot's toWorld, which narrows its cone: SpotLight
    reads the cosine from the inverse-transformed direction without
    renormalising it."""
    s = cornell_box(width, height)
    s.name = "cornell_delta_lights_%d" % width
    if not area_light:
        lm = len(s.meshes) - 1
        s.meshes[lm]["light"] = -1
        s.lights = []
    s.add_point_light((0.25, 0.8, 0.6), (0.9, 0.8, 0.6))
    c, sn = 0.0, 1.0   # rotation of +90 degrees about x: local +z -> world -y
    T = np.array([[1, 0, 0, 0.7], [0, c, -sn, 0.95], [0, sn, c, 0.5], [0, 0, 0, 1]], np.float64)
    T[:3, :3] *= spot_scale
    s.add_spot_light(T, (1.5, 1.6, 2.0), falloff_start=20.0, total_width=35.0)
    return s


def plane_room(width=64, height=64, textured=False):
    """A scene of Planes (geometricShape/Plane.cpp): a 3 x 3 floor plane
    under a rotated Diffuse panel, a tilted RoughConductor plane, and a
    0.3 x 0.3 Plane area light facing down, beside the Cornell room's tall
    box for a triangle mesh in the same render.  With `textured` the floor's
    albedo is a checker ImageTexture read at the plane's uv."""
    from .desc import BSDF_ROUGH_CONDUCTOR as RC, DIST_GGX
    s = SceneData()
    s.name = "plane_room_%d" % width
    grey = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.7, 0.7, 0.7)))
    red = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.7, 0.2, 0.15)))
    metal = s.add_bsdf(bsdf(RC, distribution=DIST_GGX, alpha=0.2, eta=AU_ETA, k=AU_K))
    lightmat = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.78, 0.78, 0.78)))
    if textured:
        t = s.add_texture(texture_image(32, 32, seed=3, kind="checker"))
        s.bsdfs[grey]["tex_albedo"] = t

    def rot_x(deg):
        a = math.radians(deg)
        return np.array([[1, 0, 0, 0], [0, math.cos(a), -math.sin(a), 0], [0, math.sin(a), math.cos(a), 0],
                         [0, 0, 0, 1]], np.float64)

    def place(scale, deg, tr):
        T = np.diag([scale[0], scale[1], 1.0, 1.0]) if len(scale) == 2 else np.diag(list(scale) + [1.0])
        M = rot_x(deg) @ T
        M[:3, 3] = tr
        return M

    s.add_plane(place((1.5, 1.5), -90.0, (0.5, 0.0, 0.5)), bsdf=grey)         # floor y = 0, normal +y
    s.add_plane(place((0.25, 0.2), -20.0, (0.3, 0.35, 0.4)), bsdf=red)       # panel
    s.add_plane(place((0.2, 0.3), -60.0, (0.75, 0.3, 0.3)), bsdf=metal)      # tilted metal sheet
    li = s.add_plane(place((0.15, 0.15), 90.0, (0.5, 0.95, 0.5)), bsdf=lightmat)   # light, normal -y
    s.spheres[li]["light"] = s.add_area_light((12.0, 11.0, 9.0), SHAPE_SPHERE, li, mesh_light=False)
    tv, tf = _box((0.6, 0.3, 0.6), (0.2, 0.6, 0.2), 15.0)
    s.add_mesh(tv, tf, bsdf=grey)
    s.camera = camera(width, height, 40.0, look_at((0.5, 0.6, 2.6), (0.5, 0.3, 0.4), (0, 1, 0)))
    s.integrator = dict(integrator=INTEGRATOR_PATH_MIS, max_depth=8, min_depth=3,
                        strategy=STRATEGY_ONE_LIGHT_UNIFORM)
    return s


def texture_image(width, height, seed=0, kind="checker"):
    """A seeded test image (H, W, 3) in [0, 1], rounded to half precision (so
    that an OpenEXR copy of it is exact): "checker" squares with a colour
    gradient, or "noise" (value noise)."""
    y, x = np.mgrid[0:height, 0:width].astype(np.float64)
    if kind == "checker":
        sq = ((x // 4 + y // 4) % 2)[..., None]
        grad = np.stack([x / max(1, width - 1), y / max(1, height - 1), 0.5 + 0 * x], axis=2)
        img = 0.15 + 0.7 * (0.6 * sq + 0.4 * grad)
    else:
        p = np.stack([x / 8.0, y / 8.0, np.full_like(x, 0.37)], axis=-1).reshape(-1, 3)
        v = value_noise(p, seed).reshape(height, width)
        img = np.repeat((0.5 + 0.5 * v)[..., None], 3, axis=2) * np.array([1.0, 0.8, 0.6])
    return np.clip(img, 0.0, 1.0).astype(np.float16).astype(np.float32)


def textured_room(width=96, height=96, max_depth=10):
    """The Cornell-box room with ImageTextures on every kind of parameter and
    every kind of texture coordinates: uv-mapped walls (repeated albedo), a
    left wall without uvs (barycentric coordinates, inverted texture), a
    RoughConductor tall box with alpha and reflectance textures, a
    RoughDielectric short box with a transmittance texture, a sphere with a
    textured Diffuse albedo (spherical coordinates) and a one-texel and a
    two-by-two texture."""
    from .desc import BSDF_CONDUCTOR
    s = SceneData()
    s.name = "textured_room_%d" % width
    checker = s.add_texture(texture_image(64, 48, 0, "checker"), scale=3.0)
    noise = s.add_texture(texture_image(32, 32, 1, "noise"))
    tiny = s.add_texture(np.array([[[0.8, 0.4, 0.2]]], np.float16).astype(np.float32))
    two = s.add_texture(np.array([[[0.9, 0.1, 0.1], [0.1, 0.9, 0.1]], [[0.1, 0.1, 0.9], [0.9, 0.9, 0.1]]],
                                 np.float16).astype(np.float32), invert_x=True, invert_y=True)
    walls = s.add_bsdf(bsdf(BSDF_DIFFUSE, tex_albedo=checker))
    left = s.add_bsdf(bsdf(BSDF_DIFFUSE, tex_albedo=two))
    green = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.12, 0.45, 0.15)))
    metal = s.add_bsdf(bsdf(BSDF_ROUGH_CONDUCTOR, distribution=DIST_GGX, eta=AU_ETA, k=AU_K, tex_alpha=noise,
                            tex_reflectance=checker))
    glass = s.add_bsdf(bsdf(BSDF_ROUGH_DIELECTRIC, distribution=DIST_GGX, alpha=0.15, eta_int=1.5,
                            tex_transmittance=noise))
    ball = s.add_bsdf(bsdf(BSDF_DIFFUSE, tex_albedo=checker))
    mirror_ball = s.add_bsdf(bsdf(BSDF_CONDUCTOR, eta=AU_ETA, k=AU_K, tex_reflectance=tiny))
    lightmat = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.78, 0.78, 0.78)))
    quad_uv = np.array([(0, 0), (1, 0), (1, 1), (0, 1)], np.float32)
    fl = _quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0))
    ce = _quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1))
    bk = _quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))
    s.add_mesh(np.concatenate([fl[0], ce[0], bk[0]]), np.concatenate([fl[1], ce[1] + 4, bk[1] + 8]), bsdf=walls,
               uvs=np.concatenate([quad_uv, quad_uv, quad_uv]))
    s.add_mesh(*_quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)), bsdf=left)
    s.add_mesh(*_quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)), bsdf=green)
    tv, tf = _box((0.33, 0.3, 0.37), (0.3, 0.6, 0.3), 15.0)
    s.add_mesh(tv, tf, bsdf=metal)
    sv, sf = _box((0.66, 0.15, 0.65), (0.3, 0.3, 0.3), -18.0)
    s.add_mesh(sv, sf, bsdf=glass)
    T = np.eye(4)
    T[:3, 3] = (0.22, 0.1, 0.78)
    T[:3, :3] = np.array([[1, 0, 0], [0, 0, -1], [0, 1, 0]])   # a pole and the uv seam toward the camera
    s.add_sphere(0.1, T, bsdf=ball)
    T2 = np.eye(4)
    T2[:3, 3] = (0.7, 0.42, 0.62)
    s.add_sphere(0.08, T2, bsdf=mirror_ball)
    h = 0.999
    lv, lfc = _quad((0.375, h, 0.375), (0.625, h, 0.375), (0.625, h, 0.625), (0.375, h, 0.625))
    lm = s.add_mesh(lv, lfc, bsdf=lightmat)
    li = s.add_area_light((17.0, 12.0, 4.0), SHAPE_MESH, lm, mesh_light=True)
    s.meshes[lm]["light"] = li
    s.camera = camera(width, height, 40.0, look_at((0.5, 0.5, 2.4), (0.5, 0.5, 0.0), (0, 1, 0)))
    s.integrator = dict(integrator=INTEGRATOR_PATH_MIS, max_depth=max_depth, min_depth=3,
                        strategy=STRATEGY_ONE_LIGHT_UNIFORM)
    return s


def displaced_icosphere(level=8, width=1024, height=1024, seed=0, alpha_bins=32,
                        env_size=(1024, 512), max_depth=16, env=None):
    """Config [1]: displaced icosphere on a ground quad under a sky (`env`:
    a precomputed sky_env image to share between scenes)."""
    s = SceneData()
    s.name = "displaced_icosphere_l%d_%d" % (level, width)
    v, f = icosphere(level)
    disp = fbm(v * 2.0 + 7.3, 5, seed)
    r = 1.0 + 0.15 * disp
    center = np.array([0.0, 1.15, 0.0])
    pos = (v * r[:, None] + center).astype(np.float32)
    rng = np.random.default_rng(seed)
    u = rng.random(len(f))
    alpha = rng.uniform(0.05, 0.5, len(f))
    abin = np.minimum((alpha - 0.05) / 0.45 * alpha_bins, alpha_bins - 1).astype(np.int64)
    group = np.where(u < 0.4, abin, np.where(u < 0.7, alpha_bins, alpha_bins + 1))
    order = np.argsort(group, kind="stable")
    f = f[order]
    group = group[order]
    bounds = np.searchsorted(group, np.arange(alpha_bins + 3))
    for g in range(alpha_bins + 2):
        a, b = bounds[g], bounds[g + 1]
        if b <= a:
            continue
        if g < alpha_bins:
            al = 0.05 + (g + 0.5) * 0.45 / alpha_bins
            m = s.add_bsdf(bsdf(BSDF_ROUGH_CONDUCTOR, distribution=DIST_GGX, alpha=al, eta=AU_ETA, k=AU_K))
        elif g == alpha_bins:
            m = s.add_bsdf(bsdf(BSDF_ROUGH_DIELECTRIC, distribution=DIST_GGX, alpha=0.1, eta_int=1.5))
        else:
            m = s.add_bsdf(bsdf(BSDF_SMOOTH_LAYERED, albedo=(0.7, 0.25, 0.2), eta_int=1.5, thickness=0.1))
        ids = f[a:b]
        uv_ids, remap = np.unique(ids.reshape(-1), return_inverse=True)
        s.add_mesh(pos[uv_ids], remap.reshape(-1, 3), bsdf=m)
    ground = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.4, 0.4, 0.4)))
    gv, gf = _quad((-12, 0, -12), (-12, 0, 12), (12, 0, 12), (12, 0, -12))
    s.add_mesh(gv, gf, bsdf=ground)
    if env is None:
        env, _ = sky_env(*env_size)
    s.add_env_light(env)
    s.camera = camera(width, height, 40.0, look_at((0.0, 2.2, 5.2), (0.0, 1.0, 0.0), (0, 1, 0)))
    s.integrator = dict(integrator=INTEGRATOR_PATH_MIS, max_depth=max_depth, min_depth=3,
                        strategy=STRATEGY_ONE_LIGHT_UNIFORM)
    return s


def density_grid(res=128, seed=0, octaves=4):
    """128^3 fBm density clamped to [0,1], x fastest (GridVolume layout)."""
    c = (np.arange(res) + 0.5) / res
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    p = np.stack([x, y, z], -1) * 4.0
    d = fbm(p, octaves, seed + 17)
    d = np.clip(0.5 + 1.2 * d, 0.0, 1.0)
    # fade to zero near the grid faces so the medium sits inside its cube
    edge = np.minimum.reduce([x, 1 - x, y, 1 - y, z, 1 - z])
    d *= np.clip(edge / 0.08, 0.0, 1.0)
    return np.ascontiguousarray(d.astype(np.float32))


def volume_grid(width=512, height=512, res=128, seed=0, max_depth=64):
    """Config [2]: grid medium in a null cube boundary, homogeneous slab below,
    sphere area light outside."""
    s = SceneData()
    s.name = "volume_grid_%d" % width
    dens = density_grid(res, seed)
    hetero = s.add_medium(dict(type=MEDIUM_HETEROGENEOUS, phase=PHASE_HG, g=0.3, scale=20.0,
                               albedo=(0.9, 0.9, 0.9), density=dens, grid_min=(0, 0, 0),
                               grid_max=(1, 1, 1), centered=1))
    slab = s.add_medium(dict(type=MEDIUM_HOMOGENEOUS, phase=PHASE_ISOTROPIC, sigma_a=(0.4, 0.4, 0.4),
                             sigma_s=(1.6, 1.6, 1.6), scale=1.0))
    cv, cf = _box((0.0, 0.75, 0.0), (1.0, 1.0, 1.0))
    s.add_mesh(cv, cf, bsdf=-1, interior=hetero)
    sv, sf = _box((0.0, 0.0, 0.0), (3.0, 0.4, 3.0))
    s.add_mesh(sv, sf, bsdf=-1, interior=slab)
    lm = s.add_bsdf(bsdf(BSDF_DIFFUSE, albedo=(0.0, 0.0, 0.0)))
    T = np.eye(4)
    T[:3, 3] = (1.1, 1.7, 0.9)
    sp = s.add_sphere(0.2, T, bsdf=lm)
    li = s.add_area_light((50.0, 50.0, 50.0), SHAPE_SPHERE, sp, mesh_light=False)
    s.spheres[sp]["light"] = li
    s.camera = camera(width, height, 35.0, look_at((0.0, 1.4, 4.2), (0.0, 0.6, 0.0), (0, 1, 0)))
    s.integrator = dict(integrator=INTEGRATOR_VOLPATH, max_depth=max_depth, min_depth=3,
                        strategy=STRATEGY_ONE_LIGHT_UNIFORM)
    return s


CONFIGS = {
    "cornell_box_256": lambda: cornell_box(),
    "displaced_icosphere_1024": lambda: displaced_icosphere(),
    "volume_grid_512": lambda: volume_grid(),
}


def batch_job(k, env=None):
    """Job k of the 64-scene batch: triangles log-uniform in [1e3, 5e5]
    (realised as the icosphere level nearest in log scale, 1,280 to 327,680
    triangles), resolution uniform over {128, 256, 512, 1024} squared, spp
    log-uniform in [4, 256], max depth 12, the displaced-icosphere material
    mix under the sky.  Returns (SceneData, spp)."""
    rng = np.random.default_rng(1000 + k)
    tris = np.exp(rng.uniform(np.log(1e3), np.log(5e5)))
    levels = np.arange(3, 8)
    level = int(levels[np.argmin(np.abs(np.log(20.0 * 4.0 ** levels) - np.log(tris)))])
    res = int(rng.choice([128, 256, 512, 1024]))
    spp = int(round(np.exp(rng.uniform(np.log(4), np.log(256)))))
    if env is None:
        env, _ = sky_env(1024, 512)
    s = displaced_icosphere(level=level, width=res, height=res, seed=k, max_depth=12, env=env)
    s.name = "batch%02d_l%d_%d_%dspp" % (k, level, res, spp)
    return s, spp
