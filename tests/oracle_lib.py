"""ctypes loader for the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg import this module.
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from raytracer_gb300 import desc as D  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build_oracle
        path = build_oracle.build_oracle()
        L = C.CDLL(path)
        L.oracle_scene_create.restype = C.c_void_p
        L.oracle_scene_create.argtypes = [C.POINTER(D.SceneDesc), C.c_int32]
        L.oracle_scene_destroy.argtypes = [C.c_void_p]
        L.oracle_render.argtypes = [C.c_void_p, C.POINTER(D.RenderDesc), C.c_void_p, C.c_int32]
        L.oracle_render_tiles.argtypes = [C.c_void_p, C.POINTER(D.RenderDesc), C.c_int32, C.c_int32, C.c_void_p,
                                          C.c_int32]
        L.oracle_render_tiles_strided.argtypes = [C.c_void_p, C.POINTER(D.RenderDesc), C.c_int32, C.c_int32,
                                                  C.c_int32, C.c_void_p, C.c_int32]
        L.oracle_render_paths.argtypes = [C.c_void_p, C.POINTER(D.RenderDesc), C.c_void_p, C.c_void_p,
                                          C.c_int32, C.c_void_p]
        L.oracle_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
        L.oracle_export_bvh.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                        C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.oracle_export_bvh.restype = C.c_int32
        L.oracle_bsdf_query.argtypes = [C.POINTER(D.BsdfDesc), C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_light_query.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_medium_query.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_scene_info.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_pcg_stream.argtypes = [C.c_uint64, C.c_uint64, C.c_int32, C.c_void_p]
        L.oracle_pcg_reals.argtypes = [C.c_uint64, C.c_uint64, C.c_int32, C.c_void_p]
        L.oracle_cdf_sample_reuse.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_cdf_sample.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
        L.oracle_camera_rays.argtypes = [C.POINTER(D.SceneDesc), C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_tex_eval.argtypes = [C.POINTER(D.TextureDesc), C.c_void_p, C.c_int32, C.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleScene:
    """A scene loaded into the CPU oracle."""

    def __init__(self, scene, strategy=None):
        self.scene = scene
        self.desc = scene.desc()
        st = scene.integrator["strategy"] if strategy is None else strategy
        self.h = lib().oracle_scene_create(C.byref(self.desc), st)

    def close(self):
        if self.h:
            lib().oracle_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def export_bvh(self):
        """The reference's two-level tree as one binary tree over the scene's
        triangles (nodes (n, 4) int32 left, right, first, count; prims), the
        form rt_scene_create_bvh takes."""
        nt = int(self.desc.n_triangles)
        nodes = np.zeros((max(1, 2 * nt), 4), np.int32)
        prims = np.zeros(max(1, nt), np.int32)
        nn, npr = C.c_int32(), C.c_int32()
        rc = lib().oracle_export_bvh(self.h, _p(nodes), len(nodes), _p(prims), len(prims), C.byref(nn), C.byref(npr))
        assert rc == 0
        return nodes[:nn.value].copy(), prims[:npr.value].copy()

    def render(self, spp, seed=0, sample_begin=0, threads=None, **over):
        rd = self.scene.render_desc(spp, seed=seed, sample_begin=sample_begin, **over)
        W, H = self.scene.camera["width"], self.scene.camera["height"]
        film = np.zeros((H, W, 4), np.float32)
        th = threads or os.cpu_count() or 1
        rc = lib().oracle_render(self.h, C.byref(rd), _p(film), th)
        assert rc == 0
        return film

    def render_tiles(self, spp, tile0, tile1, seed=0, threads=None, **over):
        rd = self.scene.render_desc(spp, seed=seed, **over)
        W, H = self.scene.camera["width"], self.scene.camera["height"]
        film = np.zeros((H, W, 4), np.float32)
        th = threads or os.cpu_count() or 1
        rc = lib().oracle_render_tiles(self.h, C.byref(rd), tile0, tile1, _p(film), th)
        assert rc == 0
        return film

    def render_tiles_strided(self, spp, tile0, count, stride, seed=0, threads=None, **over):
        """Tiles tile0, tile0 + stride, ... (count of them): a sample of the
        job grid spread over the whole frame."""
        rd = self.scene.render_desc(spp, seed=seed, **over)
        W, H = self.scene.camera["width"], self.scene.camera["height"]
        film = np.zeros((H, W, 4), np.float32)
        th = threads or os.cpu_count() or 1
        rc = lib().oracle_render_tiles_strided(self.h, C.byref(rd), tile0, count, stride, _p(film), th)
        assert rc == 0
        return film

    def render_paths(self, pixels, samples, seed=0, **over):
        rd = self.scene.render_desc(1, seed=seed, **over)
        px = np.ascontiguousarray(pixels, np.int32)
        sm = np.ascontiguousarray(samples, np.int32)
        out = np.zeros((len(px), 3), np.float32)
        lib().oracle_render_paths(self.h, C.byref(rd), _p(px), _p(sm), len(px), _p(out))
        return out

    def trace(self, rays, anyhit=False):
        rays = np.ascontiguousarray(rays, D.RAY_DTYPE)
        hits = np.zeros(len(rays), D.HIT_DTYPE)
        lib().oracle_trace(self.h, _p(rays), len(rays), int(anyhit), _p(hits))
        return hits

    def light_query(self, light, p, u):
        q = np.zeros(len(p), dtype=[("p", np.float32, 3), ("u", np.float32, 2)])
        q["p"], q["u"] = p, u
        r = np.zeros(len(p), dtype=np.dtype([("intensity", np.float32, 3), ("pdf", np.float32),
                                              ("to_light", np.float32, 3), ("distance", np.float32),
                                              ("point", np.float32, 3), ("normal", np.float32, 3),
                                              ("pdf_eval", np.float32), ("pad", np.float32)]))
        lib().oracle_light_query(self.h, light, _p(q), len(q), _p(r))
        return r

    def medium_query(self, medium, op, q):
        from raytracer_gb300.core import MEDIUM_Q, MEDIUM_R
        q = np.ascontiguousarray(q, MEDIUM_Q)
        r = np.zeros(len(q), MEDIUM_R)
        rc = lib().oracle_medium_query(self.h, medium, op, _p(q), len(q), _p(r))
        assert rc == 0
        return r

    def info(self):
        b = np.zeros(6, np.float32)
        n = np.zeros(1, np.int32)
        lib().oracle_scene_info(self.h, _p(b), _p(n))
        return b, int(n[0])

    def camera_rays(self, pxy, lens=None):
        pxy = np.ascontiguousarray(pxy, np.float32)
        out = np.zeros(len(pxy), D.RAY_DTYPE)
        ln = None if lens is None else np.ascontiguousarray(lens, np.float32)
        lib().oracle_camera_rays(C.byref(self.desc), _p(pxy), None if ln is None else _p(ln), len(pxy), _p(out))
        return out


def tex_eval(rgb, uv, scale=1.0, invert_x=False, invert_y=False):
    """The oracle's ImageTexture::eval of an (H, W, 3) image at (n, 2) uvs."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    uv = np.ascontiguousarray(uv, np.float32)
    t = D.TextureDesc(rgb.shape[1], rgb.shape[0], rgb.ctypes.data_as(C.POINTER(C.c_float)), scale,
                      int(invert_x), int(invert_y))
    out = np.zeros((len(uv), 3), np.float32)
    lib().oracle_tex_eval(C.byref(t), _p(uv), len(uv), _p(out))
    return out


BSDF_Q = np.dtype([("wi", np.float32, 3), ("wo", np.float32, 3), ("u", np.float32, 2)])
BSDF_R = np.dtype([("value", np.float32, 3), ("pdf", np.float32), ("wo", np.float32, 3),
                   ("relative_eta", np.float32), ("sampled_type", np.int32), ("pad", np.int32)])


def bsdf_query(bsdf_dict, op, q):
    b = D.bsdf_struct(bsdf_dict)
    q = np.ascontiguousarray(q, BSDF_Q)
    r = np.zeros(len(q), BSDF_R)
    lib().oracle_bsdf_query(C.byref(b), op, _p(q), len(q), _p(r))
    return r
