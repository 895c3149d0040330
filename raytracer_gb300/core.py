"""Python host binding over librtgpu.so (the C ABI in include/rtgpu.h).

This mirrors the reference's render entry points for the two path-tracing
integrators: a `Scene` is the flattened, initialised reference scene
(Scene::initialize, core/Scene.cpp:115-138) resident on the GPU, and
`Scene.render` is the render step of Scene::compute (core/Scene.cpp:83-101)
running PathTracingMIS::li or VolPathTracing::li for every path sample.
There is no CPU fallback: if the CUDA library is missing or no GPU is
present, construction raises.
"""
import ctypes as C
import os

import numpy as np

from . import desc as D

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librtgpu.so")

RT_OK = 0
_STATUS = {1: "RT_ERR_INVALID", 2: "RT_ERR_CUDA", 3: "RT_ERR_LIMIT", 4: "RT_ERR_NOMEM", 5: "RT_ERR_UNSUPPORTED"}


class ServerOpts(C.Structure):
    _fields_ = [("lanes", C.c_int32), ("max_queue", C.c_int32), ("device_budget_bytes", C.c_int64),
                ("lanes_only", C.c_int32), ("rmse_display", C.c_int32)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("spp_done", C.c_int32), ("rmse_estimate", C.c_float),
                ("queue_ms", C.c_float), ("run_ms", C.c_float), ("error", C.c_char * 128)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3


class Tuning(C.Structure):
    """rt_tuning: launch shapes, queue capacities and scheduling choices."""
    _fields_ = [("wave_paths", C.c_int32), ("lane_wave_paths", C.c_int32), ("trace_blocks_per_sm", C.c_int32),
                ("shade_blocks_per_sm", C.c_int32), ("sort_threshold", C.c_int32), ("lanes", C.c_int32),
                ("graphs", C.c_int32), ("volpath_wavefront", C.c_int32), ("batch_wavefront", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MeshData(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("vertices", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
                ("uvs", C.POINTER(C.c_float)), ("n_triangles", C.c_int32), ("indices", C.POINTER(C.c_int32))]


class RtError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_STATUS.get(status, status), msg))
        self.status = status


_lib = None


def lib():
    """Load librtgpu.so (built in-tree by raytracer_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RtError(5, "librtgpu.so not built (run raytracer_gb300.build.build())")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.rt_abi_version.restype = C.c_int32
    L.rt_last_error.restype = C.c_char_p
    L.rt_mix64.restype = C.c_uint64
    L.rt_mix64.argtypes = [C.c_uint64]
    L.rt_ctx_create.argtypes = [C.c_int32, C.POINTER(vp)]
    L.rt_ctx_destroy.argtypes = [vp]
    L.rt_ctx_set_stream.argtypes = [vp, vp]
    L.rt_scene_create.argtypes = [vp, C.POINTER(D.SceneDesc), C.POINTER(vp)]
    L.rt_scene_destroy.argtypes = [vp]
    L.rt_scene_info.argtypes = [vp, vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
    L.rt_render.argtypes = [vp, vp, C.POINTER(D.RenderDesc), vp, C.c_int32]
    L.rt_render_stats_get.argtypes = [vp, C.POINTER(D.RenderStats)]
    L.rt_ctx_set_profiling.argtypes = [vp, C.c_int32]
    L.rt_ctx_set_bvh_width.argtypes = [vp, C.c_int32]
    L.rt_ctx_set_wave_paths.argtypes = [vp, C.c_int32]
    L.rt_ctx_set_ray_sort.argtypes = [vp, C.c_int32]
    L.rt_ctx_set_graphs.argtypes = [vp, C.c_int32]
    L.rt_ctx_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.rt_ctx_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.rt_autotune.argtypes = [vp, C.POINTER(C.c_void_p), C.POINTER(D.RenderDesc), C.c_int32, C.c_int32,
                              C.POINTER(Tuning), C.POINTER(C.c_double)]
    L.rt_trace.argtypes = [vp, vp, vp, C.c_int32, C.c_int32, vp, C.c_int32]
    L.rt_render_paths.argtypes = [vp, vp, C.POINTER(D.RenderDesc), vp, vp, C.c_int32, vp]
    L.rt_render_paths.restype = C.c_int32
    L.rt_render_tile_static.argtypes = [vp, vp, C.POINTER(D.RenderDesc), C.c_int32, C.c_int32, vp]
    L.rt_render_tile_static.restype = C.c_int32
    L.rt_bsdf_query.argtypes = [vp, vp, C.c_int32, C.c_int32, vp, C.c_int32, vp]
    L.rt_light_query.argtypes = [vp, vp, C.c_int32, vp, C.c_int32, vp]
    L.rt_medium_query.argtypes = [vp, vp, C.c_int32, C.c_int32, vp, C.c_int32, vp]
    L.rt_batch_render.argtypes = [vp, C.POINTER(vp), C.POINTER(D.RenderDesc), C.c_int32, C.POINTER(vp), C.c_int32]
    L.rt_ctx_set_lanes.argtypes = [vp, C.c_int32]
    L.rt_server_start.argtypes = [vp, C.POINTER(ServerOpts), C.POINTER(vp)]
    L.rt_job_submit.argtypes = [vp, vp, C.POINTER(D.RenderDesc), C.c_float, C.POINTER(C.c_int64)]
    L.rt_job_poll.argtypes = [vp, C.c_int64, C.POINTER(JobInfo), vp]
    L.rt_job_wait.argtypes = [vp, C.c_int64, C.c_int32, C.POINTER(JobInfo), vp]
    L.rt_server_stop.argtypes = [vp]
    L.rt_obj_load.argtypes = [C.c_char_p, vp, C.POINTER(MeshData)]
    L.rt_obj_load.restype = C.c_int32
    L.rt_mesh_data_free.argtypes = [C.POINTER(MeshData)]
    L.rt_mesh_data_free.restype = None
    L.rt_hdr_load.argtypes = [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.POINTER(C.c_float))]
    L.rt_hdr_load.restype = C.c_int32
    L.rt_host_free.argtypes = [vp]
    L.rt_host_free.restype = None
    L.rt_bvh_stats.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.rt_bvh_stats.restype = C.c_int32
    L.rt_scene_create_bvh.argtypes = [vp, C.POINTER(D.SceneDesc), vp, C.c_int32, vp, C.c_int32, C.POINTER(vp)]
    L.rt_scene_create_bvh.restype = C.c_int32
    L.rt_bvh_import_check.argtypes = [vp, C.c_int32, vp, C.c_int32, vp, C.c_int32, C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32)]
    L.rt_bvh_import_check.restype = C.c_int32
    L.rt_ctx_set_bvh_builder.argtypes = [vp, C.c_int32]
    L.rt_ctx_set_bvh_builder.restype = C.c_int32
    L.rt_scene_refit.argtypes = [vp, vp, vp, vp, C.c_int32]
    L.rt_scene_refit.restype = C.c_int32
    L.rt_path_state_bytes.argtypes = [C.c_int32]
    L.rt_path_state_bytes.restype = C.c_int64
    for name in ("rt_ctx_create", "rt_ctx_destroy", "rt_ctx_set_stream", "rt_scene_create", "rt_scene_destroy",
                 "rt_scene_info", "rt_render", "rt_render_stats_get", "rt_ctx_set_profiling", "rt_ctx_set_bvh_width", "rt_ctx_set_wave_paths", "rt_ctx_set_ray_sort", "rt_ctx_set_graphs",
                 "rt_ctx_get_tuning", "rt_ctx_set_tuning", "rt_autotune",
                 "rt_trace", "rt_bsdf_query", "rt_light_query", "rt_medium_query", "rt_batch_render", "rt_ctx_set_lanes",
                 "rt_server_start", "rt_job_submit", "rt_job_poll", "rt_job_wait", "rt_server_stop"):
        getattr(L, name).restype = C.c_int32
    _lib = L
    return L


def _check(status):
    if status != RT_OK:
        raise RtError(status, lib().rt_last_error().decode())


def _p(a):
    return C.c_void_p(a.ctypes.data)


class Context:
    """One GPU and one CUDA stream (rt_ctx)."""

    def __init__(self, device=0):
        self.h = C.c_void_p()
        _check(lib().rt_ctx_create(device, C.byref(self.h)))
        self.device = device

    def close(self):
        if self.h:
            lib().rt_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        _check(lib().rt_ctx_set_stream(self.h, C.c_void_p(stream_ptr)))

    def set_profiling(self, level):
        """0 off, 1 per-kernel event timing, 2 timing + traversal counters."""
        _check(lib().rt_ctx_set_profiling(self.h, int(level)))

    def set_bvh_builder(self, device):
        """Trees of scenes created later: built on the device (True, a
        Morton-code linear BVH in milliseconds) or on the host (binned SAH)."""
        _check(lib().rt_ctx_set_bvh_builder(self.h, 1 if device else 0))

    def set_bvh_width(self, width):
        """Traversal tree for later renders and traces: 2 (default) or 8."""
        _check(lib().rt_ctx_set_bvh_width(self.h, int(width)))

    def set_wave_paths(self, paths):
        """Paths per wavefront batch of later renders (2^16..2^26)."""
        _check(lib().rt_ctx_set_wave_paths(self.h, int(paths)))

    def set_ray_sort(self, on):
        """Regroup secondary and shadow rays by octant and origin cell before tracing."""
        _check(lib().rt_ctx_set_ray_sort(self.h, int(bool(on))))

    def set_graphs(self, on):
        """Launch each PathTracingMIS batch of later renders as one CUDA graph
        with a device-controlled bounce loop (results are identical)."""
        _check(lib().rt_ctx_set_graphs(self.h, int(bool(on))))

    def set_lanes(self, lanes):
        """Concurrent worker lanes of batch_render (1..16, default 4)."""
        _check(lib().rt_ctx_set_lanes(self.h, int(lanes)))

    @staticmethod
    def _jobs(jobs):
        n = len(jobs)
        scenes = (C.c_void_p * n)()
        descs = (D.RenderDesc * n)()
        for i, (sc, spp, opt) in enumerate(jobs):
            opt = dict(opt)
            seed, sb, block = opt.pop("seed", 0), opt.pop("sample_begin", 0), opt.pop("block", 32)
            descs[i] = sc.data.render_desc(spp, seed=seed, sample_begin=sb, block=block, **opt)
            scenes[i] = sc.h
        return scenes, descs

    def batch_render(self, jobs, device_films=None):
        """Render independent jobs in one call (rt_batch_render).  `jobs` is
        a list of (Scene, spp, options) with the options of Scene.render
        (seed, sample_begin, block, max_depth, ...); returns the list of
        (H, W, 4) host films, each equal to that job's Scene.render film.
        With `device_films` (one int device address of an H*W*4 float32
        buffer per job) the films are written there and None is returned."""
        n = len(jobs)
        scenes, descs = self._jobs(jobs)
        fptr = (C.c_void_p * n)()
        if device_films is not None:
            if len(device_films) != n:
                raise ValueError("one device film per job")
            for i, f in enumerate(device_films):
                fptr[i] = int(f)
            _check(lib().rt_batch_render(self.h, scenes, descs, n, fptr, 1))
            return None
        films = []
        for i, (sc, _, _) in enumerate(jobs):
            f = np.zeros((sc.height, sc.width, 4), np.float32)
            films.append(f)
            fptr[i] = f.ctypes.data
        _check(lib().rt_batch_render(self.h, scenes, descs, n, fptr, 0))
        return films

    def get_tuning(self):
        t = Tuning()
        _check(lib().rt_ctx_get_tuning(self.h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **fields):
        """Change some rt_tuning fields (the others keep their values)."""
        t = Tuning()
        _check(lib().rt_ctx_get_tuning(self.h, C.byref(t)))
        for k, v in fields.items():
            if k not in t.as_dict():
                raise KeyError(k)
            setattr(t, k, int(v))
        _check(lib().rt_ctx_set_tuning(self.h, C.byref(t)))

    def autotune(self, jobs, max_trials=32):
        """Run the autotuner (rt_autotune) on a sample of jobs, as for
        batch_render; the best tuning stays set.  Returns (tuning dict,
        path samples per second of the sample under it)."""
        scenes, descs = self._jobs(jobs)
        t = Tuning()
        sps = C.c_double()
        _check(lib().rt_autotune(self.h, scenes, descs, len(jobs), int(max_trials), C.byref(t), C.byref(sps)))
        return t.as_dict(), sps.value

    def stats(self):
        s = D.RenderStats()
        _check(lib().rt_render_stats_get(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in D.RenderStats._fields_}


class Scene:
    """A SceneData flattened and uploaded to the device (rt_scene)."""

    def __init__(self, ctx, scene, bvh=None):
        """bvh: optional (nodes, prims) of a binary tree built elsewhere
        (rt_scene_create_bvh): nodes (n, 4) int32 rows (left, right, first,
        count), prims the triangle index of every leaf slot."""
        self.ctx = ctx
        self.data = scene
        self._desc = scene.desc()
        self.h = C.c_void_p()
        if bvh is None:
            _check(lib().rt_scene_create(ctx.h, C.byref(self._desc), C.byref(self.h)))
        else:
            nodes = np.ascontiguousarray(bvh[0], np.int32).reshape(-1, 4)
            prims = np.ascontiguousarray(bvh[1], np.int32).reshape(-1)
            _check(lib().rt_scene_create_bvh(ctx.h, C.byref(self._desc), _p(nodes), len(nodes), _p(prims), len(prims),
                                             C.byref(self.h)))
        self.width = scene.camera["width"]
        self.height = scene.camera["height"]

    def close(self):
        if self.h:
            lib().rt_scene_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def refit(self, vertices, normals=None):
        """Move the scene's vertices (n, 3) (rt_scene_refit): host arrays, or
        torch CUDA tensors for device memory."""
        if hasattr(vertices, "data_ptr"):
            _check(lib().rt_scene_refit(self.ctx.h, self.h, C.c_void_p(vertices.data_ptr()),
                                        C.c_void_p(normals.data_ptr()) if normals is not None else None, 1))
            return
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1)
        n = np.ascontiguousarray(normals, np.float32).reshape(-1) if normals is not None else None
        _check(lib().rt_scene_refit(self.ctx.h, self.h, _p(v), _p(n) if n is not None else None, 0))

    def info(self):
        b = np.zeros(6, np.float32)
        nbytes = C.c_int64()
        nodes = C.c_int32()
        _check(lib().rt_scene_info(self.h, _p(b), C.byref(nbytes), C.byref(nodes)))
        return dict(bounds=b, device_bytes=nbytes.value, bvh_nodes=nodes.value)

    def render(self, spp, seed=0, sample_begin=0, film=None, block=32, accumulate=False, out=None, **over):
        """Render `spp` samples per pixel; returns the (H, W, 4) film of
        (rgb sum, weight) in host memory (`out` when given), or writes a
        device pointer (`film` as an int address) when given.  With
        `accumulate` the samples are added to the film's contents."""
        flags = D.RENDER_ACCUMULATE if accumulate else 0
        rd = self.data.render_desc(spp, seed=seed, sample_begin=sample_begin, block=block, flags=flags, **over)
        if film is None:
            if out is None:
                out = np.zeros((self.height, self.width, 4), np.float32)
            assert out.dtype == np.float32 and out.flags.c_contiguous and out.shape == (self.height, self.width, 4)
            _check(lib().rt_render(self.ctx.h, self.h, C.byref(rd), _p(out), 0))
            return out
        _check(lib().rt_render(self.ctx.h, self.h, C.byref(rd), C.c_void_p(int(film)), 1))
        return None

    def render_tile_static(self, tile_x, tile_y, film_ptr, spp, seed=0, sample_begin=0, block=32,
                           accumulate=False, **over):
        """Allocation-free render of one job-grid tile into a device film
        (an int device address of a width*height*4 float32 buffer), added to
        the tile's pixels with `accumulate`; see rt_render_tile_static in
        include/rtgpu.h for who needs it and its limits."""
        flags = D.RENDER_ACCUMULATE if accumulate else 0
        rd = self.data.render_desc(spp, seed=seed, sample_begin=sample_begin, block=block, flags=flags, **over)
        _check(lib().rt_render_tile_static(self.ctx.h, self.h, C.byref(rd), int(tile_x), int(tile_y),
                                           C.c_void_p(int(film_ptr))))

    def render_paths(self, pixels, samples, seed=0, **over):
        """Radiance (n, 3) of the path samples (pixel index, sample index)
        through the device kernels (rt_render_paths)."""
        rd = self.data.render_desc(1, seed=seed, **over)
        px = np.ascontiguousarray(pixels, np.int32)
        sm = np.ascontiguousarray(samples, np.int32)
        out = np.zeros((len(px), 3), np.float32)
        _check(lib().rt_render_paths(self.ctx.h, self.h, C.byref(rd), _p(px), _p(sm), len(px), _p(out)))
        return out

    def trace(self, rays, anyhit=False):
        rays = np.ascontiguousarray(rays, D.RAY_DTYPE)
        hits = np.zeros(len(rays), D.HIT_DTYPE)
        _check(lib().rt_trace(self.ctx.h, self.h, _p(rays), len(rays), int(anyhit), _p(hits), 0))
        return hits

    def bsdf_query(self, bsdf, op, q):
        q = np.ascontiguousarray(q, BSDF_Q)
        r = np.zeros(len(q), BSDF_R)
        _check(lib().rt_bsdf_query(self.ctx.h, self.h, bsdf, op, _p(q), len(q), _p(r)))
        return r

    def light_query(self, light, p, u):
        q = np.zeros(len(p), LIGHT_Q)
        q["p"], q["u"] = p, u
        r = np.zeros(len(p), LIGHT_R)
        _check(lib().rt_light_query(self.ctx.h, self.h, light, _p(q), len(q), _p(r)))
        return r

    def medium_query(self, medium, op, q):
        """Medium::sampleDistance (op 0) or transmittance (op 1) for MEDIUM_Q records."""
        q = np.ascontiguousarray(q, MEDIUM_Q)
        r = np.zeros(len(q), MEDIUM_R)
        _check(lib().rt_medium_query(self.ctx.h, self.h, medium, op, _p(q), len(q), _p(r)))
        return r


class Server:
    """A render job queue on one device (rt_server_start ... rt_server_stop)."""

    def __init__(self, ctx, lanes=4, max_queue=0, device_budget_bytes=0, lanes_only=False, rmse_display=False):
        """lanes_only=False: continuous batching of PathTracingMIS jobs in
        one wavefront (other jobs on the lanes); True: every job on a lane.
        rmse_display=True: target RMSEs are over the pixel means clipped to
        [0, 1] (the displayed image) instead of the linear radiance."""
        self.ctx = ctx
        self.h = C.c_void_p()
        self._scenes = {}
        o = ServerOpts(int(lanes), int(max_queue), int(device_budget_bytes), int(bool(lanes_only)),
                       int(bool(rmse_display)))
        _check(lib().rt_server_start(ctx.h, C.byref(o), C.byref(self.h)))

    def submit(self, scene, spp, target_rmse=0.0, seed=0, sample_begin=0, block=32, **over):
        """Queue a render of `scene`; with target_rmse > 0 it renders
        progressively, at most `spp` samples.  Returns the job id."""
        rd = scene.data.render_desc(spp, seed=seed, sample_begin=sample_begin, block=block, **over)
        jid = C.c_int64()
        _check(lib().rt_job_submit(self.h, scene.h, C.byref(rd), float(target_rmse), C.byref(jid)))
        self._scenes[jid.value] = scene
        return jid.value

    @staticmethod
    def _info(ji):
        return dict(state=ji.state, spp_done=ji.spp_done, rmse_estimate=ji.rmse_estimate,
                    queue_ms=ji.queue_ms, run_ms=ji.run_ms, error=ji.error.decode())

    def poll(self, jid, fetch=False):
        """(info, film): film is the (H, W, 4) result when `fetch` is set and
        the job has finished (the job is then released), else None."""
        ji = JobInfo()
        sc = self._scenes.get(jid)
        fetch = fetch and sc is not None
        film = np.zeros((sc.height, sc.width, 4), np.float32) if fetch else None
        _check(lib().rt_job_poll(self.h, jid, C.byref(ji), _p(film) if fetch else None))
        info = self._info(ji)
        if fetch and info["state"] in (JOB_DONE, JOB_FAILED):
            self._scenes.pop(jid, None)
            return info, (film if info["state"] == JOB_DONE else None)
        return info, None

    def wait(self, jid, timeout_ms=-1):
        """Wait for a job, then (info, film) as poll(fetch=True)."""
        ji = JobInfo()
        sc = self._scenes.get(jid)
        if sc is None:
            raise RtError(1, "unknown job %d" % jid)
        film = np.zeros((sc.height, sc.width, 4), np.float32)
        _check(lib().rt_job_wait(self.h, jid, int(timeout_ms), C.byref(ji), _p(film)))
        info = self._info(ji)
        if info["state"] in (JOB_DONE, JOB_FAILED):
            self._scenes.pop(jid, None)
            return info, (film if info["state"] == JOB_DONE else None)
        return info, None

    def stop(self):
        if self.h:
            lib().rt_server_stop(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


BSDF_Q = np.dtype([("wi", np.float32, 3), ("wo", np.float32, 3), ("u", np.float32, 2)])
BSDF_R = np.dtype([("value", np.float32, 3), ("pdf", np.float32), ("wo", np.float32, 3),
                   ("relative_eta", np.float32), ("sampled_type", np.int32), ("pad", np.int32)])
LIGHT_Q = np.dtype([("p", np.float32, 3), ("u", np.float32, 2)])
LIGHT_R = np.dtype([("intensity", np.float32, 3), ("pdf", np.float32), ("to_light", np.float32, 3),
                    ("distance", np.float32), ("point", np.float32, 3), ("normal", np.float32, 3),
                    ("pdf_eval", np.float32), ("pad", np.float32)])
MEDIUM_Q = np.dtype([("o", np.float32, 3), ("mint", np.float32), ("d", np.float32, 3), ("maxt", np.float32),
                     ("seed", np.uint64), ("pixel", np.uint32), ("sample", np.uint32)])
MEDIUM_R = np.dtype([("weight", np.float32, 3), ("t", np.float32), ("scattered", np.int32), ("limit", np.int32)])
MEDIUM_OP_SAMPLE, MEDIUM_OP_TRANSMITTANCE = 0, 1
assert BSDF_Q.itemsize == C.sizeof(D.BsdfQ) and BSDF_R.itemsize == C.sizeof(D.BsdfR)
assert LIGHT_Q.itemsize == C.sizeof(D.LightQ) and LIGHT_R.itemsize == C.sizeof(D.LightR)


def path_state_bytes(integrator=0):
    """Device bytes of wavefront path state per path slot for an integrator
    (0: PathTracingMIS, 1: VolPathTracing), as a server counts them against
    its budget."""
    return int(lib().rt_path_state_bytes(int(integrator)))


def bvh_stats(tri_v, width=2, depth_cap=0):
    """Build the device tree over triangles (n, 3, 3) on the host as
    rt_scene_create would (rt_bvh_stats, no GPU needed) and return
    (deepest leaf level, node count); the binary tree is checked
    structurally.  depth_cap <= 0 is the default cap of 62 levels."""
    tv = np.ascontiguousarray(tri_v, np.float32).reshape(-1)
    d, n = C.c_int32(), C.c_int32()
    _check(lib().rt_bvh_stats(_p(tv), len(tv) // 9, width, depth_cap, C.byref(d), C.byref(n)))
    return d.value, n.value


def bvh_import_check(tri_v, nodes, prims):
    """The device image rt_scene_create_bvh would upload for a tree built
    elsewhere (rt_bvh_import_check, no GPU needed): (depth, internal nodes);
    raises RtError if the tree is malformed."""
    tv = np.ascontiguousarray(tri_v, np.float32).reshape(-1)
    nodes = np.ascontiguousarray(nodes, np.int32).reshape(-1, 4)
    prims = np.ascontiguousarray(prims, np.int32).reshape(-1)
    d, n = C.c_int32(), C.c_int32()
    _check(lib().rt_bvh_import_check(_p(tv), len(tv) // 9, _p(nodes), len(nodes), _p(prims), len(prims),
                                     C.byref(d), C.byref(n)))
    return d.value, n.value


def load_obj(path, to_world=None):
    """Read a Wavefront OBJ as the reference's ObjLoader does (rt_obj_load):
    returns (vertices (n, 3), normals (n, 3) or None, uvs (n, 2) or None,
    triangles (m, 3)), positions and normals already in world space."""
    m = MeshData()
    tw = None if to_world is None else np.ascontiguousarray(to_world, np.float32).reshape(16)
    _check(lib().rt_obj_load(os.fsencode(path), None if tw is None else _p(tw), C.byref(m)))
    try:
        def arr(ptr, n, k, dt):
            if not ptr or n == 0:
                return None
            return np.ctypeslib.as_array(ptr, shape=(n * k,)).astype(dt).reshape(n, k)
        v = arr(m.vertices, m.n_vertices, 3, np.float32)
        v = v if v is not None else np.zeros((0, 3), np.float32)
        t = arr(m.indices, m.n_triangles, 3, np.int32)
        t = t if t is not None else np.zeros((0, 3), np.int32)
        return v, arr(m.normals, m.n_vertices, 3, np.float32), arr(m.uvs, m.n_vertices, 2, np.float32), t
    finally:
        lib().rt_mesh_data_free(C.byref(m))


def load_hdr(path):
    """Read a Radiance RGBE (.hdr) image as the reference reads environment
    maps (rt_hdr_load): (height, width, 3) float32, top row first."""
    w, h = C.c_int32(), C.c_int32()
    ptr = C.POINTER(C.c_float)()
    _check(lib().rt_hdr_load(os.fsencode(path), C.byref(w), C.byref(h), C.byref(ptr)))
    try:
        return np.ctypeslib.as_array(ptr, shape=(h.value * w.value * 3,)).astype(np.float32).reshape(h.value, w.value, 3)
    finally:
        lib().rt_host_free(C.cast(ptr, C.c_void_p))


def post_process(film):
    """Screen::postProcessColor (core/Screen.cpp:8-18,113-122): colour /
    weight wherever the weight is not zero (a Mitchell-Netravali sum can be
    negative), the colour as it is elsewhere."""
    film = np.asarray(film, np.float32)
    w = film[..., 3:4]
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(w != 0, film[..., :3] / np.where(w != 0, w, 1), film[..., :3]).astype(np.float32)
