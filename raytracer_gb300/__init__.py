"""GB300-native light-transport core for Iscandel/Raytracer's PathTracingMIS
and VolPathTracing integrators.

The compute path is librtgpu.so (hand-written CUDA for sm_103a behind the C
ABI declared in include/rtgpu.h); this package holds the Python host binding
(`core`), the ctypes mirror of the scene description (`desc`), the seeded
synthetic scenes (`scenes`) and the in-tree build (`build`).
"""
from . import desc  # noqa: F401
from .core import Context, Scene, Server, RtError, post_process, lib, LIB_PATH  # noqa: F401
from .core import JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED, load_obj, load_hdr  # noqa: F401
from .core import path_state_bytes  # noqa: F401

__all__ = ["Context", "Scene", "Server", "RtError", "post_process", "lib", "desc", "LIB_PATH",
           "JOB_QUEUED", "JOB_RUNNING", "JOB_DONE", "JOB_FAILED", "load_obj", "load_hdr", "path_state_bytes"]
