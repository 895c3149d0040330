"""The C-ABI library loads, exports every entry point include/rtgpu.h
declares, and its struct layouts match the ctypes mirror (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from raytracer_gb300 import desc as D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rtgpu.h")


def _declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:rt_status|int32_t|int64_t|uint64_t|const char \*)\s*(rt_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def built():
    from raytracer_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(built):
    names = _declared_functions()
    assert len(names) >= 14
    lib = C.CDLL(built)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_path_state_bytes(built):
    """The per-slot path state a server counts against its budget: the
    wavefront arrays of a PathTracingMIS render, plus the VolPath
    wavefront's six float4 arrays; 0 for an unknown integrator."""
    import raytracer_gb300 as R
    pt, vp = R.path_state_bytes(0), R.path_state_bytes(1)
    assert pt == 16 + 10 * 16 + 3 * 4 + 2 + 11 * 4 + 3 * 4
    assert vp == pt + 6 * 16
    assert R.path_state_bytes(7) == 0


def test_struct_layout_matches_header(tmp_path):
    structs = {"rt_bsdf_desc": D.BsdfDesc, "rt_mesh_desc": D.MeshDesc, "rt_sphere_desc": D.SphereDesc,
               "rt_light_desc": D.LightDesc, "rt_medium_desc": D.MediumDesc, "rt_camera_desc": D.CameraDesc,
               "rt_scene_desc": D.SceneDesc, "rt_render_desc": D.RenderDesc, "rt_ray": D.Ray, "rt_hit": D.Hit,
               "rt_bsdf_q": D.BsdfQ, "rt_bsdf_r": D.BsdfR, "rt_light_q": D.LightQ, "rt_light_r": D.LightR,
               "rt_render_stats": D.RenderStats, "rt_texture_desc": D.TextureDesc}
    prog = ['#include <stdio.h>', '#include <stddef.h>', '#include "rtgpu.h"', "int main(void){"]
    for k in structs:
        prog.append('printf("%s %%zu\\n", sizeof(%s));' % (k, k))
    from raytracer_gb300 import core
    extra = {"rt_medium_q": core.MEDIUM_Q.itemsize, "rt_medium_r": core.MEDIUM_R.itemsize,
             "rt_server_opts": C.sizeof(core.ServerOpts), "rt_job_info": C.sizeof(core.JobInfo),
             "rt_tuning": C.sizeof(core.Tuning)}
    for k in extra:
        prog.append('printf("%s %%zu\\n", sizeof(%s));' % (k, k))
    prog.append('printf("camera_off %zu\\n", offsetof(rt_scene_desc, camera));')
    prog.append("return 0;}")
    c = tmp_path / "sz.c"
    c.write_text("\n".join(prog))
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.dirname(HEADER), str(c), "-o", str(exe)])
    out = dict(l.split() for l in subprocess.check_output([str(exe)]).decode().split("\n") if l)
    for k, cls in structs.items():
        assert int(out[k]) == C.sizeof(cls), (k, out[k], C.sizeof(cls))
    for k, size in extra.items():
        assert int(out[k]) == size, (k, out[k], size)
    assert int(out["camera_off"]) == D.SceneDesc.camera.offset


def test_mix64_matches_oracle(built):
    import numpy as np
    lib = C.CDLL(built)
    lib.rt_mix64.restype = C.c_uint64
    lib.rt_mix64.argtypes = [C.c_uint64]
    def mix64(x):
        x ^= x >> 30; x = (x * 0xbf58476d1ce4e5b9) & (2 ** 64 - 1)
        x ^= x >> 27; x = (x * 0x94d049bb133111eb) & (2 ** 64 - 1)
        return x ^ (x >> 31)
    for v in [0, 1, 2 ** 32, 123456789, 2 ** 64 - 1]:
        assert lib.rt_mix64(v) == mix64(v)


def test_no_gpu_fails_loudly(built):
    """Without a usable GPU the product raises; it never falls back to a CPU path."""
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    import raytracer_gb300 as R
    with pytest.raises(R.RtError):
        R.Context(0)
