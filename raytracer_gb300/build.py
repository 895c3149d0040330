"""In-tree build of librtgpu.so for sm_103a (GB300).

nvcc compiles the CUDA translation unit, g++ the host BVH builder, in
parallel; the shared library lands next to this file.  The device code is
compiled with -fmad=false so that every a*b+c in the shading code stays two
rounded operations, as in the reference's CPU build; the traversal kernels
use explicit fused multiply-adds where rounding cannot change a result.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librtgpu.so")

ARCH = os.environ.get("RTGPU_ARCH", "-gencode=arch=compute_103a,code=sm_103a")
NVCC = os.environ.get("NVCC", "nvcc")

CUDA_SOURCES = ["rt_api.cu"]
HOST_SOURCES = ["rt_bvh.cpp", "rt_serve.cpp", "rt_io.cpp", "rt_tune.cpp"]
HEADERS = ["rt_math.cuh", "rt_device.cuh", "rt_kernels.cuh", "rt_volpath.cuh", "rt_lbvh.cuh", "rt_bvh.h",
           "rt_internal.h"]


def _cuda_include():
    nvcc = NVCC if os.path.isabs(NVCC) else (shutil.which(NVCC) or "/usr/local/cuda/bin/nvcc")
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("build step failed: " + os.path.basename(cmd[-1]))
    return r.stdout + r.stderr


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "rtgpu.h")]
    jobs = []
    objs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            cmd = [NVCC, ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off",
                   "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            extra = os.environ.get("RTGPU_NVCC_FLAGS", "").split()
            cmd[1:1] = extra
            jobs.append(cmd)
    for s in HOST_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off",
                         "-I", os.path.join(ROOT, "include"),
                         "-I", _cuda_include(), "-c", src, "-o", obj])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([NVCC, ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
