"""Build recipe for the CPU oracle (test infrastructure only).

* liboracle.so  -- the C restatement in oracle/*.c, compiled with gcc into
  oracle/_build/.  Built on every machine (it is plain C99 + pthreads).
* libref_pin.so -- the reference's own tools/Rng.h and core/CDF.{h,cpp},
  compiled in place from the reference source tree with oracle/ref_shim.h
  force-included, into oracle/_ref/.  Built only where the reference tree is
  present; it pins the oracle's PCG32 and CDF restatements.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REF_SRC = os.environ.get("RT_REFERENCE_SRC", "/root/reference/RaytracerNew2/src")

CFLAGS = ["-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
          "-fno-strict-aliasing", "-pthread", "-Wall", "-Wno-unused-function"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("oracle build failed")


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("oracle_core.c", "oracle_bvh.c", "oracle_render.c")]
    deps = srcs + [os.path.join(HERE, "oracle.h"), os.path.join(ROOT, "include", "rtgpu.h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    tmp = out + ".tmp"
    _run(["gcc"] + CFLAGS + ["-shared", "-I", os.path.join(ROOT, "include")] + srcs + ["-o", tmp, "-lm"])
    os.replace(tmp, out)
    return out


def build_ref_pin(force=False):
    """Compile the reference's PCG32 and CDF sources in place (if present)."""
    if not os.path.isdir(REF_SRC):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    out = os.path.join(REF_OUT, "libref_pin.so")
    if not force and os.path.exists(out):
        return out
    tmp = out + ".tmp"
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
          "-include", os.path.join(HERE, "ref_shim.h"), "-I", REF_SRC,
          os.path.join(HERE, "ref_pin.cpp"), os.path.join(REF_SRC, "core", "CDF.cpp"),
          "-o", tmp])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref_pin(force=True))
