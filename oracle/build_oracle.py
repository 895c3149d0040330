"""Build recipe for the CPU oracle and the reference pin libraries (test
infrastructure only).

* liboracle.so  -- the C restatement in oracle/*.c, compiled with gcc into
  oracle/_build/.  Built on every machine (plain C99 + pthreads).
* libref_pin.so -- the reference's own tools/Rng.h and core/CDF.{h,cpp},
  compiled in place with oracle/ref_shim.h force-included, into oracle/_ref/.
* libref_hot.so -- the reference's own hot-path sources (triangle test,
  BSDFs, Fresnel, warps, microfacet distributions, lights, media, phase
  function, and for whole renders the integrators, the scene with its BVH
  and the camera; REF_HOT_SOURCES below) compiled in place against the
  project-written Eigen-subset shim and registry stand-ins in
  oracle/ref_include/, with the C entry points of oracle/ref_hot.cpp, into
  oracle/_ref/.

The two reference libraries are built only where the reference source tree
is given: the RT_REFERENCE_SRC environment variable, or the `ref_src`
argument, names its RaytracerNew2/src directory.  There is no default.

GCC and the reference.  The reference is an MSVC project.  Its sources
compile unmodified with g++ -fpermissive except for three constructs in two
headers that GCC rejects outright.  normalise_headers() writes copies of
those two headers into oracle/_ref/include/ (git-ignored, rebuilt from the
reference each time) with exactly these rewrites, each asserted to match:
  core/Color.h         the member template `tplFromSRGB` names its template
                       parameter T, shadowing the class template's T; it is
                       renamed TC_ (two sites).  Dependent-base calls to
                       coeff()/coeffRef() in TplColor get `this->`.
  tools/WithSmartPtr.h `static typename ptr` / `typename constPtr` without a
                       nested-name-specifier lose the `typename`; parameter
                       packs passed as `(args)` are expanded `(args...)`.
None of them changes arithmetic.  Standard headers that MSVC's headers
pull in transitively (cassert, cstring, vector, functional,
condition_variable, thread, mutex, unistd.h) are
force-included, and Scene.cpp's `#include <Eigen\\StdVector>` (a Windows
path separator) reaches a generated one-line header of that literal name.  GCC's -I- makes every include (also a
sibling include such as "Color.h") resolve to those copies and to the
stand-ins first; all other reference files are read where they lie.
"""
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_include")

CFLAGS = ["-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
          "-fno-strict-aliasing", "-pthread", "-Wall", "-Wno-unused-function"]

# reference translation units compiled into libref_hot.so (paths relative to
# RaytracerNew2/src): the pinned functions and what they call
REF_HOT_SOURCES = [
    "geometricShape/Triangle.cpp", "geometricShape/Sphere.cpp", "geometricShape/Mesh.cpp",
    "geometricShape/GeometricShape.cpp", "geometricShape/ISampledShape.cpp",
    "bsdf/BSDF.cpp", "bsdf/Diffuse.cpp", "bsdf/MicrofacetDistribution.cpp", "bsdf/RoughConductor.cpp",
    "bsdf/RoughDielectric.cpp", "bsdf/SmoothLayeredBSDF.cpp",
    "light/Light.cpp", "light/AreaLight.cpp", "light/MeshLight.cpp", "light/EnvironmentLight.cpp",
    "medium/Medium.cpp", "medium/Homogeneous.cpp", "medium/Heterogeneous.cpp", "medium/HGPhaseFunction.cpp",
    "medium/PhaseFunction.cpp", "medium/IsotropicPhaseFunction.cpp",
    "volume/Volume.cpp", "volume/GridVolume.cpp",
    "texture/Texture.cpp", "texture/ConstantTexture.cpp",
    "core/BoundingBox.cpp", "core/CDF.cpp", "core/Color.cpp", "core/DifferentialGeometry.cpp",
    "core/Fresnel.cpp", "core/Intersection.cpp", "core/Mapping.cpp", "core/Parameters.cpp", "core/Ray.cpp",
    "core/RaytracerObject.cpp", "core/Transform.cpp",
    "sampler/Sampler.cpp",
    "tools/Common.cpp", "tools/Logger.cpp", "tools/Filesystem.cpp", "tools/Timer.cpp",
    # whole-path renders: the integrators, the scene and its BVH, the camera
    "integrator/Integrator.cpp", "integrator/PathTracingMIS.cpp", "integrator/VolPathTracing.cpp",
    "integrator/DirectLightingMIS.cpp",
    "accelStruct/Bvh.cpp", "core/Scene.cpp", "core/Primitive.cpp",
    "camera/Camera.cpp", "camera/NoriPerspective.cpp",
    "core/Screen.cpp", "core/Job.cpp", "core/SampleJob.cpp", "core/JobManager.cpp",
    "filter/ReconstructionFilter.cpp", "filter/BoxFilter.cpp", "filter/GaussianFilter.cpp",
    "filter/MitchellNetravaliFilter.cpp",
    "thread/TaskSet.cpp", "thread/ThreadPool.cpp", "thread/Barrier.cpp",
]
REF_CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fpermissive", "-w",
                "-include", "cassert", "-include", "cstring", "-include", "vector", "-include", "functional", "-include", "condition_variable",
                "-include", "thread", "-include", "mutex", "-include", "unistd.h"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("oracle build failed: " + os.path.basename(cmd[-1]))
    return r.stdout + r.stderr


def reference_src(ref_src=None):
    """The reference's RaytracerNew2/src directory, from the argument or
    RT_REFERENCE_SRC; None when neither names an existing directory."""
    p = ref_src or os.environ.get("RT_REFERENCE_SRC")
    return p if p and os.path.isdir(p) else None


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


def build_ref_pin(force=False, ref_src=None):
    """Compile the reference's PCG32 and CDF sources in place (if given)."""
    src = reference_src(ref_src)
    if src is None:
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    out = os.path.join(REF_OUT, "libref_pin.so")
    if not force and os.path.exists(out):
        return out
    tmp = out + ".tmp"
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
          "-include", os.path.join(HERE, "ref_shim.h"), "-I", src,
          os.path.join(HERE, "ref_pin.cpp"), os.path.join(src, "core", "CDF.cpp"),
          "-o", tmp])
    os.replace(tmp, out)
    return out


def _rewrite(text, old, new, count, what):
    n = text.count(old)
    if n != count:
        raise RuntimeError("reference header changed: %s (%d matches of %r, expected %d)" % (what, n, old, count))
    return text.replace(old, new)


def normalise_headers(src, dest):
    """Copies of core/Color.h and tools/WithSmartPtr.h with the GCC-only
    rewrites listed in the module docstring, written under `dest`."""
    color = open(os.path.join(src, "core", "Color.h"), encoding="latin-1").read()
    color = _rewrite(color, "\ttemplate<class T>\n\tstatic T tplFromSRGB(", "\ttemplate<class TC_>\n\tstatic TC_ tplFromSRGB(",
                     1, "Color.h tplFromSRGB")
    color = _rewrite(color, "return T::fromRGB(fromSRGBVal(sr)", "return TC_::fromRGB(fromSRGBVal(sr)", 1,
                     "Color.h tplFromSRGB body")
    # TplColor (lines 94-343) calls coeff/coeffRef of its dependent base unqualified
    start = color.index("class TplColor : public Eigen::Array")
    end = color.index("template<class T, int N>", start)
    body = color[start:end]
    body, k = re.subn(r"(?<![\w.>])(coeffRef|coeff)\(", r"this->\1(", body)
    if k < 4:
        raise RuntimeError("reference header changed: Color.h TplColor coeff calls (%d)" % k)
    color = color[:start] + body + color[end:]
    smart = open(os.path.join(src, "tools", "WithSmartPtr.h"), encoding="latin-1").read()
    smart = smart.replace("static typename ptr ", "static ptr ").replace("static typename constPtr ", "static constPtr ")
    smart = _rewrite(smart, "std::make_shared<Derived>(args);", "std::make_shared<Derived>(args...);", 1,
                     "WithSmartPtr.h make_shared")
    smart = smart.replace("return new Derived(args);", "return new Derived(args...);")
    smart = smart.replace("return new const Derived(args);", "return new const Derived(args...);")
    # core/Scene.cpp:11 includes <Eigen\StdVector>: a file of that literal name
    files = [("core/Color.h", color), ("tools/WithSmartPtr.h", smart), ("Eigen\\StdVector", "#include <Eigen/StdVector>\n")]
    for rel, text in files:
        p = os.path.join(dest, rel)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w", encoding="latin-1") as f:
            f.write(text)


def _std_quote_dirs():
    """libstdc++ directories that its own headers reach with quoted includes
    (-I- turns off the includer's-directory lookup for them too)."""
    r = subprocess.run(["g++", "-xc++", "-E", "-v", "-"], input="", capture_output=True, text=True)
    dirs, on = [], False
    for line in r.stderr.splitlines():
        if line.startswith("#include <...> search starts here"):
            on = True
            continue
        if line.startswith("End of search list"):
            break
        if on:
            d = line.strip()
            if os.path.isdir(os.path.join(d, "pstl")):
                dirs.append(os.path.join(d, "pstl"))
    return dirs


def ref_hot_includes(src):
    norm = os.path.join(REF_OUT, "include")
    quote = [SHIM, os.path.join(SHIM, "factory"), norm, os.path.join(norm, "core"), os.path.join(norm, "tools")]
    subdirs = sorted(d for d in os.listdir(src) if os.path.isdir(os.path.join(src, d)))
    angle = [SHIM, norm, src] + [os.path.join(src, d) for d in subdirs] + _std_quote_dirs()
    flags = []
    for d in quote:
        flags += ["-I", d]
    flags.append("-I-")
    for d in angle:
        flags += ["-I", d]
    return flags


def build_ref_hot(force=False, ref_src=None):
    """Compile the reference's hot-path sources in place (if given) with the
    Eigen-subset shim, plus oracle/ref_hot.cpp, into oracle/_ref/libref_hot.so."""
    src = reference_src(ref_src)
    if src is None:
        return None
    out = os.path.join(REF_OUT, "libref_hot.so")
    if not force and os.path.exists(out):
        return out
    obj_dir = os.path.join(REF_OUT, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    normalise_headers(src, os.path.join(REF_OUT, "include"))
    inc = ref_hot_includes(src)
    jobs, objs = [], []
    for rel in REF_HOT_SOURCES:
        o = os.path.join(obj_dir, rel.replace("/", "_") + ".o")
        objs.append(o)
        jobs.append(["g++"] + REF_CXXFLAGS + inc + ["-c", os.path.join(src, rel), "-o", o])
    o = os.path.join(obj_dir, "ref_hot.o")
    objs.append(o)
    jobs.append(["g++"] + REF_CXXFLAGS + inc + ["-I", os.path.join(ROOT, "include"), "-c",
                                                 os.path.join(HERE, "ref_hot.cpp"), "-o", o])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    tmp = out + ".tmp"
    _run(["g++", "-shared", "-o", tmp] + objs + ["-lm", "-lpthread"])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else None
    print(build_oracle(force=True))
    print(build_ref_pin(force=True, ref_src=ref))
    print(build_ref_hot(force=True, ref_src=ref))
