"""Generate the golden fixtures that pin the CPU oracle to the reference.

oracle/build_oracle.py compiles the reference's own sources in place:
tools/Rng.h (PCG32) and core/CDF.{h,cpp} into libref_pin.so, and the
hot-path sources (triangle test, warps, Fresnel, microfacet distributions,
Diffuse / RoughConductor / RoughDielectric / SmoothLayeredBSDF, mesh, sphere
and environment lights, HG phase function, homogeneous and grid media) into
libref_hot.so, together with the integrators, the scene and its BVH and
the camera.  This script runs them on seeded inputs and writes the
fixtures next to itself:

* pcg32_ref.json  -- raw 32-bit outputs and mantissa floats of Rng streams
* cdf_ref.json    -- CDF::sampleAndReuse / CDF::sample on seeded pdf lists
* ref_hot.npz     -- the queries of tests/pin_cases.py with the reference's
                     answers
* ref_paths.npz   -- the radiance of every path sample of small renders of
                     the three configurations' scene families, computed by
                     the reference's own PathTracingMIS::li /
                     VolPathTracing::li over its own BVH

Run from the repository root, naming the reference's RaytracerNew2/src:
    python tests/golden/make_golden.py <reference>/RaytracerNew2/src
(or set RT_REFERENCE_SRC).
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_oracle  # noqa: E402

PIN_QUERIES = 1024   # queries per family in ref_hot.npz


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else None
    if build_oracle.reference_src(ref) is None:
        raise SystemExit("name the reference's RaytracerNew2/src directory (argument or RT_REFERENCE_SRC)")
    path = build_oracle.build_ref_pin(force=True, ref_src=ref)
    L = C.CDLL(path)
    L.ref_pcg_stream.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]
    L.ref_pcg_reals.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]
    L.ref_cdf_sample_reuse.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
    L.ref_cdf_sample.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    streams = []
    seeds = [(42, 54), (0, 0), (1, 1), (0xdeadbeefcafebabe, 7), (2 ** 64 - 1, 2 ** 63 + 5), (12345, 0)]
    # path-stream seeds: splitmix64((seed << 32) ^ pixel), sample index
    def mix64(x):
        x &= 2 ** 64 - 1
        x ^= x >> 30; x = (x * 0xbf58476d1ce4e5b9) & (2 ** 64 - 1)
        x ^= x >> 27; x = (x * 0x94d049bb133111eb) & (2 ** 64 - 1)
        x ^= x >> 31
        return x
    for pix, s in [(0, 0), (1, 0), (65535, 15), (1048575, 63)]:
        seeds.append((mix64((0 << 32) ^ pix), s))
    for st, sq in seeds:
        u = np.zeros(64, np.uint32)
        f = np.zeros(64, np.float32)
        L.ref_pcg_stream(st, sq, 64, u.ctypes.data)
        L.ref_pcg_reals(st, sq, 64, f.ctypes.data)
        streams.append(dict(initstate=str(st), initseq=str(sq), u32=[int(x) for x in u],
                            real_bits=[int(x) for x in f.view(np.uint32)]))
    json.dump(dict(source="RaytracerNew2/src/tools/Rng.h compiled in place", streams=streams),
              open(os.path.join(HERE, "pcg32_ref.json"), "w"), indent=0)
    rng = np.random.default_rng(7)
    cases = []
    for n in [1, 2, 3, 7, 32, 100, 1000]:
        pdfs = rng.random(n).astype(np.float32)
        if n > 4:
            pdfs[rng.integers(0, n, 2)] = 0.0  # zero-weight entries (empty rows / black texels)
        u = np.concatenate([rng.random(200), [0.0, 1e-9, 0.5, 0.999999, np.nextafter(np.float32(1), 0)]]).astype(np.float32)
        idx = np.zeros(len(u), np.int32)
        uo = np.zeros(len(u), np.float32)
        po = np.zeros(len(u), np.float32)
        sm = np.zeros(1, np.float32)
        L.ref_cdf_sample_reuse(pdfs.ctypes.data, n, u.ctypes.data, len(u), idx.ctypes.data, uo.ctypes.data,
                               po.ctypes.data, sm.ctypes.data)
        idx2 = np.zeros(len(u), np.int32)
        po2 = np.zeros(len(u), np.float32)
        L.ref_cdf_sample(pdfs.ctypes.data, n, u.ctypes.data, len(u), idx2.ctypes.data, po2.ctypes.data)
        cases.append(dict(pdf_bits=[int(x) for x in pdfs.view(np.uint32)], u_bits=[int(x) for x in u.view(np.uint32)],
                          index=[int(x) for x in idx], u_out_bits=[int(x) for x in uo.view(np.uint32)],
                          pdf_out_bits=[int(x) for x in po.view(np.uint32)], sum_bits=int(sm.view(np.uint32)[0]),
                          sample_index=[int(x) for x in idx2], sample_pdf_bits=[int(x) for x in po2.view(np.uint32)]))
    json.dump(dict(source="RaytracerNew2/src/core/CDF.h + CDF.cpp compiled in place", cases=cases),
              open(os.path.join(HERE, "cdf_ref.json"), "w"))
    print("wrote", os.path.join(HERE, "pcg32_ref.json"), os.path.join(HERE, "cdf_ref.json"))
    hot = build_oracle.build_ref_hot(force=True, ref_src=ref)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, ROOT)
    import pin_cases
    inp = pin_cases.inputs(n=PIN_QUERIES)
    out = pin_cases.run(C.CDLL(hot), inp)
    np.savez_compressed(os.path.join(HERE, "ref_hot.npz"),
                        **{"in_" + k: v for k, v in inp.items()}, **{"out_" + k: v for k, v in out.items()})
    print("wrote", os.path.join(HERE, "ref_hot.npz"))
    films = {}
    for name, scene, spp in pin_cases.film_scenes():
        pix, smp = pin_cases.all_paths(scene, spp)
        films[name + "_rad"] = pin_cases.reference_paths(C.CDLL(hot), scene, pix, smp, seed=0)
        films[name + "_digest"] = np.array(pin_cases.scene_digest(scene))
    np.savez_compressed(os.path.join(HERE, "ref_paths.npz"), **films)
    print("wrote", os.path.join(HERE, "ref_paths.npz"))


if __name__ == "__main__":
    main()
