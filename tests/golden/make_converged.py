"""Generate the 4096-spp CPU reference crops for the converged-image tests.

For the displaced-icosphere scene (1,310,722 triangles, sky map, 1024x1024,
max depth 16) and the grid-medium scene (128^3 fBm grid, slab, sphere light,
512x512, max depth 64) the CPU oracle renders fixed 32x32 tiles at 4096
samples per pixel twice, with two independent sample streams (seeds A and
B).  The second render calibrates the test's tolerance: the per-pixel
difference between two converged CPU renders is the Monte-Carlo noise a
converged GPU render must stay within.

Writes tests/golden/converged_4096spp.npz.  Run from the repository root
(about ten minutes on 8 cores):  python tests/golden/make_converged.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

SPP = 4096
SEED_A, SEED_B = 4242, 4343
# (scene, tile x, tile y) of the 32x32 job grid
CROPS = [("icosphere", 15, 15),   # the displaced sphere's centre (mixed materials)
         ("icosphere", 8, 12),    # its silhouette against the ground
         ("volume", 7, 6),        # inside the fBm grid medium
         ("volume", 7, 12)]       # the homogeneous slab


def scene(name):
    from raytracer_gb300 import scenes
    if name == "icosphere":
        return scenes.displaced_icosphere()
    return scenes.volume_grid()


def crop(film, tx, ty):
    return film[ty * 32:(ty + 1) * 32, tx * 32:(tx + 1) * 32].copy()


def render_crop(o, s, tx, ty, seed, threads):
    """One 32x32 tile rendered as 16 tiles of 8x8 (four rows of four, one
    worker thread per row).  With the box filter of radius 0.5 every sample
    lands in its own pixel and the per-path streams depend on the pixel and
    sample index only, so the pixels equal those of the 32x32 tile."""
    from concurrent.futures import ThreadPoolExecutor
    tiles_x8 = (s.camera["width"] + 7) // 8
    rows = [(4 * ty + r) * tiles_x8 + 4 * tx for r in range(4)]
    per = max(1, threads // 4)
    o.render_paths([0], [0], seed=seed)   # builds the light CDF before the threads share the scene
    with ThreadPoolExecutor(4) as ex:
        films = list(ex.map(lambda t: o.render_tiles(SPP, t, t + 4, seed=seed, threads=per, block=8), rows))
    return sum(films)


def main():
    import oracle_lib as O
    out = {"spp": np.int32(SPP), "seeds": np.array([SEED_A, SEED_B], np.int64)}
    cache = {}
    for name, tx, ty in CROPS:
        if name not in cache:
            s = scene(name)
            cache[name] = (s, O.OracleScene(s))
        s, o = cache[name]
        key = "%s_%d_%d" % (name, tx, ty)
        for tag, seed in (("a", SEED_A), ("b", SEED_B)):
            t0 = time.time()
            film = render_crop(o, s, tx, ty, seed, os.cpu_count() or 4)
            out[key + "_" + tag] = crop(film, tx, ty)
            print("%s %s: %.1f s" % (key, tag, time.time() - t0), flush=True)
    np.savez_compressed(os.path.join(HERE, "converged_4096spp.npz"), **out)


if __name__ == "__main__":
    main()
