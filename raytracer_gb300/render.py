"""Render a reference scene file on the GPU and save the film as OpenEXR.

    python -m raytracer_gb300.render scene.xml [-o image.exr] [--spp N] [--seed S]
                                    [--material NAME=eta_r,eta_g,eta_b:k_r,k_g,k_b ...]

The headless counterpart of the reference's main (core/main.cpp:497-563):
load the scene file, render it with its integrator, sampler count and tile
size, post-process the film and write `<fileName minus extension>.exr` (or
`-o`); without a fileName parameter, `<scene name>.exr` in the current
folder.  The window, tone mapping and PNG output of the reference are not
part of this path.
"""
import argparse
import os
import sys
import time

from .core import Context, Scene, post_process
from .exr import write_exr
from .xml_scene import load_scene


def output_path(scene, path, out=None):
    if out:
        return out
    fname = getattr(scene, "file_name", "")
    if fname:
        return fname[:-4] + ".exr" if len(fname) > 4 else fname + ".exr"
    return os.path.splitext(os.path.basename(path))[0] + ".exr"


def render_file(path, out=None, spp=None, seed=0, materials=None, ctx=None, compression="zip"):
    """Render one scene file; returns (image H x W x 3, the EXR path)."""
    s = load_scene(path, materials=materials)
    own = ctx is None
    ctx = Context() if own else ctx
    try:
        g = Scene(ctx, s)
        try:
            film = g.render(s.spp if spp is None else spp, seed=seed, block=s.block)
        finally:
            g.close()
    finally:
        if own:
            ctx.close()
    img = post_process(film)
    dst = output_path(s, path, out)
    write_exr(dst, img, compression=compression)
    return img, dst


def _material(text):
    name, rest = text.split("=", 1)
    eta, k = rest.split(":")
    return name, (tuple(float(x) for x in eta.split(",")), tuple(float(x) for x in k.split(",")))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("scene")
    ap.add_argument("-o", "--output")
    ap.add_argument("--spp", type=int)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--material", action="append", default=[], type=_material)
    ap.add_argument("--compression", choices=["zip", "none"], default="zip")
    a = ap.parse_args(argv)
    t = time.perf_counter()
    img, dst = render_file(a.scene, a.output, a.spp, a.seed, dict(a.material), compression=a.compression)
    print("Render time: %.3f s -> %s (%dx%d)" % (time.perf_counter() - t, dst, img.shape[1], img.shape[0]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
