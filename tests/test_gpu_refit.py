"""rt_scene_refit: a resident scene's triangles moved on the device, its
tree's boxes recomputed bottom-up over the unchanged topology.

Checked against the CPU oracle on a scene built from the moved positions
(the same tolerances as the other parity tests: identical hit/miss and
triangle, t and barycentrics within 2 ulp, a different triangle only at
exactly the same distance), and a refit back to the original positions must
give back the original hits exactly.
"""
import copy

import numpy as np
import pytest

import oracle_lib as O
from raytracer_gb300 import scenes

from test_gpu_parity import _random_rays, _ulp_diff

pytestmark = pytest.mark.gpu


def _moved(s, amount=0.03):
    """The scene with every vertex pushed along a smooth field (a wobble
    that keeps the mesh closed and its triangles non-degenerate)."""
    m = copy.copy(s)
    v = np.asarray(s.vertices, np.float32)
    d = np.stack([np.sin(3.1 * v[:, 1] + 0.7), np.cos(2.3 * v[:, 2] - 0.2), np.sin(1.7 * v[:, 0] + 1.3)], 1)
    m.vertices = (v + amount * d).astype(np.float32)
    return m


def _compare(hg, ho):
    hit_g, hit_o = hg["prim"] != -1, ho["prim"] != -1
    assert np.array_equal(hit_g, hit_o)
    both = hit_g & hit_o
    same = both & (hg["prim"] == ho["prim"])
    tied = both & ~same
    assert np.all(hg["t"][tied] == ho["t"][tied]), "another triangle at another distance"
    ut = _ulp_diff(hg["t"][same], ho["t"][same]).max(initial=0)
    uu = _ulp_diff(hg["u"][same], ho["u"][same]).max(initial=0)
    assert ut <= 2 and uu <= 2
    return int(both.sum()), int(tied.sum())


@pytest.mark.parametrize("width", [2, 4, 8])
@pytest.mark.parametrize("where", ["host", "device"])
def test_refit_matches_a_scene_built_from_the_moved_positions(ctx, rtlib, width, where):
    s = scenes.displaced_icosphere(level=5, width=48, height=48, env_size=(128, 64))
    moved = _moved(s)
    g = rtlib.Scene(ctx, s)
    if where == "device":
        torch = pytest.importorskip("torch")
        g.refit(torch.from_numpy(np.ascontiguousarray(moved.vertices)).cuda())
        torch.cuda.synchronize()
    else:
        g.refit(moved.vertices)
    o = O.OracleScene(moved)
    rng = np.random.default_rng(4)
    rays = _random_rays(moved, 20000, rng)
    cam = o.camera_rays(rng.random((5000, 2)) * [moved.camera["width"], moved.camera["height"]])
    rays = np.concatenate([rays, cam])
    ctx.set_bvh_width(width)
    try:
        hits, ties = _compare(g.trace(rays), o.trace(rays))
        assert np.array_equal(g.trace(rays, anyhit=True)["prim"] == 0, o.trace(rays, anyhit=True)["prim"] == 0)
        print("refit (%s, width %d): %d rays, %d hits, %d ties" % (where, width, len(rays), hits, ties))
        assert hits > 5000
        # the film over the refitted tree, against the oracle's
        fg = g.render(2, seed=3, block=16)
    finally:
        ctx.set_bvh_width(2)
    fo = o.render(2, seed=3, block=16)
    assert np.array_equal(fg[..., 3], fo[..., 3])
    err = (np.abs(fg[..., :3].astype(np.float64) - fo[..., :3]) / np.maximum(np.abs(fo[..., :3]), 1e-3)).max(-1)
    assert float(np.mean(err > 1e-3)) <= 0.002
    # the scene box follows the positions
    b = g.info()["bounds"]
    lo, hi = b[:3], b[3:]
    v = moved.vertices
    assert np.all(lo <= v.min(0)) and np.all(hi >= v.max(0))
    g.close()
    o.close()


def test_refit_back_gives_the_original_hits(ctx, rtlib):
    s = scenes.displaced_icosphere(level=4, width=40, height=40, env_size=(64, 32))
    g = rtlib.Scene(ctx, s)
    rays = _random_rays(s, 20000, np.random.default_rng(8))
    before = g.trace(rays)
    g.refit(_moved(s, 0.05).vertices)
    g.refit(s.vertices)
    after = g.trace(rays)
    for k in ("t", "u", "v", "prim"):
        assert np.array_equal(before[k], after[k]), k
    g.close()


def test_refit_refusals(ctx, rtlib):
    c = scenes.cornell_box(32, 32)          # its light is an emissive mesh
    g = rtlib.Scene(ctx, c)
    with pytest.raises(rtlib.RtError):
        g.refit(c.vertices)
    g.close()
    s = scenes.displaced_icosphere(level=3, width=32, height=32, env_size=(64, 32))
    g = rtlib.Scene(ctx, s)
    with pytest.raises(rtlib.RtError):
        g.refit(s.vertices, normals=s.vertices)   # the scene has no vertex normals
    g.close()
