"""The device tree's depth stays within the traversal stacks (no GPU needed).

The reference's traversal keeps a fixed stack of 64 entries
(accelStruct/Bvh.cpp:402) and would write past it on a tree deeper than
that.  The device traversals keep a sentinel plus one entry per level in 64
entries (RT_STACK), so the builder bounds the depth: wherever the SAH tree
would grow past the cap it splits at the object median.  rt_bvh_stats builds
the tree on the host exactly as rt_scene_create does, checks it structurally
(every triangle in one leaf, inside every box on its path) and reports the
deepest leaf.
"""
import numpy as np
import pytest

from raytracer_gb300 import core


def geometric_strip(n, ratio):
    """n triangles along +x, triangle i at x = ratio^i with size 0.1 x: the
    SAH peels off a few of the largest per level, so the tree grows deep."""
    x = ratio ** np.arange(n, dtype=np.float64)
    s = 0.1 * x
    t = np.zeros((n, 3, 3))
    t[:, 0, 0] = x
    t[:, 1, 0] = x + s
    t[:, 2, 0] = x
    t[:, 2, 1] = s
    t[:, 2, 2] = 0.5 * s
    return t.astype(np.float32)


def random_soup(n, seed):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3)) * 10.0
    return (c + rng.normal(scale=0.05, size=(n, 3, 3))).astype(np.float32)


@pytest.fixture(scope="module")
def lib():
    from raytracer_gb300 import build
    build.build()
    return core.lib()


def test_default_cap_on_deep_sah_tree(lib):
    t = geometric_strip(60, 2.0)
    d, nodes = core.bvh_stats(t)
    assert 12 < d <= 62 and nodes == 59
    d8, _ = core.bvh_stats(t, width=8)
    assert d8 <= d


@pytest.mark.parametrize("cap", [8, 12, 20])
def test_reduced_cap_bounds_the_depth(lib, cap):
    t = geometric_strip(60, 2.0)
    free, _ = core.bvh_stats(t)
    assert free > cap                      # the SAH tree alone is deeper
    # capped; rt_bvh_stats has checked that every triangle is in one leaf
    d, nodes = core.bvh_stats(t, depth_cap=cap)
    assert d <= cap and 0 < nodes <= 59
    d8, _ = core.bvh_stats(t, width=8, depth_cap=cap)
    assert d8 <= cap


def test_cap_on_a_large_soup(lib):
    t = random_soup(20000, 3)
    free, _ = core.bvh_stats(t)
    d, _ = core.bvh_stats(t, depth_cap=16)   # 2^16 >= 20000 triangles
    assert d <= 16 <= free + 16


def test_bad_caps_are_refused(lib):
    t = random_soup(100, 1)
    with pytest.raises(core.RtError):
        core.bvh_stats(t, depth_cap=5)        # 2^5 < 100 triangles
    with pytest.raises(core.RtError):
        core.bvh_stats(t, depth_cap=63)       # beyond the stack
    assert core.bvh_stats(np.zeros((0, 3, 3), np.float32)) == (0, 0)


@pytest.mark.parametrize("tris", ["strip", "soup"])
def test_four_wide_collapse(lib, tris):
    """The 4-wide tree collapsed from the binary one: rt_bvh_stats checks that
    every binary leaf is reached exactly once, with the binary tree's box, and
    that unused slots cannot be entered; it is no deeper and has fewer nodes."""
    t = geometric_strip(60, 2.0) if tris == "strip" else random_soup(20000, 3)
    d2, n2 = core.bvh_stats(t)
    d4, n4 = core.bvh_stats(t, width=4)
    assert d4 <= d2 and 0 < n4 < n2
    if tris == "soup":
        assert d4 <= (d2 + 1) // 2 + 2      # two binary levels per 4-wide level, give or take
    cap = 12 if tris == "strip" else 16
    d4c, _ = core.bvh_stats(t, width=4, depth_cap=cap)
    assert d4c <= cap


def test_reference_tree_import():
    """rt_scene_create_bvh takes the reference's own tree: the oracle builds
    the reference's two-level SAH BVH (Bvh.cpp, MeshFactory + Scene), flattens
    it into one binary tree over the triangles, and the library's host import
    turns it into the device image (rt_bvh_import_check checks every triangle
    in one leaf and inside every box on its path)."""
    import oracle_lib as O
    from raytracer_gb300 import scenes
    for s in (scenes.cornell_box(32, 32), scenes.displaced_icosphere(level=4, width=32, height=32, env_size=(64, 32))):
        o = O.OracleScene(s)
        nodes, prims = o.export_bvh()
        tri = np.asarray(s.vertices, np.float32).reshape(-1, 3)[np.asarray(s.indices).reshape(-1, 3)]
        assert sorted(prims.tolist()) == list(range(len(tri)))
        d, n = core.bvh_import_check(tri, nodes, prims)
        counts = nodes[:, 3]
        leaves = int(np.count_nonzero(counts))
        # leaves of more than 8 triangles are split in halves of their range
        extra = int(sum(int(np.ceil(c / 8.0)) - 1 for c in counts if c > 8))
        assert n >= len(nodes) - leaves + extra and 0 < d < 62
        # malformed trees are refused
        bad = nodes.copy()
        bad[0, 0] = bad[0, 1]
        with pytest.raises(core.RtError):
            core.bvh_import_check(tri, bad, prims)
        with pytest.raises(core.RtError):
            core.bvh_import_check(tri, nodes, prims[:-1])
        dup = prims.copy()
        dup[0] = dup[1]
        with pytest.raises(core.RtError):
            core.bvh_import_check(tri, nodes, dup)
        o.close()
