"""Allocation-free tile render (rt_render_tile_static) against rt_render.

rt_render_tile_static serves callers that cannot allocate device memory
while they render (plugins whose host application owns the device memory
through its own pool under a hard budget, real-time loops that forbid
cudaMalloc/cudaFree after start-up).  Its path state lives in a static
device array shared by every call.  This test renders tiles through it on two calls in a row and
checks each against the same pixels of an ordinary rt_render film: the same
kernels run on the same per-path sample streams, so the tolerance is the
parity tests' 1e-5 relative and, in practice, bitwise equality.
"""
import numpy as np
import pytest

from raytracer_gb300 import desc as D, scenes

pytestmark = pytest.mark.gpu


def _tile_box(scene, tx, ty, block):
    W, H = scene.camera["width"], scene.camera["height"]
    x0, y0 = tx * block, ty * block
    return slice(y0, min(H, y0 + block)), slice(x0, min(W, x0 + block))


@pytest.mark.parametrize("which", ["path_mis", "volpath"])
def test_static_tile_render_matches_rt_render(ctx, rtlib, which):
    torch = pytest.importorskip("torch")
    if which == "path_mis":
        s = scenes.cornell_box(80, 48)
        spp, tiles = 4, [(1, 0), (2, 1)]          # (2, 1) is a ragged 16x16 tile
    else:
        s = scenes.volume_grid(48, 40, res=32)
        spp, tiles = 2, [(0, 0), (1, 1)]
    block = 32
    g = rtlib.Scene(ctx, s)
    ref = g.render(spp, seed=3, block=block)
    H, W = ref.shape[:2]
    film = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for tx, ty in tiles:  # two calls in a row sharing the static scratch
        g.render_tile_static(tx, ty, film.data_ptr(), spp, seed=3, block=block)
    torch.cuda.synchronize()
    out = film.cpu().numpy()
    touched = np.zeros((H, W), bool)
    for tx, ty in tiles:
        ys, xs = _tile_box(s, tx, ty, block)
        touched[ys, xs] = True
        a, b = out[ys, xs], ref[ys, xs]
        assert np.array_equal(a[..., 3], b[..., 3])
        np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=1e-5, atol=1e-7)
        print("%s tile (%d,%d): bitwise equal %s" % (which, tx, ty, np.array_equal(a, b)))
    assert not out[~touched].any(), "pixels outside the requested tiles were written"
    # a repeated call overwrites its tile with the same values (scratch reuse)
    g.render_tile_static(*tiles[0], film.data_ptr(), spp, seed=3, block=block)
    torch.cuda.synchronize()
    ys, xs = _tile_box(s, *tiles[0], block)
    np.testing.assert_allclose(film.cpu().numpy()[ys, xs], ref[ys, xs], rtol=1e-5, atol=1e-7)
    g.close()


def test_static_tile_render_rejects_oversize(ctx, rtlib):
    torch = pytest.importorskip("torch")
    import raytracer_gb300 as R
    s = scenes.cornell_box(64, 64)
    g = rtlib.Scene(ctx, s)
    film = torch.zeros((64, 64, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(R.RtError) as e:
        g.render_tile_static(0, 0, film.data_ptr(), 4096, seed=0, block=32)   # 4M path samples
    assert e.value.status == 3 and "static scratch" in str(e.value)
    with pytest.raises(R.RtError):
        g.render_tile_static(5, 0, film.data_ptr(), 1, seed=0, block=32)     # outside the job grid
    g.close()


@pytest.mark.parametrize("which", ["textured", "microfacet", "textured_volpath"])
def test_static_tile_render_mixed_queue_scenes(ctx, rtlib, which):
    """Textured and Microfacet BSDFs shade from the mixed queue, which the
    static scratch holds for scenes that have such BSDFs: the tiles equal
    rt_render's (VolPathTracing applies the textures in its kernel)."""
    torch = pytest.importorskip("torch")
    if which == "microfacet":
        s = scenes.cornell_box(64, 48)
        s.meshes[0]["bsdf"] = s.add_bsdf(D.bsdf(D.BSDF_MICROFACET, albedo=(0.5, 0.5, 0.5), ks=0.3, alpha=0.2))
    else:
        s = scenes.textured_room(64, 48)
        if which == "textured_volpath":
            s.integrator = dict(s.integrator, integrator=D.INTEGRATOR_VOLPATH)
    block, spp, tiles = 32, 2, [(0, 0), (1, 1)]
    g = rtlib.Scene(ctx, s)
    ref = g.render(spp, seed=1, block=block)
    film = torch.zeros((48, 64, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for tx, ty in tiles:
        g.render_tile_static(tx, ty, film.data_ptr(), spp, seed=1, block=block)
    torch.cuda.synchronize()
    out = film.cpu().numpy()
    for tx, ty in tiles:
        ys, xs = _tile_box(s, tx, ty, block)
        a, b = out[ys, xs], ref[ys, xs]
        assert np.array_equal(a[..., 3], b[..., 3])
        np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=1e-5, atol=1e-7)
        print("%s tile (%d,%d): bitwise equal %s" % (which, tx, ty, np.array_equal(a, b)))
    g.close()


def test_static_tile_render_accumulates_sample_ranges(ctx, rtlib):
    """With RT_RENDER_ACCUMULATE, samples [0, 2) and then [2, 4) rendered
    into one tile sum to the 4-spp rt_render tile (weights exactly; rgb to
    the parity tolerance, the two partial sums being added in another
    order)."""
    torch = pytest.importorskip("torch")
    s = scenes.cornell_box(64, 48)
    block, tile = 32, (1, 0)
    g = rtlib.Scene(ctx, s)
    ref = g.render(4, seed=5, block=block)
    film = torch.zeros((48, 64, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    g.render_tile_static(*tile, film.data_ptr(), 2, seed=5, sample_begin=0, block=block, accumulate=True)
    g.render_tile_static(*tile, film.data_ptr(), 2, seed=5, sample_begin=2, block=block, accumulate=True)
    torch.cuda.synchronize()
    ys, xs = _tile_box(s, *tile, block)
    a, b = film.cpu().numpy()[ys, xs], ref[ys, xs]
    assert np.array_equal(a[..., 3], b[..., 3])
    np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=1e-5, atol=1e-6)
    g.close()


def test_static_tile_render_refuses_a_capturing_stream(rtlib):
    """The call synchronises its stream, so on a stream under capture it
    returns RT_ERR_UNSUPPORTED before it queues anything; the capture itself
    stays valid."""
    torch = pytest.importorskip("torch")
    ctx2 = rtlib.Context(0)
    stream = torch.cuda.Stream()
    ctx2.set_stream(stream.cuda_stream)
    s = scenes.cornell_box(32, 32)
    g = rtlib.Scene(ctx2, s)
    film = torch.zeros((32, 32, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        with pytest.raises(rtlib.RtError) as e:
            g.render_tile_static(0, 0, film.data_ptr(), 1, seed=0, block=32)
        film.add_(1.0)
    assert e.value.status == 5 and "captur" in str(e.value)
    graph.replay()
    torch.cuda.synchronize()
    assert float(film[0, 0, 0]) == 1.0
    g.render_tile_static(0, 0, film.data_ptr(), 1, seed=0, block=32)   # fine outside the capture
    torch.cuda.synchronize()
    g.close()
    ctx2.close()
