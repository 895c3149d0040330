"""Per-path radiance through rt_render_paths (the plugin's li(): a launch of
the (pixel, sample) paths it is asked for) against the oracle's per-path
radiance on the same streams, and against the film of rt_render.

Tolerances: per path, 1e-3 relative (floor 1e-3) on at least 99.5% of the
paths -- the same rule as the film parity tests, where a path whose branch
flips on a last-ulp difference of the device's transcendental functions is
the only source of disagreement (measured: every path within 1e-5).  The
sum of a pixel's paths equals its film entry to 1e-5 relative (the film sums
the same radiance values in sample order).
"""
import numpy as np
import pytest

import oracle_lib as O
from raytracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def _cases():
    from test_gpu_parity import _all_lights_scene
    return {
        "cornell": (scenes.cornell_box(48, 40), 4),
        "all_lights": (_all_lights_scene(), 2),
        "icosphere_env": (scenes.displaced_icosphere(level=4, width=40, height=40, env_size=(128, 64)), 2),
        "volume": (scenes.volume_grid(40, 32, res=32), 2),
    }


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return (np.abs(a - b) / np.maximum(np.abs(b), 1e-3)).max(-1)


@pytest.mark.parametrize("name", ["cornell", "all_lights", "icosphere_env", "volume"])
def test_paths_match_oracle(ctx, rtlib, name):
    s, spp = _cases()[name]
    W, H = s.camera["width"], s.camera["height"]
    rng = np.random.default_rng(5)
    n = 3000
    pix = rng.integers(0, W * H, n).astype(np.int32)
    smp = rng.integers(0, 4096, n).astype(np.int32)
    g = rtlib.Scene(ctx, s)
    o = O.OracleScene(s)
    rg = g.render_paths(pix, smp, seed=9)
    ro = o.render_paths(pix, smp, seed=9)
    err = _rel(rg, ro)
    bad = float(np.mean(err > 1e-3))
    print("%s: %d paths, identical %.4f, >1e-3 rel %.4f" % (name, n, np.mean(err == 0), bad))
    assert np.all(np.isfinite(rg))
    assert bad <= 0.005
    # one-path launches (what li() issues) give the same radiance as the batch
    for i in range(4):
        one = g.render_paths(pix[i:i + 1], smp[i:i + 1], seed=9)
        assert np.array_equal(one[0], rg[i])
    g.close()
    o.close()


def test_paths_sum_to_the_film(ctx, rtlib):
    """Box filter of radius 0.5: a sample lands in its own pixel only, so the
    film's rgb sum over spp samples is the sum of the per-path radiance."""
    s, spp = _cases()["cornell"]
    W, H = s.camera["width"], s.camera["height"]
    g = rtlib.Scene(ctx, s)
    film = g.render(spp, seed=2, block=16)
    pix = np.repeat(np.arange(W * H, dtype=np.int32), spp)
    smp = np.tile(np.arange(spp, dtype=np.int32), W * H)
    rad = g.render_paths(pix, smp, seed=2).reshape(H, W, spp, 3)
    acc = np.zeros((H, W, 3), np.float32)
    for k in range(spp):
        acc += rad[:, :, k]
    assert np.array_equal(film[..., 3], np.full((H, W), spp, np.float32))
    err = _rel(acc, film[..., :3])
    print("paths vs film: identical %.4f, max rel %.2e" % (np.mean(err == 0), err.max()))
    assert err.max() <= 1e-5
    g.close()


def test_paths_reject_bad_indices(ctx, rtlib):
    s, _ = _cases()["cornell"]
    g = rtlib.Scene(ctx, s)
    W, H = s.camera["width"], s.camera["height"]
    with pytest.raises(Exception):
        g.render_paths([W * H], [0])
    with pytest.raises(Exception):
        g.render_paths([0], [-1])
    assert g.render_paths(np.zeros(0, np.int32), np.zeros(0, np.int32)).shape == (0, 3)
    g.close()
