"""The envmap emitter on the GPU: known answer under a constant sky, the
full-size procedural sky (2048x1024, 0.5-degree sun of peak 1e4) against the
oracle path by path, and argument checks."""
import numpy as np
import pytest

import pyoracle as po
from drawlab_gb300 import abi, api, scenes
from test_envmap import constant_sky_plane

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return api.Context(0)


def test_constant_sky_direct_light_is_unbiased(ctx):
    sc = constant_sky_plane()
    gs = api.Scene.from_data(ctx, sc)
    spp = 1024
    xys = np.array([(x, y, s) for y in range(8) for x in range(8) for s in range(spp)], np.int32)
    L, _ = gs.li(abi.make_opts(spp=spp, max_depth=1, seed=3), xys)
    want = 0.6 * 0.75
    mean = L.mean(axis=0)
    sigma = L.std(axis=0) / np.sqrt(L.shape[0])
    assert np.all(np.abs(mean - want) < 4 * sigma + 1e-6), (mean, sigma)


def test_full_size_sky_matches_oracle(ctx):
    sc = scenes.env_spheres(width=40, height=24, env_width=2048, env_height=1024, sun_radius_deg=0.5,
                            sun_peak=1.0e4)
    gs = api.Scene.from_data(ctx, sc)
    orc = po.OracleScene(sc)
    opts = abi.make_opts(spp=2, max_depth=6, seed=7)
    xys = np.array([(x, y, s) for y in range(24) for x in range(40) for s in range(2)], np.int32)
    Lg, _ = gs.li(opts, xys)
    Lo, _ = orc.li(opts, xys)
    close = np.all(np.abs(Lg - Lo) <= 1e-3 * (1.0 + np.abs(Lo)), axis=1)
    assert close.mean() >= 0.99, close.mean()


def test_envmap_arguments_are_checked(ctx):
    sc = scenes.env_spheres()
    sc.lights[-1].env_rgb = sc.lights[-1].env_rgb.copy()
    sc.lights[-1].env_rgb[0, 0, 0] = -1.0
    with pytest.raises(api.DrawlabError) as e:
        api.Scene.from_data(ctx, sc)
    assert "non-negative" in str(e.value)
    sc = scenes.env_spheres()
    sc.lights.append(sc.lights[-1])
    with pytest.raises(api.DrawlabError) as e:
        api.Scene.from_data(ctx, sc)
    assert "more than one envmap" in str(e.value)
