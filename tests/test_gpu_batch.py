"""Batched rendering (dl_render_batch): requests of different scenes,
resolutions and sample counts in one wavefront give the same images as
rendering each alone; the autotuner picks a valid launch shape that renders
the same images."""
import numpy as np
import pytest

from drawlab_gb300 import abi, api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return api.Context(0)


def small_batch(ctx):
    sa = api.Scene.from_data(ctx, scenes.cornell(width=48, height=40))
    sb = api.Scene.from_data(ctx, scenes.env_spheres(width=40, height=24))
    sc = api.Scene.from_data(ctx, scenes.reference_spheres(width=32, height=20))
    return [(sa, abi.make_opts(spp=8, max_depth=6, seed=1)),
            (sb, abi.make_opts(spp=4, max_depth=8, seed=2)),
            (sc, abi.make_opts(spp=6, max_depth=5, seed=3, flags=abi.DL_RENDER_POWER_LIGHT_PICK)),
            (sa, abi.make_opts(spp=3, max_depth=2, seed=4, filter=abi.DL_FILTER_BOX))]


def test_batch_equals_single_renders(ctx):
    items = small_batch(ctx)
    outs = ctx.render_batch(items)
    st = ctx.stats()
    assert st.camera_rays == sum(s.width * s.height * o.spp for s, o in items)
    for (s, o), img in zip(items, outs):
        np.testing.assert_array_equal(img, s.render(o))


def test_batch_in_several_passes(ctx):
    # 2 x 1024^2 x 200 samples exceed one pass of the sample buffer
    s1 = api.Scene.from_data(ctx, scenes.cornell(width=1024, height=1024))
    s2 = api.Scene.from_data(ctx, scenes.env_spheres(width=1024, height=1024))
    items = [(s1, abi.make_opts(spp=200, max_depth=3, seed=5)), (s2, abi.make_opts(spp=200, max_depth=3, seed=6))]
    outs = ctx.render_batch(items)
    for (s, o), img in zip(items, outs):
        np.testing.assert_allclose(img, s.render(o), rtol=1e-5, atol=1e-6)


def test_autotune_keeps_a_valid_shape(ctx):
    items = small_batch(ctx)
    t, trials = ctx.autotune(items, trial_spp=2)
    assert trials == 19
    assert t.paths_in_flight in (1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24, 1 << 25)
    assert t.traverse_ctas_per_sm in (4, 6, 8)
    # shading block size is searched at the same threads per SM
    assert t.shade_threads in (64, 128, 256)
    assert t.shade_ctas_per_sm * t.shade_threads in (8 * 128, 16 * 128, 32 * 128)
    assert t.iterations_per_graph in (2, 4, 8)
    g = ctx.get_tune()
    assert (g.paths_in_flight, g.iterations_per_graph, g.shade_threads) == (
        t.paths_in_flight, t.iterations_per_graph, t.shade_threads)
    # images do not depend on the launch shape
    for (s, o), img in zip(items, ctx.render_batch(items)):
        np.testing.assert_array_equal(img, s.render(o))
    bad = abi.dl_tune_params(paths_in_flight=64, traverse_ctas_per_sm=8, shade_ctas_per_sm=16,
                             iterations_per_graph=3)
    with pytest.raises(api.DrawlabError):
        ctx.set_tune(bad)
    bad = abi.dl_tune_params(paths_in_flight=64, traverse_ctas_per_sm=8, shade_ctas_per_sm=16,
                             iterations_per_graph=4, shade_threads=96)
    with pytest.raises(api.DrawlabError):
        ctx.set_tune(bad)
    # every shading block size renders the same image
    s, o = items[0]
    ref = ctx.render_batch([(s, o)])[0]
    for th in (64, 256):
        ctx.set_tune(abi.dl_tune_params(paths_in_flight=1 << 20, traverse_ctas_per_sm=8, shade_ctas_per_sm=16,
                                        iterations_per_graph=4, shade_threads=th))
        np.testing.assert_array_equal(ctx.render_batch([(s, o)])[0], ref)
    ctx.set_tune(abi.dl_tune_params(paths_in_flight=1 << 22, traverse_ctas_per_sm=8, shade_ctas_per_sm=16,
                                    iterations_per_graph=4))


def test_batch_arguments_are_checked(ctx):
    other = api.Context(0)
    s_other = api.Scene.from_data(other, scenes.cornell(width=16, height=16))
    with pytest.raises(api.DrawlabError) as e:
        ctx.render_batch([(s_other, abi.make_opts(spp=1))])
    assert "another context" in str(e.value)
    s = api.Scene.from_data(ctx, scenes.cornell(width=16, height=16))
    with pytest.raises(api.DrawlabError):
        ctx.render_batch([(s, abi.make_opts(spp=0))])
    assert ctx.render_batch([]) == []


def test_camera_override_equals_a_scene_with_that_camera(ctx):
    base = scenes.cornell(width=48, height=40)
    cam = scenes.Camera(width=64, height=32, eye=(0.3, 0.1, 3.5), lookat=(0.0, -0.2, 0.0), up=(0.0, 1.0, 0.0),
                        fov=35.0)
    other = scenes.cornell(width=48, height=40)
    other.camera = cam
    sa = api.Scene.from_data(ctx, base)
    sb = api.Scene.from_data(ctx, other)
    o = abi.make_opts(spp=4, max_depth=5, seed=12)
    img, = ctx.render_batch([(sa, o, cam)])
    assert img.shape == (32, 64, 3)
    np.testing.assert_array_equal(img, sb.render(o))
