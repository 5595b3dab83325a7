"""Path-tracer parity of the GPU wavefront renderer against the oracle.

1. Path by path (dl_li vs the oracle's Li with the same per-path pcg32
   streams): the camera samples are bit-identical; the radiance agrees to
   1e-3 relative on at least 99 % of paths (the rest diverge at a discrete
   decision -- RR, Fresnel pick, a hit at a grazing edge -- that single-ulp
   differences of sin/cos/exp/log flip).
2. Films: the weight channel equals the oracle's up to float summation
   order; the per-path-stream image agrees with the oracle's per-path image.
3. Statistics against the reference semantics: per-pixel means over
   independent seeds agree with the oracle's within 3 sigma (no bias), and
   against the reference's own block renderer (golden) within a stated
   relMSE.
"""
import os

import numpy as np
import pytest

import make_golden as mg
import pyoracle as po
from drawlab_gb300 import abi, api, scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL_PATH = 1e-3
MIN_CLOSE = 0.99


@pytest.fixture(scope="module")
def ctx():
    return api.Context(0)


def path_close(a, b):
    return np.all(np.abs(a - b) <= RTOL_PATH * (1.0 + np.abs(b)), axis=1) | np.all(
        ~np.isfinite(a) & ~np.isfinite(b), axis=1)


def all_paths(w, h, spp):
    return np.array([(x, y, s) for y in range(h) for x in range(w) for s in range(spp)], np.int32)


def opencv_cornell(width=48, height=40):
    """The Cornell box through an "opencv" camera at the virtual camera's
    place: camera x right, y down, z forward (the world's -z), principal
    point off-centre, fx = fy for the same vertical field of view."""
    sc = scenes.cornell(width=width, height=height)
    f = 0.5 * height / np.tan(np.radians(39.3) / 2)
    ext = np.array([[1, 0, 0, 0], [0, -1, 0, 0], [0, 0, -1, 3.9], [0, 0, 0, 1]], np.float64)
    sc.camera = scenes.Camera(width=width, height=height, type=abi.DL_CAMERA_OPENCV, fx=f, fy=f,
                              cx=0.5 * width + 1.5, cy=0.5 * height - 2.0, transform=ext)
    return sc


LI_CASES = {
    "cornell": (lambda: scenes.cornell(width=48, height=48), dict(max_depth=0)),
    "cornell_d8": (lambda: scenes.cornell(width=48, height=48), dict(max_depth=8)),
    "refspheres": (lambda: scenes.reference_spheres(width=64, height=40), dict(max_depth=0)),
    "refspheres_fix": (lambda: scenes.reference_spheres(width=64, height=40),
                       dict(max_depth=12, flags=abi.DL_RENDER_FIX_POINT_LIGHT)),
    "spheres16": (lambda: scenes.material_spheres(width=96, height=54, num_spheres=16, level=3),
                  dict(max_depth=16)),
    "mis_plates": (lambda: scenes.mis_plates(width=96, height=54), dict(max_depth=8)),
    "env_spheres": (lambda: scenes.env_spheres(width=64, height=40), dict(max_depth=8)),
    "env_only_bg": (lambda: scenes.env_spheres(width=64, height=40, with_area_light=False, visual=0),
                    dict(max_depth=6)),
    "refspheres_power": (lambda: scenes.reference_spheres(width=64, height=40),
                         dict(max_depth=8, flags=abi.DL_RENDER_POWER_LIGHT_PICK)),
    "env_spheres_power": (lambda: scenes.env_spheres(width=64, height=40),
                          dict(max_depth=8, flags=abi.DL_RENDER_POWER_LIGHT_PICK)),
    "perspective": (lambda: mg.perspective_scene(48, 40), dict(max_depth=8)),
    "perspective_normals": (lambda: mg.perspective_scene(48, 40), dict(flags=abi.DL_RENDER_NORMALS)),
    "opencv": (lambda: opencv_cornell(), dict(max_depth=8)),
    "spheres_normals": (lambda: scenes.material_spheres(width=96, height=54, num_spheres=16, level=3),
                        dict(flags=abi.DL_RENDER_NORMALS)),
    "env_normals": (lambda: scenes.env_spheres(width=64, height=40), dict(flags=abi.DL_RENDER_NORMALS)),
    "textured": (lambda: scenes.textured_cornell(48, 48), dict(max_depth=8)),
}


@pytest.mark.parametrize("name", sorted(LI_CASES))
def test_li_matches_oracle_path_by_path(ctx, name):
    make, kw = LI_CASES[name]
    sc = make()
    gs = api.Scene.from_data(ctx, sc)
    orc = po.OracleScene(sc)
    opts = abi.make_opts(spp=2, seed=11, **kw)
    xys = all_paths(sc.camera.width, sc.camera.height, 2)
    Lg, pg = gs.li(opts, xys)
    Lo, pos_o = orc.li(opts, xys)
    np.testing.assert_array_equal(pg, pos_o)
    close = path_close(Lg, Lo)
    assert close.mean() >= MIN_CLOSE, "%s: only %.4f of paths agree" % (name, close.mean())
    # the totals agree too (divergent paths are unbiased either way)
    fin = np.isfinite(Lg).all(1) & np.isfinite(Lo).all(1)
    tg, to = Lg[fin].sum(0), Lo[fin].sum(0)
    np.testing.assert_allclose(tg, to, rtol=0.05)


@pytest.mark.parametrize("name", ["cornell", "refspheres"])
def test_li_matches_reference_golden(ctx, name):
    sc = mg.fixture_scenes()[name]
    g = np.load(os.path.join(GOLDEN, f"{name}_li.npz"))
    gs = api.Scene.from_data(ctx, sc)
    L, pos = gs.li(abi.make_opts(seed=int(g["seed"])), g["xys"])
    np.testing.assert_array_equal(pos, g["pos"])
    assert path_close(L, g["L"]).mean() >= MIN_CLOSE


def test_perspective_normals_match_reference_golden(ctx):
    """The "perspective" camera and "normals" integrator against the
    reference's own outputs (tests/golden/perspective_normals.npz)."""
    g = np.load(os.path.join(GOLDEN, "perspective_normals.npz"))
    gs = api.Scene.from_data(ctx, mg.perspective_scene())
    L, pos = gs.li(abi.make_opts(seed=int(g["seed"]), flags=abi.DL_RENDER_NORMALS), g["xys"])
    np.testing.assert_array_equal(pos, g["pos"])
    assert path_close(L, g["L"]).mean() >= 0.995


def test_normals_render_matches_oracle(ctx):
    """A normals image (dl_render, Gaussian film) of the perspective view
    equals the oracle's per-path render to float summation order."""
    sc = mg.perspective_scene(64, 48)
    gs = api.Scene.from_data(ctx, sc)
    orc = po.OracleScene(sc)
    opts = abi.make_opts(spp=4, seed=9, flags=abi.DL_RENDER_NORMALS)
    rg = gs.render(opts)
    ro, _ = orc.render_paths(opts)
    np.testing.assert_allclose(rg, ro, rtol=1e-4, atol=1e-5)
    assert rg.max() <= 1.0 + 1e-5 and rg.mean() > 0.1


@pytest.mark.parametrize("w,h,filt", [(37, 23, abi.DL_FILTER_GAUSSIAN), (33, 5, abi.DL_FILTER_BOX),
                                      (1, 1, abi.DL_FILTER_GAUSSIAN), (70, 35, abi.DL_FILTER_BOX)])
def test_film_edges_match_oracle(ctx, w, h, filt):
    # film sizes that leave partial 32x32 tiles and partial 4-row groups
    sc = scenes.cornell(width=w, height=h)
    gs = api.Scene.from_data(ctx, sc)
    orc = po.OracleScene(sc, filter=filt)
    opts = abi.make_opts(spp=3, max_depth=4, seed=11, filter=filt)
    fg = gs.render_film(opts)
    _, fo, _ = orc.render_paths(opts, film=True)
    assert fg.shape == fo.shape
    np.testing.assert_allclose(fg[..., 3], fo[..., 3], rtol=2e-5, atol=1e-6)
    # radiance: per-path float differences between the two renderers only
    rel = np.abs(fg[..., :3] - fo[..., :3]) / (np.abs(fo[..., :3]) + 1e-2)
    assert np.mean(rel < 1e-3) > 0.9


def test_film_matches_oracle_per_path_render(ctx):
    sc = scenes.cornell(width=64, height=64)
    gs = api.Scene.from_data(ctx, sc)
    orc = po.OracleScene(sc)
    opts = abi.make_opts(spp=8, max_depth=8, seed=5)
    fg = gs.render_film(opts)
    _, fo, _ = orc.render_paths(opts, film=True)
    # filter weights depend only on the (identical) sample positions
    np.testing.assert_allclose(fg[..., 3], fo[..., 3], rtol=2e-5, atol=1e-6)
    rg = gs.render(opts)
    ro, _ = orc.render_paths(opts)
    rel = np.abs(rg - ro) / (np.abs(ro) + 1e-2)
    assert np.mean(rel < 1e-3) > 0.95
    assert np.mean((rg - ro) ** 2 / (ro ** 2 + 1e-2)) < 1e-3


def test_box_filter_weights(ctx):
    sc = scenes.cornell(width=40, height=30)
    gs = api.Scene.from_data(ctx, sc)
    opts = abi.make_opts(spp=4, max_depth=2, filter=abi.DL_FILTER_BOX, seed=2)
    film = gs.render_film(opts)
    assert film.shape == (30, 40, 4)
    # each sample lands in one pixel (two on an exact pixel border)
    total = film[..., 3].sum()
    assert 40 * 30 * 4 <= total <= 40 * 30 * 4 * 1.01


def test_no_bias_against_oracle_over_seeds(ctx):
    # per-pixel mean over K independent seeds, GPU vs oracle (reference
    # semantics, per-path streams): |z| > 3 must stay rare.
    W = H = 16
    sc = scenes.cornell(width=W, height=H)
    gs = api.Scene.from_data(ctx, sc)
    orc = po.OracleScene(sc)
    K = 12
    gi = np.stack([gs.render(abi.make_opts(spp=64, seed=1000 + k)) for k in range(K)])
    oi = np.stack([orc.render_paths(abi.make_opts(spp=64, seed=2000 + k))[0] for k in range(K)])
    mg_, mo = gi.mean(0), oi.mean(0)
    se = np.sqrt(gi.var(0, ddof=1) / K + oi.var(0, ddof=1) / K) + 1e-6
    z = (mg_ - mo) / se
    assert np.mean(np.abs(z) > 3) < 0.02
    assert abs(z.mean()) < 0.2


def test_image_matches_reference_block_renderer(ctx):
    # reference (golden, its own block renderer, 4 spp, 64x64) vs GPU at
    # 256 spp.  A loose check that the low-spp golden still fits; the tight
    # image test against the reference's 4096-spp render is
    # test_gpu_configs.py::test_c1_converged_image_matches_reference_renderer.
    sc = mg.fixture_scenes()["cornell"]
    g = np.load(os.path.join(GOLDEN, "cornell_blocks.npz"))
    gs = api.Scene.from_data(ctx, sc)
    ref = g["rgb"]
    gpu = gs.render(abi.make_opts(spp=256, seed=9))
    rel = np.mean((ref - gpu) ** 2 / (gpu ** 2 + 1e-2))
    assert rel < 0.1
    assert abs(ref.mean() - gpu.mean()) / gpu.mean() < 0.03


def test_invalid_samples_are_dropped_and_counted(ctx):
    sc = scenes.cornell(width=16, height=16)
    gs = api.Scene.from_data(ctx, sc)
    gs.render(abi.make_opts(spp=4, seed=1))
    st = ctx.stats()
    assert st.camera_rays == 16 * 16 * 4
    assert st.extension_rays >= st.camera_rays
    assert st.invalid_samples >= 0


def test_invalid_arguments(ctx):
    sc = scenes.cornell(width=16, height=16)
    gs = api.Scene.from_data(ctx, sc)
    with pytest.raises(api.DrawlabError) as e:
        gs.render(abi.make_opts(spp=0))
    assert e.value.status == abi.DL_ERR_INVALID_ARG
    bad = scenes.cornell(width=16, height=16)
    bad.meshes[0].material = 99
    with pytest.raises(api.DrawlabError) as e:
        api.Scene.from_data(ctx, bad)
    assert e.value.status == abi.DL_ERR_INVALID_ARG
    bad = scenes.cornell(width=16, height=16)
    bad.lights[0].mesh = 0  # light does not point at the emitting mesh
    with pytest.raises(api.DrawlabError):
        api.Scene.from_data(ctx, bad)
    with pytest.raises(api.DrawlabError):
        gs.li(abi.make_opts(), np.array([[99, 0, 0]], np.int32))


def test_disjoint_sample_ranges_add_up(ctx):
    # replicas render disjoint sample ranges; their films sum to the film of
    # the whole range
    sc = scenes.cornell(width=24, height=24)
    gs = api.Scene.from_data(ctx, sc)
    a = gs.render_film(abi.make_opts(spp=4, spp_offset=0, seed=3, max_depth=4))
    b = gs.render_film(abi.make_opts(spp=4, spp_offset=4, seed=3, max_depth=4))
    c = gs.render_film(abi.make_opts(spp=8, spp_offset=0, seed=3, max_depth=4))
    np.testing.assert_allclose(a + b, c, rtol=1e-4, atol=1e-5)


def test_small_path_pool_matches_large(ctx):
    # the wavefront pool size changes scheduling only, not results
    sc = scenes.cornell(width=32, height=32)
    gs = api.Scene.from_data(ctx, sc)
    xys = all_paths(32, 32, 2)
    a, _ = gs.li(abi.make_opts(seed=4, max_paths_in_flight=64), xys)
    b, _ = gs.li(abi.make_opts(seed=4), xys)
    np.testing.assert_array_equal(a, b)
