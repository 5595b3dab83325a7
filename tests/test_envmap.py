"""The envmap emitter (include/optix/light/envmap.h, src/tracer/emitter/
envmap.cpp:59-141) in the oracle: the alias table reproduces the texel
importance exactly, the pdf is a normalised solid-angle density, and the
NEE + MIS estimator is unbiased under a constant sky (known answer)."""
import numpy as np
import pytest

import pyoracle as po
from drawlab_gb300 import abi, scenes


def texel_solid_angles(w, h):
    """Solid angle of each texel row, in the reference's float arithmetic
    (envmap.cpp:84-99: float theta, double cos rounded to float, float
    difference and product)."""
    pi = np.float32(np.pi)
    step_theta = np.float32(pi / np.float32(h))
    step_phi = np.float32(np.float32(2.0 * np.float64(pi)) / np.float32(w))
    theta = np.arange(h + 1, dtype=np.float32) * step_theta
    c = np.cos(theta.astype(np.float64)).astype(np.float32)
    c[0] = np.float32(1.0)
    return ((c[:-1] - c[1:]) * step_phi).astype(np.float32)


def importance(env, w, h):
    return (texel_solid_angles(w, h)[:, None] * env.max(axis=2)).astype(np.float32).astype(np.float64)


def alias_probabilities(q, alias):
    """Pick probability of every entry implied by an alias table."""
    n = q.size
    qq = np.minimum(q.ravel().astype(np.float64), 1.0)
    p = qq.copy()
    np.add.at(p, alias.ravel().astype(np.int64), 1.0 - qq)
    return p / n


@pytest.mark.parametrize("size", [(64, 32), (256, 128), (37, 19)])
def test_alias_table_reproduces_importance(size):
    w, h = size
    sc = scenes.env_spheres(env_width=w, env_height=h)
    orc = po.OracleScene(sc)
    q, alias, pdf = orc.env_tables()
    imp = importance(sc.lights[-1].env_rgb, w, h)
    want = imp / imp.sum()
    got = alias_probabilities(q, alias).reshape(h, w)
    # the residual chain runs in double: every pick probability is the
    # texel's importance share to float precision
    rel = np.abs(got - want) / want
    assert rel.max() < 1e-6, rel.max()
    assert abs(got.sum() - 1.0) < 1e-6
    assert (alias < w * h).all()


def test_alias_table_on_a_two_level_map():
    # importance 3:1 between the two halves of each row
    w, h = 16, 2
    sc = scenes.env_spheres(env_width=w, env_height=h)
    env = np.ones((h, w, 3), np.float32)
    env[:, : w // 2] = 3.0
    sc.lights[-1].env_rgb = env
    q, alias, pdf = po.OracleScene(sc).env_tables()
    got = alias_probabilities(q, alias).reshape(h, w)
    imp = importance(env, w, h)
    np.testing.assert_allclose(got, imp / imp.sum(), rtol=1e-6)


def test_pdf_is_a_solid_angle_density():
    w, h = 128, 64
    sc = scenes.env_spheres(env_width=w, env_height=h)
    q, alias, pdf = po.OracleScene(sc).env_tables()
    total = (pdf.astype(np.float64) * texel_solid_angles(w, h)[:, None].astype(np.float64)).sum()
    assert abs(total - 1.0) < 1e-4


def constant_sky_plane(value=0.75, albedo=0.6, w=8, h=8):
    s = scenes.SceneData("plane_under_sky", spp=1, max_depth=1, rr_depth=3)
    m = s.add_material(scenes.Material(albedo=(albedo, albedo, albedo)))
    p, f, n = scenes.rectangle((-1, 0, -1), (0, 0, 2), (2, 0, 0))
    s.add_mesh(scenes.Mesh(p, f, n, material=m))
    env = np.full((16, 32, 3), value, np.float32)
    s.lights.append(scenes.Light(type=abi.DL_LIGHT_ENVMAP, env_rgb=env))
    s.camera = scenes.Camera(width=w, height=h, eye=(0.0, 3.0, 0.01), lookat=(0.0, 0.0, 0.0),
                             up=(0.0, 0.0, -1.0), fov=20.0)
    return s


def test_constant_sky_direct_light_is_unbiased():
    # direct light on a diffuse plane under a constant sky c: L = albedo * c
    sc = constant_sky_plane()
    orc = po.OracleScene(sc)
    spp = 256
    xys = np.array([(x, y, s) for y in range(8) for x in range(8) for s in range(spp)], np.int32)
    L, _ = orc.li(abi.make_opts(spp=spp, max_depth=1, seed=3), xys, threads=4)
    want = 0.6 * 0.75
    mean = L.mean(axis=0)
    sigma = L.std(axis=0) / np.sqrt(L.shape[0])
    assert np.all(np.abs(mean - want) < 4 * sigma + 1e-6), (mean, sigma)


def test_camera_rays_see_sky_or_background():
    sc = scenes.env_spheres(width=32, height=20, visual=1)
    orc = po.OracleScene(sc)
    # the top rows look at the sky: radiance > 0 with visual = 1
    xys = np.array([(x, 0, 0) for x in range(32)], np.int32)
    L, _ = orc.li(abi.make_opts(max_depth=1, seed=1), xys)
    assert (L.sum(axis=1) > 0).all()
    sc0 = scenes.env_spheres(width=32, height=20, visual=0)
    L0, _ = po.OracleScene(sc0).li(abi.make_opts(max_depth=1, seed=1), xys)
    np.testing.assert_array_equal(L0, np.tile(np.float32([0.1, 0.2, 0.3]), (32, 1)))


@pytest.mark.parametrize("make", [lambda: scenes.reference_spheres(width=12, height=8),
                                  lambda: scenes.env_spheres(width=12, height=8)])
def test_power_light_pick_is_unbiased(make):
    # the power-proportional emitter pick changes the variance, not the mean
    # (with the point light in its unbiased form: the reference CPU form
    # weights a delta light by MIS against the BSDF, so its expectation
    # depends on the pick probability)
    sc = make()
    orc = po.OracleScene(sc)
    spp = 512
    xys = np.array([(x, y, s) for y in range(8) for x in range(12) for s in range(spp)], np.int32)
    means, sig = [], []
    fix = abi.DL_RENDER_FIX_POINT_LIGHT
    for flags in (fix, fix | abi.DL_RENDER_POWER_LIGHT_PICK):
        L, _ = orc.li(abi.make_opts(spp=spp, max_depth=4, seed=9 + flags, flags=flags), xys, threads=4)
        L = L[np.isfinite(L).all(1)]
        means.append(L.mean(0))
        sig.append(L.std(0) / np.sqrt(len(L)))
    z = np.abs(means[0] - means[1]) / np.sqrt(sig[0] ** 2 + sig[1] ** 2)
    assert (z < 4).all(), (means, z)
