"""The oracle against golden vectors recorded from the reference's OptiX-only
code (aniso_ggx.cu, wrap.h, envmap.h / envmap.cpp, miss.cu, opencv.h /
opencv.cpp, shader_common.h), which oracle/ref_optix.cpp compiles as host
C++; tests/golden/make_golden.py --only optix wrote the fixtures.

Tolerances: the reference computes parts of these in double (G1's 2.0 * z,
Fresnel's 1.0 - F0, the envmap's phi) and normalises by a reciprocal
multiply; the oracle follows the CPU backend's float operations.  Values
agree to a few float ulps: 1e-5 relative (floor 1e-6) for BSDF values and
weights, 2e-6 absolute for unit directions, bit-exact for the envmap's
texel pdfs and texture coordinates.
"""
import os

import numpy as np
import pytest

import make_golden as mg
import pyoracle as po
from drawlab_gb300 import abi, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def close(a, b, rel=1e-5, floor=1e-6):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    bad = np.abs(a - b) > rel * np.maximum(np.abs(b), floor)
    assert not bad.any(), "%d of %d differ, worst %s vs %s" % (
        bad.sum(), bad.size, a[bad][:3], b[bad][:3])


@pytest.mark.parametrize("k", range(4))
def test_ggx_matches_reference(k):
    g = load("optix_ggx.npz")
    pd, ps, ax, ay = mg.ggx_materials()[k]
    m = scenes.Material(type=abi.DL_MAT_ANISO_GGX, albedo=pd, specular=ps, alpha=(ax, ay))
    r = po.bsdf_query("oracle", m, g["wi"], g["wo"], g[f"m{k}_xi"])
    close(r["eval"], g[f"m{k}_eval"])
    close(r["pdf"], g[f"m{k}_pdf"])
    np.testing.assert_allclose(r["wo"], g[f"m{k}_wo"], atol=2e-6, rtol=0)
    close(r["weight"], g[f"m{k}_weight"], rel=2e-5)
    # the lobe coin splits the samples between the two lobes
    lobe = g[f"m{k}_xi"][:, 2] > 0.5
    assert 0.35 < lobe.mean() < 0.65


def env_case(name):
    return mg.env_fixture_scenes()[name]


@pytest.mark.parametrize("name", ["smooth", "sun"])
def test_envmap_tables_match_reference(name):
    e = load("optix_env.npz")
    orc = po.OracleScene(env_case(name))
    q, alias, pdf = orc.env_tables()
    # the oracle's table is the one the fixture's sampling ran on
    np.testing.assert_array_equal(q, e[f"{name}_q"])
    np.testing.assert_array_equal(alias, e[f"{name}_alias"])
    np.testing.assert_array_equal(pdf, e[f"{name}_pdf"])
    # the reference's activate(): the same pdf (its float sum vs the
    # oracle's double sum) and the same alias assignment on these maps
    close(pdf, e[f"{name}_ref_pdf"], rel=1e-5)
    np.testing.assert_array_equal(alias, e[f"{name}_ref_alias"])
    # pick probability of each texel under both tables: the oracle's equals
    # the texel's importance share; the reference's float chain drifts
    def pick(qq, aa):
        n = qq.size
        p = qq.ravel().astype(np.float64).copy()
        np.add.at(p, aa.ravel(), 1.0 - qq.ravel().astype(np.float64))
        p -= np.where(aa.ravel() == np.arange(n), 1.0 - qq.ravel(), 0.0)
        return p / n
    share = pdf.astype(np.float64).ravel()
    env = [l for l in env_case(name).lights if l.type == abi.DL_LIGHT_ENVMAP][0]
    h, w = env.env_rgb.shape[:2]
    area = (np.cos(np.arange(h) * np.pi / h) - np.cos((np.arange(h) + 1) * np.pi / h)) * 2 * np.pi / w
    share = share * np.repeat(area, w)
    share /= share.sum()
    np.testing.assert_allclose(pick(q, alias), share, rtol=1e-4, atol=1e-9)
    np.testing.assert_allclose(pick(e[f"{name}_ref_q"], e[f"{name}_ref_alias"]), share, rtol=2e-2, atol=1e-7)


@pytest.mark.parametrize("name", ["smooth", "sun"])
def test_envmap_sampling_matches_reference(name):
    e = load("optix_env.npz")
    orc = po.OracleScene(env_case(name))
    o = orc.env_query(e[f"{name}_xi"], e[f"{name}_nrm"], e[f"{name}_dirs"])
    np.testing.assert_allclose(o["s_dir"], e[f"{name}_s_dir"], atol=2e-6, rtol=0)
    np.testing.assert_array_equal(o["s_pdf"], e[f"{name}_s_pdf"])
    close(o["s_value"], e[f"{name}_s_value"])
    np.testing.assert_array_equal(o["pdf"], e[f"{name}_pdf_d"])
    close(o["value"], e[f"{name}_value"])


@pytest.mark.parametrize("name", ["smooth", "sun"])
def test_envmap_filter_weights(name):
    # the texture unit keeps 8 fractional bits per filter weight; the
    # renderer blends with fp32 weights.  Record how far apart the two are
    # on these maps (relative to the looked-up radiance): below 10 %, and
    # zero where the four texels agree.
    e = load("optix_env.npz")
    v, hw = e[f"{name}_value"].astype(np.float64), e[f"{name}_value_hw"].astype(np.float64)
    rel = np.abs(hw - v) / np.maximum(np.abs(v), 1e-3)
    assert rel.max() < 0.1
    assert np.median(rel) < 1e-2


@pytest.mark.parametrize("name", ["smooth", "sun"])
def test_env_miss_matches_reference(name):
    e = load("optix_env.npz")
    orc = po.OracleScene(env_case(name))
    out = orc.env_miss(abi.make_opts(), e[f"{name}_dirs"], e[f"{name}_depth"], e[f"{name}_bsdf_pdf"],
                       e[f"{name}_diffuse"])
    close(out, e[f"{name}_miss"])
    sc = env_case(name)
    for l in sc.lights:
        if l.type == abi.DL_LIGHT_ENVMAP:
            l.env_visual = 0
    orc0 = po.OracleScene(sc)
    n = e[f"{name}_dirs"].shape[0]
    bg = orc0.env_miss(abi.make_opts(), e[f"{name}_dirs"], np.zeros(n, np.int32), e[f"{name}_bsdf_pdf"],
                       e[f"{name}_diffuse"])
    np.testing.assert_array_equal(bg, e[f"{name}_miss_bg"])


def opencv_scene(c):
    sc = scenes.cornell(width=int(c["size"][0]), height=int(c["size"][1]))
    fx, fy, cx, cy = (float(v) for v in c["intrinsics"])
    sc.camera = scenes.Camera(width=int(c["size"][0]), height=int(c["size"][1]), type=abi.DL_CAMERA_OPENCV,
                              transform=c["extrinsic"], fx=fx, fy=fy, cx=cx, cy=cy)
    return sc


def test_opencv_camera_matches_reference():
    c = load("optix_camera.npz")
    orc = po.OracleScene(opencv_scene(c))
    # the reference's OptiX camera adds the jitter to the pixel corner; the
    # renderer uses the film position (pixel + jitter) as the sample
    film = np.stack([c["px"] + c["xi"][:, 0], c["py"] + c["xi"][:, 1]], 1)
    o, d = orc.camera_ray(film)
    np.testing.assert_allclose(o, c["o"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(d, c["d"], atol=2e-6, rtol=0)


def test_hit_data_matches_reference():
    h = load("optix_hit.npz")
    sc, _, _ = mg.hit_fixture_scene()
    orc = po.OracleScene(sc)
    for mi in range(2):
        sn, gn, st, tuv = orc.hit_data(h[f"mesh{mi}_prim"], h[f"mesh{mi}_bary"])
        np.testing.assert_allclose(sn, h[f"mesh{mi}_sn"], atol=1e-6, rtol=0)
        np.testing.assert_allclose(gn, h[f"mesh{mi}_gn"], atol=1e-6, rtol=0)
        np.testing.assert_allclose(st, h[f"mesh{mi}_st"], atol=1e-6, rtol=0)
        np.testing.assert_array_equal(tuv, h[f"mesh{mi}_uv"])
    # the textured mesh's coordinates leave [0, 1] (wrap addressing is used)
    uv = h["mesh0_uv"]
    assert (uv < 0).any() and (uv > 1).any()


def test_fixtures_reproduce_from_reference():
    """Where the reference tree is present, its code still gives the recorded
    vectors (first GGX material, both envmap tables)."""
    import pyref_optix as rx
    if not po.ref_available() or rx.lib() is None:
        pytest.skip("reference sources not present")
    g = load("optix_ggx.npz")
    pd, ps, ax, ay = mg.ggx_materials()[0]
    r = rx.ggx(pd, ps, ax, ay, g["wi"], g["wo"], g["seeds"])
    for key in ("eval", "pdf", "xi", "wo", "weight"):
        np.testing.assert_array_equal(r[key], g[f"m0_{key}"])
    e = load("optix_env.npz")
    for name in ("smooth", "sun"):
        env = [l for l in env_case(name).lights if l.type == abi.DL_LIGHT_ENVMAP][0]
        q, alias, pdf = rx.env_tables(env.env_rgb)
        np.testing.assert_array_equal(q, e[f"{name}_ref_q"])
        np.testing.assert_array_equal(alias, e[f"{name}_ref_alias"])
        np.testing.assert_array_equal(pdf, e[f"{name}_ref_pdf"])
