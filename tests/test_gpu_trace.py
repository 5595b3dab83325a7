"""First-hit and shadow-ray parity of the GPU traversal against the oracle's
octree (and the reference's golden vectors), for both GPU traversal paths:
"batch" -- the stand-alone ray-batch kernels of dl_trace_closest /
dl_trace_any -- and "wavefront" -- dl_trace_closest_wavefront /
dl_trace_any_wavefront, which run the renderer's own persistent k_traverse
kernels, the ones dl_render launches for extension and shadow rays.

Bar: the same triangle id for every ray, hit t/u/v bit-identical (the device
runs the reference's Moller-Trumbore with the same float operations),
except rays whose hit lies within 1e-6 of a triangle edge or ties two
triangles within 1e-5 in t, where the octree's and the BVH's visiting
orders may legitimately pick different triangles.  Those rays must stay
rarer than 0.2 %.
"""
import os

import numpy as np
import pytest

import make_golden as mg
import pyoracle as po
from drawlab_gb300 import abi, api, scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EDGE = 1e-6
TIE = 1e-5


@pytest.fixture(scope="module")
def ctx():
    return api.Context(0)


def near_edge(u, v, hit):
    w = 1.0 - u - v
    return hit & (np.minimum(np.minimum(u, v), w) < EDGE)


def compare_closest(g, o, max_ambiguous=2e-3):
    gp, gt, gu, gv = g
    op, ot, ou, ov = o
    ambiguous = near_edge(gu, gv, gp >= 0) | near_edge(ou, ov, op >= 0)
    both = (gp >= 0) & (op >= 0) & (gp != op)
    ambiguous |= both & (np.abs(gt - ot) <= TIE * np.maximum(np.abs(ot), 1e-30))
    keep = ~ambiguous
    assert ambiguous.mean() <= max_ambiguous, "too many ambiguous rays: %.5f" % ambiguous.mean()
    np.testing.assert_array_equal(gp[keep], op[keep])
    hit = keep & (op >= 0)
    np.testing.assert_array_equal(gt[hit], ot[hit])
    np.testing.assert_array_equal(gu[hit], ou[hit])
    np.testing.assert_array_equal(gv[hit], ov[hit])
    return keep


def scene_cases():
    return {
        "cornell": scenes.cornell(),
        "refspheres": scenes.reference_spheres(),
        "mis_plates": scenes.mis_plates(width=320, height=180),
        "spheres16": scenes.material_spheres(width=320, height=180, num_spheres=16, level=3),
    }


CASES = scene_cases()
KERNELS = ["batch", "wavefront"]


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("name", sorted(CASES))
def test_first_hit_matches_oracle(ctx, name, kernel):
    sc = CASES[name]
    gs = api.Scene.from_data(ctx, sc)
    orc = po.OracleScene(sc)
    wf = kernel == "wavefront"
    rays = mg.seeded_rays(sc, 60000, seed=17)
    keep = compare_closest(gs.trace_closest(rays, wavefront=wf), orc.trace_closest(rays))
    # any-hit on the same rays with a finite tmax halfway to the closest hit
    prim, t, _, _ = orc.trace_closest(rays)
    r2 = rays.copy()
    hit = prim >= 0
    r2[hit, 7] = np.where(np.arange(hit.sum()) % 2 == 0, 0.5 * t[hit], 1.5 * t[hit])
    g_occ = gs.trace_any(r2, wavefront=wf)
    o_occ = orc.trace_any(r2)
    near_tmax = hit & (np.abs(r2[:, 7] - t) <= TIE * np.abs(t))
    ok = keep & ~near_tmax
    np.testing.assert_array_equal(g_occ[ok], o_occ[ok])


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("name", ["cornell", "refspheres"])
def test_first_hit_matches_reference_golden(ctx, name, kernel):
    sc = mg.fixture_scenes()[name]
    g = np.load(os.path.join(GOLDEN, f"{name}_trace.npz"))
    gs = api.Scene.from_data(ctx, sc)
    wf = kernel == "wavefront"
    compare_closest(gs.trace_closest(g["rays"], wavefront=wf), (g["prim"], g["t"], g["u"], g["v"]))
    np.testing.assert_array_equal(gs.trace_any(g["rays"], wavefront=wf), g["occ"])


@pytest.mark.parametrize("kernel", KERNELS)
def test_full_material_scene_first_hits(ctx, kernel):
    # the 327,682-triangle scene, 100k seeded rays
    sc = scenes.material_spheres(width=320, height=180)
    gs = api.Scene.from_data(ctx, sc)
    info = gs.info()
    assert info.num_triangles == 64 * 5120 + 2 + 4 * 2   # spheres, ground, light quads
    assert info.bvh_depth <= 64
    orc = po.OracleScene(sc)
    rays = mg.seeded_rays(sc, 100000, seed=23)
    compare_closest(gs.trace_closest(rays, wavefront=kernel == "wavefront"), orc.trace_closest(rays))


def test_wavefront_rays_need_the_render_tmin(ctx):
    sc = scenes.cornell()
    gs = api.Scene.from_data(ctx, sc)
    rays = mg.seeded_rays(sc, 64, seed=3)
    rays[5, 3] = 1e-3
    with pytest.raises(RuntimeError, match="tmin"):
        gs.trace_closest(rays, wavefront=True)
    with pytest.raises(RuntimeError, match="tmin"):
        gs.trace_any(rays, wavefront=True)


@pytest.mark.parametrize("kernel", KERNELS)
def test_edge_cases(ctx, kernel):
    sc = scenes.cornell()
    gs = api.Scene.from_data(ctx, sc)
    wf = kernel == "wavefront"
    orc = po.OracleScene(sc)
    rays = np.zeros((7, 8), np.float32)
    rays[:, 0:3] = (0.1, 0.2, 0.05)
    rays[:, 3] = 1e-4
    rays[:, 7] = np.inf
    rays[0, 4:7] = (0, 0, 0)                 # zero direction: no hit
    rays[1, 4:7] = (0, 0, -1)                # axis-aligned, at the back wall
    rays[2, 4:7] = (1, 0, 0)                 # axis-aligned, at the green wall
    rays[3, 4:7] = (0, 0, -1)
    rays[3, 3], rays[3, 7] = 5.0, 1.0        # tmin > tmax: no hit
    rays[4, 0:3] = (0, 0, 10)
    rays[4, 4:7] = (0, 0, 1)                 # pointing away from the scene
    rays[5, 0:3] = (0.1, 2.0, 0.3)
    rays[5, 4:7] = (0, -1, 0)                # from above, through the ceiling
    rays[6, 0:3] = (0.0, 0.0, 0.0)
    rays[6, 4:7] = (0, 0, -1)                # exactly on the back wall's diagonal
    if wf:
        # the renderer's traversal starts every ray at 1e-4: the tmin > tmax
        # case becomes an empty [1e-4, 0] interval
        rays[3, 3], rays[3, 7] = 1e-4, 0.0
    g = gs.trace_closest(rays, wavefront=wf)
    o = orc.trace_closest(rays)
    keep = compare_closest(g, o, max_ambiguous=1.0 / 7)
    assert keep[:6].all()
    assert (g[0][[0, 3, 4]] == -1).all()
    assert g[0][6] >= 0                      # the diagonal ray hits one of the two triangles
    assert gs.trace_closest(rays[:0], wavefront=wf)[0].shape == (0,)
    np.testing.assert_array_equal(gs.trace_any(rays, wavefront=wf), orc.trace_any(rays))


@pytest.mark.parametrize("kernel", KERNELS)
def test_empty_scene_misses(ctx, kernel):
    sc = scenes.SceneData("empty")
    sc.materials.append(scenes.Material())
    sc.camera = scenes.Camera(width=8, height=8)
    gs = api.Scene.from_data(ctx, sc)
    rays = np.zeros((4, 8), np.float32)
    rays[:, 6] = 1
    rays[:, 7] = np.inf
    rays[:, 3] = 1e-4
    wf = kernel == "wavefront"
    prim, t, u, v = gs.trace_closest(rays, wavefront=wf)
    assert (prim == -1).all()
    assert (gs.trace_any(rays, wavefront=wf) == 0).all()


@pytest.mark.parametrize("kernel", KERNELS)
def test_one_leaf_scene(ctx, kernel):
    # two triangles make a one-leaf tree, whose root references the leaf
    # from both child slots: hits and misses still match the oracle
    sc = scenes.SceneData("one_leaf")
    m = sc.add_material(scenes.Material())
    p, f, n = scenes.rectangle((-1.0, -1.0, 0.0), (2.0, 0.0, 0.0), (0.0, 2.0, 0.0))
    sc.add_mesh(scenes.Mesh(p, f, n, material=m))
    sc.camera = scenes.Camera(width=8, height=8)
    gs = api.Scene.from_data(ctx, sc)
    assert gs.info().num_bvh_nodes == 1
    orc = po.OracleScene(sc)
    rng = np.random.default_rng(17)
    rays = np.zeros((512, 8), np.float32)
    rays[:, 0:2] = rng.uniform(-1.5, 1.5, (512, 2))
    rays[:, 2] = 2.0
    rays[:, 3] = 1e-4
    rays[:, 6] = -1.0
    rays[:, 7] = np.inf
    wf = kernel == "wavefront"
    g = gs.trace_closest(rays, wavefront=wf)
    o = orc.trace_closest(rays)
    compare_closest(g, o)
    assert (g[0] >= 0).any() and (g[0] == -1).any()
    np.testing.assert_array_equal(gs.trace_any(rays, wavefront=wf), orc.trace_any(rays))
