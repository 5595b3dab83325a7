"""The bounds-checked build (drawlab_gb300.build --checked, compiled with
-DDL_CHECKS): every queue position, path slot, path index, BVH node and
triangle index the kernels take from a queue, counter or record is checked
against its array before the access; a violation sets an error bit and the
call fails with "bounds check failed".  This stands in for a memory checker,
which the GPUs these tests run on do not offer.

The test builds that library, renders the small cases of every entry point
with it in a child process (the Cornell box, the envmap scene with its NEE /
MIS / miss paths, a three-request batch, a guided render, the wavefront ray
batches, per-path Li and the allocation-free Li), and requires no violation
and images bit-equal to the regular library's.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
sys.path[:0] = [REPO, REPO + "/tests/golden"]
from drawlab_gb300 import abi, api, scenes
import make_golden as mg
out = {}
ctx = api.Context(0)
corn = api.Scene.from_data(ctx, scenes.cornell(width=48, height=40))
out["cornell"] = corn.render(abi.make_opts(spp=8, max_depth=8, seed=3))
env = api.Scene.from_data(ctx, scenes.env_spheres(width=48, height=32))
out["env"] = env.render(abi.make_opts(spp=8, max_depth=8, seed=4))
out["env_power"] = env.render(abi.make_opts(spp=4, max_depth=8, seed=4, flags=abi.DL_RENDER_POWER_LIGHT_PICK))
small_pool = abi.make_opts(spp=4, max_depth=8, seed=5, max_paths_in_flight=256)
out["cornell_small_pool"] = corn.render(small_pool)
sph = api.Scene.from_data(ctx, scenes.material_spheres(width=64, height=36, num_spheres=16, level=2))
imgs = ctx.render_batch([(corn, abi.make_opts(spp=4, max_depth=6, seed=6)),
                         (env, abi.make_opts(spp=2, max_depth=6, seed=7)),
                         (sph, abi.make_opts(spp=4, max_depth=10, seed=8))])
for k, im in enumerate(imgs):
    out["batch%d" % k] = im
g = api.Guide(ctx, seed=9)
gimg = env.render_guided(abi.make_opts(spp=4, max_depth=6, seed=10), g)
out["guided_finite"] = np.array([float(np.isfinite(gimg).all())])
rays = mg.seeded_rays(scenes.cornell(), 4096, seed=11)
p, t, u, v = corn.trace_closest(rays, wavefront=True)
out["wf_prim"], out["wf_t"] = p, t
out["wf_occ"] = corn.trace_any(rays, wavefront=True)
out["batch_prim"] = corn.trace_closest(rays)[0]
xys = np.array([(x, y, s) for y in range(0, 32, 3) for x in range(0, 48, 3) for s in range(4)], np.int32)
out["li"] = env.li(abi.make_opts(max_depth=8, seed=12), xys)[0]
np.savez(OUT, **out)
print("child ok")
"""


def _render_set(lib_path, out_path):
    env = dict(os.environ)
    if lib_path:
        env["DRAWLAB_GB300_LIBRARY"] = str(lib_path)
    code = CHILD.replace("REPO", json.dumps(REPO)).replace("OUT", json.dumps(str(out_path)))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return dict(np.load(out_path))


def test_bounds_checked_build_renders_without_violations(tmp_path):
    from drawlab_gb300 import build
    checked = build.build(checked=True)
    regular = build.build()
    a = _render_set(checked, tmp_path / "checked.npz")
    b = _render_set(regular, tmp_path / "regular.npz")
    assert a.keys() == b.keys()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert a["guided_finite"][0] == 1.0
