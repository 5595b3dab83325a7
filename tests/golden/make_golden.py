"""Generate the golden fixtures of tests/golden/ from the reference's OWN CPU
code (oracle/_ref/libdlref.so, built by oracle/build.py from the reference
sources).  The reference ships no test vectors for its path tracer, so these
fixtures are its outputs on seeded inputs:

  <scene>_trace.npz   seeded ray batch -> closest-hit prim id, t, u, v and
                      any-hit flags (OCTree, src/tracer/accel/octree.cpp)
  <scene>_li.npz      (x, y, s) paths with per-path pcg32 streams -> Li and
                      film position (PathIntegrator::Li)
  <scene>_blocks.npz  the block renderer (spiral 32x32 blocks, per-block
                      pcg32, Gaussian film): rgb image, 1 worker thread
  <scene>_emit.npz    Scene::sampleEmitterDirection at seeded points
  bsdf.npz            BSDF eval/pdf/sample for diffuse, mirror, dielectric,
                      microfacet on seeded directions
  perspective_normals.npz
                      the Cornell box seen by the "perspective" camera
                      (PerspectiveCamera, src/tracer/camera/perspective.cpp)
                      through the "normals" integrator (NormalIntegrator,
                      src/tracer/integrator/normal.cpp): (x, y, s) paths ->
                      |shading normal| of the first hit and film position

Run from the repository root:  python tests/golden/make_golden.py
(``--only cameras`` writes perspective_normals.npz alone).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import pyoracle as po  # noqa: E402
from drawlab_gb300 import abi, scenes  # noqa: E402


def fixture_scenes():
    return {
        "cornell": scenes.cornell(width=64, height=64, spp=4, max_depth=0),
        "refspheres": scenes.reference_spheres(width=48, height=32, spp=2),
    }


def seeded_rays(scene, n, seed):
    """Half camera-like rays through the image plane, half random rays from
    points inside the scene bounds; tmin = 1e-4 (the reference default)."""
    rng = np.random.default_rng(seed)
    tri = scene.triangles().reshape(-1, 3)
    lo, hi = tri.min(0), tri.max(0)
    c = scene.camera
    eye = np.asarray(c.eye, np.float32)
    look = np.asarray(c.lookat, np.float32)
    m = n // 2
    tgt = look + rng.normal(scale=0.5 * np.linalg.norm(hi - lo) / 4, size=(m, 3)).astype(np.float32)
    d1 = tgt - eye
    o1 = np.tile(eye, (m, 1))
    o2 = (lo + (hi - lo) * rng.uniform(0.05, 0.95, size=(n - m, 3))).astype(np.float32)
    d2 = rng.normal(size=(n - m, 3)).astype(np.float32)
    o = np.concatenate([o1, o2]).astype(np.float32)
    d = np.concatenate([d1, d2]).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = 1e-4
    rays[:, 4:7] = d
    rays[:, 7] = np.inf
    return rays


def seeded_paths(scene, n, seed):
    rng = np.random.default_rng(seed)
    c = scene.camera
    return np.stack([rng.integers(0, c.width, n), rng.integers(0, c.height, n),
                     rng.integers(0, 64, n)], 1).astype(np.int32)


def bsdf_materials():
    return [
        scenes.Material(type=abi.DL_MAT_DIFFUSE, albedo=(0.3, 0.5, 0.7)),
        scenes.Material(type=abi.DL_MAT_MIRROR),
        scenes.Material(type=abi.DL_MAT_DIELECTRIC, int_ior=1.5046, ext_ior=1.000277),
        scenes.Material(type=abi.DL_MAT_MICROFACET, albedo=(0.2, 0.2, 0.4), alpha=(0.28, 0.28),
                        int_ior=1.7, ext_ior=1.000277),
        scenes.Material(type=abi.DL_MAT_MICROFACET, albedo=(0.05, 0.05, 0.05), alpha=(0.05, 0.05)),
    ]


def bsdf_inputs(n=512, seed=11):
    rng = np.random.default_rng(seed)
    wi = rng.normal(size=(n, 3)).astype(np.float32)
    wo = rng.normal(size=(n, 3)).astype(np.float32)
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    wi[: n // 2, 2] = np.abs(wi[: n // 2, 2])   # half from above the surface
    smp = rng.uniform(size=(n, 2)).astype(np.float32)
    return wi, wo, smp


def emit_inputs(scene, n=512, seed=13):
    rng = np.random.default_rng(seed)
    tri = scene.triangles().reshape(-1, 3)
    lo, hi = tri.min(0), tri.max(0)
    pts = (lo + (hi - lo) * rng.uniform(0.1, 0.9, size=(n, 3))).astype(np.float32)
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    smp = rng.uniform(size=(n, 2)).astype(np.float32)
    return pts, nrm, smp


LI_SEED = 7


def perspective_scene(width=48, height=40):
    """The Cornell box through a "perspective" camera: a <lookat> toWorld
    slightly off the box axis, horizontal fov 50, default clip planes."""
    sc = scenes.cornell(width=width, height=height, spp=2, max_depth=0)
    sc.camera = scenes.Camera(width=width, height=height, type=abi.DL_CAMERA_PERSPECTIVE, fov=50.0,
                              transform=scenes.look_at((0.3, 0.2, 3.6), (0.0, -0.1, 0.0), (0.0, 1.0, 0.0)))
    return sc


def write_camera_fixtures():
    sc = perspective_scene()
    ref = po.RefScene(sc, spp=sc.spp, normals=True)
    xys = seeded_paths(sc, 2048, seed=5)
    L, pos = ref.li(LI_SEED, xys, threads=1)
    np.savez_compressed(os.path.join(HERE, "perspective_normals.npz"), xys=xys, L=L, pos=pos,
                        seed=np.uint64(LI_SEED))
    print("perspective_normals: hits", int((L.sum(1) > 0).sum()), "of", len(L))


def main():
    if po.ref_lib() is None:
        raise SystemExit("reference harness unavailable (needs the reference sources)")
    if "--only" in sys.argv and "cameras" in sys.argv:
        write_camera_fixtures()
        return
    for name, sc in fixture_scenes().items():
        ref = po.RefScene(sc, spp=sc.spp)
        rays = seeded_rays(sc, 4096, seed=1)
        prim, t, u, v = ref.trace_closest(rays, threads=1)
        occ = ref.trace_any(rays, threads=1)
        np.savez_compressed(os.path.join(HERE, f"{name}_trace.npz"), rays=rays, prim=prim, t=t,
                            u=u, v=v, occ=occ)
        xys = seeded_paths(sc, 2048, seed=3)
        L, pos = ref.li(LI_SEED, xys, threads=1)
        np.savez_compressed(os.path.join(HERE, f"{name}_li.npz"), xys=xys, L=L, pos=pos,
                            seed=np.uint64(LI_SEED))
        rgb, _ = ref.render_blocks(threads=1)
        np.savez_compressed(os.path.join(HERE, f"{name}_blocks.npz"), rgb=rgb,
                            spp=np.int32(sc.spp))
        pts, nrm, smp = emit_inputs(sc)
        d, dist, pdf, spec = ref.emitter_sample(pts, nrm, smp)
        np.savez_compressed(os.path.join(HERE, f"{name}_emit.npz"), pts=pts, nrm=nrm, smp=smp,
                            d=d, dist=dist, pdf=pdf, spec=spec)
        print(name, "hits", int((prim >= 0).sum()), "of", len(prim))
    wi, wo, smp = bsdf_inputs()
    out = {"wi": wi, "wo": wo, "smp": smp}
    for k, m in enumerate(bsdf_materials()):
        r = po.bsdf_query("ref", m, wi, wo, smp)
        for key, val in r.items():
            out[f"m{k}_{key}"] = val
    np.savez_compressed(os.path.join(HERE, "bsdf.npz"), **out)
    print("bsdf fixtures written")
    write_camera_fixtures()


if __name__ == "__main__":
    main()
