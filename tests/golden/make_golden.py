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
  cornell_hispp.npz   the block renderer on the 64x64 Cornell box at 4096
                      spp (every core): a low-noise image of the reference
  <scene>_emit.npz    Scene::sampleEmitterDirection at seeded points
  bsdf.npz            BSDF eval/pdf/sample for diffuse, mirror, dielectric,
                      microfacet on seeded directions
  perspective_normals.npz
                      the Cornell box seen by the "perspective" camera
                      (PerspectiveCamera, src/tracer/camera/perspective.cpp)
                      through the "normals" integrator (NormalIntegrator,
                      src/tracer/integrator/normal.cpp): (x, y, s) paths ->
                      |shading normal| of the first hit and film position

and, from the reference's OptiX-only code compiled as host C++
(oracle/_ref/libdlref_optix.so, oracle/ref_optix.cpp):

  optix_ggx.npz       aniso_ggx eval / pdf / sample (aniso_ggx.cu:9-121,
                      wrap.h:54-77) of four materials on seeded directions,
                      with the three numbers the shader's rnd() drew
  optix_env.npz       two sky maps: EnvironmentMap::activate's alias table
                      and pdf (envmap.cpp:59-141); Envmap::sampleDirection /
                      pdfDirection / eval (envmap.h:25-94) run on the oracle's
                      table and texels; __miss__radiance (miss.cu:11-49)
  optix_camera.npz    OpencvCamera set-up (opencv.cpp:10-83) and sampleRay
                      (opencv.h:28-46)
  optix_hit.npz       getHitData (shader_common.h:21-143): texture
                      coordinates, world-space normal and tangent maps

Run from the repository root:  python tests/golden/make_golden.py
(``--only cameras`` writes perspective_normals.npz alone, ``--only optix``
the optix_*.npz files alone, ``--only hispp`` cornell_hispp.npz alone).
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


def ggx_materials():
    """(pd, ps, ax, ay): the material scene's GGX, an anisotropic GGX with a
    diffuse part, a coloured rough one, and the MIS plates' sharpest."""
    return [
        ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.15, 0.15),
        ((0.2, 0.2, 0.2), (0.8, 0.8, 0.8), 0.05, 0.3),
        ((0.5, 0.3, 0.1), (0.6, 0.7, 0.8), 0.4, 0.02),
        ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.005, 0.005),
    ]


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def write_ggx_fixture(rx, n=512):
    rng = np.random.default_rng(21)
    wi, wo = unit(rng, n), unit(rng, n)
    wi[: 3 * n // 4, 2] = np.abs(wi[: 3 * n // 4, 2])
    wo[: 3 * n // 4, 2] = np.abs(wo[: 3 * n // 4, 2])
    seeds = rng.integers(1, 2**32 - 1, n, dtype=np.uint64).astype(np.uint32)
    out = {"wi": wi, "wo": wo, "seeds": seeds}
    for k, (pd, ps, ax, ay) in enumerate(ggx_materials()):
        r = rx.ggx(pd, ps, ax, ay, wi, wo, seeds)
        for key, val in r.items():
            out[f"m{k}_{key}"] = val
    np.savez_compressed(os.path.join(HERE, "optix_ggx.npz"), **out)
    print("optix_ggx: specular samples above the horizon",
          int(sum((out[f"m{k}_wo"][:, 2] > 0).sum() for k in range(4))))


def env_fixture_scenes():
    """Two env scenes: a smooth sky (wide, dim sun) and the default sky with
    a 6-degree sun of peak 200, each with one area light beside the envmap."""
    return {
        "smooth": scenes.env_spheres(width=32, height=24, env_width=32, env_height=16, sun_radius_deg=25.0,
                                     sun_peak=20.0),
        "sun": scenes.env_spheres(width=32, height=24, env_width=64, env_height=32),
    }


def write_env_fixture(rx, n=1024):
    rng = np.random.default_rng(23)
    out = {}
    for name, sc in env_fixture_scenes().items():
        env_idx = [i for i, l in enumerate(sc.lights) if l.type == abi.DL_LIGHT_ENVMAP][0]
        L = sc.lights[env_idx]
        rgb = L.env_rgb
        rq, ralias, rpdf = rx.env_tables(rgb)
        orc = po.OracleScene(sc)
        q, alias, pdf = orc.env_tables()
        rx.reset_textures()
        tex = rx.texture(rgb)
        rx.env_set(tex, q, alias, pdf, scale=L.env_scale, visual=L.env_visual)
        seeds = rng.integers(1, 2**32 - 1, n, dtype=np.uint64).astype(np.uint32)
        nrm = unit(rng, n)
        p = np.zeros((n, 3), np.float32)
        dirs = unit(rng, n)
        rx.set_quantised_weights(False)
        smp = rx.env_sample(p, nrm, seeds)
        qry = rx.env_query(dirs)
        rx.set_quantised_weights(True)
        smp_q = rx.env_sample(p, nrm, seeds)
        qry_q = rx.env_query(dirs)
        rx.set_quantised_weights(False)
        depth = rng.integers(0, 3, n).astype(np.int32)
        bpdf = rng.uniform(0.01, 5.0, n).astype(np.float32)
        diffuse = rng.integers(0, 2, n).astype(np.uint8)
        miss = rx.env_miss(dirs, depth, bpdf, diffuse, len(sc.lights), env_idx, L.env_background)
        rx.env_set(tex, q, alias, pdf, scale=L.env_scale, visual=0)
        miss_bg = rx.env_miss(dirs, np.zeros(n, np.int32), bpdf, diffuse, len(sc.lights), env_idx,
                              L.env_background)
        out.update({f"{name}_ref_q": rq, f"{name}_ref_alias": ralias, f"{name}_ref_pdf": rpdf,
                    f"{name}_q": q, f"{name}_alias": alias, f"{name}_pdf": pdf,
                    f"{name}_seeds": seeds, f"{name}_nrm": nrm, f"{name}_dirs": dirs,
                    f"{name}_xi": smp["xi"], f"{name}_s_dir": smp["s_dir"], f"{name}_s_pdf": smp["s_pdf"],
                    f"{name}_s_value": smp["s_value"], f"{name}_s_value_hw": smp_q["s_value"],
                    f"{name}_pdf_d": qry["pdf"], f"{name}_value": qry["value"], f"{name}_value_hw": qry_q["value"],
                    f"{name}_uv": qry["uv"], f"{name}_depth": depth, f"{name}_bsdf_pdf": bpdf,
                    f"{name}_diffuse": diffuse, f"{name}_miss": miss, f"{name}_miss_bg": miss_bg})
    np.savez_compressed(os.path.join(HERE, "optix_env.npz"), **out)
    print("optix_env written")


def opencv_camera(width=64, height=48):
    """World-to-camera extrinsic of a camera at (0.4, 0.3, 3.5) looking at
    the origin (x right, y down, z forward) and intrinsics."""
    c2w = scenes.look_at((0.4, 0.3, 3.5), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    c2w[:3, 0] *= -1.0   # x to the right
    c2w[:3, 1] *= -1.0   # y down
    ext = np.linalg.inv(c2w)
    return dict(extrinsic=ext, fx=70.0, fy=72.0, cx=width / 2 + 0.3, cy=height / 2 - 0.6, width=width,
                height=height)


def write_camera_optix_fixture(rx, n=1024):
    rng = np.random.default_rng(25)
    c = opencv_camera()
    inv, eye = rx.opencv_setup(c["extrinsic"], c["fx"], c["fy"], c["cx"], c["cy"])
    px = rng.integers(0, c["width"], n).astype(np.int32)
    py = rng.integers(0, c["height"], n).astype(np.int32)
    seeds = rng.integers(1, 2**32 - 1, n, dtype=np.uint64).astype(np.uint32)
    xi, o, d = rx.opencv_ray(inv, eye, c["fx"], c["fy"], c["cx"], c["cy"], px, py, np.zeros(n, np.int32), 1,
                             seeds)
    np.savez_compressed(os.path.join(HERE, "optix_camera.npz"), extrinsic=c["extrinsic"], inv_ext=inv, eye=eye,
                        px=px, py=py, seeds=seeds, xi=xi, o=o, d=d,
                        intrinsics=np.array([c["fx"], c["fy"], c["cx"], c["cy"]], np.float32),
                        size=np.array([c["width"], c["height"]], np.int32))
    print("optix_camera written")


def hit_fixture_scene(seed=27):
    """A textured grid (perturbed vertex normals, texture coordinates over
    [-0.7, 1.9] to exercise wrap addressing) with world-space normal and
    tangent maps on an aniso_ggx material, and an untextured grid without
    normals on a diffuse one."""
    rng = np.random.default_rng(seed)
    s = scenes.SceneData("hit_data", spp=1)
    nmap = rng.uniform(0.0, 1.0, (8, 8, 3)).astype(np.float32)
    nmap[..., 2] = rng.uniform(0.6, 1.0, (8, 8))
    tmap = rng.uniform(0.0, 1.0, (8, 8, 3)).astype(np.float32)
    mt = s.add_material(scenes.Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0.2, 0.2, 0.2),
                                        specular=(0.8, 0.8, 0.8), alpha=(0.1, 0.2), normal_texture=nmap,
                                        tangent_texture=tmap))
    md = s.add_material(scenes.Material(type=abi.DL_MAT_DIFFUSE, albedo=(0.5, 0.5, 0.5)))
    k = 5
    gx, gz = np.meshgrid(np.linspace(-1, 1, k), np.linspace(-1, 1, k))
    pos = np.stack([gx.ravel(), 0.1 * np.sin(3 * gx.ravel()) * np.cos(2 * gz.ravel()), gz.ravel()], 1)
    idx = []
    for i in range(k - 1):
        for j in range(k - 1):
            a = i * k + j
            idx += [(a, a + 1, a + k + 1), (a, a + k + 1, a + k)]
    idx = np.array(idx, np.uint32)
    nrm = np.tile([0.0, 1.0, 0.0], (k * k, 1)) + rng.normal(scale=0.2, size=(k * k, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    uv = np.stack([-0.7 + 2.6 * (gx.ravel() + 1) / 2, 1.9 - 2.6 * (gz.ravel() + 1) / 2], 1)
    s.add_mesh(scenes.Mesh(pos.astype(np.float32), idx, nrm.astype(np.float32), uv.astype(np.float32),
                           material=mt))
    s.add_mesh(scenes.Mesh((pos + [0.0, 1.0, 0.0]).astype(np.float32), idx, None, None, material=md))
    s.camera = scenes.Camera(width=16, height=16, eye=(0, 3, 3), lookat=(0, 0, 0))
    return s, nmap, tmap


def write_hit_fixture(rx, n=1024):
    rng = np.random.default_rng(29)
    sc, nmap, tmap = hit_fixture_scene()
    rx.reset_textures()
    ntex, ttex = rx.texture(nmap), rx.texture(tmap)
    out = {}
    for mi, (m, texs) in enumerate(zip(sc.meshes, [(ntex, ttex), (0, 0)])):
        f = m.indices.shape[0]
        prim = rng.integers(0, f, n).astype(np.int32)
        b = rng.uniform(0, 1, (n, 2)).astype(np.float32)
        flip = b.sum(1) > 1
        b[flip] = 1 - b[flip]
        z3 = np.zeros((n, 3), np.float32)
        r = rx.hit_data(m.positions, m.indices.astype(np.int32), m.normals, None, m.texcoords, texs[0], texs[1],
                        prim, b, z3, z3, np.ones(n, np.float32))
        offset = sum(mm.indices.shape[0] for mm in sc.meshes[:mi])
        out.update({f"mesh{mi}_prim": prim + offset, f"mesh{mi}_bary": b, f"mesh{mi}_sn": r["sn"],
                    f"mesh{mi}_gn": r["gn"], f"mesh{mi}_st": r["st"], f"mesh{mi}_uv": r["uv"]})
    np.savez_compressed(os.path.join(HERE, "optix_hit.npz"), **out)
    print("optix_hit written")


HISPP = 4096


def write_hispp_fixture():
    sc = scenes.cornell(width=64, height=64, spp=HISPP, max_depth=0)
    ref = po.RefScene(sc, spp=HISPP)
    rgb, sec = ref.render_blocks(threads=os.cpu_count())
    np.savez_compressed(os.path.join(HERE, "cornell_hispp.npz"), rgb=rgb, spp=np.int32(HISPP))
    print("cornell_hispp: %.1f s, mean %.5f" % (sec, rgb.mean()))


def write_optix_fixtures():
    import pyref_optix as rx
    if rx.lib() is None:
        raise SystemExit("reference OptiX harness unavailable")
    write_ggx_fixture(rx)
    write_env_fixture(rx)
    write_camera_optix_fixture(rx)
    write_hit_fixture(rx)


def main():
    if po.ref_lib() is None:
        raise SystemExit("reference harness unavailable (needs the reference sources)")
    if "--only" in sys.argv and "cameras" in sys.argv:
        write_camera_fixtures()
        return
    if "--only" in sys.argv and "optix" in sys.argv:
        write_optix_fixtures()
        return
    if "--only" in sys.argv and "hispp" in sys.argv:
        write_hispp_fixture()
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
    write_optix_fixtures()
    write_hispp_fixture()


if __name__ == "__main__":
    main()
