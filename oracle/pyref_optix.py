"""ctypes wrapper of the reference's OptiX-only code compiled as host C++
(``oracle/_ref/libdlref_optix.so``, built by oracle/build.py from
oracle/ref_optix.cpp) and of the host set-up functions of ``libdlref.so``
(oracle/ref_host_setup.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/golden/make_golden.py to record
golden vectors and by tests that compare against the reference live where
the reference tree is present.  Every function here runs the reference's own
code; see oracle/ref_optix.cpp for the file:line each one drives.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_lib = None

_u64 = C.c_ulonglong
_vp = C.c_void_p
_i64 = C.c_int64
_f32 = C.c_float
_i32 = C.c_int32


def _p(a):
    return a.ctypes.data_as(_vp) if a is not None else None


def lib() -> C.CDLL | None:
    """The OptiX-side harness, built on demand; None without the reference."""
    global _lib
    if _lib is None:
        sys.path.insert(0, str(HERE))
        import build as _b  # oracle/build.py
        if _b.build_ref() is None and not (HERE / "_ref" / "libdlref_optix.so").exists():
            return None
        L = C.CDLL(str(HERE / "_ref" / "libdlref_optix.so"))
        L.refx_texture_create.restype = _u64
        L.refx_texture_create.argtypes = [_i32, _i32, _vp]
        L.refx_texture_lookup.argtypes = [_u64, _i64, _vp, _vp]
        L.refx_set_quantised_weights.argtypes = [_i32]
        L.refx_ggx.argtypes = [_i64, _vp, _vp, _f32, _f32, _u64, _u64, _u64, _vp, _vp, _vp, _vp,
                               _vp, _vp, _vp, _vp, _vp]
        L.refx_square_to_ggx.argtypes = [_i64, _f32, _f32, _vp, _vp, _vp, _vp]
        L.refx_env_set.argtypes = [_i32, _i32, _u64, _vp, _vp, _vp, _f32, _i32]
        L.refx_env_sample.argtypes = [_i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
        L.refx_env_query.argtypes = [_i64, _vp, _vp, _vp, _vp]
        L.refx_env_miss.argtypes = [_i64, _vp, _vp, _vp, _vp, _i32, _i32, _vp, _vp]
        L.refx_opencv_ray.argtypes = [_vp, _vp, _f32, _f32, _f32, _f32, _i64, _vp, _vp, _vp, _i32, _vp,
                                      _vp, _vp, _vp]
        L.refx_hit_data.argtypes = [_vp, _vp, _vp, _vp, _vp, _u64, _u64, _i64, _vp, _vp, _vp, _vp, _vp,
                                    _vp, _vp, _vp, _vp, _vp]
        _lib = L
    return _lib


def _host():
    import pyoracle
    L = pyoracle.ref_lib()
    L.refx_env_tables.argtypes = [_i32, _i32, _vp, _vp, _vp, _vp]
    L.refx_opencv_setup.argtypes = [_vp, _f32, _f32, _f32, _f32, _vp, _vp]
    return L


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def texture(rgb: np.ndarray) -> int:
    """Register an (h, w, 3) image as a texture of the host model (row 0 =
    texture coordinate v in [0, 1/h)); returns its object id."""
    h, w = rgb.shape[:2]
    rgba = np.zeros((h, w, 4), np.float32)
    rgba[..., :3] = rgb
    return int(lib().refx_texture_create(w, h, _p(rgba)))


def reset_textures():
    lib().refx_texture_reset()


def set_quantised_weights(on: bool):
    lib().refx_set_quantised_weights(1 if on else 0)


def texture_lookup(tex: int, uv):
    uv = f32(uv)
    out = np.empty((uv.shape[0], 4), np.float32)
    lib().refx_texture_lookup(tex, uv.shape[0], _p(uv), _p(out))
    return out


def ggx(pd, ps, ax, ay, wi, wo, seeds, uv=None, textures=(0, 0, 0)):
    wi, wo = f32(wi), f32(wo)
    seeds = np.ascontiguousarray(seeds, np.uint32)
    n = wi.shape[0]
    out = dict(eval=np.empty((n, 3), np.float32), pdf=np.empty(n, np.float32), xi=np.empty((n, 3), np.float32),
               wo=np.empty((n, 3), np.float32), weight=np.empty((n, 3), np.float32))
    lib().refx_ggx(n, _p(f32(pd)), _p(f32(ps)), ax, ay, textures[0], textures[1], textures[2],
                   _p(f32(uv)) if uv is not None else None, _p(wi), _p(wo), _p(seeds), _p(out["eval"]),
                   _p(out["pdf"]), _p(out["xi"]), _p(out["wo"]), _p(out["weight"]))
    return out


def env_tables(rgb: np.ndarray):
    """EnvironmentMap::activate on an (h, w, 3) bitmap: q, alias, pdf (h, w)."""
    h, w = rgb.shape[:2]
    q = np.empty((h, w), np.float32)
    alias = np.empty((h, w), np.uint32)
    pdf = np.empty((h, w), np.float32)
    if _host().refx_env_tables(w, h, _p(f32(rgb)), _p(q), _p(alias), _p(pdf)) != 0:
        raise RuntimeError("reference envmap activation failed")
    return q, alias, pdf


def env_set(tex: int, q, alias, pdf, scale=1.0, visual=1):
    h, w = q.shape
    lib().refx_env_set(w, h, tex, _p(f32(q)), _p(np.ascontiguousarray(alias, np.uint32)), _p(f32(pdf)),
                       scale, visual)


def env_sample(p, sn, seeds):
    p, sn = f32(p), f32(sn)
    seeds = np.ascontiguousarray(seeds, np.uint32)
    n = p.shape[0]
    out = dict(xi=np.empty((n, 3), np.float32), s_dir=np.empty((n, 3), np.float32),
               s_pdf=np.empty(n, np.float32), s_value=np.empty((n, 3), np.float32))
    lib().refx_env_sample(n, _p(p), _p(sn), _p(seeds), _p(out["xi"]), _p(out["s_dir"]), _p(out["s_pdf"]),
                          _p(out["s_value"]))
    return out


def env_query(dirs):
    dirs = f32(dirs)
    n = dirs.shape[0]
    out = dict(pdf=np.empty(n, np.float32), value=np.empty((n, 3), np.float32), uv=np.empty((n, 2), np.float32))
    lib().refx_env_query(n, _p(dirs), _p(out["pdf"]), _p(out["value"]), _p(out["uv"]))
    return out


def env_miss(dirs, depth, bsdf_pdf, is_diffuse, num_lights, env_idx, bg):
    dirs = f32(dirs)
    n = dirs.shape[0]
    out = np.empty((n, 3), np.float32)
    lib().refx_env_miss(n, _p(dirs), _p(np.ascontiguousarray(depth, np.int32)), _p(f32(bsdf_pdf)),
                        _p(np.ascontiguousarray(is_diffuse, np.uint8)), num_lights, env_idx, _p(f32(bg)), _p(out))
    return out


def opencv_setup(extrinsic, fx, fy, cx, cy):
    inv = np.empty(16, np.float32)
    eye = np.empty(3, np.float32)
    if _host().refx_opencv_setup(_p(f32(np.asarray(extrinsic).reshape(16))), fx, fy, cx, cy, _p(inv), _p(eye)) != 0:
        raise RuntimeError("reference OpencvCamera set-up failed")
    return inv, eye


def opencv_ray(inv_ext, eye, fx, fy, cx, cy, px, py, s, spp, seeds):
    px, py, s = (np.ascontiguousarray(a, np.int32) for a in (px, py, s))
    seeds = np.ascontiguousarray(seeds, np.uint32)
    n = px.shape[0]
    xi = np.empty((n, 2), np.float32)
    o = np.empty((n, 3), np.float32)
    d = np.empty((n, 3), np.float32)
    lib().refx_opencv_ray(_p(f32(inv_ext)), _p(f32(eye)), cx, cy, fx, fy, n, _p(px), _p(py), _p(s), spp,
                          _p(seeds), _p(xi), _p(o), _p(d))
    return xi, o, d


def hit_data(positions, indices, normals, tangents, texcoords, normal_tex, tangent_tex, prim, bary, o, d, tmax):
    prim = np.ascontiguousarray(prim, np.int32)
    n = prim.shape[0]
    sn, gn, st, p = (np.empty((n, 3), np.float32) for _ in range(4))
    uv = np.empty((n, 2), np.float32)
    keep = [f32(positions), np.ascontiguousarray(indices, np.int32),
            f32(normals) if normals is not None else None, f32(tangents) if tangents is not None else None,
            f32(texcoords) if texcoords is not None else None]
    lib().refx_hit_data(_p(keep[0]), _p(keep[2]), _p(keep[3]), _p(keep[4]), _p(keep[1]), normal_tex, tangent_tex,
                        n, _p(prim), _p(f32(bary)), _p(f32(o)), _p(f32(d)), _p(f32(tmax)), _p(sn), _p(gn),
                        _p(st), _p(uv), _p(p))
    return dict(sn=sn, gn=gn, st=st, uv=uv, p=p)
