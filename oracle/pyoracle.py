"""ctypes wrappers of the oracle (``liboracle.so``, the CPU restatement) and
of the reference harness (``libdlref.so``, the reference's own CPU code).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

from drawlab_gb300 import abi  # noqa: E402

_fp = C.POINTER(C.c_float)


def _f(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _load(path: Path) -> C.CDLL:
    return C.CDLL(str(path))


_oracle_lib = None
_ref_lib = None


def oracle_lib() -> C.CDLL:
    global _oracle_lib
    if _oracle_lib is None:
        sys.path.insert(0, str(HERE))
        import build as _b  # oracle/build.py
        path = _b.build_oracle()
        lib = _load(path)
        lib.orc_scene_create.restype = C.c_void_p
        lib.orc_last_error.restype = C.c_char_p
        _oracle_lib = lib
    return _oracle_lib


def ref_available() -> bool:
    sys.path.insert(0, str(HERE))
    import build as _b
    return _b.reference_root() is not None or (HERE / "_ref" / "libdlref.so").exists()


def ref_lib() -> C.CDLL | None:
    global _ref_lib
    if _ref_lib is None:
        sys.path.insert(0, str(HERE))
        import build as _b
        path = _b.build_ref()
        if path is None:
            p = HERE / "_ref" / "libdlref.so"
            if not p.exists():
                return None
            path = p
        lib = _load(path)
        lib.ref_scene_create.restype = C.c_void_p
        lib.ref_last_error.restype = C.c_char_p
        _ref_lib = lib
    return _ref_lib


def _threads(t):
    return int(t if t else (os.cpu_count() or 1))


class OracleScene:
    """The CPU restatement bound to one scene."""

    def __init__(self, scene, filter: int = abi.DL_FILTER_GAUSSIAN):
        self.lib = oracle_lib()
        self.scene = scene
        keep, md, nm, mat, nmat, ld, nl, cam = scene.descs()
        self._keep = keep
        h = self.lib.orc_scene_create(md, nm, mat, nmat, ld, nl, C.byref(cam), filter)
        if not h:
            raise RuntimeError("oracle scene: %s" % self.lib.orc_last_error().decode())
        self.h = C.c_void_p(h)
        self.width, self.height = scene.camera.width, scene.camera.height
        self.border = 2 if filter == abi.DL_FILTER_GAUSSIAN else 0

    def __del__(self):
        try:
            self.lib.orc_scene_destroy(self.h)
        except Exception:
            pass

    def trace_closest(self, rays: np.ndarray, threads=None):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float32) for _ in range(3))
        self.lib.orc_trace_closest(self.h, _f(rays), C.c_int64(n), _f(prim), _f(t), _f(u), _f(v),
                                   _threads(threads))
        return prim, t, u, v

    def trace_any(self, rays: np.ndarray, threads=None):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        occ = np.empty(n, np.uint8)
        self.lib.orc_trace_any(self.h, _f(rays), C.c_int64(n), _f(occ), _threads(threads))
        return occ

    def render_blocks(self, opts, threads=None, max_blocks=0, film=False):
        rgb = np.zeros((self.height, self.width, 3), np.float32)
        fb = np.zeros((self.height + 2 * self.border, self.width + 2 * self.border, 4), np.float32)
        sec = C.c_double()
        self.lib.orc_render_blocks(self.h, C.byref(opts), _threads(threads), max_blocks, _f(rgb),
                                   _f(fb), C.byref(sec))
        return (rgb, fb, sec.value) if film else (rgb, sec.value)

    def num_blocks(self) -> int:
        return int(self.lib.orc_num_blocks(self.h))

    def render_block_subset(self, opts, blocks, threads=None, film=False):
        """The block renderer over the listed blocks (positions in the
        spiral order); returns (rgb[, film], seconds)."""
        idx = np.ascontiguousarray(blocks, np.int32)
        rgb = np.zeros((self.height, self.width, 3), np.float32)
        fb = np.zeros((self.height + 2 * self.border, self.width + 2 * self.border, 4), np.float32)
        sec = C.c_double()
        if self.lib.orc_render_block_subset(self.h, C.byref(opts), _threads(threads), len(idx), _f(idx),
                                            _f(rgb), _f(fb), C.byref(sec)) != 0:
            raise ValueError("block index out of range")
        return (rgb, fb, sec.value) if film else (rgb, sec.value)

    def render_paths(self, opts, threads=None, film=False):
        rgb = np.zeros((self.height, self.width, 3), np.float32)
        fb = np.zeros((self.height + 2 * self.border, self.width + 2 * self.border, 4), np.float32)
        sec = C.c_double()
        self.lib.orc_render_paths(self.h, C.byref(opts), _threads(threads), _f(rgb), _f(fb),
                                  C.byref(sec))
        return (rgb, fb, sec.value) if film else (rgb, sec.value)

    def li(self, opts, xys: np.ndarray, threads=None):
        xys = np.ascontiguousarray(xys, np.int32)
        n = xys.shape[0]
        L = np.empty((n, 3), np.float32)
        pos = np.empty((n, 2), np.float32)
        self.lib.orc_li(self.h, C.byref(opts), C.c_int64(n), _f(xys), _f(L), _f(pos),
                        _threads(threads))
        return L, pos

    def emitter_sample(self, opts, pts, nrm, smp):
        n = pts.shape[0]
        pts, nrm, smp = (np.ascontiguousarray(a, np.float32) for a in (pts, nrm, smp))
        d = np.empty((n, 3), np.float32)
        dist = np.empty(n, np.float32)
        pdf = np.empty(n, np.float32)
        spec = np.empty((n, 3), np.float32)
        self.lib.orc_emitter_sample(self.h, C.byref(opts), C.c_int64(n), _f(pts), _f(nrm),
                                    _f(smp), _f(d), _f(dist), _f(pdf), _f(spec))
        return d, dist, pdf, spec

    def env_tables(self):
        """(q, alias, pdf) of the envmap, each (env_height, env_width)."""
        env = [x for x in self.scene.lights if x.type == abi.DL_LIGHT_ENVMAP]
        if not env:
            raise ValueError("scene has no envmap")
        h, w = env[0].env_rgb.shape[:2]
        q = np.empty((h, w), np.float32)
        alias = np.empty((h, w), np.uint32)
        pdf = np.empty((h, w), np.float32)
        if self.lib.orc_env_tables(self.h, _f(q), _f(alias), _f(pdf)) != 0:
            raise RuntimeError("oracle has no envmap tables")
        return q, alias, pdf

    def env_query(self, xi, nrm, dirs):
        """Envmap sampleDirection(xi, normal) -> s_dir, s_pdf, s_value and
        pdfDirection / eval of dirs -> pdf, value."""
        xi, nrm, dirs = (np.ascontiguousarray(a, np.float32) for a in (xi, nrm, dirs))
        n = xi.shape[0]
        out = dict(s_dir=np.empty((n, 3), np.float32), s_pdf=np.empty(n, np.float32),
                   s_value=np.empty((n, 3), np.float32), pdf=np.empty(n, np.float32),
                   value=np.empty((n, 3), np.float32))
        if self.lib.orc_env_query(self.h, C.c_int64(n), _f(xi), _f(nrm), _f(dirs), _f(out["s_dir"]),
                                  _f(out["s_pdf"]), _f(out["s_value"]), _f(out["pdf"]), _f(out["value"])) != 0:
            raise RuntimeError("scene has no envmap")
        return out

    def env_miss(self, opts, dirs, depth, bsdf_pdf, is_diffuse):
        """Radiance of rays that leave the scene along dirs (miss.cu)."""
        dirs = np.ascontiguousarray(dirs, np.float32)
        depth = np.ascontiguousarray(depth, np.int32)
        bsdf_pdf = np.ascontiguousarray(bsdf_pdf, np.float32)
        is_diffuse = np.ascontiguousarray(is_diffuse, np.uint8)
        n = dirs.shape[0]
        out = np.empty((n, 3), np.float32)
        if self.lib.orc_env_miss(self.h, C.byref(opts), C.c_int64(n), _f(dirs), _f(depth), _f(bsdf_pdf),
                                 _f(is_diffuse), _f(out)) != 0:
            raise RuntimeError("scene has no envmap")
        return out

    def camera_ray(self, film):
        film = np.ascontiguousarray(film, np.float32)
        n = film.shape[0]
        o = np.empty((n, 3), np.float32)
        d = np.empty((n, 3), np.float32)
        self.lib.orc_camera_ray(self.h, C.c_int64(n), _f(film), _f(o), _f(d))
        return o, d

    def hit_data(self, prim, bary):
        """(shading normal, geometric normal, shading tangent, texcoords) of
        global triangles prim at barycentrics bary."""
        prim = np.ascontiguousarray(prim, np.int32)
        bary = np.ascontiguousarray(bary, np.float32)
        n = prim.shape[0]
        sn, gn, st = (np.empty((n, 3), np.float32) for _ in range(3))
        tuv = np.empty((n, 2), np.float32)
        if self.lib.orc_hit_data(self.h, C.c_int64(n), _f(prim), _f(bary), _f(sn), _f(gn), _f(st), _f(tuv)) != 0:
            raise RuntimeError("bad triangle index")
        return sn, gn, st, tuv


class RefScene:
    """The reference's own CPU code bound to one scene (x86 container only)."""

    def __init__(self, scene, filter: int = abi.DL_FILTER_GAUSSIAN, spp: int = 1, normals: bool = False):
        self.lib = ref_lib()
        if self.lib is None:
            raise RuntimeError("reference harness unavailable")
        self.scene = scene
        keep, md, nm, mat, nmat, ld, nl, cam = scene.descs()
        self._keep = keep
        h = self.lib.ref_scene_create(md, nm, mat, nmat, ld, nl, C.byref(cam), filter, spp, int(normals))
        if not h:
            raise RuntimeError("reference scene: %s" % self.lib.ref_last_error().decode())
        self.h = C.c_void_p(h)
        self.width, self.height = scene.camera.width, scene.camera.height
        self.border = 2 if filter == abi.DL_FILTER_GAUSSIAN else 0

    def trace_closest(self, rays, threads=None):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float32) for _ in range(3))
        self.lib.ref_trace_closest(self.h, _f(rays), C.c_int64(n), _f(prim), _f(t), _f(u), _f(v),
                                   _threads(threads))
        return prim, t, u, v

    def trace_any(self, rays, threads=None):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        occ = np.empty(n, np.uint8)
        self.lib.ref_trace_any(self.h, _f(rays), C.c_int64(n), _f(occ), _threads(threads))
        return occ

    def render_blocks(self, threads=None, max_blocks=0, film=False):
        rgb = np.zeros((self.height, self.width, 3), np.float32)
        fb = np.zeros((self.height + 2 * self.border, self.width + 2 * self.border, 4), np.float32)
        sec = C.c_double()
        self.lib.ref_render_blocks(self.h, _threads(threads), max_blocks, _f(rgb), _f(fb),
                                   C.byref(sec))
        return (rgb, fb, sec.value) if film else (rgb, sec.value)

    def li(self, seed: int, xys, threads=None):
        xys = np.ascontiguousarray(xys, np.int32)
        n = xys.shape[0]
        L = np.empty((n, 3), np.float32)
        pos = np.empty((n, 2), np.float32)
        self.lib.ref_li(self.h, C.c_uint64(seed), C.c_int64(n), _f(xys), _f(L), _f(pos),
                        _threads(threads))
        return L, pos

    def emitter_sample(self, pts, nrm, smp):
        n = pts.shape[0]
        pts, nrm, smp = (np.ascontiguousarray(a, np.float32) for a in (pts, nrm, smp))
        d = np.empty((n, 3), np.float32)
        dist = np.empty(n, np.float32)
        pdf = np.empty(n, np.float32)
        spec = np.empty((n, 3), np.float32)
        self.lib.ref_emitter_sample(self.h, C.c_int64(n), _f(pts), _f(nrm), _f(smp), _f(d),
                                    _f(dist), _f(pdf), _f(spec))
        return d, dist, pdf, spec


def bsdf_query(lib_kind: str, mat, wi, wo, smp):
    """BSDF eval/pdf/sample through the oracle ("oracle") or the reference's
    CPU BSDFs ("ref").  smp: n x 2 (the 2D sample) or n x 3 (then the lobe
    coin that only aniso_ggx draws; the reference's CPU BSDFs take the
    first two)."""
    wi, wo, smp = (np.ascontiguousarray(a, np.float32) for a in (wi, wo, smp))
    n = wi.shape[0]
    if lib_kind == "oracle" and smp.shape[1] == 2:
        smp = np.ascontiguousarray(np.concatenate([smp, np.zeros((n, 1), np.float32)], axis=1))
    elif lib_kind != "oracle" and smp.shape[1] == 3:
        smp = np.ascontiguousarray(smp[:, :2])
    out = dict(eval=np.empty((n, 3), np.float32), pdf=np.empty(n, np.float32),
               wo=np.empty((n, 3), np.float32), weight=np.empty((n, 3), np.float32),
               eta=np.empty(n, np.float32), measure=np.empty(n, np.int32))
    md = abi.dl_material_desc()
    md.type = mat.type
    md.albedo[:] = [float(v) for v in mat.albedo]
    md.specular[:] = [float(v) for v in mat.specular]
    md.alpha[:] = [float(v) for v in mat.alpha]
    md.int_ior = mat.int_ior
    md.ext_ior = mat.ext_ior
    lib = oracle_lib() if lib_kind == "oracle" else ref_lib()
    fn = lib.orc_bsdf_query if lib_kind == "oracle" else lib.ref_bsdf_query
    fn(C.byref(md), C.c_int64(n), _f(wi), _f(wo), _f(smp), _f(out["eval"]), _f(out["pdf"]),
       _f(out["wo"]), _f(out["weight"]), _f(out["eta"]), _f(out["measure"]))
    return out


def frame(lib_kind: str, nrm):
    nrm = np.ascontiguousarray(nrm, np.float32)
    n = nrm.shape[0]
    t = np.empty((n, 3), np.float32)
    b = np.empty((n, 3), np.float32)
    if lib_kind == "oracle":
        oracle_lib().orc_frame(C.c_int64(n), _f(nrm), _f(t), _f(b))
    else:
        ref_lib().ref_frame(C.c_int64(n), _f(nrm), _f(t), _f(b))
    return t, b
