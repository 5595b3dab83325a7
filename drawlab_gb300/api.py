"""Python binding of the C ABI (include/drawlab.h) over ctypes.

The library is the in-tree ``drawlab_gb300/_build/libdlgpu.so`` built by
``drawlab_gb300.build``; there is no other code path: if the library is
missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import weakref
from pathlib import Path

import numpy as np

from . import abi
from .scenes import SceneData

# the in-tree library; DRAWLAB_GB300_LIBRARY selects another build of it (the
# bounds-checked variant of drawlab_gb300.build --checked)
_LIB_PATH = Path(os.environ.get("DRAWLAB_GB300_LIBRARY",
                                str(Path(__file__).resolve().parent / "_build" / "libdlgpu.so")))
_lib = None

# every entry point of include/drawlab.h: name -> (restype, argtypes)
_vp = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int32
SIGNATURES = {
    "dl_abi_version": (C.c_int, []),
    "dl_last_error": (C.c_char_p, [_vp]),
    "dl_context_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "dl_context_destroy": (C.c_int, [_vp]),
    "dl_scene_create_from_arrays": (C.c_int, [_vp, _vp, _i32, _vp, _i32, _vp, _i32, _vp, C.POINTER(_vp)]),
    "dl_scene_create_from_xml": (C.c_int, [_vp, C.c_char_p, C.POINTER(_vp)]),
    "dl_scene_destroy": (C.c_int, [_vp]),
    "dl_scene_get_info": (C.c_int, [_vp, _vp]),
    "dl_scene_default_opts": (C.c_int, [_vp, _vp]),
    "dl_trace_closest": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    "dl_trace_any": (C.c_int, [_vp, _vp, _i64, _vp]),
    "dl_trace_closest_device": (C.c_int, [_vp, _vp, _i64, _vp]),
    "dl_trace_any_device": (C.c_int, [_vp, _vp, _i64, _vp]),
    "dl_trace_closest_wavefront": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    "dl_trace_any_wavefront": (C.c_int, [_vp, _vp, _i64, _vp]),
    "dl_bsdf_query": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "dl_scene_env_query": (C.c_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "dl_measure_l2_read_bandwidth": (C.c_int, [_vp, _i64, _i32, _vp]),
    "dl_scene_emitter_sample": (C.c_int, [_vp, C.c_uint32, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "dl_render": (C.c_int, [_vp, _vp, _vp]),
    "dl_render_film": (C.c_int, [_vp, _vp, _vp]),
    "dl_render_film_device": (C.c_int, [_vp, _vp, _vp]),
    "dl_image_write": (C.c_int, [C.c_char_p, _i32, _i32, _vp, _i32]),
    "dl_image_read": (C.c_int, [C.c_char_p, _vp, _vp, _vp, _i64]),
    "dl_li": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "dl_stats_get": (C.c_int, [_vp, _vp]),
    "dl_render_traversal_counts": (C.c_int, [_vp, _vp, _vp]),
    "dl_context_set_kernel_timing": (C.c_int, [_vp, C.c_int]),
    "dl_li_static": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "dl_render_batch": (C.c_int, [_vp, _vp, _i32]),
    "dl_context_get_tune": (C.c_int, [_vp, _vp]),
    "dl_context_set_tune": (C.c_int, [_vp, _vp]),
    "dl_autotune": (C.c_int, [_vp, _vp, _i32, _i32, _vp, _vp]),
    "dl_guide_default_config": (C.c_int, [_vp]),
    "dl_guide_create": (C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    "dl_guide_destroy": (C.c_int, [_vp]),
    "dl_guide_get_params": (C.c_int, [_vp, _vp]),
    "dl_guide_set_params": (C.c_int, [_vp, _vp]),
    "dl_guide_forward": (C.c_int, [_vp, _i64, _vp, _vp]),
    "dl_guide_gradient": (C.c_int, [_vp, _i64, _vp, _vp, _vp]),
    "dl_guide_train": (C.c_int, [_vp, _i64, _vp, _i32, _vp]),
    "dl_render_guided": (C.c_int, [_vp, _vp, _vp, _i32, _vp]),
}


def write_image(path, rgb, fmt: int | None = None) -> None:
    """Write a (height, width, 3) float image (row 0 = top) as PNG, OpenEXR
    or PFM; the format follows the file extension unless `fmt` is given.
    Needs no GPU."""
    p = str(path)
    if fmt is None:
        ext = p.rsplit(".", 1)[-1].lower()
        fmt = {"png": abi.DL_IMAGE_PNG, "exr": abi.DL_IMAGE_EXR, "pfm": abi.DL_IMAGE_PFM}.get(ext)
        if fmt is None:
            raise ValueError("unknown image extension: %s" % p)
    a = np.ascontiguousarray(rgb, np.float32)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError("expected a (height, width, 3) image")
    L = lib()
    rc = L.dl_image_write(p.encode(), a.shape[1], a.shape[0], a.ctypes.data_as(C.c_void_p), fmt)
    if rc != abi.DL_OK:
        raise DrawlabError(rc, L.dl_last_error(None).decode())


def read_image(path) -> np.ndarray:
    """Read a PNG or PFM image as a (height, width, 3) float32 array (row 0 =
    top; PNG values are bytes / 255).  Needs no GPU."""
    L = lib()
    w, h = C.c_int32(), C.c_int32()
    p = str(path).encode()
    rc = L.dl_image_read(p, C.byref(w), C.byref(h), None, 0)
    if rc != abi.DL_OK:
        raise DrawlabError(rc, L.dl_last_error(None).decode())
    out = np.empty((h.value, w.value, 3), np.float32)
    rc = L.dl_image_read(p, C.byref(w), C.byref(h), out.ctypes.data_as(C.c_void_p), out.size)
    if rc != abi.DL_OK:
        raise DrawlabError(rc, L.dl_last_error(None).decode())
    return out


class DrawlabError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, str(status)), msg))
        self.status = status


def library_path() -> Path:
    return _LIB_PATH


def lib() -> C.CDLL:
    """Load libdlgpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError("libdlgpu.so is not built (run drawlab_gb300.build.build())")
        L = C.CDLL(str(_LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# Contexts still open at interpreter exit are closed (scenes first) before
# the CUDA runtime tears itself down.
_live_contexts = weakref.WeakSet()


@atexit.register
def _close_all():
    for c in list(_live_contexts):
        try:
            c.close()
        except Exception:
            pass


class Context:
    """A device context: one CUDA stream, device memory owned by the library."""

    def __init__(self, device: int = 0):
        self.lib = lib()
        h = C.c_void_p()
        rc = self.lib.dl_context_create(device, C.byref(h))
        if rc != abi.DL_OK:
            raise DrawlabError(rc, self.lib.dl_last_error(None).decode())
        self.h = h
        # scenes must be destroyed before their context: keep track of them
        self._scenes = weakref.WeakSet()
        _live_contexts.add(self)

    def check(self, rc: int):
        if rc != abi.DL_OK:
            raise DrawlabError(rc, self.lib.dl_last_error(self.h).decode())

    def set_kernel_timing(self, enabled: bool):
        self.check(self.lib.dl_context_set_kernel_timing(self.h, 1 if enabled else 0))

    def stats(self) -> abi.dl_stats:
        s = abi.dl_stats()
        self.check(self.lib.dl_stats_get(self.h, C.byref(s)))
        return s

    def l2_read_gbs(self, bytes_: int = 64 << 20, passes: int = 40) -> float:
        """L2 -> SM read bandwidth (GB/s) measured by the library's probe."""
        out = C.c_double()
        self.check(self.lib.dl_measure_l2_read_bandwidth(self.h, bytes_, passes, C.byref(out)))
        return out.value

    def bsdf_query(self, mat, wi, wo, smp):
        """BSDF eval / pdf of (wi, wo) and sample(wi) from smp (n x 3) of one
        material (a scenes.Material), computed on the GPU; the same keys as
        the oracle's bsdf_query."""
        wi, wo, smp = (np.ascontiguousarray(a, np.float32) for a in (wi, wo, smp))
        n = wi.shape[0]
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
        self.check(self.lib.dl_bsdf_query(self.h, C.byref(md), n, _ptr(wi), _ptr(wo), _ptr(smp),
                                          _ptr(out["eval"]), _ptr(out["pdf"]), _ptr(out["wo"]),
                                          _ptr(out["weight"]), _ptr(out["eta"]), _ptr(out["measure"])))
        return out

    @staticmethod
    def _requests(items):
        """items: (Scene, opts) or (Scene, opts, Camera override)."""
        reqs = (abi.dl_request * max(len(items), 1))()
        outs, keep = [], []
        for i, it in enumerate(items):
            scene, opts = it[0], it[1]
            cam = it[2] if len(it) > 2 else None
            w, h = (cam.width, cam.height) if cam is not None else (scene.width, scene.height)
            rgb = np.empty((h, w, 3), np.float32)
            outs.append(rgb)
            reqs[i].scene = scene.h
            reqs[i].opts = opts
            reqs[i].rgb = rgb.ctypes.data_as(C.POINTER(C.c_float))
            reqs[i].film_device = None
            if cam is not None:
                cd = cam.desc()
                keep.append(cd)
                reqs[i].camera = C.cast(C.byref(cd), C.c_void_p)
            else:
                reqs[i].camera = None
        reqs._keep = keep
        return reqs, outs

    def render_batch(self, items) -> list:
        """Render [(Scene, dl_render_opts), ...] in one wavefront; returns the
        RGB images in order."""
        reqs, outs = self._requests(items)
        self.check(self.lib.dl_render_batch(self.h, C.cast(reqs, C.c_void_p), len(items)))
        return outs

    def get_tune(self) -> abi.dl_tune_params:
        t = abi.dl_tune_params()
        self.check(self.lib.dl_context_get_tune(self.h, C.byref(t)))
        return t

    def set_tune(self, t: abi.dl_tune_params):
        self.check(self.lib.dl_context_set_tune(self.h, C.byref(t)))

    def autotune(self, items, trial_spp: int = 0):
        """Time launch shapes on [(Scene, opts), ...]; keeps and returns the
        fastest (dl_tune_params) and the number of shapes timed."""
        reqs, _ = self._requests(items)
        t = abi.dl_tune_params()
        n = C.c_int32()
        self.check(self.lib.dl_autotune(self.h, C.cast(reqs, C.c_void_p), len(items), trial_spp, C.byref(t),
                                        C.byref(n)))
        return t, n.value

    def close(self):
        if getattr(self, "h", None):
            for s in list(getattr(self, "_scenes", ())):
                s.close()
            self.lib.dl_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """A scene resident on the device (geometry, BVH, materials, lights)."""

    def __init__(self, ctx: Context, handle: C.c_void_p, data: SceneData | None = None):
        self.ctx = ctx
        self.h = handle
        self.data = data
        ctx._scenes.add(self)
        info = self.info()
        self.width, self.height = info.width, info.height

    @classmethod
    def from_data(cls, ctx: Context, data: SceneData) -> "Scene":
        keep, md, nm, mat, nmat, ld, nl, cam = data.descs()
        h = C.c_void_p()
        ctx.check(ctx.lib.dl_scene_create_from_arrays(ctx.h, C.cast(md, C.c_void_p), nm, C.cast(mat, C.c_void_p),
                                                      nmat, C.cast(ld, C.c_void_p), nl, C.byref(cam), C.byref(h)))
        del keep
        return cls(ctx, h, data)

    @classmethod
    def from_xml(cls, ctx: Context, path: str) -> "Scene":
        h = C.c_void_p()
        ctx.check(ctx.lib.dl_scene_create_from_xml(ctx.h, str(path).encode(), C.byref(h)))
        return cls(ctx, h)

    def info(self) -> abi.dl_scene_info:
        i = abi.dl_scene_info()
        self.ctx.check(self.ctx.lib.dl_scene_get_info(self.h, C.byref(i)))
        return i

    def default_opts(self) -> abi.dl_render_opts:
        o = abi.dl_render_opts()
        self.ctx.check(self.ctx.lib.dl_scene_default_opts(self.h, C.byref(o)))
        return o

    def trace_closest(self, rays: np.ndarray, wavefront: bool = False):
        """Closest hits (prim, t, u, v).  wavefront=True traces them with the
        renderer's own traversal kernel (every tmin must be 1e-4)."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float32) for _ in range(3))
        fn = self.ctx.lib.dl_trace_closest_wavefront if wavefront else self.ctx.lib.dl_trace_closest
        self.ctx.check(fn(self.h, _ptr(rays), n, _ptr(prim), _ptr(t), _ptr(u), _ptr(v)))
        return prim, t, u, v

    def trace_any(self, rays: np.ndarray, wavefront: bool = False):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        occ = np.empty(n, np.uint8)
        fn = self.ctx.lib.dl_trace_any_wavefront if wavefront else self.ctx.lib.dl_trace_any
        self.ctx.check(fn(self.h, _ptr(rays), n, _ptr(occ)))
        return occ

    def emitter_sample(self, opts, pts, nrm, smp):
        """Scene::sampleEmitterDirection without visibility on the GPU:
        (d, dist, pdf, spec, light)."""
        pts, nrm, smp = (np.ascontiguousarray(a, np.float32) for a in (pts, nrm, smp))
        n = pts.shape[0]
        d = np.empty((n, 3), np.float32)
        dist = np.empty(n, np.float32)
        pdf = np.empty(n, np.float32)
        spec = np.empty((n, 3), np.float32)
        light = np.empty(n, np.int32)
        self.ctx.check(self.ctx.lib.dl_scene_emitter_sample(self.h, opts.flags, n, _ptr(pts), _ptr(nrm), _ptr(smp),
                                                            _ptr(d), _ptr(dist), _ptr(pdf), _ptr(spec),
                                                            _ptr(light)))
        return d, dist, pdf, spec, light

    def env_query(self, xi, nrm, dirs):
        """The envmap's sampleDirection(xi, normal) -> (dir, pdf, value) and
        pdfDirection / eval of dirs, computed on the GPU."""
        xi, nrm, dirs = (np.ascontiguousarray(a, np.float32) for a in (xi, nrm, dirs))
        n = xi.shape[0]
        out = dict(s_dir=np.empty((n, 3), np.float32), s_pdf=np.empty(n, np.float32),
                   s_value=np.empty((n, 3), np.float32), pdf=np.empty(n, np.float32),
                   value=np.empty((n, 3), np.float32))
        self.ctx.check(self.ctx.lib.dl_scene_env_query(
            self.h, n, _ptr(xi), _ptr(nrm), _ptr(dirs), _ptr(out["s_dir"]), _ptr(out["s_pdf"]),
            _ptr(out["s_value"]), _ptr(out["pdf"]), _ptr(out["value"])))
        return out

    def render(self, opts: abi.dl_render_opts) -> np.ndarray:
        rgb = np.empty((self.height, self.width, 3), np.float32)
        self.ctx.check(self.ctx.lib.dl_render(self.h, C.byref(opts), _ptr(rgb)))
        return rgb

    def render_film(self, opts: abi.dl_render_opts) -> np.ndarray:
        b = 0 if opts.filter == abi.DL_FILTER_BOX else 2
        film = np.empty((self.height + 2 * b, self.width + 2 * b, 4), np.float32)
        self.ctx.check(self.ctx.lib.dl_render_film(self.h, C.byref(opts), _ptr(film)))
        return film

    def render_guided(self, opts: abi.dl_render_opts, guide, train: bool = True) -> np.ndarray:
        rgb = np.empty((self.height, self.width, 3), np.float32)
        self.ctx.check(self.ctx.lib.dl_render_guided(self.h, C.byref(opts), guide.h, 1 if train else 0, _ptr(rgb)))
        return rgb

    def li(self, opts: abi.dl_render_opts, xys: np.ndarray):
        xys = np.ascontiguousarray(xys, np.int32)
        n = xys.shape[0]
        L = np.empty((n, 3), np.float32)
        pos = np.empty((n, 2), np.float32)
        self.ctx.check(self.ctx.lib.dl_li(self.h, C.byref(opts), n, _ptr(xys), _ptr(L), _ptr(pos)))
        return L, pos

    def traversal_counts(self, opts: abi.dl_render_opts) -> abi.dl_traversal_counts:
        c = abi.dl_traversal_counts()
        self.ctx.check(self.ctx.lib.dl_render_traversal_counts(self.h, C.byref(opts), C.byref(c)))
        return c

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):   # the context still exists
                self.ctx.lib.dl_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Guide:
    """The learned guiding proposal (network parameters and Adam state on
    the device)."""

    def __init__(self, ctx: Context, **cfg):
        self.ctx = ctx
        c = abi.dl_guide_config()
        ctx.check(ctx.lib.dl_guide_default_config(C.byref(c)))
        for k, v in cfg.items():
            setattr(c, k, v)
        h = C.c_void_p()
        ctx.check(ctx.lib.dl_guide_create(ctx.h, C.byref(c), C.byref(h)))
        self.h = h
        self.config = c
        ctx._scenes.add(self)

    def params(self) -> np.ndarray:
        p = np.empty(abi.DL_GUIDE_PARAMS, np.float32)
        self.ctx.check(self.ctx.lib.dl_guide_get_params(self.h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape == (abi.DL_GUIDE_PARAMS,)
        self.ctx.check(self.ctx.lib.dl_guide_set_params(self.h, _ptr(p)))

    def forward(self, inputs) -> np.ndarray:
        x = np.ascontiguousarray(inputs, np.float32)
        out = np.empty((x.shape[0], 40), np.float32)
        self.ctx.check(self.ctx.lib.dl_guide_forward(self.h, x.shape[0], _ptr(x), _ptr(out)))
        return out

    def gradient(self, records):
        r = np.ascontiguousarray(records, np.float32)
        g = np.empty(abi.DL_GUIDE_PARAMS, np.float32)
        loss = C.c_float()
        self.ctx.check(self.ctx.lib.dl_guide_gradient(self.h, r.shape[0], _ptr(r), _ptr(g), C.byref(loss)))
        return loss.value, g

    def train(self, records, steps: int = 1) -> float:
        r = np.ascontiguousarray(records, np.float32)
        loss = C.c_float()
        self.ctx.check(self.ctx.lib.dl_guide_train(self.h, r.shape[0], _ptr(r), steps, C.byref(loss)))
        return loss.value

    def close(self):
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.ctx.lib.dl_guide_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
