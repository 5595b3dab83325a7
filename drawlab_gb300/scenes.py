"""Procedural scenes (the workloads the path tracer is measured and checked on).

No scene files ship with the reference, so every workload is generated here
from a seed:

* ``cornell()``        -- Cornell box: 5 quads + 2 rotated cuboids + ceiling
                          light, 256x256 (34 triangles).
* ``material_spheres()`` -- 64 level-4 icospheres (5120 triangles each) on a
                          40x40 ground quad with seeded materials, 4 quad area
                          lights and a point light, 1920x1080 (327,682 tris).
* ``mis_plates()``     -- four GGX plates under four spherical lights of equal
                          power, 1280x720 (Veach-style MIS stress scene).

A scene is a :class:`SceneData` holding numpy arrays; ``descs()`` packs it into
the ``dl_*_desc`` structs of include/drawlab.h for the GPU library, the oracle
and the reference harness alike.

Quads follow the reference's ``rectangle`` shape exactly
(src/tracer/mesh/rectangle.cpp:11-40): vertices pos, pos+v0, pos+v1,
pos+v0+v1, faces (0,1,2), (3,2,1), every vertex normal normalize(v0 x v1).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi


@dataclass
class Mesh:
    positions: np.ndarray           # (V, 3) float32
    indices: np.ndarray             # (F, 3) uint32
    normals: np.ndarray | None = None
    texcoords: np.ndarray | None = None
    material: int = 0
    light: int = -1


@dataclass
class Material:
    type: int = abi.DL_MAT_DIFFUSE
    albedo: tuple = (0.5, 0.5, 0.5)
    specular: tuple = (0.5, 0.5, 0.5)
    alpha: tuple = (0.1, 0.1)
    int_ior: float = 1.5046
    ext_ior: float = 1.000277
    # bitmap textures, (height, width, 3) float32, row k at t = (k + 0.5) / height
    albedo_texture: np.ndarray | None = None
    specular_texture: np.ndarray | None = None
    alpha_texture: np.ndarray | None = None
    normal_texture: np.ndarray | None = None
    tangent_texture: np.ndarray | None = None

TEXTURE_SLOTS = ("albedo_texture", "specular_texture", "alpha_texture", "normal_texture", "tangent_texture")


@dataclass
class Light:
    type: int = abi.DL_LIGHT_AREA
    mesh: int = -1
    radiance: tuple = (1.0, 1.0, 1.0)
    position: tuple = (0.0, 0.0, 0.0)
    env_rgb: np.ndarray | None = None   # (H, W, 3) float32
    env_scale: float = 1.0
    env_visual: int = 1
    env_background: tuple = (0.0, 0.0, 0.0)


@dataclass
class Camera:
    """A camera: "virtual" (eye / lookat / up, vertical fov), "perspective"
    (camera-to-world `transform`, horizontal fov, near / far clip) or
    "opencv" (intrinsics fx, fy, cx, cy and the world-to-camera `transform`)."""
    width: int = 256
    height: int = 256
    eye: tuple = (0.0, 0.0, 1.0)
    lookat: tuple = (0.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    fov: float = 30.0
    type: int = abi.DL_CAMERA_VIRTUAL
    transform: np.ndarray | None = None   # (4, 4), row-major
    near_clip: float = 1e-4
    far_clip: float = 1e4
    fx: float = 0.0
    fy: float = 0.0
    cx: float = 0.0
    cy: float = 0.0

    def desc(self) -> abi.dl_camera_desc:
        d = abi.dl_camera_desc()
        d.type = self.type
        d.width, d.height = self.width, self.height
        d.eye[:] = [float(v) for v in self.eye]
        d.lookat[:] = [float(v) for v in self.lookat]
        d.up[:] = [float(v) for v in self.up]
        d.fov = self.fov
        t = np.eye(4) if self.transform is None else np.asarray(self.transform, np.float64)
        d.transform[:] = [float(v) for v in t.reshape(16)]
        d.near_clip, d.far_clip = self.near_clip, self.far_clip
        d.fx, d.fy, d.cx, d.cy = self.fx, self.fy, self.cx, self.cy
        return d


def look_at(origin, target, up) -> np.ndarray:
    """Camera-to-world matrix of a <lookat> transform (camera looks along +z,
    x to the left: the reference's convention, parser.cpp:343-369)."""
    o = np.asarray(origin, np.float64)
    d = np.asarray(target, np.float64) - o
    d /= np.linalg.norm(d)
    left = np.cross(np.asarray(up, np.float64), d)
    left /= np.linalg.norm(left)
    nup = np.cross(d, left)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = left, nup, d, o
    return m


@dataclass
class SceneData:
    name: str
    meshes: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    lights: list = field(default_factory=list)
    camera: Camera = field(default_factory=Camera)
    spp: int = 16
    max_depth: int = 0
    rr_depth: int = 3

    @property
    def num_triangles(self) -> int:
        return int(sum(m.indices.shape[0] for m in self.meshes))

    def add_material(self, mat: Material) -> int:
        self.materials.append(mat)
        return len(self.materials) - 1

    def add_mesh(self, mesh: Mesh) -> int:
        self.meshes.append(mesh)
        return len(self.meshes) - 1

    def add_area_light(self, mesh_index: int, radiance) -> int:
        self.lights.append(Light(type=abi.DL_LIGHT_AREA, mesh=mesh_index,
                                 radiance=tuple(float(x) for x in radiance)))
        self.meshes[mesh_index].light = len(self.lights) - 1
        return len(self.lights) - 1

    def triangles(self) -> np.ndarray:
        """All triangles as (F, 3, 3) float32, meshes concatenated in order."""
        out = [m.positions[m.indices.astype(np.int64)] for m in self.meshes]
        return np.concatenate(out, axis=0).astype(np.float32)

    def descs(self):
        """Pack into ctypes descriptors.  Returns (holder, meshes, nm, mats,
        nmat, lights, nl, camera); keep ``holder`` alive while they are used."""
        keep = []

        def fptr(a):
            if a is None:
                return C.POINTER(C.c_float)()
            a = np.ascontiguousarray(a, dtype=np.float32)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_float))

        nm = len(self.meshes)
        md = (abi.dl_mesh_desc * max(nm, 1))()
        for i, m in enumerate(self.meshes):
            idx = np.ascontiguousarray(m.indices, dtype=np.uint32)
            keep.append(idx)
            md[i].positions = fptr(m.positions)
            md[i].normals = fptr(m.normals)
            md[i].texcoords = fptr(m.texcoords)
            md[i].indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
            md[i].num_vertices = m.positions.shape[0]
            md[i].num_triangles = idx.shape[0]
            md[i].material = m.material
            md[i].light = m.light
        nmat = len(self.materials)
        mat = (abi.dl_material_desc * max(nmat, 1))()
        for i, x in enumerate(self.materials):
            mat[i].type = x.type
            mat[i].albedo[:] = [float(v) for v in x.albedo]
            mat[i].specular[:] = [float(v) for v in x.specular]
            mat[i].alpha[:] = [float(v) for v in x.alpha]
            mat[i].int_ior = x.int_ior
            mat[i].ext_ior = x.ext_ior
            for slot in TEXTURE_SLOTS:
                tex = getattr(x, slot)
                if tex is not None:
                    t = getattr(mat[i], slot)
                    t.rgb = fptr(tex)
                    t.height, t.width = tex.shape[0], tex.shape[1]
        nl = len(self.lights)
        ld = (abi.dl_light_desc * max(nl, 1))()
        for i, x in enumerate(self.lights):
            ld[i].type = x.type
            ld[i].mesh = x.mesh
            ld[i].radiance[:] = [float(v) for v in x.radiance]
            ld[i].position[:] = [float(v) for v in x.position]
            if x.env_rgb is not None:
                ld[i].env_rgb = fptr(x.env_rgb)
                ld[i].env_height = x.env_rgb.shape[0]
                ld[i].env_width = x.env_rgb.shape[1]
            ld[i].env_scale = x.env_scale
            ld[i].env_visual = x.env_visual
            ld[i].env_background[:] = [float(v) for v in x.env_background]
        cam = self.camera.desc()
        keep.extend([md, mat, ld, cam])
        return keep, md, nm, mat, nmat, ld, nl, cam


# ------------------------------------------------------------------ geometry

def rectangle(pos, v0, v1) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """The reference's ``rectangle`` shape: (positions, indices, normals)."""
    pos = np.asarray(pos, np.float32)
    v0 = np.asarray(v0, np.float32)
    v1 = np.asarray(v1, np.float32)
    n = np.cross(v0, v1).astype(np.float32)
    n = (n / np.float32(np.sqrt(np.float32(n @ n)))).astype(np.float32)
    p = np.stack([pos, pos + v0, pos + v1, pos + v0 + v1]).astype(np.float32)
    f = np.array([[0, 1, 2], [3, 2, 1]], np.uint32)
    return p, f, np.tile(n, (4, 1)).astype(np.float32)


def _rot_y(deg: float) -> np.ndarray:
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float64)


def cuboid(center, size, rot_y_deg: float):
    """Axis-aligned box of `size` rotated about y, as 6 outward-facing quads
    (rectangle layout each): 24 vertices, 12 triangles, flat normals."""
    hx, hy, hz = (0.5 * s for s in size)
    R = _rot_y(rot_y_deg)
    c = np.asarray(center, np.float64)
    # (corner, edge0, edge1) with edge0 x edge1 pointing outwards
    faces = [
        ((-hx, -hy, hz), (2 * hx, 0, 0), (0, 2 * hy, 0)),    # +z
        ((hx, -hy, -hz), (-2 * hx, 0, 0), (0, 2 * hy, 0)),   # -z
        ((hx, -hy, hz), (0, 0, -2 * hz), (0, 2 * hy, 0)),    # +x
        ((-hx, -hy, -hz), (0, 0, 2 * hz), (0, 2 * hy, 0)),   # -x
        ((-hx, hy, hz), (2 * hx, 0, 0), (0, 0, -2 * hz)),    # +y
        ((-hx, -hy, -hz), (2 * hx, 0, 0), (0, 0, 2 * hz)),   # -y
    ]
    P, F, N = [], [], []
    for k, (p0, e0, e1) in enumerate(faces):
        p0 = R @ np.asarray(p0) + c
        e0 = R @ np.asarray(e0)
        e1 = R @ np.asarray(e1)
        p, f, n = rectangle(p0, e0, e1)
        P.append(p)
        F.append(f + 4 * k)
        N.append(n)
    return np.concatenate(P), np.concatenate(F).astype(np.uint32), np.concatenate(N)


def icosphere(level: int, center=(0, 0, 0), radius: float = 1.0):
    """Subdivided icosahedron: 20*4^level triangles, smooth unit normals."""
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        nf = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    Vn = np.array(V, np.float64)
    P = (Vn * radius + np.asarray(center, np.float64)).astype(np.float32)
    return P, np.array(F, np.uint32), Vn.astype(np.float32)


_ICO_CACHE: dict = {}


def _unit_icosphere(level: int):
    if level not in _ICO_CACHE:
        _ICO_CACHE[level] = icosphere(level)
    return _ICO_CACHE[level]


def sphere_mesh(level: int, center, radius: float):
    P, F, N = _unit_icosphere(level)
    Pd = (P.astype(np.float64) * radius + np.asarray(center, np.float64)).astype(np.float32)
    return Pd, F.copy(), N.copy()


# -------------------------------------------------------------------- scenes

def cornell(width: int = 256, height: int = 256, spp: int = 16, max_depth: int = 8) -> SceneData:
    """Cornell box: 2x2x2 box of 5 quads, two cuboids rotated +-17 degrees,
    0.5x0.4 ceiling area light of radiance (17, 12, 4)."""
    s = SceneData("cornell", spp=spp, max_depth=max_depth, rr_depth=3)
    grey = s.add_material(Material(albedo=(0.725, 0.725, 0.725)))
    red = s.add_material(Material(albedo=(0.63, 0.065, 0.05)))
    green = s.add_material(Material(albedo=(0.14, 0.45, 0.09)))
    black = s.add_material(Material(albedo=(0.0, 0.0, 0.0)))
    quads = [
        ((-1, -1, -1), (0, 0, 2), (2, 0, 0), grey),    # floor, +y
        ((-1, 1, -1), (2, 0, 0), (0, 0, 2), grey),     # ceiling, -y
        ((-1, -1, -1), (2, 0, 0), (0, 2, 0), grey),    # back, +z
        ((-1, -1, -1), (0, 2, 0), (0, 0, 2), red),     # left, +x
        ((1, -1, -1), (0, 0, 2), (0, 2, 0), green),    # right, -x
    ]
    for pos, v0, v1, m in quads:
        p, f, n = rectangle(pos, v0, v1)
        s.add_mesh(Mesh(p, f, n, material=m))
    # cuboids lifted 1e-3 off the floor so no face is coplanar with another
    p, f, n = cuboid((-0.33, -1 + 0.6 + 1e-3, -0.28), (0.6, 1.2, 0.6), 17.0)
    s.add_mesh(Mesh(p, f, n, material=grey))
    p, f, n = cuboid((0.34, -1 + 0.3 + 1e-3, 0.32), (0.6, 0.6, 0.6), -17.0)
    s.add_mesh(Mesh(p, f, n, material=grey))
    p, f, n = rectangle((-0.25, 0.999, -0.2), (0.5, 0, 0), (0, 0, 0.4))
    li = s.add_mesh(Mesh(p, f, n, material=black))
    s.add_area_light(li, (17.0, 12.0, 4.0))
    s.camera = Camera(width=width, height=height, eye=(0.0, 0.0, 3.9), lookat=(0.0, 0.0, 0.0),
                      up=(0.0, 1.0, 0.0), fov=39.3)
    return s


def textured_cornell(width: int = 64, height: int = 64, spp: int = 4, max_depth: int = 8, seed: int = 6) -> SceneData:
    """The Cornell box with bitmap textures: checkered albedo textures on the
    floor and back wall (texcoords over the quads, tiled twice: wrap
    addressing), and in place of the short cuboid an anisotropic GGX sphere
    with pd / ps / axay textures and world-space normal and tangent maps
    (spherical texcoords)."""
    rng = np.random.default_rng(seed)
    s = cornell(width=width, height=height, spp=spp, max_depth=max_depth)
    s.name = "textured_cornell"
    uv_quad = np.array([[0, 0], [2, 0], [0, 2], [2, 2]], np.float32)   # rectangle() vertex order

    def checker(n, a, b):
        y, x = np.mgrid[0:n, 0:n]
        m = ((x // 2 + y // 2) % 2)[..., None]
        return np.where(m, np.asarray(a, np.float32), np.asarray(b, np.float32)).astype(np.float32)

    floor_m = s.add_material(Material(albedo_texture=checker(16, (0.8, 0.75, 0.7), (0.15, 0.2, 0.3))))
    back_m = s.add_material(Material(albedo_texture=rng.uniform(0.05, 0.9, (9, 13, 3)).astype(np.float32)))
    s.meshes[0].material, s.meshes[0].texcoords = floor_m, uv_quad
    s.meshes[2].material, s.meshes[2].texcoords = back_m, uv_quad
    # the aniso sphere replaces the short cuboid
    p, f, n = sphere_mesh(3, (0.34, -0.62, 0.32), 0.38)
    d = (p - np.array([0.34, -0.62, 0.32], np.float32)) / 0.38
    uv = np.stack([np.arctan2(d[:, 2], d[:, 0]) / (2 * np.pi) + 0.5,
                   np.arccos(np.clip(d[:, 1], -1, 1)) / np.pi], 1).astype(np.float32)
    th = 24
    tw = 32
    v, u = np.mgrid[0:th, 0:tw]
    pd = np.stack([0.2 + 0.6 * (u / tw), 0.3 + 0.4 * (v / th), 0.5 + 0.0 * u], -1).astype(np.float32)
    ps = np.full((th, tw, 3), 0.6, np.float32) * (0.5 + 0.5 * ((u + v) % 2))[..., None].astype(np.float32)
    axay = np.stack([0.05 + 0.4 * (u / tw), 0.4 - 0.3 * (v / th), 0.0 * u], -1).astype(np.float32)
    # world-space maps: a perturbed outward normal, a tangent around the y axis
    phi = (u + 0.5) / tw * 2 * np.pi - np.pi
    theta = (v + 0.5) / th * np.pi
    nw = np.stack([np.sin(theta) * np.cos(phi), np.cos(theta), np.sin(theta) * np.sin(phi)], -1)
    nw = nw + 0.15 * rng.normal(size=nw.shape)
    nw /= np.linalg.norm(nw, axis=-1, keepdims=True)
    tw_ = np.stack([-np.sin(phi), np.zeros_like(phi), np.cos(phi)], -1)
    normal_map = (0.5 * (nw + 1)).astype(np.float32)
    tangent_map = (0.5 * (tw_ + 1)).astype(np.float32)
    aniso = s.add_material(Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0.5, 0.5, 0.5), specular=(0.5, 0.5, 0.5),
                                    alpha=(0.2, 0.2), albedo_texture=pd, specular_texture=ps, alpha_texture=axay,
                                    normal_texture=normal_map, tangent_texture=tangent_map))
    s.meshes[6] = Mesh(p, f, n, texcoords=uv, material=aniso)
    return s


def material_spheres(width: int = 1920, height: int = 1080, spp: int = 64, max_depth: int = 16,
                     seed: int = 2, num_spheres: int = 64, level: int = 4) -> SceneData:
    """64 icospheres on a 40x40 ground quad with seeded materials (diffuse,
    mirror, dielectric, GGX, anisotropic GGX), 4 quad area lights of radiance
    U[5,30] and one point light of intensity 200."""
    rng = np.random.default_rng(seed)
    s = SceneData("material_spheres", spp=spp, max_depth=max_depth, rr_depth=3)
    ground = s.add_material(Material(albedo=(0.5, 0.5, 0.5)))
    p, f, n = rectangle((-20, 0, -20), (0, 0, 40), (40, 0, 0))
    s.add_mesh(Mesh(p, f, n, material=ground))
    placed = []
    tries = 0
    while len(placed) < num_spheres:
        tries += 1
        if tries > 100000:
            raise RuntimeError("sphere placement failed")
        r = float(rng.uniform(0.3, 1.0))
        x, z = (float(v) for v in rng.uniform(-18.0, 18.0, size=2))
        if all((x - px) ** 2 + (z - pz) ** 2 > (r + pr + 0.05) ** 2 for px, pz, pr in placed):
            placed.append((x, z, r))
    for x, z, r in placed:
        kind = int(rng.integers(0, 5))
        if kind == 0:
            m = Material(type=abi.DL_MAT_DIFFUSE, albedo=tuple(rng.uniform(0.1, 0.9, 3)))
        elif kind == 1:
            m = Material(type=abi.DL_MAT_MIRROR)
        elif kind == 2:
            m = Material(type=abi.DL_MAT_DIELECTRIC, int_ior=1.5, ext_ior=1.000277)
        elif kind == 3:
            a = float(rng.uniform(0.05, 0.5))
            m = Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0, 0, 0), specular=(1, 1, 1), alpha=(a, a))
        else:
            ax, ay = (float(v) for v in rng.uniform(0.02, 0.4, 2))
            m = Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0, 0, 0), specular=(1, 1, 1), alpha=(ax, ay))
        mi = s.add_material(m)
        p, f, n = sphere_mesh(level, (x, r + 1e-3, z), r)
        s.add_mesh(Mesh(p, f, n, material=mi))
    black = s.add_material(Material(albedo=(0.0, 0.0, 0.0)))
    for k in range(4):
        L = float(rng.uniform(5.0, 30.0))
        cx, cz = (float(v) for v in rng.uniform(-12.0, 12.0, 2))
        w, d = (float(v) for v in rng.uniform(2.0, 4.0, 2))
        h = float(rng.uniform(8.0, 12.0))
        p, f, n = rectangle((cx - w / 2, h, cz - d / 2), (w, 0, 0), (0, 0, d))   # faces -y
        li = s.add_mesh(Mesh(p, f, n, material=black))
        s.add_area_light(li, (L, L, L))
    s.lights.append(Light(type=abi.DL_LIGHT_POINT, radiance=(200.0, 200.0, 200.0),
                          position=(0.0, 6.0, 4.0)))
    s.camera = Camera(width=width, height=height, eye=(0.0, 9.0, 26.0), lookat=(0.0, 0.0, 0.0),
                      up=(0.0, 1.0, 0.0), fov=45.0)
    return s


def mis_plates(width: int = 1280, height: int = 720, spp: int = 256, max_depth: int = 8,
               level: int = 3) -> SceneData:
    """Four 4x0.6 GGX plates (alpha 0.005, 0.02, 0.05, 0.2; pd 0, ps 1) facing
    the camera under four spherical lights of radius 0.03, 0.1, 0.3, 0.9 with
    radiance scaled as 1/r^2, in front of a diffuse 0.4 backdrop."""
    s = SceneData("mis_plates", spp=spp, max_depth=max_depth, rr_depth=3)
    eye = np.array([0.0, 2.0, 15.0])
    target = np.array([0.0, -2.0, 2.5])
    back = s.add_material(Material(albedo=(0.4, 0.4, 0.4)))
    p, f, n = rectangle((-20, -4.2, -6), (40, 0, 0), (0, 30, 0))      # back wall, +z
    s.add_mesh(Mesh(p, f, n, material=back))
    p, f, n = rectangle((-20, -4.2, -6), (0, 0, 30), (40, 0, 0))      # floor, +y
    s.add_mesh(Mesh(p, f, n, material=back))
    light_center = np.array([0.0, 2.5, 0.0])
    for k, (alpha, zc) in enumerate(zip((0.005, 0.02, 0.05, 0.2), (4.0, 2.7, 1.4, 0.1))):
        c = np.array([0.0, -2.8 + 0.25 * k, zc])
        to_eye = eye - c
        to_eye /= np.linalg.norm(to_eye)
        to_l = light_center - c
        to_l /= np.linalg.norm(to_l)
        nrm = to_eye + to_l
        nrm /= np.linalg.norm(nrm)
        ex = np.array([4.0, 0.0, 0.0])
        ey = np.cross(nrm, ex)
        ey = 0.6 * ey / np.linalg.norm(ey)
        pos = c - 0.5 * ex - 0.5 * ey
        e0, e1 = (ex, ey) if np.dot(np.cross(ex, ey), nrm) > 0 else (ey, ex)
        mi = s.add_material(Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0, 0, 0), specular=(1, 1, 1),
                                     alpha=(alpha, alpha)))
        p, f, n = rectangle(pos, e0, e1)
        s.add_mesh(Mesh(p, f, n, material=mi))
    black = s.add_material(Material(albedo=(0.0, 0.0, 0.0)))
    for x, r in zip((-3.75, -1.25, 1.25, 3.75), (0.03, 0.1, 0.3, 0.9)):
        L = 0.8 / (r * r) * 0.1
        p, f, n = sphere_mesh(level, (x, light_center[1], light_center[2]), r)
        li = s.add_mesh(Mesh(p, f, n, material=black))
        s.add_area_light(li, (L, L, L))
    s.camera = Camera(width=width, height=height, eye=tuple(eye), lookat=tuple(target),
                      up=(0.0, 1.0, 0.0), fov=28.0)
    return s


def reference_spheres(width: int = 96, height: int = 64, spp: int = 4, max_depth: int = 0,
                      seed: int = 5) -> SceneData:
    """Small scene using only what the reference CPU backend implements:
    six level-2 icospheres (diffuse, mirror, dielectric, Beckmann microfacet)
    on a ground quad, two quad area lights and a point light."""
    rng = np.random.default_rng(seed)
    s = SceneData("reference_spheres", spp=spp, max_depth=max_depth, rr_depth=3)
    ground = s.add_material(Material(albedo=(0.6, 0.6, 0.6)))
    p, f, n = rectangle((-6, 0, -6), (0, 0, 12), (12, 0, 0))
    s.add_mesh(Mesh(p, f, n, material=ground))
    kinds = [
        Material(type=abi.DL_MAT_DIFFUSE, albedo=(0.8, 0.3, 0.2)),
        Material(type=abi.DL_MAT_MIRROR),
        Material(type=abi.DL_MAT_DIELECTRIC, int_ior=1.5, ext_ior=1.000277),
        Material(type=abi.DL_MAT_MICROFACET, albedo=(0.2, 0.2, 0.4), alpha=(0.28, 0.28), int_ior=1.7),
        Material(type=abi.DL_MAT_MICROFACET, albedo=(0.5, 0.4, 0.1), alpha=(0.08, 0.08)),
        Material(type=abi.DL_MAT_DIFFUSE, albedo=(0.2, 0.7, 0.3)),
    ]
    for k, m in enumerate(kinds):
        mi = s.add_material(m)
        x = -3.75 + 1.5 * k
        z = float(rng.uniform(-1.0, 1.0))
        r = float(rng.uniform(0.45, 0.7))
        p, f, n = sphere_mesh(2, (x, r + 1e-3, z), r)
        s.add_mesh(Mesh(p, f, n, material=mi))
    black = s.add_material(Material(albedo=(0.0, 0.0, 0.0)))
    p, f, n = rectangle((-3.0, 5.0, -1.0), (2.0, 0, 0), (0, 0, 1.5))
    li = s.add_mesh(Mesh(p, f, n, material=black))
    s.add_area_light(li, (12.0, 10.0, 8.0))
    p, f, n = rectangle((1.0, 4.0, -2.5), (0, 0, 1.0), (1.5, 0, 0))
    li = s.add_mesh(Mesh(p, f, n, material=black))
    s.add_area_light(li, (5.0, 8.0, 12.0))
    s.lights.append(Light(type=abi.DL_LIGHT_POINT, radiance=(30.0, 30.0, 40.0), position=(2.0, 4.0, 2.0)))
    s.camera = Camera(width=width, height=height, eye=(0.0, 3.0, 9.0), lookat=(0.0, 0.5, 0.0),
                      up=(0.0, 1.0, 0.0), fov=40.0)
    return s


SCENES = {
    "cornell": cornell,
    "material_spheres": material_spheres,
    "mis_plates": mis_plates,
    "reference_spheres": reference_spheres,
}


# ----------------------------------------------------------------- envmaps

def sky_envmap(width: int = 2048, height: int = 1024, sun_dir=(0.35, 0.6, -0.72), sun_peak: float = 1.0e4,
               sun_radius_deg: float = 0.5, sky_scale: float = 1.0) -> np.ndarray:
    """Procedural latitude-longitude sky, (height, width, 3) float32: a
    zenith-to-horizon gradient above a dim ground, plus a sun lobe of peak
    radiance `sun_peak` and angular radius `sun_radius_deg` (smooth falloff
    over the outer fifth).  Row 0 is the +y pole; texel centres map to
    directions as the envmap emitter's lookup does."""
    y, x = np.mgrid[0:height, 0:width].astype(np.float64)
    u = (x + 0.5) / width
    v = (y + 0.5) / height
    phi = 2.0 * np.pi * u - np.pi
    theta = np.pi * v
    d = np.stack([np.cos(phi) * np.sin(theta), np.cos(theta), np.sin(phi) * np.sin(theta)], axis=-1)
    up = np.clip(d[..., 1], 0.0, 1.0)[..., None]
    zenith = np.array([0.15, 0.3, 0.8])
    horizon = np.array([0.8, 0.85, 0.9])
    ground = np.array([0.25, 0.22, 0.2])
    sky = np.where(d[..., 1:2] >= 0.0, horizon + (zenith - horizon) * np.sqrt(up), ground * 0.5)
    s = np.asarray(sun_dir, np.float64)
    s = s / np.linalg.norm(s)
    ang = np.degrees(np.arccos(np.clip(d @ s, -1.0, 1.0)))
    r = float(sun_radius_deg)
    lobe = np.clip((r - ang) / (0.2 * r), 0.0, 1.0)
    rgb = sky * sky_scale + (sun_peak * lobe)[..., None] * np.array([1.0, 0.95, 0.85])
    return np.ascontiguousarray(rgb, dtype=np.float32)


def env_spheres(width: int = 96, height: int = 64, spp: int = 4, max_depth: int = 8, env_width: int = 64,
                env_height: int = 32, sun_radius_deg: float = 6.0, sun_peak: float = 200.0,
                with_area_light: bool = True, visual: int = 1) -> SceneData:
    """Spheres of every material type on a ground quad under a procedural sky
    envmap (optionally plus one quad area light): the envmap NEE, MIS and miss
    paths.  The default map is small, with a wide sun, so the oracle stays
    fast; the 2048x1024 form with a 0.5-degree sun is sky_envmap()."""
    s = SceneData("env_spheres", spp=spp, max_depth=max_depth, rr_depth=3)
    ground = s.add_material(Material(albedo=(0.5, 0.45, 0.4)))
    p, f, n = rectangle((-8, 0, -8), (0, 0, 16), (16, 0, 0))
    s.add_mesh(Mesh(p, f, n, material=ground))
    kinds = [
        Material(type=abi.DL_MAT_DIFFUSE, albedo=(0.8, 0.3, 0.2)),
        Material(type=abi.DL_MAT_MIRROR),
        Material(type=abi.DL_MAT_DIELECTRIC, int_ior=1.5, ext_ior=1.000277),
        Material(type=abi.DL_MAT_MICROFACET, albedo=(0.2, 0.2, 0.4), alpha=(0.2, 0.2), int_ior=1.7),
        Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0, 0, 0), specular=(1, 1, 1), alpha=(0.15, 0.15)),
        Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0.2, 0.2, 0.2), specular=(0.8, 0.8, 0.8), alpha=(0.05, 0.3)),
    ]
    for k, m in enumerate(kinds):
        mi = s.add_material(m)
        p, f, n = sphere_mesh(2, (-3.75 + 1.5 * k, 0.601, 0.3 * (k % 2)), 0.6)
        s.add_mesh(Mesh(p, f, n, material=mi))
    if with_area_light:
        black = s.add_material(Material(albedo=(0.0, 0.0, 0.0)))
        p, f, n = rectangle((-1.0, 4.0, -1.0), (2.0, 0, 0), (0, 0, 1.5))
        li = s.add_mesh(Mesh(p, f, n, material=black))
        s.add_area_light(li, (6.0, 6.0, 6.0))
    env = sky_envmap(env_width, env_height, sun_peak=sun_peak, sun_radius_deg=sun_radius_deg)
    s.lights.append(Light(type=abi.DL_LIGHT_ENVMAP, env_rgb=env, env_scale=1.0, env_visual=visual,
                          env_background=(0.1, 0.2, 0.3)))
    s.camera = Camera(width=width, height=height, eye=(0.0, 2.5, 9.0), lookat=(0.0, 0.5, 0.0),
                      up=(0.0, 1.0, 0.0), fov=40.0)
    return s


def displaced_grid(center, size, n: int, height: float, seed: int = 0):
    """n x n grid over size=(sx, sz) at `center`, displaced along +y by a sum
    of seeded sines: 2 n^2 triangles, smooth normals."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-0.5, 0.5, n + 1)
    X, Z = np.meshgrid(xs * size[0], xs * size[1], indexing="xy")
    Y = np.zeros_like(X)
    for _ in range(4):
        fx, fz = rng.uniform(1.0, 6.0, 2)
        ph = rng.uniform(0, 2 * np.pi, 2)
        Y += np.sin(fx * X * 2 * np.pi / size[0] + ph[0]) * np.cos(fz * Z * 2 * np.pi / size[1] + ph[1])
    Y = height * (Y / max(1e-9, np.abs(Y).max()) * 0.5 + 0.5)
    P = np.stack([X, Y, Z], axis=-1).reshape(-1, 3) + np.asarray(center, np.float64)
    # normals from the height field gradient
    gy, gx = np.gradient(Y, xs * size[1], xs * size[0])
    N = np.stack([-gx, np.ones_like(Y), -gy], axis=-1).reshape(-1, 3)
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    i = np.arange(n)[:, None] * (n + 1) + np.arange(n)[None, :]
    a, b, c, d = i, i + 1, i + n + 1, i + n + 2
    F = np.concatenate([np.stack([a, c, b], -1).reshape(-1, 3), np.stack([b, c, d], -1).reshape(-1, 3)])
    return P.astype(np.float32), F.astype(np.uint32), N.astype(np.float32)


def guiding_room(width: int = 1920, height: int = 1080, spp: int = 16, max_depth: int = 12, grid: int = 700,
                 env_width: int = 2048, env_height: int = 1024, seed: int = 5) -> SceneData:
    """A closed 10 x 3 x 6 m room lit only through a 1 x 1 m window by the
    procedural sky (sky gradient + 0.5-degree sun of peak 1e4): diffuse walls
    0.2-0.8, furniture of cuboids (diffuse and GGX 0.1-0.4) and two
    displaced-grid 'sculptures' of 2 grid^2 triangles each (grid 700: about
    2M triangles in all).  The camera looks from the far end towards the
    window wall."""
    rng = np.random.default_rng(seed)
    s = SceneData("guiding_room", spp=spp, max_depth=max_depth, rr_depth=3)
    X0, X1, Y0, Y1, Z0, Z1 = -5.0, 5.0, 0.0, 3.0, -3.0, 3.0

    def diffuse(lo=0.2, hi=0.8):
        return s.add_material(Material(type=abi.DL_MAT_DIFFUSE, albedo=tuple(rng.uniform(lo, hi, 3))))

    def quad(pos, e0, e1, m):
        p, f, n = rectangle(pos, e0, e1)
        s.add_mesh(Mesh(p, f, n, material=m))

    # floor (+y), ceiling (-y), side walls, back wall (z = Z1, -z), window wall (z = Z0, +z)
    quad((X0, Y0, Z1), (X1 - X0, 0, 0), (0, 0, Z0 - Z1), diffuse(0.4, 0.7))
    quad((X0, Y1, Z0), (X1 - X0, 0, 0), (0, 0, Z1 - Z0), diffuse(0.6, 0.8))
    quad((X0, Y0, Z0), (0, 0, Z1 - Z0), (0, Y1 - Y0, 0), diffuse())
    quad((X1, Y0, Z1), (0, 0, Z0 - Z1), (0, Y1 - Y0, 0), diffuse())
    quad((X1, Y0, Z1), (X0 - X1, 0, 0), (0, Y1 - Y0, 0), diffuse())
    wall = diffuse(0.5, 0.8)
    wx0, wx1, wy0, wy1 = -0.5, 0.5, 1.3, 2.3        # the window opening
    quad((X0, Y0, Z0), (wx0 - X0, 0, 0), (0, Y1 - Y0, 0), wall)
    quad((wx1, Y0, Z0), (X1 - wx1, 0, 0), (0, Y1 - Y0, 0), wall)
    quad((wx0, Y0, Z0), (wx1 - wx0, 0, 0), (0, wy0 - Y0, 0), wall)
    quad((wx0, wy1, Z0), (wx1 - wx0, 0, 0), (0, Y1 - wy1, 0), wall)
    # furniture
    for k in range(6):
        sx, sy, sz = rng.uniform(0.4, 1.4), rng.uniform(0.3, 1.2), rng.uniform(0.4, 1.2)
        cx, cz = rng.uniform(X0 + 1, X1 - 1), rng.uniform(Z0 + 1.2, Z1 - 1)
        if k % 2 == 0:
            m = diffuse()
        else:
            a = float(rng.uniform(0.1, 0.4))
            m = s.add_material(Material(type=abi.DL_MAT_ANISO_GGX, albedo=tuple(rng.uniform(0.1, 0.5, 3)),
                                        specular=(0.5, 0.5, 0.5), alpha=(a, a)))
        P, F, N = cuboid((cx, Y0 + 0.5 * sy + 1e-3, cz), (sx, sy, sz), float(rng.uniform(0, 90)))
        s.add_mesh(Mesh(P, F, N, material=m))
    for k, (cx, cz) in enumerate([(-2.5, 0.5), (2.5, 1.0)]):
        m = diffuse() if k == 0 else s.add_material(Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0.3, 0.3, 0.3),
                                                             specular=(0.6, 0.6, 0.6), alpha=(0.25, 0.25)))
        P, F, N = displaced_grid((cx, Y0 + 2e-3, cz), (2.0, 2.0), grid, 0.6, seed=seed + k)
        s.add_mesh(Mesh(P, F, N, material=m))
    sky = sky_envmap(env_width, env_height, sun_dir=(0.25, 0.55, -0.8), sun_peak=1.0e4, sun_radius_deg=0.5)
    s.lights.append(Light(type=abi.DL_LIGHT_ENVMAP, env_rgb=sky, env_scale=1.0, env_visual=1))
    s.camera = Camera(width=width, height=height, eye=(0.0, 1.6, 2.7), lookat=(0.0, 1.0, -3.0),
                      up=(0.0, 1.0, 0.0), fov=60.0)
    return s


def _random_material(rng) -> Material:
    kind = int(rng.integers(0, 5))
    if kind == 0:
        return Material(type=abi.DL_MAT_DIFFUSE, albedo=tuple(rng.uniform(0.1, 0.9, 3)))
    if kind == 1:
        return Material(type=abi.DL_MAT_MIRROR)
    if kind == 2:
        return Material(type=abi.DL_MAT_DIELECTRIC, int_ior=1.5, ext_ior=1.000277)
    if kind == 3:
        a = float(rng.uniform(0.05, 0.5))
        return Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0, 0, 0), specular=(1, 1, 1), alpha=(a, a))
    ax, ay = (float(v) for v in rng.uniform(0.02, 0.4, 2))
    return Material(type=abi.DL_MAT_ANISO_GGX, albedo=(0, 0, 0), specular=(1, 1, 1), alpha=(ax, ay))


def batch_scene(triangles: int, seed: int, env: np.ndarray | None) -> SceneData:
    """A scene of about `triangles` triangles: a displaced-grid ground (half
    the budget) and level-3/4 icospheres with random materials (the other
    half), lit by `env` (the procedural sky) or by two quad area lights."""
    rng = np.random.default_rng(seed)
    s = SceneData("batch_%d" % triangles, spp=16, max_depth=8, rr_depth=3)
    n = max(4, int(math.sqrt(max(triangles // 2, 32) / 2)))
    P, F, N = displaced_grid((0.0, 0.0, 0.0), (20.0, 20.0), n, 1.0, seed=seed)
    s.add_mesh(Mesh(P, F, N, material=s.add_material(Material(albedo=tuple(rng.uniform(0.3, 0.7, 3))))))
    level = 4 if triangles >= 200_000 else 3
    per = 20 * 4 ** level
    count = max(1, (triangles - 2 * n * n) // per)
    for k in range(count):
        r = float(rng.uniform(0.2, 0.8))
        x, z = (float(v) for v in rng.uniform(-9.0, 9.0, 2))
        mi = s.add_material(_random_material(rng))
        p, f, nn = sphere_mesh(level, (x, 1.0 + r, z), r)
        s.add_mesh(Mesh(p, f, nn, material=mi))
    if env is not None:
        s.lights.append(Light(type=abi.DL_LIGHT_ENVMAP, env_rgb=env, env_scale=1.0, env_visual=1))
    else:
        black = s.add_material(Material(albedo=(0.0, 0.0, 0.0)))
        for k in range(2):
            L = float(rng.uniform(5.0, 30.0))
            cx, cz = (float(v) for v in rng.uniform(-6.0, 6.0, 2))
            p, f, nn = rectangle((cx - 1.5, 8.0, cz - 1.5), (3.0, 0, 0), (0, 0, 3.0))
            li = s.add_mesh(Mesh(p, f, nn, material=black))
            s.add_area_light(li, (L, L, L))
    s.camera = Camera(width=256, height=256, eye=(0.0, 7.0, 16.0), lookat=(0.0, 0.5, 0.0), up=(0.0, 1.0, 0.0),
                      fov=45.0)
    return s


BATCH_RESOLUTIONS = [(128, 128), (256, 256), (512, 512), (1024, 1024), (1920, 1080)]
BATCH_SPP = [4, 16, 64, 256]
BATCH_TRIANGLES = [1_000, 4_000, 16_000, 64_000, 256_000, 512_000, 1_000_000, 2_000_000]


def batch_workload(seed: int = 4, num_requests: int = 64, env_width: int = 2048, env_height: int = 1024,
                   triangles=None, resolutions=None, spp_choices=None):
    """The batched-rendering workload: `num_requests` requests drawn from
    `seed` -- a scene of 1k-2M triangles (half of the scenes lit by the
    procedural 2048x1024 sky with its 0.5-degree 1e4 sun), a resolution from
    {128^2 .. 1920x1080}, spp from {4, 16, 64, 256}, a camera orbiting the
    scene.  Returns (scenes, requests): requests are (scene index, spp,
    Camera)."""
    rng = np.random.default_rng(seed)
    tris = triangles or BATCH_TRIANGLES
    sky = sky_envmap(env_width, env_height, sun_peak=1.0e4, sun_radius_deg=0.5)
    scene_list = [batch_scene(t, seed * 100 + k, sky if k % 2 == 0 else None) for k, t in enumerate(tris)]
    reqs = []
    res = resolutions or BATCH_RESOLUTIONS
    sppc = spp_choices or BATCH_SPP
    for _ in range(num_requests):
        si = int(rng.integers(0, len(scene_list)))
        w, h = res[int(rng.integers(0, len(res)))]
        spp = int(sppc[int(rng.integers(0, len(sppc)))])
        a = float(rng.uniform(0, 2 * math.pi))
        cam = Camera(width=w, height=h, eye=(16.0 * math.sin(a), 7.0, 16.0 * math.cos(a)), lookat=(0.0, 0.5, 0.0),
                     up=(0.0, 1.0, 0.0), fov=45.0)
        reqs.append((si, spp, cam))
    return scene_list, reqs
