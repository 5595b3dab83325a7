"""ctypes mirror of include/drawlab.h (structs, enums, status codes).

One definition of the scene descriptor layout for every consumer: the product
library (``libdlgpu.so``), the oracle and the reference harness all take the
same ``dl_*_desc`` arrays.
"""
from __future__ import annotations

import ctypes as C

DL_ABI_VERSION = 8

# status
DL_OK = 0
DL_ERR_INVALID_ARG = 1
DL_ERR_OOM = 2
DL_ERR_CUDA = 3
DL_ERR_TIMEOUT = 4
DL_ERR_QUEUE_OVERFLOW = 5
DL_ERR_PARSE = 6
DL_ERR_UNSUPPORTED = 7
DL_ERR_IO = 8

STATUS_NAMES = {
    0: "DL_OK", 1: "DL_ERR_INVALID_ARG", 2: "DL_ERR_OOM", 3: "DL_ERR_CUDA",
    4: "DL_ERR_TIMEOUT", 5: "DL_ERR_QUEUE_OVERFLOW", 6: "DL_ERR_PARSE",
    7: "DL_ERR_UNSUPPORTED", 8: "DL_ERR_IO",
}

# materials
DL_MAT_DIFFUSE = 0
DL_MAT_MIRROR = 1
DL_MAT_DIELECTRIC = 2
DL_MAT_MICROFACET = 3
DL_MAT_ANISO_GGX = 4

# lights
DL_LIGHT_AREA = 0
DL_LIGHT_POINT = 1
DL_LIGHT_ENVMAP = 2

DL_CAMERA_VIRTUAL = 0
DL_CAMERA_PERSPECTIVE = 1
DL_CAMERA_OPENCV = 2

DL_FILTER_GAUSSIAN = 0
DL_FILTER_BOX = 1

DL_IMAGE_PNG = 0
DL_IMAGE_EXR = 1
DL_IMAGE_PFM = 2

DL_RENDER_FIX_POINT_LIGHT = 1 << 0
DL_RENDER_POWER_LIGHT_PICK = 1 << 1
DL_RENDER_NORMALS = 1 << 2


class dl_mesh_desc(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)),
        ("normals", C.POINTER(C.c_float)),
        ("texcoords", C.POINTER(C.c_float)),
        ("indices", C.POINTER(C.c_uint32)),
        ("num_vertices", C.c_int64),
        ("num_triangles", C.c_int64),
        ("material", C.c_int32),
        ("light", C.c_int32),
    ]


class dl_texture_desc(C.Structure):
    _fields_ = [
        ("rgb", C.POINTER(C.c_float)),
        ("width", C.c_int32),
        ("height", C.c_int32),
    ]


class dl_material_desc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("albedo", C.c_float * 3),
        ("specular", C.c_float * 3),
        ("alpha", C.c_float * 2),
        ("int_ior", C.c_float),
        ("ext_ior", C.c_float),
        ("albedo_texture", dl_texture_desc),
        ("specular_texture", dl_texture_desc),
        ("alpha_texture", dl_texture_desc),
        ("normal_texture", dl_texture_desc),
        ("tangent_texture", dl_texture_desc),
    ]


class dl_light_desc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("mesh", C.c_int32),
        ("radiance", C.c_float * 3),
        ("position", C.c_float * 3),
        ("env_rgb", C.POINTER(C.c_float)),
        ("env_width", C.c_int32),
        ("env_height", C.c_int32),
        ("env_scale", C.c_float),
        ("env_visual", C.c_int32),
        ("env_background", C.c_float * 3),
    ]


class dl_camera_desc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("eye", C.c_float * 3),
        ("lookat", C.c_float * 3),
        ("up", C.c_float * 3),
        ("fov", C.c_float),
        ("transform", C.c_float * 16),
        ("near_clip", C.c_float),
        ("far_clip", C.c_float),
        ("fx", C.c_float),
        ("fy", C.c_float),
        ("cx", C.c_float),
        ("cy", C.c_float),
    ]


class dl_scene_info(C.Structure):
    _fields_ = [
        ("num_triangles", C.c_int64),
        ("num_bvh_nodes", C.c_int64),
        ("num_meshes", C.c_int32),
        ("num_materials", C.c_int32),
        ("num_lights", C.c_int32),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("bvh_depth", C.c_int32),
        ("bvh_build_seconds", C.c_double),
        ("bvh_sah_cost", C.c_double),
        ("device_bytes", C.c_int64),
    ]


class dl_render_opts(C.Structure):
    _fields_ = [
        ("spp", C.c_int32),
        ("max_depth", C.c_int32),
        ("rr_depth", C.c_int32),
        ("filter", C.c_int32),
        ("seed", C.c_uint64),
        ("flags", C.c_uint32),
        ("spp_offset", C.c_int32),
        ("max_paths_in_flight", C.c_int64),
    ]


class dl_stats(C.Structure):
    _fields_ = [
        ("camera_rays", C.c_int64),
        ("extension_rays", C.c_int64),
        ("shadow_rays", C.c_int64),
        ("invalid_samples", C.c_int64),
        ("iterations", C.c_int64),
        ("render_ms", C.c_double),
        ("trace_ms", C.c_double),
        ("extend_ms", C.c_double),
        ("shadow_ms", C.c_double),
        ("shade_ms", C.c_double),
        ("retire_ms", C.c_double),
        ("kernel_launches", C.c_int64),
        ("guide_records", C.c_int64),
        ("guide_train_ms", C.c_double),
        ("guide_ms", C.c_double),
    ]


class dl_traversal_counts(C.Structure):
    _fields_ = [
        ("extension_rays", C.c_int64),
        ("shadow_rays", C.c_int64),
        ("extension_node_visits", C.c_int64),
        ("extension_triangle_tests", C.c_int64),
        ("shadow_node_visits", C.c_int64),
        ("shadow_triangle_tests", C.c_int64),
    ]


class dl_request(C.Structure):
    _fields_ = [
        ("scene", C.c_void_p),
        ("opts", dl_render_opts),
        ("rgb", C.POINTER(C.c_float)),
        ("film_device", C.POINTER(C.c_float)),
        ("camera", C.c_void_p),
    ]


class dl_tune_params(C.Structure):
    _fields_ = [
        ("paths_in_flight", C.c_int64),
        ("traverse_ctas_per_sm", C.c_int32),
        ("shade_ctas_per_sm", C.c_int32),
        ("iterations_per_graph", C.c_int32),
        ("shade_threads", C.c_int32),
    ]


DL_GUIDE_PARAMS = 16560


class dl_guide_config(C.Structure):
    _fields_ = [
        ("learning_rate", C.c_float),
        ("guide_fraction", C.c_float),
        ("batch", C.c_int32),
        ("steps_per_pass", C.c_int32),
        ("max_guided_depth", C.c_int32),
        ("reserved", C.c_int32),
        ("seed", C.c_uint64),
    ]


def make_opts(spp=1, max_depth=0, rr_depth=3, filter=DL_FILTER_GAUSSIAN, seed=0, flags=0,
              spp_offset=0, max_paths_in_flight=0) -> dl_render_opts:
    o = dl_render_opts()
    o.spp = spp
    o.max_depth = max_depth
    o.rr_depth = rr_depth
    o.filter = filter
    o.seed = seed
    o.flags = flags
    o.spp_offset = spp_offset
    o.max_paths_in_flight = max_paths_in_flight
    return o
