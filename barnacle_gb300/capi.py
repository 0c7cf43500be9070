"""ctypes binding of libbarnacle_gb300.so (include/barnacle_gpu.h).

The structures below mirror the C header field for field; numpy arrays are passed as plain
pointers.  Loading fails loudly when the library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libbarnacle_gb300.so"

BN_OK = 0
BN_ERR_INVALID_ARG = 1
BN_ERR_CUDA = 2
BN_ERR_NO_SCENE = 3
BN_ERR_DEVICE = 4
BN_ERR_OUT_OF_MEMORY = 5
BN_ERR_UNSUPPORTED = 6
BN_ERR_IO = 7

BN_PRIM_MESH, BN_PRIM_SPHERE = 0, 1
BN_MAT_LAMBERTIAN, BN_MAT_MIRROR, BN_MAT_DIELECTRIC, BN_MAT_PBR = 0, 1, 2, 3
BN_CAM_PINHOLE, BN_CAM_THIN_LENS = 0, 1
BN_LIGHTS_UNIFORM, BN_LIGHTS_ALIAS_TRIANGLES = 0, 1
BN_BVH_AUTO, BN_BVH_BINARY, BN_BVH_WIDE = 0, 2, 4
BN_BUILDER_AUTO, BN_BUILDER_HOST, BN_BUILDER_DEVICE = 0, 1, 2
BN_TONE_IDENTITY, BN_TONE_ACES, BN_TONE_GAMMA = 0, 1, 2
BN_TRACE_CLOSEST, BN_TRACE_ANY, BN_TRACE_WATERTIGHT, BN_TRACE_COUNT = 0x0, 0x1, 0x2, 0x4
BN_INTEGRATOR_PATH, BN_INTEGRATOR_PSSMLT, BN_INTEGRATOR_NORMAL, BN_INTEGRATOR_DIRECT = 0, 1, 2, 3
BN_MODE_MEGAKERNEL, BN_MODE_WAVEFRONT = 0, 1
BN_MUTATION_GAUSSIAN, BN_MUTATION_KELEMEN = 0, 1
BN_RENDER_WATERTIGHT, BN_RENDER_FIXED_ALIAS, BN_RENDER_NO_GRAPH, BN_RENDER_COUNT = 0x1, 0x2, 0x4, 0x8
BN_RENDER_CULL_SHADOW = 0x10
BN_DEVERR_STACK_OVERFLOW, BN_DEVERR_QUEUE_OVERFLOW, BN_DEVERR_WATCHDOG, BN_DEVERR_BAD_INDEX = 0x1, 0x2, 0x4, 0x8


class bn_mesh_desc(C.Structure):
    _fields_ = [("vertices", C.POINTER(C.c_float)), ("indices", C.POINTER(C.c_int32)),
                ("tri_material", C.POINTER(C.c_int32)), ("n_vertices", C.c_int32), ("n_triangles", C.c_int32)]


class bn_primitive_desc(C.Structure):
    _fields_ = [("type", C.c_int32), ("mesh", C.c_int32), ("radius", C.c_float)]


class bn_instance_desc(C.Structure):
    _fields_ = [("primitive", C.c_int32), ("material", C.c_int32), ("light", C.c_int32), ("pad_", C.c_int32),
                ("object_to_world", C.c_float * 16), ("world_to_object", C.c_float * 16)]


class bn_material_desc(C.Structure):
    _fields_ = [("type", C.c_int32), ("base_color", C.c_float * 3), ("ior", C.c_float), ("roughness", C.c_float),
                ("metallic", C.c_float), ("pad_", C.c_float)]


class bn_light_desc(C.Structure):
    _fields_ = [("emission", C.c_float * 3), ("two_sided", C.c_int32)]


class bn_camera_desc(C.Structure):
    _fields_ = [("type", C.c_int32), ("fov_y_degrees", C.c_float), ("aspect_ratio", C.c_float),
                ("aperture", C.c_float), ("focus_distance", C.c_float), ("push_forward", C.c_float),
                ("camera_to_world", C.c_float * 16)]


class bn_scene_desc(C.Structure):
    _fields_ = [("primitives", C.POINTER(bn_primitive_desc)), ("n_primitives", C.c_int32),
                ("meshes", C.POINTER(bn_mesh_desc)), ("n_meshes", C.c_int32),
                ("instances", C.POINTER(bn_instance_desc)), ("n_instances", C.c_int32),
                ("materials", C.POINTER(bn_material_desc)), ("n_materials", C.c_int32),
                ("lights", C.POINTER(bn_light_desc)), ("n_lights", C.c_int32),
                ("light_sampler", C.c_int32), ("bvh_width", C.c_int32), ("bvh_builder", C.c_int32)]


class bn_ray(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("direction", C.c_float * 3), ("t_max", C.c_float)]


class bn_hit(C.Structure):
    _fields_ = [("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("instance", C.c_int32),
                ("primitive", C.c_int32), ("normal", C.c_float * 3), ("position", C.c_float * 3)]


class bn_bsdf_query(C.Structure):
    _fields_ = [("material", C.c_int32), ("wo", C.c_float * 3), ("wi", C.c_float * 3), ("u_lobe", C.c_float),
                ("u_bsdf", C.c_float * 2)]


class bn_bsdf_result(C.Structure):
    _fields_ = [("bsdf", C.c_float * 3), ("pdf", C.c_float), ("wi", C.c_float * 3)]


class bn_view(C.Structure):
    _fields_ = [("camera", bn_camera_desc), ("width", C.c_int32), ("height", C.c_int32)]


class bn_render_desc(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("mode", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("rr_depth", C.c_int32), ("frame_id", C.c_int32), ("flags", C.c_uint32),
                ("n_bootstrap", C.c_int32), ("n_chains", C.c_int32), ("mutation", C.c_int32),
                ("large_step_prob", C.c_float), ("sigma", C.c_float), ("eps_min", C.c_float),
                ("eps_max", C.c_float), ("block_size", C.c_int32), ("queue_capacity", C.c_int32),
                ("pad_", C.c_int32)]


class bn_stats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("rays", C.c_uint64), ("nodes_visited", C.c_uint64),
                ("tris_tested", C.c_uint64), ("instances_visited", C.c_uint64), ("accepted", C.c_uint64),
                ("proposed", C.c_uint64), ("bootstrap_b", C.c_double), ("device_error", C.c_uint32),
                ("last_kernel_ms", C.c_float), ("last_dominant_ms", C.c_float), ("last_launches", C.c_int32)]


class bn_adjoint_desc(C.Structure):
    _fields_ = [("n_slots", C.c_int32), ("emissive_slot_base", C.c_int32), ("width", C.c_int32),
                ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32), ("rr_depth", C.c_int32),
                ("frame_id", C.c_int32), ("freeze_sampling", C.c_int32), ("pad_", C.c_int32),
                ("camera", bn_camera_desc)]


class bn_bvh_node(C.Structure):
    _fields_ = [("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3), ("right_or_offset", C.c_int32),
                ("is_leaf", C.c_uint8), ("split_axis", C.c_int8), ("count", C.c_int8),
                ("visibility_mask", C.c_uint8)]


class bn_bundle_info(C.Structure):
    _fields_ = [("scene", C.POINTER(bn_scene_desc)), ("views", C.POINTER(bn_view)), ("n_views", C.c_int32),
                ("render", bn_render_desc), ("n_triangles_unique", C.c_int64),
                ("n_triangles_instanced", C.c_int64), ("n_material_slots", C.c_int32),
                ("emissive_slot_base", C.c_int32), ("slot_params", C.POINTER(C.c_float)),
                ("tone_mapping", C.c_int32)]


# numpy dtypes matching the C structures (for bulk arrays)
RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("direction", "<f4", 3), ("t_max", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("instance", "<i4"), ("primitive", "<i4"),
                      ("normal", "<f4", 3), ("position", "<f4", 3)])
BSDF_QUERY_DTYPE = np.dtype([("material", "<i4"), ("wo", "<f4", 3), ("wi", "<f4", 3), ("u_lobe", "<f4"),
                             ("u_bsdf", "<f4", 2)])
BSDF_RESULT_DTYPE = np.dtype([("bsdf", "<f4", 3), ("pdf", "<f4"), ("wi", "<f4", 3)])
NODE_DTYPE = np.dtype([("bounds_min", "<f4", 3), ("bounds_max", "<f4", 3), ("right_or_offset", "<i4"),
                       ("is_leaf", "u1"), ("split_axis", "i1"), ("count", "i1"), ("visibility_mask", "u1")])
assert RAY_DTYPE.itemsize == C.sizeof(bn_ray)
assert HIT_DTYPE.itemsize == C.sizeof(bn_hit)
assert BSDF_QUERY_DTYPE.itemsize == C.sizeof(bn_bsdf_query)
assert BSDF_RESULT_DTYPE.itemsize == C.sizeof(bn_bsdf_result)
assert NODE_DTYPE.itemsize == C.sizeof(bn_bvh_node) == 32

# every entry point include/barnacle_gpu.h declares, with its ctypes signature
P = C.c_void_p
SIGNATURES = {
    "bn_version": (C.c_char_p, []),
    "bn_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "bn_destroy": (C.c_int, [P]),
    "bn_last_error": (C.c_int, [P, C.c_char_p, C.c_size_t]),
    "bn_scene_upload": (C.c_int, [P, C.POINTER(bn_scene_desc)]),
    "bn_scene_instance_order": (C.c_int, [P, P, C.c_int32]),
    "bn_trace": (C.c_int, [P, P, C.c_int64, C.c_uint32, P]),
    "bn_bsdf_eval": (C.c_int, [P, P, C.c_int64, P]),
    "bn_bsdf_sample": (C.c_int, [P, P, C.c_int64, P]),
    "bn_sampler_stream": (C.c_int, [P, P, C.c_int64, C.c_int32, P]),
    "bn_render": (C.c_int, [P, C.POINTER(bn_render_desc), C.POINTER(bn_view), C.c_int32, P]),
    "bn_film_download": (C.c_int, [P, P, C.c_int64]),
    "bn_film_tonemap": (C.c_int, [P, C.c_int32, P, C.c_int64]),
    "bn_image_write_png": (C.c_int, [C.c_char_p, P, C.c_int32, C.c_int32]),
    "bn_render_noalloc": (C.c_int, [P, C.POINTER(bn_render_desc), C.POINTER(bn_view), C.c_int32, P]),
    "bn_set_limits": (C.c_int, [P, C.c_int32, C.c_int32]),
    "bn_get_stats": (C.c_int, [P, C.POINTER(bn_stats)]),
    "bn_reset_stats": (C.c_int, [P]),
    "bn_forward": (C.c_int, [P, C.POINTER(bn_adjoint_desc), P, P, P]),
    "bn_backward": (C.c_int, [P, C.POINTER(bn_adjoint_desc), P, P, P, P, P]),
    "bn_bvh_build": (C.c_int, [P, C.c_int32, P, P, P]),
    "bn_bvh_build_device": (C.c_int, [P, P, C.c_int32, P, P, P]),
    "bn_mat4_invert": (C.c_int, [P, P]),
    "bn_bundle_generate": (C.c_int, [C.c_char_p, C.c_uint32, C.POINTER(P)]),
    "bn_bundle_load_json": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "bn_bundle_info_get": (C.c_int, [P, C.POINTER(bn_bundle_info)]),
    "bn_bundle_free": (C.c_int, [P]),
    "bn_host_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
}

_lib = None


def load_library() -> C.CDLL:
    """Loads the in-tree library; raises if it was not built (no CPU fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    _lib = bind(C.CDLL(str(LIB_PATH)))
    return _lib


def bind(lib: C.CDLL) -> C.CDLL:
    """Declares the signatures of every entry point the library exports (a library built from
    the host sources alone exports the scene and BVH helpers only)."""
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is not None:
            fn.restype = res
            fn.argtypes = args
    return lib


def ptr(a: np.ndarray | None) -> C.c_void_p:
    if a is None:
        return C.c_void_p()
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the C-ABI must be C-contiguous"
    return C.c_void_p(a.ctypes.data)


class BarnacleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def host_error() -> str:
    buf = C.create_string_buffer(1024)
    load_library().bn_host_last_error(buf, 1024)
    return buf.value.decode(errors="replace")
