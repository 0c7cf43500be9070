"""ORACLE — test infrastructure only.  ctypes binding of the CPU restatement
(oracle/_build/libbarnacle_oracle.so).  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker; the product never loads it."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from barnacle_gb300 import capi
from barnacle_gb300.capi import ptr

from . import build as _build

P = C.c_void_p
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        sig = {
            "or_scene_create": (C.c_int, [C.POINTER(capi.bn_scene_desc), C.POINTER(P)]),
            "or_scene_free": (None, [P]),
            "or_scene_tlas": (C.c_int, [P, P, P, P]),
            "or_scene_blas": (C.c_int, [P, C.c_int32, P, P, P]),
            "or_bvh_build": (C.c_int, [P, C.c_int32, P, P, P]),
            "or_trace": (C.c_int, [P, P, C.c_int64, C.c_uint32, P, P]),
            "or_sampler_stream": (C.c_int, [P, C.c_int64, C.c_int32, P]),
            "or_tonemap": (C.c_int, [P, C.c_int64, C.c_int32, P]),
            "or_xxhash32_two": (C.c_uint32, [C.c_uint32, C.c_uint32]),
            "or_xxhash32_three": (C.c_uint32, [C.c_uint32, C.c_uint32, C.c_uint32]),
            "or_bsdf": (C.c_int, [P, P, C.c_int64, C.c_int, C.c_int, P]),
            "or_render_pt": (C.c_int, [P, C.POINTER(capi.bn_render_desc), C.POINTER(capi.bn_view), C.c_int32,
                                       C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P]),
            "or_render_slots": (C.c_int, [P, C.POINTER(capi.bn_render_desc), C.POINTER(capi.bn_view), C.c_int32,
                                          C.c_int32, P, P, C.c_int32, P]),
            "or_render_pssmlt": (C.c_int, [P, C.POINTER(capi.bn_render_desc), C.POINTER(capi.bn_view), C.c_int32,
                                           P, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


_scenes = None


def scenes_library() -> C.CDLL:
    """The host-side scene code (procedural workloads, JSON loader) built without CUDA, for the
    CPU arms: Bundle.generate(name, seed, lib=scenes_library())."""
    global _scenes
    if _scenes is None:
        _scenes = capi.bind(C.CDLL(str(_build.build_scenes())))
    return _scenes


def bvh_build(bounds: np.ndarray):
    b = np.ascontiguousarray(bounds, np.float32).reshape(-1, 6)
    n = len(b)
    nodes = np.zeros(max(2 * n, 1), capi.NODE_DTYPE)
    nn = C.c_int32()
    perm = np.zeros(max(n, 1), np.int32)
    lib().or_bvh_build(ptr(b), n, ptr(nodes), C.byref(nn), ptr(perm))
    return nodes[: nn.value], perm[:n]


def sampler_stream(seeds: np.ndarray, n_draws: int) -> np.ndarray:
    s = np.ascontiguousarray(seeds, np.uint32).reshape(-1, 3)
    out = np.zeros((len(s), n_draws), np.float32)
    lib().or_sampler_stream(ptr(s), len(s), n_draws, ptr(out))
    return out


def tonemap(rgb: np.ndarray, tone_mapping: int) -> np.ndarray:
    """Film.PostProcess + Rgba32 packing: (..., 3) float32 -> (..., 4) uint8."""
    x = np.ascontiguousarray(rgb, np.float32)
    out = np.zeros(x.shape[:-1] + (4,), np.uint8)
    if lib().or_tonemap(ptr(x), x.size // 3, tone_mapping, ptr(out)):
        raise ValueError("unknown tone mapping")
    return out


def bsdf(materials, queries: np.ndarray, sample: bool, use_double: bool) -> np.ndarray:
    """materials: list of capi.bn_material_desc; returns (n, 7): bsdf rgb, pdf, wi xyz."""
    mats = (capi.bn_material_desc * len(materials))(*materials)
    q = np.ascontiguousarray(queries, capi.BSDF_QUERY_DTYPE)
    out = np.zeros((len(q), 7), np.float64)
    lib().or_bsdf(C.cast(mats, P), ptr(q), len(q), int(sample), int(use_double), ptr(out))
    return out


class Scene:
    def __init__(self, scene_desc):
        self._h = P()
        rc = lib().or_scene_create(scene_desc, C.byref(self._h))
        assert rc == 0
        self.n_instances = scene_desc.contents.n_instances

    def __del__(self):
        if getattr(self, "_h", None):
            lib().or_scene_free(self._h)
            self._h = None

    def tlas(self):
        nodes = np.zeros(2 * self.n_instances + 1, capi.NODE_DTYPE)
        nn = C.c_int32()
        order = np.zeros(self.n_instances, np.int32)
        lib().or_scene_tlas(self._h, ptr(nodes), C.byref(nn), ptr(order))
        return nodes[: nn.value], order

    def blas(self, mesh: int, n_tris: int):
        nodes = np.zeros(2 * n_tris + 1, capi.NODE_DTYPE)
        nn = C.c_int32()
        perm = np.zeros(max(n_tris, 1), np.int32)
        lib().or_scene_blas(self._h, mesh, ptr(nodes), C.byref(nn), ptr(perm))
        return nodes[: nn.value], perm[:n_tris]

    def trace(self, rays: np.ndarray, flags: int = 0):
        rays = np.ascontiguousarray(rays, capi.RAY_DTYPE)
        hits = np.zeros(len(rays), capi.HIT_DTYPE)
        counts = np.zeros(4, np.uint64)
        lib().or_trace(self._h, ptr(rays), len(rays), flags, ptr(hits), ptr(counts))
        return hits, counts

    def render_pt(self, desc, view, crop=None, threads: int | None = None):
        """Renders a crop (x0, y0, x1, y1) of the view; returns the (H, W, 3) film and
        counters [rays, nodes, triangles, instances]."""
        W, H = view.width, view.height
        x0, y0, x1, y1 = crop if crop else (0, 0, W, H)
        out = np.zeros((H, W, 3), np.float32)
        counts = np.zeros(4, np.uint64)
        threads = threads or os.cpu_count() or 1
        lib().or_render_pt(self._h, C.byref(desc), C.byref(view), x0, y0, x1, y1, threads, ptr(out), ptr(counts))
        return out, counts

    def render_pssmlt(self, desc, view, threads: int | None = None):
        """PSSMLTIntegrator.Render: returns (film (H, W, 3), b, accepted, proposed, bootstrap y)."""
        out = np.zeros((view.height, view.width, 3), np.float32)
        stats = np.zeros(3, np.float64)
        boot = np.zeros(max(desc.n_bootstrap, 1), np.float32)
        threads = threads or os.cpu_count() or 1
        lib().or_render_pssmlt(self._h, C.byref(desc), C.byref(view), threads, ptr(out), ptr(stats), ptr(boot))
        return out, float(stats[0]), int(stats[1]), int(stats[2]), boot

    def render_slots(self, desc, view, n_slots, emissive_base, params, sparams=None, threads: int | None = None):
        """Forward render with material slots from params (sampling from sparams, default params)."""
        out = np.zeros((view.height, view.width, 3), np.float32)
        prm = np.ascontiguousarray(params, np.float32)
        sp = prm if sparams is None else np.ascontiguousarray(sparams, np.float32)
        threads = threads or os.cpu_count() or 1
        lib().or_render_slots(self._h, C.byref(desc), C.byref(view), n_slots, emissive_base, ptr(prm), ptr(sp),
                              threads, ptr(out))
        return out
