"""Thin Python layer over the C-ABI: scene bundles (procedural workloads and the reference JSON
loader) and a device context (upload, ray queries, BSDF queries, render).

Every call goes through libbarnacle_gb300.so; errors come back as BarnacleError with the
library's message.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import BarnacleError, ptr


class Bundle:
    """A library-owned scene description plus its render settings (bn_scene_bundle)."""

    def __init__(self, handle: C.c_void_p, lib: C.CDLL | None = None):
        self._lib = lib or capi.load_library()
        self._h = handle
        self._info = capi.bn_bundle_info()
        rc = self._lib.bn_bundle_info_get(self._h, C.byref(self._info))
        if rc:
            raise BarnacleError(rc, capi.host_error())

    @classmethod
    def generate(cls, name: str, seed: int = 1, lib: C.CDLL | None = None) -> "Bundle":
        """lib: the library whose host code builds the scene (default the GPU library)."""
        lib = lib or capi.load_library()
        h = C.c_void_p()
        rc = lib.bn_bundle_generate(name.encode(), seed, C.byref(h))
        if rc:
            buf = C.create_string_buffer(1024)
            lib.bn_host_last_error(buf, 1024)
            raise BarnacleError(rc, buf.value.decode(errors="replace"))
        return cls(h, lib)

    @classmethod
    def load_json(cls, path: str) -> "Bundle":
        h = C.c_void_p()
        rc = capi.load_library().bn_bundle_load_json(str(path).encode(), C.byref(h))
        if rc:
            raise BarnacleError(rc, capi.host_error())
        return cls(h)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.bn_bundle_free(self._h)
            self._h = None

    @property
    def scene(self) -> "C.POINTER(capi.bn_scene_desc)":
        return self._info.scene

    @property
    def views(self) -> list:
        return [self._info.views[i] for i in range(self._info.n_views)]

    def views_array(self):
        arr = (capi.bn_view * self._info.n_views)()
        for i in range(self._info.n_views):
            arr[i] = self._info.views[i]
        return arr

    @property
    def render(self) -> capi.bn_render_desc:
        r = capi.bn_render_desc()
        C.pointer(r)[0] = self._info.render
        return r

    @property
    def n_triangles_unique(self) -> int:
        return int(self._info.n_triangles_unique)

    @property
    def n_triangles_instanced(self) -> int:
        return int(self._info.n_triangles_instanced)

    @property
    def n_slots(self) -> int:
        return int(self._info.n_material_slots)

    @property
    def emissive_slot_base(self) -> int:
        return int(self._info.emissive_slot_base)

    @property
    def tone_mapping(self) -> int:
        """capi.BN_TONE_*: the film's tone mapping (JSON "tone-mapping", ACES for procedural scenes)."""
        return int(self._info.tone_mapping)

    def slot_params(self) -> np.ndarray | None:
        if self.n_slots == 0:
            return None
        return np.ctypeslib.as_array(self._info.slot_params, shape=(self.n_slots * 6,)).copy()

    def materials(self) -> list:
        s = self.scene.contents
        return [s.materials[i] for i in range(s.n_materials)]


class Context:
    """A device context (bn_context) on one GPU with its own CUDA stream."""

    def __init__(self, device: int = 0):
        self.lib = capi.load_library()
        self._h = C.c_void_p()
        rc = self.lib.bn_create(device, C.byref(self._h))
        if rc:
            raise BarnacleError(rc, f"bn_create(device={device}) failed")

    def close(self):
        if getattr(self, "_h", None):
            self.lib.bn_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def error(self) -> str:
        buf = C.create_string_buffer(2048)
        self.lib.bn_last_error(self._h, buf, 2048)
        return buf.value.decode(errors="replace")

    def _check(self, rc: int):
        if rc:
            raise BarnacleError(rc, self.error())

    def upload(self, scene) -> None:
        """scene: a Bundle or a POINTER(bn_scene_desc)."""
        desc = scene.scene if isinstance(scene, Bundle) else scene
        self._check(self.lib.bn_scene_upload(self._h, desc))

    def instance_order(self, n: int) -> np.ndarray:
        out = np.zeros(n, np.int32)
        self._check(self.lib.bn_scene_instance_order(self._h, ptr(out), n))
        return out

    def trace(self, rays: np.ndarray, flags: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=capi.RAY_DTYPE)
        hits = np.zeros(len(rays), capi.HIT_DTYPE)
        self._check(self.lib.bn_trace(self._h, ptr(rays), len(rays), flags, ptr(hits)))
        return hits

    def bsdf(self, queries: np.ndarray, sample: bool) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=capi.BSDF_QUERY_DTYPE)
        out = np.zeros(len(q), capi.BSDF_RESULT_DTYPE)
        fn = self.lib.bn_bsdf_sample if sample else self.lib.bn_bsdf_eval
        self._check(fn(self._h, ptr(q), len(q), ptr(out)))
        return out

    def sampler_stream(self, seeds: np.ndarray, n_draws: int) -> np.ndarray:
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(-1, 3)
        out = np.zeros((len(seeds), n_draws), np.float32)
        self._check(self.lib.bn_sampler_stream(self._h, ptr(seeds), len(seeds), n_draws, ptr(out)))
        return out

    def render(self, desc: capi.bn_render_desc, views, to_host: bool = True) -> list | None:
        """Renders every view; returns one (H, W, 3) float32 image per view (Film.Pixels order)."""
        if isinstance(views, capi.bn_view):
            views = [views]
        arr = (capi.bn_view * len(views))(*views)
        total = sum(v.width * v.height * 3 for v in views)
        out = np.zeros(total, np.float32) if to_host else None
        self._check(self.lib.bn_render(self._h, C.byref(desc), arr, len(views), ptr(out)))
        if not to_host:
            return None
        imgs, off = [], 0
        for v in views:
            n = v.width * v.height * 3
            imgs.append(out[off:off + n].reshape(v.height, v.width, 3))
            off += n
        return imgs

    def bvh_build(self, bounds: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """BVHNode.Build on this context's GPU: the same (nodes, permutation) as bvh_build."""
        b = np.ascontiguousarray(bounds, np.float32).reshape(-1, 6)
        n = len(b)
        nodes = np.zeros(max(2 * n, 1), capi.NODE_DTYPE)
        nn = C.c_int32()
        perm = np.zeros(max(n, 1), np.int32)
        self._check(self.lib.bn_bvh_build_device(self._h, ptr(b), n, ptr(nodes), C.byref(nn), ptr(perm)))
        return nodes[: nn.value], perm[:n]

    def film_download(self, out: np.ndarray) -> None:
        self._check(self.lib.bn_film_download(self._h, ptr(out), out.size))

    def tonemap(self, tone_mapping: int, views) -> list:
        """Film.PostProcess + 8-bit packing of the last render's film on the device: one
        (H, W, 4) uint8 RGBA image per view (rows top to bottom, as Film.Save writes them)."""
        if isinstance(views, capi.bn_view):
            views = [views]
        n = sum(v.width * v.height for v in views)
        out = np.zeros(n * 4, np.uint8)
        self._check(self.lib.bn_film_tonemap(self._h, tone_mapping, ptr(out), n))
        imgs, off = [], 0
        for v in views:
            k = v.width * v.height * 4
            imgs.append(out[off:off + k].reshape(v.height, v.width, 4))
            off += k
        return imgs

    def stats(self) -> capi.bn_stats:
        s = capi.bn_stats()
        self._check(self.lib.bn_get_stats(self._h, C.byref(s)))
        return s

    def reset_stats(self) -> None:
        self._check(self.lib.bn_reset_stats(self._h))

    def forward(self, desc: capi.bn_adjoint_desc, params: np.ndarray, sampling_params: np.ndarray | None = None) -> np.ndarray:
        params = np.ascontiguousarray(params, np.float32)
        sp = None if sampling_params is None else np.ascontiguousarray(sampling_params, np.float32)
        out = np.zeros((desc.height, desc.width, 3), np.float32)
        self._check(self.lib.bn_forward(self._h, C.byref(desc), ptr(params), ptr(sp), ptr(out)))
        return out

    def backward(self, desc: capi.bn_adjoint_desc, params: np.ndarray, target: np.ndarray,
                 sampling_params: np.ndarray | None = None) -> tuple[np.ndarray, float]:
        params = np.ascontiguousarray(params, np.float32)
        sp = None if sampling_params is None else np.ascontiguousarray(sampling_params, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        grad = np.zeros(params.size, np.float64)
        loss = np.zeros(1, np.float64)
        self._check(self.lib.bn_backward(self._h, C.byref(desc), ptr(params), ptr(sp), ptr(target), ptr(grad),
                                         ptr(loss)))
        return grad, float(loss[0])


def bvh_build(bounds: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """BVHNode.Build over n boxes (n x 6: min xyz, max xyz): (nodes, permutation)."""
    b = np.ascontiguousarray(bounds, np.float32).reshape(-1, 6)
    n = len(b)
    nodes = np.zeros(max(2 * n, 1), capi.NODE_DTYPE)
    nn = C.c_int32()
    perm = np.zeros(max(n, 1), np.int32)
    rc = capi.load_library().bn_bvh_build(ptr(b), n, ptr(nodes), C.byref(nn), ptr(perm))
    if rc:
        raise BarnacleError(rc, capi.host_error())
    return nodes[: nn.value], perm[:n]


def mat4_invert(m: np.ndarray) -> np.ndarray:
    m = np.ascontiguousarray(m, np.float32).reshape(16)
    out = np.zeros(16, np.float32)
    capi.load_library().bn_mat4_invert(ptr(m), ptr(out))
    return out


def write_png(path: str, rgba: np.ndarray) -> None:
    """An (H, W, 4) uint8 image as a PNG file."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w = img.shape[:2]
    rc = capi.load_library().bn_image_write_png(str(path).encode(), ptr(img), w, h)
    if rc:
        raise BarnacleError(rc, capi.host_error())
