"""barnacle_gb300 — a GB300 (sm_103a) path-tracing core behind the render call of the Barnacle
F# renderer.  The product is libbarnacle_gb300.so (include/barnacle_gpu.h); this package holds
its build script and a thin ctypes layer."""
from .api import Bundle, Context, bvh_build, mat4_invert, write_png  # noqa: F401
from .capi import BarnacleError, load_library  # noqa: F401

__all__ = ["Bundle", "Context", "BarnacleError", "bvh_build", "mat4_invert", "write_png", "load_library"]
