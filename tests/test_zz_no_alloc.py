"""bn_render_noalloc: the render entry point for callers that cannot allocate device memory
during a render (their device memory comes from their own arena, or their frame loop must not
call cudaMalloc).  The test plays such a caller: it owns the film buffer (allocated up front, here
with torch) and renders into it twice in a row through the C-ABI; each result must equal what
bn_render produces for the same frame.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from barnacle_gb300 import Bundle, Context, capi

pytestmark = pytest.mark.gpu


def test_render_noalloc_matches_render_twice():
    torch = pytest.importorskip("torch")
    with Context(0) as ctx:
        b = Bundle.generate("cornell", 1)
        ctx.upload(b)
        v = b.views[0]
        r = b.render
        r.spp = 16
        film = torch.zeros(v.width * v.height * 3, dtype=torch.float32, device="cuda:0")
        views = (capi.bn_view * 1)(v)
        for frame in (0, 1):
            r.frame_id = frame
            want = ctx.render(r, v)[0]
            rc = ctx.lib.bn_render_noalloc(ctx._h, C.byref(r), views, 1, C.c_void_p(film.data_ptr()))
            assert rc == capi.BN_OK, ctx.error()
            torch.cuda.synchronize()
            got = film.cpu().numpy().reshape(v.height, v.width, 3)
            # same kernels, same sample chunks, same summation order: identical floats
            np.testing.assert_array_equal(got, want)
            assert got.max() > 1.0


def test_render_noalloc_rejects_oversize_and_unsupported():
    torch = pytest.importorskip("torch")
    with Context(0) as ctx:
        b = Bundle.generate("cornell", 1)
        ctx.upload(b)
        r = b.render
        r.spp = 1
        v = b.views[0]
        v.width, v.height = 1280, 1024  # 1,310,720 pixels: beyond the 1,048,576 limit
        film = torch.zeros(4, dtype=torch.float32, device="cuda:0")
        views = (capi.bn_view * 1)(v)
        rc = ctx.lib.bn_render_noalloc(ctx._h, C.byref(r), views, 1, C.c_void_p(film.data_ptr()))
        assert rc == capi.BN_ERR_INVALID_ARG and "limit" in ctx.error()
        r.mode = capi.BN_MODE_WAVEFRONT
        v.width, v.height = 8, 8
        views = (capi.bn_view * 1)(v)
        rc = ctx.lib.bn_render_noalloc(ctx._h, C.byref(r), views, 1, C.c_void_p(film.data_ptr()))
        assert rc == capi.BN_ERR_UNSUPPORTED
