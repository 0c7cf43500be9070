"""bn_render_noalloc: the render entry point for callers that cannot allocate device memory
during a render (their device memory comes from their own arena, or their frame loop must not
call cudaMalloc, which synchronises the device).  The tests play such a caller: it owns the film
buffer (allocated up front, here with torch) and renders into it several times in a row through
the C-ABI; each result must equal what bn_render produces for the same frame, and the GPU's free
memory must not change across a call once the first call on the device has done its set-up.
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from barnacle_gb300 import Bundle, Context, capi

pytestmark = pytest.mark.gpu


def _noalloc(ctx, r, views, film):
    arr = (capi.bn_view * len(views))(*views)
    return ctx.lib.bn_render_noalloc(ctx._h, C.byref(r), arr, len(views), C.c_void_p(film.data_ptr()))


def _film_image(film, views):
    out, off = [], 0
    host = film.cpu().numpy()
    for v in views:
        n = v.width * v.height * 3
        out.append(host[off:off + n].reshape(v.height, v.width, 3))
        off += n
    return out


def test_render_noalloc_matches_render_twice():
    torch = pytest.importorskip("torch")
    with Context(0) as ctx:
        b = Bundle.generate("cornell", 1)
        ctx.upload(b)
        v = b.views[0]
        r = b.render
        r.spp = 16  # 65,536 pixels x 16 chunks: exactly the 1,048,576 partial sums, no longer chunks
        film = torch.zeros(v.width * v.height * 3, dtype=torch.float32, device="cuda:0")
        for frame in (0, 1):
            r.frame_id = frame
            want = ctx.render(r, v)[0]
            rc = _noalloc(ctx, r, [v], film)
            assert rc == capi.BN_OK, ctx.error()
            torch.cuda.synchronize()
            got = _film_image(film, [v])[0]
            # same kernels, same sample chunks, same summation order: identical floats
            np.testing.assert_array_equal(got, want)
            assert got.max() > 1.0


def test_render_noalloc_allocates_nothing():
    """After the first call on the device (which resolves the static array's address), further
    calls leave the GPU's free memory exactly where it was."""
    torch = pytest.importorskip("torch")
    with Context(0) as ctx:
        b = Bundle.generate("cornell", 1)
        ctx.upload(b)
        v = b.views[0]
        r = b.render
        r.spp = 8
        film = torch.zeros(v.width * v.height * 3, dtype=torch.float32, device="cuda:0")
        r.frame_id = 0
        assert _noalloc(ctx, r, [v], film) == capi.BN_OK, ctx.error()
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info(0)
        for frame in (1, 2):
            r.frame_id = frame
            assert _noalloc(ctx, r, [v], film) == capi.BN_OK, ctx.error()
            torch.cuda.synchronize()
            free1, _ = torch.cuda.mem_get_info(0)
            assert free1 == free0, f"free device memory changed by {free0 - free1} bytes across a call"


def test_render_noalloc_three_views():
    torch = pytest.importorskip("torch")
    with Context(0) as ctx:
        b = Bundle.generate("cornell", 1)
        ctx.upload(b)
        base = b.views[0]
        views = []
        for w, h in ((256, 256), (128, 96), (64, 64)):
            v = capi.bn_view.from_buffer_copy(base)
            v.width, v.height = w, h
            views.append(v)
        r = b.render
        r.spp = 8  # 81,920 pixels x 8 chunks fit the partial sums: bit-identical
        film = torch.zeros(sum(v.width * v.height for v in views) * 3, dtype=torch.float32, device="cuda:0")
        for frame in (3, 4):
            r.frame_id = frame
            want = ctx.render(r, views)
            assert _noalloc(ctx, r, views, film) == capi.BN_OK, ctx.error()
            torch.cuda.synchronize()
            for g, w in zip(_film_image(film, views), want):
                np.testing.assert_array_equal(g, w)


def test_render_noalloc_longer_chunks():
    """512x512 at 64 spp: bn_render sums each pixel in 5 chunks of 13 samples, which would need
    1,310,720 partial sums; the static array holds 1,048,576, so this call sums 4 chunks of 16.
    The per-path radiance is the same, so the images agree to float summation order."""
    torch = pytest.importorskip("torch")
    with Context(0) as ctx:
        b = Bundle.generate("cornell", 1)
        ctx.upload(b)
        v = capi.bn_view.from_buffer_copy(b.views[0])
        v.width, v.height = 512, 512
        r = b.render
        r.spp = 64
        film = torch.zeros(v.width * v.height * 3, dtype=torch.float32, device="cuda:0")
        for frame in (5, 6):
            r.frame_id = frame
            want = ctx.render(r, v)[0]
            assert _noalloc(ctx, r, [v], film) == capi.BN_OK, ctx.error()
            torch.cuda.synchronize()
            got = _film_image(film, [v])[0]
            assert got.max() > 1.0
            np.testing.assert_allclose(got, want, rtol=2e-5, atol=1e-6)


def test_render_noalloc_rejects_oversize_and_unsupported():
    torch = pytest.importorskip("torch")
    with Context(0) as ctx:
        b = Bundle.generate("cornell", 1)
        ctx.upload(b)
        r = b.render
        r.spp = 1
        v = capi.bn_view.from_buffer_copy(b.views[0])
        v.width, v.height = 1280, 1024  # 1,310,720 pixels: beyond the 1,048,576 limit
        film = torch.zeros(8 * 8 * 3, dtype=torch.float32, device="cuda:0")
        rc = _noalloc(ctx, r, [v], film)
        assert rc == capi.BN_ERR_INVALID_ARG and "limit" in ctx.error()
        v.width, v.height = 8, 8
        r.mode = capi.BN_MODE_WAVEFRONT
        assert _noalloc(ctx, r, [v], film) == capi.BN_ERR_UNSUPPORTED
        r.mode = capi.BN_MODE_MEGAKERNEL
        r.flags |= capi.BN_RENDER_COUNT
        assert _noalloc(ctx, r, [v], film) == capi.BN_ERR_UNSUPPORTED
        r.flags &= ~capi.BN_RENDER_COUNT
        # a host buffer is rejected before anything runs on the GPU
        host = torch.zeros(8 * 8 * 3, dtype=torch.float32)
        rc = _noalloc(ctx, r, [v], host)
        assert rc == capi.BN_ERR_INVALID_ARG and "device memory" in ctx.error()
        # and the context still renders afterwards
        assert _noalloc(ctx, r, [v], film) == capi.BN_OK, ctx.error()
