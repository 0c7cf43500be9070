"""Film output on the device (Film.PostProcess + the Rgba32 packing of Film.Save) against the
oracle's restatement applied to the same float film."""
import zlib

import numpy as np
import pytest

from barnacle_gb300 import BarnacleError, Bundle, capi, write_png
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def test_tonemap_matches_oracle_on_two_views(ctx, tmp_path):
    b = Bundle.generate("instances", 1)
    ctx.upload(b)
    r = b.render
    r.spp = 1
    views = b.views[:2]
    imgs = ctx.render(r, views)
    for tm in (capi.BN_TONE_IDENTITY, capi.BN_TONE_ACES, capi.BN_TONE_GAMMA):
        got = ctx.tonemap(tm, views)
        for g, f in zip(got, imgs):
            want = pyoracle.tonemap(f, tm)
            assert g.shape == want.shape and (g[..., 3] == 255).all()
            d = np.abs(g.astype(int) - want.astype(int))
            if tm == capi.BN_TONE_GAMMA:  # powf: the device and the C library may differ by an ulp
                assert d.max() <= 1 and (d > 0).mean() < 1e-3
            else:
                assert d.max() == 0, f"{(d > 0).sum()} bytes differ"
    # the encoded image decodes to the device's bytes
    rgba = ctx.tonemap(b.tone_mapping, views[0])[0]
    p = tmp_path / "v0.png"
    write_png(p, rgba)
    data = p.read_bytes()
    idat = data[data.index(b"IDAT") + 4:data.index(b"IEND") - 8]
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(rgba.shape[0], -1)
    assert np.array_equal(raw[:, 1:].reshape(rgba.shape), rgba)


def test_tonemap_errors(ctx):
    b = Bundle.generate("cornell", 1)
    ctx.upload(b)
    r = b.render
    r.spp = 1
    ctx.render(r, b.views[0])
    n = b.views[0].width * b.views[0].height
    out = np.zeros(4 * n, np.uint8)
    tonemap = ctx.lib.bn_film_tonemap
    assert tonemap(ctx._h, capi.BN_TONE_ACES, None, n) == capi.BN_ERR_INVALID_ARG
    assert tonemap(ctx._h, capi.BN_TONE_ACES, out.ctypes.data, n + 1) == capi.BN_ERR_INVALID_ARG
    assert tonemap(ctx._h, capi.BN_TONE_ACES, out.ctypes.data, 0) == capi.BN_ERR_INVALID_ARG
    assert tonemap(ctx._h, 9, out.ctypes.data, n) == capi.BN_ERR_INVALID_ARG
    assert tonemap(ctx._h, capi.BN_TONE_ACES, out.ctypes.data, n) == capi.BN_OK
    with pytest.raises(BarnacleError):
        write_png("/nonexistent-dir/x.png", out.reshape(-1, b.views[0].width, 4))
