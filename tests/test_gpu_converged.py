"""Images against a converged reference: the oracle renders a crop at 65,536 samples per pixel
(spread over threads as independent sample ranges, averaged in FP64); the device's per-pixel means
over 64 frames must lie within 3 standard errors of it, and at equal samples per pixel the device
image's RMSE against it must be within 2% of the oracle's own."""
from concurrent.futures import ThreadPoolExecutor
import os

import numpy as np
import pytest

from barnacle_gb300 import Bundle, capi
from oracle import pyoracle

pytestmark = pytest.mark.gpu

FRAMES, SPP, CONVERGED = 64, 256, 65536


def oracle_frames(o, r, v, crop, spp, frame_ids):
    """One oracle render of the crop per frame id (each one host thread: a crop of one 16x16
    tile), run concurrently."""
    def one(f):
        rr = capi.bn_render_desc.from_buffer_copy(r)
        rr.spp = spp
        rr.frame_id = f
        return o.render_pt(rr, v, crop=crop, threads=1)[0]
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        return list(ex.map(one, frame_ids))


_CONVERGED = {}


def converged(name, o, r, v, crop):
    """16 independent 4,096-spp ranges (frame ids far from the test frames), averaged in FP64;
    computed once per scene and crop."""
    key = (name, crop)
    if key not in _CONVERGED:
        frames = oracle_frames(o, r, v, crop, CONVERGED // 16, range(100000, 100016))
        _CONVERGED[key] = crop_of(np.mean(np.stack(frames), 0, dtype=np.float64), v, crop)
    return _CONVERGED[key]


def crop_of(img, v, crop):
    x0, y0, x1, y1 = crop
    return img[v.height - y1:v.height - y0, x0:x1]  # Film.Pixels rows are flipped


@pytest.mark.parametrize("name,crop,mode,check_rmse", [
    ("cornell", (96, 120, 112, 136), capi.BN_MODE_MEGAKERNEL, True),
    ("cornell", (96, 120, 112, 136), capi.BN_MODE_WAVEFRONT, True),
    ("cornell-objects", (240, 260, 252, 272), capi.BN_MODE_MEGAKERNEL, False),
])
def test_device_image_against_converged_oracle(ctx, name, crop, mode, check_rmse):
    b = Bundle.generate(name, 1)
    ctx.upload(b)
    o = pyoracle.Scene(b.scene)
    r = b.render
    r.mode = mode
    v = b.views[0]
    conv = converged(name, o, r, v, crop)
    r.spp = SPP
    gpu = []
    for f in range(FRAMES):
        r.frame_id = f
        gpu.append(crop_of(ctx.render(r, v)[0], v, crop))
    g = np.stack(gpu).astype(np.float64)
    se = g.std(0, ddof=1) / np.sqrt(FRAMES)
    z = np.abs(g.mean(0) - conv) / np.maximum(se, 1e-12)
    assert conv.mean() > 0.01
    assert (z[se > 0] > 3).mean() < 0.02, f"{(z[se > 0] > 3).mean():.3%} of means beyond 3 standard errors"
    if check_rmse:
        cpu = np.stack([crop_of(c, v, crop) for c in
                        oracle_frames(o, r, v, crop, SPP, range(5000, 5000 + FRAMES))]).astype(np.float64)
        rmse_gpu = np.sqrt(((g - conv) ** 2).mean())
        rmse_cpu = np.sqrt(((cpu - conv) ** 2).mean())
        assert abs(rmse_gpu / rmse_cpu - 1) < 0.02, f"RMSE {rmse_gpu:.5f} (device) vs {rmse_cpu:.5f} (oracle)"
