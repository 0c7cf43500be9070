"""The reference's own scene, cbox.json (Asset/cbox.json), rendered unchanged on the GPU: loaded
through bn_bundle_load_json (Scene.Load, Extensions/Scene/Loader.fs:241-281), rendered with the
integrator the file names (PSSMLT, 16 mutations per pixel, depth 8) and with the path tracer, tone
mapped on the device with ACES (Film.PostProcess, Base/Film.fs:21-30) and compared with the two
sample images the reference ships.  Crops of its path-traced image are also checked against
converged oracle images in test_gpu_converged.py."""
import numpy as np
import pytest

from barnacle_gb300 import Bundle, capi
from cbox_common import CBOX, PSNR_MIN, block_means, psnr, samples

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cbox():
    return Bundle.load_json(str(CBOX))


def _render_tonemapped(ctx, r, v):
    img = ctx.render(r, v)[0]
    rgba = ctx.tonemap(capi.BN_TONE_ACES, v)[0]
    return img, rgba


def _pt(ctx, b, mode, spp):
    ctx.upload(b)
    r = b.render
    r.integrator = capi.BN_INTEGRATOR_PATH
    r.mode = mode
    r.spp = spp
    return _render_tonemapped(ctx, r, b.views[0])


@pytest.mark.parametrize("mode", [capi.BN_MODE_MEGAKERNEL, capi.BN_MODE_WAVEFRONT], ids=["megakernel", "wavefront"])
def test_cbox_path_tracing_matches_the_reference_samples(ctx, cbox, mode):
    img, rgba = _pt(ctx, cbox, mode, 64)
    assert np.isfinite(img).mean() > 0.999
    got = block_means(rgba)
    ref = samples()
    for k in ("pt", "pssmlt"):
        assert psnr(got, ref[k]) > PSNR_MIN, f"{k}: {psnr(got, ref[k]):.2f} dB"


def test_cbox_pssmlt_as_the_scene_file_says(ctx, cbox):
    """PSSMLT with the file's settings (16 mutations per pixel, depth 8, the loader's defaults of
    4,194,304 bootstrap paths, 1,024 chains, Gaussian mutations sigma 0.01, large-step probability
    0.5), in both chain forms: the image must agree with a 256-spp path-traced image block for
    block (both estimate the same radiance; PSSMLT.fs:322-326 normalises by the bootstrap b) and,
    the mean of four renders tone mapped, with the reference's PSSMLT sample image (one render at
    these settings is noisier, and tone mapping a noisier image lowers its block means).

    A bootstrap path can end in NaN as in the reference (a PBR sample at a grazing wo with
    wo.z = 0 exactly: specularBSDF = 0/0, PBR.fs:47), and one NaN luminance makes b, the
    float32 Array.average of 4,194,304 of them (PSSMLT.fs:394), NaN; such a render is NaN, as
    the reference's would be.  Renders whose b is NaN are counted and skipped."""
    ctx.upload(cbox)
    r = cbox.render
    v = cbox.views[0]
    assert r.integrator == capi.BN_INTEGRATOR_PSSMLT and r.spp == 16 and r.n_chains == 1024
    frames, nan_b = [], 0
    for f in range(16):
        if len(frames) == 4:
            break
        r.frame_id = f
        r.mode = capi.BN_MODE_WAVEFRONT if len(frames) % 2 else capi.BN_MODE_MEGAKERNEL
        ctx.reset_stats()
        img = ctx.render(r, v)[0]
        st = ctx.stats()
        assert st.proposed == 1024 * -(-(16 * v.width * v.height) // 1024)
        if np.isnan(st.bootstrap_b):
            nan_b += 1
            assert np.isnan(img).mean() > 0.9
            continue
        assert 0.05 < st.accepted / st.proposed < 0.95 and st.bootstrap_b > 0
        frames.append(img)
    assert len(frames) == 4 and nan_b <= 8
    stack = np.stack(frames)
    img = np.where(np.isfinite(stack), stack, 0).sum(0) / np.maximum(np.isfinite(stack).sum(0), 1)
    from oracle import pyoracle
    rgba = pyoracle.tonemap(img.astype(np.float32), capi.BN_TONE_ACES)
    pt, _ = _pt(ctx, cbox, capi.BN_MODE_WAVEFRONT, 256)
    ok = np.isfinite(img) & np.isfinite(pt)
    assert ok.mean() > 0.999
    blk = lambda x: np.where(ok, x, 0).reshape(48, 16, 64, 16, 3).sum((1, 3)) / ok.reshape(48, 16, 64, 16, 3).sum((1, 3))
    a, p = blk(img.astype(np.float64)), blk(pt.astype(np.float64))
    rel = np.abs(a - p).mean() / p.mean()
    assert rel < 0.05, f"PSSMLT vs path tracing: mean block difference {rel:.3%} of the mean"
    ref = samples()["pssmlt"]
    assert psnr(block_means(rgba), ref) > PSNR_MIN, f"{psnr(block_means(rgba), ref):.2f} dB"


def test_cbox_pssmlt_against_the_oracle(ctx, cbox):
    """The reference's scene through PSSMLT on the device and in the oracle (PSSMLT.fs:379-414 on
    the CPU), with the file's settings at the same frame: the bootstrap b agrees to rounding (the
    same 4,194,304 seeds), the acceptance rate within 1% (the chains part by transcendental
    rounding after a few mutations), and the images block for block within 5% of the mean."""
    from oracle import pyoracle
    ctx.upload(cbox)
    o = pyoracle.Scene(cbox.scene)
    v = cbox.views[0]
    for f in range(8):
        r = cbox.render
        r.frame_id = 100 + f
        ctx.reset_stats()
        g = ctx.render(r, v)[0]
        st = ctx.stats()
        c, ob, acc, prop, _ = o.render_pssmlt(r, v)
        if np.isnan(st.bootstrap_b) or np.isnan(ob):
            continue  # a NaN bootstrap path (PBR.fs:47 at wo.z = 0) makes b NaN; see above
        assert abs(st.bootstrap_b / ob - 1) < 1e-4, (st.bootstrap_b, ob)
        assert prop == st.proposed
        assert abs(st.accepted / st.proposed - acc / prop) < 0.01
        ok = np.isfinite(g) & np.isfinite(c)
        assert ok.mean() > 0.999
        blk = lambda x: np.where(ok, x, 0).reshape(48, 16, 64, 16, 3).sum((1, 3)) / ok.reshape(48, 16, 64, 16, 3).sum((1, 3))
        a, b = blk(g.astype(np.float64)), blk(c.astype(np.float64))
        rel = np.abs(a - b).mean() / b.mean()
        assert rel < 0.05, f"device vs oracle PSSMLT: mean block difference {rel:.3%} of the mean"
        return
    pytest.fail("every frame's bootstrap held a NaN path")
