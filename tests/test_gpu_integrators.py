"""The Normal and Direct integrators (Extensions/Integrator/Normal.fs, Direct.fs) in both render
forms, against the oracle's restatement.

Normal: the colour is 0.5 (n + 1) of the closest hit's shading normal, with no transcendental
function on the way, so one sample per pixel reproduces the oracle's floats exactly.  Direct: a
light sample and a BSDF sample per camera hit; diffuse and GGX sampling go through sin/cos, so it
is compared statistically, and bit-exactly on a scene of mirrors and dielectrics."""
import numpy as np
import pytest

from barnacle_gb300 import Bundle, capi
from oracle import pyoracle

pytestmark = pytest.mark.gpu

MODES = [capi.BN_MODE_MEGAKERNEL, capi.BN_MODE_WAVEFRONT]


def setup(ctx, name, integrator, spp, mode):
    b = Bundle.generate(name, 1)
    ctx.upload(b)
    r = b.render
    r.integrator = integrator
    r.spp = spp
    r.mode = mode
    r.frame_id = 0
    return b, r


def crop_rows(v, crop):
    x0, y0, x1, y1 = crop
    return slice(v.height - y1, v.height - y0), slice(x0, x1)  # Film.Pixels rows are flipped


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", ["cornell", "cornell-objects"])
def test_normal_integrator_bit_identical(ctx, name, mode):
    b, r = setup(ctx, name, capi.BN_INTEGRATOR_NORMAL, 1, mode)
    v = b.views[0]
    img = ctx.render(r, v)[0]
    crop = (0, 0, v.width, v.height) if name == "cornell" else (128, 128, 384, 384)
    ref, _ = pyoracle.Scene(b.scene).render_pt(r, v, crop=crop)
    rows, cols = crop_rows(v, crop)
    a, o = img[rows, cols], ref[rows, cols]
    assert (o > 0).mean() > 0.5 and o.max() <= 1.0
    assert np.array_equal(a.view(np.uint32), o.view(np.uint32)), f"{(a != o).any(axis=2).sum()} pixels differ"


@pytest.mark.parametrize("mode", MODES)
def test_direct_integrator_specular_scene_bit_identical(ctx, mode):
    b = Bundle.generate("cornell", 1)
    s = b.scene.contents
    for i in range(s.n_materials):
        s.materials[i].type = capi.BN_MAT_MIRROR if i % 2 == 0 else capi.BN_MAT_DIELECTRIC
    ctx.upload(b)
    r = b.render
    r.integrator = capi.BN_INTEGRATOR_DIRECT
    r.spp = 1
    r.mode = mode
    v = b.views[0]
    img = ctx.render(r, v)[0]
    ref, _ = pyoracle.Scene(b.scene).render_pt(r, v)
    assert np.isfinite(ref).all() and ref.max() > 1.0, "the light must be seen directly and through mirrors"
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), \
        f"{(img != ref).any(axis=2).sum()} pixels differ"


@pytest.mark.parametrize("mode", MODES)
def test_direct_integrator_statistically_matches_oracle(ctx, mode):
    b, r = setup(ctx, "cornell", capi.BN_INTEGRATOR_DIRECT, 16, mode)
    v = b.views[0]
    o = pyoracle.Scene(b.scene)
    crop = (64, 64, 192, 192)
    rows, cols = crop_rows(v, crop)
    gpu, cpu = [], []
    for f in range(10):
        r.frame_id = f
        gpu.append(ctx.render(r, v)[0][rows, cols])
        r.frame_id = 1000 + f
        cpu.append(o.render_pt(r, v, crop=crop)[0][rows, cols])
    g = np.stack(gpu).astype(np.float64)
    c = np.stack(cpu).astype(np.float64)
    se = np.sqrt(g.var(0, ddof=1) / len(g) + c.var(0, ddof=1) / len(c))
    z = np.abs(g.mean(0) - c.mean(0)) / np.maximum(se, 1e-12)
    assert c.mean() > 0.05
    assert (z[se > 0] > 3).mean() < 0.02
    # same per-pixel noise: RMSE of each estimator against the other's mean
    rg = np.sqrt(((g - c.mean(0)) ** 2).mean())
    rc = np.sqrt(((c - g.mean(0)) ** 2).mean())
    assert abs(rg / rc - 1) < 0.1


@pytest.mark.parametrize("integrator", [capi.BN_INTEGRATOR_NORMAL, capi.BN_INTEGRATOR_DIRECT])
def test_wavefront_equals_megakernel_other_integrators(ctx, integrator):
    """Same per-path estimator and random streams in both forms: equal up to film summation order."""
    b = Bundle.generate("cornell-objects", 1)
    ctx.upload(b)
    r = b.render
    r.integrator = integrator
    r.spp = 4
    imgs = []
    for mode in MODES:
        r.mode = mode
        imgs.append(ctx.render(r, b.views[0])[0].astype(np.float64))
    m, w = imgs
    scale = max(1e-6, float(np.abs(m).max()))
    assert scale > 0.1
    assert np.all(np.abs(w - m) <= 2e-5 * np.maximum(np.abs(m), 1e-3 * scale))


def test_direct_ignores_max_depth(ctx):
    """DirectIntegrator takes no maximum depth: depth 0 still renders (the path tracer's loop does
    not run at depth 0, so it renders black)."""
    b, r = setup(ctx, "cornell", capi.BN_INTEGRATOR_DIRECT, 2, capi.BN_MODE_WAVEFRONT)
    r.max_depth = 0
    a = ctx.render(r, b.views[0])[0]
    r.max_depth = 8
    c = ctx.render(r, b.views[0])[0]
    assert np.array_equal(a, c) and a.max() > 0.1
    r.integrator = capi.BN_INTEGRATOR_PATH
    r.max_depth = 0
    assert ctx.render(r, b.views[0])[0].max() == 0.0
