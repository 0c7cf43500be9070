"""PSSMLT on the device against the oracle's restatement of PSSMLT.fs.

The bootstrap of a scene of mirrors and dielectrics involves no transcendental function, so its
luminances and the normalisation b are bit-exact.  Chains use exp/log (Kelemen) and the BSDFs'
sin/cos, so after a few mutations the device and CPU chains part by rounding; the images are
compared statistically (block means), with the acceptance rate and b."""
import numpy as np
import pytest

from barnacle_gb300 import Bundle, capi
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def mlt_desc(b, n_boot, n_chains, spp, depth=8, kelemen=True, fixed=False, frame=0):
    r = b.render
    r.integrator = capi.BN_INTEGRATOR_PSSMLT
    r.n_bootstrap = n_boot
    r.n_chains = n_chains
    r.spp = spp
    r.max_depth = depth
    r.rr_depth = 5
    r.large_step_prob = 0.3
    r.mutation = capi.BN_MUTATION_KELEMEN if kelemen else capi.BN_MUTATION_GAUSSIAN
    r.eps_min, r.eps_max, r.sigma = 1 / 1024, 1 / 64, 1e-2
    r.flags = capi.BN_RENDER_FIXED_ALIAS if fixed else 0
    r.frame_id = frame
    return r


def small_view(b, w, h):
    v = b.views[0]
    v.width, v.height = w, h
    v.camera.aspect_ratio = w / h
    return v


def test_pssmlt_bootstrap_bit_exact_on_specular_scene(ctx):
    b = Bundle.generate("cornell", 1)
    s = b.scene.contents
    for i in range(s.n_materials):
        s.materials[i].type = capi.BN_MAT_MIRROR if i % 2 == 0 else capi.BN_MAT_DIELECTRIC
    ctx.upload(b)
    o = pyoracle.Scene(b.scene)
    v = small_view(b, 48, 48)
    r = mlt_desc(b, 1 << 14, 256, 2)
    ctx.reset_stats()
    ctx.render(r, v)
    st = ctx.stats()
    _, ob, _, _, _ = o.render_pssmlt(r, v)
    assert ob > 0 and np.float32(st.bootstrap_b) == np.float32(ob)


@pytest.mark.parametrize("kelemen,fixed", [(True, False), (True, True), (False, True)])
def test_pssmlt_matches_oracle_statistically(ctx, kelemen, fixed):
    b = Bundle.generate("cornell", 1)
    ctx.upload(b)
    o = pyoracle.Scene(b.scene)
    v = small_view(b, 64, 64)
    gpu, cpu = [], []
    acc_g = acc_c = prop = 0
    bs_g, bs_c = [], []
    for f in range(3):
        r = mlt_desc(b, 1 << 15, 2048, 32, kelemen=kelemen, fixed=fixed, frame=f)
        ctx.reset_stats()
        gpu.append(ctx.render(r, v)[0])
        st = ctx.stats()
        acc_g += st.accepted
        prop += st.proposed
        bs_g.append(st.bootstrap_b)
        img, bb, acc, pr, _ = o.render_pssmlt(r, v)
        cpu.append(img)
        acc_c += acc
        bs_c.append(bb)
    g = np.stack(gpu).astype(np.float64)
    c = np.stack(cpu).astype(np.float64)
    if fixed:
        assert np.isfinite(g).all() and np.isfinite(c).all()
    # the reference's uniform chain starts can leave NaN splats (y = 0 chains); compare the rest
    ok = np.isfinite(g).all(axis=(0, 3)) & np.isfinite(c).all(axis=(0, 3))
    assert ok.mean() > (0.99 if fixed else 0.75)
    assert abs(np.mean(bs_g) / np.mean(bs_c) - 1) < 0.03
    assert abs(acc_g / acc_c - 1) < 0.03, (acc_g, acc_c, prop)
    # 8x8-pixel block means of the frame average
    gm = np.where(ok[None, :, :, None], g, 0).mean(0)
    cm = np.where(ok[None, :, :, None], c, 0).mean(0)
    blk = lambda x: x.reshape(8, 8, 8, 8, 3).sum(axis=(1, 3))
    gb, cb = blk(gm), blk(cm)
    big = cb > 0.05 * cb.max()
    rel = np.abs(gb - cb)[big] / cb[big]
    assert np.median(rel) < 0.08 and rel.max() < 0.5, (np.median(rel), rel.max())
    assert abs(gm.sum() / cm.sum() - 1) < 0.05


def test_pssmlt_errors(ctx):
    b = Bundle.generate("cornell", 1)
    ctx.upload(b)
    r = mlt_desc(b, 0, 16, 1)
    with pytest.raises(Exception):
        ctx.render(r, b.views[0])
    r = mlt_desc(b, 1024, 16, 1)
    with pytest.raises(Exception):
        ctx.render(r, b.views + b.views)  # one view per PSSMLT render


@pytest.mark.parametrize("name,kelemen,fixed", [("cornell", True, False), ("cornell", False, True),
                                                ("cornell-objects", True, True)])
def test_pssmlt_wavefront_chains_equal_lockstep(ctx, name, kelemen, fixed):
    """The chains compacted every bounce (BN_MODE_WAVEFRONT) draw every chain's random numbers in
    the lockstep kernel's order, so each chain makes the same mutations and the same decisions:
    the accepted count and b are identical, the films equal up to the splats' summation order."""
    b = Bundle.generate(name, 1)
    ctx.upload(b)
    v = small_view(b, 64, 48)
    r = mlt_desc(b, 1 << 14, 1024, 8, depth=8 if name == "cornell" else 12, kelemen=kelemen, fixed=fixed, frame=3)
    out = {}
    for mode in (capi.BN_MODE_MEGAKERNEL, capi.BN_MODE_WAVEFRONT):
        r.mode = mode
        r.flags = capi.BN_RENDER_FIXED_ALIAS if fixed else 0
        ctx.reset_stats()
        img = ctx.render(r, v)[0]
        st = ctx.stats()
        out[mode] = (img, st.accepted, st.proposed, st.bootstrap_b)
    (a, acc_a, prop_a, b_a), (w, acc_w, prop_w, b_w) = out[capi.BN_MODE_MEGAKERNEL], out[capi.BN_MODE_WAVEFRONT]
    assert prop_a == prop_w and b_a == b_w
    assert acc_a == acc_w, (acc_a, acc_w)
    ok = np.isfinite(a) & np.isfinite(w)
    assert np.array_equal(ok, np.isfinite(a))
    assert a[ok].sum() > 0
    np.testing.assert_allclose(w[ok], a[ok], rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("depth", [1, 2])
def test_pssmlt_wavefront_short_paths_equal_lockstep(ctx, depth):
    """Paths of one or two bounces: at depth 1 every path ends at its first bounce, most with a
    shadow record still to trace, so nearly every chain waits an iteration before its Metropolis
    step; the decisions must still be the lockstep kernel's."""
    b = Bundle.generate("cornell-objects", 1)
    ctx.upload(b)
    v = small_view(b, 64, 48)
    r = mlt_desc(b, 1 << 14, 1024, 8, depth=depth, frame=5)
    out = {}
    for mode in (capi.BN_MODE_MEGAKERNEL, capi.BN_MODE_WAVEFRONT):
        r.mode = mode
        r.flags = 0
        ctx.reset_stats()
        img = ctx.render(r, v)[0]
        st = ctx.stats()
        out[mode] = (img, st.accepted, st.proposed, st.bootstrap_b)
    (a, acc_a, prop_a, b_a), (w, acc_w, prop_w, b_w) = out[capi.BN_MODE_MEGAKERNEL], out[capi.BN_MODE_WAVEFRONT]
    assert prop_a == prop_w and b_a == b_w and b_a > 0
    assert acc_a == acc_w, (acc_a, acc_w)
    ok = np.isfinite(a) & np.isfinite(w)
    assert np.array_equal(ok, np.isfinite(a)) and a[ok].sum() > 0
    np.testing.assert_allclose(w[ok], a[ok], rtol=1e-4, atol=1e-5)
