"""The batched wavefront form against the plain megakernel.

Both forms run the same per-path arithmetic and the same random streams, so their images are
the same estimator sample: equal up to the order in which the film sums the paths (the
megakernel sums chunks in order, the wavefront accumulates FP64 atomics).  That makes "paths/s at
equal image RMSE" a plain paths/s comparison."""
import numpy as np
import pytest

from barnacle_gb300 import Bundle, capi

pytestmark = pytest.mark.gpu


def render(ctx, b, views, spp, mode, flags=0, pool=0, cap=0, frame=0):
    r = b.render
    r.spp = spp
    r.mode = mode
    r.flags = flags
    r.queue_capacity = pool
    r.block_size = cap
    r.frame_id = frame
    return ctx.render(r, views)


def assert_same_image(a, b, rtol=2e-5):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(1e-6, float(np.abs(b).max()))
    err = np.abs(a - b)
    assert np.all(err <= rtol * np.maximum(np.abs(b), 1e-3 * scale)), \
        f"max abs diff {err.max():.3e}, worst rel {(err / np.maximum(np.abs(b), 1e-30)).max():.3e}"


@pytest.mark.parametrize("name,spp", [("cornell", 8), ("cornell-objects", 4)])
def test_wavefront_equals_megakernel(ctx, name, spp):
    b = Bundle.generate(name, 1)
    ctx.upload(b)
    v = b.views
    mega = render(ctx, b, v, spp, capi.BN_MODE_MEGAKERNEL)
    wave = render(ctx, b, v, spp, capi.BN_MODE_WAVEFRONT)
    for m, w in zip(mega, wave):
        assert m.max() > 0.5
        assert_same_image(w, m)


def test_wavefront_graph_and_host_loop_agree(ctx):
    b = Bundle.generate("cornell-objects", 1)
    ctx.upload(b)
    v = b.views
    g = render(ctx, b, v, 2, capi.BN_MODE_WAVEFRONT)[0]
    launches_graph = ctx.stats().last_launches
    h = render(ctx, b, v, 2, capi.BN_MODE_WAVEFRONT, flags=capi.BN_RENDER_NO_GRAPH)[0]
    assert_same_image(g, h, rtol=1e-6)
    assert launches_graph > 10


@pytest.mark.parametrize("pool", [1024, 4096])
def test_wavefront_small_pool_regenerates_correctly(ctx, pool):
    b = Bundle.generate("cornell", 1)
    ctx.upload(b)
    v = b.views[0]
    v.width, v.height = 64, 48
    mega = render(ctx, b, [v], 4, capi.BN_MODE_MEGAKERNEL)[0]
    wave = render(ctx, b, [v], 4, capi.BN_MODE_WAVEFRONT, pool=pool)[0]
    assert_same_image(wave, mega)


@pytest.mark.parametrize("pool", [1 << 20, 1 << 21, 1 << 23, 1 << 25])
def test_wavefront_sort_key_widths(ctx, pool):
    """The queues' sort keys have 16, 18, 20 and 22 bits at these pools (2^b x 8 x 2^b origin
    cells under the octant, b following the pool): sorting only reorders the rays, so every width
    gives the megakernel's image up to summation order, on the instanced scene whose keys spread
    over the most cells."""
    b = Bundle.generate("instances", 1)
    ctx.upload(b)
    views = b.views[:2]
    for v in views:
        v.width, v.height = v.width // 4, v.height // 4
    mega = render(ctx, b, views, 2, capi.BN_MODE_MEGAKERNEL)
    wave = render(ctx, b, views, 2, capi.BN_MODE_WAVEFRONT, pool=pool)
    for m, w in zip(mega, wave):
        assert float(m.sum()) > 0
        assert_same_image(w, m)


def test_wavefront_many_views_one_launch(ctx):
    b = Bundle.generate("instances", 1)
    ctx.upload(b)
    views = b.views
    for v in views:  # keep the test short: shrink every view, keep the aspect and cameras
        v.width, v.height = max(8, v.width // 8), max(8, v.height // 8)
    mega = render(ctx, b, views, 2, capi.BN_MODE_MEGAKERNEL)
    wave = render(ctx, b, views, 2, capi.BN_MODE_WAVEFRONT)
    assert len(wave) == 16
    for m, w in zip(mega, wave):
        assert_same_image(w, m)
    assert sum(float(w.sum()) for w in wave) > 0


def test_wavefront_watertight_and_depth_zero(ctx):
    b = Bundle.generate("cornell", 1)
    ctx.upload(b)
    v = b.views[0]
    v.width, v.height = 32, 32
    mega = render(ctx, b, [v], 2, capi.BN_MODE_MEGAKERNEL, flags=capi.BN_RENDER_WATERTIGHT)[0]
    wave = render(ctx, b, [v], 2, capi.BN_MODE_WAVEFRONT, flags=capi.BN_RENDER_WATERTIGHT)[0]
    assert_same_image(wave, mega)
    r = b.render
    r.max_depth = 0
    r.mode = capi.BN_MODE_WAVEFRONT
    assert np.all(ctx.render(r, [v])[0] == 0)


def test_wavefront_counting_render_and_shadow_culling(ctx):
    """A counting render walks the binary tree in the reference's order and gives the same image;
    the wavefront traces the megakernel's closest-hit rays but no shadow ray whose contribution is
    exactly zero, so it counts fewer rays than the megakernel on the same paths."""
    b = Bundle.generate("cornell-objects", 1)
    ctx.upload(b)
    v = b.views
    plain = render(ctx, b, v, 2, capi.BN_MODE_WAVEFRONT)[0]
    counts = {}
    for mode in (capi.BN_MODE_WAVEFRONT, capi.BN_MODE_MEGAKERNEL):
        ctx.reset_stats()
        img = render(ctx, b, v, 2, mode, flags=capi.BN_RENDER_COUNT)[0]
        st = ctx.stats()
        counts[mode] = (st.rays, st.nodes_visited, st.tris_tested, st.instances_visited)
        assert_same_image(img, plain)
    wf, mk = counts[capi.BN_MODE_WAVEFRONT], counts[capi.BN_MODE_MEGAKERNEL]
    assert 0 < wf[0] < mk[0] and 0 < wf[1] < mk[1]
    # every path's camera ray is traced by both
    assert wf[0] > v[0].width * v[0].height * 2
