"""Failure detection without a GPU fault: the device-side limits are lowered through
bn_set_limits so that a walk runs out of stack and the wavefront's bounce loop runs into its
watchdog.  Each must come back as BN_ERR_DEVICE with its BN_DEVERR_* bit, and the context must
render correctly afterwards (nothing traps, nothing hangs: both limits are checked on the device
and end the work with a status the host reads)."""
import numpy as np
import pytest

from barnacle_gb300 import Bundle, Context, capi
from barnacle_gb300.capi import BarnacleError

pytestmark = pytest.mark.gpu


def _limits(ctx, stack, iters):
    assert ctx.lib.bn_set_limits(ctx._h, stack, iters) == capi.BN_OK, ctx.error()


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, capi.RAY_DTYPE)
    rays["origin"] = rng.uniform(0.1, 0.9, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    rays["direction"] = d / np.sqrt((d ** 2).sum(1, dtype=np.float32))[:, None]
    rays["t_max"] = np.inf
    return rays


def test_stack_overflow_is_reported_and_the_context_recovers():
    from oracle import pyoracle
    with Context(0) as ctx:
        b = Bundle.generate("cornell-objects", 1)
        ctx.upload(b)
        rays = _rays(2048, 3)
        want = ctx.trace(rays)
        _limits(ctx, 1, 0)
        with pytest.raises(BarnacleError) as e:
            ctx.trace(rays)
        assert e.value.code == capi.BN_ERR_DEVICE
        assert ctx.stats().device_error & capi.BN_DEVERR_STACK_OVERFLOW
        r = b.render
        r.spp = 1
        for mode in (capi.BN_MODE_MEGAKERNEL, capi.BN_MODE_WAVEFRONT):
            r.mode = mode
            with pytest.raises(BarnacleError) as e:
                ctx.render(r, b.views[0])
            assert e.value.code == capi.BN_ERR_DEVICE
            assert ctx.stats().device_error & capi.BN_DEVERR_STACK_OVERFLOW
        _limits(ctx, 0, 0)
        got = ctx.trace(rays)
        assert np.array_equal(got["instance"], want["instance"]) and np.array_equal(got["primitive"], want["primitive"])
        h, _ = pyoracle.Scene(b.scene).trace(rays)
        assert np.array_equal(got["primitive"], h["primitive"])
        r.mode = capi.BN_MODE_MEGAKERNEL
        assert ctx.render(r, b.views[0])[0].max() > 0


@pytest.mark.parametrize("graph", [True, False])
def test_wavefront_watchdog_is_reported_and_the_context_recovers(graph):
    with Context(0) as ctx:
        b = Bundle.generate("cornell", 1)
        ctx.upload(b)
        r = b.render
        r.spp = 4
        r.mode = capi.BN_MODE_WAVEFRONT
        r.queue_capacity = 4096  # 262,144 paths through 4,096 slots: dozens of iterations
        if not graph:
            r.flags |= capi.BN_RENDER_NO_GRAPH
        _limits(ctx, 0, 3)
        with pytest.raises(BarnacleError) as e:
            ctx.render(r, b.views[0])
        assert e.value.code == capi.BN_ERR_DEVICE
        assert ctx.stats().device_error & capi.BN_DEVERR_WATCHDOG
        _limits(ctx, 0, 0)
        wave = ctx.render(r, b.views[0])[0]
        r.mode = capi.BN_MODE_MEGAKERNEL
        mega = ctx.render(r, b.views[0])[0]
        np.testing.assert_allclose(wave, mega, rtol=2e-5, atol=1e-6)


def test_limits_are_validated():
    with Context(0) as ctx:
        assert ctx.lib.bn_set_limits(ctx._h, 201, 0) == capi.BN_ERR_INVALID_ARG
        assert ctx.lib.bn_set_limits(ctx._h, -1, 0) == capi.BN_ERR_INVALID_ARG
        assert ctx.lib.bn_set_limits(ctx._h, 0, -5) == capi.BN_ERR_INVALID_ARG
        assert ctx.lib.bn_set_limits(ctx._h, 200, 10) == capi.BN_OK
