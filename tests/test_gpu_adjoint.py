"""The path-replay adjoint (bn_backward) on the 32-slot material workload.

* forward with the scene's own material values and unit light scales = bn_render's image;
* gradients against central finite differences (eps 1e-3) of the same estimator with common random
  numbers and sampling frozen at the evaluation point: within 1e-2 relative;
* gradients against a central finite difference of the CPU oracle's renderer with the same random
  numbers (1e-2 relative per parameter on the 12 largest entries; measured at most 5e-3; the CPU
  and device paths part only where transcendental rounding differs);
* the backward pass costs at most 3x the forward pass; Adam steps reduce the loss."""
import numpy as np
import pytest

from barnacle_gb300 import Bundle, capi
from barnacle_gb300.inverse import MaterialProblem
from oracle import pyoracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem_small(ctx):
    b = Bundle.generate("materials", 1)
    return b, MaterialProblem(ctx, b, width=64, height=64, spp=4)


def test_forward_equals_render_with_scene_materials(ctx, problem_small):
    b, pb = problem_small
    ctx.upload(b)
    params = b.slot_params()
    params.reshape(-1, 6)[:, 5] = 1.0  # lights at their scene emission
    img = pb.render(params, spp=4, frame=3)
    r = b.render
    r.spp, r.max_depth, r.rr_depth, r.frame_id = 4, pb.max_depth, pb.rr_depth, 3
    v = b.views[0]
    v.width, v.height = 64, 64
    ref = ctx.render(r, v)[0]
    np.testing.assert_allclose(img, ref, rtol=2e-5, atol=1e-6)


def test_adjoint_matches_central_finite_differences(ctx, problem_small):
    b, pb = problem_small
    ctx.upload(b)
    gt = b.slot_params()
    target = pb.render(gt, spp=16, frame=900)
    rng = np.random.default_rng(4)
    theta = pb.random_params(11).reshape(-1, 6)
    theta[:, 3] = rng.uniform(0.15, 0.85, len(theta))  # keep clear of the alpha clamp
    theta[:, 4] = rng.uniform(0.1, 0.9, len(theta))    # and of the metallic clamp
    theta = theta.reshape(-1).astype(np.float32)
    loss, g = pb.loss_and_grad(theta, target, frame=5, sampling_params=theta)
    assert np.isfinite(g).all() and loss > 0

    def loss_at(x):
        img = pb.render(x, frame=5, sampling_params=theta).astype(np.float64)
        return 0.5 * ((img - target) ** 2).sum()

    order = np.argsort(-np.abs(g))
    checked = 0
    for i in order[:16]:
        e = np.zeros_like(theta)
        e[i] = 1e-3
        xp, xm = (theta + e).astype(np.float32), (theta - e).astype(np.float32)
        fd = (loss_at(xp) - loss_at(xm)) / float(xp[i] - xm[i])
        assert abs(fd - g[i]) <= 1e-2 * abs(fd) + 1e-6, f"param {i}: adjoint {g[i]:.6g} vs FD {fd:.6g}"
        checked += 1
    assert checked == 16


def test_adjoint_agrees_with_cpu_oracle_fd(ctx, problem_small):
    """The device adjoint against a central finite difference of the CPU oracle's renderer: both
    evaluate the same estimator (sampling frozen at theta, the same frame id and so the same random
    numbers), so they agree per parameter to 1e-2 relative on the 12 largest gradient entries
    (paths where the CPU's and the device's transcendental rounding part ways are the residue)."""
    b, pb = problem_small
    ctx.upload(b)
    o = pyoracle.Scene(b.scene)
    gt = b.slot_params()
    rng = np.random.default_rng(8)
    theta = pb.random_params(3).reshape(-1, 6)
    theta[:, 3] = rng.uniform(0.15, 0.85, len(theta))  # clear of the alpha and metallic clamps
    theta[:, 4] = rng.uniform(0.1, 0.9, len(theta))
    theta = theta.reshape(-1).astype(np.float32)
    frame = 1
    r = b.render
    r.spp, r.max_depth, r.rr_depth, r.frame_id = 32, pb.max_depth, pb.rr_depth, frame
    v = b.views[0]
    v.width, v.height = 32, 32
    pb32 = MaterialProblem(ctx, b, width=32, height=32, spp=32)
    target = pb32.render(gt, spp=64, frame=77)
    _, g = pb32.loss_and_grad(theta, target, frame=frame, sampling_params=theta)
    idx = np.argsort(-np.abs(g))[:12]
    eps = 5e-3
    for i in idx:
        e = np.zeros_like(theta)
        e[i] = eps
        xp, xm = (theta + e).astype(np.float32), (theta - e).astype(np.float32)
        lp = 0.5 * ((o.render_slots(r, v, pb.n_slots, pb.emissive_base, xp, theta).astype(np.float64) - target) ** 2).sum()
        lm = 0.5 * ((o.render_slots(r, v, pb.n_slots, pb.emissive_base, xm, theta).astype(np.float64) - target) ** 2).sum()
        fd = (lp - lm) / float(xp[i] - xm[i])
        assert abs(fd - g[i]) <= 1e-2 * abs(fd), f"param {i}: adjoint {g[i]:.6g} vs oracle FD {fd:.6g}"


def test_adjoint_cost_within_3x_forward(ctx):
    b = Bundle.generate("materials", 1)
    pb = MaterialProblem(ctx, b, width=256, height=256, spp=16)
    gt = b.slot_params()
    target = pb.render(gt, spp=16, frame=1)
    theta = pb.random_params(2)
    for _ in range(2):
        pb.render(theta, frame=2)
        fwd = ctx.stats().last_kernel_ms
        pb.loss_and_grad(theta, target, frame=2)
        bwd = ctx.stats().last_kernel_ms
    assert bwd <= 3.0 * fwd, (bwd, fwd)


def test_adam_reduces_loss(ctx, problem_small):
    b, pb = problem_small
    ctx.upload(b)
    target = pb.render(b.slot_params(), spp=32, frame=500)
    x0 = pb.random_params(9)
    x, losses = pb.adam(x0, target, steps=25, lr=2e-2)
    assert np.mean(losses[-5:]) < 0.7 * np.mean(losses[:3])
    err0 = np.abs(x0 - b.slot_params()).mean()
    err1 = np.abs(x - b.slot_params()).mean()
    assert err1 < err0
