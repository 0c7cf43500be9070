"""Inverse material estimation over the C-ABI's forward/backward pair.

The scene's material slots are PBR materials parameterised per slot by
[albedo r, g, b, roughness, metallic, emission scale]; bn_forward renders them and bn_backward
returns d(0.5 * ||image - target||^2)/d(params) from the path-replay adjoint.  This module holds the
host-side loop: a target render, Adam steps with projection onto the parameter box.
"""
from __future__ import annotations

import numpy as np

from . import capi
from .api import Bundle, Context

LO = np.array([0.05, 0.05, 0.05, 0.05, 0.0, 0.05], np.float32)
HI = np.array([0.95, 0.95, 0.95, 0.9, 1.0, 5.0], np.float32)


class MaterialProblem:
    def __init__(self, ctx: Context, bundle: Bundle, width: int = 256, height: int = 256, spp: int = 16,
                 max_depth: int = 8, rr_depth: int = 5):
        if bundle.n_slots == 0:
            raise ValueError("the bundle has no material slots")
        self.ctx, self.bundle = ctx, bundle
        self.n_slots, self.emissive_base = bundle.n_slots, bundle.emissive_slot_base
        self.width, self.height, self.spp = width, height, spp
        self.max_depth, self.rr_depth = max_depth, rr_depth
        ctx.upload(bundle)
        self.camera = bundle.views[0].camera

    def desc(self, spp: int | None = None, frame: int = 0, freeze: bool = False) -> capi.bn_adjoint_desc:
        d = capi.bn_adjoint_desc()
        d.n_slots, d.emissive_slot_base = self.n_slots, self.emissive_base
        d.width, d.height = self.width, self.height
        d.spp = spp or self.spp
        d.max_depth, d.rr_depth, d.frame_id = self.max_depth, self.rr_depth, frame
        d.freeze_sampling = 1 if freeze else 0
        d.camera = self.camera
        return d

    def render(self, params: np.ndarray, spp: int | None = None, frame: int = 0,
               sampling_params: np.ndarray | None = None) -> np.ndarray:
        return self.ctx.forward(self.desc(spp, frame, sampling_params is not None), params, sampling_params)

    def loss_and_grad(self, params: np.ndarray, target: np.ndarray, frame: int = 0,
                      sampling_params: np.ndarray | None = None) -> tuple[float, np.ndarray]:
        g, loss = self.ctx.backward(self.desc(None, frame, sampling_params is not None), params, target,
                                    sampling_params)
        return loss, g

    def project(self, params: np.ndarray) -> np.ndarray:
        p = params.reshape(self.n_slots, 6)
        return np.clip(p, LO, HI).astype(np.float32).reshape(-1)

    def random_params(self, seed: int) -> np.ndarray:
        rng = np.random.default_rng(seed)
        p = rng.uniform(LO, HI, size=(self.n_slots, 6)).astype(np.float32)
        p[:, 5] = rng.uniform(0.5, 1.5, self.n_slots)
        p[: self.emissive_base, 5] = 1.0
        return p.reshape(-1)

    def adam(self, params: np.ndarray, target: np.ndarray, steps: int = 200, lr: float = 1e-2,
             beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, frame0: int = 0):
        """Adam with a fresh random stream per step; returns (params, [loss per step]).

        A step whose loss or gradient is not finite is skipped (the parameters and moments stay
        as they were; its loss is recorded as NaN): a path can end in NaN radiance as in the
        reference renderer (a PBR sample at a grazing direction with cos = 0 exactly makes the
        specular term 0/0), and one such path would otherwise poison the moments for good."""
        x = self.project(np.array(params, np.float32))
        m = np.zeros_like(x, np.float64)
        v = np.zeros_like(x, np.float64)
        losses = []
        t = 0
        for k in range(1, steps + 1):
            loss, g = self.loss_and_grad(x, target, frame=frame0 + k)
            if not (np.isfinite(loss) and np.isfinite(g).all()):
                losses.append(float("nan"))
                continue
            losses.append(loss)
            t += 1
            m = beta1 * m + (1 - beta1) * g
            v = beta2 * v + (1 - beta2) * g * g
            mh = m / (1 - beta1 ** t)
            vh = v / (1 - beta2 ** t)
            x = self.project((x - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32))
        return x, losses
