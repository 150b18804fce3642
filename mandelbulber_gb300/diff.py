"""Differentiable render: parameters theta, the config-5 workload, and a thin
torch.autograd.Function over mbgb_render_grad.

theta of one frame (MBGB_GRAD_PARAMS = 6): [0] the fractal parameter (power of the
trig_optim Mandelbulb, scale of the tglad Mandelbox), [1..3] the camera position vp,
[4] main light alpha, [5] main light beta (radians, as mbgb_scene holds them).

The forward pass renders with every hit moved onto the level set DE(P) = thr
(opts.exact_hit); the backward pass calls mbgb_render_grad, which recomputes the
forward stages and differentiates each hit pixel on the device. The autograd function
is a checking harness for that kernel (finite differences, the FP64 CPU path), not a
training framework.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import PREC_FP32_FIX, Context, finalize, mbgb_scene, scene_from_bytes, scene_bytes

GRAD_PARAMS = 6
NAMES = ("fractal", "vp_x", "vp_y", "vp_z", "light_alpha", "light_beta")


def theta_of(scene: mbgb_scene) -> np.ndarray:
    fp = scene.mboxScale if scene.formula == 8 else scene.power
    return np.array([fp, scene.vp[0], scene.vp[1], scene.vp[2], scene.mainLightAlpha, scene.mainLightBeta])


def with_theta(scene: mbgb_scene, theta) -> mbgb_scene:
    """A copy of `scene` with theta applied (derived fields rebuilt)."""
    s = scene_from_bytes(scene_bytes(scene))
    th = [float(v) for v in theta]
    if s.formula == 8:
        s.mboxScale = th[0]
    else:
        s.power = th[0]
    s.vp[0], s.vp[1], s.vp[2] = th[1], th[2], th[3]
    s.mainLightAlpha, s.mainLightBeta = th[4], th[5]
    return finalize(s)


def grad_batch(n: int = 32, size: int = 256, seed: int = 6):
    """The gradient workload: n Mandelbulb frames at size x size (the 640x480 scene's
    settings: hard shadows, no AO / fog / glow) with seeded theta -- power ~ U[6, 10],
    vp = (0, -3.5, 0) + N(0, 0.05^2) per axis, light (45 deg, 45 deg) + N(0, (5 deg)^2) --
    and target parameters theta + delta, delta = 2 % of each range (power 4, position
    4 sigma = 0.2, light 4 sigma = 20 deg) with seeded signs.
    Returns (scenes, thetas [n, 6], target_thetas [n, 6])."""
    from . import workloads as W
    rng = np.random.default_rng(seed)
    base = W.workload("mandelbulb_640x480", size, size)
    ranges = np.array([4.0, 0.2, 0.2, 0.2, math.radians(20.0), math.radians(20.0)])
    thetas, targets, scenes = [], [], []
    for _ in range(n):
        th = np.array([rng.uniform(6.0, 10.0), *(np.array([0.0, -3.5, 0.0]) + rng.normal(0.0, 0.05, 3)),
                       math.radians(45.0) + rng.normal(0.0, math.radians(5.0)),
                       math.radians(45.0) + rng.normal(0.0, math.radians(5.0))])
        sign = rng.choice([-1.0, 1.0], size=GRAD_PARAMS)
        thetas.append(th)
        targets.append(th + 0.02 * ranges * sign)
        scenes.append(with_theta(base, th))
    return scenes, np.array(thetas), np.array(targets)


class Renderer:
    """Device layers for a list of frames of equal size and the two library calls."""

    def __init__(self, ctx: Context, scenes, precision: int = PREC_FP32_FIX):
        import torch
        self.ctx, self.precision = ctx, precision
        self.scenes = list(scenes)
        self.h, self.w = self.scenes[0].image_height, self.scenes[0].image_width
        n = len(self.scenes)
        dev = torch.device("cuda")
        self.image = torch.zeros((n, self.h, self.w, 3), dtype=torch.float32, device=dev)
        self.hit = torch.zeros((n, self.h, self.w), dtype=torch.uint8, device=dev)
        self.colour = torch.zeros((n, self.h, self.w, 3), dtype=torch.uint8, device=dev)
        self.iters = torch.zeros((n, self.h, self.w), dtype=torch.int32, device=dev)

    def layers(self):
        return [{"image_float": self.image[i].data_ptr(), "hit": self.hit[i].data_ptr(),
                 "colour": self.colour[i].data_ptr(), "iters": self.iters[i].data_ptr()}
                for i in range(len(self.scenes))]

    def set_theta(self, thetas):
        self.scenes = [with_theta(s, t) for s, t in zip(self.scenes, thetas)]

    def forward(self):
        import torch
        self.ctx.render_batch_device(self.scenes, self.layers(), precision=self.precision, exact_hit=True)
        torch.cuda.synchronize()
        return self.image

    def backward(self, dL_dimage, jacobian=None):
        import torch
        g = dL_dimage.contiguous()
        ptrs = [g[i].data_ptr() for i in range(len(self.scenes))]
        jac = [jacobian[i].data_ptr() for i in range(len(self.scenes))] if jacobian is not None else None
        out = self.ctx.render_grad(self.scenes, self.layers(), dL_dimage=ptrs, jacobian=jac,
                                   precision=self.precision)
        torch.cuda.synchronize()
        return out


def render_function():
    """torch.autograd.Function: images = Render(theta); backward through mbgb_render_grad."""
    import torch

    class _Render(torch.autograd.Function):
        @staticmethod
        def forward(fctx, theta, renderer):
            renderer.set_theta(theta.detach().cpu().numpy())
            fctx.renderer = renderer
            return renderer.forward().clone()

        @staticmethod
        def backward(fctx, grad_images):
            g = fctx.renderer.backward(grad_images.float())
            return torch.as_tensor(g, dtype=torch.float64), None

    return _Render.apply
