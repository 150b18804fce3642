"""Differentiable render: the gradient stage against central finite differences (needs a GPU).

The gradient workload is the Mandelbulb scene at 256 x 256 with seeded parameters
theta = (power, camera position, light alpha / beta) and a target rendered at theta + delta
(mandelbulber_gb300.diff.grad_batch). Loss = sum over the float image of (I - target)^2.

The shaded image is piecewise smooth in theta: the hit mask, hard shadows, the integer
palette index and the orbit iteration counts at the distance samples change in jumps.
A finite difference across a jump measures the jump, not a derivative, so each check
runs on the pixels that are interior for that parameter: hit and on the level set in
the renders at theta - h, theta and theta + h, with the same colour layer and iteration
count in all three, and a second difference |I+ - 2 I0 + I-| no larger than 1e-3 of the
first difference |I+ - I-| (a jump in the normal's distance samples shows up there).
On those pixels:
  * the adjoint sums (FP64 forward state) match the FP64 central differences (h = 1e-4)
    within 1e-3 relative, per frame and parameter;
  * the same with the FP32 policy's forward state (the derivative arithmetic is FP64), on
    the pixels whose FP32 palette index and iteration count match the FP64 render's;
  * the adjoint matches central differences of the CPU oracle's own FP64 render (with
    the same level-set hits) within 1e-3 relative.
"""
import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import diff as D
from tests import metrics, oracle_lib

pytestmark = pytest.mark.gpu
H = 1e-4
REL_TOL = 1e-3
# Least fraction of all pixels each parameter's interior mask must cover: power, camera
# x / y / z, light alpha / beta. The seeded 256 x 256 frames (about 30 % of the pixels hit)
# measure 18.1 / 5.0 / 12.9 / 3.4 / 25.9 / 27.4 % on the GPU renders (both policies) and
# 17.7 / 5.1 / 13.2 / 3.7 / 25.4 / 27.0 % on the oracle's; the floors sit at ~80 % of that.
MASK_FLOOR = [0.145, 0.04, 0.103, 0.027, 0.207, 0.219]
ORACLE_MASK_FLOOR = [0.141, 0.041, 0.105, 0.029, 0.203, 0.216]


@pytest.fixture(scope="module")
def problem():
    scenes, th, tg = D.grad_batch(2, 256)
    return scenes, th, tg


def _render(ctx, scenes, thetas, precision):
    R = D.Renderer(ctx, scenes, precision)
    R.set_theta(thetas)
    R.forward()
    return R


def _target(ctx, scenes, tg):
    return _render(ctx, scenes, tg, mb.PREC_FP32_FIX).image.clone()


def _interior(Rp, R0, Rm, Ip, I0, Im):
    same = ((Rp.hit == 1) & (Rm.hit == 1) & (R0.hit == 1) & (Rp.colour == Rm.colour).all(-1)
            & (Rp.colour == R0.colour).all(-1) & (Rp.iters == Rm.iters) & (Rp.iters == R0.iters))
    d2 = (Ip - 2 * I0 + Im).abs().amax(-1)
    d1 = (Ip - Im).abs().amax(-1)
    return same & (d2 <= 1e-3 * d1 + 1e-9)


def _adjoint_vs_fd(ctx, problem, precision):
    import torch
    scenes, th, tg = problem
    n = len(scenes)
    T = _target(ctx, scenes, tg)
    R = _render(ctx, scenes, th, precision)
    I = R.image.clone()
    jac = torch.zeros((n, 256, 256, 3, 6), dtype=torch.float32, device="cuda")
    R.backward(2 * (I - T), jac)
    st = ctx.stats()
    assert st.grad_pixels > 0.5 * int((R.hit > 0).sum())
    R64 = R if precision == mb.PREC_FP64 else _render(ctx, scenes, th, mb.PREC_FP64)
    I64 = R64.image.clone()
    worst = 0.0
    for j in range(6):
        tp, tm = th.copy(), th.copy()
        tp[:, j] += H
        tm[:, j] -= H
        Rp, Rm = _render(ctx, scenes, tp, mb.PREC_FP64), _render(ctx, scenes, tm, mb.PREC_FP64)
        Ip, Im = Rp.image.clone(), Rm.image.clone()
        mask = _interior(Rp, R64, Rm, Ip, I64, Im) & (R.hit == 1)
        if R is not R64:
            # FP32 forward state: pixels whose palette index and iteration count agree with the
            # FP64 render (the FP32 colouring orbit runs N x 10 iterations and its integer
            # palette index can differ), and whose shaded value agrees to FP32 noise
            mask &= ((R.colour == R64.colour).all(-1) & (R.iters == R64.iters)
                     & ((I - I64).abs().amax(-1) <= 1e-4))
        m = mask[..., None].double()
        fd = ((((Ip.double() - T.double()) ** 2 - (Im.double() - T.double()) ** 2) * m).sum(dim=(1, 2, 3))
              / (2 * H)).cpu().numpy()
        adj = ((2 * (I.double() - T.double()))[..., None] * jac.double() * m[..., None]).sum(
            dim=(1, 2, 3))[:, j].cpu().numpy()
        frac = float(mask.float().mean())
        hit_frac = frac / max(float((R.hit == 1).float().mean()), 1e-12)
        print(f"interior mask {D.NAMES[j]}: {frac:.4f} of pixels, {hit_frac:.4f} of hits ({precision=})")
        assert frac > MASK_FLOOR[j], (D.NAMES[j], frac)
        rel = np.abs(adj - fd) / np.abs(fd)
        worst = max(worst, float(rel.max()))
        assert (rel <= REL_TOL).all(), (D.NAMES[j], fd, adj, rel)
    return worst


def test_adjoint_matches_central_differences_fp64(gpu_ctx, problem):
    _adjoint_vs_fd(gpu_ctx, problem, mb.PREC_FP64)


def test_adjoint_matches_central_differences_fp32_forward(gpu_ctx, problem):
    _adjoint_vs_fd(gpu_ctx, problem, mb.PREC_FP32_FIX)


def test_adjoint_matches_oracle_central_differences(gpu_ctx, oracle, problem):
    # CPU FD: the oracle's FP64 render (same level-set hits) at theta +- h
    import torch
    scenes, th, tg = problem
    scenes, th, tg = scenes[:1], th[:1], tg[:1]
    T = _target(gpu_ctx, scenes, tg)
    R = _render(gpu_ctx, scenes, th, mb.PREC_FP64)
    I = R.image.clone()
    jac = torch.zeros((1, 256, 256, 3, 6), dtype=torch.float32, device="cuda")
    R.backward(2 * (I - T), jac)
    Tn = T[0].double().cpu().numpy()
    c0 = oracle_lib.render_exact(oracle, D.with_theta(scenes[0], th[0]))
    for j in range(6):
        tp, tm = th[0].copy(), th[0].copy()
        tp[j] += H
        tm[j] -= H
        cp = oracle_lib.render_exact(oracle, D.with_theta(scenes[0], tp))
        cm = oracle_lib.render_exact(oracle, D.with_theta(scenes[0], tm))
        Ip, I0, Im = (x.image_float.astype(np.float64) for x in (cp, c0, cm))
        same = ((cp.hit == 1) & (c0.hit == 1) & (cm.hit == 1) & (cp.colour == cm.colour).all(-1)
                & (cp.colour == c0.colour).all(-1) & (cp.iters == cm.iters) & (cp.iters == c0.iters))
        d2 = np.abs(Ip - 2 * I0 + Im).max(-1)
        d1 = np.abs(Ip - Im).max(-1)
        mask = same & (d2 <= 1e-3 * d1 + 1e-9) & (R.hit[0].cpu().numpy() == 1)
        # and pixels where the GPU and CPU forward images agree (libm last-bit differences can
        # flip a palette index or an iteration count)
        mask &= np.abs(I[0].double().cpu().numpy() - I0).max(-1) <= 1e-9
        m = mask[..., None]
        fd = float((((Ip - Tn) ** 2 - (Im - Tn) ** 2) * m).sum() / (2 * H))
        adj = float(((2 * (I[0].double().cpu().numpy() - Tn))[..., None] * jac[0].double().cpu().numpy()
                     * m[..., None]).sum(axis=(0, 1, 2))[j])
        print(f"oracle interior mask {D.NAMES[j]}: {mask.mean():.4f} of pixels")
        assert mask.mean() > ORACLE_MASK_FLOOR[j], (D.NAMES[j], mask.mean())
        assert abs(adj - fd) <= REL_TOL * abs(fd), (D.NAMES[j], fd, adj)


def test_autograd_function(gpu_ctx, problem):
    import torch
    scenes, th, tg = problem
    T = _target(gpu_ctx, scenes, tg)
    render = D.render_function()
    R = D.Renderer(gpu_ctx, scenes, mb.PREC_FP32_FIX)
    theta = torch.tensor(th, dtype=torch.float64, requires_grad=True)
    loss = ((render(theta, R) - T) ** 2).sum()
    loss.backward()
    R2 = D.Renderer(gpu_ctx, scenes, mb.PREC_FP32_FIX)
    R2.set_theta(th)
    I = R2.forward()
    direct = R2.backward(2 * (I - T))
    np.testing.assert_allclose(theta.grad.numpy(), direct, rtol=1e-12, atol=0)
    assert np.isfinite(direct).all() and np.abs(direct).max() > 0


def test_exact_hits_stay_close_to_the_reference_render(gpu_ctx, oracle, problem):
    scenes, th, _ = problem
    sc = D.with_theta(scenes[0], th[0])
    plain = gpu_ctx.render(sc, precision=mb.PREC_FP64)
    exact = gpu_ctx.render(sc, precision=mb.PREC_FP64, exact_hit=True)
    st = gpu_ctx.stats()
    hits = int((exact.hit > 0).sum())
    assert st.level_set_missed <= 0.01 * hits, (st.level_set_missed, hits)
    m = metrics.compare(exact, plain)
    assert m["hit_mismatch"] == 0.0
    # the level set lies inside the bisection window: depth moves by a small fraction of thr
    assert m["depth_rel_p99"] < 1e-3, m
    # the oracle's level-set render: same hits and depths
    ref = oracle_lib.render_exact(oracle, sc)
    m2 = metrics.compare(exact, ref)
    assert m2["hit_mismatch"] <= 0.001 and m2["depth_rel_p99"] < 1e-9, m2


def test_grad_rejects_unsupported_scenes(gpu_ctx):
    import torch
    from mandelbulber_gb300 import workloads as W
    sc = W.workload("mandelbox_1080p", 64, 36)   # ray-traced AO, fog, glow
    img = torch.zeros((36, 64, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(mb.MbgbError):
        gpu_ctx.render_grad([sc], [{"image_float": img.data_ptr()}])
