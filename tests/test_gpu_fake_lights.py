"""Fake (orbit trap) lights on the wavefront engine (needs a GPU).

FakeLights (src/shaders.cpp:1225-1271) lights every hit by the orbit trap's distance and its
forward-difference gradient, and VolumetricShader (src/shaders.cpp:298-307) adds the trap's
glow at every step group. On the wavefront the composition stage evaluates the hit's four
orbit traps, the sample stage lists every ray's step groups, the shadow stage computes each
group's orbit trap, and the composition adds the glow in the reference's order. Checks:
  * every fake-light fixture in FP64 on the wavefront equals the per-pixel engine on hit,
    iterations and depth, float image within 60 dB;
  * the Mandelbox fixture in FP64 at a larger size equals the oracle bit for bit;
  * FP32 + FP64-fix against the oracle: hit mismatch <= 0.5 %, >= 99 % of the pixels within
    0.01 (the effect scenes' bar).
"""
import glob
import os

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from tests import metrics, oracle_lib

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EXACT = ["hit", "iters", "depth", "zbuffer", "alpha", "opacity", "colour"]


def _scene(case, w=None, h=None):
    z = np.load(os.path.join(GOLDEN, f"render_{case}.npz"))
    sc = mb.scene_from_bytes(z["scene"].tobytes())
    if w:
        sc.image_width, sc.image_height = w, h
        sc.resolution = 1.0 / w / sc.noOfTiles
    return sc


def _on_wavefront(sc) -> bool:
    return bool(sc.fakeLightsEnabled) and not (sc.slowShading or sc.limits_enabled or sc.iterThresh
                                               or sc.interiorMode)


FAKE_CASES = sorted(c for c in (os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(GOLDEN, "render_*.npz")))
                   if _on_wavefront(_scene(c)))


def test_fake_light_fixtures_reach_the_wavefront():
    assert len(FAKE_CASES) >= 2, FAKE_CASES


@pytest.mark.parametrize("case", FAKE_CASES)
def test_wavefront_fake_lights_equal_the_per_pixel_engine_in_fp64(gpu_ctx, case):
    sc = _scene(case)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=mb.ENGINE_WAVEFRONT)
    wave_launches = gpu_ctx.stats().launches
    b = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=mb.ENGINE_PER_PIXEL)
    for k in ["hit", "iters", "depth"]:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=f"{case}: {k}")
    m = metrics.compare(a, b)
    print(case, "wavefront vs per-pixel", m, "launches", wave_launches)
    assert m["psnr_float"] >= 60.0, m
    assert wave_launches >= 4, wave_launches


@pytest.mark.parametrize("case", ["fake_lights_mandelbox"])
def test_mandelbox_fake_lights_fp64_equal_the_oracle(gpu_ctx, oracle, case):
    sc = _scene(case, 128, 96)
    assert _on_wavefront(sc) and sc.formula == 8
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=mb.ENGINE_WAVEFRONT)
    for k in EXACT:
        np.testing.assert_array_equal(getattr(img, k), getattr(ref, k), err_msg=f"{case}: {k}")
    np.testing.assert_allclose(img.image_float, ref.image_float, rtol=0, atol=1e-6)


@pytest.mark.parametrize("case,w,h", [("fake_lights_mandelbox", 160, 120), ("fake_lights", 128, 96)])
def test_fp32_fake_lights_against_the_oracle(gpu_ctx, oracle, case, w, h):
    sc = _scene(case, w, h)
    assert _on_wavefront(sc)
    ref, _ = oracle_lib.render(oracle, sc)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, engine=mb.ENGINE_WAVEFRONT)
    m = metrics.compare(a, ref)
    close = float(np.mean(np.abs(a.image_float.astype(np.float64) - ref.image_float).max(-1) <= 0.01))
    print(case, "fp32 wavefront vs oracle", m, "within 0.01", close)
    assert m["hit_mismatch"] <= 0.005, m
    assert close >= 0.99, close
