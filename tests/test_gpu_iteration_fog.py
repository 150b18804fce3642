"""Iteration fog on the wavefront engine (needs a GPU).

VolumetricShader's iteration fog (src/shaders.cpp:385-466) blends into every step group of
positive opacity a fog colour chosen by the record's iteration count, lit by the main light
and the predefined aux lights through shadows traced from the group and by ray-traced AO;
every shadow, AO and aux-shadow march absorbs through the fog along the way and compares
against its samples' eye-distance thresholds at DE factor 1 (src/shaders.cpp:515-539,
646-659, 1083-1099). On the wavefront the sample stage lists the groups of positive opacity,
the shadow stage traces their shadows and AO directions next to the hits', and the
composition stage blends them in the reference's order. Checks:
  * every iteration-fog fixture the wavefront carries, in FP64, equals the per-pixel engine
    on hit, iterations and depth, float image within 60 dB;
  * the Mandelbox fixtures in FP64 at a larger size equal the oracle bit for bit;
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
    return bool(sc.iterFogEnabled) and not (sc.fakeLightsEnabled or sc.slowShading or sc.limits_enabled
                                            or sc.iterThresh or sc.interiorMode)


FOG_CASES = sorted(c for c in (os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(GOLDEN, "render_*.npz")))
                   if _on_wavefront(_scene(c)))


def test_iteration_fog_fixtures_reach_the_wavefront():
    assert len(FOG_CASES) >= 3, FOG_CASES


@pytest.mark.parametrize("case", FOG_CASES)
def test_wavefront_iteration_fog_equals_the_per_pixel_engine_in_fp64(gpu_ctx, case):
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


@pytest.mark.parametrize("case", ["ex_fx_iter_fog_1", "ex_fx_iter_fog_2"])
def test_mandelbox_iteration_fog_fp64_equals_the_oracle(gpu_ctx, oracle, case):
    sc = _scene(case, 128, 96)
    assert _on_wavefront(sc) and sc.formula == 8
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=mb.ENGINE_WAVEFRONT)
    for k in EXACT:
        np.testing.assert_array_equal(getattr(img, k), getattr(ref, k), err_msg=f"{case}: {k}")
    np.testing.assert_allclose(img.image_float, ref.image_float, rtol=0, atol=1e-6)


@pytest.mark.parametrize("case,w,h", [("ex_fx_iter_fog_2", 160, 120), ("ex_fx_iter_fog_1", 128, 96),
                                      ("iter_fog_mandelbulb", 128, 96)])
def test_fp32_iteration_fog_against_the_oracle(gpu_ctx, oracle, case, w, h):
    sc = _scene(case, w, h)
    assert _on_wavefront(sc)
    ref, _ = oracle_lib.render(oracle, sc)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, engine=mb.ENGINE_WAVEFRONT)
    m = metrics.compare(a, ref)
    close = float(np.mean(np.abs(a.image_float.astype(np.float64) - ref.image_float).max(-1) <= 0.01))
    print(case, "fp32 wavefront vs oracle", m, "within 0.01", close)
    assert m["hit_mismatch"] <= 0.005, m
    assert close >= 0.99, close
