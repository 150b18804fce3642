"""Ray-traced reflections on the wavefront engine (needs a GPU).

The reflection loop of MainThread (src/Render3D.cpp:441-566) marches the camera ray, and
from every hit on a reflecting object the mirrored ray, up to reflectionsMax times; the
colour is composed far to near, each ray's object or background blended with the farther
rays' result by its reflectance, each followed by its VolumetricShader. The wavefront engine
runs one primary pass (and FP64 polish) per depth over the rays the reflect stage spawned,
shadow and AO rays for the hits of every depth in one stage, and the far-to-near walk in the
composition stage. Checks:
  * every reflection fixture in FP64 on the wavefront equals the per-pixel engine on hit,
    iterations and depth, with the float image within 60 dB (the golden test holds both
    engines to the reference's own output, bit for bit on the Mandelbox fixtures);
  * the FP64 wavefront frame is bit-exact to the oracle on the Mandelbox reflection scenes at
    sizes the fixtures do not cover;
  * the FP32 + FP64-fix policy against the FP64 oracle: hit mismatch <= 0.5 %, >= 45 dB and
    >= 98 % of the pixels within 0.01 in every channel; a scene whose constant threshold FP32
    cannot resolve goes to FP64 under AUTO;
  * the wavefront launches its stages once per depth (the launch count grows with the depth)
    and the per-pixel engine remains selectable.
"""
import glob
import os

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from tests import metrics, oracle_lib

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REFLECTION_CASES = sorted(os.path.basename(p)[7:-4]
                          for p in glob.glob(os.path.join(GOLDEN, "render_ex_fx_reflections_*.npz")))
EXACT = ["hit", "iters", "depth", "zbuffer", "alpha", "opacity", "colour"]


def _scene(case, w=None, h=None):
    z = np.load(os.path.join(GOLDEN, f"render_{case}.npz"))
    sc = mb.scene_from_bytes(z["scene"].tobytes())
    if w:
        sc.image_width, sc.image_height = w, h
        sc.resolution = 1.0 / w / sc.noOfTiles
    return sc


def _wavefront_carries(sc) -> bool:
    """The scene's effects are the wavefront's (no aux, fake or volumetric lights, iteration fog;
    reflections without slow shading or the limit box)."""
    aux = sc.auxLightNumber > 0 or any(sc.auxLightPreEnabled[i] for i in range(4))
    return not (aux or sc.fakeLightsEnabled or sc.volumetricLightEnabledAny or sc.iterFogEnabled
                or sc.slowShading or sc.limits_enabled)


def test_reflection_fixtures_exist():
    assert len(REFLECTION_CASES) >= 6, REFLECTION_CASES


@pytest.mark.parametrize("case", REFLECTION_CASES)
def test_wavefront_reflections_equal_the_per_pixel_engine_in_fp64(gpu_ctx, case):
    sc = _scene(case)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=mb.ENGINE_WAVEFRONT)
    wave_launches = gpu_ctx.stats().launches
    b = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=mb.ENGINE_PER_PIXEL)
    pp_launches = gpu_ctx.stats().launches
    for k in ["hit", "iters", "depth"]:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=f"{case}: {k}")
    m = metrics.compare(a, b)
    print(case, "wavefront vs per-pixel", m, "launches", wave_launches, pp_launches)
    assert m["psnr_float"] >= 60.0, m
    # one primary pass per depth plus the reflect stage between depths
    if _wavefront_carries(sc):
        assert wave_launches >= 3 + 3 * sc.reflectionsMax and pp_launches <= 2, (wave_launches, pp_launches)


@pytest.mark.parametrize("case,w,h", [("ex_fx_reflections_1", 160, 90), ("ex_fx_reflections_inverted_box", 128, 96),
                                      ("ex_fx_reflections_tglad_scale_m2", 128, 96)])
def test_mandelbox_reflections_fp64_equal_the_oracle(gpu_ctx, oracle, case, w, h):
    """The Mandelbox reflection scenes at a size the fixtures do not cover: the FP64 wavefront
    frame equals the strict oracle bit for bit (float image within 1e-6)."""
    sc = _scene(case, w, h)
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=mb.ENGINE_WAVEFRONT)
    for k in EXACT:
        np.testing.assert_array_equal(getattr(img, k), getattr(ref, k), err_msg=f"{case}: {k}")
    np.testing.assert_allclose(img.image_float, ref.image_float, rtol=0, atol=1e-6)


@pytest.mark.parametrize("case,w,h", [("ex_fx_reflections_foldintpow2", 160, 120),
                                      ("ex_fx_reflections_primitives_water", 160, 120),
                                      ("ex_fx_reflections_quaternion_julia", 128, 96),
                                      ("ex_fx_reflections_tglad_scale_m2", 128, 96),
                                      ("ex_fx_reflections_inverted_box", 128, 96)])
def test_fp32_reflections_against_the_oracle(gpu_ctx, oracle, case, w, h):
    """FP32 + FP64-fix on the wavefront: hit mismatch <= 0.5 %, >= 45 dB, >= 98 % of the
    pixels within 0.01 (each reflection compounds the FP32 normal's error; the per-pixel
    engine's FP32 frames score the same)."""
    sc = _scene(case, w, h)
    assert _wavefront_carries(sc)
    ref, _ = oracle_lib.render(oracle, sc)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, engine=mb.ENGINE_WAVEFRONT)
    m = metrics.compare(a, ref)
    close = float(np.mean(np.abs(a.image_float.astype(np.float64) - ref.image_float).max(-1) <= 0.01))
    print(case, "fp32 wavefront vs oracle", m, "within 0.01", close)
    assert m["hit_mismatch"] <= 0.005, m
    assert m["psnr_float"] >= 45.0 and close >= 0.98, (m, close)


def test_auto_renders_the_fine_constant_threshold_in_fp64(gpu_ctx, oracle):
    """ex_fx_reflections_1 marches to a constant threshold of 0.0002, whose bisection window
    (0.01 x quality x threshold = 4e-10) FP32 cannot resolve at |p| ~ 4: FP32 frames (either
    engine) land at ~23 dB. AUTO's window rule picks FP64, which equals the oracle bit for bit."""
    sc = _scene("ex_fx_reflections_1", 240, 135)
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=mb.PREC_AUTO, engine=mb.ENGINE_WAVEFRONT)
    assert gpu_ctx.stats().auto_fp64 == 1
    for k in EXACT:
        np.testing.assert_array_equal(getattr(img, k), getattr(ref, k), err_msg=k)
