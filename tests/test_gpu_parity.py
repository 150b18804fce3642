"""Device kernels against the oracle and the golden vectors (needs a GPU).

Tolerances (stated per test):
  * FP64 policy, Mandelbox: only + - * / sqrt on the orbit and the march, the
    kernel is built with --fmad=false, so hit mask, depth, iterations, z-buffer,
    alpha, opacity and colour are bit-exact; the float image differs from the
    CPU only through pow() in the specular term (|diff| <= 1e-6).
  * FP64 policy, Mandelbulb: asin/atan2/pow/sincos/log come from CUDA's libm,
    which may round differently from the CPU's in the last ulp, and the orbit is
    chaotic, so a few pixels may flip: hit mismatch <= 0.5 %, iteration agreement
    >= 90 % and PSNR >= 35 dB on the 32x32 .. 64x48 golden frames (one flipped
    pixel of a 32x32 frame alone costs several dB).
  * FP32 + FP64-refinement policy: hit/miss mismatch <= 0.1 % and PSNR >= 45 dB
    of the float image against the FP64 oracle (the headline metric's bar), at sizes the
    oracle finishes in seconds.
"""
import ctypes
import glob
import os

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W
from tests import metrics, oracle_lib

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RENDERS = sorted(os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(GOLDEN, "render_*.npz")))
LAYERS = ["image_float", "zbuffer", "alpha", "opacity", "colour", "hit", "iters", "depth"]


def _golden_image(z, w, h):
    img = mb.CImage.empty(w, h)
    for k in LAYERS:
        setattr(img, k, z[k])
    return img


def _device_distance(ctx, scene, pts, detail, precision):
    import torch
    n = len(pts)
    p = torch.tensor(pts, dtype=torch.float64, device="cuda")
    d = torch.tensor(detail, dtype=torch.float64, device="cuda")
    dist = torch.zeros(n, dtype=torch.float64, device="cuda")
    it = torch.zeros(n, dtype=torch.int32, device="cuda")
    mi = torch.zeros(n, dtype=torch.uint8, device="cuda")
    ctx.distance(scene, p.data_ptr(), d.data_ptr(), n, dist.data_ptr(), it.data_ptr(), mi.data_ptr(), precision)
    torch.cuda.synchronize()
    return dist.cpu().numpy(), it.cpu().numpy(), mi.cpu().numpy()


def test_distance_fp64_mandelbox_bit_exact(gpu_ctx):
    z = np.load(os.path.join(GOLDEN, "de_mandelbox.npz"))
    sc = mb.scene_from_bytes(z["scene"].tobytes())
    d, it, mi = _device_distance(gpu_ctx, sc, z["points"], z["detail"], mb.PREC_FP64)
    np.testing.assert_array_equal(d, z["dist"])
    np.testing.assert_array_equal(it, z["iters"])
    np.testing.assert_array_equal(mi, z["max_iter"])


def test_distance_fp64_mandelbulb_close(gpu_ctx):
    z = np.load(os.path.join(GOLDEN, "de_mandelbulb.npz"))
    sc = mb.scene_from_bytes(z["scene"].tobytes())
    d, it, mi = _device_distance(gpu_ctx, sc, z["points"], z["detail"], mb.PREC_FP64)
    agree = it == z["iters"]
    assert agree.mean() >= 0.98, agree.mean()
    rel = np.abs(d[agree] - z["dist"][agree]) / np.maximum(np.abs(z["dist"][agree]), 1e-300)
    assert np.percentile(rel, 99) < 1e-9, np.percentile(rel, 99)


DES = sorted(os.path.basename(p)[3:-4] for p in glob.glob(os.path.join(GOLDEN, "de_*.npz")))
RUNTIME_DES = [d for d in DES if d not in ("mandelbulb", "mandelbox")]


def _agreement(d, it, ref, ref_it):
    """Points where the device and the reference agree in iteration count and, where either
    distance is not finite (0/0 and overflow in a few delta-DE orbits, or a forward
    difference that vanished below the escape radius' last bit), in the non-finite value;
    and the relative differences of the finite distances there."""
    fin = np.isfinite(d) & np.isfinite(ref)
    same_nonfin = (d == ref) | (np.isnan(d) & np.isnan(ref))
    agree = (it == ref_it) & (fin | same_nonfin)
    both = agree & fin
    rel = np.abs(d[both] - ref[both]) / np.maximum(np.abs(ref[both]), 1e-300)
    return agree, rel


@pytest.mark.parametrize("formula", RUNTIME_DES)
def test_distance_fp64_runtime_formulas(gpu_ctx, formula):
    """Every run-time formula (1, 3-7, 10, 11, 13-37, the hybrid sequences, the IFS pre-fold)
    against the reference's own distances: the same iteration counts (and the same value
    where a distance is not finite) on >= 98 % of the points, and there distances within
    1e-9 relative (99th percentile) for the analytic
    estimators, within 1e-4 for the delta-DE ones. The formulas built from + - * / sqrt come
    out bit for bit; in the trigonometric ones a last-bit difference of the device's and the
    C library's sin / cos / atan2 moves the escape radius by an ulp, which the forward
    difference with step 1e-10 scales by up to 1e10 / |grad r|."""
    z = np.load(os.path.join(GOLDEN, f"de_{formula}.npz"))
    sc = mb.scene_from_bytes(z["scene"].tobytes())
    d, it, mi = _device_distance(gpu_ctx, sc, z["points"], z["detail"], mb.PREC_FP64)
    agree, rel = _agreement(d, it, z["dist"], z["iters"])
    exact = float(np.mean((d == z["dist"]) | (np.isnan(d) & np.isnan(z["dist"]))))
    print(formula, "analytic", sc.analitycDE, "iters agree", agree.mean(), "bit-exact", exact,
          "rel p99", np.percentile(rel, 99), "max", rel.max())
    assert agree.mean() >= 0.98, agree.mean()
    assert np.percentile(rel, 99) < (1e-9 if sc.analitycDE else 1e-4), np.percentile(rel, 99)
    np.testing.assert_array_equal(mi[agree], z["max_iter"][agree])


@pytest.mark.parametrize("formula", DES)
def test_distance_fp32_close(gpu_ctx, formula):
    z = np.load(os.path.join(GOLDEN, f"de_{formula}.npz"))
    sc = mb.scene_from_bytes(z["scene"].tobytes())
    d, it, mi = _device_distance(gpu_ctx, sc, z["points"], z["detail"], mb.PREC_FP32_FIX)
    agree, _ = _agreement(d, it, z["dist"], z["iters"])
    assert agree.mean() >= 0.9, agree.mean()
    far = agree & (z["dist"] > 1e-3) & np.isfinite(z["dist"])
    rel = np.abs(d[far] - z["dist"][far]) / z["dist"][far]
    assert np.median(rel) < 1e-4, np.median(rel)


ENGINES = [mb.ENGINE_WAVEFRONT, mb.ENGINE_PER_PIXEL]


@pytest.mark.parametrize("engine", ENGINES, ids=["wavefront", "per_pixel"])
@pytest.mark.parametrize("case", RENDERS)
def test_render_fp64_against_reference_golden(gpu_ctx, case, engine):
    """FP64 device render vs the reference's own output (golden vectors)."""
    z = np.load(os.path.join(GOLDEN, f"render_{case}.npz"))
    sc = mb.scene_from_bytes(z["scene"].tobytes())
    img = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=engine)
    ref = _golden_image(z, sc.image_width, sc.image_height)
    m = metrics.compare(img, ref)
    # the Mandelbox frames come out bit for bit, except where the environment map's texel
    # (an 8-bit truncation of an atan2-derived coordinate) amplifies a libm last bit
    env_mapped = sc.reflect > 0 and not sc.raytracedReflections
    if sc.formula == 8 and sc.perspectiveType == 0 and not env_mapped:
        for k in ["hit", "iters", "depth", "zbuffer", "alpha", "opacity", "colour"]:
            np.testing.assert_array_equal(getattr(img, k), z[k], err_msg=f"{case}: {k}")
        np.testing.assert_allclose(img.image_float, z["image_float"], rtol=0, atol=1e-6)
    else:
        assert m["hit_mismatch"] <= 0.005, m
        if "iters_agree" in m:
            assert m["iters_agree"] >= 0.90, m
        assert m["psnr_float"] >= 35.0, m


@pytest.mark.parametrize("engine", ENGINES, ids=["wavefront", "per_pixel"])
@pytest.mark.parametrize("name,size", [("mandelbulb_640x480", (320, 240)), ("mandelbox_1080p", (480, 270))])
def test_render_fp32_fix_against_oracle(gpu_ctx, oracle, name, size, engine):
    """FP32 march + FP64 refinement vs the FP64 oracle: <= 0.1 % hit mismatch, >= 45 dB."""
    sc = W.workload(name, *size)
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, engine=engine)
    m = metrics.compare(img, ref)
    print(name, m)
    assert m["hit_mismatch"] <= 0.001, m
    assert m["psnr_float"] >= 45.0, m


def test_deep_zoom_against_oracle(gpu_ctx, oracle):
    """Deep zoom (Mandelbulb power 8, N 1000, camera 1e-6 from a seeded surface point) at
    48x48: MBGB_PREC_AUTO picks FP64 and renders the FP64 frame exactly; that frame meets
    the FP64 Mandelbulb bar against the oracle (hit mismatch <= 0.5 %, PSNR >= 35 dB)."""
    sc = W.deep_zoom(gpu_ctx, size=48)
    ref, _ = oracle_lib.render(oracle, sc)
    auto = gpu_ctx.render(sc, precision=mb.PREC_AUTO)
    assert gpu_ctx.stats().auto_fp64 == 1
    f64 = gpu_ctx.render(sc, precision=mb.PREC_FP64)
    for k in LAYERS:
        np.testing.assert_array_equal(getattr(auto, k), getattr(f64, k), err_msg=k)
    m = metrics.compare(f64, ref)
    print("deep zoom", m)
    assert m["hit_fraction"] > 0.5, m
    assert m["hit_mismatch"] <= 0.005, m
    assert m["psnr_float"] >= 35.0, m


def _fixture_scene(case, w, h):
    """The scene of render fixture `case` at another size (same perspective)."""
    z = np.load(os.path.join(GOLDEN, f"render_{case}.npz"))
    sc = mb.scene_from_bytes(z["scene"].tobytes())
    sc.image_width, sc.image_height = w, h
    sc.resolution = 1.0 / w / sc.noOfTiles
    return sc


RUNTIME_SCENES = {
    "trigde": ("mandelbulb_640x480", (160, 120), {"formula": 1, "power": 6, "angle_alfa": 30, "angle_beta": 19,
                                                 "view_point_x": 1.75, "view_point_y": -3.0, "view_point_z": -1.2}),
    "menger": ("mandelbulb_640x480", (160, 120), {"formula": 7, "N": 50, "view_point_x": 0.9, "view_point_z": 0.6,
                                                 "angle_alfa": -14, "angle_beta": -9}),
    "vary4d": ("mandelbox_1080p", (192, 108), {**W.VARY4D, "mandelbox_scale": 2.0}),
}


FIXTURE_SCENES = {"kaleidoscopic": ("ex_ifs_icosahedron", 160, 120), "smooth_mandelbox": ("smooth_mandelbox", 192, 128),
                  "fold_box": ("fold_box_icosa", 192, 128)}


@pytest.mark.parametrize("engine", ENGINES, ids=["wavefront", "per_pixel"])
@pytest.mark.parametrize("formula", sorted(RUNTIME_SCENES) + sorted(FIXTURE_SCENES))
def test_render_fp32_fix_runtime_formulas(gpu_ctx, oracle, formula, engine):
    """The FP32 policy on the analytic run-time formulas (1, 7, 10, 17, 18, 37) against the
    FP64 oracle, with the same bar as the headline scenes: <= 0.1 % hit mismatch, >= 45 dB
    float-image PSNR."""
    if formula in FIXTURE_SCENES:
        sc = _fixture_scene(*FIXTURE_SCENES[formula])
    else:
        name, size, extra = RUNTIME_SCENES[formula]
        sc = W.workload(name, *size, **extra)
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, engine=engine)
    m = metrics.compare(img, ref)
    print(formula, m)
    assert m["hit_mismatch"] <= 0.001, m
    assert m["psnr_float"] >= 45.0, m


DELTA_SCENES = [("ex_power2_default", 128, 96), ("ex_hybrid_1", 96, 64), ("ex_quaternion_lathe", 128, 96),
                ("ex_modified_mandelbulb_3", 128, 96), ("hybrid_modifiers", 96, 72)]


@pytest.mark.parametrize("case,w,h", DELTA_SCENES)
def test_delta_de_scenes_render_in_fp64(gpu_ctx, oracle, case, w, h):
    """Delta-DE formulas (src/fractal.cpp:1308-1381) render in FP64 under the FP32 policy,
    bit for bit the FP64 render, and match the FP64 oracle at sizes the fixtures do not
    cover: <= 0.5 % hit mismatch, >= 40 dB float-image PSNR (libm last-bit differences in
    the trigonometric formulas move a few hits)."""
    sc = _fixture_scene(case, w, h)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX)
    assert gpu_ctx.stats().auto_fp64 == 1
    b = gpu_ctx.render(sc, precision=mb.PREC_FP64)
    for k in LAYERS:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)
    ref, _ = oracle_lib.render(oracle, sc)
    m = metrics.compare(b, ref)
    print(case, m)
    assert m["hit_mismatch"] <= 0.005, m
    assert m["psnr_float"] >= 40.0, m


EFFECT_SCENES = [("ex_aux_coloured_lights", 96, 64), ("ex_fx_iter_fog_2", 96, 64), ("ex_fx_volumetric_light_2", 96, 64),
                 ("ex_fx_slow_interior_mandelbox", 64, 48), ("fake_lights_mandelbox", 96, 64),
                 ("envmap_mandelbulb", 96, 72), ("aux_random_visible", 96, 72)]


@pytest.mark.parametrize("case,w,h", EFFECT_SCENES)
def test_effects_fp32_against_fp64(gpu_ctx, oracle, case, w, h):
    """Secondary effects (aux / fake / volumetric lights, iteration fog, slow shading,
    environment mapping) under the FP32 policy against the FP64 render, which the fixtures
    pin to the reference, at sizes the fixtures do not cover: <= 0.5 % hit mismatch and
    >= 99 % of the pixels within 0.01 in every channel (the rest are palette-index flips of
    the FP32 colouring orbit, N x 10 iterations); and the FP64 render against the FP64
    oracle (>= 60 dB)."""
    sc = _fixture_scene(case, w, h)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX)
    b = gpu_ctx.render(sc, precision=mb.PREC_FP64)
    m = metrics.compare(a, b)
    close = float(np.mean(np.abs(a.image_float.astype(np.float64) - b.image_float).max(-1) <= 0.01))
    print(case, "fp32 vs fp64", m, "within 0.01", close)
    assert m["hit_mismatch"] <= 0.005, m
    assert close >= 0.99, close
    ref, _ = oracle_lib.render(oracle, sc)
    m2 = metrics.compare(b, ref)
    print(case, "fp64 vs oracle", m2)
    assert m2["hit_mismatch"] <= 0.005 and m2["psnr_float"] >= 60.0, m2


def test_fp32_fix_with_full_fp64_polish(gpu_ctx, oracle):
    """polish_all: every hit finishes its bisection in FP64; same parity bar, more polished hits."""
    sc = W.workload("mandelbox_1080p", 320, 180)
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, polish_all=True)
    all_polished = gpu_ctx.stats().fp64_polished
    m = metrics.compare(img, ref)
    assert m["hit_mismatch"] <= 0.001 and m["psnr_float"] >= 45.0, m
    assert all_polished == int(ref.hit.sum()) or abs(all_polished - int(img.hit.sum())) == 0
    gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX)
    assert gpu_ctx.stats().fp64_polished < all_polished


def test_full_size_fp32_fix_against_fp64(gpu_ctx):
    """At the full 1080p size: FP32+fix vs the FP64 device path (the oracle is too slow there)."""
    sc = W.workload("mandelbox_1080p")
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX)
    b = gpu_ctx.render(sc, precision=mb.PREC_FP64)
    m = metrics.compare(a, b)
    c = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=mb.ENGINE_PER_PIXEL)
    # the two engines agree exactly in FP64 on hits and depth
    np.testing.assert_array_equal(b.hit, c.hit)
    np.testing.assert_array_equal(b.depth, c.depth)
    print(m)
    assert m["hit_mismatch"] <= 0.001, m
    assert m["psnr_float"] >= 45.0, m


@pytest.mark.parametrize("engine", ENGINES, ids=["wavefront", "per_pixel"])
def test_long_rays_take_the_overflow_pass(gpu_ctx, oracle, engine):
    """Rays longer than the main pass's step records are re-rendered with full-length records."""
    sc = W.workload("mandelbox_1080p", 96, 54, DE_factor=0.01)
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=engine)
    assert gpu_ctx.stats().long_rays > 0
    for k in ["hit", "iters", "depth", "zbuffer", "alpha", "opacity", "colour"]:
        np.testing.assert_array_equal(getattr(img, k), getattr(ref, k), err_msg=k)
    np.testing.assert_allclose(img.image_float, ref.image_float, rtol=0, atol=1e-6)


def test_render_is_deterministic_and_row_ranges_compose(gpu_ctx):
    sc = W.workload("mandelbox_1080p", 320, 180)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX)
    b = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX)
    for k in LAYERS:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k))
    c = mb.CImage.empty(320, 180)
    gpu_ctx.render(sc, c, precision=mb.PREC_FP32_FIX, rows=(0, 77))
    gpu_ctx.render(sc, c, precision=mb.PREC_FP32_FIX, rows=(77, 180))
    np.testing.assert_array_equal(c.image_float, a.image_float)


def test_jitter_changes_steps_but_not_the_picture(gpu_ctx):
    """Step jitter (the reference's Random(1000) factor) perturbs the march only slightly."""
    sc = W.workload("mandelbox_1080p", 320, 180)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX)
    b = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, jitter=True, jitter_seed=7)
    m = metrics.compare(b, a)
    assert m["hit_mismatch"] <= 0.01 and m["psnr_float"] >= 30.0, m
    assert not np.array_equal(a.depth, b.depth)


def test_errors_are_status_codes(gpu_ctx):
    sc = W.workload("mandelbulb_640x480", 64, 48, formula=38)   # ocl_custom: not on the device
    with pytest.raises(mb.MbgbError) as e:
        gpu_ctx.render(sc)
    assert e.value.status == 5
    sc = W.workload("mandelbulb_640x480", 64, 48)
    with pytest.raises(mb.MbgbError) as e:
        gpu_ctx.render(sc, mb.CImage.empty(32, 32))
    assert e.value.status == 1
    with pytest.raises(mb.MbgbError) as e:
        gpu_ctx.render(sc, rows=(40, 10))
    assert e.value.status == 1
    with pytest.raises(mb.MbgbError) as e:
        gpu_ctx.render(sc, precision=9)
    assert e.value.status == 1


def test_device_deadline_returns_timeout_and_context_survives(gpu_ctx):
    """A 1 ms device budget on a full frame stops the kernel early with MBGB_ERR_TIMEOUT."""
    sc = W.workload("mandelbox_1080p")
    with pytest.raises(mb.MbgbError) as e:
        gpu_ctx.render(sc, precision=mb.PREC_FP64, deadline_ms=1)
    assert e.value.status == 4
    small = W.workload("mandelbox_1080p", 64, 36)
    img = gpu_ctx.render(small, precision=mb.PREC_FP32_FIX)
    assert img.hit.mean() > 0.5


@pytest.mark.parametrize("precision", [mb.PREC_FP64, mb.PREC_FP32_FIX], ids=["fp64", "fp32_fix"])
def test_mandelbulb_escape_radius_10_against_oracle(gpu_ctx, oracle, precision):
    """The Mandelbulb configuration's r > 10 escape radius (scene bailoutRadius; the
    reference hard-codes r > 100) on the device and in the oracle: the FP64 Mandelbulb bar
    (hit mismatch <= 0.5 %, PSNR >= 35 dB) and the FP32 policy's bar (<= 0.1 %, >= 45 dB)."""
    sc = W.workload("mandelbulb_640x480", 320, 240)
    sc.bailoutRadius = 10
    ref, _ = oracle_lib.render(oracle, sc)
    img = gpu_ctx.render(sc, precision=precision)
    m = metrics.compare(img, ref)
    print("r > 10", precision, m)
    if precision == mb.PREC_FP64:
        assert m["hit_mismatch"] <= 0.005 and m["psnr_float"] >= 35.0, m
    else:
        assert m["hit_mismatch"] <= 0.001 and m["psnr_float"] >= 45.0, m
    default = gpu_ctx.render(W.workload("mandelbulb_640x480", 320, 240), precision=precision)
    assert not np.array_equal(default.depth, img.depth)


@pytest.mark.parametrize("engine", ENGINES, ids=["wavefront", "per_pixel"])
def test_mandelbox_limit_box_on_the_lean_orbit(gpu_ctx, oracle, engine):
    """The limit box (src/fractal.cpp:1252-1262) on the Mandelbox that the lean FP32 orbit
    renders: the box test runs before the orbit and its distance bounds the result after it,
    in every stage (march, polish, shadow and AO rays, normals).
      * FP64: bit-exact to the oracle on the exact layers.
      * FP32 + FP64-fix: hit mismatch <= 0.1 %, depth within 1e-5 (p99), iterations agree on
        >= 99.9 % of hits, and >= 45 dB on the pixels the box does not cut (same hit and depth
        as without the box). The cut faces expose the fractal's interior, where the colouring
        orbit (N x 10 iterations) and the AO samples' escape test never settle: FP32 flips
        their palette index and occlusion there (about 25 dB over the whole frame, the same
        with the generic FP32 orbit), so AUTO renders limit-box scenes in FP64.
    """
    box = dict(limits_enabled=1, x_max=1.5, y_min=-2.5, z_max=2.0)
    sc = W.workload("mandelbox_1080p", 320, 180, **box)
    ref, _ = oracle_lib.render(oracle, sc)
    b = gpu_ctx.render(sc, precision=mb.PREC_FP64, engine=engine)
    for k in ["hit", "iters", "depth", "zbuffer", "alpha", "opacity", "colour"]:
        np.testing.assert_array_equal(getattr(b, k), getattr(ref, k), err_msg=k)
    a = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, engine=engine)
    m = metrics.compare(a, ref)
    plain, _ = oracle_lib.render(oracle, W.workload("mandelbox_1080p", 320, 180))
    uncut = (ref.hit == plain.hit) & (np.abs(ref.depth - plain.depth) <= 1e-9 * np.abs(plain.depth))
    m["psnr_uncut"] = metrics.psnr(a.image_float[uncut], ref.image_float[uncut])
    m["cut_fraction"] = float(1.0 - uncut.mean())
    print("limit box", engine, m)
    assert m["hit_mismatch"] <= 0.001 and m["depth_rel_p99"] <= 1e-5 and m["iters_agree"] >= 0.999, m
    assert m["psnr_uncut"] >= 45.0 and 0.1 < m["cut_fraction"] < 0.9, m
    auto = gpu_ctx.render(sc, precision=mb.PREC_AUTO, engine=engine)
    for k in ["hit", "iters", "depth", "zbuffer", "alpha", "opacity", "colour"]:
        np.testing.assert_array_equal(getattr(auto, k), getattr(ref, k), err_msg=k)
