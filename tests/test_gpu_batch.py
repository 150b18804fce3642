"""Batched frames, CUDA-graph replay and the autotuner (needs a GPU).

A batch renders frames of MainRender's keyframe / flight loops (src/Render3D.cpp:2144-2350)
in one launch sequence; every frame must come out exactly as the same frame rendered
alone, because each pixel's arithmetic does not depend on which warp or launch renders
it. The same holds for the tuned launch configurations (tile shape, threads per CTA,
CTAs per SM, refill thresholds) and for graph replays: those tests compare bit for bit.
The flight frames are also held against the FP64 oracle with the FP32 policy's bar
(hit/miss mismatch <= 0.1 %, float-image PSNR >= 45 dB).
"""
import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W
from tests import metrics, oracle_lib

pytestmark = pytest.mark.gpu
LAYERS = ["image_float", "zbuffer", "alpha", "opacity", "colour", "hit", "iters", "depth"]


def _same(a, b, what=""):
    for k in LAYERS:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=f"{what} layer {k}")


@pytest.fixture(scope="module")
def flight_small():
    # 64 frames from 80x60 to 480x270
    return W.flight(downscale=4)


def test_flight_batch_equals_single_frames(gpu_ctx, flight_small):
    batch = gpu_ctx.render_batch(flight_small)
    st = gpu_ctx.stats()
    assert st.frames == 64
    assert st.pixels == sum(f.image_width * f.image_height for f in flight_small)
    # one launch sequence: primary, polish, the hits' shadow set-up, secondary, compose, and
    # from 2^20 pixels on the three launches that put the hit list in tile order
    assert st.launches == 5 + (3 if st.pixels >= 1 << 20 else 0), st.launches
    for i in (0, 1, 7, 8, 31, 63):
        single = gpu_ctx.render(flight_small[i])
        _same(batch[i], single, f"frame {i}")


def test_graph_replay_equals_direct(gpu_ctx, flight_small):
    frames = flight_small[:16]
    direct = gpu_ctx.render_batch(frames)
    first = gpu_ctx.render_batch(frames, use_graph=True)
    assert gpu_ctx.stats().graph_replayed == 0
    again = gpu_ctx.render_batch(frames, images=[mb.CImage.empty(f.image_width, f.image_height) for f in frames],
                                 use_graph=True)
    # the host variant stages through the same device buffers, so the graph is replayed
    assert gpu_ctx.stats().graph_replayed == 1
    for i in range(len(frames)):
        _same(direct[i], first[i], f"capture frame {i}")
        _same(direct[i], again[i], f"replay frame {i}")
    # a render of something else in between, then the replay still reads its own frame table
    gpu_ctx.render(flight_small[40])
    third = gpu_ctx.render_batch(frames, use_graph=True)
    assert gpu_ctx.stats().graph_replayed == 1
    for i in range(len(frames)):
        _same(direct[i], third[i], f"replay after another render, frame {i}")


def test_autotune_and_tuned_render(gpu_ctx, flight_small):
    big = max(flight_small, key=lambda f: f.image_width * f.image_height)
    t = gpu_ctx.autotune(big)
    assert t.tile_w * t.tile_h == 32
    assert t.threads_per_cta in (64, 128)
    assert t.refill_min in (1, 4, 8, 16)
    assert t.orbit_refill in (0, 8, 16)
    assert t.trials >= 8 and 0 < t.ms <= t.ms_default * 1.0001
    ref = gpu_ctx.render_batch(flight_small[:8])
    tuned = gpu_ctx.render_batch(flight_small[:8], autotune=True)
    for i in range(8):
        _same(ref[i], tuned[i], f"tuned frame {i}")


@pytest.mark.parametrize("tile,refill,threads", [((32, 1), 16, 64), ((4, 8), 4, 128), ((16, 2), 8, 96)])
def test_launch_shapes_do_not_change_pixels(gpu_ctx, flight_small, tile, refill, threads):
    frames = flight_small[8:12]
    ref = gpu_ctx.render_batch(frames)
    got = gpu_ctx.render_batch(frames, tile=tile, refill_min=refill, threads_per_cta=threads)
    for i in range(len(frames)):
        _same(ref[i], got[i], f"frame {i}")


@pytest.mark.parametrize("orbit_refill", [-1, 1, 4, 16, 32])
def test_orbit_refill_does_not_change_pixels(gpu_ctx, flight_small, orbit_refill):
    # The shadow/AO stage's orbit-granular lane refill (lean Mandelbox and power-8
    # Mandelbulb orbits) reorders work between lanes only: every layer and the orbit and
    # distance-estimate counts of the stage match the per-estimate refill (-1) bit for bit.
    box = W.workload("mandelbox_1080p", 320, 180)
    for i, f in enumerate([box] + flight_small[8:10]):
        ref = gpu_ctx.render(f, orbit_refill=-1, profile_stages=True)
        ref_st = gpu_ctx.stats()
        got = gpu_ctx.render(f, orbit_refill=orbit_refill, profile_stages=True)
        st = gpu_ctx.stats()
        _same(ref, got, f"frame {i}, orbit_refill {orbit_refill}")
        assert st.stage_orbit[2] == ref_st.stage_orbit[2] and st.stage_de[2] == ref_st.stage_de[2]
        assert st.stage_de[2] > 0


def test_mixed_batch_groups(gpu_ctx):
    # frames that differ in fractal parameters render in separate launch sequences
    a = W.workload("mandelbulb_640x480", 96, 72)
    b = W.workload("mandelbulb_640x480", 64, 48, power=7)
    c = W.workload("mandelbox_1080p", 96, 54)
    d = W.workload("mandelbulb_640x480", 48, 36, view_point_x=0.4)
    frames = [a, b, c, d]
    batch = gpu_ctx.render_batch(frames)
    assert gpu_ctx.stats().frames == 4
    for i, f in enumerate(frames):
        _same(batch[i], gpu_ctx.render(f), f"frame {i}")


def test_batch_per_pixel_engine(gpu_ctx, flight_small):
    frames = flight_small[:3]
    batch = gpu_ctx.render_batch(frames, engine=mb.ENGINE_PER_PIXEL)
    for i, f in enumerate(frames):
        _same(batch[i], gpu_ctx.render(f, engine=mb.ENGINE_PER_PIXEL), f"frame {i}")


def test_batch_auto_precision_per_frame(gpu_ctx):
    deep = W.deep_zoom(gpu_ctx, size=64)
    plain = W.workload("mandelbulb_640x480", 64, 48)
    batch = gpu_ctx.render_batch([plain, deep], precision=mb.PREC_AUTO)
    assert gpu_ctx.stats().auto_fp64 == 1
    _same(batch[0], gpu_ctx.render(plain, precision=mb.PREC_AUTO), "plain frame")
    assert gpu_ctx.stats().auto_fp64 == 0
    _same(batch[1], gpu_ctx.render(deep, precision=mb.PREC_AUTO), "deep-zoom frame")
    assert gpu_ctx.stats().auto_fp64 == 1
    _same(batch[1], gpu_ctx.render(deep, precision=mb.PREC_FP64), "deep-zoom frame vs FP64")


def test_batch_rejects_bad_arguments(gpu_ctx, flight_small):
    with pytest.raises(mb.MbgbError):
        gpu_ctx.render_batch([])
    with pytest.raises(mb.MbgbError):
        gpu_ctx.render_batch(flight_small[:2], tile=(8, 8))
    with pytest.raises(mb.MbgbError):
        gpu_ctx.render_batch(flight_small[:2], refill_min=33)
    with pytest.raises(mb.MbgbError):
        gpu_ctx.render_batch(flight_small[:2], orbit_refill=33)
    with pytest.raises(mb.MbgbError):
        gpu_ctx.render_batch(flight_small[:2], orbit_refill=-2)
    # one AO direction table per call: frames tracing AO rays must share its quality
    q2 = W.workload("mandelbox_1080p", 64, 36)
    q3 = W.workload("mandelbox_1080p", 64, 36, ambient_occlusion_quality=3)
    with pytest.raises(mb.MbgbError):
        gpu_ctx.render_batch([q2, q3])


@pytest.mark.parametrize("frame", [0, 13, 42])
def test_flight_frames_against_oracle(gpu_ctx, oracle, frame):
    # FP32 policy against the FP64 oracle on flight frames at 1/4 resolution
    sc = W.flight(downscale=4)[frame]
    ref, _ = oracle_lib.render(oracle, sc)
    got = gpu_ctx.render_batch([sc])[0]
    m = metrics.compare(got, ref)
    assert m["hit_mismatch"] <= 0.001, m
    assert m["psnr_float"] >= 45.0, m


def test_per_frame_fractal_parameter(gpu_ctx):
    # frames that differ only in power (formula 2) or scale (formula 8) share one launch
    # sequence: the parameter travels in the frame table
    bulbs = [W.workload("mandelbulb_640x480", 64, 48, power=pw) for pw in (6.5, 7.0, 9.25)]
    batch = gpu_ctx.render_batch(bulbs)
    assert gpu_ctx.stats().launches == 5   # primary, polish, shadow set-up, secondary, compose
    for i, f in enumerate(bulbs):
        _same(batch[i], gpu_ctx.render(f), f"power frame {i}")
    boxes = [W.workload("mandelbox_1080p", 96, 54, mandelbox_scale=sc) for sc in (2.0, 2.2, -1.5)]
    batch = gpu_ctx.render_batch(boxes)
    assert gpu_ctx.stats().launches == 6   # + the overflow pass of the volumetric records
    for i, f in enumerate(boxes):
        _same(batch[i], gpu_ctx.render(f), f"scale frame {i}")
    batch = gpu_ctx.render_batch(boxes, precision=mb.PREC_FP64)
    for i, f in enumerate(boxes):
        _same(batch[i], gpu_ctx.render(f, precision=mb.PREC_FP64), f"FP64 scale frame {i}")


@pytest.mark.parametrize("size,extra", [((480, 270), {}), ((320, 180), {"ambient_occlusion_quality": 3}),
                                        ((256, 144), {"mandelbox_scale": -1.5}),
                                        ((240, 135), {"shadows_cone_angle": 2.0, "penetrating_lights": 1})])
def test_pair_rays_do_not_change_pixels(gpu_ctx, size, extra):
    """The lean Mandelbox's shadow/AO rays two per thread (packed f32x2 orbits,
    secondary_pair_kernel) give the frame of one ray per thread bit for bit, for positive
    and negative scales (|k s| from its own packed FMA) and soft / penetrating shadows."""
    sc = W.workload("mandelbox_1080p", *size, **extra)
    one = gpu_ctx.render(sc, profile_stages=True)
    st1 = gpu_ctx.stats()
    two = gpu_ctx.render(sc, pair_rays=1, profile_stages=True)
    st2 = gpu_ctx.stats()
    _same(one, two, f"pair rays {size} {extra}")
    assert st1.stage_orbit[2] == st2.stage_orbit[2] and st1.stage_de[2] == st2.stage_de[2]
    assert st2.stage_de[2] > 0


@pytest.mark.parametrize("name,size,precision", [("mandelbox_1080p", (480, 270), mb.PREC_FP32_FIX),
                                                 ("mandelbox_1080p", (320, 180), mb.PREC_FP64),
                                                 ("mandelbulb_640x480", (320, 240), mb.PREC_FP32_FIX)])
def test_hit_order_does_not_change_pixels(gpu_ctx, name, size, precision):
    """The shadow stage's jobs in the primary rays' tile order (hit_order 2, the hit list
    compacted) or in their completion order (1) give the same frame bit for bit, with the
    same shadow-stage work; a row range keeps its rows' hits only."""
    sc = W.workload(name, *size)
    frames, work = [], []
    for order in (1, 2):
        frames.append(gpu_ctx.render(sc, precision=precision, hit_order=order, profile_stages=True))
        st = gpu_ctx.stats()
        work.append((st.stage_orbit[2], st.stage_de[2]))
    _same(frames[0], frames[1], f"hit order {name} {size}")
    assert work[0] == work[1] and work[0][1] > 0
    rows = (size[1] // 3, size[1] // 2)
    part = gpu_ctx.render(sc, precision=precision, hit_order=2, rows=rows)
    full = frames[1]
    np.testing.assert_array_equal(part.hit[rows[0]:rows[1]], full.hit[rows[0]:rows[1]])
    np.testing.assert_array_equal(part.image_float[rows[0]:rows[1]], full.image_float[rows[0]:rows[1]])
