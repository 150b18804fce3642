"""Re-entrancy of the C ABI across host threads.

The reference calls Render() from its main thread only (src/Render3D.cpp:709) and
spreads the pixel rows over worker threads it joins before returning
(src/Render3D.cpp:815-849). Here every mbgb_context owns its stream, scratch and
counters, so two contexts may render at the same time from two host threads; one
context shared by two threads serialises their calls. In both cases every frame
must equal the same frame rendered alone (jitter off: the render is deterministic,
so the comparison is bit for bit on every layer). ctypes releases the GIL around
each foreign call, so the two threads' renders do overlap on the GPU.
"""
import threading

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W

pytestmark = pytest.mark.gpu
LAYERS = ("image_float", "zbuffer", "alpha", "opacity", "colour", "hit", "iters", "depth")
FRAMES = 4


def _scenes():
    return [W.workload("mandelbox_1080p", 480, 270), W.workload("mandelbulb_640x480", 320, 240)]


def _assert_same(a, b):
    for name in LAYERS:
        assert np.array_equal(getattr(a, name), getattr(b, name)), name


def _run_threads(ctxs, scenes, precision):
    out = [[None] * FRAMES for _ in scenes]
    errors = []
    start = threading.Barrier(len(scenes))

    def work(i):
        try:
            start.wait(timeout=60)
            for k in range(FRAMES):
                out[i][k] = ctxs[i].render(scenes[i], precision=precision)
        except Exception as e:  # noqa: BLE001 - reported by the main thread
            errors.append(e)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(scenes))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in threads), "a render thread did not finish"
    assert not errors, errors
    return out


@pytest.mark.parametrize("precision", [mb.PREC_FP32_FIX, mb.PREC_FP64])
def test_two_contexts_render_at_once_from_two_threads(mblib, precision):
    scenes = _scenes()
    if precision == mb.PREC_FP64:   # keep the FP64 frames small
        scenes = [W.workload("mandelbox_1080p", 160, 90), W.workload("mandelbulb_640x480", 96, 72)]
    with mb.Context(0) as a, mb.Context(0) as b:
        serial = [a.render(scenes[0], precision=precision), b.render(scenes[1], precision=precision)]
        out = _run_threads([a, b], scenes, precision)
    for i in range(len(scenes)):
        for k in range(FRAMES):
            _assert_same(out[i][k], serial[i])


def test_one_context_shared_by_two_threads(mblib):
    scenes = _scenes()
    with mb.Context(0) as ctx:
        serial = [ctx.render(sc, precision=mb.PREC_FP32_FIX) for sc in scenes]
        out = _run_threads([ctx, ctx], scenes, mb.PREC_FP32_FIX)
    for i in range(len(scenes)):
        for k in range(FRAMES):
            _assert_same(out[i][k], serial[i])
