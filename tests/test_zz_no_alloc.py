"""The allocation-free render entry point (mbgb_render_device_noalloc), through the C ABI.

Callers that cannot allocate device memory while they render (an application whose
memory manager has reserved the GPU for its own pool, a plugin inside such a host, a
frame loop that must not call cudaMalloc/cudaFree because they synchronise the
device) use this entry point; its scratch is static device memory shared by all
calls. The test renders through it three times in a row — first a scene whose long rays
go through the overflow pass, then the benchmark scene at the default launch (two CTAs
per SM) and with one CTA per SM (more step records per thread slot) — and checks each frame
against mbgb_render_device on the same scene with the FP32 parity tolerance used
by the other tests (<= 0.1 % hit mismatch, >= 45 dB PSNR of the float image).
The two entry points run the same FP32 kernel, but the allocation-free one keeps
fewer step records per thread, so more rays take the overflow pass; that pass's
inlined copy of the pixel code may contract multiply-adds differently, which moves
some float results by a few ulps — hence a tolerance, not bit equality.
This file is collected last so a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W
from tests import metrics

pytestmark = pytest.mark.gpu
LAYERS = [("image_float", 12, np.float32, (3,)), ("zbuffer", 4, np.float32, ()), ("alpha", 2, np.uint16, ()),
          ("opacity", 2, np.uint16, ()), ("colour", 3, np.uint8, (3,)), ("hit", 1, np.uint8, ()),
          ("iters", 4, np.int32, ()), ("depth", 8, np.float64, ())]


def _device_layers(w, h, fill):
    import torch
    return {name: torch.full((w * h * nbytes,), fill, dtype=torch.uint8, device="cuda")
            for name, nbytes, _, _ in LAYERS}


def _to_image(layers, w, h):
    img = mb.CImage.empty(w, h)
    for name, _, dt, extra in LAYERS:
        setattr(img, name, layers[name].cpu().numpy().view(dt).reshape((h, w) + extra))
    return img


def _c_image(layers, w, h):
    return mb.mbgb_image(w, h, *[ctypes.c_void_p(layers[name].data_ptr()) for name, _, _, _ in LAYERS])


def test_noalloc_matches_render_device_on_two_calls(mblib):
    import torch
    lib = mb.library()
    scenes = [W.workload("mandelbox_1080p", 192, 108, DE_factor=0.02),   # long rays: overflow pass
              W.workload("mandelbox_1080p", 480, 270)]
    refs = []
    with mb.Context(0) as ctx:
        for sc in scenes:
            w, h = sc.image_width, sc.image_height
            layers = _device_layers(w, h, 0)
            ctx.render_device(sc, {k: v.data_ptr() for k, v in layers.items()}, precision=mb.PREC_FP32_FIX)
            torch.cuda.synchronize()
            refs.append(_to_image(layers, w, h))
        # The first scene must send rays through the overflow pass, whose records and pixel
        # list are static arrays too. The context's per-pixel engine keeps 1024 records per
        # ray before it overflows, the allocation-free one at most 256, so a long ray there is
        # one here.
        ctx.render(scenes[0], precision=mb.PREC_FP32_FIX, engine=mb.ENGINE_PER_PIXEL)
        assert ctx.stats().long_rays > 0
    opts = [mb.make_opts(precision=mb.PREC_FP32_FIX), mb.make_opts(precision=mb.PREC_FP32_FIX),
            mb.make_opts(precision=mb.PREC_FP32_FIX, ctas_per_sm=1)]
    scenes.append(scenes[1])   # a third call: one CTA per SM, more records per thread slot
    refs.append(refs[1])
    for call, (sc, ref) in enumerate(zip(scenes, refs)):   # calls in a row share the static scratch
        w, h = sc.image_width, sc.image_height
        layers = _device_layers(w, h, 0xA5)  # garbage: every pixel must be written
        img_c = _c_image(layers, w, h)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = lib.mbgb_render_device_noalloc(ctypes.byref(sc), ctypes.byref(img_c), ctypes.byref(opts[call]))
        assert rc == 0, lib.mbgb_last_error()
        torch.cuda.synchronize()
        if call > 0:
            # after the first call (which may load the module that holds the static arrays)
            # the entry point takes no device memory at all
            assert torch.cuda.mem_get_info()[0] == free_before
        got = _to_image(layers, w, h)
        m = metrics.compare(got, ref)
        assert m["hit_mismatch"] <= 0.001 and m["psnr_float"] >= 45.0, m
        # every pixel was written (the output started as 0xA5 garbage)
        assert np.isfinite(got.image_float).all()
        assert np.all((got.hit == 0) | (got.hit == 1))


def test_noalloc_rejects_what_its_scratch_cannot_hold(mblib):
    lib = mb.library()
    big = W.workload("mandelbox_1080p", 4096, 2160)
    img = mb.mbgb_image(4096, 2160, *([None] * 8))
    assert lib.mbgb_render_device_noalloc(ctypes.byref(big), ctypes.byref(img), None) == 1
    assert b"4194304 pixels" in lib.mbgb_last_error()
    small = W.workload("mandelbox_1080p", 64, 36)
    img = mb.mbgb_image(64, 36, *([None] * 8))
    for prec in (mb.PREC_FP64, mb.PREC_AUTO):   # AUTO may pick FP64, which this entry point does not carry
        opts = mb.make_opts(precision=prec)
        assert lib.mbgb_render_device_noalloc(ctypes.byref(small), ctypes.byref(img), ctypes.byref(opts)) == 1
        assert b"FP32_FIX" in lib.mbgb_last_error()
