"""The C-ABI library loads without a GPU and exports every symbol include/mbgb.h declares."""
import ctypes

import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import _abi


def test_every_declared_symbol_is_exported(mblib):
    declared = _abi.declared_functions()
    assert len(declared) >= 14
    for name in declared:
        assert hasattr(mblib, name), f"{name} is declared in include/mbgb.h but not exported"
    assert set(declared) == set(_abi.FUNCTIONS), "Python binding table differs from the header"


def test_version_and_error_text(mblib):
    assert mblib.mbgb_version().startswith(b"mbgb ")
    s = mb.mbgb_scene()
    assert mblib.mbgb_scene_set(ctypes.byref(s), b"no_such_key", b"1") == 1
    assert b"no_such_key" in mblib.mbgb_last_error()


def test_null_arguments_are_rejected(mblib):
    assert mblib.mbgb_scene_finalize(None) == 1
    assert mblib.mbgb_scene_supported(None) == 1
    assert mblib.mbgb_render_host(None, None, None, None) == 1
    assert mblib.mbgb_context_create(0, None) == 1


def test_unsupported_features_are_reported(mblib):
    from mandelbulber_gb300 import workloads as W
    for key, value, text in [("formula", 38, "formula"),
                             ("textured_background", 1, "textured background"),
                             ("reflections_max", 11, "reflections")]:
        sc = W.workload("mandelbulb_640x480", raytraced_reflections=1, **{key: value})
        ok, why = mb.supported(sc)
        assert not ok and text in why, (key, why)
    ok, why = mb.supported(W.workload("mandelbox_1080p"))
    assert ok, why


def test_context_without_gpu_fails_loudly(mblib):
    """No CPU fallback: without a visible device the context cannot be created."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(mb.MbgbError) as e:
        mb.Context(0)
    assert e.value.status == 7


def test_option_structs_follow_the_header():
    """The Python mirrors of mbgb_opts / mbgb_tuning are read from include/mbgb.h: the launch
    options land in their fields, and the defaults (0) select the library's own choices."""
    o = mb.make_opts(refill_min=4, orbit_refill=-1, tile=(16, 2), threads_per_cta=64)
    assert (o.refill_min, o.orbit_refill, o.tile_w, o.tile_h, o.threads_per_cta) == (4, -1, 16, 2, 64)
    d = mb.make_opts()
    assert d.refill_min == 0 and d.orbit_refill == 0 and d.autotune == 0
    names = [f[0] for f in mb.mbgb_tuning._fields_]
    assert {"tile_w", "tile_h", "threads_per_cta", "ctas_per_sm", "refill_min", "orbit_refill", "ms"} <= set(names)
    assert ctypes.sizeof(mb.mbgb_opts) % 8 == 0
