"""Post-processing: CompileImage and SSAO against the reference's own code.

tests/golden/post_*.npz hold CompileImage (src/cimage.cpp:132-214) and PostRendering_SSAO
(src/image.cpp:249-478) outputs of the reference's compiled sources, applied to the
render fixtures with several brightness / contrast / gamma / HDR / SSAO-quality settings,
for the three perspective types. The oracle's restatement and the library's host
CompileImage must reproduce them exactly; the device kernels (GPU tests) exactly for the
compile step without HDR and to +-1 of 65535 where CUDA's tanh or atan round differently
from the host's libm (counted, at most 0.5 % of the values).
"""
import ctypes
import glob
import os

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from tests import oracle_lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
POSTS = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, "post_*.npz")))


def _case(name):
    z = np.load(os.path.join(GOLDEN, f"post_{name}.npz"))
    r = np.load(os.path.join(GOLDEN, f"render_{str(z['render'])}.npz"))
    sc = mb.scene_from_bytes(r["scene"].tobytes())
    sc.brightness, sc.contrast, sc.imageGamma = float(z["brightness"]), float(z["contrast"]), float(z["gamma"])
    sc.hdrEnabled = int(z["hdr"])
    sc.SSAOQuality = int(z["quality"])
    sc.globalIlum = float(z["global_ilum"])
    return z, r, sc


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_post_fixtures_present():
    assert len(POSTS) >= 4


@pytest.mark.parametrize("name", POSTS)
def test_oracle_compile_and_ssao_match_reference(name):
    z, r, sc = _case(name)
    lib = oracle_lib.load()
    h, w = r["zbuffer"].shape
    lib.oracle_compile16.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    lib.oracle_ssao.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    imf = np.ascontiguousarray(r["image_float"], np.float32)
    img16 = np.zeros((h, w, 3), np.uint16)
    lib.oracle_compile16(w, h, _p(imf), sc.brightness, sc.contrast, sc.imageGamma, sc.hdrEnabled, _p(img16))
    np.testing.assert_array_equal(img16, z["image16_compiled"])
    lib.oracle_ssao(w, h, _p(np.ascontiguousarray(r["zbuffer"])), _p(np.ascontiguousarray(r["opacity"])),
                    _p(np.ascontiguousarray(r["colour"])), sc.persp, sc.SSAOQuality, sc.perspectiveType,
                    sc.globalIlum, _p(img16))
    np.testing.assert_array_equal(img16, z["image16_ssao"])


@pytest.mark.parametrize("name", POSTS)
def test_library_host_compile_matches_reference(name):
    z, r, sc = _case(name)
    out = mb.compile_image16(sc, r["image_float"])
    np.testing.assert_array_equal(out, z["image16_compiled"])


def _within_one(got, want, what):
    d = np.abs(got.astype(np.int64) - want.astype(np.int64))
    assert d.max() <= 1, (what, int(d.max()))
    assert (d != 0).mean() <= 0.005, (what, float((d != 0).mean()))


@pytest.mark.gpu
@pytest.mark.parametrize("name", POSTS)
def test_device_compile_and_ssao_match_reference(gpu_ctx, name):
    import torch
    z, r, sc = _case(name)
    h, w = r["zbuffer"].shape
    lib = mb.library()
    imf = torch.tensor(np.ascontiguousarray(r["image_float"], np.float32), device="cuda")
    img16 = torch.zeros((h, w, 3), dtype=torch.int16, device="cuda")
    assert lib.mbgb_compile_image16_device(gpu_ctx._h, ctypes.byref(sc), imf.data_ptr(), w, h,
                                           img16.data_ptr()) == 0, lib.mbgb_last_error()
    got = img16.cpu().numpy().view(np.uint16)
    if sc.hdrEnabled:
        _within_one(got, z["image16_compiled"], "compile (tanh)")
    else:
        np.testing.assert_array_equal(got, z["image16_compiled"])
    # SSAO from the reference's compiled image (the library runs on its own stream: wait
    # for torch's copy first)
    img16.copy_(torch.tensor(z["image16_compiled"].view(np.int16), device="cuda"))
    torch.cuda.synchronize()
    zb = torch.tensor(np.ascontiguousarray(r["zbuffer"]), device="cuda")
    op = torch.tensor(np.ascontiguousarray(r["opacity"]).view(np.int16), device="cuda")
    col = torch.tensor(np.ascontiguousarray(r["colour"]), device="cuda")
    layers = mb.mbgb_image(w, h, None, ctypes.c_void_p(zb.data_ptr()), None, ctypes.c_void_p(op.data_ptr()),
                           ctypes.c_void_p(col.data_ptr()), None, None, None)
    assert lib.mbgb_ssao_device(gpu_ctx._h, ctypes.byref(sc), ctypes.byref(layers), img16.data_ptr()) == 0, \
        lib.mbgb_last_error()
    torch.cuda.synchronize()
    _within_one(img16.cpu().numpy().view(np.uint16), z["image16_ssao"], "ssao (atan)")


DOFS = sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "dof_*.npz")))


def _dof_case(name):
    z = np.load(os.path.join(GOLDEN, f"dof_{name}.npz"))
    r = np.load(os.path.join(GOLDEN, f"render_{str(z['render'])}.npz"))
    sc = mb.scene_from_bytes(r["scene"].tobytes())
    sc.DOFRadius, sc.DOFFocus = float(z["radius"]), float(z["focus"])
    return z, r, sc


@pytest.mark.parametrize("name", DOFS)
def test_oracle_dof_matches_reference(name):
    """PostRendering_DOF (src/image.cpp:57-206): the oracle's restatement of the z-buffer
    quicksort, the Random() shuffle and the in-place splats equals the reference bit for bit."""
    z, r, sc = _dof_case(name)
    lib = oracle_lib.load()
    h, w = r["zbuffer"].shape
    lib.oracle_dof.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_double, ctypes.c_double, ctypes.c_uint]
    img16 = z["image16_in"].copy()
    alpha = z["alpha_in"].copy()
    lib.oracle_dof(w, h, _p(np.ascontiguousarray(r["zbuffer"])), _p(alpha), _p(img16), sc.DOFRadius * w / 1000.0,
                   10.0 ** (sc.DOFFocus / 10.0 - 16.0), int(z["seed"]))
    np.testing.assert_array_equal(img16, z["image16_dof"])
    np.testing.assert_array_equal(alpha, z["alpha_dof"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", DOFS)
def test_device_dof_matches_reference(gpu_ctx, name):
    """mbgb_dof_device: the splat order from the host, the splats per 16 x 16 tile on the
    device, each pixel folding its splats in order: equal to the reference bit for bit."""
    import torch
    z, r, sc = _dof_case(name)
    lib = mb.library()
    h, w = r["zbuffer"].shape
    img16 = torch.tensor(z["image16_in"].view(np.int16), device="cuda")
    alpha = torch.tensor(z["alpha_in"].view(np.int16), device="cuda")
    zb = torch.tensor(np.ascontiguousarray(r["zbuffer"]), device="cuda")
    torch.cuda.synchronize()
    layers = mb.mbgb_image(w, h, None, ctypes.c_void_p(zb.data_ptr()), ctypes.c_void_p(alpha.data_ptr()), None,
                           None, None, None, None)
    assert lib.mbgb_dof_device(gpu_ctx._h, ctypes.byref(sc), ctypes.byref(layers), img16.data_ptr(),
                               int(z["seed"])) == 0, lib.mbgb_last_error()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(img16.cpu().numpy().view(np.uint16), z["image16_dof"])
    np.testing.assert_array_equal(alpha.cpu().numpy().view(np.uint16), z["alpha_dof"])
