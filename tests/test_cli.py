"""mbgb_cli: the -nogui command line (ReadComandlineParams, src/interface.cpp:3334-3540, and
MainRender's still / keyframe / flight loops, src/Render3D.cpp:1940-2480).

CPU tests check the argument handling; GPU tests render stills and animations from
.fract files, decode the PNG files and hold them against the oracle's render +
CompileImage + SSAO of the same frames (-precision fp64: equal to +-1 of 65535), and the
default FP32 policy's files against the library's own device pipeline (equal)."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W
from tests import oracle_lib

CLI = os.path.join(os.path.dirname(mb.__file__), "mbgb_cli")


@pytest.fixture(scope="module")
def cli(mblib):
    assert os.path.exists(CLI), "mbgb_cli is built with the library"
    return CLI


def _fract(path, keys):
    with open(path, "w") as f:
        for k, v in keys.items():
            f.write(f"{k} {repr(float(v)) if isinstance(v, float) else v};\n")


def _png(path):
    data = open(path, "rb").read()
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBB", body[:10])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, ctype = hdr
    ch = 4 if ctype == 6 else 3
    raw = zlib.decompress(idat)
    row = w * ch * depth // 8
    buf = b"".join(raw[y * (row + 1) + 1:(y + 1) * (row + 1)] for y in range(h))
    return np.frombuffer(buf, dtype=">u2" if depth == 16 else np.uint8).reshape(h, w, ch)


def _scene_keys(w, h, **extra):
    keys = dict(W.BASE)
    keys.update(W.MANDELBULB_640x480)
    keys.update({"image_width": w, "image_height": h, "perspective": W.fov_persp(w, h),
                 "post_SSAO_enabled": 1, "post_SSAO_quality": 12, "start_frame": 0, "end_frame": 1000})
    keys.update(extra)
    return keys


def test_cli_rejects_bad_arguments(cli, tmp_path):
    assert subprocess.run([cli, "-help"], capture_output=True).returncode == 1
    assert subprocess.run([cli, "-ip", "1.2.3.4", "x.fract"], capture_output=True).returncode == 1
    assert subprocess.run([cli, "-format", "bmp", "x.fract"], capture_output=True).returncode == 1
    r = subprocess.run([cli, "-nogui", str(tmp_path / "missing.fract")], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open settings file" in (r.stdout + r.stderr)


def _expected16(oracle, scene):
    """Oracle render, CompileImage and SSAO of the frame (FP64 CPU)."""
    import ctypes
    img, _ = oracle_lib.render(oracle, scene)
    h, w = img.zbuffer.shape
    out = np.zeros((h, w, 3), np.uint16)
    p = lambda a: np.ascontiguousarray(a).ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    f = np.ascontiguousarray(img.image_float, np.float32)
    oracle.oracle_compile16.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    oracle.oracle_ssao.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    oracle.oracle_compile16(w, h, f.ctypes.data_as(ctypes.c_void_p), scene.brightness, scene.contrast,
                            scene.imageGamma, scene.hdrEnabled, out.ctypes.data_as(ctypes.c_void_p))
    if scene.SSAOEnabled:
        z, o, c = (np.ascontiguousarray(a) for a in (img.zbuffer, img.opacity, img.colour))
        oracle.oracle_ssao(w, h, z.ctypes.data_as(ctypes.c_void_p), o.ctypes.data_as(ctypes.c_void_p),
                           c.ctypes.data_as(ctypes.c_void_p), scene.persp, scene.SSAOQuality, scene.perspectiveType,
                           scene.globalIlum, out.ctypes.data_as(ctypes.c_void_p))
    return out, img


@pytest.mark.gpu
def test_cli_still_png16_fp64_matches_oracle(cli, oracle, tmp_path):
    # -precision fp64: render, CompileImage and SSAO follow the reference's double arithmetic;
    # the 16-bit file equals the oracle's to +-1 (CUDA's atan vs the host's in SSAO)
    keys = _scene_keys(160, 120, file_destination=str(tmp_path / "img"))
    _fract(tmp_path / "s.fract", keys)
    r = subprocess.run([cli, "-nogui", "-precision", "fp64", "-format", "png16", str(tmp_path / "s.fract")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = _png(tmp_path / "img00000.png").astype(np.int64)
    scene = mb.load_settings(str(tmp_path / "s.fract"))
    want, _ = _expected16(oracle, scene)
    d = np.abs(got - want.astype(np.int64))
    assert d.max() <= 1 and (d != 0).mean() <= 0.005, (int(d.max()), float((d != 0).mean()))
    # a second run skips the existing file, as MainRender does
    r = subprocess.run([cli, "-nogui", "-format", "png16", str(tmp_path / "s.fract")], capture_output=True, text=True)
    assert "exists" in r.stdout


@pytest.mark.gpu
def test_cli_still_fp32_matches_library_pipeline(cli, gpu_ctx, tmp_path):
    # default policy (FP32 with FP64 refinement): the file equals the library's own render +
    # CompileImage + SSAO of the frame (the SSAO horizon search reacts to the FP32 depths,
    # so the comparison with the FP64 oracle is the render's own PSNR bar, not this file's)
    import ctypes
    import torch
    keys = _scene_keys(160, 120, file_destination=str(tmp_path / "img"))
    _fract(tmp_path / "s.fract", keys)
    r = subprocess.run([cli, "-nogui", "-format", "png16", str(tmp_path / "s.fract")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = _png(tmp_path / "img00000.png")
    scene = mb.load_settings(str(tmp_path / "s.fract"))
    w, h = scene.image_width, scene.image_height
    L = {"image_float": torch.zeros((h, w, 3), dtype=torch.float32, device="cuda"),
         "zbuffer": torch.zeros((h, w), dtype=torch.float32, device="cuda"),
         "alpha": torch.zeros((h, w), dtype=torch.int16, device="cuda"),
         "opacity": torch.zeros((h, w), dtype=torch.int16, device="cuda"),
         "colour": torch.zeros((h, w, 3), dtype=torch.uint8, device="cuda")}
    gpu_ctx.render_batch_device([scene], [{k: v.data_ptr() for k, v in L.items()}])
    lib = mb.library()
    i16 = torch.zeros((h, w, 3), dtype=torch.int16, device="cuda")
    assert lib.mbgb_compile_image16_device(gpu_ctx._h, ctypes.byref(scene), L["image_float"].data_ptr(), w, h,
                                           i16.data_ptr()) == 0
    lay = mb.mbgb_image(w, h, None, ctypes.c_void_p(L["zbuffer"].data_ptr()), None,
                        ctypes.c_void_p(L["opacity"].data_ptr()), ctypes.c_void_p(L["colour"].data_ptr()),
                        None, None, None)
    assert lib.mbgb_ssao_device(gpu_ctx._h, ctypes.byref(scene), ctypes.byref(lay), i16.data_ptr()) == 0
    np.testing.assert_array_equal(got, i16.cpu().numpy().view(np.uint16))


@pytest.mark.gpu
def test_cli_keyframes_and_flight(cli, oracle, tmp_path):
    base = _scene_keys(96, 72, file_destination=str(tmp_path / "anim"),
                       file_keyframes=str(tmp_path / "key"), frames_per_keyframe=2)
    _fract(tmp_path / "s.fract", base)
    for k, (x, y) in enumerate([(0.0, -3.5), (0.6, -3.3), (1.2, -3.0)]):
        _fract(tmp_path / f"key{k:05d}.fract", dict(base, view_point_x=x, view_point_y=y))
    r = subprocess.run([cli, "-nogui", "-keyframe", "-precision", "fp64", "-format", "png16alpha",
                        str(tmp_path / "s.fract")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    files = sorted(f for f in os.listdir(tmp_path) if f.startswith("anim"))
    assert files == [f"anim{i:05d}.png" for i in range(6)]
    # frame 3 = keyframe 1 + half way to keyframe 2, through the reference's spline
    keys = [mb.load_settings(str(tmp_path / f"key{k:05d}.fract")) for k in range(3)]
    main = mb.load_settings(str(tmp_path / "s.fract"))
    fr = mb.interpolate(keys, 2, 3, main)
    want, img = _expected16(oracle, fr)
    got = _png(tmp_path / "anim00003.png")
    assert got.shape[2] == 4
    np.testing.assert_array_equal(got[..., 3] > 0, img.alpha > 0)
    d = np.abs(got[..., :3].astype(np.int64) - want.astype(np.int64))
    assert d.max() <= 1, int(d.max())
    # flight: x y z alpha beta gamma per line, from start frame 1
    with open(tmp_path / "path.txt", "w") as f:
        for i in range(4):
            f.write(f"{0.1 * i:.11f} {-3.5 + 0.05 * i:.11f} 0.0 0.0 0.0 0.0\n")
    _fract(tmp_path / "f.fract", dict(base, file_destination=str(tmp_path / "fly"),
                                      file_animation_path=str(tmp_path / "path.txt")))
    r = subprocess.run([cli, "-nogui", "-flight", "-start", "1", "-precision", "fp64", "-format", "png",
                        str(tmp_path / "f.fract")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert sorted(f for f in os.listdir(tmp_path) if f.startswith("fly")) == [f"fly{i:05d}.png" for i in (1, 2, 3)]
    fr = mb.load_settings(str(tmp_path / "f.fract"))
    fr.vp[0], fr.vp[1] = 0.2, -3.4
    fr = mb.finalize(fr)
    want, _ = _expected16(oracle, fr)
    got = _png(tmp_path / "fly00002.png")
    d = np.abs(got.astype(np.int64) - (want // 256).astype(np.int64))
    assert d.max() <= 1, int(d.max())
