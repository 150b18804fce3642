"""mbgb_cli: the -nogui command line (ReadComandlineParams, src/interface.cpp:3334-3540, and
MainRender's still / keyframe / flight loops, src/Render3D.cpp:1940-2480).

CPU tests check the argument handling; GPU tests render stills and animations from
.fract files, decode the PNG files and hold them against the oracle's render +
CompileImage + SSAO of the same frames (FP32 policy bar: PSNR >= 45 dB on the 16-bit image)."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W
from tests import metrics, oracle_lib

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
                 "post_SSAO_enabled": 1, "post_SSAO_quality": 12})
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
def test_cli_still_png16_against_oracle(cli, oracle, tmp_path):
    keys = _scene_keys(160, 120, file_destination=str(tmp_path / "img"))
    _fract(tmp_path / "s.fract", keys)
    r = subprocess.run([cli, "-nogui", "-format", "png16", str(tmp_path / "s.fract")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = _png(tmp_path / "img00000.png")
    scene = mb.load_settings(str(tmp_path / "s.fract"))
    want, _ = _expected16(oracle, scene)
    assert got.shape == want.shape
    assert metrics.psnr(got.astype(np.float64), want.astype(np.float64), peak=65535.0) >= 45.0
    # a second run skips the existing file, as MainRender does
    r = subprocess.run([cli, "-nogui", "-format", "png16", str(tmp_path / "s.fract")], capture_output=True, text=True)
    assert "exists" in r.stdout


@pytest.mark.gpu
def test_cli_keyframes_and_flight(cli, oracle, tmp_path):
    base = _scene_keys(96, 72, file_destination=str(tmp_path / "anim"),
                       file_keyframes=str(tmp_path / "key"), frames_per_keyframe=2)
    _fract(tmp_path / "s.fract", base)
    for k, (x, y) in enumerate([(0.0, -3.5), (0.6, -3.3), (1.2, -3.0)]):
        _fract(tmp_path / f"key{k:05d}.fract", dict(base, view_point_x=x, view_point_y=y))
    r = subprocess.run([cli, "-nogui", "-keyframe", "-format", "png16alpha", str(tmp_path / "s.fract")],
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
    assert metrics.psnr(got[..., :3].astype(np.float64), want.astype(np.float64), peak=65535.0) >= 45.0
    # flight: x y z alpha beta gamma per line, from start frame 1
    with open(tmp_path / "path.txt", "w") as f:
        for i in range(4):
            f.write(f"{0.1 * i:.11f} {-3.5 + 0.05 * i:.11f} 0.0 0.0 0.0 0.0\n")
    _fract(tmp_path / "f.fract", dict(base, file_destination=str(tmp_path / "fly"),
                                      file_animation_path=str(tmp_path / "path.txt")))
    r = subprocess.run([cli, "-nogui", "-flight", "-start", "1", "-format", "png", str(tmp_path / "f.fract")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert sorted(f for f in os.listdir(tmp_path) if f.startswith("fly")) == [f"fly{i:05d}.png" for i in (1, 2, 3)]
    fr = mb.load_settings(str(tmp_path / "f.fract"))
    fr.vp[0], fr.vp[1] = 0.2, -3.4
    fr = mb.finalize(fr)
    want, _ = _expected16(oracle, fr)
    got = _png(tmp_path / "fly00002.png")
    assert metrics.psnr(got.astype(np.float64), (want // 256).astype(np.float64), peak=255.0) >= 40.0
