"""GB300-native drop-in for Mandelbulber 1.21's per-pixel DE ray-march render.

Python mirror of the C ABI in include/mbgb.h (libmbgb.so, built in-tree by
mandelbulber_gb300._build). It follows the reference's own interface for this
path:

* ``load_settings(path, defaults=..., overrides=...)`` is LoadSettings
  (src/settings.cpp:611-698) plus the -nogui fix-ups: it returns an
  ``mbgb_scene`` (the sParamRender fields, src/fractparams.h).
* ``Context.render(scene)`` is Render(sParamRender, cImage*) (src/Render3D.cpp:709)
  and returns a ``CImage`` holding the layers MainThread writes
  (src/Render3D.cpp:569-589): image_float, zbuffer, alpha, opacity, colour.
* ``Context.render_batch(scenes)`` renders the frames of MainRender's keyframe /
  flight loops (src/Render3D.cpp:2144-2350) in one launch sequence.

There is no CPU fallback: every render call runs the CUDA kernels and raises
``MbgbError`` when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import (PREC_AUTO, PREC_FP32_FIX, PREC_FP64, mbgb_image, mbgb_opts, mbgb_rgb, mbgb_scene, mbgb_stats,
                   mbgb_tuning)

__all__ = [
    "MbgbError", "load_settings", "scene_set", "finalize", "supported", "palette_from_seed", "Context", "CImage",
    "compile_image16", "library", "PREC_FP64", "PREC_FP32_FIX", "PREC_AUTO", "mbgb_scene",
]

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libmbgb.so")

_lib = None


class MbgbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_abi.MBGB_STATUS.get(status, status)}: {message}")
        self.status = status


def library(build_if_missing: bool = False) -> ctypes.CDLL:
    """Loads libmbgb.so (building it first when asked); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise MbgbError(3, f"{LIB_PATH} is missing: run mandelbulber_gb300._build.build()")
        from ._build import build
        build()
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _abi.FUNCTIONS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status: int):
    if status != 0:
        msg = library().mbgb_last_error()
        raise MbgbError(status, msg.decode() if msg else "")


def load_settings(path: str, defaults: str | None = None, overrides=()) -> mbgb_scene:
    """Reads a .fract file (after an optional defaults file) into a scene."""
    lib = library()
    scene = mbgb_scene()
    ov = [o.encode() if isinstance(o, str) else o for o in overrides]
    arr = (ctypes.c_char_p * max(1, len(ov)))(*ov)
    _check(lib.mbgb_scene_from_settings(defaults.encode() if defaults else None, path.encode(), arr, len(ov),
                                        ctypes.byref(scene)))
    return scene


def scene_set(scene: mbgb_scene, key: str, value) -> None:
    """Sets one settings key (LoadOneSetting semantics); call finalize() afterwards."""
    _check(library().mbgb_scene_set(ctypes.byref(scene), key.encode(), str(value).encode()))


def finalize(scene: mbgb_scene) -> mbgb_scene:
    _check(library().mbgb_scene_finalize(ctypes.byref(scene)))
    return scene


def supported(scene: mbgb_scene) -> tuple[bool, str]:
    lib = library()
    st = lib.mbgb_scene_supported(ctypes.byref(scene))
    return st == 0, (lib.mbgb_last_error() or b"").decode() if st else ""


def palette_from_seed(seed: int, saturation: float) -> np.ndarray:
    pal = (mbgb_rgb * 256)()
    library().mbgb_palette_from_seed(seed, saturation, pal)
    return np.array([[c.R, c.G, c.B] for c in pal], dtype=np.int32)


def interpolate(keys, frames_per_key: int, frame: int, base: mbgb_scene | None = None) -> mbgb_scene:
    """Scene of animation frame ``frame`` from keyframes (CMorph::CatmullRom over every
    interpolated double, src/morph.cpp:49-109, as MainRender applies it)."""
    n = len(keys)
    arr = (mbgb_scene * n)(*keys)
    out = mbgb_scene()
    _check(library().mbgb_scene_interpolate(arr, n, frames_per_key, frame,
                                            ctypes.byref(base) if base is not None else None, ctypes.byref(out)))
    return out


def scene_bytes(scene: mbgb_scene) -> bytes:
    return ctypes.string_at(ctypes.addressof(scene), ctypes.sizeof(scene))


def scene_from_bytes(raw: bytes) -> mbgb_scene:
    if len(raw) != ctypes.sizeof(mbgb_scene):
        raise ValueError(f"scene blob has {len(raw)} bytes, expected {ctypes.sizeof(mbgb_scene)}")
    s = mbgb_scene()
    ctypes.memmove(ctypes.addressof(s), raw, len(raw))
    return s


@dataclass
class CImage:
    """The cImage layers the render writes (src/cimage.hpp:155-162), row-major."""

    width: int
    height: int
    image_float: np.ndarray   # (H, W, 3) float32
    zbuffer: np.ndarray       # (H, W) float32, 1e20 for background
    alpha: np.ndarray         # (H, W) uint16
    opacity: np.ndarray       # (H, W) uint16
    colour: np.ndarray        # (H, W, 3) uint8
    hit: np.ndarray           # (H, W) uint8 (parity layer)
    iters: np.ndarray         # (H, W) int32 (parity layer)
    depth: np.ndarray         # (H, W) float64 (parity layer)

    @classmethod
    def empty(cls, width: int, height: int) -> "CImage":
        return cls(width, height,
                   np.zeros((height, width, 3), np.float32), np.full((height, width), 1e20, np.float32),
                   np.zeros((height, width), np.uint16), np.zeros((height, width), np.uint16),
                   np.zeros((height, width, 3), np.uint8), np.zeros((height, width), np.uint8),
                   np.zeros((height, width), np.int32), np.full((height, width), 1e20, np.float64))

    def as_c(self) -> mbgb_image:
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        return mbgb_image(self.width, self.height, p(self.image_float), p(self.zbuffer), p(self.alpha),
                          p(self.opacity), p(self.colour), p(self.hit), p(self.iters), p(self.depth))


ENGINE_WAVEFRONT, ENGINE_PER_PIXEL = 0, 1


def make_opts(precision: int = PREC_FP32_FIX, jitter: bool = False, jitter_seed: int = 0, rows=None,
              ctas_per_sm: int = 0, threads_per_cta: int = 0, deadline_ms: int = 0, stream: int = 0,
              engine: int = ENGINE_WAVEFRONT, profile_stages: bool = False, polish_all: bool = False,
              tile=None, refill_min: int = 0, autotune: bool = False, use_graph: bool = False,
              exact_hit: bool = False, orbit_refill: int = 0, pair_rays: int = 0, hit_order: int = 0) -> mbgb_opts:
    r0, r1 = rows if rows else (0, 0)
    tw, th = tile if tile else (0, 0)
    return mbgb_opts(precision=precision, jitter=int(jitter), jitter_seed=jitter_seed, row_begin=r0, row_end=r1,
                     ctas_per_sm=ctas_per_sm, threads_per_cta=threads_per_cta, deadline_ms=deadline_ms,
                     stream=stream if stream else None, engine=engine, profile_stages=int(profile_stages),
                     polish_all=int(polish_all), tile_w=tw, tile_h=th, refill_min=refill_min,
                     autotune=int(autotune), use_graph=int(use_graph), exact_hit=int(exact_hit),
                     orbit_refill=orbit_refill, pair_rays=pair_rays, hit_order=hit_order)


_LAYERS = ["image_float", "zbuffer", "alpha", "opacity", "colour", "hit", "iters", "depth"]


def _device_image(scene: mbgb_scene, layers: dict) -> mbgb_image:
    return mbgb_image(scene.image_width, scene.image_height,
                      *[ctypes.c_void_p(layers.get(n) or 0) if layers.get(n) else None for n in _LAYERS])


class Context:
    """One CUDA device and stream (mbgb_context)."""

    def __init__(self, device: int = 0):
        self._lib = library()
        h = ctypes.c_void_p()
        _check(self._lib.mbgb_context_create(device, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mbgb_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def render(self, scene: mbgb_scene, image: CImage | None = None, **opts) -> CImage:
        """Renders the frame into host layers; copies are part of the call."""
        if image is None:
            image = CImage.empty(scene.image_width, scene.image_height)
        img = image.as_c()
        o = make_opts(**opts)
        _check(self._lib.mbgb_render_host(self._h, ctypes.byref(scene), ctypes.byref(img), ctypes.byref(o)))
        return image

    def render_device(self, scene: mbgb_scene, layers: dict, **opts) -> None:
        """Renders into device buffers; ``layers`` maps layer names to device pointers (ints)."""
        img = _device_image(scene, layers)
        o = make_opts(**opts)
        _check(self._lib.mbgb_render_device(self._h, ctypes.byref(scene), ctypes.byref(img), ctypes.byref(o)))

    def render_batch(self, scenes, images=None, **opts) -> list:
        """Renders the frames of an animation in one launch sequence into host layers
        (mbgb_render_batch_host); returns the CImages."""
        n = len(scenes)
        if images is None:
            images = [CImage.empty(sc.image_width, sc.image_height) for sc in scenes]
        arr = (mbgb_scene * n)(*scenes)
        imgs = (mbgb_image * n)(*[im.as_c() for im in images])
        o = make_opts(**opts)
        _check(self._lib.mbgb_render_batch_host(self._h, arr, n, imgs, ctypes.byref(o)))
        return images

    def render_batch_device(self, scenes, layers: list, **opts) -> None:
        """mbgb_render_batch: frame i renders into the device pointers of ``layers[i]``."""
        n = len(scenes)
        arr = (mbgb_scene * n)(*scenes)
        imgs = (mbgb_image * n)(*[_device_image(sc, ly) for sc, ly in zip(scenes, layers)])
        o = make_opts(**opts)
        _check(self._lib.mbgb_render_batch(self._h, arr, n, imgs, ctypes.byref(o)))

    def render_grad(self, scenes, layers: list, dL_dimage=None, jacobian=None, **opts) -> np.ndarray:
        """mbgb_render_grad: renders the frames into the device layers (hits on the level set)
        and returns dL/dtheta [n, GRAD_PARAMS] for the device loss gradients ``dL_dimage``
        (list of pointers to [h, w, 3] float32, or None); ``jacobian`` optionally receives
        dI/dtheta per pixel (list of pointers to [h, w, 3, GRAD_PARAMS] float32)."""
        n = len(scenes)
        arr = (mbgb_scene * n)(*scenes)
        imgs = (mbgb_image * n)(*[_device_image(sc, ly) for sc, ly in zip(scenes, layers)])
        gin = (ctypes.c_void_p * n)(*dL_dimage) if dL_dimage is not None else None
        jac = (ctypes.c_void_p * n)(*jacobian) if jacobian is not None else None
        out = np.zeros((n, _abi.GRAD_PARAMS), np.float64)
        o = make_opts(**opts)
        _check(self._lib.mbgb_render_grad(self._h, arr, n, imgs, gin, jac,
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(o)))
        return out

    def autotune(self, scene: mbgb_scene, **opts) -> mbgb_tuning:
        """mbgb_autotune: times the launch configurations on this frame and caches the best."""
        t = mbgb_tuning()
        o = make_opts(**opts)
        _check(self._lib.mbgb_autotune(self._h, ctypes.byref(scene), ctypes.byref(o), ctypes.byref(t)))
        return t

    def distance(self, scene: mbgb_scene, points_dev: int, detail_dev: int, n: int, dist_dev: int, iters_dev: int,
                 maxiter_dev: int, precision: int = PREC_FP64) -> None:
        """CalculateDistance at n device-resident points (device pointers)."""
        _check(self._lib.mbgb_distance_device(self._h, ctypes.byref(scene), precision, points_dev, detail_dev, n,
                                              dist_dev, iters_dev, maxiter_dev))

    def stats(self) -> mbgb_stats:
        s = mbgb_stats()
        _check(self._lib.mbgb_get_stats(self._h, ctypes.byref(s)))
        return s


def compile_image16(scene: mbgb_scene, image_float: np.ndarray) -> np.ndarray:
    """CompileImage (src/cimage.cpp:183-214): float RGB -> gamma-corrected RGB16."""
    h, w = image_float.shape[:2]
    src = np.ascontiguousarray(image_float, dtype=np.float32)
    out = np.zeros((h, w, 3), np.uint16)
    _check(library().mbgb_compile_image16(ctypes.byref(scene), src.ctypes.data_as(ctypes.c_void_p), w, h,
                                          out.ctypes.data_as(ctypes.c_void_p)))
    return out
