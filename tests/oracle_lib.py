"""Loads the CPU oracle (oracle/mb_oracle.cpp) for the tests — test infrastructure only."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_cache = {}


def load(fast: bool = False) -> ctypes.CDLL:
    key = "fast" if fast else "strict"
    if key in _cache:
        return _cache[key]
    name = "libmboracle_fast.so" if fast else "libmboracle.so"
    path = os.path.join(ORACLE_DIR, "_build", name)
    subprocess.check_call(["make", "-s", "-C", ORACLE_DIR, "all"])
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    lib.oracle_distance.argtypes = [vp, vp, vp, ctypes.c_long, vp, vp, vp]
    lib.oracle_distance.restype = None
    lib.oracle_colour_value.argtypes = [vp, vp, ctypes.c_long, vp]
    lib.oracle_colour_value.restype = None
    lib.oracle_render.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp]
    lib.oracle_render.restype = ctypes.c_int
    lib.oracle_render_exact.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
    lib.oracle_compile16.restype = None
    lib.oracle_ssao.restype = None
    lib.oracle_render_exact.restype = ctypes.c_int
    lib.oracle_render_pixel_work.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp]
    lib.oracle_render_pixel_work.restype = ctypes.c_int
    _cache[key] = lib
    return lib


def ref_tree() -> str:
    """Where the reference tree lies (MBGB_REF_TREE, else oracle/Makefile's default)."""
    env = os.environ.get("MBGB_REF_TREE")
    if env:
        return env
    return subprocess.check_output(["make", "-s", "-C", ORACLE_DIR, "print-ref-tree"], text=True).strip()


def load_ref_settings():
    """The reference's own settings reader (oracle/_ref/libmbref_settings.so, built from the
    reference tree in place), or None where the tree is absent."""
    if "settings" in _cache:
        return _cache["settings"]
    lib = None
    if os.path.isfile(os.path.join(ref_tree(), "src", "settings.cpp")):
        subprocess.check_call(["make", "-s", "-C", ORACLE_DIR, "ref"])
        lib = ctypes.CDLL(os.path.join(ORACLE_DIR, "_ref", "libmbref_settings.so"))
        vp = ctypes.c_void_p
        lib.ref_scene_from_settings.argtypes = [ctypes.c_char_p, ctypes.c_char_p, vp, ctypes.c_int, vp]
        lib.ref_scene_from_settings.restype = ctypes.c_int
        lib.ref_scene_from_keys.argtypes = [vp, vp, ctypes.c_int, vp]
        lib.ref_scene_from_keys.restype = ctypes.c_int
    _cache["settings"] = lib
    return lib


def settings_value(v) -> str:
    """A settings value as the workload builder writes it (floats by repr)."""
    return repr(float(v)) if isinstance(v, float) else str(v)


def ref_scene_from_settings(lib, scene, defaults, path, overrides=()):
    """Fills the ctypes mbgb_scene `scene` through the reference's LoadSettings2 of the
    defaults file and `path` (each followed by the overrides) + the -nogui derivations."""
    ov = [o.encode() for o in overrides]
    arr = (ctypes.c_char_p * max(1, len(ov)))(*ov)
    rc = lib.ref_scene_from_settings(defaults.encode() if defaults else None, path.encode(), arr, len(ov),
                                     ctypes.addressof(scene))
    if rc != 0:
        raise RuntimeError(f"the reference's LoadSettings2 could not read {path}")
    return scene


def ref_scene_from_keys(lib, scene, keys: dict):
    """Fills `scene` through the reference's LoadOneSetting of each key (in order) on a
    zeroed sParamRender, LoadSettingsPost and the -nogui derivations."""
    ks = [k.encode() for k in keys]
    vs = [settings_value(v).encode() for v in keys.values()]
    lib.ref_scene_from_keys((ctypes.c_char_p * len(ks))(*ks), (ctypes.c_char_p * len(vs))(*vs), len(ks),
                            ctypes.addressof(scene))
    return scene


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def distance(lib, scene, points: np.ndarray, detail: np.ndarray):
    pts = np.ascontiguousarray(points, np.float64)
    det = np.ascontiguousarray(detail, np.float64)
    n = len(pts)
    d = np.zeros(n)
    it = np.zeros(n, np.int32)
    mi = np.zeros(n, np.uint8)
    lib.oracle_distance(ctypes.addressof(scene), _p(pts), _p(det), n, _p(d), _p(it), _p(mi))
    return d, it, mi


def colour_value(lib, scene, points: np.ndarray):
    pts = np.ascontiguousarray(points, np.float64)
    out = np.zeros(len(pts))
    lib.oracle_colour_value(ctypes.addressof(scene), _p(pts), len(pts), _p(out))
    return out


LAYERS = (("image_float", np.float32, 3), ("zbuffer", np.float32, 1), ("alpha", np.uint16, 1),
          ("opacity", np.uint16, 1), ("colour", np.uint8, 3), ("hit", np.uint8, 1), ("iters", np.int32, 1),
          ("depth", np.float64, 1))


class RawImage(ctypes.Structure):
    """mbgb_image (include/mbgb.h) for callers that do not load the product package."""
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32)] + [(n, ctypes.c_void_p) for n, _, _ in LAYERS]


def sample_rows(height: int, n: int) -> list:
    """`n` rows spread evenly over a frame of `height` rows (the CPU baseline's sample)."""
    n = max(1, min(n, height))
    return sorted({int((i + 0.5) * height / n) for i in range(n)})


def alloc_layers(width: int, height: int) -> dict:
    return {n: np.zeros(width * height * c, dt) for n, dt, c in LAYERS}


def render_row_list(lib, scene_ptr: int, width: int, height: int, rows, jitter=False, threads=None, layers=None):
    """Renders the listed rows of a frame on the CPU into numpy layers (`layers` from
    alloc_layers, or new ones); `scene_ptr` is the address of an mbgb_scene (a ctypes struct
    or a buffer holding its bytes). Returns (layers dict, counters). Loads nothing but the
    oracle library."""
    if layers is None:
        layers = alloc_layers(width, height)
    img = RawImage(width, height, *[layers[n].ctypes.data_as(ctypes.c_void_p) for n, _, _ in LAYERS])
    rl = np.ascontiguousarray(rows, np.int32)
    cnt = np.zeros(3, np.uint64)
    lib.oracle_render_row_list.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.oracle_render_row_list.restype = ctypes.c_int
    rc = lib.oracle_render_row_list(scene_ptr, _p(rl), len(rl), int(jitter), threads or os.cpu_count() or 1,
                                    ctypes.addressof(img), _p(cnt))
    if rc != 0:
        raise RuntimeError("oracle_render_row_list rejected its arguments")
    return layers, cnt


def render(lib, scene, rows=None, jitter=False, threads=None):
    """Renders the scene on the CPU; returns (CImage, counters)."""
    import mandelbulber_gb300 as mb
    w, h = scene.image_width, scene.image_height
    img = mb.CImage.empty(w, h)
    r0, r1 = rows if rows else (0, h)
    cnt = np.zeros(3, np.uint64)
    c = img.as_c()
    rc = lib.oracle_render(ctypes.addressof(scene), r0, r1, int(jitter), threads or os.cpu_count() or 1,
                           ctypes.addressof(c), _p(cnt))
    if rc != 0:
        raise RuntimeError("oracle_render rejected its arguments")
    return img, cnt


def render_exact(lib, scene, threads=None):
    """The oracle render with every hit moved onto the level set DE = thr (hit layer 3
    where that fails): the forward pass of the gradient checks. Returns a CImage."""
    import mandelbulber_gb300 as mb
    img = mb.CImage.empty(scene.image_width, scene.image_height)
    c = img.as_c()
    rc = lib.oracle_render_exact(ctypes.addressof(scene), 0, scene.image_height, threads or os.cpu_count() or 1,
                                 ctypes.addressof(c))
    if rc != 0:
        raise RuntimeError("oracle_render_exact rejected its arguments")
    return img


def pixel_work(lib, scene, threads=None):
    """Renders the scene on the CPU and returns (CImage, work) where work[y, x] = (orbit
    iterations, DE calls, march steps) of that pixel's rays."""
    import mandelbulber_gb300 as mb
    w, h = scene.image_width, scene.image_height
    img = mb.CImage.empty(w, h)
    work = np.zeros((h, w, 3), np.uint64)
    c = img.as_c()
    rc = lib.oracle_render_pixel_work(ctypes.addressof(scene), 0, h, threads or os.cpu_count() or 1,
                                      ctypes.addressof(c), _p(work))
    if rc != 0:
        raise RuntimeError("oracle_render_pixel_work rejected its arguments")
    return img, work
