"""ctypes mirror of the plain-C structs declared in include/mbgb.h.

The struct bodies are read from the header itself, so the Python layout cannot
drift from the C layout (tests also compare sizes with the library).
"""
from __future__ import annotations

import ctypes
import os
import re

_HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "mbgb.h")

_SCALARS = {
    "double": ctypes.c_double,
    "float": ctypes.c_float,
    "int32_t": ctypes.c_int32,
    "uint32_t": ctypes.c_uint32,
    "uint8_t": ctypes.c_uint8,
    "uint16_t": ctypes.c_uint16,
    "int64_t": ctypes.c_int64,
    "uint64_t": ctypes.c_uint64,
    "void": ctypes.c_void_p,
}


class mbgb_rgb(ctypes.Structure):
    _fields_ = [("R", ctypes.c_int32), ("G", ctypes.c_int32), ("B", ctypes.c_int32)]


def _struct_fields(name: str):
    text = open(_HEADER).read()
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S)
    if not m:
        raise RuntimeError(f"struct {name} not found in {_HEADER}")
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    fields = []
    for stmt in body.split(";"):
        stmt = stmt.strip()
        if not stmt:
            continue
        parts = stmt.split(None, 1)
        ctype, rest = parts[0], parts[1]
        if ctype == "mbgb_rgb":
            base = mbgb_rgb
        else:
            base = _SCALARS[ctype]
        for decl in rest.split(","):
            decl = decl.strip()
            ptr = decl.startswith("*")
            decl = decl.lstrip("*").strip()
            dims = [int(d) for d in re.findall(r"\[(\d+)\]", decl)]
            fname = decl.split("[")[0].strip()
            t = ctypes.c_void_p if ptr else base
            for d in reversed(dims):
                t = t * d
            fields.append((fname, t))
    return fields


class mbgb_scene(ctypes.Structure):
    _fields_ = _struct_fields("mbgb_scene")


class mbgb_image(ctypes.Structure):
    _fields_ = _struct_fields("mbgb_image")


class mbgb_opts(ctypes.Structure):
    _fields_ = _struct_fields("mbgb_opts")


class mbgb_stats(ctypes.Structure):
    _fields_ = _struct_fields("mbgb_stats")


class mbgb_tuning(ctypes.Structure):
    _fields_ = _struct_fields("mbgb_tuning")


MBGB_STATUS = {
    0: "MBGB_OK",
    1: "MBGB_ERR_BAD_PARAM",
    2: "MBGB_ERR_OOM",
    3: "MBGB_ERR_CUDA",
    4: "MBGB_ERR_TIMEOUT",
    5: "MBGB_ERR_UNSUPPORTED",
    6: "MBGB_ERR_IO",
    7: "MBGB_ERR_NO_DEVICE",
}

PREC_FP64, PREC_FP32_FIX, PREC_AUTO = 0, 1, 2
GRAD_PARAMS = 6   # MBGB_GRAD_PARAMS

# every entry point include/mbgb.h declares: name -> (restype, argtypes)
_P = ctypes.POINTER
FUNCTIONS = {
    "mbgb_version": (ctypes.c_char_p, []),
    "mbgb_last_error": (ctypes.c_char_p, []),
    "mbgb_scene_from_settings": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _P(ctypes.c_char_p), ctypes.c_int,
                                                _P(mbgb_scene)]),
    "mbgb_scene_set": (ctypes.c_int, [_P(mbgb_scene), ctypes.c_char_p, ctypes.c_char_p]),
    "mbgb_settings_string": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _P(ctypes.c_char_p), ctypes.c_int,
                                            ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32]),
    "mbgb_write_png": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_void_p]),
    "mbgb_scene_finalize": (ctypes.c_int, [_P(mbgb_scene)]),
    "mbgb_catmull_rom": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p]),
    "mbgb_scene_interpolate": (ctypes.c_int, [_P(mbgb_scene), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              _P(mbgb_scene), _P(mbgb_scene)]),
    "mbgb_palette_from_seed": (None, [ctypes.c_int32, ctypes.c_double, _P(mbgb_rgb)]),
    "mbgb_scene_supported": (ctypes.c_int, [_P(mbgb_scene)]),
    "mbgb_context_create": (ctypes.c_int, [ctypes.c_int, _P(ctypes.c_void_p)]),
    "mbgb_context_destroy": (None, [ctypes.c_void_p]),
    "mbgb_get_stats": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_stats)]),
    "mbgb_render_device": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), _P(mbgb_image), _P(mbgb_opts)]),
    "mbgb_render_host": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), _P(mbgb_image), _P(mbgb_opts)]),
    "mbgb_render_device_noalloc": (ctypes.c_int, [_P(mbgb_scene), _P(mbgb_image), _P(mbgb_opts)]),
    "mbgb_render_batch": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), ctypes.c_int32, _P(mbgb_image),
                                         _P(mbgb_opts)]),
    "mbgb_render_batch_host": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), ctypes.c_int32, _P(mbgb_image),
                                              _P(mbgb_opts)]),
    "mbgb_autotune": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), _P(mbgb_opts), _P(mbgb_tuning)]),
    "mbgb_render_grad": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), ctypes.c_int32, _P(mbgb_image),
                                        _P(ctypes.c_void_p), _P(ctypes.c_void_p), _P(ctypes.c_double),
                                        _P(mbgb_opts)]),
    "mbgb_distance_device": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "mbgb_compile_image16": (ctypes.c_int, [_P(mbgb_scene), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_void_p]),
    "mbgb_compile_image16_device": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), ctypes.c_void_p, ctypes.c_int32,
                                                   ctypes.c_int32, ctypes.c_void_p]),
    "mbgb_ssao_device": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), _P(mbgb_image), ctypes.c_void_p]),
    "mbgb_dof_device": (ctypes.c_int, [ctypes.c_void_p, _P(mbgb_scene), _P(mbgb_image), ctypes.c_void_p,
                                       ctypes.c_uint32]),
}


def declared_functions() -> list[str]:
    """Names of the functions include/mbgb.h declares (parsed from the header)."""
    text = re.sub(r"/\*.*?\*/", "", open(_HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(mbgb_[a-z0-9_]+)\s*\(", text)))
