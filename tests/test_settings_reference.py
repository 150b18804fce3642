"""The .fract settings reader against the reference's own.

mbgb_scene_from_settings / mbgb_scene_set + mbgb_scene_finalize (csrc/settings.cpp)
restate LoadSettings2 / LoadOneSetting / LoadSettingsPost (src/settings.cpp:628-698,
700-1183, 1185-1195), the -nogui tail of ReadInterface (src/interface.cpp:690-729),
the rotations of RecalculateIFSParams (src/callbacks.cpp:1538-1556) and CheckPrameters
(src/interface.cpp:3587-3602). The reference's src/settings.cpp, compiled in place
into oracle/_ref/libmbref_settings.so, reads the same inputs; the scenes must agree
byte for byte, field by field:
  * every shipped settings file: share/defaults and each share/examples/*.fract and
    share/exampleKeyframes/*.fract loaded after share/defaults, as LoadSettings does;
  * the same files with -o override strings (LoadSettings2 applies them after each file);
  * the key lists the benchmark workloads and golden scenes are built from.
tests/golden/settings_reference.npz records the reference's scenes (with the SHA-256 of
each file read); tests/golden/bench_scenes.npz the workloads' scenes, which the bench's
reference arm renders. Where the reference tree is absent, the tests that need it skip.
A palette given as an override string is left out: the override's "%1999s" stops at
the first space, so it carries one colour token, and GetPaletteFromString then reads
its buffer past the string's end (src/settings.cpp:97-111), which has no defined value.
"""
import ctypes
import hashlib
import os

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W
from tests import oracle_lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
OVERRIDES = ["image_width 333", "image_height=201", "N=77", "angle_alfa 12.5", "mandelbox_rotation_X1_beta -7",
             "ambient_occlusion_enabled 1", "fractal_constant_factor 1.25", "IFS_absX 0.5", "tiles 200",
             "ambient_occlusion_quality 40", "DE_factor 0.00001", "volumetric_light_enabled_3 1"]


def _ref():
    lib = oracle_lib.load_ref_settings()
    if lib is None:
        pytest.skip("the reference tree is absent (MBGB_REF_TREE)")
    return lib


def _files():
    root = os.path.join(oracle_lib.ref_tree(), "share")
    ex = sorted(f for f in os.listdir(os.path.join(root, "examples")) if f.endswith(".fract"))
    kf = sorted(f for f in os.listdir(os.path.join(root, "exampleKeyframes")) if f.endswith(".fract"))
    return ([("defaults", os.path.join(root, "defaults"))]
            + [("examples/" + f, os.path.join(root, "examples", f)) for f in ex]
            + [("exampleKeyframes/" + f, os.path.join(root, "exampleKeyframes", f)) for f in kf])


def _differing_fields(a: mb.mbgb_scene, b: mb.mbgb_scene) -> list:
    ra, rb = mb.scene_bytes(a), mb.scene_bytes(b)
    out = []
    for name, _ in mb.mbgb_scene._fields_:
        d = getattr(mb.mbgb_scene, name)
        if ra[d.offset:d.offset + d.size] != rb[d.offset:d.offset + d.size]:
            out.append(name)
    return out


def _both(lib, name, path, overrides=()):
    defaults = None if name == "defaults" else os.path.join(oracle_lib.ref_tree(), "share", "defaults")
    ours = mb.load_settings(path, defaults, list(overrides))
    ref = oracle_lib.ref_scene_from_settings(lib, mb.mbgb_scene(), defaults, path, list(overrides))
    return ours, ref


def test_every_shipped_settings_file_loads_as_the_reference_loads_it():
    lib = _ref()
    files = _files()
    assert len(files) == 1 + 77 + 11
    golden = np.load(os.path.join(GOLDEN, "settings_reference.npz"))
    gidx = {str(n): i for i, n in enumerate(golden["names"])}
    for name, path in files:
        ours, ref = _both(lib, name, path)
        assert _differing_fields(ours, ref) == [], name
        with open(path, "rb") as f:
            sha = hashlib.sha256(f.read()).hexdigest()
        i = gidx[name]
        if str(golden["sha256"][i]) == sha:   # the recorded reading of this very file
            assert golden["scenes"][i].tobytes() == mb.scene_bytes(ref), name


def test_override_strings_apply_as_the_reference_applies_them():
    lib = _ref()
    files = _files()
    picked = files[1::9] + [files[-1]]
    for name, path in picked:
        ours, ref = _both(lib, name, path, OVERRIDES)
        assert _differing_fields(ours, ref) == [], name
        # the overrides took effect, the clamps of CheckPrameters included
        assert (ref.image_width, ref.image_height, ref.N) == (333, 201, 77.0)
        assert ref.noOfTiles == 100 and ref.globalIlumQuality == 30 and ref.DE_factor == 0.0001
        assert ref.volumetricLightEnabledAny == 1


def test_workload_key_lists_read_as_the_reference_reads_them():
    lib = _ref()
    from tests.golden import make_golden as G
    cases = {**G.CASES, **G.FORMULA_CASES}
    for case, (wl, w, h, extra) in cases.items():
        keys = dict(W.WORKLOADS[wl])
        keys["image_width"], keys["image_height"] = w, h
        keys["perspective"] = W.fov_persp(w, h)
        keys.update(extra)
        ours = W.make_scene(keys)
        full = dict(W.BASE)
        full.update(keys)
        ref = oracle_lib.ref_scene_from_keys(lib, mb.mbgb_scene(), full)
        assert _differing_fields(ours, ref) == [], case


def test_bench_scenes_are_the_workloads():
    """Runs everywhere: the committed scenes the bench's reference arm renders (read by the
    reference's LoadOneSetting) equal the scenes the device arm builds."""
    z = np.load(os.path.join(GOLDEN, "bench_scenes.npz"))
    for name in z.files:
        sc = mb.scene_from_bytes(z[name].tobytes())
        assert _differing_fields(W.workload(name), sc) == [], name
    assert ctypes.sizeof(mb.mbgb_scene) == z["mandelbox_1080p"].size


def test_settings_golden_covers_every_shipped_file():
    """Runs everywhere: the recorded readings cover share/defaults, 77 examples and 11 keyframes,
    and each is a scene the device path accepts or rejects with a reason."""
    golden = np.load(os.path.join(GOLDEN, "settings_reference.npz"))
    names = [str(n) for n in golden["names"]]
    assert names[0] == "defaults"
    assert sum(n.startswith("examples/") for n in names) == 77
    assert sum(n.startswith("exampleKeyframes/") for n in names) == 11
    formulas = set()
    for raw in golden["scenes"]:
        sc = mb.scene_from_bytes(raw.tobytes())
        formulas.add(int(sc.formula))
        ok, why = mb.supported(sc)
        assert ok or why, "rejected without a reason"
    assert {2, 8}.issubset(formulas)
