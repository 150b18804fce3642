"""Settings reader (LoadSettings2 / LoadOneSetting / LoadSettingsPost semantics) and palette."""
import ctypes
import math

import numpy as np
import pytest

import mandelbulber_gb300 as mb

DEFAULTS = """Mandelbulber 1.1100000000000001;
image_width 800;
image_height 600;
tiles 1;
view_point_x 0;
angle_alfa -20;
angle_beta 30;
zoom 2.5;
perspective 0.5;
formula 2;
power 9;
N 250;
minN 1;
fractal_constant_factor 1;
quality 1;
shadows_enabled 1;
main_light_alfa -0.78539816339744828;
mandelbox_rotation_X1_alfa 90;
coloring_random_seed 123456;
coloring_saturation 1;
julia_mode 0;
palette 0 0 0 0 ;
"""

SCENE = """Mandelbulber 1.21;
image_width 320;
N 12.9;
formula 8;
angle_gamma 45;
julia_mode 7;
IFS_absX 0.5;
shadows_enabled 0;
coloring_random_seed 42;
some_unknown_key 5;
view_point_y -3.25;
"""


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_layering_conversions_and_derivations(mblib, tmp_path):
    d = _write(tmp_path, "defaults", DEFAULTS)
    f = _write(tmp_path, "scene.fract", SCENE)
    s = mb.load_settings(f, defaults=d, overrides=["image_height=100", "power 7.5"])
    assert s.image_width == 320 and s.image_height == 100       # file over defaults, -o over file
    assert s.power == 7.5
    assert s.N == 12.0                                            # atoi, stored as double
    assert s.formula == 8 and s.analitycDE == 1                   # noGUI analytic-DE rule
    assert math.isclose(s.alpha, -20 / 180 * math.pi) and math.isclose(s.gamma, 45 / 180 * math.pi)
    assert s.mboxRotation[0][0][0] == 90 / 180.0 * math.pi
    assert s.mainLightAlpha == -0.78539816339744828             # light angles stay radians
    assert s.juliaMode == 1 and s.ifsAbsX == 1 and s.shadow == 0
    assert s.vp[1] == -3.25
    assert s.resolution == 1.0 / 320 / 1
    assert s.settingsVersion == 1.21
    # the file carried no palette: it is regenerated from its own seed
    assert s.paletteLoaded == 0
    np.testing.assert_array_equal(np.array([[c.R, c.G, c.B] for c in s.palette]), mb.palette_from_seed(42, 1.0))


def test_clamps_of_checkparameters(mblib, tmp_path):
    f = _write(tmp_path, "c.fract", "image_width 10;\nimage_height 8;\nzoom 0;\nDE_factor 0;\nperspective 0;\n"
               "ambient_occlusion_quality 99;\ntiles 0;\nvolumetric_fog_density -3;\nsmoothness 0;\n")
    with pytest.raises(mb.MbgbError):
        mb.load_settings(f)       # tiles 0: resolution would divide by zero
    f = _write(tmp_path, "c2.fract", "image_width 10;\nimage_height 8;\nzoom 0;\nDE_factor 0;\nperspective 0;\n"
               "ambient_occlusion_quality 99;\ntiles 1;\nvolumetric_fog_density -3;\nsmoothness 0;\n")
    s = mb.load_settings(f)
    assert s.image_width == 32 and s.image_height == 32
    assert s.resolution == 1.0 / 10          # derived before the clamp, as the reference does
    assert s.zoom == 1e-15 and s.DE_factor == 0.0001 and s.persp == 0.001
    assert s.globalIlumQuality == 30 and s.fogDensity == 0.0 and s.smoothness == 0.00001


def test_palette_string(mblib, tmp_path):
    pal = " ".join(f"{(i * 65793) & 0xffffff:x}" for i in range(256))
    f = _write(tmp_path, "p.fract", f"image_width 64;\ntiles 1;\npalette {pal} ;\n")
    s = mb.load_settings(f)
    assert s.paletteLoaded == 1
    got = np.array([[c.R, c.G, c.B] for c in s.palette])
    want = np.array([[((i * 65793) & 0xffffff) // 65536, (((i * 65793) & 0xffffff) // 256) % 256,
                      ((i * 65793) & 0xffffff) % 256] for i in range(256)])
    np.testing.assert_array_equal(got, want)


def test_missing_file_is_an_io_error(mblib, tmp_path):
    with pytest.raises(mb.MbgbError) as e:
        mb.load_settings(str(tmp_path / "absent.fract"))
    assert e.value.status == 6


@pytest.mark.parametrize("seed,sat", [(123456, 1.0), (627277, 1.0), (1, 0.5), (0, 2.0), (99991, 0.0)])
def test_palette_matches_c_library_rand(mblib, seed, sat):
    """NewPalette (src/image.cpp:28-55) after srand(seed) with the C library's rand()."""
    libc = ctypes.CDLL(None)
    libc.srand(seed)
    rnd = lambda m: libc.rand() % (m + 1)  # noqa: E731  Random(max), src/common_math.cpp:25-32
    want = np.zeros((256, 3), np.int64)
    for i in range(255):
        y = int((rnd(255) - 128) / (1.0 + sat))
        for c in range(3):
            want[i, c] = min(255, max(0, int(y + 128 + (rnd(255) - 128) * sat)))
    want[255] = (255, 255, 255)
    want[254] = (0, 0, 0)
    want[253] = (0, 20, 40)
    np.testing.assert_array_equal(mb.palette_from_seed(seed, sat), want)
