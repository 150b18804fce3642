"""Keyframe interpolation against the reference's own CMorph::CatmullRom (golden vectors)."""
import ctypes
import os

import numpy as np

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_catmull_rom_bit_exact(mblib):
    z = np.load(os.path.join(GOLDEN, "catmull_rom.npz"))
    keys = np.ascontiguousarray(z["keys"])
    n_keys, size = keys.shape
    fpk = int(z["frames_per_key"])
    out = np.zeros(size)
    for frame in range(n_keys * fpk):
        rc = mblib.mbgb_catmull_rom(keys.ctypes.data, n_keys, size, fpk, frame, out.ctypes.data)
        assert rc == 0
        np.testing.assert_array_equal(out, z["out"][frame], err_msg=f"frame {frame}")


def test_scene_interpolation_passes_through_keys_and_rebuilds_derived_fields(mblib):
    keys = (mb.mbgb_scene * 3)()
    for k, y in enumerate([-3.5, -3.0, -2.5]):
        keys[k] = W.workload("mandelbulb_640x480", 64, 48, view_point_y=y, angle_alfa=10.0 * k,
                             mandelbox_rotation_main_gamma=5.0 * k, mandelbox_rotation_enabled=1)
    out = mb.mbgb_scene()
    for frame, want_y in [(0, -3.5), (4, -3.0), (8, -2.5)]:
        assert mblib.mbgb_scene_interpolate(keys, 3, 4, frame, None, ctypes.byref(out)) == 0
        assert out.vp[1] == want_y                                  # Catmull-Rom hits the keys
    assert mblib.mbgb_scene_interpolate(keys, 3, 4, 2, None, ctypes.byref(out)) == 0
    assert -3.5 < out.vp[1] < -3.0
    assert out.resolution == 1.0 / 64
    assert out.mboxMainRotZero == 0                                 # matrices rebuilt from the angles
    assert mblib.mbgb_scene_interpolate(keys, 3, 4, 12, None, ctypes.byref(out)) == 1   # past the last key
