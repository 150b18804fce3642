"""The oracle restatement against golden vectors from the reference's own compiled code.

tests/golden/*.npz were produced by tests/golden/make_golden.py, which ran the
reference's src/fractal.cpp and src/shaders.cpp (compiled in place) through
oracle/ref_harness.cpp. The oracle must reproduce them bit for bit.
"""
import glob
import json
import os

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from tests import oracle_lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LAYERS = ["image_float", "zbuffer", "alpha", "opacity", "colour", "hit", "iters", "depth"]


def _scene(z):
    return mb.scene_from_bytes(z["scene"].tobytes())


DES = sorted(os.path.basename(p)[3:-4] for p in glob.glob(os.path.join(GOLDEN, "de_*.npz")))


@pytest.mark.parametrize("formula", DES)
def test_distance_estimator_bit_exact(oracle, mblib, formula):
    z = np.load(os.path.join(GOLDEN, f"de_{formula}.npz"))
    sc = _scene(z)
    d, it, mi = oracle_lib.distance(oracle, sc, z["points"], z["detail"])
    np.testing.assert_array_equal(d, z["dist"])
    np.testing.assert_array_equal(it, z["iters"])
    np.testing.assert_array_equal(mi, z["max_iter"])


@pytest.mark.parametrize("formula", DES)
def test_colouring_value_bit_exact(oracle, mblib, formula):
    z = np.load(os.path.join(GOLDEN, f"de_{formula}.npz"))
    sc = _scene(z)
    np.testing.assert_array_equal(oracle_lib.colour_value(oracle, sc, z["points"]), z["colour"])


RENDERS = sorted(os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(GOLDEN, "render_*.npz")))


@pytest.mark.parametrize("case", RENDERS)
def test_render_bit_exact(oracle, mblib, case):
    z = np.load(os.path.join(GOLDEN, f"render_{case}.npz"))
    sc = _scene(z)
    img, _ = oracle_lib.render(oracle, sc, threads=2)
    for layer in LAYERS:
        np.testing.assert_array_equal(getattr(img, layer), z[layer], err_msg=f"{case}: layer {layer}")


KEYED = [c for c in RENDERS if "keys" in np.load(os.path.join(GOLDEN, f"render_{c}.npz")).files]


@pytest.mark.parametrize("case", KEYED)
def test_golden_scene_rebuilds_from_keys(mblib, case):
    """The stored settings keys rebuild the stored scene bytes (parser + derivations are stable).
    Fixtures made from the reference's example files store the loaded scene only."""
    from mandelbulber_gb300 import workloads as W
    z = np.load(os.path.join(GOLDEN, f"render_{case}.npz"))
    keys = json.loads(str(z["keys"]))
    assert mb.scene_bytes(W.make_scene(keys)) == z["scene"].tobytes()


def test_oracle_row_range_and_threads_agree(oracle, mblib):
    """Row subsets and thread counts do not change the (jitter-free) result."""
    z = np.load(os.path.join(GOLDEN, "render_mandelbulb_64x48.npz"))
    sc = _scene(z)
    img, _ = oracle_lib.render(oracle, sc, rows=(10, 30), threads=3)
    np.testing.assert_array_equal(img.image_float[10:30], z["image_float"][10:30])
    assert np.all(img.hit[:10] == 0) and np.all(img.hit[30:] == 0)
