"""The escape-radius option of the trigonometric formulas (mbgb_scene.bailoutRadius).

The reference hard-codes r > 100 for the distance mode of trig_DE / trig_optim
(src/fractal.cpp:1151-1157). The Mandelbulb configuration of the benchmark names r > 10,
so the scene carries an escape radius (0 = the reference's 100) that the device
kernels and the oracle honour. Here the oracle's distances with r > 10 are checked
against a plain restatement of the trig_optim orbit (src/fractal.cpp:211-225) and the
analytic estimate 0.5 r ln r / dr, and the radius is checked to change them.
"""
import math

import numpy as np

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W
from tests import oracle_lib


def _trig_optim_distance(px, py, pz, n, power, bail):
    x, y, z = px, py, pz
    r = math.sqrt(x * x + y * y + z * z)
    r_dz = 1.0
    for _ in range(n):
        th0 = math.asin(z / r)
        ph0 = math.atan2(y, x)
        rp = math.pow(r, power - 1.0)
        th, ph = th0 * power, ph0 * power
        cth = math.cos(th)
        r_dz = rp * r_dz * power + 1.0
        rp *= r
        x, y, z = cth * math.cos(ph) * rp + px, cth * math.sin(ph) * rp + py, math.sin(th) * rp + pz
        r = math.sqrt(x * x + y * y + z * z)
        if r > bail:
            return max(0.5 * r * math.log(r) / r_dz, 0.0)
    return 0.0


def test_oracle_honours_the_escape_radius(oracle):
    rng = np.random.default_rng(11)
    pts = rng.uniform(-1.4, 1.4, (300, 3))
    detail = np.full(len(pts), 1e-9)
    near = W.workload("mandelbulb_640x480", 64, 48)
    far = W.workload("mandelbulb_640x480", 64, 48)
    far.bailoutRadius = 10
    d100, it100, _ = oracle_lib.distance(oracle, near, pts, detail)
    d10, it10, _ = oracle_lib.distance(oracle, far, pts, detail)
    escaped = it10 < int(far.N)
    assert escaped.mean() > 0.5
    assert (it10[escaped] <= it100[escaped]).all() and (it10 < it100).any()
    assert np.abs(d10 - d100).max() > 0
    for k in np.flatnonzero(escaped)[:60]:
        want = _trig_optim_distance(*pts[k], int(far.N), far.power, 10.0)
        assert abs(d10[k] - want) <= 1e-10 * max(abs(want), 1e-12), (k, d10[k], want)


def test_default_scene_keeps_the_reference_radius():
    sc = W.workload("mandelbulb_640x480")
    assert sc.bailoutRadius == 0
    assert mb.mbgb_scene.bailoutRadius.size == 2
