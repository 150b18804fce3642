"""The headline frame and the Mandelbulb frame at their full sizes against the CPU oracle
(needs a GPU).

The other parity tests hold the FP32 policy against the oracle at up to 480x270. Here the
strict FP64 oracle (oracle/mb_oracle.cpp, -O2 -ffp-contract=off, bit-exact to the
reference's own compiled code on every golden) renders the frames the bench measures,
with every host thread (the 1920x1080 frame takes about a minute on 16 cores):
  * 1920x1080 Mandelbox (scale 2, N 15, hard shadow, ray AO with 29 directions,
    volumetric fog, glow): the FP64 policy equals the oracle bit for bit on hit mask,
    depth, iterations, z-buffer, alpha, opacity and colour (only + - * / sqrt on the
    path; pow() in the specular term moves the float image by <= 1e-6), as the small
    golden frames do (src/Render3D.cpp:79-199, src/fractal.cpp:467-528);
  * the same frame under the FP32 + FP64-fix policy, with the selective and with the
    full FP64 polish: hit/miss mismatch <= 0.1 % and float-image PSNR >= 45 dB against the
    oracle (the headline bar);
  * 640x480 Mandelbulb power 8, N 250, hard shadow: the FP64 policy and the FP32 policy
    each within hit/miss mismatch <= 0.1 % and PSNR >= 45 dB of the oracle (CUDA's double
    asin/atan2/pow may round a last bit differently from the host's libm, so bit equality
    is not required here).
"""
import os

import numpy as np
import pytest

import mandelbulber_gb300 as mb
from mandelbulber_gb300 import workloads as W
from tests import metrics, oracle_lib

pytestmark = pytest.mark.gpu
EXACT = ["hit", "iters", "depth", "zbuffer", "alpha", "opacity", "colour"]


@pytest.fixture(scope="module")
def box_1080p(oracle):
    sc = W.workload("mandelbox_1080p")
    ref, _ = oracle_lib.render(oracle, sc, threads=os.cpu_count())
    return sc, ref


@pytest.fixture(scope="module")
def bulb_640x480(oracle):
    sc = W.workload("mandelbulb_640x480")
    ref, _ = oracle_lib.render(oracle, sc, threads=os.cpu_count())
    return sc, ref


def test_fp64_1080p_equals_the_oracle(gpu_ctx, box_1080p):
    sc, ref = box_1080p
    img = gpu_ctx.render(sc, precision=mb.PREC_FP64)
    for k in EXACT:
        np.testing.assert_array_equal(getattr(img, k), getattr(ref, k), err_msg=k)
    np.testing.assert_allclose(img.image_float, ref.image_float, rtol=0, atol=1e-6)


@pytest.mark.parametrize("polish_all", [False, True], ids=["selective_polish", "polish_all"])
def test_fp32_fix_1080p_against_the_oracle(gpu_ctx, box_1080p, polish_all):
    sc, ref = box_1080p
    img = gpu_ctx.render(sc, precision=mb.PREC_FP32_FIX, polish_all=polish_all)
    m = metrics.compare(img, ref)
    print("1080p fp32_fix vs oracle", "polish_all" if polish_all else "selective", m)
    assert m["hit_mismatch"] <= 0.001, m
    assert m["psnr_float"] >= 45.0, m


@pytest.mark.parametrize("precision", [mb.PREC_FP64, mb.PREC_FP32_FIX], ids=["fp64", "fp32_fix"])
def test_mandelbulb_640x480_against_the_oracle(gpu_ctx, bulb_640x480, precision):
    sc, ref = bulb_640x480
    img = gpu_ctx.render(sc, precision=precision)
    m = metrics.compare(img, ref)
    print("640x480 mandelbulb vs oracle", precision, m)
    assert m["hit_mismatch"] <= 0.001, m
    assert m["psnr_float"] >= 45.0, m
