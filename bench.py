#!/usr/bin/env python
"""Benchmark of the per-pixel DE ray-march render on GB300.

Workload (default): the 1920x1080 Mandelbox scene (scale 2, 15 iterations, hard
shadows, ray-traced AO with 29 directions, volumetric fog 0.5, glow), rendered
with the FP32 march + FP64 hit refinement policy. One step = one full frame.
The same frame in the plain FP64 policy is timed beside it (the headline metric's
FP32-vs-FP64 ratio), and the two are compared (hit/miss mismatch, PSNR).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times the CPU implementation of the path (the oracle
restatement, built with the reference's -O3 -ffast-math flags, its
one-worker-per-core row claiming and rand() step jitter) on a bounded sample of
rows spread evenly over the same frame, with every host thread. It loads the
frame's scene from the committed bytes in tests/golden/bench_scenes.npz and
loads nothing but the oracle library.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1080p Mpix/s: FP32+FP64-fix vs plain FP64 at ≤0.1% hit mismatch; grads/s"
WORKLOAD = "mandelbox_1080p"
# algorithmic work of one orbit iteration / one DE evaluation (Mandelbox, no rotation):
# 3 fold add/sub + 5 for x^2+y^2+z^2 + 5 sphere fold (1 div) + 6 for z*scale+c + 2 for DE*|s|+1,
# plus sqrt and divide of each DE evaluation
FLOPS_PER_ITER = {8: 21, 2: 27}
# dram__bytes_read.sum + dram__bytes_write.sum of secondary_kernel in one full 1920x1080
# launch of this workload (a one-pass ncu capture of `bench.py --once 1920x1080`): 124.8 MB
# read (the per-hit set-up records and hit list, once per block of 4096 hits) + 157.6 MB
# written (the per-direction AO result slots that leave L2); at 480x270 both stay in L2, and
# a small capture sees almost no DRAM traffic
DRAM_BYTES_PER_LAUNCH = {"mandelbox_1080p": 282.4e6}
FLOPS_PER_DE = {8: 2, 2: 4}
PRECISION = "fp32 march/orbit/shading + fp64 ray origin and binary hit refinement"
# the single-frame workloads bench.py times (the scenes are built by mandelbulber_gb300.workloads;
# their bytes are committed in tests/golden/bench_scenes.npz for the reference arm)
WORKLOADS = {
    "mandelbox_1080p": {"width": 1920, "height": 1080,
                        "scene": "Mandelbox scale 2 (formula 8), N 15, camera (0,-20,0), 53 deg FOV, hard shadow, "
                                 "ray AO q2 (29 dirs), volumetric fog 0.5, glow"},
    "mandelbulb_640x480": {"width": 640, "height": 480,
                           "scene": "Mandelbulb power 8 (formula 2), N 250, camera (0,-3.5,0), 53 deg FOV, "
                                    "hard shadow, no AO / fog / glow"},
}
BENCH_SCENES = os.path.join(ROOT, "tests", "golden", "bench_scenes.npz")


def reference_rows(threads: int) -> int:
    """Rows of one reference-arm step: four per host thread (the dynamic row claiming then
    balances rows of unequal cost), at least 32."""
    return max(4 * threads, 32)


def bench_config(workload: str, world: int) -> dict:
    """The `config` of both arms' lines (identical, so the two lines describe one workload)."""
    wl = WORKLOADS[workload]
    threads = os.cpu_count() or 1
    return {"workload": workload, "width": wl["width"], "height": wl["height"], "scene": wl["scene"],
            "precision": PRECISION, "l2": "flushed between timed frames (512 MiB write)",
            "parallelism": f"replicas x{world}",
            "reference_sample": (f"--impl reference: {reference_rows(threads)} of the {wl['height']} rows per step, "
                                 f"spread evenly over the frame, {threads} host threads, Mpix/s of those rows")}


def bench_scene_buffer(workload: str):
    """The committed mbgb_scene bytes of a workload as a ctypes buffer (no product import)."""
    z = np.load(BENCH_SCENES)
    return ctypes.create_string_buffer(z[workload].tobytes())


def max_over_ranks(seconds: float, dist, device) -> float:
    """The slowest rank's timed region (every rank gets it); `dist` is torch.distributed or
    None for one process. `device` holds the reduction tensor (a GPU for NCCL, "cpu" for gloo)."""
    if not dist:
        return seconds
    import torch
    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_rank_step: float, steps: int, seconds: float) -> float:
    """Weak scaling: every rank processes the same units per step; the job's rate is all
    ranks' units over the slowest rank's time."""
    return world * units_per_rank_step * steps / seconds


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxs.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs), "reasons": sorted(reasons),
                "samples": len(sms)}


def cpu_sample(scene, seconds: float, jitter: bool = True):
    """Times the CPU oracle on rows spread evenly over the frame, as many as about `seconds`
    of work takes; returns (Mpix/s, desc)."""
    from tests import oracle_lib
    lib = oracle_lib.load(fast=True)
    threads = os.cpu_count() or 1
    w, h = scene.image_width, scene.image_height
    n = max(threads, 8)
    while True:
        rows = oracle_lib.sample_rows(h, n)
        t0 = time.perf_counter()
        oracle_lib.render_row_list(lib, ctypes.addressof(scene), w, h, rows, jitter=jitter, threads=threads)
        dt = time.perf_counter() - t0
        if dt >= seconds * 0.5 or len(rows) >= h:
            break
        n = min(h, int(n * max(2.0, seconds / max(dt, 1e-3) * 0.9)))
    px = len(rows) * w
    return px / dt / 1e6, {"rows": len(rows), "pixels": px, "seconds": dt, "threads": threads}


def run_reference(args, rank: int, world: int) -> int:
    """The reference arm: the CPU implementation of the path on the host cores, on the same
    workload and config as the GPU arm, one bounded row sample per step."""
    if rank != 0:
        return 0
    from tests import oracle_lib
    wl = WORKLOADS[args.workload]
    w, h = wl["width"], wl["height"]
    scene = bench_scene_buffer(args.workload)
    lib = oracle_lib.load(fast=True)
    threads = os.cpu_count() or 1
    rows = oracle_lib.sample_rows(h, reference_rows(threads))
    layers = oracle_lib.alloc_layers(w, h)
    for _ in range(args.warmup):
        oracle_lib.render_row_list(lib, ctypes.addressof(scene), w, h, rows[::4], jitter=True, threads=threads,
                                   layers=layers)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle_lib.render_row_list(lib, ctypes.addressof(scene), w, h, rows, jitter=True, threads=threads,
                                   layers=layers)
        times.append(time.perf_counter() - t0)
    px = len(rows) * w
    value = px * len(times) / sum(times) / 1e6
    sample = (f"{len(rows)} rows spread evenly over the {w}x{h} frame ({px} px per step), the CPU oracle "
              f"restatement (bit-exact to the reference's own compiled code on every golden) built with the "
              f"reference flags -O3 -ffast-math, rand() step jitter, one worker per host thread, dynamic rows")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args.workload, world),
            "cpu_baseline": {"value": value, "unit": "Mpix/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def batch_section(ctx, torch, dev, stream, flush, args, world, dist) -> dict:
    """The 64-frame flight animation (Mandelbulb power 8, per-frame resolutions 320x240 ..
    1920x1080, hard shadows + fast AO q4, FP32 with FP64 refinement) as one batch: the
    launch configuration comes from the autotuner and the launches are captured once in a
    CUDA graph and replayed. One step = one batch of 64 frames."""
    import mandelbulber_gb300 as mb
    from mandelbulber_gb300 import workloads as W
    frames = W.flight()
    npx = sum(f.image_width * f.image_height for f in frames)
    bufs, layers = [], []
    for f in frames:
        n = f.image_width * f.image_height
        b = {"image_float": torch.empty(n * 3, dtype=torch.float32, device=dev),
             "zbuffer": torch.empty(n, dtype=torch.float32, device=dev),
             "alpha": torch.empty(n, dtype=torch.int16, device=dev),
             "opacity": torch.empty(n, dtype=torch.int16, device=dev),
             "colour": torch.empty(n * 3, dtype=torch.uint8, device=dev)}
        bufs.append(b)
        layers.append({k: v.data_ptr() for k, v in b.items()})
    big = max(frames, key=lambda f: f.image_width * f.image_height)
    tuning = ctx.autotune(big)

    def run(steps, warmup, **opts):
        for _ in range(warmup):
            ctx.render_batch_device(frames, layers, stream=stream.cuda_stream, **opts)
        stream.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        for e0, e1 in evs:
            with torch.cuda.stream(stream):
                flush.zero_()
                e0.record(stream)
            ctx.render_batch_device(frames, layers, stream=stream.cuda_stream, **opts)
            e1.record(stream)
        stream.synchronize()
        total = sum(a.elapsed_time(b) for a, b in evs) / 1e3
        return max_over_ranks(total, dist, dev)

    steps = max(1, args.batch_steps)
    t_graph = run(steps, 3, autotune=True, use_graph=True)
    # counters of one batch (synchronous call)
    ctx.render_batch_device(frames, layers, autotune=True, use_graph=True)
    st = ctx.stats()
    t_plain = run(1, 1)
    return {"workload": "flight_64", "frames": len(frames), "pixels_per_batch": npx, "steps": steps,
            "value": world * npx * steps / t_graph / 1e6, "unit": "Mpix/s",
            "ms_per_batch": 1e3 * t_graph / steps,
            "untuned_ungraphed_ms_per_batch": 1e3 * t_plain,
            "graph_replayed": int(st.graph_replayed), "launches_per_batch": int(st.launches),
            "de_evaluations_per_s": world * st.de_calls * steps / t_graph,
            "tuning": {"tile": [tuning.tile_w, tuning.tile_h], "threads_per_cta": tuning.threads_per_cta,
                       "ctas_per_sm": tuning.ctas_per_sm, "refill_min": tuning.refill_min,
                       "orbit_refill": tuning.orbit_refill,
                       "tuned_ms": tuning.ms, "default_ms": tuning.ms_default, "trials": tuning.trials,
                       "tuning_frame": [big.image_width, big.image_height]},
            "scene": "Mandelbulb power 8, N 250, flight through 8 seeded keyframes (shell r 2-4, looking at "
                     "the origin), Catmull-Rom, 8 frames per key, seeded resolutions, hard shadows, fast AO q4",
            "precision": "fp32 march/orbit/shading + fp64 ray origin and binary hit refinement"}


def grad_section(ctx, torch, dev, args) -> dict:
    """The gradient workload: 32 Mandelbulb frames at 256x256 with seeded theta (power,
    camera position, light angles), loss = L2 against targets rendered at theta + delta.
    One step = the differentiable render of all 32 frames (forward stages with level-set
    hits plus the gradient stage) and the read-back of dL/dtheta; FP32 policy."""
    import mandelbulber_gb300 as mb
    from mandelbulber_gb300 import diff as D
    scenes, th, tg = D.grad_batch(32, 256)
    RT = D.Renderer(ctx, scenes, mb.PREC_FP32_FIX)
    RT.set_theta(tg)
    T = RT.forward().clone()
    R = D.Renderer(ctx, scenes, mb.PREC_FP32_FIX)
    R.set_theta(th)
    I = R.forward()
    dL = (2 * (I - T)).contiguous()
    for _ in range(3):
        R.backward(dL)
    # per-stage device times of one differentiable render of the batch
    g = ctx.render_grad(R.scenes, R.layers(), dL_dimage=[dL[i].data_ptr() for i in range(len(scenes))],
                        precision=mb.PREC_FP32_FIX, profile_stages=True)
    st = ctx.stats()
    names = ["primary_kernel", "polish_kernel", "secondary_kernel", "compose_kernel", "level_set_kernel",
             "grad_kernel"]
    stage_ms = {names[k]: float(st.stage_ms[k]) for k in range(6)}
    steps = max(1, args.grad_steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    e0.record()
    for _ in range(steps):
        g = R.backward(dL)
    e1.record()
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    st = ctx.stats()
    return {"workload": "grad_mandelbulb_32x256", "frames": len(scenes), "params_per_frame": D.GRAD_PARAMS,
            "value": len(scenes) * steps / wall, "unit": "grads/s (theta-vectors/s)", "steps": steps,
            "ms_per_batch": 1e3 * wall / steps, "device_ms_per_batch": e0.elapsed_time(e1) / steps,
            "grad_pixels": int(st.grad_pixels), "grad_skipped": int(st.grad_skipped),
            "launches_per_batch": int(st.launches), "finite": bool(np.isfinite(g).all()), "stage_ms": stage_ms,
            "precision": "fp32 forward, fp32 level-set hits and dual-number orbits (fp64 for a sample whose "
                         "tangents leave fp32's range or whose Newton step fails), fp64 shading algebra",
            "check": "tests/test_gpu_grad.py: adjoint vs central differences (h = 1e-4, FP64) within 1e-3"}


# Scenes of the other formulas and of the secondary effects (from the committed fixtures,
# which hold the reference's example scenes), rendered at a larger size for the coverage
# section: (fixture, width, height).
COVERAGE_SCENES = [
    ("trigde_40x32", 480, 270), ("ex_power2_default", 480, 270), ("ex_quaternion_lathe", 480, 270),
    ("menger_48x32", 480, 270), ("ex_ifs_icosahedron", 480, 270), ("ex_hybrid_1", 480, 270),
    ("ex_modified_mandelbulb_3", 480, 270), ("smooth_mandelbox", 480, 270), ("vary4d_48x32", 480, 270),
    ("fold_box_icosa", 480, 270), ("ex_aux_coloured_lights", 480, 270), ("ex_fx_iter_fog_2", 480, 270),
    ("ex_fx_volumetric_light_2", 480, 270), ("ex_fx_reflections_1", 480, 270), ("ex_fx_primitives_set", 480, 270),
    ("ex_fx_envmap_mandelbox", 480, 270), ("fake_lights_mandelbox", 480, 270),
    ("ex_fx_slow_interior_mandelbox", 240, 135),
]


def coverage_section(ctx) -> dict:
    """Every other formula and the secondary effects: one frame of each scene at 480x270
    (slow shading 240x135) under the FP32 policy after one untimed frame, device time from
    the library's CUDA events around its launches. Delta-DE formulas render in FP64 (the
    `fp64` flag), the effect scenes on the per-pixel engine."""
    import mandelbulber_gb300 as mb
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden")
    out = {}
    for case, w, h in COVERAGE_SCENES:
        z = np.load(os.path.join(golden, f"render_{case}.npz"))
        sc = mb.scene_from_bytes(z["scene"].tobytes())
        sc.image_width, sc.image_height = w, h
        sc.resolution = 1.0 / w / sc.noOfTiles
        ctx.render(sc, precision=mb.PREC_FP32_FIX)
        img = ctx.render(sc, precision=mb.PREC_FP32_FIX)
        st = ctx.stats()
        out[case] = {"formula": int(sc.formula), "size": [w, h], "ms": float(st.kernel_ms),
                     "mpix_per_s": w * h / (st.kernel_ms * 1e3) if st.kernel_ms > 0 else None,
                     "de_evaluations_per_s": st.de_calls / (st.kernel_ms / 1e3) if st.kernel_ms > 0 else None,
                     "fp64": bool(st.auto_fp64), "launches": int(st.launches),
                     "hit_fraction": float(img.hit.mean())}
    return out


def configs_section(ctx, cpu_seconds: float = 0.0) -> dict:
    """The other single-frame configurations at full size: config 1 (Mandelbulb power 8, N 250,
    640x480, hard shadows; at the reference's escape radius r > 100 and at the
    configuration's r > 10, with the CPU implementation's Mpix/s beside each) and config 4
    (deep zoom: Mandelbulb N 1000, 1024x1024, the camera 1e-6 from a seeded surface point).
    Per configuration and precision policy: the library's
    device time of one frame (CUDA events around its launches; best of three after a warm-up,
    one frame for FP64 and for the deep zoom, whose frames take seconds), the policy
    MBGB_PREC_AUTO picked, and the FP32_FIX frame's hit mismatch
    and float-image PSNR against the FP64 frame (the deep zoom is why AUTO exists: FP32 cannot
    resolve a 1e-6 camera distance)."""
    import mandelbulber_gb300 as mb
    from mandelbulber_gb300 import workloads as W
    from tests import metrics
    out = {}
    for name in ("mandelbulb_640x480", "mandelbulb_640x480_r10", "deep_zoom_1024"):
        if name == "deep_zoom_1024":
            sc = W.deep_zoom(ctx, size=1024)
        else:
            sc = W.workload("mandelbulb_640x480")
            if name.endswith("_r10"):
                sc.bailoutRadius = 10   # the configuration's r > 10 (the reference hard-codes r > 100)
        npx = sc.image_width * sc.image_height
        rec = {"size": [sc.image_width, sc.image_height], "formula": int(sc.formula), "N": int(sc.N),
               "escape_radius": int(sc.bailoutRadius) or 100}
        imgs = {}
        for pol, key in ((mb.PREC_FP32_FIX, "fp32_fix"), (mb.PREC_FP64, "fp64"), (mb.PREC_AUTO, "auto")):
            imgs[key] = ctx.render(sc, precision=pol)
            best = float("inf")
            for _ in range(1 if key == "fp64" or name == "deep_zoom_1024" else 3):
                ctx.render(sc, precision=pol, image=imgs[key])
                st = ctx.stats()
                best = min(best, st.kernel_ms)
            rec[key] = {"ms": best, "mpix_per_s": npx / (best * 1e3),
                        "de_evaluations_per_s": st.de_calls / (best / 1e3)}
            if key == "auto":
                rec["auto_picked_fp64"] = bool(st.auto_fp64)
        rec["fp32_fix_vs_fp64"] = metrics.compare(imgs["fp32_fix"], imgs["fp64"])
        if rec["auto_picked_fp64"]:
            rec["auto_vs_fp64_identical"] = bool(all(np.array_equal(getattr(imgs["auto"], k), getattr(imgs["fp64"], k))
                                                     for k in ("image_float", "zbuffer", "hit")))
        if cpu_seconds > 0 and name != "deep_zoom_1024":
            # the CPU implementation of the path on this configuration (the reference's
            # pthreads path restated: -O3 -ffast-math, rand() jitter, every host thread)
            v, desc = cpu_sample(sc, cpu_seconds)
            rec["cpu_reference"] = {"value": v, "unit": "Mpix/s", "cores": desc["threads"], "kind": "port",
                                    "sample": f"{desc['rows']} rows spread evenly over the frame, "
                                              f"{desc['seconds']:.1f} s"}
        out[name] = rec
    return out


def run_once(args) -> int:
    """One frame of the workload at a small size (plus `--warmup` frames): the ncu profiling case."""
    import mandelbulber_gb300 as mb
    from mandelbulber_gb300 import workloads as W
    w, h = (int(v) for v in args.once.lower().split("x"))
    if args.fixture:
        # a committed render fixture's scene (an effect scene) at this size
        z = np.load(os.path.join(ROOT, "tests", "golden", f"render_{args.fixture}.npz"))
        scene = mb.scene_from_bytes(z["scene"].tobytes())
        scene.image_width, scene.image_height = w, h
        scene.resolution = 1.0 / w / scene.noOfTiles
    else:
        scene = W.workload(args.workload, w, h)
    prec = mb.PREC_FP64 if args.precision == "fp64" else mb.PREC_FP32_FIX
    engine = mb.ENGINE_PER_PIXEL if args.engine == "per_pixel" else mb.ENGINE_WAVEFRONT
    with mb.Context(0) as ctx:
        for _ in range(args.warmup + 1):
            img = ctx.render(scene, precision=prec, engine=engine, pair_rays=int(args.pair_rays),
                             hit_order=args.hit_order)
        st = ctx.stats()
    print(json.dumps({"workload": args.fixture or args.workload, "size": [w, h], "precision": args.precision,
                      "engine": args.engine,
                      "kernel_ms": st.kernel_ms, "orbit_iterations": st.orbit_iterations, "de_calls": st.de_calls,
                      "hit_fraction": float(img.hit.mean())}))
    return 0


def run_peaks(args) -> int:
    """The ALU microbenchmarks of libmbgb_peak.so, twice each: FP32 / packed FP32 (f32x2) /
    FP64 FMA chains (TFLOP/s) and the lean Mandelbox iteration alone, scalar and two orbits
    per thread with packed FMAs (T iterations/s). The profiling case of those loops."""
    import mandelbulber_gb300 as mb
    mb.library(build_if_missing=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "mandelbulber_gb300", "libmbgb_peak.so"))
    for fn in ("mbgb_peak_tflops", "mbgb_box_orbit_rate", "mbgb_box_orbit_rate_x2"):
        getattr(lib, fn).restype = ctypes.c_double
    out = {"mode": "peaks"}
    for rep in range(2):
        out[f"rep{rep}"] = {"fp32_fma_tflops": lib.mbgb_peak_tflops(0, 0), "fp32x2_fma_tflops": lib.mbgb_peak_tflops(2, 0),
                            "fp64_fma_tflops": lib.mbgb_peak_tflops(1, 0),
                            "box_orbit_titer_per_s": lib.mbgb_box_orbit_rate(0),
                            "box_orbit_x2_titer_per_s": lib.mbgb_box_orbit_rate_x2(0)}
    print(json.dumps(out))
    return 0


def run_noise_floor(args) -> int:
    """The reference's run-to-run noise floor on the Mandelbulb configuration (640x480): the
    CPU implementation with the reference's shipped step jitter (Random() over the shared
    rand() stream, src/Render3D.cpp:129-133, src/common_math.cpp:25-32) rendered with one
    thread and with every host thread, and the two frames compared. The shared stream hands
    its numbers to whichever thread asks next, so the jitter each pixel sees depends on the
    thread count. Also each against the deterministic (jitter-off) strict FP64 oracle."""
    import mandelbulber_gb300 as mb  # noqa: F401  (CImage for the oracle's layers)
    from mandelbulber_gb300 import workloads as W
    from tests import metrics, oracle_lib
    lib = oracle_lib.load(fast=True)
    sc = W.workload("mandelbulb_640x480")
    threads = os.cpu_count() or 1
    out = {"mode": "noise_floor", "workload": "mandelbulb_640x480", "threads": [1, threads]}
    imgs = {}
    for t in (1, threads):
        t0 = time.perf_counter()
        imgs[t], _ = oracle_lib.render(lib, sc, jitter=True, threads=t)
        out[f"seconds_{t}_threads"] = time.perf_counter() - t0
    strict, _ = oracle_lib.render(oracle_lib.load(), sc, jitter=False, threads=threads)
    out["jitter_1_vs_all_threads"] = metrics.compare(imgs[1], imgs[threads])
    out["jitter_all_threads_vs_no_jitter"] = metrics.compare(imgs[threads], strict)
    print(json.dumps(out))
    return 0


def make_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-frame flight batch")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--no-grad", action="store_true", help="skip the gradient workload")
    ap.add_argument("--no-coverage", action="store_true", help="skip the other formulas / effects scenes")
    ap.add_argument("--no-configs", action="store_true", help="skip config 1 (Mandelbulb 640x480) and the deep zoom")
    ap.add_argument("--grad-steps", type=int, default=5)
    ap.add_argument("--once", default=None, metavar="WxH",
                    help="render the workload once at this size (warm-up frames first) and exit: the profiling case")
    ap.add_argument("--precision", default="fp32_fix", choices=["fp32_fix", "fp64"])
    ap.add_argument("--pair-rays", action="store_true",
                    help="with --once: the lean Mandelbox's shadow/AO rays two per thread (secondary_pair_kernel)")
    ap.add_argument("--peaks", action="store_true", help="run the ALU peak and orbit-loop microbenchmarks and exit")
    ap.add_argument("--noise-floor", action="store_true",
                    help="measure the reference's jitter noise floor on the Mandelbulb configuration (CPU) and exit")
    ap.add_argument("--hit-order", type=int, default=0, choices=[0, 1, 2],
                    help="with --once: opts.hit_order (0 automatic, 1 completion order, 2 tile order)")
    ap.add_argument("--fixture", default=None, metavar="NAME",
                    help="with --once: the scene of tests/golden/render_NAME.npz (effect scenes) instead of --workload")
    ap.add_argument("--engine", default="wavefront", choices=["wavefront", "per_pixel"],
                    help="with --once: the render engine of the profiling case")
    return ap


def main() -> int:
    args = make_parser().parse_args()
    args.warmup = max(args.warmup, 3)

    rank, world, local = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.once:
        return run_once(args)
    if args.noise_floor:
        return run_noise_floor(args)
    if args.peaks:
        return run_peaks(args)

    import torch
    import mandelbulber_gb300 as mb
    from mandelbulber_gb300 import workloads as W

    mb.library(build_if_missing=True)
    dev = local
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    scene = W.workload(args.workload)
    w, h = scene.image_width, scene.image_height
    npx = w * h
    ctx = mb.Context(dev)
    stream = torch.cuda.Stream(device=dev)

    def layers_dev():
        return {
            "image_float": torch.empty(npx * 3, dtype=torch.float32, device=dev),
            "zbuffer": torch.empty(npx, dtype=torch.float32, device=dev),
            "alpha": torch.empty(npx, dtype=torch.int16, device=dev),
            "opacity": torch.empty(npx, dtype=torch.int16, device=dev),
            "colour": torch.empty(npx * 3, dtype=torch.uint8, device=dev),
        }

    L = layers_dev()
    ptrs = {k: v.data_ptr() for k, v in L.items()}
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def timed_frames(precision, steps, warmup, **opts):
        for _ in range(warmup):
            ctx.render_device(scene, ptrs, precision=precision, stream=stream.cuda_stream, **opts)
        stream.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        t_wall = time.perf_counter()
        for e0, e1 in evs:
            with torch.cuda.stream(stream):
                flush.zero_()                      # L2 flush between timed frames (512 MiB > 129 MB L2)
                e0.record(stream)
            ctx.render_device(scene, ptrs, precision=precision, stream=stream.cuda_stream, **opts)
            e1.record(stream)
        stream.synchronize()
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t_wall
        ms = [a.elapsed_time(b) for a, b in evs]
        total = sum(ms) / 1e3
        return max_over_ranks(total, dist, dev), ms, wall

    # counters of one frame (deterministic: jitter off) for the roofline
    ctx.render_device(scene, ptrs, precision=mb.PREC_FP32_FIX)
    st32 = ctx.stats()
    with ClockSampler(dev) as clk:
        total32, ms32, wall32 = timed_frames(mb.PREC_FP32_FIX, args.steps, args.warmup)
    clocks = clk.summary()
    ctx.render_device(scene, ptrs, precision=mb.PREC_FP64)
    st64 = ctx.stats()
    total64, ms64, _ = timed_frames(mb.PREC_FP64, args.fp64_steps, 1)

    value = whole_job_rate(world, npx, args.steps, total32) / 1e6
    value64 = whole_job_rate(world, npx, args.fp64_steps, total64) / 1e6

    # parity of the two policies at full size (hit mask, PSNR of the float image)
    from tests import metrics
    a = ctx.render(scene, precision=mb.PREC_FP32_FIX)
    b = ctx.render(scene, precision=mb.PREC_FP64)
    parity = metrics.compare(a, b)

    # the same policy with every hit's bisection finished in FP64 (polish_all), beside the
    # headline's selective polish of the hits that stopped early near a window edge
    pa_steps = max(3, args.steps // 4)
    total_pa, _, _ = timed_frames(mb.PREC_FP32_FIX, pa_steps, 1, polish_all=True)
    ctx.render_device(scene, ptrs, precision=mb.PREC_FP32_FIX, polish_all=True)
    st_pa = ctx.stats()
    polish_all = {"value": whole_job_rate(world, npx, pa_steps, total_pa) / 1e6, "unit": "Mpix/s",
                  "ms_per_step": 1e3 * total_pa / pa_steps, "steps": pa_steps,
                  "fp64_polished_hits": int(st_pa.fp64_polished),
                  "parity_vs_fp64": metrics.compare(ctx.render(scene, precision=mb.PREC_FP32_FIX, polish_all=True), b)}

    # the allocation-free entry point (static scratch, per-pixel engine) on the same frame
    lib = mb.library()
    na_img = mb.mbgb_image(w, h, *[ctypes.c_void_p(ptrs[n]) for n in ("image_float", "zbuffer", "alpha",
                                                                         "opacity", "colour")], None, None, None)
    na_opts = mb.make_opts(precision=mb.PREC_FP32_FIX, stream=stream.cuda_stream)
    for _ in range(2):
        assert lib.mbgb_render_device_noalloc(ctypes.byref(scene), ctypes.byref(na_img), ctypes.byref(na_opts)) == 0, \
            lib.mbgb_last_error()
    na_steps = max(3, args.steps // 4)
    na_evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(na_steps)]
    stream.synchronize()
    for e0, e1 in na_evs:
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
        lib.mbgb_render_device_noalloc(ctypes.byref(scene), ctypes.byref(na_img), ctypes.byref(na_opts))
        e1.record(stream)
    stream.synchronize()
    na_ms = sum(a.elapsed_time(b_) for a, b_ in na_evs) / na_steps
    noalloc = {"value": npx / (na_ms * 1e3), "unit": "Mpix/s", "ms_per_step": na_ms, "steps": na_steps,
               "engine": "per-pixel (one pixel per thread), 96-thread CTAs, two per SM, 134 step records per "
                         "slot in static device arrays"}

    # end to end through the public host entry point: pinned host layers, copies inside the timed region
    host = mb.CImage.empty(w, h)
    pinned = {}
    for name in ("image_float", "zbuffer", "alpha", "opacity", "colour"):
        arr = getattr(host, name)
        t = torch.empty(arr.shape, dtype={np.float32: torch.float32, np.uint16: torch.int16,
                                          np.uint8: torch.uint8}[arr.dtype.type], pin_memory=True)
        pinned[name] = t
        setattr(host, name, t.numpy().view(arr.dtype))
    host.hit = host.iters = host.depth = None
    img_c = mb.mbgb_image(w, h, *[host.__dict__[n].ctypes.data_as(ctypes.c_void_p)
                                  for n in ("image_float", "zbuffer", "alpha", "opacity", "colour")],
                          None, None, None)
    opts = mb.make_opts(precision=mb.PREC_FP32_FIX)
    for _ in range(2):
        lib.mbgb_render_host(ctx._h, ctypes.byref(scene), ctypes.byref(img_c), ctypes.byref(opts))
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rc = lib.mbgb_render_host(ctx._h, ctypes.byref(scene), ctypes.byref(img_c), ctypes.byref(opts))
        e2e_t.append(time.perf_counter() - t0)
        assert rc == 0, lib.mbgb_last_error()
    e2e_value = world * npx * len(e2e_t) / sum(e2e_t) / 1e6
    d2h = npx * (12 + 4 + 2 + 2 + 3)

    # roofline of the dominant kernel: ALU bound. The library records CUDA events between
    # its stage launches on the launching stream (profile_stages); each stage's algorithmic
    # work comes from its own orbit/DE counters.
    peak_lib = ctypes.CDLL(os.path.join(ROOT, "mandelbulber_gb300", "libmbgb_peak.so"))
    peak_lib.mbgb_peak_tflops.restype = ctypes.c_double
    peak32 = peak_lib.mbgb_peak_tflops(0, dev)
    peak64 = peak_lib.mbgb_peak_tflops(1, dev)
    peak_lib.mbgb_box_orbit_rate.restype = ctypes.c_double
    # the lean Mandelbox iteration alone (every lane busy, no ray bookkeeping): the ceiling
    # this instruction mix allows, against which the dominant kernel's orbit rate is read
    loop_rate = peak_lib.mbgb_box_orbit_rate(dev) if scene.formula == 8 else -1.0
    f = scene.formula
    stage_names = ["primary_kernel", "polish_kernel", "secondary_kernel", "compose_kernel"]

    def stage_profile(precision, frames):
        acc = np.zeros(4)
        for _ in range(frames):
            ctx.render_device(scene, ptrs, precision=precision, profile_stages=True)
            st = ctx.stats()
            acc += np.array(list(st.stage_ms)[:4])
        acc /= frames
        work = [st.stage_orbit[k] * FLOPS_PER_ITER[f] + st.stage_de[k] * FLOPS_PER_DE[f] for k in range(4)]
        stages = {stage_names[k]: {"ms": float(acc[k]), "flops": int(work[k]), "orbit_iterations": int(st.stage_orbit[k]),
                                   "de_evaluations": int(st.stage_de[k])} for k in range(4)}
        top = max(range(4), key=lambda k: acc[k])
        return stages, stage_names[top], work[top], acc[top] / 1e3

    stages32, top32, work32, sec32 = stage_profile(mb.PREC_FP32_FIX, args.steps)
    stages64, top64, work64, sec64 = stage_profile(mb.PREC_FP64, 1)
    flops32 = st32.orbit_iterations * FLOPS_PER_ITER[f] + st32.de_calls * FLOPS_PER_DE[f]
    ach32 = work32 / sec32 / 1e12
    ach64 = work64 / sec64 / 1e12
    traffic = DRAM_BYTES_PER_LAUNCH.get(args.workload) if top32 == "secondary_kernel" else None

    # launches of one timed frame (the library counts the kernels it enqueues)
    ctx.render_device(scene, ptrs, precision=mb.PREC_FP32_FIX)
    launches_per_frame = int(ctx.stats().launches)

    batch = None if args.no_batch else batch_section(ctx, torch, dev, stream, flush, args, world, dist)
    coverage = None if args.no_coverage else coverage_section(ctx)
    configs = None if args.no_configs else configs_section(ctx, 0.0 if (args.no_cpu or rank != 0 or world > 1)
                                                               else args.cpu_seconds / 2)
    grads = None if args.no_grad else grad_section(ctx, torch, dev, args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, desc = cpu_sample(scene, args.cpu_seconds)
        cpu = {"value": v, "unit": "Mpix/s", "cores": desc["threads"], "kind": "port",
               "sample": (f"{desc['rows']} rows spread evenly over the {w}x{h} frame ({desc['pixels']} px, "
                          f"{desc['seconds']:.1f} s), CPU oracle restatement built with the reference flags "
                          f"-O3 -ffast-math, rand() step jitter, {desc['threads']} host threads")}

    line = {
        "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total32 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": bench_config(args.workload, world),
        "roofline": {"kernel": top32, "bound": "fp32_alu", "achieved": ach32, "peak": peak32, "unit": "TFLOP/s",
                     "frac": ach32 / peak32 if peak32 > 0 else None, "traffic": traffic,
                     "peak_source": "measured live: FP32 FMA-chain microbenchmark (libmbgb_peak.so)",
                     "flops_per_launch": int(work32),
                     "frame_flops": int(flops32),
                     "frame_achieved": flops32 / (total32 / args.steps) / 1e12,
                     "work": f"{FLOPS_PER_ITER[f]} FP ops per orbit iteration + {FLOPS_PER_DE[f]} per DE evaluation",
                     "orbit_loop_ceiling": None if loop_rate <= 0 else {
                         "iterations_per_s": loop_rate * 1e12,
                         "tflops": loop_rate * FLOPS_PER_ITER[f],
                         "kernel_iterations_per_s": stages32[top32]["orbit_iterations"] / sec32,
                         "frac": stages32[top32]["orbit_iterations"] / sec32 / (loop_rate * 1e12),
                         "what": "the lean Mandelbox iteration alone on bounded orbits (libmbgb_peak.so): "
                                 "the issue-bound ceiling of this instruction mix"}},
        "stages": stages32,
        "fp64_polished_hits": int(st32.fp64_polished),
        "fp64_plain": {"value": value64, "unit": "Mpix/s", "ms_per_step": 1e3 * total64 / args.fp64_steps,
                       "steps": args.fp64_steps, "stages": stages64,
                       "roofline": {"kernel": top64, "bound": "fp64_alu", "achieved": ach64, "peak": peak64,
                                    "unit": "TFLOP/s", "frac": ach64 / peak64 if peak64 > 0 else None}},
        "ratio_vs_fp64": value / value64,
        "polish_all": polish_all,
        "noalloc": noalloc,
        "parity_vs_fp64": parity,
        "e2e": {"value": e2e_value, "unit": "Mpix/s", "h2d_bytes_per_step": ctypes.sizeof(mb.mbgb_scene),
                "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps * launches_per_frame,
        "batch": batch,
        "grads": grads,
        "coverage": coverage,
        "configs": configs,
        "clocks": clocks,
        "cpu_baseline": cpu,
        "wall_s_timed_region": wall32,
    }
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
