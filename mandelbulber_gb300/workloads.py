"""Scenes of the benchmark workloads, built from settings keys.

Each workload is a dictionary of .fract keys (the names LoadOneSetting reads,
src/settings.cpp:700-1183) applied to a zeroed scene, followed by the palette
rule of LoadSettingsPost (src/settings.cpp:1185-1195) and the -nogui fix-ups.
The values not named by a workload are the hot-path entries of the
reference's default parameter set.

  mandelbulb_640x480    Mandelbulb power 8 (trig_optim, formula 2), N 250, 640x480,
                        camera (0,-3.5,0) looking +y, 53 deg horizontal FOV, DE factor 1,
                        threshold = 1 pixel footprint, light at 45/45 deg, hard shadows,
                        no AO / fog / glow.
  mandelbox_1080p       Mandelbox scale 2 (tglad, formula 8), fold limit 1 / value 2,
                        sphere fold 0.5 / 1.0, N 15 (bailout 1024), 1920x1080, camera
                        (0,-20,0) looking +y (the scale-2 box spans |y| <= 6, so a camera
                        at distance 6 would sit on its face), 53 deg FOV, hard shadows,
                        ray-traced AO (quality 2:
                        29 directions), volumetric fog density 0.5 over the primary
                        step buffer, glow on.
  flight()              64-frame flight around the Mandelbulb, per-frame resolutions from
                        320x240 to 1920x1080, hard shadows + fast AO (quality 4).
  deep_zoom()           Mandelbulb N 1000 at 1024x1024 with the camera 1e-6 from the surface.
"""
from __future__ import annotations

import math

from . import finalize, mbgb_scene, palette_from_seed, scene_set

# hot-path entries of the reference's default parameter set
BASE = {
    "image_width": 800, "image_height": 600, "tiles": 1,
    "x_min": -10, "x_max": 10, "y_min": -10, "y_max": 10, "z_min": -10, "z_max": 10,
    "view_point_x": 0, "view_point_y": 0, "view_point_z": 0,
    "angle_alfa": 0, "angle_beta": 0, "angle_gamma": 0,
    "zoom": 1e-15, "perspective": 0.5, "formula": 2, "power": 8, "N": 250, "minN": 1,
    "fractal_constant_factor": 1, "quality": 1, "smoothness": 1,
    "julia_mode": 0, "tglad_folding_mode": 0, "folding_limit": 1, "folding_value": 2,
    "spherical_folding_mode": 0, "spherical_folding_fixed": 1, "spherical_folding_min": 0.5,
    "IFS_folding_mode": 0, "iteration_threshold_mode": 0, "analityc_DE_mode": 1, "DE_factor": 1,
    "brightness": 1, "contrast": 1, "gamma": 1, "ambient": 0, "reflect": 0, "shadows_intensity": 0.7,
    "ambient_occlusion": 1, "ambient_occlusion_quality": 4, "ambient_occlusion_fast_tune": 1,
    "shading": 1, "specular": 1, "glow_intensity": 1,
    "glow_color_1_R": 40984, "glow_color_1_G": 44713, "glow_color_1_B": 49490,
    "glow_color_2_R": 57192, "glow_color_2_G": 60888, "glow_color_2_B": 62408,
    "background_color_1_R": 0, "background_color_1_G": 38306, "background_color_1_B": 65535,
    "background_color_2_R": 65535, "background_color_2_G": 65535, "background_color_2_B": 65535,
    "background_color_3_R": 0, "background_color_3_G": 10000, "background_color_3_B": 500,
    "fog_colour_1_R": 0, "fog_colour_1_G": 0, "fog_colour_1_B": 0,
    "fog_colour_2_R": 0, "fog_colour_2_G": 30000, "fog_colour_2_B": 65535,
    "fog_colour_3_R": 65535, "fog_colour_3_G": 65535, "fog_colour_3_B": 65535,
    "textured_background": 0, "shadows_enabled": 1, "ambient_occlusion_enabled": 0,
    "fast_ambient_occlusion_mode": 0, "fractal_color": 1, "coloring_random_seed": 123456,
    "coloring_saturation": 1, "coloring_speed": 1, "coloring_palette_offset": 0, "slow_shading": 0,
    "limits_enabled": 0, "post_fog_enabled": 0, "post_fog_visibility": 20,
    "post_fog_color_R": 59399, "post_fog_color_G": 61202, "post_fog_color_B": 65535,
    "post_SSAO_enabled": 0, "post_SSAO_quality": 20, "post_DOF_enabled": 0,
    "main_light_intensity": 1, "main_light_alfa": -0.78539816339744828, "main_light_beta": 0.78539816339744828,
    "main_light_colour_R": 65535, "main_light_colour_G": 65535, "main_light_colour_B": 65535,
    "aux_light_number": 0, "aux_light_visibility": 1,
    "mandelbox_scale": 2, "mandelbox_folding_limit": 1, "mandelbox_folding_value": 2,
    "mandelbox_folding_min_radius": 0.5, "mandelbox_folding_fixed_radius": 1,
    "mandelbox_color_R": 0, "mandelbox_color_X": 0.03, "mandelbox_color_Y": 0.05, "mandelbox_color_Z": 0.07,
    "mandelbox_color_Sp1": 0.2, "mandelbox_color_Sp2": 0.2, "mandelbox_rotation_enabled": 0,
    "view_distance_max": 50, "view_distance_min": 1e-15, "interior_mode": 0, "linear_DE_mode": 0,
    "constant_DE_threshold": 0, "penetrating_lights": 1, "raytraced_reflections": 0, "reflections_max": 5,
    "volumetric_fog_density": 0, "volumetric_fog_colour_1_distance": 1, "volumetric_fog_colour_2_distance": 2,
    "volumetric_fog_distance_factor": 1, "iteration_fog_enable": 0, "fish_eye": 0,
}


def fov_persp(width: int, height: int, fov_deg: float = 53.0) -> float:
    """The reference's perspective factor for a horizontal field of view.

    The view vector is (x2 * persp, 1, z2 * persp) with x2 in [-aspect/2, aspect/2)
    (src/Render3D.cpp:391-438), so tan(fov/2) = persp * aspect / 2.
    """
    return 2.0 * math.tan(math.radians(fov_deg / 2.0)) / (width / height)


MANDELBULB_640x480 = {
    "image_width": 640, "image_height": 480, "formula": 2, "power": 8, "N": 250,
    "view_point_x": 0, "view_point_y": -3.5, "view_point_z": 0,
    "perspective": fov_persp(640, 480), "DE_factor": 1, "quality": 1,
    "main_light_alfa": math.radians(45.0), "main_light_beta": math.radians(45.0),
    "shadows_enabled": 1, "shadows_cone_angle": 0, "penetrating_lights": 0,
    "ambient_occlusion_enabled": 0, "volumetric_fog_density": 0, "glow_intensity": 0,
    "post_SSAO_enabled": 0, "fractal_color": 1,
}

MANDELBOX_1080P = {
    "image_width": 1920, "image_height": 1080, "formula": 8, "N": 15,
    "mandelbox_scale": 2.0, "mandelbox_folding_limit": 1.0, "mandelbox_folding_value": 2.0,
    "mandelbox_folding_min_radius": 0.5, "mandelbox_folding_fixed_radius": 1.0,
    "view_point_x": 0, "view_point_y": -20.0, "view_point_z": 0,
    "perspective": fov_persp(1920, 1080), "DE_factor": 1, "quality": 1,
    "main_light_alfa": math.radians(45.0), "main_light_beta": math.radians(45.0),
    "shadows_enabled": 1, "shadows_cone_angle": 0, "penetrating_lights": 0,
    "ambient_occlusion_enabled": 1, "fast_ambient_occlusion_mode": 0, "ambient_occlusion_quality": 2,
    "volumetric_fog_density": 0.5, "glow_intensity": 1, "post_SSAO_enabled": 0, "fractal_color": 1,
}

WORKLOADS = {"mandelbulb_640x480": MANDELBULB_640x480, "mandelbox_1080p": MANDELBOX_1080P}

# mandelboxVaryScale4D's own parameters at the values of the reference's default settings
# (src/settings.cpp:413-417); the
# other formulas ignore them, so the base scenes keep them at zero
# Auxiliary-light settings at the reference's default values (share/defaults); the
# benchmark scenes light with the main light only
AUX_LIGHTS = {"aux_light_intensity": 1, "aux_light_random_seed": 1234, "aux_light_max_dist": 0.1,
              "aux_light_distribution_radius": 3,
              "aux_light_predefined_1_colour_R": 45761, "aux_light_predefined_1_colour_G": 53633,
              "aux_light_predefined_1_colour_B": 59498, "aux_light_predefined_2_colour_R": 62875,
              "aux_light_predefined_2_colour_G": 55818, "aux_light_predefined_2_colour_B": 50083,
              "aux_light_predefined_3_colour_R": 64884, "aux_light_predefined_3_colour_G": 64928,
              "aux_light_predefined_3_colour_B": 48848, "aux_light_predefined_4_colour_R": 52704,
              "aux_light_predefined_4_colour_G": 62492, "aux_light_predefined_4_colour_B": 45654}

VARY4D = {"formula": 18, "mandelbox_vary_scale_vary": 0.1, "mandelbox_vary_fold": 1,
          "mandelbox_vary_minr": 0.5, "mandelbox_vary_rpower": 1, "mandelbox_vary_wadd": 0}


def look_angles(d) -> tuple[float, float]:
    """Camera angles (degrees) that look along direction d.

    MainThread's view vector for the centre pixel is RotZ(alpha) RotX(beta) (0, 1, 0)
    = (-sin a cos b, cos a cos b, sin b) (src/Render3D.cpp:237-240, src/algebra.cpp:94-143).
    """
    import numpy as np
    d = np.asarray(d, float) / np.linalg.norm(d)
    return math.degrees(math.atan2(-d[0], d[1])), math.degrees(math.asin(d[2]))


def deep_zoom(ctx, size: int = 1024, seed: int = 5, N: int = 1000, **extra) -> mbgb_scene:
    """Deep-zoom Mandelbulb (power 8, N 1000): the camera sits 1e-6 before a surface point.

    A seeded direction from (0,-3.5,0) (within 15 deg of the bulb's centre) is sphere-traced
    with the device's FP64 distance estimate until the distance is below 1e-12; the camera
    is placed 1e-6 back along the ray, looking at the point, and the perspective factor is
    chosen so that the footprint scan * persp / width at scan = 1e-6 is 10**U(-9, -7).
    """
    import numpy as np
    import torch
    rng = np.random.default_rng(seed)
    origin = np.array([0.0, -3.5, 0.0])
    base = make_scene({**MANDELBULB_640x480, "N": N, "image_width": size, "image_height": size})
    pts = torch.zeros(3, dtype=torch.float64, device="cuda")
    det = torch.full((1,), 1e-13, dtype=torch.float64, device="cuda")
    dist = torch.zeros(1, dtype=torch.float64, device="cuda")
    it = torch.zeros(1, dtype=torch.int32, device="cuda")
    mi = torch.zeros(1, dtype=torch.uint8, device="cuda")
    from . import PREC_FP64
    while True:
        d = np.array([0.0, 1.0, 0.0]) + rng.normal(0.0, 0.15, 3)
        d /= np.linalg.norm(d)
        t, hit = 0.0, False
        for _ in range(20000):
            p = origin + d * t
            pts.copy_(torch.tensor(p, dtype=torch.float64))
            ctx.distance(base, pts.data_ptr(), det.data_ptr(), 1, dist.data_ptr(), it.data_ptr(), mi.data_ptr(),
                         PREC_FP64)
            de = float(dist.item())
            if de < 1e-12:
                hit = True
                break
            t += de
            if t > 10.0:
                break
        if hit:
            break
    footprint = 10.0 ** rng.uniform(-9.0, -7.0)
    cam = origin + d * (t - 1e-6)
    a, b = look_angles(d)
    keys = {**MANDELBULB_640x480, "N": N, "image_width": size, "image_height": size,
            "view_point_x": cam[0], "view_point_y": cam[1], "view_point_z": cam[2],
            "angle_alfa": a, "angle_beta": b, "perspective": footprint * size / 1e-6,
            "view_distance_min": 1e-15, "zoom": 1e-15}
    keys.update(extra)
    return make_scene(keys)


FLIGHT_RESOLUTIONS = ((320, 240), (640, 480), (1280, 720), (1920, 1080))


def flight(n_keys: int = 8, frames_per_key: int = 8, seed: int = 3, res_seed: int = 4, downscale: int = 1,
           **extra) -> list:
    """Flight animation around the power-8 Mandelbulb: n_keys x frames_per_key frames.

    Keyframe camera positions are seeded (`seed`): a direction uniform on the sphere and a
    radius r = cbrt(U (4^3 - 2^3) + 2^3), uniform in the volume of the shell 2 <= r <= 4.
    Frames follow the keyframes with the reference's Catmull-Rom spline (mbgb_scene_interpolate);
    every frame then looks at the origin from its interpolated position. Each frame's
    resolution is drawn (`res_seed`) uniformly from FLIGHT_RESOLUTIONS (divided by
    `downscale`), with a 53 deg horizontal FOV. Hard shadows and fast AO (quality 4:
    15 samples along the normal).
    """
    import numpy as np
    from . import interpolate
    rng = np.random.default_rng(seed)
    scene_keys = {**MANDELBULB_640x480, "ambient_occlusion_enabled": 1, "fast_ambient_occlusion_mode": 1,
                  "ambient_occlusion_quality": 4}
    scene_keys.update(extra)
    keys = []
    for _ in range(n_keys):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        r = (rng.uniform() * (4.0 ** 3 - 2.0 ** 3) + 2.0 ** 3) ** (1.0 / 3.0)
        pos = d * r
        a, b = look_angles(-pos)
        keys.append(make_scene({**scene_keys, "view_point_x": pos[0], "view_point_y": pos[1],
                                "view_point_z": pos[2], "angle_alfa": a, "angle_beta": b}))
    sizes = np.random.default_rng(res_seed).integers(0, len(FLIGHT_RESOLUTIONS), size=n_keys * frames_per_key)
    frames = []
    for f in range(n_keys * frames_per_key):
        sc = interpolate(keys, frames_per_key, f)
        w, h = FLIGHT_RESOLUTIONS[int(sizes[f])]
        w, h = w // downscale, h // downscale
        a, b = look_angles(-np.array([sc.vp[0], sc.vp[1], sc.vp[2]]))
        for k, v in (("image_width", w), ("image_height", h), ("perspective", repr(fov_persp(w, h))),
                     ("angle_alfa", repr(a)), ("angle_beta", repr(b))):
            scene_set(sc, k, v)
        frames.append(finalize(sc))
    return frames


def make_scene(overrides: dict, base: dict | None = None) -> mbgb_scene:
    """A finalized scene from BASE updated with `overrides` (keys as in .fract files)."""
    keys = dict(BASE if base is None else base)
    keys.update(overrides)
    s = mbgb_scene()
    for k, v in keys.items():
        scene_set(s, k, repr(float(v)) if isinstance(v, float) else v)
    pal = palette_from_seed(int(keys["coloring_random_seed"]), float(keys["coloring_saturation"]))
    for i in range(256):
        s.palette[i].R, s.palette[i].G, s.palette[i].B = (int(c) for c in pal[i])
    s.paletteLoaded = 0
    return finalize(s)


def workload(name: str, width: int | None = None, height: int | None = None, **extra) -> mbgb_scene:
    """A named workload, optionally at another resolution (FOV kept) or with extra keys."""
    keys = dict(WORKLOADS[name])
    if width and height:
        keys["image_width"], keys["image_height"] = width, height
        keys["perspective"] = fov_persp(width, height)
    keys.update(extra)
    return make_scene(keys)
