"""Generates the golden vectors under tests/golden/ from the reference's OWN code.

Runs in a container that has the reference tree: builds oracle/_ref/libmbref.so
(the reference's src/fractal.cpp, src/shaders.cpp, src/algebra.cpp,
src/common_math.cpp, src/primitives.cpp compiled in place, plus
oracle/ref_harness.cpp) and records, for seeded inputs:
  * de_<formula>.npz      CalculateDistance (distance, itersOut, max_iter) and the
                          Compute<colouring> value SurfaceColour uses, at seeded points;
  * render_<case>.npz     every cImage layer of the MainThread pixel body (jitter off)
                          for small frames covering the shading features;
  * post_<case>.npz       CompileImage (src/cimage.cpp:183-214) and PostRendering_SSAO
                          (src/image.cpp:249-478) of the reference (oracle/_ref/libmbref_post.so)
                          applied to render fixtures, for several image adjustments.
Each file also stores the scene as raw mbgb_scene bytes and its settings keys, so
the tests rebuild the exact input without the reference tree.

    python tests/golden/make_golden.py          # everything
    python tests/golden/make_golden.py post     # the post-processing fixtures only
    python tests/golden/make_golden.py formulas # the trig_DE / menger / vary4D fixtures only
    python tests/golden/make_golden.py all_formulas # every other formula: DE fixtures, example
                                                # scenes (share/examples) and synthetic scenes
    python tests/golden/make_golden.py settings # every shipped settings file as the reference
                                                # reads it, and the bench workloads' scenes

Every scene is read by the reference's own settings code (src/settings.cpp compiled in
place into oracle/_ref/libmbref_settings.so) and the -nogui derivations, never by this
library's reader: the parity tests then inherit nothing from the library's parsing. The reference tree
is found through oracle/Makefile (MBGB_REF_TREE).
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import mandelbulber_gb300 as mb  # noqa: E402
from mandelbulber_gb300 import workloads as W  # noqa: E402
from tests import oracle_lib  # noqa: E402

# Small frames covering the hot-path features; the keys are applied on top of a workload.
CASES = {
    "mandelbulb_64x48": ("mandelbulb_640x480", 64, 48, {}),
    "mandelbox_96x54": ("mandelbox_1080p", 96, 54, {}),
    "mandelbulb_soft_penetrating": ("mandelbulb_640x480", 40, 32,
                                    {"shadows_cone_angle": 1.0, "penetrating_lights": 1, "glow_intensity": 1}),
    "mandelbulb_fastao_postfog": ("mandelbulb_640x480", 40, 32,
                                  {"ambient_occlusion_enabled": 1, "fast_ambient_occlusion_mode": 1,
                                   "ambient_occlusion_quality": 4, "post_fog_enabled": 1,
                                   "post_fog_visibility": 160}),
    "mandelbulb_rayao_q1": ("mandelbulb_640x480", 32, 32,
                            {"ambient_occlusion_enabled": 1, "fast_ambient_occlusion_mode": 0,
                             "ambient_occlusion_quality": 1}),
    "mandelbulb_julia_limits": ("mandelbulb_640x480", 40, 32,
                                {"julia_mode": 1, "julia_a": 0.2, "julia_b": -0.4, "julia_c": 0.1,
                                 "limits_enabled": 1, "z_max": 0.4}),
    "mandelbulb_power6_rotated": ("mandelbulb_640x480", 40, 32,
                                  {"power": 6, "angle_alfa": 30, "angle_beta": 19, "angle_gamma": 10,
                                   "view_point_x": 1.75, "view_point_y": -3.0, "view_point_z": -1.2}),
    "mandelbox_rotated_interior": ("mandelbox_1080p", 56, 32,
                                   {"mandelbox_rotation_enabled": 1, "mandelbox_rotation_X1_alfa": 10,
                                    "mandelbox_rotation_Y2_beta": -15, "mandelbox_rotation_main_gamma": 5,
                                    "ambient_occlusion_enabled": 0, "interior_mode": 0}),
    "mandelbulb_interior": ("mandelbulb_640x480", 32, 32,
                            {"interior_mode": 1, "view_point_y": -1.0, "N": 40, "glow_intensity": 1}),
    "mandelbox_fog_colours": ("mandelbox_1080p", 56, 32,
                              {"volumetric_fog_density": 2.0, "volumetric_fog_colour_1_distance": 0.3,
                               "volumetric_fog_colour_2_distance": 0.8, "volumetric_fog_distance_factor": 0.5,
                               "ambient_occlusion_enabled": 0}),
    "mandelbox_constant_threshold_minN": ("mandelbox_1080p", 48, 32,
                                          {"constant_DE_threshold": 1, "quality": 0.002, "minN": 3,
                                           "ambient_occlusion_enabled": 1, "fast_ambient_occlusion_mode": 1,
                                           "ambient_occlusion_quality": 3}),
    "mandelbulb_tiles_equirect": ("mandelbulb_640x480", 32, 32,
                                  {"tiles": 2, "tile_no": 3, "fish_eye": 2, "perspective": 0.8}),
    "mandelbulb_fisheye_cut": ("mandelbulb_640x480", 32, 32,
                               {"fish_eye": 1, "fish_eye_180cut": 1, "perspective": 1.2}),
    "mandelbulb_prefolds_iterthresh": ("mandelbulb_640x480", 32, 32,
                                       {"tglad_folding_mode": 1, "spherical_folding_mode": 1,
                                        "iteration_threshold_mode": 1, "N": 60}),
}

# formulas selected at run time on the device: trig_DE (1), menger_sponge (7),
# mandelboxVaryScale4D (18)
FORMULA_CASES = {
    "trigde_40x32": ("mandelbulb_640x480", 40, 32, {"formula": 1}),
    "trigde_power6_rotated": ("mandelbulb_640x480", 40, 32,
                              {"formula": 1, "power": 6, "angle_alfa": 30, "angle_beta": 19,
                               "view_point_x": 1.75, "view_point_y": -3.0, "view_point_z": -1.2}),
    "menger_48x32": ("mandelbulb_640x480", 48, 32, {"formula": 7, "N": 50, "view_point_x": 0.9,
                                                    "view_point_z": 0.6, "angle_alfa": -14, "angle_beta": -9}),
    "menger_glow_fastao": ("mandelbulb_640x480", 40, 32,
                           {"formula": 7, "N": 50, "glow_intensity": 1, "ambient_occlusion_enabled": 1,
                            "fast_ambient_occlusion_mode": 1, "ambient_occlusion_quality": 3}),
    "vary4d_48x32": ("mandelbox_1080p", 48, 32, {**W.VARY4D, "ambient_occlusion_enabled": 0,
                                                 "mandelbox_scale": 2.0}),
    "vary4d_rpower_wadd": ("mandelbox_1080p", 48, 32,
                           {**W.VARY4D, "ambient_occlusion_enabled": 0, "mandelbox_scale": 2.0,
                            "view_point_y": -17.0, "angle_alfa": 20, "mandelbox_vary_rpower": 0.8, "mandelbox_vary_wadd": 0.3,
                            "mandelbox_vary_scale_vary": 0.05, "volumetric_fog_density": 0}),
}
FORMULA_DE = (("trigde", "mandelbulb_640x480", {"formula": 1}, 1.6),
              ("menger", "mandelbulb_640x480", {"formula": 7, "N": 50}, 1.5),
              ("vary4d", "mandelbox_1080p", {**W.VARY4D, "mandelbox_scale": 2.0}, 4.0))


# Example scenes of the reference (share/examples/*.fract, read by the reference's own settings
# code after share/defaults) at 48 x 32 with SSAO off; a few get one feature switched off
# that the library does not render (the override is recorded in the fixture). The fixture
# stores the loaded scene as bytes, so the tests need neither the reference tree nor the files.
EXAMPLES = {
    "ifs_sierpinski": ("IFS Sierpinski.fract", {}),
    "ifs_icosahedron": ("IFS Icosahedron.fract", {}),
    "ifs_dodecahedron": ("IFS Dodecahedron.fract", {}),
    "ifs_trees": ("IFS Trees.fract", {}),
    "hybrid_1": ("Hybrid 1.fract", {}),
    "hybrid_3": ("Hybrid 3.fract", {}),
    "hybrid_4": ("Hybrid 4.fract", {}),
    "hybrid_foldintpow2": ("FoldIntPow2 2.fract", {"raytraced_reflections": 0, "reflect": 0}),
    "modified_mandelbulb_1": ("modified mandelbulb 1.fract", {}),
    "modified_mandelbulb_2": ("modified mandelbulb 2.fract", {}),
    "modified_mandelbulb_3": ("modified mandelbulb 3.fract", {}),
    "power2_default": ("power 2 - default.fract", {}),
    "power2_limits": ("power 2 - limits.fract", {}),
    "quaternion_lathe": ("quaternion - lathe.fract", {}),
    "xenodreambuie": ("xenodreambuie's formula.fract", {}),
    "hypercomplex_ao": ("hypercomplex - ambient occlusion.fract", {"slow_shading": 0}),
    "spherical_folding_menger": ("spherical folding - menger sponge.fract", {}),
    "folded_trigonometric": ("Folded trigonometric power 8.fract", {}),
    "rotated_mandelbox_1": ("rotated mandelbox 1.fract", {}),
    "stereo_hybrid": ("stereo.fract", {}),
    # auxiliary lights: random (PlaceRandomLights), predefined, visible in the volumetric pass
    "aux_backlight": ("Mandelbulb with backlight.fract", {}),
    "aux_menger_predefined": ("menger sponge.fract", {}),
    "aux_menger_1000_lights": ("menger sponge 3.fract", {}, 32, 24),
    "aux_rotated_mandelbox_4": ("rotated mandelbox 4.fract", {}),
    "aux_coloured_lights": ("tglad - scale 2 - coloured lights.fract", {}),
    # slow shading (averaged normals), iteration fog, volumetric lights, environment mapping
    "fx_slow_hypercomplex_ao": ("hypercomplex - ambient occlusion.fract", {}, 32, 24),
    "fx_slow_interior_mandelbox": ("interior - mandelbox scale 2.fract", {}, 32, 24),
    "fx_slow_interior_power8": ("interior - mandelbulb power 8.fract", {}, 32, 24),
    "fx_iter_fog_1": ("iter fog 1.fract", {}, 32, 24),
    "fx_iter_fog_2": ("iter fog 2.fract", {}, 32, 24),
    "fx_iter_fog_3": ("iter fog 3.fract", {}, 32, 24),
    "fx_iter_fog_4": ("iter fog 4.fract", {}, 32, 24),
    "fx_volumetric_light_1": ("Volumetric light 1.fract", {}, 32, 24),
    "fx_volumetric_light_2": ("Volumetric light 2.fract", {}, 32, 24),
    "fx_volumetric_light_3": ("Volumetric light 3.fract", {}, 32, 24),
    "fx_envmap_mandelbox": ("constant factor 2.0  - mandelbox scale 2.0.fract", {}),
    "fx_envmap_hypercomplex_julia": ("hypercomplex - julia - environment mapping.fract", {"textured_background": 0}),
    "fx_envmap_power2_julia": ("power 2 - julia.fract", {"textured_background": 0}),
    # primitive objects
    "fx_primitives_inverted_box": ("primitive objects - inverted box.fract", {"raytraced_reflections": 0}),
    "fx_primitives_set": ("primitive objects - set.fract", {"raytraced_reflections": 0}),
    "fx_primitives_water": ("primitive objects - water.fract", {"raytraced_reflections": 0}),
    # ray-traced reflections
    "fx_reflections_1": ("raytraced reflections 1.fract", {"textured_background": 0}, 32, 24),
    "fx_reflections_2": ("raytraced reflections 2.fract", {"textured_background": 0}, 32, 24),
    "fx_reflections_tglad_scale_m2": ("tglad - scale -2.fract", {"textured_background": 0}, 32, 24),
    "fx_reflections_quaternion_julia": ("quaternion - julia.fract", {"textured_background": 0}, 32, 24),
    "fx_reflections_foldintpow2": ("FoldIntPow2 3.fract", {"textured_background": 0}, 32, 24),
    "fx_reflections_primitives_set": ("primitive objects - set.fract", {"textured_background": 0}, 32, 24),
    "fx_reflections_primitives_water": ("primitive objects - water.fract", {"textured_background": 0}, 32, 24),
    "fx_reflections_inverted_box": ("primitive objects - inverted box.fract", {"textured_background": 0}, 32, 24),
}

# Formulas no example uses, on the benchmark workloads' settings.
SYNTH_CASES = {
    "smooth_mandelbox": ("mandelbox_1080p", 48, 32, {"formula": 17, "mandelbox_sharpness": 3,
                                                     "ambient_occlusion_enabled": 0}),
    "fold_box_icosa": ("mandelbox_1080p", 48, 32, {"formula": 37, "mandelbox_fold_mode": 5, "mandelbox_solid": 1,
                                                   "mandelbox_melt": 0, "ambient_occlusion_enabled": 0}),
    "fold_box_prism6_melt": ("mandelbox_1080p", 48, 32, {"formula": 37, "mandelbox_fold_mode": 6,
                                                         "mandelbox_solid": 1, "mandelbox_melt": 0.1,
                                                         "ambient_occlusion_enabled": 0}),
    "fold_box_dodeca_oct_cube": ("mandelbox_1080p", 48, 32, {"formula": 37, "mandelbox_fold_mode": 3,
                                                             "mandelbox_solid": 0.9, "mandelbox_melt": 0,
                                                             "ambient_occlusion_enabled": 0,
                                                             "view_point_y": -14.0}),
    "aexion": ("mandelbulb_640x480", 40, 32, {"formula": 19, "c_add": -1.3, "N": 20, "view_point_y": -4.0}),
    "benesi": ("mandelbulb_640x480", 40, 32, {"formula": 20, "N": 30}),
    "bristorbrot": ("mandelbulb_640x480", 40, 32, {"formula": 21, "N": 30}),
    "hybrid_modifiers": ("mandelbulb_640x480", 40, 32,
                         {"formula": 12, "hybrid_formula_1": 25, "hybrid_power_1": 0.2, "hybrid_iterations_1": 1,
                          "hybrid_formula_2": 36, "hybrid_power_2": 1.5, "hybrid_iterations_2": 1,
                          "hybrid_formula_3": 27, "hybrid_power_3": 1.1, "hybrid_iterations_3": 1,
                          "hybrid_formula_4": 31, "hybrid_power_4": 0.05, "hybrid_iterations_4": 1,
                          "hybrid_formula_5": 2, "hybrid_power_5": 8, "hybrid_iterations_5": 2,
                          "hybrid_cyclic": 1, "N": 40}),
}

# Secondary effects on the benchmark workloads' settings.
EFFECT_CASES = {
    "aux_random_visible": ("mandelbulb_640x480", 40, 32,
                           {**W.AUX_LIGHTS, "aux_light_number": 6, "aux_light_random_seed": 7, "aux_light_max_dist": 0.3,
                            "aux_light_distribution_radius": 2.0, "aux_light_intensity": 1.0,
                            "aux_light_visibility": 5.0, "glow_intensity": 0}),
    "aux_predefined_penetrating": ("mandelbox_1080p", 48, 32,
                                   {**W.AUX_LIGHTS, "aux_light_predefined_1_enabled": 1, "aux_light_predefined_1_x": 2.0,
                                    "aux_light_predefined_1_y": -6.0, "aux_light_predefined_1_z": 1.0,
                                    "aux_light_predefined_1_intensity": 4.0,
                                    "aux_light_predefined_2_enabled": 1, "aux_light_predefined_2_x": -3.0,
                                    "aux_light_predefined_2_y": -5.0, "aux_light_predefined_2_z": -2.0,
                                    "aux_light_predefined_2_intensity": 2.0, "penetrating_lights": 1,
                                    "ambient_occlusion_enabled": 0, "volumetric_fog_density": 0}),
    "fake_lights": ("mandelbulb_640x480", 40, 32,
                    {"fake_lights_enabled": 1, "fake_lights_intensity": 1.0, "fake_lights_visibility": 5.0,
                     "fake_lights_visibility_size": 5.0, "fake_lights_orbit_trap_X": 2.0,
                     "fake_lights_orbit_trap_Y": 0.0, "fake_lights_orbit_trap_Z": 0.0,
                     "fake_lights_min_iter": 1, "fake_lights_max_iter": 2}),
    "fake_lights_mandelbox": ("mandelbox_1080p", 48, 32,
                              {"fake_lights_enabled": 1, "fake_lights_intensity": 0.5, "fake_lights_visibility": 2.0,
                               "fake_lights_visibility_size": 3.0, "fake_lights_orbit_trap_X": 1.0,
                               "fake_lights_orbit_trap_Y": 1.0, "fake_lights_orbit_trap_Z": 0.0,
                               "fake_lights_min_iter": 1, "fake_lights_max_iter": 3,
                               "ambient_occlusion_enabled": 0}),
    "envmap_mandelbulb": ("mandelbulb_640x480", 40, 32, {"reflect": 0.6, "ambient_occlusion_enabled": 1,
                                                         "fast_ambient_occlusion_mode": 1}),
    "slow_shading_mandelbox": ("mandelbox_1080p", 40, 32, {"slow_shading": 1, "ambient_occlusion_enabled": 0}),
    "iter_fog_mandelbulb": ("mandelbulb_640x480", 40, 32,
                            {"iteration_fog_enable": 1, "iteration_fog_opacity": 1000, "iteration_fog_opacity_trim": 4,
                             "N": 20, "ambient_occlusion_enabled": 1, "fast_ambient_occlusion_mode": 0,
                             "ambient_occlusion_quality": 1}),
    "volumetric_main_light": ("mandelbox_1080p", 40, 32,
                              {"volumetric_light_enabled_0": 1, "volumetric_light_intensity_0": 100,
                               "ambient_occlusion_enabled": 0}),
    "primitives_plane_sphere_box": ("mandelbulb_640x480", 48, 32,
                                    {"primitive_plane_enabled": 1, "primitive_plane_centre_Z": -0.9,
                                     "primitive_plane_normal_Z": 1.0, "primitive_plane_normal_X": 0.2,
                                     "primitive_sphere_enabled": 1, "primitive_sphere_centre_X": 0.9,
                                     "primitive_sphere_centre_Y": -0.6, "primitive_sphere_radius": 0.35,
                                     "primitive_box_enabled": 1, "primitive_box_centre_X": -0.9,
                                     "primitive_box_size_X": 0.4, "primitive_box_size_Y": 0.4,
                                     "primitive_box_size_Z": 0.8,
                                     "primitive_plane_colour_R": 40000, "primitive_plane_colour_G": 50000,
                                     "primitive_plane_colour_B": 60000, "primitive_sphere_colour_R": 65000,
                                     "primitive_box_colour_G": 65000}),
    "primitives_water_only_plane": ("mandelbulb_640x480", 48, 32,
                                    {"primitive_only_plane": 1, "primitive_plane_enabled": 1,
                                     "primitive_plane_centre_Z": -0.5, "primitive_plane_normal_Z": 1.0,
                                     "primitive_water_enabled": 1, "primitive_water_level": -0.3,
                                     "primitive_water_amplitude": 0.02, "primitive_water_length": 0.1,
                                     "primitive_water_rotation": 30, "primitive_water_iterations": 5,
                                     "primitive_water_anim_speed": 0.1, "frame_no": 7,
                                     "primitive_water_colour_B": 60000}),
    "aux_no_shadows": ("mandelbulb_640x480", 40, 32,
                       {**W.AUX_LIGHTS, "aux_light_number": 3, "aux_light_random_seed": 3, "aux_light_max_dist": 0.5,
                        "aux_light_distribution_radius": 2.0, "shadows_enabled": 0}),
}

# DE fixtures of every run-time formula: (name, workload or example, keys, half-size of the
# seeded point cube, points)
FORMULA_DE_ALL = (
    ("fasttrig", "mandelbulb_640x480", {"formula": 3}, 1.6),
    ("hypercomplex", "mandelbulb_640x480", {"formula": 4}, 1.6),
    ("quaternion", "mandelbulb_640x480", {"formula": 5}, 1.6),
    ("minusfasttrig", "mandelbulb_640x480", {"formula": 6}, 1.6),
    ("kaleidoscopic", "example:IFS Icosahedron.fract", {}, 2.0),
    ("ifsfold_bulb", "mandelbulb_640x480",
     {"IFS_folding_mode": 1, "IFS_scale": 1.0, "IFS_0_x": 1, "IFS_0_y": 0.3, "IFS_0_z": 0.1, "IFS_0_distance": 0.2,
      "IFS_0_enabled": 1, "IFS_0_alfa": 0.3, "IFS_absZ": 1, "IFS_rot_beta": 0.1}, 1.6),
    ("xenodreambuie", "mandelbulb_640x480", {"formula": 11}, 1.6),
    ("mandelbulb2", "mandelbulb_640x480", {"formula": 13}, 1.6),
    ("mandelbulb3", "mandelbulb_640x480", {"formula": 14}, 1.6),
    ("mandelbulb4", "mandelbulb_640x480", {"formula": 15}, 1.6),
    ("foldingintpow2", "mandelbulb_640x480", {"formula": 16, "FoldingIntPow_folding_factor": 2,
                                              "FoldingIntPow_z_factor": 5}, 1.6),
    ("smoothmandelbox", "mandelbox_1080p", {"formula": 17, "mandelbox_sharpness": 3}, 4.0),
    ("aexion", "mandelbulb_640x480", {"formula": 19, "c_add": -1.3}, 1.6),
    ("benesi", "mandelbulb_640x480", {"formula": 20}, 1.6),
    ("bristorbrot", "mandelbulb_640x480", {"formula": 21}, 1.6),
    ("foldbox_tet", "mandelbox_1080p", {"formula": 37, "mandelbox_fold_mode": 0, "mandelbox_solid": 1,
                                        "mandelbox_melt": 0}, 4.0),
    ("foldbox_cube_melt", "mandelbox_1080p", {"formula": 37, "mandelbox_fold_mode": 1, "mandelbox_solid": 1,
                                              "mandelbox_melt": 0.2}, 4.0),
    ("foldbox_oct", "mandelbox_1080p", {"formula": 37, "mandelbox_fold_mode": 2, "mandelbox_solid": 1,
                                        "mandelbox_melt": 0}, 4.0),
    ("foldbox_octcube", "mandelbox_1080p", {"formula": 37, "mandelbox_fold_mode": 4, "mandelbox_solid": 1.1,
                                            "mandelbox_melt": 0.05}, 4.0),
    ("foldbox_icosa", "mandelbox_1080p", {"formula": 37, "mandelbox_fold_mode": 5, "mandelbox_solid": 1,
                                          "mandelbox_melt": 0}, 4.0),
    ("foldbox_prism5", "mandelbox_1080p", {"formula": 37, "mandelbox_fold_mode": 7, "mandelbox_solid": 1,
                                           "mandelbox_melt": 0}, 4.0),
    ("hybrid_box_fasttrig", "example:Hybrid 1.fract", {}, 3.0),
    ("hybrid_modifiers_a", "mandelbulb_640x480",
     {"formula": 12, "hybrid_formula_1": 22, "hybrid_power_1": 0.3, "hybrid_iterations_1": 1,
      "hybrid_formula_2": 23, "hybrid_power_2": 0.2, "hybrid_iterations_2": 1,
      "hybrid_formula_3": 24, "hybrid_power_3": 0.1, "hybrid_iterations_3": 1,
      "hybrid_formula_4": 26, "hybrid_power_4": 0.1, "hybrid_iterations_4": 1,
      "hybrid_formula_5": 2, "hybrid_power_5": 8, "hybrid_iterations_5": 3, "hybrid_cyclic": 1}, 1.6),
    ("hybrid_modifiers_b", "mandelbulb_640x480",
     {"formula": 12, "hybrid_formula_1": 28, "hybrid_power_1": 1.1, "hybrid_iterations_1": 1,
      "hybrid_formula_2": 29, "hybrid_power_2": 0.9, "hybrid_iterations_2": 1,
      "hybrid_formula_3": 30, "hybrid_power_3": 1.05, "hybrid_iterations_3": 2,
      "hybrid_formula_4": 32, "hybrid_power_4": 0.1, "hybrid_iterations_4": 1,
      "hybrid_formula_5": 3, "hybrid_power_5": 2, "hybrid_iterations_5": 2, "hybrid_cyclic": 0}, 1.6),
    ("hybrid_modifiers_c", "mandelbulb_640x480",
     {"formula": 12, "hybrid_formula_1": 33, "hybrid_power_1": -0.1, "hybrid_iterations_1": 1,
      "hybrid_formula_2": 34, "hybrid_power_2": 2, "hybrid_iterations_2": 1,
      "hybrid_formula_3": 35, "hybrid_power_3": 2, "hybrid_iterations_3": 1,
      "hybrid_formula_4": 25, "hybrid_power_4": 0.4, "hybrid_iterations_4": 1,
      "hybrid_formula_5": 1, "hybrid_power_5": 8, "hybrid_iterations_5": 2, "hybrid_cyclic": 1}, 1.6),
    ("hybrid_modifiers_d", "mandelbulb_640x480",
     {"formula": 12, "hybrid_formula_1": 27, "hybrid_power_1": 1.2, "hybrid_iterations_1": 1,
      "hybrid_formula_2": 31, "hybrid_power_2": 0.2, "hybrid_iterations_2": 1,
      "hybrid_formula_3": 8, "hybrid_power_3": 2, "hybrid_iterations_3": 2,
      "hybrid_formula_4": 0, "hybrid_formula_5": 10, "hybrid_power_5": 2, "hybrid_iterations_5": 1,
      "hybrid_cyclic": 1, "IFS_scale": 2, "IFS_offsetX": 1, "IFS_offsetY": 1, "IFS_offsetZ": 1,
      "IFS_absX": 1, "IFS_absY": 1, "IFS_absZ": 1}, 2.0),
)

REF_TREE = oracle_lib.ref_tree()
DEFAULTS_FILE = os.path.join(REF_TREE, "share", "defaults")
EXAMPLES_DIR = os.path.join(REF_TREE, "share", "examples")
KEYFRAMES_DIR = os.path.join(REF_TREE, "share", "exampleKeyframes")


def ref_settings_lib():
    lib = oracle_lib.load_ref_settings()
    if lib is None:
        raise SystemExit(f"the reference tree is not at {REF_TREE} (set MBGB_REF_TREE)")
    return lib


def make_scene(overrides: dict) -> mb.mbgb_scene:
    """The scene of a key list (the workload base updated with `overrides`) as the
    reference's own LoadOneSetting / LoadSettingsPost and the -nogui derivations read it."""
    keys = dict(W.BASE)
    keys.update(overrides)
    return oracle_lib.ref_scene_from_keys(ref_settings_lib(), mb.mbgb_scene(), keys)


def workload_scene(name: str, w: int | None = None, h: int | None = None) -> mb.mbgb_scene:
    keys = dict(W.WORKLOADS[name])
    if w and h:
        keys["image_width"], keys["image_height"] = w, h
        keys["perspective"] = W.fov_persp(w, h)
    return make_scene(keys)


def example_scene(fname: str, extra: dict, w: int = 48, h: int = 32):
    """An example file read by the reference's own LoadSettings2 after share/defaults."""
    ov = [f"image_width {w}", f"image_height {h}", "post_SSAO_enabled 0"]
    ov += [f"{k} {v}" for k, v in extra.items()]
    return oracle_lib.ref_scene_from_settings(ref_settings_lib(), mb.mbgb_scene(), DEFAULTS_FILE,
                                              os.path.join(EXAMPLES_DIR, fname), ov)


def settings_files() -> list:
    """share/defaults, every share/examples/*.fract and every share/exampleKeyframes/*.fract."""
    ex = sorted(f for f in os.listdir(EXAMPLES_DIR) if f.endswith(".fract"))
    kf = sorted(f for f in os.listdir(KEYFRAMES_DIR) if f.endswith(".fract"))
    return ([("defaults", DEFAULTS_FILE)] + [("examples/" + f, os.path.join(EXAMPLES_DIR, f)) for f in ex]
            + [("exampleKeyframes/" + f, os.path.join(KEYFRAMES_DIR, f)) for f in kf])


def settings_goldens(manifest: dict):
    """settings_reference.npz: each shipped settings file as the reference reads it (after
    share/defaults, as LoadSettings does), with the SHA-256 of the file it read;
    bench_scenes.npz: the bench workloads' scenes as the reference reads their key lists."""
    import hashlib
    lib = ref_settings_lib()
    names, shas, blobs = [], [], []
    for name, path in settings_files():
        sc = oracle_lib.ref_scene_from_settings(lib, mb.mbgb_scene(), None if name == "defaults" else DEFAULTS_FILE,
                                                path)
        with open(path, "rb") as f:
            shas.append(hashlib.sha256(f.read()).hexdigest())
        names.append(name)
        blobs.append(np.frombuffer(mb.scene_bytes(sc), np.uint8))
    np.savez_compressed(os.path.join(HERE, "settings_reference.npz"), names=np.array(names), sha256=np.array(shas),
                        scenes=np.stack(blobs))
    manifest["settings_reference.npz"] = {"files": len(names), "reader": "src/settings.cpp LoadSettings2 "
                                          "(oracle/_ref/libmbref_settings.so) + -nogui derivations"}
    bench = {n: np.frombuffer(mb.scene_bytes(workload_scene(n)), np.uint8) for n in ("mandelbox_1080p",
                                                                                      "mandelbulb_640x480")}
    np.savez_compressed(os.path.join(HERE, "bench_scenes.npz"), **bench)
    manifest["bench_scenes.npz"] = {"workloads": sorted(bench), "reader": "src/settings.cpp LoadOneSetting"}
    print(len(names), "settings files;", "bench scenes", sorted(bench))


def render_example_cases(lib, manifest: dict, only=None):
    for case, spec in EXAMPLES.items():
        if only and case not in only:
            continue
        fname, extra = spec[0], spec[1]
        sc = example_scene(fname, extra, *spec[2:])
        ok, why = mb.supported(sc)
        assert ok, (case, why)
        w, h = sc.image_width, sc.image_height
        img = mb.CImage.empty(w, h)
        lib.ref_render(ctypes.byref(sc), 0, h, 0, ctypes.byref(img.as_c()))
        out = os.path.join(HERE, f"render_ex_{case}.npz")
        np.savez_compressed(out, scene=np.frombuffer(mb.scene_bytes(sc), np.uint8),
                            example=np.array(fname), overrides=np.array(json.dumps(extra)),
                            image_float=img.image_float, zbuffer=img.zbuffer, alpha=img.alpha, opacity=img.opacity,
                            colour=img.colour, hit=img.hit, iters=img.iters, depth=img.depth)
        manifest[os.path.basename(out)] = {"example": fname, "size": [w, h], "overrides": extra,
                                           "formula": int(sc.formula), "hit_fraction": float(img.hit.mean())}
        print(case, "formula", sc.formula, "hit", img.hit.mean())


def formula_de_all(lib, manifest: dict, npts: int = 400):
    for i, (name, wl, extra, half) in enumerate(FORMULA_DE_ALL):
        rng = np.random.default_rng(100 + i)
        if wl.startswith("example:"):
            sc = example_scene(wl[8:], extra, 64, 48)
        else:
            keys = dict(W.WORKLOADS[wl])
            keys["image_width"], keys["image_height"] = 64, 48
            keys["perspective"] = W.fov_persp(64, 48)
            keys.update(extra)
            sc = make_scene(keys)
        pts = np.ascontiguousarray(rng.uniform(-half, half, (npts, 3)))
        detail = np.ascontiguousarray(10.0 ** rng.uniform(-6, -2, npts))
        dist = np.zeros(npts)
        iters = np.zeros(npts, np.int32)
        mi = np.zeros(npts, np.uint8)
        lib.ref_distance(ctypes.byref(sc), ptr(pts), ptr(detail), ctypes.c_long(npts), ptr(dist), ptr(iters),
                         ptr(mi))
        colour = np.zeros(npts)
        lib.ref_colour_value(ctypes.byref(sc), ptr(pts), ctypes.c_long(npts), ptr(colour))
        out = os.path.join(HERE, f"de_{name}.npz")
        np.savez_compressed(out, scene=np.frombuffer(mb.scene_bytes(sc), np.uint8), points=pts, detail=detail,
                            dist=dist, iters=iters, max_iter=mi, colour=colour)
        manifest[os.path.basename(out)] = {"source": wl, "points": npts, "keys": extra,
                                           "formula": int(sc.formula), "analytic": int(sc.analitycDE),
                                           "max_iter_fraction": float(mi.mean())}
        print(name, "formula", sc.formula, "analytic", sc.analitycDE, "max_iter", mi.mean(),
              "iters", np.bincount(iters).nonzero()[0][:8])


def effect_goldens(manifest: dict):
    """The secondary effects' example scenes and synthetic scenes."""
    lib = build_ref()
    render_example_cases(lib, manifest, only=[k for k in EXAMPLES if k.startswith(("aux_", "fx_"))])
    render_cases(lib, EFFECT_CASES, manifest)


def build_ref() -> ctypes.CDLL:
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmbref.so"))
    return lib


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def de_points(formula: str, rng: np.random.Generator):
    """Seeded points: a uniform cube plus points near the surface along camera rays."""
    if formula == "mandelbulb":
        cube = rng.uniform(-1.6, 1.6, (2000, 3))
    else:
        cube = rng.uniform(-7.0, 7.0, (2000, 3))
    return cube


def main():
    lib = build_ref()
    manifest = {}
    for formula, wl in (("mandelbulb", "mandelbulb_640x480"), ("mandelbox", "mandelbox_1080p")):
        rng = np.random.default_rng(1234 if formula == "mandelbulb" else 5678)
        sc = workload_scene(wl, 64, 48)
        pts = np.ascontiguousarray(de_points(formula, rng))
        n = len(pts)
        detail = np.ascontiguousarray(10.0 ** rng.uniform(-6, -2, n))
        dist = np.zeros(n)
        iters = np.zeros(n, np.int32)
        mi = np.zeros(n, np.uint8)
        lib.ref_distance(ctypes.byref(sc), ptr(pts), ptr(detail), ctypes.c_long(n), ptr(dist), ptr(iters), ptr(mi))
        colour = np.zeros(n)
        lib.ref_colour_value(ctypes.byref(sc), ptr(pts), ctypes.c_long(n), ptr(colour))
        out = os.path.join(HERE, f"de_{formula}.npz")
        np.savez_compressed(out, scene=np.frombuffer(mb.scene_bytes(sc), np.uint8), points=pts, detail=detail,
                            dist=dist, iters=iters, max_iter=mi, colour=colour)
        manifest[os.path.basename(out)] = {"workload": wl, "points": n}
    for case, (wl, w, h, extra) in CASES.items():
        keys = dict(W.WORKLOADS[wl])
        keys["image_width"], keys["image_height"] = w, h
        keys["perspective"] = W.fov_persp(w, h)
        keys.update(extra)
        sc = make_scene(keys)
        img = mb.CImage.empty(w, h)
        lib.ref_render(ctypes.byref(sc), 0, h, 0, ctypes.byref(img.as_c()))
        out = os.path.join(HERE, f"render_{case}.npz")
        np.savez_compressed(out, scene=np.frombuffer(mb.scene_bytes(sc), np.uint8),
                            keys=np.array(json.dumps(keys)), image_float=img.image_float, zbuffer=img.zbuffer,
                            alpha=img.alpha, opacity=img.opacity, colour=img.colour, hit=img.hit, iters=img.iters,
                            depth=img.depth)
        manifest[os.path.basename(out)] = {"workload": wl, "size": [w, h], "keys": extra,
                                           "hit_fraction": float(img.hit.mean())}
        print(case, "hit", img.hit.mean())
    # CMorph::CatmullRom (src/morph.cpp:49-109) on seeded rows covering its branches:
    # same-sign rows with large variation (logarithmic mode), negative rows, mixed signs,
    # near-constant rows, rows crossing +-1e20 and values below 1e-20
    rng = np.random.default_rng(4242)
    n_keys, size, fpk = 8, 64, 8
    keys = np.empty((n_keys, size))
    keys[:, 0:12] = rng.uniform(0.1, 10.0, (n_keys, 12))
    keys[:, 12:24] = -rng.uniform(0.1, 10.0, (n_keys, 12))
    keys[:, 24:36] = rng.uniform(-3.0, 3.0, (n_keys, 12))
    keys[:, 36:44] = 5.0 + rng.uniform(-0.01, 0.01, (n_keys, 8))
    keys[:, 44:50] = rng.uniform(1e19, 9e20, (n_keys, 6)) * np.where(rng.random((n_keys, 6)) < 0.5, -1, 1)
    keys[:, 50:56] = rng.uniform(-1e-19, 1e-19, (n_keys, 6))
    keys[:, 56:64] = np.cumsum(rng.normal(0, 1, (n_keys, 8)), axis=0)
    keys = np.ascontiguousarray(keys)
    out = np.zeros((n_keys * fpk, size))
    lib.ref_catmull_rom(ptr(keys), n_keys, size, fpk, n_keys * fpk, ptr(out))
    np.savez_compressed(os.path.join(HERE, "catmull_rom.npz"), keys=keys, frames_per_key=fpk, out=out)
    manifest["catmull_rom.npz"] = {"keys": [n_keys, size], "frames_per_key": fpk}
    post_goldens(manifest)
    formula_goldens(manifest)
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


# render fixtures used as post-processing inputs, with (brightness, contrast, gamma, hdr,
# SSAO quality, global illumination intensity)
POST_CASES = {
    "mandelbulb_64x48": ("mandelbulb_64x48", 1.0, 1.0, 1.0, 0, 20, 1.0),
    "mandelbox_96x54": ("mandelbox_96x54", 1.3, 1.1, 0.8, 0, 7, 0.8),
    "fisheye": ("mandelbulb_fisheye_cut", 0.9, 1.4, 1.2, 1, 12, 1.0),
    "equirect": ("mandelbulb_tiles_equirect", 1.0, 0.9, 1.0, 1, 5, 1.5),
}


def post_goldens(manifest: dict):
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmbref_post.so"))
    lib.ref_compile_image.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    lib.ref_ssao.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    for case, (render, bright, contrast, gamma, hdr, quality, ilum) in POST_CASES.items():
        z = np.load(os.path.join(HERE, f"render_{render}.npz"))
        sc = mb.scene_from_bytes(z["scene"].tobytes())
        h, w = z["zbuffer"].shape
        img_f = np.ascontiguousarray(z["image_float"], np.float32)
        img16 = np.zeros((h, w, 3), np.uint16)
        lib.ref_compile_image(w, h, ptr(img_f), bright, contrast, gamma, hdr, ptr(img16))
        compiled = img16.copy()
        lib.ref_ssao(w, h, ptr(np.ascontiguousarray(z["zbuffer"])), ptr(np.ascontiguousarray(z["opacity"])),
                     ptr(np.ascontiguousarray(z["colour"])), sc.persp, quality, sc.perspectiveType, ilum, ptr(img16))
        out = os.path.join(HERE, f"post_{case}.npz")
        np.savez_compressed(out, render=np.array(render), brightness=bright, contrast=contrast, gamma=gamma,
                            hdr=hdr, quality=quality, global_ilum=ilum, image16_compiled=compiled,
                            image16_ssao=img16)
        manifest[os.path.basename(out)] = {"render": render, "ssao_quality": quality,
                                           "changed_by_ssao": float(np.mean(img16 != compiled))}
        print(case, "ssao changed", np.mean(img16 != compiled))


# Depth of field on rendered fixtures: (render fixture, DOF radius, DOF focus, seed).
DOF_CASES = {
    "mandelbox_96x54": ("mandelbox_96x54", 20.0, 162.0, 1),
    "mandelbulb_64x48": ("mandelbulb_64x48", 40.0, 155.0, 7),
    "ifs_icosahedron": ("ex_ifs_icosahedron", 80.0, 158.0, 12345),
}


def dof_goldens(manifest: dict):
    """PostRendering_DOF of the reference (libmbref_post.so) on compiled render fixtures."""
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmbref_post.so"))
    lib.ref_compile_image.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    lib.ref_dof.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_double, ctypes.c_double, ctypes.c_uint]
    for case, (render, radius, focus, seed) in DOF_CASES.items():
        z = np.load(os.path.join(HERE, f"render_{render}.npz"))
        h, w = z["zbuffer"].shape
        img_f = np.ascontiguousarray(z["image_float"], np.float32)
        img16 = np.zeros((h, w, 3), np.uint16)
        lib.ref_compile_image(w, h, ptr(img_f), 1.0, 1.0, 1.0, 0, ptr(img16))
        compiled = img16.copy()
        alpha = np.ascontiguousarray(z["alpha"]).copy()
        alpha_in = alpha.copy()
        deep = radius * w / 1000.0
        neutral = 10.0 ** (focus / 10.0 - 16.0)
        lib.ref_dof(w, h, ptr(np.ascontiguousarray(z["zbuffer"])), ptr(alpha), ptr(img16), deep, neutral, seed)
        out = os.path.join(HERE, f"dof_{case}.npz")
        np.savez_compressed(out, render=np.array(render), radius=radius, focus=focus, seed=seed,
                            image16_in=compiled, alpha_in=alpha_in, image16_dof=img16, alpha_dof=alpha)
        manifest[os.path.basename(out)] = {"render": render, "radius": radius, "focus": focus, "seed": seed,
                                           "changed_by_dof": float(np.mean(img16 != compiled))}
        print(case, "dof changed", np.mean(img16 != compiled))


def formula_goldens(manifest: dict):
    """DE and render fixtures of the run-time formulas from the reference's own code."""
    lib = build_ref()
    for name, wl, extra, half in FORMULA_DE:
        rng = np.random.default_rng({"trigde": 11, "menger": 12, "vary4d": 13}[name])
        keys = dict(W.WORKLOADS[wl])
        keys["image_width"], keys["image_height"] = 64, 48
        keys["perspective"] = W.fov_persp(64, 48)
        keys.update(extra)
        sc = make_scene(keys)
        pts = np.ascontiguousarray(rng.uniform(-half, half, (2000, 3)))
        n = len(pts)
        detail = np.ascontiguousarray(10.0 ** rng.uniform(-6, -2, n))
        dist = np.zeros(n)
        iters = np.zeros(n, np.int32)
        mi = np.zeros(n, np.uint8)
        lib.ref_distance(ctypes.byref(sc), ptr(pts), ptr(detail), ctypes.c_long(n), ptr(dist), ptr(iters), ptr(mi))
        colour = np.zeros(n)
        lib.ref_colour_value(ctypes.byref(sc), ptr(pts), ctypes.c_long(n), ptr(colour))
        out = os.path.join(HERE, f"de_{name}.npz")
        np.savez_compressed(out, scene=np.frombuffer(mb.scene_bytes(sc), np.uint8), points=pts, detail=detail,
                            dist=dist, iters=iters, max_iter=mi, colour=colour)
        manifest[os.path.basename(out)] = {"workload": wl, "points": n, "keys": extra}
    render_cases(lib, FORMULA_CASES, manifest)


def all_formula_goldens(manifest: dict):
    """Every other formula: DE fixtures, example scenes and synthetic scenes."""
    lib = build_ref()
    formula_de_all(lib, manifest)
    render_example_cases(lib, manifest)
    render_cases(lib, SYNTH_CASES, manifest)


def render_cases(lib, cases: dict, manifest: dict):
    for case, (wl, w, h, extra) in cases.items():
        keys = dict(W.WORKLOADS[wl])
        keys["image_width"], keys["image_height"] = w, h
        keys["perspective"] = W.fov_persp(w, h)
        keys.update(extra)
        sc = make_scene(keys)
        img = mb.CImage.empty(w, h)
        lib.ref_render(ctypes.byref(sc), 0, h, 0, ctypes.byref(img.as_c()))
        out = os.path.join(HERE, f"render_{case}.npz")
        np.savez_compressed(out, scene=np.frombuffer(mb.scene_bytes(sc), np.uint8),
                            keys=np.array(json.dumps(keys)), image_float=img.image_float, zbuffer=img.zbuffer,
                            alpha=img.alpha, opacity=img.opacity, colour=img.colour, hit=img.hit, iters=img.iters,
                            depth=img.depth)
        manifest[os.path.basename(out)] = {"workload": wl, "size": [w, h], "keys": extra,
                                           "hit_fraction": float(img.hit.mean())}
        print(case, "hit", img.hit.mean())


if __name__ == "__main__":
    if sys.argv[1:] in (["post"], ["formulas"], ["all_formulas"], ["effects"], ["dof"], ["settings"]):
        with open(os.path.join(HERE, "MANIFEST.json")) as f:
            manifest = json.load(f)
        {"post": post_goldens, "formulas": formula_goldens, "all_formulas": all_formula_goldens,
         "effects": effect_goldens, "dof": dof_goldens, "settings": settings_goldens}[sys.argv[1]](manifest)
        with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
            json.dump(manifest, f, indent=1, sort_keys=True)
    else:
        main()
