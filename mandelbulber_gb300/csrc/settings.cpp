// Settings reader for .fract files and the -nogui parameter derivations.
//
// Reads the same "key value;" format as LoadSettings2 (src/settings.cpp:628-698)
// with the same key names and conversions as LoadOneSetting
// (src/settings.cpp:700-1183): degrees become radians for the camera and
// Mandelbox rotation angles, booleans are "atoi(value) != 0", N is read with atoi
// and stored as double. The key set is a table keyed by name instead of the
// reference's if/else chain. After every file the palette rule of
// LoadSettingsPost (src/settings.cpp:1185-1195) applies: if the file carried no
// complete palette, NewPalette (src/image.cpp:28-55) regenerates it from
// coloring_random_seed with the C library's rand() sequence.
#include "mbgb.h"
#include "mbgb_internal.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

namespace mbgb {

// ---------------------------------------------------------------------------
// glibc rand(): the additive-feedback generator behind srand()/rand()
// (TYPE_3, degree 31, separation 3). The reference seeds it with srand(seed)
// before NewPalette; palette parity needs the same sequence on every host.
// ---------------------------------------------------------------------------
GlibcRand::GlibcRand(uint32_t seed) {
  int32_t r[34];
  if (seed == 0) seed = 1;
  r[0] = (int32_t)seed;
  for (int i = 1; i < 31; i++) {
    // r[i] = (16807 * r[i-1]) % 2147483647 computed without overflow (Schrage).
    const int32_t hi = r[i - 1] / 127773;
    const int32_t lo = r[i - 1] % 127773;
    int32_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = word;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 0; i < 34; i++) ring_[i] = (uint32_t)r[i];
  // the generator discards its first 310 outputs after seeding
  idx_ = 34;
  for (int i = 34; i < 344; i++) next_raw();
}

uint32_t GlibcRand::next_raw() {
  // o_k = r[k-31] + r[k-3] (mod 2^32), ring of 34 entries
  const uint32_t v = ring_[(idx_ - 31) % 34] + ring_[(idx_ - 3) % 34];
  ring_[idx_ % 34] = v;
  idx_++;
  return v;
}

int GlibcRand::rand() { return (int)(next_raw() >> 1); }

// Random(max) = rand() % (max + 1)  (src/common_math.cpp:25-32, non-WIN32 branch)
int GlibcRand::random(int max) { return rand() % (max + 1); }

}  // namespace mbgb

using mbgb::GlibcRand;

extern "C" void mbgb_palette_from_seed(int32_t seed, double saturation, mbgb_rgb palette[256]) {
  // NewPalette (src/image.cpp:28-55): 255 random colours around a random grey
  // level, then fixed entries 253..255.
  GlibcRand rng((uint32_t)seed);
  for (int i = 0; i < 255; i++) {
    const int Y = (int)((rng.random(255) - 128) / (1.0 + saturation));
    int R = (int)(Y + 128 + (rng.random(255) - 128) * saturation);
    int G = (int)(Y + 128 + (rng.random(255) - 128) * saturation);
    int B = (int)(Y + 128 + (rng.random(255) - 128) * saturation);
    palette[i].R = R < 0 ? 0 : (R > 255 ? 255 : R);
    palette[i].G = G < 0 ? 0 : (G > 255 ? 255 : G);
    palette[i].B = B < 0 ? 0 : (B > 255 ? 255 : B);
  }
  palette[255] = {255, 255, 255};
  palette[254] = {0, 0, 0};
  palette[253] = {0, 20, 40};
}

namespace {

enum class Kind { Dbl, Int, Bool, BoolF, Deg, Palette, Ignore };

struct Key {
  Kind kind;
  size_t off;
};

#define OFF(field) offsetof(mbgb_scene, field)

std::unordered_map<std::string, Key> build_table() {
  std::unordered_map<std::string, Key> t;
  auto D = [&](const std::string &k, size_t o) { t[k] = {Kind::Dbl, o}; };
  auto I = [&](const std::string &k, size_t o) { t[k] = {Kind::Int, o}; };
  auto B = [&](const std::string &k, size_t o) { t[k] = {Kind::Bool, o}; };
  auto A = [&](const std::string &k, size_t o) { t[k] = {Kind::Deg, o}; };
  auto RGB = [&](const std::string &prefix, size_t o) {
    I(prefix + "R", o + 0);
    I(prefix + "G", o + 4);
    I(prefix + "B", o + 8);
  };
  const char *xyz[3] = {"x", "y", "z"};
  const char *XYZ[3] = {"X", "Y", "Z"};

  // IFS vectors (src/settings.cpp:705-768); IFS angles are kept in degrees
  for (int i = 0; i < 9; i++) {
    std::string p = "IFS_" + std::to_string(i) + "_";
    for (int c = 0; c < 3; c++) D(p + xyz[c], OFF(ifsDirection) + sizeof(double) * (3 * i + c));
    D(p + "alfa", OFF(ifsAlfa) + sizeof(double) * i);
    D(p + "beta", OFF(ifsBeta) + sizeof(double) * i);
    D(p + "gamma", OFF(ifsGamma) + sizeof(double) * i);
    D(p + "distance", OFF(ifsDistance) + sizeof(double) * i);
    D(p + "intensity", OFF(ifsIntensity) + sizeof(double) * i);
    B(p + "enabled", OFF(ifsEnabled) + i);
  }
  D("Mandelbulber", OFF(settingsVersion));
  I("image_width", OFF(image_width));
  I("image_height", OFF(image_height));
  I("tiles", OFF(noOfTiles));
  D("x_min", OFF(amin)); D("x_max", OFF(amax));
  D("y_min", OFF(bmin)); D("y_max", OFF(bmax));
  D("z_min", OFF(cmin)); D("z_max", OFF(cmax));
  for (int c = 0; c < 3; c++) D(std::string("view_point_") + xyz[c], OFF(vp) + sizeof(double) * c);
  A("angle_alfa", OFF(alpha)); A("angle_beta", OFF(beta)); A("angle_gamma", OFF(gamma));
  D("zoom", OFF(zoom));
  D("perspective", OFF(persp));
  I("formula", OFF(formula));
  D("power", OFF(power));
  t["N"] = {Kind::Int, OFF(N)};  // special-cased: atoi into a double
  I("minN", OFF(minN));
  D("fractal_constant_factor", OFF(constantFactor));
  D("quality", OFF(quality));
  D("smoothness", OFF(smoothness));
  B("julia_mode", OFF(juliaMode));
  D("julia_a", OFF(julia) + 0); D("julia_b", OFF(julia) + 8); D("julia_c", OFF(julia) + 16);
  B("tglad_folding_mode", OFF(tgladFoldingMode));
  D("folding_limit", OFF(foldingLimit));
  D("folding_value", OFF(foldingValue));
  B("spherical_folding_mode", OFF(sphericalFoldingMode));
  D("spherical_folding_fixed", OFF(foldingSphericalFixed));
  D("spherical_folding_min", OFF(foldingSphericalMin));
  B("IFS_folding_mode", OFF(ifsFoldingMode));
  B("iteration_threshold_mode", OFF(iterThresh));
  B("analityc_DE_mode", OFF(analitycDE));
  D("DE_factor", OFF(DE_factor));
  D("brightness", OFF(brightness));
  D("contrast", OFF(contrast));
  D("gamma", OFF(imageGamma));
  B("hdr", OFF(hdrEnabled));
  D("ambient", OFF(ambient));
  D("reflect", OFF(reflect));
  D("shadows_intensity", OFF(directLight));
  D("shadows_cone_angle", OFF(shadowConeAngle));
  D("ambient_occlusion", OFF(globalIlum));
  I("ambient_occlusion_quality", OFF(globalIlumQuality));
  D("ambient_occlusion_fast_tune", OFF(fastAoTune));
  D("shading", OFF(shading));
  D("specular", OFF(specular));
  D("glow_intensity", OFF(glow_intensity));
  RGB("glow_color_1_", OFF(glow_color1));
  RGB("glow_color_2_", OFF(glow_color2));
  RGB("background_color_1_", OFF(background_color1));
  RGB("background_color_2_", OFF(background_color2));
  RGB("background_color_3_", OFF(background_color3));
  RGB("fog_colour_1_", OFF(fogColour1));
  RGB("fog_colour_2_", OFF(fogColour2));
  RGB("fog_colour_3_", OFF(fogColour3));
  B("textured_background", OFF(texturedBackground));
  B("background_as_fuldome", OFF(background_as_fulldome));
  B("shadows_enabled", OFF(shadow));
  B("ambient_occlusion_enabled", OFF(global_ilumination));
  B("fast_ambient_occlusion_mode", OFF(fastGlobalIllumination));
  B("fractal_color", OFF(coloringEnabled));
  I("coloring_random_seed", OFF(coloring_seed));
  D("coloring_saturation", OFF(colourSaturation));
  D("coloring_speed", OFF(coloring_speed));
  D("coloring_palette_offset", OFF(paletteOffset));
  B("slow_shading", OFF(slowShading));
  B("limits_enabled", OFF(limits_enabled));
  B("post_fog_enabled", OFF(fogEnabled));
  D("post_fog_visibility", OFF(fogVisibility));
  RGB("post_fog_color_", OFF(fogColor));
  B("post_SSAO_enabled", OFF(SSAOEnabled));
  I("post_SSAO_quality", OFF(SSAOQuality));
  B("post_DOF_enabled", OFF(DOFEnabled));
  D("post_DOF_focus", OFF(DOFFocus));
  D("post_DOF_radius", OFF(DOFRadius));
  D("main_light_intensity", OFF(mainLightIntensity));
  D("main_light_alfa", OFF(mainLightAlpha));   // radians in the file
  D("main_light_beta", OFF(mainLightBeta));
  RGB("main_light_colour_", OFF(mainLightColour));
  D("aux_light_intensity", OFF(auxLightIntensity));
  I("aux_light_random_seed", OFF(auxLightRandomSeed));
  I("aux_light_number", OFF(auxLightNumber));
  D("aux_light_max_dist", OFF(auxLightMaxDist));
  D("aux_light_distribution_radius", OFF(auxLightDistributionRadius));
  for (int i = 0; i < 4; i++) {
    std::string p = "aux_light_predefined_" + std::to_string(i + 1) + "_";
    for (int c = 0; c < 3; c++) D(p + xyz[c], OFF(auxLightPre) + sizeof(double) * (3 * i + c));
    D(p + "intensity", OFF(auxLightPreIntensity) + sizeof(double) * i);
    B(p + "enabled", OFF(auxLightPreEnabled) + i);
    RGB(p + "colour_", OFF(auxLightPreColour) + sizeof(mbgb_rgb) * i);
  }
  D("aux_light_visibility", OFF(auxLightVisibility));
  for (int c = 0; c < 3; c++)
    D(std::string("aux_light_random_center_") + XYZ[c], OFF(auxLightRandomCenter) + sizeof(double) * c);
  D("IFS_scale", OFF(ifsScale));
  D("IFS_rot_alfa", OFF(ifsRotationAlfa));
  D("IFS_rot_beta", OFF(ifsRotationBeta));
  D("IFS_rot_gamma", OFF(ifsRotationGamma));
  for (int c = 0; c < 3; c++) {
    D(std::string("IFS_offset") + XYZ[c], OFF(ifsOffset) + sizeof(double) * c);
    D(std::string("IFS_edge") + XYZ[c], OFF(ifsEdge) + sizeof(double) * c);
  }
  t["IFS_absX"] = {Kind::BoolF, OFF(ifsAbsX)};
  t["IFS_absY"] = {Kind::BoolF, OFF(ifsAbsY)};
  t["IFS_absZ"] = {Kind::BoolF, OFF(ifsAbsZ)};
  t["IFS_menger_sponge_mode"] = {Kind::BoolF, OFF(ifsMengerSpongeMode)};
  I("start_frame", OFF(startFrame));
  I("end_frame", OFF(endFrame));
  I("frames_per_keyframe", OFF(framesPerKeyframe));
  B("hybrid_cyclic", OFF(hybridCyclic));
  I("fish_eye", OFF(perspectiveType));
  B("fish_eye_180cut", OFF(fishEyeCut));
  B("stereo_enabled", OFF(stereoEnabled));
  D("stereo_eye_distance", OFF(stereoEyeDistance));
  D("mandelbox_scale", OFF(mboxScale));
  D("mandelbox_folding_limit", OFF(mboxFoldingLimit));
  D("mandelbox_folding_value", OFF(mboxFoldingValue));
  D("mandelbox_folding_min_radius", OFF(mboxFoldingSphericalMin));
  D("mandelbox_folding_fixed_radius", OFF(mboxFoldingSphericalFixed));
  D("mandelbox_sharpness", OFF(mboxSharpness));
  for (int c = 0; c < 3; c++) D(std::string("mandelbox_offset_") + XYZ[c], OFF(mboxOffset) + sizeof(double) * c);
  D("mandelbox_color_R", OFF(mboxColorFactorR));
  D("mandelbox_color_X", OFF(mboxColorFactorX));
  D("mandelbox_color_Y", OFF(mboxColorFactorY));
  D("mandelbox_color_Z", OFF(mboxColorFactorZ));
  D("mandelbox_color_Sp1", OFF(mboxColorFactorSp1));
  D("mandelbox_color_Sp2", OFF(mboxColorFactorSp2));
  B("mandelbox_rotation_enabled", OFF(mboxRotationsEnabled));
  I("mandelbox_fold_mode", OFF(genFoldBoxType));
  D("mandelbox_solid", OFF(mboxSolid));
  D("mandelbox_melt", OFF(mboxMelt));
  D("view_distance_max", OFF(viewDistanceMax));
  D("view_distance_min", OFF(viewDistanceMin));
  B("interior_mode", OFF(interiorMode));
  B("linear_DE_mode", OFF(linearDEmode));
  B("constant_DE_threshold", OFF(constantDEThreshold));
  D("FoldingIntPow_folding_factor", OFF(FoldingIntPowFoldFactor));
  D("FoldingIntPow_z_factor", OFF(FoldingIntPowZfactor));
  B("penetrating_lights", OFF(penetratingLights));
  B("raytraced_reflections", OFF(raytracedReflections));
  I("reflections_max", OFF(reflectionsMax));
  D("mandelbox_vary_scale_vary", OFF(mboxVaryScaleVary));
  D("mandelbox_vary_fold", OFF(mboxVaryFold));
  D("mandelbox_vary_minr", OFF(mboxVaryMinR));
  D("mandelbox_vary_rpower", OFF(mboxVaryRPower));
  D("mandelbox_vary_wadd", OFF(mboxVaryWadd));
  D("c_add", OFF(cadd));
  D("volumetric_fog_density", OFF(fogDensity));
  D("volumetric_fog_colour_1_distance", OFF(fogColour1Distance));
  D("volumetric_fog_colour_2_distance", OFF(fogColour2Distance));
  D("volumetric_fog_distance_factor", OFF(fogDistanceFactor));
  B("iteration_fog_enable", OFF(iterFogEnabled));
  D("iteration_fog_opacity", OFF(iterFogOpacity));
  D("iteration_fog_opacity_trim", OFF(iterFogOpacityTrim));
  B("primitive_only_plane", OFF(onlyPlane));
  // primitives (src/settings.cpp:1000-1066)
  B("primitive_plane_enabled", OFF(planeEnable));
  for (int c = 0; c < 3; c++) {
    D(std::string("primitive_plane_centre_") + XYZ[c], OFF(planeCentre) + 8 * c);
    D(std::string("primitive_plane_normal_") + XYZ[c], OFF(planeNormal) + 8 * c);
    D(std::string("primitive_box_centre_") + XYZ[c], OFF(boxCentre) + 8 * c);
    D(std::string("primitive_box_size_") + XYZ[c], OFF(boxSize) + 8 * c);
    D(std::string("primitive_invertedBox_centre_") + XYZ[c], OFF(invertedBoxCentre) + 8 * c);
    D(std::string("primitive_invertedBox_size_") + XYZ[c], OFF(invertedBoxSize) + 8 * c);
    D(std::string("primitive_sphere_centre_") + XYZ[c], OFF(sphereCentre) + 8 * c);
    D(std::string("primitive_invertedSphere_centre_") + XYZ[c], OFF(invertedSphereCentre) + 8 * c);
  }
  RGB("primitive_plane_colour_", OFF(primitivePlaneColour));
  D("primitive_plane_reflect", OFF(primitivePlaneReflect));
  B("primitive_box_enabled", OFF(boxEnable));
  RGB("primitive_box_colour_", OFF(primitiveBoxColour));
  D("primitive_box_reflect", OFF(primitiveBoxReflect));
  B("primitive_invertedBox_enabled", OFF(invertedBoxEnable));
  RGB("primitive_invertedBox_colour_", OFF(primitiveInvertedBoxColour));
  D("primitive_invertedBox_reflect", OFF(primitiveInvertedBoxReflect));
  B("primitive_sphere_enabled", OFF(sphereEnable));
  D("primitive_sphere_radius", OFF(sphereRadius));
  RGB("primitive_sphere_colour_", OFF(primitiveSphereColour));
  D("primitive_sphere_reflect", OFF(primitiveSphereReflect));
  B("primitive_invertedSphere_enabled", OFF(invertedSphereEnable));
  D("primitive_invertedSphere_radius", OFF(invertedSphereRadius));
  RGB("primitive_invertedSphere_colour_", OFF(primitiveInvertedSphereColour));
  D("primitive_invertedSphere_reflect", OFF(primitiveInvertedSphereReflect));
  B("primitive_water_enabled", OFF(waterEnable));
  D("primitive_water_level", OFF(waterHeight));
  D("primitive_water_amplitude", OFF(waterAmplitude));
  D("primitive_water_length", OFF(waterLength));
  I("primitive_water_iterations", OFF(waterIterations));
  D("primitive_water_rotation", OFF(waterRotation));
  D("primitive_water_anim_speed", OFF(waterAnimSpeed));
  RGB("primitive_water_colour_", OFF(primitiveWaterColour));
  D("primitive_water_reflect", OFF(primitiveWaterReflect));
  B("fake_lights_enabled", OFF(fakeLightsEnabled));
  I("fake_lights_min_iter", OFF(fakeLightsMinIter));
  I("fake_lights_max_iter", OFF(fakeLightsMaxIter));
  D("fake_lights_visibility", OFF(fakeLightsVisibility));
  D("fake_lights_visibility_size", OFF(fakeLightsVisibilitySize));
  D("fake_lights_intensity", OFF(fakeLightsIntensity));
  for (int c = 0; c < 3; c++)
    D(std::string("fake_lights_orbit_trap_") + XYZ[c], OFF(fakeLightsOrbitTrap) + 8 * c);
  I("frame_no", OFF(frameNo));
  I("tile_no", OFF(tileCount));
  for (const char *k : {"file_destination", "file_background", "file_envmap", "file_lightmap",
                        "file_animation_path", "file_keyframes"})
    t[k] = {Kind::Ignore, 0};
  t["palette"] = {Kind::Palette, OFF(palette)};
  for (int i = 0; i < 5; i++) {
    B("volumetric_light_enabled_" + std::to_string(i), OFF(volumetricLightEnabled) + i);
    D("volumetric_light_intensity_" + std::to_string(i), OFF(volumetricLightIntensity) + 8 * i);
  }
  for (int i = 1; i <= 5; i++) {
    I("hybrid_formula_" + std::to_string(i), OFF(hybridFormula) + 4 * (i - 1));
    I("hybrid_iterations_" + std::to_string(i), OFF(hybridIters) + 4 * (i - 1));
    D("hybrid_power_" + std::to_string(i), OFF(hybridPower) + 8 * (i - 1));
  }
  const char *comp[3] = {"alfa", "beta", "gamma"};
  for (int c = 0; c < 3; c++) A(std::string("mandelbox_rotation_main_") + comp[c], OFF(mboxRotationMain) + 8 * c);
  for (int fold = 0; fold < 2; fold++)
    for (int axis = 0; axis < 3; axis++)
      for (int c = 0; c < 3; c++)
        A(std::string("mandelbox_rotation_") + XYZ[axis] + std::to_string(fold + 1) + "_" + comp[c],
          OFF(mboxRotation) + 8 * (9 * fold + 3 * axis + c));
  return t;
}

const std::unordered_map<std::string, Key> &table() {
  static const std::unordered_map<std::string, Key> t = build_table();
  return t;
}

// GetPaletteFromString (src/settings.cpp:94-119): 256 hexadecimal tokens separated by spaces.
bool parse_palette(const char *s, mbgb_rgb *pal) {
  int index = 0;
  const size_t len = strnlen(s, 2000);
  for (size_t i = 0; i < len && i < 2000; i++) {
    unsigned int colour = 0;
    sscanf(&s[i], "%x", &colour);
    const int c = (int)colour;
    pal[index].R = c / 65536;
    pal[index].G = (c / 256) % 256;
    pal[index].B = c % 256;
    while (i < 2000 && i < len && s[i] != ' ') i++;
    index++;
    if (index == 256) return true;
  }
  return false;
}

// g_ascii_strtod: locale-independent; the process keeps the "C" numeric locale.
double atof2(const char *s) { return strtod(s, nullptr); }

}  // namespace

namespace mbgb {

// Applies one key; returns false for unknown keys (LoadOneSetting prints a warning and goes on).
bool scene_set(mbgb_scene *sc, const char *key, const char *value, bool *palette_loaded) {
  const auto &t = table();
  auto it = t.find(key);
  if (it == t.end()) return false;
  char *base = reinterpret_cast<char *>(sc);
  const Key &k = it->second;
  if (!strcmp(key, "N")) {
    sc->N = (double)atoi(value);
    return true;
  }
  switch (k.kind) {
    case Kind::Dbl: *reinterpret_cast<double *>(base + k.off) = atof2(value); break;
    case Kind::Deg: *reinterpret_cast<double *>(base + k.off) = atof2(value) / 180.0 * M_PI; break;
    case Kind::Int: *reinterpret_cast<int32_t *>(base + k.off) = atoi(value); break;
    case Kind::Bool: *reinterpret_cast<uint8_t *>(base + k.off) = atoi(value) != 0; break;
    case Kind::BoolF: *reinterpret_cast<uint8_t *>(base + k.off) = atof(value) != 0.0; break;
    case Kind::Palette:
      if (parse_palette(value, sc->palette) && palette_loaded) *palette_loaded = true;
      break;
    case Kind::Ignore: break;
  }
  return true;
}

}  // namespace mbgb

namespace {

// CRotationMatrix with its identity short-cut (src/algebra.cpp:80-218).
struct Rot {
  double m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  bool zero = true;
  void mul(const double r[9]) {
    double o[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        o[3 * i + j] = m[3 * i + 0] * r[0 + j] + m[3 * i + 1] * r[3 + j] + m[3 * i + 2] * r[6 + j];
    memcpy(m, o, sizeof(o));
    zero = false;
  }
  void rotX(double a) {
    if (a == 0.0) return;
    const double s = sin(a), c = cos(a);
    const double r[9] = {1, 0, 0, 0, c, -s, 0, s, c};
    mul(r);
  }
  void rotY(double a) {
    if (a == 0.0) return;
    const double s = sin(a), c = cos(a);
    const double r[9] = {c, 0, s, 0, 1, 0, -s, 0, c};
    mul(r);
  }
  void rotZ(double a) {
    if (a == 0.0) return;
    const double s = sin(a), c = cos(a);
    const double r[9] = {c, -s, 0, s, c, 0, 0, 0, 1};
    mul(r);
  }
  // SetRotation(double angles[3]): Z(angles[2]) then Y(angles[1]) then X(angles[0])
  void set(const double ang[3]) {
    *this = Rot();
    rotZ(ang[2]);
    rotY(ang[1]);
    rotX(ang[0]);
  }
};

}  // namespace

extern "C" mbgb_status mbgb_scene_set(mbgb_scene *scene, const char *key, const char *value) {
  if (!scene || !key || !value) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_scene_set: NULL argument");
  bool pal = false;
  if (!mbgb::scene_set(scene, key, value, &pal))
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, std::string("unknown parameter: ") + key);
  if (pal) scene->paletteLoaded = 1;
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_scene_finalize(mbgb_scene *p) {
  if (!p) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_scene_finalize: NULL scene");
  // ReadInterface -nogui tail (src/interface.cpp:690-729)
  const int f = p->formula;
  p->analitycDE = (f == 1 || f == 2 || f == 7 || f == 10 || f == 8 || f == 17 || f == 18 || f == 37);
  if (p->image_width <= 0 || p->noOfTiles == 0)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "image_width and tiles must be positive");
  p->resolution = 1.0 / p->image_width / p->noOfTiles;
  p->volumetricLightEnabledAny = 0;
  for (int i = 0; i < 5; i++)
    if (p->volumetricLightEnabled[i]) p->volumetricLightEnabledAny = 1;
  auto div256 = [](mbgb_rgb c) { return mbgb_rgb{c.R / 256, c.G / 256, c.B / 256}; };
  if (p->planeEnable) p->palette[253] = div256(p->primitivePlaneColour);
  if (p->boxEnable) p->palette[252] = div256(p->primitiveBoxColour);
  if (p->invertedBoxEnable) p->palette[251] = div256(p->primitiveInvertedBoxColour);
  if (p->sphereEnable) p->palette[250] = div256(p->primitiveSphereColour);
  if (p->invertedSphereEnable) p->palette[249] = div256(p->primitiveInvertedSphereColour);
  if (p->waterEnable) p->palette[248] = div256(p->primitiveWaterColour);
  // RecalculateIFSParams, Mandelbox part (src/callbacks.cpp:1549-1556)
  Rot main;
  main.set(p->mboxRotationMain);
  memcpy(p->mboxMainRot, main.m, sizeof(main.m));
  p->mboxMainRotZero = main.zero;
  for (int fold = 0; fold < 2; fold++)
    for (int axis = 0; axis < 3; axis++) {
      Rot r;
      r.set(p->mboxRotation[fold][axis]);
      memcpy(p->mboxRot[fold][axis], r.m, sizeof(r.m));
      p->mboxRotZero[fold][axis] = r.zero;
      double tr[9];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) tr[3 * i + j] = r.m[3 * j + i];
      memcpy(p->mboxRotInv[fold][axis], tr, sizeof(tr));
    }
  // IFS directions are normalised there too
  for (int i = 0; i < 9; i++) {
    double *d = p->ifsDirection[i];
    const double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double norm = 1.0 / len;
    d[0] *= norm; d[1] *= norm; d[2] *= norm;
  }
  // CheckPrameters (src/interface.cpp:3587-3602)
  if (p->zoom <= 1e-15) p->zoom = 1e-15;
  if (p->DE_factor <= 0.0001) p->DE_factor = 0.0001;
  if (p->smoothness <= 0.00001) p->smoothness = 0.00001;
  if (p->persp <= 0.001) p->persp = 0.001;
  if (p->globalIlumQuality >= 30) p->globalIlumQuality = 30;
  if (p->globalIlumQuality <= 1) p->globalIlumQuality = 1;
  if (p->image_width < 32) p->image_width = 32;
  if (p->image_height < 32) p->image_height = 32;
  if (p->reflectionsMax > 100) p->reflectionsMax = 100;
  if (p->noOfTiles < 1) p->noOfTiles = 1;
  if (p->noOfTiles > 100) p->noOfTiles = 100;
  if (p->fogDensity < 0.0) p->fogDensity = 0.0;
  if (p->reflect < 0.0) p->reflect = 0.0;
  return MBGB_OK;
}

namespace {

// LoadSettings2 (src/settings.cpp:628-698): token, spaces, value up to ';', rest of line.
mbgb_status load_file(const char *path, mbgb_scene *sc, const std::vector<std::string> &overrides) {
  FILE *fp = fopen(path, "r");
  if (!fp) return mbgb::set_error(MBGB_ERR_IO, std::string("cannot open settings file: ") + path);
  bool palette_loaded = false;
  sc->settingsVersion = -1;
  std::vector<char> str1(100), str2(2000);
  while (!feof(fp)) {
    int c = fscanf(fp, "%99s", str1.data());
    if (c > 0) {
      str2[0] = 0;
      c = fscanf(fp, "%1999[ ]", str2.data());
      str2[0] = 0;
      c = fscanf(fp, "%1999[^;]", str2.data());
      if (c <= 0) str2[0] = 0;
      mbgb::scene_set(sc, str1.data(), str2.data(), &palette_loaded);
      c = fscanf(fp, "%1999[^\n]", str2.data());
    }
  }
  fclose(fp);
  for (const std::string &o : overrides) {
    char k[100], v[2000];
    if (sscanf(o.c_str(), "%99[^= \t]%*1[= ]%1999s", k, v) == 2) mbgb::scene_set(sc, k, v, &palette_loaded);
  }
  // LoadSettingsPost (src/settings.cpp:1185-1195)
  if (!palette_loaded) mbgb_palette_from_seed(sc->coloring_seed, sc->colourSaturation, sc->palette);
  sc->paletteLoaded = palette_loaded;
  return MBGB_OK;
}

// The value of `key` in a settings file as LoadSettings2 reads it (the last line wins);
// false when the key does not occur.
bool find_string(const char *path, const char *key, std::string &value) {
  FILE *fp = fopen(path, "r");
  if (!fp) return false;
  bool found = false;
  std::vector<char> str1(100), str2(2000);
  while (!feof(fp)) {
    int c = fscanf(fp, "%99s", str1.data());
    if (c > 0) {
      str2[0] = 0;
      c = fscanf(fp, "%1999[ ]", str2.data());
      str2[0] = 0;
      c = fscanf(fp, "%1999[^;]", str2.data());
      if (c <= 0) str2[0] = 0;
      if (strcmp(str1.data(), key) == 0) {
        value = str2.data();
        found = true;
      }
      c = fscanf(fp, "%1999[^\n]", str2.data());
    }
  }
  fclose(fp);
  return found;
}

}  // namespace

extern "C" mbgb_status mbgb_settings_string(const char *defaults_path, const char *path,
                                            const char *const *overrides, int n_overrides, const char *key,
                                            char *out, int32_t out_len) {
  if (!path || !key || !out || out_len < 1) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_settings_string: bad argument");
  if (n_overrides < 0 || (n_overrides > 0 && !overrides))
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_settings_string: bad override list");
  std::string value;
  bool found = false;
  if (defaults_path) found = find_string(defaults_path, key, value);
  FILE *probe = fopen(path, "r");
  if (!probe) return mbgb::set_error(MBGB_ERR_IO, std::string("cannot open settings file: ") + path);
  fclose(probe);
  found = find_string(path, key, value) || found;
  for (int i = 0; i < n_overrides; i++) {
    char k[100], v[2000];
    if (overrides[i] && sscanf(overrides[i], "%99[^= \t]%*1[= ]%1999s", k, v) == 2 && strcmp(k, key) == 0) {
      value = v;
      found = true;
    }
  }
  if (!found) return mbgb::set_error(MBGB_ERR_BAD_PARAM, std::string("setting not present: ") + key);
  if ((int32_t)value.size() >= out_len) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "output buffer too small");
  memcpy(out, value.c_str(), value.size() + 1);
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_scene_from_settings(const char *defaults_path, const char *path,
                                                const char *const *overrides, int n_overrides,
                                                mbgb_scene *out) {
  if (!out || !path) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_scene_from_settings: NULL argument");
  if (n_overrides < 0 || (n_overrides > 0 && !overrides))
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_scene_from_settings: bad override list");
  std::vector<std::string> ov;
  for (int i = 0; i < n_overrides; i++) {
    if (!overrides[i]) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "NULL override string");
    ov.emplace_back(overrides[i]);
  }
  mbgb_scene sc;
  memset(&sc, 0, sizeof(sc));
  mbgb_status st;
  if (defaults_path) {
    st = load_file(defaults_path, &sc, ov);
    if (st != MBGB_OK) return st;
  }
  st = load_file(path, &sc, ov);
  if (st != MBGB_OK) return st;
  st = mbgb_scene_finalize(&sc);
  if (st != MBGB_OK) return st;
  *out = sc;
  return MBGB_OK;
}
