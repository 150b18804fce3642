// Test infrastructure: a harness around the reference's OWN settings reader.
//
// oracle/Makefile compiles the reference's src/settings.cpp in place (against
// oracle/ref_stubs_settings) together with the sources of libmbref_post.so and this
// file into oracle/_ref/libmbref_settings.so. A scene is loaded the way the -nogui
// program does it:
//   * LoadSettings (src/settings.cpp:611-626): LoadSettings2 of the defaults file, then
//     of the settings file, each followed by the -o override strings
//     (src/settings.cpp:660-676, kept in noGUIdata.overrideStrings) and LoadSettingsPost
//     (src/settings.cpp:1185-1195: NewPalette from coloring_random_seed unless the file
//     held a palette) — all the reference's compiled code;
//   * the -nogui tail of ReadInterface (src/interface.cpp:690-729) and CheckPrameters
//     (src/interface.cpp:3587-3602), restated here because src/interface.cpp is GTK code;
//     the rotation matrices of RecalculateIFSParams (src/callbacks.cpp:1538-1556) are
//     computed with the reference's own CRotationMatrix and CVector3::Normalize.
// The resulting sParamRender is copied field by field into an mbgb_scene (names follow
// the reference's fields), so tests can compare the library's settings reader with the
// reference's byte for byte. Used only by tests/golden/make_golden.py and the settings
// tests; nothing in the product loads it.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "Render3D.h"
#include "files.h"
#include "interface.h"
#include "mbgb.h"
#include "settings.h"

// defined in src/settings.cpp (no header declares it): set when a file held a palette
extern bool paletteLoadedFromSettingsFile;

// globals src/settings.cpp names that live in the reference's GUI sources
GtkWidget *window_interface = nullptr;
char *sharedDir = nullptr;   // read only by SaveSettings, which the harness never calls
GtkWidget *darea2 = nullptr, *dareaPalette = nullptr;   // src/image.cpp's GUI drawing paths
// KeepOtherSettings (src/settings.cpp:1253) reads the GUI; the harness never calls it
void ReadInterface(sParamRender *) {}
void WriteLog(const char *) {}
bool FileIfExists(const char *filename) {
  FILE *f = fopen(filename, "r");
  if (!f) return false;
  fclose(f);
  return true;
}

namespace {

static_assert(sizeof(CRotationMatrix) == sizeof(CMatrix33) + sizeof(double), "CRotationMatrix layout");

// CRotationMatrix keeps its matrix and `zero` flag private; the class is a CMatrix33 followed
// by the bool, so both are read through that layout.
void rot_out(const CRotationMatrix &r, double m[9], int32_t *zero) {
  const CMatrix33 &a = *reinterpret_cast<const CMatrix33 *>(&r);
  const double v[9] = {a.m11, a.m12, a.m13, a.m21, a.m22, a.m23, a.m31, a.m32, a.m33};
  memcpy(m, v, sizeof(v));
  if (zero) *zero = *reinterpret_cast<const bool *>(reinterpret_cast<const char *>(&r) + sizeof(CMatrix33));
}

void v3(const CVector3 &v, double *o) {
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
}
mbgb_rgb rgb(const sRGB &c) { return mbgb_rgb{c.R, c.G, c.B}; }
sRGB div256(const sRGB &c) {   // sRGBDiv256, src/interface.cpp:3623-3630
  sRGB o;
  o.R = c.R / 256;
  o.G = c.G / 256;
  o.B = c.B / 256;
  return o;
}

// The -nogui tail of ReadInterface (src/interface.cpp:690-729); InterfaceData2Params and
// the palette copy through Interface_data give the loaded values back unchanged in -nogui
// mode (src/Render3D.cpp:1797-1799, 1955; src/interface.cpp:3563-3585).
void nogui_tail(sParamRender *params) {
  const enumFractalFormula f = params->fractal.formula;
  params->fractal.analitycDE = (f == trig_DE || f == trig_optim || f == menger_sponge || f == kaleidoscopic ||
                                f == tglad || f == smoothMandelbox || f == mandelboxVaryScale4D ||
                                f == generalizedFoldBox);
  params->doubles.resolution = 1.0 / params->image_width / params->noOfTiles;
  bool volLightEnabled = false;
  for (int i = 0; i < 5; i++)
    if (params->volumetricLightEnabled[i]) volLightEnabled = true;
  params->imageSwitches.volumetricLightEnabled = volLightEnabled;
  if (params->fractal.primitives.planeEnable) params->palette[253] = div256(params->primitivePlaneColour);
  if (params->fractal.primitives.boxEnable) params->palette[252] = div256(params->primitiveBoxColour);
  if (params->fractal.primitives.invertedBoxEnable) params->palette[251] = div256(params->primitiveInvertedBoxColour);
  if (params->fractal.primitives.sphereEnable) params->palette[250] = div256(params->primitiveSphereColour);
  if (params->fractal.primitives.invertedSphereEnable)
    params->palette[249] = div256(params->primitiveInvertedSphereColour);
  if (params->fractal.primitives.waterEnable) params->palette[248] = div256(params->primitiveWaterColour);
  // RecalculateIFSParams, rotations and direction normalisation (src/callbacks.cpp:1538-1556)
  sFractal &fr = params->fractal;
  fr.IFS.mainRot.SetRotation(fr.IFS.doubles.rotationAlfa, fr.IFS.doubles.rotationBeta, fr.IFS.doubles.rotationGamma);
  for (int i = 0; i < IFS_VECTOR_COUNT; i++) {
    fr.IFS.rot[i].SetRotation(fr.IFS.doubles.alfa[i], fr.IFS.doubles.beta[i], fr.IFS.doubles.gamma[i]);
    fr.IFS.doubles.direction[i].Normalize();
  }
  fr.mandelbox.mainRot.SetRotation(fr.mandelbox.doubles.rotationMain);
  for (int fold = 0; fold < MANDELBOX_FOLDS; ++fold)
    for (int axis = 0; axis < 3; ++axis) {
      fr.mandelbox.rot[fold][axis].SetRotation(fr.mandelbox.doubles.rotation[fold][axis]);
      fr.mandelbox.rotinv[fold][axis] = fr.mandelbox.rot[fold][axis].Transpose();
    }
}

// CheckPrameters (src/interface.cpp:3587-3602), which Render() applies (src/Render3D.cpp:714).
void check_parameters(sParamRender *params) {
  if (params->doubles.zoom <= 1e-15) params->doubles.zoom = 1e-15;
  if (params->doubles.DE_factor <= 0.0001) params->doubles.DE_factor = 0.0001;
  if (params->doubles.smoothness <= 0.00001) params->doubles.smoothness = 0.00001;
  if (params->doubles.persp <= 0.001) params->doubles.persp = 0.001;
  if (params->globalIlumQuality >= 30) params->globalIlumQuality = 30;
  if (params->globalIlumQuality <= 1) params->globalIlumQuality = 1;
  if (params->image_width < 32) params->image_width = 32;
  if (params->image_height < 32) params->image_height = 32;
  if (params->reflectionsMax > 100) params->reflectionsMax = 100;
  if (params->noOfTiles < 1) params->noOfTiles = 1;
  if (params->noOfTiles > 100) params->noOfTiles = 100;
  if (params->doubles.fogDensity < 0.0) params->doubles.fogDensity = 0.0;
  if (params->doubles.imageAdjustments.reflect < 0.0) params->doubles.imageAdjustments.reflect = 0.0;
}

// sParamRender -> mbgb_scene, field by field (mbgb.h keeps the reference's field names).
void to_scene(const sParamRender &p, mbgb_scene *s) {
  memset(s, 0, sizeof(*s));
  const sParamRenderD &d = p.doubles;
  s->zoom = d.zoom; s->DE_factor = d.DE_factor; s->resolution = d.resolution; s->persp = d.persp;
  s->quality = d.quality; s->smoothness = d.smoothness; s->alpha = d.alpha; s->beta = d.beta; s->gamma = d.gamma;
  s->DOFFocus = d.DOFFocus; s->DOFRadius = d.DOFRadius;
  s->mainLightAlpha = d.mainLightAlpha; s->mainLightBeta = d.mainLightBeta;
  s->auxLightIntensity = d.auxLightIntensity; s->auxLightMaxDist = d.auxLightMaxDist;
  s->auxLightDistributionRadius = d.auxLightDistributionRadius; s->auxLightVisibility = d.auxLightVisibility;
  for (int i = 0; i < 4; i++) {
    s->auxLightPreIntensity[i] = d.auxLightPreIntensity[i];
    v3(d.auxLightPre[i], s->auxLightPre[i]);
  }
  s->stereoEyeDistance = d.stereoEyeDistance;
  s->viewDistanceMin = d.viewDistanceMin; s->viewDistanceMax = d.viewDistanceMax;
  for (int i = 0; i < 5; i++) s->volumetricLightIntensity[i] = d.volumetricLightIntensity[i];
  s->fogDensity = d.fogDensity; s->fogColour1Distance = d.fogColour1Distance;
  s->fogColour2Distance = d.fogColour2Distance; s->fogDistanceFactor = d.fogDistanceFactor;
  s->colourSaturation = d.colourSaturation; s->fastAoTune = d.fastAoTune;
  s->iterFogOpacity = d.iterFogOpacity; s->iterFogOpacityTrim = d.iterFogOpacityTrim;
  s->fakeLightsIntensity = d.fakeLightsIntensity; s->fakeLightsVisibility = d.fakeLightsVisibility;
  s->fakeLightsVisibilitySize = d.fakeLightsVisibilitySize; s->shadowConeAngle = d.shadowConeAngle;
  s->primitivePlaneReflect = d.primitivePlaneReflect; s->primitiveBoxReflect = d.primitiveBoxReflect;
  s->primitiveInvertedBoxReflect = d.primitiveInvertedBoxReflect;
  s->primitiveSphereReflect = d.primitiveSphereReflect;
  s->primitiveInvertedSphereReflect = d.primitiveInvertedSphereReflect;
  s->primitiveWaterReflect = d.primitiveWaterReflect;
  const sImageAdjustments &a = d.imageAdjustments;
  s->shading = a.shading; s->directLight = a.directLight; s->ambient = a.ambient; s->specular = a.specular;
  s->reflect = a.reflect; s->globalIlum = a.globalIlum; s->brightness = a.brightness;
  s->glow_intensity = a.glow_intensity; s->fogVisibility = a.fogVisibility; s->coloring_speed = a.coloring_speed;
  s->imageGamma = a.imageGamma; s->paletteOffset = a.paletteOffset; s->mainLightIntensity = a.mainLightIntensity;
  s->contrast = a.contrast;
  v3(d.vp, s->vp);
  v3(d.auxLightRandomCenter, s->auxLightRandomCenter);

  const sFractal &f = p.fractal;
  const sFractalD &fd = f.doubles;
  s->N = fd.N; s->amin = fd.amin; s->amax = fd.amax; s->bmin = fd.bmin; s->bmax = fd.bmax;
  s->cmin = fd.cmin; s->cmax = fd.cmax; s->constantFactor = fd.constantFactor;
  s->FoldingIntPowZfactor = fd.FoldingIntPowZfactor; s->FoldingIntPowFoldFactor = fd.FoldingIntPowFoldFactor;
  s->foldingLimit = fd.foldingLimit; s->foldingValue = fd.foldingValue;
  s->foldingSphericalMin = fd.foldingSphericalMin; s->foldingSphericalFixed = fd.foldingSphericalFixed;
  s->power = fd.power; s->cadd = fd.cadd;
  for (int i = 0; i < HYBRID_COUNT; i++) s->hybridPower[i] = fd.hybridPower[i];
  v3(fd.julia, s->julia);
  v3(fd.fakeLightsOrbitTrap, s->fakeLightsOrbitTrap);
  const sFractalPrimitivesD &pd = fd.primitives;
  v3(pd.planeCentre, s->planeCentre); v3(pd.planeNormal, s->planeNormal);
  v3(pd.boxCentre, s->boxCentre); v3(pd.boxSize, s->boxSize);
  v3(pd.invertedBoxCentre, s->invertedBoxCentre); v3(pd.invertedBoxSize, s->invertedBoxSize);
  v3(pd.sphereCentre, s->sphereCentre); s->sphereRadius = pd.sphereRadius;
  v3(pd.invertedSphereCentre, s->invertedSphereCentre); s->invertedSphereRadius = pd.invertedSphereRadius;
  s->waterHeight = pd.waterHeight; s->waterAmplitude = pd.waterAmplitude; s->waterLength = pd.waterLength;
  s->waterRotation = pd.waterRotation; s->waterAnimSpeed = pd.waterAnimSpeed;

  const sFractalMandelboxD &m = f.mandelbox.doubles;
  for (int c = 0; c < 3; c++) s->mboxRotationMain[c] = m.rotationMain[c];
  for (int fo = 0; fo < 2; fo++)
    for (int ax = 0; ax < 3; ax++)
      for (int c = 0; c < 3; c++) s->mboxRotation[fo][ax][c] = m.rotation[fo][ax][c];
  s->mboxColorFactorX = m.colorFactorX; s->mboxColorFactorY = m.colorFactorY; s->mboxColorFactorZ = m.colorFactorZ;
  s->mboxColorFactorR = m.colorFactorR; s->mboxColorFactorSp1 = m.colorFactorSp1;
  s->mboxColorFactorSp2 = m.colorFactorSp2;
  s->mboxScale = m.scale; s->mboxFoldingLimit = m.foldingLimit; s->mboxFoldingValue = m.foldingValue;
  s->mboxFoldingSphericalMin = m.foldingSphericalMin; s->mboxFoldingSphericalFixed = m.foldingSphericalFixed;
  s->mboxSharpness = m.sharpness; s->mboxSolid = m.solid; s->mboxMelt = m.melt;
  v3(m.offset, s->mboxOffset);
  s->mboxVaryFold = m.vary4D.fold; s->mboxVaryMinR = m.vary4D.minR; s->mboxVaryScaleVary = m.vary4D.scaleVary;
  s->mboxVaryWadd = m.vary4D.wadd; s->mboxVaryRPower = m.vary4D.rPower;
  rot_out(f.mandelbox.mainRot, s->mboxMainRot, &s->mboxMainRotZero);
  for (int fo = 0; fo < 2; fo++)
    for (int ax = 0; ax < 3; ax++) {
      rot_out(f.mandelbox.rot[fo][ax], s->mboxRot[fo][ax], &s->mboxRotZero[fo][ax]);
      rot_out(f.mandelbox.rotinv[fo][ax], s->mboxRotInv[fo][ax], nullptr);
    }

  const sFractalIFSD &id = f.IFS.doubles;
  s->ifsRotationGamma = id.rotationGamma; s->ifsRotationAlfa = id.rotationAlfa;
  s->ifsRotationBeta = id.rotationBeta; s->ifsScale = id.scale;
  for (int i = 0; i < IFS_VECTOR_COUNT; i++) {
    s->ifsDistance[i] = id.distance[i]; s->ifsAlfa[i] = id.alfa[i]; s->ifsBeta[i] = id.beta[i];
    s->ifsGamma[i] = id.gamma[i]; s->ifsIntensity[i] = id.intensity[i];
    v3(id.direction[i], s->ifsDirection[i]);
    s->ifsEnabled[i] = f.IFS.enabled[i];
  }
  v3(id.offset, s->ifsOffset);
  v3(id.edge, s->ifsEdge);

  s->image_width = p.image_width; s->image_height = p.image_height;
  s->globalIlumQuality = p.globalIlumQuality; s->reflectionsMax = p.reflectionsMax;
  s->coloring_seed = p.coloring_seed; s->auxLightRandomSeed = p.auxLightRandomSeed;
  s->auxLightNumber = p.auxLightNumber; s->SSAOQuality = p.SSAOQuality;
  s->startFrame = p.startFrame; s->endFrame = p.endFrame; s->framesPerKeyframe = p.framesPerKeyframe;
  s->imageFormat = p.imageFormat; s->noOfTiles = p.noOfTiles; s->tileCount = p.tileCount;
  s->perspectiveType = (int32_t)p.perspectiveType;
  s->formula = (int32_t)f.formula; s->minN = f.minN; s->frameNo = f.frameNo;
  s->fakeLightsMinIter = f.fakeLightsMinIter; s->fakeLightsMaxIter = f.fakeLightsMaxIter;
  for (int i = 0; i < HYBRID_COUNT; i++) {
    s->hybridIters[i] = f.hybridIters[i];
    s->hybridFormula[i] = (int32_t)f.hybridFormula[i];
  }
  s->genFoldBoxType = (int32_t)f.genFoldBox.type;
  s->waterIterations = f.primitives.waterIterations;

  s->shadow = p.shadow; s->global_ilumination = p.global_ilumination;
  s->fastGlobalIllumination = p.fastGlobalIllumination; s->slowShading = p.slowShading;
  s->texturedBackground = p.texturedBackground; s->background_as_fulldome = p.background_as_fulldome;
  s->SSAOEnabled = p.SSAOEnabled; s->DOFEnabled = p.DOFEnabled;
  for (int i = 0; i < 4; i++) s->auxLightPreEnabled[i] = p.auxLightPreEnabled[i];
  for (int i = 0; i < 5; i++) s->volumetricLightEnabled[i] = p.volumetricLightEnabled[i];
  s->penetratingLights = p.penetratingLights; s->stereoEnabled = p.stereoEnabled;
  s->fishEyeCut = p.fishEyeCut; s->fakeLightsEnabled = p.fakeLightsEnabled;
  s->coloringEnabled = p.imageSwitches.coloringEnabled; s->fogEnabled = p.imageSwitches.fogEnabled;
  s->raytracedReflections = p.imageSwitches.raytracedReflections;
  s->volumetricLightEnabledAny = p.imageSwitches.volumetricLightEnabled;
  s->iterFogEnabled = p.imageSwitches.iterFogEnabled; s->hdrEnabled = p.imageSwitches.hdrEnabled;
  s->limits_enabled = f.limits_enabled; s->iterThresh = f.iterThresh; s->analitycDE = f.analitycDE;
  s->juliaMode = f.juliaMode; s->tgladFoldingMode = f.tgladFoldingMode;
  s->sphericalFoldingMode = f.sphericalFoldingMode; s->interiorMode = f.interiorMode;
  s->hybridCyclic = f.hybridCyclic; s->linearDEmode = f.linearDEmode; s->constantDEThreshold = f.constantDEThreshold;
  s->mboxRotationsEnabled = f.mandelbox.rotationsEnabled;
  s->ifsFoldingMode = f.IFS.foldingMode; s->ifsAbsX = f.IFS.absX; s->ifsAbsY = f.IFS.absY; s->ifsAbsZ = f.IFS.absZ;
  s->ifsMengerSpongeMode = f.IFS.mengerSpongeMode;
  s->planeEnable = f.primitives.planeEnable; s->boxEnable = f.primitives.boxEnable;
  s->invertedBoxEnable = f.primitives.invertedBoxEnable; s->sphereEnable = f.primitives.sphereEnable;
  s->invertedSphereEnable = f.primitives.invertedSphereEnable; s->waterEnable = f.primitives.waterEnable;
  s->onlyPlane = f.primitives.onlyPlane;
  s->paletteLoaded = paletteLoadedFromSettingsFile;

  s->background_color1 = rgb(p.background_color1); s->background_color2 = rgb(p.background_color2);
  s->background_color3 = rgb(p.background_color3);
  for (int i = 0; i < 4; i++) s->auxLightPreColour[i] = rgb(p.auxLightPreColour[i]);
  s->fogColour1 = rgb(p.fogColour1); s->fogColour2 = rgb(p.fogColour2); s->fogColour3 = rgb(p.fogColour3);
  s->primitivePlaneColour = rgb(p.primitivePlaneColour); s->primitiveBoxColour = rgb(p.primitiveBoxColour);
  s->primitiveInvertedBoxColour = rgb(p.primitiveInvertedBoxColour);
  s->primitiveSphereColour = rgb(p.primitiveSphereColour);
  s->primitiveInvertedSphereColour = rgb(p.primitiveInvertedSphereColour);
  s->primitiveWaterColour = rgb(p.primitiveWaterColour);
  s->glow_color1 = rgb(p.effectColours.glow_color1); s->glow_color2 = rgb(p.effectColours.glow_color2);
  s->fogColor = rgb(p.effectColours.fogColor); s->mainLightColour = rgb(p.effectColours.mainLightColour);
  for (int i = 0; i < 256; i++) s->palette[i] = rgb(p.palette[i]);
  s->settingsVersion = p.settingsVersion;
}

void finish(sParamRender *p, mbgb_scene *out) {
  nogui_tail(p);
  check_parameters(p);
  to_scene(*p, out);
}

}  // namespace

extern "C" {

// LoadSettings (defaults file, then `path`, each with the override strings) + the -nogui
// derivations; returns 0, or 1 when a file cannot be read.
int ref_scene_from_settings(const char *defaults_path, const char *path, const char *const *overrides,
                            int n_overrides, mbgb_scene *out) {
  noGUIdata.overrideStrings.clear();
  for (int i = 0; i < n_overrides; i++) noGUIdata.overrideStrings.push_back(overrides[i]);
  sParamRender *p = new sParamRender();   // value-initialised: zeroed like the static noGUIdata
  bool ok = true;
  if (defaults_path) ok = LoadSettings2(defaults_path, *p, true);
  if (ok) ok = LoadSettings2(path, *p, true);
  noGUIdata.overrideStrings.clear();
  if (ok) finish(p, out);
  delete p;
  fflush(stdout);   // the reader's messages leave with the call that printed them
  return ok ? 0 : 1;
}

// LoadOneSetting for each (key, value) pair on a zeroed sParamRender, LoadSettingsPost, and
// the -nogui derivations: the reference's reading of a list of settings lines.
int ref_scene_from_keys(const char *const *keys, const char *const *values, int n, mbgb_scene *out) {
  sParamRender *p = new sParamRender();
  paletteLoadedFromSettingsFile = false;
  for (int i = 0; i < n; i++) LoadOneSetting(keys[i], values[i], *p, true);
  LoadSettingsPost(*p);
  finish(p, out);
  delete p;
  fflush(stdout);
  return 0;
}

}  // extern "C"
