// Test infrastructure: a harness around the reference's OWN hot-path code.
//
// oracle/Makefile compiles the reference's src/fractal.cpp, src/shaders.cpp,
// src/algebra.cpp, src/common_math.cpp and src/primitives.cpp in place (from the
// read-only reference tree, against oracle/ref_stubs) and links them with this
// file into oracle/_ref/libmbref.so. This file supplies what those sources need
// from the GTK-entangled rest of the program:
//   * the counters N_counter, Loop_counter (src/Render3D.cpp:51-52) and histogram
//     (src/image.cpp:24);
//   * cTexture's default white 100x100 bitmap (src/texture.cpp:67-116), since the
//     JPEG-loading file cannot compile here;
//   * the Mandelbox matrices of RecalculateIFSParams (src/callbacks.cpp:1549-1556);
//   * a restatement of RayMarching (src/Render3D.cpp:79-199) with the Random()
//     step jitter behind a switch, and of the MainThread pixel body
//     (src/Render3D.cpp:213-344, 389-589) with its reflection loop.
// Distance estimates, normals, shadows, AO, colouring, background and the
// volumetric pass are the reference's compiled functions.
// Used only by tests/golden/make_golden.py to produce golden vectors.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "Render3D.h"
#include "fractal.h"
#include "mbgb.h"
#include "shaders.h"
#include "morph.hpp"

guint64 N_counter = 0;
guint64 Loop_counter = 0;
#ifndef MBGB_REF_POST   // the post-processing build takes it from src/image.cpp
guint64 histogram[256];
#endif

// ---- cTexture: the default constructor's white bitmap ----
cTexture::cTexture(void) {
  width = 100;
  height = 100;
  loaded = false;
  bitmap = new sRGB8[100 * 100];
  memset(bitmap, 255, sizeof(sRGB8) * 100 * 100);
}
cTexture::~cTexture(void) { delete[] bitmap; }
sRGB8 cTexture::Pixel(double x, double y) {
  sRGB8 black = {0, 0, 0};
  if (x >= 0 && x < width && y >= 0 && y < height - 1.0) return Interpolation(x, y);
  return black;
}
sRGB8 cTexture::Interpolation(double x, double y) {
  sRGB8 c = {0, 0, 0};
  int ix = x, iy = y;
  double rx = (x - (int)x), ry = (y - (int)y);
  sRGB8 k1 = bitmap[iy * width + ix], k2 = bitmap[iy * width + ix + 1];
  sRGB8 k3 = bitmap[(iy + 1) * width + ix], k4 = bitmap[(iy + 1) * width + ix + 1];
  c.R = (k1.R * (1.0 - rx) * (1.0 - ry) + k2.R * (rx) * (1.0 - ry) + k3.R * (1.0 - rx) * ry + k4.R * (rx * ry));
  c.G = (k1.G * (1.0 - rx) * (1.0 - ry) + k2.G * (rx) * (1.0 - ry) + k3.G * (1.0 - rx) * ry + k4.G * (rx * ry));
  c.B = (k1.B * (1.0 - rx) * (1.0 - ry) + k2.B * (rx) * (1.0 - ry) + k3.B * (1.0 - rx) * ry + k4.B * (rx * ry));
  return c;
}
sRGB8 cTexture::FastPixel(int x, int y) { return bitmap[x + y * width]; }

namespace {

sRGB rgb(const mbgb_rgb &c) {
  sRGB o = {c.R, c.G, c.B};
  return o;
}
CVector3 v3(const double *d) { return CVector3(d[0], d[1], d[2]); }

// RecalculateIFSParams' face-normal tables of the generalized fold box (restated: the
// function lives in the GTK-bound src/callbacks.cpp). Only the table of the scene's type
// is filled, with the sides count the formula reads for it.
void set_fold_box(sFractalGeneralizedFoldBox &g, int type) {
  g.type = (enumGeneralizedFoldBoxType)type;
  const double q = 1.0 / sqrt(3.0);
  const CVector3 oct[8] = {CVector3(q, q, -q), CVector3(q, -q, q), CVector3(-q, q, q), CVector3(-q, -q, -q),
                           CVector3(q, q, q), CVector3(-q, -q, q), CVector3(-q, q, -q), CVector3(q, -q, -q)};
  const CVector3 cube[6] = {CVector3(1, 0, 0), CVector3(-1, 0, 0), CVector3(0, 1, 0),
                            CVector3(0, -1, 0), CVector3(0, 0, 1), CVector3(0, 0, -1)};
  for (int i = 0; i < 4; i++) g.Nv_tet[i] = oct[i];
  g.sides_tet = 4;
  for (int i = 0; i < 6; i++) g.Nv_cube[i] = cube[i];
  g.sides_cube = 6;
  for (int i = 0; i < 8; i++) g.Nv_oct[i] = oct[i];
  g.sides_oct = 8;
  for (int i = 0; i < 8; i++) g.Nv_oct_cube[i] = oct[i];
  for (int i = 0; i < 6; i++) g.Nv_oct_cube[8 + i] = cube[i];
  g.sides_oct_cube = 14;
  const double aa = ((1.0 + sqrt(5.0)) / 2.0);
  const double bb = (1.0 / sqrt(aa * aa + 1.0));
  const CVector3 dod[12] = {CVector3(0, bb, aa * bb), CVector3(0, bb, -aa * bb), CVector3(0, -bb, aa * bb),
                            CVector3(0, -bb, -aa * bb), CVector3(bb, aa * bb, 0), CVector3(bb, -aa * bb, 0),
                            CVector3(-bb, aa * bb, 0), CVector3(-bb, -aa * bb, 0), CVector3(aa * bb, 0, bb),
                            CVector3(-aa * bb, 0, bb), CVector3(aa * bb, 0, -bb), CVector3(-aa * bb, 0, -bb)};
  for (int i = 0; i < 12; i++) g.Nv_dodeca[i] = dod[i];
  g.sides_dodeca = 12;
  const double ff = sqrt(aa * aa + 1.0 / (aa * aa));
  const double cc = aa / ff;
  const double dd = 1.0 / aa / ff;
  const CVector3 ico[12] = {CVector3(0, dd, cc), CVector3(0, dd, -cc), CVector3(0, -dd, cc), CVector3(0, -dd, -cc),
                            CVector3(cc, 0, dd), CVector3(cc, 0, -dd), CVector3(-cc, 0, dd), CVector3(-cc, 0, -dd),
                            CVector3(dd, cc, 0), CVector3(dd, -cc, 0), CVector3(-dd, cc, 0), CVector3(-dd, -cc, 0)};
  for (int i = 0; i < 8; i++) g.Nv_icosa[i] = oct[i];
  for (int i = 0; i < 12; i++) g.Nv_icosa[8 + i] = ico[i];
  g.sides_icosa = 20;
  const double tha = 3.14159 * 2.0 / 6.0;
  g.Nv_box6[0] = CVector3(0, 0, 1);
  g.Nv_box6[1] = CVector3(0, 0, -1);
  for (int i = 0; i < 6; i++) g.Nv_box6[2 + i] = CVector3(cos(tha * i), sin(tha * i), 0);
  g.sides_box6 = 8;
  const double tha5 = 3.14159 * 2.0 / 5.0;
  g.Nv_box5[0] = CVector3(0, 0, 1);
  g.Nv_box5[1] = CVector3(0, 0, -1);
  for (int i = 0; i < 5; i++) g.Nv_box5[2 + i] = CVector3(cos(tha5 * i), sin(tha5 * i), 0);
  g.sides_box5 = 7;
}

// CreateFormulaSequence (restated from the GTK-bound src/callbacks.cpp:1666-1702; the loop
// is bounded here, where the reference's would not end for a sequence without iterations).
void make_formula_sequence(sFractal &f) {
  const int N = (int)f.doubles.N;
  f.formulaSequence.resize(N);
  f.hybridPowerSequence.resize(N);
  int number = 0, guard = 0;
  while (number < N && guard++ < 1000000) {
    for (int h = 0; h < HYBRID_COUNT - 1; ++h) {
      if (f.hybridFormula[h] == none) continue;
      for (int i = 0; i < f.hybridIters[h]; ++i) {
        if (number < N) {
          f.formulaSequence[number] = f.hybridFormula[h];
          f.hybridPowerSequence[number] = f.doubles.hybridPower[h];
        }
        number++;
      }
    }
    int end = N;
    if (f.hybridCyclic) end = f.hybridIters[HYBRID_COUNT - 1];
    if (f.hybridFormula[HYBRID_COUNT - 1] != none)
      for (int i = 0; i < end; i++) {
        if (number < N) {
          f.formulaSequence[number] = f.hybridFormula[HYBRID_COUNT - 1];
          f.hybridPowerSequence[number] = f.doubles.hybridPower[HYBRID_COUNT - 1];
        }
        number++;
      }
  }
}

// mbgb_scene -> sParamRender (only what the hot path reads is relevant).
sParamRender *make_params(const mbgb_scene &s) {
  sParamRender *pp = new sParamRender();
  sParamRender &p = *pp;
  sParamRenderD &d = p.doubles;
  d.zoom = s.zoom; d.DE_factor = s.DE_factor; d.resolution = s.resolution; d.persp = s.persp;
  d.quality = s.quality; d.smoothness = s.smoothness; d.alpha = s.alpha; d.beta = s.beta; d.gamma = s.gamma;
  d.DOFFocus = s.DOFFocus; d.DOFRadius = s.DOFRadius; d.mainLightAlpha = s.mainLightAlpha;
  d.mainLightBeta = s.mainLightBeta; d.auxLightIntensity = s.auxLightIntensity; d.auxLightMaxDist = s.auxLightMaxDist;
  d.auxLightDistributionRadius = s.auxLightDistributionRadius; d.auxLightVisibility = s.auxLightVisibility;
  for (int i = 0; i < 4; i++) { d.auxLightPreIntensity[i] = s.auxLightPreIntensity[i]; d.auxLightPre[i] = v3(s.auxLightPre[i]); }
  d.stereoEyeDistance = s.stereoEyeDistance; d.viewDistanceMin = s.viewDistanceMin; d.viewDistanceMax = s.viewDistanceMax;
  for (int i = 0; i < 5; i++) d.volumetricLightIntensity[i] = s.volumetricLightIntensity[i];
  d.fogDensity = s.fogDensity; d.fogColour1Distance = s.fogColour1Distance; d.fogColour2Distance = s.fogColour2Distance;
  d.fogDistanceFactor = s.fogDistanceFactor; d.colourSaturation = s.colourSaturation; d.fastAoTune = s.fastAoTune;
  d.iterFogOpacity = s.iterFogOpacity; d.iterFogOpacityTrim = s.iterFogOpacityTrim;
  d.fakeLightsIntensity = s.fakeLightsIntensity; d.fakeLightsVisibility = s.fakeLightsVisibility;
  d.fakeLightsVisibilitySize = s.fakeLightsVisibilitySize; d.shadowConeAngle = s.shadowConeAngle;
  sImageAdjustments &a = d.imageAdjustments;
  a.shading = s.shading; a.directLight = s.directLight; a.ambient = s.ambient; a.specular = s.specular;
  a.reflect = s.reflect; a.globalIlum = s.globalIlum; a.brightness = s.brightness; a.glow_intensity = s.glow_intensity;
  a.fogVisibility = s.fogVisibility; a.coloring_speed = s.coloring_speed; a.imageGamma = s.imageGamma;
  a.paletteOffset = s.paletteOffset; a.mainLightIntensity = s.mainLightIntensity; a.contrast = s.contrast;
  d.primitivePlaneReflect = s.primitivePlaneReflect; d.primitiveBoxReflect = s.primitiveBoxReflect;
  d.primitiveInvertedBoxReflect = s.primitiveInvertedBoxReflect; d.primitiveSphereReflect = s.primitiveSphereReflect;
  d.primitiveInvertedSphereReflect = s.primitiveInvertedSphereReflect;
  d.primitiveWaterReflect = s.primitiveWaterReflect;
  d.vp = v3(s.vp);
  d.auxLightRandomCenter = v3(s.auxLightRandomCenter);

  sFractal &f = p.fractal;
  f.doubles.N = s.N; f.doubles.amin = s.amin; f.doubles.amax = s.amax; f.doubles.bmin = s.bmin; f.doubles.bmax = s.bmax;
  f.doubles.cmin = s.cmin; f.doubles.cmax = s.cmax; f.doubles.constantFactor = s.constantFactor;
  f.doubles.foldingLimit = s.foldingLimit; f.doubles.foldingValue = s.foldingValue;
  f.doubles.foldingSphericalMin = s.foldingSphericalMin; f.doubles.foldingSphericalFixed = s.foldingSphericalFixed;
  f.doubles.power = s.power; f.doubles.cadd = s.cadd; f.doubles.julia = v3(s.julia);
  f.doubles.fakeLightsOrbitTrap = v3(s.fakeLightsOrbitTrap);
  f.fakeLightsMinIter = s.fakeLightsMinIter; f.fakeLightsMaxIter = s.fakeLightsMaxIter;
  f.minN = s.minN; f.limits_enabled = s.limits_enabled; f.iterThresh = s.iterThresh; f.analitycDE = s.analitycDE;
  f.juliaMode = s.juliaMode; f.tgladFoldingMode = s.tgladFoldingMode; f.sphericalFoldingMode = s.sphericalFoldingMode;
  f.interiorMode = s.interiorMode; f.linearDEmode = s.linearDEmode; f.constantDEThreshold = s.constantDEThreshold;
  f.normalCalculationMode = false; f.formula = (enumFractalFormula)s.formula; f.frameNo = s.frameNo;
  f.IFS.foldingMode = s.ifsFoldingMode;
  // kaleidoscopic IFS (sFractalIFS, src/fractal.h:102-148)
  sFractalIFS &ifs = f.IFS;
  ifs.doubles.rotationAlfa = s.ifsRotationAlfa; ifs.doubles.rotationBeta = s.ifsRotationBeta;
  ifs.doubles.rotationGamma = s.ifsRotationGamma; ifs.doubles.scale = s.ifsScale;
  ifs.doubles.offset = v3(s.ifsOffset); ifs.doubles.edge = v3(s.ifsEdge);
  ifs.absX = s.ifsAbsX; ifs.absY = s.ifsAbsY; ifs.absZ = s.ifsAbsZ; ifs.mengerSpongeMode = s.ifsMengerSpongeMode;
  for (int i = 0; i < IFS_VECTOR_COUNT; i++) {
    ifs.doubles.distance[i] = s.ifsDistance[i]; ifs.doubles.intensity[i] = s.ifsIntensity[i];
    ifs.doubles.alfa[i] = s.ifsAlfa[i]; ifs.doubles.beta[i] = s.ifsBeta[i]; ifs.doubles.gamma[i] = s.ifsGamma[i];
    // mbgb_scene_finalize already normalised the directions, as RecalculateIFSParams does once
    ifs.doubles.direction[i] = v3(s.ifsDirection[i]);
    ifs.enabled[i] = s.ifsEnabled[i];
  }
  // RecalculateIFSParams, IFS part (src/callbacks.cpp:1538-1547)
  ifs.mainRot.SetRotation(ifs.doubles.rotationAlfa, ifs.doubles.rotationBeta, ifs.doubles.rotationGamma);
  for (int i = 0; i < IFS_VECTOR_COUNT; i++)
    ifs.rot[i].SetRotation(ifs.doubles.alfa[i], ifs.doubles.beta[i], ifs.doubles.gamma[i]);
  // generalized fold box normals (src/callbacks.cpp:1557-1663)
  set_fold_box(f.genFoldBox, s.genFoldBoxType);
  f.doubles.FoldingIntPowZfactor = s.FoldingIntPowZfactor;
  f.doubles.FoldingIntPowFoldFactor = s.FoldingIntPowFoldFactor;
  // hybrid sequence (CreateFormulaSequence, src/callbacks.cpp:1666-1702)
  for (int i = 0; i < HYBRID_COUNT; i++) {
    f.hybridFormula[i] = (enumFractalFormula)s.hybridFormula[i];
    f.hybridIters[i] = s.hybridIters[i];
    f.doubles.hybridPower[i] = s.hybridPower[i];
  }
  f.hybridCyclic = s.hybridCyclic;
  make_formula_sequence(f);
  sFractalMandelboxD &m = f.mandelbox.doubles;
  for (int c = 0; c < 3; c++) m.rotationMain[c] = s.mboxRotationMain[c];
  for (int a2 = 0; a2 < 2; a2++)
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 3; c++) m.rotation[a2][b][c] = s.mboxRotation[a2][b][c];
  m.colorFactorX = s.mboxColorFactorX; m.colorFactorY = s.mboxColorFactorY; m.colorFactorZ = s.mboxColorFactorZ;
  m.colorFactorR = s.mboxColorFactorR; m.colorFactorSp1 = s.mboxColorFactorSp1; m.colorFactorSp2 = s.mboxColorFactorSp2;
  m.scale = s.mboxScale; m.foldingLimit = s.mboxFoldingLimit; m.foldingValue = s.mboxFoldingValue;
  m.foldingSphericalMin = s.mboxFoldingSphericalMin; m.foldingSphericalFixed = s.mboxFoldingSphericalFixed;
  m.offset = v3(s.mboxOffset);
  m.vary4D.fold = s.mboxVaryFold; m.vary4D.minR = s.mboxVaryMinR; m.vary4D.scaleVary = s.mboxVaryScaleVary;
  m.vary4D.wadd = s.mboxVaryWadd; m.vary4D.rPower = s.mboxVaryRPower;
  m.sharpness = s.mboxSharpness; m.solid = s.mboxSolid; m.melt = s.mboxMelt;
  f.mandelbox.rotationsEnabled = s.mboxRotationsEnabled;
  // RecalculateIFSParams, Mandelbox part (src/callbacks.cpp:1549-1556)
  f.mandelbox.mainRot.SetRotation(m.rotationMain);
  for (int fold = 0; fold < 2; fold++)
    for (int axis = 0; axis < 3; axis++) {
      f.mandelbox.rot[fold][axis].SetRotation(m.rotation[fold][axis]);
      f.mandelbox.rotinv[fold][axis] = f.mandelbox.rot[fold][axis].Transpose();
    }
  // primitive objects (sFractalPrimitives, src/fractal.h:195-222)
  f.primitives.planeEnable = s.planeEnable; f.primitives.boxEnable = s.boxEnable;
  f.primitives.invertedBoxEnable = s.invertedBoxEnable; f.primitives.sphereEnable = s.sphereEnable;
  f.primitives.invertedSphereEnable = s.invertedSphereEnable; f.primitives.waterEnable = s.waterEnable;
  f.primitives.onlyPlane = s.onlyPlane; f.primitives.waterIterations = s.waterIterations;
  sFractalPrimitivesD &pd = f.doubles.primitives;
  pd.planeCentre = v3(s.planeCentre); pd.planeNormal = v3(s.planeNormal);
  pd.boxCentre = v3(s.boxCentre); pd.boxSize = v3(s.boxSize);
  pd.invertedBoxCentre = v3(s.invertedBoxCentre); pd.invertedBoxSize = v3(s.invertedBoxSize);
  pd.sphereCentre = v3(s.sphereCentre); pd.sphereRadius = s.sphereRadius;
  pd.invertedSphereCentre = v3(s.invertedSphereCentre); pd.invertedSphereRadius = s.invertedSphereRadius;
  pd.waterHeight = s.waterHeight; pd.waterAmplitude = s.waterAmplitude; pd.waterLength = s.waterLength;
  pd.waterRotation = s.waterRotation; pd.waterAnimSpeed = s.waterAnimSpeed;

  p.image_width = s.image_width; p.image_height = s.image_height; p.globalIlumQuality = s.globalIlumQuality;
  p.reflectionsMax = s.reflectionsMax; p.coloring_seed = s.coloring_seed; p.auxLightRandomSeed = s.auxLightRandomSeed;
  p.auxLightNumber = s.auxLightNumber; p.noOfTiles = s.noOfTiles; p.tileCount = s.tileCount;
  p.perspectiveType = (enumPerspectiveType)s.perspectiveType;
  p.shadow = s.shadow; p.global_ilumination = s.global_ilumination; p.fastGlobalIllumination = s.fastGlobalIllumination;
  p.slowShading = s.slowShading; p.texturedBackground = s.texturedBackground; p.penetratingLights = s.penetratingLights;
  p.fishEyeCut = s.fishEyeCut; p.fakeLightsEnabled = s.fakeLightsEnabled;
  for (int i = 0; i < 4; i++) { p.auxLightPreEnabled[i] = s.auxLightPreEnabled[i]; p.auxLightPreColour[i] = rgb(s.auxLightPreColour[i]); }
  for (int i = 0; i < 5; i++) p.volumetricLightEnabled[i] = s.volumetricLightEnabled[i];
  p.imageSwitches.coloringEnabled = s.coloringEnabled; p.imageSwitches.fogEnabled = s.fogEnabled;
  p.imageSwitches.raytracedReflections = s.raytracedReflections;
  p.imageSwitches.volumetricLightEnabled = s.volumetricLightEnabledAny;
  p.imageSwitches.iterFogEnabled = s.iterFogEnabled; p.imageSwitches.hdrEnabled = s.hdrEnabled;
  p.primitivePlaneColour = rgb(s.primitivePlaneColour); p.primitiveBoxColour = rgb(s.primitiveBoxColour);
  p.primitiveInvertedBoxColour = rgb(s.primitiveInvertedBoxColour);
  p.primitiveSphereColour = rgb(s.primitiveSphereColour);
  p.primitiveInvertedSphereColour = rgb(s.primitiveInvertedSphereColour);
  p.primitiveWaterColour = rgb(s.primitiveWaterColour);
  p.background_color1 = rgb(s.background_color1); p.background_color2 = rgb(s.background_color2);
  p.background_color3 = rgb(s.background_color3);
  p.fogColour1 = rgb(s.fogColour1); p.fogColour2 = rgb(s.fogColour2); p.fogColour3 = rgb(s.fogColour3);
  p.effectColours.glow_color1 = rgb(s.glow_color1); p.effectColours.glow_color2 = rgb(s.glow_color2);
  p.effectColours.fogColor = rgb(s.fogColor); p.effectColours.mainLightColour = rgb(s.mainLightColour);
  for (int i = 0; i < 256; i++) p.palette[i] = rgb(s.palette[i]);
  p.lightmapTexture = new cTexture();
  p.envmapTexture = new cTexture();
  p.backgroundTexture = new cTexture();
  return pp;
}

// RayMarching (src/Render3D.cpp:79-199), restated with the jitter behind a switch.
CVector3 ray_marching(sParamRender *param, sFractal *calcParam, CVector3 start, CVector3 direction, double maxScan,
                      bool binaryEnable, sStep *stepBuff, int *buffCount, double *distThreshOut, double *lastDistOut,
                      bool *foundOut, double *depthOut, bool jitter) {
  CVector3 point;
  bool found = false;
  double scan = param->doubles.viewDistanceMin;
  double distThresh = *distThreshOut;
  double dist = 0;
  double search_accuracy = 0.01 * param->doubles.quality;
  double search_limit = 1.0 - search_accuracy;
  double step = param->doubles.viewDistanceMin;
  *buffCount = 0;
  double distThreshInit = *distThreshOut;
  for (int i = 0; i < 10000; i++) {
    point = start + direction * scan;
    bool max_iter = false;
    if (calcParam->constantDEThreshold) distThresh = param->doubles.quality;
    else distThresh = scan * param->doubles.resolution * param->doubles.persp / param->doubles.quality + distThreshInit;
    if (param->perspectiveType == equirectangular || param->perspectiveType == fishEye) distThresh *= M_PI;
    calcParam->doubles.detailSize = distThresh;
    dist = CalculateDistance(point, *calcParam, &max_iter);
    stepBuff[i].distance = dist;
    stepBuff[i].iters = calcParam->itersOut;
    stepBuff[i].distThresh = distThresh;
    if (dist > 3.0) dist = 3.0;
    if (dist < distThresh) {
      found = true;
      break;
    }
    stepBuff[i].step = step;
    const double j = jitter ? (1.0 - Random(1000) / 10000.0) : 1.0;
    if (param->fractal.interiorMode) step = (dist - 0.8 * distThresh) * param->doubles.DE_factor * j;
    else step = (dist - 0.5 * distThresh) * param->doubles.DE_factor * j;
    stepBuff[i].point = point;
    (*buffCount)++;
    scan += step;
    if (scan > maxScan) break;
  }
  if (found && binaryEnable) {
    step *= 0.5;
    for (int i = 0; i < 20; i++) {
      if (dist < distThresh && dist > distThresh * search_limit) {
        break;
      } else {
        if (dist > distThresh) {
          scan += step;
          point = start + direction * scan;
        } else if (dist < distThresh * search_limit) {
          scan -= step;
          point = start + direction * scan;
        }
      }
      if (calcParam->constantDEThreshold) distThresh = param->doubles.quality;
      else distThresh = scan * param->doubles.resolution * param->doubles.persp / param->doubles.quality + distThreshInit;
      bool max_iter = false;
      dist = CalculateDistance(point, *calcParam, &max_iter);
      step *= 0.5;
    }
  }
  *foundOut = found;
  *distThreshOut = distThresh;
  *lastDistOut = dist;
  *depthOut = scan;
  return point;
}

}  // namespace

extern "C" {

// CalculateDistance at points with detailSize = detail[i].
void ref_distance(const mbgb_scene *s, const double *pts, const double *detail, long n, double *dist, int *iters,
                  unsigned char *max_iter) {
  sParamRender *p = make_params(*s);
  sFractal calc = p->fractal;
  for (long i = 0; i < n; i++) {
    calc.doubles.detailSize = detail[i];
    bool mi = false;
    calc.itersOut = -1;
    dist[i] = CalculateDistance(CVector3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]), calc, &mi);
    iters[i] = calc.itersOut;
    max_iter[i] = mi ? 1 : 0;
  }
  delete p;
}

// Compute<colouring> with N x 10 as SurfaceColour calls it (src/shaders.cpp:855-857).
void ref_colour_value(const mbgb_scene *s, const double *pts, long n, double *out) {
  sParamRender *p = make_params(*s);
  sFractal calc = p->fractal;
  calc.doubles.N *= 10;
  for (long i = 0; i < n; i++) out[i] = Compute<colouring>(CVector3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]), calc);
  delete p;
}

// The MainThread pixel body over rows [row0, row1), single thread, reflections off.
int ref_render(const mbgb_scene *s, int row0, int row1, int jitter, const mbgb_image *img) {
  sParamRender *pp = make_params(*s);
  sParamRender &param = *pp;
  const int width = img->width, height = img->height;
  PlaceRandomLights(&param, false);
  int tiles = param.noOfTiles;
  int tile = param.tileCount;
  CVector3 vp = param.doubles.vp;
  double maxDepth = param.doubles.viewDistanceMax;
  double zoom = param.doubles.zoom;
  int AO_quality = param.globalIlumQuality;
  cTexture *lightmap_texture = param.lightmapTexture;
  CRotationMatrix mRot;
  mRot.RotateZ(param.doubles.alpha);
  mRot.RotateX(param.doubles.beta);
  mRot.RotateY(param.doubles.gamma);
  CVector3 baseY(0.0, 1.0, 0.0);
  baseY = mRot.RotateVector(baseY);
  CVector3 vector, shadowVector;
  vector.x = cos(param.doubles.mainLightAlpha - 0.5 * M_PI) * cos(-param.doubles.mainLightBeta);
  vector.y = sin(param.doubles.mainLightAlpha - 0.5 * M_PI) * cos(-param.doubles.mainLightBeta);
  vector.z = sin(-param.doubles.mainLightBeta);
  shadowVector = mRot.RotateVector(vector);
  // per-ray step buffers of the reflection loop (src/Render3D.cpp:260-268)
  int maxRay = param.reflectionsMax;
  if (!param.imageSwitches.raytracedReflections) maxRay = 0;
  struct Refl {
    CVector3 start, viewVector, point;
    bool found;
    int buffCount, objectType;
    double lastDist, depth, distThresh, reflect;
    sStep *stepBuff;
  };
  Refl *reflectBuff = new Refl[maxRay + 2];
  for (int i = 0; i < maxRay + 1; i++) reflectBuff[i].stepBuff = new sStep[10002];
  sStep *stepBuff = new sStep[10002];
  sVectorsAround *vectorsAround = new sVectorsAround[10000];
  int counter = 0;
  int lightMapWidth = lightmap_texture->Width();
  int lightMapHeight = lightmap_texture->Height();
  for (double b = -0.49 * M_PI; b < 0.49 * M_PI; b += 1.0 / AO_quality) {
    for (double a = 0.0; a < 2.0 * M_PI; a += ((2.0 / AO_quality) / cos(b))) {
      CVector3 dd;
      dd.x = cos(a + b) * cos(b);
      dd.y = sin(a + b) * cos(b);
      dd.z = sin(b);
      vectorsAround[counter].alpha = a;
      vectorsAround[counter].beta = b;
      vectorsAround[counter].v = dd;
      int X = (int)((a + b) / (2.0 * M_PI) * lightMapWidth + lightMapWidth * 8.5) % lightMapWidth;
      int Y = (int)(b / (M_PI)*lightMapHeight + lightMapHeight * 8.5) % lightMapHeight;
      vectorsAround[counter].R = lightmap_texture->FastPixel(X, Y).R;
      vectorsAround[counter].G = lightmap_texture->FastPixel(X, Y).G;
      vectorsAround[counter].B = lightmap_texture->FastPixel(X, Y).B;
      if (vectorsAround[counter].R > 10 || vectorsAround[counter].G > 10 || vectorsAround[counter].B > 10) counter++;
      if (counter >= 10000) break;
    }
    if (counter >= 10000) break;
  }
  int vectorsCount = counter;
  double aspectRatio = (double)width / height;
  enumPerspectiveType perspectiveType = param.perspectiveType;
  double fov = param.doubles.persp;
  CVector3 start;
  if (perspectiveType == fishEye || perspectiveType == equirectangular) start = vp;
  else start = vp - baseY * (1.0 / fov * zoom);
  sFractal calcParam = param.fractal;
  calcParam.normalCalculationMode = false;
  double tileXOffset = (tile % tiles);
  double tileYOffset = (tile / tiles);
  for (int yScr = row0; yScr < row1; yScr++) {
    for (int xScr = 0; xScr < width; xScr++) {
      CVector3 viewVector;
      double x2 = ((double)xScr / width / tiles - 0.5 + tileXOffset / tiles) * aspectRatio;
      double z2 = ((double)yScr / height / tiles - 0.5 + tileYOffset / tiles);
      bool hemisphereCut = false;
      if (perspectiveType == fishEye) {
        if (param.fishEyeCut && sqrt(x2 * x2 + z2 * z2) > 0.5 / fov) hemisphereCut = true;
        double x3 = x2 * M_PI, z3 = z2 * M_PI;
        double r = sqrt(x3 * x3 + z3 * z3);
        if (r == 0) {
          viewVector.x = 0.0; viewVector.z = 0.0; viewVector.y = 1.0;
        } else {
          viewVector.x = x3 / r * sin(r * fov);
          viewVector.z = z3 / r * sin(r * fov);
          viewVector.y = cos(r * fov);
        }
        viewVector.Normalize();
      } else if (perspectiveType == equirectangular) {
        double x3 = x2 * M_PI, z3 = z2 * M_PI;
        viewVector.x = sin(fov * x3) * cos(fov * z3);
        viewVector.z = sin(fov * z3);
        viewVector.y = cos(fov * x3) * cos(fov * z3);
        viewVector.Normalize();
      } else {
        viewVector.x = x2 * fov;
        viewVector.y = 1.0;
        viewVector.z = z2 * fov;
      }
      viewVector = mRot.RotateVector(viewVector);
      // the reflection loop of MainThread (src/Render3D.cpp:441-564)
      double distThresh = 0.0;
      CVector3 point;
      CVector3 startRay = start;
      sShaderOutput resultShader = {0.0, 0.0, 0.0, 0.0};
      sShaderOutput objectColour = {0.0, 0.0, 0.0, 0.0};
      int rayEnd = 0;
      int itersAtEnd = 0;
      calcParam.itersOut = 0;  // the iters layer (not a reference output) starts at 0 per pixel
      for (int ray = 0; ray <= maxRay; ray++) {
        Refl &rb = reflectBuff[ray];
        rb.start = startRay;
        rb.viewVector = viewVector;
        rb.found = false;
        rb.buffCount = 0;
        rb.depth = 0;
        rb.lastDist = 0;
        if (!hemisphereCut) {
          point = ray_marching(&param, &calcParam, startRay, viewVector, maxDepth, true, rb.stepBuff, &rb.buffCount,
                               &distThresh, &rb.lastDist, &rb.found, &rb.depth, jitter != 0);
        } else {
          rb.found = false;
        }
        if (ray == 0) itersAtEnd = calcParam.itersOut;
        rb.point = point;
        rb.distThresh = distThresh;
        rb.objectType = calcParam.objectOut;
        if (calcParam.objectOut == objFractal) rb.reflect = param.doubles.imageAdjustments.reflect;
        if (calcParam.objectOut == objWater) rb.reflect = param.doubles.primitiveWaterReflect;
        if (calcParam.objectOut == objPlane) rb.reflect = param.doubles.primitivePlaneReflect;
        if (calcParam.objectOut == objBox) rb.reflect = param.doubles.primitiveBoxReflect;
        if (calcParam.objectOut == objBoxInv) rb.reflect = param.doubles.primitiveInvertedBoxReflect;
        if (calcParam.objectOut == objSphere) rb.reflect = param.doubles.primitiveSphereReflect;
        if (calcParam.objectOut == objSphereInv) rb.reflect = param.doubles.primitiveInvertedSphereReflect;
        rayEnd = ray;
        if (!rb.found) break;
        if (rb.reflect == 0) break;
        startRay = point;
        sShaderInputData sd;
        sd.calcParam = &calcParam;
        sd.param = &param;
        sd.dist_thresh = rb.distThresh;
        sd.calcParam->doubles.detailSize = rb.distThresh;
        sd.lightVect = shadowVector;
        sd.point = point;
        sd.viewVector = viewVector;
        if (param.fractal.constantDEThreshold) sd.delta = rb.depth * param.doubles.resolution * param.doubles.persp;
        else sd.delta = rb.distThresh * param.doubles.quality;
        CVector3 vn = CalculateNormals(sd);
        viewVector = viewVector - vn * viewVector.Dot(vn) * 2.0;
        startRay = startRay + viewVector * rb.distThresh;
      }
      unsigned short opacity16 = 0, alpha16 = 0;
      for (int ray = rayEnd; ray >= 0; ray--) {
        Refl &rb = reflectBuff[ray];
        sShaderOutput objectShader = {0.0, 0.0, 0.0, 0.0};
        sShaderOutput backgroudShader = {0.0, 0.0, 0.0, 0.0};
        sShaderOutput specular = {0.0, 0.0, 0.0, 0.0};
        sShaderInputData in;
        in.calcParam = &calcParam;
        in.param = &param;
        in.dist_thresh = rb.distThresh;
        if (param.fractal.constantDEThreshold) in.delta = rb.depth * param.doubles.resolution * param.doubles.persp;
        else in.delta = rb.distThresh * param.doubles.quality;
        in.calcParam->doubles.detailSize = rb.distThresh;
        in.lightVect = shadowVector;
        in.point = rb.point;
        in.viewVector = rb.viewVector;
        in.eyePoint = start;
        in.vectorsCount = vectorsCount;
        in.vectorsAround = vectorsAround;
        in.lastDist = rb.lastDist;
        in.envMappingTexture = param.envmapTexture;
        in.depth = rb.depth;
        in.stepCount = rb.buffCount;
        in.stepBuff = rb.stepBuff;
        in.objectType = (enumObjectType)rb.objectType;
        if (rb.found) {
          objectShader = ObjectShader(in, &objectColour, &specular);
        } else {
          backgroudShader = BackgroundShader(in);
          rb.depth = 1e20;  // reflectBuff depth only; in.depth keeps the march depth (src/Render3D.cpp:528-541)
        }
        const double reflect = rb.reflect;
        sShaderOutput pixel;
        if (maxRay > 0 && rayEnd > 0 && ray != rayEnd) {
          pixel.R = resultShader.R * reflect + (1.0 - reflect) * (objectShader.R + backgroudShader.R) + specular.R;
          pixel.G = resultShader.G * reflect + (1.0 - reflect) * (objectShader.G + backgroudShader.G) + specular.G;
          pixel.B = resultShader.B * reflect + (1.0 - reflect) * (objectShader.B + backgroudShader.B) + specular.B;
        } else {
          pixel.R = objectShader.R + backgroudShader.R + specular.R;
          pixel.G = objectShader.G + backgroudShader.G + specular.G;
          pixel.B = objectShader.B + backgroudShader.B + specular.B;
        }
        pixel.alpha = objectShader.alpha + backgroudShader.alpha;
        // the reference leaves opacityOut unset when no step group is composited; 0 here
        sShaderOutput opacityOut = {0.0, 0.0, 0.0, 0.0};
        sShaderOutput vol = VolumetricShader(in, pixel, &opacityOut);
        resultShader.R = vol.R;
        resultShader.G = vol.G;
        resultShader.B = vol.B;
        if (ray == 0) {
          opacity16 = (unsigned short)(opacityOut.R * 65535.0);
          alpha16 = (unsigned short)(vol.alpha * 65535.0);
        }
      }
      const long pix = (long)yScr * width + xScr;
      if (img->opacity) img->opacity[pix] = opacity16;
      if (img->alpha) img->alpha[pix] = alpha16;
      if (img->image_float) {
        img->image_float[3 * pix + 0] = resultShader.R;
        img->image_float[3 * pix + 1] = resultShader.G;
        img->image_float[3 * pix + 2] = resultShader.B;
      }
      if (img->colour) {
        img->colour[3 * pix + 0] = objectColour.R * 255;
        img->colour[3 * pix + 1] = objectColour.G * 255;
        img->colour[3 * pix + 2] = objectColour.B * 255;
      }
      const double depth0 = reflectBuff[0].depth;
      if (img->zbuffer) img->zbuffer[pix] = (float)depth0;
      if (img->hit) img->hit[pix] = reflectBuff[0].found ? 1 : 0;
      if (img->iters) img->iters[pix] = itersAtEnd;
      if (img->depth) img->depth[pix] = depth0;
    }
  }
  for (int i = 0; i < maxRay + 1; i++) delete[] reflectBuff[i].stepBuff;
  delete[] reflectBuff;
  delete[] stepBuff;
  delete[] vectorsAround;
  delete param.lightmapTexture;
  delete param.envmapTexture;
  delete param.backgroundTexture;
  delete pp;
  return 0;
}

unsigned long long ref_orbit_counter(void) { return N_counter; }

// CMorph::CatmullRom (src/morph.cpp) over keys[n_keys][size] for frames [0, n_frames).
void ref_catmull_rom(const double *keys, int n_keys, int size, int frames_per_key, int n_frames, double *out) {
  CMorph m(n_keys, size);
  m.SetFramesPerKey(frames_per_key);
  for (int k = 0; k < n_keys; k++) m.AddData(k, const_cast<double *>(keys + (size_t)k * size));
  for (int f = 0; f < n_frames; f++) m.CatmullRom(f, out + (size_t)f * size);
}

}  // extern "C"
