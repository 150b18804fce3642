// C ABI of libmbgb: contexts, per-frame parameter derivation and the render
// entry points that stand in for Render() (src/Render3D.cpp:709).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "kernel_params.h"
#include "launch.h"
#include "mbgb.h"
#include "mbgb_internal.h"
#include "wave_launch.h"


namespace mbgb {

static thread_local std::string g_last_error;

mbgb_status set_error(mbgb_status st, const std::string &msg) {
  g_last_error = msg;
  return st;
}

static mbgb_status cuda_error(cudaError_t e, const char *what) {
  if (e == cudaErrorMemoryAllocation)
    return set_error(MBGB_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return set_error(MBGB_ERR_NO_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
  return set_error(MBGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define MBGB_CUDA(call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_error(e_, #call);  \
  } while (0)

// CRotationMatrix as built by MainThread: RotateZ(alpha), RotateX(beta), RotateY(gamma)
// (src/Render3D.cpp:237-240, src/algebra.cpp:94-143).
struct HostRot {
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
  void apply(const double v[3], double out[3]) const {
    if (zero) {
      out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
      return;
    }
    out[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    out[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
    out[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
  }
};

// Direction table for ray-traced AO (src/Render3D.cpp:272-313) with the default
// all-white 100x100 light map (src/texture.cpp:67-74): every direction is kept.
static std::vector<double> ao_vectors(int quality) {
  std::vector<double> v;
  int counter = 0;
  for (double b = -0.49 * M_PI; b < 0.49 * M_PI; b += 1.0 / quality) {
    for (double a = 0.0; a < 2.0 * M_PI; a += ((2.0 / quality) / cos(b))) {
      v.push_back(cos(a + b) * cos(b));
      v.push_back(sin(a + b) * cos(b));
      v.push_back(sin(b));
      counter++;
      if (counter >= kMaxAOVectors) break;
    }
    if (counter >= kMaxAOVectors) break;
  }
  return v;
}

// The hybrid formula's sequence (CreateFormulaSequence, src/callbacks.cpp:1666-1702) as runs
// of (formula, iterations, power): slots 1-4 that are set and have iterations, then slot 5
// for the rest of the orbit, or for its own iteration count when the sequence is cyclic;
// the runs repeat until the orbit's N entries are filled. Returns the number of runs.
static int hybrid_runs(const mbgb_scene &s, int form[5], int count[5], double power[5]) {
  int n = 0;
  for (int i = 0; i < 4; i++) {
    if (s.hybridFormula[i] == 0 || s.hybridIters[i] <= 0) continue;
    form[n] = s.hybridFormula[i];
    count[n] = s.hybridIters[i];
    power[n] = s.hybridPower[i];
    n++;
  }
  if (s.hybridFormula[4] != 0) {
    const int c = s.hybridCyclic ? s.hybridIters[4] : (int)s.N;
    if (c > 0) {
      form[n] = s.hybridFormula[4];
      count[n] = c;
      power[n] = s.hybridPower[4];
      n++;
    }
  }
  return n;
}

// Whether the orbit of scene s runs formula k: as its formula or as a run of the hybrid
// sequence.
static bool uses_formula(const mbgb_scene &s, int k) {
  if (s.formula == k) return true;
  if (s.formula != 12) return false;
  int form[5], count[5];
  double power[5];
  const int n = hybrid_runs(s, form, count, power);
  for (int i = 0; i < n; i++)
    if (form[i] == k) return true;
  return false;
}

// Face normals of the generalized fold box's polyhedra (RecalculateIFSParams,
// src/callbacks.cpp:1557-1663): tetrahedron, cube, octahedron, dodecahedron, octahedron +
// cube, icosahedron, hexagonal and pentagonal prisms; an unknown type folds like the
// tetrahedron. The prisms use the reference's 3.14159 for pi.
static int gfb_normals(int type, double nv[20][3]) {
  const double si3 = 1.0 / sqrt(3.0);
  const double oct[8][3] = {{si3, si3, -si3}, {si3, -si3, si3}, {-si3, si3, si3}, {-si3, -si3, -si3},
                            {si3, si3, si3},  {-si3, -si3, si3}, {-si3, si3, -si3}, {si3, -si3, -si3}};
  const double cube[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  int n = 0;
  auto put = [&](double x, double y, double z) {
    nv[n][0] = x; nv[n][1] = y; nv[n][2] = z;
    n++;
  };
  switch (type) {
    case 1:  // cube
      for (auto &v : cube) put(v[0], v[1], v[2]);
      break;
    case 2:  // octahedron
      for (auto &v : oct) put(v[0], v[1], v[2]);
      break;
    case 3: {  // dodecahedron
      const double aa = (1.0 + sqrt(5.0)) / 2.0;
      const double bb = 1.0 / sqrt(aa * aa + 1.0);
      put(0, bb, aa * bb); put(0, bb, -aa * bb); put(0, -bb, aa * bb); put(0, -bb, -aa * bb);
      put(bb, aa * bb, 0); put(bb, -aa * bb, 0); put(-bb, aa * bb, 0); put(-bb, -aa * bb, 0);
      put(aa * bb, 0, bb); put(-aa * bb, 0, bb); put(aa * bb, 0, -bb); put(-aa * bb, 0, -bb);
      break;
    }
    case 4:  // octahedron + cube
      for (auto &v : oct) put(v[0], v[1], v[2]);
      for (auto &v : cube) put(v[0], v[1], v[2]);
      break;
    case 5: {  // icosahedron
      const double aa = (1.0 + sqrt(5.0)) / 2.0;
      const double ff = sqrt(aa * aa + 1.0 / (aa * aa));
      const double cc = aa / ff;
      const double dd = 1.0 / aa / ff;
      for (auto &v : oct) put(v[0], v[1], v[2]);
      put(0, dd, cc); put(0, dd, -cc); put(0, -dd, cc); put(0, -dd, -cc);
      put(cc, 0, dd); put(cc, 0, -dd); put(-cc, 0, dd); put(-cc, 0, -dd);
      put(dd, cc, 0); put(dd, -cc, 0); put(-dd, cc, 0); put(-dd, -cc, 0);
      break;
    }
    case 6:
    case 7: {  // hexagonal / pentagonal prism
      const int k = type == 6 ? 6 : 5;
      const double tha = 3.14159 * 2.0 / (double)k;
      put(0, 0, 1);
      put(0, 0, -1);
      for (int i = 0; i < k; i++) put(cos(tha * i), sin(tha * i), 0);
      break;
    }
    default:  // tetrahedron
      for (int i = 0; i < 4; i++) put(oct[i][0], oct[i][1], oct[i][2]);
      break;
  }
  return n;
}

// Rays of the reflection loop per pixel: the camera ray plus reflectionsMax reflections when
// ray-traced reflections are on (src/Render3D.cpp:260-261).
static int reflection_rays(const mbgb_scene &s) {
  return 1 + ((s.raytracedReflections && s.reflectionsMax > 0) ? s.reflectionsMax : 0);
}

// Scenes with primitive objects next to (or instead of) the fractal.
static bool uses_primitives(const mbgb_scene &s) {
  return s.planeEnable || s.boxEnable || s.invertedBoxEnable || s.sphereEnable || s.invertedSphereEnable ||
         s.waterEnable || s.onlyPlane;
}

// Scenes that light with auxiliary lights: random ones or any of the four predefined.
static bool uses_aux_lights(const mbgb_scene &s) {
  if (s.auxLightNumber > 0) return true;
  for (int i = 0; i < 4; i++)
    if (s.auxLightPreEnabled[i]) return true;
  return false;
}

// The volumetric pass samples the march positions and iteration counts (sStep::point,
// iters): visible aux lights, fake lights, volumetric lights, iteration fog.
static bool need_step_points(const mbgb_scene &s) {
  return (uses_aux_lights(s) && s.auxLightVisibility > 0.0) || s.fakeLightsEnabled || s.volumetricLightEnabledAny ||
         s.iterFogEnabled;
}

static bool need_volumetric(const mbgb_scene &s) {
  return (s.glow_intensity != 0.0) || s.fogEnabled || (s.fogDensity > 0.0) || need_step_points(s);
}

// Auxiliary lights of a scene (random ones, then the four predefined): numberOfLights.
static int aux_light_count(const mbgb_scene &s) {
  return uses_aux_lights(s) ? std::max(s.auxLightNumber > 0 ? s.auxLightNumber : 0, 4) : 0;
}

// Scenes the wavefront stages do not carry render on the per-pixel engine.
// Slow shading, environment mapping and primitive objects are composition-stage work the
// wavefront carries; ray-traced reflections are further primary passes, one per depth, except
// with slow shading (whose warp-wide normals serve the camera rays only) or the limit box
// (whose early return leaves itersOut to the next ray, src/fractal.cpp:1252-1262). Auxiliary
// lights are a normal stage, AuxShadow jobs in the shadow stage and their sums in the
// composition, except with slow shading (the jobs need the normals first) or when one shadow
// factor per light and ray would pass 4 GB.
static bool per_pixel_only(const mbgb_scene &s) {
  // volumetric lights, iteration fog and fake lights: samples of the volumetric walk; the
  // shadows they trace take the detailSize of their start (src/fractal.cpp:1291-1293), which
  // the distance post-processing of limits, iteration threshold and interior mode reads as well
  if ((s.volumetricLightEnabledAny || s.iterFogEnabled || s.fakeLightsEnabled) &&
      (s.limits_enabled || s.iterThresh || s.interiorMode || s.slowShading))
    return true;
  if (reflection_rays(s) > 1 && (s.slowShading || s.limits_enabled)) return true;
  if (uses_aux_lights(s)) {
    if (s.slowShading) return true;
    const double rays = (double)s.image_width * s.image_height * reflection_rays(s);
    if (rays * aux_light_count(s) * sizeof(double) > 4e9) return true;
  }
  return false;
}

// The instantiation a scene's kernels run: Compute<orbitTrap> of the fake lights and the
// primitive objects are carried by the run-time formula path only.
static int scene_kernel_formula(const mbgb_scene &s) {
  return kernel_formula(s.formula, s.ifsFoldingMode || s.fakeLightsEnabled || uses_primitives(s));
}

// The instantiation CalculateDistance of a scene runs (the wavefront stages, distance probes,
// light placement): the primitive objects need the run-time formula path.
static int distance_kernel_formula(const mbgb_scene &s) {
  return kernel_formula(s.formula, s.ifsFoldingMode || uses_primitives(s));
}

// The lean FP32 Mandelbox orbit applies: formula 8 without rotations, offset, pre-folds,
// julia or primitive objects, fold value = 2 x fold limit, and min radius <= fixed radius (so
// that the sphere fold is a clamp). The limit box, interior mode and the iteration threshold
// only test the point before the orbit or post-process its result (limit_box, distance_post),
// which every lean path applies.
static bool fast_mandelbox(const mbgb_scene &s) {
  return s.formula == MBGB_FORMULA_TGLAD && !s.mboxRotationsEnabled && s.mboxMainRotZero && !s.juliaMode &&
         !s.tgladFoldingMode && !s.sphericalFoldingMode && !s.ifsFoldingMode && !uses_primitives(s) &&
         s.mboxOffset[0] == 0.0 && s.mboxOffset[1] == 0.0 && s.mboxOffset[2] == 0.0 &&
         s.mboxFoldingValue == 2.0 * s.mboxFoldingLimit &&
         s.mboxFoldingSphericalMin <= s.mboxFoldingSphericalFixed;
}

// The power-8 Mandelbulb orbit without transcendentals applies (formula 2, power 8,
// no pre-folds or primitive objects).
static bool fast_mandelbulb(const mbgb_scene &s) {
  return s.formula == MBGB_FORMULA_TRIG_OPTIM && s.power == 8.0 && !s.tgladFoldingMode && !s.sphericalFoldingMode &&
         !s.ifsFoldingMode && !uses_primitives(s);
}

template <typename T>
static void fill_fractal(const mbgb_scene &s, FractalT<T> &f) {
  memset(&f, 0, sizeof(f));
  f.formula = s.formula;
  f.lean = (fast_mandelbox(s) || fast_mandelbulb(s)) ? 1 : 0;
  f.N = (int)s.N;
  f.N5 = (int)(s.N * 5);
  f.N10 = (int)(s.N * 10);
  f.minN = s.minN;
  f.juliaMode = s.juliaMode;
  f.tgladFoldingMode = s.tgladFoldingMode;
  f.sphericalFoldingMode = s.sphericalFoldingMode;
  f.limits = s.limits_enabled;
  f.iterThresh = s.iterThresh;
  f.interiorMode = s.interiorMode;
  f.distPost = (s.limits_enabled || s.iterThresh || s.interiorMode) ? 1 : 0;
  f.mbRotEnabled = s.mboxRotationsEnabled;
  f.mbMainRotZero = s.mboxMainRotZero;
  f.power = (T)s.power;
  f.constantFactor = (T)s.constantFactor;
  f.bailout = s.bailoutRadius ? (T)s.bailoutRadius : T(100);
  f.bailout2 = f.bailout * f.bailout;
  for (int c = 0; c < 3; c++) {
    f.julia[c] = (T)s.julia[c];
    f.mbOffset[c] = (T)s.mboxOffset[c];
  }
  f.foldingLimit = (T)s.foldingLimit;
  f.foldingValue = (T)s.foldingValue;
  f.sphFixed = (T)s.foldingSphericalFixed;
  f.sphMin = (T)s.foldingSphericalMin;
  f.mbScale = (T)s.mboxScale;
  f.mbFoldLimit = (T)s.mboxFoldingLimit;
  f.mbFoldValue = (T)s.mboxFoldingValue;
  f.mbMinR = (T)s.mboxFoldingSphericalMin;
  f.mbFixedR = (T)s.mboxFoldingSphericalFixed;
  {
    // the same IEEE operations as a device-side derivation (no contraction in host code)
    const T mR2 = f.mbMinR * f.mbMinR, fR2 = f.mbFixedR * f.mbFixedR;
    const T km1 = fR2 / mR2 - T(1);
    f.leanKm1 = km1;
    f.leanSa = km1 > T(0) ? fR2 / km1 : T(0);
    f.leanSb = km1 > T(0) ? T(1) / km1 : T(0);
  }
  f.mbColX = (T)s.mboxColorFactorX;
  f.mbColY = (T)s.mboxColorFactorY;
  f.mbColZ = (T)s.mboxColorFactorZ;
  f.mbColR = (T)s.mboxColorFactorR;
  f.mbColSp1 = (T)s.mboxColorFactorSp1;
  f.mbColSp2 = (T)s.mboxColorFactorSp2;
  for (int i = 0; i < 9; i++) f.mbMainRot[i] = (T)s.mboxMainRot[i];
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 3; b++) {
      f.mbRotZero[a][b] = s.mboxRotZero[a][b];
      for (int i = 0; i < 9; i++) {
        f.mbRot[a][b][i] = (T)s.mboxRot[a][b][i];
        f.mbRotInv[a][b][i] = (T)s.mboxRotInv[a][b][i];
      }
    }
  f.amin = (T)s.amin; f.amax = (T)s.amax;
  f.bmin = (T)s.bmin; f.bmax = (T)s.bmax;
  f.cmin = (T)s.cmin; f.cmax = (T)s.cmax;
  f.mbVaryFold = (T)s.mboxVaryFold;
  f.mbVaryMinR = (T)s.mboxVaryMinR;
  f.mbVaryScaleVary = (T)s.mboxVaryScaleVary;
  f.mbVaryWadd = (T)s.mboxVaryWadd;
  f.mbVaryRPower = (T)s.mboxVaryRPower;
  f.analytic = s.analitycDE;
  f.linearDE = s.linearDEmode;
  if (s.ifsFoldingMode || uses_formula(s, 10)) {
    // RecalculateIFSParams, IFS part (src/callbacks.cpp:1538-1547): SetRotation(alfa, beta,
    // gamma) = RotateZ(alfa) RotateY(beta) RotateX(gamma); the directions were normalised
    // when the scene was finalised
    f.ifsFolding = s.ifsFoldingMode;
    f.ifsAbsX = s.ifsAbsX;
    f.ifsAbsY = s.ifsAbsY;
    f.ifsAbsZ = s.ifsAbsZ;
    f.ifsMenger = s.ifsMengerSpongeMode;
    HostRot mr;
    mr.rotZ(s.ifsRotationAlfa);
    mr.rotY(s.ifsRotationBeta);
    mr.rotX(s.ifsRotationGamma);
    for (int k = 0; k < 9; k++) f.ifsMainRot[k] = (T)mr.m[k];
    f.ifsMainRotZero = mr.zero;
    f.ifsScale = (T)s.ifsScale;
    for (int c = 0; c < 3; c++) {
      f.ifsOffset[c] = (T)s.ifsOffset[c];
      f.ifsEdge[c] = (T)s.ifsEdge[c];
    }
    for (int i = 0; i < 9; i++) {
      f.ifsEnabled[i] = s.ifsEnabled[i];
      HostRot r;
      r.rotZ(s.ifsAlfa[i]);
      r.rotY(s.ifsBeta[i]);
      r.rotX(s.ifsGamma[i]);
      for (int k = 0; k < 9; k++) f.ifsRot[i][k] = (T)r.m[k];
      f.ifsRotZero[i] = r.zero;
      for (int c = 0; c < 3; c++) f.ifsDir[i][c] = (T)s.ifsDirection[i][c];
      f.ifsDist[i] = (T)s.ifsDistance[i];
      f.ifsIntensity[i] = (T)s.ifsIntensity[i];
    }
  }
  if (uses_formula(s, 17)) f.mbSharpness = (T)s.mboxSharpness;
  if (uses_formula(s, 37)) {
    f.mbSolid = (T)s.mboxSolid;
    f.mbMelt = (T)s.mboxMelt;
    double nv[20][3];
    f.gfbSides = gfb_normals(s.genFoldBoxType, nv);
    for (int i = 0; i < f.gfbSides; i++)
      for (int c = 0; c < 3; c++) f.gfbNv[i][c] = (T)nv[i][c];
  }
  if (uses_formula(s, 16)) {
    f.intPowFold = (T)s.FoldingIntPowFoldFactor;
    f.intPowZ = (T)s.FoldingIntPowZfactor;
  }
  if (uses_formula(s, 19)) f.cadd = (T)s.cadd;
  if (s.formula == 12) {
    double power[5];
    f.hybridSegs = hybrid_runs(s, f.hybridForm, f.hybridCount, power);
    for (int i = 0; i < f.hybridSegs; i++) f.hybridPower[i] = (T)power[i];
  }
  if (s.fakeLightsEnabled) {
    for (int c = 0; c < 3; c++) f.fakeTrap[c] = (T)s.fakeLightsOrbitTrap[c];
    f.fakeMinIter = s.fakeLightsMinIter;
    f.fakeMaxIter = s.fakeLightsMaxIter;
  }
  if (uses_primitives(s)) {
    f.planeEnable = s.planeEnable;
    f.boxEnable = s.boxEnable;
    f.invertedBoxEnable = s.invertedBoxEnable;
    f.sphereEnable = s.sphereEnable;
    f.invertedSphereEnable = s.invertedSphereEnable;
    f.waterEnable = s.waterEnable;
    f.onlyPlane = s.onlyPlane;
    f.waterIterations = s.waterIterations;
    f.frameNo = s.frameNo;
    // PrimitivePlane normalises the normal on every call (src/primitives.cpp:15-21)
    const double *nv = s.planeNormal;
    const double norm = 1.0 / sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
    for (int c = 0; c < 3; c++) {
      f.planeCentre[c] = (T)s.planeCentre[c];
      f.planeNormal[c] = (T)(nv[c] * norm);
      f.boxCentre[c] = (T)s.boxCentre[c];
      f.boxSize[c] = (T)s.boxSize[c];
      f.invBoxCentre[c] = (T)s.invertedBoxCentre[c];
      f.invBoxSize[c] = (T)s.invertedBoxSize[c];
      f.sphereCentre[c] = (T)s.sphereCentre[c];
      f.invSphereCentre[c] = (T)s.invertedSphereCentre[c];
    }
    f.sphereRadius = (T)s.sphereRadius;
    f.invSphereRadius = (T)s.invertedSphereRadius;
    f.waterHeight = (T)s.waterHeight;
    f.waterAmplitude = (T)s.waterAmplitude;
    f.waterLength = (T)s.waterLength;
    f.waterRotation = (T)s.waterRotation;
    f.waterAnimSpeed = (T)s.waterAnimSpeed;
  }
}

// MainThread's per-frame preparation (src/Render3D.cpp:213-344) into a kernel parameter block.
template <typename T>
static void fill_params(const mbgb_scene &s, ParamsT<T> &p, const mbgb_opts &o, const T *aoVec, int aoCount) {
  memset(&p, 0, sizeof(p));
  fill_fractal<T>(s, p.f);
  p.width = s.image_width;
  p.height = s.image_height;
  p.tiles = s.noOfTiles;
  p.perspType = s.perspectiveType;
  p.fishEyeCut = s.fishEyeCut;
  p.row_begin = o.row_begin;
  p.row_end = (o.row_end > 0) ? o.row_end : s.image_height;
  p.tileXOffset = (double)(s.tileCount % s.noOfTiles);
  p.tileYOffset = (double)(s.tileCount / s.noOfTiles);
  p.aspect = (double)s.image_width / s.image_height;
  p.fov = s.persp;
  HostRot rot;
  rot.rotZ(s.alpha);
  rot.rotX(s.beta);
  rot.rotY(s.gamma);
  memcpy(p.rot, rot.m, sizeof(p.rot));
  for (int i = 0; i < 9; i++) p.rotf[i] = (float)rot.m[i];
  p.rot_zero = rot.zero;
  const double by[3] = {0.0, 1.0, 0.0};
  double baseY[3];
  rot.apply(by, baseY);
  if (s.perspectiveType == MBGB_PERSP_FISH_EYE || s.perspectiveType == MBGB_PERSP_EQUIRECT) {
    for (int c = 0; c < 3; c++) p.start[c] = s.vp[c];
  } else {
    const double k = 1.0 / s.persp * s.zoom;
    for (int c = 0; c < 3; c++) p.start[c] = s.vp[c] - baseY[c] * k;
  }
  p.viewDistanceMin = (T)s.viewDistanceMin;
  p.viewDistanceMax = (T)s.viewDistanceMax;
  p.resolution = (T)s.resolution;
  p.persp = (T)s.persp;
  p.quality = (T)s.quality;
  p.DE_factor = (T)s.DE_factor;
  p.smoothness = (T)s.smoothness;
  p.resolution_d = s.resolution;
  p.persp_d = s.persp;
  p.quality_d = s.quality;
  p.constantDEThreshold = s.constantDEThreshold;
  p.interiorMode = s.interiorMode;
  p.slowShading = s.slowShading;
  p.jitter = o.jitter;
  p.jitter_seed = o.jitter_seed;
  // main light direction, camera-relative (src/Render3D.cpp:252-256)
  const double lv[3] = {cos(s.mainLightAlpha - 0.5 * M_PI) * cos(-s.mainLightBeta),
                        sin(s.mainLightAlpha - 0.5 * M_PI) * cos(-s.mainLightBeta), sin(-s.mainLightBeta)};
  double lr[3];
  rot.apply(lv, lr);
  for (int c = 0; c < 3; c++) p.lightVect[c] = (T)lr[c];
  const int mlc[3] = {s.mainLightColour.R, s.mainLightColour.G, s.mainLightColour.B};
  for (int c = 0; c < 3; c++) p.mainLight[c] = (T)(s.mainLightIntensity * mlc[c] / 65536.0);
  p.directLight = (T)s.directLight;
  p.shading = (T)s.shading;
  p.specular = (T)s.specular;
  p.globalIlum = (T)s.globalIlum;
  p.shadow = s.shadow;
  p.penetrating = s.penetratingLights;
  const double softRange = tan(s.shadowConeAngle / 180.0 * M_PI);
  p.softRange = (T)softRange;
  // bSoft (src/shaders.cpp:501)
  p.softShadow = (!s.iterFogEnabled && !s.limits_enabled && !s.iterThresh) && softRange > 0.0;
  p.ao = s.global_ilumination;
  p.fastAO = s.fastGlobalIllumination;
  p.aoQuality = s.globalIlumQuality;
  p.fastAoTune = (T)s.fastAoTune;
  p.aoVec = aoVec;
  p.aoCount = aoCount;
  for (int c = 0; c < 3; c++) p.aoWeight[c] = (T)255;
  p.coloring = s.coloringEnabled;
  p.coloringSpeed = (T)s.coloring_speed;
  p.paletteOffset = (T)s.paletteOffset;
  for (int i = 0; i < 256; i++) {
    p.palette[i][0] = s.palette[i].R;
    p.palette[i][1] = s.palette[i].G;
    p.palette[i][2] = s.palette[i].B;
  }
  auto rgb = [](int d[3], const mbgb_rgb &c) { d[0] = c.R; d[1] = c.G; d[2] = c.B; };
  rgb(p.bg1, s.background_color1);
  rgb(p.bg2, s.background_color2);
  rgb(p.bg3, s.background_color3);
  p.glowIntensity = (T)s.glow_intensity;
  rgb(p.glow1, s.glow_color1);
  rgb(p.glow2, s.glow_color2);
  p.postFog = s.fogEnabled;
  p.fogVisibility = (T)pow(10.0, s.fogVisibility / 10 - 16.0);
  rgb(p.fogColor, s.fogColor);
  p.fogDensity = (T)s.fogDensity;
  p.fogC1Dist = (T)s.fogColour1Distance;
  p.fogC2Dist = (T)s.fogColour2Distance;
  p.fogDistFactor = (T)s.fogDistanceFactor;
  rgb(p.fogCol1, s.fogColour1);
  rgb(p.fogCol2, s.fogColour2);
  rgb(p.fogCol3, s.fogColour3);
  p.fogInvC1Dist = (T)(1.0 / s.fogColour1Distance);
  p.fogInvC2Dist = (T)(1.0 / s.fogColour2Distance);
  p.fogInvVisibility = (T)(1.0 / (double)p.fogVisibility);
  p.fogDistFactor2 = p.fogDistFactor * p.fogDistFactor;
  for (int c = 0; c < 3; c++) {
    p.fogColorS[c] = (T)p.fogColor[c] / (T)65536;
    p.fogCol1S[c] = (T)p.fogCol1[c] / (T)65536;
    p.fogCol2S[c] = (T)p.fogCol2[c] / (T)65536;
    p.fogCol3S[c] = (T)p.fogCol3[c] / (T)65536;
  }
  p.auxLightNumber = s.auxLightNumber > 0 ? s.auxLightNumber : 0;
  p.numberOfLights = uses_aux_lights(s) ? std::max(p.auxLightNumber, 4) : 0;
  p.auxLightIntensity = (T)s.auxLightIntensity;
  p.auxLightVisibility = (T)s.auxLightVisibility;
  p.lights = nullptr;
  p.iterFog = s.iterFogEnabled;
  p.volLightAny = s.volumetricLightEnabledAny;
  p.iterFogOpacity = (T)s.iterFogOpacity;
  p.iterFogOpacityTrim = (T)s.iterFogOpacityTrim;
  for (int i = 0; i < 5; i++) {
    p.volLightEnabled[i] = s.volumetricLightEnabled[i];
    p.volLightIntensity[i] = (T)s.volumetricLightIntensity[i];
  }
  rgb(p.mainLightColour, s.mainLightColour);
  p.mainLightIntensity = (T)s.mainLightIntensity;
  p.fakeLights = s.fakeLightsEnabled;
  p.fakeLightsIntensity = (T)s.fakeLightsIntensity;
  p.fakeLightsVisibility = (T)s.fakeLightsVisibility;
  p.fakeLightsVisibilitySize = (T)s.fakeLightsVisibilitySize;
  p.envMapping = !s.raytracedReflections && s.reflect > 0;
  p.reflect = (T)s.reflect;
  rgb(p.primColour[0], s.primitivePlaneColour);
  rgb(p.primColour[1], s.primitiveWaterColour);
  rgb(p.primColour[2], s.primitiveSphereColour);
  rgb(p.primColour[3], s.primitiveInvertedSphereColour);
  rgb(p.primColour[4], s.primitiveBoxColour);
  rgb(p.primColour[5], s.primitiveInvertedBoxColour);
  p.maxRay = reflection_rays(s) - 1;
  const double pr[6] = {s.primitivePlaneReflect, s.primitiveWaterReflect, s.primitiveSphereReflect,
                        s.primitiveInvertedSphereReflect, s.primitiveBoxReflect, s.primitiveInvertedBoxReflect};
  for (int i = 0; i < 6; i++) p.primReflect[i] = (T)pr[i];
  // The volumetric pass changes the pixel only through glow, post fog, volumetric fog and
  // the visible auxiliary lights.
  p.needVolumetric = need_volumetric(s);
}

struct DeviceBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t want) {
    if (bytes >= want) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) bytes = want;
    else ptr = nullptr;
    return e;
  }
};

// Parameter blocks of the FP32 render kernel for one frame, written into caller
// storage (used by the allocation-free entry point; no heap or device allocation).
mbgb_status prepare_frame_f32(const mbgb_scene &scene, const mbgb_opts &o, const float *aoVec, int aoCount,
                              ParamsT<float> *p, FractalT<double> *fd) {
  fill_params<float>(scene, *p, o, aoVec, aoCount);
  fill_fractal<double>(scene, *fd);
  return MBGB_OK;
}

// The ray-traced AO direction table (src/Render3D.cpp:272-313) written into caller
// storage of `max_vectors` x 3 floats; returns the number of directions.
int ao_vectors_into(int quality, float *out, int max_vectors) {
  int counter = 0;
  for (double b = -0.49 * M_PI; b < 0.49 * M_PI; b += 1.0 / quality) {
    for (double a = 0.0; a < 2.0 * M_PI; a += ((2.0 / quality) / cos(b))) {
      if (counter >= max_vectors) return counter;
      out[3 * counter + 0] = (float)(cos(a + b) * cos(b));
      out[3 * counter + 1] = (float)(sin(a + b) * cos(b));
      out[3 * counter + 2] = (float)sin(b);
      counter++;
      if (counter >= kMaxAOVectors) break;
    }
    if (counter >= kMaxAOVectors) break;
  }
  return counter;
}

}  // namespace mbgb

using namespace mbgb;

// Launch configuration of the wavefront stages (mbgb_tuning without the timings).
struct LaunchCfg {
  int tileW = kTileW, tileH = kTileH;   // primary-ray pixel tile of a warp
  int block = 128;                      // threads per CTA
  int ctasPerSm = 0;                    // 0 = the occupancy limit
  // idle lanes before a warp refills: each refill waits on an atomicAdd round trip, so
  // waiting for 8 idle lanes beats refilling every lane at once (1080p Mandelbox: primary
  // 2.97 -> 1.95 ms, shadow/AO 10.6 -> 9.9 ms against a threshold of 1)
  int refill = 8;
  int orbitRefill = -1;                 // ended lean orbits before a warp steps them on (0 = off,
                                        // -1 = by scene: on for the power-8 Mandelbulb's long orbits)
  bool pairRays = false;                // lean FP32 Mandelbox shadow/AO rays two per thread (packed f32x2)
};

// Scene class an autotuned configuration applies to.
using TuneKey = std::array<int, 10>;

// One launch sequence of a render call: frames sharing every non-camera parameter and
// the precision policy (wavefront), or one frame of the per-pixel engine.
struct Group {
  int prec = 1;                  // 0: FP64, 1: FP32 with FP64 refinement
  bool wave = true;
  std::vector<int> frames;       // indices into the call's frames
  int64_t npix = 0;              // full-frame pixels of the group's frames
  int64_t jobs = 0;              // primary jobs (tile-padded pixels in the row range)
  size_t cams_off = 0;           // byte offset of the group's frame table in the context's table buffer
  size_t grad_off = 0;           // differentiable render: byte offset of the group's gradient table
  LaunchCfg cfg;
};

// Device pointers of a differentiable render call (mbgb_render_grad), one per frame.
struct GradRequest {
  const float *const *dL_dimage;   // null or n pointers to [h][w][3]
  float *const *jacobian;          // null or n pointers to [h][w][3][kGradParams]
};

// What a render call enqueued; read back after the stream is synchronised.
struct CallPlan {
  std::vector<Group> groups;
  uint64_t pixels = 0;
  uint64_t frames = 0;
  uint64_t launches = 0;
  bool profile = false;
  bool grad = false;             // the gradient stage runs after composition
};

struct mbgb_context {
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  DeviceBuf step[2][5];          // per-pixel engine: [precision][step, dist, thr, scan, iters], kStepCap records per slot
  DeviceBuf ovstep[2][5];        // overflow passes: kStepSlots records per slot and ray
  DeviceBuf ovlist;              // overflow pixel list (per-pixel engine)
  DeviceBuf control;             // error flag, start time, stage counters
  DeviceBuf fctl;                // per group: wavefront stage counters / per-pixel tile counter (64 B each)
  DeviceBuf cams;                // frame tables of the wavefront groups
  DeviceBuf ao64, ao32;
  int ao_quality = -1;
  int ao_count = 0;
  DeviceBuf out[8];              // device staging for mbgb_render_host / mbgb_render_batch_host
  DeviceBuf wave[2];             // wavefront per-pixel buffers, per precision
  DeviceBuf probe;               // MBGB_PREC_AUTO: distance probes at the ray origins
  DeviceBuf lightprobe;          // PlaceRandomLights: distances at candidate positions
  DeviceBuf lights64, lights32;  // auxiliary light tables of the call's frames
  DeviceBuf tune_out;            // autotuner output layers
  DeviceBuf gradacc;             // differentiable render: per-frame dL/dtheta sums
  DeviceBuf post;                // post-processing: gamma table and SSAO direction tables
  uint64_t gen = 0;              // bumped whenever a scratch buffer is reallocated
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> gev;  // stage events, kStageEvents per group (profile_stages)
  std::map<TuneKey, mbgb_tuning> tunings;
  CallPlan plan;                 // the last call's launches
  // use_graph: the captured launches of the last such call and what they depend on
  std::vector<char> graph_key;
  uint64_t graph_gen = 0;
  cudaGraphExec_t graph = nullptr;
  CallPlan graph_plan;
  std::vector<char> graph_cams;  // host copy of the frame tables the graph reads
  bool cams_hold_graph = false;  // the table buffer holds graph_cams
  mbgb_stats stats{};
  std::mutex mu;

  cudaError_t ensure(DeviceBuf &b, size_t want) {
    void *old = b.ptr;
    cudaError_t e = b.ensure(want);
    if (b.ptr != old) gen++;
    return e;
  }
};

extern "C" const char *mbgb_version(void) { return "mbgb 0.1.0 (sm_103a)"; }

extern "C" const char *mbgb_last_error(void) { return g_last_error.c_str(); }

extern "C" mbgb_status mbgb_scene_supported(const mbgb_scene *s) {
  if (!s) return set_error(MBGB_ERR_BAD_PARAM, "NULL scene");
  if (s->formula != MBGB_FORMULA_TRIG_OPTIM && s->formula != MBGB_FORMULA_TGLAD && !runtime_formula(s->formula))
    return set_error(MBGB_ERR_UNSUPPORTED, "formula " + std::to_string(s->formula) + " is not built on the device");
  if (s->formula == 12) {
    int form[5], count[5];
    double power[5];
    const int runs = hybrid_runs(*s, form, count, power);
    if (runs == 0) return set_error(MBGB_ERR_UNSUPPORTED, "hybrid formula with an empty formula sequence");
    for (int i = 0; i < runs; i++)
      if (form[i] < 1 || form[i] > 37)
        return set_error(MBGB_ERR_UNSUPPORTED, "hybrid sequence formula " + std::to_string(form[i]) +
                                                   " is not built on the device");
  }
  if (s->raytracedReflections && s->reflectionsMax > 10)
    return set_error(MBGB_ERR_UNSUPPORTED, "ray-traced reflections: more than 10 reflections");
  if (s->texturedBackground) return set_error(MBGB_ERR_UNSUPPORTED, "textured background");
  if (s->image_width <= 0 || s->image_height <= 0 || s->image_width > 65536 || s->image_height > 65536)
    return set_error(MBGB_ERR_BAD_PARAM, "image size out of range");
  if (s->noOfTiles < 1) return set_error(MBGB_ERR_BAD_PARAM, "tiles must be >= 1");
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_context_create(int device, mbgb_context **out) {
  if (!out) return set_error(MBGB_ERR_BAD_PARAM, "NULL output");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return set_error(MBGB_ERR_NO_DEVICE, "no CUDA device visible");
  if (device < 0 || device >= n) return set_error(MBGB_ERR_BAD_PARAM, "device index out of range");
  MBGB_CUDA(cudaSetDevice(device));
  mbgb_context *c = new mbgb_context();
  c->device = device;
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    delete c;
    return cuda_error(e, "cudaGetDeviceProperties");
  }
  c->sms = prop.multiProcessorCount;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess) {
    delete c;
    return cuda_error(e, "context stream/event creation");
  }
  *out = c;
  return MBGB_OK;
}

extern "C" void mbgb_context_destroy(mbgb_context *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto &a : c->step)
    for (auto &b : a) b.release();
  for (auto &a : c->ovstep)
    for (auto &b : a) b.release();
  c->ovlist.release();
  for (auto &b : c->wave) b.release();
  c->probe.release();
  c->lightprobe.release();
  c->lights64.release();
  c->lights32.release();
  c->tune_out.release();
  c->gradacc.release();
  c->post.release();
  c->control.release();
  c->fctl.release();
  c->cams.release();
  if (c->graph) cudaGraphExecDestroy(c->graph);
  for (auto ev : c->gev)
    if (ev) cudaEventDestroy(ev);
  c->ao64.release();
  c->ao32.release();
  for (auto &b : c->out) b.release();
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" mbgb_status mbgb_get_stats(const mbgb_context *c, mbgb_stats *out) {
  if (!c || !out) return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  *out = c->stats;
  return MBGB_OK;
}

static mbgb_status ensure_ao(mbgb_context *c, int quality, cudaStream_t s) {
  if (c->ao_quality == quality) return MBGB_OK;
  std::vector<double> v = ao_vectors(quality);
  std::vector<float> vf(v.begin(), v.end());
  MBGB_CUDA(c->ensure(c->ao64, std::max<size_t>(v.size() * sizeof(double), 16)));
  MBGB_CUDA(c->ensure(c->ao32, std::max<size_t>(vf.size() * sizeof(float), 16)));
  MBGB_CUDA(cudaMemcpyAsync(c->ao64.ptr, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  MBGB_CUDA(cudaMemcpyAsync(c->ao32.ptr, vf.data(), vf.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  MBGB_CUDA(cudaStreamSynchronize(s));
  c->ao_quality = quality;
  c->ao_count = (int)(v.size() / 3);
  return MBGB_OK;
}


// Per-frame fields of ParamsT (camera, size, rows, light direction) cleared, so that
// two frames compare equal exactly when one launch sequence can render both.
template <typename T>
static void strip_camera(ParamsT<T> &p) {
  p.width = p.height = p.tiles = p.row_begin = p.row_end = 0;
  p.tileXOffset = p.tileYOffset = p.aspect = p.fov = 0.0;
  memset(p.rot, 0, sizeof(p.rot));
  memset(p.rotf, 0, sizeof(p.rotf));
  p.rot_zero = 0;
  memset(p.start, 0, sizeof(p.start));
  p.resolution = p.persp = T(0);
  p.resolution_d = p.persp_d = 0.0;
  for (int k = 0; k < 3; k++) p.lightVect[k] = T(0);
  p.aoVec = nullptr;
}

// Formulas whose main parameter is the Mandelbox scale (the device's scale_formula).
static bool scale_formula_host(int formula) {
  return formula == 8 || formula == 17 || formula == 18 || formula == 37;
}

// Fractal fields the scene's formula never reads cleared. Keyframe splines leave
// last-bit differences in parameters that stay constant over an animation
// (2 v - 5 v + 4 v - v is not exactly 0 in doubles), and those in unused fields
// must not split a batch.
template <typename T>
static void clear_unused(FractalT<T> &f) {
  if (f.formula == MBGB_FORMULA_TRIG_OPTIM) {
    f.mbRotEnabled = f.mbMainRotZero = 0;
    memset(f.mbRotZero, 0, sizeof(f.mbRotZero));
    f.mbScale = f.mbFoldLimit = f.mbFoldValue = f.mbMinR = f.mbFixedR = T(0);
    f.leanKm1 = f.leanSa = f.leanSb = T(0);
    f.mbColX = f.mbColY = f.mbColZ = f.mbColR = f.mbColSp1 = f.mbColSp2 = T(0);
    for (int k = 0; k < 3; k++) f.mbOffset[k] = T(0);
    memset(f.mbMainRot, 0, sizeof(f.mbMainRot));
    memset(f.mbRot, 0, sizeof(f.mbRot));
    memset(f.mbRotInv, 0, sizeof(f.mbRotInv));
  } else if (f.formula == MBGB_FORMULA_TGLAD) {
    f.power = T(0);
  }
}

// The formula's main parameter (power / Mandelbox scale) travels per frame (FrameCam::fparam).
template <typename T>
static void clear_fparam(FractalT<T> &f) {
  if (scale_formula_host(f.formula)) f.mbScale = T(0);
  else f.power = T(0);
}

// Whether frames a and b can share one launch sequence in precision T: every
// parameter the kernels read, other than the per-frame camera, is equal in the
// form the kernels receive it.
template <typename T>
static bool same_shared(const mbgb_scene &a, const mbgb_scene &b, const mbgb_opts &o) {
  ParamsT<T> pa, pb;
  fill_params<T>(a, pa, o, nullptr, 0);
  fill_params<T>(b, pb, o, nullptr, 0);
  strip_camera(pa);
  strip_camera(pb);
  clear_unused(pa.f);
  clear_unused(pb.f);
  clear_fparam(pa.f);
  clear_fparam(pb.f);
  if (memcmp(&pa, &pb, sizeof(pa)) != 0) return false;
  FractalT<double> fa, fb;
  fill_fractal<double>(a, fa);
  fill_fractal<double>(b, fb);
  clear_unused(fa);
  clear_unused(fb);
  clear_fparam(fa);
  clear_fparam(fb);
  // the lean orbits are chosen per launch sequence
  const bool fastA = fast_mandelbox(a) || fast_mandelbulb(a), fastB = fast_mandelbox(b) || fast_mandelbulb(b);
  return fastA == fastB && memcmp(&fa, &fb, sizeof(fa)) == 0;
}

// Camera, size, rows and output layers of one frame (MainThread's per-frame set-up,
// src/Render3D.cpp:213-344).
template <typename T>
static void fill_cam(const mbgb_scene &s, const mbgb_image &img, const mbgb_opts &o, const LaunchCfg &cfg,
                     FrameCam<T> &cam) {
  ParamsT<T> p;
  fill_params<T>(s, p, o, nullptr, 0);
  memset(&cam, 0, sizeof(cam));
  cam.width = p.width;
  cam.height = p.height;
  cam.tiles = p.tiles;
  cam.row_begin = p.row_begin;
  cam.row_end = p.row_end;
  cam.rot_zero = p.rot_zero;
  cam.tileW = cfg.tileW;
  cam.tileH = cfg.tileH;
  cam.tileXOffset = p.tileXOffset;
  cam.tileYOffset = p.tileYOffset;
  cam.aspect = p.aspect;
  cam.fov = p.fov;
  memcpy(cam.rot, p.rot, sizeof(cam.rot));
  memcpy(cam.rotf, p.rotf, sizeof(cam.rotf));
  memcpy(cam.start, p.start, sizeof(cam.start));
  cam.resolution = p.resolution;
  cam.persp = p.persp;
  cam.resolution_d = p.resolution_d;
  cam.persp_d = p.persp_d;
  for (int k = 0; k < 3; k++) cam.lightVect[k] = p.lightVect[k];
  cam.fparam = (T)(scale_formula_host(s.formula) ? s.mboxScale : s.power);
  cam.fparam_d = scale_formula_host(s.formula) ? s.mboxScale : s.power;
  cam.image_float = img.image_float;
  cam.zbuffer = img.zbuffer;
  cam.alpha = img.alpha;
  cam.opacity = img.opacity;
  cam.colour = img.colour;
  cam.hit = img.hit;
  cam.iters = img.iters;
  cam.depth = img.depth;
}


// Scenes whose distance estimate the dual-number orbit (exact hits, gradients) covers:
// formula 2, or formula 8 without rotations, offset or pre-folds, and the analytic
// estimate without limits, iteration threshold, interior mode or primitive objects.
static mbgb_status level_set_supported(const mbgb_scene &s) {
  if (s.formula != MBGB_FORMULA_TRIG_OPTIM && s.formula != MBGB_FORMULA_TGLAD)
    return set_error(MBGB_ERR_UNSUPPORTED, "exact hits / gradients: formulas 2 and 8 only");
  if (s.tgladFoldingMode || s.sphericalFoldingMode || s.ifsFoldingMode)
    return set_error(MBGB_ERR_UNSUPPORTED, "exact hits / gradients: pre-folds");
  if (s.formula == MBGB_FORMULA_TGLAD &&
      (s.mboxRotationsEnabled || !s.mboxMainRotZero || s.mboxOffset[0] != 0.0 || s.mboxOffset[1] != 0.0 ||
       s.mboxOffset[2] != 0.0))
    return set_error(MBGB_ERR_UNSUPPORTED, "exact hits / gradients: Mandelbox rotations or offset");
  if (s.limits_enabled || s.iterThresh || s.interiorMode)
    return set_error(MBGB_ERR_UNSUPPORTED, "exact hits / gradients: limits, iteration threshold or interior mode");
  if (uses_primitives(s)) return set_error(MBGB_ERR_UNSUPPORTED, "exact hits / gradients: primitive objects");
  if (reflection_rays(s) > 1) return set_error(MBGB_ERR_UNSUPPORTED, "exact hits / gradients: reflections");
  return MBGB_OK;
}

// Shading terms the gradient stage differentiates: Lambert, specular, hard shadows.
static mbgb_status grad_supported(const mbgb_scene &s) {
  if (s.global_ilumination) return set_error(MBGB_ERR_UNSUPPORTED, "gradients: ambient occlusion");
  if (need_volumetric(s)) return set_error(MBGB_ERR_UNSUPPORTED, "gradients: glow or fog");
  if (s.shadow && (s.penetratingLights || tan(s.shadowConeAngle / 180.0 * M_PI) > 0.0))
    return set_error(MBGB_ERR_UNSUPPORTED, "gradients: soft or penetrating shadows");
  // the gradient differentiates the four-sample normal of the fractal
  if (s.slowShading) return set_error(MBGB_ERR_UNSUPPORTED, "gradients: slow shading");
  if (reflection_rays(s) > 1) return set_error(MBGB_ERR_UNSUPPORTED, "gradients: reflections");
  return MBGB_OK;
}

// Gradient-stage inputs of frame i: its loss derivative and Jacobian buffers, its slot of
// the dL/dtheta sums, and the derivatives of the camera-relative light vector
// rot (cos(a) cos(b), sin(a) cos(b), sin(b)), a = alpha - pi/2, b = -beta
// (src/Render3D.cpp:252-256) by alpha and beta.
template <typename T>
static void fill_grad_cam(const mbgb_scene &s, const GradRequest &g, int i, double *acc, GradCam<T> &gc) {
  memset(&gc, 0, sizeof(gc));
  gc.dL_dimage = g.dL_dimage ? g.dL_dimage[i] : nullptr;
  gc.jacobian = g.jacobian ? g.jacobian[i] : nullptr;
  gc.dtheta = acc + (size_t)kGradParams * i;
  static_assert(kGradParams == MBGB_GRAD_PARAMS, "gradient parameter count");
  HostRot rot;
  rot.rotZ(s.alpha);
  rot.rotX(s.beta);
  rot.rotY(s.gamma);
  const double a = s.mainLightAlpha - 0.5 * M_PI, b = -s.mainLightBeta;
  const double da[3] = {-sin(a) * cos(b), cos(a) * cos(b), 0.0};
  const double db[3] = {cos(a) * sin(b), sin(a) * sin(b), -cos(b)};
  double ra[3], rb[3];
  rot.apply(da, ra);
  rot.apply(db, rb);
  for (int k = 0; k < 3; k++) {
    gc.dLight[0][k] = (T)ra[k];
    gc.dLight[1][k] = (T)rb[k];
  }
}

static TuneKey tune_key(const mbgb_scene &s, int prec) {
  return TuneKey{s.formula, (int)(fast_mandelbox(s) || fast_mandelbulb(s)), prec, (int)need_volumetric(s),
                 s.shadow, s.global_ilumination, s.fastGlobalIllumination, s.globalIlumQuality, s.perspectiveType,
                 s.interiorMode};
}

// Launch configuration of a group: explicit options first, then the cached autotuning
// (opts.autotune), then the defaults.
static LaunchCfg resolve_cfg(const mbgb_context *c, const mbgb_opts &o, const mbgb_scene &s, int prec) {
  LaunchCfg cfg;
  if (o.autotune) {
    auto it = c->tunings.find(tune_key(s, prec));
    if (it != c->tunings.end()) {
      cfg.tileW = it->second.tile_w;
      cfg.tileH = it->second.tile_h;
      cfg.block = it->second.threads_per_cta;
      cfg.ctasPerSm = it->second.ctas_per_sm;
      cfg.refill = it->second.refill_min;
      cfg.orbitRefill = it->second.orbit_refill;
    }
  }
  if (o.tile_w > 0 && o.tile_h > 0) {
    cfg.tileW = o.tile_w;
    cfg.tileH = o.tile_h;
  }
  if (o.threads_per_cta > 0) cfg.block = o.threads_per_cta;
  if (o.ctas_per_sm > 0) cfg.ctasPerSm = o.ctas_per_sm;
  if (o.refill_min > 0) cfg.refill = o.refill_min;
  if (o.orbit_refill != 0) cfg.orbitRefill = o.orbit_refill < 0 ? 0 : o.orbit_refill;
  if (o.pair_rays > 0) cfg.pairRays = true;
  // Orbit-granular refill pays where orbit lengths spread widely (Mandelbulb, N up to
  // hundreds); the Mandelbox's short orbits (bailout 1024 within ~15 iterations) lose more
  // to the extra step passes than they gain (measured at 1080p: 11.2 ms per-estimate
  // refill, 12.5-17.7 ms orbit refill 24-1).
  if (cfg.orbitRefill < 0) cfg.orbitRefill = fast_mandelbulb(s) ? 8 : 0;
  return cfg;
}

// Byte layout of the wavefront buffers for `npix` pixels (256-byte aligned pieces).
struct WaveLayout {
  size_t flags, scan, dist, thr, step, detail, bis, point, iters, count, vol, shadow, ao, hit, pol, ovl, last;
  size_t prec, pprev;
  size_t rstart, rdir, rthr, rlist, normal, auxsh, sbase, sray, srec, sstep, sres, piters, segc, hset;
  uint32_t poolCap;
  size_t total;
};

// `npixFrame` pixels with `rays` rays each (the reflection loop's depths): every per-ray array
// holds rays x npixFrame entries.
// `auxN` auxiliary lights: hit normals, and with `auxShadows` one AuxShadow factor per light.
// `sampleRes` > 0 (volumetric lights, iteration fog): the volumetric walk's samples (at most
// one per pool record) with `sampleRes` results each; `iterFog`: the records' itersOut.
// `jobs`: the primary jobs of the group, over which the hit list's compaction walks.
static WaveLayout wave_layout(int64_t npixFrame, size_t ts, int aoN, bool needVol, int rays, int auxN,
                              bool auxShadows, int sampleRes, bool iterFog, int64_t jobs) {
  const int64_t npix = npixFrame * rays;
  WaveLayout w{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off += (bytes + 255) & ~(size_t)255;
    return at;
  };
  w.flags = take(npix);
  w.scan = take(npix * ts);
  w.dist = take(npix * ts);
  w.thr = take(npix * ts);
  w.step = take(npix * ts);
  w.detail = take(npix * ts);
  w.bis = take(npix * 4);
  w.point = take(3 * npix * ts);
  w.iters = take(npix * 4);
  w.count = take(npix * 4);
  w.vol = take((needVol ? 6 : 1) * npix * ts);
  w.shadow = take(npix * ts);
  w.ao = take((size_t)aoN * npix * ts);
  w.hit = take(npix * 4);
  w.pol = take(npix * 4);
  w.ovl = take(npix * 4);
  w.last = take(npix * 4);
  // rays beyond the pool take the overflow pass (exact, but one ray per thread of a narrow
  // pass); with reflections every depth's rays share it
  const int64_t chunksPerPixel = rays > 1 ? (int64_t)kPoolChunksPerReflectedRay * rays : kPoolChunksPerPixel;
  int64_t chunks = npixFrame * chunksPerPixel;
  if (rays > 1) chunks = std::min<int64_t>(chunks, (int64_t)(8e9 / (kChunk * 4 * ts)));   // 8 GB at most
  w.poolCap = needVol ? (uint32_t)std::min<int64_t>(chunks, 0x7fffffff) : 1u;
  w.prec = take((size_t)w.poolCap * kChunk * 4 * ts);
  w.pprev = take((size_t)w.poolCap * 4);
  const size_t refl = rays > 1 ? (size_t)npix : 0;
  w.rstart = take(3 * refl * sizeof(double));
  w.rdir = take(3 * refl * sizeof(double));
  w.rthr = take(refl * sizeof(double));
  w.rlist = take((rays > 1 ? (size_t)npixFrame : 0) * 4);
  w.normal = take(auxN > 0 ? 3 * (size_t)npix * ts : 0);
  w.auxsh = take(auxN > 0 && auxShadows ? (size_t)auxN * npix * ts : 0);
  const size_t samples = sampleRes > 0 && needVol ? (size_t)w.poolCap * kChunk : 0;
  w.sbase = take(sampleRes > 0 ? (size_t)npix * 4 : 0);
  w.sray = take(samples * 4);
  w.srec = take(samples * 4);
  w.sstep = take(samples * ts);
  w.sres = take(samples * (size_t)sampleRes * ts);
  w.piters = take(iterFog && needVol ? (size_t)w.poolCap * kChunk * 4 : 0);
  w.segc = take(rays == 1 ? (size_t)((jobs + kHitSeg - 1) / kHitSeg) * kHitSegWarps * 4 : 0);
  w.hset = take(rays == 1 ? (size_t)npix * 8 * ts : 0);
  w.total = off;
  return w;
}

template <typename T>
static int wave_occupancy(int formula, int block, int which) {
  if constexpr (sizeof(T) == 8) return occupancy_wave_f64(formula, block, which);
  else return occupancy_wave_f32(formula, block, which);
}

// Enqueue the wavefront stages (wave_core.cuh) of one group: primary rays, FP64 polish
// (FP32 policy), shadow/AO rays, composition. No host round trips.
template <typename T>
static mbgb_status enqueue_wave(mbgb_context *c, const mbgb_scene *scenes, const Group &g, const mbgb_opts &o,
                                cudaStream_t s, FrameIO io, uint32_t *ctl, cudaEvent_t *ev, bool grad,
                                uint64_t *launches, int64_t lightOff) {
  const mbgb_scene &scene = scenes[g.frames[0]];
  const int prec = sizeof(T) == 8 ? 0 : 1;
  const bool needVol = need_volumetric(scene);
  const bool rayAO = scene.global_ilumination && !scene.fastGlobalIllumination;
  const int aoN = rayAO ? c->ao_count : 0;
  const int rays = reflection_rays(scene);
  const int auxN = aux_light_count(scene);
  const bool volLights =
      scene.volumetricLightEnabledAny != 0 || scene.iterFogEnabled != 0 || scene.fakeLightsEnabled != 0;
  const int sampleRes =
      volLights ? kSampleShadows + (scene.iterFogEnabled ? aoN : 0) + (scene.fakeLightsEnabled ? 1 : 0) : 0;
  const WaveLayout w = wave_layout(g.npix, sizeof(T), aoN, needVol, rays, auxN, scene.shadow != 0, sampleRes,
                                   scene.iterFogEnabled != 0, g.jobs);
  char *base = (char *)c->wave[prec].ptr;
  WaveLaunch<T> L;
  WaveBufs<T> &wb = L.wb;
  wb.flags = (uint8_t *)(base + w.flags);
  wb.scan = (T *)(base + w.scan);
  wb.dist = (T *)(base + w.dist);
  wb.thr = (T *)(base + w.thr);
  wb.step = (T *)(base + w.step);
  wb.detail = (T *)(base + w.detail);
  wb.bis_left = (int32_t *)(base + w.bis);
  wb.point = (T *)(base + w.point);
  wb.iters = (int32_t *)(base + w.iters);
  wb.count = (int32_t *)(base + w.count);
  wb.vol = (T *)(base + w.vol);
  wb.shadow = (T *)(base + w.shadow);
  wb.ao = (T *)(base + w.ao);
  wb.hit_list = (uint32_t *)(base + w.hit);
  wb.polish_list = (uint32_t *)(base + w.pol);
  wb.overflow_list = (uint32_t *)(base + w.ovl);
  wb.ctl = ctl;
  wb.last_chunk = (int32_t *)(base + w.last);
  wb.pool_rec = (T *)(base + w.prec);
  wb.pool_prev = (int32_t *)(base + w.pprev);
  wb.pool_cap = w.poolCap;
  wb.polish_all = o.polish_all;
  wb.refill_min = g.cfg.refill;
  wb.orbit_refill = g.cfg.orbitRefill;
  wb.exact_hit = o.exact_hit ? 1 : 0;
  wb.npix = g.npix * rays;
  wb.npix_frame = g.npix;
  wb.rays = rays;
  wb.depth = 0;
  wb.ray_start = (double *)(base + w.rstart);
  wb.ray_dir = (double *)(base + w.rdir);
  wb.ray_thr0 = (double *)(base + w.rthr);
  wb.ray_list = (uint32_t *)(base + w.rlist);
  wb.normal = auxN > 0 ? (T *)(base + w.normal) : nullptr;
  wb.auxsh = auxN > 0 && scene.shadow ? (T *)(base + w.auxsh) : nullptr;
  wb.sample_base = volLights ? (uint32_t *)(base + w.sbase) : nullptr;
  wb.sample_ray = volLights && needVol ? (uint32_t *)(base + w.sray) : nullptr;
  wb.sample_rec = volLights && needVol ? (int32_t *)(base + w.srec) : nullptr;
  wb.sample_step = volLights && needVol ? (T *)(base + w.sstep) : nullptr;
  wb.sample_res = volLights && needVol ? (T *)(base + w.sres) : nullptr;
  wb.sample_cap = volLights && needVol ? w.poolCap * (uint32_t)kChunk : 0u;
  wb.sample_nres = sampleRes;
  wb.pool_iters = scene.iterFogEnabled && needVol ? (int32_t *)(base + w.piters) : nullptr;
  // the hit list in tile order for the shadow stage (one ray per pixel): opts.hit_order 0 from
  // 2^20 pixels on (measured at 1080p: shadow stage 9.79 -> 9.34 ms for ~0.05 ms of
  // compaction, which a 640x480 frame does not earn back), 2 always, 1 never
  const bool tileOrder = o.hit_order == 2 || (o.hit_order == 0 && g.npix >= (int64_t)1 << 20);
  wb.seg_count = rays == 1 && tileOrder ? (uint32_t *)(base + w.segc) : nullptr;
  // shadow/AO rays two per thread (secondary_pair_kernel): the lean FP32 Mandelbox with
  // per-estimate refill, which the pair kernel's packed orbit serves
  wb.pair_rays = (sizeof(T) == 4 && fast_mandelbox(scene) && g.cfg.pairRays && g.cfg.orbitRefill <= 0) ? 1 : 0;
  MBGB_CUDA(cudaMemsetAsync(ctl, 0, 64, s));

  const int block = g.cfg.block;
  const int kf = distance_kernel_formula(scene);
  int occ1 = std::max(1, wave_occupancy<T>(kf, block, 0));
  int occ2 = std::max(1, wave_occupancy<T>(kf, block, wb.pair_rays ? 2 : 1));
  if (g.cfg.ctasPerSm > 0) {
    occ1 = std::min(occ1, g.cfg.ctasPerSm);
    occ2 = std::min(occ2, g.cfg.ctasPerSm);
  }
  L.grid = c->sms * occ1;
  L.grid2 = c->sms * occ2;
  L.block = block;
  L.ov_grid = std::max(1, kWaveOverflowThreads / block);
  L.polish_grid = c->sms * 8;
  L.compose_grid = (int)std::max<int64_t>(1, std::min<int64_t>((g.npix + block - 1) / block, (int64_t)c->sms * 32));
  L.cams = (const FrameCam<T> *)((char *)c->cams.ptr + g.cams_off);
  L.gcams = grad ? (const GradCam<T> *)((char *)c->cams.ptr + g.grad_off) : nullptr;
  L.grad_grid = L.compose_grid;
  L.ncams = (int)g.frames.size();
  L.hit_jobs = g.jobs;
  io.slots = (int64_t)L.grid * block;
  io.step_cap = kStepCap;
  io.overflow_pass = 0;
  L.io = io;
  L.ov = io;
  L.ov.overflow_pass = 1;
  L.ov.step_cap = kStepSlots;
  L.ov.slots = kWaveOverflowThreads;
  L.ov.step_step = c->ovstep[prec][0].ptr;
  L.ov.step_dist = c->ovstep[prec][1].ptr;
  L.ov.step_thr = c->ovstep[prec][2].ptr;
  // the visible auxiliary lights of a long ray sample its record positions
  L.ov.step_scan = need_step_points(scene) ? c->ovstep[prec][3].ptr : nullptr;
  L.ov.step_iters = need_step_points(scene) ? (int *)c->ovstep[prec][4].ptr : nullptr;
  L.overflow = needVol;
  for (int k = 0; k < kStageEvents; k++) L.ev[k] = ev ? ev[k] : nullptr;
  // the FAST instantiations hold no limit box test: limit-box scenes take the generic kernels,
  // whose CalculateDistance runs the lean orbit after the box test (FractalT::lean)
  L.fast = (fast_mandelbox(scene) || fast_mandelbulb(scene)) && !scene.limits_enabled;
  fill_fractal<double>(scene, L.fd);
  fill_params<T>(scene, L.p, o, (const T *)(prec == 0 ? c->ao64.ptr : c->ao32.ptr), c->ao_count);
  if (lightOff >= 0)
    L.p.lights = (const LightT<T> *)(prec == 0 ? c->lights64.ptr : c->lights32.ptr) + lightOff;
  else if (auxN > 0)
    return set_error(MBGB_ERR_CUDA, "auxiliary lights were not placed");
  // the plain variant's per-hit shadow/AO set-up (hit_setup_kernel), formed once per hit in
  // hit-list order; the effects variant sets its jobs up itself. Decided with the same test
  // as the device's launch sequence.
  const bool efx = rays > 1 || L.p.numberOfLights > 0 || L.p.volLightAny || L.p.iterFog || L.p.fakeLights;
  const bool secondaryJobs = scene.shadow != 0 || rayAO;
  wb.hit_setup = (!efx && rays == 1 && secondaryJobs) ? (T *)(base + w.hset) : nullptr;
  cudaError_t e;
  if constexpr (sizeof(T) == 8) e = launch_wave_f64(L, s);
  else e = launch_wave_f32(L, s);
  if (e != cudaSuccess) return cuda_error(e, "wavefront launch");
  // per ray depth: primary (+ overflow) pass and polish; per further depth the reflect and
  // counter kernels
  *launches += 2 + (int64_t)rays * (1 + (needVol ? 1 : 0) + (prec == 1 ? 1 : 0)) + 2 * (int64_t)(rays - 1) +
               (wb.normal ? 1 : 0) + (wb.sample_ray ? 1 : 0) + (wb.seg_count ? 3 : 0) + (wb.exact_hit ? 1 : 0) +
               (wb.hit_setup ? 1 : 0) +
               (grad ? 1 : 0);
  return MBGB_OK;
}

// Enqueue the per-pixel engine (render_core.cuh) for one frame: main pass, then (when
// the step buffer is in use) the overflow pass.
// CTAs per SM of the per-pixel engine: the occupancy limit (or the tuned value), lowered when
// the step records of the reflection loop's rays (thread slots x rays x kStepCap records)
// would pass 16 GB.
static int per_pixel_ctas(const mbgb_scene &scene, int prec, const LaunchCfg &cfg, int sms) {
  int per_sm = std::max(1, occupancy_render(prec, scene_kernel_formula(scene), cfg.block));
  if (cfg.ctasPerSm > 0) per_sm = std::min(per_sm, cfg.ctasPerSm);
  const int rays = reflection_rays(scene);
  if (rays > 1 && need_volumetric(scene)) {
    const double esz = prec == 0 ? 8.0 : 4.0;
    const double perSlot = (double)rays * kStepCap * (3 * esz + (need_step_points(scene) ? esz + 4 : 0));
    const double cap = 16e9 / (perSlot * (double)sms * cfg.block);
    per_sm = std::max(1, std::min(per_sm, (int)cap));
  }
  return per_sm;
}

// Thread slots of the per-pixel engine's overflow pass (pixels whose rays need more than
// kStepCap records): 2048, fewer when their kStepSlots records per ray of the reflection loop
// would pass 4 GB.
static int overflow_slots(const mbgb_scene &scene, int prec) {
  const double esz = prec == 0 ? 8.0 : 4.0;
  const double perSlot =
      (double)reflection_rays(scene) * kStepSlots * (3 * esz + (need_step_points(scene) ? esz + 4 : 0));
  const int slots = (int)std::min(2048.0, 4e9 / perSlot);
  return std::max(kOverflowThreads, slots / 128 * 128);
}

static mbgb_status enqueue_per_pixel(mbgb_context *c, const mbgb_scene &scene, const mbgb_image &img,
                                     const Group &g, const mbgb_opts &o, cudaStream_t s, FrameIO io, char *fctl,
                                     uint64_t *launches, int64_t lightOff) {
  const int prec = g.prec;
  const int block = g.cfg.block;
  const int kf = scene_kernel_formula(scene);
  const int grid = c->sms * per_pixel_ctas(scene, prec, g.cfg, c->sms);
  io.image_float = img.image_float;
  io.zbuffer = img.zbuffer;
  io.alpha = img.alpha;
  io.opacity = img.opacity;
  io.colour = img.colour;
  io.hit = img.hit;
  io.iters = img.iters;
  io.depth = img.depth;
  io.slots = (int64_t)grid * block;
  io.step_cap = kStepCap;
  io.overflow_pass = 0;
  io.tile_counter = (unsigned int *)(fctl + 0);
  io.overflow_count = (unsigned int *)(fctl + 4);
  const bool needVol = need_volumetric(scene);
  const bool points = need_step_points(scene);
  io.rays = reflection_rays(scene);
  if (needVol) {
    io.step_step = c->step[prec][0].ptr;
    io.step_dist = c->step[prec][1].ptr;
    io.step_thr = c->step[prec][2].ptr;
    io.step_scan = points ? c->step[prec][3].ptr : nullptr;
    io.step_iters = points ? (int *)c->step[prec][4].ptr : nullptr;
    io.overflow_list = (unsigned int *)c->ovlist.ptr;
  }
  MBGB_CUDA(cudaMemsetAsync(fctl, 0, 64, s));
  FrameIO ov = io;
  ov.overflow_pass = 1;
  ov.step_cap = kStepSlots;
  const int ovSlots = overflow_slots(scene, prec);
  ov.slots = ovSlots;
  ov.step_step = c->ovstep[prec][0].ptr;
  ov.step_dist = c->ovstep[prec][1].ptr;
  ov.step_thr = c->ovstep[prec][2].ptr;
  ov.step_scan = points ? c->ovstep[prec][3].ptr : nullptr;
  ov.step_iters = points ? (int *)c->ovstep[prec][4].ptr : nullptr;
  ov.rays = io.rays;
  const int ovBlocks = std::max(1, ovSlots / block);
  FractalT<double> fd;
  fill_fractal<double>(scene, fd);
  cudaError_t e;
  if (prec == 0) {
    ParamsT<double> p;
    fill_params<double>(scene, p, o, (const double *)c->ao64.ptr, c->ao_count);
    if (lightOff >= 0) p.lights = (const LightT<double> *)c->lights64.ptr + lightOff;
    e = launch_render_f64(kf, p, fd, io, grid, block, s);
    if (e == cudaSuccess && needVol) e = launch_render_f64(kf, p, fd, ov, ovBlocks, block, s);
  } else {
    ParamsT<float> p;
    fill_params<float>(scene, p, o, (const float *)c->ao32.ptr, c->ao_count);
    if (lightOff >= 0) p.lights = (const LightT<float> *)c->lights32.ptr + lightOff;
    e = launch_render_f32(kf, p, fd, io, grid, block, s);
    if (e == cudaSuccess && needVol) e = launch_render_f32(kf, p, fd, ov, ovBlocks, block, s);
  }
  if (e != cudaSuccess) return cuda_error(e, "render kernel launch");
  *launches += 1 + (needVol ? 1 : 0);
  return MBGB_OK;
}

// MBGB_PREC_AUTO, deep-zoom rule: FP64 for the whole frame when the hit bisection's window at
// the nearest surface, 0.01 x quality x the threshold there (src/Render3D.cpp:145-183; the
// threshold is d * resolution * persp / quality with d the FP64 distance estimate at the ray
// origin, or the constant threshold `quality`), is below 1e-7 of the scene scale
// (max(1, |origin|)): about one FP32 ulp. For quality 1 that is a pixel footprint below 1e-5
// of the scale. Scenes with the limit box render in FP64 too. One probe launch covers every
// frame of the call.
static mbgb_status auto_precision(mbgb_context *c, const mbgb_scene *scenes, int n, const mbgb_opts &o,
                                  cudaStream_t s, std::vector<int> &prec) {
  std::vector<double> pts(3 * (size_t)n), det((size_t)n, 1e-300);
  for (int i = 0; i < n; i++) {
    ParamsT<double> pp;
    fill_params<double>(scenes[i], pp, o, nullptr, 0);
    for (int k = 0; k < 3; k++) pts[3 * i + k] = pp.start[k];
  }
  const size_t nb = (size_t)n;
  const size_t o_pts = 0, o_det = o_pts + 24 * nb, o_d = o_det + 8 * nb, o_it = o_d + 8 * nb, o_mi = o_it + 4 * nb;
  MBGB_CUDA(c->ensure(c->probe, o_mi + nb + 16));
  char *pb = (char *)c->probe.ptr;
  MBGB_CUDA(cudaMemcpyAsync(pb + o_pts, pts.data(), 24 * nb, cudaMemcpyHostToDevice, s));
  MBGB_CUDA(cudaMemcpyAsync(pb + o_det, det.data(), 8 * nb, cudaMemcpyHostToDevice, s));
  std::vector<double> d((size_t)n, 0.0);
  // frames of one call may differ in fractal parameters: one probe per distinct fractal
  for (int i = 0; i < n; i++) {
    FractalT<double> fp;
    fill_fractal<double>(scenes[i], fp);
    cudaError_t pe = launch_distance_f64(distance_kernel_formula(scenes[i]), fp, (const double *)(pb + o_pts) + 3 * i,
                                         (const double *)(pb + o_det) + i, 1, (double *)(pb + o_d) + i,
                                         (int *)(pb + o_it) + i, (unsigned char *)(pb + o_mi) + i, nullptr, s);
    if (pe != cudaSuccess) return cuda_error(pe, "precision probe");
  }
  MBGB_CUDA(cudaMemcpyAsync(d.data(), pb + o_d, 8 * nb, cudaMemcpyDeviceToHost, s));
  MBGB_CUDA(cudaStreamSynchronize(s));
  prec.assign((size_t)n, 1);
  for (int i = 0; i < n; i++) {
    const double *st = &pts[3 * i];
    const double scale = std::max(1.0, sqrt(st[0] * st[0] + st[1] * st[1] + st[2] * st[2]));
    const double thr = scenes[i].constantDEThreshold
                           ? scenes[i].quality
                           : d[i] * scenes[i].resolution * scenes[i].persp / scenes[i].quality;
    const double window = 0.01 * scenes[i].quality * thr;
    prec[i] = window < 1e-7 * scale ? 0 : 1;
    // a limit box that cuts the fractal exposes its interior, where the colouring orbit
    // (N x 10 iterations) and the AO samples' escape test never settle and FP32 flips them
    if (scenes[i].limits_enabled) prec[i] = 0;
  }
  return MBGB_OK;
}

static mbgb_status check_opts(const mbgb_opts &o) {
  if (o.precision < 0 || o.precision > 2) return set_error(MBGB_ERR_BAD_PARAM, "unknown precision policy");
  if (o.threads_per_cta != 0 && (o.threads_per_cta % 32 != 0 || o.threads_per_cta < 32 || o.threads_per_cta > 128))
    return set_error(MBGB_ERR_BAD_PARAM, "threads_per_cta must be a multiple of 32, <= 128");
  if ((o.tile_w != 0 || o.tile_h != 0) && (o.tile_w <= 0 || o.tile_h <= 0 || o.tile_w * o.tile_h != 32))
    return set_error(MBGB_ERR_BAD_PARAM, "tile_w x tile_h must be 32");
  if (o.refill_min < 0 || o.refill_min > 32) return set_error(MBGB_ERR_BAD_PARAM, "refill_min must be in [0, 32]");
  if (o.orbit_refill < -1 || o.orbit_refill > 32) return set_error(MBGB_ERR_BAD_PARAM, "orbit_refill must be in [-1, 32]");
  if (o.pair_rays < 0 || o.pair_rays > 1) return set_error(MBGB_ERR_BAD_PARAM, "pair_rays must be 0 or 1");
  if (o.hit_order < 0 || o.hit_order > 2) return set_error(MBGB_ERR_BAD_PARAM, "hit_order must be 0, 1 or 2");
  if (o.ctas_per_sm < 0) return set_error(MBGB_ERR_BAD_PARAM, "negative ctas_per_sm");
  if (o.row_begin < 0 || o.row_end < 0) return set_error(MBGB_ERR_BAD_PARAM, "row range out of bounds");
  return MBGB_OK;
}

// Largest number of pixels x (1 + ray-AO directions) one wavefront group indexes with
// 32-bit pixel and job numbers.
constexpr double kMaxGroupJobs = 4.0e9;

static void key_append(std::vector<char> &k, const void *p, size_t n) {
  k.insert(k.end(), (const char *)p, (const char *)p + n);
}

// The ray-traced AO direction table of a call: a context holds one table, so the frames
// that trace AO rays must share its quality (fast AO and frames without AO read none).
static mbgb_status ensure_call_ao(mbgb_context *c, const mbgb_scene *scenes, int n, cudaStream_t s) {
  int q = -1;
  for (int i = 0; i < n; i++) {
    if (!scenes[i].global_ilumination || scenes[i].fastGlobalIllumination) continue;
    if (q < 0) q = scenes[i].globalIlumQuality;
    else if (scenes[i].globalIlumQuality != q)
      return set_error(MBGB_ERR_BAD_PARAM, "frames of one call that trace AO rays must share the AO quality");
  }
  if (q < 0) q = scenes[0].globalIlumQuality;
  return ensure_ao(c, q, s);
}

static mbgb_status read_back(mbgb_context *c, const CallPlan &plan, int replayed);
static mbgb_status autotune_impl(mbgb_context *c, const mbgb_scene *scene, const mbgb_opts &o, cudaStream_t s,
                                 mbgb_tuning *out);

// Every render call: validate, plan the groups, prepare scratch and frame tables, enqueue
// (or capture once and replay), and, for calls without a caller stream, wait and read the
// counters back.
// PlaceRandomLights (src/shaders.cpp:1134-1208): srand(seed); light after light, candidate
// positions centre + (Random(2000000) / 1e6 - 1 + Random(1000000) / 1e12 per axis) x radius x
// multiplier until CalculateDistance (detailSize 0) there is positive, below maxDist x
// multiplier and not at the iteration limit; the multiplier grows by 1.1 every 1000
// trials and resets with each light placed. Then the four predefined lights overwrite
// slots 0-3 (enabled or not). The candidates' distances come from the device, a batch of
// trials at a time: the batch is generated from a copy of the generator as if every trial
// failed, and the generator then advances to the first accepted trial.
static mbgb_status place_lights(mbgb_context *c, const mbgb_scene &s, cudaStream_t st,
                                std::vector<LightT<double>> &out) {
  const int nRandom = s.auxLightNumber > 0 ? s.auxLightNumber : 0;
  out.assign((size_t)std::max(nRandom, 4), LightT<double>{});
  GlibcRand rng((uint32_t)s.auxLightRandomSeed);
  if (nRandom > 0) {
    constexpr int kBatch = 512;
    constexpr long long kMaxTrials = 20000000;  // the reference loops for ever on a scene no light fits
    FractalT<double> f;
    fill_fractal<double>(s, f);
    const int kf = distance_kernel_formula(s);
    const size_t o_pts = 0, o_det = 24 * kBatch, o_d = o_det + 8 * kBatch, o_it = o_d + 8 * kBatch,
                 o_mi = o_it + 4 * kBatch;
    MBGB_CUDA(c->ensure(c->lightprobe, o_mi + kBatch + 16));
    char *pb = (char *)c->lightprobe.ptr;
    const std::vector<double> zeros(kBatch, 0.0);
    MBGB_CUDA(cudaMemcpyAsync(pb + o_det, zeros.data(), 8 * kBatch, cudaMemcpyHostToDevice, st));
    std::vector<double> pts(3 * kBatch), dist(kBatch);
    std::vector<unsigned char> mi(kBatch);
    std::vector<GlibcRand> after(kBatch, rng);
    std::vector<double> rmAccept(kBatch);
    std::vector<int> tnAfter(kBatch);
    int trial_number = 0;
    double radius_multiplier = 1.0;
    long long trials = 0;
    for (int i = 0; i < nRandom;) {
      GlibcRand g = rng;
      int tn = trial_number;
      double rm = radius_multiplier;
      for (int b = 0; b < kBatch; b++) {
        tn++;
        double r[3];
        for (int k = 0; k < 3; k++) {
          const int a = g.random(2000000);
          const int bb = g.random(1000000);
          r[k] = (a / 1000000.0 - 1.0) + (bb / 1.0e12);
        }
        for (int k = 0; k < 3; k++) pts[3 * b + k] = s.auxLightRandomCenter[k] + r[k] * s.auxLightDistributionRadius * rm;
        if (tn > 1000) {
          rm *= 1.1;
          tn = 0;
        }
        after[b] = g;
        rmAccept[b] = rm;
        tnAfter[b] = tn;
      }
      MBGB_CUDA(cudaMemcpyAsync(pb + o_pts, pts.data(), 24 * kBatch, cudaMemcpyHostToDevice, st));
      cudaError_t e = launch_distance_f64(kf, f, (const double *)(pb + o_pts), (const double *)(pb + o_det), kBatch,
                                          (double *)(pb + o_d), (int *)(pb + o_it), (unsigned char *)(pb + o_mi),
                                          nullptr, st);
      if (e != cudaSuccess) return cuda_error(e, "light placement distances");
      MBGB_CUDA(cudaMemcpyAsync(dist.data(), pb + o_d, 8 * kBatch, cudaMemcpyDeviceToHost, st));
      MBGB_CUDA(cudaMemcpyAsync(mi.data(), pb + o_mi, kBatch, cudaMemcpyDeviceToHost, st));
      MBGB_CUDA(cudaStreamSynchronize(st));
      int hit = -1;
      for (int b = 0; b < kBatch; b++)
        if (dist[b] > 0 && !mi[b] && dist[b] < s.auxLightMaxDist * rmAccept[b]) {
          hit = b;
          break;
        }
      if (hit < 0) {
        rng = after[kBatch - 1];
        trial_number = tnAfter[kBatch - 1];
        radius_multiplier = rmAccept[kBatch - 1];
        trials += kBatch;
        if (trials > kMaxTrials) return set_error(MBGB_ERR_UNSUPPORTED, "no position found for an auxiliary light");
        continue;
      }
      rng = after[hit];
      trial_number = tnAfter[hit];
      radius_multiplier = 1.0;
      LightT<double> &L = out[(size_t)i];
      for (int k = 0; k < 3; k++) L.pos[k] = pts[3 * hit + k];
      int col[3];
      for (int k = 0; k < 3; k++) col[k] = 20000 + rng.random(80000);
      // dMax (src/common_math.cpp:34-43)
      const double a = col[0], b = col[1], cc = col[2];
      const double maxColour = (a > b) ? ((a > cc) ? a : cc) : ((b > cc) ? b : cc);
      for (int k = 0; k < 3; k++) L.colour[k] = (int)(col[k] * 65536.0 / maxColour);
      L.intensity = dist[hit] * dist[hit] / s.auxLightMaxDist;
      L.enabled = 1;
      trials += hit + 1;
      i++;
    }
  }
  for (int i = 0; i < 4; i++) {
    LightT<double> &L = out[(size_t)i];
    if (s.auxLightPreEnabled[i]) {
      for (int k = 0; k < 3; k++) L.pos[k] = s.auxLightPre[i][k];
      L.intensity = s.auxLightPreIntensity[i];
      L.colour[0] = s.auxLightPreColour[i].R;
      L.colour[1] = s.auxLightPreColour[i].G;
      L.colour[2] = s.auxLightPreColour[i].B;
      L.enabled = 1;
    } else {
      L.enabled = 0;
    }
  }
  return MBGB_OK;
}

static mbgb_status render_frames(mbgb_context *c, const mbgb_scene *scenes, int n, const mbgb_image *imgs,
                                 const mbgb_opts *opts_in, const GradRequest *grad = nullptr) {
  if (!c || !scenes || !imgs) return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  if (n < 1) return set_error(MBGB_ERR_BAD_PARAM, "no frames");
  mbgb_opts o{};
  if (opts_in) o = *opts_in;
  if (grad) {
    o.exact_hit = 1;
    o.engine = MBGB_ENGINE_WAVEFRONT;
    o.use_graph = 0;
  }
  mbgb_status st = check_opts(o);
  if (st != MBGB_OK) return st;
  for (int i = 0; i < n; i++) {
    st = mbgb_scene_supported(&scenes[i]);
    if (st == MBGB_OK && o.exact_hit) st = level_set_supported(scenes[i]);
    if (st == MBGB_OK && grad) st = grad_supported(scenes[i]);
    if (st != MBGB_OK) return n > 1 ? set_error(st, "frame " + std::to_string(i) + ": " + mbgb_last_error()) : st;
    if (imgs[i].width != scenes[i].image_width || imgs[i].height != scenes[i].image_height)
      return set_error(MBGB_ERR_BAD_PARAM, "image size does not match the scene");
    const int r1 = o.row_end == 0 ? scenes[i].image_height : o.row_end;
    if (o.row_begin >= r1 || r1 > scenes[i].image_height)
      return set_error(MBGB_ERR_BAD_PARAM, "row range out of bounds");
  }
  MBGB_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = o.stream ? (cudaStream_t)o.stream : c->stream;
  const bool sync = o.stream == nullptr;
  // light tables are placed per call, outside any capture: such calls are not captured
  for (int i = 0; i < n; i++)
    if (uses_aux_lights(scenes[i])) o.use_graph = 0;

  // a captured graph of the same frames, outputs and options is replayed as it is
  std::vector<char> key;
  if (o.use_graph) {
    mbgb_opts ko = o;
    ko.stream = nullptr;
    key_append(key, &n, sizeof(n));
    key_append(key, scenes, sizeof(mbgb_scene) * (size_t)n);
    key_append(key, imgs, sizeof(mbgb_image) * (size_t)n);
    key_append(key, &ko, sizeof(ko));
    if (c->graph && key == c->graph_key) {
      st = ensure_call_ao(c, scenes, n, s);
      if (st != MBGB_OK) return st;
      if (c->gen == c->graph_gen) {
        if (!c->cams_hold_graph && !c->graph_cams.empty()) {
          MBGB_CUDA(cudaMemcpyAsync(c->cams.ptr, c->graph_cams.data(), c->graph_cams.size(), cudaMemcpyHostToDevice,
                                    s));
          c->cams_hold_graph = true;
        }
        MBGB_CUDA(cudaEventRecord(c->ev0, s));
        MBGB_CUDA(cudaGraphLaunch(c->graph, s));
        MBGB_CUDA(cudaEventRecord(c->ev1, s));
        c->plan = c->graph_plan;
        return sync ? read_back(c, c->plan, 1) : MBGB_OK;
      }
    }
  }

  // precision per frame
  std::vector<int> prec((size_t)n, o.precision == MBGB_PREC_FP64 ? 0 : 1);
  if (o.precision == MBGB_PREC_AUTO) {
    st = auto_precision(c, scenes, n, o, s, prec);
    if (st != MBGB_OK) return st;
  }
  // delta-DE formulas difference orbits at a step of 1e-10 (src/fractal.cpp:1310), far
  // below FP32 resolution: those frames render in FP64 under every policy
  for (int i = 0; i < n; i++)
    if (!scenes[i].analitycDE) prec[i] = 0;
  st = ensure_call_ao(c, scenes, n, s);
  if (st != MBGB_OK) return st;
  if (o.autotune) {
    // tune once per scene class, on the call's largest frame of that class
    for (int i = 0; i < n; i++) {
      if (c->tunings.count(tune_key(scenes[i], prec[i]))) continue;
      int best = i;
      for (int j = i + 1; j < n; j++)
        if (tune_key(scenes[j], prec[j]) == tune_key(scenes[i], prec[i]) &&
            (int64_t)scenes[j].image_width * scenes[j].image_height >
                (int64_t)scenes[best].image_width * scenes[best].image_height)
          best = j;
      mbgb_opts to = o;
      to.precision = prec[best] == 0 ? MBGB_PREC_FP64 : MBGB_PREC_FP32_FIX;
      to.use_graph = 0;
      mbgb_tuning t;
      st = autotune_impl(c, &scenes[best], to, s, &t);
      if (st != MBGB_OK) return st;
    }
  }

  // groups: frames with equal shared parameters and precision render in one launch sequence
  CallPlan plan;
  plan.frames = (uint64_t)n;
  plan.profile = o.profile_stages && !o.use_graph;
  plan.grad = grad != nullptr;
  for (int i = 0; i < n; i++) {
    const mbgb_scene &sc = scenes[i];
    const int r0 = o.row_begin, r1 = o.row_end == 0 ? sc.image_height : o.row_end;
    plan.pixels += (uint64_t)(r1 - r0) * (uint64_t)sc.image_width;
    const LaunchCfg cfg = resolve_cfg(c, o, sc, prec[i]);
    const int64_t fpix = (int64_t)sc.image_width * sc.image_height;
    const int64_t fjobs = (int64_t)((sc.image_width + cfg.tileW - 1) / cfg.tileW) *
                          ((r1 - r0 + cfg.tileH - 1) / cfg.tileH) * 32;
    const bool rayAO = sc.global_ilumination && !sc.fastGlobalIllumination;
    const double perPix = (1.0 + (rayAO ? c->ao_count : 0) + aux_light_count(sc)) * reflection_rays(sc);
    const bool wave = o.engine == MBGB_ENGINE_WAVEFRONT && !per_pixel_only(sc) &&
                      (double)std::max(fpix, fjobs) * perPix < kMaxGroupJobs;
    if (!wave && (grad || o.exact_hit))
      return set_error(MBGB_ERR_BAD_PARAM, "exact hits and gradients need the wavefront engine and frames below 4e9 rays");
    Group *g = nullptr;
    // a frame with auxiliary lights keeps its own group (its lights are placed for it), and so
    // does one with volumetric lights (the long rays' fold reads the scene's own parameters)
    if (wave && !uses_aux_lights(sc) && !sc.volumetricLightEnabledAny && !sc.iterFogEnabled &&
        !sc.fakeLightsEnabled) {
      for (auto &h : plan.groups) {
        if (!h.wave || h.prec != prec[i]) continue;
        if ((double)std::max(h.npix + fpix, h.jobs + fjobs) * perPix >= kMaxGroupJobs) continue;
        const mbgb_scene &rep = scenes[h.frames[0]];
        if (uses_aux_lights(rep) || rep.volumetricLightEnabledAny || rep.iterFogEnabled || rep.fakeLightsEnabled)
          continue;
        const bool same = prec[i] == 0 ? same_shared<double>(rep, sc, o) : same_shared<float>(rep, sc, o);
        if (!same) continue;
        const LaunchCfg &hc = h.cfg;
        if (hc.tileW != cfg.tileW || hc.tileH != cfg.tileH || hc.block != cfg.block ||
            hc.ctasPerSm != cfg.ctasPerSm || hc.refill != cfg.refill || hc.orbitRefill != cfg.orbitRefill)
          continue;
        g = &h;
        break;
      }
    }
    if (!g) {
      plan.groups.emplace_back();
      g = &plan.groups.back();
      g->prec = prec[i];
      g->wave = wave;
      g->cfg = cfg;
    }
    g->frames.push_back(i);
    g->npix += fpix;
    g->jobs += fjobs;
  }

  // scratch for the largest group of each kind, frame tables of all groups
  size_t wave_bytes[2] = {0, 0};
  bool volPrec[2] = {false, false};
  bool pointsPrec[2] = {false, false};
  int64_t ovRecords[2] = {kOverflowThreads, kOverflowThreads};   // overflow slots x rays
  int64_t maxPixPerPixel = 0;
  int64_t maxSlots[2] = {0, 0};
  size_t camsBytes = 0;
  for (auto &g : plan.groups) {
    const mbgb_scene &rep = scenes[g.frames[0]];
    const bool needVol = need_volumetric(rep);
    if (needVol) volPrec[g.prec] = true;
    if (need_step_points(rep)) pointsPrec[g.prec] = true;
    if (!g.wave)
      ovRecords[g.prec] =
          std::max(ovRecords[g.prec], (int64_t)overflow_slots(rep, g.prec) * reflection_rays(rep));
    else if (needVol)
      ovRecords[g.prec] = std::max<int64_t>(ovRecords[g.prec], kWaveOverflowThreads);
    if (g.wave) {
      const bool rayAO = rep.global_ilumination && !rep.fastGlobalIllumination;
      const size_t ts = g.prec == 0 ? sizeof(double) : sizeof(float);
      wave_bytes[g.prec] =
          std::max(wave_bytes[g.prec], wave_layout(g.npix, ts, rayAO ? c->ao_count : 0, needVol, reflection_rays(rep),
                                                   aux_light_count(rep), rep.shadow != 0,
                                                   (rep.volumetricLightEnabledAny || rep.iterFogEnabled ||
                                                    rep.fakeLightsEnabled)
                                                       ? kSampleShadows +
                                                             (rep.iterFogEnabled && rayAO ? c->ao_count : 0) +
                                                             (rep.fakeLightsEnabled ? 1 : 0)
                                                       : 0,
                                                   rep.iterFogEnabled != 0, g.jobs)
                                           .total);
      g.cams_off = camsBytes;
      const size_t cs = g.prec == 0 ? sizeof(FrameCam<double>) : sizeof(FrameCam<float>);
      camsBytes += (cs * g.frames.size() + 255) & ~(size_t)255;
      if (grad) {
        g.grad_off = camsBytes;
        const size_t gs = g.prec == 0 ? sizeof(GradCam<double>) : sizeof(GradCam<float>);
        camsBytes += (gs * g.frames.size() + 255) & ~(size_t)255;
      }
    } else if (needVol) {
      maxPixPerPixel = std::max(maxPixPerPixel, g.npix);
      maxSlots[g.prec] = std::max(maxSlots[g.prec], (int64_t)c->sms * per_pixel_ctas(rep, g.prec, g.cfg, c->sms) *
                                                        g.cfg.block * reflection_rays(rep));
    }
  }
  for (int p = 0; p < 2; p++) {
    if (wave_bytes[p]) MBGB_CUDA(c->ensure(c->wave[p], wave_bytes[p]));
    const size_t esz = p == 0 ? sizeof(double) : sizeof(float);
    const int arrays = pointsPrec[p] ? 5 : 3;
    auto bytes_of = [&](int k) { return k == 4 ? sizeof(int) : esz; };
    if (volPrec[p])
      for (int k = 0; k < arrays; k++)
        MBGB_CUDA(c->ensure(c->ovstep[p][k], (size_t)kStepSlots * (size_t)ovRecords[p] * bytes_of(k)));
    if (maxSlots[p])
      for (int k = 0; k < arrays; k++)
        MBGB_CUDA(c->ensure(c->step[p][k], (size_t)kStepCap * (size_t)maxSlots[p] * bytes_of(k)));
  }
  if (maxPixPerPixel) MBGB_CUDA(c->ensure(c->ovlist, (size_t)maxPixPerPixel * sizeof(unsigned int)));
  MBGB_CUDA(c->ensure(c->control, 256));
  MBGB_CUDA(c->ensure(c->fctl, 64 * plan.groups.size()));
  if (grad) MBGB_CUDA(c->ensure(c->gradacc, sizeof(double) * kGradParams * (size_t)n));
  std::vector<char> camsHost(camsBytes);
  for (auto &g : plan.groups) {
    if (!g.wave) continue;
    int64_t pixBase = 0;
    uint32_t jobBase = 0;
    for (size_t k = 0; k < g.frames.size(); k++) {
      const int i = g.frames[k];
      const mbgb_scene &sc = scenes[i];
      const int r0 = o.row_begin, r1 = o.row_end == 0 ? sc.image_height : o.row_end;
      const uint32_t jobs = (uint32_t)(((sc.image_width + g.cfg.tileW - 1) / g.cfg.tileW) *
                                       ((r1 - r0 + g.cfg.tileH - 1) / g.cfg.tileH) * 32);
      if (g.prec == 0) {
        FrameCam<double> cam;
        fill_cam<double>(sc, imgs[i], o, g.cfg, cam);
        cam.pixBase = pixBase;
        cam.jobBase = jobBase;
        cam.jobCount = jobs;
        memcpy(camsHost.data() + g.cams_off + k * sizeof(cam), &cam, sizeof(cam));
        if (grad) {
          GradCam<double> gc;
          fill_grad_cam<double>(sc, *grad, i, (double *)c->gradacc.ptr, gc);
          memcpy(camsHost.data() + g.grad_off + k * sizeof(gc), &gc, sizeof(gc));
        }
      } else {
        FrameCam<float> cam;
        fill_cam<float>(sc, imgs[i], o, g.cfg, cam);
        cam.pixBase = pixBase;
        cam.jobBase = jobBase;
        cam.jobCount = jobs;
        memcpy(camsHost.data() + g.cams_off + k * sizeof(cam), &cam, sizeof(cam));
        if (grad) {
          GradCam<float> gc;
          fill_grad_cam<float>(sc, *grad, i, (double *)c->gradacc.ptr, gc);
          memcpy(camsHost.data() + g.grad_off + k * sizeof(gc), &gc, sizeof(gc));
        }
      }
      pixBase += (int64_t)sc.image_width * sc.image_height;
      jobBase += jobs;
    }
  }
  if (camsBytes) {
    MBGB_CUDA(c->ensure(c->cams, camsBytes));
    MBGB_CUDA(cudaMemcpyAsync(c->cams.ptr, camsHost.data(), camsBytes, cudaMemcpyHostToDevice, s));
    c->cams_hold_graph = false;
  }
  if (plan.profile) {
    const size_t want = kStageEvents * plan.groups.size();
    while (c->gev.size() < want) {
      cudaEvent_t ev;
      MBGB_CUDA(cudaEventCreate(&ev));
      c->gev.push_back(ev);
    }
  }

  // auxiliary light tables of the frames that light with them
  std::vector<int64_t> lightOff((size_t)n, -1);
  {
    std::vector<LightT<double>> all64;
    for (auto &g : plan.groups) {
      if (!uses_aux_lights(scenes[g.frames[0]])) continue;
      std::vector<LightT<double>> L;
      st = place_lights(c, scenes[g.frames[0]], s, L);
      if (st != MBGB_OK) return st;
      lightOff[(size_t)g.frames[0]] = (int64_t)all64.size();
      all64.insert(all64.end(), L.begin(), L.end());
    }
    if (!all64.empty()) {
      std::vector<LightT<float>> all32(all64.size());
      for (size_t k = 0; k < all64.size(); k++) {
        for (int j = 0; j < 3; j++) {
          all32[k].pos[j] = (float)all64[k].pos[j];
          all32[k].colour[j] = all64[k].colour[j];
        }
        all32[k].intensity = (float)all64[k].intensity;
        all32[k].enabled = all64[k].enabled;
      }
      MBGB_CUDA(c->ensure(c->lights64, sizeof(LightT<double>) * all64.size()));
      MBGB_CUDA(c->ensure(c->lights32, sizeof(LightT<float>) * all32.size()));
      MBGB_CUDA(cudaMemcpyAsync(c->lights64.ptr, all64.data(), sizeof(LightT<double>) * all64.size(),
                                cudaMemcpyHostToDevice, s));
      MBGB_CUDA(cudaMemcpyAsync(c->lights32.ptr, all32.data(), sizeof(LightT<float>) * all32.size(),
                                cudaMemcpyHostToDevice, s));
    }
  }

  // enqueue (inside a capture when use_graph)
  char *ctl = (char *)c->control.ptr;
  FrameIO io{};
  io.error_flag = (int *)(ctl + 16);
  io.start_ns = (unsigned long long *)(ctl + 32);
  io.counters = (unsigned long long *)(ctl + 64);
  io.budget_ns = o.deadline_ms > 0 ? (unsigned long long)o.deadline_ms * 1000000ull : 0ull;
  auto enqueue = [&]() -> mbgb_status {
    MBGB_CUDA(cudaMemsetAsync(ctl, 0, 256, s));
    if (grad) MBGB_CUDA(cudaMemsetAsync(c->gradacc.ptr, 0, sizeof(double) * kGradParams * (size_t)n, s));
    for (size_t gi = 0; gi < plan.groups.size(); gi++) {
      const Group &g = plan.groups[gi];
      char *gctl = (char *)c->fctl.ptr + 64 * gi;
      cudaEvent_t *ev = plan.profile ? &c->gev[kStageEvents * gi] : nullptr;
      mbgb_status r;
      if (!g.wave) {
        r = enqueue_per_pixel(c, scenes[g.frames[0]], imgs[g.frames[0]], g, o, s, io, gctl, &plan.launches,
                              lightOff[(size_t)g.frames[0]]);
      } else if (g.prec == 0) {
        r = enqueue_wave<double>(c, scenes, g, o, s, io, (uint32_t *)gctl, ev, plan.grad, &plan.launches,
                                 lightOff[(size_t)g.frames[0]]);
      } else {
        r = enqueue_wave<float>(c, scenes, g, o, s, io, (uint32_t *)gctl, ev, plan.grad, &plan.launches,
                                lightOff[(size_t)g.frames[0]]);
      }
      if (r != MBGB_OK) return r;
    }
    return MBGB_OK;
  };
  if (o.use_graph) {
    if (c->graph) {
      cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
      c->graph_key.clear();
    }
    MBGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    st = enqueue();
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &graph);
    if (st != MBGB_OK) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    if (ec != cudaSuccess) return cuda_error(ec, "cudaStreamEndCapture");
    const cudaError_t ei = cudaGraphInstantiate(&c->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      c->graph = nullptr;
      return cuda_error(ei, "cudaGraphInstantiate");
    }
    c->graph_key = key;
    c->graph_gen = c->gen;
    c->graph_plan = plan;
    c->graph_cams = camsHost;
    c->cams_hold_graph = true;
    MBGB_CUDA(cudaEventRecord(c->ev0, s));
    MBGB_CUDA(cudaGraphLaunch(c->graph, s));
    MBGB_CUDA(cudaEventRecord(c->ev1, s));
  } else {
    MBGB_CUDA(cudaEventRecord(c->ev0, s));
    st = enqueue();
    if (st != MBGB_OK) return st;
    MBGB_CUDA(cudaEventRecord(c->ev1, s));
  }
  c->plan = plan;
  return sync ? read_back(c, plan, 0) : MBGB_OK;
}

// Wait for the call's stream and fill the context's counters (the reference's globals,
// src/Render3D.cpp:51-57) from the device.
static mbgb_status read_back(mbgb_context *c, const CallPlan &plan, int replayed) {
  MBGB_CUDA(cudaStreamSynchronize(c->stream));
  MBGB_CUDA(cudaEventSynchronize(c->ev1));
  char *ctl = (char *)c->control.ptr;
  unsigned long long cnt[4 * kStages];
  int flag = 0;
  MBGB_CUDA(cudaMemcpy(cnt, ctl + 64, sizeof(cnt), cudaMemcpyDeviceToHost));
  MBGB_CUDA(cudaMemcpy(&flag, ctl + 16, sizeof(flag), cudaMemcpyDeviceToHost));
  std::vector<uint32_t> gctl(16 * plan.groups.size());
  if (!gctl.empty())
    MBGB_CUDA(cudaMemcpy(gctl.data(), c->fctl.ptr, 64 * plan.groups.size(), cudaMemcpyDeviceToHost));
  mbgb_stats &S = c->stats;
  S = mbgb_stats{};
  for (int k = 0; k < kStages; k++) {
    S.stage_orbit[k] = cnt[4 * k + 0];
    S.stage_de[k] = cnt[4 * k + 1];
  }
  for (size_t gi = 0; gi < plan.groups.size(); gi++) {
    const Group &g = plan.groups[gi];
    const uint32_t *q = &gctl[16 * gi];
    if (g.wave) {
      S.long_rays += q[3];
      if (g.prec == 1) S.fp64_polished += q[6];
      S.level_set_missed += q[7];
    } else {
      S.long_rays += q[1];
    }
    if (plan.profile && g.wave) {
      // events in launch order -> stats slots (primary 0, polish 1, level set 4, shadow/AO 2,
      // compose 3, gradient 5)
      const int slot[kStages] = {0, 1, 4, 2, 3, 5};
      for (int k = 0; k < kStages; k++) {
        float sm = 0;
        if (cudaEventElapsedTime(&sm, c->gev[kStageEvents * gi + k], c->gev[kStageEvents * gi + k + 1]) ==
            cudaSuccess)
          S.stage_ms[slot[k]] += sm;
      }
    }
  }
  for (int k = 1; k < 4; k++) {
    cnt[0] += cnt[4 * k + 0];
    cnt[1] += cnt[4 * k + 1];
    cnt[2] += cnt[4 * k + 2];
    cnt[3] += cnt[4 * k + 3];
  }
  // the gradient stage's counters: orbit iterations, DE calls, pixels differentiated, skipped
  cnt[0] += cnt[20];
  cnt[1] += cnt[21];
  S.grad_pixels = plan.grad ? cnt[22] : 0;
  S.grad_skipped = plan.grad ? cnt[23] : 0;
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  S.orbit_iterations = cnt[0];
  S.de_calls = cnt[1];
  S.primary_steps = cnt[2];
  S.missed_de = cnt[3];
  S.pixels = plan.pixels;
  S.frames = plan.frames;
  S.launches = plan.launches;
  S.graph_replayed = (uint64_t)replayed;
  S.kernel_ms = ms;
  bool anyFp64 = false;
  for (auto &g : plan.groups) anyFp64 = anyFp64 || g.prec == 0;
  S.auto_fp64 = anyFp64;
  if (flag) return set_error(MBGB_ERR_TIMEOUT, "render stopped at its device deadline");
  return MBGB_OK;
}

// Autotuner: coordinate search over tile shape, threads per CTA, CTAs per SM and the
// refill threshold, each candidate timed on the device (best of two after a warm-up).
static mbgb_status autotune_impl(mbgb_context *c, const mbgb_scene *scene, const mbgb_opts &o_in, cudaStream_t s,
                                 mbgb_tuning *out) {
  const int64_t npix = (int64_t)scene->image_width * scene->image_height;
  MBGB_CUDA(c->ensure(c->tune_out, (size_t)npix * 24 + 1024));
  char *b = (char *)c->tune_out.ptr;
  mbgb_image img{};
  img.width = scene->image_width;
  img.height = scene->image_height;
  img.image_float = (float *)b;
  img.zbuffer = (float *)(b + ((npix * 12 + 255) & ~(int64_t)255));
  img.alpha = (uint16_t *)((char *)img.zbuffer + ((npix * 4 + 255) & ~(int64_t)255));
  img.opacity = (uint16_t *)((char *)img.alpha + ((npix * 2 + 255) & ~(int64_t)255));
  mbgb_opts o = o_in;
  o.autotune = 0;
  o.use_graph = 0;
  o.profile_stages = 0;
  o.stream = nullptr;
  o.engine = MBGB_ENGINE_WAVEFRONT;
  MBGB_CUDA(cudaStreamSynchronize(s));   // earlier work of the caller's stream may use the scratch
  int trials = 0;
  auto time_cfg = [&](const LaunchCfg &cfg, double *ms) -> mbgb_status {
    o.tile_w = cfg.tileW;
    o.tile_h = cfg.tileH;
    o.threads_per_cta = cfg.block;
    o.ctas_per_sm = cfg.ctasPerSm;
    o.refill_min = cfg.refill;
    o.orbit_refill = cfg.orbitRefill > 0 ? cfg.orbitRefill : (cfg.orbitRefill == 0 ? -1 : 0);
    double best = 1e30;
    for (int r = 0; r < 3; r++) {
      mbgb_status st = render_frames(c, scene, 1, &img, &o);
      if (st != MBGB_OK) return st;
      if (r > 0) best = std::min(best, c->stats.kernel_ms);
    }
    trials++;
    *ms = best;
    return MBGB_OK;
  };
  const int prec = o.precision == MBGB_PREC_FP64 ? 0 : 1;
  LaunchCfg cur;
  double curMs = 0;
  mbgb_status st = time_cfg(cur, &curMs);
  if (st != MBGB_OK) return st;
  const double defMs = curMs;
  auto consider = [&](LaunchCfg cand) -> mbgb_status {
    double ms = 0;
    mbgb_status r = time_cfg(cand, &ms);
    if (r != MBGB_OK) return r;
    if (ms < curMs) {
      cur = cand;
      curMs = ms;
    }
    return MBGB_OK;
  };
  const int tiles[3][2] = {{16, 2}, {4, 8}, {32, 1}};
  const LaunchCfg base = cur;
  for (auto &t : tiles) {
    LaunchCfg cand = base;
    cand.tileW = t[0];
    cand.tileH = t[1];
    if ((st = consider(cand)) != MBGB_OK) return st;
  }
  {
    LaunchCfg cand = cur;
    cand.block = 64;
    if ((st = consider(cand)) != MBGB_OK) return st;
  }
  {
    const int kf = distance_kernel_formula(*scene);
    const int occ = std::max(1, prec == 0 ? occupancy_wave_f64(kf, cur.block, 0) : occupancy_wave_f32(kf, cur.block, 0));
    if (occ >= 2) {
      LaunchCfg cand = cur;
      cand.ctasPerSm = occ / 2;
      if ((st = consider(cand)) != MBGB_OK) return st;
    }
  }
  const LaunchCfg before = cur;
  for (int rf : {1, 4, 16}) {
    LaunchCfg cand = before;
    cand.refill = rf;
    if ((st = consider(cand)) != MBGB_OK) return st;
  }
  if (fast_mandelbox(*scene) || fast_mandelbulb(*scene)) {
    const LaunchCfg chosen = cur;
    for (int orf : {0, 8, 16}) {
      if (orf == (fast_mandelbulb(*scene) ? 8 : 0)) continue;   // the default, timed already
      LaunchCfg cand = chosen;
      cand.orbitRefill = orf;
      if ((st = consider(cand)) != MBGB_OK) return st;
    }
  }
  mbgb_tuning t{};
  t.tile_w = cur.tileW;
  t.tile_h = cur.tileH;
  t.threads_per_cta = cur.block;
  t.ctas_per_sm = cur.ctasPerSm;
  t.refill_min = cur.refill;
  t.orbit_refill = cur.orbitRefill < 0 ? (fast_mandelbulb(*scene) ? 8 : 0) : cur.orbitRefill;
  t.ms = curMs;
  t.ms_default = defMs;
  t.trials = trials;
  c->tunings[tune_key(*scene, prec)] = t;
  if (out) *out = t;
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_render_device(mbgb_context *c, const mbgb_scene *scene, const mbgb_image *out,
                                          const mbgb_opts *opts) {
  if (!c) return set_error(MBGB_ERR_BAD_PARAM, "NULL context");
  std::lock_guard<std::mutex> lk(c->mu);
  return render_frames(c, scene, 1, out, opts);
}

extern "C" mbgb_status mbgb_render_batch(mbgb_context *c, const mbgb_scene *frames, int32_t n,
                                         const mbgb_image *outs, const mbgb_opts *opts) {
  if (!c) return set_error(MBGB_ERR_BAD_PARAM, "NULL context");
  std::lock_guard<std::mutex> lk(c->mu);
  return render_frames(c, frames, n, outs, opts);
}

extern "C" mbgb_status mbgb_render_grad(mbgb_context *c, const mbgb_scene *frames, int32_t n,
                                        const mbgb_image *outs, const float *const *dL_dimage,
                                        float *const *jacobian, double *dL_dtheta, const mbgb_opts *opts) {
  if (!c) return set_error(MBGB_ERR_BAD_PARAM, "NULL context");
  std::lock_guard<std::mutex> lk(c->mu);
  mbgb_opts o{};
  if (opts) o = *opts;
  o.stream = nullptr;   // synchronous: the sums are read back
  GradRequest gr{dL_dimage, jacobian};
  mbgb_status st = render_frames(c, frames, n, outs, &o, &gr);
  if (st != MBGB_OK) return st;
  if (dL_dtheta)
    MBGB_CUDA(cudaMemcpy(dL_dtheta, c->gradacc.ptr, sizeof(double) * kGradParams * (size_t)n, cudaMemcpyDeviceToHost));
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_autotune(mbgb_context *c, const mbgb_scene *scene, const mbgb_opts *opts,
                                     mbgb_tuning *out) {
  if (!c || !scene) return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  mbgb_opts o{};
  if (opts) o = *opts;
  if (o.precision == MBGB_PREC_AUTO) o.precision = MBGB_PREC_FP32_FIX;
  o.row_begin = o.row_end = 0;
  mbgb_status st = check_opts(o);
  if (st != MBGB_OK) return st;
  st = mbgb_scene_supported(scene);
  if (st != MBGB_OK) return st;
  MBGB_CUDA(cudaSetDevice(c->device));
  return autotune_impl(c, scene, o, c->stream, out);
}

// Host-pointer variant of render_frames: device staging per frame and layer, copies in
// the call (rows outside the row range are not copied back).
static mbgb_status render_frames_host(mbgb_context *c, const mbgb_scene *scenes, int n, const mbgb_image *outs,
                                      const mbgb_opts *opts) {
  if (!c || !scenes || !outs) return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  if (n < 1) return set_error(MBGB_ERR_BAD_PARAM, "no frames");
  MBGB_CUDA(cudaSetDevice(c->device));
  const size_t per_pix[8] = {12, 4, 2, 2, 3, 1, 4, 8};
  auto layer_ptr = [](const mbgb_image &im, int k) -> void * {
    switch (k) {
      case 0: return im.image_float;
      case 1: return im.zbuffer;
      case 2: return im.alpha;
      case 3: return im.opacity;
      case 4: return im.colour;
      case 5: return im.hit;
      case 6: return im.iters;
      default: return im.depth;
    }
  };
  // staging layout: layer k of frame i at off[i][k]
  std::vector<size_t> off((size_t)n * 8, 0);
  size_t total = 0;
  for (int i = 0; i < n; i++) {
    if (outs[i].width != scenes[i].image_width || outs[i].height != scenes[i].image_height)
      return set_error(MBGB_ERR_BAD_PARAM, "image size does not match the scene");
    const size_t npix = (size_t)outs[i].width * outs[i].height;
    for (int k = 0; k < 8; k++) {
      if (!layer_ptr(outs[i], k)) continue;
      off[8 * i + k] = total;
      total += (npix * per_pix[k] + 255) & ~(size_t)255;
    }
  }
  MBGB_CUDA(c->ensure(c->out[0], std::max<size_t>(total, 256)));
  char *stage = (char *)c->out[0].ptr;
  std::vector<mbgb_image> dev(outs, outs + n);
  for (int i = 0; i < n; i++) {
    void *p[8];
    for (int k = 0; k < 8; k++) p[k] = layer_ptr(outs[i], k) ? stage + off[8 * i + k] : nullptr;
    dev[i].image_float = (float *)p[0];
    dev[i].zbuffer = (float *)p[1];
    dev[i].alpha = (uint16_t *)p[2];
    dev[i].opacity = (uint16_t *)p[3];
    dev[i].colour = (uint8_t *)p[4];
    dev[i].hit = (uint8_t *)p[5];
    dev[i].iters = (int32_t *)p[6];
    dev[i].depth = (double *)p[7];
  }
  mbgb_opts o{};
  if (opts) o = *opts;
  cudaStream_t s = o.stream ? (cudaStream_t)o.stream : c->stream;
  mbgb_status st = render_frames(c, scenes, n, dev.data(), &o);
  if (st != MBGB_OK) return st;
  for (int i = 0; i < n; i++) {
    const int r0 = o.row_begin, r1 = o.row_end > 0 ? o.row_end : outs[i].height;
    const size_t rowpix = (size_t)outs[i].width;
    for (int k = 0; k < 8; k++) {
      void *h = layer_ptr(outs[i], k);
      if (!h) continue;
      const size_t o0 = (size_t)r0 * rowpix * per_pix[k];
      const size_t len = (size_t)(r1 - r0) * rowpix * per_pix[k];
      MBGB_CUDA(cudaMemcpyAsync((char *)h + o0, stage + off[8 * i + k] + o0, len, cudaMemcpyDeviceToHost, s));
    }
  }
  MBGB_CUDA(cudaStreamSynchronize(s));
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_render_host(mbgb_context *c, const mbgb_scene *scene, const mbgb_image *out,
                                        const mbgb_opts *opts) {
  if (!c) return set_error(MBGB_ERR_BAD_PARAM, "NULL context");
  std::lock_guard<std::mutex> lk(c->mu);
  return render_frames_host(c, scene, 1, out, opts);
}

extern "C" mbgb_status mbgb_render_batch_host(mbgb_context *c, const mbgb_scene *frames, int32_t n,
                                              const mbgb_image *outs, const mbgb_opts *opts) {
  if (!c) return set_error(MBGB_ERR_BAD_PARAM, "NULL context");
  std::lock_guard<std::mutex> lk(c->mu);
  return render_frames_host(c, frames, n, outs, opts);
}

extern "C" mbgb_status mbgb_distance_device(mbgb_context *c, const mbgb_scene *scene, int precision,
                                            const double *points, const double *detail, int64_t n, double *dist,
                                            int32_t *iters, uint8_t *max_iter) {
  if (!c || !scene || (n > 0 && (!points || !detail || !dist || !iters || !max_iter)))
    return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  if (n < 0) return set_error(MBGB_ERR_BAD_PARAM, "negative point count");
  if (scene->formula != MBGB_FORMULA_TRIG_OPTIM && scene->formula != MBGB_FORMULA_TGLAD &&
      !runtime_formula(scene->formula))
    return set_error(MBGB_ERR_UNSUPPORTED, "formula not built on the device");
  if (n == 0) return MBGB_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  MBGB_CUDA(cudaSetDevice(c->device));
  cudaError_t e;
  if (precision == MBGB_PREC_FP64 || !scene->analitycDE) {  // delta-DE: FP64 under every policy
    FractalT<double> f;
    fill_fractal<double>(*scene, f);
    e = launch_distance_f64(distance_kernel_formula(*scene), f, points, detail, n, dist, iters,
                            max_iter, nullptr, c->stream);
  } else {
    FractalT<float> f;
    fill_fractal<float>(*scene, f);
    e = launch_distance_f32(distance_kernel_formula(*scene), f, points, detail, n, dist, iters,
                            max_iter, nullptr, c->stream);
  }
  if (e != cudaSuccess) return cuda_error(e, "distance kernel launch");
  MBGB_CUDA(cudaStreamSynchronize(c->stream));
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_compile_image16_device(mbgb_context *c, const mbgb_scene *scene,
                                                   const float *image_float, int32_t width, int32_t height,
                                                   uint16_t *image16) {
  if (!c || !scene || !image_float || !image16 || width <= 0 || height <= 0)
    return set_error(MBGB_ERR_BAD_PARAM, "bad argument");
  std::lock_guard<std::mutex> lk(c->mu);
  MBGB_CUDA(cudaSetDevice(c->device));
  MBGB_CUDA(c->ensure(c->post, sizeof(int) * 65536));
  return compile16_device(*scene, image_float, width, height, image16, (int *)c->post.ptr, c->stream);
}

extern "C" mbgb_status mbgb_ssao_device(mbgb_context *c, const mbgb_scene *scene, const mbgb_image *layers,
                                        uint16_t *image16) {
  if (!c || !scene || !layers || !image16) return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  if (!layers->zbuffer || !layers->opacity || !layers->colour)
    return set_error(MBGB_ERR_BAD_PARAM, "SSAO needs the z-buffer, opacity and colour layers");
  if (layers->width <= 0 || layers->height <= 0) return set_error(MBGB_ERR_BAD_PARAM, "bad image size");
  if (scene->SSAOQuality > 1000) return set_error(MBGB_ERR_BAD_PARAM, "SSAO quality above 1000");
  std::lock_guard<std::mutex> lk(c->mu);
  MBGB_CUDA(cudaSetDevice(c->device));
  MBGB_CUDA(c->ensure(c->post, std::max<size_t>(sizeof(int) * 65536, 16 * (size_t)(scene->SSAOQuality + 1))));
  return ssao_device(*scene, *layers, image16, c->post.ptr, c->stream);
}

extern "C" mbgb_status mbgb_dof_device(mbgb_context *c, const mbgb_scene *scene, const mbgb_image *layers,
                                       uint16_t *image16, uint32_t seed) {
  if (!c || !scene || !layers || !image16) return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  if (!layers->zbuffer || !layers->alpha) return set_error(MBGB_ERR_BAD_PARAM, "DOF needs the z-buffer and alpha layers");
  if (layers->width <= 0 || layers->height <= 0) return set_error(MBGB_ERR_BAD_PARAM, "bad image size");
  std::lock_guard<std::mutex> lk(c->mu);
  MBGB_CUDA(cudaSetDevice(c->device));
  return dof_device(*scene, *layers, image16, seed, c->stream);
}

// CompileImage / CalculatePixel / CalculateGammaTable (src/cimage.cpp:132-214), progressive factor 1.
extern "C" mbgb_status mbgb_compile_image16(const mbgb_scene *scene, const float *image_float, int32_t width,
                                            int32_t height, uint16_t *image16) {
  if (!scene || !image_float || !image16 || width <= 0 || height <= 0)
    return set_error(MBGB_ERR_BAD_PARAM, "bad argument");
  std::vector<int> gamma(65536);
  for (int i = 0; i < 65536; i++) gamma[i] = (int)(pow(i / 65536.0, 1.0 / scene->imageGamma) * 65535);
  const size_t n = (size_t)width * height;
  for (size_t i = 0; i < n; i++) {
    for (int c = 0; c < 3; c++) {
      float v = image_float[3 * i + c] * scene->brightness;
      v = (v - 0.5) * scene->contrast + 0.5;
      if (v < 0.0) v = 0.0;
      if (scene->hdrEnabled) v = tanhf(v);
      if (v > 1.0) v = 1.0;
      const unsigned short q = (unsigned short)(int)(v * 65535.0);
      image16[3 * i + c] = (uint16_t)gamma[q];
    }
  }
  return MBGB_OK;
}
