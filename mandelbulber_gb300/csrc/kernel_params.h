// Host/device parameter blocks of the ray-march kernels.
//
// The host derives these once per frame from an mbgb_scene (capi.cpp) the way
// MainThread prepares its locals (src/Render3D.cpp:213-344): camera rotation,
// ray start, light vector, the ambient-occlusion direction table. They travel as
// a by-value kernel parameter, so they live in the constant bank and graph
// captures carry them. ParamsT<float> is the pre-converted copy for the FP32
// kernels, so no kernel converts doubles on its hot path.
#pragma once

#include <cstdint>

namespace mbgb {

constexpr int kMaxMarchSteps = 10000;   // RayMarching loop bound (src/Render3D.cpp:94)
constexpr int kStepSlots = 10002;       // sStep buffer length per ray (src/Render3D.cpp:267)
constexpr int kStepCap = 1024;          // step records per thread slot in the main pass
constexpr int kOverflowThreads = 128;   // threads of the pass that re-renders rays longer than kStepCap
constexpr int kMaxAOVectors = 10000;    // sVectorsAround table (src/Render3D.cpp:272)
constexpr int kTileW = 8, kTileH = 4;   // one warp renders an 8x4 pixel tile

// Formulas the kernels select at run time (FORMULA 0 of compute(), formulas.cuh): every
// formula of enumFractalFormula (src/fractal.h:25-65) from trig_DE (1) to generalizedFoldBox
// (37) but trig_optim (2) and tglad (8), which have instantiations of their own. `none` (0)
// and ocl_custom (38) are not rendered.
inline bool runtime_formula(int formula) { return formula >= 1 && formula <= 37 && formula != 2 && formula != 8; }

// The instantiation a scene runs: 2 or 8, or 0 for the run-time formula path (every other
// formula, and 2 / 8 with the kaleidoscopic IFS pre-fold, which only that path carries).
inline int kernel_formula(int formula, bool ifsFolding) {
  return ((formula == 2 || formula == 8) && !ifsFolding) ? formula : 0;
}

template <typename T>
struct FractalT;
// Primitive objects next to (or instead of) the fractal: CalculateDistance then takes the
// nearest object (src/fractal.cpp:1383-1435), which only the run-time formula path carries.
template <typename T>
inline bool fractal_has_primitives(const FractalT<T> &f);

// Fractal / distance-estimator parameters (sFractal, src/fractal.h:255-293).
template <typename T>
struct FractalT {
  int formula;
  int N;            // (int)doubles.N
  int N5;           // (int)(doubles.N * 5): CalculateNormals (src/shaders.cpp:687)
  int N10;          // (int)(doubles.N * 10): SurfaceColour (src/shaders.cpp:855)
  int minN;
  int juliaMode, tgladFoldingMode, sphericalFoldingMode;
  int limits, iterThresh, interiorMode;
  int distPost;     // limits || iterThresh || interiorMode: CalculateDistance post-processes the orbit's result
  int lean;         // the lean FP32 orbit applies (Mandelbox without rotations, offsets, pre-folds or julia;
                    // power-8 Mandelbulb without pre-folds): CalculateDistance takes it in FP32
  int mbRotEnabled, mbMainRotZero;
  int mbRotZero[2][3];
  T power, constantFactor;
  // escape radius of the trigonometric formulas' distance mode and its square (the reference's
  // r > 100, src/fractal.cpp:1151-1157, unless the scene's bailoutRadius overrides it)
  T bailout, bailout2;
  T julia[3];
  T foldingLimit, foldingValue, sphFixed, sphMin;
  T mbScale, mbFoldLimit, mbFoldValue, mbMinR, mbFixedR;
  // lean Mandelbox sphere fold, derived on the host in T's arithmetic: k1 - 1 = fR^2/mR^2 - 1,
  // fR^2/(k1 - 1) and 1/(k1 - 1) (0 when k1 <= 1)
  T leanKm1, leanSa, leanSb;
  T mbOffset[3];
  T mbColX, mbColY, mbColZ, mbColR, mbColSp1, mbColSp2;
  T mbMainRot[9];
  T mbRot[2][3][9];
  T mbRotInv[2][3][9];
  T amin, amax, bmin, bmax, cmin, cmax;
  T mbVaryFold, mbVaryMinR, mbVaryScaleVary, mbVaryWadd, mbVaryRPower;   // mandelboxVaryScale4D
  // run-time formulas (formulas.cuh); each block is filled only when the formula (or a step
  // of the hybrid sequence) reads it, so frames that differ only in unused fields still share
  // a launch sequence
  int analytic, linearDE;          // analitycDE, linearDEmode: delta-DE distance when analytic == 0
  // kaleidoscopic IFS (sFractalIFS, src/fractal.h:138-148, prepared by RecalculateIFSParams)
  int ifsFolding, ifsAbsX, ifsAbsY, ifsAbsZ, ifsMenger, ifsMainRotZero;
  int ifsEnabled[9], ifsRotZero[9];
  T ifsScale, ifsOffset[3], ifsEdge[3];
  T ifsMainRot[9];
  T ifsRot[9][9];
  T ifsDir[9][3], ifsDist[9], ifsIntensity[9];
  // smoothMandelbox / generalizedFoldBox (sFractalMandelboxD, sFractalGeneralizedFoldBox)
  T mbSharpness, mbSolid, mbMelt;
  int gfbSides;
  T gfbNv[20][3];
  T intPowFold, intPowZ, cadd;     // foldingIntPow2, aexion
  // hybrid: the formula sequence as runs of (formula, iterations, power), repeated
  int hybridSegs;
  int hybridForm[5], hybridCount[5];
  T hybridPower[5];
  // Compute<orbitTrap> of the fake lights
  T fakeTrap[3];
  int fakeMinIter, fakeMaxIter;
  // primitive objects of CalculateDistance (sFractalPrimitives, src/fractal.h:195-222;
  // src/primitives.cpp); the plane normal is stored normalised, as PrimitivePlane uses it
  int planeEnable, boxEnable, invertedBoxEnable, sphereEnable, invertedSphereEnable, waterEnable, onlyPlane;
  int waterIterations, frameNo;
  T planeCentre[3], planeNormal[3], boxCentre[3], boxSize[3], invBoxCentre[3], invBoxSize[3];
  T sphereCentre[3], sphereRadius, invSphereCentre[3], invSphereRadius;
  T waterHeight, waterAmplitude, waterLength, waterRotation, waterAnimSpeed;
};

template <typename T>
inline bool fractal_has_primitives(const FractalT<T> &f) {
  return f.planeEnable || f.boxEnable || f.invertedBoxEnable || f.sphereEnable || f.invertedSphereEnable ||
         f.waterEnable || f.onlyPlane;
}

// enumObjectType (src/fractal.h:82-91): the object a CalculateDistance call ended on.
enum { kObjFractal = 0, kObjPlane = 1, kObjWater = 2, kObjSphere = 3, kObjSphereInv = 4, kObjBox = 5, kObjBoxInv = 6 };

// One auxiliary light (sLight, src/shaders.h:25-31): placed at random around a centre
// (PlaceRandomLights, src/shaders.cpp:1134-1208) or one of the four predefined lights.
template <typename T>
struct LightT {
  T pos[3];
  int colour[3];   // sRGB, 16-bit range
  T intensity;
  int enabled;
};

// Everything MainThread and the shaders read (sParamRender, src/fractparams.h:67-146).
template <typename T>
struct ParamsT {
  FractalT<T> f;
  // camera (src/Render3D.cpp:237-333, 389-438)
  int width, height, tiles, perspType, fishEyeCut;
  int row_begin, row_end;
  double tileXOffset, tileYOffset, aspect, fov;
  double rot[9];
  float rotf[9];     // FP32 copy for the FP32 policy's camera rays
  int rot_zero;
  double start[3];
  // march (src/Render3D.cpp:79-199)
  T viewDistanceMin, viewDistanceMax, resolution, persp, quality, DE_factor, smoothness;
  double resolution_d, persp_d, quality_d;   // FP64 hit refinement
  int constantDEThreshold, interiorMode, slowShading;
  int jitter;
  uint32_t jitter_seed;
  // shading (src/shaders.cpp:21-112, 480-926)
  T lightVect[3];
  T mainLight[3];
  T directLight, shading, specular, globalIlum;
  int shadow, penetrating, softShadow;
  T softRange;
  int ao, fastAO, aoQuality, aoCount;
  T fastAoTune;
  const T *aoVec;    // aoCount x 3, device memory
  T aoWeight[3];     // lightmap colour of each direction (white default texture: 255)
  int coloring;
  T coloringSpeed, paletteOffset;
  int palette[256][3];
  int bg1[3], bg2[3], bg3[3];
  // volumetric pass (src/shaders.cpp:185-478)
  int needVolumetric;
  T glowIntensity;
  int glow1[3], glow2[3];
  int postFog;
  T fogVisibility;   // pow(10, post_fog_visibility / 10 - 16), computed on the host
  int fogColor[3];
  T fogDensity, fogC1Dist, fogC2Dist, fogDistFactor;
  int fogCol1[3], fogCol2[3], fogCol3[3];
  // the FP32 walk's forms of the above, derived on the host: reciprocals of the fog
  // distances and of the post-fog visibility, fogDistFactor^2, and every colour divided by
  // 65536 (exact)
  T fogInvC1Dist, fogInvC2Dist, fogInvVisibility, fogDistFactor2;
  T fogColorS[3], fogCol1S[3], fogCol2S[3], fogCol3S[3];
  // auxiliary lights (AuxLightsShader / LightShading / AuxShadow, src/shaders.cpp:997-1132)
  int auxLightNumber;      // random lights; the shaders also read lights 0-3 when enabled
  int numberOfLights;      // max(auxLightNumber, 4), 0 when the scene has no aux lights
  T auxLightIntensity, auxLightVisibility;
  const LightT<T> *lights; // device memory, numberOfLights entries
  int iterFog, volLightAny;  // imageSwitches.iterFogEnabled / volumetricLightEnabled
  T iterFogOpacity, iterFogOpacityTrim;
  // volumetric lights: [0] the main light, [1..4] the predefined lights
  int volLightEnabled[5];
  T volLightIntensity[5];
  int mainLightColour[3];
  T mainLightIntensity;
  // fake (orbit trap) lights (FakeLights, src/shaders.cpp:1225-1271)
  int fakeLights;
  T fakeLightsIntensity, fakeLightsVisibility, fakeLightsVisibilitySize;
  // environment mapping on the default white texture (EnvMapping, src/shaders.cpp:785-811)
  int envMapping;
  T reflect;
  // primitive colours, 16-bit range: [plane, water, sphere, inverted sphere, box, inverted box]
  int primColour[6][3];
  // ray-traced reflections (src/Render3D.cpp:441-564): reflections after the camera ray, and
  // the primitives' reflection coefficients in primColour's order (the fractal's is reflect)
  int maxRay;
  T primReflect[6];
};

// Per-frame camera, resolution, fractal parameter and output layers of a batch (device
// memory, one per frame). Everything else of the scene is shared by the batch's frames
// (ParamsT).
// Built like MainThread's per-frame set-up (src/Render3D.cpp:213-344).
template <typename T>
struct FrameCam {
  int width, height, tiles, row_begin, row_end, rot_zero;
  int tileW, tileH;             // pixel tile of one warp's first 32 jobs (autotuned)
  int64_t pixBase;              // first pixel of the frame in the per-pixel buffers
  uint32_t jobBase, jobCount;   // primary jobs of the frame: [jobBase, jobBase + jobCount)
  double tileXOffset, tileYOffset, aspect, fov;
  double rot[9];
  float rotf[9];
  double start[3];
  T resolution, persp;
  double resolution_d, persp_d;
  T lightVect[3];
  T fparam;                     // the formula's main parameter: power (2) or Mandelbox scale (8)
  double fparam_d;
  float *image_float;
  float *zbuffer;
  uint16_t *alpha;
  uint16_t *opacity;
  uint8_t *colour;
  uint8_t *hit;
  int32_t *iters;
  double *depth;
};

// Output and scratch pointers of one launch (device memory).
struct FrameIO {
  float *image_float;
  float *zbuffer;
  uint16_t *alpha;
  uint16_t *opacity;
  uint8_t *colour;
  uint8_t *hit;
  int32_t *iters;
  double *depth;
  // Scratch: per resident thread, the primary ray's step records (sStep,
  // src/Render3D.h:32-39): step, distance and threshold, each [step_cap][slots].
  // A ray that needs more than step_cap records is appended to the overflow
  // list; the overflow pass (overflow_pass = 1) re-renders those pixels with
  // step_cap = kStepSlots and its own, smaller slot set.
  void *step_step, *step_dist, *step_thr;
  // the march position and iteration count of each record (sStep::point / iters), for the
  // volumetric terms that sample there (visible aux lights); null when unused
  void *step_scan;
  int *step_iters;
  int64_t slots;
  int rays;        // record sets per slot: 1, or the rays of the reflection loop
  int step_cap;
  int overflow_pass;
  unsigned int *overflow_count;   // zeroed before the main pass
  unsigned int *overflow_list;    // pixel indices, capacity = pixels of the frame
  unsigned int *tile_counter;     // zeroed before the launch
  unsigned long long *counters;   // [0] orbit iterations, [1] DE calls, [2] primary steps, [3] missed DE
  int *error_flag;                // set to 1 when the device deadline expires
  unsigned long long *start_ns;   // %globaltimer at the first tile claim (zeroed before the launch)
  unsigned long long budget_ns;   // device-side time budget, 0 = none
};

}  // namespace mbgb
