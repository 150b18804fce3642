/*
 * mbgb.h — C ABI of the GB300-native distance-estimated ray-march renderer.
 *
 * This library replaces one seam of Mandelbulber 1.21: the per-pixel render
 *   void Render(sParamRender param, cImage *image, GtkWidget *outputDarea)
 *   (src/Render3D.cpp:709), whose CPU branch (src/Render3D.cpp:719-1158) spawns
 *   MainThread workers (src/Render3D.cpp:203) that call RayMarching
 *   (src/Render3D.cpp:79) and the shaders (src/shaders.cpp:21-757), and whose
 *   OpenCL branch (src/Render3D.cpp:1160-1252, CclSupport::Render
 *   src/cl_support.cpp:527) is the existing precedent for a device drop-in.
 *
 * Everything crossing this boundary is plain C: POD structs, pointers, sizes.
 * The scene struct mirrors the reference's sParamRender / sFractal / sImageAdjustments
 * (src/fractparams.h:18-146, src/fractal.h:104-293, src/cimage.hpp:43-80) after the
 * -nogui fix-ups (src/interface.cpp:690-729) and clamps (src/interface.cpp:3587-3602).
 * Output layers have the element types and row-major order of cImage
 * (src/cimage.hpp:155-162): x + y * width.
 */
#ifndef MBGB_H_
#define MBGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MBGB_VERSION_MAJOR 0
#define MBGB_VERSION_MINOR 1
#define MBGB_VERSION_PATCH 0

/* Status codes. The reference's Render() returns void and prints errors
 * (src/cl_support.cpp:109 checkErr); every call here returns a status instead and never aborts. */
typedef enum mbgb_status {
  MBGB_OK = 0,
  MBGB_ERR_BAD_PARAM = 1,   /* NULL pointer, size out of range, malformed settings */
  MBGB_ERR_OOM = 2,         /* device or host allocation failed */
  MBGB_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  MBGB_ERR_TIMEOUT = 4,     /* a kernel hit its device-side deadline and stopped early */
  MBGB_ERR_UNSUPPORTED = 5, /* the scene uses a feature the library does not render */
  MBGB_ERR_IO = 6,          /* settings file could not be read / image could not be written */
  MBGB_ERR_NO_DEVICE = 7    /* no CUDA device visible */
} mbgb_status;

/* enumFractalFormula (src/fractal.h:25-64). The device evaluates every value from 1 to 37
 * (Compute<Mode>, src/fractal.cpp:189-1107); `none` (0) and ocl_custom (38) are rejected.
 * Formulas 1, 2, 7, 8, 10, 17, 18 and 37 have an analytic distance estimate; the others,
 * and the hybrid (12), use the delta-DE branch of CalculateDistance
 * (src/fractal.cpp:1308-1381) and render in FP64 under every precision policy. */
enum {
  MBGB_FORMULA_TRIG_DE = 1,         /* Mandelbulb with a derivative vector, src/fractal.cpp:189-209 */
  MBGB_FORMULA_TRIG_OPTIM = 2,      /* Mandelbulb, src/fractal.cpp:211-225 */
  MBGB_FORMULA_FAST_TRIG = 3,       /* power-2 Mandelbulb without trigonometry, :321-335 */
  MBGB_FORMULA_HYPERCOMPLEX = 4,    /* :351-359 */
  MBGB_FORMULA_QUATERNION = 5,      /* :360-368 */
  MBGB_FORMULA_MINUS_FAST_TRIG = 6, /* :336-350 */
  MBGB_FORMULA_MENGER = 7,          /* Menger sponge, :369-407 */
  MBGB_FORMULA_TGLAD = 8,           /* Mandelbox, :409-529 */
  MBGB_FORMULA_KALEIDOSCOPIC = 10,  /* kaleidoscopic IFS, :837-886 */
  MBGB_FORMULA_XENODREAMBUIE = 11,  /* :300-320 */
  MBGB_FORMULA_HYBRID = 12,         /* per-iteration formula sequence (CreateFormulaSequence) */
  MBGB_FORMULA_MANDELBULB2 = 13,    /* :226-254 */
  MBGB_FORMULA_MANDELBULB3 = 14,    /* :255-282 */
  MBGB_FORMULA_MANDELBULB4 = 15,    /* :283-299 */
  MBGB_FORMULA_FOLDING_INT_POW2 = 16, /* :794-836 */
  MBGB_FORMULA_SMOOTH_MANDELBOX = 17, /* :751-793 */
  MBGB_FORMULA_MBOX_VARY4D = 18,    /* Mandelbox with varying scale, 4D, :887-915 */
  MBGB_FORMULA_AEXION = 19,         /* 19-36: aexion, benesi, bristorbrot, invert X/Y/Z/R, */
  MBGB_FORMULA_ANGLE_MULTIPLY_Z = 36, /* sphericalFold, powXYZ, scale/offset X/Y/Z, angleMultiply X/Y/Z, :916-1100 */
  MBGB_FORMULA_GENERALIZED_FOLD_BOX = 37 /* :531-750 */
};

/* enumPerspectiveType (src/common_math.h:39-42) */
enum { MBGB_PERSP_THREE_POINT = 0, MBGB_PERSP_FISH_EYE = 1, MBGB_PERSP_EQUIRECT = 2, MBGB_PERSP_FISH_EYE_CUT = 3 };

typedef struct mbgb_rgb { int32_t R, G, B; } mbgb_rgb;   /* sRGB, src/cimage.hpp:37-42 */

/* One frame's render parameters: the fields of sParamRender that the settings
 * reader fills (LoadOneSetting, src/settings.cpp:700-1183) plus the values the
 * -nogui path derives from them. Angles are radians, as stored by the reference. */
typedef struct mbgb_scene {
  /* ---- sParamRenderD (src/fractparams.h:18-65) ---- */
  double zoom, DE_factor, resolution, persp, quality, smoothness;
  double alpha, beta, gamma;
  double DOFFocus, DOFRadius;
  double mainLightAlpha, mainLightBeta;
  double auxLightIntensity, auxLightMaxDist, auxLightDistributionRadius, auxLightVisibility;
  double auxLightPreIntensity[4];
  double stereoEyeDistance;
  double viewDistanceMin, viewDistanceMax;
  double volumetricLightIntensity[5];
  double fogDensity, fogColour1Distance, fogColour2Distance, fogDistanceFactor;
  double colourSaturation, fastAoTune, iterFogOpacity, iterFogOpacityTrim;
  double fakeLightsIntensity, fakeLightsVisibility, fakeLightsVisibilitySize;
  double shadowConeAngle;
  double primitivePlaneReflect, primitiveBoxReflect, primitiveInvertedBoxReflect;
  double primitiveSphereReflect, primitiveInvertedSphereReflect, primitiveWaterReflect;
  /* sImageAdjustments (src/cimage.hpp:43-59) */
  double shading, directLight, ambient, specular, reflect, globalIlum, brightness;
  double glow_intensity, fogVisibility, coloring_speed, imageGamma, paletteOffset;
  double mainLightIntensity, contrast;
  double vp[3];
  double auxLightPre[4][3];
  double auxLightRandomCenter[3];

  /* ---- sFractalD (src/fractal.h:233-253) ---- */
  double N;                     /* stored as double, truncated to int by Compute (src/fractal.cpp:53) */
  double amin, amax, bmin, bmax, cmin, cmax;
  double constantFactor, FoldingIntPowZfactor, FoldingIntPowFoldFactor;
  double foldingLimit, foldingValue, foldingSphericalMin, foldingSphericalFixed;
  double power, cadd;
  double hybridPower[5];
  double julia[3];
  double fakeLightsOrbitTrap[3];
  /* sFractalPrimitivesD (src/fractal.h:195-211) */
  double planeCentre[3], planeNormal[3], boxCentre[3], boxSize[3];
  double invertedBoxCentre[3], invertedBoxSize[3], sphereCentre[3];
  double sphereRadius;
  double invertedSphereCentre[3];
  double invertedSphereRadius, waterHeight, waterAmplitude, waterLength, waterRotation, waterAnimSpeed;

  /* ---- sFractalMandelboxD (src/fractal.h:160-180) ---- */
  double mboxRotationMain[3];        /* radians */
  double mboxRotation[2][3][3];      /* [fold][axis][component], radians */
  double mboxColorFactorX, mboxColorFactorY, mboxColorFactorZ, mboxColorFactorR;
  double mboxColorFactorSp1, mboxColorFactorSp2;
  double mboxScale, mboxFoldingLimit, mboxFoldingValue;
  double mboxFoldingSphericalMin, mboxFoldingSphericalFixed;
  double mboxSharpness, mboxSolid, mboxMelt;
  double mboxOffset[3];
  double mboxVaryFold, mboxVaryMinR, mboxVaryScaleVary, mboxVaryWadd, mboxVaryRPower;
  /* Derived by RecalculateIFSParams (src/callbacks.cpp:1549-1556): row-major 3x3
   * CRotationMatrix contents and its `zero` (identity short-cut) flag. */
  double mboxMainRot[9];
  double mboxRot[2][3][9];
  double mboxRotInv[2][3][9];
  int32_t mboxMainRotZero;
  int32_t mboxRotZero[2][3];

  /* ---- sFractalIFSD (src/fractal.h:104-118), parsed for completeness ---- */
  double ifsRotationGamma, ifsRotationAlfa, ifsRotationBeta, ifsScale;
  double ifsDistance[9], ifsAlfa[9], ifsBeta[9], ifsGamma[9], ifsIntensity[9];
  double ifsOffset[3];
  double ifsDirection[9][3];
  double ifsEdge[3];

  /* ---- integers ---- */
  int32_t image_width, image_height;
  int32_t globalIlumQuality, reflectionsMax, coloring_seed, auxLightRandomSeed, auxLightNumber;
  int32_t SSAOQuality, startFrame, endFrame, framesPerKeyframe, imageFormat;
  int32_t noOfTiles, tileCount;
  int32_t perspectiveType;
  int32_t formula, minN, frameNo;
  int32_t fakeLightsMinIter, fakeLightsMaxIter;
  int32_t hybridIters[5], hybridFormula[5];
  int32_t genFoldBoxType, waterIterations;

  /* ---- booleans (0/1) ---- */
  uint8_t shadow, global_ilumination, fastGlobalIllumination, slowShading;
  uint8_t texturedBackground, background_as_fulldome, SSAOEnabled, DOFEnabled;
  uint8_t auxLightPreEnabled[4], volumetricLightEnabled[5];
  uint8_t penetratingLights, stereoEnabled, fishEyeCut, fakeLightsEnabled;
  /* sImageSwitches (src/cimage.hpp:69-77) */
  uint8_t coloringEnabled, fogEnabled, raytracedReflections, volumetricLightEnabledAny;
  uint8_t iterFogEnabled, hdrEnabled;
  /* sFractal switches (src/fractal.h:259-272) */
  uint8_t limits_enabled, iterThresh, analitycDE, juliaMode, tgladFoldingMode;
  uint8_t sphericalFoldingMode, interiorMode, hybridCyclic, linearDEmode, constantDEThreshold;
  uint8_t mboxRotationsEnabled;
  uint8_t ifsFoldingMode, ifsAbsX, ifsAbsY, ifsAbsZ, ifsMengerSpongeMode;
  uint8_t ifsEnabled[9];
  /* sFractalPrimitives (src/fractal.h:213-222) */
  uint8_t planeEnable, boxEnable, invertedBoxEnable, sphereEnable, invertedSphereEnable;
  uint8_t waterEnable, onlyPlane;
  uint8_t paletteLoaded;        /* palette came from the file (not generated from coloring_seed) */
  uint16_t bailoutRadius;       /* not in the reference: escape radius of the trigonometric formulas' distance
                                 * mode (trig_DE, trig_optim); 0 = the reference's hard-coded r > 100
                                 * (src/fractal.cpp:1151-1157). No settings key sets it. */

  /* ---- colours (sRGB, 16-bit range unless noted) ---- */
  mbgb_rgb background_color1, background_color2, background_color3;
  mbgb_rgb auxLightPreColour[4];
  mbgb_rgb fogColour1, fogColour2, fogColour3;
  mbgb_rgb primitivePlaneColour, primitiveBoxColour, primitiveInvertedBoxColour;
  mbgb_rgb primitiveSphereColour, primitiveInvertedSphereColour, primitiveWaterColour;
  mbgb_rgb glow_color1, glow_color2, fogColor, mainLightColour;   /* sEffectColours */
  mbgb_rgb palette[256];        /* 8-bit range */

  double settingsVersion;
} mbgb_scene;

/* Output buffers: the cImage layers (src/cimage.hpp:155-162) the render writes.
 * Any pointer may be NULL (layer not wanted). Pointers are host memory for
 * mbgb_render_host and device memory for mbgb_render_device. Row-major, x + y * width. */
typedef struct mbgb_image {
  int32_t width, height;
  float *image_float;          /* sRGBfloat, 3 floats per pixel (PutPixelImage) */
  float *zbuffer;              /* float depth, 1e20 for background (PutPixelZBuffer) */
  uint16_t *alpha;             /* PutPixelAlpha */
  uint16_t *opacity;           /* PutPixelOpacity */
  uint8_t *colour;             /* sRGB8, 3 bytes per pixel (PutPixelColour) */
  /* debug / parity layers (no reference counterpart) */
  uint8_t *hit;                /* 1 where the primary ray found the surface (3: exact_hit missed the level set) */
  int32_t *iters;              /* orbit iterations of the last DE at the hit (itersOut) */
  double *depth;               /* primary-ray depth (scan) as double, 1e20 for background */
} mbgb_image;

/* Precision policies of the device march. */
enum {
  MBGB_PREC_FP64 = 0,          /* every DE evaluation and every march in double */
  MBGB_PREC_FP32_FIX = 1,      /* FP32 march/orbit with FP64 camera origin and FP64 hit refinement */
  MBGB_PREC_AUTO = 2           /* FP32_FIX unless the hit bisection's window at the nearest surface
                                * (0.01 x quality x the threshold there: FP64 distance estimate at the ray
                                * origin x resolution x persp / quality, or the constant threshold) is below
                                * 1e-7 of the scene scale (about one FP32 ulp), or the scene has the limit box
                                * (limits_enabled: its cut faces expose the fractal's interior, whose colouring
                                * orbits FP32 does not reproduce), then FP64 for the whole frame; the probe
                                * synchronises */
};

typedef struct mbgb_opts {
  int32_t precision;           /* MBGB_PREC_* */
  int32_t jitter;              /* 0: deterministic march (parity mode); 1: per-step counter-hash jitter */
  uint32_t jitter_seed;
  int32_t row_begin, row_end;  /* render only rows [row_begin, row_end); 0,0 = all rows */
  int32_t ctas_per_sm;         /* 0 = autotuned */
  int32_t threads_per_cta;     /* 0 = autotuned */
  int32_t deadline_ms;         /* device-side deadline; 0 = none */
  void *stream;                /* cudaStream_t; NULL = the context's stream */
  int32_t engine;              /* MBGB_ENGINE_*; 0 = wavefront stages */
  int32_t profile_stages;      /* 1: record CUDA events between stages (synchronous calls fill stage_ms) */
  int32_t polish_all;          /* FP32_FIX: 1 = re-run the end of every hit's bisection in FP64; 0 = only the
                                * hits whose FP32 bisection stopped early within 1e-4 of a window edge */
  int32_t tile_w, tile_h;      /* wavefront: pixel tile of a warp's first 32 primary rays (tile_w * tile_h
                                * = 32); 0,0 = autotuned or 8 x 4 */
  int32_t refill_min;          /* wavefront: idle lanes of a warp before it claims new rays; 0 = tuned or 8 */
  int32_t autotune;            /* 1: tile shape, threads per CTA, CTAs per SM and refill_min that are 0
                                * come from mbgb_autotune, run once per scene class and context */
  int32_t use_graph;           /* 1: the launches are captured once in a CUDA graph and replayed while
                                * the frames, outputs and options stay the same */
  int32_t exact_hit;           /* wavefront: 1 = after the binary refinement every hit is moved in FP64
                                * (Newton steps) onto the level set DE(P) = thr, the surface the
                                * differentiable render differentiates; 0 = the reference's window */
  int32_t orbit_refill;        /* wavefront, lean FP32 orbits (Mandelbox, power-8 Mandelbulb), shadow/AO
                                * rays: a warp runs orbit iterations until this many of its busy lanes
                                * have ended their orbits, then steps those rays on; 0 = tuned, else 8
                                * for the Mandelbulb and off for the Mandelbox (short orbits); -1 = off:
                                * lanes step on only after every orbit of the estimate ended */
  int32_t pair_rays;           /* wavefront, lean FP32 Mandelbox (orbit_refill off), shadow/AO rays: 1 = two
                                * rays per thread whose orbits advance together in packed FP32 (f32x2)
                                * instructions; 0 = one ray per thread (faster on GB300: 9.8 against
                                * 12.1 ms on the 1080p Mandelbox). Same pixels either way */
  int32_t hit_order;           /* wavefront, one ray per pixel (no reflections): the order of the shadow/AO
                                * jobs over the hits. 2 = the primary rays' pixel-tile order (a tile's rays
                                * share a warp), 1 = the order the primary rays finished in, 0 = tile order
                                * from 2^20 pixels per launch group on. Same pixels either way */
} mbgb_opts;

/* Launch configuration picked by mbgb_autotune. */
typedef struct mbgb_tuning {
  int32_t tile_w, tile_h;      /* primary-ray pixel tile */
  int32_t threads_per_cta;     /* 64 or 128 */
  int32_t ctas_per_sm;         /* resident CTAs per SM of the ray stages */
  int32_t refill_min;          /* idle lanes before a warp refills */
  double ms;                   /* device time of the picked configuration on the tuning frame */
  double ms_default;           /* device time of the default configuration (8 x 4, 128, max, 8) */
  int32_t trials;              /* configurations timed */
  int32_t orbit_refill;        /* ended orbits before a warp steps its shadow/AO rays on (0 = off) */
} mbgb_tuning;

/* Render engines (same results within the precision policy's tolerance). */
enum {
  MBGB_ENGINE_WAVEFRONT = 0,   /* ray-granular stages with lane refill (default) */
  MBGB_ENGINE_PER_PIXEL = 1    /* one thread renders a whole pixel; smallest scratch */
};

/* Per-render counters (the reference's N_counter, DE_counter, Pixel_counter,
 * Missed_DE_counter globals, src/Render3D.cpp:51-57), kept per context here. */
typedef struct mbgb_stats {
  uint64_t orbit_iterations;   /* N_counter: sum over DE calls of (L + 1) */
  uint64_t de_calls;           /* Loop_counter: Compute<> calls */
  uint64_t primary_steps;      /* DE_counter */
  uint64_t pixels;             /* Pixel_counter */
  uint64_t missed_de;          /* Missed_DE_counter */
  uint64_t long_rays;          /* primary rays longer than the main pass's step records (re-rendered) */
  uint64_t fp64_polished;      /* FP32_FIX, wavefront: hits whose bisection was finished in FP64 */
  uint64_t auto_fp64;          /* 1 if any frame of the last call was rendered in FP64 (MBGB_PREC_FP64, MBGB_PREC_AUTO's
                                  per-frame pick, or a delta-DE formula, which renders in FP64 under every policy) */
  double kernel_ms;            /* device time of the last render */
  /* per stage: [0] primary rays (wavefront) or the per-pixel kernel, [1] FP64 hit polish,
   * [2] shadow and AO rays, [3] composition, [4] level-set refinement (exact_hit),
   * [5] gradient stage (mbgb_render_grad) */
  uint64_t stage_orbit[6];     /* orbit iterations (stages 0-3, 5) */
  uint64_t stage_de[6];        /* DE evaluations (stages 0-3, 5) */
  double stage_ms[6];          /* device time between the stage's CUDA events (profile_stages = 1) */
  uint64_t frames;             /* frames of the last call */
  uint64_t launches;           /* kernels the last call launched (graph replays included) */
  uint64_t graph_replayed;     /* 1 if the last call replayed a captured CUDA graph */
  uint64_t level_set_missed;   /* exact_hit: hits whose Newton refinement did not reach the level set */
  uint64_t grad_pixels;        /* mbgb_render_grad: hit pixels differentiated */
  uint64_t grad_skipped;       /* mbgb_render_grad: hit pixels left out (level set missed, grazing ray) */
} mbgb_stats;

typedef struct mbgb_context mbgb_context;

/* ---- version / errors ---- */
const char *mbgb_version(void);
/* Thread-local text of the last error raised on this thread. */
const char *mbgb_last_error(void);

/* ---- settings (host only; no GPU needed) ----
 * Replaces LoadSettings / LoadSettings2 / LoadOneSetting / LoadSettingsPost
 * (src/settings.cpp:611-698, 700-1183, 1185-1195) plus the -nogui fix-ups of
 * ReadInterface (src/interface.cpp:690-729), CheckPrameters (src/interface.cpp:3587)
 * and RecalculateIFSParams (src/callbacks.cpp:1538-1556).
 * `defaults_path` may be NULL (then the scene starts zeroed, as the reference's
 * static noGUIdata does). `overrides` are "key=value" strings like the -o switch
 * (src/interface.cpp:3512-3519, src/settings.cpp:660-676). */
mbgb_status mbgb_scene_from_settings(const char *defaults_path, const char *path,
                                     const char *const *overrides, int n_overrides,
                                     mbgb_scene *out);
/* A string-valued setting (file_destination, file_keyframes, file_animation_path, ...) as
 * LoadSettings reads the same files and overrides (the last occurrence wins) into `out`.
 * MBGB_ERR_BAD_PARAM when the key occurs nowhere or `out_len` is too small. */
mbgb_status mbgb_settings_string(const char *defaults_path, const char *path, const char *const *overrides,
                                 int n_overrides, const char *key, char *out, int32_t out_len);
/* Apply one "key value" pair (LoadOneSetting). Returns MBGB_ERR_BAD_PARAM for an unknown key. */
mbgb_status mbgb_scene_set(mbgb_scene *scene, const char *key, const char *value);
/* Re-derive the dependent fields (analytic-DE flag, resolution, matrices, clamps) after edits. */
mbgb_status mbgb_scene_finalize(mbgb_scene *scene);
/* Scene of animation frame `frame` from `n_keys` keyframes, `frames_per_key` frames apart:
 * CMorph::CatmullRom (src/morph.cpp:49-109) over every interpolated double, as MainRender
 * applies it in keyframe mode (src/Render3D.cpp:2280-2291). The non-interpolated fields
 * come from `base` (NULL = keys[0]); derived fields are rebuilt (mbgb_scene_finalize). */
mbgb_status mbgb_scene_interpolate(const mbgb_scene *keys, int n_keys, int frames_per_key, int frame,
                                   const mbgb_scene *base, mbgb_scene *out);
/* The same spline on plain rows: keys[n_keys][size] -> out[size] for one frame. */
mbgb_status mbgb_catmull_rom(const double *keys, int n_keys, int size, int frames_per_key, int frame, double *out);
/* Palette of NewPalette (src/image.cpp:28-55) seeded like LoadSettingsPost (src/settings.cpp:1185-1195). */
void mbgb_palette_from_seed(int32_t seed, double saturation, mbgb_rgb palette[256]);
/* Report whether the device kernels can render this scene (MBGB_OK) or why not. */
mbgb_status mbgb_scene_supported(const mbgb_scene *scene);

/* ---- context ---- */
mbgb_status mbgb_context_create(int device, mbgb_context **out);
void mbgb_context_destroy(mbgb_context *ctx);
mbgb_status mbgb_get_stats(const mbgb_context *ctx, mbgb_stats *out);

/* ---- render ----
 * One frame; the drop-in for Render() (src/Render3D.cpp:709) writing the cImage
 * layers the way MainThread does (src/Render3D.cpp:569-589). `opts` may be NULL.
 * mbgb_render_device: `out` holds device pointers; the call is asynchronous on
 * the stream unless the stream is NULL (then it synchronises).
 * mbgb_render_host: `out` holds host pointers; copies in and out are part of the call. */
mbgb_status mbgb_render_device(mbgb_context *ctx, const mbgb_scene *scene,
                               const mbgb_image *out, const mbgb_opts *opts);
mbgb_status mbgb_render_host(mbgb_context *ctx, const mbgb_scene *scene,
                             const mbgb_image *out, const mbgb_opts *opts);

/* Batch of `n` frames (MainRender's keyframe / flight loops, src/Render3D.cpp:2144-2350,
 * each frame a Render() call at :2410/:2417) in one sequence of wavefront launches: frames
 * with the same fractal, shading and fog parameters share the launches, so cameras and
 * resolutions may differ from frame to frame. frames[i] renders into outs[i].
 * mbgb_render_batch: device pointers, asynchronous on opts->stream unless it is NULL.
 * mbgb_render_batch_host: host pointers, device staging and copies are part of the call.
 * A row range in opts applies to every frame. The per-pixel engine renders the frames one
 * by one. */
mbgb_status mbgb_render_batch(mbgb_context *ctx, const mbgb_scene *frames, int32_t n,
                              const mbgb_image *outs, const mbgb_opts *opts);
mbgb_status mbgb_render_batch_host(mbgb_context *ctx, const mbgb_scene *frames, int32_t n,
                                   const mbgb_image *outs, const mbgb_opts *opts);

/* Differentiable render (no counterpart in the reference; the reference's parameters
 * are only ever set by hand or by the keyframe splines). theta of a frame has
 * MBGB_GRAD_PARAMS entries: [0] the fractal parameter (power of formula 2, Mandelbox scale
 * of formula 8), [1..3] the camera position vp, [4] main light alpha, [5] main light
 * beta (radians). frames[i] is rendered into outs[i] (device layers) with every hit moved
 * onto the level set DE(P) = thr (opts->exact_hit is implied), and differentiated at
 * that point: implicit differentiation of the hit distance, forward-mode derivatives of
 * every distance estimate (the orbits are recomputed, not stored), the reference's
 * forward-difference normal, Lambert and specular shading. Hard shadows and the palette
 * colour are piecewise constant and contribute nothing.
 * dL_dimage: NULL or n device pointers to [height][width][3] floats (dL / d image_float);
 * jacobian: NULL or n device pointers to [height][width][3][MBGB_GRAD_PARAMS] floats;
 * dL_dtheta: NULL or host [n][MBGB_GRAD_PARAMS] doubles, the sums over pixels and channels
 * of dL/dI dI/dtheta. Precision MBGB_PREC_FP64 or MBGB_PREC_FP32_FIX. Scenes: formula 2, or
 * formula 8 without rotations, offset or pre-folds; no AO, glow, fog, interior mode,
 * limits, iteration threshold, soft or penetrating shadows (MBGB_ERR_UNSUPPORTED
 * otherwise). Synchronous. */
#define MBGB_GRAD_PARAMS 6
mbgb_status mbgb_render_grad(mbgb_context *ctx, const mbgb_scene *frames, int32_t n, const mbgb_image *outs,
                             const float *const *dL_dimage, float *const *jacobian, double *dL_dtheta,
                             const mbgb_opts *opts);

/* Autotuner of the wavefront launch configuration: times the candidate tile shapes,
 * threads per CTA, CTAs per SM and refill thresholds on `scene` (a representative frame,
 * rendered into context scratch) and returns the fastest. The result is cached in the
 * context for the scene's class (formula, orbit, precision, shadow / AO / volumetric
 * switches), where renders with opts->autotune = 1 pick it up. Synchronous. */
mbgb_status mbgb_autotune(mbgb_context *ctx, const mbgb_scene *scene, const mbgb_opts *opts,
                          mbgb_tuning *out);

/* Allocation-free render (no counterpart in the reference): the FP32_FIX render of
 * mbgb_render_device for callers that cannot allocate device memory while they
 * render — an application whose memory manager has already reserved the GPU for its
 * own pool, a plugin inside such a host, or a frame loop that must not call
 * cudaMalloc/cudaFree because they synchronise the device. It needs no context and
 * calls no allocator: its scratch is a set of static device arrays (79.4 MB in total)
 * that every GPU loading this library holds until the process exits. `out` holds
 * device pointers; the render runs on the current device and on opts->stream
 * (NULL = the legacy default stream, and the call then waits for the frame and
 * reports a device-deadline timeout). `opts` may be NULL (FP32_FIX, default stream).
 * opts->ctas_per_sm (0 = 2) sets the resident 96-thread CTAs per SM: the static step
 * records are then divided among more thread slots (at least 32 per slot, else
 * MBGB_ERR_BAD_PARAM), and rays longer than a slot's records take the slower overflow pass.
 * Limits: precision MBGB_PREC_FP32_FIX only (MBGB_PREC_AUTO, which picks FP64 for deep
 * zooms, and MBGB_PREC_FP64 are rejected with MBGB_ERR_BAD_PARAM); at most 4194304
 * pixels (e.g. 2048 x 2048), larger frames are rejected with MBGB_ERR_BAD_PARAM.
 * The first call on a device resolves the arrays' device addresses, so make that
 * first call before any stream capture. A call whose AO quality (globalIlumQuality)
 * differs from the previous call's on that device copies the AO direction table from
 * host memory on opts->stream; calls at an unchanged quality copy nothing. All calls
 * share the arrays, which keep the last call's contents: calls that overlap on the
 * GPU (other streams, other host threads) race and must be serialised by the caller. */
mbgb_status mbgb_render_device_noalloc(const mbgb_scene *scene, const mbgb_image *out, const mbgb_opts *opts);

/* Distance estimate at points (CalculateDistance, src/fractal.cpp:1245-1448) with
 * detailSize = detail[i]; writes dist[i], iters[i] (itersOut) and max_iter[i].
 * All pointers are device pointers. precision: MBGB_PREC_FP64 or MBGB_PREC_FP32_FIX (float orbit). */
mbgb_status mbgb_distance_device(mbgb_context *ctx, const mbgb_scene *scene, int precision,
                                 const double *points, const double *detail, int64_t n,
                                 double *dist, int32_t *iters, uint8_t *max_iter);

/* ---- image compile (src/cimage.cpp:132-214) ----
 * Gamma/brightness/contrast/HDR of CalculatePixel + CompileImage into RGB16, host pointers. */
mbgb_status mbgb_compile_image16(const mbgb_scene *scene, const float *image_float,
                                 int32_t width, int32_t height, uint16_t *image16);

/* SavePNG / SavePNG16 / SavePNG16Alpha (src/files.cpp:385-565): a PNG file of width x height
 * pixels, `channels` 3 (RGB) or 4 (RGBA), `bit_depth` 8 (uint8_t samples) or 16 (uint16_t
 * samples in host order; big-endian in the file), rows top to bottom. The pixel data are
 * stored in uncompressed deflate blocks (no zlib needed); decoders read the same samples
 * the reference's libpng files hold. Host pointers. */
mbgb_status mbgb_write_png(const char *path, int32_t width, int32_t height, int32_t bit_depth, int32_t channels,
                           const void *pixels);

/* CompileImage (src/cimage.cpp:132-214, progressive factor 1) on the device: image_float
 * (device, RGB float) -> image16 (device, RGB16) with the scene's brightness, contrast,
 * gamma and HDR switch. Synchronous on the context's stream. */
mbgb_status mbgb_compile_image16_device(mbgb_context *ctx, const mbgb_scene *scene, const float *image_float,
                                        int32_t width, int32_t height, uint16_t *image16);

/* PostRendering_SSAO (src/image.cpp:249-478) on the device, in place on image16 (device,
 * RGB16 from CompileImage), reading the z-buffer, opacity and colour layers of `layers`
 * (device pointers): scene->SSAOQuality directions x (quality - 1) samples per pixel,
 * intensity scene->globalIlum, the scene's perspective type and persp, in double (the
 * reference's arithmetic). Synchronous. */
mbgb_status mbgb_ssao_device(mbgb_context *ctx, const mbgb_scene *scene, const mbgb_image *layers,
                             uint16_t *image16);

/* PostRendering_DOF (src/image.cpp:57-206) in place on image16 (device, RGB16) and the alpha
 * layer of `layers` (device), reading its z-buffer: radius scene->DOFRadius x width / 1000,
 * focus 10^(scene->DOFFocus / 10 - 16). The splat order is the reference's: z-buffer
 * quicksort, then its Random() shuffle drawn from rand() seeded with `seed` (the reference
 * continues its process's rand() stream there). Synchronous. */
mbgb_status mbgb_dof_device(mbgb_context *ctx, const mbgb_scene *scene, const mbgb_image *layers,
                            uint16_t *image16, uint32_t seed);

#ifdef __cplusplus
}
#endif

#endif /* MBGB_H_ */
