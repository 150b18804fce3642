// C ABI of libmbgb: contexts, per-frame parameter derivation and the render
// entry points that stand in for Render() (src/Render3D.cpp:709).
#include <cuda_runtime.h>

#include <algorithm>
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
// WaveBufs layout (must match wave_core.cuh)
template <typename T>
struct WaveBufs {
  uint8_t *flags;
  T *scan, *dist, *thr, *step, *detail;
  int32_t *bis_left;
  T *point;
  int32_t *iters, *count;
  T *vol, *shadow, *ao;
  uint32_t *hit_list, *polish_list, *ctl, *overflow_list;
  T *pool_step, *pool_dist, *pool_thr;
  int32_t *pool_prev, *last_chunk;
  uint32_t pool_cap;
  int polish_all;
  int64_t npix;
};
constexpr int kChunk = 32;
constexpr int kPoolChunksPerPixel = 4;
}  // namespace mbgb

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

template <typename T>
static void fill_fractal(const mbgb_scene &s, FractalT<T> &f) {
  memset(&f, 0, sizeof(f));
  f.formula = s.formula;
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
  f.mbRotEnabled = s.mboxRotationsEnabled;
  f.mbMainRotZero = s.mboxMainRotZero;
  f.power = (T)s.power;
  f.constantFactor = (T)s.constantFactor;
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
  // The volumetric pass changes the pixel only through glow, post fog or volumetric fog.
  p.needVolumetric = (s.glow_intensity != 0.0) || s.fogEnabled || (s.fogDensity > 0.0);
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

struct mbgb_context {
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  DeviceBuf step[2][3];          // [precision][step, dist, thr], kStepCap records per slot
  DeviceBuf ovstep[2][3];        // overflow pass: kStepSlots records per slot, kOverflowThreads slots
  DeviceBuf ovlist;              // overflow pixel list
  DeviceBuf control;              // tile counter, error flag, counters
  DeviceBuf ao64, ao32;
  int ao_quality = -1;
  int ao_count = 0;
  DeviceBuf out[8];               // device staging for mbgb_render_host
  DeviceBuf wave[2];              // wavefront per-pixel buffers, per precision
  DeviceBuf probe;                // MBGB_PREC_AUTO: one-point distance probe
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t sev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   // stage events
  mbgb_stats stats{};
  std::mutex mu;
};

extern "C" const char *mbgb_version(void) { return "mbgb 0.1.0 (sm_103a)"; }

extern "C" const char *mbgb_last_error(void) { return g_last_error.c_str(); }

extern "C" mbgb_status mbgb_scene_supported(const mbgb_scene *s) {
  if (!s) return set_error(MBGB_ERR_BAD_PARAM, "NULL scene");
  if (s->formula != MBGB_FORMULA_TRIG_OPTIM && s->formula != MBGB_FORMULA_TGLAD)
    return set_error(MBGB_ERR_UNSUPPORTED, "formula " + std::to_string(s->formula) + " is not built on the device");
  if (!s->analitycDE) return set_error(MBGB_ERR_UNSUPPORTED, "delta-DE mode is not built on the device");
  if (s->ifsFoldingMode) return set_error(MBGB_ERR_UNSUPPORTED, "IFS folding mode");
  if (s->planeEnable || s->boxEnable || s->invertedBoxEnable || s->sphereEnable || s->invertedSphereEnable ||
      s->waterEnable || s->onlyPlane)
    return set_error(MBGB_ERR_UNSUPPORTED, "primitive objects");
  if (s->iterFogEnabled) return set_error(MBGB_ERR_UNSUPPORTED, "iteration fog");
  if (s->volumetricLightEnabledAny) return set_error(MBGB_ERR_UNSUPPORTED, "volumetric lights");
  if (s->fakeLightsEnabled) return set_error(MBGB_ERR_UNSUPPORTED, "fake (orbit trap) lights");
  if (s->auxLightNumber > 0) return set_error(MBGB_ERR_UNSUPPORTED, "random auxiliary lights");
  for (int i = 0; i < 4; i++)
    if (s->auxLightPreEnabled[i]) return set_error(MBGB_ERR_UNSUPPORTED, "predefined auxiliary lights");
  if (s->raytracedReflections && s->reflectionsMax > 0)
    return set_error(MBGB_ERR_UNSUPPORTED, "ray-traced reflections");
  if (!s->raytracedReflections && s->reflect > 0)
    return set_error(MBGB_ERR_UNSUPPORTED, "environment mapping (reflect > 0)");
  if (s->texturedBackground) return set_error(MBGB_ERR_UNSUPPORTED, "textured background");
  if (s->slowShading) return set_error(MBGB_ERR_UNSUPPORTED, "slow shading (averaged normals)");
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
      (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess ||
      (e = cudaEventCreate(&c->sev[0])) != cudaSuccess || (e = cudaEventCreate(&c->sev[1])) != cudaSuccess ||
      (e = cudaEventCreate(&c->sev[2])) != cudaSuccess || (e = cudaEventCreate(&c->sev[3])) != cudaSuccess ||
      (e = cudaEventCreate(&c->sev[4])) != cudaSuccess) {
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
  c->control.release();
  c->ao64.release();
  c->ao32.release();
  for (auto &b : c->out) b.release();
  for (auto &ev : c->sev)
    if (ev) cudaEventDestroy(ev);
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
  MBGB_CUDA(c->ao64.ensure(std::max<size_t>(v.size() * sizeof(double), 16)));
  MBGB_CUDA(c->ao32.ensure(std::max<size_t>(vf.size() * sizeof(float), 16)));
  MBGB_CUDA(cudaMemcpyAsync(c->ao64.ptr, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  MBGB_CUDA(cudaMemcpyAsync(c->ao32.ptr, vf.data(), vf.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  MBGB_CUDA(cudaStreamSynchronize(s));
  c->ao_quality = quality;
  c->ao_count = (int)(v.size() / 3);
  return MBGB_OK;
}

// The lean FP32 Mandelbox orbit applies: formula 8 without rotations, offset, pre-folds,
// julia, limits, iteration threshold or interior mode, and fold value = 2 x fold limit.
static bool fast_mandelbox(const mbgb_scene &s) {
  return s.formula == MBGB_FORMULA_TGLAD && !s.mboxRotationsEnabled && s.mboxMainRotZero && !s.juliaMode &&
         !s.tgladFoldingMode && !s.sphericalFoldingMode && !s.limits_enabled && !s.iterThresh && !s.interiorMode &&
         s.mboxOffset[0] == 0.0 && s.mboxOffset[1] == 0.0 && s.mboxOffset[2] == 0.0 &&
         s.mboxFoldingValue == 2.0 * s.mboxFoldingLimit;
}

// The power-8 Mandelbulb orbit without transcendentals applies (formula 2, power 8,
// no pre-folds, limits, iteration threshold or interior mode).
static bool fast_mandelbulb(const mbgb_scene &s) {
  return s.formula == MBGB_FORMULA_TRIG_OPTIM && s.power == 8.0 && !s.tgladFoldingMode && !s.sphericalFoldingMode &&
         !s.limits_enabled && !s.iterThresh && !s.interiorMode;
}

// Wavefront stages (wave_core.cuh): primary rays, FP64 polish (FP32 policy), shadow/AO
// rays, composition. All launches are enqueued on `s` without host round trips.
template <typename T>
static mbgb_status render_wave(mbgb_context *c, const mbgb_scene *scene, const mbgb_image *img, const mbgb_opts &o,
                               cudaStream_t s, const int prec, FrameIO io, bool needVol, uint32_t **long_rays_ctl) {
  const int64_t npix = (int64_t)scene->image_width * scene->image_height;
  const int block = 128;
  const bool rayAO = scene->global_ilumination && !scene->fastGlobalIllumination;
  const int aoN = rayAO ? c->ao_count : 0;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off += (bytes + 255) & ~(size_t)255;
    return at;
  };
  const size_t ts = sizeof(T);
  const size_t o_flags = take(npix), o_scan = take(npix * ts), o_dist = take(npix * ts), o_thr = take(npix * ts);
  const size_t o_step = take(npix * ts), o_detail = take(npix * ts), o_bis = take(npix * 4);
  const size_t o_point = take(3 * npix * ts), o_iters = take(npix * 4), o_count = take(npix * 4);
  const size_t o_vol = take(6 * npix * ts), o_shadow = take(npix * ts), o_ao = take((size_t)aoN * npix * ts);
  const size_t o_hit = take(npix * 4), o_pol = take(npix * 4), o_ovl = take(npix * 4), o_ctl = take(64);
  const size_t o_last = take(npix * 4);
  const uint32_t poolCap = needVol ? (uint32_t)std::min<int64_t>(npix * kPoolChunksPerPixel, 0x7fffffff) : 1u;
  const size_t o_pstep = take((size_t)poolCap * kChunk * ts), o_pdist = take((size_t)poolCap * kChunk * ts);
  const size_t o_pthr = take((size_t)poolCap * kChunk * ts), o_pprev = take((size_t)poolCap * 4);
  MBGB_CUDA(c->wave[prec].ensure(off));
  char *base = (char *)c->wave[prec].ptr;
  WaveLaunch<T> L;
  WaveBufs<T> &wb = L.wb;
  wb.flags = (uint8_t *)(base + o_flags);
  wb.scan = (T *)(base + o_scan);
  wb.dist = (T *)(base + o_dist);
  wb.thr = (T *)(base + o_thr);
  wb.step = (T *)(base + o_step);
  wb.detail = (T *)(base + o_detail);
  wb.bis_left = (int32_t *)(base + o_bis);
  wb.point = (T *)(base + o_point);
  wb.iters = (int32_t *)(base + o_iters);
  wb.count = (int32_t *)(base + o_count);
  wb.vol = (T *)(base + o_vol);
  wb.shadow = (T *)(base + o_shadow);
  wb.ao = (T *)(base + o_ao);
  wb.hit_list = (uint32_t *)(base + o_hit);
  wb.polish_list = (uint32_t *)(base + o_pol);
  wb.overflow_list = (uint32_t *)(base + o_ovl);
  wb.ctl = (uint32_t *)(base + o_ctl);
  wb.last_chunk = (int32_t *)(base + o_last);
  wb.pool_step = (T *)(base + o_pstep);
  wb.pool_dist = (T *)(base + o_pdist);
  wb.pool_thr = (T *)(base + o_pthr);
  wb.pool_prev = (int32_t *)(base + o_pprev);
  wb.pool_cap = poolCap;
  wb.polish_all = o.polish_all;
  wb.npix = npix;
  MBGB_CUDA(cudaMemsetAsync(wb.ctl, 0, 64, s));

  int occ1 = (sizeof(T) == 8) ? occupancy_wave_f64(scene->formula, block, 0) : occupancy_wave_f32(scene->formula, block, 0);
  int occ2 = (sizeof(T) == 8) ? occupancy_wave_f64(scene->formula, block, 1) : occupancy_wave_f32(scene->formula, block, 1);
  if (occ1 < 1) occ1 = 1;
  if (occ2 < 1) occ2 = 1;
  if (o.ctas_per_sm > 0) {
    occ1 = std::min(occ1, o.ctas_per_sm);
    occ2 = std::min(occ2, o.ctas_per_sm);
  }
  L.grid = c->sms * occ1;
  L.grid2 = c->sms * occ2;
  L.block = block;
  L.ov_grid = kOverflowThreads / block > 0 ? kOverflowThreads / block : 1;
  L.polish_grid = c->sms * 8;
  const int64_t nrow = (int64_t)(o.row_end - o.row_begin) * scene->image_width;
  L.compose_grid = (int)std::min<int64_t>((nrow + block - 1) / block, (int64_t)c->sms * 32);
  if (L.compose_grid < 1) L.compose_grid = 1;
  const int64_t slots = (int64_t)L.grid * block;
  io.slots = slots;
  io.step_cap = kStepCap;
  io.overflow_pass = 0;
  const size_t esz = sizeof(T);
  if (needVol) {
    const size_t bytes = (size_t)kStepCap * (size_t)slots * esz;
    const size_t obytes = (size_t)kStepSlots * (size_t)kOverflowThreads * esz;
    for (int k = 0; k < 3; k++) {
      MBGB_CUDA(c->step[prec][k].ensure(bytes));
      MBGB_CUDA(c->ovstep[prec][k].ensure(obytes));
    }
    io.step_step = c->step[prec][0].ptr;
    io.step_dist = c->step[prec][1].ptr;
    io.step_thr = c->step[prec][2].ptr;
  }
  L.io = io;
  L.ov = io;
  L.ov.overflow_pass = 1;
  L.ov.step_cap = kStepSlots;
  L.ov.slots = kOverflowThreads;
  L.ov.step_step = c->ovstep[prec][0].ptr;
  L.ov.step_dist = c->ovstep[prec][1].ptr;
  L.ov.step_thr = c->ovstep[prec][2].ptr;
  L.overflow = needVol;
  for (int k = 0; k < 5; k++) L.ev[k] = o.profile_stages ? c->sev[k] : nullptr;
  L.fast = fast_mandelbox(*scene) || fast_mandelbulb(*scene);
  fill_fractal<double>(*scene, L.fd);
  fill_params<T>(*scene, L.p, o, (const T *)(sizeof(T) == 8 ? c->ao64.ptr : c->ao32.ptr), c->ao_count);
  cudaError_t e;
  if constexpr (sizeof(T) == 8) e = launch_wave_f64(L, s);
  else e = launch_wave_f32(L, s);
  if (e != cudaSuccess) return cuda_error(e, "wavefront launch");
  *long_rays_ctl = wb.ctl + 3;
  (void)img;
  return MBGB_OK;
}

static mbgb_status render_device_impl(mbgb_context *c, const mbgb_scene *scene, const mbgb_image *img,
                                      const mbgb_opts *opts_in) {
  if (!c || !scene || !img) return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  mbgb_status st = mbgb_scene_supported(scene);
  if (st != MBGB_OK) return st;
  if (img->width != scene->image_width || img->height != scene->image_height)
    return set_error(MBGB_ERR_BAD_PARAM, "image size does not match the scene");
  mbgb_opts o{};
  if (opts_in) o = *opts_in;
  if (o.precision < 0 || o.precision > 2) return set_error(MBGB_ERR_BAD_PARAM, "unknown precision policy");
  if (o.row_end == 0) o.row_end = scene->image_height;
  if (o.row_begin < 0 || o.row_end > scene->image_height || o.row_begin >= o.row_end)
    return set_error(MBGB_ERR_BAD_PARAM, "row range out of bounds");
  MBGB_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = o.stream ? (cudaStream_t)o.stream : c->stream;
  int prec = (o.precision == MBGB_PREC_FP64) ? 0 : 1;
  if (o.precision == MBGB_PREC_AUTO) {
    // Deep-zoom rule: FP64 for the whole frame when the pixel footprint at the nearest
    // surface, d * resolution * persp / quality with d the FP64 distance estimate at the
    // ray origin, is below 1e-5 of the scene scale (max(1, |origin|)).
    ParamsT<double> pp;
    fill_params<double>(*scene, pp, o, nullptr, 0);
    double host[5] = {pp.start[0], pp.start[1], pp.start[2], 0.0, 0.0};
    host[3] = 1e-300;
    MBGB_CUDA(c->probe.ensure(128));
    char *pb = (char *)c->probe.ptr;
    MBGB_CUDA(cudaMemcpyAsync(pb, host, 4 * sizeof(double), cudaMemcpyHostToDevice, s));
    FractalT<double> fp;
    fill_fractal<double>(*scene, fp);
    cudaError_t pe = launch_distance_f64(scene->formula, fp, (const double *)pb, (const double *)(pb + 24), 1,
                                         (double *)(pb + 32), (int *)(pb + 40), (unsigned char *)(pb + 44), nullptr, s);
    if (pe != cudaSuccess) return cuda_error(pe, "precision probe");
    double d = 0.0;
    MBGB_CUDA(cudaMemcpyAsync(&d, pb + 32, sizeof(double), cudaMemcpyDeviceToHost, s));
    MBGB_CUDA(cudaStreamSynchronize(s));
    const double scale = std::max(1.0, sqrt(host[0] * host[0] + host[1] * host[1] + host[2] * host[2]));
    const double footprint = scene->constantDEThreshold ? scene->quality
                                                        : d * scene->resolution * scene->persp / scene->quality;
    prec = footprint < 1e-5 * scale ? 0 : 1;
    c->stats.auto_fp64 = prec == 0;
  }
  st = ensure_ao(c, scene->globalIlumQuality, s);
  if (st != MBGB_OK) return st;

  const int block = o.threads_per_cta > 0 ? o.threads_per_cta : 128;
  if (block % 32 != 0 || block > 128) return set_error(MBGB_ERR_BAD_PARAM, "threads_per_cta must be a multiple of 32, <= 128");
  int per_sm = occupancy_render(prec, scene->formula, block);
  if (per_sm < 1) per_sm = 1;
  if (o.ctas_per_sm > 0) per_sm = std::min(per_sm, o.ctas_per_sm);
  const int grid = c->sms * per_sm;
  const int64_t slots = (int64_t)grid * block;

  FrameIO io{};
  io.image_float = img->image_float;
  io.zbuffer = img->zbuffer;
  io.alpha = img->alpha;
  io.opacity = img->opacity;
  io.colour = img->colour;
  io.hit = img->hit;
  io.iters = img->iters;
  io.depth = img->depth;
  io.slots = slots;
  io.step_cap = kStepCap;
  io.overflow_pass = 0;
  const bool needVol = (scene->glow_intensity != 0.0) || scene->fogEnabled || (scene->fogDensity > 0.0);
  const size_t esz = prec == 0 ? sizeof(double) : sizeof(float);
  const bool rayAOjobs = scene->global_ilumination && !scene->fastGlobalIllumination;
  const double jobs = (double)scene->image_width * scene->image_height * (1.0 + (rayAOjobs ? c->ao_count : 0));
  const bool wave = o.engine == MBGB_ENGINE_WAVEFRONT && jobs < 4.0e9;
  if (needVol && !wave) {
    const size_t bytes = (size_t)kStepCap * (size_t)slots * esz;
    const size_t obytes = (size_t)kStepSlots * (size_t)kOverflowThreads * esz;
    for (int k = 0; k < 3; k++) {
      MBGB_CUDA(c->step[prec][k].ensure(bytes));
      MBGB_CUDA(c->ovstep[prec][k].ensure(obytes));
    }
    MBGB_CUDA(c->ovlist.ensure((size_t)scene->image_width * scene->image_height * sizeof(unsigned int)));
    io.step_step = c->step[prec][0].ptr;
    io.step_dist = c->step[prec][1].ptr;
    io.step_thr = c->step[prec][2].ptr;
    io.overflow_list = (unsigned int *)c->ovlist.ptr;
  }
  MBGB_CUDA(c->control.ensure(256));
  char *ctl = (char *)c->control.ptr;
  io.tile_counter = (unsigned int *)(ctl + 0);
  io.overflow_count = (unsigned int *)(ctl + 4);
  io.error_flag = (int *)(ctl + 16);
  io.counters = (unsigned long long *)(ctl + 64);
  io.start_ns = (unsigned long long *)(ctl + 32);
  io.budget_ns = o.deadline_ms > 0 ? (unsigned long long)o.deadline_ms * 1000000ull : 0ull;
  MBGB_CUDA(cudaMemsetAsync(ctl, 0, 256, s));
  FractalT<double> fd;
  fill_fractal<double>(*scene, fd);
  MBGB_CUDA(cudaEventRecord(c->ev0, s));
  cudaError_t e;
  uint32_t *longRays = (uint32_t *)(ctl + 4);
  if (wave) {
    mbgb_status ws = prec == 0 ? render_wave<double>(c, scene, img, o, s, 0, io, needVol, &longRays)
                               : render_wave<float>(c, scene, img, o, s, 1, io, needVol, &longRays);
    if (ws != MBGB_OK) return ws;
  }
  // per-pixel engine: main pass, then (when the step buffer is in use) the overflow pass
  FrameIO ov = io;
  ov.overflow_pass = 1;
  ov.step_cap = kStepSlots;
  ov.slots = kOverflowThreads;
  ov.step_step = c->ovstep[prec][0].ptr;
  ov.step_dist = c->ovstep[prec][1].ptr;
  ov.step_thr = c->ovstep[prec][2].ptr;
  const int ovBlocks = kOverflowThreads / block > 0 ? kOverflowThreads / block : 1;
  if (wave) {
    e = cudaSuccess;
  } else if (prec == 0) {
    ParamsT<double> p;
    fill_params<double>(*scene, p, o, (const double *)c->ao64.ptr, c->ao_count);
    e = launch_render_f64(scene->formula, p, fd, io, grid, block, s);
    if (e == cudaSuccess && needVol) e = launch_render_f64(scene->formula, p, fd, ov, ovBlocks, block, s);
  } else {
    ParamsT<float> p;
    fill_params<float>(*scene, p, o, (const float *)c->ao32.ptr, c->ao_count);
    e = launch_render_f32(scene->formula, p, fd, io, grid, block, s);
    if (e == cudaSuccess && needVol) e = launch_render_f32(scene->formula, p, fd, ov, ovBlocks, block, s);
  }
  if (e != cudaSuccess) return cuda_error(e, "render kernel launch");
  MBGB_CUDA(cudaEventRecord(c->ev1, s));
  if (!o.stream) {
    MBGB_CUDA(cudaStreamSynchronize(s));
    unsigned long long cnt[16];
    int flag = 0;
    unsigned int nover = 0;
    MBGB_CUDA(cudaMemcpy(cnt, ctl + 64, sizeof(cnt), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 4; k++) {
      c->stats.stage_orbit[k] = cnt[4 * k + 0];
      c->stats.stage_de[k] = cnt[4 * k + 1];
      c->stats.stage_ms[k] = 0.0;
      if (wave && o.profile_stages) {
        float sm = 0;
        if (cudaEventElapsedTime(&sm, c->sev[k], c->sev[k + 1]) == cudaSuccess) c->stats.stage_ms[k] = sm;
      }
    }
    for (int k = 1; k < 4; k++) {
      cnt[0] += cnt[4 * k + 0];
      cnt[1] += cnt[4 * k + 1];
      cnt[2] += cnt[4 * k + 2];
      cnt[3] += cnt[4 * k + 3];
    }
    MBGB_CUDA(cudaMemcpy(&flag, ctl + 16, sizeof(flag), cudaMemcpyDeviceToHost));
    MBGB_CUDA(cudaMemcpy(&nover, longRays, sizeof(nover), cudaMemcpyDeviceToHost));
    c->stats.long_rays = nover;
    c->stats.fp64_polished = 0;
    if (wave && prec == 1) {
      uint32_t npol = 0;
      MBGB_CUDA(cudaMemcpy(&npol, longRays + 3, sizeof(npol), cudaMemcpyDeviceToHost));
      c->stats.fp64_polished = npol;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->stats.orbit_iterations = cnt[0];
    c->stats.de_calls = cnt[1];
    c->stats.primary_steps = cnt[2];
    c->stats.missed_de = cnt[3];
    c->stats.pixels = (uint64_t)(o.row_end - o.row_begin) * (uint64_t)scene->image_width;
    c->stats.kernel_ms = ms;
    if (flag) return set_error(MBGB_ERR_TIMEOUT, "render stopped at its device deadline");
  }
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_render_device(mbgb_context *c, const mbgb_scene *scene, const mbgb_image *out,
                                          const mbgb_opts *opts) {
  if (!c) return set_error(MBGB_ERR_BAD_PARAM, "NULL context");
  std::lock_guard<std::mutex> lk(c->mu);
  return render_device_impl(c, scene, out, opts);
}

extern "C" mbgb_status mbgb_render_host(mbgb_context *c, const mbgb_scene *scene, const mbgb_image *out,
                                        const mbgb_opts *opts) {
  if (!c || !scene || !out) return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (out->width != scene->image_width || out->height != scene->image_height)
    return set_error(MBGB_ERR_BAD_PARAM, "image size does not match the scene");
  MBGB_CUDA(cudaSetDevice(c->device));
  const size_t npix = (size_t)out->width * out->height;
  struct Layer {
    void *host;
    size_t bytes;
  } layers[8] = {{out->image_float, npix * 12}, {out->zbuffer, npix * 4}, {out->alpha, npix * 2},
                 {out->opacity, npix * 2},      {out->colour, npix * 3},  {out->hit, npix},
                 {out->iters, npix * 4},        {out->depth, npix * 8}};
  void *dev[8] = {nullptr};
  for (int i = 0; i < 8; i++) {
    if (!layers[i].host) continue;
    MBGB_CUDA(c->out[i].ensure(layers[i].bytes));
    dev[i] = c->out[i].ptr;
  }
  mbgb_image d = *out;
  d.image_float = (float *)dev[0];
  d.zbuffer = (float *)dev[1];
  d.alpha = (uint16_t *)dev[2];
  d.opacity = (uint16_t *)dev[3];
  d.colour = (uint8_t *)dev[4];
  d.hit = (uint8_t *)dev[5];
  d.iters = (int32_t *)dev[6];
  d.depth = (double *)dev[7];
  mbgb_opts o{};
  if (opts) o = *opts;
  cudaStream_t s = o.stream ? (cudaStream_t)o.stream : c->stream;
  o.stream = nullptr;  // synchronous render on the context stream
  if (s != c->stream) o.stream = s;
  mbgb_status st = render_device_impl(c, scene, &d, &o);
  if (st != MBGB_OK) return st;
  // rows outside [row_begin, row_end) are not copied back
  const int r0 = o.row_begin, r1 = o.row_end > 0 ? o.row_end : out->height;
  const size_t rowpix = (size_t)out->width;
  const size_t per_pix[8] = {12, 4, 2, 2, 3, 1, 4, 8};
  for (int i = 0; i < 8; i++) {
    if (!layers[i].host) continue;
    const size_t off = (size_t)r0 * rowpix * per_pix[i];
    const size_t len = (size_t)(r1 - r0) * rowpix * per_pix[i];
    MBGB_CUDA(cudaMemcpyAsync((char *)layers[i].host + off, (char *)dev[i] + off, len, cudaMemcpyDeviceToHost, s));
  }
  MBGB_CUDA(cudaStreamSynchronize(s));
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_distance_device(mbgb_context *c, const mbgb_scene *scene, int precision,
                                            const double *points, const double *detail, int64_t n, double *dist,
                                            int32_t *iters, uint8_t *max_iter) {
  if (!c || !scene || (n > 0 && (!points || !detail || !dist || !iters || !max_iter)))
    return set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  if (n < 0) return set_error(MBGB_ERR_BAD_PARAM, "negative point count");
  if (scene->formula != MBGB_FORMULA_TRIG_OPTIM && scene->formula != MBGB_FORMULA_TGLAD)
    return set_error(MBGB_ERR_UNSUPPORTED, "formula not built on the device");
  if (n == 0) return MBGB_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  MBGB_CUDA(cudaSetDevice(c->device));
  cudaError_t e;
  if (precision == MBGB_PREC_FP64) {
    FractalT<double> f;
    fill_fractal<double>(*scene, f);
    e = launch_distance_f64(scene->formula, f, points, detail, n, dist, iters, max_iter, nullptr, c->stream);
  } else {
    FractalT<float> f;
    fill_fractal<float>(*scene, f);
    e = launch_distance_f32(scene->formula, f, points, detail, n, dist, iters, max_iter, nullptr, c->stream);
  }
  if (e != cudaSuccess) return cuda_error(e, "distance kernel launch");
  MBGB_CUDA(cudaStreamSynchronize(c->stream));
  return MBGB_OK;
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
