// Allocation-free variant of the FP32 render entry point.
//
// Who needs it: callers that must not allocate device memory while they render —
// a host application whose memory manager has already reserved the GPU's memory
// for its own pool, a plugin running inside such a host, or a frame loop that
// cannot afford cudaMalloc/cudaFree (they synchronise the device and can stall it).
// Such callers pass their own input scene and output layers; the scratch this
// render needs (the primary rays' step records, the overflow pass's records and
// pixel list, the AO direction table, the tile counter and flags) lives in
// fixed-size static device arrays defined below, 79.4 MB (75.8 MiB) in total,
// which every GPU that loads the library holds until the process exits.
//
// Limits: FP32-with-FP64-refinement policy only (MBGB_PREC_FP32_FIX; MBGB_PREC_AUTO is
// refused, since it would pick FP64 for deep zooms); at most kNaMaxPixels pixels
// (the overflow pixel list is sized for that); rays longer than a thread slot's step
// records (134 at the default launch of two 96-thread CTAs per SM on 152 SMs; 256 at one,
// opts->ctas_per_sm) go to the overflow pass (exact, but slower than mbgb_render_device).
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "kernel_params.h"
#include "launch.h"
#include "mbgb.h"
#include "mbgb_internal.h"

namespace {

using mbgb::kMaxAOVectors;
using mbgb::kOverflowThreads;
using mbgb::kStepSlots;

constexpr int kNaMaxCtas = 160;                      // CTAs of the default launch: one per SM (GB300 has 152)
constexpr int kNaThreads = 96;                       // threads per CTA
constexpr int kNaSlots = kNaMaxCtas * kNaThreads;    // thread slots of the default launch
constexpr int kNaStepCap = 256;                      // step records per slot of the default launch
constexpr long long kNaRecords = (long long)kNaStepCap * kNaSlots;   // records per step array
constexpr int kNaMinStepCap = 32;                    // fewest records per slot a launch may keep
constexpr int kNaDefaultCtasPerSm = 2;               // default launch: 134 records per slot on 152 SMs
constexpr long long kNaMaxPixels = 4194304;          // 2048 x 2048; 1920 x 1080 fits
constexpr int kMaxDevices = 64;

// Static scratch (sizes in floats unless noted):
__device__ __align__(256) float g_na_steps[3][(size_t)kNaRecords];                          // 47.2 MB
__device__ __align__(256) float g_na_ovsteps[3][(size_t)kStepSlots * kOverflowThreads];    // 15.4 MB
__device__ __align__(256) unsigned int g_na_ovlist[kNaMaxPixels];                          // 16.8 MB
__device__ __align__(256) float g_na_ao[3 * kMaxAOVectors];                                // 117 KiB
__device__ __align__(256) unsigned long long g_na_control[32];                             // counters, flags

struct DeviceSymbols {
  float *steps = nullptr;
  float *ovsteps = nullptr;
  unsigned int *ovlist = nullptr;
  float *ao = nullptr;
  unsigned long long *control = nullptr;
  int sms = 0;
  bool ready = false;
  int aoQuality = -1;   // globalIlumQuality whose direction table g_na_ao holds (-1: none yet)
  int aoCount = 0;      // directions in that table
};

DeviceSymbols g_sym[kMaxDevices];
std::mutex g_setup_mu;
std::mutex g_ao_mu;
float g_ao_host[3 * kMaxAOVectors];   // host staging of the AO table (no heap use)

// Resolves the device addresses of the static arrays once per device, with that
// device current. In host code the arrays' names are host-side stand-ins, never
// device addresses; only these resolved pointers go to the kernel.
mbgb_status setup_device(int dev, DeviceSymbols **out) {
  if (dev < 0 || dev >= kMaxDevices) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceSymbols &d = g_sym[dev];
  if (!d.ready) {
    cudaError_t e;
    void *p = nullptr;
    if ((e = cudaGetSymbolAddress(&p, g_na_steps)) != cudaSuccess) goto fail;
    d.steps = (float *)p;
    if ((e = cudaGetSymbolAddress(&p, g_na_ovsteps)) != cudaSuccess) goto fail;
    d.ovsteps = (float *)p;
    if ((e = cudaGetSymbolAddress(&p, g_na_ovlist)) != cudaSuccess) goto fail;
    d.ovlist = (unsigned int *)p;
    if ((e = cudaGetSymbolAddress(&p, g_na_ao)) != cudaSuccess) goto fail;
    d.ao = (float *)p;
    if ((e = cudaGetSymbolAddress(&p, g_na_control)) != cudaSuccess) goto fail;
    d.control = (unsigned long long *)p;
    if ((e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) goto fail;
    d.ready = true;
    *out = &d;
    return MBGB_OK;
  fail:
    return mbgb::set_error(MBGB_ERR_CUDA, std::string("static scratch set-up: ") + cudaGetErrorString(e));
  }
  *out = &d;
  return MBGB_OK;
}

}  // namespace

extern "C" mbgb_status mbgb_render_device_noalloc(const mbgb_scene *scene, const mbgb_image *img,
                                                  const mbgb_opts *opts_in) {
  if (!scene || !img) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "NULL argument");
  mbgb_status st = mbgb_scene_supported(scene);
  if (st != MBGB_OK) return st;
  if (img->width != scene->image_width || img->height != scene->image_height)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "image size does not match the scene");
  if ((long long)img->width * img->height > kNaMaxPixels)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM,
                           "image larger than the allocation-free scratch allows (4194304 pixels, e.g. 2048 x 2048)");
  mbgb_opts o{};
  if (opts_in) o = *opts_in;
  else o.precision = MBGB_PREC_FP32_FIX;   // NULL options: the one policy this entry point renders
  // MBGB_PREC_AUTO is refused, not mapped to FP32_FIX: for a deep zoom AUTO picks FP64 in
  // every other entry point, and this one carries no FP64 pipeline to honour that pick.
  if (o.precision != MBGB_PREC_FP32_FIX)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM,
                           "the allocation-free entry point renders the FP32_FIX policy only (MBGB_PREC_AUTO "
                           "may pick FP64, which it does not carry)");
  if (!scene->analitycDE)
    return mbgb::set_error(MBGB_ERR_UNSUPPORTED,
                           "delta-DE formulas render in FP64, which the allocation-free entry point does not carry");
  bool auxLights = scene->auxLightNumber > 0;
  for (int i = 0; i < 4; i++) auxLights = auxLights || scene->auxLightPreEnabled[i];
  if (auxLights)
    return mbgb::set_error(MBGB_ERR_UNSUPPORTED,
                           "auxiliary lights are placed per call, which the allocation-free entry point does not do");
  if (scene->raytracedReflections && scene->reflectionsMax > 0)
    return mbgb::set_error(MBGB_ERR_UNSUPPORTED,
                           "ray-traced reflections keep per-ray records the allocation-free entry point does not have");
  if (scene->iterFogEnabled || scene->volumetricLightEnabledAny || scene->fakeLightsEnabled)
    return mbgb::set_error(MBGB_ERR_UNSUPPORTED,
                           "iteration fog, volumetric and fake lights need step positions the allocation-free "
                           "entry point does not keep");
  if (o.row_end == 0) o.row_end = scene->image_height;
  if (o.row_begin < 0 || o.row_end > scene->image_height || o.row_begin >= o.row_end)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "row range out of bounds");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return mbgb::set_error(MBGB_ERR_NO_DEVICE, cudaGetErrorString(e));
  DeviceSymbols *d = nullptr;
  st = setup_device(dev, &d);
  if (st != MBGB_OK) return st;
  cudaStream_t s = (cudaStream_t)o.stream;

  // AO direction table (src/Render3D.cpp:272-313) in the static array: uploaded only when the
  // scene's AO quality differs from the table the array already holds, so a frame loop at one
  // quality copies it once. The copy reads pageable host memory, which the runtime stages
  // before cudaMemcpyAsync returns, so the host array is free again without a stream sync.
  int aoCount = 0;
  {
    std::lock_guard<std::mutex> lk(g_ao_mu);
    if (d->aoQuality != scene->globalIlumQuality) {
      const int n = mbgb::ao_vectors_into(scene->globalIlumQuality, g_ao_host, kMaxAOVectors);
      e = cudaMemcpyAsync(d->ao, g_ao_host, sizeof(float) * 3 * (size_t)(n > 0 ? n : 1), cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) {
        d->aoQuality = -1;
        return mbgb::set_error(MBGB_ERR_CUDA, std::string("AO table copy: ") + cudaGetErrorString(e));
      }
      d->aoQuality = scene->globalIlumQuality;
      d->aoCount = n;
    }
    aoCount = d->aoCount;
  }

  // counters, tile counter, overflow count and flags must start at zero on every call
  e = cudaMemsetAsync(d->control, 0, sizeof(g_na_control), s);
  if (e != cudaSuccess) return mbgb::set_error(MBGB_ERR_CUDA, std::string("scratch clear: ") + cudaGetErrorString(e));

  mbgb::ParamsT<float> p;
  mbgb::FractalT<double> fd;
  mbgb::prepare_frame_f32(*scene, o, d->ao, aoCount, &p, &fd);

  // CTAs per SM (opts->ctas_per_sm, default 2): more resident warps, each slot then keeping
  // fewer step records (the arrays' records divided among the slots); rays longer than that
  // take the overflow pass. 1080p Mandelbox, GB300: 156 / 84 / 80 / 301 ms at 1 / 2 / 3 / 4
  // CTAs per SM (256 / 134 / 89 / 67 records per slot); 2 keeps headroom for longer rays.
  const int perSm = o.ctas_per_sm > 0 ? o.ctas_per_sm : kNaDefaultCtasPerSm;
  const long long gridL = (long long)d->sms * perSm;
  const long long slotsL = gridL * kNaThreads;
  if (kNaRecords / slotsL < kNaMinStepCap)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "ctas_per_sm leaves fewer than 32 step records per thread slot");
  const int grid = perSm == 1 && d->sms > kNaMaxCtas ? kNaMaxCtas : (int)gridL;
  const int stepCap = (int)(kNaRecords / ((long long)grid * kNaThreads));
  mbgb::FrameIO io{};
  io.image_float = img->image_float;
  io.zbuffer = img->zbuffer;
  io.alpha = img->alpha;
  io.opacity = img->opacity;
  io.colour = img->colour;
  io.hit = img->hit;
  io.iters = img->iters;
  io.depth = img->depth;
  io.step_step = d->steps + 0 * (size_t)kNaRecords;
  io.step_dist = d->steps + 1 * (size_t)kNaRecords;
  io.step_thr = d->steps + 2 * (size_t)kNaRecords;
  io.slots = (int64_t)grid * kNaThreads;
  io.step_cap = stepCap;
  io.overflow_pass = 0;
  char *ctl = (char *)d->control;
  io.tile_counter = (unsigned int *)(ctl + 0);
  io.overflow_count = (unsigned int *)(ctl + 4);
  io.error_flag = (int *)(ctl + 16);
  io.start_ns = (unsigned long long *)(ctl + 32);
  io.counters = (unsigned long long *)(ctl + 64);
  io.budget_ns = o.deadline_ms > 0 ? (unsigned long long)o.deadline_ms * 1000000ull : 0ull;
  io.overflow_list = d->ovlist;

  mbgb::FrameIO ov = io;
  ov.overflow_pass = 1;
  ov.step_cap = kStepSlots;
  ov.slots = kOverflowThreads;
  ov.step_step = d->ovsteps + 0 * (size_t)kStepSlots * kOverflowThreads;
  ov.step_dist = d->ovsteps + 1 * (size_t)kStepSlots * kOverflowThreads;
  ov.step_thr = d->ovsteps + 2 * (size_t)kStepSlots * kOverflowThreads;

  const bool needVol = (scene->glow_intensity != 0.0) || scene->fogEnabled || (scene->fogDensity > 0.0);
  const bool primitives = scene->planeEnable || scene->boxEnable || scene->invertedBoxEnable || scene->sphereEnable ||
                          scene->invertedSphereEnable || scene->waterEnable || scene->onlyPlane;
  const int kf = mbgb::kernel_formula(scene->formula, scene->ifsFoldingMode || primitives);
  e = mbgb::launch_render_f32(kf, p, fd, io, grid, kNaThreads, s);
  if (e == cudaSuccess && needVol) e = mbgb::launch_render_f32(kf, p, fd, ov, 1, kOverflowThreads, s);
  if (e != cudaSuccess) return mbgb::set_error(MBGB_ERR_CUDA, std::string("render launch: ") + cudaGetErrorString(e));
  if (!o.stream) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return mbgb::set_error(MBGB_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
    int flag = 0;
    e = cudaMemcpy(&flag, ctl + 16, sizeof(flag), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return mbgb::set_error(MBGB_ERR_CUDA, cudaGetErrorString(e));
    if (flag) return mbgb::set_error(MBGB_ERR_TIMEOUT, "render stopped at its device deadline");
  }
  return MBGB_OK;
}
