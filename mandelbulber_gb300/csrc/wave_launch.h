// Launch description of the wavefront stages (wave_core.cuh) for a batch of frames
// sharing one scene's fractal, shading and fog parameters.
#pragma once

#include <cuda_runtime.h>

#include "kernel_params.h"

namespace mbgb {

// SoA buffers of the wavefront stages over all pixels of a batch (device memory).
template <typename T>
struct WaveBufs {
  uint8_t *flags;        // [npix] bit0: hit, bit1: hemisphere cut / not marched
  T *scan;               // [npix] depth of the primary ray
  T *dist;               // [npix] last distance (lastDist)
  T *thr;                // [npix] distThresh at the hit
  T *step;               // [npix] FP32 policy: bisection step left for the FP64 polish
  T *detail;             // [npix] detailSize of the march's last step (src/Render3D.cpp:110)
  int32_t *bis_left;     // [npix] FP32 policy: bisection iterations left
  T *point;              // [3][npix] hit point in the march precision
  int32_t *iters;        // [npix] itersOut at the end of the march
  int32_t *count;        // [npix] buffCount
  T *vol;                // [6][npix] overflow pass only: A, B.r, B.g, B.b, alpha, opacity
  T *shadow;             // [npix]
  T *ao;                 // [aoCount][npix] per-direction shadowTemp
  T *normal;             // [3][npix] hit normals (auxiliary lights: null without them)
  T *auxsh;              // [numberOfLights][npix] AuxShadow of each auxiliary light at each hit
                         // (null without aux lights or shadows)
  uint32_t *hit_list;    // [npix] hits (secondary rays)
  uint32_t *polish_list; // [npix] hits the FP64 polish re-evaluates
  uint32_t *ctl;         // [0] primary jobs, [1] hits, [2] secondary jobs, [3] overflow count,
                         // [4] overflow-pass jobs, [5] pool chunks, [6] polish count,
                         // [7] exact_hit refinements that missed the level set, [8] hits before
                         // the current ray depth, [9] rays of the next depth, [10] rays of the
                         // current depth, [11] volumetric-light samples (zeroed per group)
  uint32_t *overflow_list;
  // Step records of the primary rays: chunks of kChunk records linked backwards
  // (prev), allocated by bump counter; the pixel keeps its last chunk.
  T *pool_rec;                           // [chunk * kChunk + r][4]: dist, thr, step, scan
                                         // (effects variant: one 16- or 32-byte record), or
                                         // [chunk * kChunk + r][2]: dist, thr (plain variant)
  int32_t *pool_prev;                    // [chunk]
  int32_t *last_chunk;                   // [npix], -1 = no records
  uint32_t pool_cap;                     // chunks
  int polish_all;                        // 1: every hit takes the FP64 polish
  int refill_min;                        // idle lanes of a warp before it claims new rays
  int orbit_refill;                      // lean FP32 orbits, shadow/AO stage: ended orbits of a warp
                                         // before those lanes step on; 0 = refill per distance estimate
  int exact_hit;                         // 1: hits are refined in FP64 to the level set DE = thr
  int pair_rays;                         // lean FP32 Mandelbox, shadow/AO stage: 1 = two rays per
                                         // thread with packed f32x2 orbits (secondary_pair_kernel)
  int64_t npix;                          // rays of the batch: rays x npix_frame (the stride of every
                                         // [k][npix] array above)
  // Ray-traced reflections (the reflection loop of src/Render3D.cpp:441-564): the ray of depth
  // d of pixel gp sits at index d * npix_frame + gp of every per-ray array above. reflect_kernel
  // writes the origin, direction and initial threshold of each depth's next rays.
  int64_t npix_frame;                    // pixels of the batch
  int rays;                              // 1 + reflectionsMax with reflections, else 1
  int depth;                             // ray depth of this launch (primary, polish, reflect)
  double *ray_start;                     // [3][npix] origin of a reflected ray
  double *ray_dir;                       // [3][npix] its direction
  double *ray_thr0;                      // [npix] the previous ray's distThresh, which the reflected
                                         // ray's thresholds add (src/Render3D.cpp:88, 461-462)
  uint32_t *ray_list;                    // [npix_frame] pixels whose next ray is marched
  // Volumetric lights and iteration fog (VolumetricShader, src/shaders.cpp:309-343, 385-466):
  // the step groups that the volumetric walk lights, far to near, each ray's contiguous; the
  // shadow stage traces MainShadow, the predefined lights' AuxShadow and (iteration fog) the
  // AO directions from each, the composition reads them.
  uint32_t *sample_base;                 // [npix] first sample of each ray
  uint32_t *sample_ray;                  // [sample_cap] ray of the sample
  int32_t *sample_rec;                   // [sample_cap] pool record of the group's position
  T *sample_step;                        // [sample_cap] the group's summed step
  T *sample_res;                         // [sample_nres][sample_cap] MainShadow, AuxShadow of the
                                         // predefined lights 0-3, then (iteration fog with ray AO)
                                         // each AO direction's shadowTemp
  uint32_t sample_cap;                   // samples (every group has a record: the pool's records)
  int sample_nres;                       // results per sample
  int32_t *pool_iters;                   // [chunk * kChunk + r] itersOut at each record (iteration
                                         // fog; null without)
  uint32_t *seg_count;                   // [segments][kHitSegWarps] hits per warp of each segment
                                         // of kHitSeg primary jobs (hit list in tile order; null =
                                         // kept in completion order)
  T *hit_setup;                          // [k][8] the shadow/AO set-up of hit-list entry k (plain
                                         // variant): point, thr, delta, AO end, shadow end and
                                         // start (hit_setup_kernel); null with one ray per pixel
                                         // not given
};

constexpr int kHitSegWarps = 4;          // warps per segment of the hit-list compaction
constexpr int kHitSeg = kHitSegWarps * 32 * 32;   // primary jobs per segment: 32 per lane

constexpr int kSampleShadows = 5;        // MainShadow and the four predefined lights' AuxShadow

// Stage events of one launch sequence (see WaveLaunch::ev) and the stats slot of each
// stage: primary 0, polish 1, shadow/AO 2, compose 3, level set 4, gradient 5.
constexpr int kStageEvents = 7;
constexpr int kStages = 6;

constexpr int kChunk = 32;       // step records per pool chunk
constexpr int kPoolChunksPerPixel = 4;   // pool budget; rays beyond it take the overflow pass
constexpr int kPoolChunksPerReflectedRay = 6;   // the same with reflections, per ray of the loop
constexpr int kWaveOverflowThreads = 2048;      // threads of the wavefront's overflow pass

// Parameters of the differentiable render: [0] fractal parameter (power of formula 2,
// scale of formula 8), [1..3] camera position, [4] main light alpha, [5] main light beta.
constexpr int kGradParams = 6;

// Per-frame inputs and outputs of the gradient stage (device table, one per frame).
template <typename T>
struct GradCam {
  const float *dL_dimage;   // [height][width][3] or null: the loss's derivative by the float image
  float *jacobian;          // [height][width][3][kGradParams] or null: dI/dtheta per pixel and channel
  double *dtheta;           // [kGradParams]: sum over pixels of dL/dI dI/dtheta (zeroed by the host)
  T dLight[2][3];           // d lightVect / d alpha, d lightVect / d beta (camera rotation applied)
};

template <typename T>
struct WaveLaunch {
  ParamsT<T> p;
  FractalT<double> fd;
  FrameIO io;        // main primary pass
  FrameIO ov;        // overflow primary pass (rays longer than io.step_cap records)
  WaveBufs<T> wb;
  const FrameCam<T> *cams;  // device table of the batch's frames (camera, size, rows, outputs)
  const GradCam<T> *gcams;  // differentiable render: per-frame gradient table (null = no gradient stage)
  int ncams;
  int grid, block, ov_grid, polish_grid, grid2, compose_grid;
  bool overflow;     // the step buffer is in use, so the overflow pass is enqueued
  bool fast;         // the scene qualifies for a lean FP32 orbit (Mandelbox, power-8 Mandelbulb)
  // optional stage events, in launch order: before the primary rays, after them, after the
  // polish, after the level-set refinement, after the shadow/AO rays, after composition,
  // after the gradient stage
  cudaEvent_t ev[kStageEvents];
  int grad_grid;     // blocks of the gradient stage
  int64_t hit_jobs;  // primary jobs of the batch (the hit list's compaction walks them)
};

// Stage k adds its counters at io.counters + 4 * k.
inline FrameIO stage_io(const FrameIO &io, int k) {
  FrameIO r = io;
  r.counters = io.counters + 4 * k;
  return r;
}

cudaError_t launch_wave_f64(const WaveLaunch<double> &L, cudaStream_t s);
cudaError_t launch_wave_f32(const WaveLaunch<float> &L, cudaStream_t s);
int occupancy_wave_f64(int formula, int block, int which);
int occupancy_wave_f32(int formula, int block, int which);
// the formulas compute() selects at run time (runtime_formula)
cudaError_t launch_wave_f64_runtime(const WaveLaunch<double> &L, cudaStream_t s);
cudaError_t launch_wave_f32_runtime(const WaveLaunch<float> &L, cudaStream_t s);
int occupancy_wave_f64_runtime(int block, int which);
int occupancy_wave_f32_runtime(int block, int which);

}  // namespace mbgb
