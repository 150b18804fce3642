// The launch sequence of the wavefront stages (wave_core.cuh, grad_core.cuh) for one
// launch group, shared by the translation units that instantiate it per formula.
#pragma once

#include "grad_core.cuh"
#include "wave_core.cuh"
#include "wave_launch.h"

namespace mbgb {

template <typename T, int F, bool FAST>
cudaError_t run_stages(const WaveLaunch<T> &L, cudaStream_t s) {
  auto mark = [&](int k) {
    if (L.ev[0]) cudaEventRecord(L.ev[k], s);
  };
  // the effects variant of the primary, shadow and composition stages: reflected rays,
  // auxiliary, volumetric or fake lights, iteration fog
  const bool efx = L.wb.rays > 1 || L.p.numberOfLights > 0 || L.p.volLightAny || L.p.iterFog || L.p.fakeLights;
  mark(0);
  // one primary pass (and FP64 polish) per ray depth of the reflection loop; between two
  // depths the reflect stage spawns the next depth's rays from this depth's hits
  for (int d = 0; d < L.wb.rays; d++) {
    WaveBufs<T> wbd = L.wb;
    wbd.depth = d;
    if (d > 0) {
      WaveBufs<T> wbp = L.wb;
      wbp.depth = d - 1;
      dev::reflect_kernel<T, F, FAST><<<L.polish_grid, L.block, 0, s>>>(L.p, stage_io(L.io, 0), wbp, L.cams, L.ncams);
      dev::next_depth_kernel<T><<<1, 1, 0, s>>>(L.wb.ctl);
    }
    if (efx) {
      dev::primary_kernel<T, F, FAST, true><<<L.grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.io, 0), wbd, L.cams,
                                                                        L.ncams);
      if (L.overflow)
        dev::primary_kernel<T, F, FAST, true, true><<<L.ov_grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.ov, 0), wbd,
                                                                                   L.cams, L.ncams);
    } else {
      dev::primary_kernel<T, F, FAST><<<L.grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.io, 0), wbd, L.cams, L.ncams);
      if (L.overflow)
        dev::primary_kernel<T, F, FAST><<<L.ov_grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.ov, 0), wbd, L.cams,
                                                                       L.ncams);
    }
    // with reflections the primary stage's time holds every depth's march, polish and reflection
    if (L.wb.rays == 1) mark(1);
    if constexpr (sizeof(T) == 4)
      dev::polish_kernel<F, FAST><<<L.polish_grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.io, 1), wbd, L.cams, L.ncams);
  }
  if (L.wb.rays > 1) mark(1);
  // the hit list in tile order (one ray per pixel): a tile's shadow and AO rays share a warp
  if (L.wb.seg_count) {
    const int segs = (int)((L.hit_jobs + kHitSeg - 1) / kHitSeg);
    dev::hit_count_kernel<T><<<segs, kHitSegWarps * 32, 0, s>>>(L.wb, L.cams, L.ncams);
    dev::hit_scan_kernel<T><<<1, 1024, 0, s>>>(L.wb.seg_count, (int64_t)segs * kHitSegWarps);
    dev::hit_scatter_kernel<T><<<segs, kHitSegWarps * 32, 0, s>>>(L.wb, L.cams, L.ncams);
  }
  mark(2);
  if (L.wb.exact_hit)
    dev::level_set_kernel<T, F><<<L.polish_grid, L.block, 0, s>>>(L.p, L.fd, L.wb, L.cams, L.ncams);
  mark(3);
  // volumetric lights: the volumetric walk's step groups, whose shadows the shadow stage traces
  if (L.wb.sample_ray)
    dev::sample_kernel<T><<<L.compose_grid, L.block, 0, s>>>(L.p, L.wb, L.cams, L.ncams);
  // auxiliary lights: the hit normals, which the AuxShadow jobs test (counted with composition)
  if (L.wb.normal)
    dev::normal_kernel<T, F, FAST><<<L.polish_grid, L.block, 0, s>>>(L.p, stage_io(L.io, 3), L.wb, L.cams, L.ncams);
  // the plain variant's per-hit set-up of the shadow and AO jobs
  if (L.wb.hit_setup && !efx)
    dev::hit_setup_kernel<T><<<L.polish_grid, L.block, 0, s>>>(L.p, L.wb, L.cams, L.ncams);
  bool pair = false;
  if constexpr (sizeof(T) == 4 && F == 8 && FAST) pair = L.wb.pair_rays && L.wb.orbit_refill <= 0 && !efx;
  if constexpr (sizeof(T) == 4 && F == 8 && FAST) {
    if (pair) dev::secondary_pair_kernel<8><<<L.grid2, L.block, 0, s>>>(L.p, stage_io(L.io, 2), L.wb, L.cams, L.ncams);
  }
  if (!pair) {
    if (efx)
      dev::secondary_kernel<T, F, FAST, true><<<L.grid2, L.block, 0, s>>>(L.p, stage_io(L.io, 2), L.wb, L.cams,
                                                                          L.ncams);
    else
      dev::secondary_kernel<T, F, FAST><<<L.grid2, L.block, 0, s>>>(L.p, stage_io(L.io, 2), L.wb, L.cams, L.ncams);
  }
  mark(4);
  // slow shading: one warp's 11^3 normal samples in dynamic shared memory per warp
  const size_t composeSmem = L.p.slowShading ? (size_t)(L.block / 32) * dev::kSlowSamples * sizeof(T) : 0;
  if (efx)
    dev::compose_kernel<T, F, FAST, true><<<L.compose_grid, L.block, composeSmem, s>>>(L.p, stage_io(L.io, 3), L.wb,
                                                                                     L.cams, L.ncams);
  else
    dev::compose_kernel<T, F, FAST><<<L.compose_grid, L.block, composeSmem, s>>>(L.p, stage_io(L.io, 3), L.wb, L.cams,
                                                                               L.ncams);
  mark(5);
  if (L.gcams)
    dev::grad_kernel<T, F, FAST><<<L.grad_grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.io, 5), L.wb, L.cams, L.gcams,
                                                              L.ncams);
  mark(6);
  return cudaGetLastError();
}

template <typename T, int F, bool FAST>
int stage_occupancy(int block, int which) {
  int n = 0;
  if (which == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::primary_kernel<T, F, FAST>, block, 0);
  } else if (which == 2) {   // the two-rays-per-thread shadow/AO kernel
    if constexpr (sizeof(T) == 4 && F == 8 && FAST)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::secondary_pair_kernel<8>, block, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::secondary_kernel<T, F, FAST>, block, 0);
  }
  return n;
}

}  // namespace mbgb
