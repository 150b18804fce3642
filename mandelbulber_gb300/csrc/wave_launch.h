// Launch description of the wavefront stages (wave_core.cuh) for one frame.
#pragma once

#include <cuda_runtime.h>

#include "kernel_params.h"

namespace mbgb {

template <typename T>
struct WaveBufs;

template <typename T>
struct WaveLaunch {
  ParamsT<T> p;
  FractalT<double> fd;
  FrameIO io;        // main primary pass
  FrameIO ov;        // overflow primary pass (rays longer than io.step_cap records)
  WaveBufs<T> wb;
  int grid, block, ov_grid, polish_grid, grid2, compose_grid;
  bool overflow;     // the step buffer is in use, so the overflow pass is enqueued
  bool fast;         // the scene qualifies for a lean FP32 orbit (Mandelbox, power-8 Mandelbulb)
  cudaEvent_t ev[5]; // optional: recorded before stage 0 and after each of the 4 stages
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

}  // namespace mbgb
