// Launchers of the device kernels, one translation unit per precision policy.
#pragma once

#include <cuda_runtime.h>

#include "kernel_params.h"

namespace mbgb {

cudaError_t launch_render_f64(int formula, const ParamsT<double> &p, const FractalT<double> &fd, const FrameIO &io,
                              int grid, int block, cudaStream_t s);
cudaError_t launch_render_f32(int formula, const ParamsT<float> &p, const FractalT<double> &fd, const FrameIO &io,
                              int grid, int block, cudaStream_t s);
cudaError_t launch_distance_f64(int formula, const FractalT<double> &f, const double *points, const double *detail,
                                long long n, double *dist, int *iters, unsigned char *max_iter,
                                unsigned long long *counters, cudaStream_t s);
cudaError_t launch_distance_f32(int formula, const FractalT<float> &f, const double *points, const double *detail,
                                long long n, double *dist, int *iters, unsigned char *max_iter,
                                unsigned long long *counters, cudaStream_t s);
// resident CTAs per SM of the render kernel for `block` threads
int occupancy_render(int precision, int formula, int block);

}  // namespace mbgb
