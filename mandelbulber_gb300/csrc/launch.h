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

// the formulas compute() selects at run time (runtime_formula), one translation unit each
cudaError_t launch_render_f64_runtime(const ParamsT<double> &p, const FractalT<double> &fd, const FrameIO &io,
                                      int grid, int block, cudaStream_t s);
cudaError_t launch_render_f32_runtime(const ParamsT<float> &p, const FractalT<double> &fd, const FrameIO &io,
                                      int grid, int block, cudaStream_t s);
cudaError_t launch_distance_f64_runtime(const FractalT<double> &f, const double *points, const double *detail,
                                        long long n, double *dist, int *iters, unsigned char *max_iter,
                                        unsigned long long *counters, cudaStream_t s);
cudaError_t launch_distance_f32_runtime(const FractalT<float> &f, const double *points, const double *detail,
                                        long long n, double *dist, int *iters, unsigned char *max_iter,
                                        unsigned long long *counters, cudaStream_t s);
int occupancy_render_f64_runtime(int block);
int occupancy_render_f32_runtime(int block);

}  // namespace mbgb
