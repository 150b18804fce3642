// Instantiation of the per-pixel kernels for T = double and the formulas chosen at run time
// (FORMULA 0 of compute()), in a translation unit of its own.
#include "launch.h"
#include "render_core.cuh"

namespace mbgb {

cudaError_t launch_render_f64_runtime(const ParamsT<double> &p, const FractalT<double> &fd, const FrameIO &io, int grid,
                                      int block, cudaStream_t s) {
  dev::render_kernel<double, 0><<<grid, block, 0, s>>>(p, fd, io);
  return cudaGetLastError();
}

cudaError_t launch_distance_f64_runtime(const FractalT<double> &f, const double *points, const double *detail, long long n,
                                        double *dist, int *iters, unsigned char *max_iter,
                                        unsigned long long *counters, cudaStream_t s) {
  const int block = 128;
  long long want = (n + block - 1) / block;
  const int grid = (int)(want < 4096 ? (want < 1 ? 1 : want) : 4096);
  dev::distance_kernel<double, 0><<<grid, block, 0, s>>>(f, points, detail, n, dist, iters, max_iter, counters);
  return cudaGetLastError();
}

int occupancy_render_f64_runtime(int block) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::render_kernel<double, 0>, block, 0);
  return n;
}

}  // namespace mbgb
