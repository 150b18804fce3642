// Instantiation of the ray-march kernels for T = double.
#include "launch.h"
#include "render_core.cuh"

namespace mbgb {

cudaError_t launch_render_f64(int formula, const ParamsT<double> &p, const FractalT<double> &fd, const FrameIO &io,
                              int grid, int block, cudaStream_t s) {
  switch (formula) {
    case 2: dev::render_kernel<double, 2><<<grid, block, 0, s>>>(p, fd, io); break;
    case 8: dev::render_kernel<double, 8><<<grid, block, 0, s>>>(p, fd, io); break;
    default:
      return launch_render_f64_runtime(p, fd, io, grid, block, s);
  }
  return cudaGetLastError();
}

cudaError_t launch_distance_f64(int formula, const FractalT<double> &f, const double *points, const double *detail,
                                long long n, double *dist, int *iters, unsigned char *max_iter,
                                unsigned long long *counters, cudaStream_t s) {
  const int block = 128;
  long long want = (n + block - 1) / block;
  const int grid = (int)(want < 4096 ? (want < 1 ? 1 : want) : 4096);
  switch (formula) {
    case 2: dev::distance_kernel<double, 2><<<grid, block, 0, s>>>(f, points, detail, n, dist, iters, max_iter, counters); break;
    case 8: dev::distance_kernel<double, 8><<<grid, block, 0, s>>>(f, points, detail, n, dist, iters, max_iter, counters); break;
    default:
      return launch_distance_f64_runtime(f, points, detail, n, dist, iters, max_iter, counters, s);
  }
  return cudaGetLastError();
}

int occupancy_render_f64(int formula, int block) {
  int n = 0;
  if (formula == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::render_kernel<double, 2>, block, 0);
  else if (formula == 8) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::render_kernel<double, 8>, block, 0);
  else n = occupancy_render_f64_runtime(block);
  return n;
}

}  // namespace mbgb
