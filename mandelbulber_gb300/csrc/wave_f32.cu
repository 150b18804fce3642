// Instantiation of the wavefront kernels for T = float.
#include "grad_core.cuh"
#include "wave_core.cuh"
#include "wave_launch.h"

namespace mbgb {

template <int F, bool FAST>
static cudaError_t run_stages_f32(const WaveLaunch<float> &L, cudaStream_t s) {
  auto mark = [&](int k) {
    if (L.ev[0]) cudaEventRecord(L.ev[k], s);
  };
  mark(0);
  dev::primary_kernel<float, F, FAST><<<L.grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.io, 0), L.wb, L.cams, L.ncams);
  if (L.overflow)
    dev::primary_kernel<float, F, FAST><<<L.ov_grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.ov, 0), L.wb, L.cams, L.ncams);
  mark(1);
  dev::polish_kernel<F, FAST><<<L.polish_grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.io, 1), L.wb, L.cams, L.ncams);
  mark(2);
  if (L.wb.exact_hit)
    dev::level_set_kernel<float, F><<<L.polish_grid, L.block, 0, s>>>(L.p, L.fd, L.wb, L.cams, L.ncams);
  mark(3);
  dev::secondary_kernel<float, F, FAST><<<L.grid2, L.block, 0, s>>>(L.p, stage_io(L.io, 2), L.wb, L.cams, L.ncams);
  mark(4);
  dev::compose_kernel<float, F, FAST><<<L.compose_grid, L.block, 0, s>>>(L.p, stage_io(L.io, 3), L.wb, L.cams, L.ncams);
  mark(5);
  if (L.gcams)
    dev::grad_kernel<float, F, FAST><<<L.grad_grid, L.block, 0, s>>>(L.p, L.fd, stage_io(L.io, 5), L.wb, L.cams, L.gcams,
                                                                  L.ncams);
  mark(6);
  return cudaGetLastError();
}

cudaError_t launch_wave_f32(const WaveLaunch<float> &L, cudaStream_t s) {
  if (L.p.f.formula == 2) return L.fast ? run_stages_f32<2, true>(L, s) : run_stages_f32<2, false>(L, s);
  if (L.p.f.formula == 8) return L.fast ? run_stages_f32<8, true>(L, s) : run_stages_f32<8, false>(L, s);
  return cudaErrorInvalidValue;
}

int occupancy_wave_f32(int formula, int block, int which) {
  int n = 0;
  if (which == 0) {
    if (formula == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::primary_kernel<float, 2, true>, block, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::primary_kernel<float, 8, true>, block, 0);
  } else {
    if (formula == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::secondary_kernel<float, 2, true>, block, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, dev::secondary_kernel<float, 8, true>, block, 0);
  }
  return n;
}

}  // namespace mbgb
