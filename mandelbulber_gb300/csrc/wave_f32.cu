// Instantiation of the wavefront kernels for T = float, formulas 2 and 8 (the other
// formulas are in wave_more_f32.cu).
#include "wave_stages.cuh"

namespace mbgb {

cudaError_t launch_wave_f32(const WaveLaunch<float> &L, cudaStream_t s) {
  const int kf = kernel_formula(L.p.f.formula, L.p.f.ifsFolding || fractal_has_primitives(L.p.f));
  if (kf == 2) return L.fast ? run_stages<float, 2, true>(L, s) : run_stages<float, 2, false>(L, s);
  if (kf == 8) return L.fast ? run_stages<float, 8, true>(L, s) : run_stages<float, 8, false>(L, s);
  return launch_wave_f32_runtime(L, s);
}

int occupancy_wave_f32(int formula, int block, int which) {
  if (formula == 2) return stage_occupancy<float, 2, true>(block, which);
  if (formula == 8) return stage_occupancy<float, 8, true>(block, which);
  return occupancy_wave_f32_runtime(block, which);
}

}  // namespace mbgb
