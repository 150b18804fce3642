// Instantiation of the wavefront kernels for T = double, formulas 2 and 8 (the other
// formulas are in wave_more_f64.cu).
#include "wave_stages.cuh"

namespace mbgb {

cudaError_t launch_wave_f64(const WaveLaunch<double> &L, cudaStream_t s) {
  const int kf = kernel_formula(L.p.f.formula, L.p.f.ifsFolding || fractal_has_primitives(L.p.f));
  if (kf == 2) return L.fast ? run_stages<double, 2, false>(L, s) : run_stages<double, 2, false>(L, s);
  if (kf == 8) return L.fast ? run_stages<double, 8, false>(L, s) : run_stages<double, 8, false>(L, s);
  return launch_wave_f64_runtime(L, s);
}

int occupancy_wave_f64(int formula, int block, int which) {
  if (formula == 2) return stage_occupancy<double, 2, false>(block, which);
  if (formula == 8) return stage_occupancy<double, 8, false>(block, which);
  return occupancy_wave_f64_runtime(block, which);
}

}  // namespace mbgb
