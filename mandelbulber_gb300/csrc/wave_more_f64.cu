// Instantiation of the wavefront kernels for T = double and the formulas chosen at run time
// (FORMULA 0 of compute(): trig_DE, menger_sponge, mandelboxVaryScale4D), in a translation
// unit of its own so that it compiles beside the others.
#include "wave_stages.cuh"

namespace mbgb {

cudaError_t launch_wave_f64_runtime(const WaveLaunch<double> &L, cudaStream_t s) { return run_stages<double, 0, false>(L, s); }

int occupancy_wave_f64_runtime(int block, int which) { return stage_occupancy<double, 0, false>(block, which); }

}  // namespace mbgb
