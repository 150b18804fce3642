// Instantiation of the wavefront kernels for T = float and the formulas chosen at run time
// (FORMULA 0 of compute(): trig_DE, menger_sponge, mandelboxVaryScale4D), in a translation
// unit of its own so that it compiles beside the others.
#include "wave_stages.cuh"

namespace mbgb {

cudaError_t launch_wave_f32_runtime(const WaveLaunch<float> &L, cudaStream_t s) { return run_stages<float, 0, false>(L, s); }

int occupancy_wave_f32_runtime(int block, int which) { return stage_occupancy<float, 0, false>(block, which); }

}  // namespace mbgb
