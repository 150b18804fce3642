// Internal declarations shared by the host-side translation units of libmbgb.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "mbgb.h"

namespace mbgb {

// Records `msg` as this thread's last error and returns `st` (see mbgb_last_error).
mbgb_status set_error(mbgb_status st, const std::string &msg);

// The C library's srand()/rand() sequence (glibc additive feedback generator),
// restated so palettes generated from coloring_random_seed are identical on every host.
class GlibcRand {
 public:
  explicit GlibcRand(uint32_t seed);
  int rand();
  int random(int max);

 private:
  uint32_t next_raw();
  uint32_t ring_[34];
  uint64_t idx_;
};

bool scene_set(mbgb_scene *sc, const char *key, const char *value, bool *palette_loaded);

template <typename T>
struct ParamsT;
template <typename T>
struct FractalT;
mbgb_status prepare_frame_f32(const mbgb_scene &scene, const mbgb_opts &o, const float *aoVec, int aoCount,
                              ParamsT<float> *p, FractalT<double> *fd);
int ao_vectors_into(int quality, float *out, int max_vectors);

// Post-processing on the device (post.cu): CompileImage into RGB16 and the SSAO pass.
mbgb_status compile16_device(const mbgb_scene &scene, const float *image_float, int width, int height,
                             uint16_t *image16, int *gamma_dev, cudaStream_t s);
mbgb_status ssao_device(const mbgb_scene &scene, const mbgb_image &layers, uint16_t *image16, void *tables,
                        cudaStream_t s);
mbgb_status dof_device(const mbgb_scene &scene, const mbgb_image &layers, uint16_t *image16, uint32_t seed,
                       cudaStream_t s);

}  // namespace mbgb
