// Keyframe interpolation of scenes: CMorph::CatmullRom (src/morph.cpp:49-109) applied to
// every interpolated double of the parameter blocks, as MainRender does in keyframe mode
// (src/Render3D.cpp:2280-2291): sParamRenderD, sFractalD, sFractalMandelboxD and
// sFractalIFSD. In mbgb_scene those doubles are the two contiguous runs
// [zoom, mboxMainRot) and [ifsRotationGamma, image_width); the rotation matrices in
// between are derived and are rebuilt by mbgb_scene_finalize.
#include <cmath>
#include <cstddef>
#include <cstring>

#include "mbgb.h"
#include "mbgb_internal.h"

namespace {

// One Catmull-Rom sample of value i, with the reference's logarithmic mode for four
// same-signed control values that vary by more than 10 % of their average.
double catmull_rom(const double *keys, int n_keys, int stride, int i, int frames_per_key, int frame) {
  const int key = frame / frames_per_key;
  const double factor = (frame % frames_per_key) / (double)frames_per_key;
  const double factor2 = factor * factor;
  const double factor3 = factor2 * factor;
  auto at = [&](int k) { return keys[(size_t)k * stride + i]; };
  double v1 = key >= 1 ? at(key - 1) : at(key);
  double v2 = key < n_keys ? at(key) : at(n_keys - 1);
  double v3 = key < n_keys - 1 ? at(key + 1) : at(n_keys - 1);
  double v4 = key < n_keys - 2 ? at(key + 2) : at(n_keys - 1);
  bool logaritmic = false, negative = false;
  if ((v1 > 0 && v2 > 0 && v3 > 0 && v4 > 0) || (v1 < 0 && v2 < 0 && v3 < 0 && v4 < 0)) {
    if (v1 < 0) negative = true;
    const double average = (v1 + v2 + v3 + v4) / 4.0;
    if (average > 0) {
      const double deviation = (fabs(v2 - v1) + fabs(v3 - v2) + fabs(v4 - v3)) / average;
      if (deviation > 0.1) {
        v1 = log(fabs(v1));
        v2 = log(fabs(v2));
        v3 = log(fabs(v3));
        v4 = log(fabs(v4));
        logaritmic = true;
      }
    }
  }
  double value = 0.5 * ((2 * v2) + (-v1 + v3) * factor + (2 * v1 - 5 * v2 + 4 * v3 - v4) * factor2 +
                        (-v1 + 3 * v2 - 3 * v3 + v4) * factor3);
  if (logaritmic) value = negative ? -exp(value) : exp(value);
  if (value > 1e20) value = 1e20;
  if (value < -1e20) value = 1e20;  // the reference clamps large negatives to +1e20
  if (fabs(value) < 1e-20) value = 0.0;
  return value;
}

void interpolate_run(const mbgb_scene *keys, int n_keys, int fpk, int frame, size_t begin, size_t end,
                     mbgb_scene *out) {
  const int stride = (int)(sizeof(mbgb_scene) / sizeof(double));
  const double *k0 = reinterpret_cast<const double *>(keys);
  double *o = reinterpret_cast<double *>(out);
  for (size_t i = begin / sizeof(double); i < end / sizeof(double); i++)
    o[i] = catmull_rom(k0, n_keys, stride, (int)i, fpk, frame);
}

}  // namespace

static_assert(sizeof(mbgb_scene) % sizeof(double) == 0, "mbgb_scene must be a whole number of doubles");
static_assert(offsetof(mbgb_scene, zoom) % sizeof(double) == 0 && offsetof(mbgb_scene, ifsRotationGamma) % 8 == 0,
              "double runs must be aligned");

extern "C" mbgb_status mbgb_catmull_rom(const double *keys, int n_keys, int size, int frames_per_key, int frame,
                                        double *out) {
  if (!keys || !out || n_keys < 1 || size < 1 || frames_per_key < 1 || frame < 0)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_catmull_rom: bad argument");
  if (frame / frames_per_key >= n_keys) return mbgb::set_error(MBGB_ERR_BAD_PARAM, "frame beyond the last keyframe");
  for (int i = 0; i < size; i++) out[i] = catmull_rom(keys, n_keys, size, i, frames_per_key, frame);
  return MBGB_OK;
}

extern "C" mbgb_status mbgb_scene_interpolate(const mbgb_scene *keys, int n_keys, int frames_per_key, int frame,
                                              const mbgb_scene *base, mbgb_scene *out) {
  if (!keys || !out || n_keys < 1 || frames_per_key < 1 || frame < 0)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_scene_interpolate: bad argument");
  if (frame / frames_per_key >= n_keys)
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "frame beyond the last keyframe");
  mbgb_scene r = base ? *base : keys[0];
  interpolate_run(keys, n_keys, frames_per_key, frame, offsetof(mbgb_scene, zoom), offsetof(mbgb_scene, mboxMainRot),
                  &r);
  interpolate_run(keys, n_keys, frames_per_key, frame, offsetof(mbgb_scene, ifsRotationGamma),
                  offsetof(mbgb_scene, image_width), &r);
  // MainRender after the splines (src/Render3D.cpp:2287-2290), then the derived fields
  if (r.zoom < 1e-15) r.zoom = 1e-15;
  const mbgb_status st = mbgb_scene_finalize(&r);
  if (st != MBGB_OK) return st;
  *out = r;
  return MBGB_OK;
}
