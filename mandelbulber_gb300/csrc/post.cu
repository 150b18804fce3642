// Post-processing of a rendered frame on the device: CompileImage (src/cimage.cpp:132-214)
// into the 16-bit image, and the screen-space ambient occlusion pass PostRendering_SSAO /
// ThreadSSAO (src/image.cpp:249-478), which the reference runs after CompileImage when
// post_SSAO_enabled is set (src/Render3D.cpp:1094-1099).
//
// Built with --fmad=false: the FP64 SSAO and the compile step follow the reference's
// double-precision operation order, so results match it to the last bit except where
// CUDA's atan / tanhf round differently from the host's libm.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "mbgb.h"
#include "mbgb_internal.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

// CalculatePixel (src/cimage.cpp:132-171): brightness, contrast, optional tanh, clamp,
// x 65535 and the gamma table.
__global__ void compile16_kernel(const float *__restrict__ image_float, int64_t n, double brightness,
                                 double contrast, int hdr, const int *__restrict__ gamma,
                                 uint16_t *__restrict__ image16) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += (int64_t)gridDim.x * blockDim.x) {
    float v = (float)((double)image_float[i] * brightness);
    v = (float)(((double)v - 0.5) * contrast + 0.5);
    if (v < 0.0f) v = 0.0f;
    if (hdr) v = (float)tanh((double)v);   // the host's tanhf, to the float it rounds to
    if (v > 1.0f) v = 1.0f;
    const unsigned short q = (unsigned short)((double)v * 65535.0);
    image16[i] = (uint16_t)gamma[q];
  }
}

// Screen position of a pixel sample (x, y may be fractional) at depth z in the plane
// the SSAO horizon search works in; perspective types as in ThreadSSAO. For the fish eye
// the centre pixel skips the projection where its radius is 0, while the samples test the
// search radius instead (always >= 1), as ThreadSSAO does.
template <typename T>
__device__ __forceinline__ void ssao_position(const int ptype, const T fx, const T fy, const T w, const T h,
                                              const T aspect, const T fov, const T z, const bool centre, T &ox,
                                              T &oy) {
  if (ptype == 1) {   // fish eye
    const T x2 = T(kPi) * (fx / w - T(0.5)) * aspect;
    const T y2 = T(kPi) * (fy / h - T(0.5));
    const T r = sqrt(x2 * x2 + y2 * y2);
    ox = x2;
    oy = y2;
    if (!centre || r != T(0)) {
      ox = x2 / r * sin(r * fov) * z;
      oy = y2 / r * sin(r * fov) * z;
    }
  } else if (ptype == 2) {   // equirectangular
    const T x2 = T(kPi) * (fx / w - T(0.5)) * aspect;
    const T y2 = T(kPi) * (fy / h - T(0.5));
    ox = sin(fov * x2) * cos(fov * y2) * z;
    oy = sin(fov * y2) * z;
  } else {
    ox = (fx / w - T(0.5)) * aspect;
    oy = (fy / h - T(0.5));
  }
}

// ThreadSSAO (src/image.cpp:249-417) for one pixel per thread: `quality` directions, each
// searching quality - 1 samples at radius r^2 * width / (2 quality^2) for the steepest
// horizon, ambient = mean over directions of 0.5 - atan(slope) / pi; the pixel's 16-bit
// value gains colour * ambient * intensity * (1 - opacity), clamped to 65535.
template <typename T>
__global__ void ssao_kernel(const float *__restrict__ zbuf, const uint16_t *__restrict__ opacity,
                            const uint8_t *__restrict__ colour, uint16_t *__restrict__ image16, const int width,
                            const int height, const T persp, const int quality, const int ptype, const T intensity,
                            const T *__restrict__ cs, const T *__restrict__ sn) {
  const int64_t n = (int64_t)width * height;
  const T w = (T)width, h = (T)height;
  const T scale = (T)width / (T)(quality * quality) / T(2);
  const T aspect = (T)width / (T)height;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % width), y = (int)(i / width);
    const T z = (T)zbuf[i];
    const T op = (T)opacity[i] / T(65535);
    T total = T(0);
    if (z < T(1e19)) {
      T x2, y2;
      ssao_position<T>(ptype, (T)x, (T)y, w, h, aspect, persp, z, true, x2, y2);
      if (ptype != 1 && ptype != 2) {
        x2 = x2 * z * persp;
        y2 = y2 * z * persp;
      }
      T ambient = T(0);
      for (int a = 0; a < quality; a++) {
        const T ca = cs[a], sa = sn[a];
        T maxDiff = T(-1e50);
        for (T r = T(1); r < (T)quality; r += T(1)) {
          const T rr = r * r * scale;
          const T xx = (T)x + rr * ca;
          const T yy = (T)y + rr * sa;
          if ((int)xx == x && (int)yy == y) continue;
          if (xx < T(0) || xx > (T)(width - 1) || yy < T(0) || yy > (T)(height - 1)) continue;
          const T z2 = (T)zbuf[(int64_t)(int)yy * width + (int)xx];
          T xx2, yy2;
          ssao_position<T>(ptype, xx, yy, w, h, aspect, persp, z2, false, xx2, yy2);
          if (ptype != 1 && ptype != 2) {
            xx2 = xx2 * (z2 * persp);
            yy2 = yy2 * (z2 * persp);
          }
          const T dx = xx2 - x2;
          const T dy = yy2 - y2;
          const T dz = z2 - z;
          const T dr = sqrt(dx * dx + dy * dy);
          const T diff = -dz / dr;
          if (diff > maxDiff) maxDiff = diff;
        }
        const T maxAngle = atan(maxDiff);
        ambient += -maxAngle / T(kPi) + T(0.5);
      }
      total = ambient / (T)quality;
      if (total < T(0)) total = T(0);
    }
    for (int c = 0; c < 3; c++) {
      T v = (T)image16[3 * i + c] + T(65535) * (T)colour[3 * i + c] / T(256) * total * intensity * (T(1) - op);
      if (v > T(65535)) v = T(65535);
      image16[3 * i + c] = (uint16_t)(unsigned short)v;
    }
  }
}

int grid_for(int64_t work, int block) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (work + block - 1) / block;
  const int64_t cap = (int64_t)(sms > 0 ? sms : 1) * 16;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

}  // namespace

namespace mbgb {

// CompileImage on the device (gamma table from the host's pow, as CalculateGammaTable).
mbgb_status compile16_device(const mbgb_scene &scene, const float *image_float, int width, int height,
                             uint16_t *image16, int *gamma_dev, cudaStream_t s) {
  std::vector<int> gamma(65536);
  for (int i = 0; i < 65536; i++) gamma[i] = (int)(pow(i / 65536.0, 1.0 / scene.imageGamma) * 65535);
  cudaError_t e = cudaMemcpyAsync(gamma_dev, gamma.data(), sizeof(int) * 65536, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return set_error(MBGB_ERR_CUDA, std::string("gamma table: ") + cudaGetErrorString(e));
  const int64_t n = (int64_t)width * height;
  compile16_kernel<<<grid_for(3 * n, 256), 256, 0, s>>>(image_float, n, scene.brightness, scene.contrast,
                                                        scene.hdrEnabled ? 1 : 0, gamma_dev, image16);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // the host table is released on return
  if (e != cudaSuccess) return set_error(MBGB_ERR_CUDA, std::string("compile kernel: ") + cudaGetErrorString(e));
  return MBGB_OK;
}

// PostRendering_SSAO on the device, in double (the reference's arithmetic): the sample
// positions x + r^2 s cos(a) land on the neighbouring pixel or not depending on the last
// bits of cos(a) near 0 (cos(pi / 2) = 6e-17), which float arithmetic does not keep.
// `tables` receives cos and sin of the `quality` directions.
mbgb_status ssao_device(const mbgb_scene &scene, const mbgb_image &layers, uint16_t *image16, void *tables,
                        cudaStream_t s) {
  const int q = scene.SSAOQuality;
  if (q < 1) return MBGB_OK;   // the loops of ThreadSSAO run no direction: nothing changes
  std::vector<double> t(2 * (size_t)q);
  for (int i = 0; i < q; i++) {
    t[q + i] = sin((double)i / q * 2.0 * kPi);
    t[i] = cos((double)i / q * 2.0 * kPi);
  }
  const int64_t n = (int64_t)layers.width * layers.height;
  const int block = 128;
  cudaError_t e = cudaMemcpyAsync(tables, t.data(), sizeof(double) * 2 * q, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    ssao_kernel<double><<<grid_for(n, block), block, 0, s>>>(
        layers.zbuffer, layers.opacity, layers.colour, image16, layers.width, layers.height, scene.persp, q,
        scene.perspectiveType, scene.globalIlum, (const double *)tables, (const double *)tables + q);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(MBGB_ERR_CUDA, std::string("SSAO kernel: ") + cudaGetErrorString(e));
  return MBGB_OK;
}

}  // namespace mbgb
