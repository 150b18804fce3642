// Post-processing of a rendered frame on the device: CompileImage (src/cimage.cpp:132-214)
// into the 16-bit image, the screen-space ambient occlusion pass PostRendering_SSAO /
// ThreadSSAO (src/image.cpp:249-478) and the depth of field PostRendering_DOF
// (src/image.cpp:57-206), which the reference runs in that order after the render when
// post_SSAO_enabled / post_DOF_enabled are set (src/Render3D.cpp:1093-1106).
//
// Built with --fmad=false: the FP64 SSAO and the compile step follow the reference's
// double-precision operation order, so results match it to the last bit except where
// CUDA's atan / tanhf round differently from the host's libm.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <utility>
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

// One splat of PostRendering_DOF (src/image.cpp:148-182): the pixel at (x, y) spreads its
// original RGB16 / alpha over the pixels within `size` at opacity (blur - r) / factor.
struct DofSplat {
  int x, y, size, centre;   // centre: the pixel index of (x, y)
  double blur, factor;
};

constexpr int kDofTile = 16;

// Each CTA owns one 16 x 16 tile; each thread owns one pixel of it and applies, in the
// splat order, every splat of the tile's list that covers its pixel. A pixel's value after
// the pass is the reference's sequential in-place fold: splats change only pixels they cover
// and read only the frame's original values at their centres.
__global__ void dof_kernel(const DofSplat *__restrict__ splats, const int64_t *__restrict__ tileStart,
                           const int *__restrict__ tileList, const int tilesX, const int width, const int height,
                           const uint16_t *__restrict__ image0, const uint16_t *__restrict__ alpha0,
                           uint16_t *__restrict__ image16, uint16_t *__restrict__ alpha) {
  const int tile = blockIdx.x;
  const int xx = (tile % tilesX) * kDofTile + (int)(threadIdx.x % kDofTile);
  const int yy = (tile / tilesX) * kDofTile + (int)(threadIdx.x / kDofTile);
  if (xx >= width || yy >= height) return;
  const int64_t q = (int64_t)yy * width + xx;
  uint16_t v[3] = {image16[3 * q + 0], image16[3 * q + 1], image16[3 * q + 2]};
  uint16_t a = alpha[q];
  for (int64_t k = tileStart[tile]; k < tileStart[tile + 1]; k++) {
    const DofSplat sp = splats[tileList[k]];
    const int dx = xx - sp.x, dy = yy - sp.y;
    if (dx < -sp.size || dx > sp.size || dy < -sp.size || dy > sp.size) continue;
    const double r = (double)sqrtf((float)dx * dx + dy * dy);
    double op = (sp.blur - r) / sp.factor;
    if (op > 1.0) op = 1.0;
    if (op < 0.0) op = 0.0;
    if (op > 0.0) {
      const double opN = 1.0 - op;
      for (int c = 0; c < 3; c++) v[c] = (uint16_t)(v[c] * opN + image0[3 * (int64_t)sp.centre + c] * op);
      a = (uint16_t)(a * opN + alpha0[sp.centre] * op);
    }
  }
  image16[3 * q + 0] = v[0];
  image16[3 * q + 1] = v[1];
  image16[3 * q + 2] = v[2];
  alpha[q] = a;
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

namespace {

struct SortZ {
  float z;
  int i;
};

// QuickSortZBuffer (src/common_math.h:53-84): Hoare partition around the middle element, on
// [l, p]; an explicit stack instead of recursion (the two parts are disjoint).
void quicksort_z(std::vector<SortZ> &d, int l0, int p0) {
  std::vector<std::pair<int, int>> stack{{l0, p0}};
  while (!stack.empty()) {
    const int l = stack.back().first, p = stack.back().second;
    stack.pop_back();
    int i = l, j = p;
    const SortZ x = d[(size_t)((l + p) / 2)];
    do {
      while (d[(size_t)i].z < x.z) i++;
      while (x.z < d[(size_t)j].z) j--;
      if (i <= j) {
        std::swap(d[(size_t)i], d[(size_t)j]);
        i++;
        j--;
      }
    } while (i <= j);
    if (i < p) stack.push_back({i, p});
    if (l < j) stack.push_back({l, j});
  }
}

}  // namespace

namespace mbgb {

// PostRendering_DOF (src/image.cpp:57-206). The host sorts the z-buffer with the
// reference's quicksort (element 0 stays in place, as there), shuffles it with its Random()
// swaps (rand() seeded with `seed`; the reference continues the process's rand() stream),
// and lists, per 16 x 16 tile, the splats that reach it in splat order (far to near); the
// device applies the splats (dof_kernel).
mbgb_status dof_device(const mbgb_scene &scene, const mbgb_image &layers, uint16_t *image16, uint32_t seed,
                       cudaStream_t s) {
  const int width = layers.width, height = layers.height;
  const int64_t n = (int64_t)width * height;
  if (n <= 0 || n > (int64_t)1 << 30) return set_error(MBGB_ERR_BAD_PARAM, "DOF: image size out of range");
  const double deep = scene.DOFRadius * width / 1000.0;
  const double neutral = pow(10, scene.DOFFocus / 10.0 - 16.0);
  std::vector<SortZ> sortz((size_t)n);
  std::vector<float> zb((size_t)n);
  cudaError_t e = cudaMemcpyAsync(zb.data(), layers.zbuffer, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(MBGB_ERR_CUDA, std::string("DOF z-buffer: ") + cudaGetErrorString(e));
  for (int64_t p = 0; p < n; p++) sortz[(size_t)p] = SortZ{zb[(size_t)p], (int)p};
  if (n > 2) quicksort_z(sortz, 1, (int)n - 1);
  // randomise the order within similar blur sizes (src/image.cpp:96-138)
  GlibcRand rng(seed);
  for (int64_t i = n - 1; i >= 0; i--) {
    const SortZ temp = sortz[(size_t)i];
    const double z1 = temp.z;
    const double size1 = (z1 - neutral) / z1 * deep;
    int randomStep = (int)i;
    bool done = false;
    int64_t ii;
    do {
      ii = i - rng.random(randomStep);
      if (ii <= 0) ii = 0;
      const double z2 = sortz[(size_t)ii].z;
      const double size2 = (z2 - neutral) / z2 * deep;
      if (size1 == 0 && size2 == 0) done = true;
      if (size1 * size2 > 0) {
        const double sizeCompare = size1 > 0 ? size2 / size1 : size1 / size2;
        done = sizeCompare > 0.7;
      } else {
        done = false;
      }
      randomStep = (int)(randomStep * 0.7 - 1);
      if (randomStep <= 0) done = true;
    } while (!done);
    sortz[(size_t)i] = sortz[(size_t)ii];
    sortz[(size_t)ii] = temp;
  }
  // splats in order, and the tiles each reaches
  const int tilesX = (width + kDofTile - 1) / kDofTile, tilesY = (height + kDofTile - 1) / kDofTile;
  std::vector<DofSplat> splats((size_t)n);
  std::vector<int64_t> count((size_t)tilesX * tilesY + 1, 0);
  for (int64_t k = 0; k < n; k++) {
    const int ii = sortz[(size_t)(n - k - 1)].i;
    const int x = ii % width, y = ii / width;
    const double z = zb[(size_t)ii];
    double blur = fabs(z - neutral) / z * deep;
    if (blur > 100) blur = 100.0;
    const int size = (int)blur;
    splats[(size_t)k] = DofSplat{x, y, size, ii, blur, blur * blur * sqrt(blur) * kPi / 3.0};
    const int tx0 = std::max(0, x - size) / kDofTile, tx1 = std::min(width - 1, x + size) / kDofTile;
    const int ty0 = std::max(0, y - size) / kDofTile, ty1 = std::min(height - 1, y + size) / kDofTile;
    for (int ty = ty0; ty <= ty1; ty++)
      for (int tx = tx0; tx <= tx1; tx++) count[(size_t)ty * tilesX + tx + 1]++;
  }
  for (size_t t = 1; t < count.size(); t++) count[t] += count[t - 1];
  std::vector<int> list((size_t)count.back());
  std::vector<int64_t> fill(count.begin(), count.end() - 1);
  for (int64_t k = 0; k < n; k++) {
    const DofSplat &sp = splats[(size_t)k];
    const int tx0 = std::max(0, sp.x - sp.size) / kDofTile, tx1 = std::min(width - 1, sp.x + sp.size) / kDofTile;
    const int ty0 = std::max(0, sp.y - sp.size) / kDofTile, ty1 = std::min(height - 1, sp.y + sp.size) / kDofTile;
    for (int ty = ty0; ty <= ty1; ty++)
      for (int tx = tx0; tx <= tx1; tx++) list[(size_t)fill[(size_t)ty * tilesX + tx]++] = (int)k;
  }
  // device buffers: splats, tile starts, lists, original image and alpha
  const size_t bSplat = sizeof(DofSplat) * (size_t)n, bStart = sizeof(int64_t) * count.size(),
               bList = sizeof(int) * list.size(), bImg = sizeof(uint16_t) * 3 * (size_t)n,
               bAlpha = sizeof(uint16_t) * (size_t)n;
  char *buf = nullptr;
  e = cudaMallocAsync((void **)&buf, bSplat + bStart + bList + bImg + bAlpha + 64, s);
  if (e != cudaSuccess) return set_error(MBGB_ERR_CUDA, std::string("DOF buffers: ") + cudaGetErrorString(e));
  char *pSplat = buf, *pStart = pSplat + bSplat, *pList = pStart + bStart, *pImg = pList + bList;
  pImg = (char *)(((uintptr_t)pImg + 15) & ~(uintptr_t)15);
  char *pAlpha = pImg + bImg;
  e = cudaMemcpyAsync(pSplat, splats.data(), bSplat, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(pStart, count.data(), bStart, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && bList) e = cudaMemcpyAsync(pList, list.data(), bList, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(pImg, image16, bImg, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(pAlpha, layers.alpha, bAlpha, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    dof_kernel<<<tilesX * tilesY, kDofTile * kDofTile, 0, s>>>(
        (const DofSplat *)pSplat, (const int64_t *)pStart, (const int *)pList, tilesX, width, height,
        (const uint16_t *)pImg, (const uint16_t *)pAlpha, image16, layers.alpha);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(buf, s);
  cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(MBGB_ERR_CUDA, std::string("DOF kernel: ") + cudaGetErrorString(e));
  return MBGB_OK;
}

}  // namespace mbgb
