// ALU peak microbenchmark used by bench.py as the roofline denominator of the
// ray-march kernels: dependent-free FMA chains in FP32 or FP64, sized to fill
// every SM. Reports FLOP/s counting one FMA as two operations.
// Also the orbit-loop ceiling of the lean Mandelbox iteration: the render kernels'
// iteration (lean_orbit.cuh) on bounded orbits, every lane busy, no ray bookkeeping.
#include <cuda_runtime.h>

#include <cstdint>

#include "lean_orbit.cuh"

namespace {

using mbgb::dev::LeanBoxK;

// Orbits of points near the origin (inside the scale-2 Mandelbox, so no lane leaves early),
// n iterations each through the renderer's orbit loop (box_orbit: the bailout test after
// every iteration, the count test once per block).
__global__ void box_orbit_loop(float *out, unsigned long long *count, int orbits, int n, LeanBoxK k, float s,
                               float skm1) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.0f;
  unsigned long long it = 0;
  for (int o = 0; o < orbits; o++) {
    const float cx = 1e-4f * (float)((tid + 7 * o) & 1023), cy = 1e-4f * (float)((tid * 3 + o) & 1023),
                cz = 1e-4f * (float)((tid * 5 + 3 * o) & 1023);
    int L;
    const float d = mbgb::dev::box_orbit(k, s, skm1, cx, cy, cz, cx, cy, cz, n, L);
    it += (unsigned long long)(L + 1);
    acc += d + (float)L;
  }
  if (acc == -1.2345f) out[tid] = acc;  // keeps the orbits live
  atomicAdd(count, it);
}

// The same orbits two per thread with the packed iteration (box_iteration_x2): every
// iteration of both halves is counted, the bailout test of both evaluated every iteration.
__global__ void box_orbit_loop_x2(float *out, unsigned long long *count, int orbits, int n, LeanBoxK k, float s) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.0f;
  unsigned long long it = 0;
  for (int o = 0; o < orbits; o += 2) {
    const float ax = 1e-4f * (float)((tid + 7 * o) & 1023), ay = 1e-4f * (float)((tid * 3 + o) & 1023),
                az = 1e-4f * (float)((tid * 5 + 3 * o) & 1023);
    const float bx = 1e-4f * (float)((tid + 7 * o + 7) & 1023), by = 1e-4f * (float)((tid * 3 + o + 1) & 1023),
                bz = 1e-4f * (float)((tid * 5 + 3 * o + 3) & 1023);
    mbgb::dev::BoxPair p;
    mbgb::dev::box_pair_start(p, k, 1.0f, ax, ay, az, s, bx, by, bz, s);
    int L;
#pragma unroll 5
    for (L = 0; L < n; L++) {
      const mbgb::dev::f2 r2 = mbgb::dev::box_iteration_x2(k, p);
      if (mbgb::dev::f2_lo(r2) > 1048576.0f || mbgb::dev::f2_hi(r2) > 1048576.0f) break;
    }
    it += 2ull * (unsigned long long)(L + 1);
    acc += mbgb::dev::f2_lo(p.nx) + mbgb::dev::f2_hi(p.ny) + mbgb::dev::f2_lo(p.dr) + mbgb::dev::f2_hi(p.dr);
  }
  if (acc == -1.2345f) out[tid] = acc;  // keeps the orbits live
  atomicAdd(count, it);
}

// Packed FP32 FMA chains (fma.rn.f32x2): two FMAs per instruction.
__global__ void fma_chains_x2(float *out, int iters, float a, float b) {
  using mbgb::dev::f2;
  const f2 A = mbgb::dev::f2_pack(a, a), B = mbgb::dev::f2_pack(b, b);
  const float t = (float)threadIdx.x;
  f2 x0 = mbgb::dev::f2_pack(t, t + 1), x1 = mbgb::dev::f2_pack(t + 2, t + 3), x2 = mbgb::dev::f2_pack(t + 4, t + 5),
     x3 = mbgb::dev::f2_pack(t + 6, t + 7);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      x0 = mbgb::dev::f2_fma(x0, A, B); x1 = mbgb::dev::f2_fma(x1, A, B);
      x2 = mbgb::dev::f2_fma(x2, A, B); x3 = mbgb::dev::f2_fma(x3, A, B);
    }
  }
  const float s = mbgb::dev::f2_lo(x0) + mbgb::dev::f2_hi(x1) + mbgb::dev::f2_lo(x2) + mbgb::dev::f2_hi(x3);
  if (s == -1.2345f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

template <typename T>
__global__ void fma_chains(T *out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-1.2345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

// fp64: 0 = FP32 FMA chains, 1 = FP64, 2 = packed FP32 (fma.rn.f32x2) chains.
extern "C" double mbgb_peak_tflops(int fp64, int device) {
  if (cudaSetDevice(device) != cudaSuccess) return -1.0;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return -1.0;
  const int block = 256;
  const int grid = prop.multiProcessorCount * 8;
  const int iters = fp64 == 1 ? 64 : 2048;
  void *out = nullptr;
  if (cudaMalloc(&out, (size_t)grid * block * 8) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 6; rep++) {
    cudaEventRecord(e0);
    if (fp64 == 1) fma_chains<double><<<grid, block>>>((double *)out, iters, 0.999999, 1e-7);
    else if (fp64 == 2) fma_chains_x2<<<grid, block>>>((float *)out, iters, 0.999999f, 1e-7f);
    else fma_chains<float><<<grid, block>>>((float *)out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  const double flops = 2.0 * 64.0 * (double)iters * grid * block;
  return flops / (best * 1e-3) / 1e12;
}

// Iterations per second (in units of 1e12) of the lean Mandelbox iteration in isolation, for
// scale 2, fold limit 1, min radius 0.5, fixed radius 1 (the 1080p Mandelbox workload),
// 128-thread CTAs at 10 per SM (the shadow/AO kernel's occupancy), best of five timed runs.
extern "C" double mbgb_box_orbit_rate_impl(int device, int packed);
extern "C" double mbgb_box_orbit_rate(int device) { return mbgb_box_orbit_rate_impl(device, 0); }
// The same with two orbits per thread through the packed iteration (box_iteration_x2).
extern "C" double mbgb_box_orbit_rate_x2(int device) { return mbgb_box_orbit_rate_impl(device, 1); }

extern "C" double mbgb_box_orbit_rate_impl(int device, int packed) {
  if (cudaSetDevice(device) != cudaSuccess) return -1.0;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return -1.0;
  const int block = 128, grid = prop.multiProcessorCount * 10, orbits = 64, n = 60;
  const float fR2 = 1.0f, mR2 = 0.25f, km1 = fR2 / mR2 - 1.0f, s = 2.0f;
  const LeanBoxK k{1.0f, fR2 / km1, 1.0f / km1, km1};
  void *out = nullptr, *count = nullptr;
  if (cudaMalloc(&out, (size_t)grid * block * 4) != cudaSuccess) return -1.0;
  if (cudaMalloc(&count, 8) != cudaSuccess) {
    cudaFree(out);
    return -1.0;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 6; rep++) {
    cudaMemset(count, 0, 8);
    cudaEventRecord(e0);
    if (packed) box_orbit_loop_x2<<<grid, block>>>((float *)out, (unsigned long long *)count, orbits, n, k, s);
    else box_orbit_loop<<<grid, block>>>((float *)out, (unsigned long long *)count, orbits, n, k, s, s * km1);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    unsigned long long h = 0;
    cudaMemcpy(&h, count, 8, cudaMemcpyDeviceToHost);
    const double rate = (double)h / (ms * 1e-3) / 1e12;
    if (rep > 0 && rate > best) best = rate;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  cudaFree(count);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  return best;
}
