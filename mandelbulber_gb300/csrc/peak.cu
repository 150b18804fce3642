// ALU peak microbenchmark used by bench.py as the roofline denominator of the
// ray-march kernels: dependent-free FMA chains in FP32 or FP64, sized to fill
// every SM. Reports FLOP/s counting one FMA as two operations.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

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

extern "C" double mbgb_peak_tflops(int fp64, int device) {
  if (cudaSetDevice(device) != cudaSuccess) return -1.0;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return -1.0;
  const int block = 256;
  const int grid = prop.multiProcessorCount * 8;
  const int iters = fp64 ? 64 : 2048;
  void *out = nullptr;
  if (cudaMalloc(&out, (size_t)grid * block * 8) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 6; rep++) {
    cudaEventRecord(e0);
    if (fp64) fma_chains<double><<<grid, block>>>((double *)out, iters, 0.999999, 1e-7);
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
