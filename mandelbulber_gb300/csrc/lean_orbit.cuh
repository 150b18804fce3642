// The lean FP32 Mandelbox iteration (formula 8 without rotations, offsets, pre-folds or
// julia; fold value = 2 x fold limit): shared by the render kernels (wave_core.cuh) and the
// orbit-loop microbenchmark of the peak tool (peak.cu), which times this exact iteration.
#pragma once

#include <cuda_runtime.h>

namespace mbgb {
namespace dev {

// rcp.approx.ftz.f32: the reciprocal the hardware's special-function unit returns, without
// the refinement of a correctly rounded division.
__device__ __forceinline__ float rcp_approx(const float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The lean FP32 orbits below spell out every multiply-add (fmaf, __fmul_rn) so that the
// compiler has no contraction left to choose: the one-call orbits and their resumable
// versions then round identically in every kernel that inlines them.
__device__ __forceinline__ float norm2_rn(const float x, const float y, const float z) {
  return fmaf(z, z, fmaf(y, y, __fmul_rn(x, x)));
}

// Distance estimate r / |dr| at the bailout from the squared radius, with the approximate
// square root and quotient (MUFU rsqrt/rcp; a few ulp, far inside the FP32 policy's
// tolerance): once per orbit, where the correctly rounded forms cost more than an iteration.
__device__ __forceinline__ float box_bailout_dist(const float r2, const float dr) {
  return __fdividef(__fmul_rn(r2, rsqrtf(r2)), fabsf(dr));
}

// Constants of the lean Mandelbox iteration: fold limit, and with k1 = fR2/mR2 >= 1 (min
// radius <= fixed radius) the quotients fR2/(k1 - 1), 1/(k1 - 1) and k1 - 1 (0, 0, 0 when
// k1 = 1), derived once on the host.
struct LeanBoxK {
  float fl, sa, sb, km1;
};

// One Mandelbox iteration (scale s, constant c); returns the new squared radius.
// Box fold: clamp(x) * 2 - x, identical to fv - x / -fv - x (fold value = 2 x fold limit;
// the product by 2 is exact, so the FMA rounds once, as the two-step form does). Sphere
// fold: fR2/mR2 inside mR2, fR2/r2 between mR2 and fR2, 1 outside; the clamp of fR2/r2 to
// [1, k1], written 1 + (k1 - 1) sat((fR2/r2 - 1) / (k1 - 1)) so that the clamp rides on
// the FMA pipe's saturation instead of two min/max instructions, with the approximate
// reciprocal feeding one saturating FMA (measured +11 % orbit rate).
// The scale rides on the same FMA: k s = s + (s (k1 - 1)) sat(...), with skm1 = s (k1 - 1)
// formed once per orbit (one rounding where k and k s took two; one instruction less).
__device__ __forceinline__ float box_iteration(const LeanBoxK &k, const float s, const float skm1, float &x,
                                               float &y, float &z, float &dr, const float cx, const float cy,
                                               const float cz) {
  x = fmaf(fminf(fmaxf(x, -k.fl), k.fl), 2.0f, -x);
  y = fmaf(fminf(fmaxf(y, -k.fl), k.fl), 2.0f, -y);
  z = fmaf(fminf(fmaxf(z, -k.fl), k.fl), 2.0f, -z);
  const float r2 = norm2_rn(x, y, z);
  const float ks = fmaf(__saturatef(fmaf(k.sa, rcp_approx(r2), -k.sb)), skm1, s);
  x = fmaf(x, ks, cx);
  y = fmaf(y, ks, cy);
  z = fmaf(z, ks, cz);
  dr = fmaf(dr, fabsf(ks), 1.0f);   // |k s| with the operand's absolute-value modifier
  return norm2_rn(x, y, z);
}

}  // namespace dev
}  // namespace mbgb
