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

// ---- Packed FP32 (f32x2): two orbits per thread ----
// A pair of floats in one 64-bit register pair: low half = ray A, high half = ray B. The
// f32x2 add / mul / fma each round both halves exactly as the scalar .rn instructions do,
// in one issue slot; min/max, saturation and the MUFU reciprocal have no packed form and
// stay scalar per half.
using f2 = unsigned long long;

__device__ __forceinline__ f2 f2_pack(const float lo, const float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float f2_lo(const f2 v) {
  float lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
  return lo;
}
__device__ __forceinline__ float f2_hi(const f2 v) {
  float lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
  return hi;
}
__device__ __forceinline__ f2 f2_fma(const f2 a, const f2 b, const f2 c) {
  f2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ f2 f2_mul(const f2 a, const f2 b) {
  f2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

// The state of two lean Mandelbox orbits, kept NEGATED (nx = -x, ncx = -cx): f32x2 has no
// operand negation, and with the sign folded into the state every step of box_iteration is
// one packed FMA that rounds exactly as its scalar counterpart:
//   fold   clamp(-x) = -clamp(x) (the clamp interval is symmetric), so
//          fma(clamp(nx), -2, nx) = round(2 clamp(x) - x), the scalar fold (positive form);
//   scale  fma(x, -ks, -cx) = -round(x ks + cx) (round to nearest is odd-symmetric), with
//          -ks = fma(t, -s(k1-1), -s);
//   dr     |ks| = fma(t, |s(k1-1)|, |s|): s and s(k1-1) share a sign (k1 >= 1), so this is
//          |fma(t, s(k1-1), s)| exactly.
// Squared radii are sign-free. Per ray (half): -s, -s(k1-1), |s|, |s(k1-1)|.
struct BoxPair {
  f2 nx, ny, nz, dr, ncx, ncy, ncz;
  f2 ns, nskm1, as, askm1;
};

__device__ __forceinline__ void box_pair_start(BoxPair &o, const LeanBoxK &k, const float cf, const float pxA,
                                               const float pyA, const float pzA, const float sA, const float pxB,
                                               const float pyB, const float pzB, const float sB) {
  o.nx = f2_pack(-pxA, -pxB);
  o.ny = f2_pack(-pyA, -pyB);
  o.nz = f2_pack(-pzA, -pzB);
  o.ncx = f2_pack(-__fmul_rn(pxA, cf), -__fmul_rn(pxB, cf));
  o.ncy = f2_pack(-__fmul_rn(pyA, cf), -__fmul_rn(pyB, cf));
  o.ncz = f2_pack(-__fmul_rn(pzA, cf), -__fmul_rn(pzB, cf));
  o.dr = f2_pack(1.0f, 1.0f);
  const float skA = __fmul_rn(sA, k.km1), skB = __fmul_rn(sB, k.km1);
  o.ns = f2_pack(-sA, -sB);
  o.nskm1 = f2_pack(-skA, -skB);
  o.as = f2_pack(fabsf(sA), fabsf(sB));
  o.askm1 = f2_pack(fabsf(skA), fabsf(skB));
}

// One iteration of both orbits (box_iteration per half, bit for bit); returns both new
// squared radii.
__device__ __forceinline__ f2 box_iteration_x2(const LeanBoxK &k, BoxPair &o) {
  const float fl = k.fl;
  const f2 m2 = f2_pack(-2.0f, -2.0f), one = f2_pack(1.0f, 1.0f);
  const f2 cx = f2_pack(fminf(fmaxf(f2_lo(o.nx), -fl), fl), fminf(fmaxf(f2_hi(o.nx), -fl), fl));
  const f2 cy = f2_pack(fminf(fmaxf(f2_lo(o.ny), -fl), fl), fminf(fmaxf(f2_hi(o.ny), -fl), fl));
  const f2 cz = f2_pack(fminf(fmaxf(f2_lo(o.nz), -fl), fl), fminf(fmaxf(f2_hi(o.nz), -fl), fl));
  const f2 x = f2_fma(cx, m2, o.nx), y = f2_fma(cy, m2, o.ny), z = f2_fma(cz, m2, o.nz);
  const f2 r2 = f2_fma(z, z, f2_fma(y, y, f2_mul(x, x)));
  const f2 t = f2_pack(__saturatef(fmaf(k.sa, rcp_approx(f2_lo(r2)), -k.sb)),
                       __saturatef(fmaf(k.sa, rcp_approx(f2_hi(r2)), -k.sb)));
  const f2 nks = f2_fma(t, o.nskm1, o.ns), aks = f2_fma(t, o.askm1, o.as);
  o.nx = f2_fma(x, nks, o.ncx);
  o.ny = f2_fma(y, nks, o.ncy);
  o.nz = f2_fma(z, nks, o.ncz);
  o.dr = f2_fma(o.dr, aks, one);
  return f2_fma(o.nz, o.nz, f2_fma(o.ny, o.ny, f2_mul(o.nx, o.nx)));
}

// One Mandelbox iteration (box_iteration) with x and y in one f32x2 pair, kept NEGATED
// (nxy = (-x, -y), ncxy = (-cx, -cy)), and z scalar. The box fold of x and y is one packed FMA,
// fma(clamp(-x), -2, -x) = round(2 clamp(x) - x) (the clamp interval is symmetric), which
// leaves the folded pair positive; the scale of the pair is another, fma(fx, -ks, -cx) =
// -round(fx ks + cx), with -ks = fma(t, -s(k1 - 1), -s) formed as box_iteration forms ks.
// Every lane rounds as box_iteration's scalar FMAs do, so the orbit is the same bit for bit.
__device__ __forceinline__ float box_iteration_xy(const LeanBoxK &k, const float ns, const float nskm1, f2 &nxy,
                                                  float &z, float &dr, const f2 ncxy, const float cz) {
  const float fl = k.fl;
  const f2 cl = f2_pack(fminf(fmaxf(f2_lo(nxy), -fl), fl), fminf(fmaxf(f2_hi(nxy), -fl), fl));
  const f2 fxy = f2_fma(cl, f2_pack(-2.0f, -2.0f), nxy);
  z = fmaf(fminf(fmaxf(z, -fl), fl), 2.0f, -z);
  const float r2 = norm2_rn(f2_lo(fxy), f2_hi(fxy), z);
  const float nks = fmaf(__saturatef(fmaf(k.sa, rcp_approx(r2), -k.sb)), nskm1, ns);
  nxy = f2_fma(fxy, f2_pack(nks, nks), ncxy);
  z = fmaf(z, -nks, cz);
  dr = fmaf(dr, fabsf(nks), 1.0f);
  return norm2_rn(f2_lo(nxy), f2_hi(nxy), z);
}

// The lean Mandelbox orbit of (x, y, z) with constant c, at most N iterations: returns the
// distance estimate r / |dr| at the first iteration whose radius passes the bailout
// (r^2 > 1024^2), with that iteration's index in L, or 0 with L = N when the orbit stays
// bounded. The iterations run in blocks of kBoxBlock, each followed by its bailout test,
// and the iteration count is tested once per block (a remainder loop takes N mod
// kBoxBlock), so the loop spends no instructions on the count inside a block. The iteration
// is box_iteration_xy, box_iteration's values with x and y in one packed pair.
constexpr int kBoxBlock = 5;

__device__ __forceinline__ float box_orbit(const LeanBoxK &k, const float s, const float skm1, float x, float y,
                                           float z, const float cx, const float cy, const float cz, const int N,
                                           int &L) {
  float dr = 1.0f;
  f2 nxy = f2_pack(-x, -y);
  const f2 ncxy = f2_pack(-cx, -cy);
  const float ns = -s, nskm1 = -skm1;
  int l = 0;
  for (; l <= N - kBoxBlock; l += kBoxBlock) {
#pragma unroll
    for (int u = 0; u < kBoxBlock; u++) {
      const float r2 = box_iteration_xy(k, ns, nskm1, nxy, z, dr, ncxy, cz);
      if (r2 > 1048576.0f) {
        L = l + u;
        return box_bailout_dist(r2, dr);
      }
    }
  }
#pragma unroll 1
  for (; l < N; l++) {
    const float r2 = box_iteration_xy(k, ns, nskm1, nxy, z, dr, ncxy, cz);
    if (r2 > 1048576.0f) {
      L = l;
      return box_bailout_dist(r2, dr);
    }
  }
  L = N;
  return 0.0f;
}

}  // namespace dev
}  // namespace mbgb
