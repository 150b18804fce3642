// Device side of the per-pixel distance-estimated ray march.
//
// One template body serves both precision policies:
//   * T = double, compiled with --fmad=false: every DE, march and shader runs in
//     IEEE double with the reference's operation order, so the formulas built from
//     + - * / sqrt (Mandelbox) reproduce the CPU results bit for bit.
//   * T = float: the march, the orbit iteration and the shaders run in FP32 with
//     FMA; the camera ray is formed in FP64 and the final binary hit refinement
//     runs in FP64 (FractalT<double>).
// The reference functions each part follows are cited at the function.
#pragma once

#include "lean_orbit.cuh"
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernel_params.h"

namespace mbgb {
namespace dev {

// ---------------------------------------------------------------------------
// small vector type and precision-overloaded math
// ---------------------------------------------------------------------------
template <typename T>
struct V3 {
  T x, y, z;
};
template <typename T>
__device__ __forceinline__ V3<T> operator+(const V3<T> a, const V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
__device__ __forceinline__ V3<T> operator-(const V3<T> a, const V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
__device__ __forceinline__ V3<T> operator*(const V3<T> a, const T s) { return {a.x * s, a.y * s, a.z * s}; }
// CVector3::Dot / Length (src/algebra.hpp:89-96): ((x*x + y*y) + z*z)
template <typename T>
__device__ __forceinline__ T dot3(const V3<T> a, const V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_fabs(double x) { return fabs(x); }
__device__ __forceinline__ float m_fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_asin(double x) { return asin(x); }
__device__ __forceinline__ float m_asin(float x) { return asinf(x); }
__device__ __forceinline__ double m_atan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ float m_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double m_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float m_pow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
__device__ __forceinline__ float m_log(float x) { return logf(x); }
__device__ __forceinline__ double m_floor(double x) { return floor(x); }
__device__ __forceinline__ float m_floor(float x) { return floorf(x); }
__device__ __forceinline__ void m_sincos(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void m_sincos(float x, float *s, float *c) { sincosf(x, s, c); }

template <typename T>
__device__ __forceinline__ T length3(const V3<T> a) { return m_sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// |z| of an orbit point. FP32: the squares overflow once a component passes 1.8e19, which
// an orbit of power ~10 reaches at its escape step (r^p with r up to the bailout 100);
// the length is then taken from the components scaled by the largest one. FP64 keeps the
// reference's plain expression (its range is not reached before the bailout).
template <typename T>
__device__ __forceinline__ T orbit_length(const V3<T> a) {
  const T r2 = a.x * a.x + a.y * a.y + a.z * a.z;
  if (sizeof(T) == 4 && !(r2 <= T(3.0e38))) {
    const T m = m_fabs(a.x) > m_fabs(a.y) ? (m_fabs(a.x) > m_fabs(a.z) ? m_fabs(a.x) : m_fabs(a.z))
                                           : (m_fabs(a.y) > m_fabs(a.z) ? m_fabs(a.y) : m_fabs(a.z));
    if (!(m <= T(3.0e38))) return m;   // a component already overflowed (inf) or is NaN
    const T x = a.x / m, y = a.y / m, z = a.z / m;
    return m * m_sqrt(x * x + y * y + z * z);
  }
  return m_sqrt(r2);
}

// CVector3::Normalize (src/algebra.hpp:105-112): multiply by 1/length.
template <typename T>
__device__ __forceinline__ V3<T> normalize3(const V3<T> a) {
  const T norm = T(1) / length3(a);
  return {a.x * norm, a.y * norm, a.z * norm};
}

// Conversions with the results the reference gets from x86-64 code
// (cvttsd2si to a 32-bit register, out-of-range -> INT_MIN, then truncation of
// the register to the narrower type).
__device__ __forceinline__ int to_i32_x86(double v) {
  return (v >= -2147483648.0 && v < 2147483648.0) ? (int)v : (int)0x80000000;
}
__device__ __forceinline__ unsigned short to_u16_x86(double v) { return (unsigned short)to_i32_x86(v); }
__device__ __forceinline__ unsigned char to_u8_x86(double v) { return (unsigned char)to_i32_x86(v); }

// CRotationMatrix::RotateVector with its identity short-cut (src/algebra.cpp:163-174).
template <typename T>
__device__ __forceinline__ V3<T> rotate(const T *m, int zero, const V3<T> v) {
  if (zero) return v;
  return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
          m[6] * v.x + m[7] * v.y + m[8] * v.z};
}

// Device-side deadline: true once the launch has run longer than io.budget_ns.
// The first caller stamps the launch start; every wait loop here is bounded, the
// deadline only shortens a frame that would take too long.
__device__ __forceinline__ bool deadline_passed(const FrameIO &io) {
  if (!io.budget_ns) return false;
  unsigned long long now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
  unsigned long long st = atomicCAS(io.start_ns, 0ull, now);
  if (st == 0ull) st = now;
  return now - st > io.budget_ns;
}

struct Counters {
  unsigned long long orbit;   // N_counter: sum of (L + 1)
  unsigned long long calls;   // Loop_counter
  unsigned long long steps;   // DE_counter (primary march + refinement)
  unsigned long long missed;  // Missed_DE_counter
  int objectOut;              // calcParam->objectOut: the object the last distance ended on
};

// Formulas whose main parameter is the Mandelbox scale (tglad 8, smoothMandelbox 17,
// mandelboxVaryScale4D 18, generalizedFoldBox 37); the others use the power.
__host__ __device__ __forceinline__ bool scale_formula(const int formula) {
  return formula == 8 || formula == 17 || formula == 18 || formula == 37;
}

// The formula's main parameter: the power or the Mandelbox scale.
template <typename T>
__host__ __device__ __forceinline__ T fparam_of(const FractalT<T> &f) {
  return scale_formula(f.formula) ? f.mbScale : f.power;
}

}  // namespace dev
}  // namespace mbgb

#include "formulas.cuh"

namespace mbgb {
namespace dev {

// ---------------------------------------------------------------------------
// Compute<Mode> (src/fractal.cpp:40-1241). MODE 0 = normal (returns the distance
// estimate), MODE 1 = colouring. FORMULA 2 (trig_optim) and 8 (tglad) are compiled as
// such; FORMULA 0 runs the formula f.formula selects through the run-time formula path
// (compute_runtime, formulas.cuh).
// ---------------------------------------------------------------------------
// `fparam` is the formula's main parameter: the power, or the Mandelbox scale of the
// scale formulas (a frame of a batch may carry its own; see fparam_of).
template <typename T, int FORMULA, int MODE>
__device__ __forceinline__ T compute(const FractalT<T> &f, V3<T> z, const int N, int &Lout, Counters &cnt,
                                     const T fparam) {
  if (FORMULA == 0 || MODE == kModeOrbitTrap) {
    int L;
    const T d = compute_runtime<T, MODE>(&f, z, N, 0, &L, fparam);
    cnt.orbit += (unsigned long long)(L + 1);
    cnt.calls += 1;
    Lout = L;
    return d;
  }
  T distance = T(0);
  T r_dz = T(1);
  const T p = fparam;
  const T fR2 = f.mbFixedR * f.mbFixedR;
  const T mR2 = f.mbMinR * f.mbMinR;
  const T tglad_factor1 = fR2 / mR2;
  T tgladDE = T(1);
  T tgladColor = T(1);
  const T scale = fparam;
  V3<T> constant;
  if (f.juliaMode) {
    constant = {f.julia[0], f.julia[1], f.julia[2]};
  } else {
    constant = z * f.constantFactor;
  }
  T r = orbit_length(z);
  T minv = (sizeof(T) == 8) ? T(1e200) : T(__int_as_float(0x7f800000));
  int L;
  for (L = 0; L < N; L++) {
    if (f.tgladFoldingMode) {  // src/fractal.cpp:124-156
      if (z.x > f.foldingLimit) { z.x = f.foldingValue - z.x; tgladColor *= T(0.9); }
      else if (z.x < -f.foldingLimit) { z.x = -f.foldingValue - z.x; tgladColor *= T(0.9); }
      if (z.y > f.foldingLimit) { z.y = f.foldingValue - z.y; tgladColor *= T(0.9); }
      else if (z.y < -f.foldingLimit) { z.y = -f.foldingValue - z.y; tgladColor *= T(0.9); }
      if (z.z > f.foldingLimit) { z.z = f.foldingValue - z.z; tgladColor *= T(0.9); }
      else if (z.z < -f.foldingLimit) { z.z = -f.foldingValue - z.z; tgladColor *= T(0.9); }
      r = orbit_length(z);
    }
    if (f.sphericalFoldingMode) {  // src/fractal.cpp:158-179
      const T fR2_2 = f.sphFixed * f.sphFixed;
      const T mR2_2 = f.sphMin * f.sphMin;
      const T r2_2 = r * r;
      const T tf1 = fR2_2 / mR2_2;
      if (r2_2 < mR2_2) {
        z = z * tf1; tgladDE *= tf1; tgladColor += T(1);
      } else if (r2_2 < fR2_2) {
        const T tf2 = fR2_2 / r2_2;
        z = z * tf2; tgladDE *= tf2; tgladColor += T(10);
      }
      r = orbit_length(z);
    }
    if (FORMULA == 2) {
      trig_optim_step(z, r, r_dz, p, constant);
    } else if (FORMULA == 8) {
      tglad_step(f, z, r, tgladDE, tgladColor, scale, constant, fR2, mR2, tglad_factor1);
    }
    // iteration terminate conditions (src/fractal.cpp:1133-1190)
    if (FORMULA == 8) {
      if (r > T(1024)) { distance = r / m_fabs(tgladDE); break; }
    } else {
      if (MODE == 0) {
        if (r > f.bailout) { distance = T(0.5) * r * m_log(r) / r_dz; break; }
      } else {
        distance = orbit_length(z);
        if (distance < minv) minv = distance;
        if (distance > T(1e15)) { distance = minv; break; }
      }
    }
  }
  cnt.orbit += (unsigned long long)(L + 1);
  cnt.calls += 1;
  Lout = L;
  if (MODE == 0) {
    if (L == N) distance = T(0);
    return distance;
  } else {
    if (FORMULA == 8) return tgladColor * T(100) + orbit_length(z) * f.mbColR;
    return distance * T(5000);
  }
}

// Constants of the lean Mandelbox iteration from the fractal block (the quotients are
// derived on the host: FractalT::leanKm1, leanSa, leanSb).
__device__ __forceinline__ LeanBoxK lean_box_k(const FractalT<float> &f) {
  return LeanBoxK{f.mbFoldLimit, f.leanSa, f.leanSb, f.leanKm1};
}

// Mandelbox orbit (formula 8, normal mode) for the common case: no rotation, no offset,
// no pre-folds, julia off, fold value = 2 x fold limit. Squared radius throughout: the
// bailout r > 1024 becomes r^2 > 1024^2 and the sphere fold tests r^2 directly, so the
// loop has no square root.
__device__ __forceinline__ float mandelbox_fast(const FractalT<float> &f, const float px, const float py,
                                                const float pz, const int N, int &Lout, Counters &cnt,
                                                const float s) {
  const LeanBoxK k = lean_box_k(f);
  const float skm1 = __fmul_rn(s, k.km1);
  const float cx = __fmul_rn(px, f.constantFactor), cy = __fmul_rn(py, f.constantFactor),
              cz = __fmul_rn(pz, f.constantFactor);
  int L;
  const float dist = box_orbit(k, s, skm1, px, py, pz, cx, cy, cz, N, L);
  cnt.orbit += (unsigned long long)(L + 1);
  cnt.calls += 1;
  Lout = L;
  return dist;
}

// One Mandelbulb power-8 iteration (trig_optim, src/fractal.cpp:211-225) without
// transcendentals: theta = asin(z/r) in [-pi/2, pi/2] has cos = rho/r >= 0 and sin = z/r;
// phi = atan2(y, x) has cos = x/rho, sin = y/rho (phi = 0 when rho = 0, as atan2(0, 0)).
// Three angle doublings (c, s) -> (c^2 - s^2, 2cs) give 8*theta and 8*phi; r^8 and r^7 come
// from r^2. Returns the new squared radius.
__device__ __forceinline__ float bulb8_iteration(float &x, float &y, float &z, const float r2, float &r_dz,
                                                 const float cx, const float cy, const float cz) {
  const float rho2 = fmaf(y, y, __fmul_rn(x, x));
  const float inv_r = rsqrtf(r2);
  const bool axis = rho2 == 0.0f;
  const float inv_rho = axis ? 0.0f : rsqrtf(rho2);
  float ct = __fmul_rn(__fmul_rn(rho2, inv_rho), inv_r), st = __fmul_rn(z, inv_r);
  float cp = axis ? 1.0f : __fmul_rn(x, inv_rho), sp = axis ? 0.0f : __fmul_rn(y, inv_rho);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const float ct2 = fmaf(ct, ct, -__fmul_rn(st, st)), st2 = __fmul_rn(__fmul_rn(2.0f, st), ct);
    const float cp2 = fmaf(cp, cp, -__fmul_rn(sp, sp)), sp2 = __fmul_rn(__fmul_rn(2.0f, sp), cp);
    ct = ct2; st = st2; cp = cp2; sp = sp2;
  }
  const float r4 = __fmul_rn(r2, r2);
  const float r8 = __fmul_rn(r4, r4);
  r_dz = fmaf(__fmul_rn(__fmul_rn(8.0f, r8), inv_r), r_dz, 1.0f);   // p * r^(p-1) * r_dz + 1
  const float t = __fmul_rn(ct, r8);
  x = fmaf(t, cp, cx);
  y = fmaf(t, sp, cy);
  z = fmaf(st, r8, cz);
  return norm2_rn(x, y, z);
}

// Mandelbulb power 8 orbit. MODE 0 returns the distance estimate 0.5*r*ln(r)/dr at the
// bailout r > 100 (or the scene's bailoutRadius: r^2 > FractalT::bailout2); MODE 1 returns
// the colouring value (min |z| until |z| > 1e15, times 5000). The iterations run in blocks of
// kBulbBlock with the end test after each and the count test once per block (a remainder
// loop takes N mod kBulbBlock), as the lean Mandelbox orbit's box_orbit does.
constexpr int kBulbBlock = 4;
template <int MODE>
__device__ __forceinline__ float mandelbulb8_fast(const FractalT<float> &f, const float px, const float py,
                                                  const float pz, const int N, int &Lout, Counters &cnt) {
  float cx, cy, cz;
  if (f.juliaMode) {
    cx = f.julia[0]; cy = f.julia[1]; cz = f.julia[2];
  } else {
    cx = __fmul_rn(px, f.constantFactor); cy = __fmul_rn(py, f.constantFactor); cz = __fmul_rn(pz, f.constantFactor);
  }
  float x = px, y = py, z = pz, r_dz = 1.0f, dist = 0.0f;
  float r2 = norm2_rn(x, y, z);
  float minr2 = __int_as_float(0x7f800000);
  const float bail2 = f.bailout2;
  // one iteration; true when the orbit ends at it
  auto step = [&]() -> bool {
    r2 = bulb8_iteration(x, y, z, r2, r_dz, cx, cy, cz);
    if (MODE == 0) return r2 > bail2;
    if (r2 < minr2) minr2 = r2;
    return r2 > 1.0e30f;
  };
  int L = 0;
  bool ended = false;
  while (!ended && L <= N - kBulbBlock) {
#pragma unroll
    for (int u = 0; u < kBulbBlock; u++) {
      if (step()) {
        L += u;
        ended = true;
        break;
      }
    }
    if (!ended) L += kBulbBlock;
  }
#pragma unroll 1
  for (; !ended && L < N; L++) {
    if (step()) {
      ended = true;
      break;
    }
  }
  if (MODE == 0 && ended) {
    const float r = sqrtf(r2);
    dist = __fmul_rn(__fmul_rn(0.5f, r), __logf(r)) / r_dz;
  }
  cnt.orbit += (unsigned long long)(L + 1);
  cnt.calls += 1;
  Lout = L;
  if (MODE == 0) {
    if (L == N) dist = 0.0f;
    return dist;
  }
  // colouring: min |z| after a bailout, else the last |z|
  return (L < N ? sqrtf(minr2) : sqrtf(r2)) * 5000.0f;
}

// CalculateDistance's limit box (src/fractal.cpp:1252-1262): the distance to the box, and true
// when the point lies farther from it than detailSize (the estimate is then that distance,
// with no orbit and itersOut left as it was).
template <typename T>
__device__ __forceinline__ bool limit_box(const FractalT<T> &f, const V3<T> point, const T detailSize,
                                          T &limitBoxDist) {
  if (!f.limits) return false;
  // MAX(a, b) = a > b ? a : b (gtk MAX macro)
  const T ax = point.x - f.amax, bx = -(point.x - f.amin);
  const T ay = point.y - f.bmax, by = -(point.y - f.bmin);
  const T az = point.z - f.cmax, bz = -(point.z - f.cmin);
  const T da = ax > bx ? ax : bx;
  const T db = ay > by ? ay : by;
  const T dc = az > bz ? az : bz;
  // dMax (src/common_math.cpp:34-43)
  limitBoxDist = (da > db) ? ((da > dc) ? da : dc) : ((db > dc) ? db : dc);
  return limitBoxDist > detailSize;
}

// CalculateDistance after the orbit (src/fractal.cpp:1291-1300, 1436-1445): the clamp at 0,
// minN, interior mode, the iteration threshold and the limit box, on the orbit's distance
// and end iteration Li. Shared by the generic and the lean orbits.
template <typename T>
__device__ __forceinline__ T distance_post(const FractalT<T> &f, T distance, const int Li, const int N, const int minN,
                                           const T detailSize, const bool normalMode, const T limitBoxDist,
                                           bool &maxIter) {
  maxIter = (Li == N);
  if (distance < T(0)) distance = T(0);
  if (Li < minN && distance < detailSize) distance = detailSize;
  if (!f.distPost) return distance;   // none of the three below: one uniform test per estimate
  if (f.interiorMode && !normalMode) {
    if (distance < T(0.5) * detailSize || Li == N) { distance = detailSize; maxIter = false; }
  } else if (f.interiorMode && normalMode) {
    if (distance < T(0.9) * detailSize) { distance = detailSize - distance; maxIter = false; }
  }
  if (f.iterThresh && Li < N) {
    if (distance < detailSize) distance = detailSize * T(1.01);
  }
  if (f.limits) {
    if (limitBoxDist < detailSize) distance = (distance > limitBoxDist) ? distance : limitBoxDist;
  }
  return distance;
}

// CalculateDistance, analytic branch (src/fractal.cpp:1245-1300, 1436-1445).
// `L` (itersOut) is left untouched when the limits box returns early, as in the reference.
template <typename T, int FORMULA>
__device__ __forceinline__ T calc_distance(const FractalT<T> &f, const V3<T> point, const T detailSize, const int N,
                                           const int minN, const bool normalMode, int &L, bool &maxIter,
                                           Counters &cnt, const T fparam) {
  if (FORMULA == 0)
    return calc_distance_runtime<T>(&f, point, detailSize, N, minN, normalMode, &L, &maxIter, &cnt.orbit, &cnt.calls,
                                    &cnt.objectOut, fparam);
  T limitBoxDist = T(0);
  if (limit_box(f, point, detailSize, limitBoxDist)) {
    maxIter = false;
    return limitBoxDist;
  }
  int Li;
  T distance;
  if constexpr (sizeof(T) == 4 && (FORMULA == 8 || FORMULA == 2)) {
    // the lean FP32 orbits where the fractal allows them (f.lean): the same distance estimate
    // without square roots and divisions in the loop (Mandelbox) or transcendentals (power-8
    // Mandelbulb)
    if (f.lean) {
      if constexpr (FORMULA == 8) distance = mandelbox_fast(f, point.x, point.y, point.z, N, Li, cnt, fparam);
      else distance = mandelbulb8_fast<0>(f, point.x, point.y, point.z, N, Li, cnt);
    } else {
      distance = compute<T, FORMULA, 0>(f, point, N, Li, cnt, fparam);
    }
  } else {
    distance = compute<T, FORMULA, 0>(f, point, N, Li, cnt, fparam);
  }
  L = Li;
  return distance_post(f, distance, Li, N, minN, detailSize, normalMode, limitBoxDist, maxIter);
}

// CalculateDistance with the lean orbit chosen at compile time: LEAN (the FP32 instantiations
// launched for FractalT::lean scenes) calls the lean orbit directly, so that the kernel holds
// no generic orbit; otherwise calc_distance.
template <typename T, int FORMULA, bool LEAN>
__device__ __forceinline__ T distance_est(const FractalT<T> &f, const V3<T> p, const T detail, const int N,
                                          const int minN, const bool normalMode, int &L, bool &maxIter,
                                          Counters &cnt, const T fparam) {
  if constexpr (LEAN && sizeof(T) == 4 && (FORMULA == 8 || FORMULA == 2)) {
    int Li;
    T distance;
    if constexpr (FORMULA == 8) distance = mandelbox_fast(f, p.x, p.y, p.z, N, Li, cnt, fparam);
    else distance = mandelbulb8_fast<0>(f, p.x, p.y, p.z, N, Li, cnt);
    L = Li;
    // the LEAN instantiations are launched for scenes without the limit box (its distance is 0
    // here); limit-box scenes take calc_distance, which runs the lean orbit after the box test
    return distance_post(f, distance, Li, N, minN, detail, normalMode, T(0), maxIter);
  } else {
    return calc_distance<T, FORMULA>(f, p, detail, N, minN, normalMode, L, maxIter, cnt, fparam);
  }
}

// Counter-hash stand-in for the march jitter Random(1000) (src/Render3D.cpp:129-133):
// a value in [0, 1000] from (seed, pixel, step) instead of a shared rand() stream.
__device__ __forceinline__ int jitter1000(uint32_t seed, uint32_t pixel, uint32_t step) {
  uint32_t h = seed ^ (pixel * 0x9E3779B1u) ^ (step * 0x85EBCA77u);
  h ^= h >> 16; h *= 0x7FEB352Du; h ^= h >> 15; h *= 0x846CA68Bu; h ^= h >> 16;
  return (int)(h % 1001u);
}

// Step-buffer view of one thread's scratch slot: record i at [i * slots + slot].
template <typename T>
struct StepBuf {
  T *step, *dist, *thr;
  T *scan;     // null unless the volumetric pass samples the record positions
  int *iters;
  int64_t slots, slot;   // record stride (thread slots x rays) and this thread's slot
  int64_t raySlots;      // thread slots: ray k of the reflection loop uses slot + k x raySlots
  __device__ __forceinline__ int64_t at(int i) const { return (int64_t)i * slots + slot; }
  __device__ __forceinline__ StepBuf ray(int k) const {
    StepBuf r = *this;
    r.slot = slot + (int64_t)k * raySlots;
    return r;
  }
};

// The rays of the reflection loop (sReflect, src/Render3D.h:41-56): the camera ray and up
// to kMaxRays - 1 reflections.
constexpr int kMaxRays = 11;
template <typename T>
struct RayRec {
  V3<double> start, view, point;
  bool found;
  int buffCount, objectType;
  double lastDist, depth, distThresh;
  T reflect;
};

// Per-pixel march state handed from the march to the shaders.
struct RayState {
  bool found;
  bool overflow;   // the march needed more step records than the slot holds
  int buffCount;
  int iters;
  double scan, step, dist, distThresh, detail;
  double point[3];
};

constexpr double kPI = 3.14159265358979323846;
// Upper bound of one shadow or AO march; the reference's loops have none, but a
// float accumulator can stop advancing, and every device loop here must end.
constexpr int kMaxSecondarySteps = 1 << 20;

// ---------------------------------------------------------------------------
// RayMarching march loop (src/Render3D.cpp:79-143) in precision T.
// ---------------------------------------------------------------------------
template <typename T, int FORMULA>
__device__ __forceinline__ void march(const ParamsT<T> &p, const V3<T> start, const V3<T> dir, const uint32_t pixel,
                                      const StepBuf<T> &sb, const int stepCap, RayState &rs, Counters &cnt,
                                      const T distThreshIn = T(0)) {
  T scan = p.viewDistanceMin;
  // *distThreshOut: 0.0 for the primary ray, the previous ray's threshold for a reflected
  // one (src/Render3D.cpp:88, 443, 461-462)
  T distThresh = distThreshIn;
  const T distThreshInit = distThreshIn;
  T dist = T(0);
  T step = p.viewDistanceMin;
  int buffCount = 0;
  bool found = false;
  int iters = 0;
  int counter = 0;
  const bool useSB = p.needVolumetric;
  const T thrScale = p.resolution * p.persp / p.quality;
  const T stepFrac = p.f.interiorMode ? T(0.8) : T(0.5);
  rs.overflow = false;
  for (int i = 0; i < kMaxMarchSteps; i++) {
    if (useSB && i >= stepCap) {
      rs.overflow = true;  // re-rendered by the overflow pass with full-length records
      return;
    }
    counter++;
    const V3<T> point = start + dir * scan;
    if (p.constantDEThreshold) {
      distThresh = p.quality;
    } else if (sizeof(T) == 8) {
      distThresh = scan * p.resolution * p.persp / p.quality + distThreshInit;
    } else {
      distThresh = scan * thrScale + distThreshInit;
    }
    if (p.perspType == 1 || p.perspType == 2) distThresh *= T(kPI);
    bool mi;
    dist = calc_distance<T, FORMULA>(p.f, point, distThresh, p.f.N, p.f.minN, false, iters, mi, cnt, fparam_of(p.f));
    if (useSB) {
      sb.dist[sb.at(i)] = dist;
      sb.thr[sb.at(i)] = distThresh;
      if (sb.iters) sb.iters[sb.at(i)] = iters;
    }
    if (dist > T(3)) dist = T(3);
    if (dist < distThresh) {
      if (dist < T(0.1) * distThresh) cnt.missed++;
      found = true;
      break;
    }
    if (useSB) {
      sb.step[sb.at(i)] = step;
      if (sb.scan) sb.scan[sb.at(i)] = scan;
    }
    step = (dist - stepFrac * distThresh) * p.DE_factor;
    if (p.jitter) step = step * (T(1) - T(jitter1000(p.jitter_seed, pixel, (uint32_t)i)) / T(10000));
    buffCount++;
    scan += step;
    if (scan > p.viewDistanceMax) break;
  }
  cnt.steps += (unsigned long long)counter;
  rs.found = found;
  rs.buffCount = buffCount;
  rs.iters = iters;
  rs.scan = (double)scan;
  rs.step = (double)step;
  rs.dist = (double)dist;
  rs.distThresh = (double)distThresh;
  rs.detail = (double)distThresh;
  const V3<T> pt = start + dir * scan;
  rs.point[0] = (double)pt.x;
  rs.point[1] = (double)pt.y;
  rs.point[2] = (double)pt.z;
}

// Binary hit refinement (src/Render3D.cpp:145-183) in FP64 (the FP64 policy; refine_fix below
// is the FP32 policy's).
// detailSize keeps the value of the last march step, as in the reference.
template <typename TP, int FORMULA>
__device__ __forceinline__ void refine(const ParamsT<TP> &p, const FractalT<double> &fd, const V3<double> start,
                                       const V3<double> dir, RayState &rs, Counters &cnt,
                                       const double distThreshInit = 0.0) {
  const double search_accuracy = 0.01 * p.quality_d;
  const double search_limit = 1.0 - search_accuracy;
  double scan = rs.scan;
  double step = rs.step * 0.5;
  double dist = rs.dist;
  double distThresh = rs.distThresh;
  V3<double> point{rs.point[0], rs.point[1], rs.point[2]};
  int iters = rs.iters;
  for (int i = 0; i < 20; i++) {
    cnt.steps++;
    if (dist < distThresh && dist > distThresh * search_limit) {
      break;
    } else {
      if (dist > distThresh) {
        scan += step;
        point = start + dir * scan;
      } else if (dist < distThresh * search_limit) {
        scan -= step;
        point = start + dir * scan;
      }
    }
    if (p.constantDEThreshold) {
      distThresh = p.quality_d;
    } else {
      distThresh = scan * p.resolution_d * p.persp_d / p.quality_d + distThreshInit;
    }
    bool mi;
    dist = calc_distance<double, FORMULA>(fd, point, rs.detail, fd.N, fd.minN, false, iters, mi, cnt, fparam_of(fd));
    step *= 0.5;
  }
  rs.scan = scan;
  rs.dist = dist;
  rs.distThresh = distThresh;
  rs.iters = iters;
  rs.point[0] = point.x;
  rs.point[1] = point.y;
  rs.point[2] = point.z;
}

// FP32 policy: the binary refinement in FP32, then, for a hit whose FP32 bisection stopped
// early with dist/thr within 1e-4 of a window edge, the FP64 re-evaluation at the FP32 result
// and the bisection iterations it has left in FP64 (the rule of the wavefront engine's polish
// stage). A bisection that used all 20 iterations keeps its FP32 depth: FP64 would have no
// iteration left to move it.
template <int FORMULA>
__device__ __forceinline__ void refine_fix(const ParamsT<float> &p, const FractalT<double> &fd, const V3<double> start,
                                           const V3<double> dir, RayState &rs, Counters &cnt,
                                           const double distThreshInit = 0.0) {
  using T = float;
  const T search_limit = T(1) - T(0.01) * p.quality;
  const T thrScale = p.resolution * p.persp / p.quality;
  const T thrInit = (T)distThreshInit;
  const V3<T> startT{(T)start.x, (T)start.y, (T)start.z}, dirT{(T)dir.x, (T)dir.y, (T)dir.z};
  const T detail = (T)rs.detail;
  T scan = (T)rs.scan;
  T step = (T)rs.step * T(0.5);
  T dist = (T)rs.dist;
  T thr = (T)rs.distThresh;
  V3<T> point = startT + dirT * scan;
  int iters = rs.iters;
  int bis = 0;
  for (; bis < 20; bis++) {
    cnt.steps++;
    if (dist < thr && dist > thr * search_limit) break;
    if (dist > thr) scan += step;
    else if (dist < thr * search_limit) scan -= step;
    point = startT + dirT * scan;
    thr = p.constantDEThreshold ? p.quality : scan * thrScale + thrInit;
    bool mi;
    dist = calc_distance<T, FORMULA>(p.f, point, detail, p.f.N, p.f.minN, false, iters, mi, cnt, fparam_of(p.f));
    step *= T(0.5);
  }
  const T q = dist / thr;
  const bool clear = (q > search_limit + T(1e-4)) && (q < T(1) - T(1e-4));
  if (!clear && bis < 20) {
    const double search_limit_d = 1.0 - 0.01 * p.quality_d;
    auto thr_of = [&](double sc) {
      return p.constantDEThreshold ? p.quality_d : sc * p.resolution_d * p.persp_d / p.quality_d + distThreshInit;
    };
    double scanD = (double)scan, stepD = (double)step;
    double thrD = thr_of(scanD);
    V3<double> pointD = start + dir * scanD;
    bool mi;
    double distD = calc_distance<double, FORMULA>(fd, pointD, rs.detail, fd.N, fd.minN, false, iters, mi, cnt,
                                                  fparam_of(fd));
    cnt.steps++;
    for (int it = bis; it < 20; it++) {
      if (distD < thrD && distD > thrD * search_limit_d) break;
      if (distD > thrD) scanD += stepD;
      else if (distD < thrD * search_limit_d) scanD -= stepD;
      pointD = start + dir * scanD;
      thrD = thr_of(scanD);
      distD = calc_distance<double, FORMULA>(fd, pointD, rs.detail, fd.N, fd.minN, false, iters, mi, cnt,
                                             fparam_of(fd));
      cnt.steps++;
      stepD *= 0.5;
    }
    rs.scan = scanD;
    rs.dist = distD;
    rs.distThresh = thrD;
    rs.point[0] = pointD.x;
    rs.point[1] = pointD.y;
    rs.point[2] = pointD.z;
  } else {
    rs.scan = (double)scan;
    rs.dist = (double)dist;
    rs.distThresh = (double)thr;
    rs.point[0] = (double)point.x;
    rs.point[1] = (double)point.y;
    rs.point[2] = (double)point.z;
  }
  rs.iters = iters;
}

// ---------------------------------------------------------------------------
// Shaders in precision T (src/shaders.cpp)
// ---------------------------------------------------------------------------

// CalculateNormals (src/shaders.cpp:675-757): forward differences of the distance (N x 5,
// minN 0), or with slow shading the average of point2 x distance over the 11^3 offsets
// point2 in [-1, 1]^3 (steps of 0.2, accumulated in double as the reference's loop does).
template <typename T, int FORMULA, bool LEAN = false>
__device__ __forceinline__ V3<T> calc_normal_fp(const ParamsT<T> &p, const V3<T> point, const T delta,
                                                const T dist_thresh, const T detail, Counters &cnt, const T fparam);

// CalculateNormals at the fractal's own parameter (a frame of a batch may carry its own:
// calc_normal_fp).
template <typename T, int FORMULA>
__device__ __forceinline__ V3<T> calc_normal(const ParamsT<T> &p, const V3<T> point, const T delta, const T dist_thresh,
                                             const T detail, Counters &cnt) {
  return calc_normal_fp<T, FORMULA>(p, point, delta, dist_thresh, detail, cnt, fparam_of(p.f));
}

template <typename T, int FORMULA, bool LEAN>
__device__ __forceinline__ V3<T> calc_normal_fp(const ParamsT<T> &p, const V3<T> point, const T delta,
                                                const T dist_thresh, const T detail, Counters &cnt, const T fparam) {
  T dn = delta * p.smoothness;
  if (p.f.interiorMode) dn = dist_thresh * p.quality * T(0.2) * p.smoothness;
  int L;
  bool mi;
  const int N5 = p.f.N5;
  V3<T> n;
  if (!p.slowShading) {
    const T s1 = distance_est<T, FORMULA, LEAN>(p.f, point, detail, N5, 0, true, L, mi, cnt, fparam);
    const T s2 = distance_est<T, FORMULA, LEAN>(p.f, V3<T>{point.x + dn, point.y + T(0), point.z + T(0)}, detail, N5, 0,
                                           true, L, mi, cnt, fparam);
    const T s3 = distance_est<T, FORMULA, LEAN>(p.f, V3<T>{point.x + T(0), point.y + dn, point.z + T(0)}, detail, N5, 0,
                                           true, L, mi, cnt, fparam);
    const T s4 = distance_est<T, FORMULA, LEAN>(p.f, V3<T>{point.x + T(0), point.y + T(0), point.z + dn}, detail, N5, 0,
                                           true, L, mi, cnt, fparam);
    n = V3<T>{s2 - s1, s3 - s1, s4 - s1};
  } else {
    n = V3<T>{T(0), T(0), T(0)};
    for (double px = -1.0; px <= 1.0; px += 0.2) {
      for (double py = -1.0; py <= 1.0; py += 0.2) {
        for (double pz = -1.0; pz <= 1.0; pz += 0.2) {
          const V3<T> p2{(T)px, (T)py, (T)pz};
          const T dist = distance_est<T, FORMULA, LEAN>(p.f, point + p2 * dn, detail, N5, p.f.minN, true, L, mi, cnt,
                                                   fparam);
          n = n + p2 * dist;
        }
      }
    }
  }
  if (n.x == T(0) && n.y == T(0) && n.z == T(0)) {
    n.x = T(1);
  } else {
    n = normalize3(n);
  }
  return n;
}

// IterOpacity (src/shaders.cpp:1210-1218)
template <typename T>
__device__ __forceinline__ T iter_opacity(const T step, const T iters, const T maxN, const T trim, const T opacitySp) {
  T opacity = (iters - trim) / maxN;
  if (opacity < T(0)) opacity = T(0);
  opacity *= opacity;
  opacity *= step * opacitySp;
  if (opacity > T(1)) opacity = T(1);
  return opacity;
}

// The threshold a secondary ray compares against, held in a float as the reference does:
// with iteration fog or volumetric lights the one of the sample's own distance from the
// eye, else the hit's.
template <typename T>
__device__ __forceinline__ T secondary_thresh(const ParamsT<T> &p, const V3<T> point2, const V3<T> eye,
                                              const T dist_thresh) {
  float t;
  if (p.iterFog || p.volLightAny) {
    if (!p.constantDEThreshold) t = (float)(length3(point2 - eye) * p.resolution * p.persp / p.quality);
    else t = (float)p.quality;
  } else {
    t = (float)dist_thresh;
  }
  return (T)t;
}

// MainShadow (src/shaders.cpp:480-570). `detail` is the shared detailSize state (left at the
// last float threshold), `itersOut` the shared iteration count. With iteration fog or
// volumetric lights the march steps at DE factor 1, each sample compares against its own
// eye-distance threshold and iteration fog absorbs along the way.
template <typename T, int FORMULA>
__device__ __forceinline__ T main_shadow(const ParamsT<T> &p, const V3<T> point, const T dist_thresh, const T delta,
                                         const V3<T> eye, T &detail, int &itersOut, const FrameIO &io,
                                         Counters &cnt) {
  T factor = delta / p.resolution;
  if (!p.penetrating) factor = p.viewDistanceMax;
  T dist = dist_thresh;
  detail = dist_thresh;
  const T DE_factor = (p.iterFog || p.volLightAny) ? T(1) : p.DE_factor;
  T start = dist_thresh;
  if (p.f.interiorMode) start = dist_thresh * DE_factor;
  T shadowTemp = T(1);
  const T softRange = p.softRange;
  T maxSoft = T(0);
  const bool bSoft = p.softShadow != 0;
  const V3<T> lv{p.lightVect[0], p.lightVect[1], p.lightVect[2]};
  int guard = 0;
  for (T i = start; i < factor; i += dist * DE_factor) {
    const V3<T> point2 = point + lv * i;
    const T thr = secondary_thresh(p, point2, eye, dist_thresh);
    detail = thr;
    bool mi;
    dist = calc_distance<T, FORMULA>(p.f, point2, detail, p.f.N, p.f.minN, false, itersOut, mi, cnt, fparam_of(p.f));
    if (bSoft) {
      T angle = (dist - thr) / i;
      if (angle < T(0)) angle = T(0);
      if (dist < thr) angle = T(0);
      T softShadow = (T(1) - angle / softRange);
      if (p.penetrating) softShadow *= (factor - i) / factor;
      if (softShadow < T(0)) softShadow = T(0);
      if (softShadow > maxSoft) maxSoft = softShadow;
    }
    if (p.iterFog) {
      const T opacity = iter_opacity(dist * DE_factor, T(itersOut), T(p.f.N), p.iterFogOpacityTrim, p.iterFogOpacity);
      shadowTemp -= opacity * (factor - i) / factor;
    }
    if (dist < thr || shadowTemp < T(0)) {
      shadowTemp -= (factor - i) / factor;
      if (!p.penetrating) shadowTemp = T(0);
      if (shadowTemp < T(0)) shadowTemp = T(0);
      break;
    }
    // hard bound: in FP32 `i += dist` could stop advancing when dist falls below ulp(i)
    if (++guard >= kMaxSecondarySteps) break;
    if ((guard & 1023) == 0 && deadline_passed(io)) {
      atomicExch(io.error_flag, 1);
      break;
    }
  }
  return bSoft ? (T(1) - maxSoft) : shadowTemp;
}

// FastAmbientOcclusion2 (src/shaders.cpp:585-605)
template <typename T, int FORMULA>
__device__ __forceinline__ T fast_ao(const ParamsT<T> &p, const V3<T> point, const V3<T> normal, const T dist_thresh,
                                     const T detail, Counters &cnt) {
  const T delta = dist_thresh;
  T aoTemp = T(0);
  const int q2 = p.aoQuality * p.aoQuality;
  for (int i = 1; i < q2; i++) {
    const T scan = T(i * i) * delta;
    const V3<T> pt = point + normal * scan;
    int L;
    bool mi;
    const T dist = calc_distance<T, FORMULA>(p.f, pt, detail, p.f.N, p.f.minN, false, L, mi, cnt, fparam_of(p.f));
    // 1.0 / pow(2.0, i) is exact for integral i
    aoTemp += T(1) / T(ldexp(1.0, i)) * (scan - p.fastAoTune * dist) / dist_thresh;
  }
  T ao = T(1) - T(0.2) * aoTemp;
  if (ao < T(0)) ao = T(0);
  return ao;
}

// AmbientOcclusion, ray-traced (src/shaders.cpp:607-673), white light map: every direction
// weighs (255, 255, 255). Iteration fog and volumetric lights change the threshold and add
// absorption as in MainShadow.
template <typename T, int FORMULA>
__device__ __forceinline__ V3<T> ray_ao(const ParamsT<T> &p, const V3<T> point, const T delta, const T dist_thresh,
                                        const T lastDist, const T detail, const V3<T> eye, int &itersOut,
                                        Counters &cnt) {
  const T start_dist = delta;
  const T end_dist = delta / p.resolution;
  V3<T> AO{T(0), T(0), T(0)};
  for (int v = 0; v < p.aoCount; v++) {
    const V3<T> dir{__ldg(&p.aoVec[3 * v + 0]), __ldg(&p.aoVec[3 * v + 1]), __ldg(&p.aoVec[3 * v + 2])};
    T dist = lastDist;
    T shadowTemp = T(1);
    int guard = 0;
    for (T r = start_dist; r < end_dist && guard < kMaxSecondarySteps; r += dist * T(2), guard++) {
      const V3<T> point2 = point + dir * r;
      bool mi;
      dist = calc_distance<T, FORMULA>(p.f, point2, detail, p.f.N, p.f.minN, false, itersOut, mi, cnt, fparam_of(p.f));
      if (p.iterFog) {
        const T opacity = iter_opacity(dist * T(2), T(itersOut), T(p.f.N), p.iterFogOpacityTrim, p.iterFogOpacity);
        shadowTemp -= opacity * (end_dist - r) / end_dist;
      }
      const T thr = secondary_thresh(p, point2, eye, dist_thresh);
      if (dist < thr || mi || shadowTemp < T(0)) {
        shadowTemp -= (end_dist - r) / end_dist;
        if (shadowTemp < T(0)) shadowTemp = T(0);
        break;
      }
    }
    AO.x += shadowTemp * p.aoWeight[0];
    AO.y += shadowTemp * p.aoWeight[1];
    AO.z += shadowTemp * p.aoWeight[2];
  }
  const T div = T(p.aoCount) * T(256);
  AO.x /= div;
  AO.y /= div;
  AO.z /= div;
  return AO;
}

// EnvMapping (src/shaders.cpp:785-811) on the default texture (src/texture.cpp:67-116): a
// white 100 x 100 bitmap, bilinearly interpolated, black in its last row. Evaluated in
// double under both policies: the 8-bit truncation of the interpolated texel and the black
// row turn last-bit differences of the coordinates into visible steps.
__device__ __forceinline__ double env_mapping(const V3<double> normal, const V3<double> view) {
  using T = double;
  const T d = -dot3(view, normal);
  const V3<T> reflect = normal * T(2) * d + view;
  const T alfaTexture = m_atan2(reflect.y, reflect.x) + T(kPI);
  T betaTexture = m_atan2(reflect.z, m_sqrt(reflect.x * reflect.x + reflect.y * reflect.y));
  const T texWidth = T(100), texHeight = T(100);
  if (betaTexture > T(0.5) * T(kPI)) betaTexture = T(0.5) * T(kPI) - betaTexture;
  if (betaTexture < T(-0.5) * T(kPI)) betaTexture = T(-0.5) * T(kPI) + betaTexture;
  T dtx = (alfaTexture / (T(2) * T(kPI))) * texWidth + texWidth * T(8.25);
  T dty = (betaTexture / T(kPI) + T(0.5)) * texHeight + texHeight * T(8);
  dtx = fmod(dtx, texWidth);
  dty = fmod(dty, texHeight);
  if (dtx < T(0)) dtx = T(0);
  if (dty < T(0)) dty = T(0);
  if (!(dtx >= T(0) && dtx < texWidth && dty >= T(0) && dty < texHeight - T(1))) return T(0);
  const T rx = dtx - T((int)dtx), ry = dty - T((int)dty);
  const T v = T(255) * (T(1) - rx) * (T(1) - ry) + T(255) * (rx) * (T(1) - ry) + T(255) * (T(1) - rx) * ry +
              T(255) * (rx * ry);
  return T((unsigned char)(int)v) / T(256);
}

// AuxShadow (src/shaders.cpp:1069-1132): march from the point towards a light at `distance`,
// starting and first stepping at delta. `detail` is the shared detailSize (not changed here);
// `itersOut` the shared iteration count, which a limits-box early return leaves as it was.
template <typename T, int FORMULA>
__device__ __forceinline__ T aux_shadow(const ParamsT<T> &p, const V3<T> point, const T distance, const V3<T> lightVector,
                                        const T delta, const T dist_thresh, const V3<T> eye, const T detail,
                                        int &itersOut, Counters &cnt) {
  T dist = delta;
  T shadowTemp = T(1);
  const T DE_factor = (p.iterFog || p.volLightAny) ? T(1) : p.DE_factor;
  int guard = 0;
  for (T i = delta; i < distance; i += dist * DE_factor) {
    const V3<T> point2 = point + lightVector * i;
    bool mi;
    dist = calc_distance<T, FORMULA>(p.f, point2, detail, p.f.N, p.f.minN, false, itersOut, mi, cnt, fparam_of(p.f));
    T opacity = T(0);
    if (p.iterFog)
      opacity = iter_opacity(dist * DE_factor, T(itersOut), T(p.f.N), p.iterFogOpacityTrim, p.iterFogOpacity);
    shadowTemp -= opacity * (distance - i) / distance;
    const T thr = secondary_thresh(p, point2, eye, dist_thresh);
    if (dist < thr || mi || shadowTemp < T(0)) {
      if (p.penetrating) {
        shadowTemp -= (distance - i) / distance;
        if (shadowTemp < T(0)) shadowTemp = T(0);
      } else {
        shadowTemp = T(0);
      }
      break;
    }
    // hard bound: in FP32 `i += dist` could stop advancing when dist falls below ulp(i)
    if (++guard >= kMaxSecondarySteps) break;
  }
  return shadowTemp;
}

// AuxLightsShader / LightShading (src/shaders.cpp:997-1067): Lambert and Blinn terms of each
// auxiliary light, 1 / r^2 falloff shared among `numberOfLights`, shadowed by AuxShadow when
// either term is above 0.01 (and zero when shadows are on and neither is).
template <typename T, int FORMULA>
__device__ __forceinline__ void aux_lights(const ParamsT<T> &p, const V3<T> point, const V3<T> normal, const V3<T> view,
                                           const T delta, const T dist_thresh, const V3<T> eye, const T detail,
                                           int &itersOut, Counters &cnt, T shadeSum[3], T specSum[3]) {
  shadeSum[0] = shadeSum[1] = shadeSum[2] = T(0);
  specSum[0] = specSum[1] = specSum[2] = T(0);
  const int number = p.numberOfLights;
  for (int i = 0; i < number; i++) {
    const LightT<T> L = p.lights[i];
    if (!(i < p.auxLightNumber || L.enabled)) continue;
    const V3<T> d = V3<T>{L.pos[0], L.pos[1], L.pos[2]} - point;
    const T distance = length3(d);
    const V3<T> lightVector = normalize3(d);
    const T intensity = p.auxLightIntensity * T(100) * L.intensity / (distance * distance) / T(number);
    T shade = dot3(normal, lightVector);
    if (shade < T(0)) shade = T(0);
    shade = shade * intensity;
    if (shade > T(500)) shade = T(500);
    const V3<T> half = normalize3(lightVector - view);
    T shade2 = dot3(normal, half);
    if (shade2 < T(0)) shade2 = T(0);
    shade2 = m_pow(shade2, T(30)) * T(1);
    shade2 *= intensity * p.specular;
    if (shade2 > T(15)) shade2 = T(15);
    if ((shade > T(0.01) || shade2 > T(0.01)) && p.shadow) {
      const T light = aux_shadow<T, FORMULA>(p, point, distance, lightVector, delta, dist_thresh, eye, detail, itersOut,
                                             cnt);
      shade *= light;
      shade2 *= light;
    } else if (p.shadow) {
      shade = T(0);
      shade2 = T(0);
    }
    for (int c = 0; c < 3; c++) {
      shadeSum[c] += shade * T(L.colour[c]) / T(65536);
      specSum[c] += shade2 * T(L.colour[c]) / T(65536);
    }
  }
}

// IndexToColour (src/shaders.cpp:1273-1305) -> sRGB in 8-bit range
template <typename T>
__device__ __forceinline__ void index_to_colour(const ParamsT<T> &p, int index, int rgb[3]) {
  if (index < 0) {
    rgb[0] = p.palette[255][0]; rgb[1] = p.palette[255][1]; rgb[2] = p.palette[255][2];
    return;
  }
  index = index % (255 * 256);
  const int kol = index / 256;
  rgb[0] = rgb[1] = rgb[2] = 255;
  if (kol < 255) {
    const int delta = index % 256;
    for (int c = 0; c < 3; c++) {
      const double c1 = p.palette[kol][c];
      const double c2 = p.palette[kol + 1][c];
      const double k = (c2 - c1) / 256.0;
      rgb[c] = (int)(c1 + (k * delta));
    }
  }
}

// SurfaceColour for the fractal object (src/shaders.cpp:850-879)
template <typename T, int FORMULA>
__device__ __forceinline__ V3<T> surface_colour(const ParamsT<T> &p, const V3<T> point, Counters &cnt,
                                                const T fparam, const int objectType = kObjFractal) {
  if (objectType != kObjFractal) {  // primitive colours (src/shaders.cpp:880-922)
    const int *c = p.primColour[objectType - 1];
    return V3<T>{T(c[0]) / T(65536), T(c[1]) / T(65536), T(c[2]) / T(65536)};
  }
  int L;
  T c;
  if constexpr (sizeof(T) == 4 && FORMULA == 2) {
    // the power-8 Mandelbulb's colouring orbit without transcendentals (f.lean)
    c = p.f.lean ? mandelbulb8_fast<1>(p.f, point.x, point.y, point.z, p.f.N10, L, cnt)
                 : compute<T, FORMULA, 1>(p.f, point, p.f.N10, L, cnt, fparam);
  } else {
    c = compute<T, FORMULA, 1>(p.f, point, p.f.N10, L, cnt, fparam);
  }
  int nrCol = to_i32_x86((double)m_floor(c));
  // abs(nrCol) % (248 * 256) with the magnitude taken as unsigned, as the reference
  // binary computes it: an out-of-range conversion (INT_MIN) gives 2^31 % 63488 = 2048.
  const unsigned mag = nrCol < 0 ? 0u - (unsigned)nrCol : (unsigned)nrCol;
  nrCol = (int)(mag % (248u * 256u));
  int rgb[3] = {256, 256, 256};
  if (p.coloring) {
    int color_number;
    if (nrCol >= 248 * 256) {
      color_number = nrCol;
    } else {
      color_number = to_i32_x86((double)((T)nrCol * p.coloringSpeed + T(256) * p.paletteOffset)) % 65536;
    }
    index_to_colour(p, color_number, rgb);
  }
  return V3<T>{T(rgb[0]) / T(256), T(rgb[1]) / T(256), T(rgb[2]) / T(256)};
}

// BackgroundShader, gradient branch (src/shaders.cpp:154-182)
template <typename T>
__device__ __forceinline__ V3<T> background(const ParamsT<T> &p, const V3<T> view) {
  const V3<T> vec{T(0), T(0), T(-1)};
  T grad = (dot3(view, vec) + T(1));
  int px[3];
  if (grad < T(1)) {
    const T Ngrad = T(1) - grad;
    for (int c = 0; c < 3; c++) px[c] = to_u16_x86((double)(T(p.bg3[c]) * Ngrad + T(p.bg2[c]) * grad));
  } else {
    grad = grad - T(1);
    const T Ngrad = T(1) - grad;
    for (int c = 0; c < 3; c++) px[c] = to_u16_x86((double)(T(p.bg2[c]) * Ngrad + T(p.bg1[c]) * grad));
  }
  return V3<T>{T(px[0]) / T(65536), T(px[1]) / T(65536), T(px[2]) / T(65536)};
}

// VolumetricShader (src/shaders.cpp:185-478): glow, visible aux lights, fake lights,
// volumetric lights, post fog, volumetric fog and iteration fog over the primary step
// buffer, far to near, merging steps shorter than distThresh * quality. The volumetric
// lights and the iteration fog trace MainShadow / AuxShadow / AmbientOcclusion from the
// step positions with the pixel's delta and last distance; `detail` and `itersOut` carry
// the shared CalculateDistance state through them.
template <typename T, int FORMULA>
__device__ __forceinline__ void volumetric(const ParamsT<T> &p, const StepBuf<T> &sb, const int stepCount,
                                           const T depth, const V3<T> rayStart, const V3<T> eye, const V3<T> view,
                                           const T delta,
                                           const T lastDist, T &detail, int &itersOut, const FrameIO &io,
                                           Counters &cnt, T out[4], float &totalOpacityOut, bool &opacitySet) {
  float totalOpacity = 0.0f;
  const T glow = T(stepCount) * p.glowIntensity / T(512) * p.DE_factor;
  T glowN = T(1) - glow;
  if (glowN < T(0)) glowN = T(0);
  const T glowR = (T(p.glow1[0]) * glowN + T(p.glow2[0]) * glow) / T(65536);
  const T glowG = (T(p.glow1[1]) * glowN + T(p.glow2[1]) * glow) / T(65536);
  const T glowB = (T(p.glow1[2]) * glowN + T(p.glow2[2]) * glow) / T(65536);
  const T colourThresh = p.fogC1Dist;
  const T colourThresh2 = p.fogC2Dist;
  const T fogReduce = p.fogDistFactor;
  const T fogIntensity = p.fogDensity;
  T totalStep = T(0);
  for (int index = stepCount - 1; index > 0; index--) {
    T step = sb.step[sb.at(index)];
    const T distance = sb.dist[sb.at(index)];
    const T dist_thresh = sb.thr[sb.at(index)];
    totalStep += step;
    if (totalStep < dist_thresh * p.quality) continue;
    step = totalStep;
    totalStep = T(0);
    // glow
    const T glowOpacity = glow * step / depth;
    out[0] = glowOpacity * glowR + (T(1) - glowOpacity) * out[0];
    out[1] = glowOpacity * glowG + (T(1) - glowOpacity) * out[1];
    out[2] = glowOpacity * glowB + (T(1) - glowOpacity) * out[2];
    out[3] += glowOpacity;
    // visible auxiliary lights (src/shaders.cpp:242-296): a bell-shaped glow around each
    // light, sampled in up to 50 sub-steps near the closest one
    if (p.auxLightVisibility > T(0) && p.numberOfLights > 0) {
      const V3<T> point = rayStart + view * sb.scan[sb.at(index)];
      T lowestLightSize = T(1e10);
      T lowestLightDist = T(1e10);
      for (int i = 0; i < p.numberOfLights; ++i) {
        const LightT<T> L = p.lights[i];
        if (!(i < p.auxLightNumber || L.enabled)) continue;
        const T lightDist = length3(point - V3<T>{L.pos[0], L.pos[1], L.pos[2]});
        const T lightSize = L.intensity * p.auxLightIntensity * p.auxLightVisibility;
        const T r2 = lightDist / lightSize;
        if (r2 < lowestLightSize) {
          lowestLightSize = r2;
          lowestLightDist = lightDist;
        }
      }
      int smallSteps = to_i32_x86((double)(T(10) * step / (lowestLightDist + T(1.0e-20))));
      if (smallSteps > 50) smallSteps = 50;
      int smallStep_start = 0, smallStep_end = 1;
      T step2 = step;
      if (smallSteps > 0) {
        smallStep_start = 1;
        smallStep_end = smallSteps + 1;
        step2 = step / (T(smallSteps) + T(1));
      }
      for (int smallStep = smallStep_start; smallStep < smallStep_end; smallStep++) {
        const V3<T> point2 = point - view * step2 * T(smallStep);
        for (int i = 0; i < p.numberOfLights; ++i) {
          const LightT<T> L = p.lights[i];
          if (!(i < p.auxLightNumber || L.enabled)) continue;
          const T lightDist = length3(point2 - V3<T>{L.pos[0], L.pos[1], L.pos[2]});
          const T lightSize = L.intensity * p.auxLightIntensity * p.auxLightVisibility;
          T r2 = lightDist / lightSize;
          if (r2 > T(1)) r2 = T(1);
          const T bellFunction = (m_cos(r2 * T(kPI)) + T(1)) / (r2 * r2 + T(0.02)) * T(0.3);
          const T lightDensity = step2 * bellFunction / lightSize;
          out[0] += lightDensity * T(L.colour[0]) / T(65536);
          out[1] += lightDensity * T(L.colour[1]) / T(65536);
          out[2] += lightDensity * T(L.colour[2]) / T(65536);
          out[3] += lightDensity;
        }
      }
    }
    // fake lights (orbit trap, src/shaders.cpp:298-307)
    if (p.fakeLights) {
      const V3<T> point = rayStart + view * sb.scan[sb.at(index)];
      int L;
      Counters c2{0, 0, 0, 0};
      T r = compute<T, FORMULA, 5>(p.f, point, p.f.N, L, c2, fparam_of(p.f));
      cnt.orbit += c2.orbit;
      cnt.calls += c2.calls;
      r = m_sqrt(T(1.0f) / (r + T(1.0e-30f)));
      const T fakeLight = T(1) / (m_pow(r, T(10) / p.fakeLightsVisibilitySize) *
                                      m_pow(T(10), T(10) / p.fakeLightsVisibilitySize) + T(1e-100));
      out[0] += fakeLight * step * p.fakeLightsVisibility;
      out[1] += fakeLight * step * p.fakeLightsVisibility;
      out[2] += fakeLight * step * p.fakeLightsVisibility;
      out[3] += fakeLight * step * p.fakeLightsVisibility;
    }
    // volumetric lights with shadows in fog (src/shaders.cpp:309-343)
    if (p.volLightAny) {
      const V3<T> point = rayStart + view * sb.scan[sb.at(index)];
      const T thrStep = sb.thr[sb.at(index)];
      for (int i = 0; i < 5; i++) {
        if (i == 0 && p.volLightEnabled[0]) {
          const T sh = main_shadow<T, FORMULA>(p, point, thrStep, delta, eye, detail, itersOut, io, cnt);
          out[0] += sh * step * p.volLightIntensity[0] * T(p.mainLightColour[0]) / T(65536);
          out[1] += sh * step * p.volLightIntensity[0] * T(p.mainLightColour[1]) / T(65536);
          out[2] += sh * step * p.volLightIntensity[0] * T(p.mainLightColour[2]) / T(65536);
          out[3] += (sh + sh + sh) / T(3) * step * p.volLightIntensity[0];
        }
        if (i > 0 && p.numberOfLights > 0 && p.lights[i - 1].enabled && p.volLightEnabled[i]) {
          const LightT<T> L = p.lights[i - 1];
          const V3<T> d = V3<T>{L.pos[0], L.pos[1], L.pos[2]} - point;
          const T distance = length3(d);
          const T distance2 = distance * distance;
          const V3<T> lv = normalize3(d);
          const T light = aux_shadow<T, FORMULA>(p, point, distance, lv, delta, thrStep, eye, detail, itersOut, cnt);
          out[0] += light * T(L.colour[0]) / T(65536) * p.volLightIntensity[i] * step / distance2;
          out[1] += light * T(L.colour[1]) / T(65536) * p.volLightIntensity[i] * step / distance2;
          out[2] += light * T(L.colour[2]) / T(65536) * p.volLightIntensity[i] * step / distance2;
          out[3] += light * p.volLightIntensity[i] * step / distance2;
        }
      }
    }
    // basic fog
    if (p.postFog) {
      T fogDensity = step / p.fogVisibility;
      if (fogDensity > T(1)) fogDensity = T(1);
      out[0] = fogDensity * T(p.fogColor[0]) / T(65536) + (T(1) - fogDensity) * out[0];
      out[1] = fogDensity * T(p.fogColor[1]) / T(65536) + (T(1) - fogDensity) * out[1];
      out[2] = fogDensity * T(p.fogColor[2]) / T(65536) + (T(1) - fogDensity) * out[2];
      totalOpacity = (float)(fogDensity + (T(1) - fogDensity) * (T)totalOpacity);
      out[3] = fogDensity + (T(1) - fogDensity) * out[3];
    }
    // volumetric fog
    if (fogIntensity > T(0)) {
      const T densityTemp = (step * fogReduce) / (distance * distance + fogReduce * fogReduce);
      T k = distance / colourThresh;
      if (k > T(1)) k = T(1);
      T kn = T(1) - k;
      T fr = (T(p.fogCol1[0]) * kn + T(p.fogCol2[0]) * k);
      T fg = (T(p.fogCol1[1]) * kn + T(p.fogCol2[1]) * k);
      T fb = (T(p.fogCol1[2]) * kn + T(p.fogCol2[2]) * k);
      T k2 = distance / colourThresh2 * k;
      if (k2 > T(1)) k2 = T(1);
      kn = T(1) - k2;
      fr = (fr * kn + T(p.fogCol3[0]) * k2);
      fg = (fg * kn + T(p.fogCol3[1]) * k2);
      fb = (fb * kn + T(p.fogCol3[2]) * k2);
      T fogDensity = T(0.3) * fogIntensity * densityTemp / (T(1) + fogIntensity * densityTemp);
      if (fogDensity > T(1)) fogDensity = T(1);
      out[0] = fogDensity * fr / T(65536) + (T(1) - fogDensity) * out[0];
      out[1] = fogDensity * fg / T(65536) + (T(1) - fogDensity) * out[1];
      out[2] = fogDensity * fb / T(65536) + (T(1) - fogDensity) * out[2];
      totalOpacity = (float)(fogDensity + (T(1) - fogDensity) * (T)totalOpacity);
      out[3] = fogDensity + (T(1) - fogDensity) * out[3];
    }
    // iteration fog (src/shaders.cpp:385-466): the fog colour by the record's iteration
    // count, lit by the main light and the predefined lights (shadowed) and by ray AO
    if (p.iterFog) {
      const int L = sb.iters[sb.at(index)];
      const T N = T(p.f.N);
      T opacity = iter_opacity(step, T(L), N, p.iterFogOpacityTrim, p.iterFogOpacity);
      if (opacity > T(0)) {
        const V3<T> point = rayStart + view * sb.scan[sb.at(index)];
        const T thrStep = sb.thr[sb.at(index)];
        const T iterFactor = T(2) * (T(L) - p.iterFogOpacityTrim) / (N - p.iterFogOpacityTrim);
        T k = iterFactor;
        if (k > T(1)) k = T(1);
        if (k < T(0)) k = T(0);
        T kn = T(1) - k;
        T fogCol[3];
        for (int c = 0; c < 3; c++) fogCol[c] = (T(p.fogCol1[c]) * kn + T(p.fogCol2[c]) * k);
        T k2 = iterFactor - T(1);
        if (k2 < T(0)) k2 = T(0);
        if (k2 > T(1)) k2 = T(1);
        kn = T(1) - k2;
        for (int c = 0; c < 3; c++) fogCol[c] = (fogCol[c] * kn + T(p.fogCol3[c]) * k2);
        T newColour[3] = {T(0), T(0), T(0)};
        for (int i = 0; i < 5; i++) {
          if (i == 0) {
            if (p.mainLightIntensity * p.directLight > T(0)) {
              const T sh = main_shadow<T, FORMULA>(p, point, thrStep, delta, eye, detail, itersOut, io, cnt);
              for (int c = 0; c < 3; c++)
                newColour[c] += sh * T(p.mainLightColour[c]) / T(65536) * p.mainLightIntensity * p.directLight;
            }
          }
          if (i > 0 && p.numberOfLights > 0 && p.lights[i - 1].enabled) {
            const LightT<T> Lt = p.lights[i - 1];
            const V3<T> d = V3<T>{Lt.pos[0], Lt.pos[1], Lt.pos[2]} - point;
            const T distance = length3(d);
            const T distance2 = distance * distance;
            const V3<T> lv = normalize3(d);
            const T light = aux_shadow<T, FORMULA>(p, point, distance, lv, delta, thrStep, eye, detail, itersOut, cnt);
            const T intensity = Lt.intensity * T(100);
            for (int c = 0; c < 3; c++) newColour[c] += light * T(Lt.colour[c]) / T(65536) / distance2 * intensity;
          }
        }
        if (p.ao && !p.fastAO) {
          const V3<T> AO = ray_ao<T, FORMULA>(p, point, delta, thrStep, lastDist, detail, eye, itersOut, cnt);
          newColour[0] += AO.x * p.globalIlum;
          newColour[1] += AO.y * p.globalIlum;
          newColour[2] += AO.z * p.globalIlum;
        }
        if (opacity > T(1)) opacity = T(1);
        for (int c = 0; c < 3; c++)
          out[c] = out[c] * (T(1) - opacity) + newColour[c] * opacity * fogCol[c] / T(65536);
        totalOpacity = (float)(opacity + (T(1) - opacity) * (T)totalOpacity);
        out[3] = opacity + (T(1) - opacity) * out[3];
      }
    }
    if (totalOpacity > 1.0f) totalOpacity = 1.0f;
    if (out[3] > T(1)) out[3] = T(1);
    totalOpacityOut = totalOpacity;
    opacitySet = true;
  }
}

// ObjectShader (src/shaders.cpp:21-112) at a hit: normal, main light with shadow and
// specular, surface colour, AO, environment map, aux and fake lights. Writes the object and
// specular terms and the surface colour.
template <typename T, int FORMULA>
__device__ __forceinline__ void object_shader(const ParamsT<T> &p, const V3<T> point, const V3<T> viewT,
                                              const V3<double> viewD, const V3<T> eye, const T dist_thresh,
                                              const T delta, const T lastDist, const int objectType, T &detail,
                                              int &itersOut, const FrameIO &io, Counters &cnt, T obj[3], T specOut[3],
                                              V3<T> &objColour) {
  const V3<T> n = calc_normal<T, FORMULA>(p, point, delta, dist_thresh, detail, cnt);
  const V3<T> lv{p.lightVect[0], p.lightVect[1], p.lightVect[2]};
  T shade = dot3(n, lv);
  if (shade < T(0)) shade = T(0);
  const T shadeV = p.directLight * ((T(1) - p.shading) + p.shading * shade);
  T shadow = T(1);
  if (p.shadow) shadow = main_shadow<T, FORMULA>(p, point, dist_thresh, delta, eye, detail, itersOut, io, cnt);
  // MainSpecular (src/shaders.cpp:770-783)
  V3<T> half = normalize3(lv - viewT);
  T shade2 = dot3(n, half);
  if (shade2 < T(0)) shade2 = T(0);
  shade2 = m_pow(shade2, T(30)) * T(1);
  if (shade2 > T(15)) shade2 = T(15);
  const T spec = shade2 * p.specular;
  const V3<T> colour = surface_colour<T, FORMULA>(p, point, cnt, fparam_of(p.f), objectType);
  objColour = colour;
  V3<T> ambient{T(0), T(0), T(0)};
  if (p.ao) {
    if (p.fastAO) {
      const T a = fast_ao<T, FORMULA>(p, point, n, dist_thresh, detail, cnt);
      ambient = {a, a, a};
    } else {
      ambient = ray_ao<T, FORMULA>(p, point, delta, dist_thresh, lastDist, detail, eye, itersOut, cnt);
    }
  }
  const V3<T> ambient2{ambient.x * p.globalIlum, ambient.y * p.globalIlum, ambient.z * p.globalIlum};
  // environment mapping
  const T env = (p.envMapping ? (T)env_mapping(V3<double>{(double)n.x, (double)n.y, (double)n.z}, viewD) : T(0)) *
                p.reflect;
  // auxiliary lights
  T aux[3] = {T(0), T(0), T(0)}, auxSpec[3] = {T(0), T(0), T(0)};
  if (p.numberOfLights > 0)
    aux_lights<T, FORMULA>(p, point, n, viewT, delta, dist_thresh, eye, detail, itersOut, cnt, aux, auxSpec);
  // fake (orbit trap) lights (FakeLights, src/shaders.cpp:1225-1271)
  T fake = T(0), fakeSpec = T(0);
  if (p.fakeLights) {
    const T dl = dist_thresh * p.smoothness;
    int L;
    const T rr = compute<T, FORMULA, 5>(p.f, point, p.f.N, L, cnt, fparam_of(p.f));
    const T fakeLight = p.fakeLightsIntensity / rr;
    const T r = T(1) / (rr + T(1e-30));
    const T rx = T(1) / (compute<T, FORMULA, 5>(p.f, V3<T>{point.x + dl, point.y + T(0), point.z + T(0)}, p.f.N, L,
                                                 cnt, fparam_of(p.f)) + T(1e-30));
    const T ry = T(1) / (compute<T, FORMULA, 5>(p.f, V3<T>{point.x + T(0), point.y + dl, point.z + T(0)}, p.f.N, L,
                                                 cnt, fparam_of(p.f)) + T(1e-30));
    const T rz = T(1) / (compute<T, FORMULA, 5>(p.f, V3<T>{point.x + T(0), point.y + T(0), point.z + dl}, p.f.N, L,
                                                 cnt, fparam_of(p.f)) + T(1e-30));
    V3<T> fln{r - rx, r - ry, r - rz};
    if (!(fln.x == T(0) && fln.y == T(0) && fln.z == T(0))) fln = normalize3(fln);
    T fakeLight2 = fakeLight * dot3(n, fln);
    if (fakeLight2 < T(0)) fakeLight2 = T(0);
    fake = fakeLight2;
    const V3<T> fh = normalize3(fln - viewT);
    T fs = dot3(n, fh);
    if (fs < T(0)) fs = T(0);
    fs = m_pow(fs, T(30)) * fakeLight;
    if (fs > T(15)) fs = T(15);
    fakeSpec = fs;
  }
  const T amb[3] = {ambient.x, ambient.y, ambient.z};
  const T amb2[3] = {ambient2.x, ambient2.y, ambient2.z};
  const T col[3] = {colour.x, colour.y, colour.z};
  for (int c = 0; c < 3; c++) {
    T o = env * amb[c] + (amb2[c] + p.mainLight[c] * shadeV * shadow) * col[c];
    o += (aux[c] + fake) * col[c];
    obj[c] = o;
    specOut[c] = auxSpec[c] + fakeSpec + p.mainLight[c] * spec * shadow;
  }
}

// ---------------------------------------------------------------------------
// One pixel: MainThread pixel body (src/Render3D.cpp:389-589) with its reflection loop.
// ---------------------------------------------------------------------------
template <typename T, int FORMULA>
__device__ __forceinline__ void render_pixel(const ParamsT<T> &p, const FractalT<double> &fd, const FrameIO &io,
                                             const int x, const int y, const StepBuf<T> &sb, const int stepCap,
                                             Counters &cnt) {
  const int64_t pix = (int64_t)y * p.width + x;
  // view vector (src/Render3D.cpp:389-438)
  const double x2 = ((double)x / p.width / p.tiles - 0.5 + p.tileXOffset / p.tiles) * p.aspect;
  const double z2 = ((double)y / p.height / p.tiles - 0.5 + p.tileYOffset / p.tiles);
  bool hemisphereCut = false;
  V3<double> vv;
  if (p.perspType == 1) {
    if (p.fishEyeCut && sqrt(x2 * x2 + z2 * z2) > 0.5 / p.fov) hemisphereCut = true;
    const double x3 = x2 * kPI;
    const double z3 = z2 * kPI;
    const double r = sqrt(x3 * x3 + z3 * z3);
    if (r == 0) {
      vv = {0.0, 1.0, 0.0};
    } else {
      vv.x = x3 / r * sin(r * p.fov);
      vv.z = z3 / r * sin(r * p.fov);
      vv.y = cos(r * p.fov);
    }
    vv = normalize3(vv);
  } else if (p.perspType == 2) {
    const double x3 = x2 * kPI;
    const double z3 = z2 * kPI;
    vv.x = sin(p.fov * x3) * cos(p.fov * z3);
    vv.z = sin(p.fov * z3);
    vv.y = cos(p.fov * x3) * cos(p.fov * z3);
    vv = normalize3(vv);
  } else {
    vv = {x2 * p.fov, 1.0, z2 * p.fov};
  }
  const V3<double> view = rotate(p.rot, p.rot_zero, vv);
  const V3<double> startD{p.start[0], p.start[1], p.start[2]};
  const V3<T> viewT{(T)view.x, (T)view.y, (T)view.z};
  const V3<T> startT{(T)startD.x, (T)startD.y, (T)startD.z};

  // the reflection loop (src/Render3D.cpp:441-564): ray 0 is the camera ray; each hit on a
  // reflecting object spawns the mirrored ray from just above the hit
  const int maxRay = p.maxRay;
  RayRec<T> rec[kMaxRays];
  V3<double> startRay = startD;
  V3<double> viewRay = view;
  double distThreshCarry = 0.0;
  int rayEnd = 0;
  int iters0 = 0;
  int itersState = 0;   // calcParam->itersOut
  V3<double> point{0.0, 0.0, 0.0};
  for (int ray = 0; ray <= maxRay; ray++) {
    RayRec<T> &rb = rec[ray];
    rb.start = startRay;
    rb.view = viewRay;
    RayState rs;
    rs.found = false;
    rs.overflow = false;
    rs.buffCount = 0;
    rs.iters = itersState;
    rs.distThresh = distThreshCarry;
    rs.dist = 0.0;
    rs.scan = 0.0;
    rs.point[0] = point.x;
    rs.point[1] = point.y;
    rs.point[2] = point.z;
    if (!hemisphereCut) {
      const StepBuf<T> sbr = sb.ray(ray);
      march<T, FORMULA>(p, V3<T>{(T)startRay.x, (T)startRay.y, (T)startRay.z},
                        V3<T>{(T)viewRay.x, (T)viewRay.y, (T)viewRay.z}, (uint32_t)pix, sbr, stepCap, rs, cnt,
                        (T)distThreshCarry);
      if (rs.overflow) {
        const unsigned int k = atomicAdd(io.overflow_count, 1u);
        io.overflow_list[k] = (unsigned int)pix;
        return;
      }
      if (rs.found) {
        if constexpr (sizeof(T) == 4) refine_fix<FORMULA>(p, fd, startRay, viewRay, rs, cnt, distThreshCarry);
        else refine<T, FORMULA>(p, fd, startRay, viewRay, rs, cnt, distThreshCarry);
      }
    }
    itersState = rs.iters;
    if (ray == 0) iters0 = rs.iters;
    point = V3<double>{rs.point[0], rs.point[1], rs.point[2]};
    distThreshCarry = rs.distThresh;
    rb.found = rs.found;
    rb.buffCount = rs.buffCount;
    rb.point = point;
    rb.distThresh = rs.distThresh;
    rb.lastDist = rs.dist;
    rb.depth = rs.scan;
    rb.objectType = cnt.objectOut;   // shaderInputData.objectType (src/Render3D.cpp:470)
    rb.reflect = rb.objectType == kObjFractal ? p.reflect : p.primReflect[rb.objectType - 1];
    rayEnd = ray;
    if (!rb.found) break;
    if (rb.reflect == T(0)) break;
    // mirrored direction about the hit's normal, started one threshold above the hit
    T detail = (T)rb.distThresh;
    const T thr = (T)rb.distThresh;
    T delta;
    if (p.constantDEThreshold) delta = (T)rb.depth * p.resolution * p.persp;
    else delta = thr * p.quality;
    const V3<T> vn = calc_normal<T, FORMULA>(p, V3<T>{(T)point.x, (T)point.y, (T)point.z}, delta, thr, detail, cnt);
    const V3<double> vnd{(double)vn.x, (double)vn.y, (double)vn.z};
    viewRay = viewRay - vnd * dot3(viewRay, vnd) * 2.0;
    startRay = point + viewRay * rb.distThresh;
  }

  T result[4] = {T(0), T(0), T(0), T(0)};
  V3<T> objColour{T(0), T(0), T(0)};
  float totalOpacity0 = 0.0f;
  T alpha0 = T(0);
  for (int ray = rayEnd; ray >= 0; ray--) {
    RayRec<T> &rb = rec[ray];
    const V3<T> viewT{(T)rb.view.x, (T)rb.view.y, (T)rb.view.z};
    const T dist_thresh = (T)rb.distThresh;
    T detail = (T)rb.distThresh;
    int itersOut = itersState;   // the shared calcParam->itersOut
    // shaderInputData.delta (src/Render3D.cpp:517-518), for hits and background alike
    T delta;
    if (p.constantDEThreshold) delta = (T)rb.depth * p.resolution * p.persp;
    else delta = dist_thresh * p.quality;
    T obj[3] = {T(0), T(0), T(0)}, spec[3] = {T(0), T(0), T(0)}, bg[3] = {T(0), T(0), T(0)};
    T alpha = T(0);
    if (rb.found) {
      object_shader<T, FORMULA>(p, V3<T>{(T)rb.point.x, (T)rb.point.y, (T)rb.point.z}, viewT, rb.view, startT,
                                dist_thresh, delta, (T)rb.lastDist, rb.objectType, detail, itersOut, io, cnt, obj, spec,
                                objColour);
      alpha = T(1) + T(0);
    } else {
      const V3<T> b = background(p, viewT);
      bg[0] = b.x;
      bg[1] = b.y;
      bg[2] = b.z;
    }
    const T reflect = rb.reflect;
    T pixel[4];
    for (int c = 0; c < 3; c++) {
      if (maxRay > 0 && rayEnd > 0 && ray != rayEnd)
        pixel[c] = result[c] * reflect + (T(1) - reflect) * (obj[c] + bg[c]) + spec[c];
      else
        pixel[c] = obj[c] + bg[c] + spec[c];
    }
    pixel[3] = rb.found ? alpha + T(0) : T(0) + T(0);
    float totalOpacity = 0.0f;
    bool opacitySet = false;
    // the volumetric pass sees the march depth even for background pixels: the shader
    // input is filled before the depth becomes 1e20 (src/Render3D.cpp:518-541)
    if (p.needVolumetric)
      volumetric<T, FORMULA>(p, sb.ray(ray), rb.buffCount, (T)rb.depth,
                             V3<T>{(T)rb.start.x, (T)rb.start.y, (T)rb.start.z}, startT, viewT, delta,
                             (T)rb.lastDist, detail, itersOut, io, cnt, pixel, totalOpacity, opacitySet);
    itersState = itersOut;
    result[0] = pixel[0];
    result[1] = pixel[1];
    result[2] = pixel[2];
    if (ray == 0) {
      totalOpacity0 = totalOpacity;
      alpha0 = pixel[3];
    }
  }
  const double depth = rec[0].found ? rec[0].depth : 1e20;
  const float totalOpacity = totalOpacity0;
  result[3] = alpha0;
  const bool found0 = rec[0].found;

  // buffer writes (src/Render3D.cpp:569-589)
  if (io.opacity) io.opacity[pix] = to_u16_x86((double)totalOpacity * 65535.0);
  if (io.alpha) io.alpha[pix] = to_u16_x86((double)result[3] * 65535.0);
  if (io.image_float) {
    io.image_float[3 * pix + 0] = (float)result[0];
    io.image_float[3 * pix + 1] = (float)result[1];
    io.image_float[3 * pix + 2] = (float)result[2];
  }
  if (io.colour) {
    io.colour[3 * pix + 0] = to_u8_x86((double)(objColour.x * T(255)));
    io.colour[3 * pix + 1] = to_u8_x86((double)(objColour.y * T(255)));
    io.colour[3 * pix + 2] = to_u8_x86((double)(objColour.z * T(255)));
  }
  if (io.zbuffer) io.zbuffer[pix] = (float)depth;
  if (io.hit) io.hit[pix] = found0 ? 1 : 0;
  if (io.iters) io.iters[pix] = iters0;
  if (io.depth) io.depth[pix] = depth;
}

// ---------------------------------------------------------------------------
// Persistent kernel: each warp claims 8x4 pixel tiles from a global counter
// until the frame is done, replacing the row claiming of MainThread
// (src/Render3D.cpp:352-366) and the thread spawn of Render (src/Render3D.cpp:815-849).
// ---------------------------------------------------------------------------
template <typename T, int FORMULA>
__global__ void __launch_bounds__(128) render_kernel(const __grid_constant__ ParamsT<T> p, const __grid_constant__ FractalT<double> fd, const FrameIO io) {
  const int lane = threadIdx.x & 31;
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  StepBuf<T> sb{(T *)io.step_step, (T *)io.step_dist, (T *)io.step_thr, (T *)io.step_scan, io.step_iters,
                io.slots * (io.rays > 0 ? io.rays : 1), slot, io.slots};
  Counters cnt{0, 0, 0, 0};
  const int tilesX = (p.width + kTileW - 1) / kTileW;
  const int rowTiles = (p.row_end - p.row_begin + kTileH - 1) / kTileH;
  const unsigned int nTiles = (unsigned int)(tilesX * rowTiles);
  if (io.overflow_pass) {
    // rays longer than the main pass's step_cap, one pixel per thread, full-length records
    const unsigned int n = *io.overflow_count;
    for (unsigned int k = (unsigned int)slot; k < n; k += (unsigned int)(gridDim.x * blockDim.x)) {
      const unsigned int pix = io.overflow_list[k];
      render_pixel<T, FORMULA>(p, fd, io, (int)(pix % (unsigned int)p.width), (int)(pix / (unsigned int)p.width), sb,
                               kStepSlots, cnt);
    }
  } else
  for (;;) {
    unsigned int t = 0;
    int stop = 0;
    if (lane == 0) {
      t = atomicAdd(io.tile_counter, 1u);
      if (deadline_passed(io)) { atomicExch(io.error_flag, 1); stop = 1; }
      if (io.budget_ns && *(volatile int *)io.error_flag) stop = 1;
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    stop = __shfl_sync(0xffffffffu, stop, 0);
    if (stop || t >= nTiles) break;
    const int tx = (int)(t % (unsigned int)tilesX);
    const int ty = (int)(t / (unsigned int)tilesX);
    const int x = tx * kTileW + (lane % kTileW);
    const int y = p.row_begin + ty * kTileH + (lane / kTileW);
    if (x < p.width && y < p.row_end) render_pixel<T, FORMULA>(p, fd, io, x, y, sb, io.step_cap, cnt);
  }
  // one atomic per warp for the counters
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
    cnt.steps += __shfl_down_sync(0xffffffffu, cnt.steps, off);
    cnt.missed += __shfl_down_sync(0xffffffffu, cnt.missed, off);
  }
  if (lane == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
    atomicAdd(&io.counters[2], cnt.steps);
    atomicAdd(&io.counters[3], cnt.missed);
  }
}

// CalculateDistance at arbitrary points (unit tests of the distance estimator).
template <typename T, int FORMULA>
__global__ void distance_kernel(const __grid_constant__ FractalT<T> f, const double *points, const double *detail, int64_t n,
                                double *dist, int32_t *iters, uint8_t *max_iter, unsigned long long *counters) {
  Counters cnt{0, 0, 0, 0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const V3<T> pt{(T)points[3 * i], (T)points[3 * i + 1], (T)points[3 * i + 2]};
    int L = 0;
    bool mi = false;
    const T d = calc_distance<T, FORMULA>(f, pt, (T)detail[i], f.N, f.minN, false, L, mi, cnt, fparam_of(f));
    dist[i] = (double)d;
    iters[i] = L;
    max_iter[i] = mi ? 1 : 0;
  }
  if (counters) {
    atomicAdd(&counters[0], cnt.orbit);
    atomicAdd(&counters[1], cnt.calls);
  }
}

}  // namespace dev
}  // namespace mbgb
