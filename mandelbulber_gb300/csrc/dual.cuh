// Forward-mode dual numbers for the gradient stage and the level-set hit refinement: a
// value and its derivatives along K tangent directions, propagated by the chain rule
// through the orbit iteration.
// Values come from the same math overloads as the render (m_sqrt, m_pow, ...), so a
// dual evaluation reproduces the render's distance estimate in the same precision.
#pragma once

#include "render_core.cuh"

namespace mbgb {
namespace dev {

template <typename T, int K>
struct Dual {
  T v;
  T d[K];
};

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> dconst(const T v) {
  Dual<T, K> r;
  r.v = v;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = T(0);
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> dseed(const T v, const int k0) {
  Dual<T, K> r = dconst<T, K>(v);
  r.d[k0] = T(1);
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator+(const Dual<T, K> &a, const Dual<T, K> &b) {
  Dual<T, K> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = a.d[k] + b.d[k];
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator-(const Dual<T, K> &a, const Dual<T, K> &b) {
  Dual<T, K> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = a.d[k] - b.d[k];
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator-(const Dual<T, K> &a) {
  Dual<T, K> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = -a.d[k];
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator+(const Dual<T, K> &a, const T b) {
  Dual<T, K> r = a;
  r.v = a.v + b;
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator*(const Dual<T, K> &a, const Dual<T, K> &b) {
  Dual<T, K> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator*(const Dual<T, K> &a, const T b) {
  Dual<T, K> r;
  r.v = a.v * b;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = a.d[k] * b;
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> operator/(const Dual<T, K> &a, const Dual<T, K> &b) {
  Dual<T, K> r;
  r.v = a.v / b.v;
  const T inv = T(1) / b.v;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> dsqrt(const Dual<T, K> &a) {
  Dual<T, K> r;
  r.v = m_sqrt(a.v);
  const T g = r.v > T(0) ? T(0.5) / r.v : T(0);
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = a.d[k] * g;
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> dlog(const Dual<T, K> &a) {
  Dual<T, K> r;
  r.v = m_log(a.v);
  const T g = T(1) / a.v;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = a.d[k] * g;
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> dasin(const Dual<T, K> &a) {
  Dual<T, K> r;
  r.v = m_asin(a.v);
  const T s = T(1) - a.v * a.v;
  const T g = s > T(0) ? T(1) / m_sqrt(s) : T(0);
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = a.d[k] * g;
  return r;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> datan2(const Dual<T, K> &y, const Dual<T, K> &x) {
  Dual<T, K> r;
  r.v = m_atan2(y.v, x.v);
  const T q = x.v * x.v + y.v * y.v;
  const T gx = q > T(0) ? -y.v / q : T(0);
  const T gy = q > T(0) ? x.v / q : T(0);
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = y.d[k] * gy + x.d[k] * gx;
  return r;
}

template <typename T, int K>
__device__ __forceinline__ void dsincos(const Dual<T, K> &a, Dual<T, K> &s, Dual<T, K> &c) {
  T sv, cv;
  m_sincos(a.v, &sv, &cv);
  s.v = sv;
  c.v = cv;
#pragma unroll
  for (int k = 0; k < K; k++) {
    s.d[k] = a.d[k] * cv;
    c.d[k] = -a.d[k] * sv;
  }
}

// r^q for dual base and exponent: d(r^q) = r^q (q / r dr + ln r dq).
template <typename T, int K>
__device__ __forceinline__ Dual<T, K> dpow(const Dual<T, K> &r, const Dual<T, K> &q) {
  Dual<T, K> o;
  o.v = m_pow(r.v, q.v);
  const T gr = r.v != T(0) ? o.v * q.v / r.v : T(0);
  const T gq = r.v > T(0) ? o.v * m_log(r.v) : T(0);
#pragma unroll
  for (int k = 0; k < K; k++) o.d[k] = r.d[k] * gr + q.d[k] * gq;
  return o;
}

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> dfabs(const Dual<T, K> &a) {
  return a.v < T(0) ? -a : a;
}

template <typename T, int K>
struct DV3 {
  Dual<T, K> x, y, z;
};

template <typename T, int K>
__device__ __forceinline__ Dual<T, K> dlength(const DV3<T, K> &v) {
  if constexpr (sizeof(T) == 4) {
    // FP32: the tangent as (x/r) dx + (y/r) dy + (z/r) dz, without the squares' tangents
    // 2 x dx, which leave FP32's range at an orbit's escape step (x ~ 1e16, dx ~ 1e35)
    Dual<T, K> r;
    r.v = m_sqrt(v.x.v * v.x.v + v.y.v * v.y.v + v.z.v * v.z.v);
    const T inv = r.v > T(0) ? T(1) / r.v : T(0);
    const T ux = v.x.v * inv, uy = v.y.v * inv, uz = v.z.v * inv;
#pragma unroll
    for (int k = 0; k < K; k++) r.d[k] = ux * v.x.d[k] + uy * v.y.d[k] + uz * v.z.d[k];
    return r;
  } else {
    return dsqrt(v.x * v.x + v.y * v.y + v.z * v.z);
  }
}

// Compute<normal> of formula 2 (src/fractal.cpp:211-225) or formula 8 without rotations
// and offset (src/fractal.cpp:467-528) on dual numbers: `z` is the point with its K
// tangents, `fp` the formula's parameter (power of formula 2, Mandelbox scale of formula
// 8) with its tangents. Returns the distance estimate (0 with zero derivatives when the
// orbit does not escape) and the iteration count.
template <typename T, int FORMULA, int K>
__device__ __forceinline__ Dual<T, K> de_dual_seeded(const FractalT<T> &f, DV3<T, K> z, const Dual<T, K> fp,
                                                     const int N, int &Lout) {
  using D = Dual<T, K>;
  DV3<T, K> c;
  if (f.juliaMode) {
    c = {dconst<T, K>(f.julia[0]), dconst<T, K>(f.julia[1]), dconst<T, K>(f.julia[2])};
  } else {
    c = {z.x * f.constantFactor, z.y * f.constantFactor, z.z * f.constantFactor};
  }
  D dist = dconst<T, K>(T(0));
  D r = dlength(z);
  int L;
  if (FORMULA == 2) {
    const D p = fp;
    const D pm1 = p + T(-1);
    D r_dz = dconst<T, K>(T(1));
    // FP32: the running derivative's tangents grow like r_dz^2 and leave FP32's range near
    // the surface, so they are carried relative to r_dz (q = d r_dz / r_dz), which stays small
    T rdz = T(1), q[K];
#pragma unroll
    for (int k = 0; k < K; k++) q[k] = T(0);
    for (L = 0; L < N; L++) {
      const D th0 = dasin(z.z / r);
      const D ph0 = datan2(z.y, z.x);
      D rp = dpow(r, pm1);
      const D th = th0 * p;
      const D ph = ph0 * p;
      D sth, cth, sph, cph;
      dsincos(th, sth, cth);
      dsincos(ph, sph, cph);
      if constexpr (sizeof(T) == 4) {
        // r_dz' = A r_dz + 1 with A = r^(p-1) p: d r_dz' / r_dz' = (dA + A q) r_dz / r_dz'
        const D A = rp * p;
        const T nv = A.v * rdz + T(1);
        const T ratio = rdz / nv;
#pragma unroll
        for (int k = 0; k < K; k++) q[k] = (A.d[k] + A.v * q[k]) * ratio;
        rdz = nv;
      } else {
        r_dz = rp * r_dz * p + T(1);
      }
      rp = rp * r;
      z = {(cth * cph) * rp + c.x, (cth * sph) * rp + c.y, sth * rp + c.z};
      r = dlength(z);
      if (r.v > f.bailout) {
        if constexpr (sizeof(T) == 4) {
          // dist = num / r_dz: d dist = d num / r_dz - dist q
          const D num = (r * dlog(r)) * T(0.5);
          dist.v = num.v / rdz;
#pragma unroll
          for (int k = 0; k < K; k++) dist.d[k] = num.d[k] / rdz - dist.v * q[k];
        } else {
          dist = (r * dlog(r)) * T(0.5) / r_dz;
        }
        break;
      }
    }
  } else {
    const D scale = fp;
    const T fR2 = f.mbFixedR * f.mbFixedR;
    const T mR2 = f.mbMinR * f.mbMinR;
    const T factor1 = fR2 / mR2;
    D tgladDE = dconst<T, K>(T(1));
    for (L = 0; L < N; L++) {
      if (z.x.v > f.mbFoldLimit) z.x = -z.x + f.mbFoldValue;
      else if (z.x.v < -f.mbFoldLimit) z.x = -z.x + (-f.mbFoldValue);
      if (z.y.v > f.mbFoldLimit) z.y = -z.y + f.mbFoldValue;
      else if (z.y.v < -f.mbFoldLimit) z.y = -z.y + (-f.mbFoldValue);
      if (z.z.v > f.mbFoldLimit) z.z = -z.z + f.mbFoldValue;
      else if (z.z.v < -f.mbFoldLimit) z.z = -z.z + (-f.mbFoldValue);
      r = dlength(z);
      const D r2 = r * r;
      if (r2.v < mR2) {
        z = {z.x * factor1, z.y * factor1, z.z * factor1};
        tgladDE = tgladDE * factor1;
      } else if (r2.v < fR2) {
        const D f2 = dconst<T, K>(fR2) / r2;
        z = {z.x * f2, z.y * f2, z.z * f2};
        tgladDE = tgladDE * f2;
      }
      z = {z.x * scale + c.x, z.y * scale + c.y, z.z * scale + c.z};
      tgladDE = tgladDE * dfabs(scale) + T(1);
      r = dlength(z);
      if (r.v > T(1024)) {
        dist = r / dfabs(tgladDE);
        break;
      }
    }
  }
  Lout = L;
  if (L == N || dist.v < T(0)) dist = dconst<T, K>(T(0));
  return dist;
}

// Distance estimate with derivatives by the point (tangents 0..2) and by the formula's
// parameter (tangent 3).
template <typename T, int FORMULA>
__device__ __forceinline__ Dual<T, 4> de_dual(const FractalT<T> &f, const V3<T> P, const int N, int &Lout,
                                              const T fparam) {
  const DV3<T, 4> z{dseed<T, 4>(P.x, 0), dseed<T, 4>(P.y, 1), dseed<T, 4>(P.z, 2)};
  return de_dual_seeded<T, FORMULA, 4>(f, z, dseed<T, 4>(fparam, 3), N, Lout);
}

// Distance estimate and its derivative along direction d (one tangent).
template <typename T, int FORMULA>
__device__ __forceinline__ Dual<T, 1> de_along(const FractalT<T> &f, const V3<T> P, const V3<T> d, const int N,
                                               int &Lout, const T fparam) {
  DV3<T, 1> z{dconst<T, 1>(P.x), dconst<T, 1>(P.y), dconst<T, 1>(P.z)};
  z.x.d[0] = d.x;
  z.y.d[0] = d.y;
  z.z.d[0] = d.z;
  return de_dual_seeded<T, FORMULA, 1>(f, z, dconst<T, 1>(fparam), N, Lout);
}

// Newton refinement of a hit to the level set DE(o + t d) = thr(t) in FP64 (after the
// reference's binary refinement has put it inside the window (0.99 thr, thr)). Returns
// false (and leaves t) when the level set is not reached: a grazing ray (F_t >= 0), a
// flat estimate (orbit not escaping, minN clamp), or no convergence in 16 steps.
template <int FORMULA>
__device__ __forceinline__ bool level_set_hit(const FractalT<double> &f, const V3<double> o, const V3<double> d,
                                              const double k, const double thrConst, double &t, int &iters,
                                              const double fparam) {
  double tt = t;
  for (int it = 0; it < 16; it++) {
    int L;
    const Dual<double, 1> de = de_along<double, FORMULA>(f, o + d * tt, d, f.N, L, fparam);
    const double thr = k > 0.0 ? tt * k : thrConst;
    if (L == f.N || L < f.minN) return false;
    const double F = de.v - thr;
    if (fabs(F) <= 1e-13 * thr) {
      t = tt;
      iters = L;
      return true;
    }
    const double Ft = de.d[0] - k;
    if (!(Ft < 0.0)) return false;
    double dt = -F / Ft;
    // the bisection window already brackets the root to a small fraction of thr
    const double lim = thr / sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
    if (fabs(dt) > lim) return false;
    tt += dt;
  }
  return false;
}

// The same refinement in FP32 for the FP32 policy, on its own distance estimate and ray
// (the march's): Newton steps until |F| <= 2e-5 thr, about FP32's resolution of an estimate
// near the surface, which puts t within an ulp or two of the FP32 root. Returns false where
// the FP64 refinement takes over.
template <int FORMULA>
__device__ __forceinline__ bool level_set_hit_f32(const FractalT<float> &f, const V3<float> o, const V3<float> d,
                                                  const float k, const float thrConst, float &t, int &iters,
                                                  const float fparam) {
  float tt = t;
  const float lenD = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
  for (int it = 0; it < 16; it++) {
    int L;
    const Dual<float, 1> de = de_along<float, FORMULA>(f, o + d * tt, d, f.N, L, fparam);
    const float thr = k > 0.0f ? tt * k : thrConst;
    if (L == f.N || L < f.minN || !isfinite(de.v) || !isfinite(de.d[0])) return false;
    const float F = de.v - thr;
    if (fabsf(F) <= 2e-5f * thr) {
      t = tt;
      iters = L;
      return true;
    }
    const float Ft = de.d[0] - k;
    if (!(Ft < 0.0f)) return false;
    const float dt = -F / Ft;
    // the bisection window already brackets the root to a small fraction of thr
    if (fabsf(dt) > thr / lenD) return false;
    tt += dt;
  }
  return false;
}

}  // namespace dev
}  // namespace mbgb
