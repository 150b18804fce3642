// Run-time formula path: Compute<Mode> (src/fractal.cpp:40-1241) and CalculateDistance
// (src/fractal.cpp:1245-1448) for every formula of enumFractalFormula (src/fractal.h:25-65)
// except ocl_custom, with the per-iteration formula sequence of the hybrid formula
// (CreateFormulaSequence, src/callbacks.cpp:1666-1702) and the delta-DE branch of
// CalculateDistance (src/fractal.cpp:1308-1381).
//
// trig_optim (2) and tglad (8) also have compile-time instantiations of their own
// (compute<T, 2|8, MODE> in render_core.cuh), which the headline scenes run; this path
// serves every other formula, and 2 and 8 as steps of a hybrid sequence. It is one
// non-inlined function per (precision, mode), called from every DE site of the march and
// the shaders, so the kernels that use it carry one copy of the formula bodies. The
// kernels take their parameter blocks as __grid_constant__, so the FractalT pointer
// handed in here points at the kernel's own parameter space.
//
// Included by render_core.cuh after the vector and math helpers.
#pragma once

namespace mbgb {
namespace dev {

__device__ __forceinline__ double m_acos(double x) { return acos(x); }
__device__ __forceinline__ float m_acos(float x) { return acosf(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ double m_sin(double x) { return sin(x); }
__device__ __forceinline__ float m_sin(float x) { return sinf(x); }
__device__ __forceinline__ double m_cos(double x) { return cos(x); }
__device__ __forceinline__ float m_cos(float x) { return cosf(x); }

// Compute modes (enumCalculationMode, src/fractal.h:67-70) this path evaluates.
constexpr int kModeNormal = 0, kModeColour = 1, kModeDelta1 = 3, kModeDelta2 = 4, kModeOrbitTrap = 5;

// Formulas that end their orbit at r > 1024 with distance r / |tgladDE|
// (src/fractal.cpp:1141-1148).
__host__ __device__ __forceinline__ bool box_formula(const int f) {
  return f == 8 || f == 17 || f == 18 || f == 37;
}

// 3x3 product with CMatrix33::operator*'s summation order (src/algebra.cpp:55-68).
template <typename T>
__device__ __forceinline__ void mat_mul(T *m, const T *r) {
  T o[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) o[3 * i + j] = m[3 * i + 0] * r[0 + j] + m[3 * i + 1] * r[3 + j] + m[3 * i + 2] * r[6 + j];
#pragma unroll
  for (int i = 0; i < 9; i++) m[i] = o[i];
}

// SmoothConditionAGreaterB / ALessB (src/common_math.h:87-88).
template <typename T>
__device__ __forceinline__ T smooth_greater(T a, T b, T sharpness) {
  return T(1) / (T(1) + m_exp(sharpness * (b - a)));
}
template <typename T>
__device__ __forceinline__ T smooth_less(T a, T b, T sharpness) {
  return T(1) / (T(1) + m_exp(sharpness * (a - b)));
}

// One tglad Mandelbox iteration (src/fractal.cpp:409-529): box fold (with the optional
// per-axis rotations), sphere fold about the offset, main rotation, z * scale + c.
template <typename T>
__device__ __forceinline__ void tglad_step(const FractalT<T> &f, V3<T> &z, T &r, T &tgladDE, T &tgladColor,
                                           const T scale, const V3<T> constant, const T fR2, const T mR2,
                                           const T tglad_factor1) {
  if (f.mbRotEnabled) {
    bool lockout = false;
    z = rotate(f.mbRot[0][0], f.mbRotZero[0][0], z);
    if (z.x > f.mbFoldLimit) { z.x = f.mbFoldValue - z.x; tgladColor += f.mbColX; lockout = true; }
    z = rotate(f.mbRotInv[0][0], 0, z);
    z = rotate(f.mbRot[1][0], f.mbRotZero[1][0], z);
    if (!lockout && z.x < -f.mbFoldLimit) { z.x = -f.mbFoldValue - z.x; tgladColor += f.mbColX; }
    z = rotate(f.mbRotInv[1][0], 0, z);
    lockout = false;
    z = rotate(f.mbRot[0][1], f.mbRotZero[0][1], z);
    if (z.y > f.mbFoldLimit) { z.y = f.mbFoldValue - z.y; tgladColor += f.mbColY; lockout = true; }
    z = rotate(f.mbRotInv[0][1], 0, z);
    z = rotate(f.mbRot[1][1], f.mbRotZero[1][1], z);
    if (!lockout && z.y < -f.mbFoldLimit) { z.y = -f.mbFoldValue - z.y; tgladColor += f.mbColY; }
    z = rotate(f.mbRotInv[1][1], 0, z);
    lockout = false;
    z = rotate(f.mbRot[0][2], f.mbRotZero[0][2], z);
    if (z.z > f.mbFoldLimit) { z.z = f.mbFoldValue - z.z; tgladColor += f.mbColZ; lockout = true; }
    z = rotate(f.mbRotInv[0][2], 0, z);
    z = rotate(f.mbRot[1][2], f.mbRotZero[1][2], z);
    if (!lockout && z.z < -f.mbFoldLimit) { z.z = -f.mbFoldValue - z.z; tgladColor += f.mbColZ; }
    z = rotate(f.mbRotInv[1][2], 0, z);
  } else {
    if (z.x > f.mbFoldLimit) { z.x = f.mbFoldValue - z.x; tgladColor += f.mbColX; }
    else if (z.x < -f.mbFoldLimit) { z.x = -f.mbFoldValue - z.x; tgladColor += f.mbColX; }
    if (z.y > f.mbFoldLimit) { z.y = f.mbFoldValue - z.y; tgladColor += f.mbColY; }
    else if (z.y < -f.mbFoldLimit) { z.y = -f.mbFoldValue - z.y; tgladColor += f.mbColY; }
    if (z.z > f.mbFoldLimit) { z.z = f.mbFoldValue - z.z; tgladColor += f.mbColZ; }
    else if (z.z < -f.mbFoldLimit) { z.z = -f.mbFoldValue - z.z; tgladColor += f.mbColZ; }
  }
  r = orbit_length(z);
  const T r2 = r * r;
  const V3<T> off{f.mbOffset[0], f.mbOffset[1], f.mbOffset[2]};
  z = z + off;
  if (r2 < mR2) {
    z = z * tglad_factor1; tgladDE *= tglad_factor1; tgladColor += f.mbColSp1;
  } else if (r2 < fR2) {
    const T tglad_factor2 = fR2 / r2;
    z = z * tglad_factor2; tgladDE *= tglad_factor2; tgladColor += f.mbColSp2;
  }
  z = z - off;
  z = rotate(f.mbMainRot, f.mbMainRotZero, z);
  z = z * scale + constant;
  tgladDE = tgladDE * m_fabs(scale) + T(1);
  r = orbit_length(z);
}

// One trig_optim Mandelbulb iteration (src/fractal.cpp:211-225).
template <typename T>
__device__ __forceinline__ void trig_optim_step(V3<T> &z, T &r, T &r_dz, const T p, const V3<T> constant) {
  const T th0 = m_asin(z.z / r);
  const T ph0 = m_atan2(z.y, z.x);
  T rp = m_pow(r, p - T(1));
  const T th = th0 * p;
  const T ph = ph0 * p;
  T sth, cth, sph, cph;
  m_sincos(th, &sth, &cth);
  m_sincos(ph, &sph, &cph);
  r_dz = rp * r_dz * p + T(1);
  rp *= r;
  z = V3<T>{cth * cph, cth * sph, sth} * rp + constant;
  r = orbit_length(z);
}

// Reflection across the closest cutting plane that meets the segment y + a * l, a in (0, 1]
// (the three plane searches of generalizedFoldBox, src/fractal.cpp:583-660).
template <typename T>
__device__ __forceinline__ int gfb_cut(const FractalT<T> &f, const V3<T> y, const V3<T> l, const int skip1,
                                       const int skip2, const bool from_origin, T &a) {
  a = T(1);
  int side = -1;
  for (int i = 0; i < f.gfbSides; i++) {
    if (i == skip1 || i == skip2) continue;
    const V3<T> nv{f.gfbNv[i][0], f.gfbNv[i][1], f.gfbNv[i][2]};
    const T b = from_origin ? f.mbSolid : f.mbSolid - dot3(y, nv);
    const T c = dot3(l, nv);
    if ((c > T(0)) && ((a * c) > b)) {
      side = i;
      a = b / c;
    }
  }
  return side;
}

// z moved to the far side of the melt layer around x: z + (x - z) * 2 (|x - z| - melt) /
// (|x - z| + 1e-8), when |x - z| > melt (src/fractal.cpp:664-700).
template <typename T>
__device__ __forceinline__ bool gfb_melt(V3<T> &z, const V3<T> x, const T melt) {
  const V3<T> z2X = x - z;
  if (dot3(z2X, z2X) > (melt * melt)) {
    const T mag = length3(z2X);
    z = z + z2X * (T(2) * (mag - melt) / (mag + T(.00000001)));
    return true;
  }
  return false;
}

// Compute<MODE> for the run-time formulas. `count` is deltaDE2's iteration count (the
// in/out argument iter_count of the reference); *Lout receives the last iteration index.
template <typename T, int MODE>
__device__ __noinline__ T compute_runtime(const FractalT<T> *__restrict__ fp, V3<T> z, const int N, const int count,
                                          int *Lout, const T fparam) {
  const FractalT<T> &f = *fp;
  const bool scale_main = scale_formula(f.formula);
  T p = scale_main ? f.power : fparam;    // doubles.power
  T scale = scale_main ? fparam : f.mbScale;
  T distance = T(0);
  T w = T(0), constantw = T(0);
  V3<T> dz{T(1), T(0), T(0)};
  T r_dz = T(1), ph_dz = T(0), th_dz = T(0);
  const T fR2 = f.mbFixedR * f.mbFixedR;
  const T mR2 = f.mbMinR * f.mbMinR;
  const T tglad_factor1 = fR2 / mR2;
  T tgladDE = T(1), tgladColor = T(1);
  V3<T> constant;
  if (f.juliaMode) constant = {f.julia[0], f.julia[1], f.julia[2]};
  else constant = z * f.constantFactor;
  int form = f.formula;
  const bool hybrid = form == 12;
  T r = orbit_length(z);
  T minv = (sizeof(T) == 8) ? T(1e200) : T(__int_as_float(0x7f800000));
  T orbitTrapTotal = T(0);
  int seg = 0, segk = 0;  // position in the hybrid sequence
  int L;
  for (L = 0; L < N; L++) {
    if (hybrid) {
      // formulaSequence / hybridPowerSequence hold (int)N entries; iterations past them
      // (the x5 normals and x10 colouring orbits) reuse the last entry
      if (L < f.N) {
        form = f.hybridForm[seg];
        p = f.hybridPower[seg];
        if (++segk == f.hybridCount[seg]) {
          segk = 0;
          seg = (seg + 1 == f.hybridSegs) ? 0 : seg + 1;
        }
      }
      scale = p;
    }
    if (f.ifsFolding) {  // Kaleidoscopic IFS pre-fold (src/fractal.cpp:100-123)
      if (f.ifsAbsX) z.x = m_fabs(z.x);
      if (f.ifsAbsY) z.y = m_fabs(z.y);
      if (f.ifsAbsZ) z.z = m_fabs(z.z);
      for (int i = 0; i < 9; i++) {
        if (!f.ifsEnabled[i]) continue;
        z = rotate(f.ifsRot[i], f.ifsRotZero[i], z);
        const V3<T> d{f.ifsDir[i][0], f.ifsDir[i][1], f.ifsDir[i][2]};
        const T length = dot3(z, d);
        if (length < f.ifsDist[i]) z = z - (d * T(2)) * (length - f.ifsDist[i]);
      }
      const V3<T> off{f.ifsOffset[0], f.ifsOffset[1], f.ifsOffset[2]};
      z = rotate(f.ifsMainRot, f.ifsMainRotZero, z - off) + off;
      z = z * f.ifsScale;
      z = z - off * (f.ifsScale - T(1));
      r = orbit_length(z);
    }
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
    switch (form) {
      case 1: {  // trig_DE (src/fractal.cpp:189-210)
        const T r1 = m_pow(r, p - T(1));
        const T r2 = r1 * r;
        const T th = m_atan2(z.y, z.x);
        const T ph = -m_atan2(z.z, m_sqrt(z.x * z.x + z.y * z.y));
        if (MODE == kModeNormal) {
          const T p_r1_rdz = p * r1 * r_dz;
          const T ph_phdz = (p - T(1)) * ph + ph_dz;
          const T th_thdz = (p - T(1)) * th + th_dz;
          T sb, cb, sa, ca;
          m_sincos(ph_phdz, &sb, &cb);
          m_sincos(th_thdz, &sa, &ca);
          dz = V3<T>{cb * ca * p_r1_rdz + T(1), cb * sa * p_r1_rdz + T(0), sb * p_r1_rdz + T(0)};
          r_dz = length3(dz);
          th_dz = m_atan2(dz.y, dz.x);
          ph_dz = -m_atan2(dz.z, m_sqrt(dz.x * dz.x + dz.y * dz.y));
        }
        T sb, cb, sa, ca;
        m_sincos(p * ph, &sb, &cb);
        m_sincos(p * th, &sa, &ca);
        z = V3<T>{cb * ca, cb * sa, sb} * r2 + constant;
        r = orbit_length(z);
        break;
      }
      case 2:  // trig_optim
        trig_optim_step(z, r, r_dz, p, constant);
        break;
      case 3:    // fast_trig (src/fractal.cpp:321-335)
      case 6: {  // minus_fast_trig (src/fractal.cpp:336-350): the same with +2 z sqrt(x2 + y2)
        const T x2 = z.x * z.x, y2 = z.y * z.y, z2 = z.z * z.z;
        const T temp = T(1) - z2 / (x2 + y2);
        const T newx = (x2 - y2) * temp;
        const T newy = T(2) * z.x * z.y * temp;
        const T newz = (form == 3 ? T(-2) : T(2)) * z.z * m_sqrt(x2 + y2);
        z = V3<T>{newx + constant.x, newy + constant.y, newz + constant.z};
        r = orbit_length(z);
        break;
      }
      case 4: {  // hypercomplex (src/fractal.cpp:351-359)
        const V3<T> nz{z.x * z.x - z.y * z.y - z.z * z.z - w * w, T(2) * z.x * z.y - T(2) * w * z.z,
                       T(2) * z.x * z.z - T(2) * z.y * w};
        const T nw = T(2) * z.x * w - T(2) * z.y * z.z;
        z = nz + constant;
        w = nw;
        r = m_sqrt(z.x * z.x + z.y * z.y + z.z * z.z + w * w);
        break;
      }
      case 5: {  // quaternion (src/fractal.cpp:360-368)
        const V3<T> nz{z.x * z.x - z.y * z.y - z.z * z.z - w * w, T(2) * z.x * z.y, T(2) * z.x * z.z};
        const T nw = T(2) * z.x * w;
        z = nz + constant;
        w = nw;
        r = m_sqrt(z.x * z.x + z.y * z.y + z.z * z.z + w * w);
        break;
      }
      case 7: {  // menger_sponge (src/fractal.cpp:369-407): fold into x >= y >= z >= 0
        z.x = m_fabs(z.x);
        z.y = m_fabs(z.y);
        z.z = m_fabs(z.z);
        T t;
        if (z.x - z.y < T(0)) { t = z.y; z.y = z.x; z.x = t; }
        if (z.x - z.z < T(0)) { t = z.z; z.z = z.x; z.x = t; }
        if (z.y - z.z < T(0)) { t = z.z; z.z = z.y; z.y = t; }
        if (MODE == kModeColour) {
          const T len = orbit_length(z);
          if (len < minv) minv = len;
        }
        z = z * T(3);
        z.x -= T(2);
        z.y -= T(2);
        if (z.z > T(1)) z.z -= T(2);
        r = orbit_length(z);
        tgladDE *= T(3);
        break;
      }
      case 8:  // tglad
        tglad_step(f, z, r, tgladDE, tgladColor, scale, constant, fR2, mR2, tglad_factor1);
        break;
      case 10: {  // kaleidoscopic IFS (src/fractal.cpp:837-886)
        if (f.ifsAbsX) z.x = m_fabs(z.x);
        if (f.ifsAbsY) z.y = m_fabs(z.y);
        if (f.ifsAbsZ) z.z = m_fabs(z.z);
        for (int i = 0; i < 9; i++) {
          if (!f.ifsEnabled[i]) continue;
          z = rotate(f.ifsRot[i], f.ifsRotZero[i], z);
          const V3<T> d{f.ifsDir[i][0], f.ifsDir[i][1], f.ifsDir[i][2]};
          const T length = dot3(z, d);
          if (length < f.ifsDist[i]) z = z - d * (T(2) * (length - f.ifsDist[i]) * f.ifsIntensity[i]);
        }
        const V3<T> off{f.ifsOffset[0], f.ifsOffset[1], f.ifsOffset[2]};
        z = rotate(f.ifsMainRot, f.ifsMainRotZero, z - off) + off;
        if (f.ifsEdge[0] > T(0)) z.x = f.ifsEdge[0] - m_fabs(f.ifsEdge[0] - z.x);
        if (f.ifsEdge[1] > T(0)) z.y = f.ifsEdge[1] - m_fabs(f.ifsEdge[1] - z.y);
        if (f.ifsEdge[2] > T(0)) z.z = f.ifsEdge[2] - m_fabs(f.ifsEdge[2] - z.z);
        if (MODE == kModeColour) {
          const T length2 = orbit_length(z);
          if (length2 < minv) minv = length2;
        }
        z = z * f.ifsScale;
        if (f.ifsMenger) {
          z.x -= f.ifsOffset[0] * (f.ifsScale - T(1));
          z.y -= f.ifsOffset[1] * (f.ifsScale - T(1));
          if (z.z > T(0.5) * f.ifsOffset[2] * (f.ifsScale - T(1))) z.z -= f.ifsOffset[2] * (f.ifsScale - T(1));
        } else {
          z = z - off * (f.ifsScale - T(1));
        }
        tgladDE *= f.ifsScale;
        r = orbit_length(z);
        break;
      }
      case 11: {  // xenodreambuie (src/fractal.cpp:300-320)
        const T rp = m_pow(r, p);
        const T th = m_atan2(z.y, z.x);
        T ph = m_acos(z.z / r);
        if (ph > T(0.5) * T(M_PI)) ph = T(M_PI) - ph;
        else if (ph < T(-0.5) * T(M_PI)) ph = T(-M_PI) - ph;
        z.x = rp * m_cos(th * p) * m_sin(ph * p);
        z.y = rp * m_sin(th * p) * m_sin(ph * p);
        z.z = rp * m_cos(ph * p);
        z = z + constant;
        r = orbit_length(z);
        break;
      }
      case 13: {  // mandelbulb2 (src/fractal.cpp:226-254): three plane squarings
        T temp, tempR;
        tempR = m_sqrt(z.x * z.x + z.y * z.y);
        z = z * (T(1) / tempR);
        temp = z.x * z.x - z.y * z.y;
        z.y = T(2) * z.x * z.y;
        z.x = temp;
        z = z * tempR;
        tempR = m_sqrt(z.y * z.y + z.z * z.z);
        z = z * (T(1) / tempR);
        temp = z.y * z.y - z.z * z.z;
        z.z = T(2) * z.y * z.z;
        z.y = temp;
        z = z * tempR;
        tempR = m_sqrt(z.x * z.x + z.z * z.z);
        z = z * (T(1) / tempR);
        temp = z.x * z.x - z.z * z.z;
        z.z = T(2) * z.x * z.z;
        z.x = temp;
        z = z * tempR;
        z = z * r;
        z = z + constant;
        r = orbit_length(z);
        break;
      }
      case 14: {  // mandelbulb3 (src/fractal.cpp:255-282)
        T temp, tempR;
        T sign = T(1), sign2 = T(1);
        if (z.x < T(0)) sign2 = T(-1);
        tempR = m_sqrt(z.x * z.x + z.y * z.y);
        z = z * (T(1) / tempR);
        temp = z.x * z.x - z.y * z.y;
        z.y = T(2) * z.x * z.y;
        z.x = temp;
        z = z * tempR;
        if (z.x < T(0)) sign = T(-1);
        tempR = m_sqrt(z.x * z.x + z.z * z.z);
        z = z * (T(1) / tempR);
        temp = z.x * z.x - z.z * z.z;
        z.z = T(2) * z.x * z.z * sign2;
        z.x = temp * sign;
        z = z * tempR;
        z = z * r;
        z = z + constant;
        r = orbit_length(z);
        break;
      }
      case 15: {  // mandelbulb4 (src/fractal.cpp:283-299): rotations by (p - 1) x the plane angles
        const T rp = m_pow(r, p - T(1));
        const T angZ = m_atan2(z.y, z.x);
        const T angY = m_atan2(z.z, z.x);
        const T angX = m_atan2(z.z, z.y);
        T m[9] = {T(1), T(0), T(0), T(0), T(1), T(0), T(0), T(0), T(1)};
        bool zero = true;
        const T ax = angX * (p - T(1)), ay = angY * (p - T(1)), az = angZ * (p - T(1));
        if (ax != T(0)) {
          T s, c;
          m_sincos(ax, &s, &c);
          const T rx[9] = {T(1), T(0), T(0), T(0), c, -s, T(0), s, c};
          mat_mul(m, rx);
          zero = false;
        }
        if (ay != T(0)) {
          T s, c;
          m_sincos(ay, &s, &c);
          const T ry[9] = {c, T(0), s, T(0), T(1), T(0), -s, T(0), c};
          mat_mul(m, ry);
          zero = false;
        }
        if (az != T(0)) {
          T s, c;
          m_sincos(az, &s, &c);
          const T rz[9] = {c, -s, T(0), s, c, T(0), T(0), T(0), T(1)};
          mat_mul(m, rz);
          zero = false;
        }
        z = rotate(m, zero ? 1 : 0, z) * rp + constant;
        r = orbit_length(z);
        break;
      }
      case 16: {  // foldingIntPow2 (src/fractal.cpp:794-836)
        const T ff = f.intPowFold;
        if (z.x > ff) z.x = ff * T(2) - z.x;
        else if (z.x < -ff) z.x = -ff * T(2) - z.x;
        if (z.y > ff) z.y = ff * T(2) - z.y;
        else if (z.y < -ff) z.y = -ff * T(2) - z.y;
        if (z.z > ff) z.z = ff * T(2) - z.z;
        else if (z.z < -ff) z.z = -ff * T(2) - z.z;
        r = orbit_length(z);
        const T r2_2 = r * r;
        if (r2_2 < T(0.25)) {
          z = z * T(4);
        } else if (r2_2 < T(1)) {
          z = z * (T(1) / r2_2);
        }
        z = z * T(2);
        const T x2 = z.x * z.x, y2 = z.y * z.y, z2 = z.z * z.z;
        const T temp = T(1) - z2 / (x2 + y2);
        const T newx = (x2 - y2) * temp;
        const T newy = T(2) * z.x * z.y * temp;
        const T newz = T(-2) * z.z * m_sqrt(x2 + y2);
        z = V3<T>{newx + constant.x, newy + constant.y, newz + constant.z};
        z.z *= f.intPowZ;
        r = orbit_length(z);
        break;
      }
      case 17: {  // smoothMandelbox (src/fractal.cpp:751-793)
        const T sm = f.mbSharpness;
        const T fl = f.mbFoldLimit, fv = f.mbFoldValue;
        const T zk1 = smooth_greater(z.x, fl, sm);
        const T zk2 = smooth_less(z.x, -fl, sm);
        z.x = z.x * (T(1) - zk1) + (fv - z.x) * zk1;
        z.x = z.x * (T(1) - zk2) + (-fv - z.x) * zk2;
        tgladColor += (zk1 + zk2) * f.mbColX;
        const T zk3 = smooth_greater(z.y, fl, sm);
        const T zk4 = smooth_less(z.y, -fl, sm);
        z.y = z.y * (T(1) - zk3) + (fv - z.y) * zk3;
        z.y = z.y * (T(1) - zk4) + (-fv - z.y) * zk4;
        tgladColor += (zk3 + zk4) * f.mbColY;
        const T zk5 = smooth_greater(z.z, fl, sm);
        const T zk6 = smooth_less(z.z, -fl, sm);
        z.z = z.z * (T(1) - zk5) + (fv - z.z) * zk5;
        z.z = z.z * (T(1) - zk6) + (-fv - z.z) * zk6;
        tgladColor += (zk5 + zk6) * f.mbColZ;
        r = orbit_length(z);
        const T r2 = r * r;
        const T tglad_factor2 = fR2 / r2;
        const T rk1 = smooth_less(r2, mR2, sm);
        const T rk2 = smooth_less(r2, fR2, sm);
        const T rk21 = (T(1) - rk1) * rk2;
        z = z * (T(1) - rk1) + z * (tglad_factor1 * rk1);
        z = z * (T(1) - rk21) + z * (tglad_factor2 * rk21);
        tgladDE = tgladDE * (T(1) - rk1) + tgladDE * (tglad_factor1 * rk1);
        tgladDE = tgladDE * (T(1) - rk21) + tgladDE * (tglad_factor2 * rk21);
        tgladColor += rk1 * f.mbColSp1;
        tgladColor += rk21 * f.mbColSp2;
        z = rotate(f.mbMainRot, f.mbMainRotZero, z);
        z = z * scale + constant;
        tgladDE = tgladDE * m_fabs(scale) + T(1);
        r = orbit_length(z);
        break;
      }
      case 18: {  // mandelboxVaryScale4D (src/fractal.cpp:887-915)
        scale = scale + f.mbVaryScaleVary * (m_fabs(scale) - T(1));
        const V3<T> oldz = z;
        const T fo = f.mbVaryFold;
        z.x = m_fabs(z.x + fo) - m_fabs(z.x - fo) - z.x;
        z.y = m_fabs(z.y + fo) - m_fabs(z.y - fo) - z.y;
        z.z = m_fabs(z.z + fo) - m_fabs(z.z - fo) - z.z;
        w = m_fabs(w + fo) - m_fabs(w - fo) - w;
        if (z.x != oldz.x) tgladColor += f.mbColX;
        if (z.y != oldz.y) tgladColor += f.mbColY;
        if (z.z != oldz.z) tgladColor += f.mbColZ;
        const T rr = m_pow(z.x * z.x + z.y * z.y + z.z * z.z + w * w, f.mbVaryRPower);
        T m = scale;
        if (rr < f.mbVaryMinR * f.mbVaryMinR) {
          m = scale / (f.mbVaryMinR * f.mbVaryMinR);
          tgladColor += f.mbColSp1;
        } else if (rr < T(1)) {
          m = scale / rr;
          tgladColor += f.mbColSp2;
        }
        z = z * m + constant;
        w = w * m + f.mbVaryWadd;
        tgladDE = tgladDE * m_fabs(m) + T(1);
        r = m_sqrt(z.x * z.x + z.y * z.y + z.z * z.z + w * w);
        break;
      }
      case 19: {  // aexion (src/fractal.cpp:916-947): 4D, the first iteration maps z and c
        if (L == 0) {
          const T cx = m_fabs(constant.x + constant.y + constant.z) + f.cadd;
          const T cy = m_fabs(-constant.x - constant.y + constant.z) + f.cadd;
          const T cz = m_fabs(-constant.x + constant.y - constant.z) + f.cadd;
          const T cw = m_fabs(constant.x - constant.y - constant.z) + f.cadd;
          constant = V3<T>{cx, cy, cz};
          constantw = cw;
          const T tx = m_fabs(z.x + z.y + z.z) + f.cadd;
          const T ty = m_fabs(-z.x - z.y + z.z) + f.cadd;
          const T tz = m_fabs(-z.x + z.y - z.z) + f.cadd;
          const T tw = m_fabs(z.x - z.y - z.z) + f.cadd;
          z = V3<T>{tx, ty, tz};
          w = tw;
        }
        const T tx = z.x * z.x - z.y * z.y + T(2) * w * z.z + constant.x;
        const T ty = z.y * z.y - z.x * z.x + T(2) * w * z.z + constant.y;
        const T tz = z.z * z.z - w * w + T(2) * z.x * z.y + constant.z;
        const T tw = w * w - z.z * z.z + T(2) * z.x * z.y + constantw;
        z = V3<T>{tx, ty, tz};
        w = tw;
        r = m_sqrt(z.x * z.x + z.y * z.y + z.z * z.z + w * w);
        break;
      }
      case 20: {  // benesi (src/fractal.cpp:948-970)
        T r1 = z.y * z.y + z.z * z.z;
        T newx;
        if (constant.x < T(0) || z.x < m_sqrt(r1)) newx = z.x * z.x - r1;
        else newx = -z.x * z.x + r1;
        r1 = T(-1) / m_sqrt(r1) * T(2) * m_fabs(z.x);
        const T newy = r1 * (z.y * z.y - z.z * z.z);
        const T newz = r1 * T(2) * z.y * z.z;
        z = V3<T>{newx + constant.x, newy + constant.y, newz + constant.z};
        r = orbit_length(z);
        break;
      }
      case 21: {  // bristorbrot (src/fractal.cpp:971-983)
        const T newx = z.x * z.x - z.y * z.y - z.z * z.z;
        const T newy = z.y * (T(2) * z.x - z.z);
        const T newz = z.z * (T(2) * z.x + z.y);
        z = V3<T>{newx + constant.x, newy + constant.y, newz + constant.z};
        r = orbit_length(z);
        break;
      }
      case 22:  // invertX / Y / Z (src/fractal.cpp:984-1001)
        z.x = z.x >= T(0) ? z.x * z.x / (m_fabs(z.x) + p) : -z.x * z.x / (m_fabs(z.x) + p);
        r = orbit_length(z);
        break;
      case 23:
        z.y = z.y >= T(0) ? z.y * z.y / (m_fabs(z.y) + p) : -z.y * z.y / (m_fabs(z.y) + p);
        r = orbit_length(z);
        break;
      case 24:
        z.z = z.z >= T(0) ? z.z * z.z / (m_fabs(z.z) + p) : -z.z * z.z / (m_fabs(z.z) + p);
        r = orbit_length(z);
        break;
      case 25: {  // invertR (src/fractal.cpp:1002-1010)
        const T rInv = r * r / (r + p);
        z.x = z.x / r * rInv;
        z.y = z.y / r * rInv;
        z.z = z.z / r * rInv;
        r = orbit_length(z);
        break;
      }
      case 26: {  // sphericalFold (src/fractal.cpp:1011-1029): sets every component, as written
        const T rr = r * r;
        const T pp = p * p;
        if (rr < pp) {
          z.x = T(1) / pp; z.y = T(1) / pp; z.z = T(1) / pp;
        } else if (rr < pp * T(4)) {
          z.x = T(1) / rr; z.y = T(1) / rr; z.z = T(1) / rr;
        }
        r = orbit_length(z);
        break;
      }
      case 27:  // powXYZ (src/fractal.cpp:1030-1037)
        z.x = z.x >= T(0) ? m_pow(z.x, p) : -m_pow(-z.x, p);
        z.y = z.y >= T(0) ? m_pow(z.y, p) : -m_pow(-z.y, p);
        z.z = z.z >= T(0) ? m_pow(z.z, p) : -m_pow(-z.z, p);
        r = orbit_length(z);
        break;
      case 28: z.x = z.x * p; r = orbit_length(z); break;  // scaleX / Y / Z, offsetX / Y / Z
      case 29: z.y = z.y * p; r = orbit_length(z); break;  // (src/fractal.cpp:1038-1073)
      case 30: z.z = z.z * p; r = orbit_length(z); break;
      case 31: z.x = z.x + p; r = orbit_length(z); break;
      case 32: z.y = z.y + p; r = orbit_length(z); break;
      case 33: z.z = z.z + p; r = orbit_length(z); break;
      case 34: {  // angleMultiplyX / Y / Z (src/fractal.cpp:1074-1100)
        const T angle = m_atan2(z.z, z.y) * p;
        const T tempR = m_sqrt(z.z * z.z + z.y * z.y);
        z.y = tempR * m_cos(angle);
        z.z = tempR * m_sin(angle);
        r = orbit_length(z);
        break;
      }
      case 35: {
        const T angle = m_atan2(z.z, z.x) * p;
        const T tempR = m_sqrt(z.z * z.z + z.x * z.x);
        z.x = tempR * m_cos(angle);
        z.z = tempR * m_sin(angle);
        r = orbit_length(z);
        break;
      }
      case 36: {
        const T angle = m_atan2(z.y, z.x) * p;
        const T tempR = m_sqrt(z.x * z.x + z.y * z.y);
        z.x = tempR * m_cos(angle);
        z.y = tempR * m_sin(angle);
        r = orbit_length(z);
        break;
      }
      case 37: {  // generalizedFoldBox (src/fractal.cpp:531-750)
        const T melt = f.mbMelt;
        T a;
        // closest cutting plane on the segment origin -> z
        const int side_m = gfb_cut(f, V3<T>{T(0), T(0), T(0)}, z, -1, -1, true, a);
        if (side_m != -1) {
          const V3<T> Nv_m{f.gfbNv[side_m][0], f.gfbNv[side_m][1], f.gfbNv[side_m][2]};
          const V3<T> X_m = z - Nv_m * (dot3(z, Nv_m) - f.mbSolid);
          // a plane cutting the segment Nv_m -> X_m: a rotation axis Nv_m x Nv_r
          V3<T> Lv = X_m - Nv_m;
          V3<T> Y = Nv_m;
          const int side_r = gfb_cut(f, Y, Lv, side_m, -1, false, a);
          if (side_r != -1) {
            const V3<T> Xmr_intersect = Y + Lv * a;
            const V3<T> Nv_r{f.gfbNv[side_r][0], f.gfbNv[side_r][1], f.gfbNv[side_r][2]};
            // CVector3::Cross (src/algebra.hpp:93-100)
            V3<T> L_r{Nv_m.y * Nv_r.z - Nv_m.z * Nv_r.y, -Nv_m.x * Nv_r.z + Nv_m.z * Nv_r.x,
                      Nv_m.x * Nv_r.y - Nv_m.y * Nv_r.x};
            T a_rmin = (dot3(z, L_r) - dot3(Xmr_intersect, L_r)) / (dot3(L_r, L_r));
            if (a_rmin < T(0)) {
              a_rmin = -a_rmin;
              L_r = L_r * T(-1);
            }
            const V3<T> X_r = Xmr_intersect + L_r * a_rmin;
            // a plane cutting the segment Xmr_intersect -> X_r: an inversion point
            Lv = X_r - Xmr_intersect;
            Y = Xmr_intersect;
            const int side_i = gfb_cut(f, Y, Lv, side_m, side_r, false, a);
            if (side_i != -1) {
              if (gfb_melt(z, Y + Lv * a, melt)) tgladColor += f.mbColZ;
            } else {
              if (gfb_melt(z, X_r, melt)) tgladColor += f.mbColY;
            }
          } else {
            if (gfb_melt(z, X_m, melt)) tgladColor += f.mbColX;
          }
        }
        r = orbit_length(z);
        const T r2 = r * r;
        const V3<T> off{f.mbOffset[0], f.mbOffset[1], f.mbOffset[2]};
        z = z + off;
        if (r2 < mR2) {
          z = z * tglad_factor1; tgladDE *= tglad_factor1; tgladColor += f.mbColSp1;
        } else if (r2 < fR2) {
          const T tglad_factor2 = fR2 / r2;
          z = z * tglad_factor2; tgladDE *= tglad_factor2; tgladColor += f.mbColSp2;
        }
        z = z - off;
        z = rotate(f.mbMainRot, f.mbMainRotZero, z);
        z = z * scale + constant;
        tgladDE = tgladDE * m_fabs(scale) + T(1);
        r = orbit_length(z);
        break;
      }
      default:  // none, hybrid as a step, ocl_custom: z unchanged
        break;
    }
    // iteration terminate conditions (src/fractal.cpp:1109-1190)
    if (MODE == kModeDelta1) {
      if (r > T(1e10)) break;
    } else if (MODE == kModeDelta2) {
      if (L == count) break;
    }
    if (MODE == kModeOrbitTrap) {  // src/fractal.cpp:1121-1131
      const V3<T> delta = z - V3<T>{f.fakeTrap[0], f.fakeTrap[1], f.fakeTrap[2]};
      distance = length3(delta);
      if (L >= f.fakeMinIter && L <= f.fakeMaxIter) orbitTrapTotal += T(1.0f) / (distance * distance);
      if (distance > T(1000)) {
        distance = orbitTrapTotal;
        break;
      }
    }
    if (form == 7 || form == 10) {
      if (r > T(1000)) { distance = (r - T(2)) / tgladDE; break; }
    } else if (box_formula(form)) {
      if (r > T(1024)) { distance = r / m_fabs(tgladDE); break; }
    } else {
      if (MODE == kModeNormal) {
        if (r > f.bailout) { distance = T(0.5) * r * m_log(r) / r_dz; break; }
      } else if (MODE == kModeColour) {
        if (f.onlyPlane) {
          distance = orbit_length(z);
          if (distance > T(1e15)) {
            distance = (T(L) - m_log(m_log(r) / m_log(T(N))) / m_log(p)) / T(100);
            break;
          }
        } else {
          distance = orbit_length(z);
          if (distance < minv) minv = distance;
          if (distance > T(1e15)) { distance = minv; break; }
        }
      }
    }
  }
  *Lout = L;
  if (MODE == kModeNormal) {
    if (L == N) distance = T(0);
    return distance;
  }
  if (MODE == kModeDelta1 || MODE == kModeDelta2) return r;
  if (MODE == kModeOrbitTrap) return distance;
  // colouring (src/fractal.cpp:1218-1240)
  if (hybrid) {
    if (minv > T(100)) minv = T(100);
    if (distance > T(20)) distance = T(20);
    if (tgladColor > T(1000)) tgladColor = T(1000);
    return distance * T(5000) + tgladColor * T(100) + minv * T(1000);
  }
  if (box_formula(form)) return tgladColor * T(100) + orbit_length(z) * f.mbColR;
  if (form == 10 || form == 7) return minv * T(1000);
  return distance * T(5000);
}

// CalculateDistance (src/fractal.cpp:1245-1448) for the run-time formulas, with the
// delta-DE branch (analitycDE false, src/fractal.cpp:1308-1381): the gradient length of the
// escape radius from forward differences with step 1e-10, the three perturbed orbits run
// to the unperturbed orbit's iteration count. `*Lio` receives itersOut; *orbit and
// *calls count the orbit iterations and Compute calls.
// PrimitiveWater (src/primitives.cpp:95-136): a plane at z = height with `iterations`
// octaves of sine / cosine waves within 10 x amplitude of it.
template <typename T>
__device__ __forceinline__ T primitive_water(const FractalT<T> &f, V3<T> point) {
  const V3<T> plane{T(0), T(0), T(-1)};
  const V3<T> centre{T(0), T(0), f.waterHeight};
  T planeDistance = dot3(plane, point - centre);
  if (planeDistance < f.waterAmplitude * T(10)) {
    const T ang = f.waterRotation / T(180) * T(M_PI);
    if (ang != T(0)) {
      T sn, cs;
      m_sincos(ang, &sn, &cs);
      const T m[9] = {cs, -sn, T(0), sn, cs, T(0), T(0), T(0), T(1)};
      point = rotate(m, 0, point);
    }
    const T phase = f.waterAnimSpeed * T(f.frameNo);
    const T k = T(0.23);
    T waveX = T(0), waveY = T(0);
    T pw = T(1), p2 = T(0.05);
    const T length = f.waterLength;
    for (int i = 1; i <= f.waterIterations; i++) {
      const float p3f = (float)(pw * p2);
      const T p3 = (T)p3f;
      const T shift = phase / (T(i) / T(3) + T(1));
      const T wx = m_sin(T(i) + T(0.4) * (waveX)*p3 + m_sin(k * point.y / length * p3) + point.x / length * p3 + shift) / pw;
      const T wy = m_cos(T(i) + T(0.4) * (waveY)*p3 + m_sin(point.x / length * p3) + k * point.y / length * p3 +
                         shift * T(0.23)) / pw;
      waveX += wx;
      waveY += wy;
      p2 = p2 + (T(1) - p2) * T(0.7);
      pw *= T(1.872);
    }
    planeDistance += (waveX + waveY) * f.waterAmplitude;
  }
  return planeDistance;
}

// The primitive objects of CalculateDistance (src/fractal.cpp:1383-1434): each enabled one
// replaces the distance (and the object) where it is closer.
template <typename T>
__device__ __forceinline__ T primitives(const FractalT<T> &f, const V3<T> point, T distance, int *objectOut) {
  if (f.planeEnable) {
    const V3<T> n{f.planeNormal[0], f.planeNormal[1], f.planeNormal[2]};
    const T d = dot3(n, point - V3<T>{f.planeCentre[0], f.planeCentre[1], f.planeCentre[2]});
    if (!f.onlyPlane && d < distance) *objectOut = kObjPlane;
    distance = (d < distance) ? d : distance;
  }
  if (f.boxEnable || f.invertedBoxEnable) {
    for (int inv = 0; inv < 2; inv++) {
      if (!(inv ? f.invertedBoxEnable : f.boxEnable)) continue;
      const T *c = inv ? f.invBoxCentre : f.boxCentre;
      const T *sz = inv ? f.invBoxSize : f.boxSize;
      const V3<T> c1{c[0] - T(0.5) * sz[0], c[1] - T(0.5) * sz[1], c[2] - T(0.5) * sz[2]};
      const V3<T> c2{c[0] + T(0.5) * sz[0], c[1] + T(0.5) * sz[1], c[2] + T(0.5) * sz[2]};
      // PrimitiveBox / PrimitiveInvertedBox: the planes through the corners, outward for the
      // box (max), inward for the inverted box (min); the unit normals are exact
      const T sgn = inv ? T(1) : T(-1);
      T d = dot3(V3<T>{sgn, T(0), T(0)}, point - c1);
      T q = dot3(V3<T>{-sgn, T(0), T(0)}, point - c2);
      d = inv ? ((q < d) ? q : d) : ((q > d) ? q : d);
      q = dot3(V3<T>{T(0), sgn, T(0)}, point - c1);
      d = inv ? ((q < d) ? q : d) : ((q > d) ? q : d);
      q = dot3(V3<T>{T(0), -sgn, T(0)}, point - c2);
      d = inv ? ((q < d) ? q : d) : ((q > d) ? q : d);
      q = dot3(V3<T>{T(0), T(0), sgn}, point - c1);
      d = inv ? ((q < d) ? q : d) : ((q > d) ? q : d);
      q = dot3(V3<T>{T(0), T(0), -sgn}, point - c2);
      d = inv ? ((q < d) ? q : d) : ((q > d) ? q : d);
      if (d < distance) *objectOut = inv ? kObjBoxInv : kObjBox;
      distance = (d < distance) ? d : distance;
    }
  }
  if (f.sphereEnable) {
    const T d = length3(point - V3<T>{f.sphereCentre[0], f.sphereCentre[1], f.sphereCentre[2]}) - f.sphereRadius;
    if (d < distance) *objectOut = kObjSphere;
    distance = (d < distance) ? d : distance;
  }
  if (f.invertedSphereEnable) {
    const T d =
        f.invSphereRadius - length3(point - V3<T>{f.invSphereCentre[0], f.invSphereCentre[1], f.invSphereCentre[2]});
    if (d < distance) *objectOut = kObjSphereInv;
    distance = (d < distance) ? d : distance;
  }
  if (f.waterEnable) {
    const T d = primitive_water(f, point);
    if (d < distance) *objectOut = kObjWater;
    distance = (d < distance) ? d : distance;
  }
  return distance;
}

template <typename T>
__device__ __noinline__ T calc_distance_runtime(const FractalT<T> *__restrict__ fp, V3<T> point, const T detailSize,
                                               const int N, const int minN, const bool normalMode, int *Lio,
                                               bool *maxIter, unsigned long long *orbit, unsigned long long *calls,
                                               int *objectOut, const T fparam) {
  const FractalT<T> &f = *fp;
  *objectOut = kObjFractal;
  T limitBoxDist = T(0);
  if (f.limits) {
    const T ax = point.x - f.amax, bx = -(point.x - f.amin);
    const T ay = point.y - f.bmax, by = -(point.y - f.bmin);
    const T az = point.z - f.cmax, bz = -(point.z - f.cmin);
    const T da = ax > bx ? ax : bx;
    const T db = ay > by ? ay : by;
    const T dc = az > bz ? az : bz;
    limitBoxDist = (da > db) ? ((da > dc) ? da : dc) : ((db > dc) ? db : dc);
    if (limitBoxDist > detailSize) {
      *maxIter = false;
      return limitBoxDist;
    }
  }
  T distance;
  bool mi;
  if (f.onlyPlane) {
    distance = T(10);
    mi = false;
  } else if (f.analytic) {
    int L;
    distance = compute_runtime<T, kModeNormal>(fp, point, N, 0, &L, fparam);
    *orbit += (unsigned long long)(L + 1);
    *calls += 1;
    mi = (L == N);
    *Lio = L;
    if (distance < T(0)) distance = T(0);
    if (L < minN && distance < detailSize) distance = detailSize;
    if (f.interiorMode && !normalMode) {
      if (distance < T(0.5) * detailSize || L == N) { distance = detailSize; mi = false; }
    } else if (f.interiorMode && normalMode) {
      if (distance < T(0.9) * detailSize) { distance = detailSize - distance; mi = false; }
    }
    if (f.iterThresh && L < N) {
      if (distance < detailSize) distance = detailSize * T(1.01);
    }
  } else {
    const T deltaDE = T(1e-10);
    int L;
    const T r = compute_runtime<T, kModeDelta1>(fp, point, N, 0, &L, fparam);
    *orbit += (unsigned long long)(L + 1);
    const int retval = L;
    *Lio = L;
    point.x += deltaDE;
    point.y += T(0);
    point.z += T(0);
    T r2 = compute_runtime<T, kModeDelta2>(fp, point, N, L, &L, fparam);
    *orbit += (unsigned long long)(L + 1);
    const T dr1 = m_fabs(r2 - r) / deltaDE;
    point.x -= deltaDE;
    point.y += deltaDE;
    point.z += T(0);
    r2 = compute_runtime<T, kModeDelta2>(fp, point, N, L, &L, fparam);
    *orbit += (unsigned long long)(L + 1);
    const T dr2 = m_fabs(r2 - r) / deltaDE;
    point.x += T(0);
    point.y -= deltaDE;
    point.z += deltaDE;
    r2 = compute_runtime<T, kModeDelta2>(fp, point, N, L, &L, fparam);
    *orbit += (unsigned long long)(L + 1);
    *calls += 4;
    const T dr3 = m_fabs(r2 - r) / deltaDE;
    const T dr = m_sqrt(dr1 * dr1 + dr2 * dr2 + dr3 * dr3);
    if (f.linearDE) distance = T(0.5) * r / dr;
    else distance = T(0.5) * r * m_log(r) / dr;
    if (distance < T(0)) distance = T(0);
    if (retval == N) {
      mi = true;
      distance = T(0);
    } else {
      mi = false;
    }
    if (L < minN && distance < detailSize) distance = detailSize;
    if (f.interiorMode && !normalMode) {
      if (distance < T(0.5) * detailSize || L == N) { distance = detailSize; mi = false; }
    } else if (f.interiorMode && normalMode) {
      if (distance < T(0.9) * detailSize) { distance = detailSize - distance; mi = false; }
    }
    if (f.iterThresh && retval < N) {
      if (distance < detailSize) distance = detailSize * T(1.01);
    }
  }
  distance = primitives(f, point, distance, objectOut);
  if (f.limits) {
    if (limitBoxDist < detailSize) distance = (distance > limitBoxDist) ? distance : limitBoxDist;
  }
  *maxIter = mi;
  return distance;
}

}  // namespace dev
}  // namespace mbgb
