// ORACLE — test infrastructure, not product code.
//
// A plain double-precision CPU restatement of Mandelbulber 1.21's per-pixel
// distance-estimated ray march, used (1) by the GPU parity tests as the checker
// and (2) by bench.py as the timed CPU baseline. It shares no code with the
// CUDA renderer. Parity of this restatement with the reference itself is pinned
// by tests/test_oracle_golden.py against golden vectors that
// tests/golden/make_golden.py produced by running the reference's own compiled
// fractal.cpp / shaders.cpp (oracle/_ref).
//
// Function-by-function sources (reference paths):
//   compute                           Compute<normal|colouring|deltaDE1|deltaDE2> src/fractal.cpp:40-1241
//                                     (every formula from trig_DE 1 to generalizedFoldBox 37, the
//                                     IFS / tglad / spherical pre-folds, the hybrid sequence)
//   derive                            RecalculateIFSParams / CreateFormulaSequence src/callbacks.cpp:1538-1702
//   calculate_distance                CalculateDistance, analytic and delta-DE src/fractal.cpp:1245-1448
//   ray_marching                      RayMarching                src/Render3D.cpp:79-199
//   calculate_normals                 CalculateNormals           src/shaders.cpp:675-757
//   main_shadow                       MainShadow                 src/shaders.cpp:480-570
//   fast_ao / ray_ao                  FastAmbientOcclusion2 / AmbientOcclusion src/shaders.cpp:585-673
//   surface_colour, index_to_colour   SurfaceColour / IndexToColour src/shaders.cpp:813-879, 1273-1305
//   background                        BackgroundShader           src/shaders.cpp:114-183
//   volumetric                        VolumetricShader           src/shaders.cpp:185-478
//   render_rows                       MainThread pixel body      src/Render3D.cpp:213-344, 389-589
//   compile16                         CompileImage / CalculatePixel / CalculateGammaTable src/cimage.cpp:132-214
//   ssao                              PostRendering_SSAO / ThreadSSAO src/image.cpp:249-478
//   oracle_dof                        PostRendering_DOF / QuickSortZBuffer src/image.cpp:57-206
//   level_set                         (not in the reference) Newton refinement of a hit onto
//                                     DE(P) = thr, the surface the differentiable render's
//                                     gradients are checked on; off unless oracle_render_exact
// Build: oracle/Makefile, -O2 -ffp-contract=off (parity) and -O3 -ffast-math (timing).
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include "../include/mbgb.h"

namespace {

struct Vec {
  double x, y, z;
};
inline Vec add(Vec a, Vec b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec sub(Vec a, Vec b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec mul(Vec a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double len(Vec a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline Vec normalize(Vec a) {
  double n = 1.0 / len(a);
  return {a.x * n, a.y * n, a.z * n};
}
inline Vec rot(const double *m, int zero, Vec v) {
  if (zero) return v;
  return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z, m[6] * v.x + m[7] * v.y + m[8] * v.z};
}
// x86-64 conversion results (cvttsd2si into a 32-bit register)
inline int to_i32(double v) { return (v >= -2147483648.0 && v < 2147483648.0) ? (int)v : (int)0x80000000u; }
inline unsigned short to_u16(double v) { return (unsigned short)to_i32(v); }
inline unsigned char to_u8(double v) { return (unsigned char)to_i32(v); }

struct Cnt {
  uint64_t orbit = 0, calls = 0, steps = 0;
};

// What RecalculateIFSParams and CreateFormulaSequence (src/callbacks.cpp:1538-1702) prepare
// for the orbit: the IFS rotation matrices, the generalized fold box's face normals and the
// hybrid formula sequence.
struct Derived {
  double ifsMain[9];
  int ifsMainZero;
  double ifsRot[9][9];
  int ifsRotZero[9];
  int gfbSides = 0;
  Vec gfb[20];
  std::vector<int> seqFormula;
  std::vector<double> seqPower;
};

// CRotationMatrix::SetRotation(alfa, beta, gamma): Z(alfa), then Y(beta), then X(gamma),
// each skipped for a zero angle (src/algebra.cpp:94-159).
void set_rotation(double a, double b, double g, double *m, int *zero) {
  const double id[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  memcpy(m, id, sizeof(id));
  *zero = 1;
  auto mulm = [&](const double r[9]) {
    double o[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) o[3 * i + j] = m[3 * i] * r[j] + m[3 * i + 1] * r[3 + j] + m[3 * i + 2] * r[6 + j];
    memcpy(m, o, sizeof(o));
    *zero = 0;
  };
  if (a != 0.0) { const double sn = sin(a), cs = cos(a); const double r[9] = {cs, -sn, 0, sn, cs, 0, 0, 0, 1}; mulm(r); }
  if (b != 0.0) { const double sn = sin(b), cs = cos(b); const double r[9] = {cs, 0, sn, 0, 1, 0, -sn, 0, cs}; mulm(r); }
  if (g != 0.0) { const double sn = sin(g), cs = cos(g); const double r[9] = {1, 0, 0, 0, cs, -sn, 0, sn, cs}; mulm(r); }
}

void derive(const mbgb_scene &s, Derived &d) {
  set_rotation(s.ifsRotationAlfa, s.ifsRotationBeta, s.ifsRotationGamma, d.ifsMain, &d.ifsMainZero);
  for (int i = 0; i < 9; i++) set_rotation(s.ifsAlfa[i], s.ifsBeta[i], s.ifsGamma[i], d.ifsRot[i], &d.ifsRotZero[i]);
  // face normals (src/callbacks.cpp:1557-1663)
  const double q = 1.0 / sqrt(3.0);
  const Vec oct[8] = {{q, q, -q}, {q, -q, q}, {-q, q, q}, {-q, -q, -q}, {q, q, q}, {-q, -q, q}, {-q, q, -q}, {q, -q, -q}};
  const Vec cube[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  const double aa = (1.0 + sqrt(5.0)) / 2.0;
  const double bb = 1.0 / sqrt(aa * aa + 1.0);
  const double ff = sqrt(aa * aa + 1.0 / (aa * aa));
  const double cc = aa / ff, dd = 1.0 / aa / ff;
  int n = 0;
  auto put = [&](const Vec *v, int k) {
    for (int i = 0; i < k; i++) d.gfb[n++] = v[i];
  };
  switch (s.genFoldBoxType) {
    case 1: put(cube, 6); break;
    case 2: put(oct, 8); break;
    case 3: {
      const Vec v[12] = {{0, bb, aa * bb}, {0, bb, -aa * bb}, {0, -bb, aa * bb}, {0, -bb, -aa * bb},
                         {bb, aa * bb, 0}, {bb, -aa * bb, 0}, {-bb, aa * bb, 0}, {-bb, -aa * bb, 0},
                         {aa * bb, 0, bb}, {-aa * bb, 0, bb}, {aa * bb, 0, -bb}, {-aa * bb, 0, -bb}};
      put(v, 12);
      break;
    }
    case 4: put(oct, 8); put(cube, 6); break;
    case 5: {
      const Vec v[12] = {{0, dd, cc}, {0, dd, -cc}, {0, -dd, cc}, {0, -dd, -cc}, {cc, 0, dd}, {cc, 0, -dd},
                         {-cc, 0, dd}, {-cc, 0, -dd}, {dd, cc, 0}, {dd, -cc, 0}, {-dd, cc, 0}, {-dd, -cc, 0}};
      put(oct, 8);
      put(v, 12);
      break;
    }
    case 6: case 7: {
      const int k = s.genFoldBoxType == 6 ? 6 : 5;
      const double th = 3.14159 * 2.0 / (k == 6 ? 6.0 : 5.0);
      const Vec caps[2] = {{0, 0, 1}, {0, 0, -1}};
      put(caps, 2);
      for (int i = 0; i < k; i++) d.gfb[n++] = Vec{cos(th * i), sin(th * i), 0};
      break;
    }
    default: put(oct, 4); break;
  }
  d.gfbSides = n;
  // CreateFormulaSequence
  const int N = (int)s.N;
  d.seqFormula.assign(N > 0 ? N : 0, 0);
  d.seqPower.assign(N > 0 ? N : 0, 0.0);
  if (s.formula != MBGB_FORMULA_HYBRID || N <= 0) return;
  int number = 0, guard = 0;
  while (number < N && guard++ < 1000000) {
    for (int h = 0; h < 4; h++) {
      if (s.hybridFormula[h] == 0) continue;
      for (int i = 0; i < s.hybridIters[h]; i++) {
        if (number < N) { d.seqFormula[number] = s.hybridFormula[h]; d.seqPower[number] = s.hybridPower[h]; }
        number++;
      }
    }
    const int end = s.hybridCyclic ? s.hybridIters[4] : N;
    if (s.hybridFormula[4] != 0)
      for (int i = 0; i < end; i++) {
        if (number < N) { d.seqFormula[number] = s.hybridFormula[4]; d.seqPower[number] = s.hybridPower[4]; }
        number++;
      }
  }
}

// Mutable DE state that the reference keeps in its sFractal copy.
struct Calc {
  const mbgb_scene *s;
  int N;            // (int)doubles.N, changed by normals (x5) and colouring (x10)
  int minN;
  bool normalMode;
  double detail;    // doubles.detailSize
  int itersOut;
  Cnt *cnt;
  const Derived *d;
  int objectOut = 0;  // enumObjectType of the last CalculateDistance
};

enum { kNormal = 0, kColour = 1, kDelta1 = 3, kDelta2 = 4, kOrbitTrap = 5 };

bool box_like(int f) { return f == 8 || f == 17 || f == 18 || f == 37; }

// the generalized fold box's search for the nearest cutting plane along y + a l
int gfb_search(const Derived &d, double solid, Vec y, Vec l, int skip1, int skip2, bool origin, double &a) {
  a = 1;
  int side = -1;
  for (int i = 0; i < d.gfbSides; i++) {
    if (i == skip1 || i == skip2) continue;
    const double b = origin ? solid : solid - dot(y, d.gfb[i]);
    const double c = dot(l, d.gfb[i]);
    if ((c > 0) && ((a * c) > b)) { side = i; a = b / c; }
  }
  return side;
}

bool gfb_push(Vec &z, Vec x, double melt) {
  const Vec t = sub(x, z);
  if (dot(t, t) > melt * melt) {
    const double m = len(t);
    z = add(z, mul(t, 2 * (m - melt) / (m + .00000001)));
    return true;
  }
  return false;
}

// Compute<Mode> (src/fractal.cpp:40-1241); `count` is deltaDE2's iteration count.
double compute(const Calc &c, Vec z, int mode, int count, int *Lout) {
  const mbgb_scene &s = *c.s;
  const Derived &dv = *c.d;
  const int N = c.N;
  const int Nseq = (int)s.N;
  double distance = 0;
  double w = 0, cw = 0;
  double r_dz = 1;
  double p = s.power;
  const double fR2 = s.mboxFoldingSphericalFixed * s.mboxFoldingSphericalFixed;
  const double mR2 = s.mboxFoldingSphericalMin * s.mboxFoldingSphericalMin;
  const double f1 = fR2 / mR2;
  double tDE = 1.0, tCol = 1.0;
  double scale = s.mboxScale;
  int form = s.formula;
  const bool hybrid = form == MBGB_FORMULA_HYBRID;
  // trig_DE keeps its derivative as a vector in polar form
  Vec dz{1.0, 0.0, 0.0};
  double thdz = 0.0, phdz = 0.0;
  Vec cst = s.juliaMode ? Vec{s.julia[0], s.julia[1], s.julia[2]} : mul(z, s.constantFactor);
  double r = len(z);
  double minv = 1e200;
  double trapTotal = 0.0;
  const Vec mbOff{s.mboxOffset[0], s.mboxOffset[1], s.mboxOffset[2]};
  const Vec ifsOff{s.ifsOffset[0], s.ifsOffset[1], s.ifsOffset[2]};
  int L;
  for (L = 0; L < N; L++) {
    if (hybrid) {
      const int k = L < Nseq - 1 ? L : Nseq - 1;
      form = dv.seqFormula[k];
      p = dv.seqPower[k];
      scale = p;
    }
    if (s.ifsFoldingMode) {
      if (s.ifsAbsX) z.x = fabs(z.x);
      if (s.ifsAbsY) z.y = fabs(z.y);
      if (s.ifsAbsZ) z.z = fabs(z.z);
      for (int i = 0; i < 9; i++) {
        if (!s.ifsEnabled[i]) continue;
        z = rot(dv.ifsRot[i], dv.ifsRotZero[i], z);
        const Vec dir{s.ifsDirection[i][0], s.ifsDirection[i][1], s.ifsDirection[i][2]};
        const double l = dot(z, dir);
        if (l < s.ifsDistance[i]) z = sub(z, mul(mul(dir, 2.0), l - s.ifsDistance[i]));
      }
      z = add(rot(dv.ifsMain, dv.ifsMainZero, sub(z, ifsOff)), ifsOff);
      z = mul(z, s.ifsScale);
      z = sub(z, mul(ifsOff, s.ifsScale - 1.0));
      r = len(z);
    }
    if (s.tgladFoldingMode) {
      const double fl = s.foldingLimit, fv = s.foldingValue;
      if (z.x > fl) { z.x = fv - z.x; tCol *= 0.9; } else if (z.x < -fl) { z.x = -fv - z.x; tCol *= 0.9; }
      if (z.y > fl) { z.y = fv - z.y; tCol *= 0.9; } else if (z.y < -fl) { z.y = -fv - z.y; tCol *= 0.9; }
      if (z.z > fl) { z.z = fv - z.z; tCol *= 0.9; } else if (z.z < -fl) { z.z = -fv - z.z; tCol *= 0.9; }
      r = len(z);
    }
    if (s.sphericalFoldingMode) {
      const double a = s.foldingSphericalFixed * s.foldingSphericalFixed;
      const double b = s.foldingSphericalMin * s.foldingSphericalMin;
      const double r2 = r * r;
      const double k1 = a / b;
      if (r2 < b) { z = mul(z, k1); tDE *= k1; tCol += 1; }
      else if (r2 < a) { const double k2 = a / r2; z = mul(z, k2); tDE *= k2; tCol += 10; }
      r = len(z);
    }
    switch (form) {
      case 1: {  // trig_DE
        const double r1 = pow(r, p - 1.0);
        const double r2 = r1 * r;
        const double th = atan2(z.y, z.x);
        const double ph = -atan2(z.z, sqrt(z.x * z.x + z.y * z.y));
        if (mode == kNormal) {
          const double k = p * r1 * r_dz;
          const double a = (p - 1.0) * th + thdz;
          const double b = (p - 1.0) * ph + phdz;
          dz = Vec{cos(b) * cos(a) * k + 1.0, cos(b) * sin(a) * k + 0.0, sin(b) * k + 0.0};
          r_dz = len(dz);
          thdz = atan2(dz.y, dz.x);
          phdz = -atan2(dz.z, sqrt(dz.x * dz.x + dz.y * dz.y));
        }
        z = add(mul(Vec{cos(p * ph) * cos(p * th), cos(p * ph) * sin(p * th), sin(p * ph)}, r2), cst);
        r = len(z);
        break;
      }
      case 2: {  // trig_optim
        const double th0 = asin(z.z / r);
        const double ph0 = atan2(z.y, z.x);
        double rp = pow(r, p - 1.0);
        const double th = th0 * p, ph = ph0 * p;
        const double cth = cos(th);
        r_dz = rp * r_dz * p + 1.0;
        rp *= r;
        z = add(mul(Vec{cth * cos(ph), cth * sin(ph), sin(th)}, rp), cst);
        r = len(z);
        break;
      }
      case 3: case 6: {  // fast_trig, minus_fast_trig
        const double x2 = z.x * z.x, y2 = z.y * z.y, z2 = z.z * z.z;
        const double t = 1.0 - z2 / (x2 + y2);
        const double nx = (x2 - y2) * t;
        const double ny = 2.0 * z.x * z.y * t;
        const double nz = (form == 3 ? -2.0 : 2.0) * z.z * sqrt(x2 + y2);
        z = Vec{nx + cst.x, ny + cst.y, nz + cst.z};
        r = len(z);
        break;
      }
      case 4: {  // hypercomplex
        const Vec nz{z.x * z.x - z.y * z.y - z.z * z.z - w * w, 2.0 * z.x * z.y - 2.0 * w * z.z, 2.0 * z.x * z.z - 2.0 * z.y * w};
        const double nw = 2.0 * z.x * w - 2.0 * z.y * z.z;
        z = add(nz, cst);
        w = nw;
        r = sqrt(z.x * z.x + z.y * z.y + z.z * z.z + w * w);
        break;
      }
      case 5: {  // quaternion
        const Vec nz{z.x * z.x - z.y * z.y - z.z * z.z - w * w, 2.0 * z.x * z.y, 2.0 * z.x * z.z};
        const double nw = 2.0 * z.x * w;
        z = add(nz, cst);
        w = nw;
        r = sqrt(z.x * z.x + z.y * z.y + z.z * z.z + w * w);
        break;
      }
      case 7: {  // menger_sponge
        z = Vec{fabs(z.x), fabs(z.y), fabs(z.z)};
        if (z.x - z.y < 0) std::swap(z.x, z.y);
        if (z.x - z.z < 0) std::swap(z.x, z.z);
        if (z.y - z.z < 0) std::swap(z.y, z.z);
        if (mode == kColour) {
          const double l = len(z);
          if (l < minv) minv = l;
        }
        z = mul(z, 3.0);
        z.x -= 2.0;
        z.y -= 2.0;
        if (z.z > 1.0) z.z -= 2.0;
        r = len(z);
        tDE *= 3.0;
        break;
      }
      case 8: {  // tglad
        const double fl = s.mboxFoldingLimit, fv = s.mboxFoldingValue;
        if (s.mboxRotationsEnabled) {
          bool lock = false;
          z = rot(s.mboxRot[0][0], s.mboxRotZero[0][0], z);
          if (z.x > fl) { z.x = fv - z.x; tCol += s.mboxColorFactorX; lock = true; }
          z = rot(s.mboxRotInv[0][0], 0, z);
          z = rot(s.mboxRot[1][0], s.mboxRotZero[1][0], z);
          if (!lock && z.x < -fl) { z.x = -fv - z.x; tCol += s.mboxColorFactorX; }
          z = rot(s.mboxRotInv[1][0], 0, z);
          lock = false;
          z = rot(s.mboxRot[0][1], s.mboxRotZero[0][1], z);
          if (z.y > fl) { z.y = fv - z.y; tCol += s.mboxColorFactorY; lock = true; }
          z = rot(s.mboxRotInv[0][1], 0, z);
          z = rot(s.mboxRot[1][1], s.mboxRotZero[1][1], z);
          if (!lock && z.y < -fl) { z.y = -fv - z.y; tCol += s.mboxColorFactorY; }
          z = rot(s.mboxRotInv[1][1], 0, z);
          lock = false;
          z = rot(s.mboxRot[0][2], s.mboxRotZero[0][2], z);
          if (z.z > fl) { z.z = fv - z.z; tCol += s.mboxColorFactorZ; lock = true; }
          z = rot(s.mboxRotInv[0][2], 0, z);
          z = rot(s.mboxRot[1][2], s.mboxRotZero[1][2], z);
          if (!lock && z.z < -fl) { z.z = -fv - z.z; tCol += s.mboxColorFactorZ; }
          z = rot(s.mboxRotInv[1][2], 0, z);
        } else {
          if (z.x > fl) { z.x = fv - z.x; tCol += s.mboxColorFactorX; } else if (z.x < -fl) { z.x = -fv - z.x; tCol += s.mboxColorFactorX; }
          if (z.y > fl) { z.y = fv - z.y; tCol += s.mboxColorFactorY; } else if (z.y < -fl) { z.y = -fv - z.y; tCol += s.mboxColorFactorY; }
          if (z.z > fl) { z.z = fv - z.z; tCol += s.mboxColorFactorZ; } else if (z.z < -fl) { z.z = -fv - z.z; tCol += s.mboxColorFactorZ; }
        }
        r = len(z);
        const double r2 = r * r;
        z = add(z, mbOff);
        if (r2 < mR2) { z = mul(z, f1); tDE *= f1; tCol += s.mboxColorFactorSp1; }
        else if (r2 < fR2) { const double f2 = fR2 / r2; z = mul(z, f2); tDE *= f2; tCol += s.mboxColorFactorSp2; }
        z = sub(z, mbOff);
        z = rot(s.mboxMainRot, s.mboxMainRotZero, z);
        z = add(mul(z, scale), cst);
        tDE = tDE * fabs(scale) + 1.0;
        r = len(z);
        break;
      }
      case 10: {  // kaleidoscopic
        if (s.ifsAbsX) z.x = fabs(z.x);
        if (s.ifsAbsY) z.y = fabs(z.y);
        if (s.ifsAbsZ) z.z = fabs(z.z);
        for (int i = 0; i < 9; i++) {
          if (!s.ifsEnabled[i]) continue;
          z = rot(dv.ifsRot[i], dv.ifsRotZero[i], z);
          const Vec dir{s.ifsDirection[i][0], s.ifsDirection[i][1], s.ifsDirection[i][2]};
          const double l = dot(z, dir);
          if (l < s.ifsDistance[i]) z = sub(z, mul(dir, 2.0 * (l - s.ifsDistance[i]) * s.ifsIntensity[i]));
        }
        z = add(rot(dv.ifsMain, dv.ifsMainZero, sub(z, ifsOff)), ifsOff);
        if (s.ifsEdge[0] > 0) z.x = s.ifsEdge[0] - fabs(s.ifsEdge[0] - z.x);
        if (s.ifsEdge[1] > 0) z.y = s.ifsEdge[1] - fabs(s.ifsEdge[1] - z.y);
        if (s.ifsEdge[2] > 0) z.z = s.ifsEdge[2] - fabs(s.ifsEdge[2] - z.z);
        if (mode == kColour) {
          const double l2 = len(z);
          if (l2 < minv) minv = l2;
        }
        z = mul(z, s.ifsScale);
        if (s.ifsMengerSpongeMode) {
          z.x -= s.ifsOffset[0] * (s.ifsScale - 1.0);
          z.y -= s.ifsOffset[1] * (s.ifsScale - 1.0);
          if (z.z > 0.5 * s.ifsOffset[2] * (s.ifsScale - 1.0)) z.z -= s.ifsOffset[2] * (s.ifsScale - 1.0);
        } else {
          z = sub(z, mul(ifsOff, s.ifsScale - 1.0));
        }
        tDE *= s.ifsScale;
        r = len(z);
        break;
      }
      case 11: {  // xenodreambuie
        const double rp = pow(r, p);
        const double th = atan2(z.y, z.x);
        double ph = acos(z.z / r);
        if (ph > 0.5 * M_PI) ph = M_PI - ph;
        else if (ph < -0.5 * M_PI) ph = -M_PI - ph;
        z = add(Vec{rp * cos(th * p) * sin(ph * p), rp * sin(th * p) * sin(ph * p), rp * cos(ph * p)}, cst);
        r = len(z);
        break;
      }
      case 13: case 14: {  // mandelbulb2, mandelbulb3
        double t, tr;
        double sg = 1.0, sg2 = 1.0;
        if (form == 14 && z.x < 0) sg2 = -1.0;
        tr = sqrt(z.x * z.x + z.y * z.y);
        z = mul(z, 1.0 / tr);
        t = z.x * z.x - z.y * z.y;
        z.y = 2.0 * z.x * z.y;
        z.x = t;
        z = mul(z, tr);
        if (form == 13) {
          tr = sqrt(z.y * z.y + z.z * z.z);
          z = mul(z, 1.0 / tr);
          t = z.y * z.y - z.z * z.z;
          z.z = 2.0 * z.y * z.z;
          z.y = t;
          z = mul(z, tr);
          tr = sqrt(z.x * z.x + z.z * z.z);
          z = mul(z, 1.0 / tr);
          t = z.x * z.x - z.z * z.z;
          z.z = 2.0 * z.x * z.z;
          z.x = t;
          z = mul(z, tr);
        } else {
          if (z.x < 0) sg = -1.0;
          tr = sqrt(z.x * z.x + z.z * z.z);
          z = mul(z, 1.0 / tr);
          t = z.x * z.x - z.z * z.z;
          z.z = 2.0 * z.x * z.z * sg2;
          z.x = t * sg;
          z = mul(z, tr);
        }
        z = mul(z, r);
        z = add(z, cst);
        r = len(z);
        break;
      }
      case 15: {  // mandelbulb4: identity, then RotateX, RotateY, RotateZ by (p - 1) x the angles
        const double rp = pow(r, p - 1);
        const double az = atan2(z.y, z.x), ay = atan2(z.z, z.x), ax = atan2(z.z, z.y);
        double m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        int zero = 1;
        auto mulm = [&](const double rr[9]) {
          double o[9];
          for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) o[3 * i + j] = m[3 * i] * rr[j] + m[3 * i + 1] * rr[3 + j] + m[3 * i + 2] * rr[6 + j];
          memcpy(m, o, sizeof(o));
          zero = 0;
        };
        const double a = ax * (p - 1), b = ay * (p - 1), g = az * (p - 1);
        if (a != 0.0) { const double sn = sin(a), cs = cos(a); const double rr[9] = {1, 0, 0, 0, cs, -sn, 0, sn, cs}; mulm(rr); }
        if (b != 0.0) { const double sn = sin(b), cs = cos(b); const double rr[9] = {cs, 0, sn, 0, 1, 0, -sn, 0, cs}; mulm(rr); }
        if (g != 0.0) { const double sn = sin(g), cs = cos(g); const double rr[9] = {cs, -sn, 0, sn, cs, 0, 0, 0, 1}; mulm(rr); }
        z = add(mul(rot(m, zero, z), rp), cst);
        r = len(z);
        break;
      }
      case 16: {  // foldingIntPow2
        const double F = s.FoldingIntPowFoldFactor;
        if (z.x > F) z.x = F * 2.0 - z.x; else if (z.x < -F) z.x = -F * 2.0 - z.x;
        if (z.y > F) z.y = F * 2.0 - z.y; else if (z.y < -F) z.y = -F * 2.0 - z.y;
        if (z.z > F) z.z = F * 2.0 - z.z; else if (z.z < -F) z.z = -F * 2.0 - z.z;
        r = len(z);
        const double rr = r * r;
        if (rr < 0.25) z = mul(z, 1.0 / 0.25);
        else if (rr < 1.0) z = mul(z, 1.0 / rr);
        z = mul(z, 2.0);
        const double x2 = z.x * z.x, y2 = z.y * z.y, z2 = z.z * z.z;
        const double t = 1.0 - z2 / (x2 + y2);
        z = Vec{(x2 - y2) * t + cst.x, 2.0 * z.x * z.y * t + cst.y, -2.0 * z.z * sqrt(x2 + y2) + cst.z};
        z.z *= s.FoldingIntPowZfactor;
        r = len(z);
        break;
      }
      case 17: {  // smoothMandelbox
        const double sm = s.mboxSharpness, fl = s.mboxFoldingLimit, fv = s.mboxFoldingValue;
        auto gt = [&](double a, double b) { return 1.0 / (1.0 + exp(sm * (b - a))); };
        auto lt = [&](double a, double b) { return 1.0 / (1.0 + exp(sm * (a - b))); };
        double *comp[3] = {&z.x, &z.y, &z.z};
        const double cf[3] = {s.mboxColorFactorX, s.mboxColorFactorY, s.mboxColorFactorZ};
        for (int k = 0; k < 3; k++) {
          double &v = *comp[k];
          const double k1 = gt(v, fl), k2 = lt(v, -fl);
          v = v * (1.0 - k1) + (fv - v) * k1;
          v = v * (1.0 - k2) + (-fv - v) * k2;
          tCol += (k1 + k2) * cf[k];
        }
        r = len(z);
        const double r2 = r * r;
        const double f2 = fR2 / r2;
        const double rk1 = lt(r2, mR2), rk2 = lt(r2, fR2);
        const double rk21 = (1.0 - rk1) * rk2;
        z = add(mul(z, 1.0 - rk1), mul(z, f1 * rk1));
        z = add(mul(z, 1.0 - rk21), mul(z, f2 * rk21));
        tDE = tDE * (1.0 - rk1) + tDE * (f1 * rk1);
        tDE = tDE * (1.0 - rk21) + tDE * (f2 * rk21);
        tCol += rk1 * s.mboxColorFactorSp1;
        tCol += rk21 * s.mboxColorFactorSp2;
        z = rot(s.mboxMainRot, s.mboxMainRotZero, z);
        z = add(mul(z, scale), cst);
        tDE = tDE * fabs(scale) + 1.0;
        r = len(z);
        break;
      }
      case 18: {  // mandelboxVaryScale4D
        scale = scale + s.mboxVaryScaleVary * (fabs(scale) - 1.0);
        const Vec o = z;
        const double fo = s.mboxVaryFold;
        z.x = fabs(z.x + fo) - fabs(z.x - fo) - z.x;
        z.y = fabs(z.y + fo) - fabs(z.y - fo) - z.y;
        z.z = fabs(z.z + fo) - fabs(z.z - fo) - z.z;
        w = fabs(w + fo) - fabs(w - fo) - w;
        if (z.x != o.x) tCol += s.mboxColorFactorX;
        if (z.y != o.y) tCol += s.mboxColorFactorY;
        if (z.z != o.z) tCol += s.mboxColorFactorZ;
        const double rr = pow(z.x * z.x + z.y * z.y + z.z * z.z + w * w, s.mboxVaryRPower);
        const double mr2 = s.mboxVaryMinR * s.mboxVaryMinR;
        double m = scale;
        if (rr < mr2) { m = scale / mr2; tCol += s.mboxColorFactorSp1; }
        else if (rr < 1.0) { m = scale / rr; tCol += s.mboxColorFactorSp2; }
        z = add(mul(z, m), cst);
        w = w * m + s.mboxVaryWadd;
        tDE = tDE * fabs(m) + 1.0;
        r = sqrt(z.x * z.x + z.y * z.y + z.z * z.z + w * w);
        break;
      }
      case 19: {  // aexion
        if (L == 0) {
          const double a = s.cadd;
          const Vec c0 = cst;
          cst = Vec{fabs(c0.x + c0.y + c0.z) + a, fabs(-c0.x - c0.y + c0.z) + a, fabs(-c0.x + c0.y - c0.z) + a};
          cw = fabs(c0.x - c0.y - c0.z) + a;
          const Vec z0 = z;
          z = Vec{fabs(z0.x + z0.y + z0.z) + a, fabs(-z0.x - z0.y + z0.z) + a, fabs(-z0.x + z0.y - z0.z) + a};
          w = fabs(z0.x - z0.y - z0.z) + a;
        }
        const double tx = z.x * z.x - z.y * z.y + 2.0 * w * z.z + cst.x;
        const double ty = z.y * z.y - z.x * z.x + 2.0 * w * z.z + cst.y;
        const double tz = z.z * z.z - w * w + 2.0 * z.x * z.y + cst.z;
        const double tw = w * w - z.z * z.z + 2.0 * z.x * z.y + cw;
        z = Vec{tx, ty, tz};
        w = tw;
        r = sqrt(z.x * z.x + z.y * z.y + z.z * z.z + w * w);
        break;
      }
      case 20: {  // benesi
        double r1 = z.y * z.y + z.z * z.z;
        const double nx = (cst.x < 0 || z.x < sqrt(r1)) ? z.x * z.x - r1 : -z.x * z.x + r1;
        r1 = -1.0 / sqrt(r1) * 2.0 * fabs(z.x);
        const double ny = r1 * (z.y * z.y - z.z * z.z);
        const double nz = r1 * 2.0 * z.y * z.z;
        z = Vec{nx + cst.x, ny + cst.y, nz + cst.z};
        r = len(z);
        break;
      }
      case 21: {  // bristorbrot
        const double nx = z.x * z.x - z.y * z.y - z.z * z.z;
        const double ny = z.y * (2.0 * z.x - z.z);
        const double nz = z.z * (2.0 * z.x + z.y);
        z = Vec{nx + cst.x, ny + cst.y, nz + cst.z};
        r = len(z);
        break;
      }
      case 22: case 23: case 24: {  // invertX, invertY, invertZ
        double &v = form == 22 ? z.x : (form == 23 ? z.y : z.z);
        v = v >= 0.0 ? v * v / (fabs(v) + p) : -v * v / (fabs(v) + p);
        r = len(z);
        break;
      }
      case 25: {  // invertR
        const double ri = r * r / (r + p);
        z = Vec{z.x / r * ri, z.y / r * ri, z.z / r * ri};
        r = len(z);
        break;
      }
      case 26: {  // sphericalFold
        const double rr = r * r, pp = p * p;
        if (rr < pp) z = Vec{1.0 / pp, 1.0 / pp, 1.0 / pp};
        else if (rr < pp * 4.0) z = Vec{1.0 / rr, 1.0 / rr, 1.0 / rr};
        r = len(z);
        break;
      }
      case 27: {  // powXYZ
        auto pw = [&](double v) { return v >= 0 ? pow(v, p) : -pow(-v, p); };
        z = Vec{pw(z.x), pw(z.y), pw(z.z)};
        r = len(z);
        break;
      }
      case 28: z.x *= p; r = len(z); break;
      case 29: z.y *= p; r = len(z); break;
      case 30: z.z *= p; r = len(z); break;
      case 31: z.x += p; r = len(z); break;
      case 32: z.y += p; r = len(z); break;
      case 33: z.z += p; r = len(z); break;
      case 34: {  // angleMultiplyX
        const double ang = atan2(z.z, z.y) * p;
        const double tr = sqrt(z.z * z.z + z.y * z.y);
        z.y = tr * cos(ang);
        z.z = tr * sin(ang);
        r = len(z);
        break;
      }
      case 35: {  // angleMultiplyY
        const double ang = atan2(z.z, z.x) * p;
        const double tr = sqrt(z.z * z.z + z.x * z.x);
        z.x = tr * cos(ang);
        z.z = tr * sin(ang);
        r = len(z);
        break;
      }
      case 36: {  // angleMultiplyZ
        const double ang = atan2(z.y, z.x) * p;
        const double tr = sqrt(z.x * z.x + z.y * z.y);
        z.x = tr * cos(ang);
        z.y = tr * sin(ang);
        r = len(z);
        break;
      }
      case 37: {  // generalizedFoldBox
        const double solid = s.mboxSolid, melt = s.mboxMelt;
        double a;
        const int sm = gfb_search(dv, solid, Vec{0, 0, 0}, z, -1, -1, true, a);
        if (sm != -1) {
          const Vec nm = dv.gfb[sm];
          const Vec xm = sub(z, mul(nm, dot(z, nm) - solid));
          Vec l = sub(xm, nm);
          Vec y = nm;
          const int sr = gfb_search(dv, solid, y, l, sm, -1, false, a);
          if (sr != -1) {
            const Vec xi = add(y, mul(l, a));
            const Vec nr = dv.gfb[sr];
            Vec lr{nm.y * nr.z - nm.z * nr.y, -nm.x * nr.z + nm.z * nr.x, nm.x * nr.y - nm.y * nr.x};
            double ar = (dot(z, lr) - dot(xi, lr)) / dot(lr, lr);
            if (ar < 0) { ar = -ar; lr = mul(lr, -1); }
            const Vec xr = add(xi, mul(lr, ar));
            l = sub(xr, xi);
            y = xi;
            const int si = gfb_search(dv, solid, y, l, sm, sr, false, a);
            if (si != -1) {
              if (gfb_push(z, add(y, mul(l, a)), melt)) tCol += s.mboxColorFactorZ;
            } else if (gfb_push(z, xr, melt)) {
              tCol += s.mboxColorFactorY;
            }
          } else if (gfb_push(z, xm, melt)) {
            tCol += s.mboxColorFactorX;
          }
        }
        r = len(z);
        const double r2 = r * r;
        z = add(z, mbOff);
        if (r2 < mR2) { z = mul(z, f1); tDE *= f1; tCol += s.mboxColorFactorSp1; }
        else if (r2 < fR2) { const double f2 = fR2 / r2; z = mul(z, f2); tDE *= f2; tCol += s.mboxColorFactorSp2; }
        z = sub(z, mbOff);
        z = rot(s.mboxMainRot, s.mboxMainRotZero, z);
        z = add(mul(z, scale), cst);
        tDE = tDE * fabs(scale) + 1.0;
        r = len(z);
        break;
      }
      default: break;
    }
    if (mode == kDelta1) {
      if (r > 1e10) break;
    } else if (mode == kDelta2) {
      if (L == count) break;
    }
    if (mode == kOrbitTrap) {  // src/fractal.cpp:1121-1131
      distance = len(sub(z, Vec{s.fakeLightsOrbitTrap[0], s.fakeLightsOrbitTrap[1], s.fakeLightsOrbitTrap[2]}));
      if (L >= s.fakeLightsMinIter && L <= s.fakeLightsMaxIter) trapTotal += (1.0f / (distance * distance));
      if (distance > 1000) {
        distance = trapTotal;
        break;
      }
    }
    if (form == 7 || form == 10) {
      if (r > 1000) { distance = (r - 2.0) / tDE; break; }
    } else if (box_like(form)) {
      if (r > 1024) { distance = r / fabs(tDE); break; }
    } else if (mode == kNormal) {
      // the reference's r > 100 (src/fractal.cpp:1151-1157), or the scene's bailoutRadius
      const double bail = s.bailoutRadius ? (double)s.bailoutRadius : 1e2;
      if (r > bail) { distance = 0.5 * r * log(r) / r_dz; break; }
    } else if (mode == kColour) {
      if (s.onlyPlane) {
        distance = len(z);
        if (distance > 1e15) { distance = (L - log(log(r) / log((double)N)) / log(p)) / 100.0; break; }
      } else {
        distance = len(z);
        if (distance < minv) minv = distance;
        if (distance > 1e15) { distance = minv; break; }
      }
    }
  }
  c.cnt->orbit += (uint64_t)(L + 1);
  c.cnt->calls++;
  if (Lout) *Lout = L;
  if (mode == kNormal) {
    if (L == N) distance = 0;
    return distance;
  }
  if (mode == kDelta1 || mode == kDelta2) return r;
  if (mode == kOrbitTrap) return distance;
  if (hybrid) {
    if (minv > 100) minv = 100;
    if (distance > 20) distance = 20;
    if (tCol > 1000) tCol = 1000;
    return distance * 5000.0 + tCol * 100.0 + minv * 1000.0;
  }
  if (box_like(form)) return tCol * 100.0 + len(z) * s.mboxColorFactorR;
  if (form == 7 || form == 10) return minv * 1000.0;
  return distance * 5000.0;
}

// PrimitiveWater (src/primitives.cpp:95-136)
double primitive_water(const mbgb_scene &s, Vec p) {
  double pd = dot(Vec{0, 0, -1}, sub(p, Vec{0, 0, s.waterHeight}));
  if (pd < s.waterAmplitude * 10.0) {
    const double a = s.waterRotation / 180 * M_PI;
    if (a != 0.0) {
      const double sn = sin(a), cs = cos(a);
      const double m[9] = {cs, -sn, 0, sn, cs, 0, 0, 0, 1};
      p = rot(m, 0, p);
    }
    const double phase = s.waterAnimSpeed * s.frameNo, k = 0.23, len_ = s.waterLength;
    double wx = 0, wy = 0, pw = 1.0, p2 = 0.05;
    for (int i = 1; i <= s.waterIterations; i++) {
      const float p3 = pw * p2;
      const double shift = phase / (i / 3.0 + 1.0);
      const double tx = sin(i + 0.4 * (wx)*p3 + sin(k * p.y / len_ * p3) + p.x / len_ * p3 + shift) / pw;
      const double ty = cos(i + 0.4 * (wy)*p3 + sin(p.x / len_ * p3) + k * p.y / len_ * p3 + shift * 0.23) / pw;
      wx += tx;
      wy += ty;
      p2 = p2 + (1.0 - p2) * 0.7;
      pw *= 1.872;
    }
    pd += (wx + wy) * s.waterAmplitude;
  }
  return pd;
}

// PrimitivePlane (src/primitives.cpp:15-21)
double primitive_plane(Vec p, Vec centre, Vec normal) { return dot(normalize(normal), sub(p, centre)); }

// the primitive objects of CalculateDistance (src/fractal.cpp:1383-1434)
double primitives(Calc &c, Vec p, double d) {
  const mbgb_scene &s = *c.s;
  auto take = [&](double q, int obj) {
    if (q < d) c.objectOut = obj;
    d = (q < d) ? q : d;
  };
  if (s.planeEnable) {
    const double q = primitive_plane(p, Vec{s.planeCentre[0], s.planeCentre[1], s.planeCentre[2]},
                                     Vec{s.planeNormal[0], s.planeNormal[1], s.planeNormal[2]});
    if (!s.onlyPlane && q < d) c.objectOut = 1;
    d = (q < d) ? q : d;
  }
  for (int inv = 0; inv < 2; inv++) {
    if (!(inv ? s.invertedBoxEnable : s.boxEnable)) continue;
    const double *ce = inv ? s.invertedBoxCentre : s.boxCentre;
    const double *sz = inv ? s.invertedBoxSize : s.boxSize;
    const Vec c1{ce[0] - 0.5 * sz[0], ce[1] - 0.5 * sz[1], ce[2] - 0.5 * sz[2]};
    const Vec c2{ce[0] + 0.5 * sz[0], ce[1] + 0.5 * sz[1], ce[2] + 0.5 * sz[2]};
    const double sg = inv ? 1.0 : -1.0;
    const Vec nrm[6] = {{sg, 0, 0}, {-sg, 0, 0}, {0, sg, 0}, {0, -sg, 0}, {0, 0, sg}, {0, 0, -sg}};
    double q = primitive_plane(p, c1, nrm[0]);
    for (int k = 1; k < 6; k++) {
      const double r = primitive_plane(p, (k & 1) ? c2 : c1, nrm[k]);
      q = inv ? ((r < q) ? r : q) : ((r > q) ? r : q);
    }
    take(q, inv ? 6 : 5);
  }
  if (s.sphereEnable) take(len(sub(p, Vec{s.sphereCentre[0], s.sphereCentre[1], s.sphereCentre[2]})) - s.sphereRadius, 3);
  if (s.invertedSphereEnable)
    take(s.invertedSphereRadius -
             len(sub(p, Vec{s.invertedSphereCentre[0], s.invertedSphereCentre[1], s.invertedSphereCentre[2]})),
         4);
  if (s.waterEnable) take(primitive_water(s, p), 2);
  return d;
}

double calculate_distance(Calc &c, Vec p, bool *max_iter) {
  const mbgb_scene &s = *c.s;
  c.objectOut = 0;
  double limit = 0.0;
  if (s.limits_enabled) {
    auto mx = [](double a, double b) { return a > b ? a : b; };
    const double da = mx(p.x - s.amax, -(p.x - s.amin));
    const double db = mx(p.y - s.bmax, -(p.y - s.bmin));
    const double dc = mx(p.z - s.cmax, -(p.z - s.cmin));
    limit = (da > db) ? ((da > dc) ? da : dc) : ((db > dc) ? db : dc);
    if (limit > c.detail) {
      if (max_iter) *max_iter = false;
      return limit;
    }
  }
  int L = c.itersOut;
  double d;
  int retval = 0;
  if (s.onlyPlane) {
    d = 10.0;
    if (max_iter) *max_iter = false;
  } else {
    if (s.analitycDE) {
      d = compute(c, p, kNormal, 0, &L);
      retval = L;
      if (max_iter) *max_iter = (L == c.N);
      c.itersOut = L;
      if (d < 0) d = 0;
    } else {
      // delta-DE: forward differences of the escape radius (src/fractal.cpp:1308-1381)
      const double h = 1e-10;
      const double r = compute(c, p, kDelta1, 0, &L);
      retval = L;
      c.itersOut = L;
      p.x += h; p.y += 0; p.z += 0;
      const double d1 = fabs(compute(c, p, kDelta2, L, &L) - r) / h;
      p.x -= h; p.y += h; p.z += 0;
      const double d2 = fabs(compute(c, p, kDelta2, L, &L) - r) / h;
      p.x += 0; p.y -= h; p.z += h;
      const double d3 = fabs(compute(c, p, kDelta2, L, &L) - r) / h;
      const double dr = sqrt(d1 * d1 + d2 * d2 + d3 * d3);
      d = s.linearDEmode ? 0.5 * r / dr : 0.5 * r * log(r) / dr;
      if (d < 0) d = 0;
      if (retval == c.N) {
        if (max_iter) *max_iter = true;
        d = 0;
      } else if (max_iter) {
        *max_iter = false;
      }
    }
    if (L < c.minN && d < c.detail) d = c.detail;
    if (s.interiorMode && !c.normalMode) {
      if (d < 0.5 * c.detail || L == c.N) {
        d = c.detail;
        if (max_iter) *max_iter = false;
      }
    } else if (s.interiorMode && c.normalMode) {
      if (d < 0.9 * c.detail) {
        d = c.detail - d;
        if (max_iter) *max_iter = false;
      }
    }
    if (s.iterThresh && retval < c.N) {
      if (d < c.detail) d = c.detail * 1.01;
    }
  }
  d = primitives(c, p, d);
  if (s.limits_enabled && limit < c.detail) d = d > limit ? d : limit;
  return d;
}

struct OLight {
  Vec pos;
  int col[3];
  double intensity;
  bool enabled;
};

struct Frame {
  const mbgb_scene *s;
  std::vector<OLight> lights;   // Lights[]
  int numberOfLights = 0;       // max(lightsPlaced, 4); 0 = no auxiliary lights at all
  double rm[9];
  int rzero;
  Vec start, light;
  std::vector<Vec> aoDirs;
  bool exact = false;   // level-set refinement of hits (oracle_render_exact)
  Derived d;
};

struct Step {
  double dist, step, thr;
  Vec point;   // sStep::point
  int iters;   // sStep::iters
};

struct Ray {
  bool found;
  int count;
  double thr, lastDist, depth;
  Vec point;
};

Ray ray_marching(const mbgb_scene &s, Calc &c, Vec start, Vec dir, std::vector<Step> &buf, bool jitter, Cnt &cnt,
                 double thrIn = 0.0) {
  Ray out{};
  Vec point{0, 0, 0};
  bool found = false;
  double scan = s.viewDistanceMin;
  // *distThreshOut: 0 for the camera ray, the previous ray's threshold for a reflection
  double thr = thrIn;
  const double thrInit = thrIn;
  double dist = 0;
  const double limit = 1.0 - 0.01 * s.quality;
  double step = s.viewDistanceMin;
  int count = 0;
  for (int i = 0; i < 10000; i++) {
    cnt.steps++;
    point = add(start, mul(dir, scan));
    bool mi = false;
    if (s.constantDEThreshold) thr = s.quality;
    else thr = scan * s.resolution * s.persp / s.quality + thrInit;
    if (s.perspectiveType == MBGB_PERSP_EQUIRECT || s.perspectiveType == MBGB_PERSP_FISH_EYE) thr *= M_PI;
    c.detail = thr;
    dist = calculate_distance(c, point, &mi);
    buf[i].dist = dist;
    buf[i].thr = thr;
    buf[i].iters = c.itersOut;
    if (dist > 3.0) dist = 3.0;
    if (dist < thr) {
      found = true;
      break;
    }
    buf[i].step = step;
    buf[i].point = point;
    const double j = jitter ? (1.0 - (rand() % 1001) / 10000.0) : 1.0;
    step = (dist - (s.interiorMode ? 0.8 : 0.5) * thr) * s.DE_factor * j;
    count++;
    scan += step;
    if (scan > s.viewDistanceMax) break;
  }
  if (found) {
    step *= 0.5;
    for (int i = 0; i < 20; i++) {
      cnt.steps++;
      if (dist < thr && dist > thr * limit) break;
      if (dist > thr) {
        scan += step;
        point = add(start, mul(dir, scan));
      } else if (dist < thr * limit) {
        scan -= step;
        point = add(start, mul(dir, scan));
      }
      if (s.constantDEThreshold) thr = s.quality;
      else thr = scan * s.resolution * s.persp / s.quality + thrInit;
      bool mi = false;
      dist = calculate_distance(c, point, &mi);
      step *= 0.5;
    }
  }
  out.found = found;
  out.count = count;
  out.thr = thr;
  out.lastDist = dist;
  out.depth = scan;
  out.point = point;
  return out;
}

// After RayMarching's bisection (hit inside the window (0.99 thr, thr)): Newton steps on
// F(t) = DE(start + t dir) - thr(t) with a central-difference derivative until
// |F| <= 1e-13 thr. Returns false (ray unchanged) on a flat estimate, a grazing ray
// (F' >= 0), a step longer than thr or no convergence in 16 steps.
bool level_set(const mbgb_scene &s, Calc &c, Vec start, Vec dir, Ray &ray) {
  const double k = s.constantDEThreshold ? 0.0 : s.resolution * s.persp / s.quality;
  const double dlen = len(dir);
  double t = ray.depth;
  for (int it = 0; it < 16; it++) {
    const double thr = s.constantDEThreshold ? s.quality : t * k;
    c.detail = thr;
    bool mi = false;
    const double d0 = calculate_distance(c, add(start, mul(dir, t)), &mi);
    if (mi || c.itersOut < c.minN) return false;
    const double F = d0 - thr;
    if (fabs(F) <= 1e-13 * thr) {
      ray.depth = t;
      ray.point = add(start, mul(dir, t));
      ray.thr = thr;
      ray.lastDist = d0;
      return true;
    }
    const double eps = 1e-6 * thr / dlen;
    const double dp = calculate_distance(c, add(start, mul(dir, t + eps)), &mi);
    const double dm = calculate_distance(c, add(start, mul(dir, t - eps)), &mi);
    const double Ft = (dp - dm) / (2.0 * eps) - k;
    if (!(Ft < 0.0)) return false;
    const double dt = -F / Ft;
    if (fabs(dt) > thr / dlen) return false;
    t += dt;
  }
  return false;
}

double iter_opacity(double step, double iters, double maxN, double trim, double sp) {
  double o = (iters - trim) / maxN;
  if (o < 0.0) o = 0.0;
  o *= o;
  o *= step * sp;
  if (o > 1.0) o = 1.0;
  return o;
}

// the float threshold of the secondary rays (MainShadow / AuxShadow / AmbientOcclusion)
float secondary_thresh(const mbgb_scene &s, Vec p2, Vec eye, double thr) {
  if (s.iterFogEnabled || s.volumetricLightEnabledAny) {
    if (!s.constantDEThreshold) return (float)(len(sub(p2, eye)) * s.resolution * s.persp / s.quality);
    return (float)s.quality;
  }
  return (float)thr;
}

Vec calculate_normals(const mbgb_scene &s, Calc &c, Vec p, double delta, double thr) {
  double d = delta * s.smoothness;
  if (s.interiorMode) d = thr * s.quality * 0.2 * s.smoothness;
  const int N0 = c.N, minN0 = c.minN;
  c.N = (int)(s.N * 5);
  c.minN = 0;
  c.normalMode = true;
  bool mi;
  Vec n{0, 0, 0};
  if (!s.slowShading) {
    const double s1 = calculate_distance(c, p, &mi);
    const double s2 = calculate_distance(c, Vec{p.x + d, p.y + 0.0, p.z + 0.0}, &mi);
    const double s3 = calculate_distance(c, Vec{p.x + 0.0, p.y + d, p.z + 0.0}, &mi);
    const double s4 = calculate_distance(c, Vec{p.x + 0.0, p.y + 0.0, p.z + d}, &mi);
    n = Vec{s2 - s1, s3 - s1, s4 - s1};
  } else {
    // averaged binary central difference (src/shaders.cpp:714-742): minN stays as it was
    c.minN = minN0;
    Vec q;
    for (q.x = -1.0; q.x <= 1.0; q.x += 0.2)
      for (q.y = -1.0; q.y <= 1.0; q.y += 0.2)
        for (q.z = -1.0; q.z <= 1.0; q.z += 0.2) n = add(n, mul(q, calculate_distance(c, add(p, mul(q, d)), &mi)));
  }
  c.N = N0;
  c.minN = minN0;
  c.normalMode = false;
  if (n.x == 0 && n.y == 0 && n.z == 0) n.x = 1;
  else n = normalize(n);
  return n;
}

double main_shadow(const mbgb_scene &s, Calc &c, Vec p, Vec light, double thr, double delta, Vec eye) {
  double factor = delta / s.resolution;
  if (!s.penetratingLights) factor = s.viewDistanceMax;
  double dist = thr;
  c.detail = thr;
  const double DE_factor = (s.iterFogEnabled || s.volumetricLightEnabledAny) ? 1.0 : s.DE_factor;
  double start = thr;
  if (s.interiorMode) start = thr * DE_factor;
  double shadowTemp = 1.0;
  const double softRange = tan(s.shadowConeAngle / 180.0 * M_PI);
  double maxSoft = 0.0;
  const bool bSoft = (!s.iterFogEnabled && !s.limits_enabled && !s.iterThresh) && softRange > 0.0;
  for (double i = start; i < factor; i += dist * DE_factor) {
    const Vec p2 = add(p, mul(light, i));
    const float thr_f = secondary_thresh(s, p2, eye, thr);  // the reference's float threshold
    c.detail = thr_f;
    bool mi;
    dist = calculate_distance(c, p2, &mi);
    if (bSoft) {
      double angle = (dist - thr_f) / i;
      if (angle < 0) angle = 0;
      if (dist < thr_f) angle = 0;
      double soft = (1.0 - angle / softRange);
      if (s.penetratingLights) soft *= (factor - i) / factor;
      if (soft < 0) soft = 0;
      if (soft > maxSoft) maxSoft = soft;
    }
    const double opacity = s.iterFogEnabled
                               ? iter_opacity(dist * DE_factor, c.itersOut, s.N, s.iterFogOpacityTrim, s.iterFogOpacity)
                               : 0.0;
    shadowTemp -= opacity * (factor - i) / factor;
    if (dist < thr_f || shadowTemp < 0.0) {
      shadowTemp -= (factor - i) / factor;
      if (!s.penetratingLights) shadowTemp = 0.0;
      if (shadowTemp < 0.0) shadowTemp = 0.0;
      break;
    }
  }
  return bSoft ? 1.0 - maxSoft : shadowTemp;
}

double fast_ao(const mbgb_scene &s, Calc &c, Vec p, Vec n, double thr) {
  double ao = 0;
  const double q = s.globalIlumQuality;
  for (int i = 1; i < q * q; i++) {
    const double scan = i * i * thr;
    bool mi;
    const double dist = calculate_distance(c, add(p, mul(n, scan)), &mi);
    ao += 1.0 / (pow(2.0, i)) * (scan - s.fastAoTune * dist) / thr;
  }
  double r = 1.0 - 0.2 * ao;
  return r < 0 ? 0 : r;
}

double ray_ao(const mbgb_scene &s, Calc &c, Vec p, double delta, double thr, double lastDist,
              const std::vector<Vec> &dirs, Vec eye) {
  const double end = delta / s.resolution;
  double AO = 0;
  for (const Vec &v : dirs) {
    double dist = lastDist;
    double sh = 1.0;
    for (double r = delta; r < end; r += dist * 2.0) {
      bool mi;
      const Vec p2 = add(p, mul(v, r));
      dist = calculate_distance(c, p2, &mi);
      const double opacity = s.iterFogEnabled
                                 ? iter_opacity(dist * 2.0, c.itersOut, s.N, s.iterFogOpacityTrim, s.iterFogOpacity)
                                 : 0.0;
      sh -= opacity * (end - r) / end;
      if (dist < secondary_thresh(s, p2, eye, thr) || mi || sh < 0.0) {
        sh -= (end - r) / end;
        if (sh < 0.0) sh = 0.0;
        break;
      }
    }
    AO += sh * 255;
  }
  return AO / (dirs.size() * 256.0);
}

// EnvMapping (src/shaders.cpp:785-811) on the default white 100 x 100 texture
double env_mapping(Vec n, Vec view) {
  const double d = -dot(view, n);
  const Vec r = add(mul(mul(n, 2.0), d), view);
  const double alfa = atan2(r.y, r.x) + M_PI;
  double beta = atan2(r.z, sqrt(r.x * r.x + r.y * r.y));
  if (beta > 0.5 * M_PI) beta = 0.5 * M_PI - beta;
  if (beta < -0.5 * M_PI) beta = -0.5 * M_PI + beta;
  double x = (alfa / (2.0 * M_PI)) * 100.0 + 100.0 * 8.25;
  double y = (beta / (M_PI) + 0.5) * 100.0 + 100.0 * 8.0;
  x = fmod(x, 100.0);
  y = fmod(y, 100.0);
  if (x < 0) x = 0;
  if (y < 0) y = 0;
  if (!(x >= 0 && x < 100 && y >= 0 && y < 100 - 1.0)) return 0.0;
  const double rx = (x - (int)x), ry = (y - (int)y);
  const unsigned char v = (unsigned char)(255 * (1.0 - rx) * (1.0 - ry) + 255 * (rx) * (1.0 - ry) +
                                          255 * (1.0 - rx) * ry + 255 * (rx * ry));
  return v / 256.0;
}

void index_to_colour(const mbgb_scene &s, int index, int out[3]) {
  if (index < 0) {
    out[0] = s.palette[255].R; out[1] = s.palette[255].G; out[2] = s.palette[255].B;
    return;
  }
  out[0] = out[1] = out[2] = 255;
  index = index % (255 * 256);
  const int kol = index / 256;
  if (kol < 255) {
    const int delta = index % 256;
    const int a[3] = {s.palette[kol].R, s.palette[kol].G, s.palette[kol].B};
    const int b[3] = {s.palette[kol + 1].R, s.palette[kol + 1].G, s.palette[kol + 1].B};
    for (int k = 0; k < 3; k++) {
      const double R1 = a[k], R2 = b[k];
      const double RK = (R2 - R1) / 256.0;
      out[k] = (int)(R1 + (RK * delta));
    }
  }
}

Vec surface_colour(const mbgb_scene &s, Calc &c, Vec p, int objectType) {
  const mbgb_rgb *prim[7] = {nullptr, &s.primitivePlaneColour, &s.primitiveWaterColour, &s.primitiveSphereColour,
                             &s.primitiveInvertedSphereColour, &s.primitiveBoxColour, &s.primitiveInvertedBoxColour};
  if (objectType != 0) return Vec{prim[objectType]->R / 65536.0, prim[objectType]->G / 65536.0,
                                  prim[objectType]->B / 65536.0};
  const int N0 = c.N;
  c.N = (int)(s.N * 10);
  int nr = to_i32(floor(compute(c, p, kColour, 0, nullptr)));
  c.N = N0;
  // abs(nrCol) % (248 * 256): the reference binary takes the magnitude as unsigned,
  // so an out-of-range conversion (INT_MIN) yields 2^31 % 63488 = 2048.
  const unsigned mag = nr < 0 ? 0u - (unsigned)nr : (unsigned)nr;
  nr = (int)(mag % (248u * 256u));
  int col[3] = {256, 256, 256};
  if (s.coloringEnabled) {
    int num;
    if (nr >= 248 * 256) num = nr;
    else num = to_i32(nr * s.coloring_speed + 256 * s.paletteOffset) % 65536;
    index_to_colour(s, num, col);
  }
  return {col[0] / 256.0, col[1] / 256.0, col[2] / 256.0};
}

Vec background(const mbgb_scene &s, Vec view) {
  const Vec v = normalize(Vec{0.0, 0.0, -1.0});
  double grad = (dot(view, v) + 1.0);
  const int c1[3] = {s.background_color1.R, s.background_color1.G, s.background_color1.B};
  const int c2[3] = {s.background_color2.R, s.background_color2.G, s.background_color2.B};
  const int c3[3] = {s.background_color3.R, s.background_color3.G, s.background_color3.B};
  unsigned short px[3];
  if (grad < 1) {
    const double ng = 1.0 - grad;
    for (int k = 0; k < 3; k++) px[k] = to_u16(c3[k] * ng + c2[k] * grad);
  } else {
    grad = grad - 1;
    const double ng = 1.0 - grad;
    for (int k = 0; k < 3; k++) px[k] = to_u16(c2[k] * ng + c1[k] * grad);
  }
  return {px[0] / 65536.0, px[1] / 65536.0, px[2] / 65536.0};
}

// AuxShadow (src/shaders.cpp:1069-1132)
double aux_shadow(const mbgb_scene &s, Calc &c, Vec p, double distance, Vec lv, double delta, double thr, Vec eye) {
  double dist = delta;
  double shadowTemp = 1.0;
  const double def = (s.iterFogEnabled || s.volumetricLightEnabledAny) ? 1.0 : s.DE_factor;
  for (double i = delta; i < distance; i += dist * def) {
    const Vec p2 = add(p, mul(lv, i));
    bool mi = false;
    dist = calculate_distance(c, p2, &mi);
    const double opacity = s.iterFogEnabled
                               ? iter_opacity(dist * def, c.itersOut, s.N, s.iterFogOpacityTrim, s.iterFogOpacity)
                               : 0.0;
    shadowTemp -= opacity * (distance - i) / distance;
    if (dist < secondary_thresh(s, p2, eye, thr) || mi || shadowTemp < 0.0) {
      if (s.penetratingLights) {
        shadowTemp -= (distance - i) / distance;
        if (shadowTemp < 0.0) shadowTemp = 0.0;
      } else {
        shadowTemp = 0.0;
      }
      break;
    }
  }
  return shadowTemp;
}

// AuxLightsShader / LightShading (src/shaders.cpp:997-1067)
void aux_lights(const mbgb_scene &s, const Frame &f, Calc &c, Vec p, Vec n, Vec view, double delta, double thr,
                double shade_out[3], double spec_out[3]) {
  for (int k = 0; k < 3; k++) shade_out[k] = spec_out[k] = 0.0;
  const int number = f.numberOfLights;
  for (int i = 0; i < number; i++) {
    const OLight &L = f.lights[(size_t)i];
    if (!(i < s.auxLightNumber || L.enabled)) continue;
    const Vec d = sub(L.pos, p);
    const double distance = len(d);
    const Vec lv = normalize(d);
    const double intensity = s.auxLightIntensity * 100.0 * L.intensity / (distance * distance) / number;
    double shade = dot(n, lv);
    if (shade < 0) shade = 0;
    shade = shade * intensity;
    if (shade > 500.0) shade = 500.0;
    const Vec half = normalize(sub(lv, view));
    double shade2 = dot(n, half);
    if (shade2 < 0.0) shade2 = 0.0;
    shade2 = pow(shade2, 30.0) * 1.0;
    shade2 *= intensity * s.specular;
    if (shade2 > 15.0) shade2 = 15.0;
    if ((shade > 0.01 || shade2 > 0.01) && s.shadow) {
      const double light = aux_shadow(s, c, p, distance, lv, delta, thr, f.start);
      shade *= light;
      shade2 *= light;
    } else if (s.shadow) {
      shade = 0;
      shade2 = 0;
    }
    for (int k = 0; k < 3; k++) {
      shade_out[k] += shade * L.col[k] / 65536.0;
      spec_out[k] += shade2 * L.col[k] / 65536.0;
    }
  }
}

void volumetric(const mbgb_scene &s, const Frame &f, Calc &c, const std::vector<Step> &buf, int count, double depth,
                Vec view, double delta, double lastDist, double out[4], float *opacity) {
  float total = 0.0f;
  const double glow = count * s.glow_intensity / 512.0 * s.DE_factor;
  double glowN = 1.0 - glow;
  if (glowN < 0.0) glowN = 0.0;
  const double gR = (s.glow_color1.R * glowN + s.glow_color2.R * glow) / 65536.0;
  const double gG = (s.glow_color1.G * glowN + s.glow_color2.G * glow) / 65536.0;
  const double gB = (s.glow_color1.B * glowN + s.glow_color2.B * glow) / 65536.0;
  const double fogVis = pow(10.0, s.fogVisibility / 10 - 16.0);
  const double ct1 = s.fogColour1Distance, ct2 = s.fogColour2Distance, red = s.fogDistanceFactor, I = s.fogDensity;
  double acc = 0.0;
  for (int k = count - 1; k > 0; k--) {
    double step = buf[k].step;
    const double d = buf[k].dist;
    acc += step;
    if (acc < buf[k].thr * s.quality) continue;
    step = acc;
    acc = 0.0;
    const double go = glow * step / depth;
    out[0] = go * gR + (1.0 - go) * out[0];
    out[1] = go * gG + (1.0 - go) * out[1];
    out[2] = go * gB + (1.0 - go) * out[2];
    out[3] += go;
    // visible auxiliary lights (src/shaders.cpp:242-296)
    if (s.auxLightVisibility > 0 && f.numberOfLights > 0) {
      const Vec point = buf[k].point;
      double lowSize = 1e10, lowDist = 1e10;
      for (int i = 0; i < f.numberOfLights; ++i) {
        const OLight &L = f.lights[(size_t)i];
        if (!(i < s.auxLightNumber || L.enabled)) continue;
        const double ld = len(sub(point, L.pos));
        const double size = L.intensity * s.auxLightIntensity * s.auxLightVisibility;
        const double r2 = ld / size;
        if (r2 < lowSize) {
          lowSize = r2;
          lowDist = ld;
        }
      }
      int small = to_i32(10.0 * step / (lowDist + 1.0e-20));
      if (small > 50) small = 50;
      int s0 = 0, s1 = 1;
      double step2 = step;
      if (small > 0) {
        s0 = 1;
        s1 = small + 1;
        step2 = step / (small + 1.0);
      }
      for (int ss = s0; ss < s1; ss++) {
        const Vec p2 = sub(point, mul(mul(view, step2), (double)ss));
        for (int i = 0; i < f.numberOfLights; ++i) {
          const OLight &L = f.lights[(size_t)i];
          if (!(i < s.auxLightNumber || L.enabled)) continue;
          const double ld = len(sub(p2, L.pos));
          const double size = L.intensity * s.auxLightIntensity * s.auxLightVisibility;
          double r2 = ld / size;
          if (r2 > 1.0) r2 = 1.0;
          const double bell = (cos(r2 * M_PI) + 1.0) / (r2 * r2 + 0.02) * 0.3;
          const double dens = step2 * bell / size;
          out[0] += dens * L.col[0] / 65536.0;
          out[1] += dens * L.col[1] / 65536.0;
          out[2] += dens * L.col[2] / 65536.0;
          out[3] += dens;
        }
      }
    }
    if (s.fakeLightsEnabled) {  // src/shaders.cpp:298-307
      double r = compute(c, buf[k].point, kOrbitTrap, 0, nullptr);
      r = sqrt(1.0f / (r + 1.0e-30f));
      const double fl = 1.0 / (pow(r, 10.0 / s.fakeLightsVisibilitySize) * pow(10.0, 10.0 / s.fakeLightsVisibilitySize) +
                               1e-100);
      for (int q = 0; q < 4; q++) out[q] += fl * step * s.fakeLightsVisibility;
    }
    for (int i = 0; i < 5; i++) {  // volumetric lights (src/shaders.cpp:309-343)
      if (i == 0 && s.volumetricLightEnabled[0]) {
        const double sh = main_shadow(s, c, buf[k].point, f.light, buf[k].thr, delta, f.start);
        out[0] += sh * step * s.volumetricLightIntensity[0] * s.mainLightColour.R / 65536.0;
        out[1] += sh * step * s.volumetricLightIntensity[0] * s.mainLightColour.G / 65536.0;
        out[2] += sh * step * s.volumetricLightIntensity[0] * s.mainLightColour.B / 65536.0;
        out[3] += (sh + sh + sh) / 3.0 * step * s.volumetricLightIntensity[0];
      }
      if (i > 0 && f.numberOfLights > 0 && f.lights[(size_t)i - 1].enabled && s.volumetricLightEnabled[i]) {
        const OLight &L = f.lights[(size_t)i - 1];
        const Vec d = sub(L.pos, buf[k].point);
        const double dd = len(d);
        const double d2 = dd * dd;
        const double light = aux_shadow(s, c, buf[k].point, dd, normalize(d), delta, buf[k].thr, f.start);
        for (int q = 0; q < 3; q++) out[q] += light * L.col[q] / 65536.0 * s.volumetricLightIntensity[i] * step / d2;
        out[3] += light * s.volumetricLightIntensity[i] * step / d2;
      }
    }
    if (s.fogEnabled) {
      double fd = step / fogVis;
      if (fd > 1.0) fd = 1.0;
      out[0] = fd * s.fogColor.R / 65536.0 + (1.0 - fd) * out[0];
      out[1] = fd * s.fogColor.G / 65536.0 + (1.0 - fd) * out[1];
      out[2] = fd * s.fogColor.B / 65536.0 + (1.0 - fd) * out[2];
      total = fd + (1.0 - fd) * total;
      out[3] = fd + (1.0 - fd) * out[3];
    }
    if (I > 0.0) {
      const double dt = (step * red) / (d * d + red * red);
      double kk = d / ct1;
      if (kk > 1) kk = 1.0;
      double kn = 1.0 - kk;
      double fr = (s.fogColour1.R * kn + s.fogColour2.R * kk);
      double fg = (s.fogColour1.G * kn + s.fogColour2.G * kk);
      double fb = (s.fogColour1.B * kn + s.fogColour2.B * kk);
      double k2 = d / ct2 * kk;
      if (k2 > 1) k2 = 1.0;
      kn = 1.0 - k2;
      fr = (fr * kn + s.fogColour3.R * k2);
      fg = (fg * kn + s.fogColour3.G * k2);
      fb = (fb * kn + s.fogColour3.B * k2);
      double fd = 0.3 * I * dt / (1.0 + I * dt);
      if (fd > 1) fd = 1.0;
      out[0] = fd * fr / 65536.0 + (1.0 - fd) * out[0];
      out[1] = fd * fg / 65536.0 + (1.0 - fd) * out[1];
      out[2] = fd * fb / 65536.0 + (1.0 - fd) * out[2];
      total = fd + (1.0 - fd) * total;
      out[3] = fd + (1.0 - fd) * out[3];
    }
    if (s.iterFogEnabled) {  // iteration fog (src/shaders.cpp:385-466)
      const int L = buf[k].iters;
      double op = iter_opacity(step, L, s.N, s.iterFogOpacityTrim, s.iterFogOpacity);
      if (op > 0) {
        const double itf = (double)2.0 * (L - s.iterFogOpacityTrim) / (s.N - s.iterFogOpacityTrim);
        double kk = itf;
        if (kk > 1.0) kk = 1.0;
        if (kk < 0.0) kk = 0.0;
        double kn = 1.0 - kk;
        const mbgb_rgb fc1 = s.fogColour1, fc2 = s.fogColour2, fc3 = s.fogColour3;
        double fcol[3] = {fc1.R * kn + fc2.R * kk, fc1.G * kn + fc2.G * kk, fc1.B * kn + fc2.B * kk};
        double k2 = itf - 1.0;
        if (k2 < 0.0) k2 = 0.0;
        if (k2 > 1.0) k2 = 1.0;
        kn = 1.0 - k2;
        fcol[0] = fcol[0] * kn + fc3.R * k2;
        fcol[1] = fcol[1] * kn + fc3.G * k2;
        fcol[2] = fcol[2] * kn + fc3.B * k2;
        double nc[3] = {0.0, 0.0, 0.0};
        if (s.mainLightIntensity * s.directLight > 0.0) {
          const double sh = main_shadow(s, c, buf[k].point, f.light, buf[k].thr, delta, f.start);
          nc[0] += sh * s.mainLightColour.R / 65536.0 * s.mainLightIntensity * s.directLight;
          nc[1] += sh * s.mainLightColour.G / 65536.0 * s.mainLightIntensity * s.directLight;
          nc[2] += sh * s.mainLightColour.B / 65536.0 * s.mainLightIntensity * s.directLight;
        }
        for (int i = 1; i < 5; i++) {
          if (!(f.numberOfLights > 0 && f.lights[(size_t)i - 1].enabled)) continue;
          const OLight &Lt = f.lights[(size_t)i - 1];
          const Vec dv = sub(Lt.pos, buf[k].point);
          const double dd = len(dv);
          const double d2 = dd * dd;
          const double light = aux_shadow(s, c, buf[k].point, dd, normalize(dv), delta, buf[k].thr, f.start);
          const double inten = Lt.intensity * 100.0;
          for (int q = 0; q < 3; q++) nc[q] += light * Lt.col[q] / 65536.0 / d2 * inten;
        }
        if (s.global_ilumination && !s.fastGlobalIllumination) {
          const double ao = ray_ao(s, c, buf[k].point, delta, buf[k].thr, lastDist, f.aoDirs, f.start);
          for (int q = 0; q < 3; q++) nc[q] += ao * s.globalIlum;
        }
        if (op > 1.0) op = 1.0;
        for (int q = 0; q < 3; q++) out[q] = out[q] * (1.0 - op) + nc[q] * op * fcol[q] / 65536.0;
        total = op + (1.0 - op) * total;
        out[3] = op + (1.0 - op) * out[3];
      }
    }
    if (total > 1.0) total = 1.0;
    if (out[3] > 1.0) out[3] = 1.0;
    *opacity = total;
  }
}


// PlaceRandomLights (src/shaders.cpp:1134-1208), with the C library's srand / rand.
void place_lights(const mbgb_scene &s, const Derived &d, std::vector<OLight> &L) {
  const int nr = s.auxLightNumber > 0 ? s.auxLightNumber : 0;
  L.assign((size_t)nr + 4, OLight{});
  srand((unsigned)s.auxLightRandomSeed);
  auto rnd = [](int max) { return rand() % (max + 1); };
  Cnt cnt;
  Calc c{&s, (int)s.N, s.minN, false, 0.0, 0, &cnt, &d};
  int trial = 0;
  double rm = 1.0;
  long long guard = 0;
  for (int i = 0; i < nr && guard < 20000000; i++, guard++) {
    trial++;
    double r[3];
    for (int k = 0; k < 3; k++) {
      const int a = rnd(2000000);
      const int b = rnd(1000000);
      r[k] = (a / 1000000.0 - 1.0) + (b / 1.0e12);
    }
    const Vec pos{s.auxLightRandomCenter[0] + r[0] * s.auxLightDistributionRadius * rm,
                  s.auxLightRandomCenter[1] + r[1] * s.auxLightDistributionRadius * rm,
                  s.auxLightRandomCenter[2] + r[2] * s.auxLightDistributionRadius * rm};
    bool mi = false;
    c.detail = 0.0;
    const double dist = calculate_distance(c, pos, &mi);
    if (trial > 1000) {
      rm *= 1.1;
      trial = 0;
    }
    if (dist > 0 && !mi && dist < s.auxLightMaxDist * rm) {
      rm = 1.0;
      L[i].pos = pos;
      int col[3];
      for (int k = 0; k < 3; k++) col[k] = 20000 + rnd(80000);
      const double a = col[0], b = col[1], cc = col[2];
      const double mx = (a > b) ? ((a > cc) ? a : cc) : ((b > cc) ? b : cc);
      for (int k = 0; k < 3; k++) L[i].col[k] = (int)(col[k] * 65536.0 / mx);
      L[i].intensity = dist * dist / s.auxLightMaxDist;
      L[i].enabled = true;
    } else {
      i--;
    }
  }
  for (int i = 0; i < 4; i++) {
    if (s.auxLightPreEnabled[i]) {
      L[i].pos = Vec{s.auxLightPre[i][0], s.auxLightPre[i][1], s.auxLightPre[i][2]};
      L[i].intensity = s.auxLightPreIntensity[i];
      L[i].col[0] = s.auxLightPreColour[i].R;
      L[i].col[1] = s.auxLightPreColour[i].G;
      L[i].col[2] = s.auxLightPreColour[i].B;
      L[i].enabled = true;
    } else {
      L[i].enabled = false;
    }
  }
}

void setup_frame(const mbgb_scene &s, Frame &f) {
  f.s = &s;
  derive(s, f.d);
  bool anyPre = false;
  for (int i = 0; i < 4; i++) anyPre = anyPre || s.auxLightPreEnabled[i];
  if (s.auxLightNumber > 0 || anyPre) {
    place_lights(s, f.d, f.lights);
    f.numberOfLights = s.auxLightNumber > 4 ? s.auxLightNumber : 4;
  }
  // RotateZ(alpha) * RotateX(beta) * RotateY(gamma), identity short-cut when all zero
  double m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  int zero = 1;
  auto mulm = [&](const double r[9]) {
    double o[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) o[3 * i + j] = m[3 * i] * r[j] + m[3 * i + 1] * r[3 + j] + m[3 * i + 2] * r[6 + j];
    memcpy(m, o, sizeof(o));
    zero = 0;
  };
  if (s.alpha != 0.0) { const double sn = sin(s.alpha), cs = cos(s.alpha); const double r[9] = {cs, -sn, 0, sn, cs, 0, 0, 0, 1}; mulm(r); }
  if (s.beta != 0.0) { const double sn = sin(s.beta), cs = cos(s.beta); const double r[9] = {1, 0, 0, 0, cs, -sn, 0, sn, cs}; mulm(r); }
  if (s.gamma != 0.0) { const double sn = sin(s.gamma), cs = cos(s.gamma); const double r[9] = {cs, 0, sn, 0, 1, 0, -sn, 0, cs}; mulm(r); }
  memcpy(f.rm, m, sizeof(m));
  f.rzero = zero;
  const Vec baseY = rot(f.rm, f.rzero, Vec{0.0, 1.0, 0.0});
  const Vec vp{s.vp[0], s.vp[1], s.vp[2]};
  if (s.perspectiveType == MBGB_PERSP_FISH_EYE || s.perspectiveType == MBGB_PERSP_EQUIRECT) f.start = vp;
  else f.start = sub(vp, mul(baseY, 1.0 / s.persp * s.zoom));
  const Vec lv{cos(s.mainLightAlpha - 0.5 * M_PI) * cos(-s.mainLightBeta),
               sin(s.mainLightAlpha - 0.5 * M_PI) * cos(-s.mainLightBeta), sin(-s.mainLightBeta)};
  f.light = rot(f.rm, f.rzero, lv);
  const int q = s.globalIlumQuality;
  for (double b = -0.49 * M_PI; b < 0.49 * M_PI; b += 1.0 / q) {
    for (double a = 0.0; a < 2.0 * M_PI; a += ((2.0 / q) / cos(b))) {
      f.aoDirs.push_back(Vec{cos(a + b) * cos(b), sin(a + b) * cos(b), sin(b)});
      if (f.aoDirs.size() >= 10000) break;
    }
    if (f.aoDirs.size() >= 10000) break;
  }
}

// ObjectShader (src/shaders.cpp:21-112) at a hit: object and specular terms, surface colour.
void object_shader(const mbgb_scene &s, const Frame &f, Calc &c, Vec point, Vec view, double thr, double delta,
                   double lastDist, int objectType, double obj[3], double specOut[3], Vec &objColour) {
  const Vec n = calculate_normals(s, c, point, delta, thr);
  double shade = dot(n, f.light);
  if (shade < 0) shade = 0;
  const double shadeV = s.directLight * ((1.0 - s.shading) + s.shading * shade);
  double shadow = 1.0;
  if (s.shadow) shadow = main_shadow(s, c, point, f.light, thr, delta, f.start);
  Vec half = normalize(sub(f.light, view));
  double sp = dot(n, half);
  if (sp < 0.0) sp = 0.0;
  sp = pow(sp, 30.0) * 1.0;
  if (sp > 15.0) sp = 15.0;
  sp *= s.specular;
  const Vec col = surface_colour(s, c, point, objectType);
  objColour = col;
  double amb = 0.0;
  if (s.global_ilumination) {
    if (s.fastGlobalIllumination) amb = fast_ao(s, c, point, n, thr);
    else amb = ray_ao(s, c, point, delta, thr, lastDist, f.aoDirs, f.start);
  }
  const double a2 = amb * s.globalIlum;
  const double ml[3] = {s.mainLightIntensity * s.mainLightColour.R / 65536.0,
                        s.mainLightIntensity * s.mainLightColour.G / 65536.0,
                        s.mainLightIntensity * s.mainLightColour.B / 65536.0};
  const double cc[3] = {col.x, col.y, col.z};
  const double env = ((!s.raytracedReflections && s.reflect > 0) ? env_mapping(n, view) : 0.0) * s.reflect;
  double auxS[3] = {0, 0, 0}, auxSp[3] = {0, 0, 0};
  if (f.numberOfLights > 0) aux_lights(s, f, c, point, n, view, delta, thr, auxS, auxSp);
  // FakeLights (src/shaders.cpp:1225-1271)
  double fake = 0.0, fakeSp = 0.0;
  if (s.fakeLightsEnabled) {
    const double dl = thr * s.smoothness;
    const double rr = compute(c, point, kOrbitTrap, 0, nullptr);
    const double fl = s.fakeLightsIntensity / rr;
    const double r = 1.0 / (rr + 1e-30);
    const double rx = 1.0 / (compute(c, add(point, Vec{dl, 0.0, 0.0}), kOrbitTrap, 0, nullptr) + 1e-30);
    const double ry = 1.0 / (compute(c, add(point, Vec{0.0, dl, 0.0}), kOrbitTrap, 0, nullptr) + 1e-30);
    const double rz = 1.0 / (compute(c, add(point, Vec{0.0, 0.0, dl}), kOrbitTrap, 0, nullptr) + 1e-30);
    Vec fn{r - rx, r - ry, r - rz};
    if (!(fn.x == 0 && fn.y == 0 && fn.z == 0)) fn = normalize(fn);
    fake = fl * dot(n, fn);
    if (fake < 0) fake = 0;
    double fs = dot(n, normalize(sub(fn, view)));
    if (fs < 0.0) fs = 0.0;
    fs = pow(fs, 30.0) * fl;
    if (fs > 15.0) fs = 15.0;
    fakeSp = fs;
  }
  for (int k = 0; k < 3; k++) {
    double o = env * amb + (a2 + ml[k] * shadeV * shadow) * cc[k];
    o += (auxS[k] + fake) * cc[k];
    obj[k] = o;
    specOut[k] = auxSp[k] + fakeSp + ml[k] * sp * shadow;
  }
}

void render_pixel(const Frame &f, int x, int y, std::vector<std::vector<Step>> &bufs, bool jitter,
                  const mbgb_image *img, Cnt &cnt) {
  const mbgb_scene &s = *f.s;
  const int W = img->width, H = img->height;
  const int tiles = s.noOfTiles;
  const double tx = (s.tileCount % tiles), ty = (s.tileCount / tiles);
  const double aspect = (double)W / H;
  const double fov = s.persp;
  const double x2 = ((double)x / W / tiles - 0.5 + tx / tiles) * aspect;
  const double z2 = ((double)y / H / tiles - 0.5 + ty / tiles);
  bool cut = false;
  Vec v;
  if (s.perspectiveType == MBGB_PERSP_FISH_EYE) {
    if (s.fishEyeCut && sqrt(x2 * x2 + z2 * z2) > 0.5 / fov) cut = true;
    const double x3 = x2 * M_PI, z3 = z2 * M_PI;
    const double r = sqrt(x3 * x3 + z3 * z3);
    if (r == 0) v = {0.0, 1.0, 0.0};
    else v = {x3 / r * sin(r * fov), cos(r * fov), z3 / r * sin(r * fov)};
    v = normalize(v);
  } else if (s.perspectiveType == MBGB_PERSP_EQUIRECT) {
    const double x3 = x2 * M_PI, z3 = z2 * M_PI;
    v = {sin(fov * x3) * cos(fov * z3), cos(fov * x3) * cos(fov * z3), sin(fov * z3)};
    v = normalize(v);
  } else {
    v = {x2 * fov, 1.0, z2 * fov};
  }
  const Vec view = rot(f.rm, f.rzero, v);
  Calc c{&s, (int)s.N, s.minN, false, 0.0, 0, &cnt, &f.d};
  // the reflection loop (src/Render3D.cpp:441-564)
  const int maxRay = (s.raytracedReflections && s.reflectionsMax > 0) ? s.reflectionsMax : 0;
  struct Refl {
    Vec start, view;
    Ray ray;
    int objectType;
    double reflect;
  };
  std::vector<Refl> rb((size_t)maxRay + 1);
  Vec startRay = f.start, viewRay = view;
  double thrCarry = 0.0;
  int rayEnd = 0, iters0 = 0;
  bool levelMissed = false;
  Vec lastPoint{0, 0, 0};
  for (int k = 0; k <= maxRay; k++) {
    Refl &r = rb[(size_t)k];
    r.start = startRay;
    r.view = viewRay;
    r.ray = Ray{};
    r.ray.thr = thrCarry;
    r.ray.point = lastPoint;
    if (!cut) r.ray = ray_marching(s, c, startRay, viewRay, bufs[(size_t)k], jitter, cnt, thrCarry);
    if (k == 0) {
      if (f.exact && r.ray.found) levelMissed = !level_set(s, c, f.start, view, r.ray);
      iters0 = c.itersOut;
    }
    lastPoint = r.ray.point;
    thrCarry = r.ray.thr;
    r.objectType = c.objectOut;
    const double pr[7] = {s.reflect, s.primitivePlaneReflect, s.primitiveWaterReflect, s.primitiveSphereReflect,
                          s.primitiveInvertedSphereReflect, s.primitiveBoxReflect, s.primitiveInvertedBoxReflect};
    r.reflect = pr[r.objectType];
    rayEnd = k;
    if (!r.ray.found) break;
    if (r.reflect == 0) break;
    c.detail = r.ray.thr;
    const double dl = s.constantDEThreshold ? r.ray.depth * s.resolution * s.persp : r.ray.thr * s.quality;
    const Vec vn = calculate_normals(s, c, r.ray.point, dl, r.ray.thr);
    viewRay = sub(viewRay, mul(mul(vn, dot(viewRay, vn)), 2.0));
    startRay = add(r.ray.point, mul(viewRay, r.ray.thr));
  }
  double result[3] = {0, 0, 0};
  Vec objColour{0, 0, 0};
  float opacity0 = 0.0f;
  double alpha0 = 0.0;
  for (int k = rayEnd; k >= 0; k--) {
    Refl &r = rb[(size_t)k];
    const double thr = r.ray.thr;
    c.detail = thr;
    const double delta = s.constantDEThreshold ? r.ray.depth * s.resolution * s.persp : thr * s.quality;
    double obj[3] = {0, 0, 0}, spec[3] = {0, 0, 0}, bg[3] = {0, 0, 0};
    double out[4];
    if (r.ray.found) {
      object_shader(s, f, c, r.ray.point, r.view, thr, delta, r.ray.lastDist, r.objectType, obj, spec, objColour);
    } else {
      const Vec b = background(s, r.view);
      bg[0] = b.x;
      bg[1] = b.y;
      bg[2] = b.z;
    }
    for (int q = 0; q < 3; q++) {
      if (maxRay > 0 && rayEnd > 0 && k != rayEnd)
        out[q] = result[q] * r.reflect + (1.0 - r.reflect) * (obj[q] + bg[q]) + spec[q];
      else
        out[q] = obj[q] + bg[q] + spec[q];
    }
    out[3] = r.ray.found ? 1.0 + 0.0 : 0.0 + 0.0;
    float opacity = 0.0f;
    volumetric(s, f, c, bufs[(size_t)k], r.ray.count, r.ray.depth, r.view, delta, r.ray.lastDist, out, &opacity);
    for (int q = 0; q < 3; q++) result[q] = out[q];
    if (k == 0) {
      opacity0 = opacity;
      alpha0 = out[3];
    }
  }
  const double depthZ = rb[0].ray.found ? rb[0].ray.depth : 1e20;
  const int64_t pix = (int64_t)y * W + x;
  if (img->opacity) img->opacity[pix] = to_u16((double)opacity0 * 65535.0);
  if (img->alpha) img->alpha[pix] = to_u16(alpha0 * 65535.0);
  if (img->image_float) {
    img->image_float[3 * pix + 0] = (float)result[0];
    img->image_float[3 * pix + 1] = (float)result[1];
    img->image_float[3 * pix + 2] = (float)result[2];
  }
  if (img->colour) {
    img->colour[3 * pix + 0] = to_u8(objColour.x * 255);
    img->colour[3 * pix + 1] = to_u8(objColour.y * 255);
    img->colour[3 * pix + 2] = to_u8(objColour.z * 255);
  }
  if (img->zbuffer) img->zbuffer[pix] = (float)depthZ;
  if (img->hit) img->hit[pix] = rb[0].ray.found ? (levelMissed ? 3 : 1) : 0;
  if (img->iters) img->iters[pix] = iters0;
  if (img->depth) img->depth[pix] = depthZ;
}

}  // namespace

extern "C" {

// CalculateDistance at points with detailSize = detail[i] (normal DE mode).
void oracle_distance(const mbgb_scene *s, const double *pts, const double *detail, long n, double *dist, int *iters,
                     unsigned char *max_iter) {
  Cnt cnt;
  Derived dv;
  derive(*s, dv);
  Calc c{s, (int)s->N, s->minN, false, 0.0, -1, &cnt, &dv};
  for (long i = 0; i < n; i++) {
    c.detail = detail[i];
    c.itersOut = -1;
    bool mi = false;
    dist[i] = calculate_distance(c, Vec{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, &mi);
    iters[i] = c.itersOut;
    max_iter[i] = mi ? 1 : 0;
  }
}

// Compute<colouring> with N x 10, as SurfaceColour calls it.
void oracle_colour_value(const mbgb_scene *s, const double *pts, long n, double *out) {
  Cnt cnt;
  Derived dv;
  derive(*s, dv);
  Calc c{s, (int)(s->N * 10), s->minN, false, 0.0, 0, &cnt, &dv};
  for (long i = 0; i < n; i++) out[i] = compute(c, Vec{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, kColour, 0, nullptr);
}

// Renders rows [row0, row1) with `threads` workers pulling rows from a shared
// counter (the reference's one-worker-per-core row claiming). jitter != 0 uses
// the C library's shared rand() stream, as the reference does.
// counters (may be NULL): [0] orbit iterations, [1] DE calls, [2] march steps.
// Rows [row0, row1), or the `nlist` rows of `list` when it is not NULL, claimed one at a
// time by `threads` workers (the reference's dynamic row claiming, src/Render3D.cpp:815-849).
static int render_rows(const mbgb_scene *s, int row0, int row1, int jitter, int threads, const mbgb_image *img,
                       unsigned long long *counters, bool exact, const int *list = nullptr, int nlist = 0,
                       unsigned long long *pixel_work = nullptr) {
  if (!s || !img) return 1;
  if (list) {
    if (nlist < 0) return 1;
    for (int i = 0; i < nlist; i++)
      if (list[i] < 0 || list[i] >= img->height) return 1;
    row0 = 0;
    row1 = nlist;
  } else if (row0 < 0 || row1 > img->height || row0 > row1) {
    return 1;
  }
  Frame f;
  setup_frame(*s, f);
  f.exact = exact;
  if (threads < 1) threads = 1;
  std::atomic<int> next(row0);
  std::vector<Cnt> cnts(threads);
  auto worker = [&](int t) {
    const int rays = 1 + ((s->raytracedReflections && s->reflectionsMax > 0) ? s->reflectionsMax : 0);
    std::vector<std::vector<Step>> bufs((size_t)rays, std::vector<Step>(10002));
    for (;;) {
      const int k = next.fetch_add(1);
      if (k >= row1) break;
      const int y = list ? list[k] : k;
      for (int x = 0; x < img->width; x++) {
        const Cnt before = cnts[t];
        render_pixel(f, x, y, bufs, jitter != 0, img, cnts[t]);
        if (pixel_work) {   // this pixel's orbit iterations, DE calls and march steps
          unsigned long long *w = pixel_work + 3 * ((size_t)y * img->width + x);
          w[0] = cnts[t].orbit - before.orbit;
          w[1] = cnts[t].calls - before.calls;
          w[2] = cnts[t].steps - before.steps;
        }
      }
    }
  };
  if (threads == 1) {
    worker(0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) pool.emplace_back(worker, t);
    for (auto &th : pool) th.join();
  }
  if (counters) {
    counters[0] = counters[1] = counters[2] = 0;
    for (const Cnt &c : cnts) {
      counters[0] += c.orbit;
      counters[1] += c.calls;
      counters[2] += c.steps;
    }
  }
  return 0;
}

// CompileImage with progressive factor 1: brightness and contrast in double rounded to
// float, optional float tanh, clamp to [0, 1], x 65535 truncated, gamma table.
void oracle_compile16(int w, int h, const float *image_float, double brightness, double contrast, double gamma,
                      int hdr, unsigned short *image16) {
  std::vector<int> table(65536);
  for (int i = 0; i < 65536; i++) table[i] = (int)(pow(i / 65536.0, 1.0 / gamma) * 65535);
  const long n = 3L * w * h;
  for (long i = 0; i < n; i++) {
    float v = (float)(image_float[i] * brightness);
    v = (float)((v - 0.5) * contrast + 0.5);
    if (v < 0.0f) v = 0.0f;
    if (hdr) v = tanhf(v);
    if (v > 1.0f) v = 1.0f;
    const unsigned short q = (unsigned short)(v * 65535.0);
    image16[i] = (unsigned short)table[q];
  }
}

// SSAO over an RGB16 image (in place). For each pixel on the object: `quality` directions
// at angle i / quality * 2 pi; along each, samples at radius r^2 * width / (2 quality^2),
// r = 1 .. quality - 1, skipping the pixel itself and samples off the image; the steepest
// -dz / (lateral distance) gives the horizon, ambient += 0.5 - atan(slope) / pi. Lateral
// positions follow the perspective type; the fish-eye centre skips its projection at
// radius 0, its samples do not (they test the loop radius, which is never 0).
void oracle_ssao(int w, int h, const float *zbuf, const unsigned short *opacity, const unsigned char *colour,
                 double persp, int quality, int ptype, double intensity, unsigned short *image16) {
  std::vector<double> ca(quality > 0 ? quality : 1), sa(quality > 0 ? quality : 1);
  for (int i = 0; i < quality; i++) {
    sa[i] = sin((double)i / quality * 2.0 * M_PI);
    ca[i] = cos((double)i / quality * 2.0 * M_PI);
  }
  const double scale = (double)w / (quality * quality) / 2.0;
  const double aspect = (double)w / h;
  auto lateral = [&](double fx, double fy, double z, bool centre, double &ox, double &oy) {
    if (ptype == MBGB_PERSP_FISH_EYE) {
      const double x2 = M_PI * (fx / w - 0.5) * aspect;
      const double y2 = M_PI * (fy / h - 0.5);
      const double r = sqrt(x2 * x2 + y2 * y2);
      ox = x2;
      oy = y2;
      if (!centre || r != 0.0) {
        ox = x2 / r * sin(r * persp) * z;
        oy = y2 / r * sin(r * persp) * z;
      }
    } else if (ptype == MBGB_PERSP_EQUIRECT) {
      const double x2 = M_PI * (fx / w - 0.5) * aspect;
      const double y2 = M_PI * (fy / h - 0.5);
      ox = sin(persp * x2) * cos(persp * y2) * z;
      oy = sin(persp * y2) * z;
    } else if (centre) {
      ox = (fx / w - 0.5) * aspect * z * persp;
      oy = (fy / h - 0.5) * z * persp;
    } else {
      ox = (fx / w - 0.5) * aspect * (z * persp);
      oy = (fy / h - 0.5) * (z * persp);
    }
  };
  for (int y = 0; y < h; y++) {
    for (int x = 0; x < w; x++) {
      const long p = (long)y * w + x;
      const double z = zbuf[p];
      const double op = opacity[p] / 65535.0;
      double total = 0.0;
      if (z < 1e19) {
        double x2, y2;
        lateral(x, y, z, true, x2, y2);
        double ambient = 0.0;
        for (int a = 0; a < quality; a++) {
          double best = -1e50;
          for (double r = 1.0; r < quality; r += 1.0) {
            const double rr = r * r * scale;
            const double xx = x + rr * ca[a];
            const double yy = y + rr * sa[a];
            if ((int)xx == x && (int)yy == y) continue;
            if (xx < 0 || xx > w - 1 || yy < 0 || yy > h - 1) continue;
            const double z2 = zbuf[(long)(int)yy * w + (int)xx];
            double xx2, yy2;
            lateral(xx, yy, z2, false, xx2, yy2);
            const double dx = xx2 - x2, dy = yy2 - y2, dz = z2 - z;
            const double slope = -dz / sqrt(dx * dx + dy * dy);
            if (slope > best) best = slope;
          }
          ambient += -atan(best) / M_PI + 0.5;
        }
        total = ambient / quality;
        if (total < 0) total = 0;
      }
      for (int c = 0; c < 3; c++) {
        double v = image16[3 * p + c] + 65535.0 * colour[3 * p + c] / 256.0 * total * intensity * (1.0 - op);
        if (v > 65535) v = 65535;
        image16[3 * p + c] = (unsigned short)v;
      }
    }
  }
}

// PostRendering_DOF (src/image.cpp:57-206): QuickSortZBuffer on [1, n-1], the Random()
// shuffle (srand(seed) first), then the in-place splats far to near.
void oracle_dof(int w, int h, const float *zbuffer, unsigned short *alpha, unsigned short *image16, double deep,
                double neutral, unsigned int seed) {
  const int n = w * h;
  struct SZ {
    float z;
    int i;
  };
  std::vector<SZ> d((size_t)n);
  for (int p = 0; p < n; p++) d[(size_t)p] = SZ{zbuffer[p], p};
  // Hoare partition around the middle element (src/common_math.h:53-84)
  std::vector<std::pair<int, int>> st;
  if (n > 2) st.push_back({1, n - 1});
  while (!st.empty()) {
    const int l = st.back().first, p = st.back().second;
    st.pop_back();
    int i = l, j = p;
    const SZ x = d[(size_t)((l + p) / 2)];
    do {
      while (d[(size_t)i].z < x.z) i++;
      while (x.z < d[(size_t)j].z) j--;
      if (i <= j) std::swap(d[(size_t)i++], d[(size_t)j--]);
    } while (i <= j);
    if (l < j) st.push_back({l, j});
    if (i < p) st.push_back({i, p});
  }
  srand(seed);
  for (int i = n - 1; i >= 0; i--) {
    const SZ t = d[(size_t)i];
    const double s1 = ((double)t.z - neutral) / t.z * deep;
    int rs = i, ii;
    bool done;
    do {
      ii = i - rand() % (rs + 1);
      if (ii <= 0) ii = 0;
      const double s2 = ((double)d[(size_t)ii].z - neutral) / d[(size_t)ii].z * deep;
      done = (s1 == 0 && s2 == 0);
      if (s1 * s2 > 0) done = (s1 > 0 ? s2 / s1 : s1 / s2) > 0.7;
      else done = false;
      rs = (int)(rs * 0.7 - 1);
      if (rs <= 0) done = true;
    } while (!done);
    d[(size_t)i] = d[(size_t)ii];
    d[(size_t)ii] = t;
  }
  const std::vector<unsigned short> img0(image16, image16 + 3 * (size_t)n), a0(alpha, alpha + n);
  for (int k = 0; k < n; k++) {
    const int c = d[(size_t)(n - k - 1)].i;
    const int x = c % w, y = c / w;
    const double z = zbuffer[c];
    double blur = fabs(z - neutral) / z * deep;
    if (blur > 100) blur = 100.0;
    const int size = (int)blur;
    const double factor = blur * blur * sqrt(blur) * M_PI / 3.0;
    for (int yy = y - size; yy <= y + size; yy++)
      for (int xx = x - size; xx <= x + size; xx++) {
        if (xx < 0 || xx >= w || yy < 0 || yy >= h) continue;
        const int dx = xx - x, dy = yy - y;
        const double r = sqrtf((float)dx * dx + dy * dy);
        double op = (blur - r) / factor;
        if (op > 1.0) op = 1.0;
        if (op < 0.0) op = 0.0;
        if (op > 0.0) {
          const double opN = 1.0 - op;
          const size_t q = (size_t)yy * w + xx;
          for (int ch = 0; ch < 3; ch++)
            image16[3 * q + ch] = (unsigned short)(image16[3 * q + ch] * opN + img0[3 * (size_t)c + ch] * op);
          alpha[q] = (unsigned short)(alpha[q] * opN + a0[(size_t)c] * op);
        }
      }
  }
}

int oracle_render(const mbgb_scene *s, int row0, int row1, int jitter, int threads, const mbgb_image *img,
                  unsigned long long *counters) {
  return render_rows(s, row0, row1, jitter, threads, img, counters, false);
}

// The render of an explicit list of rows (the CPU baseline's sample spread over a frame).
int oracle_render_row_list(const mbgb_scene *s, const int *rows, int nrows, int jitter, int threads,
                           const mbgb_image *img, unsigned long long *counters) {
  if (!rows) return 1;
  return render_rows(s, 0, 0, jitter, threads, img, counters, false, rows, nrows);
}

// The render of rows [row0, row1) with each pixel's work recorded: pixel_work[3 (y w + x) + k]
// = its orbit iterations, DE calls and march steps (all rays of the pixel, in order).
int oracle_render_pixel_work(const mbgb_scene *s, int row0, int row1, int threads, const mbgb_image *img,
                             unsigned long long *pixel_work) {
  if (!pixel_work) return 1;
  return render_rows(s, row0, row1, 0, threads, img, nullptr, false, nullptr, 0, pixel_work);
}

// The same render with every hit moved onto the level set DE(P) = thr after the
// bisection (hit layer 3 where that fails): the forward pass the gradient checks use.
int oracle_render_exact(const mbgb_scene *s, int row0, int row1, int threads, const mbgb_image *img) {
  return render_rows(s, row0, row1, 0, threads, img, nullptr, true);
}

}  // extern "C"
