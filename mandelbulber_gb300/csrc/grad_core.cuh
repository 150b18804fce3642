// Gradient stage of the differentiable render.
//
// Parameters theta (per frame): [0] the fractal parameter (power of the trig_optim
// Mandelbulb, scale of the tglad Mandelbox), [1..3] the camera position vp, [4] the main
// light's alpha and [5] its beta (radians, src/Render3D.cpp:252-256).
//
// For a hit pixel the shaded value (ObjectShader without AO, src/shaders.cpp:21-112) is
//   I_c = mainLight_c shadow (shadeV(n, L) colour_c + specular shade2(n, L, view))
// where the hit point P = o + t d lies on the level set F(t) = DE(o + t d) - thr(t) = 0,
// thr(t) = t k, k = resolution persp / quality (src/Render3D.cpp:105-110). Implicit
// differentiation gives dt/dtheta = -F_theta / F_t with F_t = grad DE . d - k, so
// dP/dtheta = do/dtheta + d dt/dtheta. The normal is the reference's forward difference of
// four DE values at N x 5 (src/shaders.cpp:675-711) with step dn proportional to thr, and
// is differentiated as that difference quotient (including dn's dependence on t). Shadow
// (hard) and the palette colour (integer palette index) are piecewise constant in theta
// and contribute no derivative. The derivative of every DE evaluation comes from forward
// mode: the orbit is recomputed with dual numbers along (Px, Py, Pz, fractal parameter),
// so nothing of the forward render's orbits is stored.
#pragma once

#include "dual.cuh"
#include "wave_core.cuh"

namespace mbgb {
namespace dev {

// One hit pixel: dI_c/dtheta_j into jac[3 * j + c]. Returns false for pixels that are not
// differentiated (no hit, level set not reached, grazing ray).
template <typename T, int FORMULA, bool FAST>
__device__ __forceinline__ bool pixel_jacobian(const ParamsT<T> &p, const WaveBufs<T> &wb, const FrameCam<T> &c,
                                               const GradCam<T> &g, const int64_t gp, const int x, const int y,
                                               T jac[3 * kGradParams], Counters &cnt) {
  const uint8_t flags = wb.flags[gp];
  if (!(flags & 1) || (flags & 8)) return false;
  V3<double> dview;
  camera_ray(p, c, x, y, dview);
  const V3<T> d{(T)dview.x, (T)dview.y, (T)dview.z};
  const V3<T> P{wb.point[0 * wb.npix + gp], wb.point[1 * wb.npix + gp], wb.point[2 * wb.npix + gp]};
  const T t = wb.scan[gp];
  const T k = p.constantDEThreshold ? T(0) : c.resolution * c.persp / p.quality;
  int L;
  // implicit differentiation of the hit distance
  const Dual<T, 4> de = de_dual<T, FORMULA>(p.f, P, p.f.N, L);
  const T Ft = de.d[0] * d.x + de.d[1] * d.y + de.d[2] * d.z - k;
  if (!(Ft < T(0))) return false;
  T dt[kGradParams];
  dt[0] = -de.d[3] / Ft;
  dt[1] = -de.d[0] / Ft;
  dt[2] = -de.d[1] / Ft;
  dt[3] = -de.d[2] / Ft;
  dt[4] = dt[5] = T(0);
  V3<T> dP[kGradParams];
  for (int j = 0; j < kGradParams; j++) dP[j] = d * dt[j];
  dP[1].x += T(1);
  dP[2].y += T(1);
  dP[3].z += T(1);
  // normal step dn = delta * smoothness, delta = thr * quality or scan * resolution * persp
  const T dnScale = (p.constantDEThreshold ? c.resolution * c.persp : k * p.quality) * p.smoothness;
  const T dn = p.constantDEThreshold ? t * c.resolution * c.persp * p.smoothness
                                      : wb.thr[gp] * p.quality * p.smoothness;
  const int N5 = p.f.N5;
  const Dual<T, 4> s1 = de_dual<T, FORMULA>(p.f, P, N5, L);
  const Dual<T, 4> sx = de_dual<T, FORMULA>(p.f, V3<T>{P.x + dn, P.y, P.z}, N5, L);
  const Dual<T, 4> sy = de_dual<T, FORMULA>(p.f, V3<T>{P.x, P.y + dn, P.z}, N5, L);
  const Dual<T, 4> sz = de_dual<T, FORMULA>(p.f, V3<T>{P.x, P.y, P.z + dn}, N5, L);
  const V3<T> gv{sx.v - s1.v, sy.v - s1.v, sz.v - s1.v};
  const T glen = m_sqrt(gv.x * gv.x + gv.y * gv.y + gv.z * gv.z);
  V3<T> n{T(1), T(0), T(0)};
  V3<T> dnrm[kGradParams];
  for (int j = 0; j < kGradParams; j++) dnrm[j] = {T(0), T(0), T(0)};
  if (glen > T(0)) {
    n = gv * (T(1) / glen);
    for (int j = 0; j < kGradParams; j++) {
      const T ddn = dnScale * dt[j];
      const T fpj = j == 0 ? T(1) : T(0);
      const T d1 = s1.d[0] * dP[j].x + s1.d[1] * dP[j].y + s1.d[2] * dP[j].z + s1.d[3] * fpj;
      const V3<T> dg{sx.d[0] * (dP[j].x + ddn) + sx.d[1] * dP[j].y + sx.d[2] * dP[j].z + sx.d[3] * fpj - d1,
                     sy.d[0] * dP[j].x + sy.d[1] * (dP[j].y + ddn) + sy.d[2] * dP[j].z + sy.d[3] * fpj - d1,
                     sz.d[0] * dP[j].x + sz.d[1] * dP[j].y + sz.d[2] * (dP[j].z + ddn) + sz.d[3] * fpj - d1};
      const T nd = dot3(n, dg);
      dnrm[j] = (dg - n * nd) * (T(1) / glen);
    }
  }
  // light direction and its derivatives
  const V3<T> lv{c.lightVect[0], c.lightVect[1], c.lightVect[2]};
  V3<T> dL[kGradParams];
  for (int j = 0; j < kGradParams; j++) dL[j] = {T(0), T(0), T(0)};
  dL[4] = {g.dLight[0][0], g.dLight[0][1], g.dLight[0][2]};
  dL[5] = {g.dLight[1][0], g.dLight[1][1], g.dLight[1][2]};
  // MainShading: shade = max(0, n.L)
  const T shade = dot3(n, lv);
  T dShadeV[kGradParams];
  for (int j = 0; j < kGradParams; j++)
    dShadeV[j] = shade > T(0) ? p.directLight * p.shading * (dot3(dnrm[j], lv) + dot3(n, dL[j])) : T(0);
  // MainSpecular: shade2 = min(15, max(0, n.half)^30), half = normalize(L - view)
  V3<T> view;
  camera_dir(p, c, x, y, view);
  const V3<T> hv = lv - view;
  const T hlen = m_sqrt(dot3(hv, hv));
  const V3<T> half = hv * (T(1) / hlen);
  const T s2 = dot3(n, half);
  T dSpec[kGradParams];
  for (int j = 0; j < kGradParams; j++) dSpec[j] = T(0);
  if (s2 > T(0)) {
    const T shade2 = m_pow(s2, T(30));
    if (!(shade2 > T(15))) {
      const T slope = T(30) * m_pow(s2, T(29)) * p.specular;
      for (int j = 0; j < kGradParams; j++) {
        const V3<T> dh = (dL[j] - half * dot3(half, dL[j])) * (T(1) / hlen);
        dSpec[j] = slope * (dot3(dnrm[j], half) + dot3(n, dh));
      }
    }
  }
  const T shadow = p.shadow ? wb.shadow[gp] : T(1);
  const V3<T> colour = wave_colour<T, FORMULA, FAST>(p, P, cnt);
  const T col[3] = {colour.x, colour.y, colour.z};
  for (int ch = 0; ch < 3; ch++) {
    const T ml = p.mainLight[ch] * shadow;
    for (int j = 0; j < kGradParams; j++) jac[3 * j + ch] = ml * (dShadeV[j] * col[ch] + dSpec[j]);
  }
  return true;
}

// Stage 5 (differentiable render): per-pixel Jacobians and the per-frame sums
// dL/dtheta = sum over pixels and channels of dL/dI dI/dtheta.
template <typename T, int FORMULA, bool FAST>
__global__ void __launch_bounds__(128) grad_kernel(const ParamsT<T> p, const FrameIO io, const WaveBufs<T> wb,
                                                   const FrameCam<T> *__restrict__ cams,
                                                   const GradCam<T> *__restrict__ gcams, const int ncams) {
  Counters cnt{0, 0, 0, 0};
  unsigned long long done = 0, skipped = 0;
  for (int64_t gp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gp < wb.npix;
       gp += (int64_t)gridDim.x * blockDim.x) {
    const int fr = frame_of_pixel(cams, ncams, gp);
    const FrameCam<T> &c = cams[fr];
    const GradCam<T> &g = gcams[fr];
    const int64_t pix = gp - c.pixBase;
    const int x = (int)(pix % c.width), y = (int)(pix / c.width);
    if (y < c.row_begin || y >= c.row_end) continue;
    T jac[3 * kGradParams];
    const bool ok = pixel_jacobian<T, FORMULA, FAST>(p, wb, c, g, gp, x, y, jac, cnt);
    if (!ok) {
      for (int i = 0; i < 3 * kGradParams; i++) jac[i] = T(0);
      if (wb.flags[gp] & 1) skipped++;
    } else {
      done++;
    }
    if (g.jacobian)
      for (int j = 0; j < kGradParams; j++)
        for (int ch = 0; ch < 3; ch++) g.jacobian[(pix * 3 + ch) * kGradParams + j] = (float)jac[3 * j + ch];
    if (ok && g.dL_dimage) {
      const float w0 = g.dL_dimage[3 * pix + 0], w1 = g.dL_dimage[3 * pix + 1], w2 = g.dL_dimage[3 * pix + 2];
      for (int j = 0; j < kGradParams; j++) {
        const double v = (double)w0 * (double)jac[3 * j + 0] + (double)w1 * (double)jac[3 * j + 1] +
                         (double)w2 * (double)jac[3 * j + 2];
        if (v != 0.0) atomicAdd(&g.dtheta[j], v);
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
    done += __shfl_down_sync(0xffffffffu, done, off);
    skipped += __shfl_down_sync(0xffffffffu, skipped, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
    atomicAdd(&io.counters[2], done);
    atomicAdd(&io.counters[3], skipped);
  }
}

}  // namespace dev
}  // namespace mbgb
