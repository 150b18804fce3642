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

// The distance estimate and its derivatives by the point and the fractal parameter, in the
// policy's precision: FP32 dual orbits for the FP32 policy (the running derivative's
// tangents carried relative to it, de_dual_seeded), FP64 for the FP64 policy; the shading
// algebra after them runs in FP64 for both.
template <typename T, int FORMULA>
__device__ __forceinline__ Dual<double, 4> de_dual_policy(const ParamsT<T> &p, const FractalT<double> &fd,
                                                          const V3<double> P, const int N, int &L, const T fparam,
                                                          const double fparam_d) {
  if constexpr (sizeof(T) == 4) {
    const Dual<float, 4> r = de_dual<float, FORMULA>(p.f, V3<float>{(float)P.x, (float)P.y, (float)P.z}, N, L, fparam);
    bool finite = isfinite(r.v);
#pragma unroll
    for (int k = 0; k < 4; k++) finite = finite && isfinite(r.d[k]);
    // a tangent that left FP32's range: this sample in FP64
    if (!finite) return de_dual<double, FORMULA>(fd, P, N, L, fparam_d);
    Dual<double, 4> o;
    o.v = (double)r.v;
#pragma unroll
    for (int k = 0; k < 4; k++) o.d[k] = (double)r.d[k];
    return o;
  } else {
    return de_dual<double, FORMULA>(fd, P, N, L, fparam_d);
  }
}

// One hit pixel: dI_c/dtheta_j into jac[3 * j + c]. Returns false for pixels that are not
// differentiated (no hit, level set not reached, grazing ray, non-finite result).
// The forward state (hit point, threshold, shadow, colour) is the policy's own.
template <typename T, int FORMULA, bool FAST>
__device__ __forceinline__ bool pixel_jacobian(const ParamsT<T> &p, const FractalT<double> &fd,
                                               const WaveBufs<T> &wb, const FrameCam<T> &c, const GradCam<T> &g,
                                               const int64_t gp, const int x, const int y,
                                               double jac[3 * kGradParams], Counters &cnt) {
  const uint8_t flags = wb.flags[gp];
  if (!(flags & 1) || (flags & 8)) return false;
  V3<double> d;
  camera_ray(p, c, x, y, d);
  const V3<double> P{(double)wb.point[0 * wb.npix + gp], (double)wb.point[1 * wb.npix + gp],
                     (double)wb.point[2 * wb.npix + gp]};
  const double t = (double)wb.scan[gp];
  const double thr = (double)wb.thr[gp];
  const double k = p.constantDEThreshold ? 0.0 : c.resolution_d * c.persp_d / p.quality_d;
  int L;
  // The first sample of the normal is the distance at P with N x 5 iterations. An orbit that
  // escapes within N iterations is the same computation as the N-iteration estimate the
  // implicit differentiation needs, so that one is reused (one FP64 dual orbit less per pixel).
  const Dual<double, 4> s1 = de_dual_policy<T, FORMULA>(p, fd, P, fd.N5, L, c.fparam, c.fparam_d);
  // implicit differentiation of the hit distance
  const Dual<double, 4> de = L < fd.N ? s1 : de_dual_policy<T, FORMULA>(p, fd, P, fd.N, L, c.fparam, c.fparam_d);
  const double Ft = de.d[0] * d.x + de.d[1] * d.y + de.d[2] * d.z - k;
  if (!(Ft < 0.0)) return false;
  double dt[kGradParams];
  dt[0] = -de.d[3] / Ft;
  dt[1] = -de.d[0] / Ft;
  dt[2] = -de.d[1] / Ft;
  dt[3] = -de.d[2] / Ft;
  dt[4] = dt[5] = 0.0;
  V3<double> dP[kGradParams];
  for (int j = 0; j < kGradParams; j++) dP[j] = d * dt[j];
  dP[1].x += 1.0;
  dP[2].y += 1.0;
  dP[3].z += 1.0;
  // normal step dn = delta * smoothness, delta = thr * quality (or scan * resolution * persp
  // with a constant threshold), in the policy's precision as the composition stage forms it
  const double dnScale = (p.constantDEThreshold ? c.resolution_d * c.persp_d : k * p.quality_d) *
                         (double)p.smoothness;
  const T dnT = p.constantDEThreshold ? wb.scan[gp] * c.resolution * c.persp * p.smoothness
                                      : wb.thr[gp] * p.quality * p.smoothness;
  const V3<T> PT{wb.point[0 * wb.npix + gp], wb.point[1 * wb.npix + gp], wb.point[2 * wb.npix + gp]};
  const V3<T> PxT{PT.x + dnT, PT.y, PT.z}, PyT{PT.x, PT.y + dnT, PT.z}, PzT{PT.x, PT.y, PT.z + dnT};
  const int N5 = fd.N5;
  const Dual<double, 4> sx =
      de_dual_policy<T, FORMULA>(p, fd, V3<double>{(double)PxT.x, P.y, P.z}, N5, L, c.fparam, c.fparam_d);
  const Dual<double, 4> sy =
      de_dual_policy<T, FORMULA>(p, fd, V3<double>{P.x, (double)PyT.y, P.z}, N5, L, c.fparam, c.fparam_d);
  const Dual<double, 4> sz =
      de_dual_policy<T, FORMULA>(p, fd, V3<double>{P.x, P.y, (double)PzT.z}, N5, L, c.fparam, c.fparam_d);
  const V3<double> gv{sx.v - s1.v, sy.v - s1.v, sz.v - s1.v};
  const double glen = sqrt(gv.x * gv.x + gv.y * gv.y + gv.z * gv.z);
  V3<double> n{1.0, 0.0, 0.0};
  V3<double> dnrm[kGradParams];
  for (int j = 0; j < kGradParams; j++) dnrm[j] = {0.0, 0.0, 0.0};
  if (glen > 0.0) {
    n = gv * (1.0 / glen);
    for (int j = 0; j < kGradParams; j++) {
      const double ddn = dnScale * dt[j];
      const double fpj = j == 0 ? 1.0 : 0.0;
      const double d1 = s1.d[0] * dP[j].x + s1.d[1] * dP[j].y + s1.d[2] * dP[j].z + s1.d[3] * fpj;
      const V3<double> dg{sx.d[0] * (dP[j].x + ddn) + sx.d[1] * dP[j].y + sx.d[2] * dP[j].z + sx.d[3] * fpj - d1,
                          sy.d[0] * dP[j].x + sy.d[1] * (dP[j].y + ddn) + sy.d[2] * dP[j].z + sy.d[3] * fpj - d1,
                          sz.d[0] * dP[j].x + sz.d[1] * dP[j].y + sz.d[2] * (dP[j].z + ddn) + sz.d[3] * fpj - d1};
      dnrm[j] = (dg - n * dot3(n, dg)) * (1.0 / glen);
    }
  }
  (void)thr;
  // light direction and its derivatives
  const V3<double> lv{(double)c.lightVect[0], (double)c.lightVect[1], (double)c.lightVect[2]};
  V3<double> dL[kGradParams];
  for (int j = 0; j < kGradParams; j++) dL[j] = {0.0, 0.0, 0.0};
  dL[4] = {(double)g.dLight[0][0], (double)g.dLight[0][1], (double)g.dLight[0][2]};
  dL[5] = {(double)g.dLight[1][0], (double)g.dLight[1][1], (double)g.dLight[1][2]};
  // MainShading (src/shaders.cpp:759-768): shade = max(0, n.L)
  const double shade = dot3(n, lv);
  double dShadeV[kGradParams];
  for (int j = 0; j < kGradParams; j++)
    dShadeV[j] = shade > 0.0 ? (double)p.directLight * (double)p.shading * (dot3(dnrm[j], lv) + dot3(n, dL[j]))
                             : 0.0;
  // MainSpecular (src/shaders.cpp:770-783): shade2 = min(15, max(0, n.half)^30), half = normalize(L - view)
  V3<T> viewT;
  camera_dir(p, c, x, y, viewT);
  const V3<double> view{(double)viewT.x, (double)viewT.y, (double)viewT.z};
  const V3<double> hv = lv - view;
  const double hlen = sqrt(dot3(hv, hv));
  const V3<double> half = hv * (1.0 / hlen);
  const double s2 = dot3(n, half);
  double dSpec[kGradParams];
  for (int j = 0; j < kGradParams; j++) dSpec[j] = 0.0;
  if (s2 > 0.0) {
    const double shade2 = pow(s2, 30.0);
    if (!(shade2 > 15.0)) {
      const double slope = 30.0 * pow(s2, 29.0) * (double)p.specular;
      for (int j = 0; j < kGradParams; j++) {
        const V3<double> dh = (dL[j] - half * dot3(half, dL[j])) * (1.0 / hlen);
        dSpec[j] = slope * (dot3(dnrm[j], half) + dot3(n, dh));
      }
    }
  }
  const double shadow = p.shadow ? (double)wb.shadow[gp] : 1.0;
  const V3<T> colour = wave_colour<T, FORMULA, FAST>(p, PT, cnt, c.fparam);
  const double col[3] = {(double)colour.x, (double)colour.y, (double)colour.z};
  bool finite = true;
  for (int ch = 0; ch < 3; ch++) {
    const double ml = (double)p.mainLight[ch] * shadow;
    for (int j = 0; j < kGradParams; j++) {
      jac[3 * j + ch] = ml * (dShadeV[j] * col[ch] + dSpec[j]);
      finite = finite && isfinite(jac[3 * j + ch]);
    }
  }
  return finite;
}

// Stage 5 (differentiable render): per-pixel Jacobians and the per-frame sums
// dL/dtheta = sum over pixels and channels of dL/dI dI/dtheta.
template <typename T, int FORMULA, bool FAST>
__global__ void __launch_bounds__(128) grad_kernel(const __grid_constant__ ParamsT<T> p, const __grid_constant__ FractalT<double> fd, const FrameIO io,
                                                   const WaveBufs<T> wb,
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
    double contrib[kGradParams];
    for (int j = 0; j < kGradParams; j++) contrib[j] = 0.0;
    if (y >= c.row_begin && y < c.row_end) {
      double jac[3 * kGradParams];
      const bool ok = pixel_jacobian<T, FORMULA, FAST>(p, fd, wb, c, g, gp, x, y, jac, cnt);
      if (!ok) {
        for (int i = 0; i < 3 * kGradParams; i++) jac[i] = 0.0;
        if (wb.flags[gp] & 1) skipped++;
      } else {
        done++;
      }
      if (g.jacobian)
        for (int j = 0; j < kGradParams; j++)
          for (int ch = 0; ch < 3; ch++) g.jacobian[(pix * 3 + ch) * kGradParams + j] = (float)jac[3 * j + ch];
      if (ok && g.dL_dimage) {
        const double w0 = g.dL_dimage[3 * pix + 0], w1 = g.dL_dimage[3 * pix + 1], w2 = g.dL_dimage[3 * pix + 2];
        for (int j = 0; j < kGradParams; j++) contrib[j] = w0 * jac[3 * j + 0] + w1 * jac[3 * j + 1] + w2 * jac[3 * j + 2];
      }
    }
    // dL/dtheta sums: one atomic per parameter per warp when the whole warp is on one frame
    const unsigned int m = __activemask();
    bool reduced = false;
    if (m == 0xffffffffu) {
      const int fr0 = __shfl_sync(m, fr, 0);
      if (__all_sync(m, fr == fr0)) {
        for (int j = 0; j < kGradParams; j++) {
          double v = contrib[j];
          for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(m, v, off);
          if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(&g.dtheta[j], v);
        }
        reduced = true;
      }
    }
    if (!reduced)
      for (int j = 0; j < kGradParams; j++)
        if (contrib[j] != 0.0) atomicAdd(&g.dtheta[j], contrib[j]);
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
