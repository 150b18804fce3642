// Wavefront renderer: the per-pixel pipeline of MainThread (src/Render3D.cpp:389-589)
// split into ray-granular stages so that SIMT lanes stay busy.
//
//   primary_kernel   one primary ray per job: RayMarching's march and binary refinement
//                    (src/Render3D.cpp:79-199) with lane refill; the march's step records
//                    go to a pool of chained 32-record chunks (the overflow pass, for rays
//                    the pool cannot hold, folds them into the volumetric pass's affine
//                    map at once).
//   polish_kernel    FP32 policy: the last bisection steps in FP64 for the hits whose FP32
//                    bisection stopped within 1e-4 of a window edge.
//   secondary_kernel one shadow ray (MainShadow, src/shaders.cpp:480-570) or one AO
//                    direction (AmbientOcclusion, src/shaders.cpp:607-673) per job,
//                    with lane refill; results go to per-pixel slots.
//   compose_kernel   normals, colour, specular, fast AO, background, the volumetric
//                    pass over the pooled records (or the overflow pass's affine map) and
//                    the cImage writes (ObjectShader / BackgroundShader / VolumetricShader,
//                    src/shaders.cpp:21-478).
//
// The volumetric pass is affine in the pixel colour it starts from: every glow, post-fog
// and volumetric-fog group computes out = a*C + (1 - a)*out, so the whole pass is
// out = A*base + B with one A for the three channels; alpha and opacity do not depend on
// the base colour (its alpha is 1 for a hit and 0 otherwise, known when the march ends).
// Lane refill: each warp keeps up to 32 rays in flight; once refill_min of its lanes are
// idle (or none is busy), one atomicAdd on the job counter hands them their next jobs (popc
// of the ballot).
#pragma once

#include "dual.cuh"
#include "render_core.cuh"
#include "wave_launch.h"
#include "lean_orbit.cuh"

namespace mbgb {

namespace dev {

// Resumable lean orbits (distance mode) for the orbit-granular lane refill of the shadow/AO
// stage: the state of mandelbox_fast / mandelbulb8_fast<0> between batches of kUnroll
// iterations, through the same iteration functions. start() begins the orbit of a point;
// advance() runs up to kUnroll iterations and returns true once the orbit has ended
// (bailout or N iterations), with its distance in `dist` and its end iteration in L, the
// values the one-call versions return.
template <int FORMULA>
struct LeanOrbit;

template <>
struct LeanOrbit<8> {
  static constexpr int kUnroll = 5;
  LeanBoxK k;
  float cf;
  int N;
  float x, y, z, dr, cx, cy, cz, s, skm1;
  int L;
  __device__ __forceinline__ explicit LeanOrbit(const FractalT<float> &f) : k(lean_box_k(f)) {
    cf = f.constantFactor;
    N = f.N;
    x = y = z = cx = cy = cz = s = skm1 = 0.0f;
    dr = 1.0f;
    L = 0;
  }
  // scale: the frame's Mandelbox scale
  __device__ __forceinline__ void start(const V3<float> p, const float scale) {
    x = p.x; y = p.y; z = p.z;
    cx = __fmul_rn(p.x, cf); cy = __fmul_rn(p.y, cf); cz = __fmul_rn(p.z, cf);
    dr = 1.0f;
    s = scale;
    skm1 = __fmul_rn(scale, k.km1);
    L = 0;
  }
  __device__ __forceinline__ bool advance(float &dist) {
    if (L >= N) {
      dist = 0.0f;
      return true;
    }
    if (L <= N - kUnroll) {   // a whole block: the count is tested once, after it
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        const float r2 = box_iteration(k, s, skm1, x, y, z, dr, cx, cy, cz);
        if (r2 > 1048576.0f) {
          L += u;
          dist = box_bailout_dist(r2, dr);
          return true;
        }
      }
      L += kUnroll;
      if (L == N) {
        dist = 0.0f;
        return true;
      }
      return false;
    }
#pragma unroll 1
    for (;;) {
      const float r2 = box_iteration(k, s, skm1, x, y, z, dr, cx, cy, cz);
      if (r2 > 1048576.0f) {
        dist = box_bailout_dist(r2, dr);
        return true;
      }
      if (++L == N) {
        dist = 0.0f;
        return true;
      }
    }
  }
};

template <>
struct LeanOrbit<2> {
  static constexpr int kUnroll = 2;
  float jx, jy, jz, cf, bail2;
  int N;
  bool julia;
  float x, y, z, r2, r_dz, cx, cy, cz;
  int L;
  __device__ __forceinline__ explicit LeanOrbit(const FractalT<float> &f) {
    julia = f.juliaMode;
    bail2 = f.bailout2;
    jx = f.julia[0]; jy = f.julia[1]; jz = f.julia[2];
    cf = f.constantFactor;
    N = f.N;
    x = y = z = r2 = cx = cy = cz = 0.0f;
    r_dz = 1.0f;
    L = 0;
  }
  __device__ __forceinline__ void start(const V3<float> p, const float) {
    if (julia) {
      cx = jx; cy = jy; cz = jz;
    } else {
      cx = __fmul_rn(p.x, cf); cy = __fmul_rn(p.y, cf); cz = __fmul_rn(p.z, cf);
    }
    x = p.x; y = p.y; z = p.z;
    r_dz = 1.0f;
    r2 = norm2_rn(x, y, z);
    L = 0;
  }
  __device__ __forceinline__ bool advance(float &dist) {
    if (L >= N) {
      dist = 0.0f;
      return true;
    }
    if (L <= N - kUnroll) {   // a whole block: the count is tested once, after it
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        r2 = bulb8_iteration(x, y, z, r2, r_dz, cx, cy, cz);
        if (r2 > bail2) {
          L += u;
          const float r = sqrtf(r2);
          dist = __fmul_rn(__fmul_rn(0.5f, r), __logf(r)) / r_dz;
          return true;
        }
      }
      L += kUnroll;
      if (L == N) {
        dist = 0.0f;
        return true;
      }
      return false;
    }
#pragma unroll 1
    for (;;) {
      r2 = bulb8_iteration(x, y, z, r2, r_dz, cx, cy, cz);
      if (r2 > bail2) {
        const float r = sqrtf(r2);
        dist = __fmul_rn(__fmul_rn(0.5f, r), __logf(r)) / r_dz;
        return true;
      }
      if (++L == N) {
        dist = 0.0f;
        return true;
      }
    }
  }
};

// FP64 versions of the lean orbits for the FP32 policy's FP64 polish, which needs FP64
// accuracy but not the reference's operation order: the squared radius throughout (no
// square root per iteration) and, for the Mandelbulb, no transcendentals.
__device__ __forceinline__ double mandelbox_lean_d(const FractalT<double> &f, const double px, const double py,
                                                   const double pz, const int N, int &Lout, Counters &cnt,
                                                   const double s) {
  const double fl = f.mbFoldLimit;
  const double mR2 = f.mbMinR * f.mbMinR;
  const double fR2 = f.mbFixedR * f.mbFixedR;
  const double k1 = fR2 / mR2;
  const double cx = px * f.constantFactor, cy = py * f.constantFactor, cz = pz * f.constantFactor;
  double x = px, y = py, z = pz, dr = 1.0, dist = 0.0;
  int L;
  for (L = 0; L < N; L++) {
    x = fmin(fmax(x, -fl), fl) * 2.0 - x;
    y = fmin(fmax(y, -fl), fl) * 2.0 - y;
    z = fmin(fmax(z, -fl), fl) * 2.0 - z;
    double r2 = x * x + y * y + z * z;
    const double k = fmin(fmax(fR2 / r2, 1.0), k1);
    const double ks = k * s;
    x = fma(x, ks, cx);
    y = fma(y, ks, cy);
    z = fma(z, ks, cz);
    dr = fma(dr, fabs(ks), 1.0);
    r2 = x * x + y * y + z * z;
    if (r2 > 1048576.0) {
      dist = sqrt(r2) / fabs(dr);
      break;
    }
  }
  cnt.orbit += (unsigned long long)(L + 1);
  cnt.calls += 1;
  Lout = L;
  if (L == N) dist = 0.0;
  return dist;
}

__device__ __forceinline__ double mandelbulb8_lean_d(const FractalT<double> &f, const double px, const double py,
                                                     const double pz, const int N, int &Lout, Counters &cnt) {
  double cx, cy, cz;
  if (f.juliaMode) {
    cx = f.julia[0]; cy = f.julia[1]; cz = f.julia[2];
  } else {
    cx = px * f.constantFactor; cy = py * f.constantFactor; cz = pz * f.constantFactor;
  }
  double x = px, y = py, z = pz, r_dz = 1.0, dist = 0.0;
  double r2 = x * x + y * y + z * z;
  int L;
  for (L = 0; L < N; L++) {
    const double rho2 = x * x + y * y;
    const double inv_r = rsqrt(r2);
    const bool axis = rho2 == 0.0;
    const double inv_rho = axis ? 0.0 : rsqrt(rho2);
    double ct = rho2 * inv_rho * inv_r, st = z * inv_r;
    double cp = axis ? 1.0 : x * inv_rho, sp = axis ? 0.0 : y * inv_rho;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double ct2 = ct * ct - st * st, st2 = 2.0 * st * ct;
      const double cp2 = cp * cp - sp * sp, sp2 = 2.0 * sp * cp;
      ct = ct2; st = st2; cp = cp2; sp = sp2;
    }
    const double r4 = r2 * r2;
    const double r8 = r4 * r4;
    r_dz = fma(8.0 * r8 * inv_r, r_dz, 1.0);
    const double t = ct * r8;
    x = fma(t, cp, cx);
    y = fma(t, sp, cy);
    z = fma(st, r8, cz);
    r2 = x * x + y * y + z * z;
    if (r2 > f.bailout2) {
      const double r = sqrt(r2);
      dist = 0.5 * r * log(r) / r_dz;
      break;
    }
  }
  cnt.orbit += (unsigned long long)(L + 1);
  cnt.calls += 1;
  Lout = L;
  if (L == N) dist = 0.0;
  return dist;
}

// CalculateDistance in FP64 for the polish: the lean orbits when the scene qualifies.
template <int FORMULA, bool FAST>
__device__ __forceinline__ double polish_distance(const FractalT<double> &f, const V3<double> p, const double detail,
                                                  int &L, bool &maxIter, Counters &cnt, const double fparam) {
  if constexpr (FAST) {
    int Li;
    double distance;
    if constexpr (FORMULA == 8) distance = mandelbox_lean_d(f, p.x, p.y, p.z, f.N, Li, cnt, fparam);
    else distance = mandelbulb8_lean_d(f, p.x, p.y, p.z, f.N, Li, cnt);
    L = Li;
    return distance_post(f, distance, Li, f.N, f.minN, detail, false, 0.0, maxIter);
  } else {
    return calc_distance<double, FORMULA>(f, p, detail, f.N, f.minN, false, L, maxIter, cnt, fparam);
  }
}

// CalculateDistance of the wavefront stages. The FAST instantiations (launched where the
// fractal allows the lean FP32 orbits, FractalT::lean) call the lean orbit directly, so that
// their code holds no generic orbit; the others take calc_distance.
template <typename T, int FORMULA, bool FAST>
__device__ __forceinline__ T wave_distance(const FractalT<T> &f, const V3<T> p, const T detail, const int N,
                                           const int minN, const bool normalMode, int &L, bool &maxIter,
                                           Counters &cnt, const T fparam) {
  return distance_est<T, FORMULA, FAST>(f, p, detail, N, minN, normalMode, L, maxIter, cnt, fparam);
}

// SurfaceColour (src/shaders.cpp:850-879) with the fast power-8 colouring orbit when it applies.
template <typename T, int FORMULA, bool FAST>
__device__ __forceinline__ V3<T> wave_colour(const ParamsT<T> &p, const V3<T> point, Counters &cnt,
                                             const T fparam, const int objectType = kObjFractal) {
  if constexpr (FAST && FORMULA == 2 && sizeof(T) == 4) {
    int L;
    const float c = mandelbulb8_fast<1>(p.f, point.x, point.y, point.z, p.f.N10, L, cnt);
    int nrCol = to_i32_x86((double)floorf(c));
    const unsigned mag = nrCol < 0 ? 0u - (unsigned)nrCol : (unsigned)nrCol;
    nrCol = (int)(mag % (248u * 256u));
    int rgb[3] = {256, 256, 256};
    if (p.coloring) {
      const int color_number = to_i32_x86((double)((T)nrCol * p.coloringSpeed + T(256) * p.paletteOffset)) % 65536;
      index_to_colour(p, color_number, rgb);
    }
    return V3<T>{T(rgb[0]) / T(256), T(rgb[1]) / T(256), T(rgb[2]) / T(256)};
  } else {
    return surface_colour<T, FORMULA>(p, point, cnt, fparam, objectType);
  }
}

// Warp-level job hand-out: lanes with need == true receive consecutive job indices (one
// atomicAdd per refill; a block-wise reserve with the next claim kept in flight measured
// slower at the tuned refill thresholds, 13.5 against 13.2 ms per 1080p Mandelbox frame).
__device__ __forceinline__ unsigned int claim_jobs(unsigned int *counter, const bool need) {
  const unsigned int lane = threadIdx.x & 31u;
  const unsigned int mask = __ballot_sync(0xffffffffu, need);
  unsigned int base = 0;
  if (lane == (unsigned int)(__ffs(mask) - 1) && mask) base = atomicAdd(counter, (unsigned int)__popc(mask));
  base = __shfl_sync(0xffffffffu, base, mask ? (__ffs(mask) - 1) : 0);
  return base + (unsigned int)__popc(mask & ((1u << lane) - 1u));
}

// One pooled step record: dist, thr, step in a 16-byte (float) or 32-byte (double) slot.
__device__ __forceinline__ void store_record(float *r, const float dist, const float thr, const float step,
                                             const float scan) {
  *reinterpret_cast<float4 *>(r) = make_float4(dist, thr, step, scan);
}
__device__ __forceinline__ void store_record(double *r, const double dist, const double thr, const double step,
                                             const double scan) {
  reinterpret_cast<double2 *>(r)[0] = make_double2(dist, thr);
  reinterpret_cast<double2 *>(r)[1] = make_double2(step, scan);
}
__device__ __forceinline__ void load_record(const float *r, float &dist, float &thr, float &step) {
  const float4 q = *reinterpret_cast<const float4 *>(r);
  dist = q.x; thr = q.y; step = q.z;
}
__device__ __forceinline__ void load_record(const double *r, double &dist, double &thr, double &step) {
  const double2 a = reinterpret_cast<const double2 *>(r)[0];
  const double2 b = reinterpret_cast<const double2 *>(r)[1];
  dist = a.x; thr = a.y; step = b.x;
}
// the record's march position (sStep::point = start + view * scan)
__device__ __forceinline__ float record_scan(const float *r) { return r[3]; }
__device__ __forceinline__ double record_scan(const double *r) { return r[3]; }

// The narrow record of the plain variant: distance and threshold only (8 or 16 bytes). The
// walk recomputes each record's step from the record before it (march_step), as the march
// formed it, and reads no march position.
__device__ __forceinline__ void store_record_narrow(float *r, const float dist, const float thr) {
  *reinterpret_cast<float2 *>(r) = make_float2(dist, thr);
}
__device__ __forceinline__ void store_record_narrow(double *r, const double dist, const double thr) {
  *reinterpret_cast<double2 *>(r) = make_double2(dist, thr);
}
__device__ __forceinline__ void load_record_narrow(const float *r, float &dist, float &thr) {
  const float2 q = *reinterpret_cast<const float2 *>(r);
  dist = q.x; thr = q.y;
}
__device__ __forceinline__ void load_record_narrow(const double *r, double &dist, double &thr) {
  const double2 q = *reinterpret_cast<const double2 *>(r);
  dist = q.x; thr = q.y;
}

// The march's next step after the estimate `dist` at threshold `thr` of march step i
// (src/Render3D.cpp:117, 127-134): the distance clamped at 3, less stepFrac thresholds, times
// the DE factor, with the step jitter when it is on. One function for the march and for the
// volumetric walk's recomputation, so that both round alike (the FP32 form spells out its
// multiply-add).
template <typename T>
__device__ __forceinline__ T march_step(const ParamsT<T> &p, T dist, const T thr, const T stepFrac,
                                        const uint32_t pixel, const uint32_t i) {
  if (dist > T(3)) dist = T(3);
  T step;
  if constexpr (sizeof(T) == 4) step = __fmul_rn(__fmaf_rn(-stepFrac, thr, dist), p.DE_factor);
  else step = (dist - stepFrac * thr) * p.DE_factor;
  if (p.jitter) step = step * (T(1) - T(jitter1000(p.jitter_seed, pixel, i)) / T(10000));
  return step;
}

// Backward walk over a ray's pooled records: record `index` of a chain whose last chunk
// holds the records from kChunk * (nchunks - 1) on.
template <typename T>
struct PoolRecords {
  const T *rec;            // [chunk * kChunk + r][W]: W = 4 (dist, thr, step, scan; effects
                           // variant) or 2 (dist, thr; plain variant)
  const int32_t *prev;
  int32_t last;      // chunk holding the last written record
  int lastRec;       // index of the last written record: buffCount for a hit (its hit step
                     // writes distance and threshold), buffCount - 1 otherwise
};

// The walk's next chunk (toward the ray's start) and that chunk's link, requested into L2
// while the walk reads the current chunk: the backward walk is otherwise one dependent miss
// per chunk and one miss per 128-byte line.
template <int W = 4, typename T>
__device__ __forceinline__ void prefetch_chunk(const PoolRecords<T> &pr, const int32_t chunk) {
  if (chunk < 0) return;
  const char *b = reinterpret_cast<const char *>(pr.rec + (int64_t)W * kChunk * chunk);
  for (int o = 0; o < W * kChunk * (int)sizeof(T); o += 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(b + o));
  asm volatile("prefetch.global.L2 [%0];" ::"l"(pr.prev + chunk));
}

// Frame of a primary job / of a pixel of the batch (binary search over the frame table).
template <typename T>
__device__ __forceinline__ int frame_of_job(const FrameCam<T> *__restrict__ cams, const int n, const unsigned int job) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cams[mid].jobBase <= job) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
template <typename T>
__device__ __forceinline__ int frame_of_pixel(const FrameCam<T> *__restrict__ cams, const int n, const int64_t gp) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cams[mid].pixBase <= gp) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Pixel of the batch a ray belongs to (rays of reflection depth d sit at d * npix_frame + pixel).
template <typename T>
__device__ __forceinline__ int64_t pixel_of_ray(const WaveBufs<T> &wb, const int64_t ri) {
  return ri < wb.npix_frame ? ri : ri % wb.npix_frame;
}

// Job index within a frame -> pixel: tiles of tileW x tileH (32 pixels) in row-major
// tile order, so a warp's first 32 jobs cover one tile.
__device__ __forceinline__ void job_pixel(const int width, const int row_begin, const int tileW, const int tileH,
                                          const unsigned int job, int &x, int &y) {
  const int tilesX = (width + tileW - 1) / tileW;
  const unsigned int tile = job / (unsigned int)(tileW * tileH);
  const unsigned int inTile = job % (unsigned int)(tileW * tileH);
  x = (int)(tile % (unsigned int)tilesX) * tileW + (int)(inTile % (unsigned int)tileW);
  y = row_begin + (int)(tile / (unsigned int)tilesX) * tileH + (int)(inTile / (unsigned int)tileW);
}

// Camera ray of a pixel (src/Render3D.cpp:389-438); returns false for a fisheye-cut pixel.
template <typename T>
__device__ __forceinline__ bool camera_ray(const ParamsT<T> &p, const FrameCam<T> &c, const int x, const int y,
                                           V3<double> &view) {
  const double x2 = ((double)x / c.width / c.tiles - 0.5 + c.tileXOffset / c.tiles) * c.aspect;
  const double z2 = ((double)y / c.height / c.tiles - 0.5 + c.tileYOffset / c.tiles);
  bool cut = false;
  V3<double> vv;
  if (p.perspType == 1) {
    if (p.fishEyeCut && sqrt(x2 * x2 + z2 * z2) > 0.5 / c.fov) cut = true;
    const double x3 = x2 * kPI, z3 = z2 * kPI;
    const double r = sqrt(x3 * x3 + z3 * z3);
    if (r == 0) {
      vv = {0.0, 1.0, 0.0};
    } else {
      vv.x = x3 / r * sin(r * c.fov);
      vv.z = z3 / r * sin(r * c.fov);
      vv.y = cos(r * c.fov);
    }
    vv = normalize3(vv);
  } else if (p.perspType == 2) {
    const double x3 = x2 * kPI, z3 = z2 * kPI;
    vv.x = sin(c.fov * x3) * cos(c.fov * z3);
    vv.z = sin(c.fov * z3);
    vv.y = cos(c.fov * x3) * cos(c.fov * z3);
    vv = normalize3(vv);
  } else {
    vv = {x2 * c.fov, 1.0, z2 * c.fov};
  }
  view = rotate(c.rot, c.rot_zero, vv);
  return !cut;
}

// Camera ray in the march precision: the FP32 policy forms the three-point-perspective
// direction in FP32 (the per-frame ray origin stays the FP64 value from the host); the
// FP64 policy and the fisheye/equirectangular projections use camera_ray.
template <typename T>
__device__ __forceinline__ bool camera_dir(const ParamsT<T> &p, const FrameCam<T> &c, const int x, const int y,
                                           V3<T> &dir) {
  if (sizeof(T) == 4 && p.perspType != 1 && p.perspType != 2) {
    const float x2 = ((float)x / (float)c.width / (float)c.tiles - 0.5f + (float)c.tileXOffset / (float)c.tiles) *
                     (float)c.aspect;
    const float z2 = ((float)y / (float)c.height / (float)c.tiles - 0.5f + (float)c.tileYOffset / (float)c.tiles);
    const float fov = (float)c.fov;
    const V3<float> vv{x2 * fov, 1.0f, z2 * fov};
    if (c.rot_zero) {
      dir = {(T)vv.x, (T)vv.y, (T)vv.z};
    } else {
      dir = {(T)(c.rotf[0] * vv.x + c.rotf[1] * vv.y + c.rotf[2] * vv.z),
             (T)(c.rotf[3] * vv.x + c.rotf[4] * vv.y + c.rotf[5] * vv.z),
             (T)(c.rotf[6] * vv.x + c.rotf[7] * vv.y + c.rotf[8] * vv.z)};
    }
    return true;
  }
  V3<double> view;
  const bool ok = camera_ray(p, c, x, y, view);
  dir = {(T)view.x, (T)view.y, (T)view.z};
  return ok;
}

// Visible auxiliary lights (VolumetricShader, src/shaders.cpp:242-296) at one step group of a
// ray: a bell-shaped glow around each light, sampled in up to 50 sub-steps near the closest
// one; adds to out[0..3] in the reference's order (the same arithmetic as the per-pixel
// engine's `volumetric`).
template <typename T>
__device__ __forceinline__ void visible_aux_lights(const ParamsT<T> &p, const V3<T> point, const V3<T> view,
                                                   const T step, T out[4]) {
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

// The volumetric fake light of one step group (src/shaders.cpp:298-307) from its orbit trap
// distance `r`; adds to out[0..3].
template <typename T>
__device__ __forceinline__ void fake_light_glow(const ParamsT<T> &p, T r, const T step, T out[4]) {
  r = m_sqrt(T(1.0f) / (r + T(1.0e-30f)));
  const T fakeLight = T(1) / (m_pow(r, T(10) / p.fakeLightsVisibilitySize) *
                                  m_pow(T(10), T(10) / p.fakeLightsVisibilitySize) + T(1e-100));
  out[0] += fakeLight * step * p.fakeLightsVisibility;
  out[1] += fakeLight * step * p.fakeLightsVisibility;
  out[2] += fakeLight * step * p.fakeLightsVisibility;
  out[3] += fakeLight * step * p.fakeLightsVisibility;
}

// Volumetric lights at one step group (VolumetricShader, src/shaders.cpp:309-343) from the
// group's MainShadow (`sh`, main light, volumetric light 0) and the predefined aux lights'
// AuxShadow (`aux[i]`, volumetric lights 1-4); adds to out[0..3] in the reference's order.
template <typename T>
__device__ __forceinline__ void volumetric_light_terms(const ParamsT<T> &p, const V3<T> point, const T step,
                                                       const T sh, const T aux[4], T out[4]) {
  for (int i = 0; i < 5; i++) {
    if (i == 0 && p.volLightEnabled[0]) {
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
      const T light = aux[i - 1];
      out[0] += light * T(L.colour[0]) / T(65536) * p.volLightIntensity[i] * step / distance2;
      out[1] += light * T(L.colour[1]) / T(65536) * p.volLightIntensity[i] * step / distance2;
      out[2] += light * T(L.colour[2]) / T(65536) * p.volLightIntensity[i] * step / distance2;
      out[3] += light * p.volLightIntensity[i] * step / distance2;
    }
  }
}

// The results of the shadow stage for the volumetric walk of one ray: sample `base + k` is
// the walk's k-th step group.
template <typename T>
struct VolSamples {
  const T *res;            // [WaveBufs::sample_nres][cap]
  const int32_t *iters;    // the pool records' itersOut (iteration fog)
  uint32_t cap, base;
  int fakeRes;             // the orbit trap's result (fake lights): the last one
};

// Iteration fog at one step group (VolumetricShader, src/shaders.cpp:385-466): the fog colour
// by the record's iteration count, lit by the main light and the predefined aux lights through
// the group's shadows and by the ray-traced AO, blended in by the group's opacity. `res` holds
// the group's results at stride `cap`: MainShadow, 4 AuxShadow, then the AO directions.
template <typename T>
__device__ __forceinline__ void iteration_fog_term(const ParamsT<T> &p, const V3<T> point, const T step, const int L,
                                                   const T *res, const uint32_t cap, T out[4],
                                                   float &totalOpacity) {
  const T N = T(p.f.N);
  T opacity = iter_opacity(step, T(L), N, p.iterFogOpacityTrim, p.iterFogOpacity);
  if (!(opacity > T(0))) return;
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
        const T sh = res[0];
        for (int c = 0; c < 3; c++)
          newColour[c] += sh * T(p.mainLightColour[c]) / T(65536) * p.mainLightIntensity * p.directLight;
      }
    }
    if (i > 0 && p.numberOfLights > 0 && p.lights[i - 1].enabled) {
      const LightT<T> Lt = p.lights[i - 1];
      const V3<T> d = V3<T>{Lt.pos[0], Lt.pos[1], Lt.pos[2]} - point;
      const T distance = length3(d);
      const T distance2 = distance * distance;
      const T light = res[(int64_t)i * cap];
      const T intensity = Lt.intensity * T(100);
      for (int c = 0; c < 3; c++) newColour[c] += light * T(Lt.colour[c]) / T(65536) / distance2 * intensity;
    }
  }
  if (p.ao && !p.fastAO) {
    // AmbientOcclusion (src/shaders.cpp:607-673): the directions' shadowTemp, weighed and averaged
    V3<T> AO{T(0), T(0), T(0)};
    for (int v = 0; v < p.aoCount; v++) {
      const T sh = res[(int64_t)(kSampleShadows + v) * cap];
      AO.x += sh * p.aoWeight[0];
      AO.y += sh * p.aoWeight[1];
      AO.z += sh * p.aoWeight[2];
    }
    const T div = T(p.aoCount) * T(256);
    AO.x /= div;
    AO.y /= div;
    AO.z /= div;
    newColour[0] += AO.x * p.globalIlum;
    newColour[1] += AO.y * p.globalIlum;
    newColour[2] += AO.z * p.globalIlum;
  }
  if (opacity > T(1)) opacity = T(1);
  for (int c = 0; c < 3; c++) out[c] = out[c] * (T(1) - opacity) + newColour[c] * opacity * fogCol[c] / T(65536);
  totalOpacity = (float)(opacity + (T(1) - opacity) * (T)totalOpacity);
  out[3] = opacity + (T(1) - opacity) * out[3];
}

// The volumetric pass over one ray's records (VolumetricShader's glow, post fog and
// volumetric fog, src/shaders.cpp:185-478) as the affine map out = A*base + B, plus
// the alpha and opacity it leaves for a base alpha of `alpha0`.
// Effects variant: the visible aux lights, the volumetric lights and the iteration fog, whose
// MainShadow, AuxShadow and AO (render_core.cuh's, with the ray's `delta`, last distance and
// the camera `eye`) run here in line.
template <typename T, bool EFX, int FORMULA>
__device__ __forceinline__ void volumetric_affine(const ParamsT<T> &p, const StepBuf<T> &sb, const int stepCount,
                                                  const T depth, const T alpha0, const V3<T> rayStart,
                                                  const V3<T> view, const T delta, const V3<T> eye,
                                                  const T lastDist, const FrameIO &io, Counters &cnt, T vol[6]) {
  T detail = T(0);
  int itersOut = 0;
  T A = T(1), B0 = T(0), B1 = T(0), B2 = T(0), alpha = alpha0;
  float totalOpacity = 0.0f, opacityOut = 0.0f;
  const T glow = T(stepCount) * p.glowIntensity / T(512) * p.DE_factor;
  T glowN = T(1) - glow;
  if (glowN < T(0)) glowN = T(0);
  const T gR = (T(p.glow1[0]) * glowN + T(p.glow2[0]) * glow) / T(65536);
  const T gG = (T(p.glow1[1]) * glowN + T(p.glow2[1]) * glow) / T(65536);
  const T gB = (T(p.glow1[2]) * glowN + T(p.glow2[2]) * glow) / T(65536);
  T totalStep = T(0);
  for (int index = stepCount - 1; index > 0; index--) {
    T step = sb.step[sb.at(index)];
    const T distance = sb.dist[sb.at(index)];
    const T dist_thresh = sb.thr[sb.at(index)];
    totalStep += step;
    if (totalStep < dist_thresh * p.quality) continue;
    step = totalStep;
    totalStep = T(0);
    const T go = glow * step / depth;
    A = (T(1) - go) * A;
    B0 = go * gR + (T(1) - go) * B0;
    B1 = go * gG + (T(1) - go) * B1;
    B2 = go * gB + (T(1) - go) * B2;
    alpha += go;
    if (EFX && p.auxLightVisibility > T(0) && p.numberOfLights > 0 && sb.scan) {
      // the visible lights add to the colour: the map's offset
      T add[4] = {B0, B1, B2, alpha};
      visible_aux_lights<T>(p, rayStart + view * sb.scan[sb.at(index)], view, step, add);
      B0 = add[0];
      B1 = add[1];
      B2 = add[2];
      alpha = add[3];
    }
    if (EFX && p.fakeLights && sb.scan) {
      Counters c2{0, 0, 0, 0};
      int L;
      const T r = compute<T, FORMULA, 5>(p.f, rayStart + view * sb.scan[sb.at(index)], p.f.N, L, c2, fparam_of(p.f));
      T add[4] = {B0, B1, B2, alpha};
      fake_light_glow<T>(p, r, step, add);
      B0 = add[0];
      B1 = add[1];
      B2 = add[2];
      alpha = add[3];
    }
    if (EFX && p.volLightAny && sb.scan) {
      const V3<T> point = rayStart + view * sb.scan[sb.at(index)];
      const T thrStep = sb.thr[sb.at(index)];
      T sh = T(1), aux[4] = {T(1), T(1), T(1), T(1)};
      if (p.volLightEnabled[0]) sh = main_shadow<T, FORMULA>(p, point, thrStep, delta, eye, detail, itersOut, io, cnt);
      for (int j = 0; j < 4; j++) {
        if (p.numberOfLights > 0 && p.lights[j].enabled && p.volLightEnabled[j + 1]) {
          const LightT<T> L = p.lights[j];
          const V3<T> d = V3<T>{L.pos[0], L.pos[1], L.pos[2]} - point;
          aux[j] = aux_shadow<T, FORMULA>(p, point, length3(d), normalize3(d), delta, thrStep, eye, detail, itersOut,
                                          cnt);
        }
      }
      T add[4] = {B0, B1, B2, alpha};
      volumetric_light_terms<T>(p, point, step, sh, aux, add);
      B0 = add[0];
      B1 = add[1];
      B2 = add[2];
      alpha = add[3];
    }
    if (p.postFog) {
      T fd = step / p.fogVisibility;
      if (fd > T(1)) fd = T(1);
      A = (T(1) - fd) * A;
      B0 = fd * T(p.fogColor[0]) / T(65536) + (T(1) - fd) * B0;
      B1 = fd * T(p.fogColor[1]) / T(65536) + (T(1) - fd) * B1;
      B2 = fd * T(p.fogColor[2]) / T(65536) + (T(1) - fd) * B2;
      totalOpacity = (float)(fd + (T(1) - fd) * (T)totalOpacity);
      alpha = fd + (T(1) - fd) * alpha;
    }
    if (p.fogDensity > T(0)) {
      const T red = p.fogDistFactor;
      const T dt = (step * red) / (distance * distance + red * red);
      T k = distance / p.fogC1Dist;
      if (k > T(1)) k = T(1);
      T kn = T(1) - k;
      T fr = (T(p.fogCol1[0]) * kn + T(p.fogCol2[0]) * k);
      T fg = (T(p.fogCol1[1]) * kn + T(p.fogCol2[1]) * k);
      T fb = (T(p.fogCol1[2]) * kn + T(p.fogCol2[2]) * k);
      T k2 = distance / p.fogC2Dist * k;
      if (k2 > T(1)) k2 = T(1);
      kn = T(1) - k2;
      fr = (fr * kn + T(p.fogCol3[0]) * k2);
      fg = (fg * kn + T(p.fogCol3[1]) * k2);
      fb = (fb * kn + T(p.fogCol3[2]) * k2);
      T fd = T(0.3) * p.fogDensity * dt / (T(1) + p.fogDensity * dt);
      if (fd > T(1)) fd = T(1);
      A = (T(1) - fd) * A;
      B0 = fd * fr / T(65536) + (T(1) - fd) * B0;
      B1 = fd * fg / T(65536) + (T(1) - fd) * B1;
      B2 = fd * fb / T(65536) + (T(1) - fd) * B2;
      totalOpacity = (float)(fd + (T(1) - fd) * (T)totalOpacity);
      alpha = fd + (T(1) - fd) * alpha;
    }
    if (EFX && p.iterFog && sb.iters && sb.scan) {
      // iteration fog (src/shaders.cpp:385-466) with its shadows and AO traced here
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
        if (p.mainLightIntensity * p.directLight > T(0)) {
          const T sh = main_shadow<T, FORMULA>(p, point, thrStep, delta, eye, detail, itersOut, io, cnt);
          for (int c = 0; c < 3; c++)
            newColour[c] += sh * T(p.mainLightColour[c]) / T(65536) * p.mainLightIntensity * p.directLight;
        }
        for (int i = 1; i < 5; i++) {
          if (p.numberOfLights > 0 && p.lights[i - 1].enabled) {
            const LightT<T> Lt = p.lights[i - 1];
            const V3<T> d = V3<T>{Lt.pos[0], Lt.pos[1], Lt.pos[2]} - point;
            const T distance = length3(d);
            const T distance2 = distance * distance;
            const T light =
                aux_shadow<T, FORMULA>(p, point, distance, normalize3(d), delta, thrStep, eye, detail, itersOut, cnt);
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
        A = A * (T(1) - opacity);
        B0 = B0 * (T(1) - opacity) + newColour[0] * opacity * fogCol[0] / T(65536);
        B1 = B1 * (T(1) - opacity) + newColour[1] * opacity * fogCol[1] / T(65536);
        B2 = B2 * (T(1) - opacity) + newColour[2] * opacity * fogCol[2] / T(65536);
        totalOpacity = (float)(opacity + (T(1) - opacity) * (T)totalOpacity);
        alpha = opacity + (T(1) - opacity) * alpha;
      }
    }
    if (totalOpacity > 1.0f) totalOpacity = 1.0f;
    if (alpha > T(1)) alpha = T(1);
    opacityOut = totalOpacity;
  }
  vol[0] = A;
  vol[1] = B0;
  vol[2] = B1;
  vol[3] = B2;
  vol[4] = alpha;
  vol[5] = (T)opacityOut;
}

// ---------------------------------------------------------------------------
// Stage 1: primary rays with lane refill, over every frame of the batch.
// ---------------------------------------------------------------------------
// EFX: the effects variant (reflected rays, WaveBufs::rays > 1, auxiliary or volumetric
// lights); the plain variant holds none of their state.
// OVF (effects variant): the overflow pass's instantiation, whose fold of a long ray's records
// traces the volumetric lights' shadows in line; the main pass's holds no fold.
template <typename T, int FORMULA, bool FAST, bool EFX = false, bool OVF = false>
__global__ void __launch_bounds__(128, (FAST && sizeof(T) == 4) ? 8 : 6) primary_kernel(const __grid_constant__ ParamsT<T> p, const __grid_constant__ FractalT<double> fd,
                                                      const FrameIO io, const WaveBufs<T> wb,
                                                      const FrameCam<T> *__restrict__ cams, const int ncams) {
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const StepBuf<T> sb{(T *)io.step_step, (T *)io.step_dist, (T *)io.step_thr, (T *)io.step_scan, io.step_iters,
                      io.slots, slot};
  const bool useSB = p.needVolumetric;
  const bool f64 = sizeof(T) == 8;
  const T stepFrac = p.f.interiorMode ? T(0.8) : T(0.5);
  const T search_limit = T(1) - T(0.01) * p.quality;
  const int stepCap = io.overflow_pass ? kStepSlots : io.step_cap;
  // jobs: every frame's tiles (partial tiles included), the reflected rays of this depth, or
  // the overflow list
  const int depth = EFX ? wb.depth : 0;
  const unsigned int nJobs = io.overflow_pass ? *(volatile unsigned int *)&wb.ctl[3]
                             : depth > 0      ? *(volatile unsigned int *)&wb.ctl[10]
                                              : cams[ncams - 1].jobBase + cams[ncams - 1].jobCount;
  Counters cnt{0, 0, 0, 0};
  unsigned int *jobCounter = io.overflow_pass ? (wb.ctl + 4) : (wb.ctl + 0);

  // per-lane ray state
  bool active = false, exhausted = false;
  int64_t gp = 0;   // pixel of the batch
  int64_t ri = 0;   // ray: depth * npix_frame + gp
  int phase = 0, i = 0, buffCount = 0, iters = 0, bis = 0;
  int chunk = -1;   // current pool chunk of the ray's step records (main pass)
  V3<T> dir{T(0), T(0), T(0)}, start{T(0), T(0), T(0)};
  T res = T(0), persp = T(0), thrScale = T(0), fpar = T(0);
  T thrInit = T(0);   // a reflected ray's thresholds add the previous ray's (0 for camera rays)
  T scan = T(0), step = T(0), thr = T(0), dist = T(0), detail = T(0);  // detail: detailSize of the march
  int guardSteps = 0;
  for (;;) {
    // hand out jobs to idle lanes
    // a warp claims new jobs once refill_min of its lanes are idle, or when none is busy
    const bool need = !active && !exhausted;
    const unsigned int needMask = __ballot_sync(0xffffffffu, need);
    if (needMask && (__popc(needMask) >= (unsigned int)wb.refill_min || !__any_sync(0xffffffffu, active))) {
      if (io.budget_ns && (threadIdx.x & 31) == 0 && deadline_passed(io)) atomicExch(io.error_flag, 1);
      // the flag is only ever set by an expired deadline: no read (an L2 round trip) without one
      const bool stop = io.budget_ns && *(volatile int *)io.error_flag != 0;
      const unsigned int job = claim_jobs(jobCounter, need);
      if (need) {
        if (stop || job >= nJobs) {
          exhausted = true;
        } else {
          int x, y, fr;
          if (io.overflow_pass || depth > 0) {
            ri = io.overflow_pass ? (int64_t)wb.overflow_list[job]
                                  : (int64_t)depth * wb.npix_frame + (int64_t)wb.ray_list[job];
            gp = EFX ? pixel_of_ray(wb, ri) : ri;
            fr = frame_of_pixel(cams, ncams, gp);
            const int64_t local = gp - cams[fr].pixBase;
            x = (int)(local % cams[fr].width);
            y = (int)(local / cams[fr].width);
          } else {
            fr = frame_of_job(cams, ncams, job);
            const FrameCam<T> &c = cams[fr];
            job_pixel(c.width, c.row_begin, c.tileW, c.tileH, job - c.jobBase, x, y);
            gp = c.pixBase + (int64_t)y * c.width + x;
            ri = gp;
          }
          const FrameCam<T> &c = cams[fr];
          if (x < c.width && y < c.row_end) {
            bool marched = true;
            if (!EFX || ri < wb.npix_frame) {
              marched = camera_dir(p, c, x, y, dir);
              start = {(T)c.start[0], (T)c.start[1], (T)c.start[2]};
              thrInit = T(0);
            } else {
              // a reflected ray (src/Render3D.cpp:441-462): marched in T from its FP64 origin
              // and direction, its thresholds offset by the previous ray's
              start = {(T)wb.ray_start[ri], (T)wb.ray_start[wb.npix + ri], (T)wb.ray_start[2 * wb.npix + ri]};
              dir = {(T)wb.ray_dir[ri], (T)wb.ray_dir[wb.npix + ri], (T)wb.ray_dir[2 * wb.npix + ri]};
              thrInit = (T)wb.ray_thr0[ri];
            }
            res = c.resolution;
            persp = c.persp;
            fpar = c.fparam;
            thrScale = res * persp / p.quality;
            chunk = -1;
            scan = p.viewDistanceMin;
            step = p.viewDistanceMin;
            thr = T(0);
            dist = T(0);
            i = 0;
            buffCount = 0;
            iters = 0;
            phase = 0;
            bis = 0;
            active = true;
            if (!marched) {
              // fisheye cut: no march, background with an empty step buffer
              wb.flags[ri] = 2;
              wb.scan[ri] = T(0);
              wb.count[ri] = 0;
              wb.iters[ri] = 0;
              wb.last_chunk[ri] = -1;
              active = false;
            }
          }
        }
      }
    }
    if (!__any_sync(0xffffffffu, active)) {
      if (__all_sync(0xffffffffu, exhausted)) break;
      continue;
    }
    if (active) {
      // one DE evaluation of the ray's current phase (0: march, 1: bisection)
      const V3<T> point = start + dir * scan;
      if (phase == 0) {
        if (p.constantDEThreshold) thr = p.quality;
        else if (f64) thr = EFX ? scan * res * persp / p.quality + thrInit : scan * res * persp / p.quality;
        else thr = EFX ? scan * thrScale + thrInit : scan * thrScale;
        if (p.perspType == 1 || p.perspType == 2) thr *= T(kPI);
        detail = thr;
      }
      bool mi;
      dist = wave_distance<T, FORMULA, FAST>(p.f, point, detail, p.f.N, p.f.minN, false, iters, mi, cnt, fpar);
      cnt.steps++;
      bool done = false;
      if (phase == 0) {
        int64_t rec = 0;
        if (useSB) {
          if (io.overflow_pass) {
            sb.dist[sb.at(i)] = dist;
            sb.thr[sb.at(i)] = thr;
            if constexpr (EFX) {
              if (sb.iters) sb.iters[sb.at(i)] = iters;
            }
          } else {
            // main pass: records go to the batch's pool in chunks of kChunk
            bool full = false;
            if ((i % kChunk) == 0) {
              const unsigned int cc = atomicAdd(wb.ctl + 5, 1u);
              if (cc >= wb.pool_cap) {
                full = true;
              } else {
                wb.pool_prev[cc] = chunk;
                chunk = (int)cc;
              }
            }
            if (full) {
              // the pool is spent: re-marched by the overflow pass with slot records
              const unsigned int k = atomicAdd(wb.ctl + 3, 1u);
              wb.overflow_list[k] = (unsigned int)ri;
              active = false;
              continue;
            }
            rec = (int64_t)chunk * kChunk + (i % kChunk);
            // the record's step slot holds the step that reached this point; the walk
            // never reads it for the hit record. The plain variant stores the narrow record.
            if constexpr (EFX) store_record(wb.pool_rec + 4 * rec, dist, thr, step, scan);
            else store_record_narrow(wb.pool_rec + 2 * rec, dist, thr);
            if constexpr (EFX) {
              if (wb.pool_iters) wb.pool_iters[rec] = iters;
            }
          }
        }
        if (dist > T(3)) dist = T(3);
        if (dist < thr) {
          if (dist < T(0.1) * thr) cnt.missed++;
          phase = 1;
          step *= T(0.5);
          bis = 0;
          if (dist < thr && dist > thr * search_limit) done = true;
        } else {
          if (useSB && io.overflow_pass) {
            sb.step[sb.at(i)] = step;
            if (sb.scan) sb.scan[sb.at(i)] = scan;
          }
          step = march_step(p, dist, thr, stepFrac, (uint32_t)gp, (uint32_t)i);
          buffCount++;
          scan += step;
          i++;
          if (scan > p.viewDistanceMax || i >= kMaxMarchSteps) done = true;
        }
        if (!done && phase == 1) {
          // first bisection move (src/Render3D.cpp:151-167)
          if (dist > thr) scan += step;
          else if (dist < thr * search_limit) scan -= step;
          if (p.constantDEThreshold) thr = p.quality;
          else if (f64) thr = EFX ? scan * res * persp / p.quality + thrInit : scan * res * persp / p.quality;
          else thr = EFX ? scan * thrScale + thrInit : scan * thrScale;
          bis = 1;
        }
      } else {
        // bisection iteration `bis` evaluated; next check/move
        step *= T(0.5);
        if (bis >= 20 || (dist < thr && dist > thr * search_limit)) {
          done = true;
        } else {
          if (dist > thr) scan += step;
          else if (dist < thr * search_limit) scan -= step;
          if (p.constantDEThreshold) thr = p.quality;
          else if (f64) thr = EFX ? scan * res * persp / p.quality + thrInit : scan * res * persp / p.quality;
          else thr = EFX ? scan * thrScale + thrInit : scan * thrScale;
          bis++;
        }
      }
      if (++guardSteps > (1 << 24)) done = true;
      if (done) {
        const bool found = phase == 1;
        // bits 4-6: the object the last distance estimate ended on (primitives; 0 = fractal)
        uint8_t flags = (uint8_t)((found ? 1 : 0) | ((cnt.objectOut & 7) << 4));
        if ((!EFX || OVF) && io.overflow_pass && useSB) {
          // rare long rays: fold the records now (the slot is reused); compose applies the map
          T vol[6] = {T(1), T(0), T(0), T(0), found ? T(1) : T(0), T(0)};
          const T rayDelta = p.constantDEThreshold ? scan * res * persp : thr * p.quality;
          volumetric_affine<T, EFX, FORMULA>(p, sb, buffCount, scan, found ? T(1) : T(0), start, dir, rayDelta,
                                             V3<T>{(T)cams[frame_of_pixel(cams, ncams, gp)].start[0],
                                                   (T)cams[frame_of_pixel(cams, ncams, gp)].start[1],
                                                   (T)cams[frame_of_pixel(cams, ncams, gp)].start[2]},
                                             dist, io, cnt, vol);
          for (int c = 0; c < 6; c++) wb.vol[c * wb.npix + ri] = vol[c];
          flags |= 4;
        }
        wb.flags[ri] = flags;
        wb.last_chunk[ri] = chunk;
        wb.scan[ri] = scan;
        wb.dist[ri] = dist;
        wb.thr[ri] = thr;
        wb.step[ri] = step;
        wb.detail[ri] = detail;
        wb.bis_left[ri] = 20 - bis;
        wb.count[ri] = buffCount;
        wb.iters[ri] = iters;
        const V3<T> hp = start + dir * scan;
        wb.point[0 * wb.npix + ri] = hp.x;
        wb.point[1 * wb.npix + ri] = hp.y;
        wb.point[2 * wb.npix + ri] = hp.z;
        if (found) {
          const unsigned int k = atomicAdd(wb.ctl + 1, 1u);
          wb.hit_list[k] = (unsigned int)ri;
          // FP32 policy: the FP64 polish re-checks every hit whose FP32 bisection stopped
          // early but not clearly inside the window (dist/thr within 1e-4 of an edge). A
          // bisection that used all 20 steps has none left to continue, so FP64 would keep
          // its depth: it is not re-evaluated. exact_hit: every hit goes on to the level-set
          // refinement.
          if (!f64 || wb.exact_hit) {
            const T q = dist / thr;
            const bool clear = (q > search_limit + T(1e-4)) && (q < T(1) - T(1e-4));
            if (wb.polish_all || wb.exact_hit || (!clear && bis < 20)) {
              const unsigned int m = atomicAdd(wb.ctl + 6, 1u);
              wb.polish_list[m] = (unsigned int)ri;
            }
          }
        }
        active = false;
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
    cnt.steps += __shfl_down_sync(0xffffffffu, cnt.steps, off);
    cnt.missed += __shfl_down_sync(0xffffffffu, cnt.missed, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
    atomicAdd(&io.counters[2], cnt.steps);
    atomicAdd(&io.counters[3], cnt.missed);
  }
}

// ---------------------------------------------------------------------------
// Stage 2 (FP32 policy): finish the binary refinement in FP64 (src/Render3D.cpp:145-183)
// for the hits on the polish list: the distance is re-evaluated in FP64 at the FP32
// result and the bisection continues with the iterations it has left. Scenes of the lean
// orbit class use the FP64 lean orbits (polish_distance).
// ---------------------------------------------------------------------------
template <int FORMULA, bool FAST>
__global__ void __launch_bounds__(128) polish_kernel(const __grid_constant__ ParamsT<float> p, const __grid_constant__ FractalT<double> fd,
                                                     const FrameIO io, const WaveBufs<float> wb,
                                                     const FrameCam<float> *__restrict__ cams, const int ncams) {
  // exact_hit: every hit is on the polish list for the level-set stage, which refines it
  // from the FP32 bisection (in FP32, FP64 where that fails): no FP64 bisection here
  if (wb.exact_hit) return;
  const unsigned int nh = *(volatile unsigned int *)&wb.ctl[6];
  Counters cnt{0, 0, 0, 0};
  const double search_limit = 1.0 - 0.01 * p.quality_d;
  // The FP64 pipe's time per warp instruction grows with the active lanes, so a short list
  // (a few thousand hits) is spread thin: warp w takes `lanes` consecutive items, as few as
  // fill every warp of the grid once, and goes to block w mod gridDim.x (every SM and SM
  // sub-partition). Measured at 1080p (2157 hits): 0.39 ms with 32 lanes per warp, 0.18-0.19
  // ms with 8 or 1.
  const unsigned int lane = threadIdx.x & 31u, wpb = blockDim.x >> 5;
  const unsigned int warps = gridDim.x * wpb;
  const unsigned int lanes = nh >= warps * 32u ? 32u : (nh + warps - 1) / warps;
  if (lane >= lanes) return;
  for (unsigned int w = (threadIdx.x >> 5) * gridDim.x + blockIdx.x; w * lanes < nh; w += warps) {
    const unsigned int k = w * lanes + lane;
    if (k >= nh) break;
    const int64_t gp = (int64_t)wb.polish_list[k];   // the ray (pixel + depth x npix_frame)
    const int64_t px = pixel_of_ray(wb, gp);
    const FrameCam<float> &c = cams[frame_of_pixel(cams, ncams, px)];
    const int64_t local = px - c.pixBase;
    const int x = (int)(local % c.width), y = (int)(local / c.width);
    V3<double> dir, start;
    double thrInit = 0.0;
    if (gp < wb.npix_frame) {
      camera_ray(p, c, x, y, dir);
      start = {c.start[0], c.start[1], c.start[2]};
    } else {   // a reflected ray: its FP64 origin and direction, thresholds offset
      start = {wb.ray_start[gp], wb.ray_start[wb.npix + gp], wb.ray_start[2 * wb.npix + gp]};
      dir = {wb.ray_dir[gp], wb.ray_dir[wb.npix + gp], wb.ray_dir[2 * wb.npix + gp]};
      thrInit = wb.ray_thr0[gp];
    }
    double scan = (double)wb.scan[gp];
    double step = (double)wb.step[gp];
    const double detail = (double)wb.detail[gp];
    const int left = wb.bis_left[gp];
    auto thr_of = [&](double sc) {
      return p.constantDEThreshold ? p.quality_d : sc * c.resolution_d * c.persp_d / p.quality_d + thrInit;
    };
    double thr = thr_of(scan);
    V3<double> point = start + dir * scan;
    int iters = 0;
    bool mi;
    double dist = polish_distance<FORMULA, FAST>(fd, point, detail, iters, mi, cnt, c.fparam_d);
    cnt.steps++;
    for (int it = 0; it < left; it++) {
      if (dist < thr && dist > thr * search_limit) break;
      if (dist > thr) scan += step;
      else if (dist < thr * search_limit) scan -= step;
      point = start + dir * scan;
      thr = thr_of(scan);
      dist = polish_distance<FORMULA, FAST>(fd, point, detail, iters, mi, cnt, c.fparam_d);
      cnt.steps++;
      step *= 0.5;
    }
    wb.scan[gp] = (float)scan;
    wb.dist[gp] = (float)dist;
    wb.thr[gp] = (float)thr;
    wb.iters[gp] = iters;
    wb.flags[gp] = (uint8_t)((wb.flags[gp] & 0x8f) | ((cnt.objectOut & 7) << 4));
    wb.point[0 * wb.npix + gp] = (float)point.x;
    wb.point[1 * wb.npix + gp] = (float)point.y;
    wb.point[2 * wb.npix + gp] = (float)point.z;
  }
  atomicAdd(&io.counters[0], cnt.orbit);
  atomicAdd(&io.counters[1], cnt.calls);
  atomicAdd(&io.counters[2], cnt.steps);
}

// ---------------------------------------------------------------------------
// Stage 2b (exact_hit, both policies; the differentiable render's forward pass): after
// the binary refinement, Newton steps in FP64 move every hit on the polish list onto the
// level set DE = thr. A hit that does not get there keeps its bisection result and is
// flagged (bit 3) so the gradient stage leaves it out.
// ---------------------------------------------------------------------------
template <typename T, int FORMULA>
__global__ void __launch_bounds__(128) level_set_kernel(const __grid_constant__ ParamsT<T> p, const __grid_constant__ FractalT<double> fd,
                                                        const WaveBufs<T> wb, const FrameCam<T> *__restrict__ cams,
                                                        const int ncams) {
  const unsigned int nh = *(volatile unsigned int *)&wb.ctl[6];
  unsigned int missed = 0;
  for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += gridDim.x * blockDim.x) {
    const int64_t gp = (int64_t)wb.polish_list[k];
    const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, gp)];
    const int64_t local = gp - c.pixBase;
    const int x = (int)(local % c.width), y = (int)(local / c.width);
    if constexpr (sizeof(T) == 4) {
      // FP32 policy: Newton in FP32 on the march's own ray; FP64 only where that fails
      V3<float> dirf;
      camera_dir(p, c, x, y, dirf);
      const V3<float> startf{(float)c.start[0], (float)c.start[1], (float)c.start[2]};
      const float kf = p.constantDEThreshold ? 0.0f : c.resolution * c.persp / p.quality;
      float tf = wb.scan[gp];
      int lf = wb.iters[gp];
      if (level_set_hit_f32<FORMULA>(p.f, startf, dirf, kf, p.quality, tf, lf, c.fparam)) {
        const float thr = p.constantDEThreshold ? p.quality : tf * kf;
        const V3<float> point = startf + dirf * tf;
        wb.scan[gp] = tf;
        wb.dist[gp] = thr;
        wb.thr[gp] = thr;
        wb.iters[gp] = lf;
        wb.point[0 * wb.npix + gp] = point.x;
        wb.point[1 * wb.npix + gp] = point.y;
        wb.point[2 * wb.npix + gp] = point.z;
        continue;
      }
    }
    V3<double> dir;
    camera_ray(p, c, x, y, dir);
    const V3<double> start{c.start[0], c.start[1], c.start[2]};
    const double kd = p.constantDEThreshold ? 0.0 : c.resolution_d * c.persp_d / p.quality_d;
    double t = (double)wb.scan[gp];
    int li = wb.iters[gp];
    if (level_set_hit<FORMULA>(fd, start, dir, kd, p.quality_d, t, li, c.fparam_d)) {
      const V3<double> point = start + dir * t;
      const double thr = p.constantDEThreshold ? p.quality_d : t * c.resolution_d * c.persp_d / p.quality_d;
      wb.scan[gp] = (T)t;
      wb.dist[gp] = (T)thr;
      wb.thr[gp] = (T)thr;
      wb.iters[gp] = li;
      wb.point[0 * wb.npix + gp] = (T)point.x;
      wb.point[1 * wb.npix + gp] = (T)point.y;
      wb.point[2 * wb.npix + gp] = (T)point.z;
    } else {
      wb.flags[gp] |= 8;
      missed++;
    }
  }
  if (missed) atomicAdd(wb.ctl + 7, missed);
}

// FastAmbientOcclusion2 (src/shaders.cpp:585-605) on the stage's orbit: q^2 - 1 DE samples
// along the normal at i^2 x the threshold, weighted 2^-i.
template <typename T, int FORMULA, bool FAST>
__device__ __forceinline__ T wave_fast_ao(const ParamsT<T> &p, const V3<T> point, const V3<T> normal,
                                          const T dist_thresh, const T detail, Counters &cnt, const T fparam) {
  T aoTemp = T(0);
  const int q2 = p.aoQuality * p.aoQuality;
  for (int i = 1; i < q2; i++) {
    const T scan = T(i * i) * dist_thresh;
    const V3<T> pt = point + normal * scan;
    int L;
    bool mi;
    const T dist = wave_distance<T, FORMULA, FAST>(p.f, pt, detail, p.f.N, p.f.minN, false, L, mi, cnt, fparam);
    // 1.0 / pow(2.0, i) is exact for integral i
    aoTemp += T(1) / T(ldexp(1.0, i)) * (scan - p.fastAoTune * dist) / dist_thresh;
  }
  T ao = T(1) - T(0.2) * aoTemp;
  if (ao < T(0)) ao = T(0);
  return ao;
}

// Shading-stage quantities of a hit pixel shared by the secondary and compose stages.
template <typename T>
struct HitInfo {
  V3<T> point;
  T thr, delta, scan;
};

template <typename T>
__device__ __forceinline__ HitInfo<T> hit_info(const ParamsT<T> &p, const FrameCam<T> &c, const WaveBufs<T> &wb,
                                               const int64_t gp) {
  HitInfo<T> h;
  h.point = {wb.point[0 * wb.npix + gp], wb.point[1 * wb.npix + gp], wb.point[2 * wb.npix + gp]};
  h.thr = wb.thr[gp];
  h.scan = wb.scan[gp];
  h.delta = p.constantDEThreshold ? h.scan * c.resolution * c.persp : h.thr * p.quality;
  return h;
}

// ---------------------------------------------------------------------------
// Stage 2c (ray-traced reflections, src/Render3D.cpp:441-499): every hit of the current depth
// on a reflecting object spawns the mirrored ray of the next depth, started one threshold
// above the hit. The normal is CalculateNormals at the hit (N x 5 iterations, minN 0) in the
// march precision; direction and origin are formed in FP64, as the reflection loop does.
// ---------------------------------------------------------------------------
template <typename T, int FORMULA, bool FAST>
__global__ void __launch_bounds__(128) reflect_kernel(const __grid_constant__ ParamsT<T> p, const FrameIO io,
                                                      const WaveBufs<T> wb, const FrameCam<T> *__restrict__ cams,
                                                      const int ncams) {
  // this depth's hits: the hit list from the count before its primary pass to the count now
  const unsigned int h0 = *(volatile unsigned int *)&wb.ctl[8];
  const unsigned int h1 = *(volatile unsigned int *)&wb.ctl[1];
  Counters cnt{0, 0, 0, 0};
  for (unsigned int k = h0 + blockIdx.x * blockDim.x + threadIdx.x; k < h1; k += gridDim.x * blockDim.x) {
    const int64_t ri = (int64_t)wb.hit_list[k];
    const int objectType = (wb.flags[ri] >> 4) & 7;
    // sReflect::reflect of the object the ray hit (src/Render3D.cpp:470-478)
    const T reflect = objectType == kObjFractal ? p.reflect : p.primReflect[objectType - 1];
    if (reflect == T(0)) continue;
    const int64_t gp = pixel_of_ray(wb, ri);
    const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, gp)];
    const HitInfo<T> h = hit_info(p, c, wb, ri);
    const V3<T> vn = calc_normal_fp<T, FORMULA, FAST>(p, h.point, h.delta, h.thr, h.thr, cnt, c.fparam);
    V3<double> view;
    if (ri < wb.npix_frame) {
      const int64_t local = gp - c.pixBase;
      camera_ray(p, c, (int)(local % c.width), (int)(local / c.width), view);
    } else {
      view = {wb.ray_dir[ri], wb.ray_dir[wb.npix + ri], wb.ray_dir[2 * wb.npix + ri]};
    }
    const V3<double> vnd{(double)vn.x, (double)vn.y, (double)vn.z};
    view = view - vnd * dot3(view, vnd) * 2.0;
    const double distThresh = (double)h.thr;
    const V3<double> point{(double)h.point.x, (double)h.point.y, (double)h.point.z};
    const V3<double> startRay = point + view * distThresh;
    const int64_t rn = ri + wb.npix_frame;
    wb.ray_start[rn] = startRay.x;
    wb.ray_start[wb.npix + rn] = startRay.y;
    wb.ray_start[2 * wb.npix + rn] = startRay.z;
    wb.ray_dir[rn] = view.x;
    wb.ray_dir[wb.npix + rn] = view.y;
    wb.ray_dir[2 * wb.npix + rn] = view.z;
    wb.ray_thr0[rn] = distThresh;
    const unsigned int m = atomicAdd(wb.ctl + 9, 1u);
    wb.ray_list[m] = (unsigned int)gp;
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
  }
}

// Auxiliary lights: CalculateNormals (src/shaders.cpp:675-757: 4 DEs at N x 5, minN 0) at
// every hit of every depth, before the shadow stage, whose AuxShadow jobs test each light's
// Lambert and Blinn terms; the composition stage reads the same normals.
template <typename T, int FORMULA, bool FAST>
__global__ void __launch_bounds__(128) normal_kernel(const __grid_constant__ ParamsT<T> p, const FrameIO io,
                                                     const WaveBufs<T> wb, const FrameCam<T> *__restrict__ cams,
                                                     const int ncams) {
  const unsigned int nh = *(volatile unsigned int *)&wb.ctl[1];
  Counters cnt{0, 0, 0, 0};
  for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += gridDim.x * blockDim.x) {
    const int64_t ri = (int64_t)wb.hit_list[k];
    const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, pixel_of_ray(wb, ri))];
    const HitInfo<T> h = hit_info(p, c, wb, ri);
    const V3<T> n = calc_normal_fp<T, FORMULA, FAST>(p, h.point, h.delta, h.thr, h.thr, cnt, c.fparam);
    wb.normal[ri] = n.x;
    wb.normal[wb.npix + ri] = n.y;
    wb.normal[2 * wb.npix + ri] = n.z;
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
  }
}

// The shadow/AO set-up of one hit (plain variant): the hit point, its threshold, the AO and
// shadow marches' start (delta, shadow start) and end (delta / resolution, and the shadow's
// factor: delta / resolution when penetrating, else the view distance), as
// MainShadow and AmbientOcclusion form them (src/shaders.cpp:480-570, 572-640).
template <typename T>
struct HitSetup {
  V3<T> point;
  T thr, delta, aoEnd, shadowEnd, shadowStart;
};
__device__ __forceinline__ void store_hit_setup(float *q, const HitSetup<float> &h) {
  reinterpret_cast<float4 *>(q)[0] = make_float4(h.point.x, h.point.y, h.point.z, h.thr);
  reinterpret_cast<float4 *>(q)[1] = make_float4(h.delta, h.aoEnd, h.shadowEnd, h.shadowStart);
}
__device__ __forceinline__ void store_hit_setup(double *q, const HitSetup<double> &h) {
  reinterpret_cast<double2 *>(q)[0] = make_double2(h.point.x, h.point.y);
  reinterpret_cast<double2 *>(q)[1] = make_double2(h.point.z, h.thr);
  reinterpret_cast<double2 *>(q)[2] = make_double2(h.delta, h.aoEnd);
  reinterpret_cast<double2 *>(q)[3] = make_double2(h.shadowEnd, h.shadowStart);
}
__device__ __forceinline__ HitSetup<float> load_hit_setup(const float *q) {
  const float4 a = reinterpret_cast<const float4 *>(q)[0], b = reinterpret_cast<const float4 *>(q)[1];
  return HitSetup<float>{{a.x, a.y, a.z}, a.w, b.x, b.y, b.z, b.w};
}
__device__ __forceinline__ HitSetup<double> load_hit_setup(const double *q) {
  const double2 a = reinterpret_cast<const double2 *>(q)[0], b = reinterpret_cast<const double2 *>(q)[1];
  const double2 c = reinterpret_cast<const double2 *>(q)[2], d = reinterpret_cast<const double2 *>(q)[3];
  return HitSetup<double>{{a.x, a.y, b.x}, b.y, c.x, c.y, d.x, d.y};
}
template <typename T>
__device__ __forceinline__ HitSetup<T> hit_setup(const ParamsT<T> &p, const FrameCam<T> &c, const WaveBufs<T> &wb,
                                                 const int64_t ri) {
  const HitInfo<T> h = hit_info(p, c, wb, ri);
  HitSetup<T> q;
  q.point = h.point;
  q.thr = h.thr;
  q.delta = h.delta;
  q.aoEnd = h.delta / c.resolution;
  q.shadowEnd = p.penetrating ? h.delta / c.resolution : p.viewDistanceMax;
  q.shadowStart = p.f.interiorMode ? h.thr * p.DE_factor : h.thr;
  return q;
}

// Plain variant: every hit's shadow/AO set-up in hit-list order, so that a job reads its
// hit's with two coalesced vector loads (the shadow stage claims its jobs in this order).
template <typename T>
__global__ void __launch_bounds__(128) hit_setup_kernel(const __grid_constant__ ParamsT<T> p, const WaveBufs<T> wb,
                                                        const FrameCam<T> *__restrict__ cams, const int ncams) {
  const unsigned int nh = *(volatile unsigned int *)&wb.ctl[1];
  for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += gridDim.x * blockDim.x) {
    const int64_t ri = (int64_t)wb.hit_list[k];
    const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, pixel_of_ray(wb, ri))];
    store_hit_setup(wb.hit_setup + (int64_t)8 * k, hit_setup(p, c, wb, ri));
  }
}

// Volumetric lights and iteration fog: the step groups of every ray that the volumetric walk
// lights (records summed far to near until the sum reaches thr x quality,
// src/shaders.cpp:198-205; group_has_sample), each ray's samples contiguous and in the walk's
// order. One thread per pixel walks the rays the
// reflection loop marched; long rays of the overflow pass fold theirs in that pass.
template <typename T, typename F>
__device__ __forceinline__ void walk_groups(const ParamsT<T> &p, const PoolRecords<T> &pr, const int stepCount, F fn) {
  T totalStep = T(0);
  int32_t chunk = pr.last;
  int chunkBase = (pr.lastRec / kChunk) * kChunk;
  for (int index = stepCount - 1; index > 0; index--) {
    while (index < chunkBase) {
      chunk = pr.prev[chunk];
      chunkBase -= kChunk;
    }
    const int64_t rec = (int64_t)chunk * kChunk + (index - chunkBase);
    T distance, dist_thresh, step;
    load_record(pr.rec + 4 * rec, distance, dist_thresh, step);
    totalStep += step;
    if (totalStep < dist_thresh * p.quality) continue;
    const T merged = totalStep;
    totalStep = T(0);
    fn(rec, merged);
  }
}

// A step group the shadow stage traces from: every group with volumetric or fake lights, those
// of positive iteration-fog opacity (src/shaders.cpp:387-390) with iteration fog.
template <typename T>
__device__ __forceinline__ bool group_has_sample(const ParamsT<T> &p, const int32_t *iters, const int64_t rec,
                                                 const T step) {
  if (p.volLightAny || p.fakeLights) return true;
  return p.iterFog &&
         iter_opacity(step, T(iters[rec]), T(p.f.N), p.iterFogOpacityTrim, p.iterFogOpacity) > T(0);
}

template <typename T>
__global__ void __launch_bounds__(128) sample_kernel(const __grid_constant__ ParamsT<T> p, const WaveBufs<T> wb,
                                                     const FrameCam<T> *__restrict__ cams, const int ncams) {
  for (int64_t gp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gp < wb.npix_frame;
       gp += (int64_t)gridDim.x * blockDim.x) {
    const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, gp)];
    const int64_t pix = gp - c.pixBase;
    const int y = (int)(pix / c.width);
    if (y < c.row_begin || y >= c.row_end) continue;
    int rayEnd = 0;
    for (int d = 0; d + 1 < wb.rays; d++) {
      const uint8_t f = wb.flags[(int64_t)d * wb.npix_frame + gp];
      if (!(f & 1)) break;
      const int ot = (f >> 4) & 7;
      if ((ot == kObjFractal ? p.reflect : p.primReflect[ot - 1]) == T(0)) break;
      rayEnd = d + 1;
    }
    for (int d = 0; d <= rayEnd; d++) {
      const int64_t ri = (int64_t)d * wb.npix_frame + gp;
      const uint8_t flags = wb.flags[ri];
      if (flags & 4) continue;
      const int count = wb.count[ri];
      const PoolRecords<T> pr{wb.pool_rec, wb.pool_prev, wb.last_chunk[ri], (flags & 1) ? count : count - 1};
      unsigned int n = 0;
      walk_groups(p, pr, count, [&](int64_t rec, T step) {
        if (group_has_sample(p, wb.pool_iters, rec, step)) n++;
      });
      const unsigned int base = n ? atomicAdd(wb.ctl + 11, n) : 0u;
      wb.sample_base[ri] = base;
      unsigned int k = base;
      walk_groups(p, pr, count, [&](int64_t rec, T step) {
        if (!group_has_sample(p, wb.pool_iters, rec, step)) return;
        wb.sample_ray[k] = (uint32_t)ri;
        wb.sample_rec[k] = (int32_t)rec;
        wb.sample_step[k] = step;
        k++;
      });
    }
  }
}

// The hit list in the primary jobs' tile order, for the shadow stage. The primary stage
// appends hits as rays finish, which interleaves the ~300 K rays in flight from all over the
// frame, so consecutive shadow and AO jobs would start far apart; in job order a warp's 32
// jobs are the hits of one pixel tile (8 x 4 by default). A segment of kHitSeg primary jobs is
// one block of kHitSegWarps warps, each warp 32 x 32 consecutive jobs: the count pass stores
// each warp's hits, one block turns the counts into offsets, the scatter pass writes each
// warp's hits in order at its offset. A hit is a job's pixel inside its frame's rendered rows
// whose ray found the surface (the set the primary stage counted). `gp` returns the pixel.
template <typename T>
__device__ __forceinline__ bool pixel_hit(const WaveBufs<T> &wb, const FrameCam<T> *__restrict__ cams,
                                          const int ncams, const int64_t job, int64_t &gp) {
  const unsigned int nJobs = cams[ncams - 1].jobBase + cams[ncams - 1].jobCount;
  if (job >= (int64_t)nJobs) return false;
  const FrameCam<T> &c = cams[frame_of_job(cams, ncams, (unsigned int)job)];
  int x, y;
  job_pixel(c.width, c.row_begin, c.tileW, c.tileH, (unsigned int)job - c.jobBase, x, y);
  if (x >= c.width || y >= c.row_end) return false;
  gp = c.pixBase + (int64_t)y * c.width + x;
  return (wb.flags[gp] & 1) != 0;
}

template <typename T>
__global__ void __launch_bounds__(128) hit_count_kernel(const WaveBufs<T> wb, const FrameCam<T> *__restrict__ cams,
                                                        const int ncams) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t base = (int64_t)blockIdx.x * kHitSeg + (int64_t)warp * 1024;
  unsigned int n = 0;
  for (int k = 0; k < 32; k++) {
    int64_t gp;
    n += __popc(__ballot_sync(0xffffffffu, pixel_hit(wb, cams, ncams, base + k * 32 + lane, gp)));
  }
  if (lane == 0) wb.seg_count[(int64_t)blockIdx.x * kHitSegWarps + warp] = n;
}

// Exclusive prefix sum of the `n` warp counts in place (one block of 1024 threads; T is the
// stage's precision, so that each instantiating unit has its own copy).
template <typename T>
__global__ void __launch_bounds__(1024) hit_scan_kernel(uint32_t *counts, const int64_t n) {
  __shared__ uint32_t part[1024];
  const int64_t per = (n + blockDim.x - 1) / blockDim.x;
  const int64_t b = (int64_t)threadIdx.x * per, e = b + per < n ? b + per : n;
  uint32_t sum = 0;
  for (int64_t i = b; i < e; i++) sum += counts[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (unsigned int t = 0; t < blockDim.x; t++) {
      const uint32_t v = part[t];
      part[t] = run;
      run += v;
    }
  }
  __syncthreads();
  uint32_t run = part[threadIdx.x];
  for (int64_t i = b; i < e; i++) {
    const uint32_t v = counts[i];
    counts[i] = run;
    run += v;
  }
}

template <typename T>
__global__ void __launch_bounds__(128) hit_scatter_kernel(const WaveBufs<T> wb, const FrameCam<T> *__restrict__ cams,
                                                          const int ncams) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t off = wb.seg_count[(int64_t)blockIdx.x * kHitSegWarps + warp];
  const int64_t base = (int64_t)blockIdx.x * kHitSeg + (int64_t)warp * 1024;
  for (int k = 0; k < 32; k++) {
    int64_t gp = 0;
    const bool hit = pixel_hit(wb, cams, ncams, base + k * 32 + lane, gp);
    const unsigned int m = __ballot_sync(0xffffffffu, hit);
    if (hit) wb.hit_list[off + __popc(m & ((1u << lane) - 1u))] = (uint32_t)gp;
    off += __popc(m);
  }
}

// Between two reflection depths (one thread): the next depth's rays become the current ones,
// the per-depth job, overflow and polish counters restart, the hit count so far is kept.
template <typename T>
__global__ void next_depth_kernel(uint32_t *ctl) {
  ctl[8] = ctl[1];
  ctl[10] = ctl[9];
  ctl[9] = 0;
  ctl[0] = 0;
  ctl[3] = 0;
  ctl[4] = 0;
  ctl[6] = 0;
}

// ---------------------------------------------------------------------------
// Stage 3: shadow rays and ray-traced AO directions of all hits, lane refill.
// Jobs [0, nShadow): one shadow ray per hit; then aoCount x hits AO rays,
// direction-major so a warp's initial 32 rays share a direction.
// ---------------------------------------------------------------------------

// a + b * c, spelled out so every kernel rounds it alike: in FP64 with the product and the
// sum rounded separately (the reference's order), in FP32 as one FMA.
__device__ __forceinline__ float add_mul_rn(const float a, const float b, const float c) {
  return fmaf(b, c, a);
}
__device__ __forceinline__ double add_mul_rn(const double a, const double b, const double c) {
  return __dadd_rn(a, __dmul_rn(b, c));
}
template <typename T>
__device__ __forceinline__ V3<T> ray_at(const V3<T> &o, const V3<T> &d, const T r) {
  return V3<T>{add_mul_rn(o.x, d.x, r), add_mul_rn(o.y, d.y, r), add_mul_rn(o.z, d.z, r)};
}

// Lambert and Blinn terms of one auxiliary light at a hit (LightShading, src/shaders.cpp:1023-1067),
// 1 / r^2 falloff shared among `number` lights. The shadow stage tests them to decide whether
// the light's AuxShadow is traced; the composition stage weighs them by its result.
template <typename T>
struct AuxTerms {
  T shade, shade2, distance;
  V3<T> lightVector;
};
template <typename T>
__device__ __forceinline__ AuxTerms<T> aux_light_terms(const ParamsT<T> &p, const LightT<T> &L, const int number,
                                                       const V3<T> point, const V3<T> normal, const V3<T> view) {
  AuxTerms<T> a;
  const V3<T> d = V3<T>{L.pos[0], L.pos[1], L.pos[2]} - point;
  a.distance = length3(d);
  a.lightVector = normalize3(d);
  const T intensity = p.auxLightIntensity * T(100) * L.intensity / (a.distance * a.distance) / T(number);
  T shade = dot3(normal, a.lightVector);
  if (shade < T(0)) shade = T(0);
  shade = shade * intensity;
  if (shade > T(500)) shade = T(500);
  const V3<T> half = normalize3(a.lightVector - view);
  T shade2 = dot3(normal, half);
  if (shade2 < T(0)) shade2 = T(0);
  shade2 = m_pow(shade2, T(30)) * T(1);
  shade2 *= intensity * p.specular;
  if (shade2 > T(15)) shade2 = T(15);
  a.shade = shade;
  a.shade2 = shade2;
  return a;
}

// Direction of ray `ri` in the march precision: the camera ray for depth 0, the reflected
// direction otherwise.
template <typename T>
__device__ __forceinline__ V3<T> ray_view(const ParamsT<T> &p, const FrameCam<T> &c, const WaveBufs<T> &wb,
                                          const int64_t ri, const int64_t gp) {
  V3<T> v;
  if (ri < wb.npix_frame) {
    const int64_t local = gp - c.pixBase;
    camera_dir(p, c, (int)(local % c.width), (int)(local / c.width), v);
  } else {
    v = {(T)wb.ray_dir[ri], (T)wb.ray_dir[wb.npix + ri], (T)wb.ray_dir[2 * wb.npix + ri]};
  }
  return v;
}

// Jobs of the shadow stage: one main-light shadow ray per hit, aoCount AO rays per hit, and
// (aux lights with shadows) one AuxShadow per enabled light and hit.
struct SecondaryJobs {
  unsigned int nShadow, nAO, nAux;
  unsigned int nSamples;   // volumetric-light / iteration-fog samples: WaveBufs::sample_nres jobs each
};
template <typename T, bool EFX = false>
__device__ __forceinline__ SecondaryJobs secondary_jobs(const ParamsT<T> &p, const WaveBufs<T> &wb,
                                                        const unsigned int nh) {
  SecondaryJobs j;
  j.nShadow = p.shadow ? nh : 0u;
  j.nAO = (p.ao && !p.fastAO) ? nh * (unsigned int)p.aoCount : 0u;
  j.nAux = (EFX && p.shadow && wb.auxsh) ? nh * (unsigned int)p.numberOfLights : 0u;
  j.nSamples = (EFX && wb.sample_ray) ? *(volatile unsigned int *)&wb.ctl[11] : 0u;
  return j;
}

// Hits per block of the plain variant's AO job order (a power of two).
constexpr unsigned int kAoBlock = 4096;

// State of one shadow (kind 0), AO (kind 1) or auxiliary-light shadow (kind 2) ray.
template <typename T>
struct SecondaryRay {
  int kind;
  unsigned int j;   // AO direction or auxiliary light
  int64_t gp;       // ray of the batch (pixel + reflection depth x npix_frame)
  V3<T> point, dir;
  T r, end, sh, thr, detail, maxSoft, stepMul, fpar;
  int guard;
  // effects variant: where the result goes, and with iteration fog or volumetric lights the
  // per-sample threshold of the eye distance (src/shaders.cpp:515-519, 646-650)
  T *out;
  V3<T> eye;
  T res, persp;
  int fog;
};

// AuxShadow's set-up (kind 2): it runs for an enabled light whose Lambert or Blinn term passes
// 0.01 (AuxLightsShader, src/shaders.cpp:1043-1052); the others keep the factor 1, unused.
template <typename T>
__device__ __forceinline__ void aux_shadow_begin(const ParamsT<T> &p, const WaveBufs<T> &wb, const FrameCam<T> &c,
                                              const HitInfo<T> &h, const int64_t px, SecondaryRay<T> &s) {
  const LightT<T> L = p.lights[s.j];
  bool trace = s.j < (unsigned int)p.auxLightNumber || L.enabled;
  if (trace) {
    const V3<T> nrm{wb.normal[s.gp], wb.normal[wb.npix + s.gp], wb.normal[2 * wb.npix + s.gp]};
    const AuxTerms<T> a = aux_light_terms(p, L, p.numberOfLights, h.point, nrm, ray_view(p, c, wb, s.gp, px));
    trace = a.shade > T(0.01) || a.shade2 > T(0.01);
    s.dir = a.lightVector;
    s.end = a.distance;
  }
  s.r = h.delta;
  s.stepMul = p.DE_factor;
  if (!trace) s.end = T(0);
}

// Origin and direction of ray `ri` in the march precision (the volumetric walk's rayStart and
// view): the camera's for depth 0, the reflected ray's otherwise.
template <typename T>
__device__ __forceinline__ void ray_origin_view(const ParamsT<T> &p, const FrameCam<T> &c, const WaveBufs<T> &wb,
                                                const int64_t ri, const int64_t gp, V3<T> &start, V3<T> &view) {
  if (ri < wb.npix_frame) {
    start = {(T)c.start[0], (T)c.start[1], (T)c.start[2]};
    const int64_t local = gp - c.pixBase;
    camera_dir(p, c, (int)(local % c.width), (int)(local / c.width), view);
  } else {
    start = {(T)wb.ray_start[ri], (T)wb.ray_start[wb.npix + ri], (T)wb.ray_start[2 * wb.npix + ri]};
    view = {(T)wb.ray_dir[ri], (T)wb.ray_dir[wb.npix + ri], (T)wb.ray_dir[2 * wb.npix + ri]};
  }
}

// The threshold a secondary ray compares against with iteration fog or volumetric lights:
// the one of the sample's own distance from the eye, held in a float (the per-pixel engine's
// secondary_thresh, src/shaders.cpp:515-519).
template <typename T>
__device__ __forceinline__ T fog_thresh(const ParamsT<T> &p, const V3<T> point2, const V3<T> eye, const T res,
                                        const T persp) {
  float t;
  if (!p.constantDEThreshold) t = (float)(length3(point2 - eye) * res * persp / p.quality);
  else t = (float)p.quality;
  return (T)t;
}

// The effects variant's job set-up: the plain variant's jobs (shadow, AO, AuxShadow at every
// hit of every depth) and, with volumetric lights, MainShadow and the four predefined lights'
// AuxShadow from every step group of the volumetric walk (src/shaders.cpp:309-343). With
// iteration fog or volumetric lights every march steps at DE factor 1 and compares against
// its samples' eye-distance thresholds (MainShadow, AuxShadow, AmbientOcclusion). detailSize
// after MainShadow is taken as the float threshold it starts from; CalculateDistance reads it
// only in the minN clause (src/fractal.cpp:1291-1293), whose escape in the first iteration
// gives a distance far above any threshold of these scenes.
template <typename T, int FORMULA>
__device__ __forceinline__ bool secondary_begin_efx(const ParamsT<T> &p, const WaveBufs<T> &wb,
                                                    const FrameCam<T> *__restrict__ cams, const int ncams,
                                                    const unsigned int nh, const SecondaryJobs &jn,
                                                    const unsigned int job, SecondaryRay<T> &s) {
  unsigned int q = job;
  bool sample = false;
  unsigned int si = 0;
  if (q < jn.nShadow) {
    s.kind = 0;
    s.gp = (int64_t)wb.hit_list[q];
  } else if ((q -= jn.nShadow) < jn.nAO) {
    s.kind = 1;
    s.j = q / nh;
    s.gp = (int64_t)wb.hit_list[q % nh];
  } else if ((q -= jn.nAO) < jn.nAux) {
    s.kind = 2;
    s.j = q / nh;
    s.gp = (int64_t)wb.hit_list[q % nh];
  } else {
    // sample jobs, result-major: [0] MainShadow, [1, 4] AuxShadow of predefined light r - 1,
    // [5, ...) AO direction r - 5 (iteration fog)
    q -= jn.nAux;
    sample = true;
    const unsigned int r = q / jn.nSamples;
    si = q % jn.nSamples;
    if (p.fakeLights && r == (unsigned int)wb.sample_nres - 1) {
      // the fake lights' orbit trap at the group (src/shaders.cpp:298-307): no march
      const int64_t ri = (int64_t)wb.sample_ray[si];
      const int64_t gpx = pixel_of_ray(wb, ri);
      const FrameCam<T> &cf = cams[frame_of_pixel(cams, ncams, gpx)];
      const int64_t rec = (int64_t)wb.sample_rec[si];
      V3<T> rs, rv;
      ray_origin_view(p, cf, wb, ri, gpx, rs, rv);
      Counters c2{0, 0, 0, 0};
      int L;
      wb.sample_res[(int64_t)r * wb.sample_cap + si] =
          compute<T, FORMULA, 5>(p.f, rs + rv * record_scan(wb.pool_rec + 4 * rec), p.f.N, L, c2, cf.fparam);
      return false;
    }
    s.kind = r == 0 ? 0 : (r < (unsigned int)kSampleShadows ? 2 : 1);
    s.j = r == 0 ? 0u : (r < (unsigned int)kSampleShadows ? r - 1 : r - kSampleShadows);
    s.gp = (int64_t)wb.sample_ray[si];
  }
  const int64_t px = pixel_of_ray(wb, s.gp);
  const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, px)];
  const HitInfo<T> h = hit_info(p, c, wb, s.gp);   // the ray's threshold, depth and delta
  s.fog = (p.iterFog || p.volLightAny) ? 1 : 0;
  s.eye = {(T)c.start[0], (T)c.start[1], (T)c.start[2]};
  s.res = c.resolution;
  s.persp = c.persp;
  s.fpar = c.fparam;
  s.sh = T(1);
  s.maxSoft = T(0);
  s.guard = 0;
  const T deF = s.fog ? T(1) : p.DE_factor;
  const T factor = p.penetrating ? h.delta / c.resolution : p.viewDistanceMax;
  T distThresh = h.thr;
  bool fogGroup = false;   // the group takes part in the iteration fog (positive opacity)
  if (sample) {
    // the group's position and threshold (src/shaders.cpp:309-343)
    const int64_t rec = (int64_t)wb.sample_rec[si];
    V3<T> rs, rv;
    ray_origin_view(p, c, wb, s.gp, px, rs, rv);
    s.point = rs + rv * record_scan(wb.pool_rec + 4 * rec);
    T dd, st;
    load_record(wb.pool_rec + 4 * rec, dd, distThresh, st);
    fogGroup = p.iterFog && iter_opacity(wb.sample_step[si], T(wb.pool_iters[rec]), T(p.f.N), p.iterFogOpacityTrim,
                                         p.iterFogOpacity) > T(0);
  } else {
    s.point = h.point;
  }
  // MainShadow, AmbientOcclusion and AuxShadow compare with the threshold stored in a float
  s.thr = (T)(float)distThresh;
  const T shadowStart = p.f.interiorMode ? distThresh * deF : distThresh;
  bool trace = true;
  if (s.kind == 0) {
    s.dir = {c.lightVect[0], c.lightVect[1], c.lightVect[2]};
    s.end = factor;
    s.r = shadowStart;
    s.detail = s.thr;
    s.stepMul = deF;
    // volumetric light 0, or the iteration fog's main light (src/shaders.cpp:313, 409)
    if (sample)
      trace = (p.volLightAny && p.volLightEnabled[0] != 0) || (fogGroup && p.mainLightIntensity * p.directLight > T(0));
    s.out = sample ? wb.sample_res + si : wb.shadow + s.gp;
  } else {
    // detailSize after MainShadow: the float threshold if its loop ran at least once
    s.detail = (p.shadow && shadowStart < factor) ? s.thr : distThresh;
    if (s.kind == 1) {
      s.dir = {__ldg(&p.aoVec[3 * s.j + 0]), __ldg(&p.aoVec[3 * s.j + 1]), __ldg(&p.aoVec[3 * s.j + 2])};
      s.end = h.delta / c.resolution;
      s.r = h.delta;
      s.stepMul = T(2);
      if (sample) {   // the iteration fog's AO at the group (src/shaders.cpp:444-450)
        trace = fogGroup;
        s.detail = s.thr;
        s.out = wb.sample_res + (int64_t)(kSampleShadows + s.j) * wb.sample_cap + si;
      } else {
        s.out = wb.ao + (int64_t)s.j * wb.npix + s.gp;
      }
    } else if (!sample) {
      aux_shadow_begin(p, wb, c, h, px, s);
      s.stepMul = deF;
      s.out = wb.auxsh + (int64_t)s.j * wb.npix + s.gp;
    } else {
      // the volumetric light of a predefined aux light, or its iteration-fog light
      // (src/shaders.cpp:325-341, 423-441)
      trace = p.numberOfLights > 0 && ((p.volLightAny && p.volLightEnabled[s.j + 1] != 0) || fogGroup) &&
              p.lights[s.j].enabled;
      if (trace) {
        const LightT<T> L = p.lights[s.j];
        const V3<T> d = V3<T>{L.pos[0], L.pos[1], L.pos[2]} - s.point;
        s.end = length3(d);
        s.dir = normalize3(d);
      }
      s.r = h.delta;
      s.stepMul = deF;
      s.detail = s.thr;
      s.out = wb.sample_res + (int64_t)(s.j + 1) * wb.sample_cap + si;
    }
  }
  if (!trace) s.end = T(0);
  if (!(s.r < s.end)) {
    *s.out = (s.kind == 0 && p.softShadow) ? T(1) : s.sh;
    return false;
  }
  return true;
}

// Starts job `job`: MainShadow's (src/shaders.cpp:480-570), AmbientOcclusion's
// (src/shaders.cpp:572-640) or AuxShadow's (src/shaders.cpp:1069-1132) loop set-up for one
// ray. Returns false when the loop body never runs (the result is written at once).
template <typename T, bool EFX = false>
__device__ __forceinline__ bool secondary_begin(const ParamsT<T> &p, const WaveBufs<T> &wb,
                                                const FrameCam<T> *__restrict__ cams, const int ncams,
                                                const unsigned int nh, const SecondaryJobs &jn,
                                                const unsigned int job, SecondaryRay<T> &s) {
  unsigned int k;   // the job's entry of the hit list
  if (job < jn.nShadow) {
    s.kind = 0;
    k = job;
  } else if (job < jn.nShadow + jn.nAO) {
    // AO jobs in blocks of kAoBlock hits, every direction of a block before the next block,
    // so that the block's set-up records stay in cache over its aoCount sweeps; a warp's jobs
    // are still consecutive hits (one tile) in one direction
    const unsigned int q = job - jn.nShadow;
    const unsigned int perBlock = kAoBlock * (unsigned int)p.aoCount;
    const unsigned int b = q / perBlock, r = q - b * perBlock, base = b * kAoBlock;
    s.kind = 1;
    if (nh - base >= kAoBlock) {
      s.j = r / kAoBlock;
      k = base + r % kAoBlock;
    } else {   // the last, partial block
      const unsigned int g = nh - base;
      s.j = r / g;
      k = base + (r - s.j * g);
    }
  } else {
    const unsigned int q = job - jn.nShadow - jn.nAO;
    s.kind = 2;
    s.j = q / nh;
    k = q - s.j * nh;
  }
  s.gp = (int64_t)wb.hit_list[k];
  const int64_t px = pixel_of_ray(wb, s.gp);
  const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, px)];
  // the hit's set-up, formed once per hit by hit_setup_kernel where the launch has it
  const HitSetup<T> h = wb.hit_setup ? load_hit_setup(wb.hit_setup + (int64_t)8 * k) : hit_setup(p, c, wb, s.gp);
  s.point = h.point;
  s.fpar = c.fparam;
  // MainShadow, AmbientOcclusion and AuxShadow compare with the threshold stored in a float
  s.thr = (T)(float)h.thr;
  s.sh = T(1);
  s.maxSoft = T(0);
  s.guard = 0;
  if (s.kind == 0) {
    s.dir = {c.lightVect[0], c.lightVect[1], c.lightVect[2]};
    s.end = h.shadowEnd;
    s.r = h.shadowStart;
    s.detail = s.thr;
    s.stepMul = p.DE_factor;
  } else {
    // detailSize after MainShadow: the float threshold if its loop ran at least once
    s.detail = (p.shadow && h.shadowStart < h.shadowEnd) ? s.thr : h.thr;
    if (s.kind == 1) {
      s.dir = {__ldg(&p.aoVec[3 * s.j + 0]), __ldg(&p.aoVec[3 * s.j + 1]), __ldg(&p.aoVec[3 * s.j + 2])};
      s.end = h.aoEnd;
      s.r = h.delta;
      s.stepMul = T(2);
    }
  }
  if (!(s.r < s.end)) {
    if (s.kind == 0) wb.shadow[s.gp] = p.softShadow ? T(1) : s.sh;
    else wb.ao[(int64_t)s.j * wb.npix + s.gp] = s.sh;
    return false;
  }
  return true;
}

// One loop iteration of the ray after its distance estimate `dist` (maxIter `mi`) at
// point + dir * r. Returns true when the ray has ended (its result is written).
template <typename T, bool EFX = false>
__device__ __forceinline__ bool secondary_step(const ParamsT<T> &p, const WaveBufs<T> &wb, SecondaryRay<T> &s,
                                               const T dist, const bool mi) {
  bool done = false;
  if (s.kind == 0) {
    if (p.softShadow) {
      T angle = (dist - s.thr) / s.r;
      if (angle < T(0)) angle = T(0);
      if (dist < s.thr) angle = T(0);
      T soft = (T(1) - angle / p.softRange);
      if (p.penetrating) soft *= (s.end - s.r) / s.end;
      if (soft < T(0)) soft = T(0);
      if (soft > s.maxSoft) s.maxSoft = soft;
    }
    if (dist < s.thr || s.sh < T(0)) {
      s.sh -= (s.end - s.r) / s.end;
      if (!p.penetrating) s.sh = T(0);
      if (s.sh < T(0)) s.sh = T(0);
      done = true;
    }
  } else if (!EFX || s.kind == 1) {
    if (dist < s.thr || mi || s.sh < T(0)) {
      s.sh -= (s.end - s.r) / s.end;
      if (s.sh < T(0)) s.sh = T(0);
      done = true;
    }
  } else {
    if (dist < s.thr || mi || s.sh < T(0)) {
      if (p.penetrating) {
        s.sh -= (s.end - s.r) / s.end;
        if (s.sh < T(0)) s.sh = T(0);
      } else {
        s.sh = T(0);
      }
      done = true;
    }
  }
  if (!done) {
    s.r = add_mul_rn(s.r, dist, s.stepMul);
    if (!(s.r < s.end) || ++s.guard >= kMaxSecondarySteps) done = true;
  }
  if (done) {
    if constexpr (EFX) {
      *s.out = (s.kind == 0 && p.softShadow) ? (T(1) - s.maxSoft) : s.sh;
    } else {
      if (s.kind == 0) wb.shadow[s.gp] = p.softShadow ? (T(1) - s.maxSoft) : s.sh;
      else wb.ao[(int64_t)s.j * wb.npix + s.gp] = s.sh;
    }
  }
  return done;
}

// Lean FP32 orbits: lanes are refilled per orbit rather than per distance estimate. The
// warp runs orbit iterations in batches of LeanOrbit::kUnroll until wb.orbit_refill of its
// busy lanes have ended their orbits (or all have); then those lanes take their ray's next
// step (or a new ray) and start the next orbit, while the others keep their orbit state.
// Every distance is the one mandelbox_fast / mandelbulb8_fast returns at the same point.
template <int FORMULA>
__device__ __forceinline__ void secondary_lean(const ParamsT<float> &p, const FrameIO &io, const WaveBufs<float> &wb,
                                               const FrameCam<float> *__restrict__ cams, const int ncams) {
  const unsigned int nh = *(volatile unsigned int *)&wb.ctl[1];
  const SecondaryJobs jn = secondary_jobs(p, wb, nh);
  const unsigned int njobs = jn.nShadow + jn.nAO + jn.nAux;
  const unsigned int threshold = (unsigned int)wb.orbit_refill;
  const int minN = p.f.minN;
  Counters cnt{0, 0, 0, 0};
  LeanOrbit<FORMULA> orb(p.f);
  SecondaryRay<float> s{};
  bool active = false, exhausted = false, orbiting = false;
  float odist = 0.0f;
  for (;;) {
    // lanes whose orbit ended: the distance estimate's clamps, then the ray's step
    if (active && !orbiting) {
      cnt.orbit += (unsigned long long)(orb.L + 1);
      cnt.calls += 1;
      bool mi;
      const float d = distance_post(p.f, odist, orb.L, orb.N, minN, s.detail, false, 0.0f, mi);
      if (secondary_step(p, wb, s, d, mi)) {
        active = false;
      } else {
        orb.start(ray_at(s.point, s.dir, s.r), s.fpar);
        orbiting = true;
      }
    }
    // idle lanes take new rays until every lane is busy or the jobs are spent
    for (;;) {
      const bool need = !active && !exhausted;
      if (!__any_sync(0xffffffffu, need)) break;
      if (io.budget_ns && (threadIdx.x & 31) == 0 && deadline_passed(io)) atomicExch(io.error_flag, 1);
      // the flag is only ever set by an expired deadline: no read (an L2 round trip) without one
      const bool stop = io.budget_ns && *(volatile int *)io.error_flag != 0;
      const unsigned int job = claim_jobs(wb.ctl + 2, need);
      if (need) {
        if (stop || job >= njobs) {
          exhausted = true;
        } else if (secondary_begin(p, wb, cams, ncams, nh, jn, job, s)) {
          active = true;
          orb.start(ray_at(s.point, s.dir, s.r), s.fpar);
          orbiting = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, active)) break;
    // orbit iterations until enough busy lanes have ended theirs
    for (;;) {
      if (orbiting && orb.advance(odist)) orbiting = false;
      const unsigned int busy = __ballot_sync(0xffffffffu, active);
      const unsigned int ended = __ballot_sync(0xffffffffu, active && !orbiting);
      if ((unsigned int)__popc(ended) >= threshold || ended == busy) break;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
  }
}

// Two lean Mandelbox orbits at once (mandelbox_fast for each of two points, bit for bit):
// the packed iteration box_iteration_x2 advances both until both have ended. A ray whose
// squared radius passes the bailout keeps iterating with the other (its half of the packed
// state is ignored from then on); its distance and end iteration are taken at its bailout,
// and its bailout bound becomes +inf so that it never triggers again. Returns the two
// distances (0 for an orbit that reached N) and end iterations (N when no bailout).
__device__ __forceinline__ void mandelbox_fast_x2(const FractalT<float> &f, const V3<float> a, const float sA,
                                                  const V3<float> b, const float sB, const int N, float &dA,
                                                  int &LA, float &dB, int &LB) {
  const LeanBoxK k = lean_box_k(f);
  BoxPair o;
  box_pair_start(o, k, f.constantFactor, a.x, a.y, a.z, sA, b.x, b.y, b.z, sB);
  const float kInf = __int_as_float(0x7f800000);
  float thA = 1048576.0f, thB = 1048576.0f;
  dA = dB = 0.0f;
  LA = LB = N;
#pragma unroll 5
  for (int L = 0; L < N; L++) {
    const f2 r2 = box_iteration_x2(k, o);
    const float r2A = f2_lo(r2), r2B = f2_hi(r2);
    if (r2A > thA || r2B > thB) {
      if (r2A > thA) {
        dA = box_bailout_dist(r2A, f2_lo(o.dr));
        LA = L;
        thA = kInf;
      }
      if (r2B > thB) {
        dB = box_bailout_dist(r2B, f2_hi(o.dr));
        LB = L;
        thB = kInf;
      }
      if (thA == kInf && thB == kInf) break;
    }
  }
}

// Shadow / AO rays of the lean FP32 Mandelbox two per thread (slots 0 and 1), so that the
// orbit iterations of both run as packed f32x2 instructions (one issue slot for two FMAs;
// the stage is issue-bound). Each slot follows secondary_kernel's per-estimate loop: a
// distance estimate, then the ray's step (secondary_step), refills when 2 x refill_min of
// the warp's 64 slots are idle (one atomicAdd for all of them: slot-0 jobs first, then
// slot-1 jobs). An idle slot's orbit repeats the other slot's point and is discarded.
// Results are bit-identical to secondary_kernel's: the same orbit values, clamps and steps.
// Measured on the 1080p Mandelbox (GB300): 12.1 ms against secondary_kernel's 9.8 ms. The
// packed iteration alone is 18 % faster (26 % fewer instructions, but the FMA and ALU pipes
// then throttle issue), while here the per-estimate tails run twice per lane, a pair waits for
// its longer orbit, and 80 registers leave 22 warps per SM against 36: 6 % fewer instructions
// at 70 % issue against 88 %. So it is opt-in (opts.pair_rays = 1).
// (A template, so that every translation unit that includes this header may instantiate it.)
template <int FORMULA>
__global__ void __launch_bounds__(128) secondary_pair_kernel(const __grid_constant__ ParamsT<float> p,
                                                             const FrameIO io, const WaveBufs<float> wb,
                                                             const FrameCam<float> *__restrict__ cams,
                                                             const int ncams) {
  static_assert(FORMULA == 8, "the packed orbit is the lean Mandelbox's");
  const unsigned int nh = *(volatile unsigned int *)&wb.ctl[1];
  const SecondaryJobs jn = secondary_jobs(p, wb, nh);
  const unsigned int njobs = jn.nShadow + jn.nAO + jn.nAux;
  const unsigned int lane = threadIdx.x & 31u;
  const int N = p.f.N, minN = p.f.minN;
  Counters cnt{0, 0, 0, 0};
  SecondaryRay<float> s0{}, s1{};
  bool act0 = false, act1 = false, exhausted = false;
  for (;;) {
    const bool need0 = !act0 && !exhausted, need1 = !act1 && !exhausted;
    const unsigned int m0 = __ballot_sync(0xffffffffu, need0), m1 = __ballot_sync(0xffffffffu, need1);
    const unsigned int idle = (unsigned int)(__popc(m0) + __popc(m1));
    if (idle && (idle >= 2u * (unsigned int)wb.refill_min || !__any_sync(0xffffffffu, act0 || act1))) {
      if (io.budget_ns && lane == 0 && deadline_passed(io)) atomicExch(io.error_flag, 1);
      // the flag is only ever set by an expired deadline: no read (an L2 round trip) without one
      const bool stop = io.budget_ns && *(volatile int *)io.error_flag != 0;
      unsigned int base = 0;
      const unsigned int leader = (unsigned int)(__ffs(m0 | m1) - 1);
      if (lane == leader) base = atomicAdd(wb.ctl + 2, idle);
      base = __shfl_sync(0xffffffffu, base, leader);
      const unsigned int below = (1u << lane) - 1u;
      const unsigned int job0 = base + (unsigned int)__popc(m0 & below);
      const unsigned int job1 = base + (unsigned int)__popc(m0) + (unsigned int)__popc(m1 & below);
      if (need0) {
        if (stop || job0 >= njobs) exhausted = true;
        else act0 = secondary_begin(p, wb, cams, ncams, nh, jn, job0, s0);
      }
      if (need1) {
        if (stop || job1 >= njobs) exhausted = true;
        else act1 = secondary_begin(p, wb, cams, ncams, nh, jn, job1, s1);
      }
    }
    if (!__any_sync(0xffffffffu, act0 || act1)) {
      if (__all_sync(0xffffffffu, exhausted)) break;
      continue;
    }
    if (act0 || act1) {
      const V3<float> q0 = act0 ? ray_at(s0.point, s0.dir, s0.r) : ray_at(s1.point, s1.dir, s1.r);
      const V3<float> q1 = act1 ? ray_at(s1.point, s1.dir, s1.r) : q0;
      const float f0 = act0 ? s0.fpar : s1.fpar, f1 = act1 ? s1.fpar : f0;
      float d0, d1;
      int L0, L1;
      mandelbox_fast_x2(p.f, q0, f0, q1, f1, N, d0, L0, d1, L1);
      if (act0) {   // CalculateDistance's post-processing, then the ray's step
        cnt.orbit += (unsigned long long)(L0 + 1);
        cnt.calls += 1;
        bool mi;
        d0 = distance_post(p.f, d0, L0, N, minN, s0.detail, false, 0.0f, mi);
        if (secondary_step(p, wb, s0, d0, mi)) act0 = false;
      }
      if (act1) {
        cnt.orbit += (unsigned long long)(L1 + 1);
        cnt.calls += 1;
        bool mi;
        d1 = distance_post(p.f, d1, L1, N, minN, s1.detail, false, 0.0f, mi);
        if (secondary_step(p, wb, s1, d1, mi)) act1 = false;
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
  }
  if (lane == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
  }
}

template <typename T, int FORMULA, bool FAST, bool EFX = false>
__global__ void __launch_bounds__(128) secondary_kernel(const __grid_constant__ ParamsT<T> p, const FrameIO io, const WaveBufs<T> wb,
                                                        const FrameCam<T> *__restrict__ cams, const int ncams) {
  if constexpr (FAST && !EFX && sizeof(T) == 4 && (FORMULA == 8 || FORMULA == 2)) {
    if (wb.orbit_refill > 0) {
      secondary_lean<FORMULA>(p, io, wb, cams, ncams);
      return;
    }
  }
  const unsigned int nh = *(volatile unsigned int *)&wb.ctl[1];
  const SecondaryJobs jn = secondary_jobs<T, EFX>(p, wb, nh);
  const unsigned int njobs = jn.nShadow + jn.nAO + jn.nAux + (unsigned int)wb.sample_nres * jn.nSamples;
  Counters cnt{0, 0, 0, 0};
  bool active = false, exhausted = false;
  SecondaryRay<T> s{};
  for (;;) {
    // a warp claims new jobs once refill_min of its lanes are idle, or when none is busy
    const bool need = !active && !exhausted;
    const unsigned int needMask = __ballot_sync(0xffffffffu, need);
    if (needMask && (__popc(needMask) >= (unsigned int)wb.refill_min || !__any_sync(0xffffffffu, active))) {
      if (io.budget_ns && (threadIdx.x & 31) == 0 && deadline_passed(io)) atomicExch(io.error_flag, 1);
      // the flag is only ever set by an expired deadline: no read (an L2 round trip) without one
      const bool stop = io.budget_ns && *(volatile int *)io.error_flag != 0;
      const unsigned int job = claim_jobs(wb.ctl + 2, need);
      if (need) {
        if (stop || job >= njobs) exhausted = true;
        else if constexpr (EFX) active = secondary_begin_efx<T, FORMULA>(p, wb, cams, ncams, nh, jn, job, s);
        else active = secondary_begin<T>(p, wb, cams, ncams, nh, jn, job, s);
      }
    }
    if (!__any_sync(0xffffffffu, active)) {
      if (__all_sync(0xffffffffu, exhausted)) break;
      continue;
    }
    if (active) {
      const V3<T> point2 = ray_at(s.point, s.dir, s.r);
      if constexpr (EFX) {
        if (s.fog) {   // the sample's own threshold; MainShadow's detailSize follows it
          s.thr = fog_thresh(p, point2, s.eye, s.res, s.persp);
          if (s.kind == 0) s.detail = s.thr;
        }
      }
      int L;
      bool mi;
      const T dist = wave_distance<T, FORMULA, FAST>(p.f, point2, s.detail, p.f.N, p.f.minN, false, L, mi, cnt, s.fpar);
      if constexpr (EFX) {
        // iteration fog absorbs along every march (MainShadow, AmbientOcclusion, AuxShadow:
        // src/shaders.cpp:535-539, 655-659, 1095-1099), at the march's own step factor
        if (p.iterFog)
          s.sh -= iter_opacity(dist * s.stepMul, T(L), T(p.f.N), p.iterFogOpacityTrim, p.iterFogOpacity) *
                  (s.end - s.r) / s.end;
      }
      if (secondary_step<T, EFX>(p, wb, s, dist, mi)) active = false;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
  }
}


// VolumetricShader (src/shaders.cpp:185-478; glow, visible aux lights, post fog, volumetric
// fog) reading the pooled records far to near; same arithmetic as `volumetric` in
// render_core.cuh.
template <typename T, bool EFX>
__device__ __forceinline__ void volumetric_pool(const ParamsT<T> &p, const PoolRecords<T> &pr, const int stepCount,
                                                const T depth, const V3<T> rayStart, const V3<T> view,
                                                const VolSamples<T> vs, const uint32_t pixel, T out[4],
                                                float &totalOpacityOut, bool &opacitySet) {
  uint32_t group = vs.base;
  float totalOpacity = 0.0f;
  const T glow = T(stepCount) * p.glowIntensity / T(512) * p.DE_factor;
  T glowN = T(1) - glow;
  if (glowN < T(0)) glowN = T(0);
  const T glowR = (T(p.glow1[0]) * glowN + T(p.glow2[0]) * glow) / T(65536);
  const T glowG = (T(p.glow1[1]) * glowN + T(p.glow2[1]) * glow) / T(65536);
  const T glowB = (T(p.glow1[2]) * glowN + T(p.glow2[2]) * glow) / T(65536);
  const T fogIntensity = p.fogDensity;
  // The FP32 policy's plain variant forms the group terms with the host's reciprocals and
  // pre-scaled colours and with approximate quotients (__fdividef) where the divisor varies:
  // a few ulp of the group's opacities, against five correctly rounded divisions per group.
  constexpr bool kFastTerms = sizeof(T) == 4 && !EFX;
  const T glowPerDepth = kFastTerms ? glow / depth : T(0);
  T totalStep = T(0);
  // records of W values: the effects variant's (dist, thr, step, scan), the plain variant's
  // narrow (dist, thr), whose step the walk recomputes from the record before
  constexpr int W = EFX ? 4 : 2;
  const T stepFrac = p.f.interiorMode ? T(0.8) : T(0.5);
  int32_t chunk = pr.last;
  int chunkBase = (pr.lastRec / kChunk) * kChunk;   // first record index of `chunk`
  int32_t link = (stepCount > 1 && chunk >= 0) ? pr.prev[chunk] : -1;   // the chunk before `chunk`
  prefetch_chunk<W>(pr, link);
  // the chunk holding record `at` (the walk only moves toward the ray's start)
  auto seek = [&](const int at) -> int64_t {
    while (at < chunkBase) {
      chunk = link;
      chunkBase -= kChunk;
      link = pr.prev[chunk];
      prefetch_chunk<W>(pr, link);
    }
    return (int64_t)chunk * kChunk + (at - chunkBase);
  };
  // narrow records: records `index` and index - 1 are read ahead, one turn apart, so that
  // each turn's load (of index - 2) overlaps the turn's arithmetic
  T curDist = T(0), curThr = T(0), prevDist = T(0), prevThr = T(0);
  if (!EFX && stepCount > 1) {
    load_record_narrow(pr.rec + 2 * seek(stepCount - 1), curDist, curThr);
    load_record_narrow(pr.rec + 2 * seek(stepCount - 2), prevDist, prevThr);
  }
  for (int index = stepCount - 1; index > 0; index--) {
    T distance, dist_thresh, step;
    int64_t rec = 0;
    if constexpr (EFX) {
      rec = seek(index);
      load_record(pr.rec + 4 * rec, distance, dist_thresh, step);
    } else {
      T nextDist = T(0), nextThr = T(0);
      if (index >= 2) load_record_narrow(pr.rec + 2 * seek(index - 2), nextDist, nextThr);
      // the step that reached record `index` is the march's step after record index - 1
      step = march_step(p, prevDist, prevThr, stepFrac, pixel, (uint32_t)(index - 1));
      distance = curDist;
      dist_thresh = curThr;
      curDist = prevDist;
      curThr = prevThr;
      prevDist = nextDist;
      prevThr = nextThr;
    }
    totalStep += step;
    if (totalStep < dist_thresh * p.quality) continue;
    step = totalStep;
    totalStep = T(0);
    const T glowOpacity = kFastTerms ? step * glowPerDepth : glow * step / depth;
    out[0] = glowOpacity * glowR + (T(1) - glowOpacity) * out[0];
    out[1] = glowOpacity * glowG + (T(1) - glowOpacity) * out[1];
    out[2] = glowOpacity * glowB + (T(1) - glowOpacity) * out[2];
    out[3] += glowOpacity;
    if (EFX && p.auxLightVisibility > T(0) && p.numberOfLights > 0)
      visible_aux_lights<T>(p, rayStart + view * record_scan(pr.rec + 4 * rec), view, step, out);
    // the group's shadow-stage results (fake and volumetric lights, iteration fog)
    const bool sampled =
        EFX && (p.volLightAny || p.iterFog || p.fakeLights) && group_has_sample(p, vs.iters, rec, step);
    if (EFX && p.fakeLights) fake_light_glow<T>(p, vs.res[(int64_t)vs.fakeRes * vs.cap + group], step, out);
    if (EFX && p.volLightAny) {
      const T aux[4] = {vs.res[1 * (int64_t)vs.cap + group], vs.res[2 * (int64_t)vs.cap + group],
                        vs.res[3 * (int64_t)vs.cap + group], vs.res[4 * (int64_t)vs.cap + group]};
      volumetric_light_terms<T>(p, rayStart + view * record_scan(pr.rec + 4 * rec), step, vs.res[group], aux, out);
    }
    if (p.postFog) {
      T fogDensity = kFastTerms ? step * p.fogInvVisibility : step / p.fogVisibility;
      if (fogDensity > T(1)) fogDensity = T(1);
      if constexpr (kFastTerms) {
        for (int c = 0; c < 3; c++) out[c] = fogDensity * p.fogColorS[c] + (T(1) - fogDensity) * out[c];
      } else {
        out[0] = fogDensity * T(p.fogColor[0]) / T(65536) + (T(1) - fogDensity) * out[0];
        out[1] = fogDensity * T(p.fogColor[1]) / T(65536) + (T(1) - fogDensity) * out[1];
        out[2] = fogDensity * T(p.fogColor[2]) / T(65536) + (T(1) - fogDensity) * out[2];
      }
      totalOpacity = (float)(fogDensity + (T(1) - fogDensity) * (T)totalOpacity);
      out[3] = fogDensity + (T(1) - fogDensity) * out[3];
    }
    if (kFastTerms && fogIntensity > T(0)) {
      const float densityTemp =
          __fdividef((float)step * (float)p.fogDistFactor, fmaf((float)distance, (float)distance, (float)p.fogDistFactor2));
      const float k = fminf((float)distance * (float)p.fogInvC1Dist, 1.0f);
      const float k2 = fminf((float)distance * (float)p.fogInvC2Dist * k, 1.0f);
      const float kn = 1.0f - k, kn2 = 1.0f - k2;
      const float fi = (float)fogIntensity * densityTemp;
      const float fogDensity = fminf(__fdividef(0.3f * fi, 1.0f + fi), 1.0f);
      const float keep = 1.0f - fogDensity;
      for (int c = 0; c < 3; c++) {
        const float fc = ((float)p.fogCol1S[c] * kn + (float)p.fogCol2S[c] * k) * kn2 + (float)p.fogCol3S[c] * k2;
        out[c] = (T)(fogDensity * fc + keep * (float)out[c]);
      }
      totalOpacity = fogDensity + keep * totalOpacity;
      out[3] = (T)(fogDensity + keep * (float)out[3]);
    } else if (fogIntensity > T(0)) {
      const T fogReduce = p.fogDistFactor;
      const T densityTemp = (step * fogReduce) / (distance * distance + fogReduce * fogReduce);
      T k = distance / p.fogC1Dist;
      if (k > T(1)) k = T(1);
      T kn = T(1) - k;
      T fr = (T(p.fogCol1[0]) * kn + T(p.fogCol2[0]) * k);
      T fg = (T(p.fogCol1[1]) * kn + T(p.fogCol2[1]) * k);
      T fb = (T(p.fogCol1[2]) * kn + T(p.fogCol2[2]) * k);
      T k2 = distance / p.fogC2Dist * k;
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
    if (EFX && p.iterFog && sampled)
      iteration_fog_term<T>(p, rayStart + view * record_scan(pr.rec + 4 * rec), step, vs.iters[rec], vs.res + group,
                            vs.cap, out, totalOpacity);
    if (sampled) group++;
    if (totalOpacity > 1.0f) totalOpacity = 1.0f;
    if (out[3] > T(1)) out[3] = T(1);
    totalOpacityOut = totalOpacity;
    opacitySet = true;
  }
}

// The slow shading's normal (CalculateNormals, src/shaders.cpp:713-757): the sum over the
// 11^3 offsets p2 in [-1, 1]^3 (steps of 0.2 accumulated in double, as the reference's loop
// forms them) of p2 x distance(point + p2 dn). One pixel's 1331 estimates are up to
// 1331 x N5 orbit iterations, which on one lane bound the whole frame; here the warp computes
// them for each of its hit pixels in turn, 42 per lane, into shared memory, and the pixel's
// own lane sums them in the reference's loop order (so the FP64 sum is the reference's).
// `need` marks the lanes whose pixel is a hit; each gets its unnormalised sum in `sum`.
// `axis` is the warp's 11-entry table of offsets in shared memory.
constexpr int kSlowAxis = 11, kSlowSamples = kSlowAxis * kSlowAxis * kSlowAxis;
template <typename T, int FORMULA, bool FAST>
__device__ __forceinline__ void slow_normal_warp(const ParamsT<T> &p, const WaveBufs<T> &wb,
                                              const FrameCam<T> *__restrict__ cams, const int ncams,
                                              const int64_t gw, const bool need, T *dists, T *axis, V3<T> *sum,
                                              Counters *cntOut) {
  const unsigned int lane = threadIdx.x & 31u;
  Counters cnt{0, 0, 0, 0};
  if (lane == 0) {
    double v = -1.0;
    for (int i = 0; i < kSlowAxis; i++) {   // -1.0, -0.8, ... 0.9999999999999999 (<= 1.0)
      axis[i] = (T)v;
      v += 0.2;
    }
  }
  __syncwarp();
  unsigned int mask = __ballot_sync(0xffffffffu, need);
  while (mask) {
    const unsigned int j = (unsigned int)(__ffs(mask) - 1);
    mask &= mask - 1u;
    const int64_t gj = gw + j;
    const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, gj)];
    const HitInfo<T> h = hit_info(p, c, wb, gj);
    T dn = h.delta * p.smoothness;
    if (p.f.interiorMode) dn = h.thr * p.quality * T(0.2) * p.smoothness;
    for (int k = (int)lane; k < kSlowSamples; k += 32) {
      const int ix = k / (kSlowAxis * kSlowAxis), iy = (k / kSlowAxis) % kSlowAxis, iz = k % kSlowAxis;
      const V3<T> p2{axis[ix], axis[iy], axis[iz]};
      int L;
      bool mi;
      dists[k] = distance_est<T, FORMULA, FAST>(p.f, h.point + p2 * dn, h.thr, p.f.N5, p.f.minN, true, L, mi, cnt,
                                                c.fparam);
    }
    __syncwarp();
    if (lane == j) {
      V3<T> n{T(0), T(0), T(0)};
      for (int k = 0; k < kSlowSamples; k++) {
        const int ix = k / (kSlowAxis * kSlowAxis), iy = (k / kSlowAxis) % kSlowAxis, iz = k % kSlowAxis;
        const V3<T> p2{axis[ix], axis[iy], axis[iz]};
        n = n + p2 * dists[k];
      }
      *sum = n;
    }
    __syncwarp();
  }
  cntOut->orbit += cnt.orbit;
  cntOut->calls += cnt.calls;
}

// ---------------------------------------------------------------------------
// Auxiliary lights at a hit (AuxLightsShader, src/shaders.cpp:997-1067), each weighed by its
// AuxShadow from the shadow stage: the diffuse and specular sums.
template <typename T>
__device__ __forceinline__ void aux_light_sums(const ParamsT<T> &p, const WaveBufs<T> &wb, const int64_t ri,
                                               const V3<T> point, const V3<T> nrm, const V3<T> viewT, T aux[3],
                                               T auxSpec[3]) {
  const int number = p.numberOfLights;
  for (int i = 0; i < number; i++) {
    const LightT<T> L = p.lights[i];
    if (!(i < p.auxLightNumber || L.enabled)) continue;
    const AuxTerms<T> a = aux_light_terms(p, L, number, point, nrm, viewT);
    T sh1 = a.shade, sh2 = a.shade2;
    if ((sh1 > T(0.01) || sh2 > T(0.01)) && p.shadow) {
      const T light = wb.auxsh[(int64_t)i * wb.npix + ri];
      sh1 *= light;
      sh2 *= light;
    } else if (p.shadow) {
      sh1 = T(0);
      sh2 = T(0);
    }
    for (int k = 0; k < 3; k++) {
      aux[k] += sh1 * T(L.colour[k]) / T(65536);
      auxSpec[k] += sh2 * T(L.colour[k]) / T(65536);
    }
  }
}

// Fake (orbit trap) lights at a hit (FakeLights, src/shaders.cpp:1225-1271): the trap distance
// and its gradient by forward differences of dist_thresh x smoothness give a light direction;
// Lambert and Blinn terms of that light.
template <typename T, int FORMULA>
__device__ __forceinline__ void fake_light_terms(const ParamsT<T> &p, const V3<T> point, const V3<T> n,
                                                 const V3<T> viewT, const T dist_thresh, const T fparam,
                                                 Counters &cnt, T &fake, T &fakeSpec) {
  const T dl = dist_thresh * p.smoothness;
  int L;
  const T rr = compute<T, FORMULA, 5>(p.f, point, p.f.N, L, cnt, fparam);
  const T fakeLight = p.fakeLightsIntensity / rr;
  const T r = T(1) / (rr + T(1e-30));
  const T rx = T(1) / (compute<T, FORMULA, 5>(p.f, V3<T>{point.x + dl, point.y + T(0), point.z + T(0)}, p.f.N, L, cnt,
                                               fparam) + T(1e-30));
  const T ry = T(1) / (compute<T, FORMULA, 5>(p.f, V3<T>{point.x + T(0), point.y + dl, point.z + T(0)}, p.f.N, L, cnt,
                                               fparam) + T(1e-30));
  const T rz = T(1) / (compute<T, FORMULA, 5>(p.f, V3<T>{point.x + T(0), point.y + T(0), point.z + dl}, p.f.N, L, cnt,
                                               fparam) + T(1e-30));
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


// ObjectShader (src/shaders.cpp:21-112) at the hit of ray `ri` from the stages' results: the
// normal (or the slow shading's, when `slowSum` is given), main light with its shadow and
// specular term, surface colour, AO and environment mapping. Writes the object and specular
// terms as the reflection loop combines them (src/Render3D.cpp:541-552) and the colour.
template <typename T, int FORMULA, bool FAST, bool EFX>
__device__ __forceinline__ void shade_hit(const ParamsT<T> &p, const FrameCam<T> &c, const WaveBufs<T> &wb,
                                          const int64_t ri, const uint8_t flags, const V3<T> viewT,
                                          const V3<double> viewD, const V3<T> *slowSum, Counters &cnt, T obj[3],
                                          T spec[3], V3<T> &colourOut) {
  const V3<T> lv{c.lightVect[0], c.lightVect[1], c.lightVect[2]};
  const HitInfo<T> h = hit_info(p, c, wb, ri);
  // CalculateNormals (src/shaders.cpp:675-757): 4 DEs at N x 5, minN 0, or the slow
  // shading's 11^3 samples
  V3<T> nrm;
  if (slowSum) {
    nrm = *slowSum;
    if (nrm.x == T(0) && nrm.y == T(0) && nrm.z == T(0)) nrm.x = T(1);
    else nrm = normalize3(nrm);
  } else if (EFX && wb.normal) {   // computed by the normal stage (auxiliary lights)
    nrm = {wb.normal[ri], wb.normal[wb.npix + ri], wb.normal[2 * wb.npix + ri]};
  } else {
    nrm = calc_normal_fp<T, FORMULA, FAST>(p, h.point, h.delta, h.thr, h.thr, cnt, c.fparam);
  }
  const int objectType = (flags >> 4) & 7;
  T shade = dot3(nrm, lv);
  if (shade < T(0)) shade = T(0);
  const T shadeV = p.directLight * ((T(1) - p.shading) + p.shading * shade);
  const T shadow = p.shadow ? wb.shadow[ri] : T(1);
  V3<T> half = normalize3(lv - viewT);
  T shade2 = dot3(nrm, half);
  if (shade2 < T(0)) shade2 = T(0);
  shade2 = m_pow(shade2, T(30)) * T(1);
  if (shade2 > T(15)) shade2 = T(15);
  const T specT = shade2 * p.specular;
  const V3<T> colour = wave_colour<T, FORMULA, FAST>(p, h.point, cnt, c.fparam, objectType);
  colourOut = colour;
  V3<T> ambient{T(0), T(0), T(0)};
  if (p.ao) {
    if (p.fastAO) {
      // detailSize after MainShadow: the float threshold if its loop ran
      const T factor = p.penetrating ? h.delta / c.resolution : p.viewDistanceMax;
      const T shadowStart = p.f.interiorMode ? h.thr * p.DE_factor : h.thr;
      const T detail = (p.shadow && shadowStart < factor) ? (T)(float)h.thr : h.thr;
      const T a = wave_fast_ao<T, FORMULA, FAST>(p, h.point, nrm, h.thr, detail, cnt, c.fparam);
      ambient = {a, a, a};
    } else {
      T acc = T(0);
      for (int jj = 0; jj < p.aoCount; jj++) acc += wb.ao[(int64_t)jj * wb.npix + ri] * p.aoWeight[0];
      const T div = T(p.aoCount) * T(256);
      ambient = {acc / div, acc / div, acc / div};
    }
  }
  const T a2x = ambient.x * p.globalIlum, a2y = ambient.y * p.globalIlum, a2z = ambient.z * p.globalIlum;
  // environment mapping (ObjectShader, src/shaders.cpp:71-76) of the default white texture
  const T env = (p.envMapping ? (T)env_mapping(V3<double>{(double)nrm.x, (double)nrm.y, (double)nrm.z}, viewD)
                              : T(0)) * p.reflect;
  obj[0] = env * ambient.x + (a2x + p.mainLight[0] * shadeV * shadow) * colour.x;
  obj[1] = env * ambient.y + (a2y + p.mainLight[1] * shadeV * shadow) * colour.y;
  obj[2] = env * ambient.z + (a2z + p.mainLight[2] * shadeV * shadow) * colour.z;
  if (EFX && (p.numberOfLights > 0 || p.fakeLights)) {
    // auxiliary and fake lights, added as ObjectShader does (src/shaders.cpp:98-107)
    T aux[3] = {T(0), T(0), T(0)}, auxSpec[3] = {T(0), T(0), T(0)};
    if (p.numberOfLights > 0) aux_light_sums(p, wb, ri, h.point, nrm, viewT, aux, auxSpec);
    T fake = T(0), fakeSpec = T(0);
    if (p.fakeLights) fake_light_terms<T, FORMULA>(p, h.point, nrm, viewT, h.thr, c.fparam, cnt, fake, fakeSpec);
    const T col[3] = {colour.x, colour.y, colour.z};
    for (int k = 0; k < 3; k++) {
      obj[k] += (aux[k] + fake) * col[k];
      spec[k] = auxSpec[k] + fakeSpec + p.mainLight[k] * specT * shadow;
    }
  } else {
    // no auxiliary or fake lights: their specular terms are the reference's zeros
    for (int k = 0; k < 3; k++) spec[k] = T(0) + p.mainLight[k] * specT * shadow;
  }
}

// ---------------------------------------------------------------------------
// Stage 4: per-pixel composition and the cImage writes (src/Render3D.cpp:501-589),
// over every pixel of the batch.
// ---------------------------------------------------------------------------
template <typename T, int FORMULA, bool FAST, bool EFX = false>
__global__ void __launch_bounds__(128, (FAST && sizeof(T) == 4) ? 10 : 1) compose_kernel(const __grid_constant__ ParamsT<T> p, const FrameIO io, const WaveBufs<T> wb,
                                                      const FrameCam<T> *__restrict__ cams, const int ncams) {
  Counters cnt{0, 0, 0, 0};
  const int64_t total = wb.npix_frame;
  const unsigned int lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  // a warp's 32 consecutive pixels of the float RGB and RGB8 layers, staged so that they
  // leave as 16-byte stores (cImage's interleaved layers, src/cimage.hpp:155-162)
  __shared__ __align__(16) float stageImg[4][96];
  __shared__ __align__(16) uint8_t stageCol[4][96];
  // the warp walks the pixels together, 32 at a time, so that it can vote on the vector stores
  for (int64_t gw = (int64_t)blockIdx.x * blockDim.x + warp * 32; gw < total; gw += (int64_t)gridDim.x * blockDim.x) {
    const int64_t gp = gw + lane;
    const bool inBatch = gp < total;
    const FrameCam<T> &c = cams[frame_of_pixel(cams, ncams, inBatch ? gp : total - 1)];
    const int64_t pix = gp - c.pixBase;   // pixel within the frame's own layers
    const int x = (int)(pix % c.width), y = (int)(pix / c.width);
    const bool valid = inBatch && y >= c.row_begin && y < c.row_end;
    T out0 = T(0), out1 = T(0), out2 = T(0);
    V3<T> objColour{T(0), T(0), T(0)};
    V3<T> slowSum{T(0), T(0), T(0)};
    if (p.slowShading) {   // the warp's hit pixels' slow-shading normals, computed together
      extern __shared__ __align__(16) unsigned char composeDyn[];
      __shared__ T slowAxis[4][kSlowAxis];
      T *dists = reinterpret_cast<T *>(composeDyn) + (size_t)warp * kSlowSamples;
      slow_normal_warp<T, FORMULA, FAST>(p, wb, cams, ncams, gw, valid && (wb.flags[gp] & 1), dists, slowAxis[warp],
                                         &slowSum, &cnt);
    }
    if (valid) {
    // the reflection loop (src/Render3D.cpp:441-499): ray d + 1 was marched when ray d hit an
    // object that reflects; the last ray marched closes the loop
    int rayEnd = 0;
    for (int d = 0; d + 1 < (EFX ? wb.rays : 1); d++) {
      const uint8_t f = wb.flags[(int64_t)d * wb.npix_frame + gp];
      if (!(f & 1)) break;
      const int ot = (f >> 4) & 7;
      if ((ot == kObjFractal ? p.reflect : p.primReflect[ot - 1]) == T(0)) break;
      rayEnd = d + 1;
    }
    T result[3] = {T(0), T(0), T(0)};
    T alpha = T(0), opacity = T(0);
    // far to near (src/Render3D.cpp:501-566): each ray's object or background, the farther
    // rays' result weighed by its reflectance, then its VolumetricShader
    for (int d = rayEnd; d >= 0; d--) {
      const int64_t ri = (int64_t)d * wb.npix_frame + gp;
      const uint8_t flags = wb.flags[ri];
      const bool hit = (flags & 1) != 0;
      V3<T> viewT;
      V3<double> viewD;
      if (d == 0) {
        camera_dir(p, c, x, y, viewT);
        viewD = {(double)viewT.x, (double)viewT.y, (double)viewT.z};
      } else {
        viewD = {wb.ray_dir[ri], wb.ray_dir[wb.npix + ri], wb.ray_dir[2 * wb.npix + ri]};
        viewT = {(T)viewD.x, (T)viewD.y, (T)viewD.z};
      }
      T obj[3] = {T(0), T(0), T(0)}, spec[3] = {T(0), T(0), T(0)}, bg[3] = {T(0), T(0), T(0)};
      T reflect = T(0);
      if (hit) {
        V3<T> colour;
        shade_hit<T, FORMULA, FAST, EFX>(p, c, wb, ri, flags, viewT, viewD, (p.slowShading && d == 0) ? &slowSum : nullptr,
                                    cnt, obj, spec, colour);
        if (d == 0) objColour = colour;
        const int ot = (flags >> 4) & 7;
        reflect = ot == kObjFractal ? p.reflect : p.primReflect[ot - 1];
      } else {
        const V3<T> b = background(p, viewT);
        bg[0] = b.x;
        bg[1] = b.y;
        bg[2] = b.z;
      }
      T base[3];
      for (int k = 0; k < 3; k++) {
        if (d != rayEnd) base[k] = result[k] * reflect + (T(1) - reflect) * (obj[k] + bg[k]) + spec[k];
        else base[k] = obj[k] + bg[k] + spec[k];
      }
      T a, o;
      if (flags & 4) {
        // a long ray of the overflow pass: its volumetric pass was folded into an affine map
        const T A = wb.vol[0 * wb.npix + ri];
        result[0] = A * base[0] + wb.vol[1 * wb.npix + ri];
        result[1] = A * base[1] + wb.vol[2 * wb.npix + ri];
        result[2] = A * base[2] + wb.vol[3 * wb.npix + ri];
        a = wb.vol[4 * wb.npix + ri];
        o = wb.vol[5 * wb.npix + ri];
      } else {
        // VolumetricShader over the ray's pooled step records, far to near, on this base colour
        T res[4] = {base[0], base[1], base[2], hit ? T(1) + T(0) : T(0)};
        float totalOpacity = 0.0f;
        bool set = false;
        if (p.needVolumetric) {
          const int count = wb.count[ri];
          const PoolRecords<T> pr{wb.pool_rec, wb.pool_prev, wb.last_chunk[ri], hit ? count : count - 1};
          const V3<T> rayStart = d == 0 ? V3<T>{(T)c.start[0], (T)c.start[1], (T)c.start[2]}
                                        : V3<T>{(T)wb.ray_start[ri], (T)wb.ray_start[wb.npix + ri],
                                                (T)wb.ray_start[2 * wb.npix + ri]};
          const VolSamples<T> vs{wb.sample_res, wb.pool_iters, wb.sample_cap, wb.sample_ray ? wb.sample_base[ri] : 0u,
                                 wb.sample_nres - 1};
          volumetric_pool<T, EFX>(p, pr, count, wb.scan[ri], rayStart, viewT, vs, (uint32_t)gp, res, totalOpacity,
                                  set);
        }
        result[0] = res[0];
        result[1] = res[1];
        result[2] = res[2];
        a = res[3];
        o = (T)totalOpacity;
      }
      if (d == 0) {
        alpha = a;
        opacity = o;
      }
    }
    out0 = result[0];
    out1 = result[1];
    out2 = result[2];
    const bool hit = (wb.flags[gp] & 1) != 0;
    const double depth = hit ? (double)wb.scan[gp] : 1e20;
    if (c.opacity) c.opacity[pix] = to_u16_x86((double)opacity * 65535.0);
    if (c.alpha) c.alpha[pix] = to_u16_x86((double)alpha * 65535.0);
    if (c.zbuffer) c.zbuffer[pix] = (float)depth;
    // debug layer: 0 miss, 1 hit, 3 hit whose exact_hit refinement missed the level set
    if (c.hit) c.hit[pix] = hit ? ((wb.flags[gp] & 8) ? 3 : 1) : 0;
    if (c.iters) c.iters[pix] = wb.iters[gp];
    if (c.depth) c.depth[pix] = depth;
    }
    // The interleaved layers: 16-byte stores of the warp's 32 pixels, staged in shared memory,
    // when all of them lie in one frame's rendered rows at 16-byte-aligned addresses.
    const int64_t base0 = __shfl_sync(0xffffffffu, c.pixBase, 0);
    const int64_t pix0 = gw - base0;     // the frame pixel of lane 0
    const bool aligned = (!c.image_float || ((uintptr_t)(c.image_float + 3 * pix0) & 15u) == 0) &&
                         (!c.colour || ((uintptr_t)(c.colour + 3 * pix0) & 15u) == 0);
    const bool vec = __all_sync(0xffffffffu, valid && c.pixBase == base0 && aligned);
    const uint8_t col[3] = {to_u8_x86((double)(objColour.x * T(255))), to_u8_x86((double)(objColour.y * T(255))),
                            to_u8_x86((double)(objColour.z * T(255)))};
    if (vec) {
      // 32 pixels x 12 bytes = 24 float4 stores, 32 x 3 bytes = 6 uint4 stores
      float *si = stageImg[warp];
      uint8_t *sc = stageCol[warp];
      si[3 * lane + 0] = (float)out0;
      si[3 * lane + 1] = (float)out1;
      si[3 * lane + 2] = (float)out2;
      sc[3 * lane + 0] = col[0];
      sc[3 * lane + 1] = col[1];
      sc[3 * lane + 2] = col[2];
      __syncwarp();
      if (c.image_float && lane < 24)
        reinterpret_cast<float4 *>(c.image_float + 3 * pix0)[lane] = reinterpret_cast<const float4 *>(si)[lane];
      if (c.colour && lane < 6)
        reinterpret_cast<uint4 *>(c.colour + 3 * pix0)[lane] = reinterpret_cast<const uint4 *>(sc)[lane];
      __syncwarp();
    } else if (valid) {
      if (c.image_float) {
        c.image_float[3 * pix + 0] = (float)out0;
        c.image_float[3 * pix + 1] = (float)out1;
        c.image_float[3 * pix + 2] = (float)out2;
      }
      if (c.colour) {
        c.colour[3 * pix + 0] = col[0];
        c.colour[3 * pix + 1] = col[1];
        c.colour[3 * pix + 2] = col[2];
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    cnt.orbit += __shfl_down_sync(0xffffffffu, cnt.orbit, off);
    cnt.calls += __shfl_down_sync(0xffffffffu, cnt.calls, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&io.counters[0], cnt.orbit);
    atomicAdd(&io.counters[1], cnt.calls);
  }
}

}  // namespace dev
}  // namespace mbgb
