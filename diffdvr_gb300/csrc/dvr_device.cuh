// Device building blocks of the ray marcher: camera rays, ray/box slab test,
// volume sampling, transfer functions and blending, each with its adjoint.
//
// The arithmetic restates the reference's per-step math (renderer_camera.cuh,
// renderer_utils.cuh, renderer_interpolation.cuh, renderer_tf.cuh,
// renderer_blending.cuh) in FP32 with the same operation order, so that the
// plain kernels reproduce the reference bit for bit up to the exp/rsqrt
// instruction accuracy.
#pragma once
#include <type_traits>
#include "dvr_math.cuh"
#include "dvr_params.h"

namespace dvr {

enum { kNearest = 0, kTrilinear = 1 };
enum { kTfIdentity = 0, kTfTexture = 1, kTfLinear = 2, kTfGaussian = 3 };
enum { kBeerLambert = 0, kAlphaBlend = 1 };

__device__ __forceinline__ float fexp(float x) { return __expf(x); }

// 1 - exp(-x) without the cancellation of the direct form, which loses
// relative accuracy when the per-step optical depth x is small: for
// |x| < 1/32 the Taylor series x - x^2/2 + x^3/6 - x^4/24 + x^5/120 (in
// Horner form, truncation error < x^6/720), otherwise 1 - expf(-x).
__device__ __forceinline__ float one_minus_exp_neg(float x) {
  if (fabsf(x) < 0.03125f)
    return x * (1.f - x * (0.5f - x * (0.16666667f - x * (0.041666668f - x * 0.008333334f))));
  return 1.f - expf(-x);
}

// ------------------------------------------------------------------ inputs
__device__ __forceinline__ float in1(const InView& v, int b, int i) {
  return v.p ? static_cast<const float*>(v.p)[b * v.s[0] + i * v.s[1]] : v.val[i];
}
__device__ __forceinline__ f3 in3(const InView& v, int b) { return mk3(in1(v, b, 0), in1(v, b, 1), in1(v, b, 2)); }
__device__ __forceinline__ float in_pix(const InView& v, int b, int y, int x, int i) {
  return static_cast<const float*>(v.p)[b * v.s[0] + y * v.s[1] + x * v.s[2] + i * v.s[3]];
}
__device__ __forceinline__ float step_at(const InView& v, int b, int y, int x) {
  return v.p ? static_cast<const float*>(v.p)[b * v.s[0] + y * v.s[1] + x * v.s[2]] : v.val[0];
}
__device__ __forceinline__ float mat_at(const InView& v, int b, int r, int c) {
  return v.p ? static_cast<const float*>(v.p)[b * v.s[0] + r * v.s[1] + c * v.s[2]] : 0.f;
}

// ------------------------------------------------------------------ camera
// renderer/renderer_camera.cuh:13-59.  The 4x4 value alternative of the
// inverse view matrix is carried in p.cam_value (row-major).
__device__ __forceinline__ void compute_ray(const RenderParams& p, int x, int y, int b, f3& start, f3& dir) {
  if (p.camera_mode == 0) {
    start = mk3(in_pix(p.ray_start, b, y, x, 0), in_pix(p.ray_start, b, y, x, 1), in_pix(p.ray_start, b, y, x, 2));
    dir = mk3(in_pix(p.ray_dir, b, y, x, 0), in_pix(p.ray_dir, b, y, x, 1), in_pix(p.ray_dir, b, y, x, 2));
  } else if (p.camera_mode == 1) {
    f4 row[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (p.cam.p) {
        row[i] = mk4(mat_at(p.cam, b, i, 0), mat_at(p.cam, b, i, 1), mat_at(p.cam, b, i, 2), mat_at(p.cam, b, i, 3));
      } else {
        row[i] = mk4(p.cam_value[4 * i], p.cam_value[4 * i + 1], p.cam_value[4 * i + 2], p.cam_value[4 * i + 3]);
      }
    }
    const float fx = 2 * (x + 0.5f) / float(p.W) - 1;
    const float fy = 2 * (y + 0.5f) / float(p.H) - 1;
    const f4 s0 = mk4(fx, fy, 0.f, 1.f), s1 = mk4(fx, fy, 0.9f, 1.f);
    const f4 w0 = mk4(dot4(row[0], s0), dot4(row[1], s0), dot4(row[2], s0), dot4(row[3], s0));
    const f4 w1 = mk4(dot4(row[0], s1), dot4(row[1], s1), dot4(row[2], s1), dot4(row[3], s1));
    start = mk3(w0.x / w0.w, w0.y / w0.w, w0.z / w0.w);
    const f3 end = mk3(w1.x / w1.w, w1.y / w1.w, w1.z / w1.w);
    dir = normalize3(mk3(end.x - start.x, end.y - start.y, end.z - start.z));
  } else {
    const float fovx = p.fov_y * float(p.W) / float(p.H);
    const float tan_x = tanf(fovx / 2), tan_y = tanf(p.fov_y / 2);
    const f3 eye = mk3(mat_at(p.cam, b, 0, 0), mat_at(p.cam, b, 0, 1), mat_at(p.cam, b, 0, 2));
    const f3 right = mk3(mat_at(p.cam, b, 1, 0), mat_at(p.cam, b, 1, 1), mat_at(p.cam, b, 1, 2));
    const f3 up = mk3(mat_at(p.cam, b, 2, 0), mat_at(p.cam, b, 2, 1), mat_at(p.cam, b, 2, 2));
    const f3 front = cross3(up, right);
    const float fx = 2 * (x + 0.5f) / float(p.W) - 1;
    const float fy = 2 * (y + 0.5f) / float(p.H) - 1;
    const float ax = fx * tan_x, ay = fy * tan_y;
    start = eye;
    dir = normalize3(mk3(front.x + ax * right.x + ay * up.x, front.y + ax * right.y + ay * up.y,
                         front.z + ax * right.z + ay * up.z));
  }
}

// Adjoint of the reference-frame ray generation (compute_ray, camera mode 2;
// renderer/camera_impl.cu:17-36): adds the viewport gradient of one ray with
// start/direction adjoints (adj_start, adj_dir) to g[0..8] (rows eye, right,
// up).  start = eye; dir = d / |d|, d = front + ax right + ay up,
// front = up x right.
__device__ __forceinline__ void viewport_adjoint(const RenderParams& p, int x, int y, int b, f3 adj_start, f3 adj_dir,
                                                 float* g) {
  const float fovx = p.fov_y * float(p.W) / float(p.H);
  const float tan_x = tanf(fovx / 2), tan_y = tanf(p.fov_y / 2);
  const f3 right = mk3(mat_at(p.cam, b, 1, 0), mat_at(p.cam, b, 1, 1), mat_at(p.cam, b, 1, 2));
  const f3 up = mk3(mat_at(p.cam, b, 2, 0), mat_at(p.cam, b, 2, 1), mat_at(p.cam, b, 2, 2));
  const f3 front = cross3(up, right);
  const float ax = (2 * (x + 0.5f) / float(p.W) - 1) * tan_x, ay = (2 * (y + 0.5f) / float(p.H) - 1) * tan_y;
  const f3 d = mk3(front.x + ax * right.x + ay * up.x, front.y + ax * right.y + ay * up.y,
                   front.z + ax * right.z + ay * up.z);
  const float inv = 1.f / sqrtf(dot3(d, d));
  const f3 dir = mk3(d.x * inv, d.y * inv, d.z * inv);
  const float dd = dot3(dir, adj_dir);
  const f3 ad = mk3((adj_dir.x - dir.x * dd) * inv, (adj_dir.y - dir.y * dd) * inv, (adj_dir.z - dir.z * dd) * inv);
  const f3 af_x_up = cross3(ad, up);     // adjoint of right through front = up x right
  const f3 right_x_af = cross3(right, ad);  // adjoint of up through front
  atomicAdd(g + 0, adj_start.x);
  atomicAdd(g + 1, adj_start.y);
  atomicAdd(g + 2, adj_start.z);
  atomicAdd(g + 3, ax * ad.x + af_x_up.x);
  atomicAdd(g + 4, ax * ad.y + af_x_up.y);
  atomicAdd(g + 5, ax * ad.z + af_x_up.z);
  atomicAdd(g + 6, ay * ad.x + right_x_af.x);
  atomicAdd(g + 7, ay * ad.y + right_x_af.y);
  atomicAdd(g + 8, ay * ad.z + right_x_af.z);
}

// renderer/renderer_utils.cuh:60-74 (ternary min/max: NaN handling as the reference)
__device__ __forceinline__ void ray_box(f3 s, f3 d, f3 bmin, f3 bsize, float& tmin, float& tmax) {
  const float ix = 1.0f / d.x, iy = 1.0f / d.y, iz = 1.0f / d.z;
  const float t1 = (bmin.x - s.x) * ix, t2 = (bmin.x + bsize.x - s.x) * ix;
  const float t3 = (bmin.y - s.y) * iy, t4 = (bmin.y + bsize.y - s.y) * iy;
  const float t5 = (bmin.z - s.z) * iz, t6 = (bmin.z + bsize.z - s.z) * iz;
  tmin = rmaxf(rmaxf(rminf(t1, t2), rminf(t3, t4)), rminf(t5, t6));
  tmax = rminf(rminf(rmaxf(t1, t2), rmaxf(t3, t4)), rmaxf(t5, t6));
}

// Per-ray constants of the march.
struct Ray {
  f3 start, dir, bmin, voxel;
  float step, tmin, tmax;
};

__device__ __forceinline__ void setup_ray(const RenderParams& p, int x, int y, int b, Ray& r) {
  r.bmin = in3(p.box_min, b);
  const f3 bsize = in3(p.box_size, b);
  r.voxel = mk3(bsize.x / float(p.X - 1), bsize.y / float(p.Y - 1), bsize.z / float(p.Z - 1));
  compute_ray(p, x, y, b, r.start, r.dir);
  r.step = step_at(p.step, b, y, x);
  ray_box(r.start, r.dir, r.bmin, bsize, r.tmin, r.tmax);
  r.tmin = rmaxf(r.tmin, 0.f);
}

// Upper bound on the samples of a ray, so every march terminates: the
// reference's loop (renderer/renderer_kernels.cuh:60-64) would not for a NaN
// exit distance or a non-positive step, and float(k) stops growing past 2^24.
// Such rays get no samples; regular rays stop at t > tmax long before the bound.
constexpr int kMaxSamplesPerRay = 1 << 24;
__device__ __forceinline__ int max_samples(float tmin, float tmax, float step) {
  if (!(step > 0.f) || !(tmax >= tmin)) return 0;
  const float n = floorf((tmax - tmin) / step) + 3.f;
  return n < float(kMaxSamplesPerRay) ? int(n) : kMaxSamplesPerRay;
}

__device__ __forceinline__ f3 volume_pos(const Ray& r, float t) {
  const f3 w = mk3(r.start.x + t * r.dir.x, r.start.y + t * r.dir.y, r.start.z + t * r.dir.z);
  return mk3((w.x - r.bmin.x) / r.voxel.x, (w.y - r.bmin.y) / r.voxel.y, (w.z - r.bmin.z) / r.voxel.z);
}

// ------------------------------------------------------------------ volume
// Strided volume of one batch entry with FP32 compute.
template <typename VT>
struct VolumeRef {
  const VT* p;
  int sx, sy, sz;
  int X, Y, Z;
  __device__ __forceinline__ float at(int x, int y, int z) const {
    return Storage<VT>::load(p + (x * sx + y * sy + z * sz));
  }
};

template <typename VT>
__device__ __forceinline__ VolumeRef<VT> volume_ref(const RenderParams& p, int b) {
  VolumeRef<VT> v;
  v.p = static_cast<const VT*>(p.volume.p) + b * p.volume.s[0];
  v.sx = int(p.volume.s[1]);
  v.sy = int(p.volume.s[2]);
  v.sz = int(p.volume.s[3]);
  v.X = p.X;
  v.Y = p.Y;
  v.Z = p.Z;
  return v;
}

// Nearest: clamp to [EPS, size-1-EPS], round half away from zero
// (renderer/renderer_interpolation.cuh:36-49).
__device__ __forceinline__ int nearest_coord(float v, int size) {
  const float eps = 1e-7f;
  const float one_eps = 1 + eps;
  return int(roundf(clampf(v, eps, float(size) - one_eps)));
}

// Eight cell corners, index bits (x y z) = (4 2 1), clamped to the volume
// (renderer/renderer_interpolation.cuh:193-207).
template <typename VT>
__device__ __forceinline__ void fetch_corners(const VolumeRef<VT>& v, int ix, int iy, int iz, float* d) {
  const int lx = clampi(ix, 0, v.X - 1), hx = clampi(ix + 1, 0, v.X - 1);
  const int ly = clampi(iy, 0, v.Y - 1), hy = clampi(iy + 1, 0, v.Y - 1);
  const int lz = clampi(iz, 0, v.Z - 1), hz = clampi(iz + 1, 0, v.Z - 1);
  d[0] = v.at(lx, ly, lz);
  d[1] = v.at(lx, ly, hz);
  d[2] = v.at(lx, hy, lz);
  d[3] = v.at(lx, hy, hz);
  d[4] = v.at(hx, ly, lz);
  d[5] = v.at(hx, ly, hz);
  d[6] = v.at(hx, hy, lz);
  d[7] = v.at(hx, hy, hz);
}

// lerp(lerp(lerp(d0, d4, fx), lerp(d2, d6, fx), fy),
//      lerp(lerp(d1, d5, fx), lerp(d3, d7, fx), fy), fz)
// with the x and y lerps paired: corners 0/1, 2/3, 4/5, 6/7 are z-neighbours.
__device__ __forceinline__ float trilerp(const float* d, float fx, float fy, float fz) {
  const float2 x_lo = lerp2(make_float2(d[0], d[1]), make_float2(d[4], d[5]), make_float2(fx, fx));
  const float2 x_hi = lerp2(make_float2(d[2], d[3]), make_float2(d[6], d[7]), make_float2(fx, fx));
  const float2 y = lerp2(x_lo, x_hi, make_float2(fy, fy));
  return lerp1(y.x, y.y, fz);
}

// Trilinear density and its gradient with respect to the volume position.
__device__ __forceinline__ float trilerp_grad(const float* d, float fx, float fy, float fz, f3& g) {
  const float ay0 = lerp1(d[0], d[4], fx), ay1 = lerp1(d[2], d[6], fx);
  const float by0 = lerp1(d[1], d[5], fx), by1 = lerp1(d[3], d[7], fx);
  g.x = lerp1(lerp1(d[4] - d[0], d[6] - d[2], fy), lerp1(d[5] - d[1], d[7] - d[3], fy), fz);
  g.y = lerp1(ay1 - ay0, by1 - by0, fz);
  const float lo = lerp1(ay0, ay1, fy), hi = lerp1(by0, by1, fy);
  g.z = hi - lo;
  return lerp1(lo, hi, fz);
}

// Adds adj times the trilinear weight of each corner (corner order of
// VolumeFast::corners) to g.
__device__ __forceinline__ void add_corner_weights(float* g, float adj, float fx, float fy, float fz) {
  const float gx = 1 - fx, gy = 1 - fy, gz = 1 - fz;
  g[0] += adj * (gx * gy * gz);
  g[1] += adj * (gx * gy * fz);
  g[2] += adj * (gx * fy * gz);
  g[3] += adj * (gx * fy * fz);
  g[4] += adj * (fx * gy * gz);
  g[5] += adj * (fx * gy * fz);
  g[6] += adj * (fx * fy * gz);
  g[7] += adj * (fx * fy * fz);
}

// Gradient of the trilinear interpolant w.r.t. the eight corners and the
// position, in the reference's accumulation order 000,100,010,110,001,101,011,111
// (renderer/renderer_interpolation.cuh:360-387).  acc may be nullptr.
__device__ __forceinline__ f3 trilerp_adjoint(const float* d, float fx, float fy, float fz, float adj, float* acc) {
  const float c[3] = {fx, fy, fz};
  const float f[3] = {1 - fx, 1 - fy, 1 - fz};
  float adj_c[3] = {0, 0, 0}, adj_f[3] = {0, 0, 0};
  constexpr int order[8] = {0, 4, 2, 6, 1, 5, 3, 7};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int idx = order[k];
    const int hx = (idx >> 2) & 1, hy = (idx >> 1) & 1, hz = idx & 1;
    const float wx = hx ? c[0] : f[0], wy = hy ? c[1] : f[1], wz = hz ? c[2] : f[2];
    if (acc) acc[idx] += adj * (wx * wy * wz);
    const float ad = adj * d[idx];
    if (hx) adj_c[0] += ad * wy * wz; else adj_f[0] += ad * wy * wz;
    if (hy) adj_c[1] += ad * wx * wz; else adj_f[1] += ad * wx * wz;
    if (hz) adj_c[2] += ad * wx * wy; else adj_f[2] += ad * wx * wy;
  }
  return mk3(adj_c[0] - adj_f[0], adj_c[1] - adj_f[1], adj_c[2] - adj_f[2]);
}

// ------------------------------------------------------------------ transfer functions
// TF accessor over global memory with arbitrary strides (plain kernels).
struct TfGlobal {
  const float* p;
  int64_t sr, sc;
  int R;
  __device__ __forceinline__ float at(int r, int c) const { return __ldg(p + r * sr + c * sc); }
  __device__ __forceinline__ f4 rgba(int r) const { return mk4(at(r, 0), at(r, 1), at(r, 2), at(r, 3)); }
};
// TF accessor over a dense R*C copy in shared memory (optimized kernels).
// For a piecewise-linear TF (C = 5) it records whether the control-point
// positions are non-decreasing, which lets linear_interval search them in
// log2(R) steps.
template <int C>
struct TfShared {
  const float* p;
  int R;
  bool sorted = false;
  __device__ __forceinline__ TfShared(const float* p_, int R_) : p(p_), R(R_) {
    if constexpr (C == 5) {
      bool s = true;
      for (int i = 0; i + 1 < R; ++i) s &= p[i * C + 4] <= p[(i + 1) * C + 4];
      sorted = s;
    }
  }
  __device__ __forceinline__ float at(int r, int c) const { return p[r * C + c]; }
  __device__ __forceinline__ f4 rgba(int r) const {
    if constexpr (C == 4) {
      const float4 v = reinterpret_cast<const float4*>(p)[r];
      return mk4(v.x, v.y, v.z, v.w);
    } else {
      return mk4(at(r, 0), at(r, 1), at(r, 2), at(r, 3));
    }
  }
};

template <int TF> struct TfChannels;
template <> struct TfChannels<kTfIdentity> { static constexpr int C = 2; };
template <> struct TfChannels<kTfTexture> { static constexpr int C = 4; };
template <> struct TfChannels<kTfLinear> { static constexpr int C = 5; };
template <> struct TfChannels<kTfGaussian> { static constexpr int C = 6; };

// Interval of a piecewise-linear TF: the first i in [0, R-2) whose next
// control point lies above the density, else R-2
// (renderer/renderer_tf.cuh:294-300).
template <class A>
__device__ __forceinline__ int linear_interval(const A& tf, float density) {
  int i;
  for (i = 0; i < tf.R - 2; ++i)
    if (tf.at(i + 1, 4) > density) break;
  return i;
}
// The same from a shared-memory TF: with non-decreasing positions "next
// point above the density" is monotone in i, so a binary search over
// [0, R-2] finds the same first i (a NaN density, above no point, gives
// R-2 either way) in ceil(log2(R-1)) steps that every lane takes alike;
// unsorted positions keep the reference's scan.
__device__ __forceinline__ int linear_interval(const TfShared<5>& tf, float density) {
  if (tf.sorted) {
    int lo = 0, hi = tf.R - 2;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (tf.at(mid + 1, 4) > density) hi = mid;
      else lo = mid + 1;
    }
    return lo;
  }
  int i;
  for (i = 0; i < tf.R - 2; ++i)
    if (tf.at(i + 1, 4) > density) break;
  return i;
}

__device__ __forceinline__ float gauss(float d, float mu, float sigma) {
  return expf(-(d - mu) * (d - mu) / (2 * sigma * sigma));
}
// The same with one fast reciprocal and the fast exponential instead of a
// division and expf (a few ulp apart): the optimized forward kernels' TF
// evaluation.  Every adjoint keeps gauss.
__device__ __forceinline__ float gauss_fast(float d, float mu, float sigma) {
  const float z = (d - mu) * __fdividef(1.f, sigma);
  return __expf(-0.5f * z * z);
}

// renderer/renderer_tf.cuh:62-73, :160-171, :294-313, :507-519.  FAST: the
// Gaussians by gauss_fast (the optimized forward kernels).
template <int TF, bool FAST = false, class A>
__device__ __forceinline__ f4 tf_eval(const A& tf, float density) {
  if constexpr (TF == kTfIdentity) {
    const float d = clampf(density, 0.f, 1.f);
    const float sa = tf.at(0, 0), sc = tf.at(0, 1);
    return mk4(d * sc, d * sc, d * sc, d * sa);
  } else if constexpr (TF == kTfTexture) {
    const int R = tf.R;
    const float d = density * R - 0.5f;
    const int di = int(floorf(d));
    const float df = d - di;
    const f4 a = tf.rgba(clampi(di, 0, R - 1)), c = tf.rgba(clampi(di + 1, 0, R - 1));
    const float2 xy = lerp2(make_float2(a.x, a.y), make_float2(c.x, c.y), make_float2(df, df));
    const float2 zw = lerp2(make_float2(a.z, a.w), make_float2(c.z, c.w), make_float2(df, df));
    return mk4(xy.x, xy.y, zw.x, zw.y);
  } else if constexpr (TF == kTfLinear) {
    const int i = linear_interval(tf, density);
    const f4 a = tf.rgba(i), c = tf.rgba(i + 1);
    const float p0 = tf.at(i, 4), p1 = tf.at(i + 1, 4);
    const float d = clampf(density, p0, p1);
    const float fr = (d - p0) / (p1 - p0);
    return mk4(lerp1(a.x, c.x, fr), lerp1(a.y, c.y, fr), lerp1(a.z, c.z, fr), lerp1(a.w, c.w, fr));
  } else {
    f4 acc = mk4(0, 0, 0, 0);
    for (int i = 0; i < tf.R; ++i) {
      const f4 ci = tf.rgba(i);
      const float ni = FAST ? gauss_fast(density, tf.at(i, 4), tf.at(i, 5)) : gauss(density, tf.at(i, 4), tf.at(i, 5));
      acc.x += ci.x * ni;
      acc.y += ci.y * ni;
      acc.z += ci.z * ni;
      acc.w += ci.w * ni;
    }
    return acc;
  }
}

// TF adjoint (renderer/renderer_tf.cuh:76-104, :174-220, :316-400, :563-614).
// Returns adj_density; TF gradients go to sink.add(r, c, v) when WithTfGrad.
template <int TF, bool WithTfGrad, class A, class Sink>
__device__ __forceinline__ float tf_adjoint(const A& tf, float density, f4 adj, Sink& sink) {
  if constexpr (TF == kTfIdentity) {
    const float dc = clampf(density, 0.f, 1.f);
    const float sa = tf.at(0, 0), sc = tf.at(0, 1);
    const float adj_dc = (adj.x * sc + adj.y * sc + adj.z * sc) + adj.w * sa;
    if constexpr (WithTfGrad) {
      sink.add(0, 0, adj.w * dc);
      sink.add(0, 1, adj.x * dc + adj.y * dc + adj.z * dc);
    }
    return (density > 0 && density < 1) ? adj_dc : 0.f;
  } else if constexpr (TF == kTfTexture) {
    const int R = tf.R;
    const float d = density * R - 0.5f;
    const int di = int(floorf(d));
    const float df = d - di;
    const int i0 = clampi(di, 0, R - 1), i1 = clampi(di + 1, 0, R - 1);
    const f4 a = tf.rgba(i0), c = tf.rgba(i1);
    const float adj_df = dot4(adj, mk4(c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w));
    if constexpr (WithTfGrad) {
      const float w0 = 1 - df;
      sink.add4(i0, mk4(adj.x * w0, adj.y * w0, adj.z * w0, adj.w * w0));
      sink.add4(i1, mk4(adj.x * df, adj.y * df, adj.z * df, adj.w * df));
    }
    return adj_df * R;
  } else if constexpr (TF == kTfLinear) {
    const int i = linear_interval(tf, density);
    const f4 a = tf.rgba(i), c = tf.rgba(i + 1);
    const float p0 = tf.at(i, 4), p1 = tf.at(i + 1, 4);
    const float d2 = clampf(density, p0, p1);
    const float adj_fr = dot4(adj, mk4(c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w));
    if constexpr (std::is_same<A, TfShared<5>>::value) {
      // optimized kernels: one reciprocal of the interval instead of four
      // divisions (the results differ from the quotients by rounding only)
      const float inv = 1.f / (p1 - p0);
      const float fr = (d2 - p0) * inv;
      if constexpr (WithTfGrad) {
        const float w0 = 1 - fr, inv2 = inv * inv;
        sink.add4(i, mk4(adj.x * w0, adj.y * w0, adj.z * w0, adj.w * w0));
        sink.add(i, 4, adj_fr * (d2 - p1) * inv2);
        sink.add4(i + 1, mk4(adj.x * fr, adj.y * fr, adj.z * fr, adj.w * fr));
        sink.add(i + 1, 4, adj_fr * (p0 - d2) * inv2);
      }
      return adj_fr * inv;
    } else {
      const float fr = (d2 - p0) / (p1 - p0);
      const float den = (p1 - p0) * (p1 - p0);
      if constexpr (WithTfGrad) {
        const float w0 = 1 - fr;
        sink.add4(i, mk4(adj.x * w0, adj.y * w0, adj.z * w0, adj.w * w0));
        sink.add(i, 4, adj_fr * (d2 - p1) / den);
        sink.add4(i + 1, mk4(adj.x * fr, adj.y * fr, adj.z * fr, adj.w * fr));
        sink.add(i + 1, 4, adj_fr * (p0 - d2) / den);
      }
      return adj_fr / (p1 - p0);
    }
  } else {
    float adj_density = 0;
    for (int i = 0; i < tf.R; ++i) {
      const f4 ci = tf.rgba(i);
      const float mu = tf.at(i, 4), sigma = tf.at(i, 5);
      const float s2 = sigma * sigma;
      const float ni = gauss(density, mu, sigma);
      const float f1 = (mu - density) / s2 * ni;
      adj_density += dot4(adj, mk4(ci.x * f1, ci.y * f1, ci.z * f1, ci.w * f1));
      if constexpr (WithTfGrad) {
        const float nf1 = -f1;
        const float f2 = f1 * (mu - density) / sigma;
        sink.add4(i, mk4(adj.x * ni, adj.y * ni, adj.z * ni, adj.w * ni));
        sink.add(i, 4, dot4(adj, mk4(ci.x * nf1, ci.y * nf1, ci.z * nf1, ci.w * nf1)));
        sink.add(i, 5, dot4(adj, mk4(ci.x * f2, ci.y * f2, ci.z * f2, ci.w * f2)));
      }
    }
    return adj_density;
  }
}

// ------------------------------------------------------------------ blending
// renderer/renderer_blending.cuh:54-61 (Beer-Lambert), :118-125 (alpha)
template <int BLEND>
__device__ __forceinline__ float blend_alpha(float absorption, float step) {
  if constexpr (BLEND == kBeerLambert) return one_minus_exp_neg(absorption * step);
  else return rminf(1.f, absorption * step);
}

template <int BLEND>
__device__ __forceinline__ f4 blend(f4 acc, f4 cur, float step) {
  const float a = blend_alpha<BLEND>(cur.w, step);
  const float t = 1 - acc.w;
  return mk4(acc.x + t * cur.x * a, acc.y + t * cur.y * a, acc.z + t * cur.z * a, acc.w + t * a);
}

// Adjoint of one blend step given the accumulator alpha before the step
// (alpha_in).  adj_acc is the adjoint of the accumulator after the step on
// entry and before the step on return.  Returns d(loss)/d(step) of this step.
template <int BLEND>
__device__ __forceinline__ float blend_adjoint_core(float alpha_in, f4 cur, float step, float a, f4& adj_acc,
                                                   f4& adj_cur) {
  const f4 ao = adj_acc;
  float adj_alpha = ao.w * (1 - alpha_in);
  float adj_in_alpha = ao.w * (1 - a);
  adj_alpha += ao.x * (cur.x - cur.x * alpha_in) + ao.y * (cur.y - cur.y * alpha_in) +
               ao.z * (cur.z - cur.z * alpha_in);
  adj_in_alpha += ao.x * (-cur.x * a) + ao.y * (-cur.y * a) + ao.z * (-cur.z * a);
  const float wc = a * (1 - alpha_in);
  float adj_w, adj_step;
  if constexpr (BLEND == kBeerLambert) {
    const float e = expf(-cur.w * step);
    adj_w = adj_alpha * step * e;
    adj_step = adj_alpha * cur.w * e;
  } else {
    const bool lin = cur.w * step < 1;
    adj_step = lin ? adj_alpha * cur.w : 0.f;
    adj_w = lin ? adj_alpha * step : 0.f;
  }
  adj_cur = mk4(ao.x * wc, ao.y * wc, ao.z * wc, adj_w);
  adj_acc = mk4(ao.x, ao.y, ao.z, adj_in_alpha);
  return adj_step;
}

// The reference's adjoint: recovers the accumulator before the step by
// inverting the blend (renderer/renderer_blending.cuh:63-98, :127-164).
template <int BLEND>
__device__ __forceinline__ f4 blend_adjoint_invert(f4 acc_out, f4 cur, float step, f4& adj_acc, f4& adj_cur,
                                                   float& adj_step) {
  float a;
  if constexpr (BLEND == kBeerLambert) a = one_minus_exp_neg(cur.w * step);
  else a = rminf(1.0f - 1e-5f, cur.w * step);
  const float alpha_in = (a - acc_out.w) / (a - 1);
  const float t = 1 - alpha_in;
  const f4 prev = mk4(acc_out.x - t * cur.x * a, acc_out.y - t * cur.y * a, acc_out.z - t * cur.z * a, alpha_in);
  adj_step = blend_adjoint_core<BLEND>(alpha_in, cur, step, a, adj_acc, adj_cur);
  return prev;
}

}  // namespace dvr
