// Pre-shaded volumes (VolumeFilterMode/TFMode Preshaded,
// renderer/renderer_interpolation.cuh:393-579, renderer/renderer_tf.cuh:818-854).
//
// The volume is 4 x X x Y x Z: colour (r, g, b) and absorption already
// assigned per voxel, in the first dimension, shared by every batch entry.
// Each channel is interpolated trilinearly at the sample and the "TF" passes
// the result through, so a sample reads 4 x 8 corners and no TF.  The
// adjoint scatters per-channel volume gradients (4 x 8 per cell, flushed on
// cell exit) and, for camera gradients, the position derivative of the four
// interpolants.
//
// Kernels: the forward with one warp per ray and 32 samples per step
// (compositing by warp scan, as the warp-per-ray forward of the density
// path), and the reference's adjoint algorithm (one thread per ray, the
// accumulator recovered by inverting the blend).  EXACT = false reproduces
// the reference's position adjoint, whose z term is summed with the y
// weights' selector (renderer/renderer_interpolation.cuh:543-548 against the
// scalar filter's :368-374), and its step-size adjoint, which keeps the last
// blend term only; EXACT = true gives the exact derivatives.
#pragma once
#include "dvr_kernels.h"
#include "dvr_plain.cuh"
#include "dvr_record.cuh"
#include "dvr_warpray.cuh"

namespace dvr {

// The four channel planes of a pre-shaded volume.
template <typename VT>
struct RgbaVolume {
  const VT* p;
  int64_t sc;             // channel stride
  int sx, sy, sz;
  int X1, Y1, Z1;         // size - 1
  __device__ __forceinline__ void corners(int ix, int iy, int iz, float (&d)[4][8]) const {
    const int lx = clampi(ix, 0, X1), hx = clampi(ix + 1, 0, X1);
    const int ly = clampi(iy, 0, Y1), hy = clampi(iy + 1, 0, Y1);
    const int lz = clampi(iz, 0, Z1), hz = clampi(iz + 1, 0, Z1);
    const int o[8] = {lx * sx + ly * sy + lz * sz, lx * sx + ly * sy + hz * sz, lx * sx + hy * sy + lz * sz,
                      lx * sx + hy * sy + hz * sz, hx * sx + ly * sy + lz * sz, hx * sx + ly * sy + hz * sz,
                      hx * sx + hy * sy + lz * sz, hx * sx + hy * sy + hz * sz};
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int i = 0; i < 8; ++i) d[c][i] = Storage<VT>::load(p + c * sc + o[i]);
  }
  __device__ __forceinline__ f4 sample(float3 q) const {
    const int ix = int(q.x), iy = int(q.y), iz = int(q.z);
    float d[4][8];
    corners(ix, iy, iz, d);
    const float fx = q.x - float(ix), fy = q.y - float(iy), fz = q.z - float(iz);
    return mk4(trilerp(d[0], fx, fy, fz), trilerp(d[1], fx, fy, fz), trilerp(d[2], fx, fy, fz),
               trilerp(d[3], fx, fy, fz));
  }
};

template <typename VT>
__device__ __forceinline__ RgbaVolume<VT> rgba_volume(const RenderParams& p) {
  return RgbaVolume<VT>{static_cast<const VT*>(p.volume.p), p.volume.s[0], int(p.volume.s[1]), int(p.volume.s[2]),
                        int(p.volume.s[3]), p.X - 1, p.Y - 1, p.Z - 1};
}

// Forward: one warp per ray (dynamic fetch in scanline order), 32 samples
// per step, opacity in front of each sample by an "over" scan.  With a
// sample record (p.dens), every ray with samples that finds room stores, for
// sample k, (alpha_k, opacity in front of it) as floats 2k and 2k+1 of its
// run in the pool, the format of the density path's record.
template <int BLEND, typename VT>
__global__ void __launch_bounds__(kFastThreads) preshaded_forward_kernel(const RenderParams p, int* counter) {
  const int lane = threadIdx.x & 31;
  const int rays = p.B * p.H * p.W;
  const RgbaVolume<VT> vol = rgba_volume<VT>(p);
  unsigned long long* const bump = reinterpret_cast<unsigned long long*>(counter + 2);
  while (true) {
    int pos = 0;
    if (lane == 0) pos = atomicAdd(counter, 1);
    pos = __shfl_sync(kFullMask, pos, 0);
    if (pos >= rays) break;
    const int b = pos / (p.H * p.W);
    const int rem = pos - b * p.H * p.W;
    const int y = rem / p.W, x = rem - y * p.W;
    FastRay q;
    fast_setup(p, x, y, b, q);
    const int kmax = max_samples(q.tmin, q.tmax, q.step);
    float* rec = nullptr;
    if (p.dens) {
      // room for kmax (alpha, opacity) pairs, in groups of 4 floats; -1 without samples or room
      const unsigned long long claim = static_cast<unsigned long long>((kmax + 1) >> 1);
      unsigned long long g = 0;
      if (lane == 0 && kmax > 0) g = atomicAdd(bump, claim);
      g = __shfl_sync(kFullMask, g, 0);
      const bool fits = kmax > 0 && g + claim <= static_cast<unsigned long long>(p.dens_units);
      if (lane == 0)
        static_cast<int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] + x * p.dens_off.s[2]] =
            fits ? int(g) : -1;
      if (fits) rec = p.dens + 4 * g;
    }
    float alpha = 0.f, cr = 0.f, cg = 0.f, cb = 0.f;
    int n = 0;
    for (int k0 = 0; k0 < kmax; k0 += 32) {
      const int k = k0 + lane;
      const float t = q.tmin + k * q.step;
      const bool in_ray = k < kmax && !(t > q.tmax);
      f4 c = mk4(0, 0, 0, 0);
      float a = 0.f;
      if (in_ray) {
        c = vol.sample(fast_pos(q, t));
        a = blend_alpha<BLEND>(c.w, q.step);
      }
      float incl = a;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float v = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl = over(v, incl);
      }
      float excl = __shfl_up_sync(kFullMask, incl, 1);
      if (lane == 0) excl = 0.f;
      const float a_in = over(alpha, excl);
      const bool go = in_ray && !(a_in > p.early_out);
      const unsigned gm = __ballot_sync(kFullMask, go);
      const int f = gm == kFullMask ? 32 : __ffs(~gm) - 1;
      if (lane < f) {
        if (rec) __stcs(reinterpret_cast<float2*>(rec) + k, make_float2(a, a_in));
        const float w = (1.f - a_in) * a;
        cr = fmaf(w, c.x, cr);
        cg = fmaf(w, c.y, cg);
        cb = fmaf(w, c.z, cb);
      }
      if (f < 32) {
        alpha = __shfl_sync(kFullMask, a_in, f);
        n = k0 + f;
        break;
      }
      alpha = over(alpha, __shfl_sync(kFullMask, incl, 31));
      n = k0 + 32;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      cr += __shfl_xor_sync(kFullMask, cr, o);
      cg += __shfl_xor_sync(kFullMask, cg, o);
      cb += __shfl_xor_sync(kFullMask, cb, o);
    }
    if (lane == 0) {
      float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
      col[0] = cr;
      col[p.color.s[3]] = cg;
      col[2 * p.color.s[3]] = cb;
      col[3 * p.color.s[3]] = alpha;
      static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = n;
    }
  }
}

// Forward, the reference's algorithm: one thread per ray, samples in order
// (renderer/renderer_kernels.cuh:22-90 with the pre-shaded filter and TF).
template <int BLEND>
__global__ void __launch_bounds__(256) preshaded_plain_forward_kernel(const RenderParams p) {
  const int64_t total = int64_t(p.B) * p.H * p.W;
  const RgbaVolume<float> vol = rgba_volume<float>(p);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    const int b = int(i / (int64_t(p.W) * p.H));
    const int y = int((i - int64_t(b) * p.W * p.H) / p.W);
    const int x = int(i - int64_t(p.W) * (y + int64_t(p.H) * b));
    Ray r;
    setup_ray(p, x, y, b, r);
    f4 acc = mk4(0, 0, 0, 0);
    const int kmax = max_samples(r.tmin, r.tmax, r.step);
    int k;
    for (k = 0; k < kmax; ++k) {
      const float t = r.tmin + k * r.step;
      if (t > r.tmax) break;
      if (acc.w > p.early_out) break;
      const f3 vp = volume_pos(r, t);
      acc = blend<BLEND>(acc, vol.sample(make_float3(vp.x, vp.y, vp.z)), r.step);
    }
    float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
    col[0] = acc.x;
    col[p.color.s[3]] = acc.y;
    col[2 * p.color.s[3]] = acc.z;
    col[3 * p.color.s[3]] = acc.w;
    static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = k;
  }
}

// Adjoint: one thread per ray, reverse march with blend inversion
// (renderer/renderer_kernels.cuh:315-444); volume gradients accumulated per
// cell and channel in registers, flushed on cell exit (z-adjacent corner
// pairs as one vector atomic).  Persistent: the lanes of a warp take the
// next 32 rays of the longest-first list of rays with samples together, so
// a warp's rays have similar lengths and no block idles behind one long ray.
template <int BLEND, typename VT, bool VOLGRAD, bool EXACT>
__global__ void __launch_bounds__(kFastThreads) preshaded_adjoint_kernel(const RenderParams p, const AdjointParams a,
                                                                         const RayOrder order, int* counter,
                                                                         const int* ray_list, const int* ray_count) {
  const RgbaVolume<VT> vol = rgba_volume<VT>(p);
  float* adjv = VOLGRAD ? static_cast<float*>(a.adj_volume.p) : nullptr;
  const int64_t gc = a.adj_volume.s[0], gx = a.adj_volume.s[1], gy = a.adj_volume.s[2], gz = a.adj_volume.s[3];
  const int total = *ray_count;
  const bool need_pos = a.has_camera || a.has_stepsize;
  bool exhausted = false;
  while (true) {
    const int pos = fetch_rays(counter, total, true, exhausted);
    if (__ballot_sync(kFullMask, pos >= 0) == 0u) break;
    int b = 0, x = 0, y = 0;
    // lanes without a ray skip the body; all lanes fetch together at the top
    if (pos >= 0 && order.pixel(ray_list[pos], b, x, y)) {
      Ray r;
      setup_ray(p, x, y, b, r);
      const float* fc = static_cast<const float*>(a.fwd_color.p) + b * a.fwd_color.s[0] + y * a.fwd_color.s[1] +
                        x * a.fwd_color.s[2];
      f4 acc = mk4(fc[0], fc[a.fwd_color.s[3]], fc[2 * a.fwd_color.s[3]], fc[3 * a.fwd_color.s[3]]);
      int k = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
      k = min(k, max_samples(r.tmin, r.tmax, r.step));
      const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] + y * a.adj_color.s[1] +
                        x * a.adj_color.s[2];
      f4 adj_acc = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
      float adj_step = 0.f;
      f3 adj_start = mk3(0, 0, 0), adj_dir = mk3(0, 0, 0);
      int cx = -1, cy = -1, cz = -1;
      float d[4][8], g[4][8];
#pragma unroll
      for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int q = 0; q < 8; ++q) d[c][q] = g[c][q] = 0.f;
      auto flush = [&]() {
        if constexpr (VOLGRAD) {
          if (cx < 0) return;
          const int lx = clampi(cx, 0, p.X - 1), hx = clampi(cx + 1, 0, p.X - 1);
          const int ly = clampi(cy, 0, p.Y - 1), hy = clampi(cy + 1, 0, p.Y - 1);
          const int lz = clampi(cz, 0, p.Z - 1), hz = clampi(cz + 1, 0, p.Z - 1);
          // z-adjacent corner pairs go as one vector atomic where aligned
          const bool pair = gz == 1 && hz == lz + 1;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            float* base = adjv + c * gc;
            VolGradCell<kTrilinear, true>::add_z(base + lx * gx + ly * gy, lz, hz, gz, pair, g[c][0], g[c][1]);
            VolGradCell<kTrilinear, true>::add_z(base + lx * gx + hy * gy, lz, hz, gz, pair, g[c][2], g[c][3]);
            VolGradCell<kTrilinear, true>::add_z(base + hx * gx + ly * gy, lz, hz, gz, pair, g[c][4], g[c][5]);
            VolGradCell<kTrilinear, true>::add_z(base + hx * gx + hy * gy, lz, hz, gz, pair, g[c][6], g[c][7]);
#pragma unroll
            for (int q = 0; q < 8; ++q) g[c][q] = 0.f;
          }
        }
      };
      for (--k; k >= 0; --k) {
        const float t = r.tmin + k * r.step;
        const f3 vp = volume_pos(r, t);
        const int ix = int(vp.x), iy = int(vp.y), iz = int(vp.z);
        if (ix != cx || iy != cy || iz != cz) {
          flush();
          cx = ix, cy = iy, cz = iz;
          vol.corners(ix, iy, iz, d);
        }
        const float fx = vp.x - float(ix), fy = vp.y - float(iy), fz = vp.z - float(iz);
        const f4 cur = mk4(trilerp(d[0], fx, fy, fz), trilerp(d[1], fx, fy, fz), trilerp(d[2], fx, fy, fz),
                           trilerp(d[3], fx, fy, fz));
        f4 adj_cur;
        float step_contrib;
        acc = blend_adjoint_invert<BLEND>(acc, cur, r.step, adj_acc, adj_cur, step_contrib);
        if constexpr (EXACT) adj_step += step_contrib;
        else adj_step = step_contrib;  // the reference assigns (renderer/renderer_blending.cuh:93, :158)
        const float av[4] = {adj_cur.x, adj_cur.y, adj_cur.z, adj_cur.w};
      f3 adj_vp = mk3(0, 0, 0);
      if constexpr (EXACT) {
        // the eight corner weights once for the four channels; the position
        // gradient only where camera or step-size gradients are wanted
        if constexpr (VOLGRAD) {
          const float ux = 1.f - fx, uy = 1.f - fy, uz = 1.f - fz;
          const float w8[8] = {ux * uy * uz, ux * uy * fz, ux * fy * uz, ux * fy * fz,
                               fx * uy * uz, fx * uy * fz, fx * fy * uz, fx * fy * fz};
#pragma unroll
          for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int q = 0; q < 8; ++q) g[c][q] = fmaf(av[c], w8[q], g[c][q]);
        }
        if (need_pos) {
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            f3 gc3;
            trilerp_grad(d[c], fx, fy, fz, gc3);
            adj_vp.x = fmaf(av[c], gc3.x, adj_vp.x);
            adj_vp.y = fmaf(av[c], gc3.y, adj_vp.y);
            adj_vp.z = fmaf(av[c], gc3.z, adj_vp.z);
          }
        }
      } else {
        // the reference's scatter, corner order 000,100,010,110,001,101,011,111
        const float cw[3] = {fx, fy, fz}, fw[3] = {1.f - fx, 1.f - fy, 1.f - fz};
        float adj_c[3] = {0, 0, 0}, adj_f[3] = {0, 0, 0};
        constexpr int order[8] = {0, 4, 2, 6, 1, 5, 3, 7};
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int idx = order[q];
            const int hx = (idx >> 2) & 1, hy = (idx >> 1) & 1, hz = idx & 1;
            const float wx = hx ? cw[0] : fw[0], wy = hy ? cw[1] : fw[1], wz = hz ? cw[2] : fw[2];
            if constexpr (VOLGRAD) g[c][idx] += av[c] * (wx * wy * wz);
            const float ad = av[c] * d[c][idx];
            if (hx) adj_c[0] += ad * wy * wz; else adj_f[0] += ad * wy * wz;
            if (hy) adj_c[1] += ad * wx * wz; else adj_f[1] += ad * wx * wz;
            if (hy) adj_c[2] += ad * wx * wy; else adj_f[2] += ad * wx * wy;  // y selector, as the reference
          }
        adj_vp = mk3(adj_c[0] - adj_f[0], adj_c[1] - adj_f[1], adj_c[2] - adj_f[2]);
      }
      const f3 adj_w = mk3(adj_vp.x / r.voxel.x, adj_vp.y / r.voxel.y, adj_vp.z / r.voxel.z);
        adj_start.x += adj_w.x; adj_start.y += adj_w.y; adj_start.z += adj_w.z;
        adj_dir.x += adj_w.x * t; adj_dir.y += adj_w.y * t; adj_dir.z += adj_w.z * t;
        adj_step += dot3(adj_w, r.dir) * k;
      }
      flush();
      if (a.has_stepsize) {
        float* ps = static_cast<float*>(a.adj_step.p) + b * a.adj_step.s[0] + y * a.adj_step.s[1] + x * a.adj_step.s[2];
        if (a.stepsize_broadcast) atomicAdd(ps, adj_step);
        else *ps = adj_step;
      }
      if (a.has_camera) {
        const float vs[3] = {adj_start.x, adj_start.y, adj_start.z};
        const float vd[3] = {adj_dir.x, adj_dir.y, adj_dir.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (a.camera_broadcast) {
            atomic_out(a.adj_start, b, y, x, c, vs[c]);
            atomic_out(a.adj_dir, b, y, x, c, vd[c]);
          } else {
            write_out(a.adj_start, b, y, x, c, vs[c]);
            write_out(a.adj_dir, b, y, x, c, vd[c]);
          }
        }
      }
    }
  }
}

// Adjoint from the sample record (exact derivatives): one warp per ray, lane
// j on the j-th of 32 consecutive segments of L = ceil(n / 32) samples, the
// scheme of the density path's record kernel.  The record gives every
// sample's incoming opacity, so no blend is inverted; the colours are
// gathered again.  Each lane composes its segment's affine maps of the
// opacity adjoint (adj_in = (1 - a) adj_out - a (c . adj_rgb)), a warp suffix
// scan gives the adjoint at every segment end, and each lane walks its
// segment back to front: per-cell volume-gradient registers flushed on cell
// exit, and (POS) the position chain for camera and step-size gradients,
// summed over the warp per ray.  Rays without a record go to `leftover`.
template <int BLEND, typename VT, bool VOLGRAD, bool POS>
__global__ void __launch_bounds__(kFastThreads) preshaded_record_adjoint_kernel(
    const RenderParams p, const AdjointParams a, const RayOrder order, int* counter, const int* ray_list,
    const int* ray_count, int* leftover) {
  const int lane = threadIdx.x & 31;
  const int total = *ray_count;
  const RgbaVolume<VT> vol = rgba_volume<VT>(p);
  float* adjv = VOLGRAD ? static_cast<float*>(a.adj_volume.p) : nullptr;
  const int64_t gc = a.adj_volume.s[0], gx = a.adj_volume.s[1], gy = a.adj_volume.s[2], gz = a.adj_volume.s[3];
  while (true) {
    int pos = 0;
    if (lane == 0) pos = atomicAdd(counter, 1);
    pos = __shfl_sync(kFullMask, pos, 0);
    if (pos >= total) break;
    const int id = ray_list[pos];
    int b, x, y;
    if (!order.pixel(id, b, x, y)) continue;
    const int n = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] +
                                                         x * a.fwd_term.s[2]];
    if (n <= 0) continue;
    const int g = static_cast<const int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] +
                                                        x * p.dens_off.s[2]];
    if (g < 0 || int64_t(g) + ((n + 1) >> 1) > p.dens_units) {
      if (lane == 0) leftover[atomicAdd(counter + 1, 1)] = id;
      continue;
    }
    const float2* rec = reinterpret_cast<const float2*>(p.dens + 4 * size_t(g));
    FastRay q;
    fast_setup(p, x, y, b, q);
    const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] + y * a.adj_color.s[1] +
                      x * a.adj_color.s[2];
    const f4 adj_col = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
    const int L = (n + 31) >> 5;
    const int s0 = min(n, lane * L), s1 = min(n, s0 + L);

    // cell cache of the four channels' corners
    int cx = -1, cy = -1, cz = -1;
    float d[4][8];
    auto fetch = [&](int k, float& fx, float& fy, float& fz, int& ix, int& iy, int& iz) {
      const float3 pq = fast_pos(q, q.tmin + k * q.step);
      ix = int(pq.x), iy = int(pq.y), iz = int(pq.z);
      fx = pq.x - float(ix), fy = pq.y - float(iy), fz = pq.z - float(iz);
    };

    // 1. affine map of the segment
    float A = 1.f, B = 0.f;
    for (int k = s0; k < s1; ++k) {
      float fx, fy, fz;
      int ix, iy, iz;
      fetch(k, fx, fy, fz, ix, iy, iz);
      if (ix != cx || iy != cy || iz != cz) {
        vol.corners(ix, iy, iz, d);
        cx = ix, cy = iy, cz = iz;
      }
      const f4 c = mk4(trilerp(d[0], fx, fy, fz), trilerp(d[1], fx, fy, fz), trilerp(d[2], fx, fy, fz),
                       trilerp(d[3], fx, fy, fz));
      const float ak = blend_alpha<BLEND>(c.w, q.step);
      compose(A, B, 1.f - ak, -ak * (c.x * adj_col.x + c.y * adj_col.y + c.z * adj_col.z));
    }
    // 2. opacity adjoint behind each segment: suffix composition over the lanes
    float SA = A, SB = B;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float Ao = __shfl_down_sync(kFullMask, SA, o), Bo = __shfl_down_sync(kFullMask, SB, o);
      if (lane + o < 32) compose(SA, SB, Ao, Bo);
    }
    const float NA = __shfl_down_sync(kFullMask, SA, 1), NB = __shfl_down_sync(kFullMask, SB, 1);
    f4 adj_acc = adj_col;
    if (lane < 31) adj_acc.w = fmaf(NA, adj_col.w, NB);

    // 3. reverse walk over the segment
    float gv[4][8];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int i = 0; i < 8; ++i) gv[c][i] = 0.f;
    int vx = -1, vy = -1, vz = -1;  // cell of the gradient registers
    auto flush = [&]() {
      if constexpr (VOLGRAD) {
        if (vx < 0) return;
        const int lx = clampi(vx, 0, p.X - 1), hx = clampi(vx + 1, 0, p.X - 1);
        const int ly = clampi(vy, 0, p.Y - 1), hy = clampi(vy + 1, 0, p.Y - 1);
        const int lz = clampi(vz, 0, p.Z - 1), hz = clampi(vz + 1, 0, p.Z - 1);
        const bool pair = gz == 1 && hz == lz + 1;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          float* base = adjv + c * gc;
          VolGradCell<kTrilinear, true>::add_z(base + lx * gx + ly * gy, lz, hz, gz, pair, gv[c][0], gv[c][1]);
          VolGradCell<kTrilinear, true>::add_z(base + lx * gx + hy * gy, lz, hz, gz, pair, gv[c][2], gv[c][3]);
          VolGradCell<kTrilinear, true>::add_z(base + hx * gx + ly * gy, lz, hz, gz, pair, gv[c][4], gv[c][5]);
          VolGradCell<kTrilinear, true>::add_z(base + hx * gx + hy * gy, lz, hz, gz, pair, gv[c][6], gv[c][7]);
#pragma unroll
          for (int i = 0; i < 8; ++i) gv[c][i] = 0.f;
        }
      }
    };
    f3 adj_start = mk3(0, 0, 0), adj_dir = mk3(0, 0, 0);
    float adj_step = 0.f;
    for (int k = s1 - 1; k >= s0; --k) {
      float fx, fy, fz;
      int ix, iy, iz;
      fetch(k, fx, fy, fz, ix, iy, iz);
      if (ix != cx || iy != cy || iz != cz) {
        vol.corners(ix, iy, iz, d);
        cx = ix, cy = iy, cz = iz;
      }
      if (VOLGRAD && (ix != vx || iy != vy || iz != vz)) {
        flush();
        vx = ix, vy = iy, vz = iz;
      }
      const f4 c = mk4(trilerp(d[0], fx, fy, fz), trilerp(d[1], fx, fy, fz), trilerp(d[2], fx, fy, fz),
                       trilerp(d[3], fx, fy, fz));
      const float ak = blend_alpha<BLEND>(c.w, q.step);
      const float a_in = __ldg(rec + k).y;
      f4 adj_cur;
      const float step_term = blend_adjoint_core<BLEND>(a_in, c, q.step, ak, adj_acc, adj_cur);
      const float av[4] = {adj_cur.x, adj_cur.y, adj_cur.z, adj_cur.w};
      if constexpr (VOLGRAD) {
        const float ux = 1.f - fx, uy = 1.f - fy, uz = 1.f - fz;
        const float w8[8] = {ux * uy * uz, ux * uy * fz, ux * fy * uz, ux * fy * fz,
                             fx * uy * uz, fx * uy * fz, fx * fy * uz, fx * fy * fz};
#pragma unroll
        for (int ch = 0; ch < 4; ++ch)
#pragma unroll
          for (int i = 0; i < 8; ++i) gv[ch][i] = fmaf(av[ch], w8[i], gv[ch][i]);
      }
      if constexpr (POS) {
        f3 adj_vp = mk3(0, 0, 0);
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          f3 g3;
          trilerp_grad(d[ch], fx, fy, fz, g3);
          adj_vp.x = fmaf(av[ch], g3.x, adj_vp.x);
          adj_vp.y = fmaf(av[ch], g3.y, adj_vp.y);
          adj_vp.z = fmaf(av[ch], g3.z, adj_vp.z);
        }
        const float t = q.tmin + k * q.step;
        const f3 adj_w = mk3(adj_vp.x / q.voxel.x, adj_vp.y / q.voxel.y, adj_vp.z / q.voxel.z);
        adj_start.x += adj_w.x; adj_start.y += adj_w.y; adj_start.z += adj_w.z;
        adj_dir.x += adj_w.x * t; adj_dir.y += adj_w.y * t; adj_dir.z += adj_w.z * t;
        adj_step += step_term + dot3(adj_w, q.dir) * k;
      }
    }
    flush();
    if constexpr (POS) {
      float v[7] = {adj_start.x, adj_start.y, adj_start.z, adj_dir.x, adj_dir.y, adj_dir.z, adj_step};
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < 7; ++i) v[i] += __shfl_xor_sync(kFullMask, v[i], o);
      if (lane == 0) {
        if (a.has_stepsize) {
          float* ps = static_cast<float*>(a.adj_step.p) + b * a.adj_step.s[0] + y * a.adj_step.s[1] +
                      x * a.adj_step.s[2];
          if (a.stepsize_broadcast) atomicAdd(ps, v[6]);
          else *ps = v[6];
        }
        if (a.has_camera) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            if (a.camera_broadcast) {
              atomic_out(a.adj_start, b, y, x, c, v[c]);
              atomic_out(a.adj_dir, b, y, x, c, v[3 + c]);
            } else {
              write_out(a.adj_start, b, y, x, c, v[c]);
              write_out(a.adj_dir, b, y, x, c, v[3 + c]);
            }
          }
        }
      }
    }
  }
}


}  // namespace dvr
