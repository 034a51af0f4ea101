// Optimized kernel family.
//
// Same mathematics as the reference's march (renderer/renderer_kernels.cuh:22-90
// forward, :315-444 adjoint), reorganised for GB300:
//  * rays are processed in 16x8 pixel tiles per 128-thread block, each warp
//    an 8x4 pixel patch, so the 32 rays of a warp sample neighbouring cells
//    and their corner gathers share L1 lines;
//  * the volume may be stored as FP16 or BF16 (half the bytes of every
//    gather), converted to FP32 on load; TF staged once per block in shared
//    memory as FP32;
//  * the sample position is advanced with one FMA per axis
//    (p0 + t * dp, p0 = (start - boxMin) / voxel, dp = dir / voxel);
//  * the forward pass optionally stores the accumulated opacity every K
//    samples (a transmittance checkpoint); the adjoint then re-marches each
//    K-sample segment forward from its checkpoint, keeping density and the
//    incoming opacity per step in shared memory, and runs the reverse
//    recursion over the segment without inverting the blend (the reference
//    recovers the previous accumulator by dividing by (alpha - 1),
//    renderer/renderer_blending.cuh:75-77, which is ill-conditioned as the
//    opacity approaches 1);
//  * TF gradients are accumulated per warp in shared memory and reduced into
//    the output with one global atomic per TF entry and block; the volume
//    gradient keeps the reference's per-cell register accumulation and issues
//    its eight corner reductions on cell exit.
//  * The step-size gradient is the full derivative (the reference keeps only
//    the last blend contribution, renderer/renderer_kernels.cuh:393-395).
#pragma once
#include "dvr_device.cuh"

namespace dvr {

constexpr int kTileW = 16, kTileH = 8, kFastThreads = 128;
constexpr int kMaxSegment = 32;  // checkpoint interval capacity of the adjoint

// Maps thread -> pixel within a 16x8 tile: warp w covers an 8x4 patch.
__device__ __forceinline__ void tile_pixel(int tid, int& px, int& py) {
  const int w = tid >> 5, l = tid & 31;
  px = ((w & 1) << 3) + (l & 7);
  py = ((w >> 1) << 2) + (l >> 3);
}

template <typename VT>
struct VolumeFast {
  const VT* p;
  int sx, sy, sz;
  int X1, Y1, Z1;  // size - 1
  __device__ __forceinline__ float at(int x, int y, int z) const { return Storage<VT>::load(p + (x * sx + y * sy + z * sz)); }
  __device__ __forceinline__ void corners(int ix, int iy, int iz, float* d) const {
    const int lx = clampi(ix, 0, X1), hx = clampi(ix + 1, 0, X1);
    const int ly = clampi(iy, 0, Y1), hy = clampi(iy + 1, 0, Y1);
    const int lz = clampi(iz, 0, Z1), hz = clampi(iz + 1, 0, Z1);
    const VT* pll = p + lx * sx + ly * sy;
    const VT* plh = p + lx * sx + hy * sy;
    const VT* phl = p + hx * sx + ly * sy;
    const VT* phh = p + hx * sx + hy * sy;
    const int oz = lz * sz, hz_ = hz * sz;
    d[0] = Storage<VT>::load(pll + oz);
    d[1] = Storage<VT>::load(pll + hz_);
    d[2] = Storage<VT>::load(plh + oz);
    d[3] = Storage<VT>::load(plh + hz_);
    d[4] = Storage<VT>::load(phl + oz);
    d[5] = Storage<VT>::load(phl + hz_);
    d[6] = Storage<VT>::load(phh + oz);
    d[7] = Storage<VT>::load(phh + hz_);
  }
};

__device__ __forceinline__ float tf_load(const void* base, int64_t off, int storage) {
  if (storage == kF16) return Storage<__half>::load(static_cast<const __half*>(base) + off);
  if (storage == kBF16) return Storage<__nv_bfloat16>::load(static_cast<const __nv_bfloat16*>(base) + off);
  return Storage<float>::load(static_cast<const float*>(base) + off);
}

// Copies the TF of batch entry b into shared memory as dense FP32 R*C.
__device__ __forceinline__ void stage_tf(const RenderParams& p, int b, float* s_tf) {
  const int n = p.R * p.C;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = e / p.C, c = e - r * p.C;
    s_tf[e] = tf_load(p.tf.p, b * p.tf.s[0] + r * p.tf.s[1] + c * p.tf.s[2], p.tf_storage);
  }
}

// Per-ray march state of the optimized kernels.
struct FastRay {
  float3 p0, dp;       // volume position = p0 + t * dp
  float step, tmin, tmax;
  f3 dir, voxel;
};

__device__ __forceinline__ void fast_setup(const RenderParams& p, int x, int y, int b, FastRay& fr) {
  Ray r;
  setup_ray(p, x, y, b, r);
  fr.p0 = make_float3((r.start.x - r.bmin.x) / r.voxel.x, (r.start.y - r.bmin.y) / r.voxel.y,
                      (r.start.z - r.bmin.z) / r.voxel.z);
  fr.dp = make_float3(r.dir.x / r.voxel.x, r.dir.y / r.voxel.y, r.dir.z / r.voxel.z);
  fr.step = r.step;
  fr.tmin = r.tmin;
  fr.tmax = r.tmax;
  fr.dir = r.dir;
  fr.voxel = r.voxel;
}

__device__ __forceinline__ float3 fast_pos(const FastRay& r, float t) {
  return make_float3(fmaf(t, r.dp.x, r.p0.x), fmaf(t, r.dp.y, r.p0.y), fmaf(t, r.dp.z, r.p0.z));
}

// Density at a position, with a one-cell cache (cx < 0: empty).
template <int FILTER, typename VT>
struct Sampler {
  int cx = -1, cy = -1, cz = -1;
  float d[8];
  float fx, fy, fz;
  __device__ __forceinline__ float sample(const VolumeFast<VT>& v, float3 q) {
    if constexpr (FILTER == kNearest) {
      const int ix = nearest_coord(q.x, v.X1 + 1), iy = nearest_coord(q.y, v.Y1 + 1), iz = nearest_coord(q.z, v.Z1 + 1);
      if (ix != cx || iy != cy || iz != cz) {
        d[0] = v.at(ix, iy, iz);
        cx = ix; cy = iy; cz = iz;
      }
      return d[0];
    } else {
      const int ix = int(q.x), iy = int(q.y), iz = int(q.z);
      if (ix != cx || iy != cy || iz != cz) {
        v.corners(ix, iy, iz, d);
        cx = ix; cy = iy; cz = iz;
      }
      fx = q.x - float(ix); fy = q.y - float(iy); fz = q.z - float(iz);
      return trilerp(d, fx, fy, fz);
    }
  }
};

// ----------------------------------------------------------------- forward
template <int FILTER, int TF, int BLEND, typename VT>
__device__ __forceinline__ void fast_forward_tile(const RenderParams& p, int b, int tx, int ty, float* s_tf) {
  constexpr int C = TfChannels<TF>::C;
  int px, py;
  tile_pixel(threadIdx.x, px, py);
  const int x = tx * kTileW + px, y = ty * kTileH + py;
  if (x >= p.W || y >= p.H) return;
  FastRay r;
  fast_setup(p, x, y, b, r);
  VolumeFast<VT> vol{static_cast<const VT*>(p.volume.p) + b * p.volume.s[0], int(p.volume.s[1]), int(p.volume.s[2]),
                     int(p.volume.s[3]), p.X - 1, p.Y - 1, p.Z - 1};
  const TfShared<C> tf{s_tf, p.R};
  Sampler<FILTER, VT> smp;
  f4 acc = mk4(0, 0, 0, 0);
  float* ck = p.ckpt.p ? static_cast<float*>(p.ckpt.p) + b * p.ckpt.s[0] + y * p.ckpt.s[1] + x * p.ckpt.s[2] : nullptr;
  const int K = p.ckpt_interval;
  int next_ck = K, slot = 0;
  int k;
  for (k = 0;; ++k) {
    const float t = r.tmin + k * r.step;
    if (t > r.tmax) break;
    if (acc.w > p.early_out) break;
    if (ck && k == next_ck) {  // opacity before sample k = (slot+1)*K
      if (slot < p.ckpt_slots) ck[slot * p.ckpt.s[3]] = acc.w;
      ++slot;
      next_ck += K;
    }
    const float density = smp.sample(vol, fast_pos(r, t));
    acc = blend<BLEND>(acc, tf_eval<TF>(tf, density), r.step);
  }
  float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
  col[0] = acc.x;
  col[p.color.s[3]] = acc.y;
  col[2 * p.color.s[3]] = acc.z;
  col[3 * p.color.s[3]] = acc.w;
  static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = k;
}

template <int FILTER, int TF, int BLEND, typename VT>
__global__ void __launch_bounds__(kFastThreads) fast_forward_kernel(const RenderParams p, int tiles_x, int tiles_y) {
  extern __shared__ float4 fast_smem4[];
  float* s_tf = reinterpret_cast<float*>(fast_smem4);
  const int tiles_per_b = tiles_x * tiles_y;
  const int b = blockIdx.x / tiles_per_b;
  const int rem = blockIdx.x - b * tiles_per_b;
  const int ty = rem / tiles_x, tx = rem - ty * tiles_x;
  stage_tf(p, b, s_tf);
  __syncthreads();
  fast_forward_tile<FILTER, TF, BLEND, VT>(p, b, tx, ty, s_tf);
}

// Batched variant: one block per work item (instance, batch entry, tile) of
// a list ordered by decreasing estimated cost; the instance descriptors live
// in device memory.
template <int FILTER, int TF, int BLEND, typename VT>
__global__ void __launch_bounds__(kFastThreads) fast_forward_batched_kernel(const RenderParams* __restrict__ table,
                                                                             const int4* __restrict__ items) {
  extern __shared__ float4 fast_smem4[];
  float* s_tf = reinterpret_cast<float*>(fast_smem4);
  const int4 it = items[blockIdx.x];
  const RenderParams& p = table[it.x];
  stage_tf(p, it.y, s_tf);
  __syncthreads();
  fast_forward_tile<FILTER, TF, BLEND, VT>(p, it.y, it.z, it.w, s_tf);
}

// ----------------------------------------------------------------- adjoint
// Per-warp TF gradient accumulator in shared memory.
struct TfSinkWarp {
  float* p;
  int C;
  __device__ __forceinline__ void add(int r, int c, float v) { atomicAdd(p + r * C + c, v); }
  __device__ __forceinline__ void add4(int r, f4 v) {
    float* q = p + r * C;
    atomicAdd(q + 0, v.x);
    atomicAdd(q + 1, v.y);
    atomicAdd(q + 2, v.z);
    atomicAdd(q + 3, v.w);
  }
};
struct TfSinkNone {
  __device__ __forceinline__ void add(int, int, float) {}
  __device__ __forceinline__ void add4(int, f4) {}
};

// Volume-gradient accumulator for the current cell (reference scheme).
template <int FILTER, bool VOLGRAD>
struct VolGradCell {
  int cx = -1, cy = -1, cz = -1;
  float g[8];
  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int q = 0; q < 8; ++q) g[q] = 0.f;
  }
  __device__ __forceinline__ void flush(float* adjv, const OutView& o, int X1, int Y1, int Z1) {
    if constexpr (VOLGRAD) {
      if (cx < 0) return;
      const int64_t sx = o.s[1], sy = o.s[2], sz = o.s[3];
      if constexpr (FILTER == kNearest) {
        if (g[0] != 0.f) atomicAdd(adjv + cx * sx + cy * sy + cz * sz, g[0]);
      } else {
        const int lx = clampi(cx, 0, X1), hx = clampi(cx + 1, 0, X1);
        const int ly = clampi(cy, 0, Y1), hy = clampi(cy + 1, 0, Y1);
        const int lz = clampi(cz, 0, Z1), hz = clampi(cz + 1, 0, Z1);
        atomicAdd(adjv + lx * sx + ly * sy + lz * sz, g[0]);
        atomicAdd(adjv + lx * sx + ly * sy + hz * sz, g[1]);
        atomicAdd(adjv + lx * sx + hy * sy + lz * sz, g[2]);
        atomicAdd(adjv + lx * sx + hy * sy + hz * sz, g[3]);
        atomicAdd(adjv + hx * sx + ly * sy + lz * sz, g[4]);
        atomicAdd(adjv + hx * sx + ly * sy + hz * sz, g[5]);
        atomicAdd(adjv + hx * sx + hy * sy + lz * sz, g[6]);
        atomicAdd(adjv + hx * sx + hy * sy + hz * sz, g[7]);
      }
      reset();
    }
  }
};

// One reverse step shared by both adjoint variants.  Returns the step's
// position-chain contribution to d(loss)/d(step) via adj_step.
template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT, class A, class Sink>
__device__ __forceinline__ void fast_reverse_step(const RenderParams& p, const AdjointParams& a, const FastRay& r,
                                                  const VolumeFast<VT>& vol, const A& tf, Sink& sink,
                                                  Sampler<FILTER, VT>& smp, VolGradCell<FILTER, VOLGRAD>& vg,
                                                  float* adjv, int k, float density, float alpha_in, f4& adj_acc,
                                                  f3& adj_start, f3& adj_dir, float& adj_step, bool need_pos_grad) {
  const float t = r.tmin + k * r.step;
  const f4 cur = tf_eval<TF>(tf, density);
  const float alpha = blend_alpha<BLEND>(cur.w, r.step);
  f4 adj_cur;
  adj_step += blend_adjoint_core<BLEND>(alpha_in, cur, r.step, alpha, adj_acc, adj_cur);
  const float adj_density = tf_adjoint<TF, TFGRAD>(tf, density, adj_cur, sink);
  if (!VOLGRAD && !need_pos_grad) return;
  const float3 q = fast_pos(r, t);
  if constexpr (FILTER == kNearest) {
    if constexpr (VOLGRAD) {
      const int ix = nearest_coord(q.x, p.X), iy = nearest_coord(q.y, p.Y), iz = nearest_coord(q.z, p.Z);
      if (ix != vg.cx || iy != vg.cy || iz != vg.cz) {
        vg.flush(adjv, a.adj_volume, p.X - 1, p.Y - 1, p.Z - 1);
        vg.cx = ix; vg.cy = iy; vg.cz = iz;
      }
      vg.g[0] += adj_density;
    }
  } else {
    const int ix = int(q.x), iy = int(q.y), iz = int(q.z);
    const float fx = q.x - float(ix), fy = q.y - float(iy), fz = q.z - float(iz);
    if constexpr (VOLGRAD) {
      if (ix != vg.cx || iy != vg.cy || iz != vg.cz) {
        vg.flush(adjv, a.adj_volume, p.X - 1, p.Y - 1, p.Z - 1);
        vg.cx = ix; vg.cy = iy; vg.cz = iz;
      }
    }
    if (need_pos_grad) {
      if (ix != smp.cx || iy != smp.cy || iz != smp.cz) {
        vol.corners(ix, iy, iz, smp.d);
        smp.cx = ix; smp.cy = iy; smp.cz = iz;
      }
      const f3 adj_vp = trilerp_adjoint(smp.d, fx, fy, fz, adj_density, VOLGRAD ? vg.g : nullptr);
      const f3 adj_w = mk3(adj_vp.x / r.voxel.x, adj_vp.y / r.voxel.y, adj_vp.z / r.voxel.z);
      adj_start.x += adj_w.x; adj_start.y += adj_w.y; adj_start.z += adj_w.z;
      adj_dir.x += adj_w.x * t; adj_dir.y += adj_w.y * t; adj_dir.z += adj_w.z * t;
      adj_step += dot3(adj_w, r.dir) * k;
    } else if constexpr (VOLGRAD) {
      const float gx = 1 - fx, gy = 1 - fy, gz = 1 - fz;
      vg.g[0] += adj_density * (gx * gy * gz);
      vg.g[1] += adj_density * (gx * gy * fz);
      vg.g[2] += adj_density * (gx * fy * gz);
      vg.g[3] += adj_density * (gx * fy * fz);
      vg.g[4] += adj_density * (fx * gy * gz);
      vg.g[5] += adj_density * (fx * gy * fz);
      vg.g[6] += adj_density * (fx * fy * gz);
      vg.g[7] += adj_density * (fx * fy * fz);
    }
  }
}

template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT>
__device__ __forceinline__ void fast_adjoint_tile(const RenderParams& p, const AdjointParams& a, int b, int tx, int ty,
                                                  float* s_tf, float* s_grad, float* s_seg) {
  constexpr int C = TfChannels<TF>::C;
  int px, py;
  tile_pixel(threadIdx.x, px, py);
  const int x = tx * kTileW + px, y = ty * kTileH + py;
  if (x >= p.W || y >= p.H) return;
  FastRay r;
  fast_setup(p, x, y, b, r);
  VolumeFast<VT> vol{static_cast<const VT*>(p.volume.p) + b * p.volume.s[0], int(p.volume.s[1]), int(p.volume.s[2]),
                     int(p.volume.s[3]), p.X - 1, p.Y - 1, p.Z - 1};
  const TfShared<C> tf{s_tf, p.R};
  TfSinkWarp sink{s_grad + (threadIdx.x >> 5) * p.R * C, C};
  float* adjv = VOLGRAD ? static_cast<float*>(a.adj_volume.p) + b * a.adj_volume.s[0] : nullptr;
  const bool need_pos = a.has_camera || a.has_stepsize;

  const int n = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
  const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] + y * a.adj_color.s[1] +
                    x * a.adj_color.s[2];
  f4 adj_acc = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
  float adj_step = 0;
  f3 adj_start = mk3(0, 0, 0), adj_dir = mk3(0, 0, 0);
  Sampler<FILTER, VT> smp;
  VolGradCell<FILTER, VOLGRAD> vg;
  vg.reset();

  const int K = p.ckpt_interval;
  const bool ckpt_ok = p.ckpt.p != nullptr && K <= kMaxSegment && n <= (p.ckpt_slots + 1) * K;
  if (ckpt_ok) {
    const float* ck = static_cast<const float*>(p.ckpt.p) + b * p.ckpt.s[0] + y * p.ckpt.s[1] + x * p.ckpt.s[2];
    float* seg_d = s_seg + threadIdx.x;                     // [j][thread]
    float* seg_a = s_seg + kMaxSegment * blockDim.x + threadIdx.x;
    const int nseg = (n + K - 1) / K;
    for (int j = nseg - 1; j >= 0; --j) {
      const int k0 = j * K, k1 = min(n, k0 + K);
      // re-march the segment from its checkpoint
      float alpha = j == 0 ? 0.f : ck[(j - 1) * p.ckpt.s[3]];
      for (int k = k0; k < k1; ++k) {
        const float t = r.tmin + k * r.step;
        const float density = smp.sample(vol, fast_pos(r, t));
        const float a_k = blend_alpha<BLEND>(tf_eval<TF>(tf, density).w, r.step);
        seg_d[(k - k0) * blockDim.x] = density;
        seg_a[(k - k0) * blockDim.x] = alpha;
        alpha = alpha + (1 - alpha) * a_k;
      }
      for (int k = k1 - 1; k >= k0; --k) {
        const float density = seg_d[(k - k0) * blockDim.x];
        const float alpha_in = seg_a[(k - k0) * blockDim.x];
        if constexpr (TFGRAD) {
          fast_reverse_step<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, r, vol, tf, sink, smp, vg, adjv, k, density,
                                                                    alpha_in, adj_acc, adj_start, adj_dir, adj_step,
                                                                    need_pos);
        } else {
          TfSinkNone none;
          fast_reverse_step<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, r, vol, tf, none, smp, vg, adjv, k, density,
                                                                    alpha_in, adj_acc, adj_start, adj_dir, adj_step,
                                                                    need_pos);
        }
      }
    }
  } else {
    // no checkpoints: recover the accumulator by inverting the blend, as the reference
    const float* fc = static_cast<const float*>(a.fwd_color.p) + b * a.fwd_color.s[0] + y * a.fwd_color.s[1] +
                      x * a.fwd_color.s[2];
    float alpha_out = fc[3 * a.fwd_color.s[3]];
    for (int k = n - 1; k >= 0; --k) {
      const float t = r.tmin + k * r.step;
      const float density = smp.sample(vol, fast_pos(r, t));
      const float a_k = blend_alpha<BLEND>(tf_eval<TF>(tf, density).w, r.step);
      const float a_inv = BLEND == kAlphaBlend ? rminf(1.0f - 1e-5f, a_k) : a_k;
      const float alpha_in = (a_inv - alpha_out) / (a_inv - 1);
      if constexpr (TFGRAD) {
        fast_reverse_step<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, r, vol, tf, sink, smp, vg, adjv, k, density,
                                                                  alpha_in, adj_acc, adj_start, adj_dir, adj_step,
                                                                  need_pos);
      } else {
        TfSinkNone none;
        fast_reverse_step<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, r, vol, tf, none, smp, vg, adjv, k, density,
                                                                  alpha_in, adj_acc, adj_start, adj_dir, adj_step,
                                                                  need_pos);
      }
      alpha_out = alpha_in;
    }
  }
  vg.flush(adjv, a.adj_volume, p.X - 1, p.Y - 1, p.Z - 1);

  if (a.has_stepsize) {
    float* ps = static_cast<float*>(a.adj_step.p) + b * a.adj_step.s[0] + y * a.adj_step.s[1] + x * a.adj_step.s[2];
    if (a.stepsize_broadcast) atomicAdd(ps, adj_step);
    else *ps = adj_step;
  }
  if (a.has_camera) {
    float* s0 = static_cast<float*>(a.adj_start.p) + b * a.adj_start.s[0] + y * a.adj_start.s[1] + x * a.adj_start.s[2];
    float* d0 = static_cast<float*>(a.adj_dir.p) + b * a.adj_dir.s[0] + y * a.adj_dir.s[1] + x * a.adj_dir.s[2];
    const float vs[3] = {adj_start.x, adj_start.y, adj_start.z};
    const float vd[3] = {adj_dir.x, adj_dir.y, adj_dir.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (a.camera_broadcast) {
        atomicAdd(s0 + c * a.adj_start.s[3], vs[c]);
        atomicAdd(d0 + c * a.adj_dir.s[3], vd[c]);
      } else {
        s0[c * a.adj_start.s[3]] = vs[c];
        d0[c * a.adj_dir.s[3]] = vd[c];
      }
    }
  }
}

// Shared memory of the adjoint block: TF (R*C) | per-warp TF gradients
// (4 * R*C) | segment buffers (2 * kMaxSegment * threads).
__host__ __device__ inline size_t fast_adjoint_smem(int R, int C, bool tfgrad, bool ckpt) {
  size_t n = size_t(R) * C;
  if (tfgrad) n += size_t(kFastThreads / 32) * R * C;
  if (ckpt) n += size_t(2) * kMaxSegment * kFastThreads;
  return n * sizeof(float);
}

template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT>
__device__ __forceinline__ void fast_adjoint_block(const RenderParams& p, const AdjointParams& a, int b, int tx,
                                                   int ty) {
  extern __shared__ float4 fast_smem4[];
  constexpr int C = TfChannels<TF>::C;
  float* s_tf = reinterpret_cast<float*>(fast_smem4);
  float* s_grad = s_tf + p.R * C;
  float* s_seg = s_grad + (TFGRAD ? (kFastThreads / 32) * p.R * C : 0);
  stage_tf(p, b, s_tf);
  if constexpr (TFGRAD) {
    for (int e = threadIdx.x; e < (kFastThreads / 32) * p.R * C; e += blockDim.x) s_grad[e] = 0.f;
  }
  __syncthreads();
  fast_adjoint_tile<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, b, tx, ty, s_tf, s_grad, s_seg);
  if constexpr (TFGRAD) {
    __syncthreads();
    const int n = p.R * C;
    float* g = static_cast<float*>(a.adj_tf.p) + b * a.adj_tf.s[0];
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      float v = 0.f;
#pragma unroll
      for (int w = 0; w < kFastThreads / 32; ++w) v += s_grad[w * n + e];
      const int rr = e / C, cc = e - rr * C;
      if (v != 0.f) atomicAdd(g + rr * a.adj_tf.s[1] + cc * a.adj_tf.s[2], v);
    }
  }
}

template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT>
__global__ void __launch_bounds__(kFastThreads) fast_adjoint_kernel(const RenderParams p, const AdjointParams a,
                                                                     int tiles_x, int tiles_y) {
  const int tiles_per_b = tiles_x * tiles_y;
  const int b = blockIdx.x / tiles_per_b;
  const int rem = blockIdx.x - b * tiles_per_b;
  const int ty = rem / tiles_x, tx = rem - ty * tiles_x;
  fast_adjoint_block<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, b, tx, ty);
}

template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT>
__global__ void __launch_bounds__(kFastThreads) fast_adjoint_batched_kernel(const RenderParams* __restrict__ table,
                                                                             const AdjointParams* __restrict__ atable,
                                                                             const int4* __restrict__ items) {
  const int4 it = items[blockIdx.x];
  fast_adjoint_block<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(table[it.x], atable[it.x], it.y, it.z, it.w);
}

}  // namespace dvr
