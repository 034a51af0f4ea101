// Plain FP32 kernels: one thread per ray, grid-stride over B*H*W, the
// reference's algorithm step for step.
//
//  forward  = renderer/renderer_kernels.cuh:22-106 (DvrKernelForwardImpl/Device)
//  adjoint  = renderer/renderer_kernels.cuh:315-468 (DvrKernelAdjointImpl/Device):
//             reverse march that recovers the accumulator by inverting the blend,
//             per-cell register accumulation of the volume gradient flushed by
//             eight atomics on cell exit (renderer/renderer_interpolation.cuh:299-321),
//             TF gradient either by immediate atomics or accumulated per thread in
//             shared memory and reduced across the warp at the end
//             ("delayed accumulation", renderer/renderer_tf.cuh:221-245).
//
// These are the baseline the optimized kernels are measured against.
#pragma once
#include "dvr_device.cuh"

namespace dvr {

template <int FILTER, int TF, int BLEND>
__global__ void __launch_bounds__(256) plain_forward_kernel(const RenderParams p) {
  const int64_t total = int64_t(p.B) * p.H * p.W;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    const int b = int(i / (int64_t(p.W) * p.H));
    const int y = int((i - int64_t(b) * p.W * p.H) / p.W);
    const int x = int(i - int64_t(p.W) * (y + int64_t(p.H) * b));
    Ray r;
    setup_ray(p, x, y, b, r);
    const VolumeRef<float> vol = volume_ref<float>(p, b);
    const TfGlobal tf{static_cast<const float*>(p.tf.p) + b * p.tf.s[0], p.tf.s[1], p.tf.s[2], p.R};
    f4 acc = mk4(0, 0, 0, 0);
    int cx = -1, cy = -1, cz = -1;
    float d8[8];
    const int kmax = max_samples(r.tmin, r.tmax, r.step);
    int k;
    for (k = 0; k < kmax; ++k) {
      const float t = r.tmin + k * r.step;
      if (t > r.tmax) break;
      if (acc.w > p.early_out) break;
      const f3 vp = volume_pos(r, t);
      float density;
      if constexpr (FILTER == kNearest) {
        density = vol.at(nearest_coord(vp.x, p.X), nearest_coord(vp.y, p.Y), nearest_coord(vp.z, p.Z));
      } else {
        const int ix = int(vp.x), iy = int(vp.y), iz = int(vp.z);
        if (ix != cx || iy != cy || iz != cz) {  // cell cache (renderer_interpolation.cuh:217-225)
          fetch_corners(vol, ix, iy, iz, d8);
          cx = ix; cy = iy; cz = iz;
        }
        density = trilerp(d8, vp.x - float(ix), vp.y - float(iy), vp.z - float(iz));
      }
      acc = blend<BLEND>(acc, tf_eval<TF>(tf, density), r.step);
    }
    float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
    col[0] = acc.x;
    col[p.color.s[3]] = acc.y;
    col[2 * p.color.s[3]] = acc.z;
    col[3 * p.color.s[3]] = acc.w;
    static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = k;
  }
}

// TF gradient sinks ---------------------------------------------------------
struct TfSinkAtomic {  // immediate global atomics
  float* p;
  int64_t sr, sc;
  __device__ __forceinline__ void add(int r, int c, float v) { atomicAdd(p + r * sr + c * sc, v); }
  __device__ __forceinline__ void add4(int r, f4 v) {
    add(r, 0, v.x); add(r, 1, v.y); add(r, 2, v.z); add(r, 3, v.w);
  }
};
struct TfSinkThread {  // per-thread slots in shared memory, interleaved [entry][thread]
  float* p;
  int C, stride;
  __device__ __forceinline__ void add(int r, int c, float v) { p[(r * C + c) * stride] += v; }
  __device__ __forceinline__ void add4(int r, f4 v) {
    add(r, 0, v.x); add(r, 1, v.y); add(r, 2, v.z); add(r, 3, v.w);
  }
};

__device__ __forceinline__ void atomic_out(const OutView& o, int b, int y, int x, int c, float v) {
  atomicAdd(static_cast<float*>(o.p) + b * o.s[0] + y * o.s[1] + x * o.s[2] + c * o.s[3], v);
}
__device__ __forceinline__ void write_out(const OutView& o, int b, int y, int x, int c, float v) {
  static_cast<float*>(o.p)[b * o.s[0] + y * o.s[1] + x * o.s[2] + c * o.s[3]] = v;
}

template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD>
__global__ void __launch_bounds__(256) plain_adjoint_kernel(const RenderParams p, const AdjointParams a) {
  extern __shared__ float plain_smem[];
  constexpr int C = TfChannels<TF>::C;
  const bool delayed = TFGRAD && a.tf_delayed;
  const int tf_entries = p.R * C;
  if (delayed) {
    for (int e = 0; e < tf_entries; ++e) plain_smem[e * blockDim.x + threadIdx.x] = 0.f;
  }
  int last_b = -1;  // batch index of the per-thread TF slots (flushed on change)

  const int64_t total = int64_t(p.B) * p.H * p.W;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    const int b = int(i / (int64_t(p.W) * p.H));
    const int y = int((i - int64_t(b) * p.W * p.H) / p.W);
    const int x = int(i - int64_t(p.W) * (y + int64_t(p.H) * b));
    if (delayed && last_b >= 0 && b != last_b && a.adj_tf.s[0] != 0) {
      // a thread crossing into the next batch entry flushes its slots directly
      for (int e = 0; e < tf_entries; ++e) {
        float& s = plain_smem[e * blockDim.x + threadIdx.x];
        if (s != 0.f) atomicAdd(static_cast<float*>(a.adj_tf.p) + last_b * a.adj_tf.s[0] + (e / C) * a.adj_tf.s[1] +
                                    (e % C) * a.adj_tf.s[2], s);
        s = 0.f;
      }
    }
    last_b = b;
    Ray r;
    setup_ray(p, x, y, b, r);
    const VolumeRef<float> vol = volume_ref<float>(p, b);
    const TfGlobal tf{static_cast<const float*>(p.tf.p) + b * p.tf.s[0], p.tf.s[1], p.tf.s[2], p.R};
    TfSinkAtomic sink_atomic{static_cast<float*>(a.adj_tf.p) + b * a.adj_tf.s[0], a.adj_tf.s[1], a.adj_tf.s[2]};
    TfSinkThread sink_thread{plain_smem + threadIdx.x, C, int(blockDim.x)};

    const float* fc = static_cast<const float*>(a.fwd_color.p) + b * a.fwd_color.s[0] + y * a.fwd_color.s[1] +
                      x * a.fwd_color.s[2];
    f4 acc = mk4(fc[0], fc[a.fwd_color.s[3]], fc[2 * a.fwd_color.s[3]], fc[3 * a.fwd_color.s[3]]);
    int k = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
    k = min(k, max_samples(r.tmin, r.tmax, r.step));
    const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] + y * a.adj_color.s[1] +
                      x * a.adj_color.s[2];
    f4 adj_acc = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
    float adj_step = 0;
    f3 adj_start = mk3(0, 0, 0), adj_dir = mk3(0, 0, 0);

    // volume-gradient state: current cell (or voxel) and its accumulators
    int cx = -1, cy = -1, cz = -1;
    float d8[8], g8[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) { d8[q] = 0; g8[q] = 0; }
    float nearest_val = 0, nearest_acc = 0;
    float* adjv = VOLGRAD ? static_cast<float*>(a.adj_volume.p) + b * a.adj_volume.s[0] : nullptr;
    auto flush = [&]() {
      if constexpr (VOLGRAD) {
        if constexpr (FILTER == kNearest) {
          if (nearest_acc != 0) {
            atomicAdd(adjv + cx * a.adj_volume.s[1] + cy * a.adj_volume.s[2] + cz * a.adj_volume.s[3], nearest_acc);
            nearest_acc = 0;
          }
        } else if (cx >= 0) {
          const int lx = clampi(cx, 0, p.X - 1), hx = clampi(cx + 1, 0, p.X - 1);
          const int ly = clampi(cy, 0, p.Y - 1), hy = clampi(cy + 1, 0, p.Y - 1);
          const int lz = clampi(cz, 0, p.Z - 1), hz = clampi(cz + 1, 0, p.Z - 1);
          const int64_t sx = a.adj_volume.s[1], sy = a.adj_volume.s[2], sz = a.adj_volume.s[3];
          atomicAdd(adjv + lx * sx + ly * sy + lz * sz, g8[0]);
          atomicAdd(adjv + lx * sx + ly * sy + hz * sz, g8[1]);
          atomicAdd(adjv + lx * sx + hy * sy + lz * sz, g8[2]);
          atomicAdd(adjv + lx * sx + hy * sy + hz * sz, g8[3]);
          atomicAdd(adjv + hx * sx + ly * sy + lz * sz, g8[4]);
          atomicAdd(adjv + hx * sx + ly * sy + hz * sz, g8[5]);
          atomicAdd(adjv + hx * sx + hy * sy + lz * sz, g8[6]);
          atomicAdd(adjv + hx * sx + hy * sy + hz * sz, g8[7]);
#pragma unroll
          for (int q = 0; q < 8; ++q) g8[q] = 0;
        }
      }
    };

    for (--k; k >= 0; --k) {
      const float t = r.tmin + k * r.step;
      const f3 vp = volume_pos(r, t);
      float density, fx = 0, fy = 0, fz = 0;
      if constexpr (FILTER == kNearest) {
        const int ix = nearest_coord(vp.x, p.X), iy = nearest_coord(vp.y, p.Y), iz = nearest_coord(vp.z, p.Z);
        if (ix != cx || iy != cy || iz != cz) {
          flush();
          cx = ix; cy = iy; cz = iz;
          nearest_val = vol.at(ix, iy, iz);
        }
        density = nearest_val;
      } else {
        const int ix = int(vp.x), iy = int(vp.y), iz = int(vp.z);
        if (ix != cx || iy != cy || iz != cz) {
          flush();
          cx = ix; cy = iy; cz = iz;
          fetch_corners(vol, ix, iy, iz, d8);
        }
        fx = vp.x - float(ix); fy = vp.y - float(iy); fz = vp.z - float(iz);
        density = trilerp(d8, fx, fy, fz);
      }
      const f4 cur = tf_eval<TF>(tf, density);
      f4 adj_cur;
      float step_contrib;
      acc = blend_adjoint_invert<BLEND>(acc, cur, r.step, adj_acc, adj_cur, step_contrib);
      // the reference assigns the blend's step adjoint to the running sum
      // (renderer_blending.cuh:93 with renderer_kernels.cuh:393-395)
      adj_step = step_contrib;
      float adj_density;
      if (delayed) adj_density = tf_adjoint<TF, TFGRAD>(tf, density, adj_cur, sink_thread);
      else adj_density = tf_adjoint<TF, TFGRAD>(tf, density, adj_cur, sink_atomic);
      f3 adj_vp;
      if constexpr (FILTER == kNearest) {
        nearest_acc += adj_density;
        adj_vp = mk3(0, 0, 0);
      } else {
        adj_vp = trilerp_adjoint(d8, fx, fy, fz, adj_density, VOLGRAD ? g8 : nullptr);
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

  if (delayed) {
    // warp-reduce the per-thread slots, lane 0 adds them to the TF gradient.
    // Lanes may belong to different batch entries when adj_tf is not broadcast;
    // reduce per batch entry by masking.
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int my_b = last_b;
    for (int e = 0; e < tf_entries; ++e) {
      float v = plain_smem[e * blockDim.x + threadIdx.x];
      if (a.adj_tf.s[0] == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(full, v, o);
        if (lane == 0 && v != 0.f)
          atomicAdd(static_cast<float*>(a.adj_tf.p) + (e / C) * a.adj_tf.s[1] + (e % C) * a.adj_tf.s[2], v);
      } else if (my_b >= 0 && v != 0.f) {
        atomicAdd(static_cast<float*>(a.adj_tf.p) + my_b * a.adj_tf.s[0] + (e / C) * a.adj_tf.s[1] +
                      (e % C) * a.adj_tf.s[2], v);
      }
    }
  }
}

}  // namespace dvr
