// Persistent adjoint kernel with per-lane ray refill, and the ray numbering
// and work fetching shared by the persistent kernels.
//
// One block per SM slot stays resident; each warp pulls rays from a global
// counter whenever some of its lanes are idle (one atomicAdd per refill for
// all idle lanes), so lanes are not left waiting for the longest ray of a
// fixed 32-ray patch and warps are not left waiting for the slowest warp of
// a block.  Rays are numbered in 8x4-pixel patches (patches row-major, then
// batch entries), so the rays a warp fetches together are neighbours and their
// corner gathers share cache lines.
//
// The adjoint keeps the lanes of a warp in lock step at segment granularity: per
// round each active lane re-marches one K-sample segment of its ray from its
// checkpoint and runs the reverse recursion over it; lanes may be on different
// rays and segment indices.  The per-step math is that of dvr_fast.cuh.
#pragma once
#include "dvr_cells.cuh"

namespace dvr {

constexpr int kPatchW = 8, kPatchH = 4;
constexpr unsigned kFullMask = 0xffffffffu;

// Ray numbering in 8x4 patches.
struct RayOrder {
  int W, H, B, pxn, pyn;
  __host__ __device__ static RayOrder make(int W, int H, int B) {
    RayOrder o;
    o.W = W;
    o.H = H;
    o.B = B;
    o.pxn = (W + kPatchW - 1) / kPatchW;
    o.pyn = (H + kPatchH - 1) / kPatchH;
    return o;
  }
  __host__ __device__ int64_t total() const { return int64_t(B) * pxn * pyn * 32; }
  __device__ __forceinline__ bool pixel(int id, int& b, int& x, int& y) const {
    const int per_img = pxn * pyn * 32;
    b = id / per_img;
    const int rem = id - b * per_img;
    const int patch = rem >> 5, l = rem & 31;
    const int py_ = patch / pxn, px_ = patch - py_ * pxn;
    x = px_ * kPatchW + (l & 7);
    y = py_ * kPatchH + (l >> 3);
    return x < W && y < H;
  }
};

// Hands the next ray ids to the idle lanes of the warp (all 32 lanes call
// it).  Returns this lane's new id, or -1.  `exhausted` becomes true for the
// whole warp once the counter has passed the last ray.
__device__ __forceinline__ int fetch_rays(int* counter, int total, bool idle, bool& exhausted) {
  const unsigned mask = __ballot_sync(kFullMask, idle);
  if (mask == 0u || exhausted) return -1;
  const int cnt = __popc(mask);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0) base = atomicAdd(counter, cnt);
  base = __shfl_sync(kFullMask, base, 0);
  if (base + cnt >= total) exhausted = true;
  if (!idle) return -1;
  const int id = base + __popc(mask & ((1u << lane) - 1u));
  return id < total ? id : -1;
}

__device__ __forceinline__ int tf_copies(const RenderParams& p) { return p.tf.s[0] == 0 ? 1 : p.B; }

// ----------------------------------------------------------------- adjoint
template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT>
__global__ void __launch_bounds__(kFastThreads) fast_adjoint_persistent_kernel(const RenderParams p,
                                                                                const AdjointParams a,
                                                                                const RayOrder order, int* counter,
                                                                                float* tf_scratch,
                                                                                const int* ray_list,
                                                                                const int* ray_count,
                                                                                const TexGather tg) {
  extern __shared__ float4 fast_smem4[];
  if (ray_count && *ray_count == 0) return;  // an empty list: nothing to add
  constexpr int C = TfChannels<TF>::C;
  float* smem = reinterpret_cast<float*>(fast_smem4);
  const int copies = tf_copies(p);
  const int K = p.ckpt_interval;
  const int seg_len = p.ckpt.p ? K : 0;
  const AdjointSmem L(TF, p.R, C, int(blockDim.x), TFGRAD, seg_len, copies);
  float* s_tf = smem + L.tf;
  for (int bb = 0; bb < copies; ++bb) stage_tf(p, bb, s_tf + bb * p.R * C);
  // this block's slice of the TF-gradient scratch: control points leaving a
  // lane's window are added there with fire-and-forget global reductions
  float* block_slice = tf_scratch + size_t(blockIdx.x) * p.R * C;
  if constexpr (TFGRAD) {
    for (int e = threadIdx.x; e < L.seg - L.warp; e += blockDim.x) smem[L.warp + e] = 0.f;
    for (int e = threadIdx.x; e < p.R * C; e += blockDim.x) block_slice[e] = 0.f;
  }
  __syncthreads();

  // viewport gradient of the block, per batch entry, after the layout
  float* s_vp = smem + L.total;
  if (a.has_viewport)
    for (int e = threadIdx.x; e < p.B * 9; e += blockDim.x) s_vp[e] = 0.f;
  __syncthreads();

  const bool tf_per_batch = TFGRAD && a.adj_tf.s[0] != 0;
  float* s_grad_warp = smem + L.warp + (threadIdx.x >> 5) * p.R * C;
  TfGradAccum<TF, TFGRAD> tacc;
  tacc.bind(smem + L.lane, int(blockDim.x), int(threadIdx.x), L.slots, p.R);
  if (!tf_per_batch) tacc.set_evict_target(block_slice, C, 1);
  int cur_b = -1;  // batch entry of the accumulated TF gradient (per-batch outputs)
  const bool need_pos = a.has_camera || a.has_stepsize || a.has_viewport;
  float* seg_d = smem + L.seg + threadIdx.x;  // [offset][thread]
  float* seg_a = smem + L.seg + K * blockDim.x + threadIdx.x;

  // rays to process: the whole order, or the first *ray_count entries of ray_list
  const int total = ray_count ? *ray_count : int(order.total());
  bool exhausted = false, active = false;
  int b = 0, x = 0, y = 0, n = 0, j = 0;
  bool ckpt_ray = false;
  float alpha_out = 0.f;  // inversion mode: accumulator alpha after the current sample
  FastRay r{};
  f4 adj_acc = mk4(0, 0, 0, 0);
  float adj_step = 0.f;
  f3 adj_start = mk3(0, 0, 0), adj_dir = mk3(0, 0, 0);
  Sampler<FILTER, VT> smp;
  VolGradCell<FILTER, VOLGRAD> vg;
  // trilinear corners from the slab gather texture when the call built one
  AdjVolume<VT> vol(VolumeFast<VT>{static_cast<const VT*>(p.volume.p), int(p.volume.s[1]), int(p.volume.s[2]),
                                   int(p.volume.s[3]), p.X - 1, p.Y - 1, p.Z - 1},
                    TexVolume<VT>{tg, 0, p.X - 1, p.Y - 1, p.Z - 1}, tg.tex != 0);
  TfShared<C> tf{s_tf, p.R};
  float* adjv = nullptr;
  const float* ck = nullptr;
  const float2* drow = nullptr;  // the ray's recorded (density, incoming opacity) pairs, if any

  auto write_ray_grads = [&]() {
    if (a.has_viewport) viewport_adjoint(p, x, y, b, adj_start, adj_dir, s_vp + b * 9);
    if (a.has_stepsize) {
      float* ps = static_cast<float*>(a.adj_step.p) + b * a.adj_step.s[0] + y * a.adj_step.s[1] + x * a.adj_step.s[2];
      if (a.stepsize_broadcast) atomicAdd(ps, adj_step);
      else *ps = adj_step;
    }
    if (a.has_camera) {
      float* s0 = static_cast<float*>(a.adj_start.p) + b * a.adj_start.s[0] + y * a.adj_start.s[1] +
                  x * a.adj_start.s[2];
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
  };

  while (true) {
    // refill idle lanes; rays without samples are finished right here
    while (true) {
      int id = fetch_rays(counter, total, !active, exhausted);
      if (id >= 0 && ray_list) id = ray_list[id];
      if (id >= 0 && order.pixel(id, b, x, y)) {
        n = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
        adj_step = 0.f;
        adj_start = mk3(0, 0, 0);
        adj_dir = mk3(0, 0, 0);
        fast_setup(p, x, y, b, r);
        n = min(n, max_samples(r.tmin, r.tmax, r.step));
        if (n <= 0) {
          write_ray_grads();
        } else {
          active = true;
          const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] +
                            y * a.adj_color.s[1] + x * a.adj_color.s[2];
          adj_acc = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
          smp.cx = -1;
          vg.cx = -1;
          vg.reset();
          vol.v.p = static_cast<const VT*>(p.volume.p) + b * p.volume.s[0];
          vol.t.s0 = p.volume.s[0] != 0 ? b * p.X : 0;
          tf = TfShared<C>(s_tf + (copies > 1 ? b : 0) * p.R * C, p.R);
          adjv = VOLGRAD ? static_cast<float*>(a.adj_volume.p) + b * a.adj_volume.s[0] : nullptr;
          if (VOLGRAD && a.cell_grad)
            vg.cg = a.cell_grad + (a.adj_volume.s[0] != 0 ? size_t(b) : 0) * 8 * size_t(p.X) * p.Y * p.Z;
          ckpt_ray = p.ckpt.p != nullptr && n <= (p.ckpt_slots + 1) * K;
          drow = nullptr;
          if (ckpt_ray) {
            ck = static_cast<const float*>(p.ckpt.p) + b * p.ckpt.s[0] + y * p.ckpt.s[1] + x * p.ckpt.s[2];
            j = (n + K - 1) / K - 1;
            if (p.dens) {
              const int g = static_cast<const int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] +
                                                                  x * p.dens_off.s[2]];
              if (g >= 0 && int64_t(g) + ((n + 1) >> 1) <= p.dens_units)
                drow = reinterpret_cast<const float2*>(p.dens + 4 * size_t(g));
            }
          } else {
            // no checkpoints: invert the blend from the final colour, K samples per round
            const float* fc = static_cast<const float*>(a.fwd_color.p) + b * a.fwd_color.s[0] +
                              y * a.fwd_color.s[1] + x * a.fwd_color.s[2];
            alpha_out = fc[3 * a.fwd_color.s[3]];
            j = n - 1;  // next sample to process
          }
          if (tf_per_batch && b != cur_b) {
            if (cur_b >= 0)
              tacc.flush_global(static_cast<float*>(a.adj_tf.p) + cur_b * a.adj_tf.s[0], a.adj_tf.s[1],
                                a.adj_tf.s[2], s_grad_warp);
            cur_b = b;
            tacc.set_evict_target(static_cast<float*>(a.adj_tf.p) + b * a.adj_tf.s[0], a.adj_tf.s[1],
                                  a.adj_tf.s[2]);
          }
        }
      }
      if (exhausted || __ballot_sync(kFullMask, !active) == 0u) break;
    }
    if (__ballot_sync(kFullMask, active) == 0u) break;

    // one round: K samples of the current segment of each active lane's ray
    const int k0 = ckpt_ray ? j * K : 0;
    const int k1 = ckpt_ray ? min(n, k0 + K) : 0;
    if (seg_len > 0) {
      float alpha = (active && ckpt_ray && j > 0 && !drow) ? ck[(j - 1) * p.ckpt.s[3]] : 0.f;
      for (int kk = 0; kk < K; ++kk) {
        const int k = k0 + kk;
        if (active && ckpt_ray && k < k1) {
          if (drow) {  // recorded density and incoming opacity
            const float2 v = __ldg(drow + k);
            seg_d[kk * blockDim.x] = v.x;
            seg_a[kk * blockDim.x] = v.y;
          } else {
            const float t = r.tmin + k * r.step;
            const float density = smp.sample(vol, fast_pos(r, t));
            const float a_k = blend_alpha<BLEND>(tf_eval<TF>(tf, density).w, r.step);
            seg_d[kk * blockDim.x] = density;
            seg_a[kk * blockDim.x] = alpha;
            alpha = alpha + (1 - alpha) * a_k;
          }
        }
      }
      __syncwarp();
    }
    for (int kk = K - 1; kk >= 0; --kk) {
      if (active) {
        if (ckpt_ray) {
          const int k = k0 + kk;
          if (k < k1) {
            fast_reverse_step<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(
                p, a, r, vol, tf, tacc, s_grad_warp, smp, vg, adjv, k, seg_d[kk * blockDim.x],
                seg_a[kk * blockDim.x], adj_acc, adj_start, adj_dir, adj_step, need_pos);
          }
        } else {
          const int k = j - (K - 1 - kk);
          if (k >= 0) {
            const float t = r.tmin + k * r.step;
            const float density = smp.sample(vol, fast_pos(r, t));
            const float a_k = blend_alpha<BLEND>(tf_eval<TF>(tf, density).w, r.step);
            const float a_inv = BLEND == kAlphaBlend ? rminf(1.0f - 1e-5f, a_k) : a_k;
            const float alpha_in = (a_inv - alpha_out) / (a_inv - 1);
            fast_reverse_step<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, r, vol, tf, tacc, s_grad_warp, smp, vg,
                                                                      adjv, k, density, alpha_in, adj_acc,
                                                                      adj_start, adj_dir, adj_step, need_pos);
            alpha_out = alpha_in;
          }
        }
      }
      __syncwarp();
    }
    if (active) {
      j -= ckpt_ray ? 1 : K;
      if (j < 0) {  // ray done
        vg.flush(adjv, a.adj_volume, p.X - 1, p.Y - 1, p.Z - 1);
        write_ray_grads();
        active = false;
      }
    }
  }

  // TF gradient of the block
  if constexpr (TFGRAD) {
    if (tf_per_batch) {
      if (cur_b >= 0)
        tacc.flush_global(static_cast<float*>(a.adj_tf.p) + cur_b * a.adj_tf.s[0], a.adj_tf.s[1], a.adj_tf.s[2],
                          s_grad_warp);
    } else {
      tacc.finish(smem + L.lane, int(blockDim.x), int(threadIdx.x),
                  reinterpret_cast<int*>(smem + L.lo) + threadIdx.x);
      __syncthreads();
      reduce_tf_grad<TF>(L, smem, p.R, static_cast<float*>(a.adj_tf.p), 0, a.adj_tf.s[1], a.adj_tf.s[2], 0,
                         block_slice);
    }
  }
  // viewport gradient of the block
  if (a.has_viewport) {
    __syncthreads();
    for (int e = threadIdx.x; e < p.B * 9; e += blockDim.x) {
      const float v = s_vp[e];
      const int bb = e / 9, r = (e - bb * 9) / 3, c = e - bb * 9 - r * 3;
      if (v != 0.f)
        atomicAdd(static_cast<float*>(a.adj_viewport.p) + bb * a.adj_viewport.s[0] + r * a.adj_viewport.s[1] +
                      c * a.adj_viewport.s[2],
                  v);
    }
  }
}

}  // namespace dvr
