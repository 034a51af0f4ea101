// Adjoint for the TF-gradient-only case with a texture TF, read from the
// forward's sample-density record.
//
// When only the TF gradient is wanted and the forward recorded every sample's
// density, the adjoint of a ray needs no volume access and no ray geometry:
// per K-sample segment it rebuilds the incoming opacity of each sample from
// the segment's checkpoint and the recorded densities, then runs the reverse
// recursion (renderer/renderer_kernels.cuh:367-444 with the blend adjoint of
// renderer/renderer_blending.cuh:63-98, the accumulator taken from the
// rebuilt segment instead of the blend inversion).  The state of a lane is a
// handful of registers, so more warps fit per SM than in the general kernel:
//  * TF gradient: the two control points of the current texel in registers;
//    a point leaving them is added with a fire-and-forget global reduction to
//    the warp's slice of an L2-resident scratch (or to the per-batch output);
//    the slices are summed per block at the end.
//  * rays the record does not cover (pool full, or more samples than the
//    checkpoint buffer spans) are appended to a leftover list that the
//    general kernel processes afterwards.
#pragma once
#include "dvr_persist.cuh"

namespace dvr {

// Shared-memory layout of the record adjoint (floats).
struct RecordSmem {
  int tf, warp, seg, total;
  __host__ __device__ RecordSmem(int R, int C, int threads, int seg_len, int tf_copies, bool warp_copies) {
    int o = 0;
    tf = o;
    o += (tf_copies * R * C + 3) & ~3;
    warp = o;
    if (warp_copies) o += ((threads / 32) * R * C + 3) & ~3;
    seg = o;
    o += 2 * seg_len * threads;
    total = o;
  }
};

// A lane's TF-gradient accumulator: the pair of texels (i, i+1) in registers,
// other points added atomically to dst (point t, channel c at dst[t*sr + c*sc]).
struct TexelPairAtomic {
  int i = -1;
  f4 a0, a1;
  float* dst = nullptr;
  int64_t sr = 4, sc = 1;
  int R = 0;
  __device__ __forceinline__ void put(int t, f4 v) const {
    if (t < 0 || t >= R) return;
    float* e = dst + t * sr;
    if (v.x != 0.f) atomicAdd(e, v.x);
    if (v.y != 0.f) atomicAdd(e + sc, v.y);
    if (v.z != 0.f) atomicAdd(e + 2 * sc, v.z);
    if (v.w != 0.f) atomicAdd(e + 3 * sc, v.w);
  }
  __device__ __forceinline__ void flush() {
    if (i < 0) return;
    put(i, a0);
    put(i + 1, a1);
    i = -1;
  }
  // adds k0 * v to texel i0 and k1 * v to texel i1 (i1 = i0 + 1, or i0 at the clamped ends)
  __device__ __forceinline__ void add(int i0, int i1, f4 v, float k0, float k1) {
    if (i0 != i) {
      const f4 z = mk4(0, 0, 0, 0);
      if (i >= 0 && i0 == i + 1) {
        put(i, a0);
        a0 = a1;
        a1 = z;
      } else if (i >= 0 && i0 == i - 1) {
        put(i + 1, a1);
        a1 = a0;
        a0 = z;
      } else {
        flush();
        a0 = z;
        a1 = z;
      }
      i = i0;
    }
    const bool same = i1 == i0;
    const float q0 = same ? k0 + k1 : k0, q1 = same ? 0.f : k1;
    a0 = mk4(fmaf(v.x, q0, a0.x), fmaf(v.y, q0, a0.y), fmaf(v.z, q0, a0.z), fmaf(v.w, q0, a0.w));
    a1 = mk4(fmaf(v.x, q1, a1.x), fmaf(v.y, q1, a1.y), fmaf(v.z, q1, a1.z), fmaf(v.w, q1, a1.w));
  }
};

// Rays whose adjoint this kernel leaves to the general kernel: leftover[0..*n_left).
// tf_slices: (blocks x warps) slices of R*C floats, one per warp (TF gradient
// of a broadcast TF), zeroed here.
template <int BLEND>
__global__ void __launch_bounds__(kFastThreads) fast_adjoint_record_kernel(const RenderParams p, const AdjointParams a,
                                                                            const RayOrder order, int* counter,
                                                                            const int* ray_list, int* leftover,
                                                                            float* tf_slices) {
  extern __shared__ float4 fast_smem4[];
  constexpr int C = 4;
  float* smem = reinterpret_cast<float*>(fast_smem4);
  const int copies = tf_copies(p);
  const int K = p.ckpt_interval;
  const bool per_batch = a.adj_tf.s[0] != 0;
  const RecordSmem L(p.R, C, int(blockDim.x), K, copies, false);
  float* s_tf = smem + L.tf;
  for (int bb = 0; bb < copies; ++bb) stage_tf(p, bb, s_tf + bb * p.R * C);
  const int n_tf = p.R * C;
  const int warps = int(blockDim.x) / 32;
  float* block_slices = tf_slices + size_t(blockIdx.x) * warps * n_tf;
  if (!per_batch)
    for (int e = threadIdx.x; e < warps * n_tf; e += blockDim.x) block_slices[e] = 0.f;
  __syncthreads();

  int* const n_left = counter + 1;
  const int total = int(order.total());
  float* seg_d = smem + L.seg + threadIdx.x;  // [offset][thread]
  float* seg_a = smem + L.seg + K * blockDim.x + threadIdx.x;

  TexelPairAtomic acc_tf;
  acc_tf.R = p.R;
  if (!per_batch) acc_tf.dst = block_slices + (threadIdx.x >> 5) * n_tf;
  int cur_b = -1;

  bool exhausted = false, active = false;
  int n = 0, j = 0;
  float step = 0.f;
  f4 adj_acc = mk4(0, 0, 0, 0);
  const float* ck = nullptr;
  const float4* drow = nullptr;
  TfShared<C> tf{s_tf, p.R};

  while (true) {
    while (true) {
      int id = fetch_rays(counter, total, !active, exhausted);
      if (id >= 0 && ray_list) id = ray_list[id];
      int b, x, y;
      if (id >= 0 && order.pixel(id, b, x, y)) {
        n = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
        FastRay r;
        fast_setup(p, x, y, b, r);
        n = min(n, max_samples(r.tmin, r.tmax, r.step));
        if (n > 0) {
          const int g = static_cast<const int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] +
                                                              x * p.dens_off.s[2]];
          if (g < 0 || n > (p.ckpt_slots + 1) * K) {
            leftover[atomicAdd(n_left, 1)] = id;
          } else {
            active = true;
            step = r.step;
            j = (n + K - 1) / K - 1;
            const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] +
                              y * a.adj_color.s[1] + x * a.adj_color.s[2];
            adj_acc = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
            ck = static_cast<const float*>(p.ckpt.p) + b * p.ckpt.s[0] + y * p.ckpt.s[1] + x * p.ckpt.s[2];
            drow = reinterpret_cast<const float4*>(p.dens) + g;
            tf.p = s_tf + (copies > 1 ? b : 0) * n_tf;
            if (per_batch && b != cur_b) {
              acc_tf.flush();
              cur_b = b;
              acc_tf.dst = static_cast<float*>(a.adj_tf.p) + b * a.adj_tf.s[0];
              acc_tf.sr = a.adj_tf.s[1];
              acc_tf.sc = a.adj_tf.s[2];
            }
          }
        }
      }
      if (exhausted || __ballot_sync(kFullMask, !active) == 0u) break;
    }
    if (__ballot_sync(kFullMask, active) == 0u) break;

    // rebuild segment j: incoming opacity of each sample from the checkpoint
    const int k0 = j * K;
    const int k1 = min(n, k0 + K);
    {
      float alpha = (active && j > 0) ? ck[(j - 1) * p.ckpt.s[3]] : 0.f;
      float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int kk = 0; kk < K; ++kk) {
        const int k = k0 + kk;
        if (active && k < k1) {
          if (kk == 0 || (k & 3) == 0) q = __ldcs(drow + (k >> 2));
          const int c = k & 3;
          const float density = c == 0 ? q.x : c == 1 ? q.y : c == 2 ? q.z : q.w;
          const float a_k = blend_alpha<BLEND>(tf_eval<kTfTexture>(tf, density).w, step);
          seg_d[kk * blockDim.x] = density;
          seg_a[kk * blockDim.x] = alpha;
          alpha = alpha + (1 - alpha) * a_k;
        }
      }
      __syncwarp();
    }
    // reverse recursion over the segment
    for (int kk = K - 1; kk >= 0; --kk) {
      if (active && k0 + kk < k1) {
        const float density = seg_d[kk * blockDim.x];
        const float alpha_in = seg_a[kk * blockDim.x];
        const int R = tf.R;
        const float d = density * R - 0.5f;
        const int di = int(floorf(d));
        const float df = d - di;
        const int i0 = clampi(di, 0, R - 1), i1 = clampi(di + 1, 0, R - 1);
        const f4 t0 = tf.rgba(i0), t1 = tf.rgba(i1);
        const f4 cur = mk4(lerp1(t0.x, t1.x, df), lerp1(t0.y, t1.y, df), lerp1(t0.z, t1.z, df),
                           lerp1(t0.w, t1.w, df));
        const float a_k = blend_alpha<BLEND>(cur.w, step);
        f4 adj_cur;
        blend_adjoint_core<BLEND>(alpha_in, cur, step, a_k, adj_acc, adj_cur);
        acc_tf.add(i0, i1, adj_cur, 1 - df, df);
      }
    }
    __syncwarp();
    if (active && --j < 0) active = false;
  }

  // TF gradient of the block
  acc_tf.flush();
  if (!per_batch) {
    __syncthreads();
    float* out = static_cast<float*>(a.adj_tf.p);
    for (int e = threadIdx.x; e < n_tf; e += blockDim.x) {
      float v = 0.f;
      for (int w = 0; w < warps; ++w) v += __ldcg(block_slices + w * n_tf + e);
      const int t = e / C, c = e - t * C;
      if (v != 0.f) atomicAdd(out + t * a.adj_tf.s[1] + c * a.adj_tf.s[2], v);
    }
  }
}

}  // namespace dvr
