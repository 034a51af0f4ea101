// Adjoint for the TF-gradient-only case with a texture TF, read from the
// forward's sample record.
//
// The forward records, per sample, the density and the opacity accumulated in
// front of the sample.  With those, the adjoint of a ray needs no volume
// access, no ray geometry and no checkpoints: each lane walks its ray back to
// front through the record and runs the reverse recursion
// (renderer/renderer_kernels.cuh:367-444 with the blend adjoint of
// renderer/renderer_blending.cuh:63-98, the accumulator before each sample
// read from the record instead of recovered by inverting the blend).  The
// state of a lane is a few registers, so many warps fit per SM, and lanes
// whose ray is done take the next ray from the longest-first order.
//  * TF gradient: the two texels (i, i+1) of the current sample in registers;
//    a texel leaving them is added with fire-and-forget global reductions to
//    the warp's slice of an L2-resident scratch (or to the per-batch output);
//    the slices are summed per block at the end.
//  * rays without a record (the pool was full) are appended to a leftover
//    list that the general kernel processes afterwards.
// The record and the termination indices must come from the same forward
// pass; reads stay inside the pool in any case.
#pragma once
#include "dvr_warpray.cuh"

namespace dvr {

// Shared memory of the record adjoint (floats): the TF copies.
__host__ __device__ inline int record_smem_floats(int R, int C, int tf_copies) { return (tf_copies * R * C + 3) & ~3; }

// A lane's TF-gradient accumulator: the pair of texels (i, i+1) in registers,
// other texels added atomically to dst (texel t, channel c at dst[t*sr + c*sc]).
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

// One reverse step of the TF-only adjoint: sample with density d and incoming
// opacity a_in; updates the accumulator adjoint and the TF gradient.
template <int BLEND>
__device__ __forceinline__ void record_reverse_step(const TfShared<4>& tf, float step, float d, float a_in,
                                                    f4& adj_acc, TexelPairAtomic& acc_tf) {
  const int R = tf.R;
  const float dd = d * R - 0.5f;
  const int di = int(floorf(dd));
  const float df = dd - di;
  const int i0 = clampi(di, 0, R - 1), i1 = clampi(di + 1, 0, R - 1);
  const f4 t0 = tf.rgba(i0), t1 = tf.rgba(i1);
  const f4 cur = mk4(lerp1(t0.x, t1.x, df), lerp1(t0.y, t1.y, df), lerp1(t0.z, t1.z, df), lerp1(t0.w, t1.w, df));
  const float a_k = blend_alpha<BLEND>(cur.w, step);
  f4 adj_cur;
  blend_adjoint_core<BLEND>(a_in, cur, step, a_k, adj_acc, adj_cur);
  acc_tf.add(i0, i1, adj_cur, 1 - df, df);
}

// ray_list[0 .. *ray_count): the rays with samples; leftover[0 .. counter[1]):
// the rays left to the general kernel.  tf_slices: (blocks x warps) slices of
// R*C floats, one per warp (TF gradient of a broadcast TF), zeroed here.
template <int BLEND>
__global__ void __launch_bounds__(kFastThreads) fast_adjoint_record_kernel(const RenderParams p, const AdjointParams a,
                                                                            const RayOrder order, int* counter,
                                                                            const int* ray_list, const int* ray_count,
                                                                            int* leftover, float* tf_slices) {
  extern __shared__ float4 fast_smem4[];
  constexpr int C = 4;
  float* s_tf = reinterpret_cast<float*>(fast_smem4);
  const int copies = tf_copies(p);
  for (int bb = 0; bb < copies; ++bb) stage_tf(p, bb, s_tf + bb * p.R * C);
  const int n_tf = p.R * C;
  const int warps = int(blockDim.x) / 32;
  const bool per_batch = a.adj_tf.s[0] != 0;
  float* block_slices = tf_slices + size_t(blockIdx.x) * warps * n_tf;
  if (!per_batch)
    for (int e = threadIdx.x; e < warps * n_tf; e += blockDim.x) block_slices[e] = 0.f;
  __syncthreads();

  const int total = *ray_count;
  TexelPairAtomic acc_tf;
  acc_tf.R = p.R;
  if (!per_batch) acc_tf.dst = block_slices + (threadIdx.x >> 5) * n_tf;
  int cur_b = -1;

  // The record of a ray is read as groups of 4 floats (samples 2m and 2m+1);
  // a round walks back over two groups, the next round's two are loaded
  // during it.
  bool exhausted = false, active = false;
  int n = 0, m = 0;  // samples of the ray; the round's upper group
  float step = 0.f;
  f4 adj_acc = mk4(0, 0, 0, 0);
  const float4* rec = nullptr;
  float4 g0 = make_float4(0.f, 0.f, 0.f, 0.f), g1 = g0;  // groups m and m - 1
  TfShared<C> tf{s_tf, p.R};

  while (true) {
    while (true) {
      int id = fetch_rays(counter, total, !active, exhausted);
      if (id >= 0) id = ray_list[id];
      int b, x, y;
      if (id >= 0 && order.pixel(id, b, x, y)) {
        n = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
        if (n > 0) {
          const int g = static_cast<const int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] +
                                                              x * p.dens_off.s[2]];
          // the ray's ceil(n / 2) groups must lie inside the pool
          if (g < 0 || int64_t(g) + ((n + 1) >> 1) > p.dens_units) {
            leftover[atomicAdd(counter + 1, 1)] = id;
          } else {
            active = true;
            step = step_at(p.step, b, y, x);
            const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] +
                              y * a.adj_color.s[1] + x * a.adj_color.s[2];
            adj_acc = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
            rec = reinterpret_cast<const float4*>(p.dens) + g;
            m = (n - 1) >> 1;
            g0 = __ldcs(rec + m);
            g1 = m >= 1 ? __ldcs(rec + m - 1) : make_float4(0.f, 0.f, 0.f, 0.f);
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

#pragma unroll 1
    for (int round = 0; round < 2; ++round) {
      if (active) {
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 h0 = m >= 2 ? __ldcs(rec + m - 2) : z;  // next round's groups
        const float4 h1 = m >= 3 ? __ldcs(rec + m - 3) : z;
        if (2 * m + 1 < n) record_reverse_step<BLEND>(tf, step, g0.z, g0.w, adj_acc, acc_tf);
        record_reverse_step<BLEND>(tf, step, g0.x, g0.y, adj_acc, acc_tf);
        if (m >= 1) {
          record_reverse_step<BLEND>(tf, step, g1.z, g1.w, adj_acc, acc_tf);
          record_reverse_step<BLEND>(tf, step, g1.x, g1.y, adj_acc, acc_tf);
        }
        m -= 2;
        g0 = h0;
        g1 = h1;
        if (m < 0) active = false;
      }
      __syncwarp();
    }
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
