// Adjoint for the TF-gradient-only case with a texture TF, read from the
// forward's sample record.
//
// The forward records, per sample, the density and the opacity accumulated in
// front of the sample.  With those, the adjoint of a ray needs no volume
// access, no ray geometry and no checkpoints: the reverse recursion
// (renderer/renderer_kernels.cuh:367-444 with the blend adjoint of
// renderer/renderer_blending.cuh:63-98, the accumulator before each sample
// read from the record instead of recovered by inverting the blend) runs over
// the record, split over the 32 lanes of a warp (see the kernel).
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

// composition of affine maps x -> A x + B: (A, B) becomes f o g with g = (Ag, Bg)
__device__ __forceinline__ void compose(float& A, float& B, float Ag, float Bg) {
  B = fmaf(A, Bg, B);
  A = A * Ag;
}

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
    if (sc == 1 && (reinterpret_cast<uintptr_t>(e) & 15u) == 0u) {
      if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f)
        atomicAdd(reinterpret_cast<float4*>(e), make_float4(v.x, v.y, v.z, v.w));
      return;
    }
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
  // one texel's four channels: a single 16-byte vector reduction when the
  // channels are contiguous and aligned (the per-warp slices are), else four
  __device__ __forceinline__ void red4(float* e, f4 v) const {
    if (sc == 1 && (reinterpret_cast<uintptr_t>(e) & 15u) == 0u) {
      atomicAdd(reinterpret_cast<float4*>(e), make_float4(v.x, v.y, v.z, v.w));
      return;
    }
    atomicAdd(e, v.x);
    atomicAdd(e + sc, v.y);
    atomicAdd(e + 2 * sc, v.z);
    atomicAdd(e + 3 * sc, v.w);
  }
  // adds k0 * v to texel i0 and k1 * v to texel i1 (i1 = i0 + 1, or i0 at the
  // clamped ends).  Branch-light: about one lane in ten moves to another texel
  // per sample, so nearly every warp step has a mover; the moves are
  // predicates and selects rather than nested branches.
  __device__ __forceinline__ void add(int i0, int i1, f4 v, float k0, float k1) {
    const bool moved = i0 != i, held = i >= 0;
    const bool up = moved && held && i0 == i + 1, down = moved && held && i0 == i - 1;
    const bool jump = moved && held && !up && !down;
    if (up || jump) red4(dst + i * sr, a0);
    if ((down || jump) && i + 1 < R) red4(dst + (i + 1) * sr, a1);
    const f4 z = mk4(0, 0, 0, 0);
    const f4 n0 = up ? a1 : (moved ? z : a0);
    const f4 n1 = down ? a0 : (moved ? z : a1);
    a0 = n0;
    a1 = n1;
    i = i0;
    const bool same = i1 == i0;
    const float q0 = same ? k0 + k1 : k0, q1 = same ? 0.f : k1;
    // the same fused multiply-adds, two channels per packed instruction
    const float2 vxy = make_float2(v.x, v.y), vzw = make_float2(v.z, v.w);
    const float2 a0xy = __ffma2_rn(vxy, make_float2(q0, q0), make_float2(a0.x, a0.y));
    const float2 a0zw = __ffma2_rn(vzw, make_float2(q0, q0), make_float2(a0.z, a0.w));
    const float2 a1xy = __ffma2_rn(vxy, make_float2(q1, q1), make_float2(a1.x, a1.y));
    const float2 a1zw = __ffma2_rn(vzw, make_float2(q1, q1), make_float2(a1.z, a1.w));
    a0 = mk4(a0xy.x, a0xy.y, a0zw.x, a0zw.y);
    a1 = mk4(a1xy.x, a1xy.y, a1zw.x, a1zw.y);
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
  const float2 xy = lerp2(make_float2(t0.x, t0.y), make_float2(t1.x, t1.y), make_float2(df, df));
  const float2 zw = lerp2(make_float2(t0.z, t0.w), make_float2(t1.z, t1.w), make_float2(df, df));
  const f4 cur = mk4(xy.x, xy.y, zw.x, zw.y);
  const float a_k = blend_alpha<BLEND>(cur.w, step);
  f4 adj_cur;
  blend_adjoint_core<BLEND>(a_in, cur, step, a_k, adj_acc, adj_cur);
  acc_tf.add(i0, i1, adj_cur, 1 - df, df);
}

// Affine map x -> A x + B of the opacity adjoint across one sample:
// adj_in = (1 - a) adj_out - a (c . adj_rgb)   (renderer/renderer_blending.cuh:75-93)
template <int BLEND>
__device__ __forceinline__ void record_sample_map(const TfShared<4>& tf, float step, float d, f4 adj_rgb, float& A,
                                                  float& B) {
  const f4 cur = tf_eval<kTfTexture>(tf, d);
  const float a_k = blend_alpha<BLEND>(cur.w, step);
  A = 1.f - a_k;
  B = -a_k * (cur.x * adj_rgb.x + cur.y * adj_rgb.y + cur.z * adj_rgb.z);
}

// The TF-only reverse pass over a run of recorded samples [0, len) of one
// ray, split over the 32 lanes of the calling warp: lane j takes the j-th of
// 32 consecutive segments of L = ceil(len / 32) samples.  Each lane composes
// the affine maps of its segment, a warp suffix scan gives the opacity
// adjoint at the end of every segment, and each lane then walks its segment
// back to front with the full reverse step.  The serial depth is 2 L samples
// instead of len.  adj: the accumulator adjoint behind the run (the colour
// adjoint, constant along the ray, and the opacity adjoint at the run's
// end).  rec(k) returns sample k's (density, incoming opacity).  Returns the
// opacity adjoint in front of the lane's segment: lane 0's value is the one
// in front of the run.
template <int BLEND, class Rec>
__device__ __forceinline__ float record_run_adjoint(const TfShared<4>& tf, float step, int len, const f4 adj, Rec rec,
                                                    TexelPairAtomic& acc_tf) {
  const int lane = threadIdx.x & 31;
  const int L = (len + 31) >> 5;
  const int s0 = min(len, lane * L), s1 = min(len, s0 + L);

  // 1. affine map of the segment: G = f_s0 o f_s0+1 o ... o f_s1-1
  float A = 1.f, B = 0.f;
  {
    int k = s0;
    for (; k + 1 < s1; k += 2) {
      const float2 v0 = rec(k), v1 = rec(k + 1);
      float A0, B0, A1, B1;
      record_sample_map<BLEND>(tf, step, v0.x, adj, A0, B0);
      record_sample_map<BLEND>(tf, step, v1.x, adj, A1, B1);
      compose(A0, B0, A1, B1);
      compose(A, B, A0, B0);
    }
    if (k < s1) {
      float A0, B0;
      record_sample_map<BLEND>(tf, step, rec(k).x, adj, A0, B0);
      compose(A, B, A0, B0);
    }
  }
  // 2. opacity adjoint behind each segment: suffix composition over the lanes
  float SA = A, SB = B;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float Ao = __shfl_down_sync(kFullMask, SA, o), Bo = __shfl_down_sync(kFullMask, SB, o);
    if (lane + o < 32) compose(SA, SB, Ao, Bo);
  }
  const float NA = __shfl_down_sync(kFullMask, SA, 1), NB = __shfl_down_sync(kFullMask, SB, 1);
  f4 adj_acc = adj;
  if (lane < 31) adj_acc.w = fmaf(NA, adj.w, NB);

  // 3. reverse walk over the segment
  {
    int k = s1 - 1;
    float2 v0 = k >= s0 ? rec(k) : make_float2(0.f, 0.f);
    float2 v1 = k - 1 >= s0 ? rec(k - 1) : make_float2(0.f, 0.f);
    for (; k - 1 >= s0; k -= 2) {
      const float2 u0 = k - 2 >= s0 ? rec(k - 2) : make_float2(0.f, 0.f);  // next pair, in flight
      const float2 u1 = k - 3 >= s0 ? rec(k - 3) : make_float2(0.f, 0.f);
      record_reverse_step<BLEND>(tf, step, v0.x, v0.y, adj_acc, acc_tf);
      record_reverse_step<BLEND>(tf, step, v1.x, v1.y, adj_acc, acc_tf);
      v0 = u0;
      v1 = u1;
    }
    if (k >= s0) record_reverse_step<BLEND>(tf, step, v0.x, v0.y, adj_acc, acc_tf);
  }
  return adj_acc.w;
}

// ray_list[0 .. *ray_count): the rays with samples; leftover[0 .. counter[1]):
// the rays left to the general kernel.  tf_slices: (blocks x warps) slices of
// R*C floats, one per warp (TF gradient of a broadcast TF), zeroed here.
//
// One warp per ray: record_run_adjoint over the ray's n recorded samples.
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

  const int lane = threadIdx.x & 31;
  const int total = *ray_count;
  TexelPairAtomic acc_tf;
  acc_tf.R = p.R;
  if (!per_batch) acc_tf.dst = block_slices + (threadIdx.x >> 5) * n_tf;
  int cur_b = -1;

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
    // the ray's ceil(n / 2) groups of 4 floats must lie inside the pool
    if (g < 0 || int64_t(g) + ((n + 1) >> 1) > p.dens_units) {
      if (lane == 0) leftover[atomicAdd(counter + 1, 1)] = id;
      continue;
    }
    const float step = step_at(p.step, b, y, x);
    const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] + y * a.adj_color.s[1] +
                      x * a.adj_color.s[2];
    const f4 adj_col = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
    const float2* rec = reinterpret_cast<const float2*>(p.dens + 4 * size_t(g));
    const TfShared<C> tf{s_tf + (copies > 1 ? b : 0) * n_tf, p.R};
    if (per_batch && b != cur_b) {
      acc_tf.flush();
      cur_b = b;
      acc_tf.dst = static_cast<float*>(a.adj_tf.p) + b * a.adj_tf.s[0];
      acc_tf.sr = a.adj_tf.s[1];
      acc_tf.sc = a.adj_tf.s[2];
    }

    record_run_adjoint<BLEND>(tf, step, n, adj_col, [rec](int k) { return __ldg(rec + k); }, acc_tf);
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

// Samples of one re-marched chunk: each warp's shared-memory run of
// (density, incoming opacity) pairs holds this many.
constexpr int kRemarchCap = 512;

// The chunk length of the re-march adjoint for checkpoint interval K: a
// multiple of K (every chunk starts at a checkpoint) and of 2, at most
// kRemarchCap; 0 when no such length fits (never for the intervals the entry
// points accept, 1 to 64).
__host__ __device__ inline int remarch_chunk(int K) {
  const int unit = K % 2 == 0 ? K : 2 * K;
  return K > 0 && unit <= kRemarchCap ? unit * (kRemarchCap / unit) : 0;
}

// Entries of a warp's run: the chunk's pairs and up to 32 pad entries.
__host__ __device__ inline int remarch_run_entries(int chunk) { return chunk + 32; }

// Shared memory of the re-march adjoint (floats): the TF copies, then each
// warp's run of (density, opacity) pairs.
__host__ __device__ inline int remarch_smem_floats(int R, int C, int tf_copies, int warps, int chunk) {
  return record_smem_floats(R, C, tf_copies) + warps * remarch_run_entries(chunk) * 2;
}

// TF-gradient-only adjoint of a texture TF from the transmittance
// checkpoints alone (no sample record): the memory-lean path.  One warp per
// ray takes the ray's n samples in chunks of `chunk` samples from the back.
// A chunk is re-marched from the checkpoint at its start (the opacity in
// front of sample c0, written by the forward) with the forward's warp scan,
// 64 samples per step and two per lane, into the warp's shared-memory run,
// and that run is reversed by record_run_adjoint with the opacity adjoint
// carried from the chunk behind it.  The adjoint needs O(warps) memory
// instead of the record's O(samples), and each sample is gathered once more
// than with the record.  Rays the checkpoints do not cover (n above
// (slots + 1) K) go to leftover for the general kernel.  ray_list, leftover
// and tf_slices as fast_adjoint_record_kernel; GATHER as the forward's
// (direct loads or the slab texture tg).
template <int FILTER, int BLEND, typename VT, int GATHER>
__global__ void __launch_bounds__(kFastThreads, 6)
    fast_adjoint_remarch_kernel(const RenderParams p, const AdjointParams a, const RayOrder order, int* counter,
                                const int* ray_list, const int* ray_count, int* leftover, float* tf_slices,
                                const TexGather tg, int chunk) {
  extern __shared__ float4 fast_smem4[];
  constexpr int C = 4;
  float* s_tf = reinterpret_cast<float*>(fast_smem4);
  const int copies = tf_copies(p);
  for (int bb = 0; bb < copies; ++bb) stage_tf(p, bb, s_tf + bb * p.R * C);
  const int n_tf = p.R * C;
  const int warps = int(blockDim.x) / 32;
  // the warp's run of remarch_run_entries(chunk) pairs
  float2* run = reinterpret_cast<float2*>(s_tf + record_smem_floats(p.R, C, copies)) +
                size_t(threadIdx.x >> 5) * remarch_run_entries(chunk);
  const bool per_batch = a.adj_tf.s[0] != 0;
  float* block_slices = tf_slices + size_t(blockIdx.x) * warps * n_tf;
  if (!per_batch)
    for (int e = threadIdx.x; e < warps * n_tf; e += blockDim.x) block_slices[e] = 0.f;
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int total = *ray_count;
  const int K = p.ckpt_interval;
  TexelPairAtomic acc_tf;
  acc_tf.R = p.R;
  if (!per_batch) acc_tf.dst = block_slices + (threadIdx.x >> 5) * n_tf;
  int cur_b = -1;

  while (true) {
    int pos = 0;
    if (lane == 0) pos = atomicAdd(counter, 1);
    pos = __shfl_sync(kFullMask, pos, 0);
    if (pos >= total) break;
    const int id = ray_list[pos];
    int b, x, y;
    if (!order.pixel(id, b, x, y)) continue;
    FastRay q;
    fast_setup(p, x, y, b, q);
    const int n = min(static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] +
                                                             x * a.fwd_term.s[2]],
                      max_samples(q.tmin, q.tmax, q.step));
    if (n <= 0) continue;
    // every chunk start c0 < n is a multiple of K with c0 / K - 1 < slots
    if (n > (p.ckpt_slots + 1) * K) {
      if (lane == 0) leftover[atomicAdd(counter + 1, 1)] = id;
      continue;
    }
    const float* ck = static_cast<const float*>(p.ckpt.p) + b * p.ckpt.s[0] + y * p.ckpt.s[1] + x * p.ckpt.s[2];
    const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] + y * a.adj_color.s[1] +
                      x * a.adj_color.s[2];
    f4 adj = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
    const TfShared<C> tf{s_tf + (copies > 1 ? b : 0) * n_tf, p.R};
    if (per_batch && b != cur_b) {
      acc_tf.flush();
      cur_b = b;
      acc_tf.dst = static_cast<float*>(a.adj_tf.p) + b * a.adj_tf.s[0];
      acc_tf.sr = a.adj_tf.s[1];
      acc_tf.sc = a.adj_tf.s[2];
    }
    const VolumeFast<VT> vol{static_cast<const VT*>(p.volume.p) + b * p.volume.s[0], int(p.volume.s[1]),
                             int(p.volume.s[2]), int(p.volume.s[3]), p.X - 1, p.Y - 1, p.Z - 1};
    const TexVolume<VT> tv{tg, p.volume.s[0] != 0 ? b * p.X : 0, p.X - 1, p.Y - 1, p.Z - 1};

    for (int c0 = ((n - 1) / chunk) * chunk; c0 >= 0; c0 -= chunk) {
      const int len = min(n - c0, chunk);
      // The reverse pass reads lane j's segment [j L, j L + L) of the run
      // (L = ceil(len / 32)) one entry per lane at a time.  Sample i is stored
      // at i + pad floor(i / L), one pad entry after every segment when L is
      // even, so the lanes' entries lie an odd number L + pad of pairs apart
      // and a half-warp's reads fall in distinct banks.  At most 31 pads.
      const int L = (len + 31) >> 5;
      const int pad = (L & 1) ^ 1;
      const float inv_L = 1.f / float(L);
      // 1. re-march [c0, c0 + len) from the opacity in front of sample c0
      float alpha = c0 > 0 ? ck[(c0 / K - 1) * p.ckpt.s[3]] : 0.f;
      for (int s0 = 0; s0 < len; s0 += 64) {
        const int i0 = s0 + 2 * lane;  // the lane's samples: run entries i0 and i0 + 1
        const bool in0 = i0 < len, in1 = i0 + 1 < len;
        float d[2], a_s[2] = {0.f, 0.f};
        // lanes past the chunk's end gather at its first sample (inside the
        // ray) and discard the value
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const int k = c0 + ((i == 0 ? in0 : in1) ? i0 + i : 0);
          const float3 q3 = fast_pos(q, q.tmin + k * q.step);
          if constexpr (GATHER == kGatherTexture) d[i] = tv.sample(q3);
          else d[i] = sample_density<FILTER, VT>(vol, q3);
        }
        if (in0) a_s[0] = blend_alpha<BLEND>(tf_eval<kTfTexture>(tf, d[0]).w, q.step);
        if (in1) a_s[1] = blend_alpha<BLEND>(tf_eval<kTfTexture>(tf, d[1]).w, q.step);
        // incoming opacity of each sample: exclusive "over" scan of the pairs
        float incl = over(a_s[0], a_s[1]);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float v = __shfl_up_sync(kFullMask, incl, o);
          if (lane >= o) incl = over(v, incl);
        }
        float excl = __shfl_up_sync(kFullMask, incl, 1);
        if (lane == 0) excl = 0.f;
        const float a_in0 = over(alpha, excl), a_in1 = over(a_in0, a_s[0]);
        // floor(i / L) for i < 512, L <= 16: (i + 1/2) / L is at least 1/32
        // from an integer, far above the rounding of one multiplication
        if (pad) {
          if (in0) run[i0 + __float2int_rz((float(i0) + 0.5f) * inv_L)] = make_float2(d[0], a_in0);
          if (in1) run[i0 + 1 + __float2int_rz((float(i0) + 1.5f) * inv_L)] = make_float2(d[1], a_in1);
        } else {
          if (in0) run[i0] = make_float2(d[0], a_in0);
          if (in1) run[i0 + 1] = make_float2(d[1], a_in1);
        }
        alpha = over(alpha, __shfl_sync(kFullMask, incl, 31));
      }
      __syncwarp();
      // 2. reverse the chunk; the opacity adjoint in front of it goes on to
      // the chunk before
      // lane j reads only its own segment: entry k sits at k + j pad
      const float2* seg = run + lane * pad;
      adj.w = __shfl_sync(kFullMask,
                          record_run_adjoint<BLEND>(tf, q.step, len, adj, [seg](int k) { return seg[k]; }, acc_tf), 0);
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
