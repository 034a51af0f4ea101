// Forward-mode differentiation of the march (renderer::Renderer::
// renderForwardGradients, renderer/renderer_kernels.cuh:131-240) and the
// contraction of its forward variables with an output adjoint
// (forwardVariablesToGradients, renderer/renderer_kernels.cuh:505-560).
//
// The output of the forward mode is, per pixel, the 4 x D Jacobian of the
// colour with respect to D selected variables: the step size, the components
// of the ray start and direction (after ray generation) and TF entries.  The
// reference carries D derivatives through every step of a thread's march
// (dual numbers), O(D) work per sample.  Here the derivative recurrence is
// split by linearity: one blend step maps the accumulator's derivatives as
//
//   d rgb' = d rgb - c a dA + (1 - A) (a dc + c da)
//   d A'   = (1 - a) dA     + (1 - A) da
//
// (A = opacity in front of the sample, a = sample alpha, c = sample colour),
// i.e. a homogeneous part M = (rgb, A) -> (rgb - Q A, P A) with Q = c a,
// P = 1 - a, common to all D derivatives, plus the sample's local seeds (dc,
// da), non-zero only for the few variables the sample touches.  Homogeneous
// maps compose front to back like colours: M1 then M2 = (Q1 + P1 Q2, P1 P2).
// One warp marches a ray 32 samples at a time (one sample per lane, as the
// warp-per-ray forward does); a warp suffix scan of the maps gives, for each
// sample, the map of the samples behind it in the chunk, which carries the
// sample's seeds to the chunk end directly.  The Jacobian block of the ray
// (D x 4 floats in shared memory) is mapped once per chunk by the whole
// chunk's map and receives the seeds by shared-memory atomics; the seven
// camera/step-size derivatives, which every sample touches, are per-lane
// registers reduced over the warp at the end of the ray.  Work per sample is
// O(variables touched), not O(D).
//
// Derivative semantics follow the reference's forward mode: the entry and
// exit distances are not traced; nearest sampling has no position
// derivative; clamps select an operand together with its derivative (the
// identity TF passes the density derivative strictly inside (0, 1), like its
// adjoint; the linear TF's clamp of the density to [p0, p1] takes the
// derivative of the bound it clamps to).
#pragma once
#include <algorithm>
#include <climits>
#include "dvr_kernels.h"
#include "dvr_persist.cuh"
#include "dvr_warpray.cuh"

namespace dvr {

// d c / d density of the TF (renderer/renderer_tf.cuh:122-150, :256-290,
// :437-486, :522-560 with a traced density).
template <int TF, class A>
__device__ __forceinline__ f4 tf_slope(const A& tf, float density) {
  if constexpr (TF == kTfIdentity) {
    if (!(density > 0.f && density < 1.f)) return mk4(0, 0, 0, 0);
    const float sa = tf.at(0, 0), sc = tf.at(0, 1);
    return mk4(sc, sc, sc, sa);
  } else if constexpr (TF == kTfTexture) {
    const int R = tf.R;
    const int di = int(floorf(density * R - 0.5f));
    const f4 a = tf.rgba(clampi(di, 0, R - 1)), c = tf.rgba(clampi(di + 1, 0, R - 1));
    return mk4(R * (c.x - a.x), R * (c.y - a.y), R * (c.z - a.z), R * (c.w - a.w));
  } else if constexpr (TF == kTfLinear) {
    const int i = linear_interval(tf, density);
    const float p0 = tf.at(i, 4), p1 = tf.at(i + 1, 4);
    if (density < p0 || density > p1) return mk4(0, 0, 0, 0);
    const f4 a = tf.rgba(i), c = tf.rgba(i + 1);
    const float inv = 1.f / (p1 - p0);
    return mk4((c.x - a.x) * inv, (c.y - a.y) * inv, (c.z - a.z) * inv, (c.w - a.w) * inv);
  } else {
    f4 s = mk4(0, 0, 0, 0);
    for (int i = 0; i < tf.R; ++i) {
      const f4 ci = tf.rgba(i);
      const float mu = tf.at(i, 4), sigma = tf.at(i, 5);
      const float f = gauss(density, mu, sigma) * (mu - density) / (sigma * sigma);
      s.x += ci.x * f;
      s.y += ci.y * f;
      s.z += ci.z * f;
      s.w += ci.w * f;
    }
    return s;
  }
}

// Per-lane weights of one sample's seeds: a colour derivative dc of the
// sample changes the chunk-end state by
//   rgb: Ta dc.rgb + e (Taw dc.w),   A: Ep Taw dc.w
// with Ta = (1 - A) a, Taw = (1 - A) d alpha / d absorption and e = c - (the
// colour behind the sample in the chunk), Ep = the transmittance behind it.
// All zero for lanes whose sample is not taken.
struct SeedWeights {
  float Ta, Taw, er, eg, eb, Ep;
  __device__ __forceinline__ f4 of(f4 dc) const {
    const float u = Taw * dc.w;
    return mk4(fmaf(Ta, dc.x, er * u), fmaf(Ta, dc.y, eg * u), fmaf(Ta, dc.z, eb * u), Ep * u);
  }
};

// Sums v over the run of consecutive lanes with this lane's key, from this
// lane to the run's end (suffix segmented scan); returns whether the lane
// starts its run, i.e. holds the run's total.
template <int N>
__device__ __forceinline__ bool run_sums(float (&v)[N], int key, int lane) {
  const int prev = __shfl_up_sync(kFullMask, key, 1);
  const bool head = lane == 0 || prev != key;
  const unsigned after = __ballot_sync(kFullMask, head) & ~((2u << lane) - 1u);
  const int last = after ? __ffs(after) - 2 : 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const float t = __shfl_down_sync(kFullMask, v[i], o);
      if (lane + o <= last) v[i] += t;
    }
  }
  return head;
}

// Sums v over the warp into lane 0.
template <int N>
__device__ __forceinline__ void warp_sums(float (&v)[N]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] += __shfl_down_sync(kFullMask, v[i], o);
}

// Adds (x, y, z, w) to the Jacobian row of TF entry (r, c) when it is traced
// in this pass.  Entries may share an index, so the adds are atomic.
struct TfRows {
  float4* J;
  const int* dtf;
  int64_t s1, s2;
  int d0, dn;
  __device__ __forceinline__ void add(int r, int c, float x, float y, float z, float w) const {
    const int idx = __ldg(dtf + r * s1 + c * s2) - d0;
    if (idx < 0 || idx >= dn) return;
    float* jp = reinterpret_cast<float*>(J + idx);
    if (x != 0.f) atomicAdd(jp + 0, x);
    if (y != 0.f) atomicAdd(jp + 1, y);
    if (z != 0.f) atomicAdd(jp + 2, z);
    if (w != 0.f) atomicAdd(jp + 3, w);
  }
};

// The TF-entry seeds of the warp's 32 samples (renderer/renderer_tf.cuh, the
// evalForwardGradients overloads with TF derivatives), summed over the lanes
// that touch the same entries before they reach shared memory: runs of
// consecutive samples in one texel cell / control-point interval (texture,
// linear), the whole warp (identity and Gaussian TFs, whose samples all touch
// every entry).  Called by all 32 lanes.
template <int TF, class A>
__device__ __forceinline__ void tf_seeds_warp(const A& tf, float density, bool used, const SeedWeights& w,
                                              const TfRows& rows, int lane) {
  if constexpr (TF == kTfIdentity) {
    // (0,0) absorption scale: dc = (0,0,0,d); (0,1) colour scale: dc = (d,d,d,0)
    const float d = used ? clampf(density, 0.f, 1.f) : 0.f;
    float v[5] = {w.er * w.Taw * d, w.eg * w.Taw * d, w.eb * w.Taw * d, w.Ep * w.Taw * d, w.Ta * d};
    warp_sums(v);
    if (lane == 0) {
      rows.add(0, 0, v[0], v[1], v[2], v[3]);
      rows.add(0, 1, v[4], v[4], v[4], 0.f);
    }
  } else if constexpr (TF == kTfTexture) {
    const int R = tf.R;
    const float dd = density * R - 0.5f;
    const int di = int(floorf(dd));
    const float df = dd - di;
    const float w0 = 1.f - df;
    const float u0 = w.Taw * w0, u1 = w.Taw * df;
    // texel i0: rgb entries get Ta w0 in their channel, the absorption entry (e u0, Ep u0); texel i1 likewise
    float v[10] = {w.Ta * w0, w.er * u0, w.eg * u0, w.eb * u0, w.Ep * u0,
                   w.Ta * df, w.er * u1, w.eg * u1, w.eb * u1, w.Ep * u1};
    const bool head = run_sums(v, used ? di : INT_MIN, lane);
    if (head && used) {
      const int i0 = clampi(di, 0, R - 1), i1 = clampi(di + 1, 0, R - 1);
      rows.add(i0, 0, v[0], 0.f, 0.f, 0.f);
      rows.add(i0, 1, 0.f, v[0], 0.f, 0.f);
      rows.add(i0, 2, 0.f, 0.f, v[0], 0.f);
      rows.add(i0, 3, v[1], v[2], v[3], v[4]);
      rows.add(i1, 0, v[5], 0.f, 0.f, 0.f);
      rows.add(i1, 1, 0.f, v[5], 0.f, 0.f);
      rows.add(i1, 2, 0.f, 0.f, v[5], 0.f);
      rows.add(i1, 3, v[6], v[7], v[8], v[9]);
    }
  } else if constexpr (TF == kTfLinear) {
    const int i = used ? linear_interval(tf, density) : 0;
    const float p0 = tf.at(i, 4), p1 = tf.at(i + 1, 4);
    const bool inside = !(density < p0) && !(density > p1);
    const float d2 = density < p0 ? p0 : (density > p1 ? p1 : density);
    const float den = p1 - p0;
    const float fr = (d2 - p0) / den;
    const float w0 = 1.f - fr;
    const float u0 = w.Taw * w0, u1 = w.Taw * fr;
    f4 k0 = mk4(0, 0, 0, 0), k1 = mk4(0, 0, 0, 0);  // control-point position seeds
    if (inside && used) {
      const f4 a = tf.rgba(i), c = tf.rgba(i + 1);
      const f4 K = w.of(mk4(c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w));
      const float den2 = den * den;
      const float g0 = (d2 - p1) / den2, g1 = (p0 - d2) / den2;
      k0 = mk4(K.x * g0, K.y * g0, K.z * g0, K.w * g0);
      k1 = mk4(K.x * g1, K.y * g1, K.z * g1, K.w * g1);
    }
    float v[18] = {w.Ta * w0, w.er * u0, w.eg * u0, w.eb * u0, w.Ep * u0, k0.x, k0.y, k0.z, k0.w,
                   w.Ta * fr, w.er * u1, w.eg * u1, w.eb * u1, w.Ep * u1, k1.x, k1.y, k1.z, k1.w};
    const bool head = run_sums(v, used ? i : INT_MIN, lane);
    if (head && used) {
      rows.add(i, 0, v[0], 0.f, 0.f, 0.f);
      rows.add(i, 1, 0.f, v[0], 0.f, 0.f);
      rows.add(i, 2, 0.f, 0.f, v[0], 0.f);
      rows.add(i, 3, v[1], v[2], v[3], v[4]);
      rows.add(i, 4, v[5], v[6], v[7], v[8]);
      rows.add(i + 1, 0, v[9], 0.f, 0.f, 0.f);
      rows.add(i + 1, 1, 0.f, v[9], 0.f, 0.f);
      rows.add(i + 1, 2, 0.f, 0.f, v[9], 0.f);
      rows.add(i + 1, 3, v[10], v[11], v[12], v[13]);
      rows.add(i + 1, 4, v[14], v[15], v[16], v[17]);
    }
  } else {
    for (int i = 0; i < tf.R; ++i) {
      // entry (i, c<3): Ta n; (i, 3): (e, Ep) Taw n; mean and sigma: their dc through the seed weights
      const f4 ci = tf.rgba(i);
      const float mu = tf.at(i, 4), sigma = tf.at(i, 5);
      const float n = used ? gauss(density, mu, sigma) : 0.f;
      const float e = density - mu, s2 = sigma * sigma;
      const float gm = n * e / s2, gs = n * e * e / (s2 * sigma);
      const f4 K = w.of(ci);
      const float u = w.Taw * n;
      float v[13] = {w.Ta * n, w.er * u, w.eg * u, w.eb * u, w.Ep * u, K.x * gm, K.y * gm, K.z * gm, K.w * gm,
                     K.x * gs, K.y * gs, K.z * gs, K.w * gs};
      warp_sums(v);
      if (lane == 0) {
        rows.add(i, 0, v[0], 0.f, 0.f, 0.f);
        rows.add(i, 1, 0.f, v[0], 0.f, 0.f);
        rows.add(i, 2, 0.f, 0.f, v[0], 0.f);
        rows.add(i, 3, v[1], v[2], v[3], v[4]);
        rows.add(i, 4, v[5], v[6], v[7], v[8]);
        rows.add(i, 5, v[9], v[10], v[11], v[12]);
      }
    }
  }
}

// Seven per-ray variables: ray start x y z, direction x y z, step size.
struct RoleSums {
  float v[7][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int r = 0; r < 7; ++r) v[r][0] = v[r][1] = v[r][2] = v[r][3] = 0.f;
  }
  __device__ __forceinline__ void map(float qr, float qg, float qb, float pp) {
#pragma unroll
    for (int r = 0; r < 7; ++r) {
      const float A = v[r][3];
      v[r][0] = fmaf(-qr, A, v[r][0]);
      v[r][1] = fmaf(-qg, A, v[r][1]);
      v[r][2] = fmaf(-qb, A, v[r][2]);
      v[r][3] = pp * A;
    }
  }
};

// ROLES: some of the seven per-ray variables are traced in this pass.
template <int FILTER, int TF, int BLEND, typename VT, bool ROLES>
__global__ void __launch_bounds__(kFwdThreads) forward_gradients_kernel(const RenderParams p, const FwdGradParams g,
                                                                        int* counter) {
  extern __shared__ float4 fwd_smem4[];
  constexpr int C = TfChannels<TF>::C;
  float* s_tf = reinterpret_cast<float*>(fwd_smem4);
  const int copies = tf_copies(p);
  for (int bb = 0; bb < copies; ++bb) stage_tf(p, bb, s_tf + bb * p.R * C);
  const int tf_f4 = (copies * p.R * C + 3) >> 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float4* J = fwd_smem4 + tf_f4 + warp * g.dn;  // this ray's Jacobian block, dn x (r, g, b, A)
  __syncthreads();

  // the seven per-ray variables that fall into this pass: slot in J, or -1
  int role[7];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    role[c] = g.d_start[c] - g.d0;
    role[3 + c] = g.d_dir[c] - g.d0;
  }
  role[6] = g.d_step - g.d0;
#pragma unroll
  for (int r = 0; r < 7; ++r)
    if (role[r] < 0 || role[r] >= g.dn) role[r] = -1;
  const bool need_slope = ROLES && FILTER == kTrilinear &&
                          (role[0] >= 0 || role[1] >= 0 || role[2] >= 0 || role[3] >= 0 || role[4] >= 0 ||
                           role[5] >= 0 || role[6] >= 0);
  const int rays = p.B * p.H * p.W;

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
    if (kmax == 0) {
      // no samples: zero colour and derivatives, written straight to the outputs
      float* out = g.grad + b * g.grad_s[0] + y * g.grad_s[1] + x * g.grad_s[2] + g.d0 * g.grad_s[3];
      for (int e = lane; e < 4 * g.dn; e += 32) out[(e >> 2) * g.grad_s[3] + (e & 3) * g.grad_s[4]] = 0.f;
      if (lane == 0) {
        float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
        col[0] = col[p.color.s[3]] = col[2 * p.color.s[3]] = col[3 * p.color.s[3]] = 0.f;
        static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = 0;
      }
      continue;
    }
    for (int i = lane; i < g.dn; i += 32) J[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    const VolumeFast<VT> vol{static_cast<const VT*>(p.volume.p) + b * p.volume.s[0], int(p.volume.s[1]),
                             int(p.volume.s[2]), int(p.volume.s[3]), p.X - 1, p.Y - 1, p.Z - 1};
    const TfShared<C> tf{s_tf + (copies > 1 ? b : 0) * p.R * C, p.R};
    const TfRows rows{J, g.has_tf ? g.d_tf + b * g.dtf_s[0] : nullptr, g.dtf_s[1], g.dtf_s[2], g.d0, g.dn};
    const f3 gsc = mk3(1.f / q.voxel.x, 1.f / q.voxel.y, 1.f / q.voxel.z);

    RoleSums rs;
    if constexpr (ROLES) rs.zero();
    float alpha = 0.f, cr = 0.f, cg = 0.f, cb = 0.f;
    int n = 0;
    for (int k0 = 0;; k0 += 32) {
      const int k = k0 + lane;
      const float t = q.tmin + k * q.step;
      const bool in_ray = k < kmax && !(t > q.tmax);
      float density = 0.f, a = 0.f;
      f3 grad = mk3(0, 0, 0);
      f4 c = mk4(0, 0, 0, 0);
      if (in_ray) {
        const float3 pq = fast_pos(q, t);
        if constexpr (FILTER == kNearest) {
          density = sample_density<FILTER, VT>(vol, pq);
        } else {
          const int ix = int(pq.x), iy = int(pq.y), iz = int(pq.z);
          float d[8];
          vol.corners(ix, iy, iz, d);
          density = trilerp_grad(d, pq.x - float(ix), pq.y - float(iy), pq.z - float(iz), grad);
        }
        c = tf_eval<TF>(tf, density);
        a = blend_alpha<BLEND>(c.w, q.step);
      }
      // opacity in front of each sample: exclusive "over" scan
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
      const bool used = lane < f;

      // homogeneous blend map of each sample; the samples not taken are identities
      float Qr = used ? c.x * a : 0.f, Qg = used ? c.y * a : 0.f, Qb = used ? c.z * a : 0.f;
      float P = used ? 1.f - a : 1.f;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {  // inclusive suffix composition, this sample first
        const float r2 = __shfl_down_sync(kFullMask, Qr, o), g2 = __shfl_down_sync(kFullMask, Qg, o);
        const float b2 = __shfl_down_sync(kFullMask, Qb, o), p2 = __shfl_down_sync(kFullMask, P, o);
        if (lane + o < 32) {
          Qr = fmaf(P, r2, Qr);
          Qg = fmaf(P, g2, Qg);
          Qb = fmaf(P, b2, Qb);
          P *= p2;
        }
      }
      // map of the samples behind this one in the chunk
      float Er = __shfl_down_sync(kFullMask, Qr, 1), Eg = __shfl_down_sync(kFullMask, Qg, 1);
      float Eb = __shfl_down_sync(kFullMask, Qb, 1), Ep = __shfl_down_sync(kFullMask, P, 1);
      if (lane == 31) Er = Eg = Eb = 0.f, Ep = 1.f;
      const float Mr = __shfl_sync(kFullMask, Qr, 0), Mg = __shfl_sync(kFullMask, Qg, 0);
      const float Mb = __shfl_sync(kFullMask, Qb, 0), Mp = __shfl_sync(kFullMask, P, 0);

      // carry the state in front of the chunk through the chunk
      if (g.has_tf && f > 0) {
        for (int i = lane; i < g.dn; i += 32) {
          float4 v = J[i];
          v.x = fmaf(-Mr, v.w, v.x);
          v.y = fmaf(-Mg, v.w, v.y);
          v.z = fmaf(-Mb, v.w, v.z);
          v.w *= Mp;
          J[i] = v;
        }
      }
      if constexpr (ROLES) rs.map(Mr, Mg, Mb, Mp);
      __syncwarp();

      // d alpha / d absorption and / d step (renderer/renderer_blending.cuh:40-52, :104-116)
      float aw, as;
      if constexpr (BLEND == kBeerLambert) {
        const float e = 1.f - a;
        aw = q.step * e;
        as = c.w * e;
      } else {
        const bool lin = c.w * q.step < 1.f;
        aw = lin ? q.step : 0.f;
        as = lin ? c.w : 0.f;
      }
      const float T = used ? 1.f - a_in : 0.f;
      const SeedWeights sw{T * a, T * aw, c.x - Er, c.y - Eg, c.z - Eb, Ep};
      if (g.has_tf && f > 0) tf_seeds_warp<TF>(tf, density, used, sw, rows, lane);
      if constexpr (ROLES) {
        if (used) {
          f4 kd = mk4(0, 0, 0, 0);  // state change per unit density derivative
          f3 gs = mk3(0, 0, 0);      // d density / d ray start
          if (need_slope) {
            kd = sw.of(tf_slope<TF>(tf, density));
            gs = mk3(grad.x * gsc.x, grad.y * gsc.y, grad.z * gsc.z);
          }
          const float dd[7] = {gs.x, gs.y, gs.z, t * gs.x, t * gs.y, t * gs.z,
                               k * (gs.x * q.dir.x + gs.y * q.dir.y + gs.z * q.dir.z)};
#pragma unroll
          for (int r = 0; r < 7; ++r) {
            rs.v[r][0] = fmaf(kd.x, dd[r], rs.v[r][0]);
            rs.v[r][1] = fmaf(kd.y, dd[r], rs.v[r][1]);
            rs.v[r][2] = fmaf(kd.z, dd[r], rs.v[r][2]);
            rs.v[r][3] = fmaf(kd.w, dd[r], rs.v[r][3]);
          }
          // the step size's own alpha dependence: d alpha = as
          const float u = T * as;
          rs.v[6][0] = fmaf(sw.er, u, rs.v[6][0]);
          rs.v[6][1] = fmaf(sw.eg, u, rs.v[6][1]);
          rs.v[6][2] = fmaf(sw.eb, u, rs.v[6][2]);
          rs.v[6][3] = fmaf(sw.Ep, u, rs.v[6][3]);
        }
      }
      if (used) {
        const float wgt = (1.f - a_in) * a;
        cr = fmaf(wgt, c.x, cr);
        cg = fmaf(wgt, c.y, cg);
        cb = fmaf(wgt, c.z, cb);
      }
      __syncwarp();
      if (f < 32) {
        alpha = __shfl_sync(kFullMask, a_in, f);
        n = k0 + f;
        break;
      }
      alpha = over(alpha, __shfl_sync(kFullMask, incl, 31));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      cr += __shfl_xor_sync(kFullMask, cr, o);
      cg += __shfl_xor_sync(kFullMask, cg, o);
      cb += __shfl_xor_sync(kFullMask, cb, o);
    }
    if constexpr (ROLES) {
#pragma unroll
      for (int r = 0; r < 7; ++r)
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          float v = rs.v[r][ch];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
          rs.v[r][ch] = v;
        }
    }
    if (lane == 0) {
      float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
      col[0] = cr;
      col[p.color.s[3]] = cg;
      col[2 * p.color.s[3]] = cb;
      col[3 * p.color.s[3]] = alpha;
      static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = n;
      if constexpr (ROLES) {
        // several variables may share an index: their derivatives add up
#pragma unroll
        for (int r = 0; r < 7; ++r)
          if (role[r] >= 0) {
            float4 v = J[role[r]];
            v.x += rs.v[r][0];
            v.y += rs.v[r][1];
            v.z += rs.v[r][2];
            v.w += rs.v[r][3];
            J[role[r]] = v;
          }
      }
    }
    __syncwarp();
    float* out = g.grad + b * g.grad_s[0] + y * g.grad_s[1] + x * g.grad_s[2] + g.d0 * g.grad_s[3];
    const float* js = reinterpret_cast<const float*>(J);
    for (int e = lane; e < 4 * g.dn; e += 32) out[(e >> 2) * g.grad_s[3] + (e & 3) * g.grad_s[4]] = js[e];
    __syncwarp();
  }
}

#ifdef DVR_FWDVARS_DEFINE
// Forward variables [b][y][x][d][c] contracted with adj_color [b][y][x][c].
// One warp per pixel (grid-stride over the pixels of batch entry blockIdx.y),
// so a pixel's D x 4 variables are read as one contiguous run.  Lanes 0-6
// write the pixel's ray and step-size gradients; TF entries are spread over
// the lanes and summed per warp in shared memory (a lane owns its entries:
// plain adds), then over the block, then added to adj_tf once per block.
__global__ void __launch_bounds__(kFwdVarsThreads) forward_variables_to_gradients_kernel(const FwdVarsParams v) {
  extern __shared__ float fv_smem[];
  constexpr int nw = kFwdVarsThreads / 32;
  const int b = blockIdx.y;
  const int E = v.has_tf ? v.R * v.C : 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // shared memory: the warps' TF sums, then each entry's derivative index
  const bool tf_smem = E > 0 && E * (nw + 1) <= kFwdVarsSmemFloats;
  float* acc = fv_smem + warp * E;
  int* s_idx = reinterpret_cast<int*>(fv_smem + nw * E);
  const int* dtf = E > 0 ? v.d_tf + b * v.dtf_s[0] : nullptr;
  if (tf_smem) {
    for (int e = lane; e < E; e += 32) acc[e] = 0.f;
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const int r = e / v.C, c = e - r * v.C;
      const int idx = __ldg(dtf + r * v.dtf_s[1] + c * v.dtf_s[2]);
      s_idx[e] = idx >= 0 && idx < v.D ? idx : -1;
    }
    __syncthreads();
  }
  float* tf_out = E > 0 ? v.adj_tf + b * v.tf_s[0] : nullptr;
  const bool vec = v.fwd_s[4] == 1 && v.fwd_s[3] == 4 && (reinterpret_cast<uintptr_t>(v.fwd) & 15u) == 0 &&
                   (v.fwd_s[2] & 3) == 0 && (v.fwd_s[1] & 3) == 0 && (v.fwd_s[0] & 3) == 0;
  // the per-pixel variable this lane writes (lanes 0-6: start xyz, dir xyz, step)
  int my_d = -1;
  float* my_out = nullptr;
  int64_t my_s0 = 0, my_s1 = 0, my_s2 = 0;
  bool my_acc = false;
  if (lane < 3 && v.has_camera) {
    my_d = v.d_start[0] * (lane == 0) + v.d_start[1] * (lane == 1) + v.d_start[2] * (lane == 2);
    my_out = v.adj_start + lane * v.start_s[3];
    my_s0 = v.start_s[0], my_s1 = v.start_s[1], my_s2 = v.start_s[2];
    my_acc = v.camera_broadcast;
  } else if (lane >= 3 && lane < 6 && v.has_camera) {
    my_d = v.d_dir[0] * (lane == 3) + v.d_dir[1] * (lane == 4) + v.d_dir[2] * (lane == 5);
    my_out = v.adj_dir + (lane - 3) * v.dir_s[3];
    my_s0 = v.dir_s[0], my_s1 = v.dir_s[1], my_s2 = v.dir_s[2];
    my_acc = v.camera_broadcast;
  } else if (lane == 6 && v.has_step) {
    my_d = v.d_step;
    my_out = v.adj_step;
    my_s0 = v.step_s[0], my_s1 = v.step_s[1], my_s2 = v.step_s[2];
    my_acc = v.step_broadcast;
  }
  const int pixels = v.H * v.W;
  for (int pix = blockIdx.x * nw + warp; pix < pixels; pix += gridDim.x * nw) {
    const int y = pix / v.W, x = pix - y * v.W;
    const float* fv = v.fwd + b * v.fwd_s[0] + y * v.fwd_s[1] + x * v.fwd_s[2];
    const float* gp = v.adj_color + b * v.adj_s[0] + y * v.adj_s[1] + x * v.adj_s[2];
    const f4 gc = mk4(__ldg(gp), __ldg(gp + v.adj_s[3]), __ldg(gp + 2 * v.adj_s[3]), __ldg(gp + 3 * v.adj_s[3]));
    auto dotd = [&](int d) {
      if (vec) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(fv) + d);
        return gc.x * q.x + gc.y * q.y + gc.z * q.z + gc.w * q.w;
      }
      const float* q = fv + d * v.fwd_s[3];
      return gc.x * q[0] + gc.y * q[v.fwd_s[4]] + gc.z * q[2 * v.fwd_s[4]] + gc.w * q[3 * v.fwd_s[4]];
    };
    if (my_d >= 0) {
      float* o = my_out + b * my_s0 + y * my_s1 + x * my_s2;
      const float val = dotd(my_d);
      if (my_acc) atomicAdd(o, val);
      else *o = val;
    }
    if (tf_smem) {
      // indices from shared memory: the row reads of a pixel are independent
#pragma unroll 4
      for (int e = lane; e < E; e += 32) {
        const int idx = s_idx[e];
        if (idx >= 0) acc[e] += dotd(idx);
      }
    } else {
      for (int e = lane; e < E; e += 32) {
        const int r = e / v.C, c = e - r * v.C;
        const int idx = __ldg(dtf + r * v.dtf_s[1] + c * v.dtf_s[2]);
        if (idx < 0 || idx >= v.D) continue;
        atomicAdd(tf_out + r * v.tf_s[1] + c * v.tf_s[2], dotd(idx));
      }
    }
  }
  if (tf_smem) {
    __syncthreads();
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      float sum = 0.f;
#pragma unroll
      for (int w = 0; w < nw; ++w) sum += fv_smem[w * E + e];
      const int r = e / v.C, c = e - r * v.C;
      if (sum != 0.f) atomicAdd(tf_out + r * v.tf_s[1] + c * v.tf_s[2], sum);
    }
  }
}
#endif

#ifdef DVR_FWDGRAD_DEFINE
template <int FILTER, int TF, int BLEND, typename VT, bool ROLES>
static cudaError_t forward_gradients_roles(const RenderParams& p, const FwdGradParams& g, const LaunchInfo& li,
                                           cudaStream_t s) {
  auto kernel = forward_gradients_kernel<FILTER, TF, BLEND, VT, ROLES>;
  const int copies = p.tf.s[0] == 0 ? 1 : p.B;
  const size_t smem = size_t((copies * p.R * TfChannels<TF>::C + 3) / 4) * 16 + size_t(kFwdThreads / 32) * g.dn * 16;
  if (smem > size_t(li.max_smem_optin)) return cudaErrorInvalidConfiguration;
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kFwdThreads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int64_t rays = int64_t(p.B) * p.H * p.W;
  const int64_t need = (rays + kFwdThreads / 32 - 1) / (kFwdThreads / 32);
  const int grid = int(std::min<int64_t>(need, int64_t(per_sm) * li.num_sms));
  cudaError_t err = cudaSuccess;
  int* counter = acquire_counter(li.device, s, err);
  if (err != cudaSuccess) return err;
  kernel<<<grid, kFwdThreads, smem, s>>>(p, g, counter);
  return cudaGetLastError();
}

template <int FILTER, int TF, int BLEND, typename VT>
static cudaError_t forward_gradients_go(const RenderParams& p, const FwdGradParams& g, const LaunchInfo& li,
                                        cudaStream_t s) {
  bool roles = false;
  for (int c = 0; c < 3; ++c)
    roles |= (g.d_start[c] >= g.d0 && g.d_start[c] < g.d0 + g.dn) || (g.d_dir[c] >= g.d0 && g.d_dir[c] < g.d0 + g.dn);
  roles |= g.d_step >= g.d0 && g.d_step < g.d0 + g.dn;
  return roles ? forward_gradients_roles<FILTER, TF, BLEND, VT, true>(p, g, li, s)
               : forward_gradients_roles<FILTER, TF, BLEND, VT, false>(p, g, li, s);
}

template <int TF, typename VT>
cudaError_t launch_forward_gradients_vt(const RenderParams& p, const FwdGradParams& g, int filter, int blend,
                                        const LaunchInfo& li, cudaStream_t s) {
  if (filter == kNearest)
    return blend == kBeerLambert ? forward_gradients_go<kNearest, TF, kBeerLambert, VT>(p, g, li, s)
                                 : forward_gradients_go<kNearest, TF, kAlphaBlend, VT>(p, g, li, s);
  return blend == kBeerLambert ? forward_gradients_go<kTrilinear, TF, kBeerLambert, VT>(p, g, li, s)
                               : forward_gradients_go<kTrilinear, TF, kAlphaBlend, VT>(p, g, li, s);
}

template <int TF>
cudaError_t launch_forward_gradients(const RenderParams& p, const FwdGradParams& g, int filter, int blend,
                                     const LaunchInfo& li, cudaStream_t s) {
  switch (p.vol_storage) {
    case kF16: return launch_forward_gradients_vt<TF, __half>(p, g, filter, blend, li, s);
    case kBF16: return launch_forward_gradients_vt<TF, __nv_bfloat16>(p, g, filter, blend, li, s);
    default: return launch_forward_gradients_vt<TF, float>(p, g, filter, blend, li, s);
  }
}
#endif

}  // namespace dvr
