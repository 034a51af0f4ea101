// Forward march with one warp per ray.
//
// The 32 lanes of a warp take 64 consecutive samples of the same ray at once,
// two adjacent ones per lane: each lane gathers its samples' densities and
// evaluates the TF, then the warp composites the 64 samples front to back.
// Compositing is associative (the "over" operator: opacity a then b gives
// a + (1 - a) b, colour likewise), so a 5-step warp scan over the lanes'
// pairs gives every sample's incoming opacity, from which follow the
// early-termination point (the first sample whose incoming opacity exceeds
// blendingEarlyOut, renderer/renderer_kernels.cuh:55-58), each sample's
// colour contribution (1 - incoming opacity) a c (summed per lane, then over
// the warp at the end of the ray) and the transmittance checkpoints.  The
// per-sample arithmetic is the reference's
// (renderer/renderer_blending.cuh:30-49); only the order of the compositing
// sums differs, by rounding.
//
// All 64 gathers of a step are independent and issued together, lanes never
// diverge on cell or termination events, and a lane keeps no per-ray state,
// so registers are few and many warps fit per SM.  Warps fetch one ray at a
// time from the longest-first order of the rays with samples.
#pragma once
#include "dvr_cells.cuh"
#include "dvr_persist.cuh"

namespace dvr {

template <int FILTER, typename VT>
__device__ __forceinline__ float sample_density(const VolumeFast<VT>& v, float3 q) {
  if constexpr (FILTER == kNearest) {
    return v.at(nearest_coord(q.x, v.X1 + 1), nearest_coord(q.y, v.Y1 + 1), nearest_coord(q.z, v.Z1 + 1));
  } else {
    const int ix = int(q.x), iy = int(q.y), iz = int(q.z);
    float d[8];
    v.corners(ix, iy, iz, d);
    return trilerp(d, q.x - float(ix), q.y - float(iy), q.z - float(iz));
  }
}

// opacity a, then b: a + (1 - a) b
__device__ __forceinline__ float over(float a, float b) { return a + (1.f - a) * b; }

// How a trilinear sample reads its eight corners.
enum { kGatherDirect = 0, kGatherCells = 1, kGatherTexture = 2 };

// Marches ray (b, x, y) with the 32 lanes of the calling warp, 64
// consecutive samples per step, two adjacent ones per lane (lane l takes
// samples 2l and 2l + 1 of the step): writes its colour and termination
// index, and per sample the (density, incoming opacity) pair to rec (when not
// nullptr) or the opacity before every K-th sample to the checkpoints ck
// (when not nullptr).  sample(float3 q) returns the density at volume
// position q.  Every lane of the warp calls it with the same ray.
//
// Two samples per lane halve the scan, ballot and loop work per sample, put
// four independent texture gathers (or sixteen corner loads) of a lane in
// flight at once, and store a lane's two record entries as one 16-byte
// store.  A ray that terminates early computes at most 63 samples past its
// end, against 31 with one sample per lane.
template <int TF, int BLEND, class Sample>
__device__ __forceinline__ void warp_march_ray(const RenderParams& p, int b, int x, int y, const FastRay& q,
                                               int kmax, const TfShared<TfChannels<TF>::C>& tf, float* rec,
                                               float* ck, Sample sample) {
  const int lane = threadIdx.x & 31;
  const int K = p.ckpt_interval;
  const int kshift = (K & (K - 1)) == 0 ? __ffs(K) - 1 : -1;  // log2 K for a power-of-two interval
  // sample 0 lies in the volume whenever the ray has samples: lanes whose
  // samples are past the ray's end gather there, so every lane issues its
  // gathers unconditionally and the result is discarded
  const bool has = kmax > 0 && !(q.tmin > q.tmax);
  float alpha = 0.f;  // accumulated opacity before the step
  float cr = 0.f, cg = 0.f, cb = 0.f;  // this lane's samples' colour contributions
  int n = 0;
  for (int k0 = 0;; k0 += 64) {
    const int k = k0 + 2 * lane;  // the lane's samples k and k + 1
    float density[2] = {0.f, 0.f}, a[2] = {0.f, 0.f};
    f4 c[2] = {mk4(0, 0, 0, 0), mk4(0, 0, 0, 0)};
    bool in_ray[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) in_ray[i] = k + i < kmax && !(q.tmin + (k + i) * q.step > q.tmax);
    if (has) {
      float d[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) d[i] = sample(fast_pos(q, q.tmin + (in_ray[i] ? k + i : 0) * q.step));
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        if (in_ray[i]) {
          density[i] = d[i];
          c[i] = tf_eval<TF, true>(tf, d[i]);
          a[i] = blend_alpha<BLEND>(c[i].w, q.step);
        }
      }
    }
    // incoming opacity of each pair: exclusive "over" scan of the lanes' pairs
    float incl = over(a[0], a[1]);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float v = __shfl_up_sync(kFullMask, incl, o);
      if (lane >= o) incl = over(v, incl);
    }
    float excl = __shfl_up_sync(kFullMask, incl, 1);
    if (lane == 0) excl = 0.f;
    float a_in[2];
    a_in[0] = over(alpha, excl);
    a_in[1] = over(a_in[0], a[0]);
    // first sample of the step not taken: past the ray's end or behind the
    // early-termination opacity
    const unsigned m0 = __ballot_sync(kFullMask, in_ray[0] && !(a_in[0] > p.early_out));
    const unsigned m1 = __ballot_sync(kFullMask, in_ray[1] && !(a_in[1] > p.early_out));
    const int f = min(m0 == kFullMask ? 64 : 2 * (__ffs(~m0) - 1), m1 == kFullMask ? 64 : 2 * __ffs(~m1) - 1);
    const bool used0 = 2 * lane < f, used1 = 2 * lane + 1 < f;
    if (rec) {
      if (used1) __stcs(reinterpret_cast<float4*>(rec + 2 * k), make_float4(density[0], a_in[0], density[1], a_in[1]));
      else if (used0) __stcs(reinterpret_cast<float2*>(rec) + k, make_float2(density[0], a_in[0]));
    }
    if (ck) {
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int ki = k + i;
        if ((i == 0 ? used0 : used1) && ki > 0) {
          // opacity before sample (slot + 1) * K
          const bool at = kshift >= 0 ? (ki & (K - 1)) == 0 : ki % K == 0;
          const int slot = (kshift >= 0 ? ki >> kshift : ki / K) - 1;
          if (at && slot < p.ckpt_slots) ck[slot * p.ckpt.s[3]] = a_in[i];
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      if (i == 0 ? used0 : used1) {
        const float w = (1.f - a_in[i]) * a[i];
        const float2 rg = __ffma2_rn(make_float2(w, w), make_float2(c[i].x, c[i].y), make_float2(cr, cg));
        cr = rg.x;
        cg = rg.y;
        cb = fmaf(w, c[i].z, cb);
      }
    }
    if (f < 64) {
      alpha = __shfl_sync(kFullMask, (f & 1) ? a_in[1] : a_in[0], f >> 1);
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
  if (lane == 0) {
    float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
    col[0] = cr;
    col[p.color.s[3]] = cg;
    col[2 * p.color.s[3]] = cb;
    col[3 * p.color.s[3]] = alpha;
    static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = n;
  }
}

// ray_list[0 .. *ray_count): the rays with samples (longest first); the
// ordering pass has already finished the others.  GATHER: trilinear samples
// load the corners directly from the volume, read the cell-corner volume
// `cells`, or gather them from the slab texture `tg`.
template <int FILTER, int TF, int BLEND, typename VT, int GATHER>
__global__ void __launch_bounds__(kFastThreads) fast_forward_warp_kernel(const RenderParams p, const RayOrder order,
                                                                         int* counter, const int* ray_list,
                                                                         const int* ray_count,
                                                                         const CellWords<VT>* cells,
                                                                         const TexGather tg) {
  extern __shared__ float4 fast_smem4[];
  constexpr int C = TfChannels<TF>::C;
  float* s_tf = reinterpret_cast<float*>(fast_smem4);
  const int copies = tf_copies(p);
  for (int bb = 0; bb < copies; ++bb) stage_tf(p, bb, s_tf + bb * p.R * C);
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int total = *ray_count;
  unsigned long long* const bump = reinterpret_cast<unsigned long long*>(counter + 2);

  while (true) {
    int pos = 0;
    if (lane == 0) pos = atomicAdd(counter, 1);
    pos = __shfl_sync(kFullMask, pos, 0);
    if (pos >= total) break;
    int b, x, y;
    if (!order.pixel(ray_list[pos], b, x, y)) continue;
    FastRay q;
    fast_setup(p, x, y, b, q);
    const int kmax = max_samples(q.tmin, q.tmax, q.step);

    float* rec = nullptr;
    if (p.dens) {
      // room for kmax (density, incoming opacity) pairs, in groups of 4 floats
      const unsigned long long claim = static_cast<unsigned long long>((kmax + 1) >> 1);
      unsigned long long g = 0;
      if (lane == 0) g = atomicAdd(bump, claim);
      g = __shfl_sync(kFullMask, g, 0);
      const bool fits = g + claim <= static_cast<unsigned long long>(p.dens_units);
      if (lane == 0)
        static_cast<int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] + x * p.dens_off.s[2]] =
            fits ? int(g) : -1;
      if (fits) rec = p.dens + 4 * g;
    }
    const VolumeFast<VT> vol{static_cast<const VT*>(p.volume.p) + b * p.volume.s[0], int(p.volume.s[1]),
                             int(p.volume.s[2]), int(p.volume.s[3]), p.X - 1, p.Y - 1, p.Z - 1};
    const size_t vb = p.volume.s[0] != 0 ? size_t(b) * p.X * p.Y * p.Z : 0;
    const CellVolume<VT> cv{cells ? cells + vb : nullptr, p.X - 1, p.Y - 1, p.Z - 1};
    const TexVolume<VT> tv{tg, p.volume.s[0] != 0 ? b * p.X : 0, p.X - 1, p.Y - 1, p.Z - 1};
    const TfShared<C> tf{s_tf + (copies > 1 ? b : 0) * p.R * C, p.R};
    // a recorded ray carries its opacities in the record: no checkpoints
    float* ck = p.ckpt.p && !rec
                    ? static_cast<float*>(p.ckpt.p) + b * p.ckpt.s[0] + y * p.ckpt.s[1] + x * p.ckpt.s[2]
                    : nullptr;

    warp_march_ray<TF, BLEND>(p, b, x, y, q, kmax, tf, rec, ck, [&](float3 pos) {
      if constexpr (GATHER == kGatherCells) return cv.sample(pos);
      else if constexpr (GATHER == kGatherTexture) return tv.sample(pos);
      else return sample_density<FILTER, VT>(vol, pos);
    });
  }
}

}  // namespace dvr
