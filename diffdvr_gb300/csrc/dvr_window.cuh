// Window adjoint: the volume-gradient adjoint for rays with a sample record,
// organised around the volume instead of around the rays.
//
// The reference scatters each sample's volume gradient with eight global
// atomics on cell exit (renderer/renderer_interpolation.cuh:299-321).  With
// many views of one volume nearly every voxel receives hundreds of such
// additions, and the adjoint is bound by L2 atomic throughput.  Here a block
// takes a 16x8 tile of one view's rays (one ray per thread; neighbouring rays
// run nearly parallel) and walks them back to front in slabs of equal ray
// distance t: in slab [T - dt, T) every thread runs the reverse recursion over
// its own samples with t in that range.  The slab's samples touch a compact
// box of voxels, computed per slab as the bounding box of the tile's first and
// last cells in the slab (positions along a ray are monotone per axis).  The
// block accumulates the slab's volume gradient in a dense shared-memory copy
// of that box (shared atomics, per-cell register accumulation in front of
// them), then adds every non-zero group of four z-neighbours to global memory
// with one 16-byte vector reduction and zeroes it behind itself.  Where the
// camera or step-size gradient needs the eight corner densities of a sample,
// the slab's box of the volume is first staged into shared memory with bulk
// copies (cp.async.bulk, one per (x, y) row of 16-byte aligned storage,
// completion on an mbarrier), so corner reads come from shared memory instead
// of scattered global loads.
//
// The slab depth adapts: it halves while the box exceeds the shared-memory
// window and grows again when the box is small.  A slab whose box does not fit
// even at one step of depth falls back to global atomics.  Rays without a
// record go to a leftover list for the general adjoint kernel.  The reverse
// step's arithmetic is that of dvr_fast.cuh (exact recursion from the
// recorded incoming opacity).
#pragma once
#include "dvr_persist.cuh"

namespace dvr {

constexpr int kWinTileW = 16, kWinTileH = 8;     // rays of a block: one per thread
constexpr float kWinInitVoxels = 8.f;            // initial slab depth in voxels
constexpr float kWinMaxVoxels = 32.f;
constexpr long long kWinSpinLimit = 1ll << 26;   // mbarrier polls before giving up

// Tiles of the window kernel: row-major per batch entry.
struct WinTiles {
  int W, H, B, nx, ny;
  __host__ __device__ static WinTiles make(int W, int H, int B) {
    return WinTiles{W, H, B, (W + kWinTileW - 1) / kWinTileW, (H + kWinTileH - 1) / kWinTileH};
  }
  __host__ __device__ int total() const { return B * nx * ny; }
};

// RayOrder id of pixel (x, y) of batch entry b (8x4 patches), for the
// leftover list of the general kernel.
__device__ __forceinline__ int ray_order_id(const RayOrder& o, int b, int x, int y) {
  return b * (o.pxn * o.pyn * 32) + ((y / kPatchH) * o.pxn + x / kPatchW) * 32 + (y % kPatchH) * kPatchW +
         (x % kPatchW);
}

// The slab's box: voxels [x0, x0 + nx) x [y0, y0 + ny) x [z0, z0 + nz); the
// gradient window rounds z to multiples of 4 floats, the staged volume to
// multiples of 16 bytes of storage.
struct WinBox {
  int x0, y0, z0, nx, ny, nz;   // gradient window (z0 % 4 == 0, nz % 4 == 0)
  int vz0, vnz;                 // staged volume rows (16-byte aligned)
};

// Distance of sample k along the ray, one rounding (the same expression
// wherever a slab's box and its samples are computed, so the box holds every
// cell its samples touch).
__device__ __forceinline__ float sample_t(const FastRay& r, int k) { return __fmaf_rn(float(k), r.step, r.tmin); }

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// ---- bulk copies into shared memory (the copy engine's non-tensor mode)
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
// true once the phase of parity `parity` has completed
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Per-cell register accumulation of the volume gradient (as VolGradCell),
// flushed into the slab's shared-memory window, or into global memory with
// atomics when the slab has no window.
struct WinGradCell {
  int cx = -1, cy = -1, cz = -1;
  float g[8];
  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int q = 0; q < 8; ++q) g[q] = 0.f;
  }
  __device__ __forceinline__ void flush(float* win, const WinBox& w, float* adjv, const OutView& o, int X1, int Y1,
                                        int Z1) {
    if (cx < 0) return;
    const int lx = clampi(cx, 0, X1), hx = clampi(cx + 1, 0, X1);
    const int ly = clampi(cy, 0, Y1), hy = clampi(cy + 1, 0, Y1);
    const int lz = clampi(cz, 0, Z1), hz = clampi(cz + 1, 0, Z1);
    // a cell outside the window (the box is built to hold every cell of the
    // slab, so this does not happen) goes to global memory
    if (win && (lx < w.x0 || hx >= w.x0 + w.nx || ly < w.y0 || hy >= w.y0 + w.ny || lz < w.z0 || hz >= w.z0 + w.nz))
      win = nullptr;
    if (win) {
      const int ax = (lx - w.x0) * w.ny, bx = (hx - w.x0) * w.ny;
      const int ay = ly - w.y0, by = hy - w.y0;
      const int az = lz - w.z0, bz = hz - w.z0;
      atomicAdd(win + (ax + ay) * w.nz + az, g[0]);
      atomicAdd(win + (ax + ay) * w.nz + bz, g[1]);
      atomicAdd(win + (ax + by) * w.nz + az, g[2]);
      atomicAdd(win + (ax + by) * w.nz + bz, g[3]);
      atomicAdd(win + (bx + ay) * w.nz + az, g[4]);
      atomicAdd(win + (bx + ay) * w.nz + bz, g[5]);
      atomicAdd(win + (bx + by) * w.nz + az, g[6]);
      atomicAdd(win + (bx + by) * w.nz + bz, g[7]);
    } else {
      const int64_t sx = o.s[1], sy = o.s[2], sz = o.s[3];
      atomicAdd(adjv + lx * sx + ly * sy + lz * sz, g[0]);
      atomicAdd(adjv + lx * sx + ly * sy + hz * sz, g[1]);
      atomicAdd(adjv + lx * sx + hy * sy + lz * sz, g[2]);
      atomicAdd(adjv + lx * sx + hy * sy + hz * sz, g[3]);
      atomicAdd(adjv + hx * sx + ly * sy + lz * sz, g[4]);
      atomicAdd(adjv + hx * sx + ly * sy + hz * sz, g[5]);
      atomicAdd(adjv + hx * sx + hy * sy + lz * sz, g[6]);
      atomicAdd(adjv + hx * sx + hy * sy + hz * sz, g[7]);
    }
    cx = -1;
    reset();
  }
};

// Corner densities of cell (ix, iy, iz) (clamped corners) from the staged
// window of the volume (plain shared-memory loads), or from global memory.
template <typename VT>
__device__ __forceinline__ void win_corners(const VT* sv, const WinBox& w, const VolumeFast<VT>& vol, int ix, int iy,
                                            int iz, float* d) {
  const int lx = clampi(ix, 0, vol.X1), hx = clampi(ix + 1, 0, vol.X1);
  const int ly = clampi(iy, 0, vol.Y1), hy = clampi(iy + 1, 0, vol.Y1);
  const int lz = clampi(iz, 0, vol.Z1) - w.vz0, hz = clampi(iz + 1, 0, vol.Z1) - w.vz0;
  // a cell outside the staged box (not expected) is read from global memory
  if (sv && lx >= w.x0 && hx < w.x0 + w.nx && ly >= w.y0 && hy < w.y0 + w.ny && lz >= 0 && hz < w.vnz) {
    const VT* pll = sv + ((lx - w.x0) * w.ny + (ly - w.y0)) * w.vnz;
    const VT* plh = sv + ((lx - w.x0) * w.ny + (hy - w.y0)) * w.vnz;
    const VT* phl = sv + ((hx - w.x0) * w.ny + (ly - w.y0)) * w.vnz;
    const VT* phh = sv + ((hx - w.x0) * w.ny + (hy - w.y0)) * w.vnz;
    d[0] = to_float(pll[lz]);
    d[1] = to_float(pll[hz]);
    d[2] = to_float(plh[lz]);
    d[3] = to_float(plh[hz]);
    d[4] = to_float(phl[lz]);
    d[5] = to_float(phl[hz]);
    d[6] = to_float(phh[lz]);
    d[7] = to_float(phh[hz]);
  } else {
    vol.corners(ix, iy, iz, d);
  }
}

// Block-wide min (lo) and max (hi) of three ints each; red: 6 * warps ints.
__device__ __forceinline__ void block_box(int lo[3], int hi[3], int* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    lo[c] = __reduce_min_sync(kFullMask, lo[c]);
    hi[c] = __reduce_max_sync(kFullMask, hi[c]);
  }
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      red[warp * 6 + c] = lo[c];
      red[warp * 6 + 3 + c] = hi[c];
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    int l = red[c], h = red[3 + c];
    for (int w = 1; w < nw; ++w) {
      l = min(l, red[w * 6 + c]);
      h = max(h, red[w * 6 + 3 + c]);
    }
    lo[c] = l;
    hi[c] = h;
  }
  __syncthreads();
}

// Block-wide maximum of one float per thread; red: one float per warp.
__device__ __forceinline__ float block_max(float v, int* red) {
  float* f = reinterpret_cast<float*>(red);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFullMask, v, o));
  if ((threadIdx.x & 31) == 0) f[threadIdx.x >> 5] = v;
  __syncthreads();
  v = f[0];
  for (int w = 1; w < int(blockDim.x >> 5); ++w) v = fmaxf(v, f[w]);
  __syncthreads();
  return v;
}

// Shared-memory layout of the window kernel (floats): the adjoint layout
// without segment buffers, then the gradient window, the staged volume
// window, the box reduction, the tile index and the mbarrier.
struct WinSmem {
  int base, grad, vol, red, bar, total;
  __host__ __device__ WinSmem(int tf_mode, int R, int C, bool tfgrad, int copies, int grad_cap, int vol_bytes) {
    const AdjointSmem L(tf_mode, R, C, kFastThreads, tfgrad, 0, copies);
    base = L.total;
    grad = (base + 3) & ~3;
    vol = grad + grad_cap;
    red = vol + ((vol_bytes + 15) / 16) * 4;
    bar = red + 6 * (kFastThreads / 32) + 4;
    bar = (bar + 3) & ~3;
    total = bar + 4;
  }
};

// STAGE: stage the slab's volume box in shared memory for the corner reads of
// the position derivative (camera / step-size gradients).
template <int TF, int BLEND, bool TFGRAD, bool STAGE, typename VT>
__global__ void __launch_bounds__(kFastThreads) window_adjoint_kernel(const RenderParams p, const AdjointParams a,
                                                                       const WinTiles tiles, const RayOrder order,
                                                                       int* counters, float* tf_scratch,
                                                                       int* leftover, int grad_cap, int vol_cap) {
  extern __shared__ float4 fast_smem4[];
  constexpr int C = TfChannels<TF>::C;
  float* smem = reinterpret_cast<float*>(fast_smem4);
  const int copies = tf_copies(p);
  const AdjointSmem L(TF, p.R, C, kFastThreads, TFGRAD, 0, copies);
  const WinSmem S(TF, p.R, C, TFGRAD, copies, grad_cap, STAGE ? vol_cap * int(sizeof(VT)) : 0);
  float* s_tf = smem + L.tf;
  float* win = smem + S.grad;
  VT* svol = reinterpret_cast<VT*>(smem + S.vol);
  int* red = reinterpret_cast<int*>(smem + S.red);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + S.bar);
  int* s_tile = red + 6 * (kFastThreads / 32);
  for (int bb = 0; bb < copies; ++bb) stage_tf(p, bb, s_tf + bb * p.R * C);
  float* block_slice = tf_scratch ? tf_scratch + size_t(blockIdx.x) * p.R * C : nullptr;
  if constexpr (TFGRAD) {
    for (int e = threadIdx.x; e < L.seg - L.warp; e += blockDim.x) smem[L.warp + e] = 0.f;
    for (int e = threadIdx.x; e < p.R * C; e += blockDim.x) block_slice[e] = 0.f;
  }
  // the gradient window starts at zero; each slab's flush zeroes what it used
  for (int e = threadIdx.x * 4; e < grad_cap; e += blockDim.x * 4)
    *reinterpret_cast<float4*>(win + e) = make_float4(0.f, 0.f, 0.f, 0.f);
  if (STAGE && threadIdx.x == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  unsigned phase = 0;

  const bool tf_per_batch = TFGRAD && a.adj_tf.s[0] != 0;
  float* s_grad_warp = smem + L.warp + (threadIdx.x >> 5) * p.R * C;
  TfGradAccum<TF, TFGRAD> tacc;
  tacc.bind(smem + L.lane, int(blockDim.x), int(threadIdx.x), L.slots, p.R);
  if (!tf_per_batch) tacc.set_evict_target(block_slice, C, 1);
  int cur_b = -1;
  const bool need_pos = a.has_camera || a.has_stepsize;
  const int X1 = p.X - 1, Y1 = p.Y - 1, Z1 = p.Z - 1;
  const int64_t gsx = a.adj_volume.s[1], gsy = a.adj_volume.s[2];
  const int vsx = int(p.volume.s[1]), vsy = int(p.volume.s[2]);
  constexpr int kVtPerRow = 16 / int(sizeof(VT));  // storage elements per 16 bytes
  bool failed = false;

  while (true) {
    if (threadIdx.x == 0) *s_tile = atomicAdd(counters, 1);
    __syncthreads();
    const int tile = *s_tile;
    __syncthreads();
    if (tile >= tiles.total()) break;
    const int per_b = tiles.nx * tiles.ny;
    const int b = tile / per_b;
    const int rem = tile - b * per_b;
    const int ty = rem / tiles.nx, tx = rem - ty * tiles.nx;
    int px, py;
    tile_pixel(threadIdx.x, px, py);
    const int x = tx * kWinTileW + px, y = ty * kWinTileH + py;
    const bool valid = x < p.W && y < p.H;

    FastRay r{};
    int n = 0, n_ray = 0;
    const float2* drow = nullptr;
    if (valid) {
      fast_setup(p, x, y, b, r);
      n = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
      n = min(n, max_samples(r.tmin, r.tmax, r.step));
      n_ray = n;
      if (n > 0) {
        const int g = static_cast<const int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] +
                                                            x * p.dens_off.s[2]];
        if (g >= 0 && int64_t(g) + ((n + 1) >> 1) <= p.dens_units) {
          drow = reinterpret_cast<const float2*>(p.dens + 4 * size_t(g));
        } else {
          // no record: the general kernel takes this ray
          leftover[atomicAdd(counters + 1, 1)] = ray_order_id(order, b, x, y);
          n = 0;
        }
      }
    }
    f4 adj_acc = mk4(0, 0, 0, 0);
    if (n > 0) {
      const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] + y * a.adj_color.s[1] +
                        x * a.adj_color.s[2];
      adj_acc = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
    }
    if (tf_per_batch && b != cur_b) {
      if (cur_b >= 0)
        tacc.flush_global(static_cast<float*>(a.adj_tf.p) + cur_b * a.adj_tf.s[0], a.adj_tf.s[1], a.adj_tf.s[2],
                          s_grad_warp);
      cur_b = b;
      tacc.set_evict_target(static_cast<float*>(a.adj_tf.p) + b * a.adj_tf.s[0], a.adj_tf.s[1], a.adj_tf.s[2]);
    }
    const VolumeFast<VT> vol{static_cast<const VT*>(p.volume.p) + b * p.volume.s[0], vsx, vsy,
                             int(p.volume.s[3]), X1, Y1, Z1};
    const TfShared<C> tf{s_tf + (copies > 1 ? b : 0) * p.R * C, p.R};
    float* adjv = static_cast<float*>(a.adj_volume.p) + b * a.adj_volume.s[0];
    float adj_step = 0.f;
    f3 adj_start = mk3(0, 0, 0), adj_dir = mk3(0, 0, 0);
    WinGradCell vg;
    vg.reset();
    float d8[8];
    int scx = -1, scy = -1, scz = -1;  // cell of d8

    // the slab front: the largest remaining sample distance of the tile; the
    // slab depth and its lower bound are the same for every thread (the
    // smallest voxel edge and step of the tile's rays with samples)
    int k = n - 1;
    float T = block_max(k >= 0 ? sample_t(r, k) : -INFINITY, red);
    const float vmin = -block_max(n > 0 ? -fminf(r.voxel.x, fminf(r.voxel.y, r.voxel.z)) : -INFINITY, red);
    const float step_min = -block_max(n > 0 ? -r.step : -INFINITY, red);
    float dt = kWinInitVoxels * vmin;

    while (T > -INFINITY && !failed) {
      // the slab [T - dt, T): this thread's samples k_stop .. k
      int k_stop = k + 1;
      WinBox w{};
      bool direct = false;
      float dt_used = dt;
      while (true) {
        const float T_lo = T - dt;
        k_stop = k + 1;
        int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
        if (k >= 0) {
          const float f = ceilf((T_lo - r.tmin) / r.step);
          k_stop = f <= 0.f ? 0 : (f > float(k) ? k + 1 : int(f));
          if (sample_t(r, k) >= T) k_stop = min(k_stop, k);  // the front ray always advances
          if (k_stop <= k) {
            const float3 qa = fast_pos(r, sample_t(r, k_stop)), qb = fast_pos(r, sample_t(r, k));
            const int ca[3] = {int(qa.x), int(qa.y), int(qa.z)}, cb[3] = {int(qb.x), int(qb.y), int(qb.z)};
            const int mx[3] = {X1, Y1, Z1};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              lo[c] = clampi(min(ca[c], cb[c]), 0, mx[c]);
              hi[c] = clampi(max(ca[c], cb[c]) + 1, 0, mx[c]);
            }
          }
        }
        block_box(lo, hi, red);
        if (lo[0] > hi[0]) {
          // no samples in [T - dt, T): jump to the largest remaining sample
          T = block_max(k >= 0 ? sample_t(r, k) : -INFINITY, red);
          if (T == -INFINITY) break;
          continue;
        }
        w.x0 = lo[0];
        w.y0 = lo[1];
        w.z0 = lo[2] & ~3;
        w.nx = hi[0] - lo[0] + 1;
        w.ny = hi[1] - lo[1] + 1;
        w.nz = ((hi[2] | 3) - w.z0) + 1;
        w.vz0 = lo[2] & ~(kVtPerRow - 1);
        w.vnz = ((hi[2] | (kVtPerRow - 1)) - w.vz0) + 1;
        const bool fits = w.nx * w.ny * w.nz <= grad_cap && (!STAGE || w.nx * w.ny * w.vnz <= vol_cap);
        if (fits) {
          dt_used = dt;
          if (w.nx * w.ny * w.nz * 3 < grad_cap && dt < kWinMaxVoxels * vmin) dt *= 1.5f;  // next slab deeper
          break;
        }
        if (dt <= step_min) {
          direct = true;  // even one step's box is too large: global atomics for this slab
          dt_used = dt;
          break;
        }
        dt = fmaxf(dt * 0.5f, step_min);
      }
      if (T == -INFINITY) break;

      // stage the volume box (the gradient window is all zero here)
      if (STAGE && !direct) {
        const unsigned row_bytes = unsigned(w.vnz * sizeof(VT));
        if (threadIdx.x == 0) mbar_arrive_expect(bar, row_bytes * unsigned(w.nx * w.ny));
        __syncthreads();
        for (int row = threadIdx.x; row < w.nx * w.ny; row += blockDim.x) {
          const int ix = row / w.ny, iy = row - ix * w.ny;
          bulk_load(svol + row * w.vnz, vol.p + (w.x0 + ix) * vsx + (w.y0 + iy) * vsy + w.vz0, row_bytes, bar);
        }
        long long spins = 0;
        while (!mbar_try_wait(bar, phase)) {
          if (++spins > kWinSpinLimit) {
            failed = true;
            // wait once more, again bounded, for the copies still in flight
            for (long long again = 0; again < kWinSpinLimit && !mbar_try_wait(bar, phase); ++again) {
            }
            break;
          }
        }
        phase ^= 1u;
        if (__syncthreads_or(failed)) {
          failed = true;
          break;
        }
      }

      // reverse steps over this thread's samples of the slab
      const VT* sv = (STAGE && !direct) ? svol : nullptr;
      float* wv = direct ? nullptr : win;
      for (; k >= k_stop; --k) {
        const float2 rec = __ldg(drow + k);
        const float density = rec.x, alpha_in = rec.y;
        const float t = sample_t(r, k);
        const f4 cur = tf_eval<TF>(tf, density);
        const float alpha = blend_alpha<BLEND>(cur.w, r.step);
        f4 adj_cur;
        adj_step += blend_adjoint_core<BLEND>(alpha_in, cur, r.step, alpha, adj_acc, adj_cur);
        const float adj_density = tacc.adjoint(tf, density, adj_cur, s_grad_warp);
        const float3 q = fast_pos(r, t);
        const int ix = int(q.x), iy = int(q.y), iz = int(q.z);
        const float fx = q.x - float(ix), fy = q.y - float(iy), fz = q.z - float(iz);
        if (ix != vg.cx || iy != vg.cy || iz != vg.cz) {
          vg.flush(wv, w, adjv, a.adj_volume, X1, Y1, Z1);
          vg.cx = ix;
          vg.cy = iy;
          vg.cz = iz;
        }
        if (need_pos) {
          if (ix != scx || iy != scy || iz != scz) {
            win_corners<VT>(sv, w, vol, ix, iy, iz, d8);
            scx = ix;
            scy = iy;
            scz = iz;
          }
          f3 g;
          trilerp_grad(d8, fx, fy, fz, g);
          add_corner_weights(vg.g, adj_density, fx, fy, fz);
          const f3 adj_w = mk3(adj_density * g.x * r.inv_voxel.x, adj_density * g.y * r.inv_voxel.y,
                               adj_density * g.z * r.inv_voxel.z);
          adj_start.x += adj_w.x; adj_start.y += adj_w.y; adj_start.z += adj_w.z;
          adj_dir.x += adj_w.x * t; adj_dir.y += adj_w.y * t; adj_dir.z += adj_w.z * t;
          adj_step += dot3(adj_w, r.dir) * k;
        } else {
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
      vg.flush(wv, w, adjv, a.adj_volume, X1, Y1, Z1);
      scx = -1;  // the staged box changes with the slab

      const bool any_left = __syncthreads_or(k >= 0);
      if (!direct) {
        // the window's non-zero groups of 4 z-neighbours, one 16-byte vector
        // reduction each, and the window zeroed behind them
        const int nwin = w.nx * w.ny * w.nz;
        for (int e = threadIdx.x * 4; e < nwin; e += blockDim.x * 4) {
          float4* g4 = reinterpret_cast<float4*>(win + e);
          const float4 v = *g4;
          if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {
            const int row = e / w.nz, zz = e - row * w.nz;
            const int ix = row / w.ny, iy = row - ix * w.ny;
            atomicAdd(reinterpret_cast<float4*>(adjv + (w.x0 + ix) * gsx + (w.y0 + iy) * gsy + w.z0 + zz), v);
            *g4 = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
      }
      // the next slab starts where this one ended; the next box reduction
      // orders the zeroing above before any addition of the next slab
      T = any_left ? T - dt_used : -INFINITY;
    }
    if (failed) break;

    // per-ray outputs (rays handed to the general kernel write their own)
    if (valid && (drow || n_ray <= 0)) {
      if (a.has_stepsize) {
        float* ps =
            static_cast<float*>(a.adj_step.p) + b * a.adj_step.s[0] + y * a.adj_step.s[1] + x * a.adj_step.s[2];
        if (a.stepsize_broadcast) atomicAdd(ps, adj_step);
        else *ps = adj_step;
      }
      if (a.has_camera) {
        float* s0 = static_cast<float*>(a.adj_start.p) + b * a.adj_start.s[0] + y * a.adj_start.s[1] +
                    x * a.adj_start.s[2];
        float* d0 =
            static_cast<float*>(a.adj_dir.p) + b * a.adj_dir.s[0] + y * a.adj_dir.s[1] + x * a.adj_dir.s[2];
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
  }
  if (failed) {
    if (threadIdx.x == 0) atomicExch(counters + 3, 1);  // a bulk copy did not complete in time
    return;
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
}

}  // namespace dvr
