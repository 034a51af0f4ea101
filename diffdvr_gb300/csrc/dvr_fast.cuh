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
//  * TF gradients are accumulated per thread in registers (see TfGradAccum),
//    flushed to a per-warp copy in shared memory, and reduced into the output
//    with one global atomic per TF entry and block; the volume gradient keeps
//    the reference's per-cell register accumulation and issues its eight
//    corner reductions on cell exit.
//  * The step-size gradient is the full derivative (the reference keeps only
//    the last blend contribution, renderer/renderer_kernels.cuh:393-395).
#pragma once
#include "dvr_device.cuh"

namespace dvr {

constexpr int kFastThreads = 128;

// Batched launches carry their instance descriptors in the kernel parameter
// (up to 32 KB since CUDA 12.1), so a batched call needs no staging copy and
// no device workspace and can be captured into a CUDA graph.  One block per
// (instance, batch entry, tile) item; instances are ordered by decreasing
// cost and item_end[i] is the end of instance i's items.
constexpr int kBatchMax = 24;  // instances per launch: 24 * (752 + 400) B of descriptors fit

// Tile shapes of the batched launches: every warp covers an 8x4 pixel patch
// and the four warps of a block sit side by side in tile_warps_x(shape)
// columns (DvrTileShape): 16x8 (2 x 2 warps), 32x4 (4 x 1), 8x16 (1 x 4).
__host__ __device__ constexpr int tile_warps_x(int shape) { return shape == 1 ? 4 : (shape == 2 ? 1 : 2); }
__host__ __device__ constexpr int tile_w(int shape) { return 8 * tile_warps_x(shape); }
__host__ __device__ constexpr int tile_h(int shape) { return 4 * (4 / tile_warps_x(shape)); }

struct BatchForwardTable {
  int n;
  int item_end[kBatchMax];
  unsigned char shape[kBatchMax];  // tile shape of each instance
  RenderParams p[kBatchMax];
};
struct BatchAdjointTable {
  int n;
  int item_end[kBatchMax];
  unsigned char shape[kBatchMax];
  RenderParams p[kBatchMax];
  AdjointParams a[kBatchMax];
};
static_assert(sizeof(BatchAdjointTable) <= 32764, "kernel parameter limit");

__device__ __forceinline__ void batch_item(const int* item_end, const unsigned char* shapes, int n,
                                           const RenderParams* ps, int item, int& inst, int& b, int& tx, int& ty) {
  inst = 0;
  while (inst + 1 < n && item >= item_end[inst]) ++inst;
  const int local = item - (inst > 0 ? item_end[inst - 1] : 0);
  const int tw = tile_w(shapes[inst]), th = tile_h(shapes[inst]);
  const int tiles_x = (ps[inst].W + tw - 1) / tw, tiles_y = (ps[inst].H + th - 1) / th;
  const int per_b = tiles_x * tiles_y;
  b = local / per_b;
  const int r = local - b * per_b;
  ty = r / tiles_x;
  tx = r - ty * tiles_x;
}
constexpr int kMaxSegment = 64;  // largest checkpoint interval

// Maps thread -> pixel within a tile of the given shape: warp w covers an
// 8x4 patch, the warps sit in tile_warps_x(shape) columns.  Shape 0 is the
// 16x8 tile of the window kernel.
__device__ __forceinline__ void tile_pixel(int tid, int& px, int& py, int shape = 0) {
  const int w = tid >> 5, l = tid & 31, wx = tile_warps_x(shape);
  px = (w % wx) * 8 + (l & 7);
  py = (w / wx) * 4 + (l >> 3);
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
  f3 dir, voxel, inv_voxel;  // inv_voxel = 1 / voxel: position derivatives scale by it
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
  fr.inv_voxel = mk3(1.f / r.voxel.x, 1.f / r.voxel.y, 1.f / r.voxel.z);
}

__device__ __forceinline__ float3 fast_pos(const FastRay& r, float t) {
  const float2 xy = __ffma2_rn(make_float2(t, t), make_float2(r.dp.x, r.dp.y), make_float2(r.p0.x, r.p0.y));
  return make_float3(xy.x, xy.y, fmaf(t, r.dp.z, r.p0.z));
}

// Density at a position, with a one-cell cache (cx < 0: empty).
template <int FILTER, typename VT>
struct Sampler {
  int cx = -1, cy = -1, cz = -1;
  float d[8];
  float fx, fy, fz;
  // V: VolumeFast, or any accessor with at(), corners() and X1/Y1/Z1
  template <class V>
  __device__ __forceinline__ float sample(const V& v, float3 q) {
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
__device__ __forceinline__ void fast_forward_tile(const RenderParams& p, int b, int tx, int ty, float* s_tf,
                                                  int shape) {
  constexpr int C = TfChannels<TF>::C;
  int px, py;
  tile_pixel(threadIdx.x, px, py, shape);
  const int x = tx * tile_w(shape) + px, y = ty * tile_h(shape) + py;
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
  const int kmax = max_samples(r.tmin, r.tmax, r.step);
  // sample record: every ray owns a fixed run of the pool (pool / rays
  // groups of 4 floats, in pixel order), so no counter is needed; a ray
  // whose samples do not fit gets offset -1 and is re-marched by the adjoint
  float2* rec = nullptr;
  if (p.dens) {
    const int64_t rays = int64_t(p.B) * p.H * p.W;
    const int64_t cap = p.dens_units / rays;
    const int64_t g = ((int64_t(b) * p.H + y) * p.W + x) * cap;
    const bool fits = int64_t((kmax + 1) >> 1) <= cap && g <= 0x7fffffff;
    static_cast<int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] + x * p.dens_off.s[2]] =
        fits ? int(g) : -1;
    if (fits) rec = reinterpret_cast<float2*>(p.dens + 4 * g);
  }
  int k;
  for (k = 0; k < kmax; ++k) {
    const float t = r.tmin + k * r.step;
    if (t > r.tmax) break;
    if (acc.w > p.early_out) break;
    if (ck && k == next_ck) {  // opacity before sample k = (slot+1)*K
      if (slot < p.ckpt_slots) ck[slot * p.ckpt.s[3]] = acc.w;
      ++slot;
      next_ck += K;
    }
    const float density = smp.sample(vol, fast_pos(r, t));
    if (rec) rec[k] = make_float2(density, acc.w);
    acc = blend<BLEND>(acc, tf_eval<TF, true>(tf, density), r.step);
  }
  float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
  col[0] = acc.x;
  col[p.color.s[3]] = acc.y;
  col[2 * p.color.s[3]] = acc.z;
  col[3 * p.color.s[3]] = acc.w;
  static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = k;
}

// Batched variant: one block per work item (instance, batch entry, tile) of
// a list ordered by decreasing estimated cost; the instance descriptors live
// in device memory.
template <int FILTER, int TF, int BLEND, typename VT>
__global__ void __launch_bounds__(kFastThreads) fast_forward_batched_kernel(const __grid_constant__ BatchForwardTable t) {
  extern __shared__ float4 fast_smem4[];
  float* s_tf = reinterpret_cast<float*>(fast_smem4);
  int inst, b, tx, ty;
  batch_item(t.item_end, t.shape, t.n, t.p, int(blockIdx.x), inst, b, tx, ty);
  const RenderParams& p = t.p[inst];
  stage_tf(p, b, s_tf);
  __syncthreads();
  fast_forward_tile<FILTER, TF, BLEND, VT>(p, b, tx, ty, s_tf, t.shape[inst]);
}

// ----------------------------------------------------------------- adjoint
// TF-gradient accumulation.  Every adjoint sample adds to a few TF entries.
// Adding each one to shared memory with atomics makes the 32 lanes of a warp,
// whose rays see similar densities, collide on the same addresses, and float
// atomics on shared memory serialise on conflicts.  So every lane owns its
// accumulators and nothing is shared until the block ends:
//  * identity (2 entries) and Gaussian with R <= kGaussRegs: registers, stored
//    into the lane's shared-memory slots when the ray is done;
//  * texture / linear (and larger Gaussian TFs): registers for the two
//    control points of the current interval (PairCache), added when the
//    density leaves them into a private store of up to kLaneWin control
//    points per lane in shared memory, laid out [slot][lane] so the accesses
//    of a warp never share a bank.  For R <= kLaneWin it holds
//    the whole TF; else it is a circular window over the control points near
//    the current density, and a point that leaves the window (the density
//    drifted by more than kLaneWin points along the ray) is added to the
//    warp's shared copy.
// At the end of the block all lane stores and warp copies are summed per
// entry and added to the output with one global atomic per entry.
constexpr int kLaneWin = 16;   // window of the lane stores (power of two)
constexpr int kGaussRegs = 4;

// Shared-memory layout of the adjoint block (offsets in floats), computed
// identically on host and device.
struct AdjointSmem {
  int tf, warp, lane, lo, seg, total;
  int slots;  // control points per lane store
  __host__ __device__ static int slots_for(int tf_mode, int R) {
    if (tf_mode == kTfIdentity) return 1;
    return R <= kLaneWin ? R : kLaneWin;
  }
  __host__ __device__ AdjointSmem(int tf_mode, int R, int C, int threads, bool tfgrad, int seg_len,
                                  int tf_copies = 1) {
    int o = 0;
    tf = o;
    o += (tf_copies * R * C + 3) & ~3;
    slots = slots_for(tf_mode, R);
    warp = o;
    if (tfgrad) o += ((threads / 32) * R * C + 3) & ~3;
    lane = o;
    if (tfgrad) o += slots * C * threads;
    lo = o;
    if (tfgrad) o += threads;
    seg = o;
    o += 2 * seg_len * threads;
    total = o;
  }
};

// A lane's private accumulators: C channels per control point, stored
// [slot][lane] as float4 for channels 0-3 and [slot][k][lane] floats for the
// extra channels (linear: position; Gaussian: mean, sigma).
template <int C>
struct LaneStore {
  float* base;   // the block's lane-store region
  int T, tid;
  int slots;     // slots per lane
  int R;
  int lo = -1;   // first control point of the window; -1 = empty
  __device__ __forceinline__ float4* q(int slot) const { return reinterpret_cast<float4*>(base) + slot * T + tid; }
  __device__ __forceinline__ float* x(int slot, int k) const {
    return base + 4 * slots * T + (slot * (C - 4) + k) * T + tid;
  }
  __device__ __forceinline__ bool windowed() const { return R > slots; }
  __device__ __forceinline__ int slot_of(int t) const { return windowed() ? (t & (kLaneWin - 1)) : t; }
  __device__ __forceinline__ void clear(int s) {
    *q(s) = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (C > 4) {
#pragma unroll
      for (int k = 0; k < C - 4; ++k) *x(s, k) = 0.f;
    }
  }
  // where evicted control points go: the warp's dense R*C copy in shared
  // memory, or (per-batch TF gradients) the global output with its strides
  float* ev_base = nullptr;
  int64_t ev_sr = C, ev_sc = 1;
  __device__ __forceinline__ void add_to(float* g, int64_t sr, int64_t sc, int t, int s) const {
    const float4 v = *q(s);
    float* e = g + t * sr;
    if (v.x != 0.f) atomicAdd(e, v.x);
    if (v.y != 0.f) atomicAdd(e + sc, v.y);
    if (v.z != 0.f) atomicAdd(e + 2 * sc, v.z);
    if (v.w != 0.f) atomicAdd(e + 3 * sc, v.w);
    if constexpr (C > 4) {
#pragma unroll
      for (int k = 0; k < C - 4; ++k) {
        const float xv = *x(s, k);
        if (xv != 0.f) atomicAdd(e + (4 + k) * sc, xv);
      }
    }
  }
  __device__ __forceinline__ void evict(int t, float* warp_copy) {
    const int s = slot_of(t);
    if (t >= 0 && t < R) {
      if (ev_base) add_to(ev_base, ev_sr, ev_sc, t, s);
      else add_to(warp_copy, C, 1, t, s);
    }
    clear(s);
  }
  // adds every held control point to g (strides sr, sc) and empties the store
  __device__ __forceinline__ void flush_all(float* g, int64_t sr, int64_t sc) {
    if (windowed()) {
      if (lo >= 0) {
        for (int t = lo; t < lo + kLaneWin; ++t) {
          if (t < R) add_to(g, sr, sc, t, slot_of(t));
          clear(slot_of(t));
        }
      }
      lo = -1;
    } else {
      for (int t = 0; t < R; ++t) {
        add_to(g, sr, sc, t, t);
        clear(t);
      }
    }
  }
  // makes control points [t0, t1] resident (window mode only)
  __device__ __forceinline__ void ensure(int t0, int t1, float* warp_copy) {
    if (!windowed()) return;
    if (lo < 0) {
      lo = max(0, min(t0 - kLaneWin / 2, R - kLaneWin));
      return;
    }
    while (t1 >= lo + kLaneWin) {
      evict(lo, warp_copy);
      ++lo;
    }
    while (t0 < lo) {
      --lo;
      evict(lo + kLaneWin, warp_copy);
    }
  }
  __device__ __forceinline__ void add(int t, f4 v, float e0 = 0.f, float e1 = 0.f) {
    const int s = slot_of(t);
    float4* p = q(s);
    float4 a = *p;
    a.x += v.x;
    a.y += v.y;
    a.z += v.z;
    a.w += v.w;
    *p = a;
    if constexpr (C > 4) *x(s, 0) += e0;
    if constexpr (C > 5) *x(s, 1) += e1;
  }
  __device__ __forceinline__ int window_lo() const { return windowed() ? max(lo, 0) : 0; }
};

// Pair cache in front of a lane store: registers for the two control points
// of the current interval (i, i+1).  When the density crosses into the next
// or previous interval the point that leaves is added to the lane store and
// the other one shifts over; a larger jump flushes both.  Per sample this is
// a compare and 2*C FMAs.
template <int C>
struct PairCache {
  int i = -1;
  float a0[C], a1[C];
  __device__ __forceinline__ void put(LaneStore<C>& st, int t, const float* v, float* warp_copy) {
    if (t < 0 || t >= st.R) return;
    st.ensure(t, t, warp_copy);
    if constexpr (C == 4) st.add(t, mk4(v[0], v[1], v[2], v[3]));
    else st.add(t, mk4(v[0], v[1], v[2], v[3]), v[4]);
  }
  __device__ __forceinline__ void flush(LaneStore<C>& st, float* warp_copy) {
    if (i < 0) return;
    put(st, i, a0, warp_copy);
    put(st, i + 1, a1, warp_copy);
    i = -1;
  }
  // adds k0 * v (+ e0 on channel 4) to point i0 and k1 * v (+ e1) to point i1,
  // where i1 is i0 + 1 or, at the clamped ends of a texture TF, i0 itself
  __device__ __forceinline__ void add(int i0, int i1, f4 v, float k0, float k1, float e0, float e1,
                                      LaneStore<C>& st, float* warp_copy) {
    if (i0 != i) {
      if (i >= 0 && i0 == i + 1) {
        put(st, i, a0, warp_copy);
#pragma unroll
        for (int c = 0; c < C; ++c) { a0[c] = a1[c]; a1[c] = 0.f; }
      } else if (i >= 0 && i0 == i - 1) {
        put(st, i + 1, a1, warp_copy);
#pragma unroll
        for (int c = 0; c < C; ++c) { a1[c] = a0[c]; a0[c] = 0.f; }
      } else {
        flush(st, warp_copy);
#pragma unroll
        for (int c = 0; c < C; ++c) { a0[c] = 0.f; a1[c] = 0.f; }
      }
      i = i0;
    }
    const bool same = i1 == i0;
    const float q0 = same ? k0 + k1 : k0, q1 = same ? 0.f : k1;
    a0[0] += v.x * q0; a0[1] += v.y * q0; a0[2] += v.z * q0; a0[3] += v.w * q0;
    a1[0] += v.x * q1; a1[1] += v.y * q1; a1[2] += v.z * q1; a1[3] += v.w * q1;
    if constexpr (C == 5) {
      a0[4] += same ? e0 + e1 : e0;
      a1[4] += same ? 0.f : e1;
    }
  }
};

template <int TF, bool TFGRAD>
struct TfGradAccum;

template <bool TFGRAD>
struct TfGradAccum<kTfIdentity, TFGRAD> {
  float ga = 0.f, gc = 0.f;
  __device__ __forceinline__ void bind(float*, int, int, int, int) {}
  template <class A>
  __device__ __forceinline__ float adjoint(const A& tf, float density, f4 adj, float*) {
    const float dc = clampf(density, 0.f, 1.f);
    const float sa = tf.at(0, 0), sc = tf.at(0, 1);
    if constexpr (TFGRAD) {
      ga += adj.w * dc;
      gc += adj.x * dc + adj.y * dc + adj.z * dc;
    }
    const float adj_dc = (adj.x * sc + adj.y * sc + adj.z * sc) + adj.w * sa;
    return (density > 0 && density < 1) ? adj_dc : 0.f;
  }
  __device__ __forceinline__ void set_evict_target(float*, int64_t, int64_t) {}
  // adds the accumulated gradient to g (strides sr, sc) and restarts from zero
  __device__ __forceinline__ void flush_global(float* g, int64_t, int64_t sc, float*) {
    if constexpr (TFGRAD) {
      if (ga != 0.f) atomicAdd(g, ga);
      if (gc != 0.f) atomicAdd(g + sc, gc);
      ga = gc = 0.f;
    }
  }
  // identity lane store: 2 floats [channel][lane]
  __device__ __forceinline__ void finish(float* lane_base, int T, int tid, int* lo_out) {
    if constexpr (TFGRAD) {
      lane_base[tid] = ga;
      lane_base[T + tid] = gc;
      *lo_out = 0;
    }
  }
};

template <bool TFGRAD>
struct TfGradAccum<kTfTexture, TFGRAD> {
  LaneStore<4> st;
  PairCache<4> win;
  float* warp_copy = nullptr;
  __device__ __forceinline__ void bind(float* lane_base, int T, int tid, int slots, int R) {
    st.base = lane_base;
    st.T = T;
    st.tid = tid;
    st.slots = slots;
    st.R = R;
  }
  template <class A>
  __device__ __forceinline__ float adjoint(const A& tf, float density, f4 adj, float* wc) {
    const int R = tf.R;
    const float d = density * R - 0.5f;
    const int di = int(floorf(d));
    const float df = d - di;
    const int i0 = clampi(di, 0, R - 1), i1 = clampi(di + 1, 0, R - 1);
    const f4 a = tf.rgba(i0), c = tf.rgba(i1);
    if constexpr (TFGRAD) {
      warp_copy = wc;
      win.add(i0, i1, adj, 1 - df, df, 0.f, 0.f, st, wc);
    }
    return dot4(adj, mk4(c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w)) * R;
  }
  __device__ __forceinline__ void set_evict_target(float* base, int64_t sr, int64_t sc) {
    st.ev_base = base;
    st.ev_sr = sr;
    st.ev_sc = sc;
  }
  __device__ __forceinline__ void flush_global(float* g, int64_t sr, int64_t sc, float* wc) {
    if constexpr (TFGRAD) {
      win.flush(st, wc);
      st.flush_all(g, sr, sc);
    }
  }
  __device__ __forceinline__ void finish(float*, int, int, int* lo_out) {
    if constexpr (TFGRAD) {
      win.flush(st, warp_copy);
      *lo_out = st.window_lo();
    }
  }
};

template <bool TFGRAD>
struct TfGradAccum<kTfLinear, TFGRAD> {
  LaneStore<5> st;
  PairCache<5> win;
  float* warp_copy = nullptr;
  __device__ __forceinline__ void bind(float* lane_base, int T, int tid, int slots, int R) {
    st.base = lane_base;
    st.T = T;
    st.tid = tid;
    st.slots = slots;
    st.R = R;
  }
  template <class A>
  __device__ __forceinline__ float adjoint(const A& tf, float density, f4 adj, float* wc) {
    const int i = linear_interval(tf, density);
    const f4 a = tf.rgba(i), c = tf.rgba(i + 1);
    const float p0 = tf.at(i, 4), p1 = tf.at(i + 1, 4);
    const float d2 = clampf(density, p0, p1);
    const float fr = (d2 - p0) / (p1 - p0);
    const float adj_fr = dot4(adj, mk4(c.x - a.x, c.y - a.y, c.z - a.z, c.w - a.w));
    if constexpr (TFGRAD) {
      const float den = (p1 - p0) * (p1 - p0);
      warp_copy = wc;
      win.add(i, i + 1, adj, 1 - fr, fr, adj_fr * (d2 - p1) / den, adj_fr * (p0 - d2) / den, st, wc);
    }
    return adj_fr / (p1 - p0);
  }
  __device__ __forceinline__ void set_evict_target(float* base, int64_t sr, int64_t sc) {
    st.ev_base = base;
    st.ev_sr = sr;
    st.ev_sc = sc;
  }
  __device__ __forceinline__ void flush_global(float* g, int64_t sr, int64_t sc, float* wc) {
    if constexpr (TFGRAD) {
      win.flush(st, wc);
      st.flush_all(g, sr, sc);
    }
  }
  __device__ __forceinline__ void finish(float*, int, int, int* lo_out) {
    if constexpr (TFGRAD) {
      win.flush(st, warp_copy);
      *lo_out = st.window_lo();
    }
  }
};

template <bool TFGRAD>
struct TfGradAccum<kTfGaussian, TFGRAD> {
  float acc[kGaussRegs][6];
  LaneStore<6> st;
  bool regs = true;
  __device__ __forceinline__ void bind(float* lane_base, int T, int tid, int slots, int R) {
#pragma unroll
    for (int i = 0; i < kGaussRegs; ++i)
#pragma unroll
      for (int c = 0; c < 6; ++c) acc[i][c] = 0.f;
    regs = R <= kGaussRegs;
    st.base = lane_base;
    st.T = T;
    st.tid = tid;
    st.slots = slots;
    st.R = R;
  }
  template <class A>
  __device__ __forceinline__ float adjoint(const A& tf, float density, f4 adj, float* warp_copy) {
    float adj_density = 0;
    for (int i = 0; i < tf.R; ++i) {
      const f4 ci = tf.rgba(i);
      const float mu = tf.at(i, 4), sigma = tf.at(i, 5);
      const float s2 = sigma * sigma;
      const float ni = gauss(density, mu, sigma);
      const float f1 = (mu - density) / s2 * ni;
      const float d1 = dot4(adj, mk4(ci.x * f1, ci.y * f1, ci.z * f1, ci.w * f1));
      adj_density += d1;
      if constexpr (TFGRAD) {
        const float f2 = f1 * (mu - density) / sigma;
        const float gs = dot4(adj, mk4(ci.x * f2, ci.y * f2, ci.z * f2, ci.w * f2));
        const f4 gc = mk4(adj.x * ni, adj.y * ni, adj.z * ni, adj.w * ni);
        if (regs) {
#pragma unroll
          for (int r = 0; r < kGaussRegs; ++r) {
            if (r == i) {
              acc[r][0] += gc.x;
              acc[r][1] += gc.y;
              acc[r][2] += gc.z;
              acc[r][3] += gc.w;
              acc[r][4] += -d1;
              acc[r][5] += gs;
            }
          }
        } else {
          st.ensure(i, i, warp_copy);
          st.add(i, gc, -d1, gs);
        }
      }
    }
    return adj_density;
  }
  __device__ __forceinline__ void set_evict_target(float* base, int64_t sr, int64_t sc) {
    st.ev_base = base;
    st.ev_sr = sr;
    st.ev_sc = sc;
  }
  __device__ __forceinline__ void flush_global(float* g, int64_t sr, int64_t sc, float*) {
    if constexpr (TFGRAD) {
      if (regs) {
#pragma unroll
        for (int r = 0; r < kGaussRegs; ++r) {
          if (r < st.R) {
#pragma unroll
            for (int c = 0; c < 6; ++c) {
              if (acc[r][c] != 0.f) atomicAdd(g + r * sr + c * sc, acc[r][c]);
              acc[r][c] = 0.f;
            }
          }
        }
      } else {
        st.flush_all(g, sr, sc);
      }
    }
  }
  __device__ __forceinline__ void finish(float*, int, int, int* lo_out) {
    if constexpr (TFGRAD) {
      if (regs) {
#pragma unroll
        for (int r = 0; r < kGaussRegs; ++r) {
          if (r < st.R) {
            *st.q(r) = make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
            *st.x(r, 0) = acc[r][4];
            *st.x(r, 1) = acc[r][5];
          }
        }
      }
      *lo_out = st.window_lo();
    }
  }
};

// Sums the lane stores and warp copies of the block into the output TF
// gradient (one global atomic per entry).
template <int TF>
__device__ __forceinline__ void reduce_tf_grad(const AdjointSmem& L, const float* smem, int R, float* out,
                                               int64_t sb, int64_t sr, int64_t sc, int b,
                                               const float* extra = nullptr) {
  constexpr int C = TfChannels<TF>::C;
  const int T = blockDim.x;
  const int n = R * C;
  const float* lane = smem + L.lane;
  const int* lo = reinterpret_cast<const int*>(smem + L.lo);
  const float* warp = smem + L.warp;
  const bool window = TF != kTfIdentity && R > L.slots;
  for (int e = threadIdx.x; e < n; e += T) {
    const int t = e / C, c = e - t * C;
    float v = extra ? extra[e] : 0.f;
    for (int w = 0; w < T / 32; ++w) v += warp[w * n + e];
    if constexpr (TF == kTfIdentity) {
      for (int l = 0; l < T; ++l) v += lane[c * T + l];
    } else {
      const int slot = window ? (t & (kLaneWin - 1)) : t;
      for (int l = 0; l < T; ++l) {
        if (window) {
          const int l0 = lo[l];
          if (t < l0 || t >= l0 + kLaneWin) continue;
        }
        v += c < 4 ? lane[(slot * T + l) * 4 + c] : lane[4 * L.slots * T + (slot * (C - 4) + (c - 4)) * T + l];
      }
    }
    if (v != 0.f) atomicAdd(out + b * sb + t * sr + c * sc, v);
  }
}

// Volume-gradient accumulator for the current cell (reference scheme).
template <int FILTER, bool VOLGRAD>
struct VolGradCell {
  int cx = -1, cy = -1, cz = -1;
  float g[8];
  // the cell-corner gradient of this ray's volume batch entry
  // (AdjointParams::cell_grad), or nullptr
  float* cg = nullptr;
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
      } else if (cg) {
        // the cell's eight sums as two aligned 16-byte reductions; a cell
        // index above size - 1 (a sample within rounding of the far face)
        // has the same clamped corners as cell size - 1, which stands for it
        float* e = cg + ((size_t(clampi(cx, 0, X1)) * (Y1 + 1) + clampi(cy, 0, Y1)) * (Z1 + 1) + clampi(cz, 0, Z1)) * 8;
        atomicAdd(reinterpret_cast<float4*>(e), make_float4(g[0], g[1], g[2], g[3]));
        atomicAdd(reinterpret_cast<float4*>(e + 4), make_float4(g[4], g[5], g[6], g[7]));
      } else {
        const int lx = clampi(cx, 0, X1), hx = clampi(cx + 1, 0, X1);
        const int ly = clampi(cy, 0, Y1), hy = clampi(cy + 1, 0, Y1);
        const int lz = clampi(cz, 0, Z1), hz = clampi(cz + 1, 0, Z1);
        const bool pair = sz == 1 && hz == lz + 1;  // the two z corners are adjacent floats
        add_z(adjv + lx * sx + ly * sy, lz, hz, sz, pair, g[0], g[1]);
        add_z(adjv + lx * sx + hy * sy, lz, hz, sz, pair, g[2], g[3]);
        add_z(adjv + hx * sx + ly * sy, lz, hz, sz, pair, g[4], g[5]);
        add_z(adjv + hx * sx + hy * sy, lz, hz, sz, pair, g[6], g[7]);
      }
      reset();
    }
  }
  // adds u at z = lz and v at z = hz of one (x, y) row of the gradient: one
  // vector atomic when the two are adjacent floats inside an aligned 8- or
  // 16-byte block, else two scalar atomics
  __device__ __forceinline__ static void add_z(float* row, int lz, int hz, int64_t sz, bool pair, float u, float v) {
    float* e = row + lz * sz;
    const unsigned mis = static_cast<unsigned>(reinterpret_cast<uintptr_t>(e)) & 15u;
    if (pair && (mis & 7u) == 0u) {
      atomicAdd(reinterpret_cast<float2*>(e), make_float2(u, v));
    } else if (pair && mis == 4u) {
      atomicAdd(reinterpret_cast<float4*>(e - 1), make_float4(0.f, u, v, 0.f));
    } else {
      atomicAdd(e, u);
      atomicAdd(row + hz * sz, v);
    }
  }
};

// One reverse step shared by both adjoint variants.  Returns the step's
// position-chain contribution to d(loss)/d(step) via adj_step.
template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT, class A, class V>
__device__ __forceinline__ void fast_reverse_step(const RenderParams& p, const AdjointParams& a, const FastRay& r,
                                                  const V& vol, const A& tf,
                                                  TfGradAccum<TF, TFGRAD>& tacc, float* s_grad_warp,
                                                  Sampler<FILTER, VT>& smp, VolGradCell<FILTER, VOLGRAD>& vg,
                                                  float* adjv, int k, float density, float alpha_in, f4& adj_acc,
                                                  f3& adj_start, f3& adj_dir, float& adj_step, bool need_pos_grad) {
  const float t = r.tmin + k * r.step;
  const f4 cur = tf_eval<TF>(tf, density);
  const float alpha = blend_alpha<BLEND>(cur.w, r.step);
  f4 adj_cur;
  adj_step += blend_adjoint_core<BLEND>(alpha_in, cur, r.step, alpha, adj_acc, adj_cur);
  const float adj_density = tacc.adjoint(tf, density, adj_cur, s_grad_warp);
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
      // position derivative in difference form (the same derivative as the
      // reference's per-corner sums, renderer/renderer_interpolation.cuh:360-387,
      // in about half the instructions), scaled to world units
      f3 g;
      trilerp_grad(smp.d, fx, fy, fz, g);
      if constexpr (VOLGRAD) add_corner_weights(vg.g, adj_density, fx, fy, fz);
      const f3 adj_w = mk3(adj_density * g.x * r.inv_voxel.x, adj_density * g.y * r.inv_voxel.y,
                           adj_density * g.z * r.inv_voxel.z);
      adj_start.x += adj_w.x; adj_start.y += adj_w.y; adj_start.z += adj_w.z;
      adj_dir.x += adj_w.x * t; adj_dir.y += adj_w.y * t; adj_dir.z += adj_w.z * t;
      adj_step += dot3(adj_w, r.dir) * k;
    } else if constexpr (VOLGRAD) {
      add_corner_weights(vg.g, adj_density, fx, fy, fz);
    }
  }
}

template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT>
__device__ __forceinline__ void fast_adjoint_tile(const RenderParams& p, const AdjointParams& a, int b, int tx, int ty,
                                                  int shape, float* s_tf, float* s_grad, float* s_lane,
                                                  int s_lane_slots, int* s_lo, float* s_seg) {
  constexpr int C = TfChannels<TF>::C;
  constexpr unsigned kFull = 0xffffffffu;
  int px, py;
  tile_pixel(threadIdx.x, px, py, shape);
  const int x = tx * tile_w(shape) + px, y = ty * tile_h(shape) + py;
  // every lane stays in the loops below (pixels outside the image have no
  // samples) so that the warp can reconverge explicitly after each step
  const bool valid = x < p.W && y < p.H;
  FastRay r{};
  if (valid) fast_setup(p, x, y, b, r);
  VolumeFast<VT> vol{static_cast<const VT*>(p.volume.p) + b * p.volume.s[0], int(p.volume.s[1]), int(p.volume.s[2]),
                     int(p.volume.s[3]), p.X - 1, p.Y - 1, p.Z - 1};
  const TfShared<C> tf{s_tf, p.R};
  float* s_grad_warp = s_grad + (threadIdx.x >> 5) * p.R * C;
  TfGradAccum<TF, TFGRAD> tacc;
  tacc.bind(s_lane, int(blockDim.x), int(threadIdx.x), s_lane_slots, p.R);
  float* adjv = VOLGRAD ? static_cast<float*>(a.adj_volume.p) + b * a.adj_volume.s[0] : nullptr;
  const bool need_pos = a.has_camera || a.has_stepsize;

  int n = 0;
  f4 adj_acc = mk4(0, 0, 0, 0);
  if (valid) {
    n = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
    n = min(n, max_samples(r.tmin, r.tmax, r.step));
    const float* ac = static_cast<const float*>(a.adj_color.p) + b * a.adj_color.s[0] + y * a.adj_color.s[1] +
                      x * a.adj_color.s[2];
    adj_acc = mk4(ac[0], ac[a.adj_color.s[3]], ac[2 * a.adj_color.s[3]], ac[3 * a.adj_color.s[3]]);
  }
  float adj_step = 0;
  f3 adj_start = mk3(0, 0, 0), adj_dir = mk3(0, 0, 0);
  Sampler<FILTER, VT> smp;
  VolGradCell<FILTER, VOLGRAD> vg;
  vg.reset();

  const int K = p.ckpt_interval;
  const bool ckpt_ok = valid && p.ckpt.p != nullptr && n <= (p.ckpt_slots + 1) * K;
  // checkpointed rays: segments [jK, (j+1)K) from last to first, all lanes on
  // the same segment index and sample offset (predicated per lane)
  const int nseg = ckpt_ok ? (n + K - 1) / K : 0;
  const int nseg_max = int(__reduce_max_sync(kFull, unsigned(nseg)));
  const float* ck = ckpt_ok ? static_cast<const float*>(p.ckpt.p) + b * p.ckpt.s[0] + y * p.ckpt.s[1] +
                                  x * p.ckpt.s[2]
                            : nullptr;
  float* seg_d = s_seg + threadIdx.x;  // [offset][thread]
  float* seg_a = s_seg + K * blockDim.x + threadIdx.x;
  // the forward's sample record, when the ray has one: density and incoming
  // opacity of every sample, no re-march
  const float2* drow = nullptr;
  if (ckpt_ok && p.dens) {
    const int g = static_cast<const int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] +
                                                        x * p.dens_off.s[2]];
    if (g >= 0 && int64_t(g) + ((n + 1) >> 1) <= p.dens_units)
      drow = reinterpret_cast<const float2*>(p.dens + 4 * size_t(g));
  }
  for (int j = nseg_max - 1; j >= 0; --j) {
    const int k0 = j * K;
    const int k1 = j < nseg ? min(n, k0 + K) : k0;
    // re-march the segment from its checkpoint, or read it from the record
    float alpha = (j > 0 && j < nseg && !drow) ? ck[(j - 1) * p.ckpt.s[3]] : 0.f;
    for (int kk = 0; kk < K; ++kk) {
      const int k = k0 + kk;
      if (k < k1) {
        if (drow) {
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
      __syncwarp();
    }
    for (int kk = K - 1; kk >= 0; --kk) {
      const int k = k0 + kk;
      if (k < k1) {
        const float density = seg_d[kk * blockDim.x];
        const float alpha_in = seg_a[kk * blockDim.x];
        fast_reverse_step<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, r, vol, tf, tacc, s_grad_warp, smp, vg, adjv,
                                                                  k, density, alpha_in, adj_acc, adj_start, adj_dir,
                                                                  adj_step, need_pos);
      }
      __syncwarp();
    }
  }
  // rays without checkpoints: recover the accumulator by inverting the blend,
  // as the reference
  const int ninv = (valid && !ckpt_ok) ? n : 0;
  const int ninv_max = int(__reduce_max_sync(kFull, unsigned(ninv)));
  if (ninv_max > 0) {
    float alpha_out = 0.f;
    if (ninv > 0) {
      const float* fc = static_cast<const float*>(a.fwd_color.p) + b * a.fwd_color.s[0] + y * a.fwd_color.s[1] +
                        x * a.fwd_color.s[2];
      alpha_out = fc[3 * a.fwd_color.s[3]];
    }
    for (int k = ninv_max - 1; k >= 0; --k) {
      if (k < ninv) {
        const float t = r.tmin + k * r.step;
        const float density = smp.sample(vol, fast_pos(r, t));
        const float a_k = blend_alpha<BLEND>(tf_eval<TF>(tf, density).w, r.step);
        const float a_inv = BLEND == kAlphaBlend ? rminf(1.0f - 1e-5f, a_k) : a_k;
        const float alpha_in = (a_inv - alpha_out) / (a_inv - 1);
        fast_reverse_step<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, r, vol, tf, tacc, s_grad_warp, smp, vg, adjv,
                                                                  k, density, alpha_in, adj_acc, adj_start, adj_dir,
                                                                  adj_step, need_pos);
        alpha_out = alpha_in;
      }
      __syncwarp();
    }
  }
  vg.flush(adjv, a.adj_volume, p.X - 1, p.Y - 1, p.Z - 1);
  tacc.finish(s_lane, int(blockDim.x), int(threadIdx.x), s_lo + threadIdx.x);
  if (!valid) return;

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

// Shared memory of the adjoint block, in bytes.
__host__ __device__ inline size_t fast_adjoint_smem(int tf_mode, int R, int C, bool tfgrad, int seg_len) {
  return size_t(AdjointSmem(tf_mode, R, C, kFastThreads, tfgrad, seg_len).total) * sizeof(float);
}

template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT>
__device__ __forceinline__ void fast_adjoint_block(const RenderParams& p, const AdjointParams& a, int b, int tx,
                                                   int ty, int shape) {
  extern __shared__ float4 fast_smem4[];
  constexpr int C = TfChannels<TF>::C;
  float* smem = reinterpret_cast<float*>(fast_smem4);
  const int seg_len = p.ckpt.p ? p.ckpt_interval : 0;
  const AdjointSmem L(TF, p.R, C, int(blockDim.x), TFGRAD, seg_len);
  float* s_grad = smem + L.warp;
  stage_tf(p, b, smem + L.tf);
  if constexpr (TFGRAD) {
    // warp copies, lane stores and window bases start at zero
    for (int e = threadIdx.x; e < L.seg - L.warp; e += blockDim.x) s_grad[e] = 0.f;
  }
  __syncthreads();
  fast_adjoint_tile<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(p, a, b, tx, ty, shape, smem + L.tf, s_grad, smem + L.lane,
                                                            L.slots, reinterpret_cast<int*>(smem + L.lo),
                                                            smem + L.seg);
  if constexpr (TFGRAD) {
    __syncthreads();
    reduce_tf_grad<TF>(L, smem, p.R, static_cast<float*>(a.adj_tf.p), a.adj_tf.s[0], a.adj_tf.s[1], a.adj_tf.s[2],
                       b);
  }
}

template <int FILTER, int TF, int BLEND, bool VOLGRAD, bool TFGRAD, typename VT>
__global__ void __launch_bounds__(kFastThreads) fast_adjoint_batched_kernel(const __grid_constant__ BatchAdjointTable t) {
  int inst, b, tx, ty;
  batch_item(t.item_end, t.shape, t.n, t.p, int(blockIdx.x), inst, b, tx, ty);
  fast_adjoint_block<FILTER, TF, BLEND, VOLGRAD, TFGRAD, VT>(t.p[inst], t.a[inst], b, tx, ty, t.shape[inst]);
}

}  // namespace dvr
