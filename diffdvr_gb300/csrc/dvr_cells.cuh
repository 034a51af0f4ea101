// Cell-corner volume: the eight corners of every trilinear cell stored
// together, so a sample reads its cell with one 16-byte load (two for FP32)
// instead of eight scattered element loads with their address arithmetic.
//
// Cell (x, y, z), x in [0, X-1], holds the voxels at x and min(x+1, X-1)
// (likewise y, z) in the corner order of VolumeFast::corners, i.e. exactly
// the clamped corners the reference's trilinear fetch reads for a sample in
// that cell (renderer/renderer_interpolation.cuh:179-253).  A sample at voxel
// coordinate q uses cell min(int(q), X-1) and the fractional part
// q - int(q) of the unclamped cell index, as the reference does; samples lie
// inside the box, so int(q) >= 0.  Built per forward call by one pass over the
// volume (V x 16 bytes written for BF16/FP16, V x 32 for FP32).
#pragma once
#include <type_traits>
#include "dvr_fast.cuh"

namespace dvr {

template <typename VT>
struct CellWords;  // raw storage of one cell
template <>
struct __align__(16) CellWords<__nv_bfloat16> {
  uint4 w;
};
template <>
struct __align__(16) CellWords<__half> {
  uint4 w;
};
template <>
struct __align__(16) CellWords<float> {
  float4 lo, hi;
};

__device__ __forceinline__ void unpack2(unsigned w, __nv_bfloat16*, float& a, float& b) {
  a = __uint_as_float(w << 16);
  b = __uint_as_float(w & 0xffff0000u);
}
__device__ __forceinline__ void unpack2(unsigned w, __half*, float& a, float& b) {
  const __half2 h = *reinterpret_cast<const __half2*>(&w);
  const float2 f = __half22float2(h);
  a = f.x;
  b = f.y;
}

template <typename VT>
__device__ __forceinline__ void cell_load(const CellWords<VT>* cells, size_t i, float* d) {
  if constexpr (sizeof(VT) == 4) {
    const float4 lo = __ldg(&cells[i].lo), hi = __ldg(&cells[i].hi);
    d[0] = lo.x; d[1] = lo.y; d[2] = lo.z; d[3] = lo.w;
    d[4] = hi.x; d[5] = hi.y; d[6] = hi.z; d[7] = hi.w;
  } else {
    const uint4 w = __ldg(&cells[i].w);
    unpack2(w.x, static_cast<VT*>(nullptr), d[0], d[1]);
    unpack2(w.y, static_cast<VT*>(nullptr), d[2], d[3]);
    unpack2(w.z, static_cast<VT*>(nullptr), d[4], d[5]);
    unpack2(w.w, static_cast<VT*>(nullptr), d[6], d[7]);
  }
}

// The cells of one volume batch entry.
template <typename VT>
struct CellVolume {
  const CellWords<VT>* cells;
  int X1, Y1, Z1;
  __device__ __forceinline__ float sample(float3 q) const {
    const int ix = int(q.x), iy = int(q.y), iz = int(q.z);
    const int cx = min(max(ix, 0), X1), cy = min(max(iy, 0), Y1), cz = min(max(iz, 0), Z1);
    float d[8];
    cell_load(cells, (size_t(cx) * (Y1 + 1) + cy) * (Z1 + 1) + cz, d);
    return trilerp(d, q.x - float(ix), q.y - float(iy), q.z - float(iz));
  }
};

template <typename T>
__device__ __forceinline__ unsigned short raw16(T v) {
  return *reinterpret_cast<const unsigned short*>(&v);
}

// One warp per (batch entry, x, y) row of cells, lanes along z: the row's
// index arithmetic is done once per warp, and the corner loads and the cell
// stores of a warp are contiguous in z.
template <typename VT>
__global__ void build_cells_kernel(const RenderParams p, int bv, CellWords<VT>* cells) {
  const int X = p.X, Y = p.Y, Z = p.Z;
  const int lane = threadIdx.x & 31;
  const int64_t rows = int64_t(bv) * X * Y;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  const int64_t sx = p.volume.s[1], sy = p.volume.s[2], sz = p.volume.s[3];
  for (int64_t row = blockIdx.x * int64_t(blockDim.x >> 5) + (threadIdx.x >> 5); row < rows; row += warps) {
    const int64_t bx = row / Y;
    const int y = int(row - bx * Y);
    const int b = int(bx / X), x = int(bx - int64_t(b) * X);
    const VT* v = static_cast<const VT*>(p.volume.p) + b * p.volume.s[0];
    const int hx = min(x + 1, X - 1), hy = min(y + 1, Y - 1);
    const VT* r00 = v + x * sx + y * sy;
    const VT* r01 = v + x * sx + hy * sy;
    const VT* r10 = v + hx * sx + y * sy;
    const VT* r11 = v + hx * sx + hy * sy;
    CellWords<VT>* dst = cells + row * Z;
    for (int z = lane; z < Z; z += 32) {
      const int hz = min(z + 1, Z - 1);
      const VT c[8] = {r00[z * sz], r00[hz * sz], r01[z * sz], r01[hz * sz],
                       r10[z * sz], r10[hz * sz], r11[z * sz], r11[hz * sz]};
      CellWords<VT> out;
      if constexpr (sizeof(VT) == 4) {
        out.lo = make_float4(c[0], c[1], c[2], c[3]);
        out.hi = make_float4(c[4], c[5], c[6], c[7]);
      } else {
        out.w = make_uint4(raw16(c[0]) | (unsigned(raw16(c[1])) << 16), raw16(c[2]) | (unsigned(raw16(c[3])) << 16),
                           raw16(c[4]) | (unsigned(raw16(c[5])) << 16), raw16(c[6]) | (unsigned(raw16(c[7])) << 16));
      }
      dst[z] = out;
    }
  }
}


// Gather texture: the volume's x slabs (Y x Z voxels of every volume batch
// entry) tiled into one 2D CUDA array created with the gather flag, each slab
// inside a one-texel apron that repeats its edge voxels.  Slab s sits at tile
// column s & (2^tshift - 1), tile row s >> tshift; voxel (y, z) of a slab at
// texel (1 + z, 1 + y) of its tile.  tex2Dgather returns the four texels of a
// 2x2 footprint, so a trilinear sample reads its eight corners with two
// texture instructions, one per slab, and no per-corner address arithmetic.
// With the slab index clamped to [0, X-1] and the footprint start clamped to
// [-1, size-1] (the apron), the texels read are exactly the clamped corners of
// VolumeFast::corners for every cell index (renderer/renderer_interpolation.cuh:193-207).
// Texture fetches clamp their coordinates to the array, so no index reads
// outside it.  Texels hold the stored values exactly (TexelFormat).
struct TexGather {
  cudaTextureObject_t tex;
  int tshift;  // tiles per texture row = 2^tshift
  int tw, th;  // tile size in texels: Z + 2, Y + 2
};

// How the gather texture holds a volume's values, exactly in every case:
//  kTexelF32:  32-bit float texels: FP32 volumes (and BF16 volumes widened,
//              a BF16 value being the upper half of its FP32 bits, when
//              kWideBf16Texels);
//  kTexelF16:  16-bit float texels, which the texture unit returns as FP32;
//  kTexelRaw16: the BF16 bits as 16-bit unsigned texels, widened in
//              registers.
// Widening BF16 saves the eight conversions per sample but doubles the
// texture's bytes, and measured slower (256^3 forward 0.69 -> 0.78 ms,
// 512^3 24.6 -> 25.8 ms), so BF16 volumes keep 16-bit texels.
enum { kTexelF32 = 0, kTexelF16 = 1, kTexelRaw16 = 2 };
constexpr bool kWideBf16Texels = false;
template <typename VT> struct TexelFormat;
template <> struct TexelFormat<float> {
  static constexpr int kind = kTexelF32;
  using T = float;
};
template <> struct TexelFormat<__half> {
  static constexpr int kind = kTexelF16;
  using T = unsigned short;
};
template <> struct TexelFormat<__nv_bfloat16> {
  static constexpr int kind = kWideBf16Texels ? kTexelF32 : kTexelRaw16;
  using T = typename std::conditional<kWideBf16Texels, float, unsigned short>::type;
};

// The four corners (y, z) of one slab in the corner order of
// VolumeFast::corners: (ly lz), (ly hz), (hy lz), (hy hz).  tex2Dgather
// returns the footprint counter-clockwise from the texel at (u0, v1):
// x = (u0, v1), y = (u1, v1), z = (u1, v0), w = (u0, v0).
template <typename VT>
__device__ __forceinline__ void gather_slab(cudaTextureObject_t tex, float u, float v, float* d) {
  if constexpr (TexelFormat<VT>::kind == kTexelRaw16) {
    const ushort4 g = tex2Dgather<ushort4>(tex, u, v, 0);
    d[0] = __uint_as_float(unsigned(g.w) << 16); d[1] = __uint_as_float(unsigned(g.z) << 16);
    d[2] = __uint_as_float(unsigned(g.x) << 16); d[3] = __uint_as_float(unsigned(g.y) << 16);
  } else {
    const float4 g = tex2Dgather<float4>(tex, u, v, 0);
    d[0] = g.w; d[1] = g.z; d[2] = g.x; d[3] = g.y;
  }
}

// The gather texture seen from one volume batch entry.
template <typename VT>
struct TexVolume {
  TexGather g;
  int s0;  // slab of x = 0 of this batch entry
  int X1, Y1, Z1;
  // Texture coordinate of the footprint whose first texel is (tile origin +
  // (cz2 - 1, cy2 - 1)): the texel corner between the four, exact in FP32
  // (integers below 2^23 converted with the 2^23 bias).
  __device__ __forceinline__ float2 coord(int x, int cz2, int cy2) const {
    const int s = s0 + x;
    const int iu = (s & ((1 << g.tshift) - 1)) * g.tw + cz2;
    const int iv = (s >> g.tshift) * g.th + cy2;
    return __fadd2_rn(make_float2(__int_as_float(iu + 0x4B000000), __int_as_float(iv + 0x4B000000)),
                      make_float2(-8388608.f, -8388608.f));
  }
  __device__ __forceinline__ void corners(int ix, int iy, int iz, float* d) const {
    const int lx = min(max(ix, 0), X1), hx = min(max(ix + 1, 0), X1);
    // footprint start in [-1, size-1]: texel 1 + start and the next one
    const int cy2 = min(max(iy, -1), Y1) + 2, cz2 = min(max(iz, -1), Z1) + 2;
    const float2 a = coord(lx, cz2, cy2), b = coord(hx, cz2, cy2);
    gather_slab<VT>(g.tex, a.x, a.y, d);
    gather_slab<VT>(g.tex, b.x, b.y, d + 4);
  }
  __device__ __forceinline__ float sample(float3 q) const {
    const int ix = int(q.x), iy = int(q.y), iz = int(q.z);
    float d[8];
    corners(ix, iy, iz, d);
    return trilerp(d, q.x - float(ix), q.y - float(iy), q.z - float(iz));
  }
};

// The volume as the general adjoint reads it: trilinear corners from the
// slab gather texture when the call built one (tex), else loaded directly;
// single voxels (nearest filtering) always directly.  Both give the same
// values.
template <typename VT>
struct AdjVolume {
  VolumeFast<VT> v;
  TexVolume<VT> t;
  bool tex;
  int X1, Y1, Z1;
  __device__ __forceinline__ AdjVolume(const VolumeFast<VT>& v_, const TexVolume<VT>& t_, bool tex_)
      : v(v_), t(t_), tex(tex_), X1(v_.X1), Y1(v_.Y1), Z1(v_.Z1) {}
  __device__ __forceinline__ float at(int x, int y, int z) const { return v.at(x, y, z); }
  __device__ __forceinline__ void corners(int ix, int iy, int iz, float* d) const {
    if (tex) t.corners(ix, iy, iz, d);
    else v.corners(ix, iy, iz, d);
  }
};

// The texel (u, v) of the tiled, aproned slab image: one warp per texel row
// of one tile (blockIdx.x = tile column, warps over texel rows), lanes along
// z, so the row's index arithmetic is done once per warp and the volume reads
// and texel writes of a warp are contiguous.  Texels of tiles past the last
// slab are zero.  put(u, v, texel) stores one texel.
template <typename VT, class Put>
__device__ __forceinline__ void gather_image_rows(const RenderParams& p, int bv, int tshift, int H, Put put) {
  using Texel = typename TexelFormat<VT>::T;
  const int X = p.X, Y = p.Y, Z = p.Z, tw = Z + 2, th = Y + 2;
  const int lane = threadIdx.x & 31;
  const int tc = blockIdx.x;
  const int64_t slabs = int64_t(X) * bv;
  for (int v = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5); v < H; v += gridDim.y * (blockDim.x >> 5)) {
    const int tr = v / th;
    const int64_t s = (int64_t(tr) << tshift) + tc;
    const int u0 = tc * tw;
    if (s >= slabs) {
      for (int u = lane; u < tw; u += 32) put(u0 + u, v, Texel(0));
      continue;
    }
    const int b = int(s / X), x = int(s - int64_t(b) * X);
    const int y = min(max(v - tr * th - 1, 0), Y - 1);
    const VT* src = static_cast<const VT*>(p.volume.p) + b * p.volume.s[0] + x * p.volume.s[1] + y * p.volume.s[2];
    const int64_t sz = p.volume.s[3];
    for (int u = lane; u < tw; u += 32) {
      const VT e = src[min(max(u - 1, 0), Z - 1) * sz];
      if constexpr (TexelFormat<VT>::kind == kTexelF32) put(u0 + u, v, Texel(float(e)));
      else put(u0 + u, v, Texel(raw16(e)));
    }
  }
}

// The slab image written to memory (W x H texels, row-major, pitch W), then
// copied into the texture's array.
template <typename VT>
__global__ void build_gather_image_kernel(const RenderParams p, int bv, int tshift, int W, int H,
                                          typename TexelFormat<VT>::T* out) {
  using Texel = typename TexelFormat<VT>::T;
  gather_image_rows<VT>(p, bv, tshift, H, [&](int u, int v, Texel t) { out[int64_t(v) * W + u] = t; });
}

// The slab image written straight into the texture's array by surface
// stores (u < W and v < H by construction; stores outside would be dropped).
template <typename VT>
__global__ void build_gather_surface_kernel(const RenderParams p, int bv, int tshift, int H,
                                            cudaSurfaceObject_t surf) {
  using Texel = typename TexelFormat<VT>::T;
  gather_image_rows<VT>(p, bv, tshift, H, [&](int u, int v, Texel t) {
    surf2Dwrite<Texel>(t, surf, u * int(sizeof(Texel)), v, cudaBoundaryModeZero);
  });
}

}  // namespace dvr
