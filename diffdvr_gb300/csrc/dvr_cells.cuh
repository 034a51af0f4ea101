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

// One thread per cell of every volume batch entry.
template <typename VT>
__global__ void build_cells_kernel(const RenderParams p, int bv, CellWords<VT>* cells) {
  const int X = p.X, Y = p.Y, Z = p.Z;
  const size_t V = size_t(X) * Y * Z;
  const size_t n = V * bv;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const int b = int(i / V);
    size_t r = i - size_t(b) * V;
    const int z = int(r % Z);
    r /= Z;
    const int y = int(r % Y), x = int(r / Y);
    const VT* v = static_cast<const VT*>(p.volume.p) + b * p.volume.s[0];
    const int64_t sx = p.volume.s[1], sy = p.volume.s[2], sz = p.volume.s[3];
    const int hx = min(x + 1, X - 1), hy = min(y + 1, Y - 1), hz = min(z + 1, Z - 1);
    const VT c[8] = {v[x * sx + y * sy + z * sz],   v[x * sx + y * sy + hz * sz],  v[x * sx + hy * sy + z * sz],
                     v[x * sx + hy * sy + hz * sz], v[hx * sx + y * sy + z * sz],  v[hx * sx + y * sy + hz * sz],
                     v[hx * sx + hy * sy + z * sz], v[hx * sx + hy * sy + hz * sz]};
    CellWords<VT> out;
    if constexpr (sizeof(VT) == 4) {
      out.lo = make_float4(c[0], c[1], c[2], c[3]);
      out.hi = make_float4(c[4], c[5], c[6], c[7]);
    } else {
      out.w = make_uint4(raw16(c[0]) | (unsigned(raw16(c[1])) << 16), raw16(c[2]) | (unsigned(raw16(c[3])) << 16),
                         raw16(c[4]) | (unsigned(raw16(c[5])) << 16), raw16(c[6]) | (unsigned(raw16(c[7])) << 16));
    }
    cells[i] = out;
  }
}

}  // namespace dvr
