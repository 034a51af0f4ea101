// Fold of the cell-corner volume gradient into the volume gradient.
//
// The general adjoint can accumulate its volume gradient per cell: the eight
// corner sums of cell (x, y, z) at AdjointParams::cell_grad[((x*Y + y)*Z +
// z)*8 + qx*4 + qy*2 + qz], in the corner order of the trilinear fetch
// (renderer/renderer_interpolation.cuh:193-207; corner (qx, qy, qz) of cell c
// is voxel min(c + q, size - 1) on every axis).  A cell's flush is then two
// aligned 16-byte reductions instead of four z-pair reductions on rows of
// arbitrary alignment.  This pass adds, for every voxel, the sums of the
// (cell, corner) pairs that name it: on each axis (c, 0) with c = v, (c, 1)
// with c = v - 1, and on the last voxel also (c, 1) with c = v (the clamped
// upper corner of the last cell).
#include <algorithm>
#include "dvr_kernels.h"

namespace dvr {
namespace {

// One warp per (volume batch entry, x, y) row of voxels, lanes along z.
__global__ void fold_cell_grad_kernel(const float* __restrict__ cg, OutView out, int X, int Y, int Z, int vb) {
  const int lane = threadIdx.x & 31;
  const int64_t rows = int64_t(vb) * X * Y;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  const size_t cells = size_t(X) * Y * Z;
  for (int64_t row = blockIdx.x * int64_t(blockDim.x >> 5) + (threadIdx.x >> 5); row < rows; row += warps) {
    const int64_t bx = row / Y;
    const int y = int(row - bx * Y);
    const int b = int(bx / X), x = int(bx - int64_t(b) * X);
    const float* c = cg + size_t(b) * cells * 8;
    // (cell, corner) pairs naming coordinate v of an axis of n voxels
    int ax[3], aq[3], na = 0, ay[3], aqy[3], nb = 0;
    ax[na] = x; aq[na++] = 0;
    if (x >= 1) { ax[na] = x - 1; aq[na++] = 1; }
    if (x == X - 1) { ax[na] = x; aq[na++] = 1; }
    ay[nb] = y; aqy[nb++] = 0;
    if (y >= 1) { ay[nb] = y - 1; aqy[nb++] = 1; }
    if (y == Y - 1) { ay[nb] = y; aqy[nb++] = 1; }
    float* dst = static_cast<float*>(out.p) + b * out.s[0] + x * out.s[1] + y * out.s[2];
    for (int z = lane; z < Z; z += 32) {
      float sum = 0.f;
      for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) {
          const float* cr = c + ((size_t(ax[i]) * Y + ay[j]) * Z) * 8 + aq[i] * 4 + aqy[j] * 2;
          sum += cr[size_t(z) * 8];                           // (z, 0)
          if (z >= 1) sum += cr[size_t(z - 1) * 8 + 1];       // (z - 1, 1)
          if (z == Z - 1) sum += cr[size_t(z) * 8 + 1];       // (z, 1), clamped
        }
      if (sum != 0.f) dst[z * out.s[3]] += sum;
    }
  }
}

}  // namespace

cudaError_t fold_cell_grad(const float* cell_grad, const OutView& adj_volume, int X, int Y, int Z, int vb,
                           const LaunchInfo& li, cudaStream_t s) {
  const int64_t rows = int64_t(vb) * X * Y;
  if (rows == 0) return cudaSuccess;
  const int blocks = int(std::min<int64_t>((rows + 7) / 8, int64_t(li.num_sms) * 32));
  fold_cell_grad_kernel<<<blocks, 256, 0, s>>>(cell_grad, adj_volume, X, Y, Z, vb);
  return cudaGetLastError();
}

}  // namespace dvr
