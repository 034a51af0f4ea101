// Launch logic of the optimized kernels for one TF mode and one volume
// storage type (included by dvr_fast_tf*_*.cu).  One block per 16x8 pixel
// tile; the hardware block scheduler balances tiles of unequal cost.
#pragma once
#include "dvr_fast.cuh"
#include "dvr_kernels.h"

namespace dvr {

template <int TF, typename VT>
cudaError_t launch_fast_forward_vt(const RenderParams& p, int filter, int blend, const LaunchInfo& li,
                                   cudaStream_t s);
template <int TF, typename VT>
cudaError_t launch_fast_adjoint_vt(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                   const LaunchInfo& li, cudaStream_t s);

template <int TF, typename VT>
cudaError_t launch_fast_forward_batched_vt(const RenderParams* table, const int4* items, int n_items, size_t smem,
                                           int filter, int blend, cudaStream_t s);
template <int TF, typename VT>
cudaError_t launch_fast_adjoint_batched_vt(const RenderParams* table, const AdjointParams* atable, const int4* items,
                                           int n_items, size_t smem, int filter, int blend, bool volgrad, bool tfgrad,
                                           cudaStream_t s);

#ifdef DVR_FAST_DEFINE
template <typename K>
static cudaError_t set_smem(K kernel, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  return cudaSuccess;
}

template <int TF, typename VT>
cudaError_t launch_fast_forward_batched_vt(const RenderParams* table, const int4* items, int n_items, size_t smem,
                                           int filter, int blend, cudaStream_t s) {
  if (n_items == 0) return cudaSuccess;
  auto go = [&](auto kernel) {
    cudaError_t e = set_smem(kernel, smem);
    if (e != cudaSuccess) return e;
    kernel<<<unsigned(n_items), kFastThreads, smem, s>>>(table, items);
    return cudaGetLastError();
  };
  if (filter == kNearest)
    return blend == kBeerLambert ? go(fast_forward_batched_kernel<kNearest, TF, kBeerLambert, VT>)
                                 : go(fast_forward_batched_kernel<kNearest, TF, kAlphaBlend, VT>);
  return blend == kBeerLambert ? go(fast_forward_batched_kernel<kTrilinear, TF, kBeerLambert, VT>)
                               : go(fast_forward_batched_kernel<kTrilinear, TF, kAlphaBlend, VT>);
}

template <int FILTER, int TF, int BLEND, typename VT>
static cudaError_t fast_adjoint_batched_go(const RenderParams* table, const AdjointParams* atable, const int4* items,
                                           int n_items, size_t smem, bool volgrad, bool tfgrad, cudaStream_t s) {
  auto go = [&](auto kernel) {
    cudaError_t e = set_smem(kernel, smem);
    if (e != cudaSuccess) return e;
    kernel<<<unsigned(n_items), kFastThreads, smem, s>>>(table, atable, items);
    return cudaGetLastError();
  };
  if (volgrad)
    return tfgrad ? go(fast_adjoint_batched_kernel<FILTER, TF, BLEND, true, true, VT>)
                  : go(fast_adjoint_batched_kernel<FILTER, TF, BLEND, true, false, VT>);
  return tfgrad ? go(fast_adjoint_batched_kernel<FILTER, TF, BLEND, false, true, VT>)
                : go(fast_adjoint_batched_kernel<FILTER, TF, BLEND, false, false, VT>);
}

template <int TF, typename VT>
cudaError_t launch_fast_adjoint_batched_vt(const RenderParams* table, const AdjointParams* atable, const int4* items,
                                           int n_items, size_t smem, int filter, int blend, bool volgrad, bool tfgrad,
                                           cudaStream_t s) {
  if (n_items == 0) return cudaSuccess;
  if (filter == kNearest)
    return blend == kBeerLambert
               ? fast_adjoint_batched_go<kNearest, TF, kBeerLambert, VT>(table, atable, items, n_items, smem, volgrad, tfgrad, s)
               : fast_adjoint_batched_go<kNearest, TF, kAlphaBlend, VT>(table, atable, items, n_items, smem, volgrad, tfgrad, s);
  return blend == kBeerLambert
             ? fast_adjoint_batched_go<kTrilinear, TF, kBeerLambert, VT>(table, atable, items, n_items, smem, volgrad, tfgrad, s)
             : fast_adjoint_batched_go<kTrilinear, TF, kAlphaBlend, VT>(table, atable, items, n_items, smem, volgrad, tfgrad, s);
}

template <int TF, typename VT>
cudaError_t launch_fast_forward_vt(const RenderParams& p, int filter, int blend, const LaunchInfo&,
                                   cudaStream_t s) {
  const int tiles_x = (p.W + kTileW - 1) / kTileW, tiles_y = (p.H + kTileH - 1) / kTileH;
  const int64_t blocks = int64_t(tiles_x) * tiles_y * p.B;
  if (blocks == 0) return cudaSuccess;
  if (blocks > 0x7fffffff) return cudaErrorInvalidConfiguration;
  const size_t smem = size_t(p.R) * p.C * sizeof(float);
  auto go = [&](auto kernel) {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e != cudaSuccess) return e;
    }
    kernel<<<unsigned(blocks), kFastThreads, smem, s>>>(p, tiles_x, tiles_y);
    return cudaGetLastError();
  };
  if (filter == kNearest)
    return blend == kBeerLambert ? go(fast_forward_kernel<kNearest, TF, kBeerLambert, VT>)
                                 : go(fast_forward_kernel<kNearest, TF, kAlphaBlend, VT>);
  return blend == kBeerLambert ? go(fast_forward_kernel<kTrilinear, TF, kBeerLambert, VT>)
                               : go(fast_forward_kernel<kTrilinear, TF, kAlphaBlend, VT>);
}

template <int FILTER, int TF, int BLEND, typename VT>
static cudaError_t fast_adjoint_go(const RenderParams& p, const AdjointParams& a, cudaStream_t s) {
  const int tiles_x = (p.W + kTileW - 1) / kTileW, tiles_y = (p.H + kTileH - 1) / kTileH;
  const int64_t blocks = int64_t(tiles_x) * tiles_y * p.B;
  if (blocks == 0) return cudaSuccess;
  if (blocks > 0x7fffffff) return cudaErrorInvalidConfiguration;
  constexpr int C = TfChannels<TF>::C;
  const bool tfgrad = a.has_tf != 0, volgrad = a.has_volume != 0;
  const size_t smem = fast_adjoint_smem(TF, p.R, C, tfgrad, p.ckpt.p ? p.ckpt_interval : 0);
  auto go = [&](auto kernel) {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e != cudaSuccess) return e;
    }
    kernel<<<unsigned(blocks), kFastThreads, smem, s>>>(p, a, tiles_x, tiles_y);
    return cudaGetLastError();
  };
  if (volgrad)
    return tfgrad ? go(fast_adjoint_kernel<FILTER, TF, BLEND, true, true, VT>)
                  : go(fast_adjoint_kernel<FILTER, TF, BLEND, true, false, VT>);
  return tfgrad ? go(fast_adjoint_kernel<FILTER, TF, BLEND, false, true, VT>)
                : go(fast_adjoint_kernel<FILTER, TF, BLEND, false, false, VT>);
}

template <int TF, typename VT>
cudaError_t launch_fast_adjoint_vt(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                   const LaunchInfo&, cudaStream_t s) {
  if (filter == kNearest)
    return blend == kBeerLambert ? fast_adjoint_go<kNearest, TF, kBeerLambert, VT>(p, a, s)
                                 : fast_adjoint_go<kNearest, TF, kAlphaBlend, VT>(p, a, s);
  return blend == kBeerLambert ? fast_adjoint_go<kTrilinear, TF, kBeerLambert, VT>(p, a, s)
                               : fast_adjoint_go<kTrilinear, TF, kAlphaBlend, VT>(p, a, s);
}
#endif

}  // namespace dvr

#define DVR_INSTANTIATE_FAST(TF, VT)                                                                        \
  template cudaError_t dvr::launch_fast_forward_vt<TF, VT>(const RenderParams&, int, int, const LaunchInfo&, \
                                                           cudaStream_t);                                    \
  template cudaError_t dvr::launch_fast_adjoint_vt<TF, VT>(const RenderParams&, const AdjointParams&, int, int, \
                                                           const LaunchInfo&, cudaStream_t);                 \
  template cudaError_t dvr::launch_fast_forward_batched_vt<TF, VT>(const RenderParams*, const int4*, int, size_t, \
                                                                   int, int, cudaStream_t);                  \
  template cudaError_t dvr::launch_fast_adjoint_batched_vt<TF, VT>(const RenderParams*, const AdjointParams*,  \
                                                                   const int4*, int, size_t, int, int, bool, bool, \
                                                                   cudaStream_t);
