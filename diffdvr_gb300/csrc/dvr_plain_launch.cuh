// Launch logic of the plain kernels for one TF mode (included by
// dvr_plain_tf*.cu).  Grid sizing follows the reference's occupancy-based
// choice (renderer/renderer_cuda.cpp:97-108, :273-307): a grid-stride loop
// over B*H*W with at most the resident number of blocks.
#pragma once
#include "dvr_kernels.h"
#include "dvr_plain.cuh"

namespace dvr {

template <typename K>
static int resident_grid(K kernel, int block, size_t smem, int64_t work, const LaunchInfo& li) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int64_t need = (work + block - 1) / block;
  const int64_t cap = int64_t(per_sm) * li.num_sms;
  return int(need < cap ? (need > 0 ? need : 1) : cap);
}

template <int TF>
cudaError_t launch_plain_forward(const RenderParams& p, int filter, int blend, const LaunchInfo& li,
                                 cudaStream_t s) {
  const int64_t work = int64_t(p.B) * p.H * p.W;
  if (work == 0) return cudaSuccess;
  const int block = 256;
  auto go = [&](auto kernel) {
    kernel<<<resident_grid(kernel, block, 0, work, li), block, 0, s>>>(p);
    return cudaGetLastError();
  };
  if (filter == kNearest) {
    return blend == kBeerLambert ? go(plain_forward_kernel<kNearest, TF, kBeerLambert>)
                                 : go(plain_forward_kernel<kNearest, TF, kAlphaBlend>);
  }
  return blend == kBeerLambert ? go(plain_forward_kernel<kTrilinear, TF, kBeerLambert>)
                               : go(plain_forward_kernel<kTrilinear, TF, kAlphaBlend>);
}

template <int FILTER, int TF, int BLEND>
static cudaError_t plain_adjoint_go(const RenderParams& p, const AdjointParams& a, const LaunchInfo& li,
                                    cudaStream_t s) {
  const int64_t work = int64_t(p.B) * p.H * p.W;
  constexpr int C = TfChannels<TF>::C;
  const bool volgrad = a.has_volume != 0, tfgrad = a.has_tf != 0;
  AdjointParams aa = a;
  int block = 256;
  size_t smem = 0;
  if (tfgrad && aa.tf_delayed) {
    // per-thread TF slots: pick the largest block whose slots fit
    const size_t per_thread = size_t(p.R) * C * sizeof(float);
    const size_t budget = size_t(li.max_smem_optin);
    while (block > 32 && per_thread * block > budget) block >>= 1;
    if (per_thread * block > budget) aa.tf_delayed = 0;  // too large: immediate atomics
    else smem = per_thread * block;
  }
  auto go = [&](auto kernel) {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e != cudaSuccess) return e;
    }
    kernel<<<resident_grid(kernel, block, smem, work, li), block, smem, s>>>(p, aa);
    return cudaGetLastError();
  };
  if (volgrad) {
    return tfgrad ? go(plain_adjoint_kernel<FILTER, TF, BLEND, true, true>)
                  : go(plain_adjoint_kernel<FILTER, TF, BLEND, true, false>);
  }
  return tfgrad ? go(plain_adjoint_kernel<FILTER, TF, BLEND, false, true>)
                : go(plain_adjoint_kernel<FILTER, TF, BLEND, false, false>);
}

template <int TF>
cudaError_t launch_plain_adjoint(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                 const LaunchInfo& li, cudaStream_t s) {
  if (int64_t(p.B) * p.H * p.W == 0) return cudaSuccess;
  if (filter == kNearest) {
    return blend == kBeerLambert ? plain_adjoint_go<kNearest, TF, kBeerLambert>(p, a, li, s)
                                 : plain_adjoint_go<kNearest, TF, kAlphaBlend>(p, a, li, s);
  }
  return blend == kBeerLambert ? plain_adjoint_go<kTrilinear, TF, kBeerLambert>(p, a, li, s)
                               : plain_adjoint_go<kTrilinear, TF, kAlphaBlend>(p, a, li, s);
}

}  // namespace dvr

#define DVR_INSTANTIATE_PLAIN(TF)                                                                           \
  template cudaError_t dvr::launch_plain_forward<TF>(const RenderParams&, int, int, const LaunchInfo&,     \
                                                     cudaStream_t);                                        \
  template cudaError_t dvr::launch_plain_adjoint<TF>(const RenderParams&, const AdjointParams&, int, int,  \
                                                     const LaunchInfo&, cudaStream_t);
