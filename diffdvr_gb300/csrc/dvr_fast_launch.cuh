// Launch logic of the optimized kernels for one TF mode and one volume
// storage type (included by dvr_fast_tf*_*.cu).  Single-instance calls use
// the persistent kernels (dvr_persist.cuh) with a work counter from the
// library's pool; batched calls launch one block per (instance, batch entry,
// tile) work item.
#pragma once
#include "dvr_record.cuh"
#include "dvr_warpray.cuh"
#include "dvr_window.cuh"
#include "dvr_kernels.h"

namespace dvr {

template <int TF, typename VT>
cudaError_t launch_fast_forward_vt(const RenderParams& p, int filter, int blend, const LaunchInfo& li,
                                   cudaStream_t s);
template <int TF, typename VT>
cudaError_t launch_fast_adjoint_vt(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                   const LaunchInfo& li, cudaStream_t s);

template <int TF, typename VT>
cudaError_t launch_fast_forward_batched_vt(const BatchForwardTable& t, int n_items, size_t smem, int filter, int blend,
                                           cudaStream_t s);
template <int TF, typename VT>
cudaError_t launch_fast_adjoint_batched_vt(const BatchAdjointTable& t, int n_items, size_t smem, int filter, int blend,
                                           bool volgrad, bool tfgrad, cudaStream_t s);
template <int TF, typename VT>
cudaError_t launch_fast_adjoint_into_vt(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                        const LaunchInfo& li, const CallerScratch& sc, cudaStream_t s);

#ifdef DVR_FAST_DEFINE
template <typename K>
static cudaError_t set_smem(K kernel, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  return cudaSuccess;
}

template <int TF, typename VT>
cudaError_t launch_fast_forward_batched_vt(const BatchForwardTable& t, int n_items, size_t smem, int filter, int blend,
                                           cudaStream_t s) {
  if (n_items == 0) return cudaSuccess;
  auto go = [&](auto kernel) {
    cudaError_t e = set_smem(kernel, smem);
    if (e != cudaSuccess) return e;
    kernel<<<unsigned(n_items), kFastThreads, smem, s>>>(t);
    return cudaGetLastError();
  };
  if (filter == kNearest)
    return blend == kBeerLambert ? go(fast_forward_batched_kernel<kNearest, TF, kBeerLambert, VT>)
                                 : go(fast_forward_batched_kernel<kNearest, TF, kAlphaBlend, VT>);
  return blend == kBeerLambert ? go(fast_forward_batched_kernel<kTrilinear, TF, kBeerLambert, VT>)
                               : go(fast_forward_batched_kernel<kTrilinear, TF, kAlphaBlend, VT>);
}

template <int FILTER, int TF, int BLEND, typename VT>
static cudaError_t fast_adjoint_batched_go(const BatchAdjointTable& t, int n_items, size_t smem, bool volgrad,
                                           bool tfgrad, cudaStream_t s) {
  auto go = [&](auto kernel) {
    cudaError_t e = set_smem(kernel, smem);
    if (e != cudaSuccess) return e;
    kernel<<<unsigned(n_items), kFastThreads, smem, s>>>(t);
    return cudaGetLastError();
  };
  if (volgrad)
    return tfgrad ? go(fast_adjoint_batched_kernel<FILTER, TF, BLEND, true, true, VT>)
                  : go(fast_adjoint_batched_kernel<FILTER, TF, BLEND, true, false, VT>);
  return tfgrad ? go(fast_adjoint_batched_kernel<FILTER, TF, BLEND, false, true, VT>)
                : go(fast_adjoint_batched_kernel<FILTER, TF, BLEND, false, false, VT>);
}

template <int TF, typename VT>
cudaError_t launch_fast_adjoint_batched_vt(const BatchAdjointTable& t, int n_items, size_t smem, int filter, int blend,
                                           bool volgrad, bool tfgrad, cudaStream_t s) {
  if (n_items == 0) return cudaSuccess;
  if (filter == kNearest)
    return blend == kBeerLambert
               ? fast_adjoint_batched_go<kNearest, TF, kBeerLambert, VT>(t, n_items, smem, volgrad, tfgrad, s)
               : fast_adjoint_batched_go<kNearest, TF, kAlphaBlend, VT>(t, n_items, smem, volgrad, tfgrad, s);
  return blend == kBeerLambert
             ? fast_adjoint_batched_go<kTrilinear, TF, kBeerLambert, VT>(t, n_items, smem, volgrad, tfgrad, s)
             : fast_adjoint_batched_go<kTrilinear, TF, kAlphaBlend, VT>(t, n_items, smem, volgrad, tfgrad, s);
}

// Grid of a persistent launch: every resident block slot, but no more
// blocks than 128-ray groups of work.
template <typename K>
static int persistent_grid(K kernel, size_t smem, int64_t rays, const LaunchInfo& li) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kFastThreads, smem) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int64_t need = (rays + kFastThreads - 1) / kFastThreads;
  const int64_t cap = int64_t(per_sm) * li.num_sms;
  return int(need < cap ? (need > 0 ? need : 1) : cap);
}

// Largest cell-corner volume gradient (8 floats per cell and volume batch
// entry) the general adjoint accumulates into: it must stay in L2 beside the
// volume and the sample record's stream.
constexpr size_t kCellGradMaxBytes = size_t(80) << 20;

// Volume batch entries of a call (1 for a broadcast volume).
static inline int volume_entries(const RenderParams& p) { return p.volume.s[0] != 0 ? p.B : 1; }

// Whether a trilinear call reads its corners from the slab gather texture
// (DvrForwardGather): TEXTURE, or AUTO with cell records larger than 64 MB
// (smaller ones stay in L2 and are read as cells by the forward).
template <typename VT>
static bool texture_gather_wanted(const RenderParams& p) {
  const int mode = forward_gather_mode();
  const size_t cell_bytes = size_t(p.X) * p.Y * p.Z * volume_entries(p) * sizeof(CellWords<VT>);
  return mode == DVR_GATHER_TEXTURE || (mode == DVR_GATHER_AUTO && cell_bytes > (size_t(64) << 20));
}

// Builds the slab gather texture of the volume (TexGather): the tiled,
// aproned slab image is written to scratch and copied into the texture's
// array.  cudaErrorNotSupported when the slabs exceed the gather texture's
// size limits (the caller then reads the volume directly).
template <typename VT>
static cudaError_t build_gather_texture(const RenderParams& p, int bv, const LaunchInfo& li, cudaStream_t s,
                                        TexGather& tg) {
  int max_w = 0, max_h = 0;
  cudaError_t err = cudaDeviceGetAttribute(&max_w, cudaDevAttrMaxTexture2DGatherWidth, li.device);
  if (err != cudaSuccess) return err;
  err = cudaDeviceGetAttribute(&max_h, cudaDevAttrMaxTexture2DGatherHeight, li.device);
  if (err != cudaSuccess) return err;
  const int64_t slabs = int64_t(p.X) * bv, tw = p.Z + 2, th = p.Y + 2;
  int shift = 0;
  while (shift < 16 && ((slabs + (int64_t(1) << shift) - 1) >> shift) * th > max_h) ++shift;
  const int64_t per_row = std::min<int64_t>(int64_t(1) << shift, slabs);
  const int64_t W = per_row * tw, H = ((slabs + (int64_t(1) << shift) - 1) >> shift) * th;
  if (W > max_w || H > max_h) return cudaErrorNotSupported;
  using Texel = typename TexelFormat<VT>::T;
  constexpr int bytes = int(sizeof(Texel));
  cudaArray_t array = nullptr;
  cudaSurfaceObject_t surf = 0;
  err = acquire_gather_texture(li.device, s, int(W), int(H), TexelFormat<VT>::kind, array, tg.tex, surf);
  if (err != cudaSuccess) return err;
  // a block per tile column and 8 texel rows (one per warp)
  const dim3 grid(unsigned(per_row), unsigned(std::min<int64_t>((H + 7) / 8, 65535)));
  if (surf) {
    build_gather_surface_kernel<VT><<<grid, 256, 0, s>>>(p, bv, shift, int(H), surf);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  } else {
    auto* image = static_cast<Texel*>(acquire_scratch(li.device, s, size_t(W) * H * bytes, err, 1));
    if (!image) return err;
    build_gather_image_kernel<VT><<<grid, 256, 0, s>>>(p, bv, shift, int(W), int(H), image);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    err = cudaMemcpy2DToArrayAsync(array, 0, 0, image, size_t(W) * bytes, size_t(W) * bytes, size_t(H),
                                   cudaMemcpyDeviceToDevice, s);
    if (err != cudaSuccess) return err;
  }
  tg.tshift = shift;
  tg.tw = int(tw);
  tg.th = int(th);
  return cudaSuccess;
}

template <int TF, typename VT>
cudaError_t launch_fast_forward_vt(const RenderParams& p, int filter, int blend, const LaunchInfo& li,
                                   cudaStream_t s) {
  const RayOrder order = RayOrder::make(p.W, p.H, p.B);
  if (order.total() == 0) return cudaSuccess;
  if (order.total() > 0x7fffffff) return cudaErrorInvalidConfiguration;
  const int copies = p.tf.s[0] == 0 ? 1 : p.B;
  const size_t smem = size_t(copies) * p.R * p.C * sizeof(float);
  if (smem > size_t(li.max_smem_optin)) return cudaErrorInvalidConfiguration;
  cudaError_t err;
  int* counter = acquire_counter(li.device, s, err);
  if (!counter) return err;
  int* order_ints = static_cast<int*>(acquire_scratch(li.device, s, work_order_ints(p) * sizeof(int), err));
  if (!order_ints) return err;
  err = order_rays_by_work(p, nullptr, order_ints, li, s);
  if (err != cudaSuccess) return err;
  // Trilinear corners (DvrForwardGather).  AUTO: the cell-corner volume when
  // the cells fit in L2 with room to spare (64 MB of its 129 MB); else the
  // slab gather texture; where the slabs exceed the texture's size limits,
  // the cell-corner volume when the volume itself is too large for L2 (one
  // 16-byte sector per sample then replaces about four), else direct loads.
  // Measured forward (GB300, BF16): 128^3 cells 1.85 ms, texture 1.92 (64
  // views of 256^2); 256^3 texture 0.75 ms, direct 0.80, cells 0.82 (8 views
  // of 256^2); 512^3 texture 25.1 ms, cells 27.8 (16 views of 1024^2).
  const CellWords<VT>* cells = nullptr;
  TexGather tg{};
  int gather = kGatherDirect;
  if (filter != kNearest) {
    const int mode = forward_gather_mode();
    const int bv = p.volume.s[0] != 0 ? p.B : 1;
    const size_t n = size_t(p.X) * p.Y * p.Z * bv;
    const size_t cell_bytes = n * sizeof(CellWords<VT>), raw_bytes = n * sizeof(VT);
    const bool cells_in_l2 = cell_bytes <= (size_t(64) << 20);
    if (texture_gather_wanted<VT>(p)) {
      err = build_gather_texture<VT>(p, bv, li, s, tg);
      if (err == cudaSuccess) gather = kGatherTexture;
      else if (err != cudaErrorNotSupported) return err;
    }
    const bool cells_auto =
        cells_in_l2 || (raw_bytes > (size_t(64) << 20) && cell_bytes <= (size_t(8) << 30));
    if (gather == kGatherDirect && (mode == DVR_GATHER_CELLS || (mode != DVR_GATHER_DIRECT && cells_auto))) {
      auto* c = static_cast<CellWords<VT>*>(acquire_scratch(li.device, s, cell_bytes, err, 1));
      if (!c) return err;
      // one warp per row of Z cells, 8 rows per block
      const int blocks = int(std::min<size_t>((n / p.Z + 7) / 8, size_t(li.num_sms) * 32));
      build_cells_kernel<VT><<<blocks, 256, 0, s>>>(p, bv, c);
      err = cudaGetLastError();
      if (err != cudaSuccess) return err;
      cells = c;
      gather = kGatherCells;
    }
  }
  auto go = [&](auto kernel) {
    cudaError_t e = set_smem(kernel, smem);
    if (e != cudaSuccess) return e;
    // one warp per ray: as many warps as fit, up to one per ray
    kernel<<<persistent_grid(kernel, smem, order.total() * 32, li), kFastThreads, smem, s>>>(
        p, order, counter, order_ints + work_order_list_offset, order_ints + work_order_count_offset, cells, tg);
    return cudaGetLastError();
  };
  if (filter == kNearest)
    return blend == kBeerLambert ? go(fast_forward_warp_kernel<kNearest, TF, kBeerLambert, VT, kGatherDirect>)
                                 : go(fast_forward_warp_kernel<kNearest, TF, kAlphaBlend, VT, kGatherDirect>);
  if (gather == kGatherCells)
    return blend == kBeerLambert ? go(fast_forward_warp_kernel<kTrilinear, TF, kBeerLambert, VT, kGatherCells>)
                                 : go(fast_forward_warp_kernel<kTrilinear, TF, kAlphaBlend, VT, kGatherCells>);
  if (gather == kGatherTexture)
    return blend == kBeerLambert ? go(fast_forward_warp_kernel<kTrilinear, TF, kBeerLambert, VT, kGatherTexture>)
                                 : go(fast_forward_warp_kernel<kTrilinear, TF, kAlphaBlend, VT, kGatherTexture>);
  return blend == kBeerLambert ? go(fast_forward_warp_kernel<kTrilinear, TF, kBeerLambert, VT, kGatherDirect>)
                               : go(fast_forward_warp_kernel<kTrilinear, TF, kAlphaBlend, VT, kGatherDirect>);
}

// TF-gradient-only adjoint of a texture TF from the sample-density record:
// longest-first order, the record kernel, then the general kernel over the
// rays the record does not cover (usually none; a small grid).
template <int FILTER, int BLEND, typename VT>
static cudaError_t fast_adjoint_record_go(const RenderParams& p, const AdjointParams& a, const RayOrder& order,
                                          int* counter, size_t rsmem, size_t gsmem, const LaunchInfo& li,
                                          cudaStream_t s) {
  constexpr int C = 4;
  const int64_t total = order.total();
  auto rec = fast_adjoint_record_kernel<BLEND>;
  auto gen = fast_adjoint_persistent_kernel<FILTER, kTfTexture, BLEND, false, true, VT>;
  cudaError_t e = set_smem(rec, rsmem);
  if (e != cudaSuccess) return e;
  e = set_smem(gen, gsmem);
  if (e != cudaSuccess) return e;
  const int rgrid = persistent_grid(rec, rsmem, total * 32, li);  // one warp per ray
  const int ggrid = li.num_sms;
  // scratch: order ints, leftover list, the general kernel's TF-gradient slices
  const size_t order_bytes = (work_order_ints(p) * sizeof(int) + 255) & ~size_t(255);
  const size_t left_bytes = (size_t(total) * sizeof(int) + 255) & ~size_t(255);
  const size_t tf_bytes = (size_t(ggrid) * p.R * C * sizeof(float) + 255) & ~size_t(255);
  const size_t slice_bytes = size_t(rgrid) * (kFastThreads / 32) * p.R * C * sizeof(float);
  char* scratch =
      static_cast<char*>(acquire_scratch(li.device, s, order_bytes + left_bytes + tf_bytes + slice_bytes, e));
  if (!scratch) return e;
  int* order_ints = reinterpret_cast<int*>(scratch);
  int* leftover = reinterpret_cast<int*>(scratch + order_bytes);
  e = order_rays_by_work(p, &a, order_ints, li, s);
  if (e != cudaSuccess) return e;
  rec<<<rgrid, kFastThreads, rsmem, s>>>(p, a, order, counter, order_ints + work_order_list_offset,
                                         order_ints + work_order_count_offset, leftover,
                                         reinterpret_cast<float*>(scratch + order_bytes + left_bytes + tf_bytes));
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int* counter2 = acquire_counter(li.device, s, e);
  if (!counter2) return e;
  gen<<<ggrid, kFastThreads, gsmem, s>>>(p, a, order, counter2,
                                         reinterpret_cast<float*>(scratch + order_bytes + left_bytes), leftover,
                                         counter + 1, TexGather{});
  return cudaGetLastError();
}

// TF-gradient-only adjoint of a texture TF from the checkpoints alone (no
// sample record): longest-first order, the re-march kernel (chunks
// re-marched from their checkpoints into shared memory, through the slab
// gather texture where the forward would use it), then the general kernel
// over the rays the checkpoints do not cover.
template <int FILTER, int BLEND, typename VT>
static cudaError_t fast_adjoint_remarch_go(const RenderParams& p, const AdjointParams& a, const RayOrder& order,
                                           int* counter, int chunk, size_t rsmem, size_t gsmem, const LaunchInfo& li,
                                           cudaStream_t s) {
  constexpr int C = 4;
  const int64_t total = order.total();
  TexGather tg{};
  if (FILTER == kTrilinear && texture_gather_wanted<VT>(p)) {
    cudaError_t e = build_gather_texture<VT>(p, volume_entries(p), li, s, tg);
    if (e == cudaErrorNotSupported) tg = TexGather{};
    else if (e != cudaSuccess) return e;
  }
  auto go = [&](auto rem) {
    auto gen = fast_adjoint_persistent_kernel<FILTER, kTfTexture, BLEND, false, true, VT>;
    cudaError_t e = set_smem(rem, rsmem);
    if (e != cudaSuccess) return e;
    e = set_smem(gen, gsmem);
    if (e != cudaSuccess) return e;
    const int rgrid = persistent_grid(rem, rsmem, total * 32, li);  // one warp per ray
    const int ggrid = li.num_sms;
    // scratch: order ints, leftover list, the general kernel's TF-gradient slices, the
    // re-march kernel's per-warp slices
    const size_t order_bytes = (work_order_ints(p) * sizeof(int) + 255) & ~size_t(255);
    const size_t left_bytes = (size_t(total) * sizeof(int) + 255) & ~size_t(255);
    const size_t tf_bytes = (size_t(ggrid) * p.R * C * sizeof(float) + 255) & ~size_t(255);
    const size_t slice_bytes = size_t(rgrid) * (kFastThreads / 32) * p.R * C * sizeof(float);
    char* scratch =
        static_cast<char*>(acquire_scratch(li.device, s, order_bytes + left_bytes + tf_bytes + slice_bytes, e));
    if (!scratch) return e;
    int* order_ints = reinterpret_cast<int*>(scratch);
    int* leftover = reinterpret_cast<int*>(scratch + order_bytes);
    e = order_rays_by_work(p, &a, order_ints, li, s);
    if (e != cudaSuccess) return e;
    rem<<<rgrid, kFastThreads, rsmem, s>>>(p, a, order, counter, order_ints + work_order_list_offset,
                                           order_ints + work_order_count_offset, leftover,
                                           reinterpret_cast<float*>(scratch + order_bytes + left_bytes + tf_bytes),
                                           tg, chunk);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int* counter2 = acquire_counter(li.device, s, e);
    if (!counter2) return e;
    gen<<<ggrid, kFastThreads, gsmem, s>>>(p, a, order, counter2,
                                           reinterpret_cast<float*>(scratch + order_bytes + left_bytes), leftover,
                                           counter + 1, TexGather{});
    return cudaGetLastError();
  };
  if constexpr (FILTER == kTrilinear) {
    if (tg.tex) return go(fast_adjoint_remarch_kernel<FILTER, BLEND, VT, kGatherTexture>);
  }
  return go(fast_adjoint_remarch_kernel<FILTER, BLEND, VT, kGatherDirect>);
}

// The window kernel (dvr_window.cuh) adds its gradient window to global
// memory in 16-byte groups and stages the volume in 16-byte rows: both
// tensors must be z-contiguous with 16-byte aligned rows.
static bool rows_aligned(const void* base, const int64_t* st, int Z, int per16) {
  return st[3] == 1 && st[0] % per16 == 0 && st[1] % per16 == 0 && st[2] % per16 == 0 && Z % per16 == 0 &&
         (reinterpret_cast<uintptr_t>(base) & 15u) == 0;
}
constexpr int kWinGradCap = 6144;    // floats of the gradient window (24 KB)
constexpr int kWinVolBytes = 16384;  // bytes of the staged volume window

// Volume-gradient adjoint from the sample record: the window kernel over
// 16x8 tiles, then the general kernel over the rays without a record.
template <int TF, int BLEND, typename VT>
static cudaError_t fast_adjoint_window_go(const RenderParams& p, const AdjointParams& a, const RayOrder& order,
                                          int* counter, size_t gsmem, const LaunchInfo& li, cudaStream_t s) {
  constexpr int C = TfChannels<TF>::C;
  const bool tfgrad = a.has_tf != 0;
  const bool stage = (a.has_camera || a.has_stepsize) &&
                     rows_aligned(p.volume.p, p.volume.s, p.Z, 16 / int(sizeof(VT)));
  const int copies = p.tf.s[0] == 0 ? 1 : p.B;
  const int vol_cap = kWinVolBytes / int(sizeof(VT));
  const WinSmem S(TF, p.R, C, tfgrad, copies, kWinGradCap, stage ? kWinVolBytes : 0);
  const size_t wsmem = size_t(S.total) * sizeof(float);
  if (wsmem > size_t(li.max_smem_optin)) return cudaErrorInvalidConfiguration;
  const WinTiles tiles = WinTiles::make(p.W, p.H, p.B);
  auto launch = [&](auto wk, auto gk) -> cudaError_t {
    cudaError_t e = set_smem(wk, wsmem);
    if (e != cudaSuccess) return e;
    e = set_smem(gk, gsmem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wk, kFastThreads, wsmem) != cudaSuccess || per_sm < 1)
      per_sm = 1;
    const int wgrid = std::max(1, std::min(tiles.total(), per_sm * li.num_sms));
    const int ggrid = li.num_sms;
    // scratch: leftover ray list, the two kernels' TF-gradient slices
    const size_t left_bytes = (size_t(order.total()) * sizeof(int) + 255) & ~size_t(255);
    const size_t wtf = tfgrad ? ((size_t(wgrid) * p.R * C * sizeof(float) + 255) & ~size_t(255)) : 0;
    const size_t gtf = tfgrad ? size_t(ggrid) * p.R * C * sizeof(float) : 0;
    char* scratch = static_cast<char*>(acquire_scratch(li.device, s, left_bytes + wtf + gtf, e));
    if (!scratch) return e;
    int* leftover = reinterpret_cast<int*>(scratch);
    wk<<<wgrid, kFastThreads, wsmem, s>>>(p, a, tiles, order, counter,
                                          tfgrad ? reinterpret_cast<float*>(scratch + left_bytes) : nullptr,
                                          leftover, kWinGradCap, vol_cap);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int* counter2 = acquire_counter(li.device, s, e);
    if (!counter2) return e;
    gk<<<ggrid, kFastThreads, gsmem, s>>>(p, a, order, counter2,
                                          tfgrad ? reinterpret_cast<float*>(scratch + left_bytes + wtf) : nullptr,
                                          leftover, counter + 1, TexGather{});
    return cudaGetLastError();
  };
  if (tfgrad)
    return stage ? launch(window_adjoint_kernel<TF, BLEND, true, true, VT>,
                          fast_adjoint_persistent_kernel<kTrilinear, TF, BLEND, true, true, VT>)
                 : launch(window_adjoint_kernel<TF, BLEND, true, false, VT>,
                          fast_adjoint_persistent_kernel<kTrilinear, TF, BLEND, true, true, VT>);
  return stage ? launch(window_adjoint_kernel<TF, BLEND, false, true, VT>,
                        fast_adjoint_persistent_kernel<kTrilinear, TF, BLEND, true, false, VT>)
               : launch(window_adjoint_kernel<TF, BLEND, false, false, VT>,
                        fast_adjoint_persistent_kernel<kTrilinear, TF, BLEND, true, false, VT>);
}

template <int FILTER, int TF, int BLEND, typename VT>
static cudaError_t fast_adjoint_go(const RenderParams& p, const AdjointParams& a, const LaunchInfo& li,
                                   cudaStream_t s) {
  const RayOrder order = RayOrder::make(p.W, p.H, p.B);
  if (order.total() == 0) return cudaSuccess;
  if (order.total() > 0x7fffffff) return cudaErrorInvalidConfiguration;
  constexpr int C = TfChannels<TF>::C;
  const bool tfgrad = a.has_tf != 0, volgrad = a.has_volume != 0;
  const int copies = p.tf.s[0] == 0 ? 1 : p.B;
  const size_t smem = (size_t(AdjointSmem(TF, p.R, C, kFastThreads, tfgrad, p.ckpt.p ? p.ckpt_interval : 0, copies)
                                  .total) + (a.has_viewport ? size_t(p.B) * 9 : 0)) * sizeof(float);
  if (smem > size_t(li.max_smem_optin)) return cudaErrorInvalidConfiguration;
  cudaError_t err;
  int* counter = acquire_counter(li.device, s, err);
  if (!counter) return err;
  auto go = [&](auto kernel) {
    cudaError_t e = set_smem(kernel, smem);
    if (e != cudaSuccess) return e;
    const int grid = persistent_grid(kernel, smem, order.total(), li);
    // scratch: the longest-first ray list, then the blocks' TF-gradient slices
    const size_t list_bytes = (work_order_ints(p) * sizeof(int) + 255) & ~size_t(255);
    const size_t tf_bytes = tfgrad ? size_t(grid) * p.R * C * sizeof(float) : 0;
    char* scratch = static_cast<char*>(acquire_scratch(li.device, s, list_bytes + tf_bytes, e));
    if (!scratch) return e;
    int* order_ints = reinterpret_cast<int*>(scratch);
    e = order_rays_by_work(p, &a, order_ints, li, s);
    if (e != cudaSuccess) return e;
    // the slab gather texture serves the re-march of rays without a record
    // and the corner reads of position derivatives; with a record and no
    // position derivatives the kernel reads no volume (only the rare rays
    // the pool could not hold do, from the volume directly)
    TexGather tg{};
    if (FILTER == kTrilinear && (!p.dens || a.has_camera || a.has_stepsize || a.has_viewport) &&
        texture_gather_wanted<VT>(p)) {
      e = build_gather_texture<VT>(p, volume_entries(p), li, s, tg);
      if (e == cudaErrorNotSupported) tg = TexGather{};
      else if (e != cudaSuccess) return e;
    }
    // volume gradient through the cell-corner buffer where it stays in L2
    AdjointParams ac = a;
    const int vb = a.adj_volume.s[0] != 0 ? p.B : 1;
    const size_t cell_bytes = size_t(p.X) * p.Y * p.Z * vb * 8 * sizeof(float);
    if (FILTER == kTrilinear && volgrad && cell_bytes <= kCellGradMaxBytes) {
      ac.cell_grad = static_cast<float*>(acquire_scratch(li.device, s, cell_bytes, e, 2));
      if (!ac.cell_grad) return e;
      e = cudaMemsetAsync(ac.cell_grad, 0, cell_bytes, s);
      if (e != cudaSuccess) return e;
    }
    kernel<<<grid, kFastThreads, smem, s>>>(p, ac, order, counter, tfgrad ? reinterpret_cast<float*>(scratch + list_bytes)
                                                                        : nullptr,
                                            order_ints + work_order_list_offset, nullptr, tg);
    e = cudaGetLastError();
    if (e != cudaSuccess || !ac.cell_grad) return e;
    return fold_cell_grad(ac.cell_grad, a.adj_volume, p.X, p.Y, p.Z, vb, li, s);
  };
  if constexpr (TF == kTfTexture) {
    // TF gradient only, from the sample-density record
    if (tfgrad && !volgrad && !a.has_camera && !a.has_stepsize && !a.has_viewport && p.dens && p.ckpt.p) {
      const bool per_batch = a.adj_tf.s[0] != 0;
      (void)per_batch;
      const size_t rsmem = size_t(record_smem_floats(p.R, C, copies)) * sizeof(float);
      if (rsmem <= size_t(li.max_smem_optin)) {
        last_adjoint_path() = DVR_PATH_RECORD;
        return fast_adjoint_record_go<FILTER, BLEND, VT>(p, a, order, counter, rsmem, smem, li, s);
      }
    }
    // TF gradient only, from the checkpoints alone: the re-march kernel
    const int chunk = p.ckpt.p ? remarch_chunk(p.ckpt_interval) : 0;
    if (tfgrad && !volgrad && !a.has_camera && !a.has_stepsize && !a.has_viewport && !p.dens && chunk > 0) {
      const size_t rsmem =
          size_t(remarch_smem_floats(p.R, C, copies, kFastThreads / 32, chunk)) * sizeof(float);
      if (rsmem <= size_t(li.max_smem_optin)) {
        last_adjoint_path() = DVR_PATH_REMARCH;
        return fast_adjoint_remarch_go<FILTER, BLEND, VT>(p, a, order, counter, chunk, rsmem, smem, li, s);
      }
    }
  }
  if constexpr (FILTER == kTrilinear) {
    // volume gradients from the sample record: the window kernel
    if (volgrad && p.dens && p.ckpt.p && !a.has_viewport && window_adjoint_on() &&
        rows_aligned(a.adj_volume.p, a.adj_volume.s, p.Z, 4)) {
      last_adjoint_path() = DVR_PATH_WINDOW;
      return fast_adjoint_window_go<TF, BLEND, VT>(p, a, order, counter, smem, li, s);
    }
  }
  if (volgrad)
    return tfgrad ? go(fast_adjoint_persistent_kernel<FILTER, TF, BLEND, true, true, VT>)
                  : go(fast_adjoint_persistent_kernel<FILTER, TF, BLEND, true, false, VT>);
  return tfgrad ? go(fast_adjoint_persistent_kernel<FILTER, TF, BLEND, false, true, VT>)
                : go(fast_adjoint_persistent_kernel<FILTER, TF, BLEND, false, false, VT>);
}

template <int TF, typename VT>
cudaError_t launch_fast_adjoint_vt(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                   const LaunchInfo& li, cudaStream_t s) {
  if (filter == kNearest)
    return blend == kBeerLambert ? fast_adjoint_go<kNearest, TF, kBeerLambert, VT>(p, a, li, s)
                                 : fast_adjoint_go<kNearest, TF, kAlphaBlend, VT>(p, a, li, s);
  return blend == kBeerLambert ? fast_adjoint_go<kTrilinear, TF, kBeerLambert, VT>(p, a, li, s)
                               : fast_adjoint_go<kTrilinear, TF, kAlphaBlend, VT>(p, a, li, s);
}

// Same kernels as fast_adjoint_go; the work counter and the TF-gradient
// slices come from the caller, so nothing is allocated.
template <int FILTER, int TF, int BLEND, typename VT>
static cudaError_t fast_adjoint_into_go(const RenderParams& p, const AdjointParams& a, const LaunchInfo& li,
                                        const CallerScratch& sc, cudaStream_t s) {
  const RayOrder order = RayOrder::make(p.W, p.H, p.B);
  if (order.total() == 0) return cudaSuccess;
  if (order.total() > 0x7fffffff) return cudaErrorInvalidConfiguration;
  constexpr int C = TfChannels<TF>::C;
  const bool tfgrad = a.has_tf != 0, volgrad = a.has_volume != 0;
  const int copies = p.tf.s[0] == 0 ? 1 : p.B;
  const size_t smem = (size_t(AdjointSmem(TF, p.R, C, kFastThreads, tfgrad, p.ckpt.p ? p.ckpt_interval : 0, copies)
                                  .total) + (a.has_viewport ? size_t(p.B) * 9 : 0)) * sizeof(float);
  if (smem > size_t(li.max_smem_optin)) return cudaErrorInvalidConfiguration;
  const size_t slice = size_t(p.R) * C * sizeof(float);
  const int64_t fit = tfgrad ? int64_t(sc.tf_bytes / slice) : int64_t(1) << 30;
  if (fit < 1) return cudaErrorInvalidValue;
  cudaError_t err = cudaMemsetAsync(sc.counter, 0, sizeof(int), s);
  if (err != cudaSuccess) return err;
  auto go = [&](auto kernel) {
    cudaError_t e = set_smem(kernel, smem);
    if (e != cudaSuccess) return e;
    const int grid = int(std::min<int64_t>(persistent_grid(kernel, smem, order.total(), li), fit));
    kernel<<<grid, kFastThreads, smem, s>>>(p, a, order, sc.counter, sc.tf, nullptr, nullptr, TexGather{});
    return cudaGetLastError();
  };
  if (volgrad)
    return tfgrad ? go(fast_adjoint_persistent_kernel<FILTER, TF, BLEND, true, true, VT>)
                  : go(fast_adjoint_persistent_kernel<FILTER, TF, BLEND, true, false, VT>);
  return tfgrad ? go(fast_adjoint_persistent_kernel<FILTER, TF, BLEND, false, true, VT>)
                : go(fast_adjoint_persistent_kernel<FILTER, TF, BLEND, false, false, VT>);
}

template <int TF, typename VT>
cudaError_t launch_fast_adjoint_into_vt(const RenderParams& p, const AdjointParams& a, int filter, int blend,
                                        const LaunchInfo& li, const CallerScratch& sc, cudaStream_t s) {
  if (filter == kNearest)
    return blend == kBeerLambert ? fast_adjoint_into_go<kNearest, TF, kBeerLambert, VT>(p, a, li, sc, s)
                                 : fast_adjoint_into_go<kNearest, TF, kAlphaBlend, VT>(p, a, li, sc, s);
  return blend == kBeerLambert ? fast_adjoint_into_go<kTrilinear, TF, kBeerLambert, VT>(p, a, li, sc, s)
                               : fast_adjoint_into_go<kTrilinear, TF, kAlphaBlend, VT>(p, a, li, sc, s);
}
#endif

}  // namespace dvr

#define DVR_INSTANTIATE_FAST(TF, VT)                                                                        \
  template cudaError_t dvr::launch_fast_forward_vt<TF, VT>(const RenderParams&, int, int, const LaunchInfo&, \
                                                           cudaStream_t);                                    \
  template cudaError_t dvr::launch_fast_adjoint_vt<TF, VT>(const RenderParams&, const AdjointParams&, int, int, \
                                                           const LaunchInfo&, cudaStream_t);                 \
  template cudaError_t dvr::launch_fast_forward_batched_vt<TF, VT>(const BatchForwardTable&, int, size_t, int, int, \
                                                                   cudaStream_t);                            \
  template cudaError_t dvr::launch_fast_adjoint_batched_vt<TF, VT>(const BatchAdjointTable&, int, size_t, int, int, \
                                                                   bool, bool, cudaStream_t);                            \
  template cudaError_t dvr::launch_fast_adjoint_into_vt<TF, VT>(const RenderParams&, const AdjointParams&, int,  \
                                                                int, const LaunchInfo&, const CallerScratch&,  \
                                                                cudaStream_t);
