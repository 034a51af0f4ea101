// Launchers of the pre-shaded kernels (all blend modes and volume storage types).
#include "dvr_preshaded.cuh"

namespace dvr {

namespace {
template <typename K>
int grid_for(K kernel, int block, int64_t work, const LaunchInfo& li) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  const int64_t need = (work + block - 1) / block;
  const int64_t cap = int64_t(per_sm) * li.num_sms;
  return int(need < cap ? (need > 0 ? need : 1) : cap);
}

template <int BLEND, typename VT>
cudaError_t forward_go(const RenderParams& p, const LaunchInfo& li, cudaStream_t s) {
  auto kernel = preshaded_forward_kernel<BLEND, VT>;
  cudaError_t err = cudaSuccess;
  int* counter = acquire_counter(li.device, s, err);
  if (err != cudaSuccess) return err;
  const int64_t rays = int64_t(p.B) * p.H * p.W;
  // one warp per ray: rays x 32 threads of work
  kernel<<<grid_for(kernel, kFastThreads, rays * 32, li), kFastThreads, 0, s>>>(p, counter);
  return cudaGetLastError();
}

template <int BLEND, typename VT, bool EXACT>
cudaError_t adjoint_go(const RenderParams& p, const AdjointParams& a, const LaunchInfo& li, cudaStream_t s) {
  const RayOrder order = RayOrder::make(p.W, p.H, p.B);
  const int64_t total = order.total();
  if (total > 0x7fffffff) return cudaErrorInvalidConfiguration;
  // the warp-per-ray record kernel pays off when the rays are too few to fill
  // the GPU one per lane (1 view of 256^2: 1.2 ms against 4.1 ms); with more
  // rays the per-lane kernel, which gathers each sample once, is faster
  // (8 views: 9.5 ms against 12.1 ms)
  bool record = false;
  if (EXACT && p.dens != nullptr) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, preshaded_adjoint_kernel<BLEND, VT, true, EXACT>,
                                                      kFastThreads, 0) != cudaSuccess || per_sm < 1)
      per_sm = 1;
    record = int64_t(p.B) * p.H * p.W <= 2 * int64_t(per_sm) * li.num_sms * kFastThreads;
  }
  // scratch: the longest-first order, and the leftover list of the record kernel
  const size_t order_bytes = (work_order_ints(p) * sizeof(int) + 255) & ~size_t(255);
  const size_t left_bytes = record ? size_t(total) * sizeof(int) : 0;
  cudaError_t err = cudaSuccess;
  char* scratch = static_cast<char*>(acquire_scratch(li.device, s, order_bytes + left_bytes, err));
  if (!scratch) return err;
  int* ints = reinterpret_cast<int*>(scratch);
  err = order_rays_by_work(p, &a, ints, li, s);
  if (err != cudaSuccess) return err;
  int* counter = acquire_counter(li.device, s, err);
  if (err != cudaSuccess) return err;
  const int* list = ints + work_order_list_offset;
  const int* count = ints + work_order_count_offset;
  auto run = [&](auto kernel, int* ctr, const int* l, const int* c) {
    kernel<<<grid_for(kernel, kFastThreads, total, li), kFastThreads, 0, s>>>(p, a, order, ctr, l, c);
    return cudaGetLastError();
  };
  auto per_lane = [&](int* ctr, const int* l, const int* c) {
    return a.has_volume ? run(preshaded_adjoint_kernel<BLEND, VT, true, EXACT>, ctr, l, c)
                        : run(preshaded_adjoint_kernel<BLEND, VT, false, EXACT>, ctr, l, c);
  };
  if (!record) return per_lane(counter, list, count);
  // one warp per recorded ray, then one lane per leftover ray
  int* leftover = reinterpret_cast<int*>(scratch + order_bytes);
  const bool pos = a.has_camera || a.has_stepsize;
  auto rec = [&](auto kernel) {
    kernel<<<grid_for(kernel, kFastThreads, total * 32, li), kFastThreads, 0, s>>>(p, a, order, counter, list, count,
                                                                                  leftover);
    return cudaGetLastError();
  };
  err = a.has_volume ? (pos ? rec(preshaded_record_adjoint_kernel<BLEND, VT, true, true>)
                            : rec(preshaded_record_adjoint_kernel<BLEND, VT, true, false>))
                     : (pos ? rec(preshaded_record_adjoint_kernel<BLEND, VT, false, true>)
                            : rec(preshaded_record_adjoint_kernel<BLEND, VT, false, false>));
  if (err != cudaSuccess) return err;
  int* counter2 = acquire_counter(li.device, s, err);
  if (err != cudaSuccess) return err;
  return per_lane(counter2, leftover, counter + 1);
}

template <typename VT>
cudaError_t adjoint_vt(const RenderParams& p, const AdjointParams& a, int blend, bool exact, const LaunchInfo& li,
                       cudaStream_t s) {
  if (blend == kBeerLambert)
    return exact ? adjoint_go<kBeerLambert, VT, true>(p, a, li, s) : adjoint_go<kBeerLambert, VT, false>(p, a, li, s);
  return exact ? adjoint_go<kAlphaBlend, VT, true>(p, a, li, s) : adjoint_go<kAlphaBlend, VT, false>(p, a, li, s);
}
}  // namespace

cudaError_t launch_preshaded_forward(const RenderParams& p, int blend, bool plain, const LaunchInfo& li,
                                     cudaStream_t s) {
  const int64_t rays = int64_t(p.B) * p.H * p.W;
  if (rays == 0) return cudaSuccess;
  if (plain) {
    auto run = [&](auto kernel) {
      kernel<<<grid_for(kernel, 256, rays, li), 256, 0, s>>>(p);
      return cudaGetLastError();
    };
    return blend == kBeerLambert ? run(preshaded_plain_forward_kernel<kBeerLambert>)
                                 : run(preshaded_plain_forward_kernel<kAlphaBlend>);
  }
  switch (p.vol_storage) {
    case kF16: return blend == kBeerLambert ? forward_go<kBeerLambert, __half>(p, li, s)
                                            : forward_go<kAlphaBlend, __half>(p, li, s);
    case kBF16: return blend == kBeerLambert ? forward_go<kBeerLambert, __nv_bfloat16>(p, li, s)
                                             : forward_go<kAlphaBlend, __nv_bfloat16>(p, li, s);
    default: return blend == kBeerLambert ? forward_go<kBeerLambert, float>(p, li, s)
                                          : forward_go<kAlphaBlend, float>(p, li, s);
  }
}

cudaError_t launch_preshaded_adjoint(const RenderParams& p, const AdjointParams& a, int blend, bool exact,
                                     const LaunchInfo& li, cudaStream_t s) {
  if (int64_t(p.B) * p.H * p.W == 0) return cudaSuccess;
  switch (p.vol_storage) {
    case kF16: return adjoint_vt<__half>(p, a, blend, exact, li, s);
    case kBF16: return adjoint_vt<__nv_bfloat16>(p, a, blend, exact, li, s);
    default: return adjoint_vt<float>(p, a, blend, exact, li, s);
  }
}

}  // namespace dvr
