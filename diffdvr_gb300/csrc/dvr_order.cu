// Longest-first ray order for the persistent kernels.
//
// With one or two rays per resident lane, fetching rays in pixel order lets a
// long ray fetched late set the end of the launch while the other warps wait.
// These kernels bucket the ray ids by descending work n (key = 255 -
// min(255, floor(4 sqrt(n))): buckets a few samples wide for short rays, a
// few tens for rays of thousands of samples) so the tail of the launch is made
// of short rays.  The adjoint's n is exact, the forward's termination index;
// the forward's is the ray's sample bound from the box entry and exit (early
// termination may end it sooner).  Within a bucket, ids of one block of
// consecutive rays stay together, so neighbouring rays are still fetched by
// the same warp.
//
// For the forward, rays without samples (outside the image or missing the
// box) form the last bucket; the scatter pass writes their outputs (zero
// colour and sample count, no density record) and the scan publishes the
// number of rays before that bucket, which is all the forward kernel marches.
#include "dvr_kernels.h"
#include "dvr_persist.cuh"

namespace dvr {
namespace {

constexpr int kBuckets = 256;
constexpr int kOrderThreads = 256;
static_assert(work_order_count_offset == 2 * kBuckets && work_order_list_offset > work_order_count_offset,
              "histogram, bucket starts, count of rays with work, list");

template <bool FWD>
__device__ __forceinline__ int work_key(const RenderParams& p, const AdjointParams& a, const RayOrder& o, int id) {
  int b, x, y;
  if (!o.pixel(id, b, x, y)) return kBuckets - 1;
  int n;
  if constexpr (FWD) {
    FastRay r;
    fast_setup(p, x, y, b, r);
    n = max_samples(r.tmin, r.tmax, r.step);
  } else {
    n = static_cast<const int*>(a.fwd_term.p)[b * a.fwd_term.s[0] + y * a.fwd_term.s[1] + x * a.fwd_term.s[2]];
  }
  const int r = n <= 0 ? 0 : min(kBuckets - 1, int(sqrtf(float(n)) * 4.f));
  return kBuckets - 1 - r;
}

// keys[id] keeps each ray's bucket for the scatter pass
template <bool FWD>
__global__ void __launch_bounds__(kOrderThreads) work_histogram_kernel(const RenderParams p, const AdjointParams a,
                                                                       const RayOrder o, int* hist,
                                                                       unsigned char* keys) {
  __shared__ int sh[kBuckets];
  sh[threadIdx.x] = 0;
  __syncthreads();
  const int total = int(o.total());
  for (int id = blockIdx.x * kOrderThreads + threadIdx.x; id < total; id += gridDim.x * kOrderThreads) {
    const int key = work_key<FWD>(p, a, o, id);
    keys[id] = static_cast<unsigned char>(key);
    atomicAdd(&sh[key], 1);
  }
  __syncthreads();
  if (sh[threadIdx.x] > 0) atomicAdd(&hist[threadIdx.x], sh[threadIdx.x]);
}

// exclusive scan of the histogram into the bucket starts (one block); the
// start of the last bucket (rays without samples) is the number of rays with work
__global__ void __launch_bounds__(kOrderThreads) work_scan_kernel(const int* hist, int* start, int* with_work) {
  __shared__ int sh[kBuckets];
  sh[threadIdx.x] = hist[threadIdx.x];
  __syncthreads();
  for (int o = 1; o < kBuckets; o <<= 1) {
    const int v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  start[threadIdx.x] = sh[threadIdx.x] - hist[threadIdx.x];
  if (threadIdx.x == kBuckets - 1) *with_work = sh[threadIdx.x] - hist[threadIdx.x];
}

// outputs of a forward ray without samples
__device__ __forceinline__ void finish_empty_ray(const RenderParams& p, const RayOrder& o, int id) {
  int b, x, y;
  if (!o.pixel(id, b, x, y)) return;
  float* col = static_cast<float*>(p.color.p) + b * p.color.s[0] + y * p.color.s[1] + x * p.color.s[2];
  col[0] = 0.f;
  col[p.color.s[3]] = 0.f;
  col[2 * p.color.s[3]] = 0.f;
  col[3 * p.color.s[3]] = 0.f;
  static_cast<int*>(p.term.p)[b * p.term.s[0] + y * p.term.s[1] + x * p.term.s[2]] = 0;
  if (p.dens) static_cast<int*>(p.dens_off.p)[b * p.dens_off.s[0] + y * p.dens_off.s[1] + x * p.dens_off.s[2]] = -1;
}

template <bool FWD>
__global__ void __launch_bounds__(kOrderThreads) work_scatter_kernel(const RenderParams p, const RayOrder o,
                                                                     const unsigned char* keys, int* start,
                                                                     int* list) {
  __shared__ int cnt[kBuckets];
  __shared__ int base[kBuckets];
  const int total = int(o.total());
  for (int first = blockIdx.x * kOrderThreads; first < total; first += gridDim.x * kOrderThreads) {
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int id = first + threadIdx.x;
    const int key = id < total ? int(keys[id]) : 0;
    const int rank = id < total ? atomicAdd(&cnt[key], 1) : 0;
    __syncthreads();
    if (cnt[threadIdx.x] > 0) base[threadIdx.x] = atomicAdd(&start[threadIdx.x], cnt[threadIdx.x]);
    __syncthreads();
    if (id < total) {
      list[base[key] + rank] = id;
      if (FWD && key == kBuckets - 1) finish_empty_ray(p, o, id);
    }
    __syncthreads();
  }
}

}  // namespace

// histogram, bucket starts, count, list (total ints), keys (total bytes)
size_t work_order_ints(const RenderParams& p) {
  const size_t total = size_t(RayOrder::make(p.W, p.H, p.B).total());
  return work_order_list_offset + total + (total + 3) / 4;
}

cudaError_t order_rays_by_work(const RenderParams& p, const AdjointParams* a, int* scratch, const LaunchInfo& li,
                               cudaStream_t s) {
  const RayOrder o = RayOrder::make(p.W, p.H, p.B);
  const int64_t total = o.total();
  if (total == 0) return cudaSuccess;
  int* hist = scratch;
  int* start = scratch + kBuckets;
  int* with_work = scratch + work_order_count_offset;
  int* list = scratch + work_order_list_offset;
  unsigned char* keys = reinterpret_cast<unsigned char*>(list + total);
  cudaError_t e = cudaMemsetAsync(hist, 0, kBuckets * sizeof(int), s);
  if (e != cudaSuccess) return e;
  const int blocks = int(std::min<int64_t>((total + kOrderThreads - 1) / kOrderThreads, int64_t(li.num_sms) * 8));
  if (a) {
    work_histogram_kernel<false><<<blocks, kOrderThreads, 0, s>>>(p, *a, o, hist, keys);
    work_scan_kernel<<<1, kOrderThreads, 0, s>>>(hist, start, with_work);
    work_scatter_kernel<false><<<blocks, kOrderThreads, 0, s>>>(p, o, keys, start, list);
  } else {
    const AdjointParams none{};
    work_histogram_kernel<true><<<blocks, kOrderThreads, 0, s>>>(p, none, o, hist, keys);
    work_scan_kernel<<<1, kOrderThreads, 0, s>>>(hist, start, with_work);
    work_scatter_kernel<true><<<blocks, kOrderThreads, 0, s>>>(p, o, keys, start, list);
  }
  return cudaGetLastError();
}

}  // namespace dvr
