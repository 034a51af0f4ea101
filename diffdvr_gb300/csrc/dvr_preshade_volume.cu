// Pre-shading of a density volume (TFUtils::preshadeVolume,
// renderer/tf_utils.cpp:160-249, renderer/tf_utils_impl.cu:16-170): the
// colour volume 4 x X x Y x Z of a density volume 1 x X x Y x Z through the
// TF of batch entry 0, and its adjoint d loss / d density.  One thread per
// voxel in z-fastest order, the TF staged in shared memory; HBM-bound (4 B
// read and 16 B written per voxel forward, 20 B read and 4 B written
// adjoint).
#include "dvr_kernels.h"
#include "dvr_device.cuh"

namespace dvr {

namespace {
struct Dummy {
  __device__ __forceinline__ void add(int, int, float) {}
};

__device__ __forceinline__ void stage(const PreshadeParams& q, float* s_tf) {
  for (int e = threadIdx.x; e < q.R * q.C; e += blockDim.x) {
    const int r = e / q.C, c = e - r * q.C;
    s_tf[e] = q.tf[r * q.tf_s[1] + c * q.tf_s[2]];
  }
  __syncthreads();
}

template <int TF>
__global__ void __launch_bounds__(256) preshade_kernel(const PreshadeParams q) {
  extern __shared__ float s_tf[];
  stage(q, s_tf);
  constexpr int C = TfChannels<TF>::C;
  const TfShared<C> tf{s_tf, q.R};
  const int64_t n = int64_t(q.X) * q.Y * q.Z;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int z = int(i % q.Z);
    const int64_t r = i / q.Z;
    const int y = int(r % q.Y), x = int(r / q.Y);
    const float d = q.density[x * q.d_s[1] + y * q.d_s[2] + z * q.d_s[3]];
    const f4 c = tf_eval<TF>(tf, d);
    float* o = q.out + x * q.o_s[1] + y * q.o_s[2] + z * q.o_s[3];
    o[0] = c.x;
    o[q.o_s[0]] = c.y;
    o[2 * q.o_s[0]] = c.z;
    o[3 * q.o_s[0]] = c.w;
  }
}

template <int TF>
__global__ void __launch_bounds__(256) preshade_adjoint_kernel(const PreshadeParams q) {
  extern __shared__ float s_tf[];
  stage(q, s_tf);
  constexpr int C = TfChannels<TF>::C;
  const TfShared<C> tf{s_tf, q.R};
  const int64_t n = int64_t(q.X) * q.Y * q.Z;
  Dummy none;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int z = int(i % q.Z);
    const int64_t r = i / q.Z;
    const int y = int(r % q.Y), x = int(r / q.Y);
    const float d = q.density[x * q.d_s[1] + y * q.d_s[2] + z * q.d_s[3]];
    const float* a = q.adj_color + x * q.a_s[1] + y * q.a_s[2] + z * q.a_s[3];
    const f4 adj = mk4(a[0], a[q.a_s[0]], a[2 * q.a_s[0]], a[3 * q.a_s[0]]);
    q.out[x * q.o_s[1] + y * q.o_s[2] + z * q.o_s[3]] = tf_adjoint<TF, false>(tf, d, adj, none);
  }
}

template <int TF>
cudaError_t go(const PreshadeParams& q, bool adjoint, const LaunchInfo& li, cudaStream_t s) {
  const int64_t n = int64_t(q.X) * q.Y * q.Z;
  if (n == 0) return cudaSuccess;
  const size_t smem = size_t(q.R) * q.C * sizeof(float);
  auto kernel = adjoint ? preshade_adjoint_kernel<TF> : preshade_kernel<TF>;
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
  const int64_t need = (n + 255) / 256;
  const int grid = int(need < int64_t(per_sm) * li.num_sms ? need : int64_t(per_sm) * li.num_sms);
  kernel<<<grid, 256, smem, s>>>(q);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_preshade_volume(const PreshadeParams& q, int tf_mode, bool adjoint, const LaunchInfo& li,
                                   cudaStream_t s) {
  switch (tf_mode) {
    case kTfIdentity: return go<kTfIdentity>(q, adjoint, li, s);
    case kTfTexture: return go<kTfTexture>(q, adjoint, li, s);
    case kTfLinear: return go<kTfLinear>(q, adjoint, li, s);
    default: return go<kTfGaussian>(q, adjoint, li, s);
  }
}

}  // namespace dvr
