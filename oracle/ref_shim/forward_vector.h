// Declaration-only stand-in for the forward-mode AD header of the reference's
// absent cudAD submodule. The forward and adjoint ray marchers compile against
// these declarations without instantiating any dual-number arithmetic; only the
// plain-vector accessors are defined. Test infrastructure only.
#pragma once
#include <cuda_runtime.h>
namespace cudAD {
namespace internal { template <typename T, int N> struct array { T v[N]; }; }
template <typename T, int D> struct fvar {
  T value_;
  __host__ __device__ const T& value() const { return value_; }
  __host__ __device__ explicit operator T() const { return value_; }
  template <int I> static __host__ __device__ fvar input(const T& v);
  static __host__ __device__ fvar input(const T& v, int idx);
  static __host__ __device__ fvar constant(const T& v);
  __host__ __device__ T derivative(int) const;
  template <int I> __host__ __device__ T derivative() const;
};
#define DVR_SHIM_ACCESSORS(TYPE, ELEM)                                              \
  __host__ __device__ inline ELEM getX(const TYPE& v) { return v.x; }               \
  __host__ __device__ inline ELEM getY(const TYPE& v) { return v.y; }
DVR_SHIM_ACCESSORS(float2, float)
DVR_SHIM_ACCESSORS(double2, double)
DVR_SHIM_ACCESSORS(float3, float)
DVR_SHIM_ACCESSORS(double3, double)
DVR_SHIM_ACCESSORS(float4, float)
DVR_SHIM_ACCESSORS(double4, double)
#undef DVR_SHIM_ACCESSORS
__host__ __device__ inline float getZ(const float3& v) { return v.z; }
__host__ __device__ inline double getZ(const double3& v) { return v.z; }
__host__ __device__ inline float getZ(const float4& v) { return v.z; }
__host__ __device__ inline double getZ(const double4& v) { return v.z; }
__host__ __device__ inline float getW(const float4& v) { return v.w; }
__host__ __device__ inline double getW(const double4& v) { return v.w; }
template <int D> __host__ __device__ fvar<float3, D> make_float3in(const float3&, const int3&);
template <int D> __host__ __device__ fvar<double3, D> make_double3in(const double3&, const int3&);
template <int D> __host__ __device__ fvar<float4, D> make_float4in(const float4&, const int4&);
template <int D> __host__ __device__ fvar<double4, D> make_double4in(const double4&, const int4&);
template <typename T> __host__ __device__ T broadcast3(const T& v);
template <typename T> __host__ __device__ T broadcast4(const T& v);
}  // namespace cudAD
