// Small float3/float4 helpers for the ray-marcher kernels.
//
// Operation order follows the reference's vector math where results must
// match it bit for bit on identical inputs: dot = x*x' + y*y' + z*z' [+ w*w'],
// lerp(a, b, t) = a + t*(b - a), clamp = fmax(lo, fmin(v, hi)), and rmin/rmax
// as ternaries (renderer/helper_math.cuh:86-100, :1835-1850, :1898-1908).
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace dvr {

struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

__host__ __device__ __forceinline__ f3 mk3(float x, float y, float z) { return {x, y, z}; }
__host__ __device__ __forceinline__ f4 mk4(float x, float y, float z, float w) { return {x, y, z, w}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float dot4(f4 a, f4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
__device__ __forceinline__ float lerp1(float a, float b, float t) { return a + t * (b - a); }
// Two lerps as one pair of packed FP32 operations (FADD2, FFMA2 on sm_100
// and later): per element the subtraction and the fused multiply-add that
// lerp1 compiles to, half the instructions.
__device__ __forceinline__ float2 lerp2(float2 a, float2 b, float2 t) {
  return __ffma2_rn(t, __fadd2_rn(b, make_float2(-a.x, -a.y)), a);
}
__device__ __forceinline__ float rminf(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float rmaxf(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fmaxf(lo, fminf(v, hi)); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return max(lo, min(v, hi)); }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ f3 normalize3(f3 v) {
  const float inv = rsqrtf(dot3(v, v));
  return mk3(v.x * inv, v.y * inv, v.z * inv);
}

// Storage types of the density volume / transfer function and their
// conversion to the FP32 compute type.
template <typename T> struct Storage;
template <> struct Storage<float> {
  static __device__ __forceinline__ float load(const float* p) { return __ldg(p); }
};
template <> struct Storage<__half> {
  static __device__ __forceinline__ float load(const __half* p) { return __half2float(__ldg(p)); }
};
template <> struct Storage<__nv_bfloat16> {
  static __device__ __forceinline__ float load(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }
};

// Conversion of one stored value to FP32 without a read-only global load:
// for copies of the volume staged in shared memory (Storage<T>::load reads
// through the non-coherent global path, which is for global memory only).
__device__ __forceinline__ float to_float(float v) { return v; }
__device__ __forceinline__ float to_float(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_float(__nv_bfloat16 v) { return __bfloat162float(v); }

}  // namespace dvr
