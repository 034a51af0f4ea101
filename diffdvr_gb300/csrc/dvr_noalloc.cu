// dvr_render_adjoint_noalloc: the optimized adjoint with its scratch in a
// file-scope device array instead of memory the library allocates.
//
// dvr_render_adjoint takes its work counters and TF-gradient scratch from
// pools that it grows with cudaMalloc on first use.  Some callers cannot let
// a library allocate device memory: applications that hand the whole device
// to their own allocator or run under a hard memory budget, and render loops
// that must not meet cudaMalloc's implicit device synchronisation.  This entry
// point makes no device allocation at all; its scratch is the static array
// below, sized kNoAllocScratchBytes per device.
//
//   bytes [0, 256)      the persistent kernel's work counter, set to zero with
//                       cudaMemsetAsync on the caller's stream before each launch
//   bytes [256, 4 MiB)  TF-gradient slices, R*C floats per block, which each
//                       block zeroes itself before use
//
// Because every call on a device shares this one array, calls that may
// overlap on the same device (other streams, other host threads) race; the
// caller serialises them.
//
// The array's device address is resolved once per device, on the first call
// there, and kept for the life of the process.  cudaDeviceReset destroys the
// context that address belongs to: a process that resets a device must not
// call this entry point on that device afterwards.
#include <cuda_runtime.h>

#include <mutex>

#include "dvr_entry.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr size_t kCounterBytes = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_base[kMaxDevices] = {};

// Resolves the array's address once per device; `device` is current here.
const char* noalloc_scratch(int device, dvr::CallerScratch* out) {
  if (device < 0 || device >= kMaxDevices) return "device index out of range for the no-allocation adjoint";
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_base[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return "cudaGetSymbolAddress failed for the no-allocation adjoint's scratch array";
    }
    g_scratch_base[device] = static_cast<unsigned char*>(p);
  }
  unsigned char* base = g_scratch_base[device];
  out->counter = reinterpret_cast<int*>(base);
  out->tf = reinterpret_cast<float*>(base + kCounterBytes);
  out->tf_bytes = kNoAllocScratchBytes - kCounterBytes;
  return nullptr;
}

}  // namespace

extern "C" int dvr_render_adjoint_noalloc(const DvrRendererInputs* inputs,
                                          const DvrRendererOutputs* outputs_from_forward,
                                          const DvrTensor* adj_color, const DvrAdjointOutputs* adj_outputs,
                                          void* cuda_stream) {
  return dvr::render_adjoint_into(inputs, outputs_from_forward, adj_color, adj_outputs, cuda_stream,
                                  noalloc_scratch);
}
