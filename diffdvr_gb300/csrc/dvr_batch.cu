// Batched rendering of uneven instances in one launch.
//
// The host builds a work list of (instance, batch entry, tile) items ordered
// by decreasing estimated cost (pixels of the tile times samples per ray), so
// the block scheduler starts the longest tiles first and the tail of the
// launch is made of short ones.  Instance descriptors and the list are copied
// through a pinned staging buffer into a per-device workspace that the
// library owns and grows on demand.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "dvr_batch.h"
#include "dvr_fast_launch.cuh"

namespace dvr {
namespace {

struct Workspace {
  void* dev = nullptr;
  size_t dev_bytes = 0;
  void* host = nullptr;       // pinned staging
  size_t host_bytes = 0;
  cudaEvent_t copied = nullptr;  // staging may be rewritten once this fired
  std::mutex mutex;
};
Workspace g_ws[64];

cudaError_t ensure(Workspace& w, size_t bytes) {
  cudaError_t e = cudaSuccess;
  if (!w.copied) {
    e = cudaEventCreateWithFlags(&w.copied, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
  }
  if (w.host_bytes < bytes) {
    if (w.host) {
      cudaEventSynchronize(w.copied);
      cudaFreeHost(w.host);
    }
    w.host = nullptr;
    w.host_bytes = 0;
    e = cudaMallocHost(&w.host, bytes * 2);
    if (e != cudaSuccess) return e;
    w.host_bytes = bytes * 2;
  }
  if (w.dev_bytes < bytes) {
    if (w.dev) {
      // earlier launches may still read the old table
      e = cudaDeviceSynchronize();
      if (e != cudaSuccess) return e;
      cudaFree(w.dev);
    }
    w.dev = nullptr;
    w.dev_bytes = 0;
    e = cudaMalloc(&w.dev, bytes * 2);
    if (e != cudaSuccess) return e;
    w.dev_bytes = bytes * 2;
  }
  return cudaSuccess;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Samples per ray, from the volume diagonal in voxels and the step in voxels
// (step given by value; a step-size tensor counts as one voxel).
double cost_per_ray(const RenderParams& p) {
  const double diag = std::sqrt(double(p.X) * p.X + double(p.Y) * p.Y + double(p.Z) * p.Z);
  double step_vox = 1.0;
  if (p.step.p == nullptr && p.box_size.p == nullptr) {
    const double vx = p.box_size.val[0] / std::max(1, p.X - 1);
    if (vx > 0 && p.step.val[0] > 0) step_vox = p.step.val[0] / vx;
  }
  return diag / std::max(step_vox, 1e-3);
}

std::vector<int4> build_items(const RenderParams* ps, int n) {
  struct Inst {
    int i;
    double cost;
  };
  std::vector<Inst> order(n);
  for (int i = 0; i < n; ++i) order[i] = {i, cost_per_ray(ps[i])};
  std::stable_sort(order.begin(), order.end(), [](const Inst& a, const Inst& b) { return a.cost > b.cost; });
  std::vector<int4> items;
  for (const Inst& o : order) {
    const RenderParams& p = ps[o.i];
    const int tx = (p.W + kTileW - 1) / kTileW, ty = (p.H + kTileH - 1) / kTileH;
    for (int b = 0; b < p.B; ++b)
      for (int y = 0; y < ty; ++y)
        for (int x = 0; x < tx; ++x) items.push_back(make_int4(o.i, b, x, y));
  }
  return items;
}

template <typename T>
cudaError_t stage(Workspace& w, const std::vector<std::pair<const void*, size_t>>& parts, std::vector<size_t>& offs,
                  cudaStream_t s) {
  size_t total = 0;
  offs.clear();
  for (auto& pr : parts) {
    offs.push_back(total);
    total = align_up(total + pr.second, 256);
  }
  cudaError_t e = ensure(w, total);
  if (e != cudaSuccess) return e;
  e = cudaEventSynchronize(w.copied);  // the previous upload has left the staging buffer
  if (e != cudaSuccess) return e;
  for (size_t i = 0; i < parts.size(); ++i)
    std::memcpy(static_cast<char*>(w.host) + offs[i], parts[i].first, parts[i].second);
  e = cudaMemcpyAsync(w.dev, w.host, total, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  return cudaEventRecord(w.copied, s);
}

size_t max_tf_entries(const RenderParams* ps, int n) {
  size_t m = 0;
  for (int i = 0; i < n; ++i) m = std::max(m, size_t(ps[i].R) * ps[i].C);
  return m;
}

template <int TF>
cudaError_t fwd_tf(const RenderParams* t, const int4* items, int n_items, size_t smem, int vst, int filter, int blend,
                   cudaStream_t s) {
  switch (vst) {
    case kF16: return launch_fast_forward_batched_vt<TF, __half>(t, items, n_items, smem, filter, blend, s);
    case kBF16: return launch_fast_forward_batched_vt<TF, __nv_bfloat16>(t, items, n_items, smem, filter, blend, s);
    default: return launch_fast_forward_batched_vt<TF, float>(t, items, n_items, smem, filter, blend, s);
  }
}

template <int TF>
cudaError_t adj_tf(const RenderParams* t, const AdjointParams* at, const int4* items, int n_items, size_t smem,
                   int vst, int filter, int blend, bool vg, bool tg, cudaStream_t s) {
  switch (vst) {
    case kF16:
      return launch_fast_adjoint_batched_vt<TF, __half>(t, at, items, n_items, smem, filter, blend, vg, tg, s);
    case kBF16:
      return launch_fast_adjoint_batched_vt<TF, __nv_bfloat16>(t, at, items, n_items, smem, filter, blend, vg, tg, s);
    default:
      return launch_fast_adjoint_batched_vt<TF, float>(t, at, items, n_items, smem, filter, blend, vg, tg, s);
  }
}

std::mutex g_counter_mutex;
int* g_counters[64] = {};
unsigned g_counter_next[64] = {};
constexpr unsigned kCounters = 4096;
constexpr unsigned kCounterInts = 4;  // 16 bytes per launch

struct ScratchSlot {
  int device = -1;
  cudaStream_t stream = nullptr;
  void* ptr = nullptr;
  size_t bytes = 0;
};
std::mutex g_scratch_mutex;
std::vector<ScratchSlot> g_scratch;

}  // namespace

void* acquire_scratch(int device, cudaStream_t s, size_t bytes, cudaError_t& err) {
  err = cudaSuccess;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  ScratchSlot* slot = nullptr;
  for (auto& e : g_scratch)
    if (e.device == device && e.stream == s) slot = &e;
  if (!slot) {
    g_scratch.push_back(ScratchSlot{device, s, nullptr, 0});
    slot = &g_scratch.back();
  }
  if (slot->bytes < bytes) {
    if (slot->ptr) {
      // earlier launches on this stream may still use the old buffer
      err = cudaStreamSynchronize(s);
      if (err != cudaSuccess) return nullptr;
      cudaFree(slot->ptr);
      slot->ptr = nullptr;
      slot->bytes = 0;
    }
    const size_t want = std::max(bytes, size_t(1) << 20);
    err = cudaMalloc(&slot->ptr, want);
    if (err != cudaSuccess) return nullptr;
    slot->bytes = want;
  }
  return slot->ptr;
}

int* acquire_counter(int device, cudaStream_t s, cudaError_t& err) {
  err = cudaSuccess;
  int* c = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_counter_mutex);
    const int d = device & 63;
    if (!g_counters[d]) {
      err = cudaMalloc(&g_counters[d], kCounters * kCounterInts * sizeof(int));
      if (err != cudaSuccess) return nullptr;
    }
    // launches in flight at the same time get different counters as long as
    // fewer than kCounters of them overlap
    c = g_counters[d] + (g_counter_next[d]++ % kCounters) * kCounterInts;
  }
  err = cudaMemsetAsync(c, 0, kCounterInts * sizeof(int), s);
  return err == cudaSuccess ? c : nullptr;
}

cudaError_t launch_batched_forward(const RenderParams* ps, int n, int filter, int tf_mode, int blend, int device,
                                   const LaunchInfo&, cudaStream_t s) {
  std::vector<int4> items = build_items(ps, n);
  if (items.empty()) return cudaSuccess;
  if (items.size() > 0x7fffffffu) return cudaErrorInvalidConfiguration;
  Workspace& w = g_ws[device & 63];
  std::lock_guard<std::mutex> lock(w.mutex);
  std::vector<size_t> offs;
  cudaError_t e = stage<int>(w, {{ps, sizeof(RenderParams) * n}, {items.data(), sizeof(int4) * items.size()}}, offs, s);
  if (e != cudaSuccess) return e;
  const RenderParams* dt = reinterpret_cast<const RenderParams*>(static_cast<char*>(w.dev) + offs[0]);
  const int4* di = reinterpret_cast<const int4*>(static_cast<char*>(w.dev) + offs[1]);
  const size_t smem = max_tf_entries(ps, n) * sizeof(float);
  const int ni = int(items.size()), vst = ps[0].vol_storage;
  switch (tf_mode) {
    case 0: return fwd_tf<0>(dt, di, ni, smem, vst, filter, blend, s);
    case 1: return fwd_tf<1>(dt, di, ni, smem, vst, filter, blend, s);
    case 2: return fwd_tf<2>(dt, di, ni, smem, vst, filter, blend, s);
    default: return fwd_tf<3>(dt, di, ni, smem, vst, filter, blend, s);
  }
}

cudaError_t launch_batched_adjoint(const RenderParams* ps, const AdjointParams* as, int n, int filter, int tf_mode,
                                   int blend, int device, const LaunchInfo&, cudaStream_t s) {
  std::vector<int4> items = build_items(ps, n);
  if (items.empty()) return cudaSuccess;
  if (items.size() > 0x7fffffffu) return cudaErrorInvalidConfiguration;
  Workspace& w = g_ws[device & 63];
  std::lock_guard<std::mutex> lock(w.mutex);
  std::vector<size_t> offs;
  cudaError_t e = stage<int>(w,
                             {{ps, sizeof(RenderParams) * n},
                              {as, sizeof(AdjointParams) * n},
                              {items.data(), sizeof(int4) * items.size()}},
                             offs, s);
  if (e != cudaSuccess) return e;
  const RenderParams* dt = reinterpret_cast<const RenderParams*>(static_cast<char*>(w.dev) + offs[0]);
  const AdjointParams* da = reinterpret_cast<const AdjointParams*>(static_cast<char*>(w.dev) + offs[1]);
  const int4* di = reinterpret_cast<const int4*>(static_cast<char*>(w.dev) + offs[2]);
  const bool tg = as[0].has_tf != 0, vg = as[0].has_volume != 0;
  size_t smem = 0;
  for (int i = 0; i < n; ++i) {
    const int seg = ps[i].ckpt.p ? ps[i].ckpt_interval : 0;
    smem = std::max(smem, fast_adjoint_smem(tf_mode, ps[i].R, ps[i].C, tg, seg));
  }
  const int ni = int(items.size()), vst = ps[0].vol_storage;
  switch (tf_mode) {
    case 0: return adj_tf<0>(dt, da, di, ni, smem, vst, filter, blend, vg, tg, s);
    case 1: return adj_tf<1>(dt, da, di, ni, smem, vst, filter, blend, vg, tg, s);
    case 2: return adj_tf<2>(dt, da, di, ni, smem, vst, filter, blend, vg, tg, s);
    default: return adj_tf<3>(dt, da, di, ni, smem, vst, filter, blend, vg, tg, s);
  }
}

}  // namespace dvr
