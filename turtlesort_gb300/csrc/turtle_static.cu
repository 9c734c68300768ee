// Allocation-free sort entry point: turtle_sort_device_noalloc.
//
// Some callers cannot allocate device memory at the time they need a sort:
// code that runs inside a host that owns a fixed device-memory pool and
// forbids further allocations after start-up, plugins that are handed device
// pointers but no allocator, and real-time loops that must not block on the
// allocator.  For them this entry point sorts keys (and ids) that the caller
// already holds in device memory using only a scratch area compiled into the
// library: a file-scope `static __device__` array of kStaticScratchBytes.
// Every GPU that loads the library holds that array until the process exits.
//
// Limits and rules:
//   * at most kStaticMaxElements keys per call (any of the eight dtypes, with
//     or without ids); larger calls return TURTLE_ERR_TOO_LARGE;
//   * all calls share the one array and it keeps the previous call's
//     contents; the work-list header is cleared at the start of every call.
//     Calls whose work overlaps on the GPU (several host threads, or several
//     streams) race on the array and corrupt each other's results;
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress (and prepares the kernels);
//   * the call waits for its own stream (the status words are read with one
//     copy ordered on that stream) and returns the device-side status;
//   * nothing here calls cudaMalloc, cudaFree or any other allocating routine.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstring>
#include <mutex>

#include "../../include/turtle_gb300.h"
#include "turtle_device.cuh"
#include "turtle_internal.h"
#include "turtle_layout.cuh"

namespace {

constexpr long long kStaticMaxElements = 1LL << 20;   // 1,048,576 keys per call
constexpr size_t kStaticScratchBytes = 16u << 20;     // 16 MiB per device

// Scratch for one sort: keys B | ids B | work lists (layout from make_layout).
static __device__ __align__(256) unsigned char g_turtle_scratch[kStaticScratchBytes];

struct DeviceState {
  bool ready = false;
  char* base = nullptr;    // device address of g_turtle_scratch on this device
  int grid[9][2] = {};     // cooperative grid per key width and id flag
};

constexpr int kMaxDevices = 64;
std::mutex g_mu;
DeviceState g_state[kMaxDevices];

struct Plan {
  turtle::WsLayout lay;
  size_t offIdx = 0, offWs = 0, bytes = 0;
};

Plan plan_for(int width) {
  Plan p;
  p.lay = turtle::make_layout(kStaticMaxElements, turtle::kernels_tile_elems(width),
                              turtle::kernels_leaf_max(width), 0, false);
  p.offIdx = turtle::align_up((size_t)kStaticMaxElements * width, 256);
  p.offWs = turtle::align_up(p.offIdx + (size_t)kStaticMaxElements * sizeof(int32_t), 256);
  p.bytes = p.offWs + p.lay.bytes;
  return p;
}

turtle_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return TURTLE_OK;
  cudaGetLastError();
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return TURTLE_ERR_NO_DEVICE;
  return TURTLE_ERR_CUDA;
}

// Once per device, with that device current: the scratch array's device
// address and the kernels' launch geometry.
turtle_status setup(int dev, DeviceState** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState& st = g_state[dev];
  if (!st.ready) {
    void* addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_turtle_scratch);
    if (e != cudaSuccess || addr == nullptr) return cuda_status(e != cudaSuccess ? e : cudaErrorUnknown);
    for (int w : {1, 2, 4, 8}) {
      if (plan_for(w).bytes > kStaticScratchBytes) return TURTLE_ERR_CAPACITY;
      for (int i = 0; i < 2; ++i) {
        e = turtle::kernels_prepare(w, i != 0, dev, &st.grid[w][i]);
        if (e != cudaSuccess) return cuda_status(e);
      }
    }
    st.base = (char*)addr;
    st.ready = true;
  }
  *out = &st;
  return TURTLE_OK;
}

}  // namespace

extern "C" turtle_status turtle_sort_device_noalloc(turtle_dtype dtype, void* d_keys,
                                                    int32_t* d_idx, int64_t n, void* stream) {
  const int width = turtle::dtype_width(dtype);
  if (width == 0 || n < 0 || (!d_keys && n > 0)) return TURTLE_ERR_INVALID_ARGUMENT;
  if (n > kStaticMaxElements) return TURTLE_ERR_TOO_LARGE;
  if (((uintptr_t)d_keys % 16) != 0 || ((uintptr_t)d_idx % 16) != 0) return TURTLE_ERR_ALIGNMENT;
  if (n < 2) return TURTLE_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  if (dev < 0 || dev >= kMaxDevices) return TURTLE_ERR_NO_DEVICE;
  DeviceState* st = nullptr;
  turtle_status ts = setup(dev, &st);
  if (ts != TURTLE_OK) return ts;
  const Plan p = plan_for(width);
  const bool hasIdx = d_idx != nullptr;
  cudaStream_t cs = (cudaStream_t)stream;
  // the compile-time defaults: the scratch array is laid out for them
  turtle::SortArgs a = turtle::bind_args(d_keys, d_idx, st->base, (int*)(st->base + p.offIdx),
                                         st->base + p.offWs, p.lay, nullptr, 0, n, dtype,
                                         turtle::kRuleAuto, turtle::tune_defaults(width, n));
  // the previous call's work-list header must not leak into this one
  if ((e = cudaMemsetAsync(a.ctrl, 0, sizeof(turtle::Control), cs)) != cudaSuccess)
    return cuda_status(e);
  for (int round = 0;; ++round) {
    e = turtle::kernels_launch_persistent(width, hasIdx, a, st->grid[width][hasIdx ? 1 : 0], cs);
    if (e != cudaSuccess) return cuda_status(e);
    // the status words (Control::error .. Control::yield) in one copy ordered
    // on the caller's stream, so the call waits for its own work only
    constexpr size_t kFrom = offsetof(turtle::Control, error);
    constexpr size_t kTo = offsetof(turtle::Control, yield) + sizeof(int);
    static_assert(kFrom < kTo, "error precedes yield in the control block");
    unsigned char words[kTo - kFrom];
    if ((e = cudaMemcpyAsync(words, (const unsigned char*)a.ctrl + kFrom, kTo - kFrom,
                             cudaMemcpyDeviceToHost, cs)) != cudaSuccess)
      return cuda_status(e);
    if ((e = cudaStreamSynchronize(cs)) != cudaSuccess) return cuda_status(e);
    int error = 0, yielded = 0;
    std::memcpy(&error, words, sizeof(int));
    std::memcpy(&yielded, words + (kTo - kFrom - sizeof(int)), sizeof(int));
    if (error == turtle::kDevTimeout) return TURTLE_ERR_TIMEOUT;
    if (error == turtle::kDevCapacity) return TURTLE_ERR_CAPACITY;
    if (error != 0) return TURTLE_ERR_CUDA;
    if (!yielded) return TURTLE_OK;
    if (round > 100000) return TURTLE_ERR_CAPACITY;
    a.resume = 1;  // the leaf lists filled up: continue from the saved level
  }
}

extern "C" int64_t turtle_noalloc_max_elements(void) { return kStaticMaxElements; }
