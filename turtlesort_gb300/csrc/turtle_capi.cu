// C ABI of the GB300 TurtleSort path (declared in include/turtle_gb300.h).
//
// A turtle_sorter is the GB300 counterpart of Turtle::TurtleSort<T,TrackIndex>
// (turtle-sort.cuh:31-283): it owns the device buffers (driver VMM memory, see
// turtle_vmm.cu), a private non-blocking stream, the work lists of the
// persistent sort kernel and a pinned status block.  Entry points return
// status codes; nothing calls exit().
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/turtle_gb300.h"
#include "turtle_device.cuh"
#include "turtle_internal.h"
#include "turtle_layout.cuh"
#include "turtle_tuning.h"

using turtle::DevBuffer;
using turtle::WsLayout;
using turtle::make_layout;
using turtle::dtype_width;
using turtle::dtype_flip;

namespace {

constexpr long long kMaxElements = (1LL << 31) - 1;  // int32 ids and in-segment offsets
// StartSorting of at least this many keys into pinned host buffers sorts the
// leaves in kMaxSlices position slices and copies each finished slice back
// while the later slices are still being sorted.
constexpr long long kOverlapMinKeys = 1LL << 22;

}  // namespace

struct turtle_sorter {
  int dtype = 0;
  int width = 0;
  unsigned long long flip = 0;
  long long maxN = 0;
  bool trackIdx = false;
  bool compressRequested = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  DevBuffer keysA, idxA, keysB, idxB, ws, offsets;
  DevBuffer idxC;  // late ids of StartSorting (allocated on first use)
  WsLayout lay;
  int grid[2] = {0, 0};
  turtle::Control* hctrl = nullptr;  // pinned status block
  // StartSorting / Sync state
  void* hostKeys = nullptr;
  int32_t* hostIdx = nullptr;
  long long n = 0;
  bool pending = false;
  std::chrono::steady_clock::time_point t0;
  std::atomic<long long> launches{0};
  int lastLevels = 0;
  std::string lastCuda;
  struct GraphEntry {
    void* keys; int32_t* idx; const long long* offs; long long num, total;
    cudaGraphExec_t exec;
  };
  std::vector<GraphEntry> graphs;
  std::mutex mu;
  // last persistent launch, for resuming a partition that yielded
  turtle::SortArgs lastArgs;
  bool lastHasIdx = false;
  bool lastValid = false;
  cudaStream_t lastStream = nullptr;
  int pivotRule = turtle::kRuleAuto;
  // overlapped device-to-host copies of StartSorting (pinned host buffers)
  cudaStream_t copyStream = nullptr;
  cudaEvent_t sliceEv[turtle::kMaxSlices] = {};
  bool overlapped = false;  // this StartSorting's result copies are queued on copyStream
  bool yielded = false;     // the partition yielded: those copies may be stale
  int leafYield = 0;        // test threshold for yields (0: default)
  long long barrierPolls = 0;  // test limit of the grid-barrier / look-back wait (0: default)
  long long radixStall = 0;    // test: radix tile + 1 that never publishes (0: none)
  // launch configuration: the tuned table (default), the compile-time
  // defaults, or one pinned configuration
  bool tuning = true;
  bool pinned = false;
  turtle::TuneParams pin = {};
  // optional kernel timing: events around the two launches of each sort
  static constexpr int kRing = 64;
  bool timeKernels = false;
  cudaEvent_t ev[kRing][4] = {};  // start, partition end, end, partition start
  int lastForm = turtle::kRuleAuto;  // form of the last enqueued sort
  long long timed = 0;
};

namespace {

turtle_status from_cuda(turtle_sorter* s, cudaError_t e) {
  if (e == cudaSuccess) return TURTLE_OK;
  if (s) s->lastCuda = cudaGetErrorString(e);
  cudaGetLastError();  // clear sticky-free errors
  if (e == cudaErrorMemoryAllocation) return TURTLE_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return TURTLE_ERR_NO_DEVICE;
  return TURTLE_ERR_CUDA;
}

#define TRY_CUDA(s, call)                               \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return from_cuda((s), e_);   \
  } while (0)

void free_graphs(turtle_sorter* s) {
  for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
  s->graphs.clear();
}

// The work lists are laid out for the smallest tile and leaf cut any
// configuration of this sorter can use (table entries up to max_n, with and
// without ids, and a pinned configuration).
turtle_status alloc_workspace(turtle_sorter* s, long long extraLeaves) {
  turtle::vmm_free(&s->ws);
  int ts0 = 0, lc0 = 0, ts1 = 0, lc1 = 0;
  turtle::tune_layout_bounds(s->width, false, s->maxN, &ts0, &lc0);
  turtle::tune_layout_bounds(s->width, true, s->maxN, &ts1, &lc1);
  int ts = ts0 < ts1 ? ts0 : ts1, lc = lc0 < lc1 ? lc0 : lc1;
  if (s->pinned) {
    const turtle::TuneParams p = turtle::tune_sanitize(s->width, s->pin);
    ts = p.tileShift < ts ? p.tileShift : ts;
    lc = p.leafCut < lc ? p.leafCut : lc;
  }
  s->lay = make_layout(s->maxN, 1 << ts, lc, extraLeaves, true, s->width);
  TRY_CUDA(s, turtle::vmm_alloc(&s->ws, s->lay.bytes, s->device, false));
  return TURTLE_OK;
}

turtle::TuneParams pick_params(turtle_sorter* s, bool hasIdx, long long n) {
  if (s->pinned) return s->pin;
  return s->tuning ? turtle::tune_lookup(s->width, hasIdx, n) : turtle::tune_defaults(s->width, n);
}

turtle::SortArgs make_args(turtle_sorter* s, void* keys, int32_t* idx, const long long* offs,
                           long long num, long long n, int slices = 1) {
  turtle::SortArgs a = turtle::bind_args(keys, idx, s->keysB.ptr, (int*)s->idxB.ptr,
                                         (char*)s->ws.ptr, s->lay, offs, num, n, s->dtype,
                                         s->pivotRule, pick_params(s, idx != nullptr, n));
  a.slices = slices;
  a.leafYield = s->leafYield;
  a.barrierPolls = s->barrierPolls;
  a.radixStall = s->radixStall;
  a.idxC = (int*)s->idxC.ptr;
  return a;
}

// Enqueue: reset the control block, run the persistent kernel, copy the
// control block to the pinned status block.
cudaError_t enqueue_persistent(turtle_sorter* s, const turtle::SortArgs& a, bool hasIdx,
                               cudaStream_t st, bool allowTiming = true,
                               const cudaEvent_t* keysReady = nullptr, int keyChunks = 0) {
  if (!a.resume) {
    cudaError_t e = cudaMemsetAsync(a.ctrl, 0, sizeof(turtle::Control), st);
    if (e != cudaSuccess) return e;
  }
  const bool timing = allowTiming && s->timeKernels;
  cudaEvent_t* ev = s->ev[s->timed % turtle_sorter::kRing];
  cudaError_t e = cudaSuccess;
  if (timing && (e = cudaEventRecord(ev[0], st)) != cudaSuccess) return e;
  const int full = s->grid[hasIdx ? 1 : 0];
  const int grid = full / (a.gridDiv > 0 ? a.gridDiv : 1);
  e = turtle::kernels_launch_persistent(s->width, hasIdx, a, grid > 0 ? grid : 1, st,
                                        timing ? ev[1] : nullptr,
                                        a.slices > 1 ? s->sliceEv : nullptr,
                                        timing ? ev[3] : nullptr, keysReady, keyChunks);
  if (e != cudaSuccess) return e;
  if (timing) {
    if ((e = cudaEventRecord(ev[2], st)) != cudaSuccess) return e;
    ++s->timed;
  }
  // partition + leaf launches, or the radix form's kernels
  s->launches.fetch_add(a.radix ? turtle::radix_launches(s->width) : 1 + a.slices);
  s->lastForm = a.radix ? turtle::kRuleRadix
                        : a.samples == turtle::kWideSamples ? turtle::kRuleTwoLevel
                        : a.samples == 3 ? turtle::kRuleReference : turtle::kRuleSampled;
  s->lastArgs = a;
  s->lastArgs.resume = 1;
  s->lastHasIdx = hasIdx;
  s->lastStream = st;
  s->lastValid = true;
  return cudaMemcpyAsync(s->hctrl, a.ctrl, sizeof(turtle::Control), cudaMemcpyDeviceToHost, st);
}

// After the stream of the last sort has been synchronized: if the partition
// yielded (its leaf lists filled up), relaunch it from the saved level until
// it completes.  Only pathological inputs ever take this path.
turtle_status finish_yields(turtle_sorter* s);

cudaStream_t pick_stream(turtle_sorter* s, void* stream) {
  return stream ? (cudaStream_t)stream : s->stream;
}

turtle_status check_idx(turtle_sorter* s, const int32_t* idx) {
  if (idx && !s->trackIdx) return TURTLE_ERR_INVALID_ARGUMENT;
  return TURTLE_OK;
}

turtle_status device_status(turtle_sorter* s) {
  turtle_status y = finish_yields(s);
  if (y != TURTLE_OK) return y;
  s->lastLevels = s->hctrl->levels;
  switch (s->hctrl->error) {
    case 0: return TURTLE_OK;
    case turtle::kDevTimeout: return TURTLE_ERR_TIMEOUT;
    case turtle::kDevCapacity: return TURTLE_ERR_CAPACITY;
    default: return TURTLE_ERR_CUDA;
  }
}

turtle_status finish_yields(turtle_sorter* s) {
  int rounds = 0;
  while (s->lastValid && s->hctrl->error == 0 && s->hctrl->yield != 0) {
    if (++rounds > 100000) return TURTLE_ERR_CAPACITY;
    s->yielded = true;
    TRY_CUDA(s, enqueue_persistent(s, s->lastArgs, s->lastHasIdx, s->lastStream));
    TRY_CUDA(s, cudaStreamSynchronize(s->lastStream));
  }
  return TURTLE_OK;
}

turtle_status sort_device_impl(turtle_sorter* s, void* keys, int32_t* idx, long long n,
                               cudaStream_t st, int slices = 1) {
  if (n < 2) return TURTLE_OK;
  const bool hasIdx = idx != nullptr;
  turtle::SortArgs a = make_args(s, keys, idx, nullptr, 0, n, slices);
  TRY_CUDA(s, enqueue_persistent(s, a, hasIdx, st));
  return TURTLE_OK;
}

bool host_pinned(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

// Result copies of StartSorting: after leaf launch sl, keys [lo, hi) of slice
// sl are final (the leaves of a slice start inside it), so copyStream brings
// them back while the later slices are sorted.
turtle_status queue_slice_copies(turtle_sorter* s, int slices) {
  const long long n = s->n;
  for (int sl = 0; sl < slices; ++sl) {
    const long long lo = (sl * n + slices - 1) / slices;
    const long long hi = ((sl + 1) * n + slices - 1) / slices;
    TRY_CUDA(s, cudaStreamWaitEvent(s->copyStream, s->sliceEv[sl], 0));
    if (hi <= lo) continue;
    TRY_CUDA(s, cudaMemcpyAsync((char*)s->hostKeys + lo * s->width,
                                (const char*)s->keysA.ptr + lo * s->width,
                                (size_t)(hi - lo) * s->width, cudaMemcpyDeviceToHost,
                                s->copyStream));
    if (s->hostIdx)
      TRY_CUDA(s, cudaMemcpyAsync(s->hostIdx + lo, (const int32_t*)s->idxA.ptr + lo,
                                  (size_t)(hi - lo) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                  s->copyStream));
  }
  return TURTLE_OK;
}

}  // namespace

extern "C" {

turtle_status turtle_create(turtle_dtype dtype, int64_t max_n, int track_index, int compress,
                            int device, turtle_sorter** out) {
  if (!out) return TURTLE_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const int width = dtype_width(dtype);
  if (width == 0 || max_n < 0) return TURTLE_ERR_INVALID_ARGUMENT;
  if (max_n > kMaxElements) return TURTLE_ERR_TOO_LARGE;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return TURTLE_ERR_NO_DEVICE;
  }
  if (device < 0) {
    if (cudaGetDevice(&device) != cudaSuccess) return TURTLE_ERR_NO_DEVICE;
  }
  if (device >= ndev) return TURTLE_ERR_INVALID_ARGUMENT;
  turtle_sorter* s = new turtle_sorter();
  s->dtype = dtype;
  s->width = width;
  s->flip = dtype_flip(dtype);
  s->maxN = max_n < 2 ? 2 : max_n;
  s->trackIdx = track_index != 0;
  s->compressRequested = compress != 0;
  s->device = device;
  auto fail = [&](turtle_status st) {
    turtle_destroy(s);
    return st;
  };
  if (cudaSetDevice(device) != cudaSuccess) return fail(TURTLE_ERR_NO_DEVICE);
  turtle_status st;
  cudaError_t e;
  const size_t kbytes = (size_t)s->maxN * width;
  const size_t ibytes = (size_t)s->maxN * sizeof(int32_t);
  if ((e = turtle::vmm_alloc(&s->keysA, kbytes, device, s->compressRequested)) != cudaSuccess)
    return fail(from_cuda(s, e));
  if ((e = turtle::vmm_alloc(&s->keysB, kbytes, device, s->compressRequested)) != cudaSuccess)
    return fail(from_cuda(s, e));
  if (s->trackIdx) {
    if ((e = turtle::vmm_alloc(&s->idxA, ibytes, device, s->compressRequested)) != cudaSuccess)
      return fail(from_cuda(s, e));
    if ((e = turtle::vmm_alloc(&s->idxB, ibytes, device, s->compressRequested)) != cudaSuccess)
      return fail(from_cuda(s, e));
  }
  if ((st = alloc_workspace(s, 0)) != TURTLE_OK) return fail(st);
  if ((e = cudaHostAlloc((void**)&s->hctrl, sizeof(turtle::Control), cudaHostAllocDefault)) !=
      cudaSuccess)
    return fail(from_cuda(s, e));
  std::memset(s->hctrl, 0, sizeof(turtle::Control));
  if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail(from_cuda(s, e));
  if ((e = cudaStreamCreateWithFlags(&s->copyStream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail(from_cuda(s, e));
  for (auto& ev : s->sliceEv)
    if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
      return fail(from_cuda(s, e));
  if ((e = turtle::kernels_prepare(width, false, device, &s->grid[0])) != cudaSuccess)
    return fail(from_cuda(s, e));
  if ((e = turtle::kernels_prepare(width, true, device, &s->grid[1])) != cudaSuccess)
    return fail(from_cuda(s, e));
  *out = s;
  return TURTLE_OK;
}

turtle_status turtle_destroy(turtle_sorter* s) {
  if (!s) return TURTLE_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->lastStream) cudaStreamSynchronize(s->lastStream);
  if (s->copyStream) cudaStreamSynchronize(s->copyStream);
  for (auto& ev : s->sliceEv)
    if (ev) { cudaEventDestroy(ev); ev = nullptr; }
  for (auto& r : s->ev)
    for (auto& e : r)
      if (e) { cudaEventDestroy(e); e = nullptr; }
  free_graphs(s);
  turtle::vmm_free(&s->keysA);
  turtle::vmm_free(&s->keysB);
  turtle::vmm_free(&s->idxA);
  turtle::vmm_free(&s->idxB);
  turtle::vmm_free(&s->idxC);
  turtle::vmm_free(&s->ws);
  turtle::vmm_free(&s->offsets);
  if (s->hctrl) cudaFreeHost(s->hctrl);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->copyStream) cudaStreamDestroy(s->copyStream);
  cudaGetLastError();
  delete s;
  return TURTLE_OK;
}

int turtle_compression_ok(const turtle_sorter* s) {
  return (s && s->keysA.compressed) ? 1 : 0;
}

// StartSorting with ids in pinned host memory under the radix form: the ids'
// host-to-device copy runs while the digit passes sort the keys with element
// positions as payload (the ids are not needed until the end), then one
// gather turns positions into ids; the keys' copy back overlaps the gather.
// The keys come in kKeyChunks chunks on the copy stream; the histogram of
// each chunk runs as soon as it is in, under the copy of the next.
// Stream order: keys in, chunk by chunk, then ids in (copy stream) |
// histogram chunks, plan, passes, finish -> keys out (copy stream) | wait ids
// in -> gather -> ids out (copy stream).
static turtle_status start_late_ids(turtle_sorter* s, void* host_keys, int32_t* host_idx,
                                     long long n) {
  constexpr int kKeyChunks = 4;
  static_assert(4 + kKeyChunks <= turtle::kMaxSlices, "the slice events hold both sets");
  cudaEvent_t* ev = s->sliceEv;  // ids in, keys final, ids final, sorter stream ready
  cudaEvent_t* chunkEv = s->sliceEv + 4;
  // the copy stream starts after whatever the sorter's stream holds
  TRY_CUDA(s, cudaEventRecord(ev[3], s->stream));
  TRY_CUDA(s, cudaStreamWaitEvent(s->copyStream, ev[3], 0));
  for (int c = 0; c < kKeyChunks; ++c) {
    const long long lo = c * n / kKeyChunks, hi = (c + 1) * n / kKeyChunks;
    TRY_CUDA(s, cudaMemcpyAsync((char*)s->keysA.ptr + lo * s->width,
                                (const char*)host_keys + lo * s->width, (size_t)(hi - lo) * s->width,
                                cudaMemcpyHostToDevice, s->copyStream));
    TRY_CUDA(s, cudaEventRecord(chunkEv[c], s->copyStream));
  }
  TRY_CUDA(s, cudaMemcpyAsync(s->idxC.ptr, host_idx, (size_t)n * sizeof(int32_t),
                              cudaMemcpyHostToDevice, s->copyStream));
  TRY_CUDA(s, cudaEventRecord(ev[0], s->copyStream));
  turtle::SortArgs a = make_args(s, s->keysA.ptr, (int32_t*)s->idxA.ptr, nullptr, 0, n);
  a.idsLate = 1;
  TRY_CUDA(s, enqueue_persistent(s, a, true, s->stream, true, chunkEv, kKeyChunks));
  TRY_CUDA(s, cudaEventRecord(ev[1], s->stream));
  TRY_CUDA(s, cudaStreamWaitEvent(s->copyStream, ev[1], 0));
  TRY_CUDA(s, cudaMemcpyAsync(host_keys, s->keysA.ptr, (size_t)n * s->width,
                              cudaMemcpyDeviceToHost, s->copyStream));
  TRY_CUDA(s, cudaStreamWaitEvent(s->stream, ev[0], 0));
  TRY_CUDA(s, turtle::kernels_launch_radix_gather(a, s->stream));
  s->launches.fetch_add(1);
  TRY_CUDA(s, cudaEventRecord(ev[2], s->stream));
  TRY_CUDA(s, cudaStreamWaitEvent(s->copyStream, ev[2], 0));
  TRY_CUDA(s, cudaMemcpyAsync(host_idx, s->idxA.ptr, (size_t)n * sizeof(int32_t),
                              cudaMemcpyDeviceToHost, s->copyStream));
  s->overlapped = true;
  s->pending = true;
  return TURTLE_OK;
}

turtle_status turtle_start(turtle_sorter* s, void* host_keys, int32_t* host_idx, int64_t n) {
  if (!s || (!host_keys && n > 0) || n < 0) return TURTLE_ERR_INVALID_ARGUMENT;
  if (n > s->maxN) return TURTLE_ERR_TOO_LARGE;
  turtle_status st = check_idx(s, host_idx);
  if (st != TURTLE_OK) return st;
  if (s->pending) return TURTLE_ERR_STATE;
  cudaSetDevice(s->device);
  s->t0 = std::chrono::steady_clock::now();
  s->hostKeys = host_keys;
  s->hostIdx = host_idx;
  s->n = n;
  std::memset(s->hctrl, 0, sizeof(turtle::Control));
  s->yielded = false;
  const bool pinned = n > 0 && host_pinned(host_keys) && (!host_idx || host_pinned(host_idx));
  if (host_idx && pinned && n >= kOverlapMinKeys &&
      make_args(s, s->keysA.ptr, (int32_t*)s->idxA.ptr, nullptr, 0, n).radix) {
    bool ready = s->idxC.ptr != nullptr;
    if (!ready) {  // the ids' landing buffer, once per sorter; without it, the plain path
      ready = turtle::vmm_alloc(&s->idxC, (size_t)s->maxN * sizeof(int32_t), s->device,
                                s->compressRequested) == cudaSuccess;
      cudaGetLastError();
    }
    if (ready) return start_late_ids(s, host_keys, host_idx, n);
  }
  if (n > 0) {
    TRY_CUDA(s, cudaMemcpyAsync(s->keysA.ptr, host_keys, (size_t)n * s->width,
                                cudaMemcpyHostToDevice, s->stream));
    if (host_idx)
      TRY_CUDA(s, cudaMemcpyAsync(s->idxA.ptr, host_idx, (size_t)n * sizeof(int32_t),
                                  cudaMemcpyHostToDevice, s->stream));
  }
  const int slices = (n >= kOverlapMinKeys && pinned) ? turtle::kMaxSlices : 1;
  st = sort_device_impl(s, s->keysA.ptr, host_idx ? (int32_t*)s->idxA.ptr : nullptr, n,
                        s->stream, slices);
  if (st != TURTLE_OK) return st;
  if (slices > 1) {
    if ((st = queue_slice_copies(s, slices)) != TURTLE_OK) return st;
    s->overlapped = true;
  }
  s->pending = true;
  return TURTLE_OK;
}

turtle_status turtle_sync(turtle_sorter* s, double* seconds) {
  if (!s) return TURTLE_ERR_INVALID_ARGUMENT;
  if (!s->pending) return TURTLE_ERR_STATE;
  cudaSetDevice(s->device);
  s->pending = false;
  TRY_CUDA(s, cudaStreamSynchronize(s->stream));
  turtle_status st = device_status(s);
  const bool overlapped = s->overlapped;
  s->overlapped = false;
  // the slice copies finish before any copy below (they may be stale after
  // a yield, and must not land on top of the final result)
  if (overlapped) TRY_CUDA(s, cudaStreamSynchronize(s->copyStream));
  if (st != TURTLE_OK) return st;
  if (s->n > 0 && (!overlapped || s->yielded)) {
    TRY_CUDA(s, cudaMemcpyAsync(s->hostKeys, s->keysA.ptr, (size_t)s->n * s->width,
                                cudaMemcpyDeviceToHost, s->stream));
    if (s->hostIdx)
      TRY_CUDA(s, cudaMemcpyAsync(s->hostIdx, s->idxA.ptr, (size_t)s->n * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, s->stream));
    TRY_CUDA(s, cudaStreamSynchronize(s->stream));
  }
  const auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - s->t0).count();
  s->hostKeys = nullptr;
  s->hostIdx = nullptr;
  return TURTLE_OK;
}

turtle_status turtle_multisort_device(turtle_sorter* s, void* d_keys, int32_t* d_idx,
                                      int64_t arr_size, int64_t num_arrays, void* stream) {
  if (!s || arr_size < 0 || num_arrays < 0 || (!d_keys && arr_size * num_arrays > 0))
    return TURTLE_ERR_INVALID_ARGUMENT;
  turtle_status st = check_idx(s, d_idx);
  if (st != TURTLE_OK) return st;
  if (arr_size > 0 && num_arrays > s->maxN / arr_size) return TURTLE_ERR_TOO_LARGE;
  if (arr_size < 2 || num_arrays == 0) return TURTLE_OK;
  cudaSetDevice(s->device);
  cudaStream_t cs = pick_stream(s, stream);
  // shared-memory geometry: the tuned one for this array length, if it holds
  // the arrays, else the smallest geometry that does
  int geom = s->tuning ? turtle::tune_multi_lookup(s->width, d_idx != nullptr, (int)arr_size) : -1;
  int cap = 0;
  if (geom >= 0) turtle::kernels_leaf_geometry(s->width, geom, nullptr, nullptr, &cap, nullptr);
  if (geom < 0 || arr_size > cap) {
    geom = -1;
    for (int g : {turtle::kDefaultLeafGeometry, 2}) {
      turtle::kernels_leaf_geometry(s->width, g, nullptr, nullptr, &cap, nullptr);
      if (arr_size <= cap) { geom = g; break; }
    }
  }
  if (geom >= 0) {
    TRY_CUDA(s, turtle::kernels_launch_multisort(s->width, d_idx != nullptr, d_keys, d_idx,
                                                 num_arrays, (int)arr_size, s->flip,
                                                 turtle::dtype_fbits(s->dtype), geom, cs));
    s->launches.fetch_add(1);
    std::memset(s->hctrl, 0, sizeof(turtle::Control));
    return TURTLE_OK;
  }
  // long arrays: batched persistent path with uniform offsets
  std::vector<long long> offs((size_t)num_arrays + 1);
  for (long long i = 0; i <= num_arrays; ++i) offs[(size_t)i] = i * arr_size;
  const size_t ob = offs.size() * sizeof(long long);
  if (s->offsets.bytes < ob) {
    TRY_CUDA(s, cudaStreamSynchronize(cs));
    turtle::vmm_free(&s->offsets);
    TRY_CUDA(s, turtle::vmm_alloc(&s->offsets, ob, s->device, false));
  }
  TRY_CUDA(s, cudaMemcpyAsync(s->offsets.ptr, offs.data(), ob, cudaMemcpyHostToDevice, cs));
  TRY_CUDA(s, cudaStreamSynchronize(cs));  // offs is a host temporary
  return turtle_sort_batched_device(s, d_keys, d_idx, (const int64_t*)s->offsets.ptr, num_arrays,
                                    arr_size * num_arrays, stream);
}

turtle_status turtle_multisort_idx(turtle_sorter* s, void* host_keys, int32_t* host_idx,
                                   int64_t arr_size, int64_t num_arrays, int block_size,
                                   double* seconds) {
  if (!s || arr_size < 0 || num_arrays < 0 || (!host_keys && arr_size * num_arrays > 0))
    return TURTLE_ERR_INVALID_ARGUMENT;
  turtle_status st = check_idx(s, host_idx);
  if (st != TURTLE_OK) return st;
  if (block_size > 0 && num_arrays % block_size != 0) return TURTLE_ERR_INVALID_ARGUMENT;
  if (arr_size > 0 && num_arrays > s->maxN / arr_size) return TURTLE_ERR_TOO_LARGE;
  if (s->pending) return TURTLE_ERR_STATE;
  cudaSetDevice(s->device);
  const auto t0 = std::chrono::steady_clock::now();
  const long long total = arr_size * num_arrays;
  const size_t bytes = (size_t)total * s->width;
  if (bytes > 0) {
    int32_t* dIdx = host_idx ? (int32_t*)s->idxA.ptr : nullptr;
    TRY_CUDA(s, cudaMemcpyAsync(s->keysA.ptr, host_keys, bytes, cudaMemcpyHostToDevice, s->stream));
    if (dIdx)
      TRY_CUDA(s, cudaMemcpyAsync(dIdx, host_idx, (size_t)total * sizeof(int32_t),
                                  cudaMemcpyHostToDevice, s->stream));
    st = turtle_multisort_device(s, s->keysA.ptr, dIdx, arr_size, num_arrays, s->stream);
    if (st != TURTLE_OK) return st;
    TRY_CUDA(s, cudaMemcpyAsync(host_keys, s->keysA.ptr, bytes, cudaMemcpyDeviceToHost, s->stream));
    if (dIdx)
      TRY_CUDA(s, cudaMemcpyAsync(host_idx, dIdx, (size_t)total * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, s->stream));
    TRY_CUDA(s, cudaStreamSynchronize(s->stream));
    st = device_status(s);
    if (st != TURTLE_OK) return st;
  }
  const auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  return TURTLE_OK;
}

turtle_status turtle_multisort(turtle_sorter* s, void* host_keys, int64_t arr_size,
                               int64_t num_arrays, int block_size, double* seconds) {
  return turtle_multisort_idx(s, host_keys, nullptr, arr_size, num_arrays, block_size, seconds);
}

turtle_status turtle_sort_device(turtle_sorter* s, void* d_keys, int32_t* d_idx, int64_t n,
                                 void* stream) {
  if (!s || n < 0 || (!d_keys && n > 0)) return TURTLE_ERR_INVALID_ARGUMENT;
  if (n > s->maxN) return TURTLE_ERR_TOO_LARGE;
  turtle_status st = check_idx(s, d_idx);
  if (st != TURTLE_OK) return st;
  if (((uintptr_t)d_keys % 16) != 0 || ((uintptr_t)d_idx % 16) != 0)
    return TURTLE_ERR_ALIGNMENT;
  cudaSetDevice(s->device);
  std::memset(s->hctrl, 0, sizeof(turtle::Control));
  return sort_device_impl(s, d_keys, d_idx, n, pick_stream(s, stream));
}

turtle_status turtle_sort_batched_device(turtle_sorter* s, void* d_keys, int32_t* d_idx,
                                         const int64_t* d_offsets, int64_t num, int64_t total,
                                         void* stream) {
  if (!s || num < 0 || total < 0 || (num > 0 && (!d_offsets || (!d_keys && total > 0))))
    return TURTLE_ERR_INVALID_ARGUMENT;
  if (total > s->maxN) return TURTLE_ERR_TOO_LARGE;
  turtle_status st = check_idx(s, d_idx);
  if (st != TURTLE_OK) return st;
  if (((uintptr_t)d_keys % 16) != 0 || ((uintptr_t)d_idx % 16) != 0 ||
      ((uintptr_t)d_offsets % 8) != 0)
    return TURTLE_ERR_ALIGNMENT;
  cudaSetDevice(s->device);
  std::memset(s->hctrl, 0, sizeof(turtle::Control));
  if (num == 0 || total < 2) return TURTLE_OK;
  cudaStream_t cs = pick_stream(s, stream);
  std::lock_guard<std::mutex> lk(s->mu);
  // every small array may become one leaf at once
  if ((long long)s->lay.leafCap < num + 16LL * (s->lay.segCap + 1) + 4096) {
    TRY_CUDA(s, cudaDeviceSynchronize());
    free_graphs(s);
    if ((st = alloc_workspace(s, num)) != TURTLE_OK) return st;
  }
  const bool hasIdx = d_idx != nullptr;
  for (auto& g : s->graphs) {
    if (g.keys == d_keys && g.idx == d_idx && g.offs == (const long long*)d_offsets &&
        g.num == num && g.total == total) {
      TRY_CUDA(s, cudaGraphLaunch(g.exec, cs));
      s->launches.fetch_add(2);
      s->lastArgs = make_args(s, d_keys, d_idx, (const long long*)d_offsets, num, total);
      s->lastArgs.resume = 1;
      s->lastHasIdx = hasIdx;
      s->lastStream = cs;
      s->lastValid = true;
      return TURTLE_OK;
    }
  }
  turtle::SortArgs a = make_args(s, d_keys, d_idx, (const long long*)d_offsets, num, total);
  // capture memset + persistent kernel + status copy into a graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  TRY_CUDA(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t ce = enqueue_persistent(s, a, hasIdx, s->stream, false);
  s->launches.fetch_sub(2);  // counted when the graph is launched
  cudaError_t ee = cudaStreamEndCapture(s->stream, &graph);
  if (ce != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return from_cuda(s, ce); }
  if (ee != cudaSuccess) return from_cuda(s, ee);
  ee = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ee != cudaSuccess) return from_cuda(s, ee);
  if (s->graphs.size() >= 16) {
    cudaGraphExecDestroy(s->graphs.front().exec);
    s->graphs.erase(s->graphs.begin());
  }
  s->graphs.push_back({d_keys, d_idx, (const long long*)d_offsets, num, total, exec});
  TRY_CUDA(s, cudaGraphLaunch(exec, cs));
  s->launches.fetch_add(2);
  s->lastStream = cs;
  return TURTLE_OK;
}

turtle_status turtle_stream_status(turtle_sorter* s, void* stream) {
  if (!s) return TURTLE_ERR_INVALID_ARGUMENT;
  cudaSetDevice(s->device);
  TRY_CUDA(s, cudaStreamSynchronize(pick_stream(s, stream)));
  return device_status(s);
}

int64_t turtle_launch_count(const turtle_sorter* s) { return s ? s->launches.load() : 0; }

int turtle_last_levels(const turtle_sorter* s) { return s ? s->lastLevels : 0; }

int turtle_last_form(const turtle_sorter* s) { return s ? s->lastForm : -1; }

int64_t turtle_max_elements(turtle_dtype dtype, int track_index) {
  (void)track_index;
  return dtype_width(dtype) ? kMaxElements : 0;
}

int64_t turtle_smem_capacity(turtle_dtype dtype, int track_index) {
  (void)track_index;
  const int w = dtype_width(dtype);
  return w ? turtle::kernels_leaf_max(w) : 0;
}

const char* turtle_status_string(turtle_status st) {
  switch (st) {
    case TURTLE_OK: return "ok";
    case TURTLE_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TURTLE_ERR_TOO_LARGE: return "size above the sorter's capacity";
    case TURTLE_ERR_CUDA: return "CUDA error";
    case TURTLE_ERR_OUT_OF_MEMORY: return "out of memory";
    case TURTLE_ERR_TIMEOUT: return "device-side wait timed out";
    case TURTLE_ERR_CAPACITY: return "device work list capacity exceeded";
    case TURTLE_ERR_STATE: return "call out of order";
    case TURTLE_ERR_ALIGNMENT: return "misaligned device pointer";
    case TURTLE_ERR_NO_DEVICE: return "no CUDA device";
    case TURTLE_ERR_BUDGET: return "request larger than the memory budget";
    default: return "unknown status";
  }
}

const char* turtle_last_cuda_error(const turtle_sorter* s) {
  return s ? s->lastCuda.c_str() : "";
}

void turtle_debug_fail_allocations(int count) { turtle::vmm_inject_failures(count); }

void turtle_debug_fail_allocation_at(int k) { turtle::vmm_inject_failure_at(k); }

int turtle_debug_timeline(const turtle_sorter* s, uint64_t* ns, int32_t* info, int max) {
  if (!s || !s->hctrl) return 0;
  const int n = std::min(std::min(s->hctrl->tlCount, turtle::kTimeline), max - 1);
  if (n <= 0) return 0;
  for (int i = 0; i < n; ++i) {
    ns[i] = s->hctrl->tl[i];
    info[i] = s->hctrl->tlInfo[i];
  }
  ns[n] = s->hctrl->tEnd;
  info[n] = -2;
  return n + 1;
}

turtle_status turtle_set_pivot_rule(turtle_sorter* s, int rule) {
  if (!s || rule < turtle::kRuleReference || rule > turtle::kRuleRadix)
    return TURTLE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  free_graphs(s);  // captured launches hold the old rule
  s->pivotRule = rule;
  return TURTLE_OK;
}

turtle_status turtle_debug_time_kernels(turtle_sorter* s, int enable) {
  if (!s) return TURTLE_ERR_INVALID_ARGUMENT;
  cudaSetDevice(s->device);
  if (enable && !s->ev[0][0]) {
    for (auto& r : s->ev)
      for (auto& e : r) TRY_CUDA(s, cudaEventCreate(&e));
  }
  s->timeKernels = enable != 0;
  s->timed = 0;
  return TURTLE_OK;
}

int turtle_debug_kernel_times(turtle_sorter* s, int last, double* partition_ms, double* leaf_ms) {
  if (!s || !s->timeKernels || last <= 0) return 0;
  const long long n = std::min<long long>(std::min<long long>(last, s->timed), turtle_sorter::kRing);
  double pm = 0, lm = 0;
  for (long long k = s->timed - n; k < s->timed; ++k) {
    cudaEvent_t* ev = s->ev[k % turtle_sorter::kRing];
    float a = 0, b = 0;
    if (cudaEventSynchronize(ev[2]) != cudaSuccess || cudaEventElapsedTime(&a, ev[0], ev[1]) != cudaSuccess ||
        cudaEventElapsedTime(&b, ev[1], ev[2]) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    pm += a;
    lm += b;
  }
  if (partition_ms) *partition_ms = pm;
  if (leaf_ms) *leaf_ms = lm;
  return (int)n;
}

int turtle_debug_pass_times(turtle_sorter* s, int last, double* setup_ms, double* pass_ms) {
  if (!s || !s->timeKernels || last <= 0) return 0;
  const long long n = std::min<long long>(std::min<long long>(last, s->timed), turtle_sorter::kRing);
  double su = 0, pm = 0;
  for (long long k = s->timed - n; k < s->timed; ++k) {
    cudaEvent_t* ev = s->ev[k % turtle_sorter::kRing];
    float a = 0, b = 0;
    if (cudaEventSynchronize(ev[2]) != cudaSuccess || cudaEventElapsedTime(&a, ev[0], ev[3]) != cudaSuccess ||
        cudaEventElapsedTime(&b, ev[3], ev[1]) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    su += a;
    pm += b;
  }
  if (setup_ms) *setup_ms = su;
  if (pass_ms) *pass_ms = pm;
  return (int)n;
}

int turtle_debug_error_site(const turtle_sorter* s, int* site, int* block, int* info) {
  if (!s || !s->hctrl) return 0;
  if (site) *site = s->hctrl->errSite;
  if (block) *block = s->hctrl->errBlock;
  if (info) *info = s->hctrl->errInfo;
  return s->hctrl->error;
}

turtle_status turtle_debug_yield_threshold(turtle_sorter* s, int32_t leaves) {
  if (!s || leaves < 0) return TURTLE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  s->leafYield = leaves;
  free_graphs(s);  // captured launches carry the old threshold
  return TURTLE_OK;
}

turtle_status turtle_debug_barrier_polls(turtle_sorter* s, int64_t polls) {
  if (!s || polls < 0) return TURTLE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  s->barrierPolls = polls;
  free_graphs(s);  // captured launches carry the old limit
  return TURTLE_OK;
}

turtle_status turtle_debug_radix_stall(turtle_sorter* s, int64_t tile) {
  if (!s) return TURTLE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  s->radixStall = tile < 0 ? 0 : tile + 1;
  return TURTLE_OK;
}

turtle_status turtle_set_tuning(turtle_sorter* s, int enable) {
  if (!s) return TURTLE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  s->tuning = enable != 0;
  free_graphs(s);  // captured launches carry the old configuration
  return TURTLE_OK;
}

turtle_status turtle_set_config(turtle_sorter* s, int form, int tile_shift, int leaf_geometry,
                                int leaf_cut, int grid_div) {
  if (!s) return TURTLE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  free_graphs(s);
  if (form < 0) {
    s->pinned = false;
    return TURTLE_OK;
  }
  if ((form != turtle::kRuleSampled && form != turtle::kRuleTwoLevel &&
       form != turtle::kRuleRadix) ||
      tile_shift < turtle::kMinTileShift || tile_shift > turtle::kMaxTileShift ||
      leaf_geometry < 0 || leaf_geometry >= turtle::kLeafGeometries ||
      (grid_div != 1 && grid_div != 2 && grid_div != 4))
    return TURTLE_ERR_INVALID_ARGUMENT;
  int cap = 0;
  turtle::kernels_leaf_geometry(s->width, leaf_geometry, nullptr, nullptr, &cap, nullptr);
  if (leaf_cut < turtle::kMinLeafCut || leaf_cut > cap) return TURTLE_ERR_INVALID_ARGUMENT;
  turtle::TuneParams p;
  p.form = form;  // TURTLE_FORM_RADIX: radix for plain sorts, two-level passes for batched ones
  p.tileShift = tile_shift;
  p.leafGeom = leaf_geometry;
  p.leafCut = leaf_cut;
  p.gridDiv = grid_div;
  p.radix = 0;
  p = turtle::tune_sanitize(s->width, p);
  const bool relayout = tile_shift < s->lay.tileShift || leaf_cut < s->lay.leafMax;
  s->pin = p;
  s->pinned = true;
  if (relayout) {
    cudaSetDevice(s->device);
    if (cudaDeviceSynchronize() != cudaSuccess) return from_cuda(s, cudaGetLastError());
    return alloc_workspace(s, 0);
  }
  return TURTLE_OK;
}

turtle_status turtle_tuning_lookup(turtle_dtype dtype, int track_index, int64_t n,
                                   int32_t* out6) {
  const int w = turtle::dtype_width(dtype);
  if (!w || !out6 || n < 0) return TURTLE_ERR_INVALID_ARGUMENT;
  const turtle::TuneParams p = turtle::tune_lookup(w, track_index != 0, n);
  out6[0] = p.form;
  out6[1] = p.tileShift;
  out6[2] = p.leafGeom;
  out6[3] = p.leafCut;
  out6[4] = p.gridDiv;
  out6[5] = p.radix;
  return TURTLE_OK;
}

int turtle_tuning_multisort_geometry(turtle_dtype dtype, int track_index, int64_t arr_size) {
  const int w = turtle::dtype_width(dtype);
  if (!w || arr_size < 0 || arr_size > (1LL << 30)) return -1;
  return turtle::tune_multi_lookup(w, track_index != 0, (int)arr_size);
}

const char* turtle_tuning_source(void) { return turtle::tune_source(); }

turtle_status turtle_debug_multisort_geometry(turtle_dtype dtype, void* d_keys, int32_t* d_idx,
                                              int64_t arr_size, int64_t num_arrays, int geometry,
                                              void* stream) {
  const int w = turtle::dtype_width(dtype);
  if (!w || arr_size < 0 || num_arrays < 0 || geometry < 0 ||
      geometry >= turtle::kLeafGeometries || (!d_keys && arr_size * num_arrays > 0))
    return TURTLE_ERR_INVALID_ARGUMENT;
  int cap = 0;
  turtle::kernels_leaf_geometry(w, geometry, nullptr, nullptr, &cap, nullptr);
  if (arr_size > cap) return TURTLE_ERR_TOO_LARGE;
  if (arr_size < 2 || num_arrays == 0) return TURTLE_OK;
  int dev = 0, grid = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return from_cuda(nullptr, cudaGetLastError());
  cudaError_t e = turtle::kernels_prepare(w, d_idx != nullptr, dev, &grid);
  if (e == cudaSuccess)
    e = turtle::kernels_launch_multisort(w, d_idx != nullptr, d_keys, d_idx, num_arrays,
                                         (int)arr_size, dtype_flip(dtype),
                                         turtle::dtype_fbits(dtype), geometry,
                                         (cudaStream_t)stream);
  return from_cuda(nullptr, e);
}

int turtle_leaf_geometry(turtle_dtype dtype, int geometry, int32_t* out4) {
  const int w = turtle::dtype_width(dtype);
  if (!w || !out4 || geometry < 0 || geometry >= turtle::kLeafGeometries) return 0;
  turtle::kernels_leaf_geometry(w, geometry, &out4[0], &out4[1], &out4[2], &out4[3]);
  return 1;
}

const char* turtle_version(void) { return "turtle-gb300 0.1 (sm_103a)"; }

}  // extern "C"
