// Serving loop: continuous batching of sort requests under an HBM budget.
//
// No reference counterpart: the reference sorts one array per
// StartSorting/Sync call (turtle-sort.cuh:124-258).  Here requests of mixed
// sizes and dtypes arrive at any time from any host thread.  A scheduler
// thread
//   * retires finished batches (their device memory returns to the budget);
//   * admits waiting requests while the HBM budget allows: the oldest waiting
//     request opens a batch, and every request of its (dtype, ids) group
//     within the first kWindow waiting requests joins it (in arrival order),
//     up to the batch limits -- one batched persistent launch with the arrays
//     packed back to back and an offsets array, exactly the
//     turtle_sort_batched_device form; requests of other groups keep their
//     place in the queue.  A request of at least kSoloKeys keys is sorted
//     alone, as a plain sort (radix form);
//   * keeps up to kSlots batches in flight as a pipeline of copy-in, sort and
//     copy-out streams, so one batch's copies overlap other batches' sorts.
//     Requests that arrive while batches are on the GPU join the next batch as
//     memory frees up.
// Sorts of different batches run on kSortStreams streams at once.  Each
// batch's partition kernel is a cooperative launch on 1/kSortStreams of the
// resident CTAs, so the partition grids of all streams fit on the GPU
// together whatever order their CTAs are dispatched in.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/turtle_gb300.h"
#include "turtle_device.cuh"
#include "turtle_internal.h"
#include "turtle_layout.cuh"

namespace {

constexpr int kSlots = 8;        // batches in flight
constexpr int kSortStreams = 2;  // batches sorting at once
constexpr int kWindow = 256;     // waiting requests scanned for a batch's group
// Requests of at least kSoloKeys keys are batches of their own: a plain sort,
// which takes the radix form where the tuned table says so (at 2^20 keys it
// sorts about 4x faster than a batched pivot sort of the same keys).
constexpr long long kSoloKeys = 1LL << 20;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t ticket = 0;
  int dtype = 0;
  int width = 0;
  void* hostKeys = nullptr;
  int32_t* hostIdx = nullptr;
  long long n = 0;
  double tSubmit = 0, tDone = 0;
  turtle_status status = TURTLE_OK;
  bool done = false;
  long long offset = 0;  // inside its batch
};

struct Batch {
  int slot = -1;
  int dtype = 0, width = 0;
  bool hasIdx = false;
  std::vector<Request*> reqs;
  long long total = 0;
  size_t bytes = 0;
  char* dev = nullptr;  // one stream-ordered allocation: keys | ids | keysB | idsB | offsets | ws
  turtle::WsLayout lay;
  turtle::SortArgs args;
  bool launched = false;
};

struct Slot {
  cudaEvent_t inDone = nullptr, sortDone = nullptr, outDone = nullptr;
  long long* hOffs = nullptr;          // pinned offsets staging
  turtle::Control* hCtrl = nullptr;    // pinned status block
  Batch* batch = nullptr;
};

}  // namespace

struct turtle_server {
  int device = 0;
  long long budget = 0;
  int maxBatchRequests = 4096;
  long long maxBatchKeys = 32ll << 20;
  cudaStream_t sIn = nullptr, sOut = nullptr;
  cudaStream_t sSort[kSortStreams] = {};
  cudaMemPool_t pool = nullptr;  // the server's own stream-ordered pool (keeps freed batches)
  int grid[9][2] = {};
  Slot slots[kSlots];
  std::mutex mu;
  std::condition_variable cv, cvDone;
  std::deque<Request*> waiting;
  std::unordered_map<uint64_t, Request*> all;
  std::vector<double> latencies;
  long long inUse = 0;
  uint64_t nextTicket = 1;
  long long submitted = 0, completed = 0, failed = 0, batches = 0, keysDone = 0;
  double tFirst = 0, tLast = 0;
  bool stop = false;
  std::thread worker;
  int inflight = 0;
};

namespace {

size_t batch_bytes(int width, bool hasIdx, long long total, long long num, turtle::WsLayout* layOut) {
  int ts = 0, lc = 0;  // laid out for the configuration the table gives this batch
  turtle::tune_layout_bounds(width, hasIdx, std::max(total, 2LL), &ts, &lc);
  // a batch of one request is a plain sort: room for the radix form too
  const turtle::WsLayout lay = turtle::make_layout(std::max(total, 2LL), 1 << ts, lc, num, true,
                                                   num == 1 ? width : 0);
  size_t b = 0;
  const size_t kb = turtle::align_up((size_t)total * width + 16, 256);
  const size_t ib = hasIdx ? turtle::align_up((size_t)total * 4 + 16, 256) : 0;
  b += 2 * kb + 2 * ib;
  b += turtle::align_up((size_t)(num + 1) * sizeof(long long), 256);
  b += lay.bytes;
  if (layOut) *layOut = lay;
  return b;
}

void fail_request(turtle_server* s, Request* r, turtle_status st) {
  r->status = st;
  r->done = true;
  r->tDone = now_s();
  s->failed++;
}

// Partition CTAs of a batch: at most 1/kSortStreams of the resident grid (so
// the cooperative grids of all sort streams are co-resident together), less
// when the tuned configuration asks for a smaller grid.
int batch_grid(const turtle_server* s, const Batch* b) {
  const int full = s->grid[b->width][b->hasIdx ? 1 : 0];
  const int div = std::max(kSortStreams, b->args.gridDiv > 0 ? b->args.gridDiv : 1);
  return std::max(1, full / div);
}

// Launch a formed batch into slot `slot` (called with the lock released: the
// batch and slot are owned by the worker thread).
turtle_status launch_batch(turtle_server* s, Batch* b) {
  Slot& sl = s->slots[b->slot];
  const long long num = (long long)b->reqs.size();
  cudaError_t e = cudaMallocFromPoolAsync((void**)&b->dev, b->bytes, s->pool, s->sIn);
  if (e != cudaSuccess) { cudaGetLastError(); return TURTLE_ERR_OUT_OF_MEMORY; }
  const size_t kb = turtle::align_up((size_t)b->total * b->width + 16, 256);
  const size_t ib = b->hasIdx ? turtle::align_up((size_t)b->total * 4 + 16, 256) : 0;
  char* keys = b->dev;
  int* idx = b->hasIdx ? (int*)(b->dev + kb) : nullptr;
  char* keysB = b->dev + kb + ib;
  int* idxB = b->hasIdx ? (int*)(b->dev + 2 * kb + ib) : nullptr;
  long long* offs = (long long*)(b->dev + 2 * kb + 2 * ib);
  char* ws = b->dev + 2 * kb + 2 * ib + turtle::align_up((size_t)(num + 1) * sizeof(long long), 256);
  // copy in: keys / ids packed back to back, then the offsets
  long long o = 0;
  for (long long i = 0; i < num; ++i) {
    Request* r = b->reqs[(size_t)i];
    r->offset = o;
    sl.hOffs[i] = o;
    if (r->n > 0) {
      cudaMemcpyAsync(keys + o * b->width, r->hostKeys, (size_t)r->n * b->width,
                      cudaMemcpyHostToDevice, s->sIn);
      if (b->hasIdx)
        cudaMemcpyAsync(idx + o, r->hostIdx, (size_t)r->n * 4, cudaMemcpyHostToDevice, s->sIn);
    }
    o += r->n;
  }
  sl.hOffs[num] = o;
  cudaMemcpyAsync(offs, sl.hOffs, (size_t)(num + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                  s->sIn);
  cudaEventRecord(sl.inDone, s->sIn);
  // sort
  // one request: a plain sort (the tuned form, radix included); else batched
  b->args = turtle::bind_args(keys, idx, keysB, idxB, ws, b->lay, num == 1 ? nullptr : offs,
                              num == 1 ? 0 : num, b->total, b->dtype, turtle::kRuleAuto,
                              turtle::tune_lookup(b->width, b->hasIdx, b->total));
  cudaStream_t ss = s->sSort[b->slot % kSortStreams];
  cudaStreamWaitEvent(ss, sl.inDone, 0);
  cudaMemsetAsync(b->args.ctrl, 0, sizeof(turtle::Control), ss);
  e = turtle::kernels_launch_persistent(b->width, b->hasIdx, b->args, batch_grid(s, b), ss);
  if (e != cudaSuccess) { cudaGetLastError(); return TURTLE_ERR_CUDA; }
  cudaMemcpyAsync(sl.hCtrl, b->args.ctrl, sizeof(turtle::Control), cudaMemcpyDeviceToHost, ss);
  cudaEventRecord(sl.sortDone, ss);
  // copy out
  cudaStreamWaitEvent(s->sOut, sl.sortDone, 0);
  for (Request* r : b->reqs) {
    if (r->n <= 0) continue;
    cudaMemcpyAsync(r->hostKeys, keys + r->offset * b->width, (size_t)r->n * b->width,
                    cudaMemcpyDeviceToHost, s->sOut);
    if (b->hasIdx)
      cudaMemcpyAsync(r->hostIdx, idx + r->offset, (size_t)r->n * 4, cudaMemcpyDeviceToHost,
                      s->sOut);
  }
  cudaEventRecord(sl.outDone, s->sOut);
  b->launched = true;
  return TURTLE_OK;
}

// Finish a batch whose copy-out event has fired (worker thread, no lock).
turtle_status finish_batch(turtle_server* s, Batch* b) {
  Slot& sl = s->slots[b->slot];
  turtle_status st = TURTLE_OK;
  // a partition that yielded (leaf lists full) continues here before the
  // results are trusted; pathological inputs only
  int rounds = 0;
  while (sl.hCtrl->error == 0 && sl.hCtrl->yield != 0) {
    if (++rounds > 100000) {
      st = TURTLE_ERR_CAPACITY;  // still yielding: the keys are only partly sorted
      break;
    }
    b->args.resume = 1;
    cudaStream_t ss = s->sSort[b->slot % kSortStreams];
    cudaError_t e = turtle::kernels_launch_persistent(b->width, b->hasIdx, b->args,
                                                      batch_grid(s, b), ss);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(sl.hCtrl, b->args.ctrl, sizeof(turtle::Control),
                          cudaMemcpyDeviceToHost, ss);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ss);
    if (e != cudaSuccess) {
      cudaGetLastError();
      st = TURTLE_ERR_CUDA;
      break;
    }
  }
  // the copy-out that ran before the relaunches read partly sorted keys:
  // copy the finished result again
  if (rounds > 0 && st == TURTLE_OK && sl.hCtrl->error == 0) {
    cudaError_t e = cudaSuccess;
    cudaStream_t ss = s->sSort[b->slot % kSortStreams];
    for (Request* r : b->reqs) {
      if (r->n <= 0 || e != cudaSuccess) continue;
      e = cudaMemcpyAsync(r->hostKeys, b->dev + r->offset * b->width, (size_t)r->n * b->width,
                          cudaMemcpyDeviceToHost, ss);
      if (e == cudaSuccess && b->hasIdx)
        e = cudaMemcpyAsync(r->hostIdx, (const int*)b->args.idxA + r->offset, (size_t)r->n * 4,
                            cudaMemcpyDeviceToHost, ss);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ss);
    if (e != cudaSuccess) {
      cudaGetLastError();
      st = TURTLE_ERR_CUDA;
    }
  }
  if (sl.hCtrl->error == turtle::kDevTimeout) st = TURTLE_ERR_TIMEOUT;
  else if (sl.hCtrl->error == turtle::kDevCapacity) st = TURTLE_ERR_CAPACITY;
  else if (sl.hCtrl->error != 0) st = TURTLE_ERR_CUDA;
  cudaFreeAsync(b->dev, s->sOut);
  b->dev = nullptr;
  return st;
}

void worker_loop(turtle_server* s) {
  cudaSetDevice(s->device);
  std::vector<Batch*> live(kSlots, nullptr);
  for (;;) {
    // 1. retire finished batches
    bool any = false;
    for (int k = 0; k < kSlots; ++k) {
      Batch* b = live[k];
      if (!b || cudaEventQuery(s->slots[k].outDone) != cudaSuccess) continue;
      const turtle_status st = finish_batch(s, b);
      const double t = now_s();
      {
        std::lock_guard<std::mutex> lk(s->mu);
        for (Request* r : b->reqs) {
          r->status = st;
          r->done = true;
          r->tDone = t;
          if (st == TURTLE_OK) {
            s->completed++;
            s->keysDone += r->n;
            s->latencies.push_back(r->tDone - r->tSubmit);
          } else {
            s->failed++;
          }
        }
        s->inUse -= (long long)b->bytes;
        s->inflight--;
        s->tLast = t;
      }
      s->cvDone.notify_all();
      delete b;
      live[k] = nullptr;
      any = true;
    }
    cudaGetLastError();
    // 2. admit and launch new batches
    for (int k = 0; k < kSlots; ++k) {
      if (live[k]) continue;
      Batch* b = nullptr;
      {
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->waiting.empty()) break;
        Request* head = s->waiting.front();
        const bool hasIdx = head->hostIdx != nullptr;
        b = new Batch();
        b->slot = k;
        b->dtype = head->dtype;
        b->width = head->width;
        b->hasIdx = hasIdx;
        // requests of the head's group among the first kWindow waiting ones,
        // in arrival order, within the batch limits; others keep their place.
        // A large head is sorted alone; large requests join no batch.
        const bool solo = head->n >= kSoloKeys;
        int scanned = 0;
        for (auto it = s->waiting.begin(); it != s->waiting.end() && scanned < kWindow; ++scanned) {
          Request* r = *it;
          if (r->dtype != b->dtype || (r->hostIdx != nullptr) != hasIdx ||
              (r != head && (solo || r->n >= kSoloKeys))) {
            ++it;
            continue;
          }
          if ((long long)b->reqs.size() >= s->maxBatchRequests) break;
          if (!b->reqs.empty() && b->total + r->n > s->maxBatchKeys) break;
          const size_t need = batch_bytes(b->width, hasIdx, b->total + r->n,
                                          (long long)b->reqs.size() + 1, nullptr);
          if ((long long)need + s->inUse > s->budget) {
            if (b->reqs.empty() && s->inflight == 0) {
              // can never fit, even on an idle GPU
              fail_request(s, r, TURTLE_ERR_BUDGET);
              it = s->waiting.erase(it);
              s->cvDone.notify_all();
              continue;
            }
            break;
          }
          b->reqs.push_back(r);
          b->total += r->n;
          it = s->waiting.erase(it);
          if (solo) break;
        }
        if (b->reqs.empty()) {
          delete b;
          b = nullptr;
          break;  // wait for memory
        }
        b->bytes = batch_bytes(b->width, hasIdx, b->total, (long long)b->reqs.size(), &b->lay);
        s->inUse += (long long)b->bytes;
        s->inflight++;
        s->batches++;
      }
      const turtle_status st = launch_batch(s, b);
      if (st != TURTLE_OK) {
        std::lock_guard<std::mutex> lk(s->mu);
        for (Request* r : b->reqs) fail_request(s, r, st);
        s->inUse -= (long long)b->bytes;
        s->inflight--;
        if (b->dev) cudaFreeAsync(b->dev, s->sIn);
        delete b;
        s->cvDone.notify_all();
        continue;
      }
      live[k] = b;
      any = true;
    }
    // 3. sleep until something can happen
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop && s->waiting.empty() && s->inflight == 0) break;
      if (!any) s->cv.wait_for(lk, std::chrono::microseconds(s->inflight ? 50 : 2000));
    }
  }
}

turtle_status from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return TURTLE_OK;
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return TURTLE_ERR_OUT_OF_MEMORY;
  return TURTLE_ERR_CUDA;
}

}  // namespace

extern "C" {

turtle_status turtle_server_create(int device, int64_t hbm_budget_bytes, int max_batch_requests,
                                   int64_t max_batch_keys, turtle_server** out) {
  if (!out || hbm_budget_bytes <= 0) return TURTLE_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return TURTLE_ERR_NO_DEVICE;
  }
  if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return TURTLE_ERR_NO_DEVICE;
  if (device >= ndev) return TURTLE_ERR_INVALID_ARGUMENT;
  turtle_server* s = new turtle_server();
  s->device = device;
  s->budget = hbm_budget_bytes;
  if (max_batch_requests > 0) s->maxBatchRequests = max_batch_requests;
  // one launch addresses its keys with 32-bit positions
  if (max_batch_keys > 0) s->maxBatchKeys = std::min<long long>(max_batch_keys, (1LL << 31) - 1);
  cudaSetDevice(device);
  cudaError_t e = cudaSuccess;
  for (int w : {1, 2, 4, 8})
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = turtle::kernels_prepare(w, i != 0, device, &s->grid[w][i]);
  if (e == cudaSuccess) {
    // a private pool whose freed blocks stay mapped up to the budget, so a
    // steady request stream does not map and unmap device memory per batch
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
      unsigned long long keep = (unsigned long long)hbm_budget_bytes;
      e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->sIn, cudaStreamNonBlocking);
  for (int k = 0; k < kSortStreams && e == cudaSuccess; ++k)
    e = cudaStreamCreateWithFlags(&s->sSort[k], cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->sOut, cudaStreamNonBlocking);
  for (int k = 0; k < kSlots && e == cudaSuccess; ++k) {
    Slot& sl = s->slots[k];
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.inDone, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.sortDone, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.outDone, cudaEventDisableTiming);
    if (e == cudaSuccess)
      e = cudaHostAlloc((void**)&sl.hOffs, (size_t)(s->maxBatchRequests + 1) * sizeof(long long),
                        cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&sl.hCtrl, sizeof(turtle::Control), cudaHostAllocDefault);
  }
  if (e != cudaSuccess) {
    turtle_server_destroy(s);
    return from_cuda(e);
  }
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return TURTLE_OK;
}

turtle_status turtle_server_submit(turtle_server* s, turtle_dtype dtype, void* host_keys,
                                   int32_t* host_idx, int64_t n, uint64_t* ticket) {
  if (!s || !ticket || n < 0 || (!host_keys && n > 0)) return TURTLE_ERR_INVALID_ARGUMENT;
  const int width = turtle::dtype_width(dtype);
  if (!width) return TURTLE_ERR_INVALID_ARGUMENT;
  if (n > (1LL << 31) - 1) return TURTLE_ERR_TOO_LARGE;
  Request* r = new Request();
  r->dtype = dtype;
  r->width = width;
  r->hostKeys = host_keys;
  r->hostIdx = host_idx;
  r->n = n;
  r->tSubmit = now_s();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->nextTicket++;
    s->all[r->ticket] = r;
    s->waiting.push_back(r);
    s->submitted++;
    if (s->submitted == 1) s->tFirst = r->tSubmit;
    *ticket = r->ticket;
  }
  s->cv.notify_all();
  return TURTLE_OK;
}

turtle_status turtle_server_poll(turtle_server* s, uint64_t ticket, int* done) {
  if (!s || !done) return TURTLE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return TURTLE_ERR_INVALID_ARGUMENT;
  *done = it->second->done ? 1 : 0;
  return TURTLE_OK;
}

turtle_status turtle_server_wait(turtle_server* s, uint64_t ticket, double* latency_seconds) {
  if (!s) return TURTLE_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return TURTLE_ERR_INVALID_ARGUMENT;
  Request* r = it->second;
  s->cvDone.wait(lk, [&] { return r->done; });
  if (latency_seconds) *latency_seconds = r->tDone - r->tSubmit;
  const turtle_status st = r->status;
  s->all.erase(it);
  delete r;
  return st;
}

turtle_status turtle_server_drain(turtle_server* s) {
  if (!s) return TURTLE_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cvDone.wait(lk, [&] { return s->waiting.empty() && s->inflight == 0; });
  return TURTLE_OK;
}

turtle_status turtle_server_get_stats(turtle_server* s, turtle_server_stats* out) {
  if (!s || !out) return TURTLE_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->batches = s->batches;
  out->keys = s->keysDone;
  std::vector<double> l = s->latencies;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) {
      const size_t i = (size_t)std::min<double>((double)l.size() - 1, p * (double)(l.size() - 1) + 0.5);
      return l[i];
    };
    double sum = 0;
    for (double x : l) sum += x;
    out->p50_ms = 1e3 * pct(0.50);
    out->p99_ms = 1e3 * pct(0.99);
    out->mean_ms = 1e3 * sum / (double)l.size();
    out->max_ms = 1e3 * l.back();
  }
  const double span = s->tLast - s->tFirst;
  out->span_s = span;
  out->keys_per_s = span > 0 ? (double)s->keysDone / span : 0.0;
  out->in_use_bytes = s->inUse;
  return TURTLE_OK;
}

turtle_status turtle_server_destroy(turtle_server* s) {
  if (!s) return TURTLE_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->device);
  if (s->sIn) cudaStreamSynchronize(s->sIn);
  for (cudaStream_t ss : s->sSort)
    if (ss) cudaStreamSynchronize(ss);
  if (s->sOut) cudaStreamSynchronize(s->sOut);
  for (int k = 0; k < kSlots; ++k) {
    Slot& sl = s->slots[k];
    if (sl.inDone) cudaEventDestroy(sl.inDone);
    if (sl.sortDone) cudaEventDestroy(sl.sortDone);
    if (sl.outDone) cudaEventDestroy(sl.outDone);
    if (sl.hOffs) cudaFreeHost(sl.hOffs);
    if (sl.hCtrl) cudaFreeHost(sl.hCtrl);
  }
  if (s->pool) cudaMemPoolDestroy(s->pool);
  if (s->sIn) cudaStreamDestroy(s->sIn);
  for (cudaStream_t ss : s->sSort)
    if (ss) cudaStreamDestroy(ss);
  if (s->sOut) cudaStreamDestroy(s->sOut);
  for (auto& kv : s->all) delete kv.second;
  cudaGetLastError();
  delete s;
  return TURTLE_OK;
}

}  // extern "C"
