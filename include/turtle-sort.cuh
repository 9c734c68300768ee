// turtle-sort.cuh -- drop-in C++ host API of the GB300 TurtleSort sort path.
//
// Re-creates the reference's header-only API (tugrul512bit/TurtleSort,
// turtle-sort.cuh:31-283, turtle-globals.cuh:33-58) on top of the C ABI in
// turtle_gb300.h, so programs written against the reference compile and run
// unchanged:
//
//     #include "turtle-sort.cuh"
//     Turtle::TurtleSort<int> sorter(n, compress);
//     sorter.StartSorting(&values, &index);     // asynchronous
//     double seconds = sorter.Sync();
//     sorter.MultiSort<int, 1024, 32>(numArrays, hostPtr);
//
// This header is plain C++11 (g++ or nvcc); it includes no CUDA headers.
// Link with libturtle_gb300.so.
//
// Error behaviour matches the reference (turtle-globals.cuh:18-30): a failing
// call prints a message to stderr and exits with the status code.  Define
// TURTLE_THROW_ON_ERROR before including this header to get a
// Turtle::TurtleError exception instead.
#pragma once
#ifndef TURTLE_SORT_GB300_CUH
#define TURTLE_SORT_GB300_CUH

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "turtle_gb300.h"

namespace TurtleGlobals {

// Same semantics as the reference's RAII timer (turtle-globals.cuh:33-58):
// writes elapsed nanoseconds to *target on destruction, or prints seconds
// when target is null.
class Bench {
 public:
  explicit Bench(size_t* targetPtr) : target(targetPtr) {
    t1 = std::chrono::duration_cast<std::chrono::nanoseconds>(
        std::chrono::high_resolution_clock::now().time_since_epoch());
    t2 = t1;
  }
  ~Bench() {
    t2 = std::chrono::duration_cast<std::chrono::nanoseconds>(
        std::chrono::high_resolution_clock::now().time_since_epoch());
    if (target)
      *target = (size_t)(t2.count() - t1.count());
    else
      std::cout << static_cast<double>(t2.count() - t1.count()) / 1000000000.0 << " seconds"
                << std::endl;
  }

 private:
  size_t* target;
  std::chrono::nanoseconds t1, t2;
};

}  // namespace TurtleGlobals

namespace Turtle {

using TurtleGlobals::Bench;

class TurtleError : public std::runtime_error {
 public:
  TurtleError(turtle_status st, const std::string& what)
      : std::runtime_error(what), status(st) {}
  turtle_status status;
};

namespace detail {

inline void check(turtle_status st, const char* where, const turtle_sorter* s = nullptr) {
  if (st == TURTLE_OK) return;
  std::string msg = std::string("TurtleSort ") + where + ": " + turtle_status_string(st);
  if (s) {
    const char* c = turtle_last_cuda_error(s);
    if (c && *c) msg += std::string(" (") + c + ")";
  }
#ifdef TURTLE_THROW_ON_ERROR
  throw TurtleError(st, msg);
#else
  std::fprintf(stderr, "%s\n", msg.c_str());
  std::exit((int)st);
#endif
}

// Key type -> turtle_dtype.  char follows the platform's signedness; float
// and double sort in IEEE-754 totalOrder.
template <typename T, size_t S = sizeof(T), bool Signed = std::is_signed<T>::value>
struct dtype_of {
  static_assert(std::is_integral<T>::value && !std::is_same<T, bool>::value,
                "TurtleSort on GB300 sorts integer (int8 .. uint64), float and double keys");
};
template <> struct dtype_of<float, 4, true> { static const turtle_dtype value = TURTLE_FLOAT32; };
template <> struct dtype_of<double, 8, true> { static const turtle_dtype value = TURTLE_FLOAT64; };
template <typename T> struct dtype_of<T, 1, true> { static const turtle_dtype value = TURTLE_INT8; };
template <typename T> struct dtype_of<T, 1, false> { static const turtle_dtype value = TURTLE_UINT8; };
template <typename T> struct dtype_of<T, 2, true> { static const turtle_dtype value = TURTLE_INT16; };
template <typename T> struct dtype_of<T, 2, false> { static const turtle_dtype value = TURTLE_UINT16; };
template <typename T> struct dtype_of<T, 4, true> { static const turtle_dtype value = TURTLE_INT32; };
template <typename T> struct dtype_of<T, 4, false> { static const turtle_dtype value = TURTLE_UINT32; };
template <typename T> struct dtype_of<T, 8, true> { static const turtle_dtype value = TURTLE_INT64; };
template <typename T> struct dtype_of<T, 8, false> { static const turtle_dtype value = TURTLE_UINT64; };

}  // namespace detail

// Mirror of Turtle::TurtleSort<Type, TrackIndex> (turtle-sort.cuh:31-283).
template <typename Type, bool TrackIndex = true>
struct TurtleSort {
 public:
  // turtle-sort.cuh:63 -- device buffers for maxElements keys (+ ids).
  TurtleSort(int maxElements, bool optInCompression = false) : handle(nullptr) {
    detail::check(turtle_create(detail::dtype_of<Type>::value, (int64_t)maxElements,
                                TrackIndex ? 1 : 0, optInCompression ? 1 : 0, -1, &handle),
                  "constructor");
  }

  TurtleSort(const TurtleSort&) = delete;
  TurtleSort& operator=(const TurtleSort&) = delete;

  // turtle-sort.cuh:115
  bool MemoryCompressionSuccessful() { return turtle_compression_ok(handle) != 0; }

  // turtle-sort.cuh:124 -- starts sorting, returns immediately.  The vectors
  // must stay alive and unresized until Sync() returns.
  void StartSorting(std::vector<Type>* arrayToSort, std::vector<int>* indicesToTrack = nullptr) {
    int32_t* ids = nullptr;
    if (TrackIndex && indicesToTrack != nullptr) {
      if (indicesToTrack->size() != arrayToSort->size())
        detail::check(TURTLE_ERR_INVALID_ARGUMENT, "StartSorting (index size differs)");
      ids = reinterpret_cast<int32_t*>(indicesToTrack->data());
    }
    detail::check(turtle_start(handle, arrayToSort->data(), ids, (int64_t)arrayToSort->size()),
                  "StartSorting", handle);
  }

  // turtle-sort.cuh:188 -- waits, writes results back, returns seconds since
  // StartSorting (end to end, including both copies).
  double Sync() {
    double s = 0.0;
    detail::check(turtle_sync(handle, &s), "Sync", handle);
    return s;
  }

  // turtle-sort.cuh:265 -- sorts numArraysToSort arrays of ArrSize keys in
  // place; returns seconds including the copies.  BlockSize and
  // UseSharedMemory are accepted for source compatibility (the GB300 kernel
  // always sorts in shared memory); numArraysToSort must be a multiple of
  // BlockSize, as in the reference.
  template <typename MType, int ArrSize, int BlockSize = 32, bool UseSharedMemory = false>
  double MultiSort(const int numArraysToSort, MType* hostDataToSort) {
    static_assert(std::is_same<MType, Type>::value,
                  "MultiSort sorts the sorter's own key type (as the reference's buffers do)");
    double s = 0.0;
    detail::check(turtle_multisort(handle, hostDataToSort, (int64_t)ArrSize,
                                   (int64_t)numArraysToSort, BlockSize, &s),
                  "MultiSort", handle);
    return s;
  }

  // MultiSort with an id per key (not in the reference): hostIdx holds
  // numArraysToSort * ArrSize int ids, permuted with the keys, stably within
  // each array.  The sorter must track indices.
  template <typename MType, int ArrSize, int BlockSize = 32, bool UseSharedMemory = false>
  double MultiSort(const int numArraysToSort, MType* hostDataToSort, int* hostIdx) {
    static_assert(std::is_same<MType, Type>::value,
                  "MultiSort sorts the sorter's own key type (as the reference's buffers do)");
    double s = 0.0;
    detail::check(turtle_multisort_idx(handle, hostDataToSort, reinterpret_cast<int32_t*>(hostIdx),
                                       (int64_t)ArrSize, (int64_t)numArraysToSort, BlockSize, &s),
                  "MultiSort", handle);
    return s;
  }

  // Device-resident sort of n keys (and ids) already in device memory; the
  // stream is a cudaStream_t (nullptr = the sorter's own stream).
  void SortDevice(Type* dKeys, int* dIdx, int64_t n, void* stream = nullptr) {
    detail::check(turtle_sort_device(handle, dKeys, reinterpret_cast<int32_t*>(dIdx), n, stream),
                  "SortDevice", handle);
  }

  ~TurtleSort() { turtle_destroy(handle); }

  turtle_sorter* native() { return handle; }

 private:
  turtle_sorter* handle;
};

}  // namespace Turtle

#endif  // TURTLE_SORT_GB300_CUH
