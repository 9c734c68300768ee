// Internal declarations shared by the kernel and host translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace turtle {

struct SortArgs;

// ---- kernels (turtle_sort.cu) ----
// width = key bytes (1, 2, 4, 8); hasIdx = int32 payload present.
cudaError_t kernels_prepare(int width, bool hasIdx, int device, int* grid);
// Launches the partition kernel and the leaf kernel on `stream`; when `mid`
// is not null it is recorded between the two launches.
// Partition kernel, then a.slices leaf launches; sliceDone[s] (optional) is
// recorded after leaf launch s, when every key below slice s's end is final.
// passStart (optional) is recorded where the partition (or the radix form's
// digit passes) begins.  keysReady (radix form, optional): the keys arrive
// in keyChunks equal chunks, chunk c complete at event keysReady[c]; the
// histogram of each chunk starts when it has arrived.
cudaError_t kernels_launch_persistent(int width, bool hasIdx, const SortArgs& a, int grid,
                                      cudaStream_t stream, cudaEvent_t mid = nullptr,
                                      const cudaEvent_t* sliceDone = nullptr,
                                      cudaEvent_t passStart = nullptr,
                                      const cudaEvent_t* keysReady = nullptr, int keyChunks = 0);
// LSD radix form of a plain sort (a.radix == 1; turtle_radix.cu): histogram,
// plan, one pass per key byte, finish.  Same events as the partition path;
// every slice event is recorded at the end.
cudaError_t kernels_launch_radix(int width, bool hasIdx, const SortArgs& a, cudaStream_t stream,
                                 cudaEvent_t mid = nullptr, const cudaEvent_t* sliceDone = nullptr,
                                 cudaEvent_t passStart = nullptr,
                                 const cudaEvent_t* keysReady = nullptr, int keyChunks = 0);
// Kernel launches of one radix-form sort of `width`-byte keys.
int radix_launches(int width);
// Late ids (a.idsLate): idxA[i] = idxC[position of i], after the radix kernels
// and once the caller's ids are in idxC.
cudaError_t kernels_launch_radix_gather(const SortArgs& a, cudaStream_t stream);
cudaError_t kernels_launch_multisort(int width, bool hasIdx, void* keys, int* idx,
                                     long long numArrays, int arrSize, unsigned long long flip,
                                     int fbits, int geometry, cudaStream_t stream);
int kernels_tile_elems(int width);
int kernels_leaf_max(int width);
// Geometry g (0..3) of the leaf / MultiSort kernels for keys of `width` bytes.
void kernels_leaf_geometry(int width, int g, int* threads, int* items, int* capacity,
                           int* classes);

// ---- device buffers on the driver VMM API (turtle_vmm.cu) ----
// Replaces TurtleBuffer::Buffer (turtle-buffer.cuh:7-100) and
// QuickHelper::allocateCompressible/freeCompressible (quick-helper.cuh:39-127).
struct DevBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;        // requested
  size_t mapped = 0;       // rounded to the allocation granularity
  bool vmm = false;        // false: cudaMalloc fallback
  bool compressed = false; // generic compression really granted
};

// Allocates `bytes` on `device`.  want_compression asks for
// CU_MEM_ALLOCATION_COMP_GENERIC; if the device does not support it or the
// driver does not grant it, the buffer is allocated uncompressed.  Returns a
// CUDA error code (cudaSuccess on success).
cudaError_t vmm_alloc(DevBuffer* b, size_t bytes, int device, bool want_compression);
void vmm_free(DevBuffer* b);
bool vmm_compression_supported(int device);

// Test hook: make the next `count` VMM allocations fail (host-side fault
// injection; the buffer layer then reports cudaErrorMemoryAllocation).
void vmm_inject_failures(int count);
// Test hook: only the k-th device-buffer allocation from now on fails (k = 1:
// the next one); 0 cancels.
void vmm_inject_failure_at(int k);

}  // namespace turtle
