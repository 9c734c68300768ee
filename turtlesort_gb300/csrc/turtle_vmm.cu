// Device buffers on the CUDA driver virtual-memory API.
//
// Replaces TurtleBuffer::Buffer (turtle-buffer.cuh:27-99) and the VMM helper
// QuickHelper::allocateCompressible / freeCompressible (quick-helper.cuh:57-127):
// physical memory is created with cuMemCreate (optionally with
// CU_MEM_ALLOCATION_COMP_GENERIC), a virtual range is reserved with
// cuMemAddressReserve, the two are mapped with cuMemMap and made read/write for
// the owning device with cuMemSetAccess.  Sizes are rounded to the allocation
// granularity.  Differences from the reference: failures are reported as
// status codes instead of exit(), a refused compression request falls back to
// uncompressed VMM memory (then to cudaMalloc) and the "compressed" flag
// reflects what the driver actually granted.
//
// The driver entry points are resolved at run time through
// cudaGetDriverEntryPointByVersion, so the library does not link libcuda and
// loads on machines without a driver.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <mutex>

#include "turtle_internal.h"

namespace turtle {
namespace {

struct DriverApi {
  PFN_cuMemGetAllocationGranularity_v10020 getGranularity = nullptr;
  PFN_cuMemAddressReserve_v10020 addressReserve = nullptr;
  PFN_cuMemAddressFree_v10020 addressFree = nullptr;
  PFN_cuMemCreate_v10020 create = nullptr;
  PFN_cuMemRelease_v10020 release = nullptr;
  PFN_cuMemMap_v10020 map = nullptr;
  PFN_cuMemUnmap_v10020 unmap = nullptr;
  PFN_cuMemSetAccess_v10020 setAccess = nullptr;
  PFN_cuMemGetAllocationPropertiesFromHandle_v10020 getProps = nullptr;
  PFN_cuDeviceGetAttribute_v2000 devAttr = nullptr;
  PFN_cuDeviceGet_v2000 devGet = nullptr;
  bool ok = false;
};

std::once_flag g_once;
DriverApi g_api;
std::atomic<int> g_inject{0};
std::atomic<int> g_injectAt{0};  // > 0: the allocation this many calls ahead fails

template <typename F>
bool resolve(const char* name, F* fn) {
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  void* p = nullptr;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || p == nullptr)
    return false;
  *fn = reinterpret_cast<F>(p);
  return true;
}

const DriverApi& api() {
  std::call_once(g_once, [] {
    DriverApi a;
    bool ok = true;
    ok &= resolve("cuMemGetAllocationGranularity", &a.getGranularity);
    ok &= resolve("cuMemAddressReserve", &a.addressReserve);
    ok &= resolve("cuMemAddressFree", &a.addressFree);
    ok &= resolve("cuMemCreate", &a.create);
    ok &= resolve("cuMemRelease", &a.release);
    ok &= resolve("cuMemMap", &a.map);
    ok &= resolve("cuMemUnmap", &a.unmap);
    ok &= resolve("cuMemSetAccess", &a.setAccess);
    ok &= resolve("cuMemGetAllocationPropertiesFromHandle", &a.getProps);
    ok &= resolve("cuDeviceGetAttribute", &a.devAttr);
    ok &= resolve("cuDeviceGet", &a.devGet);
    a.ok = ok;
    g_api = a;
  });
  return g_api;
}

// One VMM allocation attempt; returns false (and leaves nothing mapped) on
// any failure.
bool vmm_try(DevBuffer* b, size_t bytes, int device, bool compress) {
  const DriverApi& d = api();
  if (!d.ok) return false;
  CUdevice dev;
  if (d.devGet(&dev, device) != CUDA_SUCCESS) return false;
  CUmemAllocationProp prop;
  std::memset(&prop, 0, sizeof(prop));
  prop.type = CU_MEM_ALLOCATION_TYPE_PINNED;
  prop.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
  prop.location.id = dev;
  if (compress) prop.allocFlags.compressionType = CU_MEM_ALLOCATION_COMP_GENERIC;
  size_t gran = 0;
  if (d.getGranularity(&gran, &prop, CU_MEM_ALLOC_GRANULARITY_RECOMMENDED) != CUDA_SUCCESS ||
      gran == 0)
    return false;
  const size_t size = ((bytes + gran - 1) / gran) * gran;
  CUdeviceptr va = 0;
  if (d.addressReserve(&va, size, gran, 0, 0) != CUDA_SUCCESS) return false;
  CUmemGenericAllocationHandle h;
  if (d.create(&h, size, &prop, 0) != CUDA_SUCCESS) {
    d.addressFree(va, size);
    return false;
  }
  bool granted = false;
  if (compress) {
    CUmemAllocationProp got;
    std::memset(&got, 0, sizeof(got));
    if (d.getProps(&got, h) == CUDA_SUCCESS)
      granted = got.allocFlags.compressionType == CU_MEM_ALLOCATION_COMP_GENERIC;
  }
  if (d.map(va, size, 0, h, 0) != CUDA_SUCCESS) {
    d.release(h);
    d.addressFree(va, size);
    return false;
  }
  d.release(h);  // the mapping keeps the physical memory alive
  CUmemAccessDesc acc;
  std::memset(&acc, 0, sizeof(acc));
  acc.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
  acc.location.id = dev;
  acc.flags = CU_MEM_ACCESS_FLAGS_PROT_READWRITE;
  if (d.setAccess(va, size, &acc, 1) != CUDA_SUCCESS) {
    d.unmap(va, size);
    d.addressFree(va, size);
    return false;
  }
  b->ptr = reinterpret_cast<void*>(va);
  b->bytes = bytes;
  b->mapped = size;
  b->vmm = true;
  b->compressed = granted;
  return true;
}

}  // namespace

bool vmm_compression_supported(int device) {
  const DriverApi& d = api();
  if (!d.ok) return false;
  CUdevice dev;
  if (d.devGet(&dev, device) != CUDA_SUCCESS) return false;
  int v = 0;
  if (d.devAttr(&v, CU_DEVICE_ATTRIBUTE_GENERIC_COMPRESSION_SUPPORTED, dev) != CUDA_SUCCESS)
    return false;
  return v != 0;
}

void vmm_inject_failures(int count) { g_inject.store(count < 0 ? 0 : count); }

void vmm_inject_failure_at(int k) { g_injectAt.store(k < 0 ? 0 : k); }

cudaError_t vmm_alloc(DevBuffer* b, size_t bytes, int device, bool want_compression) {
  *b = DevBuffer();
  if (bytes == 0) bytes = 256;
  if (g_inject.load() > 0) {  // injected failure: nothing is allocated
    g_inject.fetch_sub(1);
    return cudaErrorMemoryAllocation;
  }
  if (g_injectAt.load() > 0 && g_injectAt.fetch_sub(1) == 1)
    return cudaErrorMemoryAllocation;  // the one chosen allocation fails
  if (want_compression && vmm_compression_supported(device) && vmm_try(b, bytes, device, true))
    return cudaSuccess;
  if (vmm_try(b, bytes, device, false)) return cudaSuccess;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return e;
  b->ptr = p;
  b->bytes = bytes;
  b->mapped = bytes;
  b->vmm = false;
  b->compressed = false;
  return cudaSuccess;
}

void vmm_free(DevBuffer* b) {
  if (b->ptr == nullptr) return;
  if (b->vmm) {
    const DriverApi& d = api();
    const CUdeviceptr va = reinterpret_cast<CUdeviceptr>(b->ptr);
    d.unmap(va, b->mapped);
    d.addressFree(va, b->mapped);
  } else {
    cudaFree(b->ptr);
  }
  *b = DevBuffer();
}

}  // namespace turtle
