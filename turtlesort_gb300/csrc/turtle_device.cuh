// Device-side building blocks of the GB300 TurtleSort path.
//
//  * key handling: the eight integer dtypes are sorted as unsigned words; a
//    signed key is mapped to its order-preserving unsigned image by flipping
//    the sign bit in registers on load and back on store (no extra pass).
//    1- and 2-byte keys are widened to 32 bits inside the kernels.
//  * work-list descriptors (segments, leaves, pivot-run fills) that replace the
//    reference's (start, stop) int task arrays (turtle-sort.cuh:41-46) and its
//    CDP task flip (turtle-sort.cu:35-111).
//  * a bounded grid barrier for the persistent cooperative kernel.
//  * the stable one-CTA shared-memory sort (register odd-even transposition +
//    merge-path merges) that replaces sortByNetwork (turtle-sort.cu:392-559)
//    and bruteSort (turtle-sort.cu:118-188).
#pragma once

#include <cuda/atomic>
#include <cstdint>

namespace turtle {

constexpr int kThreads = 512;            // CTA size of every sort kernel
constexpr int kWarps = kThreads / 32;
constexpr int kMinBlocks = 2;            // resident CTAs per SM we compile for
constexpr int kFillChunk = 1 << 16;      // pivot-run fill work unit (elements)
constexpr int kDepthSwitch = 48;         // levels of start/mid/stop pivots before
                                         // switching to sampled quartile pivots
constexpr int kMaxLevels = 4096;         // hard cap on partition levels
constexpr int kLeafClasses = 10;         // group sizes 1, 2, 4, ..., 512 threads
constexpr long long kSpinLimit = 40000000LL;  // bounded barrier spin iterations

// Device status words (match turtle_status in turtle_gb300.h)
constexpr int kDevOk = 0;
constexpr int kDevTimeout = 5;
constexpr int kDevCapacity = 6;

// Key width traits: KT is the in-kernel key word, kItems the elements per
// thread for both the partition tile and the shared-memory sort.
template <typename U> struct KeyCfg;
template <> struct KeyCfg<uint8_t> { using KT = uint32_t; static constexpr int kItems = 16; };
template <> struct KeyCfg<uint16_t> { using KT = uint32_t; static constexpr int kItems = 16; };
template <> struct KeyCfg<uint32_t> { using KT = uint32_t; static constexpr int kItems = 16; };
template <> struct KeyCfg<uint64_t> { using KT = uint64_t; static constexpr int kItems = 8; };

template <typename U>
struct Geom {
  using KT = typename KeyCfg<U>::KT;
  static constexpr int kItems = KeyCfg<U>::kItems;
  static constexpr int kTile = kThreads * kItems;       // partition tile = smem sort capacity
  static constexpr int kWarpChunk = 32 * kItems;        // elements per warp in a tile
  static constexpr int kKeyPadShift = sizeof(KT) == 8 ? 4 : 5;
  static constexpr int kKeySlots = kTile + (kTile >> kKeyPadShift) + 8;
  static constexpr int kIdxSlots = kTile + (kTile >> 5) + 8;
};

// Bank-conflict padding for shared-memory element arrays.
template <typename KT>
__device__ __forceinline__ int kpad(int p) {
  return p + (p >> (sizeof(KT) == 8 ? 4 : 5));
}
__device__ __forceinline__ int ipad(int p) { return p + (p >> 5); }

template <typename KT>
__device__ __forceinline__ KT key_max() {
  return ~KT(0);
}

// ---- work-list descriptors ----
struct SegDesc {        // a segment partitioned by the multi-CTA 3-pivot pass
  long long start;
  long long n;
  int tileBase;         // first entry in this level's tile arrays
  int ntiles;
  int done;             // count-phase tiles finished (last one plans)
  int pad;
};
struct LeafDesc {       // a segment finished by the shared-memory sort
  long long start;
  int n;
  int inB;              // 1: data lives in the scratch buffer, 0: in place
};
struct FillDesc {       // a pivot run parked in scratch: keys filled by value
  long long start;
  int n;
  int pad;
  unsigned long long value;  // unsigned image of the pivot key
};

struct Control {
  unsigned long long segTile[2];  // packed (segments << 32 | tiles) per level parity
  int leafCount;
  int fillCount;
  int classCount[16];
  int classFill[16];
  unsigned int work[4];           // ring of per-phase work counters
  unsigned int barCount;
  unsigned int barGen;
  int error;
  int levels;
  int pad[2];
};

struct SortArgs {
  void* keysA;            // input and final output
  int* idxA;
  void* keysB;            // scratch of the same size
  int* idxB;
  const long long* offsets;  // nullptr: one array of n elements
  long long numArrays;
  long long n;
  unsigned long long flip;   // sign-bit mask for signed dtypes (0 otherwise)
  SegDesc* segs[2];
  int* tileCnt[2];           // [tile][8] class counts
  long long* tileOff[2];     // [tile][8] global destination of each class
  LeafDesc* leaves;
  LeafDesc* leavesSorted;
  FillDesc* fills;
  int segCap, tileCap, leafCap, fillCap;
  Control* ctrl;
};

// ---- atomics / barrier ----
__device__ __forceinline__ unsigned ld_acquire(unsigned* p) {
  cuda::atomic_ref<unsigned, cuda::thread_scope_device> a(*p);
  return a.load(cuda::memory_order_acquire);
}
__device__ __forceinline__ int ld_acquire_int(int* p) {
  cuda::atomic_ref<int, cuda::thread_scope_device> a(*p);
  return a.load(cuda::memory_order_acquire);
}
__device__ __forceinline__ void set_error(Control* c, int code) {
  cuda::atomic_ref<int, cuda::thread_scope_device> a(c->error);
  int expected = 0;
  a.compare_exchange_strong(expected, code, cuda::memory_order_acq_rel);
}

// Grid-wide barrier for a cooperatively launched grid.  The spin is bounded:
// after kSpinLimit polls the CTA records kDevTimeout and leaves; a CTA also
// leaves as soon as any other CTA has recorded an error.  Returns true when
// no error is recorded.
__device__ __forceinline__ bool grid_barrier(Control* c) {
  __syncthreads();
  __shared__ int s_err;
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(c->barGen);
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> cnt(c->barCount);
    const unsigned g = gen.load(cuda::memory_order_acquire);
    const unsigned arrived = cnt.fetch_add(1u, cuda::memory_order_acq_rel) + 1u;
    if (arrived == gridDim.x) {
      cnt.store(0u, cuda::memory_order_relaxed);
      gen.store(g + 1u, cuda::memory_order_release);
    } else {
      long long it = 0;
      unsigned ns = 32;
      while (gen.load(cuda::memory_order_acquire) == g) {
        if (ld_acquire_int(&c->error) != 0) break;
        if (++it > kSpinLimit) {
          set_error(c, kDevTimeout);
          break;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
      }
    }
    s_err = ld_acquire_int(&c->error);
  }
  __syncthreads();
  return s_err == 0;
}

// Claim the next work item of a phase (CTA-uniform result).
__device__ __forceinline__ int claim_item(unsigned* ctr) {
  __shared__ int s_item;
  __syncthreads();
  if (threadIdx.x == 0) s_item = (int)atomicAdd(ctr, 1u);
  __syncthreads();
  return s_item;
}

// ---- key load/store with the sign flip ----
template <typename U, typename KT>
__device__ __forceinline__ KT kload(const U* p, long long i, KT flip) {
  return KT(p[i]) ^ flip;
}
template <typename U, typename KT>
__device__ __forceinline__ void kstore(U* p, long long i, KT v, KT flip) {
  p[i] = U(v ^ flip);
}

// Class of a key against sorted pivots p1 <= p2 <= p3, tested in the
// reference's order (turtle-sort.cu:688-718): ==p1, ==p2, ==p3, <p1, <p2, <p3.
// 0:<p1 1:==p1 2:(p1,p2) 3:==p2 4:(p2,p3) 5:==p3 6:>p3
template <typename KT>
__device__ __forceinline__ int classify(KT k, KT p1, KT p2, KT p3) {
  return (k == p1) ? 1 : (k == p2) ? 3 : (k == p3) ? 5 : (k < p1) ? 0 : (k < p2) ? 2 : (k < p3) ? 4 : 6;
}

// ---- stable one-CTA shared-memory sort ----
//
// The CTA is split into groups of P threads (P a power of two); group g sorts
// the kItems*P elements in smem[g*P*kItems, (g+1)*P*kItems) of the key and id
// arrays (unused tail slots hold key_max and come last, so real keys equal to
// key_max stay in front of them).  Each thread sorts kItems consecutive
// elements in registers by odd-even transposition (stable), then log2(P)
// rounds of merge-path merges (ties taken from the left run) produce the
// sorted group.  Results are left in shared memory.  All threads of the CTA
// must call it (it synchronizes).
template <typename KT, int kItems, bool kIdx>
__device__ __forceinline__ void block_sort_groups(KT* sk, int* si, int P) {
  const int tid = threadIdx.x;
  KT k[kItems];
  int v[kItems];
  const int base = tid * kItems;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    k[i] = sk[kpad<KT>(base + i)];
    if (kIdx) v[i] = si[ipad(base + i)];
  }
  // odd-even transposition: swap only on strict inversion -> stable
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
#pragma unroll
    for (int i = (r & 1); i + 1 < kItems; i += 2) {
      if (k[i + 1] < k[i]) {
        KT t = k[i]; k[i] = k[i + 1]; k[i + 1] = t;
        if (kIdx) { int u = v[i]; v[i] = v[i + 1]; v[i + 1] = u; }
      }
    }
  }
  const int lane_in_group = tid & (P - 1);
  const int group_first = tid - lane_in_group;
  for (int w = 1; w < P; w <<= 1) {
    // registers -> smem (blocked)
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      sk[kpad<KT>(base + i)] = k[i];
      if (kIdx) si[ipad(base + i)] = v[i];
    }
    __syncthreads();
    // merge runs of w threads pairwise: my pair starts at thread pf
    const int pair_lane = lane_in_group & (2 * w - 1);
    const int pf = tid - pair_lane;
    const int a0 = pf * kItems;
    const int len = w * kItems;
    const int b0 = a0 + len;
    const int diag = pair_lane * kItems;
    int lo = diag > len ? diag - len : 0;
    int hi = diag < len ? diag : len;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      // take more from A while A[mid] <= B[diag-1-mid]
      if (!(sk[kpad<KT>(b0 + diag - 1 - mid)] < sk[kpad<KT>(a0 + mid)])) lo = mid + 1;
      else hi = mid;
    }
    int ia = lo, ib = diag - lo;
    KT ka = ia < len ? sk[kpad<KT>(a0 + ia)] : key_max<KT>();
    KT kb = ib < len ? sk[kpad<KT>(b0 + ib)] : key_max<KT>();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const bool takeA = (ib >= len) || (ia < len && !(kb < ka));
      if (takeA) {
        k[i] = ka;
        if (kIdx) v[i] = si[ipad(a0 + ia)];
        ++ia;
        ka = ia < len ? sk[kpad<KT>(a0 + ia)] : key_max<KT>();
      } else {
        k[i] = kb;
        if (kIdx) v[i] = si[ipad(b0 + ib)];
        ++ib;
        kb = ib < len ? sk[kpad<KT>(b0 + ib)] : key_max<KT>();
      }
    }
  }
  (void)group_first;
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    sk[kpad<KT>(base + i)] = k[i];
    if (kIdx) si[ipad(base + i)] = v[i];
  }
  __syncthreads();
}

// Size class of a leaf: the smallest power-of-two thread group whose
// registers hold it (class c uses P = 1 << c threads).
template <int kItems>
__device__ __forceinline__ int leaf_class(int n) {
  int p = (n + kItems - 1) / kItems;
  int c = 0;
  while ((1 << c) < p) ++c;
  return c;
}

}  // namespace turtle
