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
//  * the stable one-CTA shared-memory sort (packed key/position words, a
//    register sorting network + merge-path merges) that replaces
//    sortByNetwork (turtle-sort.cu:392-559) and bruteSort
//    (turtle-sort.cu:118-188).
#pragma once

#include <cuda/atomic>
#include <climits>
#include <cstdint>
#include <type_traits>

namespace turtle {

#ifndef TURTLE_PART_THREADS
#define TURTLE_PART_THREADS 768
#endif
#ifndef TURTLE_PART_BLOCKS
#define TURTLE_PART_BLOCKS 1
#endif
constexpr int kThreads = TURTLE_PART_THREADS;  // CTA size of the partition kernel
constexpr int kWarps = kThreads / 32;
constexpr int kMinBlocks = TURTLE_PART_BLOCKS; // resident partition CTAs per SM we compile for
#ifndef TURTLE_PART_TILE
#define TURTLE_PART_TILE 2048
#endif
constexpr int kPartTile = TURTLE_PART_TILE;  // partition tile (keys), a power of two
constexpr int kLThreads = 512;           // CTA size of the default leaf / batched geometry
constexpr int kFillChunk = 1 << 16;      // pivot-run fill work unit (elements)
#ifndef TURTLE_DEPTH_SWITCH
#define TURTLE_DEPTH_SWITCH 48
#endif
constexpr int kDepthSwitch = TURTLE_DEPTH_SWITCH;  // levels of start/mid/stop pivots
                                         // before switching to sampled quartile pivots
constexpr int kMaxLevels = 4096;         // hard cap on partition levels
constexpr int kSamples = 31;             // evenly spaced pivot samples (one-level sampled rule)
constexpr int kWideSamples = 63;         // pivot samples of a segment in two-level passes
constexpr int kRow = 32;                 // per-tile row: 32 class counts / offsets / sample keys
constexpr int kMaxSlices = 8;
constexpr int kSmallPlanTiles = 64;      // segments this small are planned by one warp            // leaf phase split by position (one launch each)
constexpr long long kSpinLimit = 40000000LL;  // bounded barrier spin iterations
constexpr int kTimeline = 160;           // phase timestamps kept per launch

// Device status words (match turtle_status in turtle_gb300.h)
constexpr int kDevOk = 0;
constexpr int kDevTimeout = 5;
constexpr int kDevCapacity = 6;

// Key width traits: KT is the in-kernel key word, kItems the elements per
// thread for both the partition tile and the shared-memory sort.
template <typename U> struct KeyCfg;
// kItems: per thread in the partition kernel; kLItems: per thread in the
// shared-memory (leaf / batched) sort.
template <> struct KeyCfg<uint8_t> { using KT = uint32_t; static constexpr int kItems = 8, kLItems = 16; };
template <> struct KeyCfg<uint16_t> { using KT = uint32_t; static constexpr int kItems = 8, kLItems = 16; };
template <> struct KeyCfg<uint32_t> { using KT = uint32_t; static constexpr int kItems = 8, kLItems = 16; };
template <> struct KeyCfg<uint64_t> { using KT = uint64_t; static constexpr int kItems = 4, kLItems = 8; };

// Geometries of the shared-memory sort (leaf kernel and MultiSort kernel),
// selected at run time: CTA size x keys per thread.  kLItems (16 for keys of
// up to 32 bits, 8 for 64-bit keys) is the size of the register network;
// geometry 3 halves it, so an array gets twice the threads.
//   0: 256 threads x kLItems      (capacity 4096 / 2048)
//   1: 512 threads x kLItems      (capacity 8192 / 4096, the default)
//   2: 1024 threads x kLItems     (capacity 16384 / 8192)
//   3: 512 threads x kLItems / 2  (capacity 4096 / 2048)
constexpr int kLeafGeometries = 4;
constexpr int kDefaultLeafGeometry = 1;
template <typename U, int kV>
struct LeafGeom {
  static constexpr int kThreads = kV == 0 ? 256 : kV == 2 ? 1024 : 512;
  static constexpr int kItems = kV == 3 ? KeyCfg<U>::kLItems / 2 : KeyCfg<U>::kLItems;
  static constexpr int kMax = kThreads * kItems;
  static constexpr int kBlocks = 1024 / kThreads;  // resident CTAs per SM at 64 registers
  static constexpr int kClasses = kV == 0 ? 9 : kV == 2 ? 11 : 10;  // groups of 1 .. kThreads threads
};

template <typename U>
struct Geom {
  using KT = typename KeyCfg<U>::KT;
  static constexpr int kItems = KeyCfg<U>::kItems;
  static constexpr int kLItems = KeyCfg<U>::kLItems;
  static constexpr int kTile = kPartTile;               // partition tile
  static constexpr int kLeafMax = kLThreads * kLItems;  // capacity of the default leaf geometry
  static constexpr int kWarpChunk = 32 * kItems;        // elements per warp chunk
};

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
  unsigned long long samp[64]; // pivot samples (unsigned images): a[start+n/2], a[start],
                               // a[stop] under the reference rule, else evenly spaced
                               // keys (one-level) or up to kWideSamples keys (two-level)
  int nsamp;            // valid entries of samp (two-level passes)
  unsigned lut;         // class remap for equal pivots, set by the plan
  unsigned long long pivS[3];  // one-level: sorted pivots (unsigned images), set by the plan
  long long cbase[32];  // class boundaries after planning (one-level: 8, two-level: 32)
  int childSeg[16];     // next-level segments (one-level: 4 children, two-level: 16 grandchildren)
  alignas(16) int tot[32];  // class totals, summed by COUNT (zeroed with 16-byte stores)
  int planBase;         // first plan item of this segment
  unsigned parkMask;    // two-level: classes whose keys wait in B for a fill
};
// Sorted pivots and class table of one 3-pivot split (16 bytes for 32-bit
// keys: one shared-memory load).
template <typename KT>
struct alignas(16) PivotSet {
  KT p[3];
  unsigned lut;
};
// Pivots of a segment and of its four children (two-level passes).
template <typename KT>
struct WidePivots {
  PivotSet<KT> par;       // the segment's pivots
  PivotSet<KT> child[4];  // child ci's (parent classes 0, 2, 4, 6)
};
struct TileDesc {       // one partition tile: [lo, hi) of segment seg
  long long lo;
  long long hi;
  int seg;
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
  int planCount[2];               // plan items per level parity
  int planSmallCount[2];          // small segments (one warp plans each) per level parity
  int planMulti[2];               // 1: some segment of the level has several plan items
  unsigned int smallWork;         // small-segment plan counter of the current level
  int leafCount;
  int fillCount;
  int classCount[kMaxSlices * 16];  // leaves per (slice, size class)
  int classFill[kMaxSlices * 16];
  unsigned int work[4];           // ring of per-phase work counters
  unsigned int barCount;
  unsigned int barGen;
  int error;
  int levels;
  int tlCount;                    // timeline entries written (block 0)
  int finished;                   // CTAs that reached the end of the kernel
  int leafItems[kMaxSlices];      // leaf work items of each slice
  int fillItems;                  // parked pivot-run fills (done with slice 0)
  int classItemsG[kMaxSlices * 16];  // first item of each (slice, size class) in its slice
  int classOffG[kMaxSlices * 16];    // first sorted leaf of each (slice, size class)
  unsigned int leafWork[kMaxSlices];  // leaf-kernel work counter of each slice
  int leafDone;                   // leaf-kernel CTAs finished (all slices)
  int yield;                      // 1: partition stopped early to drain the leaf lists
  int resumeLevel;                // level to continue from after a yield
  int resumePhase;                // work-counter ring position at the yield
  int errSite;                    // which bounded wait or check recorded `error`
  int errBlock;                   // the CTA that recorded it
  int errInfo;                    // site-specific detail
  unsigned long long tEnd;        // globaltimer when the last CTA finished
  unsigned long long tl[kTimeline];  // globaltimer (ns) after each grid barrier
  int tlInfo[kTimeline];             // work items of the phase that just ended
};

// ---- LSD radix form (turtle_radix.cu) ----
// One pass per 8-bit digit; a pass CTA of kRadixThreads threads ranks a tile
// of kRadixThreads x radix_items(width) keys (4096, or 2048 for 64-bit keys).
// Measured on 2^26 int32 keys + ids: 1.76 ms with 256 x 16, 2.12 ms with
// 512 x 8 (more resident warps, but longer CTA barriers and half the threads
// idle in the per-digit steps); 256 x 12: 1.835 vs 1.669 ms; 256 x 24: 1.70
// vs 1.67 ms (0.198 vs 0.172 ms at 2^22).
// Large sorts of 8- to 32-bit keys without ids take kRadixWideItems keys a
// thread (6144-key tiles): 1.207 vs 1.305 ms for 2^26 uint32 keys, 0.396 vs
// 0.425 ms for uint8.  Below kRadixWideMinKeys (fewer tiles than a few waves
// of resident CTAs) the longer tiles were not measured to pay, and the
// 4096-key tiles stay.
constexpr int kRadixThreads = 256;
constexpr int kRadixBins = 256;
constexpr long long kRadixMaxN = (1LL << 31) - 2;  // look-back words hold prefix + 1 in 31 bits
constexpr int kRadixWideItems = 24;
constexpr long long kRadixWideMinKeys = 1LL << 24;
__host__ __device__ constexpr int radix_items(int width) { return width == 8 ? 8 : 16; }
// The smallest pass tile of a key width: look-back rows are sized and
// cleared for this many tiles, an upper bound for every pass.
__host__ __device__ constexpr int radix_tile(int width) { return kRadixThreads * radix_items(width); }

struct RadixCtl {
  int ord[8];            // rank of digit p among the digits that move keys (-1: skipped)
  unsigned tileCtr[8];   // tile claim counter of digit p's pass
  int active;            // digits that move keys
  int last;              // the last of them (-1: none)
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
  TileDesc* tiles[2];
  int* tileCnt[2];           // [tile][kRow]: one-level: #(k<p1), #(k<=p1), #(k<p2), #(k<=p2),
                             // #(k<p3), #(k<=p3), #keys; two-level: the 31 class counts
  long long* tileOff[2];     // [tile][kRow] global destination of each class
  int* planSmall[2];         // one-level passes: segments of at most kSmallPlanTiles tiles,
                             // each planned by one warp
  int* planSeg[2];           // segment of each plan item
  int* itemTot[2];           // [item][kRow] column sums of each plan item's count rows
  unsigned char* cls;        // two-level passes: class of each key, written by COUNT for SCATTER (kPartTile * kThreads keys)
  LeafDesc* leaves;
  LeafDesc* leavesSorted;
  FillDesc* fills;
  int segCap, tileCap, leafCap, fillCap, planCap;
  int resume;                // 1: continue a partition that yielded
  int slices;                // leaf launches, one per position slice (1..kMaxSlices)
  int fbits;                 // float keys (32 / 64): sorted as totalOrder images, else 0
  int leafYield;             // > 0: yield when more leaves are pending (testing)
  int samples;               // pivot samples per segment: 3 (reference rule, one-level
                             // passes) or kWideSamples (sampled rule, two-level passes)
  long long barrierPolls;    // > 0: grid-barrier poll limit (testing the timeout), else kSpinLimit
  int tileShift;             // partition tile = 1 << tileShift keys (10..12)
  int leafCut;               // segments of at most leafCut keys become leaves
  int leafItems;             // keys per thread of the leaf sort (size classes)
  int leafClasses;           // leaf size classes: thread groups of 1, 2, ..., 2^(leafClasses-1)
  int leafVariant;           // geometry of the leaf kernel (see kernels_leaf_geometry)
  int gridDiv;               // the partition kernel runs on (resident CTAs) / gridDiv CTAs
  Control* ctrl;
  int radix;                 // 1: LSD radix form (radix kernels instead of partition + leaf)
  int radixTiles;            // rows of each look-back region
  unsigned* radixHist;       // [key bytes][256] digit counts
  unsigned* radixBase;       // [key bytes][256] first output position of each digit
  RadixCtl* radixCtl;
  unsigned* radixStatus;     // [2][radixTiles][256] look-back words
  long long radixStall;      // testing: tile + 1 whose look-back words are never published (0: none)
  int* idxC;                 // late ids (radix form): the caller's ids, gathered after the passes
  int idsLate;               // 1: the passes carry element positions; radix_gather_kernel then
                             // writes idxA[i] = idxC[position of i]
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
// Error sites recorded with the first error (Control::errSite).
constexpr int kSiteBarrier = 1;    // grid_barrier spin limit
constexpr int kSiteBulk = 3;       // bulk-copy barrier wait limit
constexpr int kSiteCapacity = 4;   // a work list was full
constexpr int kSiteLookback = 5;   // radix look-back poll limit

__device__ __forceinline__ void set_error(Control* c, int code, int site = 0, int info = 0) {
  cuda::atomic_ref<int, cuda::thread_scope_device> a(c->error);
  int expected = 0;
  if (a.compare_exchange_strong(expected, code, cuda::memory_order_acq_rel)) {
    c->errSite = site;
    c->errBlock = (int)blockIdx.x;
    c->errInfo = info;
  }
}

// Grid-wide barrier for a cooperatively launched grid.  The spin is bounded:
// after `limit` polls (kSpinLimit unless a test lowers it) the CTA records
// kDevTimeout and leaves; a CTA also leaves as soon as any other CTA has
// recorded an error.  Returns true when no error is recorded.
__device__ __forceinline__ bool grid_barrier(Control* c, long long limit = kSpinLimit) {
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
        if (++it > limit) {
          set_error(c, kDevTimeout, kSiteBarrier, (int)g);
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

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Block 0 records a timestamp and a work-item count (phase timeline; read by
// the host for profiling).  Call right after a grid barrier.
__device__ __forceinline__ void timeline_mark(Control* c, int info) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int i = c->tlCount;
    if (i < kTimeline) {
      c->tl[i] = global_ns();
      c->tlInfo[i] = info;
      c->tlCount = i + 1;
    }
  }
}

// Asynchronous 4-byte global -> shared copy (Ampere+ cp.async); the issuing
// thread waits for its own copies with cp_async_wait_all().
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// ---- bulk asynchronous copies (TMA, non-tensor form) with an mbarrier ----
// One warp-private mbarrier tracks the bulk copies of one chunk: lane 0 arms it
// with the byte count and issues the copies; every lane then waits for the
// phase flip.  Both addresses and the size of a bulk copy must be multiples of
// 16 bytes; callers check this and fall back to plain loads otherwise.
constexpr long long kTmaSpinLimit = 1LL << 22;  // bounded mbarrier polls

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(m)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
// Orders this thread's earlier generic-proxy accesses (shared and global)
// before its later bulk copies: the copies read global data that other CTAs
// wrote before the last grid barrier and overwrite shared bytes this warp has
// just read.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async;\n" ::: "memory");
}
// The same for shared memory only (buffer reuse inside a warp).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arm(unsigned long long* m, unsigned bytes) {
  asm volatile(
      "{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(
          smem_u32(m)),
      "r"(bytes)
      : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* m) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(m))
      : "memory");
}
// Bounded wait for phase `parity` of the mbarrier; false after kTmaSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* m, unsigned parity) {
  const unsigned a = smem_u32(m);
  for (long long it = 0; it < kTmaSpinLimit; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
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

// ---- blocked tile I/O and cheap classification ----

// Thread-blocked chunk of a tile: elements [e0, e0 + kItems) relative to the
// tile base `tb` (absolute index tbAbs).  16-byte vector loads when the chunk
// lies inside the array (the tile base is 16-byte aligned because tiles start
// on absolute multiples of the tile size and the buffers are 16-byte
// aligned); per-element loads at the array end.  Elements outside [rlo, rhi)
// are masked out of the returned bit mask.
template <typename U, typename KT, int kItems>
__device__ __forceinline__ unsigned load_chunk(const U* tb, long long tbAbs, long long nTotal,
                                               int e0, int rlo, int rhi, KT flip, KT* key) {
  constexpr int kBytes = kItems * (int)sizeof(U);
  static_assert(kBytes % 8 == 0, "chunk must be whole 8-byte vectors");
  using V = typename std::conditional<kBytes % 16 == 0, uint4, uint2>::type;
  constexpr int kVec = kBytes / (int)sizeof(V);
  unsigned ok = 0;
#pragma unroll
  for (int i = 0; i < kItems; ++i) ok |= (e0 + i >= rlo && e0 + i < rhi) ? (1u << i) : 0u;
  if (ok == 0) return 0;
  if (tbAbs + e0 + kItems <= nTotal) {
    V v[kVec];
    const V* src = reinterpret_cast<const V*>(tb + e0);
#pragma unroll
    for (int j = 0; j < kVec; ++j) v[j] = __ldcg(src + j);
    const U* u = reinterpret_cast<const U*>(v);
#pragma unroll
    for (int i = 0; i < kItems; ++i) key[i] = KT(u[i]) ^ flip;
  } else {
#pragma unroll
    for (int i = 0; i < kItems; ++i) key[i] = (ok >> i & 1u) ? (KT(__ldcg(tb + e0 + i)) ^ flip) : KT(0);
  }
  return ok;
}

template <int kItems>
__device__ __forceinline__ void load_ids(const int* tb, long long tbAbs, long long nTotal, int e0,
                                         unsigned ok, int* id) {
  static_assert(kItems % 4 == 0, "ids are loaded as int4");
  if (ok == 0) return;
  if (tbAbs + e0 + kItems <= nTotal) {
    const int4* src = reinterpret_cast<const int4*>(tb + e0);
#pragma unroll
    for (int j = 0; j < kItems / 4; ++j) {
      const int4 v = __ldcg(src + j);
      id[4 * j] = v.x; id[4 * j + 1] = v.y; id[4 * j + 2] = v.z; id[4 * j + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < kItems; ++i) id[i] = (ok >> i & 1u) ? __ldcg(tb + e0 + i) : 0;
  }
}

// 7-class code of a key from comparison counts: 2 * #{pivots < k} +
// #{pivots == k}, remapped through a per-segment table for equal pivots so
// the classes follow the reference's test order (==p1, ==p2, ==p3 first).
__device__ __forceinline__ unsigned pivot_lut(bool eq12, bool eq23) {
  unsigned lut = 0u | 1u << 3 | 2u << 6 | 3u << 9 | 4u << 12 | 5u << 15 | 6u << 18;
  auto set = [&](int j, unsigned v) { lut = (lut & ~(7u << (3 * j))) | (v << (3 * j)); };
  if (eq12 && eq23) set(3, 1);
  else if (eq12) set(2, 1);
  else if (eq23) set(4, 3);
  return lut;
}
template <typename KT>
__device__ __forceinline__ int class_lut(KT k, KT p1, KT p2, KT p3, unsigned lut) {
  const int cp = (k > p1) + (k >= p1) + (k > p2) + (k >= p2) + (k > p3) + (k >= p3);
  return (int)((lut >> (3 * cp)) & 7u);
}

// ---- stable one-CTA shared-memory sort of packed words ----
//
// The shared-memory sort (leaves, MultiSort arrays) moves one word per key.
// With ids, the key is packed with its position in its array, so every word
// is distinct: any sorting network or merge then yields the stable order
// (ties by position), and each id is fetched once, by position, when the
// result is written out.  Without ids the word is the key itself (equal keys
// are indistinguishable, so stability does not arise).  Padding slots hold
// the largest word, which sorts behind every real one.
template <typename U, bool kIdx> struct LeafWord;

// 8- and 16-bit keys: (key << 16 | position), 32-bit words.
template <bool kIdx>
struct LeafWordNarrow {
  using W = uint32_t;
  __device__ __forceinline__ static W make(uint32_t k, int pos) {
    return kIdx ? (k << 16) | (uint32_t)pos : k;
  }
  __device__ __forceinline__ static uint32_t key(W w) { return kIdx ? w >> 16 : w; }
  __device__ __forceinline__ static int pos(W w) { return (int)(w & 0xFFFFu); }
  __device__ __forceinline__ static bool less(W a, W b) { return a < b; }
  __device__ __forceinline__ static W sent() { return ~0u; }
};
template <bool kIdx> struct LeafWord<uint8_t, kIdx> : LeafWordNarrow<kIdx> {};
template <bool kIdx> struct LeafWord<uint16_t, kIdx> : LeafWordNarrow<kIdx> {};

// 32-bit keys: the key alone, or (key << 32 | position).
template <>
struct LeafWord<uint32_t, false> {
  using W = uint32_t;
  __device__ __forceinline__ static W make(uint32_t k, int) { return k; }
  __device__ __forceinline__ static uint32_t key(W w) { return w; }
  __device__ __forceinline__ static int pos(W) { return 0; }
  __device__ __forceinline__ static bool less(W a, W b) { return a < b; }
  __device__ __forceinline__ static W sent() { return ~0u; }
};
template <>
struct LeafWord<uint32_t, true> {
  using W = unsigned long long;
  __device__ __forceinline__ static W make(uint32_t k, int pos) {
    return ((W)k << 32) | (uint32_t)pos;
  }
  __device__ __forceinline__ static uint32_t key(W w) { return (uint32_t)(w >> 32); }
  __device__ __forceinline__ static int pos(W w) { return (int)(uint32_t)w; }
  __device__ __forceinline__ static bool less(W a, W b) { return a < b; }
  __device__ __forceinline__ static W sent() { return ~0ull; }
};

// 64-bit keys: the key alone, or the key with its position beside it.
template <>
struct LeafWord<uint64_t, false> {
  using W = unsigned long long;
  __device__ __forceinline__ static W make(unsigned long long k, int) { return k; }
  __device__ __forceinline__ static unsigned long long key(W w) { return w; }
  __device__ __forceinline__ static int pos(W) { return 0; }
  __device__ __forceinline__ static bool less(W a, W b) { return a < b; }
  __device__ __forceinline__ static W sent() { return ~0ull; }
};
struct alignas(16) KeyPos64 {
  unsigned long long k;
  unsigned p;
};
template <>
struct LeafWord<uint64_t, true> {
  using W = KeyPos64;
  __device__ __forceinline__ static W make(unsigned long long k, int pos) {
    W w;
    w.k = k;
    w.p = (unsigned)pos;
    return w;
  }
  __device__ __forceinline__ static unsigned long long key(W w) { return w.k; }
  __device__ __forceinline__ static int pos(W w) { return (int)w.p; }
  __device__ __forceinline__ static bool less(W a, W b) {
    return a.k < b.k || (a.k == b.k && a.p < b.p);
  }
  __device__ __forceinline__ static W sent() {
    W w;
    w.k = ~0ull;
    w.p = ~0u;
    return w;
  }
};

// Range-packed words for arrays whose keys span a narrow range (the leaves of
// the partition lie between two pivots): the key minus the array's smallest
// key, shifted above a `sh`-bit position when there are ids (sh = log2 of
// the group's slot count, so every position fits).  Usable when
// max - min <= max_range(sh), which keeps every real word below the padding
// word.  Narrower words halve the ALU work of every compare and select in the
// network and the merges.
template <typename KT, typename Wt, bool kIdx>
struct RangeWord {
  using W = Wt;
  __host__ __device__ static constexpr unsigned long long max_range(int sh) {
    return (unsigned long long)(W(~W(0)) >> (kIdx ? sh : 0)) - (kIdx ? 1ull : 0ull);
  }
  __device__ __forceinline__ static W make(KT k, KT lo, int pos, int sh) {
    return kIdx ? (W(k - lo) << sh) | W((unsigned)pos) : W(k - lo);
  }
  __device__ __forceinline__ static KT key(W w, KT lo, int sh) {
    return lo + KT(kIdx ? w >> sh : w);
  }
  __device__ __forceinline__ static int pos(W w, int sh) {
    return kIdx ? (int)(w & W((1ull << sh) - 1ull)) : 0;
  }
  __device__ __forceinline__ static bool less(W a, W b) { return a < b; }
  __device__ __forceinline__ static W sent() { return W(~W(0)); }
};

// Adapter giving LeafWord the (key, lo) interface of RangeWord (lo unused).
template <typename U, bool kIdx>
struct FullWord : LeafWord<U, kIdx> {
  using Base = LeafWord<U, kIdx>;
  using W = typename Base::W;
  template <typename KT>
  __device__ __forceinline__ static W make(KT k, KT, int pos, int) { return Base::make(k, pos); }
  template <typename KT>
  __device__ __forceinline__ static KT key(W w, KT, int) { return (KT)Base::key(w); }
  __device__ __forceinline__ static int pos(W w, int) { return Base::pos(w); }
};

// Bank-conflict padding for word arrays: one spare slot per 128 bytes, so a
// thread's kItems consecutive words (blocked layout) start in another bank
// than its neighbour's.
template <typename W>
__device__ __forceinline__ int wpad(int p) {
  return p + p / (int)(128 / sizeof(W));
}
template <typename W>
constexpr int word_slots(int n) {
  return n + n / (int)(128 / sizeof(W)) + 8;
}

template <class LW>
__device__ __forceinline__ void cex(typename LW::W& a, typename LW::W& b) {
  const bool sw = LW::less(b, a);
  const typename LW::W lo = sw ? b : a;
  const typename LW::W hi = sw ? a : b;
  a = lo;
  b = hi;
}

// Batcher's odd-even merge sort of N register words (63 comparators for 16,
// 19 for 8; each list passes the 0-1 principle on all 2^N inputs).  The
// comparators are written out so every index is a literal and the words stay
// in registers.
template <class LW, int N> struct Network;
#define TURTLE_C(x, y) cex<LW>(v[x], v[y]);
template <class LW>
struct Network<LW, 4> {
  __device__ __forceinline__ static void sort(typename LW::W* v) {
    TURTLE_C(0,1) TURTLE_C(2,3) TURTLE_C(0,2) TURTLE_C(1,3) TURTLE_C(1,2)
  }
};
template <class LW>
struct Network<LW, 8> {
  __device__ __forceinline__ static void sort(typename LW::W* v) {
    TURTLE_C(0,1) TURTLE_C(2,3) TURTLE_C(4,5) TURTLE_C(6,7) TURTLE_C(0,2) TURTLE_C(1,3)
    TURTLE_C(4,6) TURTLE_C(5,7) TURTLE_C(1,2) TURTLE_C(5,6) TURTLE_C(0,4) TURTLE_C(1,5)
    TURTLE_C(2,6) TURTLE_C(3,7) TURTLE_C(2,4) TURTLE_C(3,5) TURTLE_C(1,2) TURTLE_C(3,4)
    TURTLE_C(5,6)
  }
};
template <class LW>
struct Network<LW, 16> {
  __device__ __forceinline__ static void sort(typename LW::W* v) {
    TURTLE_C(0,1) TURTLE_C(2,3) TURTLE_C(4,5) TURTLE_C(6,7) TURTLE_C(8,9) TURTLE_C(10,11)
    TURTLE_C(12,13) TURTLE_C(14,15) TURTLE_C(0,2) TURTLE_C(1,3) TURTLE_C(4,6) TURTLE_C(5,7)
    TURTLE_C(8,10) TURTLE_C(9,11) TURTLE_C(12,14) TURTLE_C(13,15) TURTLE_C(1,2) TURTLE_C(5,6)
    TURTLE_C(9,10) TURTLE_C(13,14) TURTLE_C(0,4) TURTLE_C(1,5) TURTLE_C(2,6) TURTLE_C(3,7)
    TURTLE_C(8,12) TURTLE_C(9,13) TURTLE_C(10,14) TURTLE_C(11,15) TURTLE_C(2,4) TURTLE_C(3,5)
    TURTLE_C(10,12) TURTLE_C(11,13) TURTLE_C(1,2) TURTLE_C(3,4) TURTLE_C(5,6) TURTLE_C(9,10)
    TURTLE_C(11,12) TURTLE_C(13,14) TURTLE_C(0,8) TURTLE_C(1,9) TURTLE_C(2,10) TURTLE_C(3,11)
    TURTLE_C(4,12) TURTLE_C(5,13) TURTLE_C(6,14) TURTLE_C(7,15) TURTLE_C(4,8) TURTLE_C(5,9)
    TURTLE_C(6,10) TURTLE_C(7,11) TURTLE_C(2,4) TURTLE_C(3,5) TURTLE_C(6,8) TURTLE_C(7,9)
    TURTLE_C(10,12) TURTLE_C(11,13) TURTLE_C(1,2) TURTLE_C(3,4) TURTLE_C(5,6) TURTLE_C(7,8)
    TURTLE_C(9,10) TURTLE_C(11,12) TURTLE_C(13,14)
#undef TURTLE_C
  }
};

// The CTA is split into groups of P threads (P a power of two); group g sorts
// the kItems*P words in sw[g*P*kItems, (g+1)*P*kItems) (addressed through
// wpad).  Each thread sorts its kItems consecutive words in registers, then
// log2(P) rounds of merge-path merges double the sorted runs; a round whose
// two runs lie inside one warp synchronizes that warp only.  Results are left
// in sw.  All threads of the CTA must call it; only threads below `active`
// (a multiple of P) touch the words.  `nReal` is the number of real words of
// the calling thread's group, in front of its padding: a thread whose kItems
// output slots all lie at or after nReal holds only padding after every
// round (padding sorts last), so it skips the network, the merges and the
// stores.
template <class LW, int kItems>
__device__ __forceinline__ void block_sort_words(typename LW::W* sw, int P, int active,
                                                 int nReal) {
  using W = typename LW::W;
  const int tid = threadIdx.x;
  const int lane_in_group = tid & (P - 1);
  const bool on = tid < active && lane_in_group * kItems < nReal;
  const int base = tid * kItems;
  W v[kItems];
  if (on) {
#pragma unroll
    for (int i = 0; i < kItems; ++i) v[i] = sw[wpad<W>(base + i)];
    Network<LW, kItems>::sort(v);
  }
  for (int w = 1; w < P; w <<= 1) {
    const bool inWarp = 2 * w <= 32;  // the pair of runs lies in one warp
    if (inWarp) __syncwarp(); else __syncthreads();
    if (on) {
#pragma unroll
      for (int i = 0; i < kItems; ++i) sw[wpad<W>(base + i)] = v[i];
    }
    if (inWarp) __syncwarp(); else __syncthreads();
    if (on) {
      // merge runs A = [a0, a0+len) and B = [b0, b0+len) of the pair; this
      // thread produces merged outputs [diag, diag + kItems)
      const int pair_lane = lane_in_group & (2 * w - 1);
      const int a0 = (tid - pair_lane) * kItems;
      const int len = w * kItems;
      const int b0 = a0 + len;
      const int diag = pair_lane * kItems;
      int lo = diag > len ? diag - len : 0;
      int hi = diag < len ? diag : len;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        // take more from A while A[mid] <= B[diag-1-mid] (ties from A: stable)
        if (!LW::less(sw[wpad<W>(b0 + diag - 1 - mid)], sw[wpad<W>(a0 + mid)])) lo = mid + 1;
        else hi = mid;
      }
      int ia = lo, ib = diag - lo;
      W a = ia < len ? sw[wpad<W>(a0 + ia)] : LW::sent();
      W b = ib < len ? sw[wpad<W>(b0 + ib)] : LW::sent();
#pragma unroll
      for (int i = 0; i < kItems; ++i) {
        const bool takeB = LW::less(b, a);
        v[i] = takeB ? b : a;
        ia += takeB ? 0 : 1;
        ib += takeB ? 1 : 0;
        if (i + 1 < kItems) {
          // one load: the next word of the run the output came from
          const int r = takeB ? ib : ia;
          const int at = takeB ? b0 + ib : a0 + ia;
          const W x = r < len ? sw[wpad<W>(at)] : LW::sent();
          a = takeB ? a : x;
          b = takeB ? x : b;
        }
      }
    }
  }
  if (P <= 32) __syncwarp(); else __syncthreads();
  if (on) {
#pragma unroll
    for (int i = 0; i < kItems; ++i) sw[wpad<W>(base + i)] = v[i];
  }
  __syncthreads();
}

// Size class of a leaf: the smallest power-of-two thread group whose
// registers hold it (class c uses P = 1 << c threads of `items` keys each).
__device__ __forceinline__ int leaf_class(int n, int items) {
  const int p = (n + items - 1) / items;
  int c = 0;
  while ((1 << c) < p) ++c;
  return c;
}

}  // namespace turtle
