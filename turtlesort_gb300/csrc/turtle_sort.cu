// GB300 TurtleSort kernels: the persistent work-list quicksort, the leaf
// kernel and the fixed-size batched (MultiSort) kernel.
//
// persistent_sort_kernel (replaces the CDP2 chain copyTasksBack ->
// resetNumTasks -> quickSortWithoutStreamCompaction / bruteSort,
// turtle-sort.cu:35-188,573-934): one cooperative launch of one CTA per SM
// walks the partition tree level by level.  Every level has three phases
// separated by a bounded grid barrier:
//   COUNT   one warp per tile (kTile keys of one segment, aligned to absolute
//           kTile boundaries) counts its keys against the segment's pivots
//           (six predicate totals per tile; class totals per segment).
//   PLAN    one CTA per plan item (kThreads tiles of one segment) turns the
//           per-tile totals into per-tile destination offsets (class order as
//           in turtle-sort.cu:755-761, then tiles in memory order: stable);
//           a segment's first item also routes its children (next-level
//           segments with their tiles, leaves, parked pivot runs;
//           turtle-sort.cu:857-933).
//   SCATTER one warp per tile, 256-key chunks prefetched into shared memory
//           by bulk asynchronous copies (TMA).  Per chunk the warp ranks the
//           keys stably per class (4-bit per-lane counters, one warp scan),
//           stages them by class in shared memory and writes each class run
//           coalesced to its destination in the other buffer.  Pivot runs are
//           written by value and never recursed into.  The warp whose chunk
//           holds a child's first, middle or last key reads it from the stage
//           and records it: those three keys are the child's pivots.
// Children live in the other buffer (ping-pong A <-> B), so there is no
// copy-back pass.  At the end the kernel buckets the leaves by size and hands
// them to leaf_kernel, which sorts them in shared memory (register network +
// merge-path merge) and fills the parked pivot runs.  If the leaf lists would
// overflow before the tree is done (pathological inputs only), the kernel
// yields: the host runs leaf_kernel and relaunches the partition from the
// saved level.
//
// Pivots are the reference's: sorted{a[start + n/2], a[start], a[stop]}
// (turtle-sort.cu:641-655).  From kDepthSwitch levels on, a segment's pivots
// are the quartiles of 31 evenly spaced samples instead, which bounds the
// depth on inputs built against median-of-3; the output does not depend on
// the pivots (every step is stable, so the result equals a stable sort by
// key).
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <cstdio>

#include "turtle_device.cuh"
#include "turtle_internal.h"

namespace turtle {

// Leaf size classes: class c uses P = 1 << c threads of the leaf CTA, each
// group sorted by the register network + merge-path merges (a shared-memory
// radix sort of the same leaves measured slower for every class on GB300).

constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }
#ifndef TURTLE_COUNT_RING
#define TURTLE_COUNT_RING 2
#endif
constexpr int kMaxRing = 8;  // deepest COUNT chunk ring (bulk-copy barriers per warp)
static_assert(TURTLE_COUNT_RING >= 2 && TURTLE_COUNT_RING <= kMaxRing, "COUNT ring depth");
constexpr unsigned kFull = 0xffffffffu;

template <typename U, bool kIdx>
struct Persist {
  using G = Geom<U>;
  using KT = typename G::KT;
  static constexpr int kItems = G::kItems;
  static constexpr int kWCH = G::kWarpChunk;
  static_assert(kWCH == 32 * kItems && kWCH <= 256, "stage slots are 8-bit");
  static_assert(kItems <= 8, "per-lane class counters are 4-bit");

  // One per warp: the chunk double buffer (bulk-copy destinations), the
  // class-ordered stage and the warp's destination tables.
  struct alignas(16) WarpArea {
    U pk[2][kWCH];                  // raw keys of the chunks in flight
    int pi[2][kIdx ? kWCH : 4];     // their ids
    KT sk[kWCH];                    // staged keys (class order)
    int si[kIdx ? kWCH : 4];        // staged ids
    unsigned char sc[kWCH];         // class of each stage slot
    alignas(16) unsigned char pc[2][kWCH];  // two-level SCATTER: class bytes of the chunks in flight
    struct OneLevel {               // tables of a one-level pass (7 classes)
      long long delta[8];           // destination minus stage slot, per class
      long long wbase[8];           // running destination per class
      long long cpos[4][32];        // children's pivot sample positions
      int cseg[4];                  // the child segments (-1: none)
    };
    struct TwoLevel {               // tables of a two-level pass (31 classes)
      long long delta[32];          // destination minus stage slot, per class
      long long wbase[32];          // running destination per class
      long long capP[32];           // next sample position of each grandchild class
      int cnt[32];                  // running count of each class in the chunk (ranking)
      int cs[32];                   // start of each class in the stage
      int capI[32];                 // index of that sample
      WidePivots<KT> wp;            // pivots of segment pivSeg
      KT q[16];                     // the same 15 pivots as one sorted sequence
      int pivSeg;
    };
    union {
      OneLevel o;
      TwoLevel t;
    };
    unsigned long long mbar[kMaxRing];  // bulk-copy completion barriers (one per slot)
  };
  // COUNT reads keys only: its chunk ring spans pk, pi, sk and si (contiguous)
  static constexpr int kChunkBytes = kWCH * (int)sizeof(U);
  static constexpr int kRingBytes = 2 * kWCH * (int)sizeof(U) + 2 * (kIdx ? kWCH : 4) * 4 +
                                    kWCH * (int)sizeof(KT) + (kIdx ? kWCH : 4) * 4;
  // two slots measured fastest on GB300 (a 1 KB bulk copy per warp with one in
  // flight streams at HBM speed; deeper rings streamed slower)
  static constexpr int kCountRing = TURTLE_COUNT_RING < kRingBytes / kChunkBytes
                                        ? TURTLE_COUNT_RING
                                        : kRingBytes / kChunkBytes;
  static_assert(kCountRing >= 2, "COUNT double-buffers at least");

  struct Smem {  // partition CTA
    WarpArea w[kWarps];
    int red[kWarps][8];
    int pre[8];
    int tot[8];
    int cbase[8];                   // class boundaries relative to the segment start
    int childSeg[4];
    int childTb[4], childNt[4];
    long long childStart[4], childN[4];
    KT piv[3];
    unsigned lut;
    int rowSum[kWarps][kRow];       // plan item totals: per-warp column sums
    int preAll[kRow];               // column sums of the item's segment before the item
    int classOff[kMaxSlices * 16];  // leaf buckets: (slice, size class)
    int classItems[kMaxSlices * 16];
    // two-level plan
    int wcb[33];                    // class starts relative to the segment
    int gSeg[16], gTb[16], gNt[16]; // the grandchild segments
    long long gStart[16], gN[16];
    WidePivots<KT> wpiv;
  };

};

// Shared memory of a leaf / MultiSort CTA of geometry kV.
template <typename U, bool kIdx, int kV>
struct LeafCfg {
  using LG = LeafGeom<U, kV>;
  using KT = typename KeyCfg<U>::KT;
  static constexpr int kThreads = LG::kThreads, kItems = LG::kItems, kMax = LG::kMax;
  static constexpr int kWarps = kThreads / 32;
  using LW = LeafWord<U, kIdx>;
  using LWord = typename LW::W;
  static constexpr size_t cmax(size_t x, size_t y) { return x > y ? x : y; }
  // the word buffer holds the full-range words, the range-packed 32-bit words,
  // for 64-bit keys with ids 64-bit words, and the raw keys while they load
  static constexpr size_t kWordBytes = cmax(
      cmax(sizeof(LWord) * (size_t)word_slots<LWord>(kMax), 4 * (size_t)word_slots<uint32_t>(kMax)),
      cmax((sizeof(U) == 8 && kIdx) ? 8 * (size_t)word_slots<uint64_t>(kMax) : 0,
           sizeof(KT) * (size_t)kMax));
  struct Smem {
    alignas(16) unsigned char wbytes[kWordBytes];  // packed key (+ position) words
    int idx[kIdx ? kMax + 8 : 4];                   // ids by position
    KT gmin[kWarps], gmax[kWarps];                  // per-warp key range of the loaded leaves
    KT glo[kThreads];                               // smallest key of each group's leaf
    int item;
    int classOff[16];
    int classItems[16];
    __device__ LWord* words() { return reinterpret_cast<LWord*>(wbytes); }
  };
};

template <typename U, bool kIdx>
struct RingLayoutCheck {
  using W = typename Persist<U, kIdx>::WarpArea;
  static_assert(offsetof(W, sc) - offsetof(W, pk) == (size_t)Persist<U, kIdx>::kRingBytes,
                "the COUNT ring spans pk, pi, sk and si without padding");
  static_assert(offsetof(W, pk) % 16 == 0 && Persist<U, kIdx>::kChunkBytes % 16 == 0,
                "bulk-copy destinations are 16-byte aligned");
};
template struct RingLayoutCheck<uint8_t, false>;
template struct RingLayoutCheck<uint8_t, true>;
template struct RingLayoutCheck<uint16_t, false>;
template struct RingLayoutCheck<uint16_t, true>;
template struct RingLayoutCheck<uint32_t, false>;
template struct RingLayoutCheck<uint32_t, true>;
template struct RingLayoutCheck<uint64_t, false>;
template struct RingLayoutCheck<uint64_t, true>;

template <typename U, bool kIdx>
constexpr size_t persist_smem_bytes() {
  return sizeof(typename Persist<U, kIdx>::Smem);
}
template <typename U, bool kIdx, int kV>
constexpr size_t leaf_smem_bytes() {
  return sizeof(typename LeafCfg<U, kIdx, kV>::Smem);
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

template <typename KT>
__device__ __forceinline__ void sort3(KT s0, KT s1, KT s2, KT* piv) {
  // compareSwap(0,1), (0,2), (1,2) as in turtle-sort.cu:647-649
  KT t;
  if (s1 < s0) { t = s0; s0 = s1; s1 = t; }
  if (s2 < s0) { t = s0; s0 = s2; s2 = t; }
  if (s2 < s1) { t = s1; s1 = s2; s2 = t; }
  piv[0] = s0; piv[1] = s1; piv[2] = s2;
}

// Quartiles of 31 evenly spaced samples (deep levels only).
template <typename KT, typename U>
__device__ __noinline__ void sampled_pivots(const U* src, long long start, long long n, KT flip,
                                            KT* piv) {
  KT s[31];
  for (int i = 0; i < 31; ++i)
    s[i] = KT(__ldcg(src + start + (n * (2 * i + 1)) / 62)) ^ flip;
  for (int i = 1; i < 31; ++i) {
    KT x = s[i];
    int j = i - 1;
    while (j >= 0 && x < s[j]) { s[j + 1] = s[j]; --j; }
    s[j + 1] = x;
  }
  piv[0] = s[7]; piv[1] = s[15]; piv[2] = s[23];
}

// Position of pivot sample i of a segment [start, start+n): the reference's
// a[start+n/2], a[start], a[stop] (turtle-sort.cu:641-655) for 3 samples,
// else evenly spaced keys.
__device__ __forceinline__ long long sample_pos(long long start, long long n, int i, int ns) {
  if (ns == 3) return i == 0 ? start + n / 2 : i == 1 ? start : start + n - 1;
  return start + ((2 * (long long)i + 1) * n) / (2 * ns);
}

// Sorted pivots of a segment on deep levels (quartiles of samples of its
// keys) or under the reference rule (its three captured samples, sorted);
// segment_pivots_warp ranks the sampled rule's kSamples samples.
template <typename KT, typename U>
__device__ __forceinline__ void segment_pivots(const SegDesc* sd, const U* src, int level, KT flip,
                                               int ns, KT* piv) {
  if (level >= kDepthSwitch) {
    sampled_pivots<KT, U>(src, __ldcg(&sd->start), __ldcg(&sd->n), flip, piv);
  } else {
    sort3<KT>((KT)__ldcg(&sd->samp[0]), (KT)__ldcg(&sd->samp[1]), (KT)__ldcg(&sd->samp[2]), piv);
  }
}

// segment_pivots for a whole warp: the kSamples samples are ranked one per
// lane with shuffles instead of by every lane.
template <typename KT, typename U>
__device__ __forceinline__ void segment_pivots_warp(const SegDesc* sd, const U* src, int level,
                                                    KT flip, int ns, KT* piv) {
  if (level >= kDepthSwitch || ns == 3) {
    segment_pivots<KT, U>(sd, src, level, flip, ns, piv);
    return;
  }
  const int lane = threadIdx.x & 31;
  const KT v = lane < kSamples ? (KT)__ldcg(&sd->samp[lane]) : KT(0);
  int r = 0;
#pragma unroll
  for (int j = 0; j < kSamples; ++j) {
    const KT w = __shfl_sync(kFull, v, j);
    r += (w < v) || (w == v && j < lane);
  }
  static_assert(kSamples <= 32, "one sample per lane");
  const bool in = lane < kSamples;
  const int l1 = __ffs(__ballot_sync(kFull, in && r == kSamples / 4)) - 1;
  const int l2 = __ffs(__ballot_sync(kFull, in && r == kSamples / 2)) - 1;
  const int l3 = __ffs(__ballot_sync(kFull, in && r == (3 * kSamples) / 4)) - 1;
  piv[0] = __shfl_sync(kFull, v, l1);
  piv[1] = __shfl_sync(kFull, v, l2);
  piv[2] = __shfl_sync(kFull, v, l3);
}

__device__ __forceinline__ long long tiles_of(long long start, long long n, int shift) {
  return ((start + n - 1) >> shift) - (start >> shift) + 1;
}

// Allocate a next-level segment (tile range allocated with the same 64-bit
// atomic, so tileBase grows with the segment index).  Returns the segment
// index or -1 on overflow.  The caller writes the tile descriptors.  With
// smallPlans, a segment of at most kSmallPlanTiles tiles goes to the list of
// segments planned by one warp instead of getting CTA plan items.
__device__ int alloc_segment(const SortArgs& a, int par, long long start, long long n,
                             int* tbOut, int* ntOut, bool smallPlans) {
  const long long nt = tiles_of(start, n, a.tileShift);
  const unsigned long long old =
      atomicAdd(&a.ctrl->segTile[par], (1ull << 32) | (unsigned long long)nt);
  const int si = (int)(old >> 32);
  const long long tb = (long long)(old & 0xffffffffull);
  const bool small = smallPlans && nt <= kSmallPlanTiles;
  const int np = small ? 0 : (int)((nt + kThreads - 1) / kThreads);  // plan items
  const int pb = small ? atomicAdd(&a.ctrl->planSmallCount[par], 1)
                       : atomicAdd(&a.ctrl->planCount[par], np);
  if (si >= a.segCap || tb + nt > a.tileCap || (small ? pb >= a.segCap : pb + np > a.planCap)) {
    set_error(a.ctrl, kDevCapacity, kSiteCapacity, 1);
    return -1;
  }
  if (small) a.planSmall[par][pb] = si;
  if (np > 1) a.ctrl->planMulti[par] = 1;  // the plan sums per-item totals first
  // only the fields read before the plan writes them: the samples come from
  // the parent's scatter, pivots, class bases and children from the plan
  SegDesc* d = &a.segs[par][si];
  d->start = start;
  d->n = n;
  d->tileBase = (int)tb;
  d->ntiles = (int)nt;
  d->nsamp = 0;
  d->planBase = small ? -1 : pb;
  int4* tot = reinterpret_cast<int4*>(d->tot);  // COUNT adds into the class totals
#pragma unroll
  for (int c = 0; c < 8; ++c) tot[c] = make_int4(0, 0, 0, 0);
  for (int k = 0; k < np; ++k) a.planSeg[par][pb + k] = si;
  *tbOut = (int)tb;
  *ntOut = (int)nt;
  return si;
}

// Tile descriptors of a segment, written by threads [t0, t0+stride) of a group.
__device__ void write_tiles(const SortArgs& a, int par, int si, int tb, int nt, long long start,
                            long long n, int t0, int stride) {
  const int sh = a.tileShift;
  const long long tile = 1LL << sh;
  const long long first = start >> sh;
  const long long end = start + n;
  for (int i = t0; i < nt; i += stride) {
    const long long abs0 = (first + i) << sh;
    TileDesc d;
    d.lo = abs0 > start ? abs0 : start;
    d.hi = (abs0 + tile) < end ? (abs0 + tile) : end;
    d.seg = si;
    d.pad = 0;
    a.tiles[par][tb + i] = d;
  }
}

// Tile descriptor written by another CTA in an earlier phase (L2 read).
__device__ __forceinline__ TileDesc load_tile(const TileDesc* p) {
  TileDesc d;
  d.lo = __ldcg(&p->lo);
  d.hi = __ldcg(&p->hi);
  d.seg = __ldcg(&p->seg);
  d.pad = 0;
  return d;
}

__device__ void push_leaf(const SortArgs& a, long long start, long long n, int inB) {
  const int li = atomicAdd(&a.ctrl->leafCount, 1);
  if (li >= a.leafCap) { set_error(a.ctrl, kDevCapacity, kSiteCapacity, 2); return; }
  LeafDesc d;
  d.start = start; d.n = (int)n; d.inB = inB;
  a.leaves[li] = d;
}

__device__ void push_fill(const SortArgs& a, long long start, long long n, unsigned long long v) {
  for (long long o = 0; o < n; o += kFillChunk) {
    const int fi = atomicAdd(&a.ctrl->fillCount, 1);
    if (fi >= a.fillCap) { set_error(a.ctrl, kDevCapacity, kSiteCapacity, 3); return; }
    FillDesc d;
    d.start = start + o;
    d.n = (int)((n - o) < kFillChunk ? (n - o) : kFillChunk);
    d.pad = 0;
    d.value = v;
    a.fills[fi] = d;
  }
}

// Route one input array at init: nothing, leaf, or level-0 segment (with its
// pivot candidates, unless the caller reads them; its tiles are written when
// writeTiles).
template <typename U>
__device__ void route_input(const SortArgs& a, long long start, long long n, bool writeTiles,
                            int* siOut, int* tbOut, int* ntOut, bool samples = true) {
  *siOut = -1;
  *tbOut = 0;
  *ntOut = 0;
  if (n <= 1) return;
  if (n <= a.leafCut) { push_leaf(a, start, n, 0); return; }
  int tb = 0, nt = 0;
  const int si = alloc_segment(a, 0, start, n, &tb, &nt, true);
  if (si < 0) return;
  using KT = typename KeyCfg<U>::KT;
  const U* src = (const U*)a.keysA;
  const KT flip = (KT)a.flip;
  SegDesc* sd = &a.segs[0][si];
  sd->nsamp = a.samples;
  for (int i = 0; samples && i < a.samples; ++i)
    sd->samp[i] = (unsigned long long)kload<U, KT>(src, sample_pos(start, n, i, a.samples), flip);
  if (writeTiles) write_tiles(a, 0, si, tb, nt, start, n, 0, 1);
  *siOut = si; *tbOut = tb; *ntOut = nt;
}

// Class counts from the six predicate totals #(k<p1), #(k<=p1), #(k<p2),
// #(k<=p2), #(k<p3), #(k<=p3) of nt elements: class boundaries b1..b6 (max()
// keeps them ordered when pivots are equal, which sends every key equal to a
// pivot to the first equal pivot's class, as the reference's test order
// does).  The map is additive over disjoint element sets.
__device__ __forceinline__ void classes_from_predicates(const int* pc, int nt, int* cnt) {
  int b[8];
  b[0] = 0;
  b[1] = pc[0];
  b[2] = pc[1];
  b[3] = max(pc[2], b[2]);
  b[4] = max(pc[3], b[3]);
  b[5] = max(pc[4], b[4]);
  b[6] = max(pc[5], b[5]);
  b[7] = nt;
#pragma unroll
  for (int c = 0; c < 7; ++c) cnt[c] = b[c + 1] - b[c];
}

// Class counts of one tile from its row of predicate totals (L2 reads).
__device__ __forceinline__ void tile_classes(const int* row, int* cnt) {
  const int4 r0 = __ldcg(reinterpret_cast<const int4*>(row));
  const int4 r1 = __ldcg(reinterpret_cast<const int4*>(row) + 1);
  const int pc[6] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y};
  classes_from_predicates(pc, r1.z, cnt);
}

// ---------------------------------------------------------------------------
// chunk pipeline (COUNT and SCATTER)
// ---------------------------------------------------------------------------

// A chunk can be bulk-copied when it lies inside the array and both source
// addresses are 16-byte aligned (tiles start on absolute multiples of the
// tile size, so this holds whenever the buffers are 16-byte aligned; the
// check keeps any other case on plain loads).
template <typename U, bool kIdx>
__device__ __forceinline__ bool chunk_bulk_ok(const U* srcK, const int* srcI, long long c0,
                                              long long n) {
  constexpr int kWCH = Persist<U, kIdx>::kWCH;
  if (c0 + kWCH > n) return false;
  const unsigned long long ak = (unsigned long long)(srcK + c0);
  const unsigned long long ai = kIdx ? (unsigned long long)(srcI + c0) : 0ull;
  return ((ak | ai) & 15ull) == 0;
}

// Lane 0: bulk-copy the chunk at c0 (keys, and ids when withIds) into buffer b.
template <typename U, bool kIdx, bool withIds>
__device__ __forceinline__ void chunk_bulk_issue(typename Persist<U, kIdx>::WarpArea& ws, int b,
                                                 const U* srcK, const int* srcI, long long c0) {
  constexpr int kWCH = Persist<U, kIdx>::kWCH;
  constexpr bool kI = kIdx && withIds;
  constexpr unsigned kBytes = kWCH * sizeof(U) + (kI ? kWCH * 4 : 0);
  fence_proxy_async_smem();
  mbar_arm(&ws.mbar[b], kBytes);
  bulk_g2s(ws.pk[b], srcK + c0, kWCH * sizeof(U), &ws.mbar[b]);
  if (kI) bulk_g2s(ws.pi[b], srcI + c0, kWCH * 4, &ws.mbar[b]);
}

// The lane's kItems consecutive keys of buffer b (flipped to unsigned images).
template <typename U, bool kIdx>
__device__ __forceinline__ void chunk_keys(const typename Persist<U, kIdx>::WarpArea& ws, int b,
                                           int lane, typename Persist<U, kIdx>::KT flip,
                                           typename Persist<U, kIdx>::KT* key) {
  using KT = typename Persist<U, kIdx>::KT;
  constexpr int kItems = Persist<U, kIdx>::kItems;
  constexpr int kBytes = kItems * (int)sizeof(U);
  using V = typename std::conditional<kBytes % 16 == 0, uint4, uint2>::type;
  V v[kBytes / (int)sizeof(V)];
  const V* pk = reinterpret_cast<const V*>(ws.pk[b] + lane * kItems);
#pragma unroll
  for (int j = 0; j < kBytes / (int)sizeof(V); ++j) v[j] = pk[j];
  const U* u = reinterpret_cast<const U*>(v);
#pragma unroll
  for (int i = 0; i < kItems; ++i) key[i] = KT(u[i]) ^ flip;
}

// Bounded wait for buffer b's bulk copies; phases holds one parity bit per buffer.
template <typename U, bool kIdx>
__device__ __forceinline__ void chunk_wait(typename Persist<U, kIdx>::WarpArea& ws, int b,
                                           unsigned& phases, Control* c) {
  if (!mbar_wait(&ws.mbar[b], (phases >> b) & 1u))
    set_error(c, kDevTimeout, kSiteBulk, (int)(threadIdx.x >> 5) * 16 + b * 2 + (int)((phases >> b) & 1u));
  phases ^= 1u << b;
}

// ---------------------------------------------------------------------------
// COUNT phase: one tile per warp
// ---------------------------------------------------------------------------

// Lane 0: bulk-copy the keys of the chunk at c0 into COUNT ring slot r.
template <typename U, bool kIdx>
__device__ __forceinline__ void ring_issue(typename Persist<U, kIdx>::WarpArea& ws, int r,
                                           const U* src, long long c0) {
  constexpr int kCB = Persist<U, kIdx>::kChunkBytes;
  fence_proxy_async_smem();
  mbar_arm(&ws.mbar[r], kCB);
  bulk_g2s(reinterpret_cast<unsigned char*>(ws.pk) + r * kCB, src + c0, kCB, &ws.mbar[r]);
}

// Tile t, counted by one warp against its segment's pivots, chunk by chunk.
// Up to kCountRing - 1 chunks are bulk-copied ahead into a ring of slots
// (COUNT needs neither ids nor the stage, so the ring uses their shared
// memory too); lanes 0..6 store the tile's predicate totals and key count.
template <typename U, bool kIdx>
__device__ __forceinline__ void count_tile_warp(const SortArgs& a, int level, int t,
                                                typename Persist<U, kIdx>::WarpArea& ws,
                                                unsigned& phases, int& accSeg, int& accCnt) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kItems = P::kItems, kWCH = P::kWCH;
  const int kShift = a.tileShift;
  constexpr int kR = P::kCountRing, kCB = P::kChunkBytes;
  const int par = level & 1;
  const int lane = threadIdx.x & 31;
  const U* src = (const U*)(par ? a.keysB : a.keysA);
  const KT flip = (KT)a.flip;
  const TileDesc td = load_tile(&a.tiles[par][t]);
  const long long abs0 = (td.lo >> kShift) << kShift;
  const int rlo = (int)(td.lo - abs0), rhi = (int)(td.hi - abs0);
  const int chBeg = rlo / kWCH, chEnd = (rhi + kWCH - 1) / kWCH;
  if (lane == 0) {
    for (int q = 0; q < kR - 1 && chBeg + q < chEnd; ++q) {
      const long long c0 = abs0 + (long long)(chBeg + q) * kWCH;
      if (chunk_bulk_ok<U, false>(src, nullptr, c0, a.n)) ring_issue<U, kIdx>(ws, q, src, c0);
    }
  }
  KT piv[3];
  segment_pivots_warp<KT, U>(&a.segs[par][td.seg], src, level, flip, a.samples, piv);
  unsigned w0 = 0, w1 = 0, w2 = 0;  // (k<p | k<=p << 16) for p1, p2, p3
  int r = 0;                        // ring slot of chunk ch
  for (int ch = chBeg; ch < chEnd; ++ch) {
    const long long c0 = abs0 + (long long)ch * kWCH;
    {
      // refill the slot freed by the previous chunk
      const int ahead = ch + kR - 1;
      const int ra = r == 0 ? kR - 1 : r - 1;
      const long long ca = abs0 + (long long)ahead * kWCH;
      if (ahead < chEnd && lane == 0 && chunk_bulk_ok<U, false>(src, nullptr, ca, a.n))
        ring_issue<U, kIdx>(ws, ra, src, ca);
    }
    const int e0 = ch * kWCH + lane * kItems;
    KT key[kItems];
    // keys of the lane inside the tile (every key of an interior chunk)
    unsigned okm = (1u << kItems) - 1u;
    if (ch * kWCH < rlo || (ch + 1) * kWCH > rhi) {
      okm = 0;
#pragma unroll
      for (int i = 0; i < kItems; ++i) okm |= (e0 + i >= rlo && e0 + i < rhi) ? (1u << i) : 0u;
    }
    if (chunk_bulk_ok<U, false>(src, nullptr, c0, a.n)) {
      if (!mbar_wait(&ws.mbar[r], (phases >> r) & 1u))
        set_error(a.ctrl, kDevTimeout, kSiteBulk, (int)(threadIdx.x >> 5) * 16 + r * 2 + (int)((phases >> r) & 1u));
      phases ^= 1u << r;
      constexpr int kBytes = kItems * (int)sizeof(U);
      using V = typename std::conditional<kBytes % 16 == 0, uint4, uint2>::type;
      V v[kBytes / (int)sizeof(V)];
      const V* pk = reinterpret_cast<const V*>(reinterpret_cast<const unsigned char*>(ws.pk) +
                                               r * kCB + lane * kBytes);
#pragma unroll
      for (int j = 0; j < kBytes / (int)sizeof(V); ++j) v[j] = pk[j];
      const U* u = reinterpret_cast<const U*>(v);
#pragma unroll
      for (int i = 0; i < kItems; ++i) key[i] = KT(u[i]) ^ flip;
    } else {
      load_chunk<U, KT, kItems>(src + abs0, abs0, a.n, e0, rlo, rhi, flip, key);
    }
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      if (okm >> i & 1u) {
        const KT x = key[i];
        w0 += (x < piv[0] ? 1u : 0u) + (x <= piv[0] ? 0x10000u : 0u);
        w1 += (x < piv[1] ? 1u : 0u) + (x <= piv[1] ? 0x10000u : 0u);
        w2 += (x < piv[2] ? 1u : 0u) + (x <= piv[2] ? 0x10000u : 0u);
      }
    }
    __syncwarp();
    r = r + 1 == kR ? 0 : r + 1;
  }
  w0 = __reduce_add_sync(kFull, w0);
  w1 = __reduce_add_sync(kFull, w1);
  w2 = __reduce_add_sync(kFull, w2);
  if (lane < 8) {
    const unsigned w = lane < 2 ? w0 : lane < 4 ? w1 : w2;
    int v = (lane & 1) ? (int)(w >> 16) : (int)(w & 0xffffu);
    if (lane == 6) v = rhi - rlo;
    if (lane == 7) v = 0;
    a.tileCnt[par][(long long)t * kRow + lane] = v;
  }
  // the tile's class counts go to the warp's running total of its segment
  {
    const int pc[6] = {(int)(w0 & 0xffffu), (int)(w0 >> 16), (int)(w1 & 0xffffu),
                       (int)(w1 >> 16), (int)(w2 & 0xffffu), (int)(w2 >> 16)};
    int cc[7];
    classes_from_predicates(pc, rhi - rlo, cc);
    int mine = 0;
#pragma unroll
    for (int c = 0; c < 7; ++c) mine = lane == c ? cc[c] : mine;
    if (td.seg != accSeg) {
      if (accSeg >= 0 && lane < 7 && accCnt) atomicAdd(&a.segs[par][accSeg].tot[lane], accCnt);
      accSeg = td.seg;
      accCnt = 0;
    }
    accCnt += mine;
  }
}

// ---------------------------------------------------------------------------
// PLAN phase: one plan item per CTA
// ---------------------------------------------------------------------------

// PLAN, first step (levels with segments of several plan items): the column
// sums of one item's count rows (warp w sums rows w, w + kWarps, ...; lane =
// column), so that the plan of a later item of the segment reads the totals
// of the items before it instead of all their rows.
template <typename U, bool kIdx>
__device__ __noinline__ void item_totals(const SortArgs& a, int level, int item,
                                         typename Persist<U, kIdx>::Smem& sm) {
  const int par = level & 1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int seg = __ldcg(&a.planSeg[par][item]);
  const SegDesc* sdp = &a.segs[par][seg];
  const int j = item - __ldcg(&sdp->planBase);
  const int tileBase = __ldcg(&sdp->tileBase), nt = __ldcg(&sdp->ntiles);
  const int t0 = j * kThreads, t1 = nt < t0 + kThreads ? nt : t0 + kThreads;
  const int* cnt = a.tileCnt[par] + (long long)tileBase * kRow;
  int acc = 0;
#pragma unroll 8
  for (int t = t0 + warp; t < t1; t += kWarps) acc += __ldcg(cnt + (long long)t * kRow + lane);
  sm.rowSum[warp][lane] = acc;
  __syncthreads();
  if (tid < kRow) {
    int s = 0;
    for (int w = 0; w < kWarps; ++w) s += sm.rowSum[w][tid];
    a.itemTot[par][(long long)item * kRow + tid] = s;
  }
  __syncthreads();
}

// Column sums of the items of a segment before item j (threads 0..kRow-1),
// into sm.preAll.  The caller synchronizes.
template <typename U, bool kIdx>
__device__ __forceinline__ void item_prefix(const SortArgs& a, int par, int planBase, int j,
                                            typename Persist<U, kIdx>::Smem& sm) {
  const int tid = threadIdx.x;
  if (tid < kRow) {
    // independent loads, several in flight (the chain of adds is cheap)
    const int* col = a.itemTot[par] + (long long)planBase * kRow + tid;
    int s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    int i = 0;
    for (; i + 4 <= j; i += 4) {
      s0 += __ldcg(col + (long long)i * kRow);
      s1 += __ldcg(col + (long long)(i + 1) * kRow);
      s2 += __ldcg(col + (long long)(i + 2) * kRow);
      s3 += __ldcg(col + (long long)(i + 3) * kRow);
    }
    for (; i < j; ++i) s0 += __ldcg(col + (long long)i * kRow);
    sm.preAll[tid] = s0 + s1 + s2 + s3;
  }
}

// One plan item: kThreads consecutive tiles (item j of segment `seg`, one
// tile per thread).  The class bases of the segment follow from its class
// totals (summed by COUNT) in class order as in turtle-sort.cu:755-761; the
// tiles before the item contribute their counts (summed by the whole CTA),
// and the item's own tiles are scanned in memory order, which makes the
// partition stable.  Item 0 of a segment also routes the children
// (turtle-sort.cu:857-933) and stores the segment's sorted pivots, class
// table and children for SCATTER.  Large segments are thus planned by many
// CTAs at once.
template <typename U, bool kIdx>
__device__ __noinline__ void plan_item(const SortArgs& a, int level, int item,
                                       typename Persist<U, kIdx>::Smem& sm) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  const int kLeafMax = a.leafCut;
  const int par = level & 1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int seg = __ldcg(&a.planSeg[par][item]);
  SegDesc* sdp = &a.segs[par][seg];
  const int planBase = __ldcg(&sdp->planBase);
  const int j = item - planBase;
  const long long sdStart = __ldcg(&sdp->start);
  const int tileBase = __ldcg(&sdp->tileBase);
  const int nt = __ldcg(&sdp->ntiles);
  const int* cnt = a.tileCnt[par] + (long long)tileBase * kRow;
  const int t0 = j * kThreads;
  if (tid < 7) sm.tot[tid] = __ldcg(&sdp->tot[tid]);
  // the segment's tiles before this item: their raw predicate totals (the
  // class map is additive over tiles) from the item totals
  item_prefix<U, kIdx>(a, par, planBase, j, sm);
  if (j == 0 && warp == 0) {
    KT piv[3];
    segment_pivots_warp<KT, U>(sdp, (const U*)(par ? a.keysB : a.keysA), level, (KT)a.flip,
                               a.samples, piv);
    if (lane == 0) {
      sm.piv[0] = piv[0]; sm.piv[1] = piv[1]; sm.piv[2] = piv[2];
      sm.lut = pivot_lut(piv[0] == piv[1], piv[1] == piv[2]);
    }
  }
  // counts of this thread's tile
  int v[7];
#pragma unroll
  for (int c = 0; c < 7; ++c) v[c] = 0;
  const int myTile = t0 + tid;
  if (myTile < nt) tile_classes(cnt + (long long)myTile * kRow, v);
  int inc[7];
#pragma unroll
  for (int c = 0; c < 7; ++c) {
    int x = v[c];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    inc[c] = x;
    if (lane == 31) sm.red[warp][c] = x;
  }
  __syncthreads();
  if (tid < 7) {
    int acc = 0;
    for (int w = 0; w < kWarps; ++w) {
      const int x = sm.red[w][tid];
      sm.red[w][tid] = acc;
      acc += x;
    }
  }
  if (tid == 7) {
    int pre[7];
    const int pc[6] = {sm.preAll[0], sm.preAll[1], sm.preAll[2], sm.preAll[3], sm.preAll[4],
                       sm.preAll[5]};
    classes_from_predicates(pc, sm.preAll[6], pre);
    for (int c = 0; c < 7; ++c) sm.pre[c] = pre[c];
  }
  if (tid == 0) {
    int b = 0;
    for (int c = 0; c < 7; ++c) { sm.cbase[c] = b; b += sm.tot[c]; }
    sm.cbase[7] = b;
  }
  __syncthreads();
  if (myTile < nt) {
    long long o[7];
#pragma unroll
    for (int c = 0; c < 7; ++c)
      o[c] = sdStart + sm.cbase[c] + sm.pre[c] + sm.red[warp][c] + (inc[c] - v[c]);
    longlong2* dst = reinterpret_cast<longlong2*>(a.tileOff[par] + (long long)(tileBase + myTile) * kRow);
    dst[0] = make_longlong2(o[0], o[1]);
    dst[1] = make_longlong2(o[2], o[3]);
    dst[2] = make_longlong2(o[4], o[5]);
    dst[3] = make_longlong2(o[6], 0);
  }
  if (j != 0) {
    __syncthreads();
    return;
  }

  // item 0: children -- thread c routes class c (fill, leaf or next-level
  // segment); the CTA then writes the new segments' tile descriptors
  const bool dstIsA = (par == 1);
  const int nextPar = par ^ 1;
  if (tid < 7) {
    const int c = tid;
    const long long pos = sdStart + sm.cbase[c];
    const long long m = sm.cbase[c + 1] - sm.cbase[c];
    if (c & 1) {
      if (m > 0 && !dstIsA) push_fill(a, pos, m, (unsigned long long)sm.piv[c >> 1]);
    } else {
      const int ci = c >> 1;
      int si = -1;
      if (m > 1 || (m == 1 && !dstIsA)) {
        if (m <= kLeafMax) {
          push_leaf(a, pos, m, dstIsA ? 0 : 1);
        } else {
          int tb = 0, ntc = 0;
          si = alloc_segment(a, nextPar, pos, m, &tb, &ntc, true);
          sm.childTb[ci] = tb;
          sm.childNt[ci] = si >= 0 ? ntc : 0;
          sm.childStart[ci] = pos;
          sm.childN[ci] = m;
        }
      }
      sm.childSeg[ci] = si;
      sdp->childSeg[ci] = si;
    }
    sdp->cbase[c] = pos;
    if (c == 6) sdp->cbase[7] = sdStart + sm.cbase[7];
    if (c < 3) sdp->pivS[c] = (unsigned long long)sm.piv[c];
    if (c == 3) sdp->lut = sm.lut;
  }
  __syncthreads();
  for (int ci = 0; ci < 4; ++ci) {
    if (sm.childSeg[ci] >= 0)
      write_tiles(a, nextPar, sm.childSeg[ci], sm.childTb[ci], sm.childNt[ci],
                         sm.childStart[ci], sm.childN[ci], tid, kThreads);
  }
  __syncthreads();
}

// plan_item for a segment of at most kSmallPlanTiles tiles, by one warp (lane
// l owns tiles 2l and 2l+1, so a warp scan gives the offsets in memory
// order).  The deep levels hold thousands of such segments; one warp each
// keeps the CTA's other warps planning other segments meanwhile.
template <typename U, bool kIdx>
__device__ __noinline__ void plan_small_warp(const SortArgs& a, int level, int seg) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  const int kLeafMax = a.leafCut;
  static_assert(kSmallPlanTiles == 64, "two tiles per lane");
  const int par = level & 1;
  const int lane = threadIdx.x & 31;
  SegDesc* sdp = &a.segs[par][seg];
  const long long sdStart = __ldcg(&sdp->start);
  const int tileBase = __ldcg(&sdp->tileBase);
  const int nt = __ldcg(&sdp->ntiles);
  const int* cnt = a.tileCnt[par] + (long long)tileBase * kRow;
  KT piv[3];
  segment_pivots_warp<KT, U>(sdp, (const U*)(par ? a.keysB : a.keysA), level, (KT)a.flip,
                             a.samples, piv);
  const int t0 = 2 * lane, t1 = 2 * lane + 1;
  int v0[7], v1[7];
#pragma unroll
  for (int c = 0; c < 7; ++c) { v0[c] = 0; v1[c] = 0; }
  if (t0 < nt) tile_classes(cnt + (long long)t0 * kRow, v0);
  if (t1 < nt) tile_classes(cnt + (long long)t1 * kRow, v1);
  long long* off0 = a.tileOff[par] + (long long)(tileBase + t0) * kRow;
  long long* off1 = off0 + kRow;
  int base = 0, myBase = 0, myTot = 0;
#pragma unroll
  for (int c = 0; c < 7; ++c) {
    const int sum = v0[c] + v1[c];
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    const int tot = __shfl_sync(kFull, x, 31);
    const long long o = sdStart + base + (x - sum);
    if (t0 < nt) off0[c] = o;
    if (t1 < nt) off1[c] = o + v0[c];
    if (lane == c) { myBase = base; myTot = tot; }
    base += tot;
  }
  // lane c routes class c (fill, leaf or next-level segment)
  const bool dstIsA = (par == 1);
  const int nextPar = par ^ 1;
  int si = -1, tb = 0, ntc = 0;
  long long pos = 0, m = 0;
  if (lane < 7) {
    const int c = lane;
    pos = sdStart + myBase;
    m = myTot;
    if (c & 1) {
      if (m > 0 && !dstIsA) push_fill(a, pos, m, (unsigned long long)piv[c >> 1]);
    } else {
      if (m > 1 || (m == 1 && !dstIsA)) {
        if (m <= kLeafMax) push_leaf(a, pos, m, dstIsA ? 0 : 1);
        else si = alloc_segment(a, nextPar, pos, m, &tb, &ntc, true);
      }
      sdp->childSeg[c >> 1] = si;
    }
    sdp->cbase[c] = pos;
    if (c == 6) sdp->cbase[7] = sdStart + base;
    if (c < 3) sdp->pivS[c] = (unsigned long long)piv[c];
    if (c == 3) sdp->lut = pivot_lut(piv[0] == piv[1], piv[1] == piv[2]);
  }
  // tiles of the new segments
#pragma unroll
  for (int ci = 0; ci < 4; ++ci) {
    const int s = __shfl_sync(kFull, si, 2 * ci);
    if (s >= 0) {
      const int ctb = __shfl_sync(kFull, tb, 2 * ci);
      const int cnt2 = __shfl_sync(kFull, ntc, 2 * ci);
      const long long cs = __shfl_sync(kFull, pos, 2 * ci);
      const long long cn = __shfl_sync(kFull, m, 2 * ci);
      write_tiles(a, nextPar, s, ctb, cnt2, cs, cn, lane, 32);
    }
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// SCATTER phase: one tile per warp
// ---------------------------------------------------------------------------

// The warp walks its tile chunk by chunk (the next chunk is bulk-copied into
// the other buffer while the current one is processed).  Per chunk: class of
// every key (comparison sum through the segment's class table), lane-local
// ranks in 4-bit counters, one warp scan of the packed counters, the chunk
// staged by class, and each class run written to base[class] + rank, where
// base[class] starts at the tile's offset from the plan and advances by each
// chunk's class counts: class runs of one chunk are contiguous and
// consecutive chunks continue them.  Lane 8*ci + j watches pivot samples j
// and j + 8 of child ci (sample_pos) and copies the staged key that lands
// there into the child's descriptor.
template <typename U, bool kIdx>
__device__ __forceinline__ void scatter_tile_warp(const SortArgs& a, int level, int t,
                                                  typename Persist<U, kIdx>::WarpArea& ws,
                                                  unsigned& phases) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kItems = P::kItems, kWCH = P::kWCH;
  const int kShift = a.tileShift;
  const int par = level & 1;
  const KT flip = (KT)a.flip;
  const int lane = threadIdx.x & 31;
  const TileDesc td = load_tile(&a.tiles[par][t]);
  const long long abs0 = (td.lo >> kShift) << kShift;
  const int rlo = (int)(td.lo - abs0), rhi = (int)(td.hi - abs0);
  const U* srcK = (const U*)(par ? a.keysB : a.keysA);
  const int* srcI = par ? a.idxB : a.idxA;
  const int chBeg = rlo / kWCH, chEnd = (rhi + kWCH - 1) / kWCH;
  if (lane == 0 && chunk_bulk_ok<U, kIdx>(srcK, srcI, abs0 + (long long)chBeg * kWCH, a.n))
    chunk_bulk_issue<U, kIdx, true>(ws, 0, srcK, srcI, abs0 + (long long)chBeg * kWCH);
  const SegDesc* sdp = &a.segs[par][td.seg];
  const KT p1 = (KT)__ldcg(&sdp->pivS[0]), p2 = (KT)__ldcg(&sdp->pivS[1]),
           p3 = (KT)__ldcg(&sdp->pivS[2]);
  const unsigned lut = __ldcg(&sdp->lut);
  // running destination of each class; pivot positions of the children
  if (lane < 7) ws.o.wbase[lane] = __ldcg(&a.tileOff[par][(long long)t * kRow + lane]);
  const int ns = a.samples;
  // lane 8*ci + j watches samples j, j+8, ... of child ci; it keeps the next
  // one at or after the tile's first destination of the child's class
  const int myci = lane >> 3, myj = lane & 7;
  int nextQ = 0;
  long long nextPos = LLONG_MAX;
  {
    const int child = __ldcg(&sdp->childSeg[myci]);
    if (myj == 0) ws.o.cseg[myci] = child;
    if (child >= 0 && myj < ns) {
      const long long cb = __ldcg(&sdp->cbase[2 * myci]);
      const long long cn = __ldcg(&sdp->cbase[2 * myci + 1]) - cb;
      const long long tStart = __ldcg(&a.tileOff[par][(long long)t * kRow + 2 * myci]);
      for (int q = myj; q < ns; q += 8) {
        const long long p = sample_pos(cb, cn, q, ns);
        ws.o.cpos[myci][q] = p;
        if (nextPos == LLONG_MAX && p >= tStart) { nextQ = q; nextPos = p; }
      }
    }
  }
  __syncwarp();

  for (int ch = chBeg; ch < chEnd; ++ch) {
    const int b = (ch - chBeg) & 1;
    const long long c0 = abs0 + (long long)ch * kWCH;
    if (ch + 1 < chEnd && lane == 0 && chunk_bulk_ok<U, kIdx>(srcK, srcI, c0 + kWCH, a.n))
      chunk_bulk_issue<U, kIdx, true>(ws, b ^ 1, srcK, srcI, c0 + kWCH);
    const int e0 = ch * kWCH + lane * kItems;  // tile-relative index of the lane's first key
    KT key[kItems];
    // keys of the lane inside the tile (every key of an interior chunk)
    unsigned okm = (1u << kItems) - 1u;
    if (ch * kWCH < rlo || (ch + 1) * kWCH > rhi) {
      okm = 0;
#pragma unroll
      for (int i = 0; i < kItems; ++i) okm |= (e0 + i >= rlo && e0 + i < rhi) ? (1u << i) : 0u;
    }
    if (chunk_bulk_ok<U, kIdx>(srcK, srcI, c0, a.n)) {
      chunk_wait<U, kIdx>(ws, b, phases, a.ctrl);
      chunk_keys<U, kIdx>(ws, b, lane, flip, key);
    } else {
      // array end: plain loads; the ids go through the buffer like bulk ones
      load_chunk<U, KT, kItems>(srcK + abs0, abs0, a.n, e0, rlo, rhi, flip, key);
      if (kIdx) {
        int id[kItems];
        load_ids<kItems>(srcI + abs0, abs0, a.n, e0, okm, id);
#pragma unroll
        for (int i = 0; i < kItems; ++i) ws.pi[b][lane * kItems + i] = id[i];
      }
    }

    // classes (3 bits each, 7 = no key) and lane-local ranks (4 bits each)
    unsigned cw = 0, rw = 0, acc = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      unsigned c = 7u;
      if (okm >> i & 1u) {
        const KT k = key[i];
        const unsigned cp = (unsigned)((k > p1) + (k >= p1) + (k > p2) + (k >= p2) + (k > p3) +
                                       (k >= p3));
        c = (lut >> (3u * cp)) & 7u;
        rw |= ((acc >> (4u * c)) & 15u) << (4 * i);
        acc += 1u << (4u * c);
      }
      cw |= c << (3 * i);
    }
    // warp exclusive scan of the lane counts (8-bit fields; exclusive sums
    // stay below 256, so the packed arithmetic is exact)
    const unsigned a0 = (acc & 0xFu) | ((acc & 0xF0u) << 4) | ((acc & 0xF00u) << 8) |
                        ((acc & 0xF000u) << 12);
    const unsigned a1 = ((acc >> 16) & 0xFu) | ((acc >> 12) & 0xF00u) | ((acc >> 8) & 0xF0000u);
    unsigned i0 = a0, i1 = a1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y0 = __shfl_up_sync(kFull, i0, o), y1 = __shfl_up_sync(kFull, i1, o);
      if (lane >= o) { i0 += y0; i1 += y1; }
    }
    // class totals of the chunk (16-bit fields) and class starts in the stage
    const unsigned t01 = __reduce_add_sync(kFull, (acc & 0xFu) | ((acc & 0xF0u) << 12));
    const unsigned t23 = __reduce_add_sync(kFull, ((acc >> 8) & 0xFu) | ((acc & 0xF000u) << 4));
    const unsigned t45 = __reduce_add_sync(kFull, ((acc >> 16) & 0xFu) | ((acc >> 4) & 0xF0000u));
    const unsigned t6 = __reduce_add_sync(kFull, (acc >> 24) & 0xFu);
    const unsigned cs1 = t01 & 0xFFFFu;
    const unsigned cs2 = cs1 + (t01 >> 16);
    const unsigned cs3 = cs2 + (t23 & 0xFFFFu);
    const unsigned cs4 = cs3 + (t23 >> 16);
    const unsigned cs5 = cs4 + (t45 & 0xFFFFu);
    const unsigned cs6 = cs5 + (t45 >> 16);
    const unsigned nv = cs6 + t6;
    // stage the chunk: per lane and class, the slot of the lane's first key of
    // that class is a packed 8-bit field of b0 (classes 0-3) or b1 (4-6)
    {
      const unsigned b0 = (cs1 << 8) + (cs2 << 16) + (cs3 << 24) + (i0 - a0);
      const unsigned b1 = cs4 + (cs5 << 8) + (cs6 << 16) + (i1 - a1);
#pragma unroll
      for (int h = 0; h < kItems; h += 4) {
        int4 idv = make_int4(0, 0, 0, 0);
        if (kIdx) idv = *reinterpret_cast<const int4*>(&ws.pi[b][lane * kItems + h]);
        const int idq[4] = {idv.x, idv.y, idv.z, idv.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = h + u;
          const unsigned c = (cw >> (3 * i)) & 7u;
          if (c != 7u) {
            const unsigned w = c < 4u ? b0 : b1;
            const unsigned pos = ((w >> ((c & 3u) * 8u)) & 0xFFu) + ((rw >> (4 * i)) & 15u);
            ws.sk[pos] = key[i];
            if (kIdx) ws.si[pos] = idq[u];
            ws.sc[pos] = (unsigned char)c;
          }
        }
      }
    }
    // lanes 0..6: destination table of the chunk, then advance the bases
    if (lane < 7) {
      const unsigned csl = lane == 1 ? cs1 : lane == 2 ? cs2 : lane == 3 ? cs3 : lane == 4 ? cs4
                         : lane == 5 ? cs5 : lane == 6 ? cs6 : 0u;
      const unsigned cel = lane == 0 ? cs1 : lane == 1 ? cs2 : lane == 2 ? cs3 : lane == 3 ? cs4
                         : lane == 4 ? cs5 : lane == 5 ? cs6 : nv;
      const long long wb = ws.o.wbase[lane];
      ws.o.delta[lane] = wb - (long long)csl;
      ws.o.wbase[lane] = wb + (long long)(cel - csl);
    }
    __syncwarp();
    // write-out: consecutive stage slots of one class go to consecutive addresses
    {
      U* dstK = (U*)(par ? a.keysA : a.keysB);
      int* dstI = par ? a.idxA : a.idxB;
      const bool parkPivots = (par == 0);  // children in B: pivot-run keys wait for their fill
#pragma unroll
      for (int j = 0; j < kItems; ++j) {
        const int sl = 32 * j + lane;
        if (sl < (int)nv) {
          const unsigned c = ws.sc[sl];
          const long long d = ws.o.delta[c] + sl;
          if (!(parkPivots && (c & 1u))) dstK[d] = U(ws.sk[sl] ^ flip);
          if (kIdx) dstI[d] = ws.si[sl];
        }
      }
    }
    // a child's pivot sample written by this chunk (its class run ends at the
    // advanced base): copy the staged key
    if (nextPos < ws.o.wbase[2 * myci]) {
      const int child = ws.o.cseg[myci];
      const long long dl = ws.o.delta[2 * myci];
      const long long end = ws.o.wbase[2 * myci];
      do {
        a.segs[par ^ 1][child].samp[nextQ] = (unsigned long long)ws.sk[nextPos - dl];
        nextQ += 8;
        nextPos = nextQ < ns ? ws.o.cpos[myci][nextQ] : LLONG_MAX;
      } while (nextPos < end);
    }
    __syncwarp();
  }
}

}  // namespace turtle

#include "turtle_wide.cuh"

namespace turtle {

// ---------------------------------------------------------------------------
// leaf bucketing (end of the partition kernel)
// ---------------------------------------------------------------------------

// Slice of a leaf or fill: the position slice holding its first key.  Leaf
// launch s sorts the leaves of slice s (launch 0 also fills every parked
// pivot run), so once launch s is done every key below the end of slice s is
// final.
__device__ __forceinline__ int leaf_slice(long long start, long long n, int slices) {
  const long long s = (start * slices) / (n > 0 ? n : 1);
  return (int)(s < slices - 1 ? s : slices - 1);
}

// Bucket the leaves by (slice, size class) -- slices in order, largest class
// first within a slice -- and publish the leaf work items in the control
// block.  Uses 2 grid barriers; returns false on error.
template <typename U, bool kIdx>
__device__ __noinline__ bool leaf_bucket(const SortArgs& a, typename Persist<U, kIdx>::Smem& sm) {
  const int items = a.leafItems, classes = a.leafClasses;
  constexpr int kB = kMaxSlices * 16;
  Control* c = a.ctrl;
  const long long polls = a.barrierPolls > 0 ? a.barrierPolls : kSpinLimit;
  const int tid = threadIdx.x;
  const int S = a.slices;
  const int nLeaves = ld_acquire_int(&c->leafCount);
  const int nFills = ld_acquire_int(&c->fillCount);
  const int nl = nLeaves < a.leafCap ? nLeaves : a.leafCap;
  const int nf = nFills < a.fillCap ? nFills : a.fillCap;
  // bucket 1: counts
  for (int b = tid; b < kB; b += kThreads) sm.classItems[b] = 0;
  __syncthreads();
  for (int i = blockIdx.x * kThreads + tid; i < nl; i += gridDim.x * kThreads) {
    const LeafDesc d = a.leaves[i];
    atomicAdd(&sm.classItems[leaf_slice(d.start, a.n, S) * 16 + leaf_class(d.n, items)], 1);
  }
  __syncthreads();
  for (int b = tid; b < S * 16; b += kThreads)
    if (sm.classItems[b]) atomicAdd(&c->classCount[b], sm.classItems[b]);
  if (!grid_barrier(c, polls)) return false;
  timeline_mark(c, nl);
  // bucket 2: scatter into per-bucket ranges
  if (tid == 0) {
    int acc = 0;
    for (int s = 0; s < S; ++s) {
      for (int k = classes - 1; k >= 0; --k) {
        sm.classOff[s * 16 + k] = acc;
        acc += ld_acquire_int(&c->classCount[s * 16 + k]);
      }
    }
  }
  __syncthreads();
  for (int i = blockIdx.x * kThreads + tid; i < nl; i += gridDim.x * kThreads) {
    const LeafDesc d = a.leaves[i];
    const int b = leaf_slice(d.start, a.n, S) * 16 + leaf_class(d.n, items);
    const int pos = sm.classOff[b] + atomicAdd(&c->classFill[b], 1);
    a.leavesSorted[pos] = d;
  }
  if (blockIdx.x == 0 && tid == 0) {
    for (int s = 0; s < S; ++s) {
      int acc = 0;
      for (int k = classes - 1; k >= 0; --k) {
        const int groups = (1 << (classes - 1)) >> k;
        const int cnt = ld_acquire_int(&c->classCount[s * 16 + k]);
        c->classItemsG[s * 16 + k] = acc;  // first item of class k in slice s
        c->classOffG[s * 16 + k] = sm.classOff[s * 16 + k];
        acc += (cnt + groups - 1) / groups;
      }
      c->leafItems[s] = acc;
    }
    c->fillItems = nf;
  }
  if (!grid_barrier(c, polls)) return false;
  timeline_mark(c, nf);
  return true;
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------

// Tiles of a level, claimed one at a time by each warp (lane 0 claims the
// next tile before the warp works on the current one).
// kWide: two-level pass (31 classes) instead of one level (7 classes).
template <typename U, bool kIdx, int kPhase, bool kWide>
__device__ __forceinline__ void stream_tiles(const SortArgs& a, int level, int ntiles,
                                             unsigned* wc,
                                             typename Persist<U, kIdx>::WarpArea& ws,
                                             unsigned& mphase) {
  const int lane = threadIdx.x & 31;
  // the bulk copies of this phase read what other CTAs wrote before the
  // grid barrier: order the async proxy after it
  if (lane == 0) fence_proxy_async();
  if (kWide) ws.t.pivSeg = -1;  // segment indices are per pass
  __syncwarp();
  unsigned t = 0;
  if (lane == 0) t = atomicAdd(wc, 1u);
  t = __shfl_sync(kFull, t, 0);
  int accSeg = -1, accCnt = 0;
  while ((int)t < ntiles) {
    unsigned nxt = 0;
    if (lane == 0) nxt = atomicAdd(wc, 1u);
    if (kWide) {
      if (kPhase == 0) count31_tile_warp<U, kIdx>(a, level, (int)t, ws, mphase, accSeg, accCnt);
      else scatter31_tile_warp<U, kIdx>(a, level, (int)t, ws, mphase);
    } else {
      if (kPhase == 0) count_tile_warp<U, kIdx>(a, level, (int)t, ws, mphase, accSeg, accCnt);
      else scatter_tile_warp<U, kIdx>(a, level, (int)t, ws, mphase);
    }
    t = __shfl_sync(kFull, nxt, 0);
  }
  if (kPhase == 0 && accSeg >= 0 && lane < (kWide ? 32 : 7) && accCnt)
    atomicAdd(&a.segs[level & 1][accSeg].tot[lane], accCnt);
}

// kWide: two-level passes (sampled pivots from kWideSamples keys) instead of
// one level per pass; each form is its own kernel with its own registers.
template <typename U, bool kIdx, bool kWide>
__global__ void __launch_bounds__(kThreads, kMinBlocks) persistent_sort_kernel(SortArgs a) {
  using P = Persist<U, kIdx>;
  const int kLeafMax = a.leafCut;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename P::Smem& sm = *reinterpret_cast<typename P::Smem*>(smem_raw);
  Control* c = a.ctrl;
  const long long polls = a.barrierPolls > 0 ? a.barrierPolls : kSpinLimit;
  const int tid = threadIdx.x;
  typename P::WarpArea& ws = sm.w[tid >> 5];
  unsigned mphase = 0;  // parity bit of each chunk buffer's barrier
  if ((tid & 31) == 0)
    for (int r = 0; r < kMaxRing; ++r) mbar_init(&ws.mbar[r], 1);
  __syncwarp();
  int phase = 0;
  int level = 0;
  timeline_mark(c, -1);

  if (a.resume) {
    // continue after a yield: the leaf lists were drained by leaf_kernel
    level = c->resumeLevel;
    phase = c->resumePhase;
    if (blockIdx.x == 0 && tid == 0) {
      c->leafCount = 0;
      c->fillCount = 0;
      for (int k = 0; k < kMaxSlices; ++k) c->leafWork[k] = 0;
      c->leafDone = 0;
      c->yield = 0;
      for (int k = 0; k < kMaxSlices * 16; ++k) { c->classCount[k] = 0; c->classFill[k] = 0; }
    }
  } else if (a.offsets == nullptr) {
    // init: route the input array (level-0 list is parity 0)
    if (blockIdx.x == 0) {
      if (tid == 0) {
        int si, tb, nt;
        route_input<U>(a, 0, a.n, false, &si, &tb, &nt, false);
        sm.childSeg[0] = si;
        sm.childTb[0] = tb;
        sm.childNt[0] = nt;
      }
      __syncthreads();
      if (sm.childSeg[0] >= 0 && tid < a.samples)  // pivot candidates, one per thread
        a.segs[0][sm.childSeg[0]].samp[tid] = (unsigned long long)kload<U, typename P::KT>(
            (const U*)a.keysA, sample_pos(0, a.n, tid, a.samples), (typename P::KT)a.flip);
      if (sm.childSeg[0] >= 0)
        write_tiles(a, 0, sm.childSeg[0], sm.childTb[0], sm.childNt[0], 0, a.n, tid,
                           kThreads);
    }
  } else {
    for (long long i = (long long)blockIdx.x * kThreads + tid; i < a.numArrays;
         i += (long long)gridDim.x * kThreads) {
      const long long s = a.offsets[i], e = a.offsets[i + 1];
      int si, tb, nt;
      route_input<U>(a, s, e - s, true, &si, &tb, &nt);
    }
  }
  if (!grid_barrier(c, polls)) return;
  timeline_mark(c, 0);

  // one level adds at most 4 leaves and 3 fills (+ chunks) per segment, a
  // two-level pass 16 leaves and 15 fills; stop and hand the lists to
  // leaf_kernel before a level could overflow them
  constexpr bool wide = kWide;
  const int leafRoom = (wide ? 16 : 4) * (a.segCap + 1);
  const int fillRoom = (wide ? 15 : 3) * (a.segCap + 1) + a.tileCap;
  for (;; ++level) {
    const int par = level & 1;
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> st(c->segTile[par]);
    const unsigned long long v = st.load(cuda::memory_order_acquire);
    const int nsegs = (int)(v >> 32);
    const int ntiles = (int)(v & 0xffffffffull);
    const int nplan = ld_acquire_int(&c->planCount[par]);
    if (nsegs == 0) break;
    if (level >= kMaxLevels) { if (tid == 0) set_error(c, kDevCapacity); return; }
    if (ld_acquire_int(&c->leafCount) > (a.leafYield > 0 ? a.leafYield : a.leafCap - leafRoom) ||
        ld_acquire_int(&c->fillCount) > a.fillCap - fillRoom) {
      if (blockIdx.x == 0 && tid == 0) {
        c->yield = 1;
        c->resumeLevel = level;
        c->resumePhase = phase;
      }
      break;
    }

    // COUNT: per-tile predicate totals
    if (blockIdx.x == 0 && tid == 0) c->work[(phase + 2) & 3] = 0;
    stream_tiles<U, kIdx, 0, kWide>(a, level, ntiles, &c->work[phase & 3], ws, mphase);
    ++phase;
    __threadfence();
    if (!grid_barrier(c, polls)) return;
    timeline_mark(c, ntiles);

    // PLAN, first step when a segment has several plan items: item totals
    if (ld_acquire_int(&c->planMulti[par])) {
      unsigned* wc = &c->work[phase & 3];
      if (blockIdx.x == 0 && tid == 0) c->work[(phase + 2) & 3] = 0;
      for (;;) {
        const int it = claim_item(wc);
        if (it >= nplan) break;
        item_totals<U, kIdx>(a, level, it, sm);
      }
      ++phase;
      __threadfence();
      if (!grid_barrier(c, polls)) return;
    }
    // PLAN: one item (kThreads tiles of one segment) per CTA
    {
      unsigned* wc = &c->work[phase & 3];
      if (blockIdx.x == 0 && tid == 0) c->work[(phase + 2) & 3] = 0;
      for (;;) {
        const int it = claim_item(wc);
        if (it >= nplan) break;
        if (kWide) plan31_item<U, kIdx>(a, level, it, sm);
        else plan_item<U, kIdx>(a, level, it, sm);
      }
      {
        // small segments: one warp each
        const int nsmall = ld_acquire_int(&c->planSmallCount[par]);
        for (;;) {
          unsigned it = 0;
          if ((tid & 31) == 0) it = atomicAdd(&c->smallWork, 1u);
          it = __shfl_sync(kFull, it, 0);
          if ((int)it >= nsmall) break;
          if (kWide) plan31_small_warp<U, kIdx>(a, level, __ldcg(&a.planSmall[par][it]), &ws.t.wp);
          else plan_small_warp<U, kIdx>(a, level, __ldcg(&a.planSmall[par][it]));
        }
      }
      ++phase;
    }
    __threadfence();
    if (!grid_barrier(c, polls)) return;
    timeline_mark(c, nsegs);

    // SCATTER
    if (blockIdx.x == 0 && tid == 0) {
      // this level's list was read by everyone before the last barrier;
      // level+2 appends to it during the next PLAN phase
      st.store(0ull, cuda::memory_order_relaxed);
      c->planCount[par] = 0;
      c->planSmallCount[par] = 0;
      c->planMulti[par] = 0;
      c->smallWork = 0;
      c->work[(phase + 2) & 3] = 0;
    }
    stream_tiles<U, kIdx, 1, kWide>(a, level, ntiles, &c->work[phase & 3], ws, mphase);
    ++phase;
    __threadfence();
    if (!grid_barrier(c, polls)) return;
    timeline_mark(c, nsegs);
  }
  if (blockIdx.x == 0 && tid == 0) c->levels = wide ? 2 * level : level;
  // publish the leaves for leaf_kernel (launched right after on the stream)
  leaf_bucket<U, kIdx>(a, sm);
}

// ---------------------------------------------------------------------------
// LEAF kernel
// ---------------------------------------------------------------------------

// Sort the loaded leaves of the CTA's groups as words of codec LW and write
// keys and ids to A.  Each thread's raw keys wait in the word buffer at the
// slots it wrote; the group's smallest key is `lo`.  What the output needs
// after the sort (the leaf descriptor, lo) is reloaded then, which keeps the
// sort within the register budget.
template <typename U, bool kIdx, int kV, class LW>
__device__ __forceinline__ void leaf_words_sort(const SortArgs& a,
                                                typename LeafCfg<U, kIdx, kV>::Smem& sm, int P,
                                                int li, int last,
                                                typename KeyCfg<U>::KT lo, int sh) {
  using KT = typename KeyCfg<U>::KT;
  using W = typename LW::W;
  constexpr int kItems = LeafCfg<U, kIdx, kV>::kItems;
  constexpr int kLT = LeafCfg<U, kIdx, kV>::kThreads;
  const int tid = threadIdx.x;
  const int g = tid / P, q = tid & (P - 1);
  const int n = li < last ? __ldcg(&a.leavesSorted[li].n) : 0;
  W* words = reinterpret_cast<W*>(sm.wbytes);
  {
    const int region = g * P * kItems;
    KT lk[kItems];
    const KT* raw = reinterpret_cast<const KT*>(sm.wbytes);
#pragma unroll
    for (int i = 0; i < kItems; ++i) lk[i] = raw[region + q + i * P];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int j = q + i * P;
      words[wpad<W>(region + j)] = j < n ? LW::make(lk[i], lo, j, sh) : LW::sent();
    }
  }
  if (q == 0) sm.glo[g] = lo;
  __syncthreads();
  block_sort_words<LW, kItems>(words, P, kLT, n);
  if (li < last) {
    const LeafDesc d = a.leavesSorted[li];
    const KT base = sm.glo[g];
    const int region = g * P * kItems;
    U* dst = (U*)a.keysA;
    int* dstI = a.idxA;
    const KT flip = (KT)a.flip;
    for (int j = q; j < d.n; j += P) {
      const W w = words[wpad<W>(region + j)];
      kstore<U, KT>(dst, d.start + j, (KT)LW::key(w, base, sh), flip);
      if (kIdx) dstI[d.start + j] = sm.idx[region + LW::pos(w, sh)];
    }
  }
}

// Sort up to kThreads/P leaves of size class cls (P = 1 << cls threads each)
// from leavesSorted[first, last), results to A.  The keys are loaded once;
// when every leaf of the CTA spans a narrow key range (the leaves of the
// partition lie between two pivots) they are sorted as range-packed 32-bit
// words (64-bit words for 64-bit keys with ids when that range fits), else as
// full-range words.
template <typename U, bool kIdx, int kV>
__device__ void sort_leaf_group(const SortArgs& a, int cls, int first, int last,
                                typename LeafCfg<U, kIdx, kV>::Smem& sm) {
  using KT = typename KeyCfg<U>::KT;
  constexpr int kItems = LeafCfg<U, kIdx, kV>::kItems;
  const int P = 1 << cls;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = tid / P, q = tid & (P - 1);
  const int li = first + g;
  const int region = g * P * kItems;
  const KT flip = (KT)a.flip;
  LeafDesc d;
  d.start = 0; d.n = 0; d.inB = 0;
  if (li < last) d = a.leavesSorted[li];
  const U* src = (const U*)(d.inB ? a.keysB : a.keysA);
  const int* srcI = d.inB ? a.idxB : a.idxA;
  // a thread's kItems slots are q, q + P, ...: all its loads are issued before
  // the first shared-memory store, so they overlap instead of queueing.  Keys
  // and ids go to shared memory as loaded (ids are fetched by position once
  // the words are sorted); the thread keeps the range of its keys.
  KT tmin = key_max<KT>(), tmax = KT(0);
  {
    KT lk[kItems];
    int lv[kItems];
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int j = q + i * P;
      const bool ok = j < d.n;
      lk[i] = ok ? kload<U, KT>(src, d.start + j, flip) : KT(0);
      if (kIdx) lv[i] = ok ? srcI[d.start + j] : 0;
    }
    KT* raw = reinterpret_cast<KT*>(sm.wbytes);
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int j = q + i * P;
      if (j < d.n) {
        tmin = lk[i] < tmin ? lk[i] : tmin;
        tmax = lk[i] > tmax ? lk[i] : tmax;
        if (kIdx) sm.idx[region + j] = lv[i];
      }
      raw[region + j] = lk[i];
    }
  }
  // key range of the group: its lanes, then its warps
  const int span = P < 32 ? P : 32;
  for (int o = 1; o < span; o <<= 1) {
    const KT m0 = __shfl_xor_sync(kFull, tmin, o), m1 = __shfl_xor_sync(kFull, tmax, o);
    tmin = m0 < tmin ? m0 : tmin;
    tmax = m1 > tmax ? m1 : tmax;
  }
  if (P > 32) {
    if (lane == 0) { sm.gmin[warp] = tmin; sm.gmax[warp] = tmax; }
    __syncthreads();
    const int w0 = (g * P) >> 5;
    for (int w = w0; w < w0 + (P >> 5); ++w) {
      tmin = sm.gmin[w] < tmin ? sm.gmin[w] : tmin;
      tmax = sm.gmax[w] > tmax ? sm.gmax[w] : tmax;
    }
  }
  const unsigned long long range = d.n > 0 ? (unsigned long long)(tmax - tmin) : 0ull;
  // positions of a group need log2(P * kItems) bits
  int sh = 0;
  while ((1 << sh) < P * kItems) ++sh;
  using Narrow = RangeWord<KT, uint32_t, kIdx>;
  using Mid = RangeWord<KT, uint64_t, kIdx>;
  using Full = FullWord<U, kIdx>;
  // 8/16-bit keys and 32-bit keys without ids already sort 32-bit words
  constexpr bool kNarrowOpt = !(sizeof(U) <= 2 || (sizeof(U) == 4 && !kIdx));
  if (kNarrowOpt && __syncthreads_and(range <= Narrow::max_range(sh))) {
    leaf_words_sort<U, kIdx, kV, Narrow>(a, sm, P, li, last, tmin, sh);
  } else if (sizeof(U) == 8 && kIdx && __syncthreads_and(range <= Mid::max_range(sh))) {
    leaf_words_sort<U, kIdx, kV, Mid>(a, sm, P, li, last, tmin, sh);
  } else {
    leaf_words_sort<U, kIdx, kV, Full>(a, sm, P, li, last, tmin, sh);
  }
  __syncthreads();
}

template <typename U, bool kIdx>
__device__ void fill_run(const SortArgs& a, const FillDesc& f) {
  using KT = typename Persist<U, kIdx>::KT;
  U* dst = (U*)a.keysA;
  const KT flip = (KT)a.flip;
  const KT v = (KT)f.value;
  for (int j = threadIdx.x; j < f.n; j += blockDim.x) {
    kstore<U, KT>(dst, f.start + j, v, flip);
    if (kIdx) a.idxA[f.start + j] = a.idxB[f.start + j];
  }
}

// The LEAF phase: sorts the leaves published by persistent_sort_kernel and
// fills the parked pivot runs.  An ordinary launch (no grid barrier) with its
// own register budget and the larger leaf CTA.
// Launch `slice` handles the leaves of that position slice; launch 0 also
// fills the parked pivot runs.
template <typename U, bool kIdx, int kV>
__global__ void __launch_bounds__(LeafGeom<U, kV>::kThreads, LeafGeom<U, kV>::kBlocks)
    leaf_kernel(SortArgs a, int slice) {
  using LC = LeafCfg<U, kIdx, kV>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename LC::Smem& sm = *reinterpret_cast<typename LC::Smem*>(smem_raw);
  Control* c = a.ctrl;
  const int tid = threadIdx.x;
  if (ld_acquire_int(&c->error) != 0) return;
  const int sb = slice * 16;
  unsigned* wc = &c->leafWork[slice];
  if (tid < 16) {
    sm.classItems[tid] = ld_acquire_int(&c->classItemsG[sb + tid]);
    sm.classOff[tid] = ld_acquire_int(&c->classOffG[sb + tid]);
  }
  if (tid == 0) sm.item = (int)atomicAdd(wc, 1u);
  __syncthreads();
  const int leafItems = ld_acquire_int(&c->leafItems[slice]);
  const int nf = slice == 0 ? ld_acquire_int(&c->fillItems) : 0;
  int it = sm.item;
  while (it < leafItems + nf) {
    unsigned nxt = 0;
    if (tid == 0) nxt = atomicAdd(wc, 1u);  // claim ahead
    if (it < leafItems) {
      // class k covers items [classItems[k], classItems[k-1])
      int k = LeafGeom<U, kV>::kClasses - 1;
      while (k > 0 && it >= sm.classItems[k - 1]) --k;
      const int groups = LC::kThreads >> k;
      const int first = sm.classOff[k] + (it - sm.classItems[k]) * groups;
      const int last = sm.classOff[k] + ld_acquire_int(&c->classCount[sb + k]);
      const int end = first + groups < last ? first + groups : last;
      sort_leaf_group<U, kIdx, kV>(a, k, first, end, sm);
    } else {
      fill_run<U, kIdx>(a, a.fills[it - leafItems]);
    }
    __syncthreads();
    if (tid == 0) sm.item = (int)nxt;
    __syncthreads();
    it = sm.item;
  }
  __syncthreads();
  if (tid == 0 && atomicAdd(&c->leafDone, 1) == (slice + 1) * (int)gridDim.x - 1)
    c->tEnd = global_ns();
}

// ---------------------------------------------------------------------------
// fixed-size batched sort (MultiSort): each CTA sorts kThreads/P arrays of
// arrSize <= kMax keys that lie back to back in memory.  Replaces the
// per-thread heap sort of turtle-multi-sort.cuh:87-182.
// ---------------------------------------------------------------------------
template <typename U, bool kIdx, int kV>
__global__ void __launch_bounds__(LeafGeom<U, kV>::kThreads, LeafGeom<U, kV>::kBlocks)
    multisort_kernel(U* keys, int* idx, long long numArrays, int arrSize, int cls,
                     unsigned long long flip64) {
  using LC = LeafCfg<U, kIdx, kV>;
  using KT = typename KeyCfg<U>::KT;
  constexpr int kItems = LC::kItems;
  constexpr int kLT = LC::kThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename LC::Smem& sm = *reinterpret_cast<typename LC::Smem*>(smem_raw);
  const KT flip = (KT)flip64;
  const int P = 1 << cls;
  const int groups = kLT / P;
  const int tid = threadIdx.x;
  const long long first = (long long)blockIdx.x * groups;
  const long long na = (numArrays - first) < groups ? (numArrays - first) : groups;
  const long long base = first * arrSize;
  const int total = (int)(na * arrSize);
  using LW = typename LC::LW;
  using W = typename LW::W;
  // pad every group's tail
  {
    const int g = tid / P, q = tid & (P - 1);
    for (int j = arrSize + q; j < P * kItems; j += P) sm.words()[wpad<W>(g * P * kItems + j)] = LW::sent();
  }
  // coalesced load of the whole range
  for (int j = tid; j < total; j += kLT) {
    const int g = j / arrSize, e = j - g * arrSize;
    const int slot = g * P * kItems + e;
    sm.words()[wpad<W>(slot)] = LW::make(kload<U, KT>(keys, base + j, flip), e);
    if (kIdx) sm.idx[slot] = idx[base + j];
  }
  __syncthreads();
  block_sort_words<LW, kItems>(sm.words(), P, kLT, tid / P < na ? arrSize : 0);
  for (int j = tid; j < total; j += kLT) {
    const int g = j / arrSize, e = j - g * arrSize;
    const int region = g * P * kItems;
    const W w = sm.words()[wpad<W>(region + e)];
    kstore<U, KT>(keys, base + j, (KT)LW::key(w), flip);
    if (kIdx) idx[base + j] = sm.idx[region + LW::pos(w)];
  }
}

// ---------------------------------------------------------------------------
// float keys: IEEE-754 totalOrder images
// ---------------------------------------------------------------------------

// keys[lo, hi) to their totalOrder images (negative: all bits flipped,
// positive: sign bit set), or back with `inverse`.  As unsigned integers the
// images order -NaN < -inf < ... < -0 < +0 < ... < +inf < +NaN.  With a
// control block, the map back is skipped when the partition yielded (the keys
// are still mid-sort; the resumed launch maps them back).
template <typename U>
__global__ void __launch_bounds__(256) float_order_kernel(U* keys, long long lo, long long hi,
                                                          int inverse, Control* ctrl) {
  if (ctrl != nullptr && ld_acquire_int(&ctrl->yield) != 0) return;
  constexpr U kSign = U(1) << (8 * sizeof(U) - 1);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += stride) {
    const U b = keys[i];
    const bool top = (b & kSign) != 0;
    // forward: negative (top set) -> ~b, else b | sign; inverse: an image with
    // the top bit set was positive -> b ^ sign, else -> ~b
    const U mask = (top != (inverse != 0)) ? U(~U(0)) : kSign;
    keys[i] = b ^ mask;
  }
}

template <typename U>
static cudaError_t launch_float_order(void* keys, long long lo, long long hi, bool inverse,
                                      Control* ctrl, cudaStream_t stream) {
  if (hi <= lo) return cudaSuccess;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (hi - lo + 255) / 256;
  const long long cap = (long long)(sms > 0 ? sms : 1) * 8;
  float_order_kernel<U><<<(unsigned)(want < cap ? want : cap), 256, 0, stream>>>(
      (U*)keys, lo, hi, inverse ? 1 : 0, ctrl);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
// Resident CTAs per SM of each leaf geometry (set by prepare_persistent).
static int g_leafBlocks[9][2][kLeafGeometries];

template <typename U, bool kIdx, int kV>
static cudaError_t prepare_leaf_geometry() {
  const int lsmem = (int)leaf_smem_bytes<U, kIdx, kV>();
  cudaError_t e = cudaFuncSetAttribute(multisort_kernel<U, kIdx, kV>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, lsmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(leaf_kernel<U, kIdx, kV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           lsmem);
  if (e != cudaSuccess) return e;
  int perSM = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, leaf_kernel<U, kIdx, kV>,
                                                    LeafGeom<U, kV>::kThreads, lsmem);
  if (e != cudaSuccess) return e;
  if (perSM < 1) return cudaErrorInvalidConfiguration;
  g_leafBlocks[sizeof(U)][kIdx ? 1 : 0][kV] = perSM;
  return cudaSuccess;
}

template <typename U, bool kIdx>
static cudaError_t prepare_persistent(int device, int* gridOut) {
  const size_t smem = persist_smem_bytes<U, kIdx>();
  cudaError_t e = cudaFuncSetAttribute(persistent_sort_kernel<U, kIdx, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(persistent_sort_kernel<U, kIdx, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if ((e = prepare_leaf_geometry<U, kIdx, 0>()) != cudaSuccess) return e;
  if ((e = prepare_leaf_geometry<U, kIdx, 1>()) != cudaSuccess) return e;
  if ((e = prepare_leaf_geometry<U, kIdx, 2>()) != cudaSuccess) return e;
  if ((e = prepare_leaf_geometry<U, kIdx, 3>()) != cudaSuccess) return e;
  int perSM = 0, perSMWide = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, persistent_sort_kernel<U, kIdx, false>,
                                                    kThreads, smem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSMWide,
                                                    persistent_sort_kernel<U, kIdx, true>, kThreads,
                                                    smem);
  if (e != cudaSuccess) return e;
  perSM = perSM < perSMWide ? perSM : perSMWide;  // one grid serves both forms
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  if (perSM < 1) return cudaErrorInvalidConfiguration;
  *gridOut = perSM * sms;
  return cudaSuccess;
}

template <typename U, bool kIdx, int kV>
static cudaError_t launch_leaf(const SortArgs& a, int slice, int sms, cudaStream_t stream) {
  const int per = g_leafBlocks[sizeof(U)][kIdx ? 1 : 0][kV];
  leaf_kernel<U, kIdx, kV><<<(unsigned)(sms * (per > 0 ? per : 1)), LeafGeom<U, kV>::kThreads,
                             leaf_smem_bytes<U, kIdx, kV>(), stream>>>(a, slice);
  return cudaGetLastError();
}

// The partition kernel on `grid` CTAs (at most the resident maximum), then
// the leaf kernel of geometry a.leafVariant once per position slice.
template <typename U, bool kIdx>
static cudaError_t launch_persistent(const SortArgs& a, int grid, cudaStream_t stream,
                                     cudaEvent_t mid, const cudaEvent_t* sliceDone) {
  constexpr bool kFloatable = sizeof(U) >= 4;  // float32 / float64 storage
  cudaError_t e = cudaSuccess;
  if (kFloatable && a.fbits != 0 && !a.resume &&
      (e = launch_float_order<U>(a.keysA, 0, a.n, false, nullptr, stream)) != cudaSuccess)
    return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = persist_smem_bytes<U, kIdx>();
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = a.samples == kWideSamples
          ? cudaLaunchKernelEx(&cfg, persistent_sort_kernel<U, kIdx, true>, a)
          : cudaLaunchKernelEx(&cfg, persistent_sort_kernel<U, kIdx, false>, a);
  if (e != cudaSuccess) return e;
  if (mid != nullptr && (e = cudaEventRecord(mid, stream)) != cudaSuccess) return e;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) sms = 1;
  for (int sl = 0; sl < a.slices; ++sl) {
    switch (a.leafVariant) {
      case 0: e = launch_leaf<U, kIdx, 0>(a, sl, sms, stream); break;
      case 2: e = launch_leaf<U, kIdx, 2>(a, sl, sms, stream); break;
      case 3: e = launch_leaf<U, kIdx, 3>(a, sl, sms, stream); break;
      default: e = launch_leaf<U, kIdx, 1>(a, sl, sms, stream); break;
    }
    if (e != cudaSuccess) return e;
    if (kFloatable && a.fbits != 0) {
      // keys of this slice are final: back from totalOrder images
      const long long lo = (sl * a.n + a.slices - 1) / a.slices;
      const long long hi = ((sl + 1) * a.n + a.slices - 1) / a.slices;
      if ((e = launch_float_order<U>(a.keysA, lo, hi, true, a.ctrl, stream)) != cudaSuccess)
        return e;
    }
    if (sliceDone != nullptr && (e = cudaEventRecord(sliceDone[sl], stream)) != cudaSuccess)
      return e;
  }
  return cudaSuccess;
}

template <typename U, bool kIdx, int kV>
static cudaError_t launch_multisort_geom(void* keys, int* idx, long long numArrays, int arrSize,
                                         unsigned long long flip, cudaStream_t stream) {
  constexpr int kItems = LeafGeom<U, kV>::kItems, kLT = LeafGeom<U, kV>::kThreads;
  int cls = 0;
  while ((1 << cls) * kItems < arrSize) ++cls;
  const int groups = kLT >> cls;
  const long long blocks = (numArrays + groups - 1) / groups;
  if (blocks <= 0) return cudaSuccess;
  multisort_kernel<U, kIdx, kV><<<(unsigned)blocks, kLT, leaf_smem_bytes<U, kIdx, kV>(), stream>>>(
      (U*)keys, idx, numArrays, arrSize, cls, flip);
  return cudaGetLastError();
}

template <typename U, bool kIdx>
static cudaError_t launch_multisort(void* keys, int* idx, long long numArrays, int arrSize,
                                    unsigned long long flip, int fbits, int geometry,
                                    cudaStream_t stream) {
  if (numArrays <= 0) return cudaSuccess;
  constexpr bool kFloatable = sizeof(U) >= 4;
  const long long total = numArrays * (long long)arrSize;
  cudaError_t e;
  if (kFloatable && fbits != 0 &&
      (e = launch_float_order<U>(keys, 0, total, false, nullptr, stream)) != cudaSuccess)
    return e;
  switch (geometry) {
    case 0: e = launch_multisort_geom<U, kIdx, 0>(keys, idx, numArrays, arrSize, flip, stream); break;
    case 2: e = launch_multisort_geom<U, kIdx, 2>(keys, idx, numArrays, arrSize, flip, stream); break;
    case 3: e = launch_multisort_geom<U, kIdx, 3>(keys, idx, numArrays, arrSize, flip, stream); break;
    default: e = launch_multisort_geom<U, kIdx, 1>(keys, idx, numArrays, arrSize, flip, stream); break;
  }
  if (e != cudaSuccess) return e;
  if (kFloatable && fbits != 0) return launch_float_order<U>(keys, 0, total, true, nullptr, stream);
  return cudaSuccess;
}

// dispatch on key width / index
#define TURTLE_WIDTH_DISPATCH(width, hasIdx, CALL)                                  \
  switch (width) {                                                                  \
    case 1: if (hasIdx) { using U = uint8_t; constexpr bool I = true; return CALL; } \
            else { using U = uint8_t; constexpr bool I = false; return CALL; }        \
    case 2: if (hasIdx) { using U = uint16_t; constexpr bool I = true; return CALL; } \
            else { using U = uint16_t; constexpr bool I = false; return CALL; }       \
    case 4: if (hasIdx) { using U = uint32_t; constexpr bool I = true; return CALL; } \
            else { using U = uint32_t; constexpr bool I = false; return CALL; }       \
    case 8: if (hasIdx) { using U = uint64_t; constexpr bool I = true; return CALL; } \
            else { using U = uint64_t; constexpr bool I = false; return CALL; }       \
    default: return cudaErrorInvalidValue;                                          \
  }

cudaError_t kernels_prepare(int width, bool hasIdx, int device, int* grid) {
  TURTLE_WIDTH_DISPATCH(width, hasIdx, (prepare_persistent<U, I>(device, grid)));
}

cudaError_t kernels_launch_persistent(int width, bool hasIdx, const SortArgs& a, int grid,
                                      cudaStream_t stream, cudaEvent_t mid,
                                      const cudaEvent_t* sliceDone, cudaEvent_t passStart,
                                      const cudaEvent_t* keysReady, int keyChunks) {
  if (a.radix)
    return kernels_launch_radix(width, hasIdx, a, stream, mid, sliceDone, passStart, keysReady,
                                keyChunks);
  if (passStart != nullptr) {
    const cudaError_t e = cudaEventRecord(passStart, stream);
    if (e != cudaSuccess) return e;
  }
  TURTLE_WIDTH_DISPATCH(width, hasIdx,
                        (launch_persistent<U, I>(a, grid, stream, mid, sliceDone)));
}

cudaError_t kernels_launch_multisort(int width, bool hasIdx, void* keys, int* idx,
                                     long long numArrays, int arrSize, unsigned long long flip,
                                     int fbits, int geometry, cudaStream_t stream) {
  TURTLE_WIDTH_DISPATCH(width, hasIdx, (launch_multisort<U, I>(keys, idx, numArrays, arrSize, flip,
                                                               fbits, geometry, stream)));
}

int kernels_tile_elems(int width) {
  switch (width) {
    case 1: return Geom<uint8_t>::kTile;
    case 2: return Geom<uint16_t>::kTile;
    case 4: return Geom<uint32_t>::kTile;
    case 8: return Geom<uint64_t>::kTile;
    default: return 0;
  }
}

// Geometry of leaf / MultiSort variant g for keys of `width` bytes: CTA
// threads, keys per thread, capacity, size classes.
void kernels_leaf_geometry(int width, int g, int* threads, int* items, int* capacity,
                           int* classes) {
  const int base = width == 8 ? 8 : 16;
  const int t = g == 0 ? 256 : g == 2 ? 1024 : 512;
  const int it = g == 3 ? base / 2 : base;
  if (threads) *threads = t;
  if (items) *items = it;
  if (capacity) *capacity = t * it;
  if (classes) {
    int c = 1;
    while ((1 << (c - 1)) < t) ++c;
    *classes = c;
  }
}

int kernels_leaf_max(int width) {
  int cap = 0;
  kernels_leaf_geometry(width, kDefaultLeafGeometry, nullptr, nullptr, &cap, nullptr);
  return (width == 1 || width == 2 || width == 4 || width == 8) ? cap : 0;
}

}  // namespace turtle
