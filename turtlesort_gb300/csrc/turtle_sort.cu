// GB300 TurtleSort kernels: the persistent work-list quicksort, the leaf
// kernel and the fixed-size batched (MultiSort) kernel.
//
// persistent_sort_kernel (replaces the CDP2 chain copyTasksBack ->
// resetNumTasks -> quickSortWithoutStreamCompaction / bruteSort,
// turtle-sort.cu:35-188,573-934): one cooperative launch of (SMs x 2) blocks
// walks the partition tree level by level.  Every level has two phases
// separated by a bounded grid barrier:
//   COUNT   each tile (kTile elements of one segment, aligned to absolute
//           kTile boundaries) counts its keys against the segment's pivots;
//           the CTA that completes a segment's last tile plans it: per-class
//           totals, per-tile destination offsets and the children
//           (next-level segments with their tile descriptors, leaves, parked
//           pivot runs).
//   SCATTER each tile re-reads its keys (+ids), ranks them stably per class
//           (thread-local counts + one block scan), stages them by class in
//           shared memory and writes each class run coalesced to its
//           destination in the other buffer.  Pivot runs are written by value
//           and never recursed into.  The tile that writes a child's first,
//           middle or last element records it in the child's descriptor:
//           those are the child's pivots.
// Children live in the other buffer (ping-pong A <-> B), so there is no
// copy-back pass.  At the end the kernel buckets the leaves by size and hands
// them to leaf_kernel, which sorts them in shared memory (short leaves with the
// register network + merge-path merge, long ones with the stable radix groups)
// and fills the parked pivot runs.  If the leaf lists would overflow before
// the tree is done (pathological inputs only), the kernel yields: the host
// runs leaf_kernel and relaunches the partition from the saved level.
//
// Pivots are the reference's: sorted{a[start + n/2], a[start], a[stop]}
// (turtle-sort.cu:641-655).  After kDepthSwitch levels a segment's pivots are
// the quartiles of 31 evenly spaced samples instead, which bounds the depth on
// inputs built against median-of-3; the output does not depend on the pivots
// (every step is stable, so the result equals a stable sort by key).
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "turtle_device.cuh"
#include "turtle_internal.h"

namespace turtle {

// Leaf size classes: class c uses P = 1 << c threads of the leaf CTA.
// Classes up to kMergeClassMax use the register network + merge-path groups;
// larger ones the radix groups of P / 32 warps.
constexpr int kMergeClassMax = 4;
// The merge-path groups measured faster than the radix groups for every leaf
// class on GB300, so the radix groups are compiled out of the leaf sort.
constexpr bool kRadixLeaves = false;
constexpr int kCountBatch = 8;  // tiles per COUNT work item

template <typename U, bool kIdx>
struct Persist {
  using G = Geom<U>;
  using KT = typename G::KT;
  static constexpr int kItems = G::kItems;
  static constexpr int kTile = G::kTile;
  static constexpr int kLeafMax = G::kLeafMax;
  static constexpr int kIdxSlots = kIdx ? G::kIdxSlots : 4;

  struct Smem {  // partition CTA
    KT keys[G::kKeySlots];
    int idx[kIdxSlots];
    int classStart[8];
    int cnt[8];
    long long toff[8];
    long long red[kWarps][8];
    long long carry[8];
    long long tot[8];
    long long cbase[8];
    long long ppos[4][3];       // child pivot positions (start+n/2, start, stop)
    long long dbias[8];         // per-class destination minus stage index
    unsigned wpred[kWarps][4];  // COUNT: per-warp predicate totals
    unsigned wscan[kWarps][4];  // SCATTER: per-warp class-count totals
    long long wbase[kWarps][8];  // SCATTER: per-warp destination base per class
    unsigned dstRel[kWarps * (32 * kItems + kItems)];  // SCATTER: staged destinations
    unsigned wpre[kWarps][4];   // SCATTER: exclusive warp prefixes
    TileDesc tds[kCountBatch];
    int childSeg[4];
    int childTb[4], childNt[4];
    long long childStart[4], childN[4];
    KT piv[3];
    unsigned lut;
    int seg, item, nPlan;
    int segList[kCountBatch];
    int planList[kCountBatch];
    int classOff[16];
    int classItems[16];
  };

  static constexpr int kLIdxSlots = kIdx ? G::kLeafIdxSlots : 4;
  struct LeafSmem {  // leaf / batched CTA
    KT keys[G::kLeafKeySlots];
    int idx[kLIdxSlots];
    int rcnt[kLWarps * 256 + kLWarps];
    KT rred[2 * kLWarps];
    int rpass;
    int item;
    int classOff[16];
    int classItems[16];
  };
};

template <typename U, bool kIdx>
constexpr size_t persist_smem_bytes() {
  return sizeof(typename Persist<U, kIdx>::Smem);
}
template <typename U, bool kIdx>
constexpr size_t leaf_smem_bytes() {
  return sizeof(typename Persist<U, kIdx>::LeafSmem);
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
  for (int i = 0; i < 31; ++i) s[i] = kload<U, KT>(src, start + (n * (2 * i + 1)) / 62, flip);
  for (int i = 1; i < 31; ++i) {
    KT x = s[i];
    int j = i - 1;
    while (j >= 0 && x < s[j]) { s[j + 1] = s[j]; --j; }
    s[j + 1] = x;
  }
  piv[0] = s[7]; piv[1] = s[15]; piv[2] = s[23];
}

// Pivots of a segment: the captured candidates, or samples on deep levels.
template <typename KT, typename U>
__device__ __forceinline__ void segment_pivots(const SegDesc& sd, const U* src, int level, KT flip,
                                               KT* piv) {
  if (level < kDepthSwitch)
    sort3<KT>((KT)__ldcg(&sd.piv[0]), (KT)__ldcg(&sd.piv[1]), (KT)__ldcg(&sd.piv[2]), piv);
  else
    sampled_pivots<KT, U>(src, __ldcg(&sd.start), __ldcg(&sd.n), flip, piv);
}

template <int kTile>
__device__ __forceinline__ long long tiles_of(long long start, long long n) {
  return (start + n - 1) / kTile - start / kTile + 1;
}

// Allocate a next-level segment (tile range allocated with the same 64-bit
// atomic, so tileBase grows with the segment index).  Returns the segment
// index or -1 on overflow.  The caller writes the tile descriptors.
template <int kTile>
__device__ int alloc_segment(const SortArgs& a, int par, long long start, long long n,
                             int* tbOut, int* ntOut) {
  const long long nt = tiles_of<kTile>(start, n);
  const unsigned long long old =
      atomicAdd(&a.ctrl->segTile[par], (1ull << 32) | (unsigned long long)nt);
  const int si = (int)(old >> 32);
  const long long tb = (long long)(old & 0xffffffffull);
  if (si >= a.segCap || tb + nt > a.tileCap) {
    set_error(a.ctrl, kDevCapacity);
    return -1;
  }
  SegDesc d;
  d.start = start; d.n = n; d.tileBase = (int)tb; d.ntiles = (int)nt; d.done = 0; d.pad = 0;
  d.piv[0] = d.piv[1] = d.piv[2] = 0;
  for (int c = 0; c < 8; ++c) d.cbase[c] = 0;
  for (int c = 0; c < 4; ++c) d.childSeg[c] = -1;
  a.segs[par][si] = d;
  *tbOut = (int)tb;
  *ntOut = (int)nt;
  return si;
}

// Tile descriptors of a segment, written by threads [t0, t0+stride) of a group.
template <int kTile>
__device__ void write_tiles(const SortArgs& a, int par, int si, int tb, int nt, long long start,
                            long long n, int t0, int stride) {
  const long long first = start / kTile;
  const long long end = start + n;
  for (int i = t0; i < nt; i += stride) {
    const long long abs0 = (first + i) * (long long)kTile;
    TileDesc d;
    d.lo = abs0 > start ? abs0 : start;
    d.hi = (abs0 + kTile) < end ? (abs0 + kTile) : end;
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
  if (li >= a.leafCap) { set_error(a.ctrl, kDevCapacity); return; }
  LeafDesc d;
  d.start = start; d.n = (int)n; d.inB = inB;
  a.leaves[li] = d;
}

__device__ void push_fill(const SortArgs& a, long long start, long long n, unsigned long long v) {
  for (long long o = 0; o < n; o += kFillChunk) {
    const int fi = atomicAdd(&a.ctrl->fillCount, 1);
    if (fi >= a.fillCap) { set_error(a.ctrl, kDevCapacity); return; }
    FillDesc d;
    d.start = start + o;
    d.n = (int)((n - o) < kFillChunk ? (n - o) : kFillChunk);
    d.pad = 0;
    d.value = v;
    a.fills[fi] = d;
  }
}

// Route one input array at init: nothing, leaf, or level-0 segment (whose
// pivots this thread reads, and whose tiles it writes when writeTiles).
template <typename U, int kTile, int kLeafMax>
__device__ void route_input(const SortArgs& a, long long start, long long n, bool writeTiles,
                            int* siOut, int* tbOut, int* ntOut) {
  *siOut = -1;
  *tbOut = 0;
  *ntOut = 0;
  if (n <= 1) return;
  if (n <= kLeafMax) { push_leaf(a, start, n, 0); return; }
  int tb = 0, nt = 0;
  const int si = alloc_segment<kTile>(a, 0, start, n, &tb, &nt);
  if (si < 0) return;
  using KT = typename KeyCfg<U>::KT;
  const U* src = (const U*)a.keysA;
  const KT flip = (KT)a.flip;
  SegDesc* sd = &a.segs[0][si];
  sd->piv[0] = (unsigned long long)kload<U, KT>(src, start + n / 2, flip);
  sd->piv[1] = (unsigned long long)kload<U, KT>(src, start, flip);
  sd->piv[2] = (unsigned long long)kload<U, KT>(src, start + n - 1, flip);
  if (writeTiles) write_tiles<kTile>(a, 0, si, tb, nt, start, n, 0, 1);
  *siOut = si; *tbOut = tb; *ntOut = nt;
}

// ---------------------------------------------------------------------------
// COUNT phase: one warp chunk (kWarpChunk elements of a tile)
// ---------------------------------------------------------------------------

// Class counts from the six predicate totals #(k<p1), #(k<=p1), #(k<p2),
// #(k<=p2), #(k<p3), #(k<=p3) of nt elements: class boundaries b1..b6 (max()
// keeps them ordered when pivots are equal, which sends every key equal to a
// pivot to the first equal pivot's class, as the reference's test order
// does).  The map is additive over disjoint element sets, so per-chunk counts
// sum to per-tile counts.
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

// Tile t, counted by one warp: the tile's keys against the segment's pivots,
// chunk by chunk (the next chunk loads while the current one is counted); the
// tile's class counts go to tileCnt.  Warps stream independently.
template <typename U, bool kIdx>
__device__ __forceinline__ void count_tile_warp(const SortArgs& a, int level, int t) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kItems = P::kItems, kTile = P::kTile, kWCH = Geom<U>::kWarpChunk;
  const int par = level & 1;
  const int lane = threadIdx.x & 31;
  const U* src = (const U*)(par ? a.keysB : a.keysA);
  const KT flip = (KT)a.flip;
  const TileDesc td = load_tile(&a.tiles[par][t]);
  const long long abs0 = (td.lo / kTile) * (long long)kTile;
  const int rlo = (int)(td.lo - abs0), rhi = (int)(td.hi - abs0);
  const U* tb = src + abs0;
  const int chBeg = rlo / kWCH, chEnd = (rhi + kWCH - 1) / kWCH;
  KT key[kItems];
  unsigned okm = load_chunk<U, KT, kItems>(tb, abs0, a.n, chBeg * kWCH + lane * kItems, rlo, rhi,
                                           flip, key);
  KT piv[3];
  segment_pivots<KT, U>(a.segs[par][td.seg], src, level, flip, piv);
  unsigned w0 = 0, w1 = 0, w2 = 0;  // (k<p | k<=p << 16) for p1, p2, p3
  for (int ch = chBeg; ch < chEnd; ++ch) {
    KT keyn[kItems];
    unsigned okn = 0;
    if (ch + 1 < chEnd)
      okn = load_chunk<U, KT, kItems>(tb, abs0, a.n, (ch + 1) * kWCH + lane * kItems, rlo, rhi,
                                      flip, keyn);
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      if (okm >> i & 1u) {
        const KT x = key[i];
        w0 += (x < piv[0] ? 1u : 0u) + (x <= piv[0] ? 0x10000u : 0u);
        w1 += (x < piv[1] ? 1u : 0u) + (x <= piv[1] ? 0x10000u : 0u);
        w2 += (x < piv[2] ? 1u : 0u) + (x <= piv[2] ? 0x10000u : 0u);
      }
    }
    okm = okn;
#pragma unroll
    for (int i = 0; i < kItems; ++i) key[i] = keyn[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    w0 += __shfl_xor_sync(0xffffffffu, w0, o);
    w1 += __shfl_xor_sync(0xffffffffu, w1, o);
    w2 += __shfl_xor_sync(0xffffffffu, w2, o);
  }
  int pc[6], cc[7];
  pc[0] = (int)(w0 & 0xffffu); pc[1] = (int)(w0 >> 16);
  pc[2] = (int)(w1 & 0xffffu); pc[3] = (int)(w1 >> 16);
  pc[4] = (int)(w2 & 0xffffu); pc[5] = (int)(w2 >> 16);
  classes_from_predicates(pc, rhi - rlo, cc);
  if (lane < 8) {
    int v = 0;
#pragma unroll
    for (int c = 0; c < 7; ++c) v = (lane == c) ? cc[c] : v;
    a.tileCnt[par][(long long)t * 8 + lane] = v;
  }
}

// ---------------------------------------------------------------------------
// PLAN phase: one segment per CTA
// ---------------------------------------------------------------------------

// Turns the per-tile class counts of segment `seg` into destination offsets
// (class bases as in turtle-sort.cu:755-761, then tiles in memory order, which
// makes the partition stable), routes the children (turtle-sort.cu:857-933)
// and stores the segment's sorted pivots and class table for SCATTER.
template <typename U, bool kIdx>
__device__ __noinline__ void plan_segment(const SortArgs& a, int level, int seg,
                                          typename Persist<U, kIdx>::Smem& sm) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kTile = P::kTile, kLeafMax = P::kLeafMax;
  const int par = level & 1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  SegDesc* sdp = &a.segs[par][seg];
  if (tid == 0)
    segment_pivots<KT, U>(*sdp, (const U*)(par ? a.keysB : a.keysA), level, (KT)a.flip, sm.piv);
  const long long sdStart = __ldcg(&sdp->start);
  const int tileBase = __ldcg(&sdp->tileBase);
  const int nt = __ldcg(&sdp->ntiles);
  const int* cnt = a.tileCnt[par] + (long long)tileBase * 8;
  long long* off = a.tileOff[par] + (long long)tileBase * 8;

  // thread `tid` owns the consecutive tiles [tid*per, (tid+1)*per)
  const int per = (nt + kThreads - 1) / kThreads;
  const int tBeg = min(nt, tid * per), tEnd = min(nt, tBeg + per);
  long long s[7];
#pragma unroll
  for (int c = 0; c < 7; ++c) s[c] = 0;
  const int4* cnt4 = reinterpret_cast<const int4*>(cnt);
  for (int t0 = tBeg; t0 < tEnd; t0 += 4) {
    int4 r[8];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const bool ok = t0 + u < tEnd;
      r[2 * u] = ok ? __ldcg(&cnt4[(long long)(t0 + u) * 2]) : make_int4(0, 0, 0, 0);
      r[2 * u + 1] = ok ? __ldcg(&cnt4[(long long)(t0 + u) * 2 + 1]) : make_int4(0, 0, 0, 0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      s[0] += r[2 * u].x; s[1] += r[2 * u].y; s[2] += r[2 * u].z; s[3] += r[2 * u].w;
      s[4] += r[2 * u + 1].x; s[5] += r[2 * u + 1].y; s[6] += r[2 * u + 1].z;
    }
  }
  // block exclusive scan of the per-thread sums, and the class totals
  long long inc[7];
#pragma unroll
  for (int c = 0; c < 7; ++c) {
    long long x = s[c];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    inc[c] = x;
  }
  if (lane == 31) {
#pragma unroll
    for (int c = 0; c < 7; ++c) sm.red[warp][c] = inc[c];
  }
  __syncthreads();
  if (tid < 7) {
    long long acc = 0;
    for (int w = 0; w < kWarps; ++w) {
      const long long x = sm.red[w][tid];
      sm.red[w][tid] = acc;
      acc += x;
    }
    sm.tot[tid] = acc;
  }
  __syncthreads();
  if (tid == 0) {
    long long b = sdStart;
    for (int c = 0; c < 7; ++c) { sm.cbase[c] = b; b += sm.tot[c]; }
    sm.cbase[7] = b;
  }
  __syncthreads();
  {
    long long run[7];
#pragma unroll
    for (int c = 0; c < 7; ++c) run[c] = sm.cbase[c] + sm.red[warp][c] + (inc[c] - s[c]);
    for (int t0 = tBeg; t0 < tEnd; t0 += 4) {
      int4 r[8];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const bool ok = t0 + u < tEnd;
        r[2 * u] = ok ? __ldcg(&cnt4[(long long)(t0 + u) * 2]) : make_int4(0, 0, 0, 0);
        r[2 * u + 1] = ok ? __ldcg(&cnt4[(long long)(t0 + u) * 2 + 1]) : make_int4(0, 0, 0, 0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (t0 + u < tEnd) {
          const int v[7] = {r[2 * u].x, r[2 * u].y, r[2 * u].z, r[2 * u].w,
                            r[2 * u + 1].x, r[2 * u + 1].y, r[2 * u + 1].z};
          longlong2* o = reinterpret_cast<longlong2*>(off + (long long)(t0 + u) * 8);
          o[0] = make_longlong2(run[0], run[1]);
          o[1] = make_longlong2(run[2], run[3]);
          o[2] = make_longlong2(run[4], run[5]);
          o[3] = make_longlong2(run[6], 0);
#pragma unroll
          for (int c = 0; c < 7; ++c) run[c] += v[c];
        }
      }
    }
  }

  // children: thread 0 routes them; the CTA writes the tile descriptors
  const bool dstIsA = (par == 1);
  const int nextPar = par ^ 1;
  if (tid == 0) {
    for (int c = 0; c < 7; ++c) {
      const long long pos = sm.cbase[c];
      const long long m = sm.cbase[c + 1] - pos;
      if (c & 1) {
        if (m > 0 && !dstIsA) push_fill(a, pos, m, (unsigned long long)sm.piv[c >> 1]);
        continue;
      }
      const int ci = c >> 1;
      sm.childSeg[ci] = -1;
      if (m <= 0 || (m == 1 && dstIsA)) continue;
      if (m <= kLeafMax) {
        push_leaf(a, pos, m, dstIsA ? 0 : 1);
        continue;
      }
      int tb = 0, ntc = 0;
      const int si = alloc_segment<kTile>(a, nextPar, pos, m, &tb, &ntc);
      sm.childSeg[ci] = si;
      sm.childTb[ci] = tb;
      sm.childNt[ci] = si >= 0 ? ntc : 0;
      sm.childStart[ci] = pos;
      sm.childN[ci] = m;
    }
    for (int c = 0; c < 8; ++c) sdp->cbase[c] = sm.cbase[c];
    for (int ci = 0; ci < 4; ++ci) sdp->childSeg[ci] = sm.childSeg[ci];
    for (int k = 0; k < 3; ++k) sdp->pivS[k] = (unsigned long long)sm.piv[k];
    sdp->lut = pivot_lut(sm.piv[0] == sm.piv[1], sm.piv[1] == sm.piv[2]);
  }
  __syncthreads();
  for (int ci = 0; ci < 4; ++ci) {
    if (sm.childSeg[ci] >= 0)
      write_tiles<kTile>(a, nextPar, sm.childSeg[ci], sm.childTb[ci], sm.childNt[ci],
                         sm.childStart[ci], sm.childN[ci], tid, kThreads);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// SCATTER phase: one tile per warp
// ---------------------------------------------------------------------------
// The warp walks its tile chunk by chunk (kWarpChunk elements; the next chunk
// loads while the current one is written).  Per chunk it ranks the keys stably
// per class (lane-local counts + a warp scan) and writes every element straight
// to base[class] + rank, where base[class] starts at the tile's offset from the
// plan and advances by each chunk's class counts.  Class runs of one chunk are
// contiguous, and consecutive chunks continue each other's runs.
template <typename U, bool kIdx>
__device__ __forceinline__ void scatter_tile_warp(const SortArgs& a, int level, int t,
                                                  typename Persist<U, kIdx>::Smem& sm) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kItems = P::kItems, kTile = P::kTile, kWCH = Geom<U>::kWarpChunk;
  const int par = level & 1;
  const bool dstIsA = (par == 1);
  const KT flip = (KT)a.flip;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const TileDesc td = load_tile(&a.tiles[par][t]);
  const long long abs0 = (td.lo / kTile) * (long long)kTile;
  const int rlo = (int)(td.lo - abs0), rhi = (int)(td.hi - abs0);
  const U* tb = (const U*)(par ? a.keysB : a.keysA) + abs0;
  const int* tbI = (par ? a.idxB : a.idxA) + abs0;
  const int chBeg = rlo / kWCH, chEnd = (rhi + kWCH - 1) / kWCH;
  KT key[kItems];
  int id[kIdx ? kItems : 1];
  unsigned okm = load_chunk<U, KT, kItems>(tb, abs0, a.n, chBeg * kWCH + lane * kItems, rlo, rhi,
                                           flip, key);
  if (kIdx) load_ids<kItems>(tbI, abs0, a.n, chBeg * kWCH + lane * kItems, okm, id);
  // segment metadata written by the plan (L2 reads: the plan ran on another SM)
  const SegDesc* sdp = &a.segs[par][td.seg];
  const KT p1 = (KT)__ldcg(&sdp->pivS[0]), p2 = (KT)__ldcg(&sdp->pivS[1]),
           p3 = (KT)__ldcg(&sdp->pivS[2]);
  const unsigned lut = __ldcg(&sdp->lut);
  // lanes 0..6: running destination base of class `lane`; lanes 0..11: the
  // children's pivot candidate positions a[start+n/2], a[start], a[stop]
  long long base = lane < 7 ? __ldcg(&a.tileOff[par][(long long)t * 8 + lane]) : 0;
  long long cpos = -1;
  int cchild = -1;
  if (lane < 12) {
    const int ci = lane / 3, j = lane - 3 * ci, c = 2 * ci;
    cchild = __ldcg(&sdp->childSeg[ci]);
    if (cchild >= 0) {
      const long long cb = __ldcg(&sdp->cbase[c]), cn = __ldcg(&sdp->cbase[c + 1]) - cb;
      cpos = j == 0 ? cb + cn / 2 : j == 1 ? cb : cb + cn - 1;
    }
  }
  U* dst = (U*)(par ? a.keysA : a.keysB);
  int* dstI = par ? a.idxA : a.idxB;
  long long* wb = sm.wbase[warp];
  constexpr int kStride = kWCH + kWCH / 32;  // padded stage slice per warp
  static_assert(kWarps * kStride <= Geom<U>::kKeySlots, "stage slices exceed the key stage");
  static_assert(!kIdx || kWarps * kStride <= Geom<U>::kIdxSlots, "stage slices exceed the id stage");
  KT* skeys = sm.keys + warp * kStride;
  int* sidx = sm.idx + (kIdx ? warp * kStride : 0);
  unsigned* sdst = sm.dstRel + warp * kStride;
  const long long segStartOf = __ldcg(&sdp->start);
  for (int ch = chBeg; ch < chEnd; ++ch) {
    KT keyn[kItems];
    int idn[kIdx ? kItems : 1];
    unsigned okn = 0;
    if (ch + 1 < chEnd) {
      const int en = (ch + 1) * kWCH + lane * kItems;
      okn = load_chunk<U, KT, kItems>(tb, abs0, a.n, en, rlo, rhi, flip, keyn);
      if (kIdx) load_ids<kItems>(tbI, abs0, a.n, en, okn, idn);
    }
    // classes and lane-local ranks (memory order inside the lane's items)
    unsigned long long acc = 0;       // 8-bit count per class
    unsigned info[(kItems + 3) / 4];  // (class | local rank << 3) per element
#pragma unroll
    for (int j = 0; j < (kItems + 3) / 4; ++j) info[j] = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      unsigned code = 0xffu;
      if (okm >> i & 1u) {
        const int c = class_lut<KT>(key[i], p1, p2, p3, lut);
        const unsigned lr = (unsigned)(acc >> (8 * c)) & 0xffu;
        acc += 1ull << (8 * c);
        code = (unsigned)c | (lr << 3);
      }
      info[i >> 2] |= code << (8 * (i & 3));
    }
    // warp exclusive scan of the lane counts (four words of 16-bit fields)
    unsigned w[4], ex[4], tot[4];
    w[0] = (unsigned)(acc & 0xff) | (unsigned)((acc >> 8) & 0xff) << 16;
    w[1] = (unsigned)((acc >> 16) & 0xff) | (unsigned)((acc >> 24) & 0xff) << 16;
    w[2] = (unsigned)((acc >> 32) & 0xff) | (unsigned)((acc >> 40) & 0xff) << 16;
    w[3] = (unsigned)((acc >> 48) & 0xff);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      unsigned x = w[q];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      ex[q] = x - w[q];
      tot[q] = __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane < 7) wb[lane] = base;
    __syncwarp();
    // stage the chunk class by class in the warp's slice, with each element's
    // destination relative to the segment start (bit 31: a pivot-run key that
    // waits in B for its fill)
    int cs[8];
    {
      int run = 0;
#pragma unroll
      for (int c = 0; c < 7; ++c) {
        cs[c] = run;
        run += (int)((tot[c >> 1] >> (16 * (c & 1))) & 0xffffu);
      }
      cs[7] = run;
    }
    const long long segStart = segStartOf;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const unsigned code = (info[i >> 2] >> (8 * (i & 3))) & 0xffu;
      if (code != 0xffu) {
        const int c = code & 7;
        const int q = c >> 1;
        const unsigned eq = q == 0 ? ex[0] : q == 1 ? ex[1] : q == 2 ? ex[2] : ex[3];
        const unsigned rk = ((eq >> (16 * (c & 1))) & 0xffffu) + (code >> 3);
        const int pos = cs[c] + (int)rk;
        const int sp = pos + (pos >> 5);
        skeys[sp] = key[i];
        if (kIdx) sidx[sp] = id[i];
        const unsigned rel = (unsigned)(wb[c] - segStart) + rk;
        sdst[sp] = ((c & 1) && !dstIsA) ? (rel | 0x80000000u) : rel;
      }
    }
    __syncwarp();
    // write out: consecutive stage slots of one class go to consecutive addresses
    {
      const int n = cs[7];
#pragma unroll
      for (int j = 0; j < kItems; ++j) {
        const int i = lane + 32 * j;
        if (i < n) {
          const int sp = i + (i >> 5);
          const unsigned rel = sdst[sp];
          const long long d = segStart + (long long)(rel & 0x7fffffffu);
          if (!(rel & 0x80000000u)) dst[d] = U(skeys[sp] ^ flip);
          if (kIdx) dstI[d] = sidx[sp];
        }
      }
    }
    // a child pivot candidate written by this chunk: the lane holding it
    // records the key (rare; one ballot otherwise)
    {
      bool in = false;
      long long r = 0;
      if (lane < 12 && cchild >= 0) {
        const int c = 2 * (lane / 3);
        const unsigned cnt = (tot[c >> 1] >> (16 * (c & 1))) & 0xffffu;
        r = cpos - wb[c];
        in = r >= 0 && r < (long long)cnt;
      }
      unsigned m = __ballot_sync(0xffffffffu, in);
      while (m) {
        const int srcl = __ffs(m) - 1;
        m &= m - 1;
        const int c = 2 * (srcl / 3), j = srcl - 3 * (srcl / 3);
        const int rr = (int)__shfl_sync(0xffffffffu, r, srcl);
        const int child = __shfl_sync(0xffffffffu, cchild, srcl);
        const unsigned eq = (ex[c >> 1] >> (16 * (c & 1))) & 0xffffu;
        const unsigned cn = (w[c >> 1] >> (16 * (c & 1))) & 0xffffu;
        if ((unsigned)rr >= eq && (unsigned)rr < eq + cn) {  // exactly one lane
          const unsigned want = (unsigned)rr - eq;
#pragma unroll
          for (int i = 0; i < kItems; ++i) {
            const unsigned code = (info[i >> 2] >> (8 * (i & 3))) & 0xffu;
            if (code != 0xffu && (int)(code & 7) == c && (code >> 3) == want)
              a.segs[par ^ 1][child].piv[j] = (unsigned long long)key[i];
          }
        }
      }
    }
    __syncwarp();
    // advance the running bases by this chunk's class counts
    if (lane < 7) base += (long long)((tot[lane >> 1] >> (16 * (lane & 1))) & 0xffffu);
    okm = okn;
#pragma unroll
    for (int i = 0; i < kItems; ++i) key[i] = keyn[i];
    if (kIdx) {
#pragma unroll
      for (int i = 0; i < kItems; ++i) id[i] = idn[i];
    }
  }
}

// ---------------------------------------------------------------------------
// leaf bucketing (end of the partition kernel)
// ---------------------------------------------------------------------------

// Bucket the leaves by size class (largest class first) and publish the leaf
// work items in the control block.  Uses 2 grid barriers; returns false on
// error.
template <typename U, bool kIdx>
__device__ __noinline__ bool leaf_bucket(const SortArgs& a, typename Persist<U, kIdx>::Smem& sm) {
  constexpr int kItems = Geom<U>::kLItems;
  Control* c = a.ctrl;
  const int tid = threadIdx.x;
  const int nLeaves = ld_acquire_int(&c->leafCount);
  const int nFills = ld_acquire_int(&c->fillCount);
  const int nl = nLeaves < a.leafCap ? nLeaves : a.leafCap;
  const int nf = nFills < a.fillCap ? nFills : a.fillCap;
  // bucket 1: class counts
  if (tid < 16) sm.classItems[tid] = 0;
  __syncthreads();
  for (int i = blockIdx.x * kThreads + tid; i < nl; i += gridDim.x * kThreads)
    atomicAdd(&sm.classItems[leaf_class<kItems>(a.leaves[i].n)], 1);
  __syncthreads();
  if (tid < kLeafClasses && sm.classItems[tid]) atomicAdd(&c->classCount[tid], sm.classItems[tid]);
  if (!grid_barrier(c)) return false;
  timeline_mark(c, nl);
  // bucket 2: scatter into per-class ranges (largest class first)
  if (tid == 0) {
    int acc = 0;
    for (int k = kLeafClasses - 1; k >= 0; --k) {
      sm.classOff[k] = acc;
      acc += ld_acquire_int(&c->classCount[k]);
    }
  }
  __syncthreads();
  for (int i = blockIdx.x * kThreads + tid; i < nl; i += gridDim.x * kThreads) {
    const LeafDesc d = a.leaves[i];
    const int k = leaf_class<kItems>(d.n);
    const int pos = sm.classOff[k] + atomicAdd(&c->classFill[k], 1);
    a.leavesSorted[pos] = d;
  }
  if (blockIdx.x == 0 && tid == 0) {
    int acc = 0;
    for (int k = kLeafClasses - 1; k >= 0; --k) {
      const int groups = kLThreads >> k;
      const int cnt = ld_acquire_int(&c->classCount[k]);
      c->classItemsG[k] = acc;  // first item of class k
      c->classOffG[k] = sm.classOff[k];
      acc += (cnt + groups - 1) / groups;
    }
    c->leafItems = acc;
    c->fillItems = nf;
  }
  if (!grid_barrier(c)) return false;
  timeline_mark(c, nf);
  return true;
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------

// Tiles of a level, claimed one at a time by each warp (lane 0 claims the
// next tile before the warp works on the current one).
template <typename U, bool kIdx, int kPhase>
__device__ __forceinline__ void stream_tiles(const SortArgs& a, int level, int ntiles,
                                             unsigned* wc, typename Persist<U, kIdx>::Smem& sm) {
  const int lane = threadIdx.x & 31;
  unsigned t = 0;
  if (lane == 0) t = atomicAdd(wc, 1u);
  t = __shfl_sync(0xffffffffu, t, 0);
  while ((int)t < ntiles) {
    unsigned nxt = 0;
    if (lane == 0) nxt = atomicAdd(wc, 1u);
    if (kPhase == 0) count_tile_warp<U, kIdx>(a, level, (int)t);
    else scatter_tile_warp<U, kIdx>(a, level, (int)t, sm);
    t = __shfl_sync(0xffffffffu, nxt, 0);
  }
}

template <typename U, bool kIdx>
__global__ void __launch_bounds__(kThreads, kMinBlocks) persistent_sort_kernel(SortArgs a) {
  using P = Persist<U, kIdx>;
  constexpr int kTile = P::kTile, kLeafMax = P::kLeafMax;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename P::Smem& sm = *reinterpret_cast<typename P::Smem*>(smem_raw);
  Control* c = a.ctrl;
  const int tid = threadIdx.x;
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
      c->leafWork = 0;
      c->leafDone = 0;
      c->yield = 0;
      for (int k = 0; k < 16; ++k) { c->classCount[k] = 0; c->classFill[k] = 0; }
    }
  } else if (a.offsets == nullptr) {
    // init: route the input array (level-0 list is parity 0)
    if (blockIdx.x == 0) {
      if (tid == 0) {
        int si, tb, nt;
        route_input<U, kTile, kLeafMax>(a, 0, a.n, false, &si, &tb, &nt);
        sm.childSeg[0] = si;
        sm.childTb[0] = tb;
        sm.childNt[0] = nt;
      }
      __syncthreads();
      if (sm.childSeg[0] >= 0)
        write_tiles<kTile>(a, 0, sm.childSeg[0], sm.childTb[0], sm.childNt[0], 0, a.n, tid,
                           kThreads);
    }
  } else {
    for (long long i = (long long)blockIdx.x * kThreads + tid; i < a.numArrays;
         i += (long long)gridDim.x * kThreads) {
      const long long s = a.offsets[i], e = a.offsets[i + 1];
      int si, tb, nt;
      route_input<U, kTile, kLeafMax>(a, s, e - s, true, &si, &tb, &nt);
    }
  }
  if (!grid_barrier(c)) return;
  timeline_mark(c, 0);

  // one level adds at most 4 leaves and 3 fills (+ chunks) per segment; stop
  // and hand the lists to leaf_kernel before a level could overflow them
  const int leafRoom = 4 * (a.segCap + 1);
  const int fillRoom = 3 * (a.segCap + 1) + a.tileCap;
  for (;; ++level) {
    const int par = level & 1;
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> st(c->segTile[par]);
    const unsigned long long v = st.load(cuda::memory_order_acquire);
    const int nsegs = (int)(v >> 32);
    const int ntiles = (int)(v & 0xffffffffull);
    if (nsegs == 0) break;
    if (level >= kMaxLevels) { if (tid == 0) set_error(c, kDevCapacity); return; }
    if (ld_acquire_int(&c->leafCount) > a.leafCap - leafRoom ||
        ld_acquire_int(&c->fillCount) > a.fillCap - fillRoom) {
      if (blockIdx.x == 0 && tid == 0) {
        c->yield = 1;
        c->resumeLevel = level;
        c->resumePhase = phase;
      }
      break;
    }

    // COUNT: per-tile class counts
    if (blockIdx.x == 0 && tid == 0) c->work[(phase + 2) & 3] = 0;
    stream_tiles<U, kIdx, 0>(a, level, ntiles, &c->work[phase & 3], sm);
    ++phase;
    __threadfence();
    if (!grid_barrier(c)) return;
    timeline_mark(c, ntiles);

    // PLAN: one segment per CTA
    {
      unsigned* wc = &c->work[phase & 3];
      if (blockIdx.x == 0 && tid == 0) c->work[(phase + 2) & 3] = 0;
      for (;;) {
        const int sgi = claim_item(wc);
        if (sgi >= nsegs) break;
        plan_segment<U, kIdx>(a, level, sgi, sm);
      }
      ++phase;
    }
    __threadfence();
    if (!grid_barrier(c)) return;
    timeline_mark(c, nsegs);

    // SCATTER
    if (blockIdx.x == 0 && tid == 0) {
      // this level's list was read by everyone before the last barrier;
      // level+2 appends to it during the next PLAN phase
      st.store(0ull, cuda::memory_order_relaxed);
      c->work[(phase + 2) & 3] = 0;
    }
    stream_tiles<U, kIdx, 1>(a, level, ntiles, &c->work[phase & 3], sm);
    ++phase;
    __threadfence();
    if (!grid_barrier(c)) return;
    timeline_mark(c, nsegs);
  }
  if (blockIdx.x == 0 && tid == 0) c->levels = level;
  // publish the leaves for leaf_kernel (launched right after on the stream)
  leaf_bucket<U, kIdx>(a, sm);
}

// ---------------------------------------------------------------------------
// LEAF kernel
// ---------------------------------------------------------------------------

// Sort up to kLThreads/P leaves of size class cls (P = 1 << cls threads each)
// from leavesSorted[first, last), results to A.
template <typename U, bool kIdx>
__device__ void sort_leaf_group(const SortArgs& a, int cls, int first, int last,
                                typename Persist<U, kIdx>::LeafSmem& sm) {
  using P_ = Persist<U, kIdx>;
  using KT = typename P_::KT;
  constexpr int kItems = Geom<U>::kLItems;
  const int P = 1 << cls;
  const int tid = threadIdx.x;
  const int g = tid / P, q = tid & (P - 1);
  const int li = first + g;
  const int region = g * P * kItems;
  const KT flip = (KT)a.flip;
  LeafDesc d;
  d.start = 0; d.n = 0; d.inB = 0;
  if (li < last) d = a.leavesSorted[li];
  const U* src = (const U*)(d.inB ? a.keysB : a.keysA);
  const int* srcI = d.inB ? a.idxB : a.idxA;
  for (int j = q; j < P * kItems; j += P) {
    const bool ok = j < d.n;
    sm.keys[kpad<KT>(region + j)] = ok ? kload<U, KT>(src, d.start + j, flip) : key_max<KT>();
    if (kIdx) sm.idx[ipad(region + j)] = ok ? srcI[d.start + j] : 0;
  }
  __syncthreads();
  if (!kRadixLeaves || cls <= kMergeClassMax)
    block_sort_groups<KT, kItems, kIdx>(sm.keys, sm.idx, P);
  else
    group_radix_sort<KT, kItems, kIdx, kLWarps>(sm.keys, sm.idx, d.n, P >> 5, sm.rcnt, sm.rred,
                                                &sm.rpass);
  U* dst = (U*)a.keysA;
  int* dstI = a.idxA;
  for (int j = q; j < d.n; j += P) {
    kstore<U, KT>(dst, d.start + j, sm.keys[kpad<KT>(region + j)], flip);
    if (kIdx) dstI[d.start + j] = sm.idx[ipad(region + j)];
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
template <typename U, bool kIdx>
__global__ void __launch_bounds__(kLThreads, 2) leaf_kernel(SortArgs a) {
  using P = Persist<U, kIdx>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename P::LeafSmem& sm = *reinterpret_cast<typename P::LeafSmem*>(smem_raw);
  Control* c = a.ctrl;
  const int tid = threadIdx.x;
  if (ld_acquire_int(&c->error) != 0) return;
  unsigned* wc = &c->leafWork;
  if (tid < 16) {
    sm.classItems[tid] = ld_acquire_int(&c->classItemsG[tid]);
    sm.classOff[tid] = ld_acquire_int(&c->classOffG[tid]);
  }
  if (tid == 0) sm.item = (int)atomicAdd(wc, 1u);
  __syncthreads();
  const int leafItems = ld_acquire_int(&c->leafItems);
  const int nf = ld_acquire_int(&c->fillItems);
  int it = sm.item;
  while (it < leafItems + nf) {
    unsigned nxt = 0;
    if (tid == 0) nxt = atomicAdd(wc, 1u);  // claim ahead
    if (it < leafItems) {
      // class k covers items [classItems[k], classItems[k-1])
      int k = kLeafClasses - 1;
      while (k > 0 && it >= sm.classItems[k - 1]) --k;
      const int groups = kLThreads >> k;
      const int first = sm.classOff[k] + (it - sm.classItems[k]) * groups;
      const int last = sm.classOff[k] + ld_acquire_int(&c->classCount[k]);
      const int end = first + groups < last ? first + groups : last;
      sort_leaf_group<U, kIdx>(a, k, first, end, sm);
    } else {
      fill_run<U, kIdx>(a, a.fills[it - leafItems]);
    }
    __syncthreads();
    if (tid == 0) sm.item = (int)nxt;
    __syncthreads();
    it = sm.item;
  }
  __syncthreads();
  if (tid == 0 && atomicAdd(&c->leafDone, 1) == (int)gridDim.x - 1) c->tEnd = global_ns();
}

// ---------------------------------------------------------------------------
// fixed-size batched sort (MultiSort): each CTA sorts kLThreads/P arrays of
// arrSize <= kLeafMax keys that lie back to back in memory.  Replaces the
// per-thread heap sort of turtle-multi-sort.cuh:87-182.
// ---------------------------------------------------------------------------
template <typename U, bool kIdx>
__global__ void __launch_bounds__(kLThreads, 2)
    multisort_kernel(U* keys, int* idx, long long numArrays, int arrSize, int cls,
                     unsigned long long flip64) {
  using P_ = Persist<U, kIdx>;
  using KT = typename P_::KT;
  constexpr int kItems = Geom<U>::kLItems;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename P_::LeafSmem& sm = *reinterpret_cast<typename P_::LeafSmem*>(smem_raw);
  const KT flip = (KT)flip64;
  const int P = 1 << cls;
  const int groups = kLThreads / P;
  const int tid = threadIdx.x;
  const long long first = (long long)blockIdx.x * groups;
  const long long na = (numArrays - first) < groups ? (numArrays - first) : groups;
  const long long base = first * arrSize;
  const int total = (int)(na * arrSize);
  // pad every group's tail
  {
    const int g = tid / P, q = tid & (P - 1);
    for (int j = arrSize + q; j < P * kItems; j += P) {
      sm.keys[kpad<KT>(g * P * kItems + j)] = key_max<KT>();
      if (kIdx) sm.idx[ipad(g * P * kItems + j)] = 0;
    }
  }
  // coalesced load of the whole range
  for (int j = tid; j < total; j += kLThreads) {
    const int g = j / arrSize, e = j - g * arrSize;
    const int slot = g * P * kItems + e;
    sm.keys[kpad<KT>(slot)] = kload<U, KT>(keys, base + j, flip);
    if (kIdx) sm.idx[ipad(slot)] = idx[base + j];
  }
  __syncthreads();
  if (!kRadixLeaves || cls <= kMergeClassMax) {
    block_sort_groups<KT, kItems, kIdx>(sm.keys, sm.idx, P);
  } else {
    const int g = tid / P;
    group_radix_sort<KT, kItems, kIdx, kLWarps>(sm.keys, sm.idx, g < na ? arrSize : 0, P >> 5,
                                                sm.rcnt, sm.rred, &sm.rpass);
  }
  for (int j = tid; j < total; j += kLThreads) {
    const int g = j / arrSize, e = j - g * arrSize;
    const int slot = g * P * kItems + e;
    kstore<U, KT>(keys, base + j, sm.keys[kpad<KT>(slot)], flip);
    if (kIdx) idx[base + j] = sm.idx[ipad(slot)];
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
template <typename U, bool kIdx>
static cudaError_t prepare_persistent(int device, int* gridOut) {
  const size_t smem = persist_smem_bytes<U, kIdx>();
  const size_t lsmem = leaf_smem_bytes<U, kIdx>();
  cudaError_t e = cudaFuncSetAttribute(persistent_sort_kernel<U, kIdx>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(multisort_kernel<U, kIdx>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)lsmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(leaf_kernel<U, kIdx>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)lsmem);
  if (e != cudaSuccess) return e;
  int perSM = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, persistent_sort_kernel<U, kIdx>,
                                                    kThreads, smem);
  if (e != cudaSuccess) return e;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  if (perSM < 1) return cudaErrorInvalidConfiguration;
  *gridOut = perSM * sms;
  return cudaSuccess;
}

template <typename U, bool kIdx>
static cudaError_t launch_persistent(const SortArgs& a, int grid, cudaStream_t stream) {
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
  cudaError_t e = cudaLaunchKernelEx(&cfg, persistent_sort_kernel<U, kIdx>, a);
  if (e != cudaSuccess) return e;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  leaf_kernel<U, kIdx><<<(unsigned)(sms > 0 ? 2 * sms : 2), kLThreads, leaf_smem_bytes<U, kIdx>(),
                         stream>>>(a);
  return cudaGetLastError();
}

template <typename U, bool kIdx>
static cudaError_t launch_multisort(void* keys, int* idx, long long numArrays, int arrSize,
                                    unsigned long long flip, cudaStream_t stream) {
  constexpr int kItems = Geom<U>::kLItems;
  int cls = 0;
  while ((1 << cls) * kItems < arrSize) ++cls;
  const int groups = kLThreads >> cls;
  const long long blocks = (numArrays + groups - 1) / groups;
  if (blocks <= 0) return cudaSuccess;
  multisort_kernel<U, kIdx><<<(unsigned)blocks, kLThreads, leaf_smem_bytes<U, kIdx>(), stream>>>(
      (U*)keys, idx, numArrays, arrSize, cls, flip);
  return cudaGetLastError();
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
                                      cudaStream_t stream) {
  TURTLE_WIDTH_DISPATCH(width, hasIdx, (launch_persistent<U, I>(a, grid, stream)));
}

cudaError_t kernels_launch_multisort(int width, bool hasIdx, void* keys, int* idx,
                                     long long numArrays, int arrSize, unsigned long long flip,
                                     cudaStream_t stream) {
  TURTLE_WIDTH_DISPATCH(width, hasIdx,
                        (launch_multisort<U, I>(keys, idx, numArrays, arrSize, flip, stream)));
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

int kernels_leaf_max(int width) {
  switch (width) {
    case 1: return Geom<uint8_t>::kLeafMax;
    case 2: return Geom<uint16_t>::kLeafMax;
    case 4: return Geom<uint32_t>::kLeafMax;
    case 8: return Geom<uint64_t>::kLeafMax;
    default: return 0;
  }
}

}  // namespace turtle
