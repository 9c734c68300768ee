// GB300 TurtleSort kernels: the persistent work-list quicksort and the
// fixed-size batched (MultiSort) kernel.
//
// Persistent kernel (replaces the CDP2 chain copyTasksBack -> resetNumTasks ->
// quickSortWithoutStreamCompaction / bruteSort, turtle-sort.cu:35-188,573-934):
// one cooperative launch of (SMs x resident CTAs) blocks walks the partition
// tree level by level.  Every level has two phases separated by a bounded grid
// barrier:
//   COUNT  each tile (kTile elements of one segment, aligned to absolute
//          kTile boundaries) counts its keys in the 7 pivot classes.  The CTA
//          that finishes the last tile of a segment plans it: per-class totals,
//          per-tile destination offsets, and the children (next-level
//          segments, shared-memory leaves, parked pivot runs).
//   SCATTER each tile re-reads its keys (+ids), ranks them stably per class
//          with warp ballots, stages them by class in shared memory and writes
//          each class run coalesced to its destination in the other buffer.
//          Pivot runs are written by value (keys) and never recursed into.
// Children live in the other buffer (ping-pong A <-> B), so there is no
// copy-back pass.  Leaves (segments of at most kTile elements) and pivot runs
// parked in B are finished by the LEAF phase: leaves are bucketed by size and
// sorted by groups of 1..512 threads with the stable shared-memory sort; parked
// pivot runs get their keys filled in A and their ids copied from B.  Leaves
// are also flushed between levels whenever the lists run near capacity, which
// bounds the work-list memory independently of the tree depth.
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

template <typename U, bool kIdx>
struct Persist {
  using G = Geom<U>;
  using KT = typename G::KT;
  static constexpr int kItems = G::kItems;
  static constexpr int kTile = G::kTile;
  static constexpr int kWCH = G::kWarpChunk;
  static constexpr int kIdxSlots = kIdx ? G::kIdxSlots : 4;

  struct Smem {
    KT keys[G::kKeySlots];
    int idx[kIdxSlots];
    int warpRun[kWarps][8];
    int warpOff[kWarps][8];
    int classStart[8];
    int cnt[8];
    long long toff[8];
    long long red[kWarps][8];
    long long carry[8];
    long long tot[8];
    KT piv[3];
    long long lo, hi, segStart, segN;
    int segIdx, tileInSeg, ntiles, isLast;
    int classOff[16];
    int classItems[16];
  };
};

template <typename U, bool kIdx>
constexpr size_t persist_smem_bytes() {
  return sizeof(typename Persist<U, kIdx>::Smem);
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

template <typename KT, typename U>
__device__ void pick_pivots(const U* src, long long start, long long n, int level, KT flip,
                            KT* piv) {
  if (level < kDepthSwitch) {
    KT s0 = kload<U, KT>(src, start + n / 2, flip);
    KT s1 = kload<U, KT>(src, start, flip);
    KT s2 = kload<U, KT>(src, start + n - 1, flip);
    KT t;
    if (s1 < s0) { t = s0; s0 = s1; s1 = t; }
    if (s2 < s0) { t = s0; s0 = s2; s2 = t; }
    if (s2 < s1) { t = s1; s1 = s2; s2 = t; }
    piv[0] = s0; piv[1] = s1; piv[2] = s2;
  } else {
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
}

__device__ __forceinline__ int find_seg(const SegDesc* segs, int nsegs, int t) {
  int lo = 0, hi = nsegs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].tileBase <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <int kTile>
__device__ __forceinline__ long long tiles_of(long long start, long long n) {
  return (start + n - 1) / kTile - start / kTile + 1;
}

// Append a segment to the next level's list (tile range allocated with the
// same 64-bit atomic, so tileBase grows with the segment index).
template <int kTile>
__device__ void push_segment(const SortArgs& a, int par, long long start, long long n) {
  const long long nt = tiles_of<kTile>(start, n);
  const unsigned long long old =
      atomicAdd(&a.ctrl->segTile[par], (1ull << 32) | (unsigned long long)nt);
  const int si = (int)(old >> 32);
  const long long tb = (long long)(old & 0xffffffffull);
  if (si >= a.segCap || tb + nt > a.tileCap) {
    set_error(a.ctrl, kDevCapacity);
    return;
  }
  SegDesc d;
  d.start = start; d.n = n; d.tileBase = (int)tb; d.ntiles = (int)nt; d.done = 0; d.pad = 0;
  a.segs[par][si] = d;
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

// Route one array / child: nothing, leaf, or next-level segment.
template <int kTile>
__device__ void route_child(const SortArgs& a, int nextPar, long long start, long long n,
                            bool inB) {
  if (n <= 0) return;
  if (n == 1 && !inB) return;  // already final in A
  if (n <= kTile) push_leaf(a, start, n, inB ? 1 : 0);
  else push_segment<kTile>(a, nextPar, start, n);
}

// ---------------------------------------------------------------------------
// COUNT phase: one tile
// ---------------------------------------------------------------------------
template <typename U, bool kIdx>
__device__ void plan_segment(const SortArgs& a, int level, typename Persist<U, kIdx>::Smem& sm);

template <typename U, bool kIdx>
__device__ void count_tile(const SortArgs& a, int level, int t, int nsegs,
                           typename Persist<U, kIdx>::Smem& sm) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kItems = P::kItems, kTile = P::kTile, kWCH = P::kWCH;
  const int par = level & 1;
  const U* src = (const U*)(par ? a.keysB : a.keysA);
  const KT flip = (KT)a.flip;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    const int si = find_seg(a.segs[par], nsegs, t);
    const SegDesc sd = a.segs[par][si];
    sm.segIdx = si;
    sm.tileInSeg = t - sd.tileBase;
    sm.ntiles = sd.ntiles;
    sm.segStart = sd.start;
    sm.segN = sd.n;
    const long long abs0 = (sd.start / kTile + sm.tileInSeg) * (long long)kTile;
    sm.lo = abs0 > sd.start ? abs0 : sd.start;
    const long long e = sd.start + sd.n;
    sm.hi = (abs0 + kTile) < e ? (abs0 + kTile) : e;
    pick_pivots<KT, U>(src, sd.start, sd.n, level, flip, sm.piv);
  }
  if (tid < 8) sm.cnt[tid] = 0;
  __syncthreads();
  const long long lo = sm.lo, hi = sm.hi;
  const long long abs0 = (lo / kTile) * (long long)kTile;
  const KT p1 = sm.piv[0], p2 = sm.piv[1], p3 = sm.piv[2];
  KT key[kItems];
  bool ok[kItems];
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const long long s = abs0 + warp * kWCH + r * 32 + lane;
    ok[r] = (s >= lo) && (s < hi);
    key[r] = ok[r] ? kload<U, KT>(src, s, flip) : KT(0);
  }
  unsigned long long accLo = 0, accHi = 0;  // 16-bit fields: classes 0-3 / 4-6
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    if (ok[r]) {
      const int c = classify<KT>(key[r], p1, p2, p3);
      if (c < 4) accLo += 1ull << (16 * c);
      else accHi += 1ull << (16 * (c - 4));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    accLo += __shfl_xor_sync(0xffffffffu, accLo, o);
    accHi += __shfl_xor_sync(0xffffffffu, accHi, o);
  }
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int x = (int)((accLo >> (16 * c)) & 0xffff);
      if (x) atomicAdd(&sm.cnt[c], x);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int x = (int)((accHi >> (16 * c)) & 0xffff);
      if (x) atomicAdd(&sm.cnt[4 + c], x);
    }
  }
  __syncthreads();
  if (tid < 8) {
    a.tileCnt[par][(long long)t * 8 + tid] = sm.cnt[tid];
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) {
    SegDesc* sd = &a.segs[par][sm.segIdx];
    cuda::atomic_ref<int, cuda::thread_scope_device> done(sd->done);
    const int old = done.fetch_add(1, cuda::memory_order_acq_rel);
    sm.isLast = (old == sm.ntiles - 1);
  }
  __syncthreads();
  if (sm.isLast) {
    __threadfence();
    plan_segment<U, kIdx>(a, level, sm);
  }
}

// The CTA that counted the last tile of segment sm.segIdx turns the per-tile
// counts into destination offsets (class bases as in turtle-sort.cu:755-761,
// then tiles in memory order, which makes the partition stable) and routes the
// children (turtle-sort.cu:857-933).
template <typename U, bool kIdx>
__device__ void plan_segment(const SortArgs& a, int level, typename Persist<U, kIdx>::Smem& sm) {
  using P = Persist<U, kIdx>;
  constexpr int kTile = P::kTile;
  const int par = level & 1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const SegDesc sd = a.segs[par][sm.segIdx];
  const int* cnt = a.tileCnt[par] + (long long)sd.tileBase * 8;
  long long* off = a.tileOff[par] + (long long)sd.tileBase * 8;
  const int nt = sd.ntiles;

  // 1. class totals
  long long s[7];
#pragma unroll
  for (int c = 0; c < 7; ++c) s[c] = 0;
  for (int t = tid; t < nt; t += kThreads) {
#pragma unroll
    for (int c = 0; c < 7; ++c) s[c] += __ldcg(&cnt[(long long)t * 8 + c]);
  }
#pragma unroll
  for (int c = 0; c < 7; ++c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 7; ++c) sm.red[warp][c] = s[c];
  }
  __syncthreads();
  if (tid < 7) {
    long long x = 0;
    for (int w = 0; w < kWarps; ++w) x += sm.red[w][tid];
    sm.tot[tid] = x;
  }
  __syncthreads();
  if (tid == 0) {
    long long b = sd.start;
    for (int c = 0; c < 7; ++c) { sm.carry[c] = b; b += sm.tot[c]; }
  }
  __syncthreads();

  // 2. exclusive scan over tiles, per class, in chunks of kThreads tiles
  for (int c0 = 0; c0 < nt; c0 += kThreads) {
    const int t = c0 + tid;
    int v[7];
#pragma unroll
    for (int c = 0; c < 7; ++c) v[c] = (t < nt) ? __ldcg(&cnt[(long long)t * 8 + c]) : 0;
    int inc[7];
#pragma unroll
    for (int c = 0; c < 7; ++c) {
      int x = v[c];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      inc[c] = x;
    }
    if (lane == 31) {
#pragma unroll
      for (int c = 0; c < 7; ++c) sm.red[warp][c] = inc[c];
    }
    __syncthreads();
    if (tid < 7) {  // exclusive prefix of warp totals, in place
      long long acc = 0;
      for (int w = 0; w < kWarps; ++w) {
        const long long x = sm.red[w][tid];
        sm.red[w][tid] = acc;
        acc += x;
      }
      sm.tot[tid] = acc;  // chunk total (class totals no longer needed)
    }
    __syncthreads();
    if (t < nt) {
#pragma unroll
      for (int c = 0; c < 7; ++c)
        off[(long long)t * 8 + c] = sm.carry[c] + sm.red[warp][c] + (inc[c] - v[c]);
      off[(long long)t * 8 + 7] = 0;
    }
    __syncthreads();
    if (tid < 7) sm.carry[tid] += sm.tot[tid];
    __syncthreads();
  }
  // sm.carry[c] now = end of class c = start of class c + its total
  // 3. children
  if (tid == 0) {
    const bool dstIsA = (par == 1);
    const int nextPar = par ^ 1;
    long long pos = sd.start;
    for (int c = 0; c < 7; ++c) {
      const long long m = sm.carry[c] - pos;
      if (m > 0) {
        if (c & 1) {
          if (!dstIsA) push_fill(a, pos, m, (unsigned long long)sm.piv[c >> 1]);
        } else {
          route_child<kTile>(a, nextPar, pos, m, !dstIsA);
        }
      }
      pos = sm.carry[c];
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// SCATTER phase: one tile
// ---------------------------------------------------------------------------
template <typename U, bool kIdx>
__device__ void scatter_tile(const SortArgs& a, int level, int t, int nsegs,
                             typename Persist<U, kIdx>::Smem& sm) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kItems = P::kItems, kTile = P::kTile, kWCH = P::kWCH;
  const int par = level & 1;
  const U* src = (const U*)(par ? a.keysB : a.keysA);
  const int* srcI = par ? a.idxB : a.idxA;
  U* dst = (U*)(par ? a.keysA : a.keysB);
  int* dstI = par ? a.idxA : a.idxB;
  const bool dstIsA = (par == 1);
  const KT flip = (KT)a.flip;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    const int si = find_seg(a.segs[par], nsegs, t);
    const SegDesc sd = a.segs[par][si];
    const int tis = t - sd.tileBase;
    const long long abs0 = (sd.start / kTile + tis) * (long long)kTile;
    sm.lo = abs0 > sd.start ? abs0 : sd.start;
    const long long e = sd.start + sd.n;
    sm.hi = (abs0 + kTile) < e ? (abs0 + kTile) : e;
    pick_pivots<KT, U>(src, sd.start, sd.n, level, flip, sm.piv);
  }
  if (tid < 8) sm.toff[tid] = __ldcg(&a.tileOff[par][(long long)t * 8 + tid]);
  if (tid < kWarps * 8) (&sm.warpRun[0][0])[tid] = 0;
  __syncthreads();
  const long long lo = sm.lo, hi = sm.hi;
  const long long abs0 = (lo / kTile) * (long long)kTile;
  const KT p1 = sm.piv[0], p2 = sm.piv[1], p3 = sm.piv[2];
  KT key[kItems];
  int id[kItems];
  unsigned rk[(kItems + 1) / 2];  // (class | rank << 3) per element, 16 bits each
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const long long s = abs0 + warp * kWCH + r * 32 + lane;
    const bool ok = (s >= lo) && (s < hi);
    key[r] = ok ? kload<U, KT>(src, s, flip) : KT(0);
    if (kIdx) id[r] = ok ? srcI[s] : 0;
  }
  const unsigned lt = lanemask_lt();
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const long long s = abs0 + warp * kWCH + r * 32 + lane;
    const bool ok = (s >= lo) && (s < hi);
    const int c = classify<KT>(key[r], p1, p2, p3);
    const unsigned bv = __ballot_sync(0xffffffffu, ok);
    const unsigned b0 = __ballot_sync(0xffffffffu, ok && (c & 1));
    const unsigned b1 = __ballot_sync(0xffffffffu, ok && (c & 2));
    const unsigned b2 = __ballot_sync(0xffffffffu, ok && (c & 4));
    const unsigned m = bv & ((c & 1) ? b0 : ~b0) & ((c & 2) ? b1 : ~b1) & ((c & 4) ? b2 : ~b2);
    int run = 0;
    if (ok) run = sm.warpRun[warp][c];
    const int rank = run + __popc(m & lt);
    __syncwarp();
    if (ok && (m >> lane) == 1u) sm.warpRun[warp][c] = run + __popc(m);
    __syncwarp();
    const unsigned packed = ok ? (unsigned)(c | (rank << 3)) : 0xffffu;
    if (r & 1) rk[r >> 1] |= packed << 16;
    else rk[r >> 1] = packed;
  }
  __syncthreads();
  if (tid < 7) {
    int acc = 0;
    for (int w = 0; w < kWarps; ++w) {
      const int x = sm.warpRun[w][tid];
      sm.warpOff[w][tid] = acc;
      acc += x;
    }
    sm.cnt[tid] = acc;
  }
  __syncthreads();
  if (tid == 0) {
    int acc = 0;
    for (int c = 0; c < 7; ++c) { sm.classStart[c] = acc; acc += sm.cnt[c]; }
    sm.classStart[7] = acc;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const unsigned packed = (rk[r >> 1] >> ((r & 1) * 16)) & 0xffffu;
    if (packed != 0xffffu) {
      const int c = packed & 7;
      const int pos = sm.classStart[c] + sm.warpOff[warp][c] + (int)(packed >> 3);
      if (!(c & 1)) sm.keys[kpad<KT>(pos)] = key[r];
      if (kIdx) sm.idx[ipad(pos)] = id[r];
    }
  }
  __syncthreads();
  const int cntTile = (int)(hi - lo);
  int cs[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) cs[c] = sm.classStart[c];
  for (int i = tid; i < cntTile; i += kThreads) {
    int c = 0;
#pragma unroll
    for (int q = 1; q < 7; ++q) c += (i >= cs[q]) ? 1 : 0;
    const long long d = sm.toff[c] + (i - cs[c]);
    if (c & 1) {
      if (dstIsA) kstore<U, KT>(dst, d, sm.piv[c >> 1], flip);
    } else {
      kstore<U, KT>(dst, d, sm.keys[kpad<KT>(i)], flip);
    }
    if (kIdx) dstI[d] = sm.idx[ipad(i)];
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// LEAF phase
// ---------------------------------------------------------------------------

// Sort up to kThreads/P leaves of size class c (P = 1 << c threads each).
template <typename U, bool kIdx>
__device__ void sort_leaf_group(const SortArgs& a, int cls, int first, int last,
                                typename Persist<U, kIdx>::Smem& sm) {
  using P_ = Persist<U, kIdx>;
  using KT = typename P_::KT;
  constexpr int kItems = P_::kItems;
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
  block_sort_groups<KT, kItems, kIdx>(sm.keys, sm.idx, P);
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
  for (int j = threadIdx.x; j < f.n; j += kThreads) {
    kstore<U, KT>(dst, f.start + j, v, flip);
    if (kIdx) a.idxA[f.start + j] = a.idxB[f.start + j];
  }
}

// Bucket the leaves by size class, sort them (largest class first) and fill
// the parked pivot runs.  Uses 3 barriers; returns false on error.
template <typename U, bool kIdx>
__device__ bool leaf_phase(const SortArgs& a, int& phase, typename Persist<U, kIdx>::Smem& sm) {
  using P_ = Persist<U, kIdx>;
  constexpr int kItems = P_::kItems;
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
  if (!grid_barrier(c)) return false;
  // items: per class ceil(count / groups), then fills
  if (tid == 0) {
    int acc = 0;
    for (int k = kLeafClasses - 1; k >= 0; --k) {
      const int groups = kThreads >> k;
      const int cnt = ld_acquire_int(&c->classCount[k]);
      sm.classItems[k] = acc;  // first item of class k
      acc += (cnt + groups - 1) / groups;
    }
    sm.classItems[15] = acc;  // total leaf items
  }
  __syncthreads();
  const int leafItems = sm.classItems[15];
  unsigned* wc = &c->work[phase & 3];
  if (blockIdx.x == 0 && tid == 0) c->work[(phase + 2) & 3] = 0;
  for (;;) {
    const int it = claim_item(wc);
    if (it >= leafItems + nf) break;
    if (it < leafItems) {
      int k = kLeafClasses - 1;
      while (k > 0 && it >= (k == 0 ? leafItems : sm.classItems[k - 1])) --k;
      // class k covers items [classItems[k], classItems[k-1]) (k-1 is the next smaller class)
      const int groups = kThreads >> k;
      const int first = sm.classOff[k] + (it - sm.classItems[k]) * groups;
      const int last = sm.classOff[k] + ld_acquire_int(&c->classCount[k]);
      const int end = first + groups < last ? first + groups : last;
      sort_leaf_group<U, kIdx>(a, k, first, end, sm);
    } else {
      fill_run<U, kIdx>(a, a.fills[it - leafItems]);
      __syncthreads();
    }
  }
  ++phase;
  return true;
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------
template <typename U, bool kIdx>
__global__ void __launch_bounds__(kThreads, kMinBlocks) persistent_sort_kernel(SortArgs a) {
  using P = Persist<U, kIdx>;
  constexpr int kTile = P::kTile;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename P::Smem& sm = *reinterpret_cast<typename P::Smem*>(smem_raw);
  Control* c = a.ctrl;
  const int tid = threadIdx.x;
  int phase = 0;

  // init: route every input array (level-0 list is parity 0)
  if (a.offsets == nullptr) {
    if (blockIdx.x == 0 && tid == 0) route_child<kTile>(a, 0, 0, a.n, false);
  } else {
    for (long long i = (long long)blockIdx.x * kThreads + tid; i < a.numArrays;
         i += (long long)gridDim.x * kThreads) {
      const long long s = a.offsets[i], e = a.offsets[i + 1];
      route_child<kTile>(a, 0, s, e - s, false);
    }
  }
  if (!grid_barrier(c)) return;

  // flush threshold: one level can add at most 4 leaves / 3 fills (+chunks)
  // per segment; flush before a level could overflow the lists.
  const int leafRoom = 4 * (a.segCap + 1);
  int level = 0;
  for (;; ++level) {
    const int par = level & 1;
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> st(c->segTile[par]);
    const unsigned long long v = st.load(cuda::memory_order_acquire);
    const int nsegs = (int)(v >> 32);
    const int ntiles = (int)(v & 0xffffffffull);
    if (nsegs == 0) break;
    if (level >= kMaxLevels) { if (tid == 0) set_error(c, kDevCapacity); return; }

    // flush leaves/fills early if the next level could overflow the lists
    if (ld_acquire_int(&c->leafCount) > a.leafCap - leafRoom ||
        ld_acquire_int(&c->fillCount) > a.fillCap - (3 * (a.segCap + 1) + a.tileCap)) {
      if (!leaf_phase<U, kIdx>(a, phase, sm)) return;
      if (!grid_barrier(c)) return;
      if (blockIdx.x == 0 && tid == 0) {
        c->leafCount = 0;
        c->fillCount = 0;
        for (int k = 0; k < 16; ++k) { c->classCount[k] = 0; c->classFill[k] = 0; }
      }
      if (!grid_barrier(c)) return;
    }

    // COUNT (+ plan by the last tile of each segment)
    {
      unsigned* wc = &c->work[phase & 3];
      if (blockIdx.x == 0 && tid == 0) c->work[(phase + 2) & 3] = 0;
      for (;;) {
        const int t = claim_item(wc);
        if (t >= ntiles) break;
        count_tile<U, kIdx>(a, level, t, nsegs, sm);
      }
      ++phase;
    }
    if (!grid_barrier(c)) return;

    // SCATTER
    {
      unsigned* wc = &c->work[phase & 3];
      if (blockIdx.x == 0 && tid == 0) {
        c->work[(phase + 2) & 3] = 0;
        // this level's list was read by everyone before the last barrier;
        // level+2 appends to it during the next COUNT phase
        st.store(0ull, cuda::memory_order_relaxed);
      }
      for (;;) {
        const int t = claim_item(wc);
        if (t >= ntiles) break;
        scatter_tile<U, kIdx>(a, level, t, nsegs, sm);
      }
      ++phase;
    }
    if (!grid_barrier(c)) return;
  }
  if (blockIdx.x == 0 && tid == 0) c->levels = level;
  leaf_phase<U, kIdx>(a, phase, sm);
}

// ---------------------------------------------------------------------------
// fixed-size batched sort (MultiSort): each CTA sorts kThreads/P arrays of
// arrSize <= kTile keys that lie back to back in memory.  Replaces the
// per-thread heap sort of turtle-multi-sort.cuh:87-182.
// ---------------------------------------------------------------------------
template <typename U, bool kIdx>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    multisort_kernel(U* keys, int* idx, long long numArrays, int arrSize, int cls,
                     unsigned long long flip64) {
  using P_ = Persist<U, kIdx>;
  using KT = typename P_::KT;
  constexpr int kItems = P_::kItems;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename P_::Smem& sm = *reinterpret_cast<typename P_::Smem*>(smem_raw);
  const KT flip = (KT)flip64;
  const int P = 1 << cls;
  const int groups = kThreads / P;
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
  for (int j = tid; j < total; j += kThreads) {
    const int g = j / arrSize, e = j - g * arrSize;
    const int slot = g * P * kItems + e;
    sm.keys[kpad<KT>(slot)] = kload<U, KT>(keys, base + j, flip);
    if (kIdx) sm.idx[ipad(slot)] = idx[base + j];
  }
  __syncthreads();
  block_sort_groups<KT, kItems, kIdx>(sm.keys, sm.idx, P);
  for (int j = tid; j < total; j += kThreads) {
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
  cudaError_t e = cudaFuncSetAttribute(persistent_sort_kernel<U, kIdx>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(multisort_kernel<U, kIdx>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
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
  return cudaLaunchKernelEx(&cfg, persistent_sort_kernel<U, kIdx>, a);
}

template <typename U, bool kIdx>
static cudaError_t launch_multisort(void* keys, int* idx, long long numArrays, int arrSize,
                                    unsigned long long flip, cudaStream_t stream) {
  constexpr int kItems = Geom<U>::kItems;
  int cls = 0;
  while ((1 << cls) * kItems < arrSize) ++cls;
  const int groups = kThreads >> cls;
  const long long blocks = (numArrays + groups - 1) / groups;
  if (blocks <= 0) return cudaSuccess;
  multisort_kernel<U, kIdx><<<(unsigned)blocks, kThreads, persist_smem_bytes<U, kIdx>(), stream>>>(
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

}  // namespace turtle
