// LSD radix form of the plain sort (TURTLE_FORM_RADIX).
//
// The reference sorts by 3-pivot partitioning (turtle-sort.cu:573-934) and
// its output is the stable order of the keys (ids of equal keys in input
// order), which every stable sort produces.  This form reaches the same bytes
// in passes over 8-bit digits, least significant first; each pass is a stable
// counting scatter, so the composition is the stable sort:
//
//   radix_hist_kernel    one read of the keys: the 256-bin histogram of every
//                        digit at once (float keys are mapped to their
//                        totalOrder images here, in place);
//   radix_plan_kernel    one CTA: the first output position of each digit
//                        value (exclusive prefix of each histogram); a digit
//                        whose keys all share one value is skipped, its
//                        scatter would be the identity;
//   radix_pass_kernel    one launch per digit, one CTA per tile of
//                        kRadixThreads x radix_items keys (4096, 2048 for
//                        64-bit keys; 6144 for large sorts of 8- to 32-bit
//                        keys without ids), tiles claimed in
//                        order with an atomic counter.  The CTA counts its
//                        keys' digit values and publishes the counts, ranks
//                        its keys by digit (per-warp running counts; the lanes
//                        of one digit value found with shared-memory atomicOr,
//                        which measured 2.5x faster than a match instruction
//                        on ~30 distinct values per warp), adds the counts of
//                        the tiles before it by a decoupled look-back over
//                        their published words, stages the tile in shared
//                        memory in digit order and writes it out, consecutive
//                        keys of a digit to consecutive addresses;
//   radix_finish_kernel  the result back into the caller's buffer when an odd
//                        number of passes left it in the scratch buffer (and
//                        float keys back from their images when no pass ran);
//   radix_gather_kernel  late ids (StartSorting): the passes carried element
//                        positions; this writes the ids in sorted order.
//
// Every pass reads keys + ids once and writes them once; the histogram pass
// reads the keys once more.  A look-back wait is bounded: past the poll limit
// the CTA records kDevTimeout, publishes its word (so later tiles go on) and
// writes nothing.
#include <cuda_runtime.h>

#include <cuda/atomic>
#include <type_traits>

#include "turtle_device.cuh"
#include "turtle_internal.h"

namespace turtle {
namespace {

constexpr unsigned kRFull = 0xffffffffu;
constexpr unsigned kLbInclusive = 0x80000000u;  // word holds the inclusive prefix, else the tile's count
constexpr int kRWarps = kRadixThreads / 32;
constexpr int kBinWarps = kRadixBins / 32;  // warps whose threads each own one digit value
constexpr int kLbWindow = 4;  // look-back words loaded per round trip
static_assert(kRadixThreads >= kRadixBins && kRadixThreads % kRadixBins == 0,
              "threads 0..255 of a pass CTA each own one digit value");

// Look-back words: 0 = not published; else flag | (value + 1).
__device__ __forceinline__ unsigned lb_load(const unsigned* p) {
  cuda::atomic_ref<const unsigned, cuda::thread_scope_device> a(*p);
  return a.load(cuda::memory_order_relaxed);
}
__device__ __forceinline__ void lb_store(unsigned* p, unsigned v) {
  cuda::atomic_ref<unsigned, cuda::thread_scope_device> a(*p);
  a.store(v, cuda::memory_order_relaxed);
}

// totalOrder image of an IEEE-754 bit pattern (forward), or back (inverse).
template <typename U>
__device__ __forceinline__ U float_image(U b, bool inverse) {
  constexpr U kSign = U(1) << (8 * sizeof(U) - 1);
  const bool top = (b & kSign) != 0;
  const U mask = (top != inverse) ? U(~U(0)) : kSign;
  return b ^ mask;
}

// Keys [lo, hi) (the keys may arrive in chunks, one launch each); `clear`:
// this launch also clears look-back region 0.
template <typename U>
__global__ void __launch_bounds__(kRadixThreads) radix_hist_kernel(SortArgs a, long long lo,
                                                                    long long hi, int clear) {
  using KT = typename KeyCfg<U>::KT;
  constexpr int P = sizeof(U);
  __shared__ unsigned h[P * kRadixBins];
  const int tid = threadIdx.x, lane = tid & 31;
  for (int i = tid; i < P * kRadixBins; i += kRadixThreads) h[i] = 0u;
  // the first moving pass uses look-back region 0: clear its rows
  if (clear) {
    const long long rows = (a.n + radix_tile(P) - 1) / radix_tile(P);
    const long long words = rows * kRadixBins;
    for (long long i = (long long)blockIdx.x * kRadixThreads + tid; i < words;
         i += (long long)gridDim.x * kRadixThreads)
      a.radixStatus[i] = 0u;
  }
  __syncthreads();
  U* keys = (U*)a.keysA;
  const KT flip = (KT)a.flip;
  const bool fl = sizeof(U) >= 4 && a.fbits != 0;
  const long long step = (long long)gridDim.x * kRadixThreads * 4;
  // a warp takes 128 consecutive keys per round (four coalesced loads)
  for (long long base = lo + ((long long)blockIdx.x * kRadixThreads + (tid & ~31)) * 4; base < hi;
       base += step) {
    KT k[4];
    bool ok[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long e = base + 32 * q + lane;
      ok[q] = e < hi;
      U raw = ok[q] ? keys[e] : U(0);
      if (fl && ok[q]) {
        raw = float_image<U>(raw, false);
        keys[e] = raw;
      }
      k[q] = KT(raw) ^ flip;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const unsigned d = (unsigned)(k[q] >> (8 * p)) & 255u;
        // one shared atomic per key and digit: measured faster than first
        // testing whether the warp's 32 keys share the value (1.675 vs
        // 1.740 ms per 2^26 int32 + id sort; sorted input 1.646 vs 1.751 ms)
        if (ok[q]) atomicAdd(&h[p * kRadixBins + d], 1u);
      }
    }
  }
  __syncthreads();
  for (int i = tid; i < P * kRadixBins; i += kRadixThreads)
    if (h[i] != 0u) atomicAdd(&a.radixHist[i], h[i]);
}

template <typename U>
__global__ void __launch_bounds__(kRadixBins) radix_plan_kernel(SortArgs a) {
  constexpr int P = sizeof(U);
  const int b = threadIdx.x, lane = b & 31, warp = b >> 5;
  __shared__ unsigned wsum[kRadixBins / 32];
  RadixCtl* c = a.radixCtl;
  int ord = 0, last = -1;
  for (int p = 0; p < P; ++p) {
    const unsigned cnt = a.radixHist[p * kRadixBins + b];
    const int skip = __syncthreads_or(cnt == (unsigned)a.n);
    unsigned x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(kRFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    unsigned pre = 0;
    for (int w = 0; w < warp; ++w) pre += wsum[w];
    a.radixBase[p * kRadixBins + b] = pre + x - cnt;
    __syncthreads();
    if (b == 0) {
      c->ord[p] = skip ? -1 : ord;
      c->tileCtr[p] = 0u;
    }
    if (!skip) {
      last = p;
      ++ord;
    }
  }
  if (b == 0) {
    for (int p = P; p < 8; ++p) c->ord[p] = -1;
    c->active = ord;
    c->last = last;
    a.ctrl->levels = ord;
  }
}

// Digit p (byte p) of an unsigned key image: one byte-permute for 32-bit
// words.
template <typename KT>
__device__ __forceinline__ unsigned digit_of(KT k, int p) {
  if constexpr (sizeof(KT) == 8) {
    const unsigned half = p >= 4 ? (unsigned)((unsigned long long)k >> 32) : (unsigned)k;
    return __byte_perm(half, 0u, 0x4440u | (unsigned)(p & 3));
  } else {
    return __byte_perm((unsigned)k, 0u, 0x4440u | (unsigned)p);
  }
}

// The same digit through an opaque byte-permute: keeps the compiler from
// holding every item's digit in a register from the ranking to the staging.
template <typename KT>
__device__ __forceinline__ unsigned digit_again(KT k, int p) {
  unsigned half, d;
  if constexpr (sizeof(KT) == 8) half = p >= 4 ? (unsigned)((unsigned long long)k >> 32) : (unsigned)k;
  else half = (unsigned)k;
  asm volatile("prmt.b32 %0, %1, 0, %2;" : "=r"(d) : "r"(half), "r"(0x4440u | (unsigned)(p & 3)));
  return d;
}

template <typename U, bool kIdx, int kItems>
struct RadixSmem {
  static constexpr int kTile = kRadixThreads * kItems;
  unsigned short wc[kRWarps][kRadixBins];  // warp running counts, then staging starts per warp
  unsigned mm[kRWarps][kRadixBins];        // lanes of each digit value (one item)
  unsigned cnt[kRadixBins];                // the tile's count of each digit value, then its
                                           // first staging slot of each value
  int dst[kRadixBins];                     // the pass's first output position of each value,
                                           // then the output position of staging slot 0
  unsigned wsum[kBinWarps];
  int tile, fail;
  // the tile in digit order: (key, id) pairs for keys of up to 4 bytes with
  // ids (one 8-byte store and load per key: 1.73 vs 1.80 ms for 2^26 int32
  // keys + ids against separate key and id arrays), else keys and ids apart
  static constexpr bool kPair = kIdx && sizeof(U) <= 4;
  alignas(16) uint2 kv[kPair ? kTile : 1];
  alignas(16) U k[kPair ? 1 : kTile];
  int i[kIdx && !kPair ? kTile : 1];
};

// The work of one tile (`valid` keys; kFull: all kTile).  Order: load; count
// the tile's digit values (shared atomics) and publish the counts at once, so
// later tiles can add them; rank (no other tile needed); look back and publish
// the inclusive prefix; stage and write.  Measured on 2^26 int32 keys + ids:
// 1.88 ms in this order, 1.99 ms when the look-back runs before the ranking
// (with or without its first loads issued early), 2.53 ms when the counts are
// published only after the ranking.
// Late ids: the passes carry element positions instead of ids.  The first
// moving pass makes them; the pass of rank k writes them to idxB when
// active - 1 - k is even, else to idxA, so the last one leaves them in idxB
// for the gather.
__device__ __forceinline__ int* late_positions(const SortArgs& a, int active, int k) {
  return ((active - 1 - k) & 1) == 0 ? a.idxB : a.idxA;
}

template <typename U, bool kIdx, int kItems, bool kFull>
__device__ __forceinline__ void radix_pass_tile(const SortArgs& a, int p, int ord, bool lastPass,
                                                int active, RadixSmem<U, kIdx, kItems>& sm,
                                                int tile, int valid) {
  using KT = typename KeyCfg<U>::KT;
  constexpr int kTile = kRadixThreads * kItems;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int b = tid;  // threads b < 256: the digit value they publish, scan and look back for
  const bool binT = b < kRadixBins;
  const bool fromB = (ord & 1) != 0;
  const KT flip = (KT)a.flip;
  // warp-striped items: item i of this lane is tile element e0 + 32 i
  const int e0 = warp * 32 * kItems + lane;
  unsigned okm = (1u << kItems) - 1u;
  if (!kFull) {
    okm = 0u;
#pragma unroll
    for (int i = 0; i < kItems; ++i) okm |= (e0 + 32 * i < valid ? 1u : 0u) << i;
  }
  KT key[kItems];
  int id[kIdx ? kItems : 1];
  {
    const long long tbase = (long long)tile * kTile;
    const U* tk = (const U*)(fromB ? a.keysB : a.keysA) + tbase;
    // ids, or (late ids) the positions of the previous moving pass; the first
    // moving pass makes the positions
    const bool makePos = a.idsLate && ord == 0;
    const int* ti = !kIdx || makePos ? nullptr
                    : (a.idsLate ? late_positions(a, active, ord - 1) : (fromB ? a.idxB : a.idxA)) + tbase;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const bool ok = kFull || ((okm >> i) & 1u);
      key[i] = ok ? KT(__ldcs(tk + e0 + 32 * i)) ^ flip : KT(0);
      if (kIdx) id[i] = !ok ? 0 : makePos ? (int)(tbase + e0 + 32 * i) : __ldcs(ti + e0 + 32 * i);
    }
  }
  // 1. the tile's digit counts, published at once; the tile's staging start
  // of each digit value (exclusive prefix over the values)
#pragma unroll
  for (int i = 0; i < kItems; ++i)
    if (kFull || ((okm >> i) & 1u)) atomicAdd(&sm.cnt[digit_of<KT>(key[i], p)], 1u);
  __syncthreads();
  const unsigned cnt = binT ? sm.cnt[b] : 0u;
  const bool mute = a.radixStall == (long long)tile + 1;  // testing: later tiles wait in vain
  if (binT && !mute)
    lb_store(a.radixStatus + ((size_t)(ord & 1) * a.radixTiles + tile) * kRadixBins + b,
             (tile == 0 ? kLbInclusive : 0u) | (cnt + 1u));
  {
    unsigned x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(kRFull, x, o);
      if (lane >= o) x += y;
    }
    if (binT && lane == 31) sm.wsum[warp] = x;
    __syncthreads();
    if (binT) {
      unsigned pre = 0;
#pragma unroll
      for (int w = 0; w < kBinWarps; ++w) pre += w < warp ? sm.wsum[w] : 0u;
      sm.cnt[b] = pre + x - cnt;  // thread b alone reads and writes entry b
    }
  }
  // 2. rank: item by item in memory order (stable).  The lanes of one digit
  // value are found by each setting its bit in the warp's word for that value;
  // the warp's running count of the value is updated by the group's highest lane.
  const unsigned lanebit = 1u << lane, lt = lanebit - 1u;
  unsigned rk[kItems / 2];
  unsigned short* wc = sm.wc[warp];
  unsigned* mm = sm.mm[warp];
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    const bool ok = kFull || ((okm >> i) & 1u);
    const unsigned d = digit_of<KT>(key[i], p);
    if (ok) atomicOr(&mm[d], lanebit);
    __syncwarp();
    unsigned peers = 0u, base = 0u;
    if (ok) {
      peers = mm[d];
      base = wc[d];
    }
    __syncwarp();
    if (ok && (peers >> lane) == 1u) {
      wc[d] = (unsigned short)(base + __popc(peers));
      mm[d] = 0u;
    }
    __syncwarp();
    const unsigned r = base + __popc(peers & lt);
    if (i & 1) rk[i >> 1] |= r << 16;
    else rk[i >> 1] = r;
  }
  __syncthreads();
  // 3. staging start of digit value b for each warp: the tile's start of b
  // plus the counts of b in the warps before
  if (binT) {
    unsigned run = sm.cnt[b];
#pragma unroll
    for (int w = 0; w < kRWarps; ++w) {
      const unsigned x = sm.wc[w][b];
      sm.wc[w][b] = (unsigned short)run;
      run += x;
    }
  }
  // 4. decoupled look-back: add the published words of the tiles before this
  // one, kLbWindow at a time, back to the first inclusive prefix
  unsigned excl = 0;
  const unsigned* own = a.radixStatus + (size_t)(ord & 1) * a.radixTiles * kRadixBins;
  if (binT && tile > 0) {
    const long long limit = a.barrierPolls > 0 ? a.barrierPolls : kSpinLimit;
    long long polls = 0;
    long long j = tile - 1;
    for (;;) {
      unsigned w[kLbWindow];
#pragma unroll
      for (int q = 0; q < kLbWindow; ++q)
        w[q] = j - q >= 0 ? lb_load(own + (size_t)(j - q) * kRadixBins + b) : (kLbInclusive | 1u);
      bool stop = false, incl = false;
      int used = 0;
#pragma unroll
      for (int q = 0; q < kLbWindow; ++q) {
        if (!stop) {
          if (w[q] == 0u) {
            stop = true;  // not published yet: poll it again
          } else {
            excl += (w[q] & ~kLbInclusive) - 1u;
            ++used;
            if (w[q] & kLbInclusive) incl = stop = true;
          }
        }
      }
      if (incl) break;
      j -= used;
      if (used == 0 &&
          (++polls > limit || ((polls & 255) == 0 && ld_acquire_int(&a.ctrl->error) != 0))) {
        set_error(a.ctrl, kDevTimeout, kSiteLookback, tile);
        sm.fail = 1;
        break;
      }
    }
    if (!mute)
      lb_store(a.radixStatus + ((size_t)(ord & 1) * a.radixTiles + tile) * kRadixBins + b,
               kLbInclusive | (excl + cnt + 1u));
  }
  if (binT) sm.dst[b] = sm.dst[b] + (int)excl - (int)sm.cnt[b];
  __syncthreads();
  // 5. stage the tile in digit order
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    if (kFull || ((okm >> i) & 1u)) {
      const unsigned d = digit_again<KT>(key[i], p);
      const unsigned r = (i & 1) ? rk[i >> 1] >> 16 : rk[i >> 1] & 0xFFFFu;
      const int pos = (int)sm.wc[warp][d] + (int)r;
      if constexpr (RadixSmem<U, kIdx, kItems>::kPair) {
        sm.kv[pos] = make_uint2((unsigned)U(key[i] ^ flip), (unsigned)id[i]);
      } else {
        sm.k[pos] = U(key[i] ^ flip);
        if (kIdx) sm.i[pos] = id[i];
      }
    }
  }
  __syncthreads();
  if (sm.fail) return;
  // 6. write-out: thread t takes staging slots t, t + 256, ...; consecutive
  // slots of one digit value go to consecutive addresses
  const unsigned un = (unsigned)a.n;
  U* dstK = (U*)(fromB ? a.keysA : a.keysB);
  int* dstI = a.idsLate ? late_positions(a, active, ord) : (fromB ? a.idxA : a.idxB);
  auto write = [&](auto unmap) {
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int sl = i * kRadixThreads + tid;
      if (kFull || sl < valid) {
        U raw;
        int idv = 0;
        if constexpr (RadixSmem<U, kIdx, kItems>::kPair) {
          const uint2 v = sm.kv[sl];
          raw = (U)v.x;
          idv = (int)v.y;
        } else {
          raw = sm.k[sl];
          if (kIdx) idv = sm.i[sl];
        }
        const int dst = sm.dst[digit_of<KT>(KT(raw) ^ flip, p)] + sl;
        if ((unsigned)dst < un) {  // always, when the look-back completed
          if constexpr (decltype(unmap)::value) raw = float_image<U>(raw, true);
          dstK[dst] = raw;
          if (kIdx) dstI[dst] = idv;
        }
      }
    }
  };
  if (sizeof(U) >= 4 && lastPass && a.fbits != 0) write(std::true_type{});
  else write(std::false_type{});
}

// One pass over digit p (bits 8p .. 8p+7 of the unsigned key image).  With
// ids a thread holds 2 x kItems loaded words: three resident CTAs per SM
// leave it enough registers; without ids 16 (or 8) keys a thread fit four,
// kRadixWideItems keys three.  The shared block (RadixSmem) is dynamic.
template <typename U, bool kIdx, int kItems>
__global__ void __launch_bounds__(kRadixThreads, kIdx || kItems > 16 ? 3 : 4)
    radix_pass_kernel(SortArgs a, int p) {
  constexpr int kTile = RadixSmem<U, kIdx, kItems>::kTile;
  static_assert(kTile <= 65535, "per-warp counts and staging starts are 16-bit");
  extern __shared__ __align__(16) unsigned char radix_smem[];
  RadixSmem<U, kIdx, kItems>& sm = *reinterpret_cast<RadixSmem<U, kIdx, kItems>*>(radix_smem);
  const RadixCtl* c = a.radixCtl;
  const int ord = c->ord[p];
  if (ord < 0) return;  // every key has the same digit: nothing moves
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long n = a.n;
  const long long tiles = (n + kTile - 1) / kTile;
  if (tid == 0) {
    sm.tile = (int)atomicAdd(&a.radixCtl->tileCtr[p], 1u);
    sm.fail = 0;
  }
  for (int i = lane; i < kRadixBins; i += 32) {
    sm.wc[warp][i] = 0;
    sm.mm[warp][i] = 0u;
  }
  if (tid < kRadixBins) {
    sm.cnt[tid] = 0u;
    sm.dst[tid] = (int)a.radixBase[p * kRadixBins + tid];
  }
  __syncthreads();
  const int tile = sm.tile;
  if (tile >= tiles) return;  // the grid is exactly `tiles` CTAs
  // the next moving pass uses the other look-back region: clear this tile's
  // row of it (the pass that used it last has finished)
  if (tid < kRadixBins)
    a.radixStatus[(size_t)((ord & 1) ^ 1) * a.radixTiles * kRadixBins + (size_t)tile * kRadixBins + tid] = 0u;
  const bool lastPass = p == c->last;
  const int active = c->active;
  const long long left = n - (long long)tile * kTile;
  if (left >= kTile)
    radix_pass_tile<U, kIdx, kItems, true>(a, p, ord, lastPass, active, sm, tile, kTile);
  else
    radix_pass_tile<U, kIdx, kItems, false>(a, p, ord, lastPass, active, sm, tile, (int)left);
}

template <typename U, bool kIdx>
__global__ void __launch_bounds__(256) radix_finish_kernel(SortArgs a) {
  const int active = a.radixCtl->active;
  const bool inB = (active & 1) != 0;
  const bool unmap = sizeof(U) >= 4 && active == 0 && a.fbits != 0;
  if (!inB && !unmap) return;
  U* ka = (U*)a.keysA;
  const U* kb = (const U*)a.keysB;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    if (inB) {
      ka[i] = kb[i];  // the last pass already mapped float images back
      if (kIdx && !a.idsLate) a.idxA[i] = a.idxB[i];  // late ids: radix_gather_kernel
    } else {
      ka[i] = float_image<U>(ka[i], true);
    }
  }
}

// Late ids: idxA[i] = idxC[position of the key now at i] (identity when no
// pass moved keys).  Sequential position reads, gathered id reads.
__global__ void __launch_bounds__(256) radix_gather_kernel(SortArgs a) {
  const int active = a.radixCtl->active;
  const int* pos = active > 0 ? a.idxB : nullptr;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long n = a.n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const long long src = pos ? (long long)__ldcs(pos + i) : i;
    a.idxA[i] = (src >= 0 && src < n) ? a.idxC[src] : 0;  // positions are always in range
  }
}

int device_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

// The P digit passes, one CTA per tile of kRadixThreads x kItems keys (no
// more tiles than the look-back rows, which are counted in the smallest tile).
template <typename U, bool kIdx, int kItems>
cudaError_t launch_radix_passes(const SortArgs& a, cudaStream_t stream) {
  using Smem = RadixSmem<U, kIdx, kItems>;
  constexpr int smem = (int)sizeof(Smem);
  cudaError_t e = cudaFuncSetAttribute(radix_pass_kernel<U, kIdx, kItems>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const long long passTiles = (a.n + Smem::kTile - 1) / Smem::kTile;
  for (int p = 0; p < (int)sizeof(U); ++p)
    radix_pass_kernel<U, kIdx, kItems><<<(unsigned)passTiles, kRadixThreads, smem, stream>>>(a, p);
  return cudaGetLastError();
}

template <typename U, bool kIdx>
cudaError_t launch_radix(const SortArgs& a, cudaStream_t stream, cudaEvent_t mid,
                         const cudaEvent_t* sliceDone, cudaEvent_t passStart,
                         const cudaEvent_t* keysReady, int keyChunks) {
  constexpr int P = sizeof(U);
  const long long tiles = (a.n + radix_tile(P) - 1) / radix_tile(P);
  if (a.n < 2) return cudaSuccess;
  if (tiles > a.radixTiles || a.radixHist == nullptr) return cudaErrorInvalidValue;
  const int sms = device_sms();
  cudaError_t e = cudaMemsetAsync(a.radixHist, 0, (size_t)P * kRadixBins * sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  // the histogram, in one launch or one per chunk of keys as the chunks arrive
  const int chunks = keysReady != nullptr && keyChunks > 1 ? keyChunks : 1;
  for (int c = 0; c < chunks; ++c) {
    const long long lo = c * a.n / chunks, hi = (c + 1) * a.n / chunks;
    if (keysReady != nullptr && (e = cudaStreamWaitEvent(stream, keysReady[c], 0)) != cudaSuccess)
      return e;
    const long long hb = (hi - lo + 4LL * kRadixThreads - 1) / (4LL * kRadixThreads);
    const long long histBlocks = hb < 8LL * sms ? hb : 8LL * sms;
    radix_hist_kernel<U><<<(unsigned)(histBlocks > 0 ? histBlocks : 1), kRadixThreads, 0, stream>>>(
        a, lo, hi, c == 0 ? 1 : 0);
  }
  radix_plan_kernel<U><<<1, kRadixBins, 0, stream>>>(a);
  if (passStart != nullptr && (e = cudaEventRecord(passStart, stream)) != cudaSuccess) return e;
  constexpr bool kWideOk = !kIdx && P <= 4;
  e = kWideOk && a.n >= kRadixWideMinKeys
          ? launch_radix_passes<U, kIdx, kWideOk ? kRadixWideItems : radix_items(P)>(a, stream)
          : launch_radix_passes<U, kIdx, radix_items(P)>(a, stream);
  if (e != cudaSuccess) return e;
  if (mid != nullptr && (e = cudaEventRecord(mid, stream)) != cudaSuccess) return e;
  const long long fb = (a.n + 255) / 256;
  radix_finish_kernel<U, kIdx><<<(unsigned)(fb < 8LL * sms ? fb : 8LL * sms), 256, 0, stream>>>(a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // every key is final only now: all result slices complete together
  if (sliceDone != nullptr)
    for (int sl = 0; sl < a.slices; ++sl)
      if ((e = cudaEventRecord(sliceDone[sl], stream)) != cudaSuccess) return e;
  return cudaSuccess;
}

}  // namespace

int radix_launches(int width) { return width + 3; }

cudaError_t kernels_launch_radix_gather(const SortArgs& a, cudaStream_t stream) {
  if (a.n < 1 || !a.idsLate || a.idxC == nullptr) return cudaErrorInvalidValue;
  const long long fb = (a.n + 255) / 256;
  const long long cap = 8LL * device_sms();
  radix_gather_kernel<<<(unsigned)(fb < cap ? fb : cap), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t kernels_launch_radix(int width, bool hasIdx, const SortArgs& a, cudaStream_t stream,
                                 cudaEvent_t mid, const cudaEvent_t* sliceDone,
                                 cudaEvent_t passStart, const cudaEvent_t* keysReady,
                                 int keyChunks) {
#define TURTLE_RADIX_LAUNCH(UU, II) \
  launch_radix<UU, II>(a, stream, mid, sliceDone, passStart, keysReady, keyChunks)
  switch (width) {
    case 1: return hasIdx ? TURTLE_RADIX_LAUNCH(uint8_t, true) : TURTLE_RADIX_LAUNCH(uint8_t, false);
    case 2: return hasIdx ? TURTLE_RADIX_LAUNCH(uint16_t, true) : TURTLE_RADIX_LAUNCH(uint16_t, false);
    case 4: return hasIdx ? TURTLE_RADIX_LAUNCH(uint32_t, true) : TURTLE_RADIX_LAUNCH(uint32_t, false);
    case 8: return hasIdx ? TURTLE_RADIX_LAUNCH(uint64_t, true) : TURTLE_RADIX_LAUNCH(uint64_t, false);
#undef TURTLE_RADIX_LAUNCH
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace turtle
