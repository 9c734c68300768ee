// Two-level partition passes of persistent_sort_kernel (the default for
// large sorts; rule TURTLE_PIVOTS_TWO_LEVEL).
//
// One pass applies two levels of the 3-pivot partition at once.  A key's
// class c1 against its segment's pivots (7 classes) and, when c1 is not a
// pivot run, its class c2 against child c1/2's pivots give one of 31 classes
// k = 8*(c1/2) + (c1 odd ? 7 : c2), in key order, so one stable counting pass
// (COUNT, PLAN, SCATTER as in the one-level pass) moves every key straight to
// its grandchild: half the passes over the data, half the grid barriers.  A
// segment's pivots are the quartiles of its kWideSamples evenly spaced
// samples; child ci's pivots are the quartiles of the samples that fall in
// child ci.  COUNT computes each key's class once (a lower bound over the 15
// pivots in key order) and stores it as a byte for SCATTER.  SCATTER records
// the samples of every new grandchild segment as it writes the keys at the
// sample positions.  Every step is stable, so the output is the stable sort
// by key whatever the samples are.
#pragma once

namespace turtle {

constexpr int kWideClasses = 31;  // classes of a two-level pass (class 31 unused)

// Position of sample i of ns in a segment of m keys starting at pos.
__device__ __forceinline__ long long wide_sample_pos(long long pos, long long m, int i, int ns) {
  return pos + ((2 * (long long)i + 1) * m) / (2 * ns);
}

// The pivots of a segment and of its four children from its samples, by one
// warp (every caller gets the same result).  The samples (two per lane) are
// sorted by a bitonic network; the parent pivots are ranks ns/4, ns/2, 3ns/4.
// The samples of parent class 2ci are contiguous in the sorted order; child
// ci's pivots are their quartiles, or the neighbouring parent pivots when the
// class holds no sample.
template <typename KT>
__device__ __noinline__ void wide_pivots_warp(const SegDesc* sd, WidePivots<KT>* out) {
  const int lane = threadIdx.x & 31;
  const int ns = __ldcg(&sd->nsamp);
  const int e0 = 2 * lane, e1 = 2 * lane + 1;
  KT x0 = e0 < ns ? (KT)__ldcg(&sd->samp[e0]) : key_max<KT>();
  KT x1 = e1 < ns ? (KT)__ldcg(&sd->samp[e1]) : key_max<KT>();
#pragma unroll
  for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j == 1) {
        const bool asc = (e0 & k) == 0;
        const KT lo = x0 < x1 ? x0 : x1, hi = x0 < x1 ? x1 : x0;
        x0 = asc ? lo : hi;
        x1 = asc ? hi : lo;
      } else {
        const KT y0 = __shfl_xor_sync(0xffffffffu, x0, j >> 1);
        const KT y1 = __shfl_xor_sync(0xffffffffu, x1, j >> 1);
        const bool keepMin0 = ((e0 & k) == 0) == ((e0 & j) == 0);
        const bool keepMin1 = ((e1 & k) == 0) == ((e1 & j) == 0);
        x0 = keepMin0 ? (y0 < x0 ? y0 : x0) : (y0 < x0 ? x0 : y0);
        x1 = keepMin1 ? (y1 < x1 ? y1 : x1) : (y1 < x1 ? x1 : y1);
      }
    }
  }
  // sorted sample of rank r (warp-uniform r)
  auto at = [&](int r) -> KT {
    return __shfl_sync(0xffffffffu, (r & 1) ? x1 : x0, (r >> 1) & 31);
  };
  WidePivots<KT> wp;
  PivotSet<KT>& pp = wp.par;
  pp.p[0] = at(ns / 4);
  pp.p[1] = at(ns / 2);
  pp.p[2] = at((3 * ns) / 4);
  pp.lut = pivot_lut(pp.p[0] == pp.p[1], pp.p[1] == pp.p[2]);
  const int c0 = e0 < ns ? class_lut<KT>(x0, pp.p[0], pp.p[1], pp.p[2], pp.lut) : 99;
  const int c1 = e1 < ns ? class_lut<KT>(x1, pp.p[0], pp.p[1], pp.p[2], pp.lut) : 99;
#pragma unroll
  for (int ci = 0; ci < 4; ++ci) {
    const int want = 2 * ci;
    const int below = __popc(__ballot_sync(0xffffffffu, c0 < want)) +
                      __popc(__ballot_sync(0xffffffffu, c1 < want));
    const int cnt = __popc(__ballot_sync(0xffffffffu, c0 == want)) +
                    __popc(__ballot_sync(0xffffffffu, c1 == want));
    PivotSet<KT>& cs = wp.child[ci];
    if (cnt > 0) {
      cs.p[0] = at(below + cnt / 4);
      cs.p[1] = at(below + cnt / 2);
      cs.p[2] = at(below + (3 * cnt) / 4);
    } else {
      const KT lo = ci == 0 ? pp.p[0] : pp.p[ci - 1];
      const KT hi = ci == 3 ? pp.p[2] : pp.p[ci];
      cs.p[0] = lo;
      cs.p[1] = lo;
      cs.p[2] = hi;
    }
    cs.lut = pivot_lut(cs.p[0] == cs.p[1], cs.p[1] == cs.p[2]);
  }
  if (lane == 0) *out = wp;
  __syncwarp();
}

// The 15 pivots of a two-level pass in key order: child ci's three pivots,
// then the parent's pivot ci (for ci < 3).  Child ci's pivots lie between the
// parent pivots around it, so the sequence is sorted.  The class of key k is
// then 2 * #{q < k} + [k equals the first q not below it]: a key equal to a
// pivot goes to the first run of that value, every other key to its gap.
// Lanes 0..14 write the sequence; the caller synchronizes the warp.
template <typename KT>
__device__ __forceinline__ void wide_sequence(const WidePivots<KT>& wp, KT* q) {
  const int lane = threadIdx.x & 31;
  if (lane < 15) {
    const int ci = lane >> 2, j = lane & 3;
    q[lane] = j < 3 ? wp.child[ci].p[j] : wp.par.p[ci];
  }
}

// Class (0..30) of key k from the sorted 15-pivot sequence (branchless lower
// bound: four probes, then one equality test).
template <typename KT>
__device__ __forceinline__ unsigned wide_class_seq(KT k, const KT* q) {
  int r = q[7] < k ? 8 : 0;
  r += q[r + 3] < k ? 4 : 0;
  r += q[r + 1] < k ? 2 : 0;
  r += q[r] < k ? 1 : 0;
  const bool eq = q[r < 15 ? r : 14] == k && r < 15;
  return 2u * (unsigned)r + (eq ? 1u : 0u);
}

// COUNT of a two-level pass: tile t's 31 class counts go to its row of
// tileCnt and each key's class to its byte of a.cls (for SCATTER); the warp's
// running class totals of the segment (accSeg / accCnt, lane k holds class k)
// go to the segment when the warp moves on.
template <typename U, bool kIdx>
__device__ __forceinline__ void count31_tile_warp(const SortArgs& a, int pass, int t,
                                                  typename Persist<U, kIdx>::WarpArea& ws,
                                                  unsigned& phases, int& accSeg, int& accCnt) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kItems = P::kItems, kWCH = P::kWCH;
  // tiles are at most 4096 keys: a lane tallies at most 128 keys of a tile
  const int kShift = a.tileShift;
  const int par = pass & 1;
  const int lane = threadIdx.x & 31;
  const U* src = (const U*)(par ? a.keysB : a.keysA);
  const KT flip = (KT)a.flip;
  const TileDesc td = load_tile(&a.tiles[par][t]);
  const long long abs0 = (td.lo >> kShift) << kShift;
  const int rlo = (int)(td.lo - abs0), rhi = (int)(td.hi - abs0);
  const int chBeg = rlo / kWCH, chEnd = (rhi + kWCH - 1) / kWCH;
  if (lane == 0 && chunk_bulk_ok<U, false>(src, nullptr, abs0 + (long long)chBeg * kWCH, a.n))
    chunk_bulk_issue<U, kIdx, false>(ws, 0, src, nullptr, abs0 + (long long)chBeg * kWCH);
  if (td.seg != ws.t.pivSeg) {  // pivots of the warp's last segment are kept
    wide_pivots_warp<KT>(&a.segs[par][td.seg], &ws.t.wp);
    wide_sequence<KT>(ws.t.wp, ws.t.q);
    __syncwarp();
    ws.t.pivSeg = td.seg;
  }
  const KT* q = ws.t.q;
  // per-lane class tallies, one byte each (a lane sees at most tile / 32 <=
  // 128 keys of a tile): cnt[32 * k + lane], in the stage buffer, which COUNT
  // does not use otherwise
  static_assert(sizeof(ws.sk) >= 32 * 32, "the stage holds 32 x 32 byte tallies");
  unsigned char* cnt = reinterpret_cast<unsigned char*>(ws.sk);
  {
    unsigned* z = reinterpret_cast<unsigned*>(cnt);
#pragma unroll
    for (int j = 0; j < 8; ++j) z[32 * j + lane] = 0u;
  }
  __syncwarp();
  for (int ch = chBeg; ch < chEnd; ++ch) {
    const int b = (ch - chBeg) & 1;
    const long long c0 = abs0 + (long long)ch * kWCH;
    if (ch + 1 < chEnd && lane == 0 && chunk_bulk_ok<U, false>(src, nullptr, c0 + kWCH, a.n))
      chunk_bulk_issue<U, kIdx, false>(ws, b ^ 1, src, nullptr, c0 + kWCH);
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
      chunk_wait<U, kIdx>(ws, b, phases, a.ctrl);
      chunk_keys<U, kIdx>(ws, b, lane, flip, key);
    } else {
      load_chunk<U, KT, kItems>(src + abs0, abs0, a.n, e0, rlo, rhi, flip, key);
    }
    unsigned cb0 = 0, cb1 = 0;  // the keys' classes, one byte each, for SCATTER
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      if (okm >> i & 1u) {
        const unsigned k = wide_class_seq<KT>(key[i], q);
        cnt[32 * k + lane] += 1;
        if (i < 4) cb0 |= k << (8 * i);
        else cb1 |= k << (8 * (i - 4));
      }
    }
    {
      unsigned char* cdst = a.cls + c0 + lane * kItems;
      if (okm == (1u << kItems) - 1u) {
        if (kItems == 8) *reinterpret_cast<uint2*>(cdst) = make_uint2(cb0, cb1);
        else *reinterpret_cast<unsigned*>(cdst) = cb0;
      } else {
#pragma unroll
        for (int i = 0; i < kItems; ++i)
          if (okm >> i & 1u) cdst[i] = (unsigned char)((i < 4 ? cb0 >> (8 * i) : cb1 >> (8 * (i - 4))) & 0xFFu);
      }
    }
    __syncwarp();
  }
  // lane k sums class k's 32 lane tallies (four bytes per word)
  unsigned sum = 0u;
  {
    const unsigned* row = reinterpret_cast<const unsigned*>(cnt + 32 * lane);
#pragma unroll
    for (int j = 0; j < 8; ++j) sum = __dp4a(row[j], 0x01010101u, sum);
  }
  const int mine = (int)sum;
  __syncwarp();
  a.tileCnt[par][(long long)t * kRow + lane] = mine;
  if (td.seg != accSeg) {
    if (accSeg >= 0 && accCnt) atomicAdd(&a.segs[par][accSeg].tot[lane], accCnt);
    accSeg = td.seg;
    accCnt = 0;
  }
  accCnt += mine;
}

// PLAN of a two-level pass, one plan item (kThreads tiles of one segment):
// the destination of every tile and class (class bases from the segment's
// class totals, then the tiles in memory order: stable).  Item 0 also routes
// the 31 classes (SCATTER takes the classes from COUNT): the parent's pivot runs
// and the children's pivot runs are parked for a fill when the keys go to the
// scratch buffer; a child of at most kLeafMax keys becomes one leaf whatever
// its second-level classes; every other grandchild becomes a leaf or a
// next-pass segment.
template <typename U, bool kIdx>
__device__ __noinline__ void plan31_item(const SortArgs& a, int pass, int item,
                                         typename Persist<U, kIdx>::Smem& sm) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  const int kLeafMax = a.leafCut;  // at least kWideSamples: every segment holds its samples
  const int par = pass & 1;
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
  const int myTile = t0 + tid;
  // class counts of the segment's tiles before this item, from the item totals
  item_prefix<U, kIdx>(a, par, planBase, j, sm);
  if (tid < 32) {
    int x = tid < kWideClasses ? __ldcg(&sdp->tot[tid]) : 0;
    const int tot = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    sm.wcb[tid] = x - tot;  // class start relative to the segment
    if (tid == 31) sm.wcb[32] = x;
  }
  if (j == 0 && warp == 1) wide_pivots_warp<KT>(sdp, &sm.wpiv);
  // offsets, eight classes per round
  for (int g = 0; g < 4; ++g) {
    int v[8], inc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = 0;
    if (myTile < nt) {
      const int4* row = reinterpret_cast<const int4*>(cnt + (long long)myTile * kRow + 8 * g);
      const int4 x = __ldcg(row), y = __ldcg(row + 1);
      v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
      v[4] = y.x; v[5] = y.y; v[6] = y.z; v[7] = y.w;
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
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
    if (tid < 8) {
      int acc = 0;
      for (int w = 0; w < kWarps; ++w) {
        const int x = sm.red[w][tid];
        sm.red[w][tid] = acc;
        acc += x;
      }
      sm.pre[tid] = sm.preAll[8 * g + tid];
    }
    __syncthreads();
    if (myTile < nt) {
      longlong2* dst = reinterpret_cast<longlong2*>(a.tileOff[par] +
                                                    (long long)(tileBase + myTile) * kRow + 8 * g);
#pragma unroll
      for (int c = 0; c < 8; c += 2) {
        const long long o0 =
            sdStart + sm.wcb[8 * g + c] + sm.pre[c] + sm.red[warp][c] + (inc[c] - v[c]);
        const long long o1 = sdStart + sm.wcb[8 * g + c + 1] + sm.pre[c + 1] +
                             sm.red[warp][c + 1] + (inc[c + 1] - v[c + 1]);
        dst[c / 2] = make_longlong2(o0, o1);
      }
    }
    __syncthreads();
  }
  if (j != 0) return;

  // item 0: routing (warp 0, lane k = class k)
  const bool dstIsA = (par == 1);
  const int nextPar = par ^ 1;
  if (warp == 0) {
    const int k = lane, ci = k >> 3, jj = k & 7;
    unsigned park = 0u;
    if (k < kWideClasses) {
      const long long pos = sdStart + sm.wcb[k];
      const long long m = sm.wcb[k + 1] - sm.wcb[k];
      const long long cStart = sdStart + sm.wcb[8 * ci];
      const long long cN = (long long)sm.wcb[8 * ci + 7] - sm.wcb[8 * ci];  // child ci
      const bool leafChild = cN <= kLeafMax;
      if (jj == 7) {  // the parent's pivot run ci
        if (m > 0 && !dstIsA) {
          push_fill(a, pos, m, (unsigned long long)sm.wpiv.par.p[ci]);
          park = 1u;
        }
      } else if (leafChild) {
        if (jj == 0) {
          if (cN > 1 || (cN == 1 && !dstIsA)) push_leaf(a, cStart, cN, dstIsA ? 0 : 1);
          for (int q = 0; q < 4; ++q) sm.gSeg[ci * 4 + q] = -1;
        }
      } else if (jj & 1) {  // child ci's pivot run jj/2
        if (m > 0 && !dstIsA) {
          push_fill(a, pos, m, (unsigned long long)sm.wpiv.child[ci].p[jj >> 1]);
          park = 1u;
        }
      } else {  // grandchild g
        const int g = ci * 4 + (jj >> 1);
        int si = -1;
        if (m > 1 || (m == 1 && !dstIsA)) {
          if (m <= kLeafMax) {
            push_leaf(a, pos, m, dstIsA ? 0 : 1);
          } else {
            int tb = 0, ntc = 0;
            si = alloc_segment(a, nextPar, pos, m, &tb, &ntc, true);
            if (si >= 0) a.segs[nextPar][si].nsamp = kWideSamples;
            sm.gTb[g] = tb;
            sm.gNt[g] = si >= 0 ? ntc : 0;
            sm.gStart[g] = pos;
            sm.gN[g] = m;
          }
        }
        sm.gSeg[g] = si;
      }
      sdp->cbase[k] = pos;
    } else {
      sdp->cbase[31] = sdStart + sm.wcb[32];
    }
    const unsigned pm = __ballot_sync(kFull, park != 0u);
    if (lane == 0) sdp->parkMask = pm;
  }
  __syncthreads();
  if (tid < 16) sdp->childSeg[tid] = sm.gSeg[tid];
  for (int g = 0; g < 16; ++g) {
    if (sm.gSeg[g] >= 0)
      write_tiles(a, nextPar, sm.gSeg[g], sm.gTb[g], sm.gNt[g], sm.gStart[g], sm.gN[g],
                         tid, kThreads);
  }
  __syncthreads();
}

// plan31_item for a segment of at most kSmallPlanTiles tiles, by one warp:
// lane k owns class k, so the destinations of the segment's tiles are a
// running prefix over its tiles in memory order (one 128-byte row read and
// one 256-byte row write per tile); the warp then routes the 31 classes as
// item 0 does.  `scratch` is the warp's own pivot slot (idle during PLAN).
template <typename U, bool kIdx>
__device__ __noinline__ void plan31_small_warp(const SortArgs& a, int pass, int seg,
                                               WidePivots<typename Persist<U, kIdx>::KT>* scratch) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  const int kLeafMax = a.leafCut;
  const int par = pass & 1;
  const int lane = threadIdx.x & 31;
  SegDesc* sdp = &a.segs[par][seg];
  const long long sdStart = __ldcg(&sdp->start);
  const int tileBase = __ldcg(&sdp->tileBase);
  const int nt = __ldcg(&sdp->ntiles);
  const int* cnt = a.tileCnt[par] + (long long)tileBase * kRow;
  long long* off = a.tileOff[par] + (long long)tileBase * kRow;
  const int tot = lane < kWideClasses ? __ldcg(&sdp->tot[lane]) : 0;
  int incl = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += y;
  }
  const int base = incl - tot;                   // class start relative to the segment
  const int end = __shfl_sync(kFull, incl, 31);  // segment size
  {
    long long run = sdStart + base;
#pragma unroll 4
    for (int t = 0; t < nt; ++t) {
      const int v = __ldcg(cnt + (long long)t * kRow + lane);
      off[(long long)t * kRow + lane] = run;
      run += v;
    }
  }
  wide_pivots_warp<KT>(sdp, scratch);
  const WidePivots<KT> wp = *scratch;
  // routing: lane k = class k; child ci is classes 8ci .. 8ci+6
  const bool dstIsA = (par == 1);
  const int nextPar = par ^ 1;
  const int k = lane, ci = k >> 3, jj = k & 7;
  const int cBase = __shfl_sync(kFull, base, 8 * ci);
  const int cEnd = __shfl_sync(kFull, base, 8 * ci + 7);  // start of class 8ci+7
  unsigned park = 0u;
  int si = -1, tb = 0, ntc = 0;
  const long long pos = sdStart + base;
  const long long m = tot;
  if (k < kWideClasses) {
    const long long cStart = sdStart + cBase;
    const long long cN = (long long)cEnd - cBase;
    const bool leafChild = cN <= kLeafMax;
    if (jj == 7) {  // the parent's pivot run ci
      if (m > 0 && !dstIsA) {
        push_fill(a, pos, m, (unsigned long long)wp.par.p[ci]);
        park = 1u;
      }
    } else if (leafChild) {
      if (jj == 0 && (cN > 1 || (cN == 1 && !dstIsA))) push_leaf(a, cStart, cN, dstIsA ? 0 : 1);
    } else if (jj & 1) {  // child ci's pivot run jj/2
      if (m > 0 && !dstIsA) {
        push_fill(a, pos, m, (unsigned long long)wp.child[ci].p[jj >> 1]);
        park = 1u;
      }
    } else if (m > 1 || (m == 1 && !dstIsA)) {  // grandchild
      if (m <= kLeafMax) {
        push_leaf(a, pos, m, dstIsA ? 0 : 1);
      } else {
        si = alloc_segment(a, nextPar, pos, m, &tb, &ntc, true);
        if (si >= 0) a.segs[nextPar][si].nsamp = kWideSamples;
      }
    }
    sdp->cbase[k] = pos;
  } else {
    sdp->cbase[31] = sdStart + end;
  }
  const unsigned pm = __ballot_sync(kFull, park != 0u);
  // tiles of the new segments; grandchild g = 4ci + q is class 8ci + 2q
  int gseg = -1;
#pragma unroll
  for (int g = 0; g < 16; ++g) {
    const int src = 8 * (g >> 2) + 2 * (g & 3);
    const int s = __shfl_sync(kFull, si, src);
    if (lane == g) gseg = s;
    if (s >= 0) {
      const int ctb = __shfl_sync(kFull, tb, src);
      const int cnt2 = __shfl_sync(kFull, ntc, src);
      const long long cs = __shfl_sync(kFull, pos, src);
      const long long cn = __shfl_sync(kFull, m, src);
      write_tiles(a, nextPar, s, ctb, cnt2, cs, cn, lane, 32);
    }
  }
  if (lane < 16) sdp->childSeg[lane] = gseg;
  if (lane == 0) sdp->parkMask = pm;
  __syncwarp();
}

// Lane 0: bulk-copy keys, ids and class bytes of the chunk at c0 into buffer b.
template <typename U, bool kIdx>
__device__ __forceinline__ void wide_bulk_issue(typename Persist<U, kIdx>::WarpArea& ws, int b,
                                                const U* srcK, const int* srcI,
                                                const unsigned char* cls, long long c0) {
  constexpr int kWCH = Persist<U, kIdx>::kWCH;
  constexpr unsigned kBytes = kWCH * sizeof(U) + (kIdx ? kWCH * 4 : 0) + kWCH;
  fence_proxy_async_smem();
  mbar_arm(&ws.mbar[b], kBytes);
  bulk_g2s(ws.pk[b], srcK + c0, kWCH * sizeof(U), &ws.mbar[b]);
  if (kIdx) bulk_g2s(ws.pi[b], srcI + c0, kWCH * 4, &ws.mbar[b]);
  bulk_g2s(ws.pc[b], cls + c0, kWCH, &ws.mbar[b]);
}

// SCATTER of a two-level pass: scatter_tile_warp with 31 classes.  The keys'
// classes come from COUNT (one byte per key, bulk-copied with the keys and
// ids).  Items are lane-strided (item i of lane l is chunk element 32i + l),
// so ranking them item by item keeps memory order: the lanes of one class
// are found with one match instruction, and a per-warp running count per
// class gives the rank.  The class starts come from a lane scan of the chunk's
// class totals.  Lane k also watches the sample positions of grandchild class
// k and copies the staged key written there into the new segment's samples.
template <typename U, bool kIdx>
__device__ __forceinline__ void scatter31_tile_warp(const SortArgs& a, int pass, int t,
                                                    typename Persist<U, kIdx>::WarpArea& ws,
                                                    unsigned& phases) {
  using P = Persist<U, kIdx>;
  using KT = typename P::KT;
  constexpr int kItems = P::kItems, kWCH = P::kWCH;
  const int kShift = a.tileShift;
  const int par = pass & 1;
  const KT flip = (KT)a.flip;
  const int lane = threadIdx.x & 31;
  const TileDesc td = load_tile(&a.tiles[par][t]);
  const long long abs0 = (td.lo >> kShift) << kShift;
  const int rlo = (int)(td.lo - abs0), rhi = (int)(td.hi - abs0);
  const U* srcK = (const U*)(par ? a.keysB : a.keysA);
  const int* srcI = par ? a.idxB : a.idxA;
  const int chBeg = rlo / kWCH, chEnd = (rhi + kWCH - 1) / kWCH;
  if (lane == 0 && chunk_bulk_ok<U, kIdx>(srcK, srcI, abs0 + (long long)chBeg * kWCH, a.n))
    wide_bulk_issue<U, kIdx>(ws, 0, srcK, srcI, a.cls, abs0 + (long long)chBeg * kWCH);
  const SegDesc* sdp = &a.segs[par][td.seg];
  const unsigned parkMask = __ldcg(&sdp->parkMask);
  {
    // running destination of class `lane`, and its next sample position
    const long long wb = __ldcg(&a.tileOff[par][(long long)t * kRow + lane]);
    ws.t.wbase[lane] = wb;
    long long nextP = LLONG_MAX;
    int nextI = 0;
    const int jj = lane & 7;
    if (lane < kWideClasses && jj < 7 && !(jj & 1)) {
      const int gs = __ldcg(&sdp->childSeg[(lane >> 3) * 4 + (jj >> 1)]);
      if (gs >= 0) {
        const long long gpos = __ldcg(&sdp->cbase[lane]);
        const long long m = __ldcg(&sdp->cbase[lane + 1]) - gpos;
        const long long r = wb - gpos;  // class rank of the tile's first key of the class
        // first sample i with floor((2i+1) m / 2ns) >= r
        const long long q = (2 * (long long)kWideSamples * r + m - 1) / m;
        nextI = (int)(q / 2);
        if (nextI < kWideSamples) nextP = wide_sample_pos(gpos, m, nextI, kWideSamples);
      }
    }
    ws.t.capP[lane] = nextP;
    ws.t.capI[lane] = nextI;
  }
  __syncwarp();
  U* dstK = (U*)(par ? a.keysA : a.keysB);
  int* dstI = par ? a.idxA : a.idxB;

  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  for (int ch = chBeg; ch < chEnd; ++ch) {
    const int b = (ch - chBeg) & 1;
    const long long c0 = abs0 + (long long)ch * kWCH;
    if (ch + 1 < chEnd && lane == 0 && chunk_bulk_ok<U, kIdx>(srcK, srcI, c0 + kWCH, a.n))
      wide_bulk_issue<U, kIdx>(ws, b ^ 1, srcK, srcI, a.cls, c0 + kWCH);
    // lane-strided items: item i of this lane is chunk element 32 * i + lane,
    // so ranking item by item follows memory order (stable)
    const bool inner = ch * kWCH >= rlo && (ch + 1) * kWCH <= rhi;
    KT key[kItems];
    if (chunk_bulk_ok<U, kIdx>(srcK, srcI, c0, a.n)) {
      chunk_wait<U, kIdx>(ws, b, phases, a.ctrl);
#pragma unroll
      for (int i = 0; i < kItems; ++i) key[i] = KT(ws.pk[b][32 * i + lane]) ^ flip;
    } else {
      // array end: plain loads; ids and classes go through the buffers like bulk ones
#pragma unroll
      for (int i = 0; i < kItems; ++i) {
        const int e = ch * kWCH + 32 * i + lane;
        const bool ok = e >= rlo && e < rhi;
        key[i] = ok ? KT(__ldcg(srcK + abs0 + e)) ^ flip : KT(0);
        if (kIdx) ws.pi[b][32 * i + lane] = ok ? __ldcg(srcI + abs0 + e) : 0;
        ws.pc[b][32 * i + lane] = ok ? __ldcg(a.cls + abs0 + e) : (unsigned char)31;
      }
      __syncwarp();
    }
    ws.t.cnt[lane] = 0;
    __syncwarp();
    // class (5 bits, 31 = no key) and rank in the chunk (8 bits) of each item
    unsigned cwLo = 0, cwHi = 0, rk0 = 0, rk1 = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int e = ch * kWCH + 32 * i + lane;
      const unsigned k = (inner || (e >= rlo && e < rhi)) ? (unsigned)ws.pc[b][32 * i + lane] : 31u;
      // lanes of the same class (one match instruction; measured a little
      // faster than one vote per class bit)
      const unsigned peers = __match_any_sync(kFull, k);
      const int base = ws.t.cnt[k];
      const unsigned r = (unsigned)(base + __popc(peers & lt));
      __syncwarp();
      if ((peers >> lane) == 1u) ws.t.cnt[k] = base + __popc(peers);  // highest lane of the class
      __syncwarp();
      if (i < 4) rk0 |= r << (8 * i);
      else rk1 |= r << (8 * (i - 4));
      if (i < 6) cwLo |= k << (5 * i);
      else cwHi |= k << (5 * (i - 6));
    }
    // class starts in the stage (lane k: class k; class 31 holds no key)
    const int totk = lane < kWideClasses ? ws.t.cnt[lane] : 0;
    int csk = totk;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, csk, o);
      if (lane >= o) csk += y;
    }
    const int nv = __shfl_sync(kFull, csk, 31);
    csk -= totk;
    ws.t.cs[lane] = csk;
    // destination table of the chunk: delta[k] = running base - class start
    const long long wbLo = ws.t.wbase[lane];
    ws.t.delta[lane] = wbLo - (long long)csk;
    ws.t.wbase[lane] = wbLo + totk;
    __syncwarp();
    // stage by class
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const unsigned k = i < 6 ? (cwLo >> (5 * i)) & 31u : (cwHi >> (5 * (i - 6))) & 31u;
      if (k != 31u) {
        const unsigned pos = (unsigned)ws.t.cs[k] + ((i < 4 ? rk0 >> (8 * i) : rk1 >> (8 * (i - 4))) & 0xFFu);
        ws.sk[pos] = key[i];
        if (kIdx) ws.si[pos] = ws.pi[b][32 * i + lane];
        ws.sc[pos] = (unsigned char)k;
      }
    }
    __syncwarp();
    // write-out: consecutive stage slots of one class go to consecutive addresses
#pragma unroll
    for (int jw = 0; jw < kItems; ++jw) {
      const int sl = 32 * jw + lane;
      if (sl < nv) {
        const unsigned k = ws.sc[sl];
        const long long d = ws.t.delta[k] + sl;
        if (!((parkMask >> k) & 1u)) dstK[d] = U(ws.sk[sl] ^ flip);
        if (kIdx) dstI[d] = ws.si[sl];
      }
    }
    // samples of grandchild class `lane` written by this chunk
    {
      long long nextP = ws.t.capP[lane];
      const long long hiP = wbLo + totk;
      if (nextP < hiP) {
        const int gs = __ldcg(&sdp->childSeg[(lane >> 3) * 4 + ((lane & 7) >> 1)]);
        const long long gpos = __ldcg(&sdp->cbase[lane]);
        const long long m = __ldcg(&sdp->cbase[lane + 1]) - gpos;
        int nextI = ws.t.capI[lane];
        SegDesc* gd = &a.segs[par ^ 1][gs];
        while (nextP < hiP) {
          gd->samp[nextI] = (unsigned long long)ws.sk[csk + (int)(nextP - wbLo)];
          ++nextI;
          nextP = nextI < kWideSamples ? wide_sample_pos(gpos, m, nextI, kWideSamples) : LLONG_MAX;
        }
        ws.t.capP[lane] = nextP;
        ws.t.capI[lane] = nextI;
      }
    }
    __syncwarp();
  }
}

}  // namespace turtle
