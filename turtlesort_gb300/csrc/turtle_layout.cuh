// Work-list layout inside one workspace allocation, shared by the sorter
// (turtle_capi.cu) and the allocation-free entry point (turtle_static.cu).
#pragma once

#include <algorithm>
#include <cstring>

#include "../../include/turtle_gb300.h"
#include "turtle_device.cuh"
#include "turtle_internal.h"
#include "turtle_tuning.h"

namespace turtle {

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct WsLayout {
  int segCap = 0, tileCap = 0, leafCap = 0, fillCap = 0, planCap = 0;
  size_t offPlanSeg[2] = {0, 0}, offPlanSmall[2] = {0, 0}, offItemTot[2] = {0, 0};
  size_t offCtrl = 0, offSegs[2] = {0, 0}, offTiles[2] = {0, 0}, offTileCnt[2] = {0, 0},
         offTileOff[2] = {0, 0};
  size_t offLeaves = 0, offLeavesSorted = 0, offFills = 0, bytes = 0;
  bool hasCls = false;   // per-key class bytes (two-level passes need them)
  size_t offCls = 0;
  int tileShift = 11;    // the smallest partition tile the lists are sized for
  int leafMax = 0;       // the smallest leaf cut the lists are sized for
  int radixTiles = 0;    // look-back rows of the radix form (0: no radix form)
  size_t offRadixHist = 0, offRadixBase = 0, offRadixCtl = 0, offRadixStatus = 0;
};

// classBytes: room for the per-key class bytes of two-level passes (without
// it, sorts use one-level passes only).  radixWidth: key bytes of the radix
// form's histograms and look-back words (0: no radix form).
inline WsLayout make_layout(long long maxN, int tile, int leafMax, long long extraLeaves,
                            bool classBytes = true, int radixWidth = 0) {
  WsLayout L;
  L.tileShift = 0;
  while ((1 << L.tileShift) < tile) ++L.tileShift;
  L.leafMax = leafMax;
  // segments of one level are disjoint and longer than leafMax
  const long long segCap = maxN / leafMax + 66;
  const long long tileCap = maxN / tile + 2 * segCap + 64;
  // leaf / fill lists: roomy enough that a partition never has to yield on
  // ordinary inputs (one level adds at most 4 leaves and 3 fills per segment)
  // (a two-level pass adds up to 16 leaves and 15 fills per segment)
  const long long leafCap = std::max(24 * (segCap + 1), maxN / 64) + extraLeaves + 4096;
  const long long fillCap = 2 * (15 * (segCap + 1) + tileCap) + maxN / 64 + 4096;
  // plan items: kThreads tiles each, at least one per segment
  const long long planCap = tileCap / turtle::kThreads + segCap + 64;
  L.planCap = (int)planCap;
  L.segCap = (int)segCap;
  L.tileCap = (int)tileCap;
  L.leafCap = (int)leafCap;
  L.fillCap = (int)fillCap;
  size_t o = 0;
  L.offCtrl = o; o = align_up(o + sizeof(turtle::Control), 256);
  for (int p = 0; p < 2; ++p) { L.offSegs[p] = o; o = align_up(o + segCap * sizeof(turtle::SegDesc), 256); }
  for (int p = 0; p < 2; ++p) { L.offTiles[p] = o; o = align_up(o + tileCap * sizeof(turtle::TileDesc), 256); }
  for (int p = 0; p < 2; ++p) { L.offTileCnt[p] = o; o = align_up(o + tileCap * turtle::kRow * sizeof(int), 256); }
  for (int p = 0; p < 2; ++p) { L.offTileOff[p] = o; o = align_up(o + tileCap * turtle::kRow * sizeof(long long), 256); }
  for (int p = 0; p < 2; ++p) { L.offPlanSeg[p] = o; o = align_up(o + planCap * sizeof(int), 256); }
  for (int p = 0; p < 2; ++p) { L.offPlanSmall[p] = o; o = align_up(o + segCap * sizeof(int), 256); }
  for (int p = 0; p < 2; ++p) { L.offItemTot[p] = o; o = align_up(o + planCap * turtle::kRow * sizeof(int), 256); }
  L.offLeaves = o; o = align_up(o + leafCap * sizeof(turtle::LeafDesc), 256);
  L.offLeavesSorted = o; o = align_up(o + leafCap * sizeof(turtle::LeafDesc), 256);
  L.offFills = o; o = align_up(o + fillCap * sizeof(turtle::FillDesc), 256);
  if (classBytes) { L.hasCls = true; L.offCls = o; o = align_up(o + (size_t)maxN + 16, 256); }
  if (radixWidth > 0) {
    const long long rt = (maxN + radix_tile(radixWidth) - 1) / radix_tile(radixWidth);
    L.radixTiles = (int)(rt > 0 ? rt : 1);
    const size_t hb = (size_t)8 * kRadixBins * sizeof(unsigned);
    L.offRadixHist = o; o = align_up(o + hb, 256);
    L.offRadixBase = o; o = align_up(o + hb, 256);
    L.offRadixCtl = o; o = align_up(o + sizeof(RadixCtl), 256);
    L.offRadixStatus = o;
    o = align_up(o + (size_t)2 * L.radixTiles * kRadixBins * sizeof(unsigned), 256);
  }
  L.bytes = o;
  return L;
}

inline int dtype_width(int dt) {
  switch (dt) {
    case TURTLE_INT8: case TURTLE_UINT8: return 1;
    case TURTLE_INT16: case TURTLE_UINT16: return 2;
    case TURTLE_INT32: case TURTLE_UINT32: case TURTLE_FLOAT32: return 4;
    case TURTLE_INT64: case TURTLE_UINT64: case TURTLE_FLOAT64: return 8;
    default: return 0;
  }
}

inline unsigned long long dtype_flip(int dt) {
  switch (dt) {
    case TURTLE_INT8: return 0x80ull;
    case TURTLE_INT16: return 0x8000ull;
    case TURTLE_INT32: return 0x80000000ull;
    case TURTLE_INT64: return 0x8000000000000000ull;
    default: return 0ull;  // unsigned keys; float keys are mapped by dtype_fbits
  }
}

// Float keys: bits of the IEEE-754 format (32 or 64), else 0.  The sort
// kernels see float keys as their totalOrder images (an elementwise map
// before the sort and its inverse after it).
inline int dtype_fbits(int dt) {
  return dt == TURTLE_FLOAT32 ? 32 : dt == TURTLE_FLOAT64 ? 64 : 0;
}

// Kernel arguments for sorting `keys` (+ `idx`) with scratch buffers
// keysB / idxB and the work lists laid out by L inside `ws`.
// Pivot rules: the reference's median of a[start+n/2], a[start], a[stop]
// (3 samples), the quartiles of kSamples evenly spaced samples, or two-level
// passes with kWideSamples samples.  All give the same output (every step is
// stable); the sampled rules need fewer levels.
constexpr int kRuleReference = 0;
constexpr int kRuleSampled = 1;
constexpr int kRuleTwoLevel = 2;
constexpr int kRuleAuto = 3;                      // two-level from kAutoTwoLevelKeys keys up
constexpr int kRuleRadix = 4;                     // LSD radix passes (plain sorts)
constexpr long long kAutoTwoLevelKeys = 1LL << 23;  // measured crossover on GB300
inline int rule_samples(int rule) {
  return rule == kRuleReference ? 3 : rule == kRuleTwoLevel ? kWideSamples : kSamples;
}

// Launch configuration tp (see turtle_tuning.h) decides the pass form under
// kRuleAuto, the tile, the leaf geometry and cut; it is clamped to what the
// work lists were laid out for.
inline SortArgs bind_args(void* keys, int* idx, void* keysB, int* idxB, char* ws, const WsLayout& L,
                          const long long* offs, long long num, long long n, int dtype,
                          int rule, TuneParams tp) {
  SortArgs a;
  std::memset(&a, 0, sizeof(a));
  a.keysA = keys;
  a.idxA = idx;
  a.keysB = keysB;
  a.idxB = idxB;
  a.offsets = offs;
  a.numArrays = num;
  a.n = n;
  a.flip = dtype_flip(dtype);
  a.fbits = dtype_fbits(dtype);
  for (int p = 0; p < 2; ++p) {
    a.segs[p] = (SegDesc*)(ws + L.offSegs[p]);
    a.tiles[p] = (TileDesc*)(ws + L.offTiles[p]);
    a.tileCnt[p] = (int*)(ws + L.offTileCnt[p]);
    a.tileOff[p] = (long long*)(ws + L.offTileOff[p]);
    a.planSeg[p] = (int*)(ws + L.offPlanSeg[p]);
    a.planSmall[p] = (int*)(ws + L.offPlanSmall[p]);
    a.itemTot[p] = (int*)(ws + L.offItemTot[p]);
  }
  a.leaves = (LeafDesc*)(ws + L.offLeaves);
  a.leavesSorted = (LeafDesc*)(ws + L.offLeavesSorted);
  a.fills = (FillDesc*)(ws + L.offFills);
  a.segCap = L.segCap;
  a.tileCap = L.tileCap;
  a.leafCap = L.leafCap;
  a.fillCap = L.fillCap;
  a.planCap = L.planCap;
  a.ctrl = (Control*)(ws + L.offCtrl);
  const int width = dtype_width(dtype);
  tp = tune_sanitize(width, tp);
  int cap = 0;
  kernels_leaf_geometry(width, tp.leafGeom, nullptr, nullptr, &cap, nullptr);
  if (L.leafMax > cap) {  // the lists need longer leaves than this geometry holds
    tp.leafGeom = kDefaultLeafGeometry;
    kernels_leaf_geometry(width, tp.leafGeom, nullptr, nullptr, &cap, nullptr);
  }
  if (tp.leafCut < L.leafMax) tp.leafCut = L.leafMax < cap ? L.leafMax : cap;
  if (tp.tileShift < L.tileShift) tp.tileShift = L.tileShift;
  if (rule == kRuleAuto) rule = tp.radix ? kRuleRadix : tp.form;
  if (rule == kRuleRadix) {
    // one array whose tiles fit the look-back rows; otherwise the pivot form
    const long long rt = (n + radix_tile(width) - 1) / radix_tile(width);
    if (offs == nullptr && L.radixTiles > 0 && rt <= L.radixTiles && n <= kRadixMaxN) a.radix = 1;
    rule = tp.form;
  }
  if (rule == kRuleTwoLevel && !L.hasCls) rule = kRuleSampled;
  if (L.radixTiles > 0) {
    a.radixTiles = L.radixTiles;
    a.radixHist = (unsigned*)(ws + L.offRadixHist);
    a.radixBase = (unsigned*)(ws + L.offRadixBase);
    a.radixCtl = (RadixCtl*)(ws + L.offRadixCtl);
    a.radixStatus = (unsigned*)(ws + L.offRadixStatus);
  }
  a.cls = L.hasCls ? (unsigned char*)(ws + L.offCls) : nullptr;
  a.samples = rule_samples(rule);
  a.slices = 1;
  a.leafYield = 0;
  a.tileShift = tp.tileShift;
  a.leafCut = tp.leafCut;
  a.leafVariant = tp.leafGeom;
  a.gridDiv = tp.gridDiv;
  kernels_leaf_geometry(width, tp.leafGeom, nullptr, &a.leafItems, nullptr, &a.leafClasses);
  return a;
}

}  // namespace turtle
