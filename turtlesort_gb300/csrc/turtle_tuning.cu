// Launch configurations by key width x index flag x size band (see
// turtle_tuning.h).  The table itself is generated by turtlesort_gb300/tune.py.
#include "turtle_tuning.h"

#include "turtle_internal.h"
#include "turtle_layout.cuh"

namespace {
#include "turtle_tuning_table.inc"
}  // namespace

namespace turtle {

TuneParams tune_defaults(int width, long long n) {
  TuneParams p;
  p.form = n >= kAutoTwoLevelKeys ? kRuleTwoLevel : kRuleSampled;
  p.tileShift = 11;
  p.leafGeom = kDefaultLeafGeometry;
  int cap = 0;
  kernels_leaf_geometry(width, p.leafGeom, nullptr, nullptr, &cap, nullptr);
  p.leafCut = cap;
  p.gridDiv = 1;
  p.radix = 0;
  return p;
}

TuneParams tune_sanitize(int width, TuneParams p) {
  if (p.form == kRuleRadix) {  // radix for plain sorts, two-level passes for batched ones
    p.form = kRuleTwoLevel;
    p.radix = 1;
  }
  if (p.form != kRuleSampled && p.form != kRuleTwoLevel && p.form != kRuleReference)
    p.form = kRuleSampled;
  p.radix = p.radix != 0 ? 1 : 0;
  if (p.tileShift < kMinTileShift) p.tileShift = kMinTileShift;
  if (p.tileShift > kMaxTileShift) p.tileShift = kMaxTileShift;
  if (p.leafGeom < 0 || p.leafGeom >= kLeafGeometries) p.leafGeom = kDefaultLeafGeometry;
  int cap = 0;
  kernels_leaf_geometry(width, p.leafGeom, nullptr, nullptr, &cap, nullptr);
  if (p.leafCut > cap || p.leafCut <= 0) p.leafCut = cap;
  if (p.leafCut < kMinLeafCut) p.leafCut = kMinLeafCut < cap ? kMinLeafCut : cap;
  if (p.gridDiv != 1 && p.gridDiv != 2 && p.gridDiv != 4) p.gridDiv = 1;
  return p;
}

TuneParams tune_lookup(int width, bool ids, long long n) {
  const TuneEntry* best = nullptr;
  for (const TuneEntry& e : kTuneTable) {
    if (e.width != width || e.ids != (ids ? 1 : 0)) continue;
    best = &e;  // entries of one (width, ids) are in increasing maxN
    if (n <= e.maxN) break;
  }
  return best ? tune_sanitize(width, best->p) : tune_defaults(width, n);
}

int tune_multi_lookup(int width, bool ids, int arrSize) {
  int g = -1;
  for (const MultiEntry& e : kMultiTable) {
    if (e.width != width || e.ids != (ids ? 1 : 0)) continue;
    g = e.geom;
    if (arrSize <= e.maxArr) break;
  }
  return g;
}

void tune_layout_bounds(int width, bool ids, long long maxN, int* tileShift, int* leafCut) {
  const TuneParams d = tune_defaults(width, maxN);
  int ts = d.tileShift, lc = d.leafCut;
  long long prev = 0;
  for (const TuneEntry& e : kTuneTable) {
    if (e.width != width || e.ids != (ids ? 1 : 0)) continue;
    if (prev <= maxN) {  // this band holds sizes the sorter can be asked for
      const TuneParams p = tune_sanitize(width, e.p);
      ts = p.tileShift < ts ? p.tileShift : ts;
      lc = p.leafCut < lc ? p.leafCut : lc;
    }
    prev = e.maxN + 1;
  }
  *tileShift = ts;
  *leafCut = lc;
}

const char* tune_source() { return kTuneSourceText; }

int tune_entries() {
  int k = 0;
  for (const TuneEntry& e : kTuneTable) k += e.width != 0;
  return k;
}

}  // namespace turtle
