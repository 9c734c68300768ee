// Launch configuration of a sort, picked per key width x index flag x size
// band from a table that turtlesort_gb300/tune.py measures on the GPU and
// writes to turtle_tuning_table.inc.
//
// The reference fixes its geometry at compile time (BRUTE_FORCE_LIMIT and
// DIRECTLY_COMPUTE_LIMIT at turtle-sort.cu:7,12; ArrSize / BlockSize template
// parameters of MultiSort, turtle-multi-sort.cuh:11,13).  Here every knob the
// tuner sweeps is a run-time value:
//   form       one-level passes (3-pivot, sampled pivots) or two-level passes
//   tileShift  partition tile of 1 << tileShift keys (1024 .. 4096)
//   leafGeom   CTA size x keys per thread of the shared-memory sort (0..3,
//              kernels_leaf_geometry)
//   leafCut    segments of at most leafCut keys go to the shared-memory sort
//              (at most the geometry's capacity)
//   gridDiv    the partition kernel runs on (resident CTAs) / gridDiv CTAs
//   radix      1: plain (one-array) sorts use the LSD radix form instead; the
//              pivot values above still configure batched sorts
#pragma once

#include <cstdint>

namespace turtle {

struct TuneParams {
  int form;       // kRuleSampled or kRuleTwoLevel
  int tileShift;
  int leafGeom;
  int leafCut;
  int gridDiv;
  int radix;
};

struct TuneEntry {  // plain and batched sorts: n (total keys) up to maxN
  int width;
  int ids;
  long long maxN;
  TuneParams p;
};

struct MultiEntry {  // fixed-size arrays (MultiSort): arrays of up to maxArr keys
  int width;
  int ids;
  int maxArr;
  int geom;
};

constexpr int kMinTileShift = 10, kMaxTileShift = 12;
constexpr int kMinLeafCut = 1024;

// Compile-time defaults (the configuration before tuning): two-level passes
// from 2^23 keys, 2048-key tiles, 512 x 16 (512 x 8 for 64-bit keys) leaf
// geometry at full capacity, every resident CTA, no radix form.
TuneParams tune_defaults(int width, long long n);
// Table entry for (width, ids, n), else the defaults.
TuneParams tune_lookup(int width, bool ids, long long n);
// Leaf geometry for MultiSort arrays of arrSize keys (-1: use the default).
int tune_multi_lookup(int width, bool ids, int arrSize);
// Smallest tile shift and leaf cut any table entry uses for (width, ids) at
// sizes up to maxN: the work lists of a sorter are laid out for them.
void tune_layout_bounds(int width, bool ids, long long maxN, int* tileShift, int* leafCut);
// Clamps p to what the geometry allows.
TuneParams tune_sanitize(int width, TuneParams p);
// Description of the table (device, date), and its entry count.
const char* tune_source();
int tune_entries();

}  // namespace turtle
