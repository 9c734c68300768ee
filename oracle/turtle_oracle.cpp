// TurtleSort oracle -- TEST INFRASTRUCTURE ONLY.
//
// This file is the CPU checker for the GB300 sort path.  Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference leg
// may load it, and only to check or to time a CPU baseline; the product path
// (turtlesort_gb300/) never calls it.
//
// What it restates (reference = tugrul512bit/TurtleSort):
//   * oracle_turtle_sort: the 3-pivot quicksort of
//     turtle-sort.cu:573-934 (quickSortWithoutStreamCompaction):
//       - pivots = sorted{a[start + num/2], a[start], a[stop]}   (:641-655)
//       - 7 classes, tested in the order ==p1, ==p2, ==p3, then <p1,
//         (p1,p2), (p2,p3), >p3                                 (:682-721)
//       - class offsets = running sum in class order            (:755-761)
//       - pivot runs are written by value and never recursed    (:832-851)
//       - children with more than one element are pushed        (:857-933)
//     The reference scatters with shared-memory atomics, so its tie order is
//     not defined.  The restatement fixes the tie order to the stable one
//     (elements of a class keep their input order) and finishes segments of
//     at most `leaf_max` elements with a stable insertion/merge sort in place
//     of sortByNetwork (:392-559) and bruteSort (:118-188; odd-even
//     transposition is itself stable).  With a stable partition and stable
//     leaves the (key, idx) output equals std::stable_sort by key, which is
//     what oracle_stable_sort computes independently.
//   * oracle_multisort_heap: the per-array heap sort of
//     turtle-multi-sort.cuh:33-84 (insert/remove) and :110-126 (the sort loop).
//   * oracle_segmented_sort: per-array stable sort, the checker for the
//     batched uneven form (no reference counterpart).
//   * cpu_* : the CPU baselines the reference README times
//     (README.md:174-181): std::sort of {key, int idx} structs on one thread,
//     std::sort(std::execution::par_unseq) and __gnu_parallel::sort (OpenMP).
#include <algorithm>
#include <array>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <execution>
#include <parallel/algorithm>
#include <omp.h>
#include <thread>
#include <vector>

namespace {

enum Dtype { I8 = 0, U8 = 1, I16 = 2, U16 = 3, I32 = 4, U32 = 5, I64 = 6, U64 = 7 };

template <typename K>
struct Pair {
  K key;
  int32_t idx;
};

// ---- restatement of quickSortWithoutStreamCompaction (stable tie order) ----

template <typename K>
struct Seg {
  int64_t start, n;
};

template <typename K>
void stable_leaf(K* a, int32_t* id, int64_t n) {
  // Stable: insertion sort for short runs, std::stable_sort of pairs otherwise.
  if (n <= 64) {
    for (int64_t i = 1; i < n; ++i) {
      K k = a[i];
      int32_t v = id ? id[i] : 0;
      int64_t j = i - 1;
      while (j >= 0 && k < a[j]) {
        a[j + 1] = a[j];
        if (id) id[j + 1] = id[j];
        --j;
      }
      a[j + 1] = k;
      if (id) id[j + 1] = v;
    }
    return;
  }
  std::vector<Pair<K>> p(n);
  for (int64_t i = 0; i < n; ++i) p[i] = {a[i], id ? id[i] : 0};
  std::stable_sort(p.begin(), p.end(),
                   [](const Pair<K>& x, const Pair<K>& y) { return x.key < y.key; });
  for (int64_t i = 0; i < n; ++i) {
    a[i] = p[i].key;
    if (id) id[i] = p[i].idx;
  }
}

// Class of one key against sorted pivots p1 <= p2 <= p3, in the reference's
// test order (turtle-sort.cu:688-718).  0:<p1 1:==p1 2:(p1,p2) 3:==p2
// 4:(p2,p3) 5:==p3 6:>p3.
template <typename K>
inline int classify(K d, K p1, K p2, K p3) {
  if (d == p1) return 1;
  if (d == p2) return 3;
  if (d == p3) return 5;
  if (d < p1) return 0;
  if (d < p2) return 2;
  if (d < p3) return 4;
  return 6;
}

// One stable 7-class partition of a[start, start+n); returns class sizes.
// `threads` > 1 splits the count and the scatter into contiguous chunks, the
// way a multi-CTA partition would; the result does not depend on it.
template <typename K>
void partition_segment(K* a, int32_t* id, K* ta, int32_t* tid, int64_t start, int64_t n,
                       int64_t cnt[7], int threads) {
  K s0 = a[start + n / 2], s1 = a[start], s2 = a[start + n - 1];
  // compareSwap(0,1), (0,2), (1,2)  (turtle-sort.cu:647-649)
  if (s1 < s0) std::swap(s0, s1);
  if (s2 < s0) std::swap(s0, s2);
  if (s2 < s1) std::swap(s1, s2);
  const K p1 = s0, p2 = s1, p3 = s2;
  int T = threads;
  if (n < (int64_t(1) << 20)) T = 1;
  std::vector<std::array<int64_t, 7>> part(T);
  const int64_t chunk = (n + T - 1) / T;
#pragma omp parallel for num_threads(T) schedule(static) if (T > 1)
  for (int t = 0; t < T; ++t) {
    std::array<int64_t, 7> c{};
    const int64_t b = start + t * chunk, e = std::min(start + n, b + chunk);
    for (int64_t i = b; i < e; ++i) c[classify(a[i], p1, p2, p3)]++;
    part[t] = c;
  }
  for (int k = 0; k < 7; ++k) {
    cnt[k] = 0;
    for (int t = 0; t < T; ++t) cnt[k] += part[t][k];
  }
  // class bases (turtle-sort.cu:755-761), then per-chunk offsets
  std::vector<std::array<int64_t, 7>> off(T);
  int64_t base = start;
  for (int k = 0; k < 7; ++k) {
    int64_t run = base;
    for (int t = 0; t < T; ++t) {
      off[t][k] = run;
      run += part[t][k];
    }
    base += cnt[k];
  }
#pragma omp parallel for num_threads(T) schedule(static) if (T > 1)
  for (int t = 0; t < T; ++t) {
    std::array<int64_t, 7> o = off[t];
    const int64_t b = start + t * chunk, e = std::min(start + n, b + chunk);
    for (int64_t i = b; i < e; ++i) {
      const int k = classify(a[i], p1, p2, p3);
      const int64_t dst = o[k]++;
      ta[dst] = a[i];
      if (id) tid[dst] = id[i];
    }
  }
  // copy back; pivot runs are written by value (turtle-sort.cu:832-851)
  const K pv[7] = {K(0), p1, K(0), p2, K(0), p3, K(0)};
  int64_t pos = start;
  for (int k = 0; k < 7; ++k) {
    if (k & 1) {
      std::fill(a + pos, a + pos + cnt[k], pv[k]);
    } else {
      std::memcpy(a + pos, ta + pos, cnt[k] * sizeof(K));
    }
    if (id) std::memcpy(id + pos, tid + pos, cnt[k] * sizeof(int32_t));
    pos += cnt[k];
  }
}

template <typename K>
void turtle_sort_impl(K* a, int32_t* id, int64_t n, int64_t leaf_max, int threads) {
  if (n < 2) return;
  if (leaf_max < 1) leaf_max = 1;
  std::vector<K> ta(n);
  std::vector<int32_t> tid(id ? n : 0);
  // Explicit work list in place of the CDP recursion (turtle-sort.cu:35-111).
  std::vector<Seg<K>> big{{0, n}};
  std::vector<Seg<K>> leaves;
  while (!big.empty()) {
    std::vector<Seg<K>> next;
    // Large segments are partitioned with all threads, small ones in parallel.
    std::vector<Seg<K>> small;
    for (auto& s : big) {
      if (s.n >= (int64_t(1) << 20) && threads > 1) {
        int64_t c[7];
        partition_segment(a, id, ta.data(), id ? tid.data() : nullptr, s.start, s.n, c, threads);
        int64_t pos = s.start;
        for (int k = 0; k < 7; ++k) {
          if (!(k & 1) && c[k] > 1) {
            if (c[k] <= leaf_max) leaves.push_back({pos, c[k]});
            else next.push_back({pos, c[k]});
          }
          pos += c[k];
        }
      } else {
        small.push_back(s);
      }
    }
    std::vector<std::vector<Seg<K>>> nx(small.size()), lv(small.size());
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1) if (threads > 1)
    for (int64_t i = 0; i < (int64_t)small.size(); ++i) {
      // depth-first inside one thread
      std::vector<Seg<K>> stack{small[i]};
      while (!stack.empty()) {
        Seg<K> s = stack.back();
        stack.pop_back();
        int64_t c[7];
        partition_segment(a, id, ta.data(), id ? tid.data() : nullptr, s.start, s.n, c, 1);
        int64_t pos = s.start;
        for (int k = 0; k < 7; ++k) {
          if (!(k & 1) && c[k] > 1) {
            if (c[k] <= leaf_max) lv[i].push_back({pos, c[k]});
            else stack.push_back({pos, c[k]});
          }
          pos += c[k];
        }
      }
    }
    for (auto& v : lv) leaves.insert(leaves.end(), v.begin(), v.end());
    big.swap(next);
  }
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16) if (threads > 1)
  for (int64_t i = 0; i < (int64_t)leaves.size(); ++i)
    stable_leaf(a + leaves[i].start, id ? id + leaves[i].start : nullptr, leaves[i].n);
}

template <typename K>
void stable_sort_impl(K* a, int32_t* id, int64_t n) {
  std::vector<Pair<K>> p(n);
  for (int64_t i = 0; i < n; ++i) p[i] = {a[i], id ? id[i] : 0};
  std::stable_sort(p.begin(), p.end(),
                   [](const Pair<K>& x, const Pair<K>& y) { return x.key < y.key; });
  for (int64_t i = 0; i < n; ++i) {
    a[i] = p[i].key;
    if (id) id[i] = p[i].idx;
  }
}

// ---- restatement of the MultiSort heap sort (turtle-multi-sort.cuh) ----
// insert (:33-47): sift a new element up; remove (:49-84): sift the root down
// choosing the larger child, ties going to the right child.
template <typename K>
void heap_insert(K* b, int64_t index) {
  while (true) {
    const int64_t parent = ((index + 1) / 2) - 1;
    if (parent < 0 || parent == index) return;
    if (b[parent] < b[index]) {
      std::swap(b[parent], b[index]);
      index = parent;
    } else {
      return;
    }
  }
}
template <typename K>
void heap_remove(K* b, int64_t index, int64_t size) {
  while (true) {
    const int64_t l = ((index + 1) * 2) - 1, r = l + 1;
    int64_t child;
    if (l < size && r < size) child = (b[l] > b[r]) ? l : r;
    else if (l < size) child = l;
    else return;
    if (b[index] < b[child]) {
      std::swap(b[index], b[child]);
      index = child;
    } else {
      return;
    }
  }
}
template <typename K>
void heap_sort_one(K* b, int64_t n) {
  for (int64_t i = 1; i < n; ++i) heap_insert(b, i);  // :112-115
  for (int64_t i = 0; i < n; ++i) {                    // :117-126
    const int64_t cur = n - i;
    K top = b[0];
    b[0] = b[cur - 1];
    heap_remove(b, 0, cur - 1);
    b[cur - 1] = top;
  }
}

template <typename K>
void multisort_impl(K* a, int64_t arr_size, int64_t num_arrays, int threads) {
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
  for (int64_t i = 0; i < num_arrays; ++i) heap_sort_one(a + i * arr_size, arr_size);
}

template <typename K>
void segmented_impl(K* a, int32_t* idx, const int64_t* offsets, int64_t num, int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64) if (threads > 1)
  for (int64_t i = 0; i < num; ++i)
    stable_sort_impl<K>(a + offsets[i], idx ? idx + offsets[i] : nullptr,
                        offsets[i + 1] - offsets[i]);
}

template <typename K>
double time_std_sort(K* a, int32_t* id, int64_t n, int mode, int threads) {
  std::vector<Pair<K>> p(n);
  for (int64_t i = 0; i < n; ++i) p[i] = {a[i], id ? id[i] : 0};
  auto cmp = [](const Pair<K>& x, const Pair<K>& y) { return x.key < y.key; };
  auto t0 = std::chrono::steady_clock::now();
  if (mode == 0) {
    std::sort(p.begin(), p.end(), cmp);
  } else if (mode == 1) {
    std::sort(std::execution::par_unseq, p.begin(), p.end(), cmp);
  } else {
    omp_set_num_threads(threads);
    __gnu_parallel::sort(p.begin(), p.end(), cmp, __gnu_parallel::parallel_tag(threads));
  }
  auto t1 = std::chrono::steady_clock::now();
  for (int64_t i = 0; i < n; ++i) {
    a[i] = p[i].key;
    if (id) id[i] = p[i].idx;
  }
  return std::chrono::duration<double>(t1 - t0).count();
}

#define DISPATCH(dtype, CALL)                              \
  switch (dtype) {                                         \
    case I8: { using K = int8_t; CALL; } break;            \
    case U8: { using K = uint8_t; CALL; } break;           \
    case I16: { using K = int16_t; CALL; } break;          \
    case U16: { using K = uint16_t; CALL; } break;         \
    case I32: { using K = int32_t; CALL; } break;          \
    case U32: { using K = uint32_t; CALL; } break;         \
    case I64: { using K = int64_t; CALL; } break;          \
    case U64: { using K = uint64_t; CALL; } break;         \
    default: return -1;                                    \
  }

}  // namespace

extern "C" {

// Restated reference 3-pivot quicksort with stable tie order.  In place.
int oracle_turtle_sort(int dtype, void* keys, int32_t* idx, int64_t n, int64_t leaf_max,
                       int threads) {
  if (threads < 1) threads = 1;
  DISPATCH(dtype, turtle_sort_impl<K>((K*)keys, idx, n, leaf_max, threads));
  return 0;
}

// Independent check: std::stable_sort of (key, idx) pairs by key.  In place.
int oracle_stable_sort(int dtype, void* keys, int32_t* idx, int64_t n) {
  DISPATCH(dtype, stable_sort_impl<K>((K*)keys, idx, n));
  return 0;
}

// Restated MultiSort heap sort: num_arrays contiguous arrays of arr_size keys.
int oracle_multisort_heap(int dtype, void* keys, int64_t arr_size, int64_t num_arrays,
                          int threads) {
  if (threads < 1) threads = 1;
  DISPATCH(dtype, multisort_impl<K>((K*)keys, arr_size, num_arrays, threads));
  return 0;
}

// Per-array stable sort of arrays [offsets[i], offsets[i+1]).
int oracle_segmented_sort(int dtype, void* keys, int32_t* idx, const int64_t* offsets,
                          int64_t num, int threads) {
  if (threads < 1) threads = 1;
  DISPATCH(dtype, segmented_impl<K>((K*)keys, idx, offsets, num, threads));
  return 0;
}

// CPU baselines; return seconds spent in the sort call alone (not the
// struct packing), or a negative value on a bad dtype.
// mode 0: std::sort, 1 thread.  mode 1: std::sort(par_unseq) (serial when
// libstdc++ has no TBB backend).  mode 2: __gnu_parallel::sort on `threads`.
double cpu_sort_pairs(int dtype, void* keys, int32_t* idx, int64_t n, int mode, int threads) {
  double s = -1.0;
  switch (dtype) {
    case I8: s = time_std_sort((int8_t*)keys, idx, n, mode, threads); break;
    case U8: s = time_std_sort((uint8_t*)keys, idx, n, mode, threads); break;
    case I16: s = time_std_sort((int16_t*)keys, idx, n, mode, threads); break;
    case U16: s = time_std_sort((uint16_t*)keys, idx, n, mode, threads); break;
    case I32: s = time_std_sort((int32_t*)keys, idx, n, mode, threads); break;
    case U32: s = time_std_sort((uint32_t*)keys, idx, n, mode, threads); break;
    case I64: s = time_std_sort((int64_t*)keys, idx, n, mode, threads); break;
    case U64: s = time_std_sort((uint64_t*)keys, idx, n, mode, threads); break;
    default: break;
  }
  return s;
}

int oracle_hardware_threads(void) { return (int)std::thread::hardware_concurrency(); }

}  // extern "C"
