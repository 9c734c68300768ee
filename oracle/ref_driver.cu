// Reference runner -- TEST INFRASTRUCTURE ONLY (pins the oracle and the
// GB300 path to the reference's own output bytes).
//
// Calls the reference's public API, exactly as its README programs do
// (tugrul512bit/TurtleSort: Turtle::TurtleSort<Type>(maxN) at
// turtle-sort.cuh:63-113, StartSorting at turtle-sort.cuh:124-184, Sync at
// turtle-sort.cuh:188-258, MultiSort<Type,ArrSize,BlockSize,true> at
// turtle-sort.cuh:265-276), on input files written by
// tests/golden/make_ref_golden.py, and writes the sorted outputs next to
// them.  It is compiled against a staged copy of the reference sources by
// oracle/ref_build.sh into oracle/_ref/ (never committed) and only runs on a
// machine with a GPU.
//
// Case file: one case per line,
//   <name> <type> <n> <ids> <reps> <input file> <output file>
// type: i8 u8 i16 u16 i32 u32 i64 u64 f32 f64 (StartSorting / Sync) or
//       m<ArrSize>x<BlockSize> (MultiSort of int arrays, shared-memory form);
// ids:  1 = an int32 index array follows the keys in the input file and is
//       passed to StartSorting, 0 = keys only (for MultiSort, n = arrays);
// reps: sorts of the same input (the first result is written; each sort's
//       Sync seconds are printed).
// Input file: n keys, then n int32 ids when ids = 1.  The output file has the
// same layout.
#include "turtle-sort.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

bool read_file(const std::string& path, void* dst, size_t bytes) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  f.read(static_cast<char*>(dst), (std::streamsize)bytes);
  return (size_t)f.gcount() == bytes;
}

bool write_file(const std::string& path, const void* a, size_t abytes, const void* b,
                size_t bbytes) {
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  f.write(static_cast<const char*>(a), (std::streamsize)abytes);
  if (bbytes) f.write(static_cast<const char*>(b), (std::streamsize)bbytes);
  return (bool)f;
}

template <typename T>
int run_sort(const std::string& name, long long n, bool ids, int reps, const std::string& in,
             const std::string& out) {
  std::vector<T> src(n), keys(n);
  std::vector<int> srcId(ids ? n : 0), id(ids ? n : 0);
  if (!read_file(in, src.data(), n * sizeof(T)) ||
      (ids && !read_file(in + ".ids", srcId.data(), n * sizeof(int)))) {
    std::printf("%s: cannot read input\n", name.c_str());
    return 1;
  }
  // capacity of at least 64: StartSorting copies two task pairs (4 ints)
  // into task buffers of maxN ints even for a single task
  // (turtle-sort.cuh:174), which fails for maxN < 4
  Turtle::TurtleSort<T> sorter((int)std::max<long long>(n, 64));
  std::vector<T> firstK;
  std::vector<int> firstI;
  for (int r = 0; r < reps; ++r) {
    keys = src;
    if (ids) id = srcId;
    sorter.StartSorting(&keys, ids ? &id : nullptr);
    const double s = sorter.Sync();
    std::printf("%s rep %d sync_seconds %.6f\n", name.c_str(), r, s);
    if (r == 0) {
      firstK = keys;
      firstI = id;
    }
  }
  if (!write_file(out, firstK.data(), n * sizeof(T), ids ? firstI.data() : nullptr,
                  ids ? n * sizeof(int) : 0)) {
    std::printf("%s: cannot write output\n", name.c_str());
    return 1;
  }
  return 0;
}

template <int A, int B>
int run_multi(const std::string& name, long long num, int reps, const std::string& in,
              const std::string& out) {
  const long long n = num * A;
  std::vector<int> src(n), keys(n), first;
  if (!read_file(in, src.data(), n * sizeof(int))) {
    std::printf("%s: cannot read input\n", name.c_str());
    return 1;
  }
  Turtle::TurtleSort<int> sorter((int)n);
  for (int r = 0; r < reps; ++r) {
    keys = src;
    const double s = sorter.MultiSort<int, A, B, true>((int)num, keys.data());
    std::printf("%s rep %d multisort_seconds %.6f\n", name.c_str(), r, s);
    if (r == 0) first = keys;
  }
  return write_file(out, first.data(), n * sizeof(int), nullptr, 0) ? 0 : 1;
}

int run_case(const std::string& line) {
  std::istringstream is(line);
  std::string name, type, in, out;
  long long n = 0;
  int ids = 0, reps = 1;
  if (!(is >> name >> type >> n >> ids >> reps >> in >> out)) return 0;  // blank / comment
  const bool withIds = ids != 0;
  // int8 keys: the reference's `char` instantiation (unsigned on Arm hosts)
  if (type == "i8") return run_sort<char>(name, n, withIds, reps, in, out);
  if (type == "u8") return run_sort<unsigned char>(name, n, withIds, reps, in, out);
  if (type == "i16") return run_sort<short>(name, n, withIds, reps, in, out);
  if (type == "u16") return run_sort<unsigned short>(name, n, withIds, reps, in, out);
  if (type == "i32") return run_sort<int>(name, n, withIds, reps, in, out);
  if (type == "u32") return run_sort<unsigned int>(name, n, withIds, reps, in, out);
  if (type == "i64") return run_sort<long>(name, n, withIds, reps, in, out);
  if (type == "u64") return run_sort<unsigned long>(name, n, withIds, reps, in, out);
  if (type == "f32") return run_sort<float>(name, n, withIds, reps, in, out);
  if (type == "f64") return run_sort<double>(name, n, withIds, reps, in, out);
  if (type == "m10x64") return run_multi<10, 64>(name, n, reps, in, out);
  if (type == "m32x32") return run_multi<32, 32>(name, n, reps, in, out);
  if (type == "m128x32") return run_multi<128, 32>(name, n, reps, in, out);
  std::printf("%s: unknown type %s\n", name.c_str(), type.c_str());
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf("usage: %s <case file>\n", argv[0]);
    return 2;
  }
  std::ifstream cases(argv[1]);
  std::string line;
  int bad = 0;
  while (std::getline(cases, line)) {
    if (line.empty() || line[0] == '#') continue;
    const int rc = run_case(line);
    std::printf("case_done %s rc %d\n", line.substr(0, line.find(' ')).c_str(), rc);
    std::fflush(stdout);
    bad += rc != 0;
  }
  return bad ? 1 : 0;
}
