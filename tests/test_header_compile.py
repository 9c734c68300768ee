"""The drop-in C++ header compiles with g++ (no CUDA headers needed), accepts
the reference's call syntax, and links against the C ABI library."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

PROGRAM = r'''
#include "turtle-sort.cuh"
#include <vector>
#include <iostream>
int main() {
  using Type = int;
  const int n = 1000;
  Turtle::TurtleSort<Type> sortVal(n, false);               // turtle-sort.cuh:63
  std::vector<Type> sample = {5, 4, 3, 9, 8, 1};
  std::vector<int> index = {0, 1, 2, 3, 4, 5};
  sortVal.StartSorting(&sample, &index);                    // turtle-sort.cuh:124
  double t = sortVal.Sync();                                // turtle-sort.cuh:188
  for (auto& e : sample) std::cout << e << " ";
  std::cout << std::endl;
  bool ok = sortVal.MemoryCompressionSuccessful() || true;  // turtle-sort.cuh:115
  std::vector<Type> arrays(64 * 10);
  double s = sortVal.MultiSort<Type, 10, 64>(64, arrays.data());  // turtle-sort.cuh:265
  size_t ns = 0;
  { Turtle::Bench b(&ns); }                                 // README.md:146
  { TurtleGlobals::Bench b(&ns); }                          // turtle-globals.cuh:33
  Turtle::TurtleSort<unsigned char, false> keysOnly(16);
  Turtle::TurtleSort<long> wide(16);
  Turtle::TurtleSort<char> c8(16);
  Turtle::TurtleSort<short> s16(16);
  // float keys, as the reference's main.cpp (MultiSort<float, 2038, 32>)
  Turtle::TurtleSort<float> f32(32 * 2038);
  std::vector<float> fv = {2.5f, -1.0f, 0.0f, -0.0f, 7.0f, -3.25f};
  f32.StartSorting(&fv);
  f32.Sync();
  bool fok = true;
  for (size_t i = 1; i < fv.size(); ++i) fok = fok && !(fv[i] < fv[i - 1]);
  std::vector<float> farrays(32 * 2038);
  for (size_t i = 0; i < farrays.size(); ++i) farrays[i] = (float)((i * 7919u) % 1000u) - 500.0f;
  f32.MultiSort<float, 2038, 32>(32, farrays.data());
  for (size_t a = 0; a < 32; ++a)
    for (size_t i = 1; i < 2038; ++i) fok = fok && !(farrays[a * 2038 + i] < farrays[a * 2038 + i - 1]);
  Turtle::TurtleSort<double, false> f64(16);
  return (ok && fok && t >= 0 && s >= 0) ? 0 : 1;
}
'''


@pytest.fixture(scope="module")
def compiled(tmp_path_factory, native_lib):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("hdr")
    src = d / "readme_sample.cpp"
    src.write_text(PROGRAM)
    exe = d / "readme_sample"
    lib_dir = ROOT / "turtlesort_gb300"
    cmd = [gxx, "-std=c++11", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
           str(src), "-o", str(exe), "-L", str(lib_dir), "-lturtle_gb300",
           f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_readme_program_compiles_and_links(compiled):
    assert compiled.exists()


@pytest.mark.gpu
def test_readme_program_runs(compiled):
    r = subprocess.run([str(compiled)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split()[:6] == ["1", "3", "4", "5", "8", "9"]
