"""Host check of the bit-level FP64 <-> double-float conversions
(s2let_gb300/csrc/dfconv.h) used by the split-precision kernels: a small C++
harness is compiled with g++ and run on random and edge-case values."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "s2let_gb300", "csrc")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "dfconv.h"
using namespace s2g;
int main() {
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-300, 300);
  double worst_split = 0, worst_join = 0;
  long flushed_wrong = 0, bad_norm = 0;
  for (int i = 0; i < 2000000; ++i) {
    double v = std::ldexp(u(g), ex(g));
    if (i % 97 == 0) v = 0.0;
    int emax = exp_field(v) + (i % 5 == 0 ? (i % 200) : 0);  // block max at or above v
    int e = block_scale(emax);
    float hi, lo;
    split_scaled(v, e, hi, lo);
    double s = std::ldexp(v, -e);
    if (!(std::fabs(s) < 1.0)) return 2;
    double back = (double)hi + (double)lo;
    if (std::fabs(s) >= std::ldexp(1.0, -126)) {
      // guarantee: |error| <= max(2^-47 |s|, 2^-126) relative to the block maximum 1
      double err = std::fabs(back - s) / std::fmax(std::ldexp(std::fabs(s), -47), std::ldexp(1.0, -126));
      if (err > worst_split) worst_split = err;
      if (std::fabs(lo) > std::ldexp(std::fabs((double)hi), -24)) ++bad_norm;
      double j = join_scaled(hi, lo, e);
      double ej = std::fabs(std::ldexp(j - v, -e)) / std::fmax(std::ldexp(std::fabs(s), -47), std::ldexp(1.0, -126));
      if (ej > worst_join) worst_join = ej;
    } else if (std::fabs(s) > 0 && back != 0.0 && std::fabs(back - s) > std::ldexp(1.0, -126)) {
      ++flushed_wrong;
    }
  }
  // exact widening of normal floats
  for (int k = -40; k <= 40; ++k)
    for (float x : {1.0f, -1.5f, 3.1415927f, 1.1754944e-38f, 3.4e38f})
      if (widen_scaled(x, k) != std::ldexp((double)x, k)) return 3;
  std::printf("%.6f %.6f %ld %ld\n", worst_split, worst_join, flushed_wrong, bad_norm);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_dfconv_round_trip(tmp_path):
    src = tmp_path / "h.cpp"
    exe = tmp_path / "h"
    src.write_text(HARNESS)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.returncode
    ws, wj, flushed_wrong, bad_norm = out.stdout.split()
    # 24 + 24 significant bits: |error| <= max(2^-47 |v 2^-e|, 2^-126), the
    # floor being where the low word leaves the float normal range
    assert float(ws) <= 1.0 and float(wj) <= 1.0
    assert int(flushed_wrong) == 0 and int(bad_norm) == 0


DIGITS = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "dfconv.h"
using namespace s2g;
int main() {
  std::mt19937_64 g(11);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-200, 200);
  double worst = 0.0;
  long big = 0, inexact = 0;
  for (int it = 0; it < 2000000; ++it) {
    double v = std::ldexp(u(g), ex(g));
    if (it % 101 == 0) v = 0.0;
    const int emax = exp_field(v) + (it % 7 == 0 ? it % 50 : 0);  // column maximum at or above v
    const int e = block_scale(emax);
    uint32_t d[7];
    split_digits_fp32<7>(v, e, d);
    long double acc = 0.0L;
    for (int j = 0; j < 7; ++j) {
      const uint32_t b = d[j] << 16;
      float f;
      std::memcpy(&f, &b, 4);
      if (std::fabs(f) > 64.0f) ++big;
      if (f != std::nearbyint(f)) ++inexact;
      acc += (long double)f * std::pow(2.0L, -6 - 7 * j);
    }
    const double err = (double)std::fabs(acc - std::ldexp((long double)v, -e));
    if (err > worst) worst = err;
  }
  std::printf("%.6e %ld %ld\n", worst, big, inexact);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_fp32_digit_split(tmp_path):
    """split_digits_fp32 (the coefficient slicing of the tensor-core
    contraction): 7 balanced base-128 digits, each an integer of magnitude
    <= 64 exactly held by its bf16 pattern, reconstructing v 2^-e to 2^-47."""
    src = tmp_path / "d.cpp"
    exe = tmp_path / "d"
    src.write_text(DIGITS)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.returncode
    worst, big, inexact = out.stdout.split()
    assert int(big) == 0 and int(inexact) == 0
    assert float(worst) <= 2.0 ** -47
