"""The Stockham radix plans of pfdd_gb300/csrc/pfdd_fft.cuh (8 and 16 values per
thread, both signs, L = 8..512), run on the host stage by stage with the
kernels' own stage function and checked against a direct DFT in long double.

Each stage reads every team thread's values before any thread writes, as the
block barrier between a stage's reads and its in-place writes does on the GPU."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>
#include "pfdd_fft.cuh"
using namespace pfdd;

template <typename V, int S, int NV>
static double run(int lgL, std::mt19937_64 &rng) {
  using T = decltype(V{}.x);
  const int L = 1 << lgL, lgNV = NV == 16 ? 4 : 3, LV = L >> lgNV;
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::vector<V> line(L), tw(L);
  std::vector<long double> re(L), im(L);
  for (int i = 0; i < L; ++i) {
    line[i].x = (T)u(rng); line[i].y = (T)u(rng);
    re[i] = line[i].x; im[i] = line[i].y;
    const long double ang = -2.0L * 3.14159265358979323846264338327950288L * i / L;
    tw[i].x = (T)std::cos(ang); tw[i].y = (T)std::sin(ang);
  }
  const int nst = stockham_stages(lgL, NV);
  std::vector<V> regs((size_t)LV * NV);
  for (int st = 0; st < nst; ++st) {
    for (int th = 0; th < LV; ++th)
      for (int m = 0; m < NV; ++m) regs[(size_t)th * NV + m] = line[th + m * LV];
    for (int th = 0; th < LV; ++th)
      stockham_plan_stage<S, NV>(&regs[(size_t)th * NV], th, lgL, st, tw.data(),
                                 [&](int l) { return &line[l]; });
  }
  double err = 0.0, mag = 0.0;
  for (int k = 0; k < L; ++k) {
    long double sr = 0, si = 0;
    for (int n = 0; n < L; ++n) {
      const long double ang = S * 2.0L * 3.14159265358979323846264338327950288L * (long double)((long long)n * k % L) / L;
      sr += re[n] * std::cos(ang) - im[n] * std::sin(ang);
      si += re[n] * std::sin(ang) + im[n] * std::cos(ang);
    }
    err = std::fmax(err, (double)std::fabs(sr - line[k].x));
    err = std::fmax(err, (double)std::fabs(si - line[k].y));
    mag = std::fmax(mag, (double)std::fabs(sr));
  }
  return err / mag;
}

int main() {
  std::mt19937_64 rng(7);
  for (int lgL = 3; lgL <= 9; ++lgL) {
    double e[8] = {run<double2, -1, 8>(lgL, rng), run<double2, 1, 8>(lgL, rng),
                   lgL >= 4 ? run<double2, -1, 16>(lgL, rng) : 0.0, lgL >= 4 ? run<double2, 1, 16>(lgL, rng) : 0.0,
                   run<float2, -1, 8>(lgL, rng), run<float2, 1, 8>(lgL, rng),
                   lgL >= 4 ? run<float2, -1, 16>(lgL, rng) : 0.0, lgL >= 4 ? run<float2, 1, 16>(lgL, rng) : 0.0};
    printf("%d", lgL);
    for (double v : e) printf(" %.3e", v);
    printf("\n");
  }
  return 0;
}
"""


def test_stockham_radix_plans_match_dft(tmp_path):
    src = tmp_path / "plan.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "plan"
    subprocess.run(["nvcc", "-std=c++17", "-O2", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", str(ROOT / "pfdd_gb300" / "csrc"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [list(map(float, r.split())) for r in out if r.strip()]
    assert [int(r[0]) for r in rows] == list(range(3, 10))
    for r in rows:
        fp64, fp32 = r[1:5], r[5:9]
        assert max(fp64) < 2e-15, r   # max error relative to the largest output
        assert max(fp32) < 1e-6, r
