"""The integer-pipe binary64 <-> binary32 conversions used by the FP32-FFT form's
update (pfdd_gb300/csrc/pfdd_convert.cuh), compiled for the host and checked
against the C compiler's own IEEE conversions on 2M random patterns plus edge cases."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

HARNESS = r"""
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <random>
#include "pfdd_convert.cuh"
using namespace pfdd;

static uint64_t db(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static uint32_t fb(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static double mkd(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static float mkf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

int main() {
  std::mt19937_64 rng(12345);
  long bad = 0, checked = 0;
  // binary32 -> binary64: every normal float converts exactly
  for (int i = 0; i < 1000000; ++i) {
    uint32_t u = (uint32_t)rng();
    float f = mkf(u);
    uint32_t e = (u >> 23) & 0xff;
    if (e == 0 || e == 0xff) continue;
    ++checked;
    if (db(f32_to_f64_int(f)) != db((double)f)) ++bad;
  }
  // binary64 -> binary32 within the normal float range, including exact ties
  for (int i = 0; i < 1000000; ++i) {
    uint64_t m = rng() & 0xfffffffffffffull;
    if (i % 4 == 0) m = (m & ~0x1fffffffull) | (1ull << 28);  // tie: half an ulp exactly
    int e = 1023 - 126 + (int)(rng() % 253);
    uint64_t s = (rng() & 1) ? (1ull << 63) : 0;
    double d = mkd(s | ((uint64_t)e << 52) | m);
    float ref = (float)d;
    if (!std::isfinite(ref) || std::fabs(ref) < FLT_MIN) continue;
    ++checked;
    if (fb(f64_to_f32_int(d)) != fb(ref)) ++bad;
  }
  // edge cases
  int edge = 0;
  edge += fb(f64_to_f32_int(0.0)) != 0u;
  edge += fb(f64_to_f32_int(-0.0)) != 0x80000000u;
  edge += fb(f64_to_f32_int(1e300)) != 0x7f800000u;
  edge += fb(f64_to_f32_int(-1e300)) != 0xff800000u;
  edge += fb(f64_to_f32_int(1e-300)) != 0u;
  edge += !std::isnan(f64_to_f32_int(NAN));
  edge += !std::isinf(f64_to_f32_int(INFINITY));
  edge += db(f32_to_f64_int(0.0f)) != 0u;
  edge += db(f32_to_f64_int(-0.0f)) != (1ull << 63);
  edge += !std::isnan(f32_to_f64_int(NAN));
  edge += f32_to_f64_int(-INFINITY) != -INFINITY;
  edge += f32_to_f64_int(1e-45f) != 0.0;  // subnormal input flushes
  edge += f64_to_f32_int((double)FLT_MAX) != FLT_MAX;
  edge += f64_to_f32_int(1.0 + 1e-9) != 1.0f;
  // the 32-bit-word short paths agree with the general functions on every
  // pattern class (random bits across all exponents, ties, zeros, Inf/NaN)
  long fastbad = 0;
  for (int i = 0; i < 1000000; ++i) {
    uint64_t u = rng();
    if (i % 3 == 0) u = (u & ~0x7ff0000000000000ull) | ((uint64_t)(880 + rng() % 290) << 52);
    if (i % 7 == 0) u = (u & ~0x1fffffffull) | (1ull << 28);
    if (fb(f64bits_to_f32_fast(u)) != fb(f64bits_to_f32_int(u))) ++fastbad;
    uint32_t w = (uint32_t)rng();
    if (f32_to_f64bits_fast(mkf(w)) != f32_to_f64bits_int(mkf(w))) ++fastbad;
  }
  for (uint64_t u : std::initializer_list<uint64_t>{0ull, 1ull << 63, 0x7ff0000000000000ull, 0xfff8000000000001ull,
                                                    db(FLT_MAX), db(FLT_MIN), db((double)FLT_MAX * (1 + 1e-9)), db(1.0)})
    if (fb(f64bits_to_f32_fast(u)) != fb(f64bits_to_f32_int(u))) ++fastbad;
  printf("%ld %ld %d %ld\n", checked, bad, edge, fastbad);
  return 0;
}
"""


def test_integer_conversions_match_ieee(tmp_path):
    src = tmp_path / "conv.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "conv"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "pfdd_gb300" / "csrc"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    checked, bad, edge, fastbad = map(int, out)
    assert checked > 1_500_000
    assert bad == 0
    assert edge == 0
    assert fastbad == 0
