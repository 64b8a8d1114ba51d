"""The B(k) tile table of the FP32 stored-table form (pfdd_gb300/csrc/pfdd_launch.h,
b_index in pfdd_kernels.cuh), checked on the host for every grid the tests and
workloads use: every line sits in exactly one tile; a mirrored tile pairs a line
with its mirror through the origin and neither has a Nyquist y or z index;
every stored (pair, point) has its own slot inside the allocation; exactly the
second line's non-Nyquist x points are not stored, and their mirror is; every
tile's block starts and ends on a 16-byte boundary; the frequencies of a point
and of its mirror are negatives of each other exactly when the point is not
stored (so B(-f) = B(f) makes the shared slot exact)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

HARNESS = r"""
#include <cstdio>
#include <vector>
#include "pfdd_launch.h"
using namespace pfdd;
static double frec_h(int i, int n) {  // frec with d = 1 (F:2683-2754)
  double v = 0.0;
  if (i >= 1 && i < n / 2) v = (double)i / (double)n;
  if (i >= n / 2) v = ((double)i - (double)n) / (double)n;
  return v;
}
int main() {
  const int sizes[][3] = {{8, 8, 8}, {16, 16, 16}, {32, 32, 32}, {128, 16, 8}, {8, 16, 32}, {32, 2, 32},
                          {16, 8, 32}, {2, 4, 8}, {1, 16, 32}, {16, 1, 16}, {16, 16, 1}, {4, 4, 4}, {2, 64, 2},
                          {1, 1, 1}, {64, 8, 2}};
  long bad = 0, checked = 0;
  for (auto &sz : sizes)
    for (int ns : {1, 3, 12})
      for (bool sym : {true, false}) {
        const int n1 = sz[0], n2 = sz[1], n3 = sz[2], P = ns * (ns + 1) / 2;
        const long long inner = (long long)n2 * n3, N = inner * n1;
        TileTable t = make_tile_table(n1, n2, n3, P, sym);
        const long long total = t.toff.back();
        const long long cap = (long long)P * inner * ((n1 + 3) / 4 * 4);  // the context's allocation
        if (total > cap) ++bad;
        std::vector<int> seen(inner, 0);
        for (size_t i = 0; i < t.tiles.size(); ++i) {
          const int2 tp = t.tiles[i];
          if ((t.toff[i] * 4) % 16 || (t.toff[i + 1] * 4) % 16) ++bad;  // FP32 blocks on 16-byte boundaries
          seen[tp.x]++;
          if (t.line_tile[tp.x] != (int)(2 * i)) ++bad;
          if (tp.y >= 0) {
            seen[tp.y]++;
            if (t.line_tile[tp.y] != (int)(2 * i + 1) || !sym) ++bad;
            const int j = tp.x / n3, k = tp.x % n3;
            if (tp.y != b_mirror(j, n2) * n3 + b_mirror(k, n3) || tp.y == tp.x) ++bad;
            if (j == n2 / 2 || k == n3 / 2) ++bad;
          }
        }
        for (long long c = 0; c < inner; ++c) if (seen[c] != 1) ++bad;
        BLayout bl{N, inner, n1, 1, P, t.tiles.data(), t.toff.data(), t.line_tile.data()};
        std::vector<unsigned char> used(total, 0);
        for (int p = 0; p < P; ++p)
          for (long long pt = 0; pt < N; ++pt) {
            ++checked;
            const long long x = pt / inner, c = pt - x * inner;
            const long long bi = b_index(bl, p, pt);
            const int2 tp = t.tiles[t.line_tile[c] >> 1];
            const bool second = tp.y >= 0 && (t.line_tile[c] & 1);
            const bool nyqx = x == n1 / 2;
            if (bi < 0) {
              if (!second || nyqx) { ++bad; continue; }
              // the stored mirror: frequency -f exactly
              const long long mpt = (long long)b_mirror((int)x, n1) * inner + tp.x;
              if (b_index(bl, p, mpt) < 0) ++bad;
              const int j = (int)(c / n3), k = (int)(c % n3), mj = (int)(tp.x / n3), mk = (int)(tp.x % n3);
              if (frec_h((int)x, n1) != -frec_h(b_mirror((int)x, n1), n1) || frec_h(j, n2) != -frec_h(mj, n2) ||
                  frec_h(k, n3) != -frec_h(mk, n3)) ++bad;
              continue;
            }
            if (second && !nyqx) ++bad;
            if (bi >= total) { ++bad; continue; }
            if (used[bi]++) ++bad;  // two (pair, point) in one slot
          }
      }
  std::printf("%ld %ld\n", checked, bad);
  return 0;
}
"""


def test_b_tile_table(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    src = tmp_path / "bt.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "bt"
    subprocess.run([nvcc, "-std=c++17", "-O2", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", str(ROOT / "pfdd_gb300" / "csrc"), "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True)
    checked, bad = map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split())
    assert checked > 1_000_000
    assert bad == 0
