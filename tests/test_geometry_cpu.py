"""Launch geometry checked on the host before any GPU run: for every grid the
workloads and tests use (and every autotune candidate), the shared memory, thread
counts and tilings that the kernels assume hold.  The geometry code is the
library's own header, compiled here with nvcc as host code (no GPU needed)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

HARNESS = r"""
#include <cstdio>
#include "pfdd_launch.h"
using namespace pfdd;
static int bad = 0, checked = 0;
// threads per line as the kernels compute it: 16 values per thread for lines
// of 16, 128 and 256 in the strided passes, the FP64 z-pass and the FP32
// x-pass (whose compiled-in lengths are 32..256), else 8; lines shorter than
// that: one thread.  kind: 0 strided, 1 z-pass, 2 x-pass.
static int team_of(int L, int kind, size_t vs) {
  bool nv16 = L == 16 || L == 128 || L == 256;
  if (kind == 1 && vs == 8) nv16 = false;
  if (kind == 2 && (vs == 16 || L == 16)) nv16 = false;
  const int nv = nv16 ? 16 : 8;
  return L < nv ? 1 : L / nv;
}
#define CHECK(c, what) do { if (!(c)) { ++bad; std::printf("FAIL %s n=%dx%dx%d ns=%d v=%zu b=%zu\n", what, n1, n2, n3, ns, vs, bs); } } while (0)
static void z_ok(const Geometry &g, int n1, int n2, int n3, int ns, size_t vs, size_t bs) {
  const int team = team_of(n3, 1, vs);
  CHECK((g.zTL & (g.zTL - 1)) == 0 && g.zTL <= n1 && n1 % g.zTL == 0, "z lines");
  CHECK(g.zThreads == g.zTL * team && g.zThreads <= kThreads, "z threads");
  CHECK(g.zSmem <= kMaxDynSmem && g.zPitch >= n3 + 1, "z smem/pitch");
  CHECK((long long)g.zNparts * g.zTL == (long long)n1 * n2, "z parts");
}
static void y_ok(const Geometry &g, int n1, int n2, int n3, int ns, size_t vs, size_t bs) {
  const long long inner = (long long)n3 * n1;
  const int team = team_of(n2, 0, vs);
  const int TI = 1 << g.lgTI[0];
  CHECK(TI <= inner && inner % TI == 0 && g.tiles[0] * TI == inner, "y tiles");
  CHECK(g.threads[0] == TI * team && g.threads[0] <= kThreads && g.smem[0] <= kMaxDynSmem, "y threads/smem");
}
static void x_ok(const Geometry &g, int n1, int n2, int n3, int ns, size_t vs, size_t bs) {
  const int team = team_of(n1, 2, vs);
  const int cap = vs == 16 ? 256 : 384;
  CHECK(g.xTiles << g.xLgT == (long long)n2 * n3, "x tiles");
  CHECK(g.xThreads >= team && g.xThreads % team == 0 && g.xThreads <= cap, "x threads");
  CHECK(g.xSmem == (g.xWarp ? xw_smem(ns, ilog2(n1), g.xLgT, bs) : x_fused_smem(ns, n1, g.xLgT, g.xPitch, vs, bs)) &&
            g.xSmem <= kMaxDynSmem, "x smem");
}
int main() {
  const int sizes[][3] = {{8, 8, 8}, {16, 16, 16}, {32, 32, 32}, {64, 64, 64}, {128, 128, 128}, {256, 256, 256},
                          {8, 16, 32}, {32, 2, 32}, {16, 8, 32}, {32, 16, 64}, {8, 16, 16}, {16, 8, 16}, {16, 16, 32},
                          {512, 8, 8}, {8, 8, 512}, {4, 4, 4}, {2, 64, 2}, {16, 1, 16}, {1, 16, 32}, {16, 16, 1},
                          {2, 4, 8}, {512, 2, 2}, {2, 2, 512}, {1, 1, 1}, {32, 8, 16}, {16, 32, 8}, {32, 16, 8}};
  const size_t vb[3][2] = {{16, 8}, {8, 4}, {8, 0}};
  for (auto &sz : sizes)
    for (int ns : {1, 3, 12})
      for (auto &p : vb) {
        const int n1 = sz[0], n2 = sz[1], n3 = sz[2];
        const size_t vs = p[0], bs = p[1];
        if (bs == 0 && (n1 < 32 || n1 > 256)) continue;  // the on-the-fly form's range
        Geometry g = make_geometry(n1, n2, n3, ns, vs, bs, true);
        const bool expect_fit = x_fused_smem(ns, n1, 0, line_pitch(n1), vs, bs) <= kMaxDynSmem;
        CHECK(g.valid == expect_fit, "validity");
        if (vs == 8 && bs == 4) {  // the FP32 stored-table form: mirrored tile table
          const long long tiles = (long long)make_tile_table(n1, n2, n3, ns * (ns + 1) / 2, true).tiles.size();
          Geometry t = make_geometry(n1, n2, n3, ns, vs, bs, true, tiles);
          const bool fit = x_fused_smem(ns, n1, 0, line_pitch(n1), vs, bs, true) <= kMaxDynSmem;
          CHECK(t.valid == fit && (!fit || (t.xTable && t.xLgT <= 1)), "table validity");
          if (t.valid) {
            CHECK(t.xTiles == (t.xLgT == 1 ? tiles : (long long)n2 * n3), "table tiles");
            CHECK(t.xSmem == x_fused_smem(ns, n1, t.xLgT, t.xPitch, vs, bs, true), "table smem");
            for (int lg = 0; lg <= 1; ++lg)
              for (bool warp : {false, true}) {
                Geometry h = t;
                if (!set_x_geometry(h, n1, n2, n3, ns, vs, bs, lg, false, warp, tiles)) continue;
                CHECK(h.xTable && h.xSmem <= kMaxDynSmem && h.xThreads % 32 == 0 && h.xThreads <= 384, "table x");
                CHECK(h.xSmem == (warp ? xw_smem(ns, ilog2(n1), lg, bs, true)
                                       : x_fused_smem(ns, n1, lg, h.xPitch, vs, bs, true)), "table x smem");
                CHECK(!h.xSplit, "split only when asked");
                // the warp-team kernel with its B block in two halves: half the pair
                // rows (rounded up) in shared memory, at most one point a thread
                Geometry hs = t;
                if (warp && set_x_geometry(hs, n1, n2, n3, ns, vs, bs, lg, false, true, tiles, true)) {
                  const size_t P = (size_t)ns * (ns + 1) / 2;
                  CHECK(hs.xSplit && hs.xWarp && ns >= 2 && (n1 << lg) <= hs.xThreads, "split x");
                  CHECK(hs.xSmem == xw_smem(ns, ilog2(n1), lg, bs, true, true) &&
                        hs.xSmem == h.xSmem - (P / 2) * (size_t)(n1 + 4) * bs, "split smem");
                  CHECK(((P / 2) * (size_t)(n1 + 4) * bs) % 16 == 0, "split halves on 16-byte boundaries");
                }
              }
          }
        }
        if (!g.valid) continue;
        ++checked;
        z_ok(g, n1, n2, n3, ns, vs, bs); y_ok(g, n1, n2, n3, ns, vs, bs); x_ok(g, n1, n2, n3, ns, vs, bs);
        const int cap = (int)std::min<long long>((long long)n1 * n2, (long long)g.zNparts * 4);
        for (int lg = 0; lg <= 5; ++lg) {
          Geometry h = g;
          if (set_z_geometry(h, n1, n2, n3, vs, 1 << lg) && h.zNparts <= cap) z_ok(h, n1, n2, n3, ns, vs, bs);
          h = g;
          if (set_x_geometry(h, n1, n2, n3, ns, vs, bs, lg, false, true)) {  // warp-team x-pass
            x_ok(h, n1, n2, n3, ns, vs, bs);
            CHECK(vs == 8 && n1 >= 32 && n1 <= 256 && h.xWarp, "x warp form");
            CHECK(h.xSmem == xw_smem(ns, ilog2(n1), h.xLgT, bs) && h.xPitch == xw_pitch(ilog2(n1)) &&
                  h.xThreads % 32 == 0, "x warp smem/pitch/threads");
          }
          for (bool wide : {false, true}) {
            h = g;
            if (set_x_geometry(h, n1, n2, n3, ns, vs, bs, lg, wide)) x_ok(h, n1, n2, n3, ns, vs, bs);
          }
        }
        for (int lg = 0; lg <= 7; ++lg) {
          Geometry h = g;
          if (set_strided_geometry(h, 0, n2, (long long)n3 * n1, lg, vs)) y_ok(h, n1, n2, n3, ns, vs, bs);
        }
      }
  std::printf("%d %d\n", checked, bad);
  return 0;
}
"""


def test_launch_geometry_invariants(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    src = tmp_path / "geom.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "geom"
    subprocess.run([nvcc, "-std=c++17", "-O1", "-I", str(ROOT / "pfdd_gb300" / "csrc"), "-I", str(ROOT / "include"),
                    str(src), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    *fails, last = out.strip().splitlines()
    checked, bad = map(int, last.split())
    assert bad == 0, fails[:20]
    assert checked > 100
