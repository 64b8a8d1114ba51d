// pfdd_launch.h -- host launchers of the templated kernels.  Each kernel is
// instantiated for every power-of-two line length it runs (log2 L known at
// compile time) in its own translation unit, so the build compiles in
// parallel: pfdd_fftpass.cu (z-pass, strided passes), pfdd_xpass_f32.cu and
// pfdd_xpass_f64.cu (fused x-pass).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "pfdd_kernels.cuh"

namespace pfdd {
// z-pass for lgL in [0, 9]; prec 0 = FP64 spectra, 1 = FP32; nv: values a
// thread (8, or 16 for lgL >= 4; 0: zpass_nv)
cudaError_t launch_zpass(int prec, int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                         const ZParams &p, int nv = 0);
// strided line FFT (sign -1 forward, +1 inverse) for lgL in [0, 9]; nv as
// launch_zpass (0: fft_nv)
cudaError_t launch_strided(int prec, int sign, int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                           void *data, int lgTI, long long inner, long long tiles_per_outer, const void *tw,
                           const uint8_t *active, long long outer_per_rep, int pitch, bool rev = false, int nv = 0);
// fused x-pass (x-forward FFT, contraction, x-inverse FFT) for ns in [1, 12]
cudaError_t launch_x_fused_f32(int ns, unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p);
cudaError_t launch_x_fused_f64(int ns, unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p);
// FP32 x-pass evaluating B(k) in registers, N1 in [32, 256]
cudaError_t launch_x_fused_f32_bfly(int ns, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                                    const XParams &p);
// warp-team FP32 x-pass (stored or register-evaluated B(k)), N1 in [32, 256]
cudaError_t launch_x_warp_f32(int ns, bool bfly, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                              const XParams &p);


// Launch geometry of the z-pass, the strided passes and the fused x-pass for one
// grid (ns = 0: FFT-boundary plans without the x-pass).  Sizes: powers of two <= 512.
constexpr int kThreads = 256;

inline bool pow2_ok(int n) { return n >= 1 && n <= 512 && (n & (n - 1)) == 0; }

inline int ilog2(long long v) {
  int l = 0;
  while ((1LL << l) < v) ++l;
  return l;
}

// threads per line (team) of the strided passes and the z-pass, which have
// every line length compiled in, and of the fused x-pass, which has N1 =
// 32..256 compiled in and runs other lengths with 8 values per thread
inline int line_team(int L, int nv = 0) { return L / std::min(nv ? nv : fft_nv(ilog2(L)), L); }
inline int z_line_team(int L, size_t vsize, int nv = 0) {
  return L / std::min(nv ? nv : zpass_nv(ilog2(L), (int)vsize), L);
}
// the radix plans a line of L can run: 8 values a thread, and 16 from L = 16 on
inline bool nv_ok(int L, int nv) { return nv == 0 || nv == 8 || (nv == 16 && L >= 16); }
inline int x_line_team(int n1, size_t vsize) {
  const int lg = ilog2(n1);
  return n1 / std::min(lg >= 5 && lg <= 8 ? xpass_nv(lg, (int)vsize) : 8, n1);
}

// dynamic shared memory a kernel may opt into (227 KB per block on GB300,
// less the kernels' few hundred bytes of static shared memory)
constexpr size_t kMaxDynSmem = 226 * 1024;

struct Geometry {
  bool valid = true;  // false: the fused x-pass tile of this grid does not fit
  // spectral layout of a context's S: x fastest ([y][z][x] per field); the
  // FFT-boundary plans keep the natural [x][y][z]
  bool xfast = false;
  // z-pass; zNV: values a thread (the radix plan; 0: zpass_nv)
  int zTL = 1, zThreads = 1, zPitch = 1, zNparts = 1, lgL3 = 0, zNV = 0;
  size_t zSmem = 0;
  // strided passes (y: axis 1, x: axis 0; x only in the FFT-boundary plans);
  // nv: values a thread (0: fft_nv)
  int lgTI[2] = {0, 0}, threads[2] = {1, 1}, pitch[2] = {1, 1}, nv[2] = {0, 0};
  long long tiles[2] = {1, 1};
  size_t smem[2] = {0, 0};
  // fused x-pass; xWarp: the warp-team kernel (x_warp_kernel); xTable: the
  // B(k) tile-table layout (see BLayout), xTiles then the table's tile count
  int xLgT = 0, xPitch = 1, xThreads = 256;
  // xSplit (warp teams on the tile table): the tile's B block arrives in two
  // halves of its pair rows through one buffer of half the size
  bool xWide = false, xWarp = false, xTable = false, xSplit = false;
  long long xTiles = 1;
  size_t xSmem = 0;
};

inline int line_pitch(int L) { return L + 1; }  // odd pitch: lanes on different lines hit different banks

// Pitch of the z-pass lines, whose consecutive lanes walk TL lines and then the
// next position of the same lines.  A shared-memory phase serves 128 bytes,
// i.e. u = 128 / vsize lanes; with TL >= u they all sit on different lines and
// an odd pitch spreads them, with TL < u each line holds u / TL consecutive
// lanes and a pitch of u / TL (mod u) puts the lines side by side.
inline int z_line_pitch(int L, int TL, size_t vsize) {
  const int u = (int)(128 / vsize);
  return TL >= u ? L + 1 : L + u / TL;
}

// z-pass with TL lines per block (the x-fastest layout needs TL <= N1) and nv
// values a thread (0: the default radix plan).
inline bool set_z_geometry(Geometry &g, int n1, int n2, int n3, size_t vsize, int TL, int nv = 0) {
  if (!nv_ok(n3, nv)) return false;
  const int L3 = n3, team3 = z_line_team(L3, vsize, nv);
  const long long lines = (long long)n1 * n2;
  if (TL < 1 || TL > lines || (g.xfast && TL > n1) || (long long)TL * team3 > kThreads) return false;
  g.zNV = nv;
  g.zTL = TL;
  g.zThreads = TL * team3;
  g.zPitch = z_line_pitch(L3, TL, vsize);
  g.zNparts = (int)(lines / TL);
  // twiddles + padded S lines (16-byte aligned) + FP64 xi tile
  g.zSmem = ((((size_t)L3 + (size_t)TL * g.zPitch) * vsize + 15) & ~(size_t)15) + (size_t)TL * L3 * 16;
  g.lgL3 = ilog2(L3);
  return g.zSmem <= kMaxDynSmem;
}

// Strided pass along axis ax (0: y, 1: x) with TI = 2^lgTI columns per tile
// and nv values a thread (0: the default radix plan).
inline bool set_strided_geometry(Geometry &g, int ax, int L, long long inner, int lgTI, size_t vsize, int nv = 0) {
  if (!nv_ok(L, nv)) return false;
  const int team = line_team(L, nv);
  const int TI = 1 << lgTI;
  if (TI > inner || (long long)TI * team > kThreads) return false;  // fft_strided_kernel launch bounds
  g.nv[ax] = nv;
  g.lgTI[ax] = lgTI;
  g.threads[ax] = TI * team;
  g.pitch[ax] = TI >= 8 ? TI + 1 : TI;
  g.tiles[ax] = inner / TI;
  g.smem[ax] = ((size_t)L + (size_t)L * g.pitch[ax]) * vsize;
  return g.smem[ax] <= kMaxDynSmem;
}

// Fused x-pass with tiles of T = 2^lgT inner indices (all N1 x, all ns fields,
// the tile's B(k)).  False when the tile does not fit.
// wide: enough threads that the lines of a tile fill whole shared-memory
// phases (16 lanes of 8 bytes, 8 of 16 bytes), i.e. every phase of an FFT
// stage touches as many different lines as it has lanes (no bank conflicts),
// at the price of idle threads when the tile has fewer lines.
// table_tiles > 0: the tile-table layout with that many tiles (T = 2: a CTA
// per tile, T = 1: a CTA per line).
inline bool set_x_geometry(Geometry &g, int n1, int n2, int n3, int ns, size_t vsize, size_t bsize, int lgT,
                           bool wide = false, bool warp = false, long long table_tiles = 0, bool split = false) {
  const long long innerx = (long long)n2 * n3;
  if ((1LL << lgT) > innerx && table_tiles == 0) return false;
  if (table_tiles > 0 && lgT > 1) return false;
  if (split && (!warp || table_tiles == 0 || ns < 2)) return false;
  if (warp) {  // FP32 spectra, N1 = 32..256; a thread a point, at most 384
    const int lgL = ilog2(n1);
    if (wide || vsize != 8 || n1 < 32 || n1 > 256) return false;
    const size_t smem = xw_smem(ns, lgL, lgT, bsize, table_tiles > 0, split);
    if (smem > kMaxDynSmem) return false;
    const int lpw = 32 / xw_lv(lgL), lines = ns << lgT;
    int thr = std::max(n1 << lgT, (lines + lpw - 1) / lpw * 32);
    thr = std::min(384, (thr + 31) / 32 * 32);
    if (split && (n1 << lgT) > thr) return false;  // the split contraction takes one point a thread
    g.xPitch = xw_pitch(lgL);
    g.xLgT = lgT;
    g.xTiles = table_tiles > 0 ? (lgT == 1 ? table_tiles : innerx) : innerx >> lgT;
    g.xSmem = smem;
    g.xThreads = thr;
    g.xWide = false;
    g.xWarp = true;
    g.xTable = table_tiles > 0;
    g.xSplit = split;
    return true;
  }
  g.xWarp = false;
  g.xSplit = false;
  const int pitch = line_pitch(n1);
  const size_t smem = x_fused_smem(ns, n1, lgT, pitch, vsize, bsize, table_tiles > 0);
  if (smem > kMaxDynSmem) return false;
  const int team = x_line_team(n1, vsize), lines = ns << lgT, npt = n1 << lgT;
  const int unit = std::max(32, team);
  const int cap = vsize == sizeof(double2) ? 256 : 384;  // x_fused_kernel launch bounds
  if (unit > cap) return false;
  const int phase = (int)(128 / vsize);
  const int lines_eff = wide ? (lines + phase - 1) / phase * phase : lines;
  if (wide && (lines_eff == lines || lines_eff * team > cap)) return false;  // nothing to widen / too wide
  int thr = std::min(cap, std::max(npt, lines_eff * team));
  thr = (thr + unit - 1) / unit * unit;
  g.xPitch = pitch;
  g.xLgT = lgT;
  g.xTiles = table_tiles > 0 ? (lgT == 1 ? table_tiles : innerx) : innerx >> lgT;
  g.xTable = table_tiles > 0;
  g.xSmem = smem;
  g.xThreads = std::min(thr, cap / unit * unit);
  g.xWide = wide;
  return true;
}

// ns = 0: no fused x-pass (FFT-boundary plans).  bsize: bytes of a stored B(k)
// value, 0 when the x-pass evaluates B(k) itself.  The strided and x-pass tile
// widths chosen here are the defaults; a context's first step may retune them
// (they do not change any result).
inline Geometry make_geometry(int n1, int n2, int n3, int ns, size_t vsize, size_t bsize, bool xfast = false,
                              long long table_tiles = 0) {
  Geometry g;
  g.xfast = xfast;
  const int L3 = n3, team3 = z_line_team(L3, vsize);
  const long long lines = (long long)n1 * n2;
  int TL = std::max(1, kThreads / team3);
  while ((long long)TL > lines || (xfast && TL > n1)) TL >>= 1;  // x-fastest: a block's lines share y
  set_z_geometry(g, n1, n2, n3, vsize, TL);
  const int Ls[2] = {n2, n1};
  const long long inner[2] = {xfast ? (long long)n3 * n1 : (long long)n3, (long long)n2 * n3};
  for (int ax = 0; ax < 2; ++ax) {
    const int L = Ls[ax], team = line_team(L);
    int TI = std::max(1, kThreads / team);
    while ((long long)TI > inner[ax]) TI >>= 1;
    set_strided_geometry(g, ax, L, inner[ax], ilog2(TI), vsize);
  }
  if (ns > 0) {
    // default x tile: the widest T <= 32 whose tile fits two CTAs per SM (<= 110 KB)
    int lgT = 5;
    while (lgT > 0 && ((1LL << lgT) > (long long)n2 * n3 ||
                       x_fused_smem(ns, n1, lgT, line_pitch(n1), vsize, bsize) > 110 * 1024))
      --lgT;
    // tile table: a CTA per line pair with warp teams (the autotuner's choice at
    // 128^3 x 12), else with block teams, or per line when a pair's tile does not fit
    g.valid = table_tiles > 0 ? (set_x_geometry(g, n1, n2, n3, ns, vsize, bsize, 1, false, true, table_tiles) ||
                                 set_x_geometry(g, n1, n2, n3, ns, vsize, bsize, 1, false, false, table_tiles) ||
                                 set_x_geometry(g, n1, n2, n3, ns, vsize, bsize, 0, false, false, table_tiles))
                              : set_x_geometry(g, n1, n2, n3, ns, vsize, bsize, lgT);
  }
  return g;
}

// B(k) tile table (see BLayout): symmetric: a mirrored tile for each line pair
// (c, m(c)) whose indices j, k are below Nyquist (c != m(c)), single tiles for
// the other lines; otherwise single tiles only.  Offsets in values.
struct TileTable {
  std::vector<int2> tiles;
  std::vector<long long> toff;
  std::vector<int> line_tile, order;  // order: the lines tile by tile
};
inline TileTable make_tile_table(int n1, int n2, int n3, int P, bool symmetric) {
  TileTable t;
  const int inner = n2 * n3;
  t.line_tile.assign(inner, -1);
  const long long ws = (n1 + 3) / 4 * 4, wm = b_wm(n1);
  auto nyq = [](int i, int n) { return i == n / 2; };  // its own mirror, nonzero frequency
  long long off = 0;
  for (int c = 0; c < inner; ++c) {
    if (t.line_tile[c] >= 0) continue;  // the second line of a mirrored tile
    const int j = c / n3, k = c % n3, m = b_mirror(j, n2) * n3 + b_mirror(k, n3);
    const int id = (int)t.tiles.size();
    t.toff.push_back(off);
    if (symmetric && !nyq(j, n2) && !nyq(k, n3) && m != c) {
      t.tiles.push_back(make_int2(c, m));
      t.line_tile[c] = 2 * id;
      t.line_tile[m] = 2 * id + 1;
      t.order.push_back(c);
      t.order.push_back(m);
      off += P * wm;
    } else {
      t.tiles.push_back(make_int2(c, -1));
      t.line_tile[c] = 2 * id;
      t.order.push_back(c);
      off += P * ws;
    }
  }
  t.toff.push_back(off);
  return t;
}

// Launches a step kernel with programmatic dependent launch allowed (see
// griddep_wait): its CTAs may be scheduled while the previous kernel on the
// stream finishes; the kernel orders its dependent reads itself.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned blocks, int threads, size_t smem, cudaStream_t st,
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Per-kernel record of the dynamic shared memory opted into on each device.
// Contexts on different host threads (the server's workers) launch the same
// kernels concurrently, so updates are serialised and only ever raise it.
constexpr int kMaxDevices = 64;
struct SmemOptIn {
  std::mutex mu;
  size_t bytes[kMaxDevices] = {};
};

// opts a kernel into `smem` bytes of dynamic shared memory on the current
// device, once per size increase
template <typename K>
inline cudaError_t ensure_smem(K kernel, size_t smem, SmemOptIn &rec) {
  if (smem <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  std::lock_guard<std::mutex> lk(rec.mu);
  if (smem <= rec.bytes[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) rec.bytes[dev] = smem;
  return e;
}
}  // namespace pfdd
