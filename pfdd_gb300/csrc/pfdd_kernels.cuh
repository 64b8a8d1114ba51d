// pfdd_kernels.cuh -- kernels of the PFDD TDGL step (any power-of-two grid,
// FP64 or FP32 spectral precision).
//
// Device data (N = N1*N2*N3, R replicas, ns slip systems):
//   xi   double2 [R][ns][N]   order parameter, FP64 state (F:4146), [x][y][z]
//   S    T2      [R][ns][N]   spectral work buffer (T = double or float), in a
//                step's context x fastest: [y][z][x] per field
//   B    T       packed symmetric B(k), P = ns(ns+1)/2 pairs a <= b in
//                row-major order, stored in the tile order of the fused
//                x-pass (see BLayout) so each tile streams one contiguous block
//   bc   uint32  bit mask     bit (r*ns+a)*N+pt set = pinned (xi_bc != 0)
//
// One TDGL step is four launches:
//   y-forward FFT, x-pass (x-forward FFT -> B(k) contraction -> x-inverse FFT),
//   y-inverse FFT, z-pass (z-inverse FFT -> Euler update + gamma partials ->
//   z-forward FFT of the new state).
// S therefore holds the (y,z)-transformed state between steps.
#pragma once
#include <climits>
#include <type_traits>

#include "pfdd_convert.cuh"
#include "pfdd_fft.cuh"
#include "pfdd_tma.cuh"

namespace pfdd {

constexpr int kMaxNs = 16;
constexpr double kPiTrunc = 3.141592654;  // PFDD_Final_GPU.c:95
// sin(2 * pi_trunc * x) = sinpi(x * kTwoPiTruncOverPi)
constexpr double kTwoPiTruncOverPi = 2.0 * 3.141592654 / 3.14159265358979323846;

// z-pass stages: load (S, or xi with Z_SRC_XI) -> [inverse z FFT] -> [update]
// -> [forward z FFT] -> [store S]
enum ZFlags { Z_INV = 1, Z_UPDATE = 2, Z_FWD = 4, Z_SRC_XI = 8, Z_STORE = 16 };

struct ZParams {
  void *S;
  double2 *xi;
  const uint32_t *bc;
  const double *tau;        // [step][R][ns]: tau/dslip (no field) or ramp multiplier (field)
  const double *tau_field;  // [ns][N] or null
  const double *dslip;      // [ns] (field mode)
  long long *part;          // [step][R*ns][nparts] exact fixed-point partial sums (LLONG_MIN: overflow)
  const uint8_t *active;    // [R] or null
  const void *tw;           // forward twiddles of length L
  int *err;                 // set when a bounded wait times out (may be null)
  const int *step_ctr;      // step index within the chunk, advanced by the x-pass (null: use `step`)
  long long N, lines_per_field;
  int step, L, lgL, ns, R, TL, nparts, flags, pitch;
  // S layout: 0 = natural [x][y][z] (z fastest, like xi); 1 = x fastest,
  // [y][z][x] per field (the step's spectral buffer).  With 1 a block takes the
  // TL lines (x0..x0+TL-1, y) and n1, n2, lgTL describe the grid.
  int sxf, n1, n2, lgTL;
  double inv_n, uq2;
  double cd2[kMaxNs], asf_pi[kMaxNs], uq2cd2[kMaxNs];
};

template <typename V> __device__ __forceinline__ V from_xi(double2 x);
template <> __device__ __forceinline__ double2 from_xi<double2>(double2 x) { return x; }
template <> __device__ __forceinline__ float2 from_xi<float2>(double2 x) {
  return make_float2(f64_to_f32_int(x.x), f64_to_f32_int(x.y));
}

// plasticevolv (F:3470-3501) for one point, plain FP64 form: the reference's
// expression in double precision (pi truncated as F:95).
__device__ __forceinline__ void tdgl_point(double2 &x, double2 f, double cd2, double asf_pi, double uq2,
                                           double uq2cd2, double ctau, double inv_n) {
  const double s = sinpi(x.x * kTwoPiTruncOverPi);
  x.x = x.x - cd2 * (uq2 * f.x * inv_n + asf_pi * s - ctau);
  x.y = x.y - uq2cd2 * (f.y * inv_n);
}
// FP32-FFT form (inlined in the z-pass): the increment -- force, core term
// on the FP32-rounded state, stress -- is evaluated in FP32, then subtracted
// from the FP64 state; the FP64 <-> FP32 conversions run on the integer pipe.

template <typename T> struct UpdCoef;
template <> struct UpdCoef<double> {
  double cd2, asf_pi, uq2, uq2cd2, inv_n;
  __device__ UpdCoef(const ZParams &p, int a) : cd2(p.cd2[a]), asf_pi(p.asf_pi[a]), uq2(p.uq2), uq2cd2(p.uq2cd2[a]),
                                                inv_n(p.inv_n) {}
  __device__ double tau(double t) const { return t; }
};
template <> struct UpdCoef<float> {
  float cd2, asf_pi, uq2, uq2cd2, inv_n;
  __device__ UpdCoef(const ZParams &p, int a)
      : cd2((float)p.cd2[a]), asf_pi((float)p.asf_pi[a]), uq2((float)p.uq2), uq2cd2((float)p.uq2cd2[a]),
        inv_n((float)p.inv_n) {}
  __device__ float tau(double t) const { return (float)t; }
};

// Exact accumulation of FP64 values in 64-bit fixed point with 2^-44
// resolution, on the integer pipe (FP64 adds run at 1/58 of the FP32 rate on
// GB300).  round(d * 2^44) is formed from the bit pattern; |d| must stay below
// 2^7 so that the 2048 values of one block cannot overflow (anything larger,
// or non-finite, raises `big`, which the caller turns into a NaN partial: the
// divergence watchdog).  The sums are exact, hence independent of the order.
constexpr int kFixBits = 44;
__device__ __forceinline__ long long to_fixed_bits(unsigned long long u, bool &big) {
  const int e = (int)((u >> 52) & 0x7ff);
  if (e >= 1023 + 7) { big = true; return 0; }
  const int sh = 1075 - kFixBits - e;  // |d| = m * 2^(e-1075) = (m >> sh) units of 2^-44; >= 2 here
  if (sh >= 64) return 0;               // includes e == 0
  const unsigned long long m = (u & 0xfffffffffffffull) | (1ull << 52);
  const long long v = (long long)((m + (1ull << (sh - 1))) >> sh);
  return (u >> 63) ? -v : v;
}
__device__ __forceinline__ long long to_fixed(double d, bool &big) {
  return to_fixed_bits((unsigned long long)__double_as_longlong(d), big);
}

__device__ __forceinline__ long long block_sum_i64(long long v, long long *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  long long s = 0;
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int i = 0; i < nw; ++i) s += red[i];
  }
  return s;
}

// The FP32-FFT form's Euler update of one z-pass tile (TL lines of L = 2^LG,
// nel = TL*L points, element e = line * L + z): the force from the FP32
// spectrum sm (line pitch P), the FP64 state from xsb (the tile in shared
// memory, as bit patterns).  Writes the evolved state to xg (the field's xi)
// and its FP32 copy back to sm; returns the tile's exact fixed-point sum of
// Re xi (big: see to_fixed_bits).  The FP64 state stays in integer registers;
// FP64 arithmetic is exactly the two subtractions (the compiler otherwise
// routes 64-bit register moves through the FP64 pipe).  kGeneral: pinned
// points or a stress field (read per point); otherwise every point evolves
// under the tile's one stress value.
template <bool kGeneral, int LG>
__device__ __forceinline__ long long update_tile_f32(const ZParams &p, const UpdCoef<float> &k, float ctau0, double tv,
                                                     int a, long long fbase, int lb, int ls, int nel, int P,
                                                     float2 *sm, const ulonglong2 *xsb, ulonglong2 *xg, bool &big) {
  constexpr int L = 1 << LG;
  long long acc = 0;
#pragma unroll 1  // measured: 261 us against 277 (unroll 2), 280 (4), 288 (8) at 128^3 x 12
  for (int e = threadIdx.x; e < nel; e += blockDim.x) {
    float2 *sp = &sm[(e >> LG) * P + (e & (L - 1))];
    ulonglong2 xb = xsb[e];
    const int pt = lb + (e >> LG) * ls + (e & (L - 1));
    bool evolve = true;
    float ctau = ctau0;
    if constexpr (kGeneral) {
      if (p.bc) {
        const long long bit = fbase + pt;
        evolve = ((p.bc[bit >> 5] >> (bit & 31)) & 1u) == 0u;
      }
      if (p.tau_field) ctau = k.tau((p.tau_field[(long long)a * p.N + pt] * tv) / p.dslip[a]);
    }
    if (evolve) {
      const float2 f = *sp;
      const float xr = f64bits_to_f32_fast(xb.x);
      const float s = sinpif(2.0f * xr);
      const float dre = k.cd2 * (k.uq2 * f.x * k.inv_n + k.asf_pi * s - ctau);
      const float dim = k.uq2cd2 * (f.y * k.inv_n);
      xb.x = (unsigned long long)__double_as_longlong(__longlong_as_double((long long)xb.x) -
                                                      __longlong_as_double((long long)f32_to_f64bits_fast(dre)));
      xb.y = (unsigned long long)__double_as_longlong(__longlong_as_double((long long)xb.y) -
                                                      __longlong_as_double((long long)f32_to_f64bits_fast(dim)));
      __stcs(&xg[pt], xb);  // read again only by the next step's z-pass: evict first
    }
    acc += to_fixed_bits(xb.x, big);
    float2 o;
    o.x = f64bits_to_f32_fast(xb.x);
    o.y = f64bits_to_f32_fast(xb.y);
    *sp = o;
  }
  return acc;
}

// z-pass: TL lines of length L along z (one field), see ZFlags.
// Shared memory: twiddles [L] | S lines [TL][pitch] (z_line_pitch) | xi tile
// [TL][L] double2 (update only).  The FP64 xi lines arrive by TMA bulk copies
// that overlap the inverse FFT.  Natural layout: the block's lines are
// consecutive (x, y) pairs, whose S values arrive by cp.async; x-fastest S
// layout (sxf): the lines (x0 + t, y) of one y, whose S values sit TL to a
// contiguous run and go straight between global memory and registers.
// NV: values a thread holds (8 or 16: the radix plan, see stockham_plan_stage).
template <typename T, int LG, int NV>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) zpass_kernel(ZParams p) {
  using V = typename cpx<T>::t;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ long long red[32];
  static_assert(LG >= 0, "the z-pass is instantiated per line length");
  static_assert(NV == 8 || NV == 16, "8 or 16 values a thread");
  constexpr int L = 1 << LG, lgL = LG;
  const int TL = p.TL, P = p.pitch;
  V *tws = reinterpret_cast<V *>(smraw);
  V *sm = tws + L;
  double2 *xs = reinterpret_cast<double2 *>(smraw + ((((size_t)L + (size_t)TL * P) * sizeof(V) + 15) & ~(size_t)15));
  const int E = L >= NV ? NV : L, team = L / E;
  const long long line0 = (long long)blockIdx.x * TL;
  const long long rf = line0 / p.lines_per_field;
  const int r = (int)(rf / p.ns), a = (int)(rf % p.ns);
  if (p.active && !p.active[r]) return;
  const int lf0 = (int)(line0 - rf * p.lines_per_field);
  const bool xf = p.sxf != 0;
  // block within the field -> (x block, y) for the x-fastest layout (x block fastest)
  const int xblocks = xf ? p.n1 >> p.lgTL : 1;
  const int bf = lf0 / TL;
  const int x0 = xf ? (bf % xblocks) * TL : 0, yj = xf ? bf / xblocks : 0;
  // field-relative offsets (< 2^31): xi element (line t, z = k) at lb + t*ls + k,
  // S element at sb + t + k*sk (x-fastest layout; sb + t*L + k in the natural one)
  const int lb = xf ? (x0 * p.n2 + yj) * L : lf0 * L, ls = xf ? p.n2 * L : L;
  const int sb = xf ? yj * L * p.n1 + x0 : lf0 * L, sk = xf ? p.n1 : 1;
  const long long fbase = rf * p.N;  // element / bit base of this field
  const int nel = TL << lgL;
  const int tid = threadIdx.x, nthr = blockDim.x;
  V *Sf = reinterpret_cast<V *>(p.S) + fbase;
  double2 *xif = p.xi + fbase;
  const bool upd = (p.flags & Z_UPDATE) != 0;
  auto sidx = [&](int e) { return (e >> lgL) * P + (e & (L - 1)); };

  __shared__ __align__(8) uint64_t xbar;  // completion of the FP64 state tile
  if (upd && tid == 0) {  // TMA bulk copies: one block (natural) or one per line
    mbar_init(&xbar, 1);
    mbar_arrive_expect_tx(&xbar, (unsigned)nel * 16u);
    if (xf)
      for (int t = 0; t < TL; ++t) bulk_copy(xs + (t << lgL), xif + lb + t * ls, (unsigned)L * 16u, &xbar);
    else
      bulk_copy(xs, xif + lb, (unsigned)nel * 16u, &xbar);
  }
  // x-fastest layout with a forward transform that ends in the store: the S
  // lines go global <-> registers (consecutive lanes on consecutive x, so every
  // access covers whole TL-element runs), shared memory only between stages
  constexpr bool kIO = LG >= 3;
  const bool direct = kIO && xf && (p.flags & Z_FWD) && (p.flags & Z_STORE);
  // S and the step counter come from the kernels before this one (and the
  // FFT-boundary plans write their twiddles right before it); xi (the TMA
  // copy above) from the z-pass before those, complete by then
  griddep_wait();
  load_twiddles(tws, reinterpret_cast<const V *>(p.tw), L);
  if (p.flags & Z_SRC_XI) {
    for (int e = tid; e < nel; e += nthr)
      sm[sidx(e)] = from_xi<V>(xif[lb + (e >> lgL) * ls + (e & (L - 1))]);
  } else if (direct) {
    // (the inverse transform loads its input itself)
  } else if (xf) {
    // consecutive lanes on consecutive x: TL-element runs in global memory
    for (int e = tid; e < nel; e += nthr) {
      const int t = e & (TL - 1), k = e >> p.lgTL;
      cp_async_elem(&sm[t * P + k], &Sf[sb + t + k * sk]);
    }
  } else {
    for (int e = tid; e < nel; e += nthr) cp_async_elem(&sm[sidx(e)], &Sf[sb + e]);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int t = tid % TL, th = tid / TL;  // consecutive lanes on consecutive lines
  const bool act = th < team;
  auto line = [&](int l) { return &sm[t * P + l]; };
  auto gline = [&](int l) { return &Sf[sb + t + l * sk]; };  // S element z = l of line t
  V v[NV];
  if (p.flags & Z_INV) {
    if constexpr (kIO) {
      if (direct && !(p.flags & Z_SRC_XI)) {
        constexpr int LV = L / NV;
        if (act) {
#pragma unroll
          for (int m = 0; m < NV; ++m) v[m] = *gline(th + m * LV);
        }
        line_fft_io<+1, LG, true, false, NV>(v, th, tws, line, line, act);
      } else {
        line_fft<+1, LG, NV>(th, lgL, tws, line, act);
      }
    } else {
      line_fft<+1, LG, NV>(th, lgL, tws, line, act);
    }
  }

  if (upd) {
    mbar_wait(&xbar, 0, p.err);
    __syncthreads();  // the update reads elements of other teams' lines
    const UpdCoef<T> k(p, a);
    const int step = p.step_ctr ? *p.step_ctr : p.step;
    const double tv = p.tau[((long long)step * p.R + r) * p.ns + a];
    const auto ctau0 = k.tau(tv);
    long long acc = 0;
    bool big = false;
    if constexpr (sizeof(V) == sizeof(float2)) {
      const ulonglong2 *xsb = reinterpret_cast<const ulonglong2 *>(xs);
      ulonglong2 *xg = reinterpret_cast<ulonglong2 *>(xif);
      if (p.bc || p.tau_field)
        acc = update_tile_f32<true, LG>(p, k, ctau0, tv, a, fbase, lb, ls, nel, P, sm, xsb, xg, big);
      else
        acc = update_tile_f32<false, LG>(p, k, ctau0, tv, a, fbase, lb, ls, nel, P, sm, xsb, xg, big);
    } else {
      for (int e = tid; e < nel; e += nthr) {
        V *sp = &sm[sidx(e)];
        double2 x = xs[e];
        const int pt = lb + (e >> lgL) * ls + (e & (L - 1));
        bool evolve = true;
        if (p.bc) {
          const long long bit = fbase + pt;
          evolve = ((p.bc[bit >> 5] >> (bit & 31)) & 1u) == 0u;
        }
        if (evolve) {
          auto ctau = ctau0;
          if (p.tau_field) ctau = k.tau((p.tau_field[(long long)a * p.N + pt] * tv) / p.dslip[a]);
          tdgl_point(x, *sp, k.cd2, k.asf_pi, k.uq2, k.uq2cd2, ctau, k.inv_n);
          xif[pt] = x;
        }
        acc += to_fixed(x.x, big);
        *sp = from_xi<V>(x);
      }
    }
    const long long s = block_sum_i64(acc, red);
    const int anybig = __syncthreads_or(big);
    if (tid == 0) p.part[((long long)step * p.R * p.ns + rf) * p.nparts + lf0 / TL] = anybig ? LLONG_MIN : s;
    __syncthreads();
  }

  if constexpr (kIO) {
    if (direct) {  // forward transform, last stage straight to S
      line_fft_io<-1, LG, false, true, NV>(v, th, tws, line, gline, act);
      return;
    }
  }
  if (p.flags & Z_FWD) line_fft<-1, LG, NV>(th, lgL, tws, line, act);
  if (p.flags & Z_STORE) {
    __syncthreads();
    if (xf) {
      for (int e = tid; e < nel; e += nthr) {
        const int t = e & (TL - 1), k = e >> p.lgTL;
        Sf[sb + t + k * sk] = sm[t * P + k];
      }
    } else {
      for (int e = tid; e < nel; e += nthr) Sf[sb + e] = sm[sidx(e)];
    }
  }
}

// Batched line FFT along a strided axis: data viewed as [outer][L][inner],
// one CTA transforms an L x TI tile (TI contiguous inner columns).
// Shared memory: twiddles [L] | tile [L][pitch].
// NV: values a thread holds (8 or 16) for L >= 8.
template <typename T, int S, int LG, int NV>
__global__ void __launch_bounds__(256)
fft_strided_kernel(void *data_, int lgL, int lgTI, long long inner, long long tiles_per_outer, const void *tw_,
                   const uint8_t *active, long long outer_per_rep, int pitch, int rev) {
  static_assert(NV == 8 || NV == 16, "8 or 16 values a thread");
  using V = typename cpx<T>::t;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int L = 1 << lgL, TI = 1 << lgTI;
  V *tws = reinterpret_cast<V *>(smraw);
  V *sm = tws + L;
  // rev: the blocks run from the last down, so that the first take the
  // fields the previous pass wrote last (still in L2)
  const long long bid = rev ? gridDim.x - 1 - blockIdx.x : blockIdx.x;
  const long long o = bid / tiles_per_outer;
  const long long c0 = (bid - o * tiles_per_outer) << lgTI;
  if (active && !active[o / outer_per_rep]) return;
  V *base = reinterpret_cast<V *>(data_) + o * (long long)L * inner + c0;
  const int nel = L << lgTI, tid = threadIdx.x, nthr = blockDim.x;
  // the lines come from the kernel before this one (and the FFT-boundary
  // plans write their twiddles right before it)
  griddep_wait();
  load_twiddles(tws, reinterpret_cast<const V *>(tw_), L);
  if constexpr (LG >= 3) {
    // lines straight from global memory into registers (consecutive lanes on
    // consecutive columns: coalesced), the last stage straight back; shared
    // memory only between stages.  The first stage uses no twiddles, and the
    // barrier after it orders the twiddle table before the second.
    constexpr int LV = (1 << LG) / NV;
    const int t = tid & (TI - 1), th = tid >> lgTI;
    V *col = base + t;
    const int in32 = (int)inner;  // a line spans L * inner < 2^31 values
    V v[NV];
#pragma unroll
    for (int m = 0; m < NV; ++m) v[m] = col[(th + m * LV) * in32];
    line_fft_io<S, LG, true, true, NV>(v, th, tws, [&](int l) { return &sm[l * pitch + t]; },
                                       [&](int l) { return &col[l * in32]; }, true);
  } else {
    for (int e = tid; e < nel; e += nthr) {
      const int l = e >> lgTI, t = e & (TI - 1);
      cp_async_elem(&sm[l * pitch + t], &base[(long long)l * inner + t]);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    const int E = L >= 8 ? 8 : L, team = L / E;  // LG < 3 here: one thread per line
    const int t = tid & (TI - 1), th = tid >> lgTI;  // consecutive lanes on consecutive lines
    const bool act = th < team;
    line_fft<S, LG>(th, lgL, tws, [&](int l) { return &sm[l * pitch + t]; }, act);
    __syncthreads();
    for (int e = tid; e < nel; e += nthr) {
      const int l = e >> lgTI, tt = e & (TI - 1);
      base[(long long)l * inner + tt] = sm[l * pitch + tt];
    }
  }
}

// Device order of B(k), by fused x-pass tile (every x of its inner indices
// c = j*N3 + k), each tile one contiguous block.
// Consecutive tiles (tiles == null): tile c holds T consecutive inner indices,
//   index = (c*P + p) * (T*N1) + t*N1 + x,  inner index = c*T + t.
// Tile table (the FP32 stored-table form): tile i holds the lines tiles[i] =
// (ca, cb) from offset toff[i].  B(k) built from the closed form satisfies
// B(-k) = B(k) bit for bit (every product in it is even in f), and the point
// mirrored through the origin, ((N1-x)%N1, (N2-j)%N2, (N3-k)%N3), has
// frequency -f unless one of its indices is a Nyquist index N/2 (its own
// mirror with a nonzero frequency; for N = 1 index 0, which frec maps to -1).
// So a line ca with j and k below Nyquist and its mirror line
// cb = m(ca) form one "mirrored" tile that stores only ca's row per pair, W =
// b_wm(N1) values: x < N1 for ca, and at x = N1 the value of cb at its Nyquist
// x = N1/2 (the one point of cb that is not a mirror of ca); cb's other points
// read ca's row at (N1 - x) % N1.  Other lines are "single" tiles (cb = -1)
// of one row of W = N1 rounded up to 4 per pair.  A B(k) given by the caller
// that lacks the symmetry gets single tiles only.  line_tile[c] = tile*2 + role
// (0: ca, 1: cb).
struct BLayout {
  long long N, inner;
  int L, lgT, P;
  const int2 *tiles;          // null: consecutive tiles
  const long long *toff;      // [ntiles + 1] offsets (values)
  const int *line_tile;       // [inner]
};
__host__ __device__ __forceinline__ int b_mirror(int i, int n) { return (n - i) & (n - 1); }
// row width of a mirrored tile (N1 values + the Nyquist column, a multiple of
// 4 so every block is a whole number of 16-byte units)
__host__ __device__ constexpr int b_wm(int L) { return (L + 4) / 4 * 4; }
// -1: not stored (the mirror's value, see BLayout)
__host__ __device__ __forceinline__ long long b_index(const BLayout &bl, int p, long long pt) {
  const long long x = pt / bl.inner, c = pt - x * bl.inner;
  if (!bl.tiles) {
    const long long tile = c >> bl.lgT, t = c & ((1LL << bl.lgT) - 1);
    return (tile * bl.P + p) * ((long long)bl.L << bl.lgT) + t * bl.L + x;
  }
  const int lt = bl.line_tile[c], tile = lt >> 1, role = lt & 1;
  const long long base = bl.toff[tile];
  if (bl.tiles[tile].y < 0) return base + (long long)p * ((bl.toff[tile + 1] - base) / bl.P) + x;
  const long long W = b_wm(bl.L);
  if (role == 0) return base + p * W + x;
  return x == bl.L / 2 ? base + p * W + bl.L : -1;
}

// Constants of the closed-form B(k) for the x-pass that evaluates the
// contraction in FP32 registers instead of streaming a stored table (see
// x_fused_kernel, BFLY).  Symmetric tensors as six components c = xx, yy, zz,
// xy, xz, yz; m_c = 1 (diagonal) or 2 (off-diagonal) folds the double
// contraction of two symmetric tensors into six products.
struct BFlyParams {
  int n2, n3, lgN3;
  float d[3], mu, ll, mup;
  float sig6[kMaxNs][6];  // sigma_b = C : eps_b
  float pe6[kMaxNs][6];   // m_c sym(eps_a)_c / mu
  float qs6[kMaxNs][6];   // -m_c sigma_a,c / mu
};

struct XParams {
  void *S;
  const void *B;
  const int2 *xt;            // tile table (null: tiles of T consecutive inner indices), see BLayout
  const long long *xtoff;
  const int *xline;          // line -> tile * 2 + role
  const int *xord;           // T = 1: the CTA's line (lines tile by tile)
  const uint8_t *active;
  const void *tw;          // x-axis forward twiddles (length L = N1)
  long long inner, tiles;  // inner = N2*N3, tiles = inner / T per field row
  int L, lgL, lgT, pitch, R;
  int *err;                // set when a bounded wait times out (may be null)
  int *step_ctr;           // incremented once per launch (null: none); the z-pass reads it
  // failure test (0 in normal runs): CTA 0 announces its B tile's bytes on the
  // mbarrier but issues no copy, so its bounded wait (limit wait_ns) runs out;
  // nothing is left in flight
  int drop_bulk;
  unsigned long long wait_ns;
  // > 0 (warp teams on the tile table): the B block's first bsplit pair rows
  // arrive first; the rest reuse the same buffer once those have been used
  int bsplit;
  BFlyParams bf;
};

// frec (F:2683-2754) in FP32: exact for power-of-two n and unit spacing
__device__ __forceinline__ float frec_f(int i, int n, float d) {
  float v = 0.0f;
  if (i >= 1 && i < n / 2) v = (float)i / (float)n / d;
  if (i >= n / 2) v = ((float)i - (float)n) / (float)n / d;
  return v;
}

// k-space contraction of one point, S_a <- sum_b B_ab S_b (F:4609-4629, b
// ascending), with the point's B(k) in the shared-memory tile Bs: pair p's
// value at Bs[p * W + bx].  at(a) is the point's value of field a (read, then
// overwritten).  IN_REGS keeps the NS inputs in registers.
// WC > 0: the row width is that compile-time W (the B loads then address off
// one base register with immediate offsets).
template <typename T, int NS, bool IN_REGS, int WC = 0, typename At>
__device__ __forceinline__ void contract_table(const T *Bs, int Wrt, int bx, At at) {
  using V = typename cpx<T>::t;
  const int W = WC > 0 ? WC : Wrt;
  Bs += bx;
  V out[NS];
  V in[IN_REGS ? NS : 1];
#pragma unroll
  for (int a = 0; a < NS; ++a) {
    out[a] = V{0, 0};
    if (IN_REGS) in[a] = at(a);
  }
  int pidx = 0;
#pragma unroll
  for (int a = 0; a < NS; ++a) {
    const V ina = IN_REGS ? in[a] : at(a);
#pragma unroll
    for (int b = a; b < NS; ++b, ++pidx) {
      const T v = Bs[pidx * W];
      const V inb = IN_REGS ? in[b] : at(b);
      out[a].x += inb.x * v;
      out[a].y += inb.y * v;
      if (b != a) {
        out[b].x += ina.x * v;
        out[b].y += ina.y * v;
      }
    }
  }
#pragma unroll
  for (int a = 0; a < NS; ++a) at(a) = out[a];
}

// contract_table (FP32, inputs in registers, row width WC) with the tile's pair
// rows in two halves through one buffer: rows [0, P/2) are in Bs on entry;
// at pair P/2 every thread calls mid(), which refills Bs with rows [P/2, P).
// The additions are those of contract_table in the same order (the same
// bits).  has: this thread has a point (a thread without one still calls
// mid(), which holds block barriers).
template <int NS, int WC, typename At, typename Mid>
__device__ __forceinline__ void contract_table_split(const float *Bs, int bx, bool has, At at, Mid mid) {
  constexpr int P = NS * (NS + 1) / 2, P0 = P / 2;
  Bs += bx;
  float2 out[NS], in[NS];
#pragma unroll
  for (int a = 0; a < NS; ++a) {
    out[a] = make_float2(0.f, 0.f);
    in[a] = has ? at(a) : make_float2(0.f, 0.f);
  }
  int pidx = 0;
#pragma unroll
  for (int a = 0; a < NS; ++a) {
#pragma unroll
    for (int b = a; b < NS; ++b, ++pidx) {
      if (pidx == P0) mid();
      const float v = Bs[(pidx < P0 ? pidx : pidx - P0) * WC];
      out[a].x += in[b].x * v;
      out[a].y += in[b].y * v;
      if (b != a) {
        out[b].x += in[a].x * v;
        out[b].y += in[a].y * v;
      }
    }
  }
  if (has) {
#pragma unroll
    for (int a = 0; a < NS; ++a) at(a) = out[a];
  }
}

// The same contraction with the closed form of Bmatrix (F:328-412) in FP32:
// B_ab(k) = (E_ab - u_a . t_b) / mu with E_ab = eps_a : sigma_b, t_b = sigma_b f,
// u_a = G(f) t_a, applied in factored form: with W = sum_b sigma_b S_b (a
// symmetric tensor), w = W f and g = G w,
//   sum_b B_ab S_b = (eps_a : W - sigma_a : sym(g f)) / mu,
// 24 products per field instead of 2 NS per pair; k = 0 gives 0.  x: the
// point's x index (N1 = L), c: its inner index j * N3 + k.
template <int NS, typename At>
__device__ __forceinline__ void contract_bfly(const BFlyParams &bf, At at, int x, int L, long long c) {
  using V = float2;
  const int j = (int)(c >> bf.lgN3), kz = (int)(c & (bf.n3 - 1));
  const float f0 = frec_f(x, L, bf.d[0]), f1 = frec_f(j, bf.n2, bf.d[1]), f2 = frec_f(kz, bf.n3, bf.d[2]);
  const float ff = f0 * f0 + f1 * f1 + f2 * f2;
  if (!(ff > 0.0f)) {
#pragma unroll
    for (int a = 0; a < NS; ++a) at(a) = V{0, 0};
    return;
  }
  V W[6];
#pragma unroll
  for (int cc = 0; cc < 6; ++cc) W[cc] = V{0, 0};
#pragma unroll
  for (int b = 0; b < NS; ++b) {
    const V in = at(b);
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) {
      W[cc].x += bf.sig6[b][cc] * in.x;
      W[cc].y += bf.sig6[b][cc] * in.y;
    }
  }
  // G(f) (the inverse acoustic tensor over |f|^2, as in Bmatrix)
  const float inv = 1.0f / ff;
  const float z0 = f0 * f0 * inv, z1 = f1 * f1 * inv, z2 = f2 * f2 * inv;
  const float d0 = bf.mu + bf.mup * z0, d1 = bf.mu + bf.mup * z1, d2 = bf.mu + bf.mup * z2;
  const float i0 = 1.0f / d0, i1 = 1.0f / d1, i2 = 1.0f / d2;
  const float kk = 1.0f + (bf.mu + bf.ll) * (i0 * z0 + i1 * z1 + i2 * z2);
  const float cg = (bf.mu + bf.ll) / kk * inv;
  const float G00 = inv * (i0 - f0 * f0 * i0 * i0 * cg);
  const float G11 = inv * (i1 - f1 * f1 * i1 * i1 * cg);
  const float G22 = inv * (i2 - f2 * f2 * i2 * i2 * cg);
  const float G01 = -inv * f0 * f1 * i0 * i1 * cg;
  const float G02 = -inv * f0 * f2 * i0 * i2 * cg;
  const float G12 = -inv * f1 * f2 * i1 * i2 * cg;
  // w = W f, g = G w
  V w0, w1, w2, g0, g1, g2;
  w0.x = W[0].x * f0 + W[3].x * f1 + W[4].x * f2;  w0.y = W[0].y * f0 + W[3].y * f1 + W[4].y * f2;
  w1.x = W[3].x * f0 + W[1].x * f1 + W[5].x * f2;  w1.y = W[3].y * f0 + W[1].y * f1 + W[5].y * f2;
  w2.x = W[4].x * f0 + W[5].x * f1 + W[2].x * f2;  w2.y = W[4].y * f0 + W[5].y * f1 + W[2].y * f2;
  g0.x = G00 * w0.x + G01 * w1.x + G02 * w2.x;  g0.y = G00 * w0.y + G01 * w1.y + G02 * w2.y;
  g1.x = G01 * w0.x + G11 * w1.x + G12 * w2.x;  g1.y = G01 * w0.y + G11 * w1.y + G12 * w2.y;
  g2.x = G02 * w0.x + G12 * w1.x + G22 * w2.x;  g2.y = G02 * w0.y + G12 * w1.y + G22 * w2.y;
  // H = sym(g f)
  V H[6];
  H[0].x = g0.x * f0;  H[0].y = g0.y * f0;
  H[1].x = g1.x * f1;  H[1].y = g1.y * f1;
  H[2].x = g2.x * f2;  H[2].y = g2.y * f2;
  H[3].x = 0.5f * (g0.x * f1 + g1.x * f0);  H[3].y = 0.5f * (g0.y * f1 + g1.y * f0);
  H[4].x = 0.5f * (g0.x * f2 + g2.x * f0);  H[4].y = 0.5f * (g0.y * f2 + g2.y * f0);
  H[5].x = 0.5f * (g1.x * f2 + g2.x * f1);  H[5].y = 0.5f * (g1.y * f2 + g2.y * f1);
  // partial unroll: the per-field constants then come through uniform
  // registers (a full unroll spills at 80 registers a thread)
#pragma unroll 4
  for (int a = 0; a < NS; ++a) {
    V o{0, 0};
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) {
      o.x += bf.pe6[a][cc] * W[cc].x + bf.qs6[a][cc] * H[cc].x;
      o.y += bf.pe6[a][cc] * W[cc].y + bf.qs6[a][cc] * H[cc].y;
    }
    at(a) = o;
  }
}

// Shared-memory bytes of the fused x-pass for a tile of T = 2^lgT.
// table: the tile-table layout (T = 2, B rows of at most L + 4 values).
__host__ __device__ __forceinline__ size_t x_fused_smem(int ns, int L, int lgT, int pitch, size_t vsize,
                                                        size_t bsize, bool table = false) {
  const size_t head = ((size_t)L + (size_t)ns * ((size_t)1 << lgT) * pitch) * vsize;
  const size_t P = (size_t)ns * (ns + 1) / 2;
  return ((head + 15) & ~(size_t)15) + P * (table ? (size_t)L + 4 : ((size_t)L << lgT)) * bsize;
}

// Fused x-pass on a tile of T consecutive inner indices, all N1 x-values and
// all NS fields of one replica: forward FFT along x, k-space contraction
// S[a](k) <- sum_b B_ab(k) S[b](k) (F:4609-4629, b ascending), inverse FFT
// along x.  S is in the x-fastest layout ([a][y][z][x] per replica), so every
// line of the tile is L contiguous values.  Shared memory: twiddles [L] | tile
// [a][t][x] (odd line pitch) | B tile [P][T*L].  The lines arrive by cp.async
// (whole 128-byte lines per warp), the B tile by TMA bulk copies that stream in
// during the forward FFT.  One point per thread
// in the contraction; IN_REGS keeps its NS inputs in registers (FP32, up to
// 384 threads); FP64 reads them from shared memory and runs at most 256 threads.
// BFLY (FP32 only): the contraction with the closed form of Bmatrix
// (F:328-412) evaluated per point in FP32 registers, factored through the
// symmetric tensor W = sum_b sigma_b S_b; no B table is read (the x-pass then
// moves only the fields).
template <typename T, int NS, bool IN_REGS, int LG, bool BFLY>
__global__ void __launch_bounds__((IN_REGS || BFLY) ? 384 : 256, 2) x_fused_kernel(XParams p) {
  using V = typename cpx<T>::t;
  constexpr int P = NS * (NS + 1) / 2;
  extern __shared__ __align__(16) unsigned char smraw[];
  // line length and pitch fixed at compile time when LG is (the host's pitch
  // is line_pitch(N1) = N1 + 1), so the shared-memory addressing folds
  const int L = LG >= 0 ? 1 << LG : p.L, lgL = LG >= 0 ? LG : p.lgL, lgT = p.lgT, TT = 1 << lgT;
  const int LP = LG >= 0 ? (1 << LG) + 1 : p.pitch;
  V *tws = reinterpret_cast<V *>(smraw);
  V *sm = tws + L;
  const size_t head = (((size_t)L + (size_t)NS * TT * LP) * sizeof(V) + 15) & ~(size_t)15;
  T *Bs = reinterpret_cast<T *>(smraw + head);
  // replicas of one tile on consecutive CTAs: a batch's CTAs that read the
  // same B block run together, so it comes from HBM once and then from L2
  const long long r = blockIdx.x % p.R;
  const long long tile = blockIdx.x / p.R;
  const bool idle = p.active && !p.active[r];
  const long long c0 = tile << lgT;
  const int npt = L << lgT;
  V *S = reinterpret_cast<V *>(p.S);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int nel = (NS * L) << lgT;
  auto sidx = [&](int a, int t, int x) { return (a * TT + t) * LP + x; };
  constexpr int NV = LG >= 0 ? xpass_nv(LG, (int)sizeof(V)) : 8;
  const int E = L >= NV ? NV : L, team = L / E, teams = nthr / team;
  const int lines = NS << lgT;
  const int my_team = tid % teams, th = tid / teams;  // consecutive lanes on consecutive lines
  // tile table (see BLayout): T = 2, a CTA per tile (its lines ca and cb in
  // slots 0 and 1, slot 1 empty for a single tile); T = 1, a CTA per line
  // (xord lists the lines tile by tile, so the two CTAs of a mirrored tile
  // run back to back and the second reads the shared B block from L2)
  int2 tp = make_int2(0, 0);
  long long tix = tile;
  int role0 = 0;
  if (p.xt) {
    if (lgT == 0) {
      const int c = p.xord[tile], lt = p.xline[c];
      tix = lt >> 1;
      role0 = lt & 1;
      tp = make_int2(c, -1);
    } else {
      tp = p.xt[tile];
    }
  }
  const int tl = p.xt && tp.y < 0 ? 1 : TT;
  auto cidx = [&](int t) { return p.xt ? (t ? tp.y : tp.x) : (int)(c0 + t); };
  const long long boff = p.xt ? p.xtoff[tix] : tile * P * (long long)npt;
  const int bvals = p.xt ? (int)(p.xtoff[tix + 1] - boff) : P * npt;
  const bool mirrored = p.xt && p.xt[tix].y >= 0;
  const int W = p.xt ? (mirrored ? b_wm(L) : bvals / P) : npt;
  const T *Bt = reinterpret_cast<const T *>(p.B) + boff;
  // S is x-fastest: line (a, t) of the tile is L contiguous values; consecutive
  // lanes copy consecutive x (whole 128-byte lines per warp)
  // element x of tile line ln sits at Sr[goff(ln) + x]: 32-bit offsets from the
  // replica's base (a replica's ns fields hold fewer than 2^31 values)
  V *Sr = S + (long long)r * NS * p.inner * L;
  const int fstride = (int)p.inner * L;
  auto goff = [&](int ln) { return (ln >> lgT) * fstride + cidx(ln & (TT - 1)) * L; };
  auto live = [&](int ln) { return (ln & (TT - 1)) < tl; };
  // B tile: one contiguous block of bvals values, TMA bulk copies issued by
  // one thread so it streams in during the forward FFT; B(k) and the
  // twiddles are constant, so they load before the previous kernel is done
  __shared__ __align__(8) uint64_t bbar;
  const int bbytes = BFLY ? 0 : bvals * (int)sizeof(T);
  const bool bulk = !BFLY && (bbytes & 15) == 0 && ((boff * (long long)sizeof(T)) & 15) == 0;
  if (!idle) {
    if (bulk && tid == 0) {
      mbar_init(&bbar, 1);
      if (p.drop_bulk && blockIdx.x == 0) mbar_arrive_expect_tx(&bbar, (unsigned)bbytes);
      else bulk_load(Bs, Bt, (unsigned)bbytes, &bbar);
    }
    if (!BFLY && !bulk)
      for (int i = tid; i < bvals; i += nthr) Bs[i] = Bt[i];
    load_twiddles(tws, reinterpret_cast<const V *>(p.tw), L);
  }
  griddep_wait();  // S and the step counter come from the kernels before this one
  if (p.step_ctr && blockIdx.x == 0 && threadIdx.x == 0) *p.step_ctr += 1;
  if (idle) return;
  for (int e = tid; e < nel; e += nthr) {
    const int x = e & (L - 1), ln = e >> lgL;
    if (live(ln)) cp_async_elem(&sm[ln * LP + x], Sr + goff(ln) + x);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  for (int l0 = 0; l0 < lines; l0 += teams) {
    const int ln = l0 + my_team, a = ln >> lgT, t = ln & (TT - 1);
    line_fft<-1, LG, NV>(th, lgL, tws, [&](int l) { return &sm[sidx(a, t, l)]; }, ln < lines && live(ln));
  }
  if (bulk) mbar_wait(&bbar, 0, p.err, p.wait_ns);
  __syncthreads();
  for (int q = tid; q < (tl << lgL); q += nthr) {
    const int t = q >> lgL, x = q & (L - 1);
    auto at = [&](int a) -> V & { return sm[sidx(a, t, x)]; };
    if constexpr (BFLY) {
      contract_bfly<NS>(p.bf, at, x, L, c0 + t);
    } else {
      // the point's column in the B block: consecutive tiles q; tile table
      // x, or for a mirrored tile's second line the mirror x (its Nyquist x
      // has a column of its own)
      const int role = lgT == 0 ? role0 : t;
      const int bx = !p.xt ? q : (role == 0 ? x : (x == L / 2 ? L : b_mirror(x, L)));
      contract_table<T, NS, IN_REGS>(Bs, W, bx, at);
    }
  }
  __syncthreads();
  for (int l0 = 0; l0 < lines; l0 += teams) {
    const int ln = l0 + my_team, a = ln >> lgT, t = ln & (TT - 1);
    line_fft<+1, LG, NV>(th, lgL, tws, [&](int l) { return &sm[sidx(a, t, l)]; }, ln < lines && live(ln));
  }
  __syncthreads();
  for (int e = tid; e < nel; e += nthr) {
    const int x = e & (L - 1), ln = e >> lgL;
    if (live(ln)) Sr[goff(ln) + x] = sm[ln * LP + x];
  }
}

// Line pitch and swizzle of the warp-team x-pass (FP32 spectra, 8-byte
// elements): element l of a tile line sits at line * xw_pitch(L) + (l ^ ((l >>
// lgNV) & (LV - 1))) with LV = L / NV lanes per line.  The pitch puts the
// 16 / LV lines of one 128-byte shared-memory phase side by side and the XOR
// spreads a stage's strided writes, so no FFT stage and no contraction access
// has a bank conflict (checked for N1 = 32..256 by the host tests).
__host__ __device__ constexpr int xw_lv(int lgL) { return (1 << lgL) / xpass_nv(lgL, 8); }
__host__ __device__ constexpr int xw_pitch(int lgL) { return (1 << lgL) + (xw_lv(lgL) < 16 ? xw_lv(lgL) : 16); }
__host__ __device__ __forceinline__ int xw_swz(int l, int lgL) {
  const int lgNV = xpass_nv(lgL, 8) == 16 ? 4 : 3;
  return l ^ ((l >> lgNV) & (xw_lv(lgL) - 1));
}

// Shared-memory bytes of the warp-team x-pass: twiddles | tile lines |
// B tile (bsize 0: B evaluated in registers; split: the larger half of its
// pair rows, P - P/2).
__host__ __device__ __forceinline__ size_t xw_smem(int ns, int lgL, int lgT, size_t bsize, bool table = false,
                                                   bool split = false) {
  const size_t head = (((size_t)1 << lgL) + (size_t)ns * ((size_t)1 << lgT) * xw_pitch(lgL)) * 8;
  const size_t P = (size_t)ns * (ns + 1) / 2, rows = split ? P - P / 2 : P;
  return ((head + 15) & ~(size_t)15) + rows * (table ? ((size_t)1 << lgL) + 4 : (size_t)1 << (lgL + lgT)) * bsize;
}

// Fused x-pass with warp-resident line teams (FP32 spectra, N1 = 32..256):
// the same transform, contraction and results as x_fused_kernel, laid out so
// that each line's L/NV threads are lanes of one warp.  A line goes straight
// from global memory into registers (lanes on consecutive x), through the
// forward FFT's stages in the warp's own lines of shared memory (warp
// barriers only), and back out of the inverse FFT's last stage straight to
// global memory; the block synchronises only around the contraction, which
// mixes the fields of a point.  The B tile (table form) streams in by TMA
// bulk copies during the forward FFT.
template <int NS, int LG, bool BFLY>
__global__ void __launch_bounds__(384, 2) x_warp_kernel(XParams p) {
  using V = float2;
  static_assert(LG >= 5 && LG <= 8, "the warp-team x-pass covers N1 = 32..256");
  constexpr int L = 1 << LG, P = NS * (NS + 1) / 2;
  constexpr int NV = xpass_nv(LG, 8), LV = L / NV, LPW = 32 / LV, LP = xw_pitch(LG);
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lgT = p.lgT, TT = 1 << lgT, lines = NS << lgT, npt = L << lgT;
  V *tws = reinterpret_cast<V *>(smraw);
  V *sm = tws + L;
  const size_t head = (((size_t)L + (size_t)lines * LP) * sizeof(V) + 15) & ~(size_t)15;
  float *Bs = reinterpret_cast<float *>(smraw + head);
  // replicas of one tile on consecutive CTAs: a batch's CTAs that read the
  // same B block run together, so it comes from HBM once and then from L2
  const long long r = blockIdx.x % p.R;
  const long long tile = blockIdx.x / p.R;
  const bool idle = p.active && !p.active[r];
  const long long c0 = tile << lgT;
  const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
  const int th = lane & (LV - 1), wl = lane / LV;  // team thread, line of the warp
  // tile table (stored-table form, see BLayout and x_fused_kernel): T = 2, a
  // CTA per tile; T = 1, a CTA per line
  int2 tp = make_int2(0, 0);
  long long tix = tile;
  int role0 = 0;
  if (!BFLY && p.xt) {
    if (lgT == 0) {
      const int c = p.xord[tile], lt = p.xline[c];
      tix = lt >> 1;
      role0 = lt & 1;
      tp = make_int2(c, -1);
    } else {
      tp = p.xt[tile];
    }
  }
  const bool tabled = !BFLY && p.xt;
  const int tl = tabled && tp.y < 0 ? 1 : TT;
  auto cidx = [&](int t) { return tabled ? (t ? tp.y : tp.x) : (int)(c0 + t); };
  auto live = [&](int ln) { return (ln & (TT - 1)) < tl; };
  const long long boff = tabled ? p.xtoff[tix] : tile * P * (long long)npt;
  const int bvals = BFLY ? 0 : (tabled ? (int)(p.xtoff[tix + 1] - boff) : P * npt);
  const bool mirrored = tabled && p.xt[tix].y >= 0;
  const int W = tabled ? (mirrored ? b_wm(L) : bvals / P) : npt;
  V *Sr = reinterpret_cast<V *>(p.S) + (long long)r * NS * p.inner * L;
  const int fstride = (int)p.inner * L;
  auto goff = [&](int ln) { return (ln >> lgT) * fstride + cidx(ln & (TT - 1)) * L; };
  __shared__ __align__(8) uint64_t bbar;
  // B(k) and the twiddles are constant: they load before the previous kernel is done
  if (!idle) {
    if (!BFLY && tid == 0) {  // B tile: bvals contiguous values (a multiple of 16 bytes)
      mbar_init(&bbar, 1);
      // split: the first p.bsplit pair rows now, the rest during the contraction
      const int first = p.bsplit ? p.bsplit * W : bvals;
      if (p.drop_bulk && blockIdx.x == 0) mbar_arrive_expect_tx(&bbar, (unsigned)(first * 4));
      else bulk_load_evict_first(Bs, reinterpret_cast<const float *>(p.B) + boff, (unsigned)(first * 4), &bbar);
    }
    load_twiddles(tws, reinterpret_cast<const V *>(p.tw), L);
  }
  griddep_wait();  // S and the step counter come from the kernels before this one
  if (p.step_ctr && blockIdx.x == 0 && threadIdx.x == 0) *p.step_ctr += 1;
  if (idle) return;
  __syncthreads();  // twiddles (the second stage on) and the barrier's initialisation
  for (int ln0 = warp * LPW; ln0 < lines; ln0 += nwarps * LPW) {
    const int ln = ln0 + wl;
    const bool act = ln < lines && live(ln);
    V *line = sm + ln * LP;
    V v[NV];
    if (act) {
      const V *g = Sr + goff(ln) + th;
#pragma unroll
      for (int m = 0; m < NV; ++m) v[m] = g[m * LV];
    }
    line_fft_io<-1, LG, true, false, NV, true>(v, th, tws, [&](int l) { return &line[xw_swz(l, LG)]; },
                                               [&](int l) { return &line[xw_swz(l, LG)]; }, act);
  }
  bool bok = true;
  if (!BFLY) bok = mbar_wait(&bbar, 0, p.err, p.wait_ns);
  __syncthreads();
  if (!BFLY && p.bsplit) {
    // B block in two halves (the host checks that the tile has at most one
    // point a thread): every thread takes part in the buffer swap
    const int q = tid;
    const bool has = q < (tl << LG);
    const int t = has ? q >> LG : 0, x = has ? q & (L - 1) : 0;
    V *const pt = sm + t * LP + xw_swz(x, LG);
    const int role = lgT == 0 ? role0 : t;
    const int bx = !has ? 0 : (role == 0 ? x : (x == L / 2 ? L : b_mirror(x, L)));
    auto mid = [&]() {
      // every thread is past the first rows (and they had arrived): refill the
      // buffer with the rest (generic-proxy reads before the bulk copy's writes)
      if (__syncthreads_and(bok)) {
        if (tid == 0) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          bulk_load_evict_first(Bs, reinterpret_cast<const float *>(p.B) + boff + (long long)p.bsplit * W,
                                (unsigned)((bvals - p.bsplit * W) * 4), &bbar);
        }
        mbar_wait(&bbar, 1, p.err, p.wait_ns);
      }
    };
    auto split = [&](auto wc, auto tc) {
      constexpr int WC = decltype(wc)::value, TC = decltype(tc)::value;
      contract_table_split<NS, WC>(Bs, bx, has, [&](int a) -> V & { return pt[a * TC * LP]; }, mid);
    };
    using I = std::integral_constant<int, 1>;
    using II = std::integral_constant<int, 2>;
    using WM = std::integral_constant<int, b_wm(L)>;
    using WS = std::integral_constant<int, L>;
    if (mirrored && lgT == 1) split(WM{}, II{});
    else if (mirrored) split(WM{}, I{});
    else if (lgT == 1) split(WS{}, II{});
    else split(WS{}, I{});
  } else {
    for (int q = tid; q < (tl << LG); q += nthr) {
      const int t = q >> LG, x = q & (L - 1), sx = xw_swz(x, LG);
      V *const pt = sm + t * LP + sx;  // the point's value of field a at pt[a * T * LP]
      if constexpr (BFLY) {
        contract_bfly<NS>(p.bf, [&](int a) -> V & { return pt[a * TT * LP]; }, x, L, c0 + t);
      } else {
        const int role = lgT == 0 ? role0 : t;
        const int bx = !tabled ? q : (role == 0 ? x : (x == L / 2 ? L : b_mirror(x, L)));
        // the table form's row widths (a mirrored pair, a single line) and tile
        // widths (T = 1, 2) as constants: every shared-memory access of the
        // contraction is an immediate offset from pt or from the B row
        auto table = [&](auto wc, auto tc) {
          constexpr int WC = decltype(wc)::value, TC = decltype(tc)::value;
          contract_table<float, NS, true, WC>(Bs, W, bx, [&](int a) -> V & { return pt[a * TC * LP]; });
        };
        using I = std::integral_constant<int, 1>;
        using II = std::integral_constant<int, 2>;
        using WM = std::integral_constant<int, b_wm(L)>;
        using WS = std::integral_constant<int, L>;
        if (tabled && mirrored && lgT == 1) table(WM{}, II{});
        else if (tabled && mirrored && lgT == 0) table(WM{}, I{});
        else if (tabled && W == L && lgT == 1) table(WS{}, II{});
        else if (tabled && W == L && lgT == 0) table(WS{}, I{});
        else contract_table<float, NS, true>(Bs, W, bx, [&](int a) -> V & { return pt[a * TT * LP]; });
      }
    }
  }
  __syncthreads();
  for (int ln0 = warp * LPW; ln0 < lines; ln0 += nwarps * LPW) {
    const int ln = ln0 + wl;
    const bool act = ln < lines && live(ln);
    V *line = sm + ln * LP;
    V *g = Sr + (act ? goff(ln) : 0);
    V v[NV];
    line_fft_io<+1, LG, false, true, NV, true>(v, th, tws, [&](int l) { return &line[xw_swz(l, LG)]; },
                                               [&](int l) { return &g[l]; }, act);
  }
}

// Forward twiddle table w[t] = exp(-2 pi i t / L), t < L (sincospi in FP64).
template <typename T>
__global__ void twiddle_kernel(void *tw_, int L) {
  using V = typename cpx<T>::t;
  V *tw = reinterpret_cast<V *>(tw_);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= L) return;
  double s, c;
  sincospi(-2.0 * (double)t / (double)L, &s, &c);
  V w;
  w.x = (T)c;
  w.y = (T)s;
  tw[t] = w;
}

struct BBuildParams {
  int n1, n2, n3, ns;
  double d1, d2, d3, mu, ll, mup, mu_inv;
  double sig[kMaxNs][3][3];     // sigma_a = C : eps_a
  double E[kMaxNs][kMaxNs];     // eps_a : C : eps_b
};

__device__ __forceinline__ double frec_dev(int i, int n, double d) {
  double v = 0.0;  // frec, F:2683-2754 (same order of tests)
  if (i >= 1 && i < n / 2) v = (double)(i) / (double)(n) / d;
  if (i >= n / 2) v = ((double)(i) - (double)(n)) / (double)(n) / d;
  return v;
}

}  // namespace pfdd
