// pfdd_fft.cuh -- Stockham FFT building blocks for sm_103a.
//
// A line of length L (power of two) is transformed by a team of L/NV threads
// that each hold NV = 8 or 16 complex values in registers (L < 8: one thread
// holds the whole line).  Every stage reads the thread's NV values from shared
// memory at positions th + m*L/NV (m < NV), applies the stage twiddles, runs
// radix-NV butterflies (or NV/R of radix R = 8, 4, 2 in the last stage) in
// registers and writes the results back in Stockham (self-sorting) order, so
// the final stage leaves the transform in natural order.  NV = 16 needs one
// shared-memory round trip fewer for L = 128 and 256 (two stages, not three).
// All index arithmetic is shifts and masks; the twiddles come from a table in
// shared memory.  Signs follow the reference's
// fft_forward / fft_backward (PFDD_Final_GPU.c:209-273): forward
// exp(-2 pi i nk/L), backward exp(+2 pi i nk/L), no normalisation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pfdd {

template <typename T> struct cpx;
template <> struct cpx<float> { using t = float2; };
template <> struct cpx<double> { using t = double2; };

template <typename V> __host__ __device__ __forceinline__ V cadd(V a, V b) { V r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename V> __host__ __device__ __forceinline__ V csub(V a, V b) { V r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }

// a * w (S < 0) or a * conj(w) (S > 0) where w is a forward-sign table entry
template <int S, typename V> __host__ __device__ __forceinline__ V ctw(V a, V w) {
  V r;
  if (S < 0) { r.x = a.x * w.x - a.y * w.y; r.y = a.x * w.y + a.y * w.x; }
  else       { r.x = a.x * w.x + a.y * w.y; r.y = a.y * w.x - a.x * w.y; }
  return r;
}
// a * (S i)
template <int S, typename V> __host__ __device__ __forceinline__ V mul_si(V a) {
  V r;
  if (S < 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
  return r;
}
// a * exp(S 2 pi i / 8) = a (1 + S i) / sqrt2
template <int S, typename V> __host__ __device__ __forceinline__ V mul_w8(V a) {
  using T = decltype(a.x);
  const T h = (T)0.70710678118654752440;
  V r;
  if (S < 0) { r.x = (a.x + a.y) * h; r.y = (a.y - a.x) * h; }
  else       { r.x = (a.x - a.y) * h; r.y = (a.x + a.y) * h; }
  return r;
}
// a * exp(S 2 pi i 3/8) = a (-1 + S i) / sqrt2
template <int S, typename V> __host__ __device__ __forceinline__ V mul_w83(V a) {
  using T = decltype(a.x);
  const T h = (T)0.70710678118654752440;
  V r;
  if (S < 0) { r.x = (a.y - a.x) * h; r.y = -(a.x + a.y) * h; }
  else       { r.x = -(a.x + a.y) * h; r.y = (a.x - a.y) * h; }
  return r;
}

template <int S, typename V> __host__ __device__ __forceinline__ void dft2(V &a, V &b) {
  V t = a; a = cadd(t, b); b = csub(t, b);
}
template <int S, typename V> __host__ __device__ __forceinline__ void dft4(V &x0, V &x1, V &x2, V &x3) {
  V t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), t3 = mul_si<S>(csub(x1, x3));
  x0 = cadd(t0, t2); x2 = csub(t0, t2); x1 = cadd(t1, t3); x3 = csub(t1, t3);
}
// in place: x[q] <- sum_r x[r] w^{rq}, w = exp(S 2 pi i / 8)
template <int S, typename V> __host__ __device__ __forceinline__ void dft8(V *x) {
  V e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
  V o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
  dft4<S>(e0, e1, e2, e3);
  dft4<S>(o0, o1, o2, o3);
  o1 = mul_w8<S>(o1); o2 = mul_si<S>(o2); o3 = mul_w83<S>(o3);
  x[0] = cadd(e0, o0); x[4] = csub(e0, o0);
  x[1] = cadd(e1, o1); x[5] = csub(e1, o1);
  x[2] = cadd(e2, o2); x[6] = csub(e2, o2);
  x[3] = cadd(e3, o3); x[7] = csub(e3, o3);
}
// a * exp(S 2 pi i m / 16) for m = 1, 3 (cos/sin of pi/8 and 3 pi/8)
template <int S, int M, typename V> __host__ __device__ __forceinline__ V mul_w16(V a) {
  using T = decltype(a.x);
  const T c = (T)0.92387953251128675613, s = (T)0.38268343236508977173;
  const T wr = M == 1 ? c : s, wi = (T)S * (M == 1 ? s : c);
  V r;
  r.x = a.x * wr - a.y * wi;
  r.y = a.x * wi + a.y * wr;
  return r;
}
// in place: x[q] <- sum_r x[r] w^{rq}, w = exp(S 2 pi i / 16), as 4 x 4:
// r = 4 r1 + r2, q = q1 + 4 q2; DFT-4 over r1, twiddle w^{r2 q1}, DFT-4 over r2
template <int S, typename V> __host__ __device__ __forceinline__ void dft16(V *x) {
#pragma unroll
  for (int r2 = 0; r2 < 4; ++r2) dft4<S>(x[r2], x[4 + r2], x[8 + r2], x[12 + r2]);
  // x[4 q1 + r2] now holds the r2-th partial at q1; twiddles w^{r2 q1}
  x[5] = mul_w16<S, 1>(x[5]);   // q1 = 1, r2 = 1: w^1
  x[6] = mul_w8<S>(x[6]);       // q1 = 1, r2 = 2: w^2
  x[7] = mul_w16<S, 3>(x[7]);   // q1 = 1, r2 = 3: w^3
  x[9] = mul_w8<S>(x[9]);       // q1 = 2, r2 = 1: w^2
  x[10] = mul_si<S>(x[10]);     // q1 = 2, r2 = 2: w^4
  x[11] = mul_w83<S>(x[11]);    // q1 = 2, r2 = 3: w^6
  x[13] = mul_w16<S, 3>(x[13]); // q1 = 3, r2 = 1: w^3
  x[14] = mul_w83<S>(x[14]);    // q1 = 3, r2 = 2: w^6
  {                             // q1 = 3, r2 = 3: w^9 = -w^1
    const V t = mul_w16<S, 1>(x[15]);
    x[15].x = -t.x; x[15].y = -t.y;
  }
  V y[16];
#pragma unroll
  for (int q1 = 0; q1 < 4; ++q1) {
    V a0 = x[4 * q1], a1 = x[4 * q1 + 1], a2 = x[4 * q1 + 2], a3 = x[4 * q1 + 3];
    dft4<S>(a0, a1, a2, a3);
    y[q1] = a0; y[q1 + 4] = a1; y[q1 + 8] = a2; y[q1 + 12] = a3;
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) x[q] = y[q];
}

// One Stockham stage of radix R = 2^lgR for a team thread th holding
// v[m] = line[th + m*L/NV] (m < NV).  Ns = 2^lgNs radices already applied;
// the thread runs NV/R butterflies, butterfly u on the R values
// line[j + r*L/R] with j = th + u*L/NV.  Host-callable for the CPU check of
// the radix plans (sm is then any addressable buffer).
template <int S, int R, int NV = 8, typename V, typename Addr>
__host__ __device__ __forceinline__ void stockham_stage(V *v, int th, int lgL, int lgNs, const V *tw, Addr sm) {
  static_assert(R <= NV && (NV == 8 || NV == 16), "radix above the values a thread holds");
  constexpr int NB = NV / R;  // butterflies per thread
  constexpr int lgR = R == 16 ? 4 : (R == 8 ? 3 : (R == 4 ? 2 : 1));
  constexpr int lgNV = NV == 16 ? 4 : 3;
  const int LV = 1 << (lgL - lgNV);
  const int Ns = 1 << lgNs;
  const int tsh = lgL - lgNs - lgR;  // twiddle index step = k << tsh
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int j = th + u * LV;
    const int k = j & (Ns - 1);
    V a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = v[u + r * NB];
    if (lgNs > 0) {
      const int ts = k << tsh;
#pragma unroll
      for (int r = 1; r < R; ++r) a[r] = ctw<S>(a[r], tw[r * ts]);
    }
    if constexpr (R == 16) dft16<S>(a);
    else if constexpr (R == 8) dft8<S>(a);
    else if constexpr (R == 4) dft4<S>(a[0], a[1], a[2], a[3]);
    else dft2<S>(a[0], a[1]);
    const int base = ((j - k) << lgR) + k;  // (j / Ns) * Ns * R + k
#pragma unroll
    for (int q = 0; q < R; ++q) *sm(base + (q << lgNs)) = a[q];
  }
}

// Stage st of the radix plan for NV values per thread: radix NV while at
// least NV remain, then one stage of the remainder (8, 4 or 2).
template <int S, int NV, typename V, typename Addr>
__host__ __device__ __forceinline__ void stockham_plan_stage(V *v, int th, int lgL, int st, const V *tw, Addr sm) {
  constexpr int lgNV = NV == 16 ? 4 : 3;
  const int lgNs = lgNV * st, rem = lgL - lgNs;
  if (rem >= lgNV) stockham_stage<S, NV, NV>(v, th, lgL, lgNs, tw, sm);
  else if (rem == 3) stockham_stage<S, 8, NV>(v, th, lgL, lgNs, tw, sm);  // NV = 16 only
  else if (rem == 2) stockham_stage<S, 4, NV>(v, th, lgL, lgNs, tw, sm);
  else stockham_stage<S, 2, NV>(v, th, lgL, lgNs, tw, sm);
}

// Values per thread (NV) for a line of 2^lgL known at compile time: 16 where
// that saves a stage (L = 16, 128, 256), else 8.  A line of L has a team of
// max(1, L / NV) threads.  Each kernel takes this or 8 (zpass_nv, xpass_nv):
// at 128^3 x 12 on GB300 the 16-value plan made the FP32 x-pass 222 -> 203 us,
// the y passes 70 -> 66 us and the FP64 z-pass 3.13 -> 3.06 ms, but the FP32
// z-pass (64 registers a thread for four 256-thread CTAs per SM) 280 -> 355 us
// and the FP64 x-pass (spills) 2.98 -> 3.52 ms, so those two stay at 8.
// These are the defaults; the z-pass and the strided passes are compiled for
// both 8 and 16 where they differ (L >= 16), and a context's autotuner times
// both (the x-pass keeps xpass_nv).
__host__ __device__ constexpr int fft_nv(int lgL) { return (lgL == 4 || lgL == 7 || lgL == 8) ? 16 : 8; }
__host__ __device__ constexpr int zpass_nv(int lgL, int vsize) { return vsize == 8 ? 8 : fft_nv(lgL); }
__host__ __device__ constexpr int xpass_nv(int lgL, int vsize) { return vsize == 8 ? fft_nv(lgL) : 8; }

// Stage count of a line of 2^lgL with NV values per thread.
__host__ __device__ constexpr int stockham_stages(int lgL, int NV) {
  return NV == 16 ? (lgL + 3) / 4 : (lgL + 2) / 3;
}

// Full transform of the team's line, data in shared memory in natural order
// before and after; sm(l) addresses element l.  tw: forward twiddles of
// length L (shared memory).  Every thread of the block must call it (the
// stages end with block barriers); the caller synchronises the block before
// the first stage.  Kernels map consecutive lanes to different lines (the
// twiddle loads of a warp are then broadcasts) and give lines an odd pitch.
// LG >= 0 fixes log2(L) at compile time (stage loop unrolled, all index
// arithmetic folded); LG < 0 takes it from lgL at run time.  A team has
// L/NV threads, so L >= NV (or L < 8: one thread, a single DFT-2 or DFT-4).
template <int S, int LG, int NV = 8, typename V, typename Addr>
__device__ __forceinline__ void line_fft(int th, int lgL_rt, const V *tw, Addr sm, bool active) {
  constexpr int lgNV = NV == 16 ? 4 : 3;
  const int lgL = LG >= 0 ? LG : lgL_rt;
  if (lgL >= 3) {
    const int LV = 1 << (lgL > lgNV ? lgL - lgNV : 0);  // (L >= NV whenever this runs)
    // stage count (run time: at most 4 for L <= 4096)
    constexpr int NST = LG >= 0 ? stockham_stages(LG, NV) : stockham_stages(12, NV);
#pragma unroll
    for (int st = 0; st < NST; ++st) {
      if (LG < 0 && lgNV * st >= lgL) break;
      V v[NV];
      if (active) {
#pragma unroll
        for (int m = 0; m < NV; ++m) v[m] = *sm(th + m * LV);
      }
      __syncthreads();
      if (active) stockham_plan_stage<S, NV>(v, th, lgL, st, tw, sm);
      __syncthreads();
    }
  } else if (lgL >= 1) {
    if (active) {
      if (lgL == 2) {
        V a0 = *sm(0), a1 = *sm(1), a2 = *sm(2), a3 = *sm(3);
        dft4<S>(a0, a1, a2, a3);
        *sm(0) = a0; *sm(1) = a1; *sm(2) = a2; *sm(3) = a3;
      } else {
        V a0 = *sm(0), a1 = *sm(1);
        dft2<S>(a0, a1);
        *sm(0) = a0; *sm(1) = a1;
      }
    }
  }
}

// Same transform (compile-time L = 2^LG >= NV) with register input and/or a
// direct output.  IN_REGS: v[m] already holds line[th + m*L/NV] (loaded by
// the caller straight from global memory), so the first stage skips its
// shared-memory read.  OUT_DIRECT: the last stage writes through `out` (e.g.
// global memory, natural order) instead of `sm`, and no barrier follows it.
// `sm` holds the line between stages; every thread of the block must call it.
// WARP: the team's threads sit in one warp (the line lives in the warp's own
// part of shared memory), so the stages synchronise the warp, not the block;
// every lane of a warp that calls it must call it.
template <int S, int LG, bool IN_REGS, bool OUT_DIRECT, int NV = 8, bool WARP = false, typename V, typename AddrS,
          typename AddrO>
__device__ __forceinline__ void line_fft_io(V *v, int th, const V *tw, AddrS sm, AddrO out, bool active) {
  constexpr int lgNV = NV == 16 ? 4 : 3;
  static_assert(LG >= lgNV, "line_fft_io needs L >= NV");
  constexpr int NST = stockham_stages(LG, NV);
  constexpr int LV = 1 << (LG - lgNV);
#pragma unroll
  for (int st = 0; st < NST; ++st) {
    if (st > 0 || !IN_REGS) {
      if (active) {
#pragma unroll
        for (int m = 0; m < NV; ++m) v[m] = *sm(th + m * LV);
      }
      if (WARP) __syncwarp();  // every read of this stage precedes its in-place writes
      else __syncthreads();
    }
    if (active) {
      if (OUT_DIRECT && st == NST - 1) stockham_plan_stage<S, NV>(v, th, LG, st, tw, out);
      else stockham_plan_stage<S, NV>(v, th, LG, st, tw, sm);
    }
    if (!(OUT_DIRECT && st == NST - 1)) {
      if (WARP) __syncwarp();
      else __syncthreads();
    }
  }
}

// Copies a length-L twiddle table to shared memory (caller synchronises).
template <typename V>
__device__ __forceinline__ void load_twiddles(V *dst, const V *__restrict__ src, int L) {
  for (int i = threadIdx.x; i < L; i += blockDim.x) dst[i] = src[i];
}

// ---- asynchronous global -> shared copies (cp.async, completion groups) ----
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
template <typename V> __device__ __forceinline__ void cp_async_elem(V *smem, const V *gmem) {
  if (sizeof(V) == 16) cp_async16(smem, gmem);
  else cp_async8(smem, gmem);
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

}  // namespace pfdd
