// pfdd_fft.cuh -- Stockham FFT building blocks for sm_103a.
//
// A line of length L (power of two) is transformed by a team of L/8 threads
// that each hold 8 complex values in registers (L < 8: one thread holds the
// whole line).  Every stage reads the thread's 8 values from shared memory at
// positions th + m*L/8 (m = 0..7), applies the stage twiddles, runs radix-8
// (or two radix-4, or four radix-2) butterflies in registers and writes the
// results back in Stockham (self-sorting) order, so the final stage leaves the
// transform in natural order.  All index arithmetic is shifts and masks; the
// twiddles come from a table in shared memory.  Signs follow the reference's
// fft_forward / fft_backward (PFDD_Final_GPU.c:209-273): forward
// exp(-2 pi i nk/L), backward exp(+2 pi i nk/L), no normalisation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pfdd {

template <typename T> struct cpx;
template <> struct cpx<float> { using t = float2; };
template <> struct cpx<double> { using t = double2; };

template <typename V> __device__ __forceinline__ V cadd(V a, V b) { V r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { V r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }

// a * w (S < 0) or a * conj(w) (S > 0) where w is a forward-sign table entry
template <int S, typename V> __device__ __forceinline__ V ctw(V a, V w) {
  V r;
  if (S < 0) { r.x = a.x * w.x - a.y * w.y; r.y = a.x * w.y + a.y * w.x; }
  else       { r.x = a.x * w.x + a.y * w.y; r.y = a.y * w.x - a.x * w.y; }
  return r;
}
// a * (S i)
template <int S, typename V> __device__ __forceinline__ V mul_si(V a) {
  V r;
  if (S < 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
  return r;
}
// a * exp(S 2 pi i / 8) = a (1 + S i) / sqrt2
template <int S, typename V> __device__ __forceinline__ V mul_w8(V a) {
  using T = decltype(a.x);
  const T h = (T)0.70710678118654752440;
  V r;
  if (S < 0) { r.x = (a.x + a.y) * h; r.y = (a.y - a.x) * h; }
  else       { r.x = (a.x - a.y) * h; r.y = (a.x + a.y) * h; }
  return r;
}
// a * exp(S 2 pi i 3/8) = a (-1 + S i) / sqrt2
template <int S, typename V> __device__ __forceinline__ V mul_w83(V a) {
  using T = decltype(a.x);
  const T h = (T)0.70710678118654752440;
  V r;
  if (S < 0) { r.x = (a.y - a.x) * h; r.y = -(a.x + a.y) * h; }
  else       { r.x = -(a.x + a.y) * h; r.y = (a.x - a.y) * h; }
  return r;
}

template <int S, typename V> __device__ __forceinline__ void dft2(V &a, V &b) {
  V t = a; a = cadd(t, b); b = csub(t, b);
}
template <int S, typename V> __device__ __forceinline__ void dft4(V &x0, V &x1, V &x2, V &x3) {
  V t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), t3 = mul_si<S>(csub(x1, x3));
  x0 = cadd(t0, t2); x2 = csub(t0, t2); x1 = cadd(t1, t3); x3 = csub(t1, t3);
}
// in place: x[q] <- sum_r x[r] w^{rq}, w = exp(S 2 pi i / 8)
template <int S, typename V> __device__ __forceinline__ void dft8(V *x) {
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

// One Stockham stage of radix R = 2^lgR for a team thread th holding
// v[m] = line[th + m*L/8].  Ns = 2^lgNs radices already applied.
template <int S, int R, typename V, typename Addr>
__device__ __forceinline__ void stockham_stage(V *v, int th, int lgL, int lgNs, const V *tw, Addr sm) {
  constexpr int NB = 8 / R;  // butterflies per thread
  constexpr int lgR = R == 8 ? 3 : (R == 4 ? 2 : 1);
  const int L8 = 1 << (lgL - 3);
  const int Ns = 1 << lgNs;
  const int tsh = lgL - lgNs - lgR;  // twiddle index step = k << tsh
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int j = th + u * L8;
    const int k = j & (Ns - 1);
    V a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = v[u + r * NB];
    if (lgNs > 0) {
      const int ts = k << tsh;
#pragma unroll
      for (int r = 1; r < R; ++r) a[r] = ctw<S>(a[r], tw[r * ts]);
    }
    if (R == 8) dft8<S>(a);
    else if (R == 4) dft4<S>(a[0], a[1], a[2], a[3]);
    else dft2<S>(a[0], a[1]);
    const int base = ((j - k) << lgR) + k;  // (j / Ns) * Ns * R + k
#pragma unroll
    for (int q = 0; q < R; ++q) *sm(base + (q << lgNs)) = a[q];
  }
}

// Full transform of the team's line, data in shared memory in natural order
// before and after; sm(l) addresses element l.  tw: forward twiddles of
// length L (shared memory).  Every thread of the block must call it (the
// stages end with block barriers); the caller synchronises the block before
// the first stage.  Kernels map consecutive lanes to different lines (the
// twiddle loads of a warp are then broadcasts) and give lines an odd pitch.
// LG >= 0 fixes log2(L) at compile time (stage loop unrolled, all index
// arithmetic folded); LG < 0 takes it from lgL at run time.
template <int S, int LG, typename V, typename Addr>
__device__ __forceinline__ void line_fft(int th, int lgL_rt, const V *tw, Addr sm, bool active) {
  const int lgL = LG >= 0 ? LG : lgL_rt;
  if (lgL >= 3) {
    const int L8 = 1 << (lgL - 3);
    constexpr int NST = LG >= 0 ? (LG + 2) / 3 : 4;  // stage count (run time: at most 4 for L <= 4096)
#pragma unroll
    for (int st = 0; st < NST; ++st) {
      const int lgNs = 3 * st;  // every stage before the last is radix 8
      if (LG < 0 && lgNs >= lgL) break;
      const int rem = lgL - lgNs;
      V v[8];
      if (active) {
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = *sm(th + m * L8);
      }
      __syncthreads();
      if (active) {
        if (rem >= 3) stockham_stage<S, 8>(v, th, lgL, lgNs, tw, sm);
        else if (rem == 2) stockham_stage<S, 4>(v, th, lgL, lgNs, tw, sm);
        else stockham_stage<S, 2>(v, th, lgL, lgNs, tw, sm);
      }
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

// Same transform (compile-time L = 2^LG >= 8) with register input and/or a
// direct output.  IN_REGS: v[m] already holds line[th + m*L/8] (loaded by the
// caller straight from global memory), so the first stage skips its shared-
// memory read.  OUT_DIRECT: the last stage writes through `out` (e.g. global
// memory, natural order) instead of `sm`, and no barrier follows it.  `sm`
// holds the line between stages; every thread of the block must call it.
template <int S, int LG, bool IN_REGS, bool OUT_DIRECT, typename V, typename AddrS, typename AddrO>
__device__ __forceinline__ void line_fft_io(V *v, int th, const V *tw, AddrS sm, AddrO out, bool active) {
  static_assert(LG >= 3, "line_fft_io needs L >= 8");
  constexpr int NST = (LG + 2) / 3;
  constexpr int L8 = 1 << (LG - 3);
#pragma unroll
  for (int st = 0; st < NST; ++st) {
    const int lgNs = 3 * st;
    const int rem = LG - lgNs;
    if (st > 0 || !IN_REGS) {
      if (active) {
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = *sm(th + m * L8);
      }
      __syncthreads();  // every read of this stage precedes its in-place writes
    }
    if (active) {
      if (OUT_DIRECT && st == NST - 1) {
        if (rem >= 3) stockham_stage<S, 8>(v, th, LG, lgNs, tw, out);
        else if (rem == 2) stockham_stage<S, 4>(v, th, LG, lgNs, tw, out);
        else stockham_stage<S, 2>(v, th, LG, lgNs, tw, out);
      } else {
        if (rem >= 3) stockham_stage<S, 8>(v, th, LG, lgNs, tw, sm);
        else if (rem == 2) stockham_stage<S, 4>(v, th, LG, lgNs, tw, sm);
        else stockham_stage<S, 2>(v, th, LG, lgNs, tw, sm);
      }
    }
    if (!(OUT_DIRECT && st == NST - 1)) __syncthreads();
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
