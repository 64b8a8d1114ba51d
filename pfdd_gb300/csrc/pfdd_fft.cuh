// pfdd_fft.cuh -- Stockham FFT building blocks for sm_103a.
//
// A line of length L (power of two) is transformed by a team of L/8 threads
// that each hold 8 complex values in registers (L < 8: one thread holds the
// whole line).  Every stage reads the thread's 8 values from shared memory at
// positions th + m*L/8 (m = 0..7), applies the stage twiddles, runs radix-8
// (or two radix-4, or four radix-2) butterflies in registers and writes the
// results back in Stockham (self-sorting) order, so the final stage leaves the
// transform in natural order.  Signs follow the reference's fft_forward /
// fft_backward (PFDD_Final_GPU.c:209-273): forward exp(-2 pi i nk/L),
// backward exp(+2 pi i nk/L), no normalisation.
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

// One Stockham stage of radix R (R in {2,4,8}) for a team thread th holding
// v[m] = line[th + m*L/8].  Ns = product of the radices already applied.
// sm(l) addresses element l of this thread's line in shared memory.
template <int S, int R, typename V, typename Addr>
__device__ __forceinline__ void stockham_stage(V *v, int th, int L, int Ns, const V *__restrict__ tw, Addr sm) {
  constexpr int NB = 8 / R;  // butterflies per thread
  const int L8 = L >> 3;
  const int LR = L / R;
#pragma unroll
  for (int u = 0; u < NB; ++u) {
    const int j = th + u * L8;
    const int k = j & (Ns - 1);
    V a[R];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r] = v[u + r * NB];
    if (Ns > 1) {
      const int tstep = k * (L / (Ns * R));
#pragma unroll
      for (int r = 1; r < R; ++r) a[r] = ctw<S>(a[r], __ldg(&tw[r * tstep]));
    }
    if (R == 8) dft8<S>(a);
    else if (R == 4) dft4<S>(a[0], a[1], a[2], a[3]);
    else dft2<S>(a[0], a[1]);
    const int base = (j - k) * R + k;  // (j / Ns) * Ns * R + k
#pragma unroll
    for (int q = 0; q < R; ++q) *sm(base + q * Ns) = a[q];
  }
  (void)LR;
}

// Full transform of the team's line, data in shared memory in natural order
// before and after.  Every thread of the block must call it (it synchronises).
template <int S, typename V, typename Addr>
__device__ __forceinline__ void line_fft(int th, int L, const V *__restrict__ tw, Addr sm, bool active) {
  if (L >= 8) {
    const int L8 = L >> 3;
    int Ns = 1;
    while (Ns < L) {
      const int rem = L / Ns;
      V v[8];
      if (active) {
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = *sm(th + m * L8);
      }
      __syncthreads();
      if (active) {
        if (rem >= 8) stockham_stage<S, 8>(v, th, L, Ns, tw, sm);
        else if (rem == 4) stockham_stage<S, 4>(v, th, L, Ns, tw, sm);
        else stockham_stage<S, 2>(v, th, L, Ns, tw, sm);
      }
      __syncthreads();
      Ns *= (rem >= 8 ? 8 : rem);
    }
  } else if (L == 4 || L == 2) {
    if (active) {
      if (L == 4) {
        V a0 = *sm(0), a1 = *sm(1), a2 = *sm(2), a3 = *sm(3);
        dft4<S>(a0, a1, a2, a3);
        *sm(0) = a0; *sm(1) = a1; *sm(2) = a2; *sm(3) = a3;
      } else {
        V a0 = *sm(0), a1 = *sm(1);
        dft2<S>(a0, a1);
        *sm(0) = a0; *sm(1) = a1;
      }
    }
    __syncthreads();
  }
}

}  // namespace pfdd
