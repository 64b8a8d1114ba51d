// pfdd_kernels.cuh -- kernels of the PFDD TDGL step (generic path, any
// power-of-two grid, FP64 or FP32 spectral precision).
//
// Device data (N = N1*N2*N3, R replicas, ns slip systems):
//   xi   double2 [R][ns][N]   order parameter, FP64 state (F:4146)
//   S    T2      [R][ns][N]   spectral work buffer (T = double or float)
//   B    T       [P][N]       packed symmetric B(k), P = ns(ns+1)/2 pairs
//                             a <= b in row-major order
//   bc   uint32  bit mask     bit (r*ns+a)*N+pt set = pinned (xi_bc != 0)
//
// One TDGL step of the generic path is six launches:
//   y-forward, x-forward, contraction, x-inverse, y-inverse,
//   z-pass (z-inverse -> Euler update + gamma partials -> z-forward).
// The z-forward of the new state is fused into the update so S always holds
// the z-transformed state between steps.
#pragma once
#include "pfdd_fft.cuh"

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
  double *part;             // [step][R*ns][nparts]
  const uint8_t *active;    // [R] or null
  const void *tw;           // forward twiddles of length L
  long long N, lines_per_field;
  int step, L, ns, R, TL, nparts, flags, pitch;
  double inv_n, uq2;
  double cd2[kMaxNs], asf_pi[kMaxNs], uq2cd2[kMaxNs];
};

template <typename V> __device__ __forceinline__ V from_xi(double2 x);
template <> __device__ __forceinline__ double2 from_xi<double2>(double2 x) { return x; }
template <> __device__ __forceinline__ float2 from_xi<float2>(double2 x) { return make_float2((float)x.x, (float)x.y); }

// plasticevolv (F:3470-3501) for one point.  FP64 form: the reference's
// expression in double precision.  FP32 form: force and core term evaluated
// in FP32 (sin of an FP64-reduced argument), then accumulated into the FP64
// state.
__device__ __forceinline__ void tdgl_point(double2 &x, double2 f, double cd2, double asf_pi, double uq2,
                                           double uq2cd2, double ctau, double inv_n) {
  const double s = sinpi(x.x * kTwoPiTruncOverPi);
  x.x = x.x - cd2 * (uq2 * f.x * inv_n + asf_pi * s - ctau);
  x.y = x.y - uq2cd2 * (f.y * inv_n);
}
__device__ __forceinline__ void tdgl_point(double2 &x, float2 f, double cd2, double asf_pi, double uq2,
                                           double uq2cd2, double ctau, double inv_n) {
  const double nr = rint(x.x);
  const float r = (float)(x.x - nr);
  const float s = sinpif(2.0f * r);
  const float fi = (float)inv_n;
  const float inner = (float)uq2 * f.x * fi + (float)asf_pi * s - (float)ctau;
  const float dre = (float)cd2 * inner;
  const float dim = (float)uq2cd2 * (f.y * fi);
  x.x = x.x - (double)dre;
  x.y = x.y - (double)dim;
}

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int i = 0; i < nw; ++i) s += red[i];
  }
  return s;
}

// z-pass: TL contiguous lines of length L (one field), see ZFlags.
template <typename T>
__global__ void __launch_bounds__(256) zpass_kernel(ZParams p) {
  using V = typename cpx<T>::t;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double red[32];
  V *sm = reinterpret_cast<V *>(smraw);
  const int L = p.L, TL = p.TL, P = p.pitch;
  const int E = L >= 8 ? 8 : L, team = L / E;
  const long long line0 = (long long)blockIdx.x * TL;
  const long long rf = line0 / p.lines_per_field;
  const int r = (int)(rf / p.ns), a = (int)(rf % p.ns);
  if (p.active && !p.active[r]) return;
  const long long lf0 = line0 - rf * p.lines_per_field;
  const long long e0 = line0 * L;
  const int nel = TL * L;
  const int tid = threadIdx.x, nthr = blockDim.x;
  V *S = reinterpret_cast<V *>(p.S);
  const V *tw = reinterpret_cast<const V *>(p.tw);

  if (p.flags & Z_SRC_XI) {
    for (int e = tid; e < nel; e += nthr) sm[(e / L) * P + (e % L)] = from_xi<V>(p.xi[e0 + e]);
  } else {
    for (int e = tid; e < nel; e += nthr) sm[(e / L) * P + (e % L)] = S[e0 + e];
  }
  __syncthreads();
  const int t = tid / team, th = tid - t * team;
  const bool act = t < TL;
  auto line = [&](int l) { return &sm[t * P + l]; };
  if (p.flags & Z_INV) line_fft<+1>(th, L, tw, line, act);

  if (p.flags & Z_UPDATE) {
    const double cd2 = p.cd2[a], asf_pi = p.asf_pi[a], uq2cd2 = p.uq2cd2[a];
    const double tv = p.tau[((long long)p.step * p.R + r) * p.ns + a];
    const long long fbase = rf * p.N;  // bit / element base of this field
    double acc = 0.0;
    for (int e = tid; e < nel; e += nthr) {
      V *sp = &sm[(e / L) * P + (e % L)];
      double2 x = p.xi[e0 + e];
      const long long pt = lf0 * L + e;
      bool evolve = true;
      if (p.bc) {
        const long long bit = fbase + pt;
        evolve = ((p.bc[bit >> 5] >> (bit & 31)) & 1u) == 0u;
      }
      if (evolve) {
        double ctau = tv;
        if (p.tau_field) ctau = (p.tau_field[(long long)a * p.N + pt] * tv) / p.dslip[a];
        tdgl_point(x, *sp, cd2, asf_pi, p.uq2, uq2cd2, ctau, p.inv_n);
        p.xi[e0 + e] = x;
      }
      acc += x.x;
      *sp = from_xi<V>(x);
    }
    const double s = block_sum(acc, red);
    if (tid == 0) p.part[((long long)p.step * p.R * p.ns + rf) * p.nparts + lf0 / TL] = s;
    __syncthreads();
  }

  if (p.flags & Z_FWD) line_fft<-1>(th, L, tw, line, act);
  if (p.flags & Z_STORE) {
    if (L < 8) __syncthreads();
    for (int e = tid; e < nel; e += nthr) S[e0 + e] = sm[(e / L) * P + (e % L)];
  }
}

// Batched line FFT along a strided axis: data viewed as [outer][L][inner],
// one CTA transforms an L x TI tile (TI contiguous inner columns).
template <typename T, int S>
__global__ void __launch_bounds__(256)
fft_strided_kernel(void *data_, int L, long long inner, int TI, long long tiles_per_outer, const void *tw_,
                   const uint8_t *active, long long outer_per_rep, int pitch) {
  using V = typename cpx<T>::t;
  extern __shared__ __align__(16) unsigned char smraw[];
  V *sm = reinterpret_cast<V *>(smraw);
  const long long o = blockIdx.x / tiles_per_outer;
  const long long c0 = (blockIdx.x - o * tiles_per_outer) * (long long)TI;
  if (active && !active[o / outer_per_rep]) return;
  V *base = reinterpret_cast<V *>(data_) + o * (long long)L * inner + c0;
  const V *tw = reinterpret_cast<const V *>(tw_);
  const int nel = L * TI, tid = threadIdx.x, nthr = blockDim.x;
  for (int e = tid; e < nel; e += nthr) {
    const int l = e / TI, t = e - l * TI;
    sm[l * pitch + t] = base[(long long)l * inner + t];
  }
  __syncthreads();
  const int E = L >= 8 ? 8 : L, team = L / E;
  const int t = tid % TI, th = tid / TI;
  const bool act = th < team;
  line_fft<S>(th, L, tw, [&](int l) { return &sm[l * pitch + t]; }, act);
  for (int e = tid; e < nel; e += nthr) {
    const int l = e / TI, tt = e - l * TI;
    base[(long long)l * inner + tt] = sm[l * pitch + tt];
  }
}

// k-space contraction (F:4609-4629): S[r][a](k) <- sum_b B_ab(k) S[r][b](k),
// b ascending for every a, RC replicas per pass so each B value is loaded once
// per RC replicas.
template <typename T, int NS, int RC>
__global__ void __launch_bounds__(256)
contract_kernel(void *S_, const T *__restrict__ B, long long N, int R, const uint8_t *active) {
  using V = typename cpx<T>::t;
  V *S = reinterpret_cast<V *>(S_);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += stride) {
    for (int r0 = 0; r0 < R; r0 += RC) {
      V in[RC][NS], out[RC][NS];
      bool on[RC];
#pragma unroll
      for (int q = 0; q < RC; ++q) {
        on[q] = (r0 + q < R) && (!active || active[r0 + q]);
#pragma unroll
        for (int b = 0; b < NS; ++b) {
          in[q][b] = on[q] ? S[((long long)(r0 + q) * NS + b) * N + pt] : V{0, 0};
          out[q][b] = V{0, 0};
        }
      }
      int pidx = 0;
#pragma unroll
      for (int a = 0; a < NS; ++a) {
#pragma unroll
        for (int b = a; b < NS; ++b, ++pidx) {
          const T v = __ldg(&B[(long long)pidx * N + pt]);
#pragma unroll
          for (int q = 0; q < RC; ++q) {
            out[q][a].x += in[q][b].x * v;
            out[q][a].y += in[q][b].y * v;
            if (b != a) {
              out[q][b].x += in[q][a].x * v;
              out[q][b].y += in[q][a].y * v;
            }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < RC; ++q)
        if (on[q]) {
#pragma unroll
          for (int b = 0; b < NS; ++b) S[((long long)(r0 + q) * NS + b) * N + pt] = out[q][b];
        }
    }
  }
}

// Deterministic second stage of the gamma sums: one thread per (step, replica).
__global__ void gamma_reduce_kernel(const double *part, int nparts, int R, int ns, int nsteps, double inv_n,
                                    double *gamma_a, double *gamma) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nsteps * R) return;
  const int s = idx / R, r = idx - s * R;
  double tot = 0.0;
  for (int a = 0; a < ns; ++a) {
    const double *pp = part + ((long long)s * R * ns + (long long)r * ns + a) * nparts;
    double acc = 0.0;
    for (int c = 0; c < nparts; ++c) acc += pp[c];
    gamma_a[((long long)s * R + r) * ns + a] = acc * inv_n;
    tot += acc;
  }
  gamma[idx] = tot * inv_n;
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

// B(k) of Bmatrix (F:328-412) in closed form:
//   B_ab = (E_ab - t_a^T G t_b) / mu,  t_a = sigma_a f,
//   G_ki = (1/f^2) [delta_ik / (mu + mu' z_k)
//                   - f_i f_k / f^2 / (mu + mu' z_i) / (mu + mu' z_k) (mu + lambda) / kk]
// with z_i = f_i^2 / f^2 and kk = 1 + (mu + lambda) sum_j z_j / (mu + mu' z_j).
__global__ void build_B_kernel(const BBuildParams *__restrict__ bp, double *Bd, float *Bf, long long N) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int ns = bp->ns;
  const long long P = (long long)ns * (ns + 1) / 2;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += stride) {
    const int k3 = (int)(pt % bp->n3), k2 = (int)((pt / bp->n3) % bp->n2), k1 = (int)(pt / ((long long)bp->n3 * bp->n2));
    const double f[3] = {frec_dev(k1, bp->n1, bp->d1), frec_dev(k2, bp->n2, bp->d2), frec_dev(k3, bp->n3, bp->d3)};
    const double f2 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    if (!(f2 > 0)) {
      for (long long q = 0; q < P; ++q) {
        if (Bd) Bd[q * N + pt] = 0.0;
        if (Bf) Bf[q * N + pt] = 0.0f;
      }
      continue;
    }
    const double mu = bp->mu, ll = bp->ll, mup = bp->mup;
    double z[3], den[3];
    for (int i = 0; i < 3; ++i) { z[i] = f[i] * f[i] / f2; den[i] = mu + mup * z[i]; }
    const double kk = 1.0 + (mu + ll) * (1 / den[0] * z[0] + 1 / den[1] * z[1] + 1 / den[2] * z[2]);
    double G[3][3];
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k)
        G[i][k] = 1 / f2 * ((i == k ? 1.0 : 0.0) / den[k] - f[i] * f[k] / f2 / den[i] / den[k] * (mu + ll) / kk);
    double t[kMaxNs][3], u[kMaxNs][3];
    for (int a = 0; a < ns; ++a) {
      for (int i = 0; i < 3; ++i)
        t[a][i] = bp->sig[a][i][0] * f[0] + bp->sig[a][i][1] * f[1] + bp->sig[a][i][2] * f[2];
      for (int i = 0; i < 3; ++i) u[a][i] = G[i][0] * t[a][0] + G[i][1] * t[a][1] + G[i][2] * t[a][2];
    }
    long long q = 0;
    for (int a = 0; a < ns; ++a)
      for (int b = a; b < ns; ++b, ++q) {
        const double v = (bp->E[a][b] - (t[a][0] * u[b][0] + t[a][1] * u[b][1] + t[a][2] * u[b][2])) * bp->mu_inv;
        if (Bd) Bd[q * N + pt] = v;
        if (Bf) Bf[q * N + pt] = (float)v;
      }
  }
}

// Packs a host-layout B ([kb][ka][N], FP64) already on the device into the
// pair layout, optionally rounding to FP32.
__global__ void pack_B_kernel(const double *src, int ns, long long N, double *Bd, float *Bf) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += stride) {
    long long q = 0;
    for (int a = 0; a < ns; ++a)
      for (int b = a; b < ns; ++b, ++q) {
        const double v = src[((long long)b * ns + a) * N + pt];
        if (Bd) Bd[q * N + pt] = v;
        if (Bf) Bf[q * N + pt] = (float)v;
      }
  }
}

// xi_bc -> pinned bit mask (bit set where xi_bc[..][0] != 0; the reference
// evolves a point where XI_BC(...,0) == 0, F:3481).  `src` holds count
// interleaved [re, im] pairs for bits bit0 .. bit0+count-1; each warp builds its
// 32 bits with a ballot and merges them into at most two mask words.
__global__ void pack_bc_kernel(const double *src, long long count, long long bit0, uint32_t *mask) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31LL; base < count; base += stride) {
    const long long e = base + (threadIdx.x & 31);
    const bool pin = e < count && src[2 * e] != 0.0;
    const uint32_t bal = __ballot_sync(0xffffffffu, pin);
    if ((threadIdx.x & 31) == 0) {
      const long long n = count - base < 32 ? count - base : 32;
      const long long b = bit0 + base;
      const int sh = (int)(b & 31);
      const unsigned long long m64 = (n == 32 ? 0xffffffffull : ((1ull << n) - 1)) << sh;
      const unsigned long long p64 = ((unsigned long long)bal & (n == 32 ? 0xffffffffull : ((1ull << n) - 1))) << sh;
      uint32_t *w = mask + (b >> 5);
      atomicAnd(w, ~(uint32_t)m64);
      atomicOr(w, (uint32_t)p64);
      if (m64 >> 32) {
        atomicAnd(w + 1, ~(uint32_t)(m64 >> 32));
        atomicOr(w + 1, (uint32_t)(p64 >> 32));
      }
    }
  }
}

__global__ void mask_any_kernel(const uint32_t *mask, long long words, int *any) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  int found = 0;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += stride) found |= mask[w] != 0u;
  if (__syncthreads_or(found) && threadIdx.x == 0) atomicOr(any, 1);
}

// Inverse of pack_B_kernel: pair layout (FP64 or FP32) -> [kb][ka][N] FP64.
__global__ void unpack_B_kernel(const double *Bd, const float *Bf, int ns, long long N, double *dst) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += stride) {
    long long q = 0;
    for (int a = 0; a < ns; ++a)
      for (int b = a; b < ns; ++b, ++q) {
        const double v = Bd ? Bd[q * N + pt] : (double)Bf[q * N + pt];
        dst[((long long)b * ns + a) * N + pt] = v;
        dst[((long long)a * ns + b) * N + pt] = v;
      }
  }
}

}  // namespace pfdd
