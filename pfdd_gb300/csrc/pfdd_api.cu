// pfdd_api.cu -- C ABI of the PFDD TDGL hot path (include/pfdd_gpu.h).
//
// A context owns, on one GPU and one CUDA stream, everything a solve (or a
// batch of replicas sharing B(k)) needs between steps: the FP64 state xi,
// the spectral buffer S, the packed B(k), the pinned-point bit mask, the
// per-step stress table and the gamma partial sums.  Nothing is copied
// between host and device inside a step; pfdd_step uploads the stresses of a
// chunk of steps once and reads back gamma once per chunk.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/pfdd_gpu.h"
#include "pfdd_converge.h"
#include "pfdd_launch.h"

namespace pfdd {

__global__ void fill_u64_kernel(unsigned long long *p, long long n, unsigned long long v) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

// Exact sums of the z-pass's fixed-point partials (units of 2^-44) per
// (step, replica): 128-bit integer accumulation, so gamma_a and gamma do not
// depend on how the points were split into blocks; one conversion at the end.
__device__ __forceinline__ double i128_to_double(__int128 v) {
  const bool neg = v < 0;
  const unsigned __int128 u = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const double d = (double)(unsigned long long)(u >> 64) * 18446744073709551616.0 + (double)(unsigned long long)u;
  return neg ? -d : d;
}

// Second stage of the gamma sums: a block per (step, replica), kGammaWarps
// warps per system (block of kGammaWarps * 32 * ns threads).  The sums are
// exact integers, so neither the split of the partials over lanes nor the
// order of the additions changes a result.
constexpr int kGammaWarps = 2;

__device__ __forceinline__ __int128 shfl_down_i128(__int128 v, int o) {
  const unsigned long long lo = __shfl_down_sync(0xffffffffu, (unsigned long long)v, o);
  const long long hi = __shfl_down_sync(0xffffffffu, (long long)(v >> 64), o);
  return (__int128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}

__global__ void __launch_bounds__(kGammaWarps * 32 * kMaxNs) gamma_reduce_kernel(const long long *part, int nparts,
                                                                                int R, int ns, double scale,
                                                                                double *gamma_a, double *gamma) {
  __shared__ __int128 red[kGammaWarps * kMaxNs];
  __shared__ int redbad[kGammaWarps * kMaxNs];
  const int s = blockIdx.x / R, r = blockIdx.x - s * R;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = w / kGammaWarps, part0 = (w % kGammaWarps) * 32 + lane;
  const long long *pp = part + ((long long)s * R * ns + (long long)r * ns + a) * nparts;
  __int128 acc = 0;
  int bad = 0;
#pragma unroll 8
  for (int c = part0; c < nparts; c += kGammaWarps * 32) {
    const long long v = pp[c];
    bad |= v == LLONG_MIN;
    acc += v == LLONG_MIN ? 0 : v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += shfl_down_i128(acc, o);
  bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) {
    red[w] = acc;
    redbad[w] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __int128 tot = 0;
    int totbad = 0;
    for (int b = 0; b < ns; ++b) {
      __int128 sa = 0;
      int ba = 0;
      for (int k = 0; k < kGammaWarps; ++k) {
        sa += red[b * kGammaWarps + k];
        ba |= redbad[b * kGammaWarps + k];
      }
      gamma_a[((long long)s * R + r) * ns + b] = ba ? __longlong_as_double(0x7ff8000000000000ll)
                                                    : i128_to_double(sa) * scale;
      tot += sa;
      totbad |= ba;
    }
    gamma[blockIdx.x] = totbad ? __longlong_as_double(0x7ff8000000000000ll) : i128_to_double(tot) * scale;
  }
}

// Interface-plane diagnostics: copies Re xi of every field at the listed points
// (the plane's, then the residual line's) into out[step][field][point], the
// step from the device counter (0 without one).
__global__ void diag_gather_kernel(const double2 *__restrict__ xi, const long long *__restrict__ pts, int npts,
                                   int RF, long long N, const int *step_ctr, double *out) {
  const long long step = step_ctr ? *step_ctr : 0;
  const long long per = (long long)RF * npts;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < per; i += (long long)gridDim.x * blockDim.x) {
    const long long f = i / npts, q = i - f * npts;
    out[step * per + i] = xi[f * N + pts[q]].x;
  }
}

// ---- strain and stress fields (diagnostics) --------------------------------

struct StrainParams {
  int n1, n2, n3, ns;
  double d1, d2, d3, mu, ll, mup;
  double sig[kMaxNs][3][3];  // sigma_a = C : eps_a
  double eps[kMaxNs][3][3];
  double avepst_sym[3][3];   // (avepst + avepst^T) / 2
  double inv_n;
};

// Symmetric strain in k-space.  The reference's F matrix (F:414-598) is
// F_a,ij = sum_klmn C_klmn G_jk eps_a,mn f_i f_l = f_i (G t_a)_j with
// t_a = sigma_a f, so beta_ij(k) = sum_a F_a,ij xi_a(k) = f_i w_j with
// w = sum_a u_a xi_a, u_a = G t_a (strain, F:761-778); the kernel writes the
// six components (f_i w_j + f_j w_i)/2, c = 00, 01, 02, 11, 12, 22.
__global__ void strain_spec_kernel(const StrainParams *__restrict__ sp, const double2 *__restrict__ xhat,
                                   double2 *__restrict__ E, long long N) {
  const int ns = sp->ns;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += (long long)gridDim.x * blockDim.x) {
    const int k3 = (int)(pt % sp->n3), k2 = (int)((pt / sp->n3) % sp->n2), k1 = (int)(pt / ((long long)sp->n3 * sp->n2));
    const double f[3] = {frec_dev(k1, sp->n1, sp->d1), frec_dev(k2, sp->n2, sp->d2), frec_dev(k3, sp->n3, sp->d3)};
    const double f2 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    double2 w[3] = {{0, 0}, {0, 0}, {0, 0}};
    if (f2 > 0) {
      const double mu = sp->mu, ll = sp->ll, mup = sp->mup;
      double z[3], den[3];
      for (int i = 0; i < 3; ++i) { z[i] = f[i] * f[i] / f2; den[i] = mu + mup * z[i]; }
      const double kk = 1.0 + (mu + ll) * (1 / den[0] * z[0] + 1 / den[1] * z[1] + 1 / den[2] * z[2]);
      double G[3][3];
      for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k)
          G[i][k] = 1 / f2 * ((i == k ? 1.0 : 0.0) / den[k] - f[i] * f[k] / f2 / den[i] / den[k] * (mu + ll) / kk);
      for (int a = 0; a < ns; ++a) {
        double t[3], u[3];
        for (int i = 0; i < 3; ++i) t[i] = sp->sig[a][i][0] * f[0] + sp->sig[a][i][1] * f[1] + sp->sig[a][i][2] * f[2];
        for (int j = 0; j < 3; ++j) u[j] = G[j][0] * t[0] + G[j][1] * t[1] + G[j][2] * t[2];
        const double2 x = xhat[(long long)a * N + pt];
        for (int j = 0; j < 3; ++j) { w[j].x += u[j] * x.x; w[j].y += u[j] * x.y; }
      }
    }
    int c = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j, ++c) {
        double2 e;
        e.x = 0.5 * (f[i] * w[j].x + f[j] * w[i].x);
        e.y = 0.5 * (f[i] * w[j].y + f[j] * w[i].y);
        E[(long long)c * N + pt] = e;
      }
  }
}

// Real-space strain and stress per point (strain F:792-812, stress F:885-921):
// eps_ij = Re E_ij / N + sym(avepst)_ij, sigma_ij = C_ijkl (eps_kl - eps_d,kl),
// eps_d = sum_a eps_a Re xi_a.  Outputs [3 i + j][N] (either may be null) and
// per-block partial sums of both (18 values per block, summed on the host in
// block order, so the means do not depend on scheduling).
__global__ void __launch_bounds__(256) strain_real_kernel(const StrainParams *__restrict__ sp,
                                                          const double2 *__restrict__ E,
                                                          const double2 *__restrict__ xi, double *eps_out,
                                                          double *sig_out, double *partial, long long N) {
  __shared__ double red[18][256];
  double acc[18];
  for (int q = 0; q < 18; ++q) acc[q] = 0.0;
  const int ns = sp->ns;
  const double mu = sp->mu, ll = sp->ll, mup = sp->mup;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += (long long)gridDim.x * blockDim.x) {
    double e[3][3], ed[3][3];
    int c = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j, ++c) {
        e[i][j] = E[(long long)c * N + pt].x * sp->inv_n + sp->avepst_sym[i][j];
        e[j][i] = e[i][j];
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) ed[i][j] = 0.0;
    for (int a = 0; a < ns; ++a) {
      const double x = xi[(long long)a * N + pt].x;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) ed[i][j] += sp->eps[a][i][j] * x;
    }
    double d[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) d[i][j] = e[i][j] - ed[i][j];
    const double tr = d[0][0] + d[1][1] + d[2][2];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        // C_ijkl d_kl of the cubic/isotropic C (F:869-877)
        const double s = mu * (d[i][j] + d[j][i]) + (i == j ? ll * tr + mup * d[i][i] : 0.0);
        if (eps_out) eps_out[(long long)(3 * i + j) * N + pt] = e[i][j];
        if (sig_out) sig_out[(long long)(3 * i + j) * N + pt] = s;
        acc[3 * i + j] += e[i][j];
        acc[9 + 3 * i + j] += s;
      }
  }
  for (int q = 0; q < 18; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 18; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 18) partial[(long long)blockIdx.x * 18 + threadIdx.x] = red[threadIdx.x][0];
}

// B(k) of Bmatrix (F:328-412) in closed form:
//   B_ab = (E_ab - t_a^T G t_b) / mu,  t_a = sigma_a f,
//   G_ki = (1/f^2) [delta_ik / (mu + mu' z_k)
//                   - f_i f_k / f^2 / (mu + mu' z_i) / (mu + mu' z_k) (mu + lambda) / kk]
// with z_i = f_i^2 / f^2 and kk = 1 + (mu + lambda) sum_j z_j / (mu + mu' z_j).
__global__ void build_B_kernel(const BBuildParams *__restrict__ bp, BLayout bl, double *Bd, float *Bf) {
  const long long N = bl.N;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int ns = bp->ns;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += stride) {
    const int k3 = (int)(pt % bp->n3), k2 = (int)((pt / bp->n3) % bp->n2), k1 = (int)(pt / ((long long)bp->n3 * bp->n2));
    const double f[3] = {frec_dev(k1, bp->n1, bp->d1), frec_dev(k2, bp->n2, bp->d2), frec_dev(k3, bp->n3, bp->d3)};
    const double f2 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    if (!(f2 > 0)) {
      for (int q = 0; q < bl.P; ++q) {
        const long long bi = b_index(bl, q, pt);
        if (bi < 0) continue;  // held by the mirrored point (tile table)
        if (Bd) Bd[bi] = 0.0;
        if (Bf) Bf[bi] = 0.0f;
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
    int q = 0;
    for (int a = 0; a < ns; ++a)
      for (int b = a; b < ns; ++b, ++q) {
        const long long bi = b_index(bl, q, pt);
        if (bi < 0) continue;
        const double v = (bp->E[a][b] - (t[a][0] * u[b][0] + t[a][1] * u[b][1] + t[a][2] * u[b][2])) * bp->mu_inv;
        if (Bd) Bd[bi] = v;
        if (Bf) Bf[bi] = (float)v;
      }
  }
}

// Host-layout B ([kb][ka][N], FP64, on the device) -> device layout.
__global__ void pack_B_kernel(const double *src, int ns, BLayout bl, double *Bd, float *Bf) {
  const long long N = bl.N;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += stride) {
    int q = 0;
    for (int a = 0; a < ns; ++a)
      for (int b = a; b < ns; ++b, ++q) {
        const long long bi = b_index(bl, q, pt);
        if (bi < 0) continue;  // the mirrored point's value (checked equal on the host)
        const double v = src[((long long)b * ns + a) * N + pt];
        if (Bd) Bd[bi] = v;
        if (Bf) Bf[bi] = (float)v;
      }
  }
}

// Device layout (FP64 or FP32) -> [kb][ka][N] FP64.
__global__ void unpack_B_kernel(const double *Bd, const float *Bf, int ns, BLayout bl, double *dst) {
  const long long N = bl.N;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x; pt < N; pt += stride) {
    int q = 0;
    for (int a = 0; a < ns; ++a)
      for (int b = a; b < ns; ++b, ++q) {
        long long bi = b_index(bl, q, pt);
        if (bi < 0) {  // a mirrored tile's second line: B at the point mirrored through the origin
          const long long x = pt / bl.inner, cc = pt - x * bl.inner;
          const int2 tp = bl.tiles[bl.line_tile[cc] >> 1];
          bi = b_index(bl, q, (long long)b_mirror((int)x, bl.L) * bl.inner + tp.x);
        }
        const double v = Bd ? Bd[bi] : (double)Bf[bi];
        dst[((long long)b * ns + a) * N + pt] = v;
        dst[((long long)a * ns + b) * N + pt] = v;
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
      const unsigned long long lowmask = n == 32 ? 0xffffffffull : ((1ull << n) - 1);
      const unsigned long long m64 = lowmask << sh;
      const unsigned long long p64 = ((unsigned long long)bal & lowmask) << sh;
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

}  // namespace pfdd

using namespace pfdd;

namespace {

// kernels of a step, for the optional per-kernel event timing
enum KId { K_Z_PROLOGUE, K_Z_STEP, K_FFT_Y_FWD, K_FFT_X_FWD, K_CONTRACT, K_FFT_X_INV, K_FFT_Y_INV, K_GAMMA,
           K_X_FUSED, K_PLANE, K_PLANE_PROLOGUE, K_DIAG, K_COUNT };
const char *const kKernelNames[K_COUNT] = {"z_prologue", "z_step", "fft_y_fwd", "fft_x_fwd", "contract",
                                           "fft_x_inv", "fft_y_inv", "gamma_reduce", "x_fused", "plane",
                                           "plane_prologue", "diag_gather"};

struct KTiming {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  std::vector<int> ids;
  size_t used = 0;
  double ms[K_COUNT] = {};
  long long cnt[K_COUNT] = {};
};

}  // namespace

struct pfdd_ctx {
  int n[3] = {0, 0, 0};
  int ns = 0, nrep = 0, prec = 0, dev = 0;
  // replicas a step's grids cover: up to the last active one (idle replicas
  // below it are skipped by the kernels; those above it cost no CTAs at all)
  int krep = 0;
  long long N = 0;
  cudaStream_t st = nullptr;
  void *S = nullptr;
  double2 *xi = nullptr;
  uint32_t *bc = nullptr;
  void *B = nullptr;
  double *tau = nullptr, *gam_a = nullptr, *gam = nullptr;
  long long *part = nullptr;  // fixed-point gamma partials
  double *tau_field = nullptr, *dslip_dev = nullptr;
  uint8_t *active = nullptr;
  int *flag = nullptr, *errflag = nullptr, *h_errflag = nullptr;
  void *tw[3] = {nullptr, nullptr, nullptr};
  double *h_gam_a = nullptr, *h_gam = nullptr, *h_tau = nullptr;
  std::vector<uint8_t> h_active;
  bool hasB = false, hasParams = false, hasState = false, specValid = false, anyBc = false;
  double cd2[kMaxNs] = {}, asf[kMaxNs] = {}, dslip[kMaxNs] = {}, uq2 = 1.0;
  int kchunk = 1;
  Geometry g;
  BLayout bl{};
  // B(k) tile table of the FP32 stored-table form (see BLayout); xtSym: the
  // mirrored layout (B(-k) = B(k)) is in use, else single tiles only
  int2 *xt = nullptr;
  long long *xtoff = nullptr;
  int *xline = nullptr, *xord = nullptr;
  long long ntiles = 0, bvals = 0;
  bool xtSym = true;
  // the step's y passes take the fields from the last down: the z-pass runs
  // them upwards, so each y pass starts on the fields that the pass before it
  // wrote last, which are still in L2 (the x-pass takes every field per tile)
  bool yRev = true;
  BFlyParams bf{};
  long long launches = 0;
  KTiming tm;
  std::string err;
  // step counter on the device (the x-pass advances it, the z-pass reads it),
  // so one captured sequence of steps replays at any position in a chunk
  int *step_ctr = nullptr;
  // captured CUDA graphs of kGraphSteps steps and of one step; rebuilt when a
  // captured argument changes (gen counts those changes)
  cudaGraphExec_t graph_many = nullptr, graph_one = nullptr;
  unsigned gen = 0, graph_gen = ~0u;
  bool primed = false, use_graphs = true;
  // launch plan: tile widths timed on the first step (autotune), as JSON
  // elastic constants, eigenstrains and spacings of pfdd_build_B (strain/stress)
  bool hasElastic = false;
  double Cel[3] = {0, 0, 0}, dsp[3] = {1, 1, 1};
  std::vector<double> epsv;
  bool tuned = false, tune = true;
  int zparts_cap = 0;  // z-pass blocks per field the partial buffer holds
  std::string plan;  // the autotune record of the plan (JSON), reported with the current geometry
  // failure tests, set from the host environment (0 in normal runs):
  // PFDD_TEST_DROP_BULK=1 makes the x-pass's first CTA wait for B-tile bytes
  // that are never copied (its bounded wait runs out: pfdd_step returns
  // PFDD_ETIMEOUT); PFDD_TEST_FAIL_ALLOC=k makes the k-th device or pinned
  // allocation of pfdd_create fail (PFDD_ENOMEM)
  int drop_bulk = 0;
  int alloc_count = 0, fail_alloc_at = 0;
  // work buffers of pfdd_strain_stress, allocated by its first call and kept
  // (a free inside a running server would synchronise the whole device)
  pfdd_fft_plan *sp_plan = nullptr;
  double2 *sp_E = nullptr;
  double *sp_eps = nullptr, *sp_sig = nullptr, *sp_part = nullptr;
  StrainParams *sp_dp = nullptr;
  // interface-plane diagnostics (pfdd_set_diagnostics): the gathered points
  // (the plane's in the reference's row-major order, then the residual line's),
  // the per-step gathers of a chunk and the energies of the last pfdd_step
  bool diagOn = false;
  pfdd_diag_params dgp{};
  std::vector<long long> dpts;
  int dplane = 0, dline = 0;
  long long *d_dpts = nullptr;
  double *d_dgat = nullptr;
  std::vector<double> h_dgat, h_diag;
  int diag_steps = 0;
  // the inner loop's convergence stop (plasticconverge, F:3732-3785), one
  // tracker a replica (pfdd_step_converge, pfdd_step_converge_batched)
  std::vector<ConvergeTracker> cv;
};

// wait limit of the bounded device waits under PFDD_TEST_DROP_BULK (the normal
// limit is kWaitNs)
constexpr unsigned long long kTestWaitNs = 2ull * 1000 * 1000;

struct pfdd_fft_plan {
  int n[3] = {0, 0, 0};
  int prec = 0, dev = 0, max_batch = 0;
  long long N = 0;
  cudaStream_t st = nullptr;
  void *buf = nullptr;
  void *tw[3] = {nullptr, nullptr, nullptr};
  Geometry g;
};

static pfdd_status fail(pfdd_ctx *c, pfdd_status s, const char *fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return s;
}

#define CK(ctx, call)                                                                         \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) {                                                                  \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? PFDD_ENOMEM : PFDD_ECUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                          \
    }                                                                                         \
  } while (0)

// CUDA event pair around one kernel launch (timing mode only)
static void t_begin(pfdd_ctx *c) {
  if (!c->tm.on) return;
  while (c->tm.pool.size() < c->tm.used + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) { c->tm.on = false; return; }
    c->tm.pool.push_back(e);
  }
  cudaEventRecord(c->tm.pool[c->tm.used], c->st);
}
static void t_end(pfdd_ctx *c, int id) {
  c->launches++;
  if (!c->tm.on) return;
  cudaEventRecord(c->tm.pool[c->tm.used + 1], c->st);
  c->tm.ids.push_back(id);
  c->tm.used += 2;
}

// Stockham radices of a line of length n transformed with nv values per
// thread (radix nv while at least nv remain, then the remainder).
static std::string radix_plan(int n, int nv) {
  std::string r;
  int lg = 0;
  while ((1 << lg) < n) ++lg;
  if (lg == 0) return "1";
  const int lgNV = nv == 16 ? 4 : 3;
  while (lg > 0) {
    const int k = lg >= lgNV ? lgNV : lg;
    r += (r.empty() ? "" : "x") + std::to_string(1 << k);
    lg -= k;
  }
  return r;
}

static size_t vsize_of(int prec) { return prec == PFDD_FP64 ? sizeof(double2) : sizeof(float2); }
// bytes of a stored B(k) value; 0: the x-pass evaluates B(k) itself
static size_t bsize_of(int prec) {
  return prec == PFDD_FP64 ? sizeof(double) : (prec == PFDD_FFT_FP32 ? sizeof(float) : 0);
}
static bool prec_ok(int prec) { return prec == PFDD_FP64 || prec == PFDD_FFT_FP32 || prec == PFDD_FFT_FP32_BFLY; }

// The FP32 stored-table form keeps B(k) in the tile-table layout.
static bool uses_tile_table(int prec) { return prec == PFDD_FFT_FP32; }

// B(k) values a context stores (the single-tile table is the largest layout)
static size_t b_values(int n1, int n2, int n3, int ns, int prec) {
  const size_t P = (size_t)ns * (ns + 1) / 2, N = (size_t)n1 * n2 * n3;
  if (!uses_tile_table(prec)) return bsize_of(prec) ? P * N : 0;
  return P * (size_t)n2 * n3 * (size_t)((n1 + 3) / 4 * 4);
}

extern "C" size_t pfdd_required_bytes(int n1, int n2, int n3, int ns, int nrep, int precision) {
  const size_t N = (size_t)n1 * n2 * n3, P = (size_t)ns * (ns + 1) / 2, RF = (size_t)nrep * ns;
  size_t b = RF * N * (sizeof(double2) + vsize_of(precision));  // xi + S
  b += b_values(n1, n2, n3, ns, precision) * bsize_of(precision);  // B
  (void)P;
  b += (RF * N + 31) / 32 * 4;                                   // bc mask
  b += 64u << 20;                                                // partials, tables, slack
  return b;
}

extern "C" const char *pfdd_status_string(int s) {
  switch (s) {
    case PFDD_OK: return "ok";
    case PFDD_EINVAL: return "invalid argument";
    case PFDD_ENOMEM: return "out of memory";
    case PFDD_ECUDA: return "CUDA error";
    case PFDD_ETIMEOUT: return "device wait timed out";
    case PFDD_ENONFINITE: return "state became non-finite";
    case PFDD_ENOTREADY: return "input not set";
    case PFDD_ELIMIT: return "size beyond a fixed capacity";
    default: return "unknown status";
  }
}

extern "C" const char *pfdd_last_error(const pfdd_ctx *c) { return c ? c->err.c_str() : "null context"; }
extern "C" long long pfdd_last_launch_count(const pfdd_ctx *c) { return c ? c->launches : 0; }

static cudaError_t make_twiddles(void **tw, const int n[3], int prec, cudaStream_t st) {
  for (int ax = 0; ax < 3; ++ax) {
    const int L = n[ax];
    cudaError_t e = cudaMalloc(&tw[ax], (size_t)std::max(L, 1) * vsize_of(prec));
    if (e != cudaSuccess) return e;
    if (prec == PFDD_FP64) twiddle_kernel<double><<<(L + 127) / 128, 128, 0, st>>>(tw[ax], L);
    else twiddle_kernel<float><<<(L + 127) / 128, 128, 0, st>>>(tw[ax], L);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
static pfdd_status autotune(pfdd_ctx *c);

// Copies a tile table to the context's device arrays (sized for the single-
// tile table, the largest) and records its tile count.
static cudaError_t upload_tile_table(pfdd_ctx *c, const TileTable &t) {
  cudaError_t e = cudaMemcpyAsync(c->xt, t.tiles.data(), t.tiles.size() * sizeof(int2), cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->xtoff, t.toff.data(), t.toff.size() * sizeof(long long), cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->xline, t.line_tile.data(), t.line_tile.size() * sizeof(int), cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->xord, t.order.data(), t.order.size() * sizeof(int), cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);  // the host vectors go out of scope
  c->ntiles = (long long)t.tiles.size();
  return e;
}

// Switches the FP32 stored-table form between the mirrored tile table and the
// single-tile one (a B(k) without the mirror symmetry); the x-pass grid changes
// with it.
static pfdd_status set_tile_layout(pfdd_ctx *c, bool symmetric) {
  if (!uses_tile_table(c->prec) || c->xtSym == symmetric) return PFDD_OK;
  const TileTable t = make_tile_table(c->n[0], c->n[1], c->n[2], c->ns * (c->ns + 1) / 2, symmetric);
  CK(c, upload_tile_table(c, t));
  c->xtSym = symmetric;
  Geometry g = c->g;
  if (!set_x_geometry(g, c->n[0], c->n[1], c->n[2], c->ns, vsize_of(c->prec), bsize_of(c->prec), g.xLgT, g.xWide,
                      false, c->ntiles))
    return fail(c, PFDD_EINVAL, "B(k) tile layout: the x-pass tile does not fit");
  c->g = g;
  c->gen++;  // captured x-pass launch shape
  return PFDD_OK;
}

// Device and pinned allocations of a context, counted so a failure test can
// make the k-th one fail (PFDD_TEST_FAIL_ALLOC=k) as an exhausted device would.
static cudaError_t ctx_malloc(pfdd_ctx *c, void **p, size_t bytes) {
  if (c->fail_alloc_at > 0 && ++c->alloc_count == c->fail_alloc_at) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}
static cudaError_t ctx_malloc_host(pfdd_ctx *c, void **p, size_t bytes) {
  if (c->fail_alloc_at > 0 && ++c->alloc_count == c->fail_alloc_at) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocHost(p, bytes);
}
template <typename P> static cudaError_t ctx_malloc(pfdd_ctx *c, P **p, size_t bytes) {
  return ctx_malloc(c, reinterpret_cast<void **>(p), bytes);
}
template <typename P> static cudaError_t ctx_malloc_host(pfdd_ctx *c, P **p, size_t bytes) {
  return ctx_malloc_host(c, reinterpret_cast<void **>(p), bytes);
}

extern "C" pfdd_status pfdd_create_batched(pfdd_ctx **out, int n1, int n2, int n3, int ns, int nrep, int precision,
                                           int device) {
  if (!out) return PFDD_EINVAL;
  *out = nullptr;
  if (!pow2_ok(n1) || !pow2_ok(n2) || !pow2_ok(n3) || ns < 1 || ns > 12 || nrep < 1 || !prec_ok(precision))
    return PFDD_EINVAL;
  if (precision == PFDD_FFT_FP32_BFLY && (n1 < 32 || n1 > 256)) return PFDD_EINVAL;
  pfdd_ctx *c = new pfdd_ctx();
  *out = c;
  c->n[0] = n1; c->n[1] = n2; c->n[2] = n3;
  c->ns = ns; c->nrep = nrep; c->krep = nrep; c->prec = precision; c->dev = device;
  c->N = (long long)n1 * n2 * n3;
  if (const char *v = std::getenv("PFDD_TEST_FAIL_ALLOC")) c->fail_alloc_at = std::atoi(v);
  CK(c, cudaSetDevice(device));
  CK(c, cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
  TileTable tt;
  if (uses_tile_table(precision)) {
    tt = make_tile_table(n1, n2, n3, ns * (ns + 1) / 2, true);
    c->ntiles = (long long)tt.tiles.size();
  }
  c->g = make_geometry(n1, n2, n3, ns, vsize_of(precision), bsize_of(precision), /*xfast=*/true, c->ntiles);
  if (!c->g.valid)
    return fail(c, PFDD_EINVAL,
                "pfdd_create: one x-line tile of %d systems x N1=%d with its B(k) does not fit in shared memory in "
                "this precision", ns, n1);
  const size_t RF = (size_t)nrep * ns, N = (size_t)c->N, P = (size_t)ns * (ns + 1) / 2;
  CK(c, ctx_malloc(c, &c->xi, RF * N * sizeof(double2)));
  CK(c, ctx_malloc(c, &c->S, RF * N * vsize_of(precision)));
  c->bvals = (long long)b_values(n1, n2, n3, ns, precision);
  if (c->bvals) CK(c, ctx_malloc(c, &c->B, (size_t)c->bvals * bsize_of(precision)));
  if (uses_tile_table(precision)) {
    const size_t inner = (size_t)n2 * n3;
    CK(c, ctx_malloc(c, &c->xt, inner * sizeof(int2)));
    CK(c, ctx_malloc(c, &c->xtoff, (inner + 1) * sizeof(long long)));
    CK(c, ctx_malloc(c, &c->xline, inner * sizeof(int)));
    CK(c, ctx_malloc(c, &c->xord, inner * sizeof(int)));
    CK(c, upload_tile_table(c, tt));
  }
  CK(c, ctx_malloc(c, &c->active, nrep));
  CK(c, ctx_malloc(c, &c->dslip_dev, kMaxNs * sizeof(double)));
  CK(c, ctx_malloc(c, &c->flag, sizeof(int)));
  CK(c, ctx_malloc(c, &c->errflag, sizeof(int)));
  CK(c, ctx_malloc(c, &c->step_ctr, sizeof(int)));
  if (const char *g = std::getenv("PFDD_NO_GRAPHS")) c->use_graphs = g[0] == '\0' || g[0] == '0';
  if (const char *g = std::getenv("PFDD_NO_TUNE")) c->tune = g[0] == '\0' || g[0] == '0';
  CK(c, cudaMemsetAsync(c->errflag, 0, sizeof(int), c->st));
  CK(c, ctx_malloc_host(c, &c->h_errflag, sizeof(int)));
  // partial sums for a chunk of steps, bounded to ~32 MB; sized for the
  // smallest z-pass block the autotuner may pick (a quarter of the default)
  c->zparts_cap = (int)std::min<long long>((long long)n1 * n2, (long long)c->g.zNparts * 4);
  const size_t per_step = RF * (size_t)c->zparts_cap;
  c->kchunk = (int)std::max<size_t>(1, std::min<size_t>(1024, (4u << 20) / per_step));
  CK(c, ctx_malloc(c, &c->part, per_step * c->kchunk * sizeof(long long)));
  CK(c, ctx_malloc(c, &c->tau, (size_t)c->kchunk * RF * sizeof(double)));
  CK(c, ctx_malloc(c, &c->gam_a, (size_t)c->kchunk * RF * sizeof(double)));
  CK(c, ctx_malloc(c, &c->gam, (size_t)c->kchunk * nrep * sizeof(double)));
  CK(c, ctx_malloc_host(c, &c->h_gam_a, (size_t)c->kchunk * RF * sizeof(double)));
  CK(c, ctx_malloc_host(c, &c->h_gam, (size_t)c->kchunk * nrep * sizeof(double)));
  CK(c, ctx_malloc_host(c, &c->h_tau, (size_t)c->kchunk * RF * sizeof(double)));
  CK(c, make_twiddles(c->tw, c->n, precision, c->st));
  c->h_active.assign(nrep, 1);
  CK(c, cudaMemcpyAsync(c->active, c->h_active.data(), nrep, cudaMemcpyHostToDevice, c->st));
  // tile widths are timed on the (zeroed) buffers before B(k) is laid out in
  // the chosen x-pass tile order
  CK(c, cudaMemsetAsync(c->S, 0, RF * N * vsize_of(precision), c->st));
  if (c->B) CK(c, cudaMemsetAsync(c->B, 0, (size_t)c->bvals * bsize_of(precision), c->st));
  {
    const pfdd_status st = precision == PFDD_FP64 ? autotune<double>(c) : autotune<float>(c);
    if (st != PFDD_OK) return st;
  }
  c->bl = BLayout{c->N, (long long)n2 * n3, n1, c->g.xLgT, ns * (ns + 1) / 2, c->g.xTable ? c->xt : nullptr,
                  c->g.xTable ? c->xtoff : nullptr, c->g.xTable ? c->xline : nullptr};
  (void)P;
  CK(c, cudaStreamSynchronize(c->st));
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_create(pfdd_ctx **out, int n1, int n2, int n3, int ns, int precision, int device) {
  return pfdd_create_batched(out, n1, n2, n3, ns, 1, precision, device);
}

extern "C" void pfdd_destroy(pfdd_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->dev);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->graph_many) cudaGraphExecDestroy(c->graph_many);
  if (c->graph_one) cudaGraphExecDestroy(c->graph_one);
  void *dp[] = {c->S, c->xi, c->bc, c->B, c->tau, c->part, c->gam_a, c->gam, c->tau_field, c->dslip_dev,
                c->active, c->flag, c->errflag, c->step_ctr, c->tw[0], c->tw[1], c->tw[2],
                c->xt, c->xtoff, c->xline, c->xord, c->sp_E, c->sp_eps, c->sp_sig, c->sp_part, c->sp_dp,
                c->d_dpts, c->d_dgat};
  if (c->sp_plan) pfdd_fft_plan_destroy(c->sp_plan);
  if (c->h_errflag) cudaFreeHost(c->h_errflag);
  for (auto &ev : c->tm.pool) cudaEventDestroy(ev);
  for (void *p : dp)
    if (p) cudaFree(p);
  if (c->h_gam_a) cudaFreeHost(c->h_gam_a);
  if (c->h_gam) cudaFreeHost(c->h_gam);
  if (c->h_tau) cudaFreeHost(c->h_tau);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

extern "C" pfdd_status pfdd_set_B(pfdd_ctx *c, const double *B) {
  if (!c || !B) return fail(c, PFDD_EINVAL, "pfdd_set_B: null argument");
  if (c->prec == PFDD_FFT_FP32_BFLY)
    return fail(c, PFDD_EINVAL, "pfdd_set_B: this context evaluates B(k) itself; use pfdd_build_B");
  CK(c, cudaSetDevice(c->dev));
  if (uses_tile_table(c->prec)) {
    // the mirrored tile layout holds one of each pair of points mirrored
    // through the origin (see BLayout): use it only when the given B(k) has
    // the same bits at both (a B(k) from the reference's formula does)
    const int n1 = c->n[0], n2 = c->n[1], n3 = c->n[2], ns = c->ns;
    const long long inner = (long long)n2 * n3, N = c->N;
    bool sym = true;
    for (long long cc = 0; cc < inner && sym; ++cc) {
      const int j = (int)(cc / n3), k = (int)(cc % n3);
      if (j == n2 / 2 || k == n3 / 2) continue;  // Nyquist lines are single tiles
      const long long m = (long long)b_mirror(j, n2) * n3 + b_mirror(k, n3);
      if (m <= cc) continue;
      for (int x = 0; x < n1 && sym; ++x) {
        if (x == n1 / 2) continue;  // stored for both lines
        const long long p1 = (long long)x * inner + cc, p2 = (long long)b_mirror(x, n1) * inner + m;
        for (int aa = 0; aa < ns && sym; ++aa)
          for (int bb = aa; bb < ns; ++bb) {
            const double *row = B + ((long long)bb * ns + aa) * N;
            if (std::memcmp(row + p1, row + p2, sizeof(double)) != 0) { sym = false; break; }
          }
      }
    }
    const pfdd_status st = set_tile_layout(c, sym);
    if (st != PFDD_OK) return st;
  }
  const size_t full = (size_t)c->ns * c->ns * c->N * sizeof(double);
  double *tmp = nullptr;
  CK(c, cudaMalloc(&tmp, full));
  cudaError_t e = cudaMemcpyAsync(tmp, B, full, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) {
    pack_B_kernel<<<1216, kThreads, 0, c->st>>>(tmp, c->ns, c->bl, c->prec == PFDD_FP64 ? (double *)c->B : nullptr,
                                                 c->prec == PFDD_FP64 ? nullptr : (float *)c->B);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaFree(tmp);
  CK(c, e);
  c->hasB = true;
  c->gen++;  // captured x-pass arguments (B(k) constants) may differ
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_get_B(pfdd_ctx *c, double *B) {
  if (!c || !B) return fail(c, PFDD_EINVAL, "pfdd_get_B: null argument");
  if (!c->hasB) return fail(c, PFDD_ENOTREADY, "pfdd_get_B: B(k) not set");
  if (c->prec == PFDD_FFT_FP32_BFLY) return fail(c, PFDD_EINVAL, "pfdd_get_B: no stored B(k) in this context");
  CK(c, cudaSetDevice(c->dev));
  const size_t full = (size_t)c->ns * c->ns * c->N * sizeof(double);
  double *tmp = nullptr;
  CK(c, cudaMalloc(&tmp, full));
  unpack_B_kernel<<<1216, kThreads, 0, c->st>>>(c->prec == PFDD_FP64 ? (const double *)c->B : nullptr,
                                                c->prec == PFDD_FP64 ? nullptr : (const float *)c->B, c->ns, c->bl, tmp);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(B, tmp, full, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaFree(tmp);
  CK(c, e);
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_build_B(pfdd_ctx *c, double C11, double C12, double C44, const double *eps, double d1,
                                    double d2, double d3) {
  if (!c || !eps) return fail(c, PFDD_EINVAL, "pfdd_build_B: null argument");
  if (!(C44 != 0.0) || !(d1 > 0) || !(d2 > 0) || !(d3 > 0)) return fail(c, PFDD_EINVAL, "pfdd_build_B: bad constants");
  CK(c, cudaSetDevice(c->dev));
  BBuildParams hp;
  std::memset(&hp, 0, sizeof hp);
  hp.n1 = c->n[0]; hp.n2 = c->n[1]; hp.n3 = c->n[2]; hp.ns = c->ns;
  hp.d1 = d1; hp.d2 = d2; hp.d3 = d3;
  hp.mu = C44; hp.ll = C12; hp.mup = C11 - C12 - 2 * C44; hp.mu_inv = 1. / hp.mu;
  // C_ijkl of Bmatrix (F:347-357), sigma_a = C : eps_a, E_ab = eps_a : C : eps_b
  double Cc[3][3][3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k)
        for (int m = 0; m < 3; ++m)
          Cc[i][j][k][m] = hp.mu * ((i == k) * (j == m) + (i == m) * (j == k)) + hp.ll * (i == j) * (k == m) +
                           hp.mup * ((i == j) && (j == k) && (k == m));
  for (int a = 0; a < c->ns; ++a)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0;
        for (int m = 0; m < 3; ++m)
          for (int n = 0; n < 3; ++n) s += Cc[i][j][m][n] * eps[(a * 3 + m) * 3 + n];
        hp.sig[a][i][j] = s;
      }
  for (int a = 0; a < c->ns; ++a)
    for (int b = 0; b < c->ns; ++b) {
      double s = 0;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) s += eps[(a * 3 + i) * 3 + j] * hp.sig[b][i][j];
      hp.E[a][b] = s;
    }
  c->Cel[0] = C11; c->Cel[1] = C12; c->Cel[2] = C44;
  c->dsp[0] = d1; c->dsp[1] = d2; c->dsp[2] = d3;
  c->epsv.assign(eps, eps + 9 * c->ns);
  c->hasElastic = true;
  if (c->prec == PFDD_FFT_FP32_BFLY) {  // the x-pass evaluates the same closed form in FP32
    BFlyParams &bf = c->bf;
    bf.n2 = c->n[1]; bf.n3 = c->n[2]; bf.lgN3 = ilog2(c->n[2]);
    bf.d[0] = (float)d1; bf.d[1] = (float)d2; bf.d[2] = (float)d3;
    bf.mu = (float)hp.mu; bf.ll = (float)hp.ll; bf.mup = (float)hp.mup;
    static const int comp[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
    for (int a = 0; a < c->ns; ++a)
      for (int cc = 0; cc < 6; ++cc) {
        const int i = comp[cc][0], j = comp[cc][1];
        const double m = i == j ? 1.0 : 2.0;
        const double se = 0.5 * (eps[(a * 3 + i) * 3 + j] + eps[(a * 3 + j) * 3 + i]);  // eps_a : W = sym(eps_a) : W
        bf.sig6[a][cc] = (float)hp.sig[a][i][j];
        bf.pe6[a][cc] = (float)(m * se * hp.mu_inv);
        bf.qs6[a][cc] = (float)(-m * hp.sig[a][i][j] * hp.mu_inv);
      }
    c->hasB = true;
    return PFDD_OK;
  }
  {
    const pfdd_status st = set_tile_layout(c, true);  // the closed form has B(-k) = B(k) bit for bit
    if (st != PFDD_OK) return st;
  }
  BBuildParams *dp = nullptr;
  CK(c, cudaMalloc(&dp, sizeof hp));
  cudaError_t e = cudaMemcpyAsync(dp, &hp, sizeof hp, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) {
    // a block per 128 points (each CTA short): a grid of SM-long CTAs would hold
    // every SM for the whole build (46 ms at 256^3 x 12), and other contexts'
    // kernels, whatever their stream priority, would wait for it
    const long long blocks = std::min<long long>((c->N + 127) / 128, 0x7fffffffLL);
    build_B_kernel<<<(unsigned)blocks, 128, 0, c->st>>>(dp, c->bl, c->prec == PFDD_FP64 ? (double *)c->B : nullptr,
                                                        c->prec == PFDD_FP64 ? nullptr : (float *)c->B);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaFree(dp);
  CK(c, e);
  c->hasB = true;
  c->gen++;  // captured x-pass arguments (B(k) constants) may differ
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_set_params(pfdd_ctx *c, const double *cd2, const double *asf, const double *dslip,
                                       double uq2) {
  if (!c || !cd2 || !asf || !dslip) return fail(c, PFDD_EINVAL, "pfdd_set_params: null argument");
  for (int a = 0; a < c->ns; ++a) {
    if (!(dslip[a] != 0.0)) return fail(c, PFDD_EINVAL, "pfdd_set_params: dslip[%d] == 0", a);
    c->cd2[a] = cd2[a]; c->asf[a] = asf[a]; c->dslip[a] = dslip[a];
  }
  c->uq2 = uq2;
  CK(c, cudaSetDevice(c->dev));
  CK(c, cudaMemcpyAsync(c->dslip_dev, c->dslip, sizeof(double) * kMaxNs, cudaMemcpyHostToDevice, c->st));
  CK(c, cudaStreamSynchronize(c->st));
  c->hasParams = true;
  c->gen++;  // the captured z-pass arguments hold the coefficients
  return PFDD_OK;
}

// Upload xi (and the pinned mask) of replicas [r0, r0+nr).  xi_bc is staged
// through the spectral buffer S (invalidated by a state change anyway) in
// chunks and packed to bits on the device, so no host pass over it is needed.
// A host <-> device copy of a state in pieces of 64 MB, each waited for before
// the next is queued: the copy engines take copies in the order they are
// queued, so a 3.2 GB state copied in one piece holds up every small copy of
// the other contexts on the device (the server's other classes) until it is
// done; in pieces those go through in between.
static cudaError_t copy_in_pieces(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
  constexpr size_t kPiece = (size_t)64 << 20;
  for (size_t off = 0; off < bytes; off += kPiece) {
    const size_t n = std::min(kPiece, bytes - off);
    cudaError_t e = cudaMemcpyAsync(static_cast<char *>(dst) + off, static_cast<const char *>(src) + off, n, kind, st);
    if (e == cudaSuccess && off + n < bytes) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

static pfdd_status upload_state(pfdd_ctx *c, int r0, int nr, const double *xi, const double *bc) {
  CK(c, cudaSetDevice(c->dev));
  const size_t fieldN = (size_t)c->N, RFn = (size_t)nr * c->ns;
  CK(c, copy_in_pieces(c->xi + (size_t)r0 * c->ns * fieldN, xi, RFn * fieldN * sizeof(double2),
                       cudaMemcpyHostToDevice, c->st));
  const size_t total_bits = (size_t)c->nrep * c->ns * fieldN, words = (total_bits + 31) / 32;
  if (bc && !c->bc) {
    CK(c, cudaMalloc(&c->bc, words * 4));
    CK(c, cudaMemsetAsync(c->bc, 0, words * 4, c->st));
  }
  if (c->bc) {
    const size_t count = RFn * fieldN, b0 = (size_t)r0 * c->ns * fieldN;
    if (!bc) {
      // every point of these replicas evolves: clear their bits
      CK(c, cudaMemsetAsync(c->S, 0, std::min(count, (size_t)c->nrep * c->ns * fieldN * vsize_of(c->prec) / 16) * 16,
                            c->st));
    }
    const size_t chunk = (size_t)c->nrep * c->ns * fieldN * vsize_of(c->prec) / (2 * sizeof(double));
    for (size_t off = 0; off < count; off += chunk) {
      const size_t n = std::min(chunk, count - off);
      if (bc) CK(c, copy_in_pieces(c->S, bc + 2 * off, n * 2 * sizeof(double), cudaMemcpyHostToDevice, c->st));
      pack_bc_kernel<<<1216, kThreads, 0, c->st>>>((const double *)c->S, (long long)n, (long long)(b0 + off), c->bc);
      CK(c, cudaGetLastError());
    }
    CK(c, cudaMemsetAsync(c->flag, 0, sizeof(int), c->st));
    mask_any_kernel<<<304, kThreads, 0, c->st>>>(c->bc, (long long)words, c->flag);
    CK(c, cudaGetLastError());
    int any = 0;
    CK(c, cudaMemcpyAsync(&any, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    if (c->anyBc != (any != 0)) c->gen++;  // the captured z-pass reads the mask or not
    c->anyBc = any != 0;
  }
  CK(c, cudaStreamSynchronize(c->st));
  c->hasState = true;
  c->specValid = false;
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_set_state(pfdd_ctx *c, const double *xi, const double *bc) {
  if (!c || !xi) return fail(c, PFDD_EINVAL, "pfdd_set_state: null argument");
  return upload_state(c, 0, c->nrep, xi, bc);
}

extern "C" pfdd_status pfdd_set_replica_state(pfdd_ctx *c, int r, const double *xi, const double *bc) {
  if (!c || !xi || r < 0 || r >= c->nrep) return fail(c, PFDD_EINVAL, "pfdd_set_replica_state: bad argument");
  return upload_state(c, r, 1, xi, bc);
}

extern "C" pfdd_status pfdd_set_tau_field(pfdd_ctx *c, const double *tf) {
  if (!c) return PFDD_EINVAL;
  CK(c, cudaSetDevice(c->dev));
  if (!tf) {
    if (c->tau_field) CK(c, cudaFree(c->tau_field));
    c->tau_field = nullptr;
    c->gen++;
    return PFDD_OK;
  }
  const size_t N = (size_t)c->N, ns = (size_t)c->ns;
  std::vector<double> t(ns * N);
  for (size_t pt = 0; pt < N; ++pt)
    for (size_t a = 0; a < ns; ++a) t[a * N + pt] = tf[pt * ns + a];
  if (!c->tau_field) {
    CK(c, cudaMalloc(&c->tau_field, ns * N * sizeof(double)));
    c->gen++;
  }
  CK(c, cudaMemcpyAsync(c->tau_field, t.data(), ns * N * sizeof(double), cudaMemcpyHostToDevice, c->st));
  CK(c, cudaStreamSynchronize(c->st));
  return PFDD_OK;
}

// Grid extent of a step: replicas up to the last active one (at least one,
// so an all-idle step still launches valid, empty grids).
static void update_krep(pfdd_ctx *c) {
  int k = 0;
  for (int r = 0; r < c->nrep; ++r)
    if (c->h_active[r]) k = r + 1;
  k = std::max(k, 1);
  if (k != c->krep) {
    c->krep = k;
    c->gen++;  // captured grid sizes change
  }
}

extern "C" pfdd_status pfdd_set_replica_active(pfdd_ctx *c, int r, int on) {
  if (!c || r < 0 || r >= c->nrep) return fail(c, PFDD_EINVAL, "pfdd_set_replica_active: bad replica");
  // a replica that was idle when the spectral buffer was last rebuilt from xi
  // has no spectral state: the next step rebuilds it
  if (on && !c->h_active[r]) c->specValid = false;
  c->h_active[r] = on ? 1 : 0;
  update_krep(c);
  CK(c, cudaSetDevice(c->dev));
  CK(c, cudaMemcpyAsync(c->active, c->h_active.data(), c->nrep, cudaMemcpyHostToDevice, c->st));
  CK(c, cudaStreamSynchronize(c->st));
  return PFDD_OK;
}

static int prec_code(int prec) { return prec == PFDD_FP64 ? 0 : 1; }

static cudaError_t ctx_zpass(pfdd_ctx *c, ZParams &zp, int flags) {
  zp.flags = flags;
  const long long blocks = (long long)c->krep * c->ns * c->g.zNparts;
  t_begin(c);
  cudaError_t e =
      launch_zpass(prec_code(c->prec), c->g.lgL3, (unsigned)blocks, c->g.zThreads, c->g.zSmem, c->st, zp, c->g.zNV);
  t_end(c, (flags & Z_UPDATE) ? K_Z_STEP : K_Z_PROLOGUE);
  return e;
}

static cudaError_t ctx_strided(pfdd_ctx *c, int sign, int ax /*0: y, 1: x*/) {
  const int L = ax == 0 ? c->n[1] : c->n[0];
  if (L == 1) return cudaSuccess;
  const int gi = ax == 0 ? 0 : 1;
  // y lines: stride N3*N1 in the x-fastest layout, N3 in the natural one
  const long long inner = ax == 0 ? (c->g.xfast ? (long long)c->n[2] * c->n[0] : (long long)c->n[2])
                                  : (long long)c->n[1] * c->n[2];
  const long long outer = ax == 0 ? (long long)c->krep * c->ns * (c->g.xfast ? 1 : c->n[0])
                                  : (long long)c->krep * c->ns;
  const long long outer_per_rep = outer / c->krep;
  const long long blocks = outer * c->g.tiles[gi];
  t_begin(c);
  cudaError_t e = launch_strided(prec_code(c->prec), sign, ilog2(L), (unsigned)blocks, c->g.threads[gi], c->g.smem[gi],
                                 c->st, c->S, c->g.lgTI[gi], inner, c->g.tiles[gi], c->tw[ax == 0 ? 1 : 0],
                                 c->active, outer_per_rep, c->g.pitch[gi], ax == 0 && c->yRev, c->g.nv[gi]);
  t_end(c, ax == 0 ? (sign < 0 ? K_FFT_Y_FWD : K_FFT_Y_INV) : (sign < 0 ? K_FFT_X_FWD : K_FFT_X_INV));
  return e;
}

template <typename T>
static cudaError_t launch_x_fused(pfdd_ctx *c) {
  XParams xp;
  xp.S = c->S; xp.B = c->B; xp.active = c->active; xp.tw = c->tw[0];
  xp.xt = c->g.xTable ? c->xt : nullptr;
  xp.xtoff = c->g.xTable ? c->xtoff : nullptr;
  xp.xline = c->g.xTable ? c->xline : nullptr;
  xp.xord = c->g.xTable ? c->xord : nullptr;
  xp.inner = (long long)c->n[1] * c->n[2]; xp.tiles = c->g.xTiles;
  xp.L = c->n[0]; xp.lgL = ilog2(c->n[0]); xp.lgT = c->g.xLgT; xp.pitch = c->g.xPitch; xp.R = c->krep;
  xp.step_ctr = c->step_ctr;
  const unsigned blocks = (unsigned)(c->krep * c->g.xTiles);
  t_begin(c);
  xp.bf = c->bf;
  xp.err = c->errflag;
  xp.drop_bulk = c->drop_bulk;
  xp.bsplit = c->g.xSplit ? c->ns * (c->ns + 1) / 4 : 0;  // P / 2 pair rows first
  xp.wait_ns = c->drop_bulk ? kTestWaitNs : kWaitNs;
  cudaError_t e = c->g.xWarp
                      ? launch_x_warp_f32(c->ns, c->prec == PFDD_FFT_FP32_BFLY, blocks, c->g.xThreads, c->g.xSmem, c->st, xp)
                  : c->prec == PFDD_FFT_FP32_BFLY
                      ? launch_x_fused_f32_bfly(c->ns, blocks, c->g.xThreads, c->g.xSmem, c->st, xp)
                      : (std::is_same<T, float>::value
                             ? launch_x_fused_f32(c->ns, blocks, c->g.xThreads, c->g.xSmem, c->st, xp)
                             : launch_x_fused_f64(c->ns, blocks, c->g.xThreads, c->g.xSmem, c->st, xp));
  t_end(c, K_X_FUSED);
  return e;
}

constexpr int kGraphSteps = 16;

// z-pass arguments of a step of this context (the step index comes from the
// device counter that the x-pass advances)
static ZParams make_zparams(const pfdd_ctx *c) {
  ZParams zp;
  std::memset(&zp, 0, sizeof zp);
  zp.S = c->S; zp.xi = c->xi; zp.bc = c->anyBc ? c->bc : nullptr; zp.tau = c->tau; zp.tau_field = c->tau_field;
  zp.dslip = c->dslip_dev; zp.part = c->part; zp.err = c->errflag;
  zp.active = c->active;
  zp.step_ctr = c->step_ctr;
  zp.tw = c->tw[2];
  zp.N = c->N; zp.lines_per_field = (long long)c->n[0] * c->n[1];
  zp.L = c->n[2]; zp.lgL = c->g.lgL3; zp.ns = c->ns; zp.R = c->nrep; zp.TL = c->g.zTL; zp.nparts = c->g.zNparts;
  zp.pitch = c->g.zPitch;
  zp.sxf = c->g.xfast ? 1 : 0;
  zp.n1 = c->n[0]; zp.n2 = c->n[1]; zp.lgTL = ilog2(c->g.zTL);
  zp.inv_n = 1.0 / (double)c->N;  // N is a power of two: exact, same as dividing by nsize
  zp.uq2 = c->uq2;
  for (int a = 0; a < c->ns; ++a) {
    zp.cd2[a] = c->cd2[a];
    zp.asf_pi[a] = c->asf[a] * kPiTrunc;  // Asf2[isa]*pi, F:3488
    zp.uq2cd2[a] = c->uq2 * c->cd2[a];    // uq2*CD2[isa], F:3489
  }
  return zp;
}

static std::string plan_json(const pfdd_ctx *c, const std::string &tuning) {
  const Geometry &g = c->g;
  const int vs = (int)vsize_of(c->prec), lgx = ilog2(c->n[0]);
  const int xnv = lgx >= 5 && lgx <= 8 ? xpass_nv(lgx, vs) : 8;  // the x-pass's compiled-in lengths
  char b[1024];  // the fixed part; the autotune timings follow
  snprintf(b, sizeof b,
           "{\"x_pass\": {\"tile_columns\": %d, \"threads\": %d, \"smem\": %zu, \"ctas\": %lld, \"warp_teams\": %d, "

           "\"b_tiles\": %lld, \"b_mirrored\": %d, \"b_split\": %d}, "
           "\"y_pass\": {\"tile_columns\": %d, \"threads\": %d, \"smem\": %zu, \"tiles_per_field\": %lld}, "
           "\"z_pass\": {\"lines\": %d, \"threads\": %d, \"smem\": %zu}, "
           "\"radix_plan\": [\"%s\", \"%s\", \"%s\"], \"graph_steps\": %d, \"autotune\": ",
           1 << g.xLgT, g.xThreads, g.xSmem, (long long)c->nrep * g.xTiles, (int)g.xWarp,
           g.xTable ? c->ntiles : 0LL, (int)(g.xTable && c->xtSym), (int)g.xSplit, 1 << g.lgTI[0], g.threads[0], g.smem[0],
           g.tiles[0], g.zTL, g.zThreads, g.zSmem, radix_plan(c->n[0], xnv).c_str(),
           radix_plan(c->n[1], g.nv[0] ? g.nv[0] : fft_nv(ilog2(c->n[1]))).c_str(),
           radix_plan(c->n[2], g.zNV ? g.zNV : zpass_nv(ilog2(c->n[2]), vs)).c_str(), kGraphSteps);
  return std::string(b) + tuning + "}";
}

// Tuned plans by grid shape (N1, N2, N3, ns, precision, device): a process
// times each shape once; later contexts of the shape (serving classes, batch
// re-creation) reuse the plan instead of timing under whatever else is running.
struct TunedPlan {
  int zTL, xLgT, yLgTI, zNV, yNV;
  bool xWide, xWarp, xSplit;
  std::string timings;
};
static std::mutex g_plan_mu;
static std::map<std::string, TunedPlan> g_plans;

static std::string plan_key(const pfdd_ctx *c) {
  return std::to_string(c->n[0]) + "x" + std::to_string(c->n[1]) + "x" + std::to_string(c->n[2]) + "/" +
         std::to_string(c->ns) + "/" + std::to_string(c->prec) + "/" + std::to_string(c->dev);
}

// Times every tile width of the fused x-pass and of the y-pass that fits, on
// the context's own buffers (3 launches each after one warm-up), and keeps the
// fastest.  Tile widths change no result: every line and every point is
// computed by the same instructions whatever the tile.  The trial launches
// overwrite the spectral buffer, which the next step rebuilds from xi.
// A pinned radix plan with the widest tile (z lines per block, y columns) up
// to the current one that fits its thread count.
static bool pin_z_radix(const pfdd_ctx *c, Geometry &g, size_t vs, int nv) {
  for (int TL = g.zTL; TL >= 1; TL >>= 1)
    if (set_z_geometry(g, c->n[0], c->n[1], c->n[2], vs, TL, nv) && g.zNparts <= c->zparts_cap) return true;
  return false;
}
static bool pin_y_radix(const pfdd_ctx *c, Geometry &g, size_t vs, int nv) {
  for (int lgTI = g.lgTI[0]; lgTI >= 0; --lgTI)
    if (set_strided_geometry(g, 0, c->n[1], (long long)c->n[2] * c->n[0], lgTI, vs, nv)) return true;
  return false;
}

template <typename T>
static pfdd_status autotune(pfdd_ctx *c) {
  c->tuned = true;
  std::string tuning = "null";
  // PFDD_PLAN="z=<lines>,n=<8|16>,x=<tile columns>,w=<0|1|2>,y=<tile columns>,m=<8|16>,f=<0|1>"
  // pins the plan (each entry optional, ignored when it does not fit; n and m:
  // values a thread of the z-pass and the y passes, the radix plans; w=1, the
  // warp-team x-pass, after x, w=2 the same with its B block in two halves;
  // f=0, the y passes in ascending field order)
  // instead of timing it, e.g. to profile the plan a timed run chose (a
  // profiler distorts the timings)
  if (const char *pin = std::getenv("PFDD_PLAN")) {
    const size_t vs = vsize_of(c->prec), bs = bsize_of(c->prec);
    for (const char *q = pin; *q;) {
      char key = 0;
      int v = 0;
      const bool kv = std::sscanf(q, "%c=%d", &key, &v) == 2;
      if (kv && key == 'f') c->yRev = v != 0;
      if (kv && v > 0) {
        Geometry g = c->g;
        const long long tt = uses_tile_table(c->prec) ? c->ntiles : 0;
        const bool ok = key == 'z'   ? set_z_geometry(g, c->n[0], c->n[1], c->n[2], vs, v, g.zNV) &&
                                           g.zNparts <= c->zparts_cap
                        : key == 'n' ? pin_z_radix(c, g, vs, v)
                        : key == 'm' ? pin_y_radix(c, g, vs, v)
                        : key == 'x' ? set_x_geometry(g, c->n[0], c->n[1], c->n[2], c->ns, vs, bs, ilog2(v), false,
                                                      false, tt)
                        : key == 'w' ? set_x_geometry(g, c->n[0], c->n[1], c->n[2], c->ns, vs, bs, g.xLgT, false,
                                                      v >= 1, tt, v == 2)
                        : key == 'y' ? set_strided_geometry(g, 0, c->n[1], (long long)c->n[2] * c->n[0], ilog2(v), vs,
                                                            g.nv[0])
                                     : false;
        if (ok) c->g = g;
      }
      const char *comma = std::strchr(q, ',');
      if (!comma) break;
      q = comma + 1;
    }
    c->gen++;
    c->plan = "\"pinned\"";
    return PFDD_OK;
  }
  if (c->tune) {
    const size_t vs = vsize_of(c->prec), bs = bsize_of(c->prec);
    const std::string key = plan_key(c);
    {
      std::lock_guard<std::mutex> lk(g_plan_mu);
      auto it = g_plans.find(key);
      if (it != g_plans.end()) {
        Geometry g = c->g;
        if (set_z_geometry(g, c->n[0], c->n[1], c->n[2], vs, it->second.zTL, it->second.zNV) &&
            g.zNparts <= c->zparts_cap &&
            set_x_geometry(g, c->n[0], c->n[1], c->n[2], c->ns, vs, bs, it->second.xLgT, it->second.xWide,
                           it->second.xWarp, uses_tile_table(c->prec) ? c->ntiles : 0, it->second.xSplit) &&
            (c->n[1] == 1 ||
             set_strided_geometry(g, 0, c->n[1], (long long)c->n[2] * c->n[0], it->second.yLgTI, vs,
                                  it->second.yNV))) {
          c->g = g;
          c->gen++;
          c->plan = "{\"cached\": true, \"timings\": " + it->second.timings + "}";
          return PFDD_OK;
        }
      }
    }
    const bool timing = c->tm.on;
    c->tm.on = false;
    const long long l0 = c->launches;
    cudaEvent_t e0, e1;
    CK(c, cudaEventCreate(&e0));
    CK(c, cudaEventCreate(&e1));
    auto time_us = [&](auto launch) -> double {
      if (launch() != cudaSuccess) { cudaGetLastError(); return -1.0; }
      cudaEventRecord(e0, c->st);
      for (int i = 0; i < 3; ++i)
        if (launch() != cudaSuccess) { cudaGetLastError(); return -1.0; }
      cudaEventRecord(e1, c->st);
      if (cudaEventSynchronize(e1) != cudaSuccess) return -1.0;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      return 1e3 * ms / 3.0;
    };
    std::string xs, ys, zs;
    Geometry best = c->g;
    double bt = 1e30;
    // the timings take one replica (the kernels skip idle ones), so tuning a
    // batched context costs what tuning one solve does
    const int krep_saved = c->krep;
    if (c->nrep > 1) {
      std::vector<uint8_t> one(c->nrep, 0);
      one[0] = 1;
      CK(c, cudaMemcpyAsync(c->active, one.data(), c->nrep, cudaMemcpyHostToDevice, c->st));
      CK(c, cudaStreamSynchronize(c->st));
      c->krep = 1;  // grids over replica 0 alone
    }
    // z-pass lines per block (the gamma partials are exact integer sums, so
    // the split of points into blocks changes no result); a typical state
    // (0.5) and zero stresses so the update takes its usual path
    fill_u64_kernel<<<1216, kThreads, 0, c->st>>>(reinterpret_cast<unsigned long long *>(c->xi),
                                                  (long long)c->ns * c->N * 2, 0x3fe0000000000000ull);
    cudaMemsetAsync(c->tau, 0, (size_t)c->nrep * c->ns * sizeof(double), c->st);
    // z-pass lines per block and radix plan (values a thread: 8, 16): the
    // plans round differently, the line counts change no result
    for (int cand = 0; cand < 2 * 6; ++cand) {
      const int lgTL = cand >> 1, nv = (cand & 1) ? 16 : 8;
      Geometry g = c->g;
      if (!set_z_geometry(g, c->n[0], c->n[1], c->n[2], vs, 1 << lgTL, nv) || g.zNparts > c->zparts_cap) continue;
      c->g = g;
      ZParams zp = make_zparams(c);
      zp.step_ctr = nullptr;
      zp.step = 0;
      const double us = time_us([&] { return ctx_zpass(c, zp, Z_INV | Z_UPDATE | Z_FWD | Z_STORE); });
      if (us > 0 && us < bt) { bt = us; best = g; }
      char b[64];
      snprintf(b, sizeof b, "%s\"%d/%d\": %.1f", zs.empty() ? "" : ", ", 1 << lgTL, nv, us);
      zs += b;
    }
    c->g = best;
    bt = 1e30;
    // tile widths 1..64, each with the block-team kernel (plain and wide) and
    // the warp-team kernel (key suffix "v"; "s": its B block in two halves, for
    // a fourth CTA on an SM); all compute the same bits
    for (int cand = 0; cand <= 4 * 7 - 1; ++cand) {
      const int lgT = cand / 4, form = cand % 4;
      const bool wide = form == 1, warp = form >= 2, split = form == 3;
      Geometry g = c->g;
      if (!set_x_geometry(g, c->n[0], c->n[1], c->n[2], c->ns, vs, bs, lgT, wide, warp,
                          uses_tile_table(c->prec) ? c->ntiles : 0, split))
        continue;
      c->g = g;
      const double us = time_us([&] { return launch_x_fused<T>(c); });
      if (us > 0 && us < bt) { bt = us; best = g; }
      char b[64];
      snprintf(b, sizeof b, "%s\"%d%s\": %.1f", xs.empty() ? "" : ", ", 1 << lgT,
               wide ? "w" : (split ? "s" : (warp ? "v" : "")), us);
      xs += b;
    }
    c->g = best;
    if (c->n[1] > 1) {
      bt = 1e30;
      for (int cand = 0; cand < 2 * 8; ++cand) {
        const int lgTI = cand >> 1, nv = (cand & 1) ? 16 : 8;
        Geometry g = c->g;
        if (!set_strided_geometry(g, 0, c->n[1], (long long)c->n[2] * c->n[0], lgTI, vs, nv)) continue;
        c->g = g;
        const double us = time_us([&] { return ctx_strided(c, -1, 0); });
        if (us > 0 && us < bt) { bt = us; best = g; }
        char b[64];
        snprintf(b, sizeof b, "%s\"%d/%d\": %.1f", ys.empty() ? "" : ", ", 1 << lgTI, nv, us);
        ys += b;
      }
      c->g = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->launches = l0;
    c->tm.on = timing;
    if (c->nrep > 1) {  // every replica active again
      CK(c, cudaMemcpyAsync(c->active, c->h_active.data(), c->nrep, cudaMemcpyHostToDevice, c->st));
      CK(c, cudaStreamSynchronize(c->st));
      c->krep = krep_saved;
    }
    c->specValid = false;
    c->gen++;  // captured launch shapes change
    tuning = "{\"z_pass_us_by_lines\": {" + zs + "}, \"x_pass_us_by_tile\": {" + xs + "}, \"y_pass_us_by_tile\": {" +
             ys + "}}";
    {
      std::lock_guard<std::mutex> lk(g_plan_mu);
      g_plans[key] = TunedPlan{c->g.zTL, c->g.xLgT, c->g.lgTI[0], c->g.zNV, c->g.nv[0],
                               c->g.xWide, c->g.xWarp, c->g.xSplit, tuning};
    }
    cudaMemsetAsync(c->errflag, 0, sizeof(int), c->st);
  }
  c->plan = tuning;
  return PFDD_OK;
}

static cudaError_t launch_diag_gather(pfdd_ctx *c, const int *step_ctr) {
  const int RF = c->nrep * c->ns, npts = (int)c->dpts.size();
  const long long per = (long long)RF * npts;
  const int blocks = (int)std::max<long long>(1, std::min<long long>(152, (per + 255) / 256));
  t_begin(c);
  diag_gather_kernel<<<blocks, 256, 0, c->st>>>(c->xi, c->d_dpts, npts, RF, c->N, step_ctr, c->d_dgat);
  t_end(c, K_DIAG);
  return cudaGetLastError();
}

// Energies of the gathered values g (field a's point q at g[a * npts + q]) in
// the reference's order of summation (avestrain F:641-749 for the plane sums,
// ResidualEnergy F:3920-3945 for the line): out[6] = energy_in, energy_in2,
// energy_in3, energy_in4 (one call's worth), energy_Residual, their sum.
static void diag_energies(const pfdd_ctx *c, const double *g, double *out) {
  const pfdd_diag_params &d = c->dgp;
  const int ns = c->ns, npts = (int)c->dpts.size(), nspm = d.ns_per_material > 0 ? d.ns_per_material : ns;
  auto dl = [](int i, int j) { return i == j ? 1 : 0; };
  auto dl4 = [](int i, int j, int k, int l) { return (i == j && j == k && k == l) ? 1 : 0; };
  double S[3][3][3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l)
          S[i][j][k][l] = (d.S11 + 2 * d.S12) / 3.0 * dl(i, j) * dl(k, l) +
                          d.S44 / 4.0 * (dl(i, k) * dl(j, l) + dl(i, l) * dl(j, k)) - d.S44 / 2.0 * dl4(i, j, k, l) +
                          (d.S11 - d.S12) * (dl4(i, j, k, l) - dl(i, j) * dl(k, l) / 3.0);
  double e3 = 0.0, e4 = 0.0;
  for (int q = 0; q < c->dplane; ++q) {
    double sp[3][3];
    for (int u = 0; u < 3; ++u)
      for (int v = 0; v < 3; ++v) {
        sp[u][v] = 0.0;
        for (int a = 0; a < ns; ++a) sp[u][v] += g[(size_t)a * npts + q] * c->epsv[(a * 3 + u) * 3 + v];
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        e3 += -(sp[i][j] + 0.0) * (d.sigma[i][j]);  // + the virtual strain, zero here
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) e4 += -S[i][j][k][l] * d.sigma[k][l] * d.sigma[i][j] * 0.5 * d.mu;
      }
  }
  const double D00 = d.D[0], D01 = d.D[1], D10 = d.D[2], D11 = d.D[3];
  double er = 0.0;
  for (int j = 0; j < c->dline; ++j) {
    double x0 = 0.0, x1 = 0.0;
    for (int a = 0; a < ns; ++a) {
      const int m = a / nspm;
      if (m == 0) x0 += g[(size_t)a * npts + c->dplane + j];
      if (m == 1) x1 += g[(size_t)a * npts + c->dplane + j];
    }
    er = er + std::fabs(-D11 * x1 * x1 + (D10 + D01) * x1 * x0 - D00 * x0 * x0);
  }
  out[0] = 0.0;  // energy_in: no virtual strain fields
  out[1] = 0.0;  // energy_in2: no virtual strain fields
  out[2] = e3;
  out[3] = e4;
  out[4] = er;
  out[5] = out[0] + out[1] + out[2] + out[3] + out[4];
}

// The launches of one TDGL step (step index taken from the device counter).
template <typename T>
static cudaError_t launch_step(pfdd_ctx *c, ZParams &zp) {
  cudaError_t e = ctx_strided(c, -1, 0);
  if (e == cudaSuccess) e = launch_x_fused<T>(c);
  if (e == cudaSuccess) e = ctx_strided(c, +1, 0);
  if (e == cudaSuccess) e = ctx_zpass(c, zp, Z_INV | Z_UPDATE | Z_FWD | Z_STORE);
  if (e == cudaSuccess && c->diagOn) e = launch_diag_gather(c, c->step_ctr);
  return e;
}

// Captures `steps` steps on the context's stream into an executable graph.
template <typename T>
static cudaError_t capture_steps(pfdd_ctx *c, ZParams &zp, int steps, cudaGraphExec_t *out) {
  cudaError_t e = cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t le = cudaSuccess;
  for (int s = 0; s < steps && le == cudaSuccess; ++s) le = launch_step<T>(c, zp);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(c->st, &g);
  if (le != cudaSuccess) e = le;
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  return e;
}

template <typename T>
static pfdd_status run_steps(pfdd_ctx *c, int nsteps, const double *tau, double *gamma, double *gamma_a) {
  ZParams zp = make_zparams(c);
  const int RF = c->nrep * c->ns;
  const size_t dper = (size_t)RF * c->dpts.size();  // gathered values per step (diagnostics)
  if (c->diagOn) {
    c->h_diag.assign((size_t)nsteps * c->nrep * 6, 0.0);
    c->diag_steps = nsteps;
  }
  if (!c->specValid) {
    CK(c, ctx_zpass(c, zp, Z_SRC_XI | Z_FWD | Z_STORE));
    c->specValid = true;
  }
  for (int s0 = 0; s0 < nsteps; s0 += c->kchunk) {
    const int ks = std::min(c->kchunk, nsteps - s0);
    // per-step stress table: tau/dslip (F:3488) or the tau-field multiplier
    for (int s = 0; s < ks; ++s)
      for (int r = 0; r < c->nrep; ++r)
        for (int a = 0; a < c->ns; ++a) {
          const double t = tau[((size_t)(s0 + s) * c->nrep + r) * c->ns + a];
          c->h_tau[((size_t)s * c->nrep + r) * c->ns + a] = c->tau_field ? t : t / c->dslip[a];
        }
    CK(c, cudaMemcpyAsync(c->tau, c->h_tau, (size_t)ks * RF * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(c, cudaMemsetAsync(c->step_ctr, 0xff, sizeof(int), c->st));  // -1: the first x-pass makes it 0
    int done = 0;
    const bool direct = c->tm.on || !c->use_graphs;
    if (direct || !c->primed) {
      // direct launches: timing mode, and the first step of a context (it
      // also sets every kernel's shared-memory opt-in before any capture)
      const int n = direct ? ks : 1;
      for (; done < n; ++done) CK(c, launch_step<T>(c, zp));
      c->primed = true;
    }
    if (done < ks) {
      if (c->graph_gen != c->gen) {
        if (c->graph_many) cudaGraphExecDestroy(c->graph_many);
        if (c->graph_one) cudaGraphExecDestroy(c->graph_one);
        c->graph_many = c->graph_one = nullptr;
        const long long l0 = c->launches;
        CK(c, capture_steps<T>(c, zp, kGraphSteps, &c->graph_many));
        CK(c, capture_steps<T>(c, zp, 1, &c->graph_one));
        c->launches = l0;  // captured, not launched
        c->graph_gen = c->gen;
      }
      const int per_step = 4 + (c->diagOn ? 1 : 0);
      for (; done + kGraphSteps <= ks; done += kGraphSteps) {
        CK(c, cudaGraphLaunch(c->graph_many, c->st));
        c->launches += (long long)per_step * kGraphSteps;
      }
      for (; done < ks; ++done) {
        CK(c, cudaGraphLaunch(c->graph_one, c->st));
        c->launches += per_step;
      }
    }
    const int nt = ks * c->nrep;
    t_begin(c);
    gamma_reduce_kernel<<<nt, kGammaWarps * 32 * c->ns, 0, c->st>>>(c->part, c->g.zNparts, c->nrep, c->ns,
                                                                   0x1p-44 * zp.inv_n, c->gam_a, c->gam);
    t_end(c, K_GAMMA);
    CK(c, cudaGetLastError());
    CK(c, cudaMemcpyAsync(c->h_gam_a, c->gam_a, (size_t)ks * RF * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaMemcpyAsync(c->h_gam, c->gam, (size_t)nt * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaMemcpyAsync(c->h_errflag, c->errflag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    if (*c->h_errflag) {
      CK(c, cudaMemsetAsync(c->errflag, 0, sizeof(int), c->st));
      CK(c, cudaStreamSynchronize(c->st));
      c->specValid = false;
      return fail(c, PFDD_ETIMEOUT, "pfdd_step: a bounded device wait for a bulk copy ran out within steps %d..%d",
                  s0, s0 + ks - 1);
    }
    bool finite = true;
    for (int q = 0; q < nt; ++q)
      if (c->h_active[q % c->nrep] && !std::isfinite(c->h_gam[q])) finite = false;
    if (c->diagOn) {
      CK(c, cudaMemcpyAsync(c->h_dgat.data(), c->d_dgat, (size_t)ks * dper * sizeof(double), cudaMemcpyDeviceToHost,
                            c->st));
      CK(c, cudaStreamSynchronize(c->st));
      for (int s = 0; s < ks; ++s)
        for (int r = 0; r < c->nrep; ++r)
          diag_energies(c, c->h_dgat.data() + ((size_t)s * c->nrep + r) * c->ns * c->dpts.size(),
                        c->h_diag.data() + (((size_t)(s0 + s)) * c->nrep + r) * 6);
    }
    if (gamma) std::memcpy(gamma + (size_t)s0 * c->nrep, c->h_gam, (size_t)nt * sizeof(double));
    if (gamma_a) std::memcpy(gamma_a + (size_t)s0 * RF, c->h_gam_a, (size_t)ks * RF * sizeof(double));
    if (!finite) return fail(c, PFDD_ENONFINITE, "pfdd_step: state became non-finite within steps %d..%d", s0, s0 + ks - 1);
  }
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_step(pfdd_ctx *c, int nsteps, const double *tau, double *gamma, double *gamma_a) {
  if (!c || nsteps < 0 || (nsteps > 0 && !tau)) return fail(c, PFDD_EINVAL, "pfdd_step: bad argument");
  if (!c->hasB) return fail(c, PFDD_ENOTREADY, "pfdd_step: B(k) not set");
  if (!c->hasParams) return fail(c, PFDD_ENOTREADY, "pfdd_step: parameters not set");
  if (!c->hasState) return fail(c, PFDD_ENOTREADY, "pfdd_step: state not set");
  c->launches = 0;
  if (nsteps == 0) return PFDD_OK;
  {
    const char *v = std::getenv("PFDD_TEST_DROP_BULK");
    const int want = v && v[0] && v[0] != '0';
    if (want != c->drop_bulk) {
      c->drop_bulk = want;
      c->gen++;  // captured x-pass arguments
    }
  }
  CK(c, cudaSetDevice(c->dev));
  return c->prec == PFDD_FP64 ? run_steps<double>(c, nsteps, tau, gamma, gamma_a)
                              : run_steps<float>(c, nsteps, tau, gamma, gamma_a);
}

static void ensure_trackers(pfdd_ctx *c) {
  if ((int)c->cv.size() != c->nrep) c->cv.assign(c->nrep, ConvergeTracker());
}

extern "C" pfdd_status pfdd_converge_reset(pfdd_ctx *c, double gamma_prev) {
  if (!c) return PFDD_EINVAL;
  ensure_trackers(c);
  for (auto &t : c->cv) t.reset(gamma_prev);
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_converge_reset_batched(pfdd_ctx *c, const double *gamma_prev) {
  if (!c || !gamma_prev) return fail(c, PFDD_EINVAL, "pfdd_converge_reset_batched: null argument");
  ensure_trackers(c);
  for (int r = 0; r < c->nrep; ++r) c->cv[r].reset(gamma_prev[r]);
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_step_converge(pfdd_ctx *c, int max_steps, const double *tau, double *gamma,
                                          double *gamma_a, int *steps_done) {
  if (!c || max_steps < 0 || (max_steps > 0 && (!tau || !gamma)) || !steps_done)
    return fail(c, PFDD_EINVAL, "pfdd_step_converge: bad argument");
  if (c->nrep != 1) return fail(c, PFDD_EINVAL, "pfdd_step_converge: one solve per context (nrep == 1)");
  return pfdd_step_converge_batched(c, max_steps, tau, gamma, gamma_a, steps_done);
}

extern "C" pfdd_status pfdd_step_converge_batched(pfdd_ctx *c, int max_steps, const double *tau, double *gamma,
                                                  double *gamma_a, int *steps_done) {
  if (!c || max_steps < 0 || (max_steps > 0 && (!tau || !gamma)) || !steps_done)
    return fail(c, PFDD_EINVAL, "pfdd_step_converge_batched: bad argument");
  const int R = c->nrep, ns = c->ns;
  for (int r = 0; r < R; ++r) steps_done[r] = 0;
  if (max_steps == 0) return PFDD_OK;
  if (!c->hasState) return fail(c, PFDD_ENOTREADY, "pfdd_step_converge_batched: state not set");
  ensure_trackers(c);
  // the replicas that take part: the active ones; each leaves (idle, its state
  // kept) at its stop, and the ones that left are active again at the end
  std::vector<uint8_t> run(R, 0), left(R, 0);
  for (int r = 0; r < R; ++r) run[r] = c->h_active[r];
  std::vector<double> g, ga;
  int done = 0;
  pfdd_status st = PFDD_OK;
  while (done < max_steps) {
    // a chunk no longer than the fewest steps to any running replica's next
    // possible stop: a replica can stop at its last step at the earliest
    int k = std::min(c->kchunk, max_steps - done), nrun = 0;
    for (int r = 0; r < R; ++r)
      if (run[r]) {
        k = std::min(k, c->cv[r].min_steps());
        ++nrun;
      }
    if (!nrun) break;
    g.assign((size_t)k * R, 0.0);
    ga.assign((size_t)k * R * ns, 0.0);
    st = pfdd_step(c, k, tau + (size_t)done * R * ns, g.data(), ga.data());
    if (st != PFDD_OK) break;
    for (int r = 0; r < R; ++r) {
      if (!run[r]) continue;
      int stop = -1;
      for (int j = 0; j < k; ++j) {
        gamma[(size_t)(done + j) * R + r] = g[(size_t)j * R + r];
        if (gamma_a)
          for (int a = 0; a < ns; ++a)
            gamma_a[((size_t)(done + j) * R + r) * ns + a] = ga[((size_t)j * R + r) * ns + a];
        if (c->cv[r].update(g[(size_t)j * R + r])) stop = j;
      }
      steps_done[r] = done + k;
      if (stop >= 0 && stop != k - 1) {
        st = fail(c, PFDD_EINVAL, "pfdd_step_converge: replica %d stops at step %d inside a chunk of %d", r,
                  done + stop, k);
        break;
      }
      if (stop >= 0) {
        run[r] = 0;
        if (R > 1) {
          st = pfdd_set_replica_active(c, r, 0);
          if (st != PFDD_OK) break;
          left[r] = 1;
        }
      }
    }
    if (st != PFDD_OK) break;
    done += k;
  }
  for (int r = 0; r < R; ++r)
    if (left[r]) {
      const pfdd_status e = pfdd_set_replica_active(c, r, 1);
      if (st == PFDD_OK) st = e;
    }
  return st;
}

extern "C" pfdd_status pfdd_get_plan(pfdd_ctx *c, char *buf, size_t len) {
  if (!c || !buf || len == 0) return fail(c, PFDD_EINVAL, "pfdd_get_plan: bad argument");
  const std::string p = plan_json(c, c->tuned ? c->plan : std::string("null"));
  if (p.size() + 1 > len) return fail(c, PFDD_EINVAL, "pfdd_get_plan: buffer of %zu bytes, need %zu", len, p.size() + 1);
  std::memcpy(buf, p.c_str(), p.size() + 1);
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_set_diagnostics(pfdd_ctx *c, const pfdd_diag_params *p) {
  if (!c) return PFDD_EINVAL;
  if (!p) {
    if (c->diagOn) c->gen++;  // captured steps lose the gather
    c->diagOn = false;
    return PFDD_OK;
  }
  if (!c->hasElastic) return fail(c, PFDD_ENOTREADY, "pfdd_set_diagnostics: needs the eigenstrains of pfdd_build_B");
  const int n1 = c->n[0], n2 = c->n[1], n3 = c->n[2];
  for (int ax = 0; ax < 3; ++ax)
    if (p->ppoint[ax] < 0 || p->ppoint[ax] >= c->n[ax])
      return fail(c, PFDD_EINVAL, "pfdd_set_diagnostics: ppoint outside the grid");
  if (p->ns_per_material < 0) return fail(c, PFDD_EINVAL, "pfdd_set_diagnostics: ns_per_material < 0");
  // the plane's points in the reference's row-major order (avestrain's test,
  // F:691 and F:702), then the residual line (ppoint_x, j, ppoint_z), j ascending
  std::vector<long long> pts;
  const double *nv = p->interface_n;
  for (int k1 = 0; k1 < n1; ++k1)
    for (int k2 = 0; k2 < n2; ++k2)
      for (int k3 = 0; k3 < n3; ++k3)
        if (std::fabs(nv[0] * (k1 - p->ppoint[0]) + nv[1] * (k2 - p->ppoint[1]) + nv[2] * (k3 - p->ppoint[2])) <= 1.0 &&
            k1 == p->ppoint[0])
          pts.push_back(((long long)k1 * n2 + k2) * n3 + k3);
  const int nplane = (int)pts.size();
  for (int j = 0; j < n2; ++j) pts.push_back(((long long)p->ppoint[0] * n2 + j) * n3 + p->ppoint[2]);
  CK(c, cudaSetDevice(c->dev));
  CK(c, cudaStreamSynchronize(c->st));
  if (c->d_dpts) CK(c, cudaFree(c->d_dpts));
  if (c->d_dgat) CK(c, cudaFree(c->d_dgat));
  c->d_dpts = nullptr;
  c->d_dgat = nullptr;
  const size_t dper = (size_t)c->nrep * c->ns * pts.size();
  CK(c, cudaMalloc(&c->d_dpts, pts.size() * sizeof(long long)));
  CK(c, cudaMalloc(&c->d_dgat, (size_t)c->kchunk * dper * sizeof(double)));
  CK(c, cudaMemcpy(c->d_dpts, pts.data(), pts.size() * sizeof(long long), cudaMemcpyHostToDevice));
  c->h_dgat.assign((size_t)c->kchunk * dper, 0.0);
  c->dpts = pts;
  c->dplane = nplane;
  c->dline = n2;
  c->dgp = *p;
  c->diagOn = true;
  c->diag_steps = 0;
  c->gen++;  // captured steps gain the gather
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_get_diagnostics(pfdd_ctx *c, int nsteps, double *out) {
  if (!c || !out || nsteps < 0) return fail(c, PFDD_EINVAL, "pfdd_get_diagnostics: bad argument");
  if (!c->diagOn || nsteps != c->diag_steps)
    return fail(c, PFDD_ENOTREADY, "pfdd_get_diagnostics: no diagnostics of a %d-step call", nsteps);
  std::memcpy(out, c->h_diag.data(), (size_t)nsteps * c->nrep * 6 * sizeof(double));
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_state_diagnostics(pfdd_ctx *c, double *out) {
  if (!c || !out) return fail(c, PFDD_EINVAL, "pfdd_state_diagnostics: bad argument");
  if (!c->diagOn) return fail(c, PFDD_ENOTREADY, "pfdd_state_diagnostics: diagnostics not set");
  if (!c->hasState) return fail(c, PFDD_ENOTREADY, "pfdd_state_diagnostics: state not set");
  CK(c, cudaSetDevice(c->dev));
  CK(c, launch_diag_gather(c, nullptr));
  const size_t per = (size_t)c->ns * c->dpts.size();
  CK(c, cudaMemcpyAsync(c->h_dgat.data(), c->d_dgat, (size_t)c->nrep * per * sizeof(double), cudaMemcpyDeviceToHost,
                        c->st));
  CK(c, cudaStreamSynchronize(c->st));
  for (int r = 0; r < c->nrep; ++r) diag_energies(c, c->h_dgat.data() + (size_t)r * per, out + (size_t)r * 6);
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_get_state(pfdd_ctx *c, double *xi) {
  if (!c || !xi) return fail(c, PFDD_EINVAL, "pfdd_get_state: null argument");
  CK(c, cudaSetDevice(c->dev));
  CK(c, copy_in_pieces(xi, c->xi, (size_t)c->nrep * c->ns * c->N * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
  CK(c, cudaStreamSynchronize(c->st));
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_get_replica_state(pfdd_ctx *c, int r, double *xi) {
  if (!c || !xi || r < 0 || r >= c->nrep) return fail(c, PFDD_EINVAL, "pfdd_get_replica_state: bad argument");
  CK(c, cudaSetDevice(c->dev));
  const size_t fl = (size_t)c->ns * c->N;
  CK(c, copy_in_pieces(xi, c->xi + (size_t)r * fl, fl * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
  CK(c, cudaStreamSynchronize(c->st));
  return PFDD_OK;
}

extern "C" void *pfdd_get_stream(pfdd_ctx *c) { return c ? (void *)c->st : nullptr; }

extern "C" pfdd_status pfdd_set_stream_priority(pfdd_ctx *c, int priority) {
  if (!c) return PFDD_EINVAL;
  CK(c, cudaSetDevice(c->dev));
  int lo = 0, hi = 0;  // least, greatest (numerically lowest) priority
  CK(c, cudaDeviceGetStreamPriorityRange(&lo, &hi));
  priority = std::min(lo, std::max(hi, priority));
  cudaStream_t ns = nullptr;
  CK(c, cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, priority));
  cudaError_t e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) {
    cudaStreamDestroy(ns);
    CK(c, e);
  }
  cudaStreamDestroy(c->st);
  c->st = ns;
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_set_kernel_timing(pfdd_ctx *c, int enable) {
  if (!c) return PFDD_EINVAL;
  c->tm.on = enable != 0;
  c->tm.used = 0;
  c->tm.ids.clear();
  for (int k = 0; k < K_COUNT; ++k) { c->tm.ms[k] = 0; c->tm.cnt[k] = 0; }
  return PFDD_OK;
}

extern "C" pfdd_status pfdd_kernel_stat(pfdd_ctx *c, int idx, const char **name, long long *launches,
                                        double *total_ms) {
  if (!c || idx < 0 || idx >= K_COUNT) return PFDD_EINVAL;
  if (c->tm.used) {  // fold recorded event pairs into the totals
    CK(c, cudaStreamSynchronize(c->st));
    for (size_t q = 0; q < c->tm.ids.size(); ++q) {
      float ms = 0.f;
      CK(c, cudaEventElapsedTime(&ms, c->tm.pool[2 * q], c->tm.pool[2 * q + 1]));
      c->tm.ms[c->tm.ids[q]] += ms;
      c->tm.cnt[c->tm.ids[q]] += 1;
    }
    c->tm.used = 0;
    c->tm.ids.clear();
  }
  if (name) *name = kKernelNames[idx];
  if (launches) *launches = c->tm.cnt[idx];
  if (total_ms) *total_ms = c->tm.ms[idx];
  return PFDD_OK;
}

// ---------------------------------------------------------------------------
// FFT boundary (fft_forward / fft_backward of F:209-273)

extern "C" pfdd_status pfdd_fft_plan_create(pfdd_fft_plan **out, int n1, int n2, int n3, int precision,
                                            int max_batch, int device) {
  if (!out) return PFDD_EINVAL;
  *out = nullptr;
  if (!pow2_ok(n1) || !pow2_ok(n2) || !pow2_ok(n3) || max_batch < 1 ||
      (precision != PFDD_FP64 && precision != PFDD_FFT_FP32))
    return PFDD_EINVAL;
  pfdd_fft_plan *p = new pfdd_fft_plan();
  p->n[0] = n1; p->n[1] = n2; p->n[2] = n3;
  p->prec = precision; p->dev = device; p->max_batch = max_batch;
  p->N = (long long)n1 * n2 * n3;
  p->g = make_geometry(n1, n2, n3, 0, vsize_of(precision), bsize_of(precision));
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&p->buf, (size_t)max_batch * p->N * vsize_of(precision));
  if (e == cudaSuccess) e = make_twiddles(p->tw, p->n, precision, p->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->st);
  if (e != cudaSuccess) {
    pfdd_fft_plan_destroy(p);
    return e == cudaErrorMemoryAllocation ? PFDD_ENOMEM : PFDD_ECUDA;
  }
  *out = p;
  return PFDD_OK;
}

extern "C" void pfdd_fft_plan_destroy(pfdd_fft_plan *p) {
  if (!p) return;
  cudaSetDevice(p->dev);
  if (p->st) cudaStreamSynchronize(p->st);
  if (p->buf) cudaFree(p->buf);
  for (void *t : p->tw)
    if (t) cudaFree(t);
  if (p->st) cudaStreamDestroy(p->st);
  delete p;
}

static cudaError_t fft_exec(pfdd_fft_plan *p, void *dbuf, int batch, int sign) {
  const Geometry &g = p->g;
  const int pc = prec_code(p->prec);
  ZParams zp;
  std::memset(&zp, 0, sizeof zp);
  zp.S = dbuf; zp.tw = p->tw[2]; zp.N = p->N; zp.lines_per_field = (long long)p->n[0] * p->n[1];
  zp.L = p->n[2]; zp.lgL = g.lgL3; zp.ns = batch; zp.R = 1; zp.TL = g.zTL; zp.nparts = g.zNparts; zp.pitch = g.zPitch;
  const unsigned zblocks = (unsigned)((long long)batch * g.zNparts);
  auto strided = [&](int ax, int s) -> cudaError_t {
    const int L = ax == 0 ? p->n[1] : p->n[0];
    if (L == 1) return cudaSuccess;
    const int gi = ax == 0 ? 0 : 1;
    const long long inner = ax == 0 ? (long long)p->n[2] : (long long)p->n[1] * p->n[2];
    const long long outer = ax == 0 ? (long long)batch * p->n[0] : (long long)batch;
    const long long blocks = outer * g.tiles[gi];
    return launch_strided(pc, s, ilog2(L), (unsigned)blocks, g.threads[gi], g.smem[gi], p->st, dbuf, g.lgTI[gi], inner,
                          g.tiles[gi], p->tw[ax == 0 ? 1 : 0], nullptr, outer, g.pitch[gi]);
  };
  cudaError_t e;
  if (sign < 0) {
    zp.flags = Z_FWD | Z_STORE;
    if ((e = launch_zpass(pc, g.lgL3, zblocks, g.zThreads, g.zSmem, p->st, zp)) != cudaSuccess) return e;
    if ((e = strided(0, -1)) != cudaSuccess) return e;
    return strided(1, -1);
  }
  if ((e = strided(1, +1)) != cudaSuccess) return e;
  if ((e = strided(0, +1)) != cudaSuccess) return e;
  zp.flags = Z_INV | Z_STORE;
  return launch_zpass(pc, g.lgL3, zblocks, g.zThreads, g.zSmem, p->st, zp);
}

static pfdd_status fft_call(pfdd_fft_plan *p, void *data, int batch, int on_device, int sign) {
  if (!p || !data || batch < 1 || batch > p->max_batch) return PFDD_EINVAL;
  if (cudaSetDevice(p->dev) != cudaSuccess) return PFDD_ECUDA;
  const size_t bytes = (size_t)batch * p->N * vsize_of(p->prec);
  void *d = on_device ? data : p->buf;
  cudaError_t e = cudaSuccess;
  if (!on_device) e = cudaMemcpyAsync(d, data, bytes, cudaMemcpyHostToDevice, p->st);
  if (e == cudaSuccess) e = fft_exec(p, d, batch, sign);
  if (e == cudaSuccess && !on_device) e = cudaMemcpyAsync(data, d, bytes, cudaMemcpyDeviceToHost, p->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->st);
  return e == cudaSuccess ? PFDD_OK : PFDD_ECUDA;
}

extern "C" pfdd_status pfdd_fft_forward(pfdd_fft_plan *p, void *data, int batch, int on_device) {
  return fft_call(p, data, batch, on_device, -1);
}
extern "C" pfdd_status pfdd_fft_backward(pfdd_fft_plan *p, void *data, int batch, int on_device) {
  return fft_call(p, data, batch, on_device, +1);
}

// ---- strain and stress fields of a state (strain F:752-835, stress F:837-972)

extern "C" pfdd_status pfdd_strain_stress(pfdd_ctx *c, int r, const double *sigma_app, double *eps, double *sigma,
                                          double *aveps, double *avesigma) {
  if (!c || !sigma_app || r < 0 || r >= c->nrep) return fail(c, PFDD_EINVAL, "pfdd_strain_stress: bad argument");
  if (!c->hasElastic)
    return fail(c, PFDD_ENOTREADY, "pfdd_strain_stress: needs the elastic constants and eigenstrains of pfdd_build_B");
  if (!c->hasState) return fail(c, PFDD_ENOTREADY, "pfdd_strain_stress: state not set");
  CK(c, cudaSetDevice(c->dev));
  CK(c, cudaStreamSynchronize(c->st));  // the state is current
  const int ns = c->ns;
  const long long N = c->N;
  const double C11 = c->Cel[0], C12 = c->Cel[1], C44 = c->Cel[2];
  StrainParams hp;
  std::memset(&hp, 0, sizeof hp);
  hp.n1 = c->n[0]; hp.n2 = c->n[1]; hp.n3 = c->n[2]; hp.ns = ns;
  hp.d1 = c->dsp[0]; hp.d2 = c->dsp[1]; hp.d3 = c->dsp[2];
  hp.mu = C44; hp.ll = C12; hp.mup = C11 - C12 - 2 * C44;
  hp.inv_n = 1.0 / (double)N;
  double Cc[3][3][3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k)
        for (int m = 0; m < 3; ++m)
          Cc[i][j][k][m] = hp.mu * ((i == k) * (j == m) + (i == m) * (j == k)) + hp.ll * (i == j) * (k == m) +
                           hp.mup * ((i == j) && (j == k) && (k == m));
  for (int a = 0; a < ns; ++a)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0;
        for (int m = 0; m < 3; ++m)
          for (int n = 0; n < 3; ++n) s += Cc[i][j][m][n] * c->epsv[(a * 3 + m) * 3 + n];
        hp.sig[a][i][j] = s;
        hp.eps[a][i][j] = c->epsv[(a * 3 + i) * 3 + j];
      }
  // FP64 work: a natural-layout FFT plan whose buffer holds the state's
  // transform, the six strain components and the outputs; allocated by the
  // first call, kept by the context
  if (!c->sp_plan) {
    pfdd_status st = pfdd_fft_plan_create(&c->sp_plan, c->n[0], c->n[1], c->n[2], PFDD_FP64, std::max(ns, 6), c->dev);
    if (st != PFDD_OK) {
      c->sp_plan = nullptr;
      return fail(c, st, "pfdd_strain_stress: work buffers (%s)", pfdd_status_string(st));
    }
  }
  pfdd_fft_plan *p = c->sp_plan;
  const int blocks = (int)std::min<long long>(1216, (N + 255) / 256);
  if (!c->sp_E) CK(c, cudaMalloc(&c->sp_E, 6 * N * sizeof(double2)));
  if (eps && !c->sp_eps) CK(c, cudaMalloc(&c->sp_eps, 9 * N * sizeof(double)));
  if (sigma && !c->sp_sig) CK(c, cudaMalloc(&c->sp_sig, 9 * N * sizeof(double)));
  if (!c->sp_part) CK(c, cudaMalloc(&c->sp_part, 1216 * 18 * sizeof(double)));
  if (!c->sp_dp) CK(c, cudaMalloc(&c->sp_dp, sizeof(StrainParams)));
  double2 *E = c->sp_E;
  double *d_eps = eps ? c->sp_eps : nullptr, *d_sig = sigma ? c->sp_sig : nullptr, *part = c->sp_part;
  StrainParams *dp = c->sp_dp;
  std::vector<double2> dc(ns);
  std::vector<double> hpart((size_t)blocks * 18);
  double2 *W = reinterpret_cast<double2 *>(p->buf);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(W, c->xi + (size_t)r * ns * N, (size_t)ns * N * sizeof(double2), cudaMemcpyDeviceToDevice, p->st);
  if (e == cudaSuccess) e = fft_exec(p, W, ns, -1);
  // the k = 0 coefficients are the field sums: <Re xi_a> for avepsd (avestrain, F:670-688)
  for (int a = 0; e == cudaSuccess && a < ns; ++a)
    e = cudaMemcpyAsync(&dc[a], W + (size_t)a * N, sizeof(double2), cudaMemcpyDeviceToHost, p->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->st);
  if (e == cudaSuccess) {
    // avepst = S : sigma_app mu + avepsd (F:726-741), S of F:661-664 with S11, S12, S44 of F:4261-4263
    const double S11 = 1. / 3. * (1 / (C11 + 2 * C12) + 2 / (C11 - C12));
    const double S12 = 1. / 3. * (1 / (C11 + 2 * C12) - 1 / (C11 - C12));
    const double S44 = 1 / C44;
    double avepst[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.;
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) {
            const double dij = i == j, dkl = k == l, d4 = (i == j) && (j == k) && (k == l);
            const double Sijkl = (S11 + 2 * S12) / 3.0 * dij * dkl + S44 / 4.0 * ((i == k) * (j == l) + (i == l) * (j == k)) -
                                 S44 / 2.0 * d4 + (S11 - S12) * (d4 - dij * dkl / 3.0);
            s += Sijkl * sigma_app[3 * k + l] * C44;
          }
        double ad = 0.;
        for (int a = 0; a < ns; ++a) ad += hp.eps[a][i][j] * (dc[a].x / (double)N);
        avepst[i][j] = s + ad;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) hp.avepst_sym[i][j] = 0.5 * (avepst[i][j] + avepst[j][i]);
    e = cudaMemcpyAsync(dp, &hp, sizeof hp, cudaMemcpyHostToDevice, p->st);
  }
  if (e == cudaSuccess) {
    strain_spec_kernel<<<1216, 256, 0, p->st>>>(dp, W, E, N);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = fft_exec(p, E, 6, +1);
  if (e == cudaSuccess) {
    strain_real_kernel<<<blocks, 256, 0, p->st>>>(dp, E, c->xi + (size_t)r * ns * N, d_eps, d_sig, part, N);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && eps) e = cudaMemcpyAsync(eps, d_eps, 9 * N * sizeof(double), cudaMemcpyDeviceToHost, p->st);
  if (e == cudaSuccess && sigma) e = cudaMemcpyAsync(sigma, d_sig, 9 * N * sizeof(double), cudaMemcpyDeviceToHost, p->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(hpart.data(), part, hpart.size() * sizeof(double), cudaMemcpyDeviceToHost, p->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->st);
  if (e == cudaSuccess) {
    for (int q = 0; q < 9; ++q) {
      double se = 0., ss = 0.;
      for (int b = 0; b < blocks; ++b) {
        se += hpart[(size_t)b * 18 + q];
        ss += hpart[(size_t)b * 18 + 9 + q];
      }
      if (aveps) aveps[q] = se / (double)N;
      if (avesigma) avesigma[q] = ss / (double)N;
    }
  }
  CK(c, e);
  return PFDD_OK;
}
