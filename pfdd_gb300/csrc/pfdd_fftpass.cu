// pfdd_fftpass.cu -- instantiations of the strided FFT passes for every line
// length 2^0 .. 2^9, both spectral precisions, both signs and both radix plans
// (8 or 16 values a thread; 16 from L = 16 on).
#include "pfdd_launch.h"

namespace pfdd {

struct StridedArgs {
  void *data;
  int lgTI;
  long long inner, tiles;
  const void *tw;
  const uint8_t *active;
  long long outer_per_rep;
  int pitch, rev;
};

template <typename T, int S, int LG, int NV>
static cudaError_t strided_lg(unsigned blocks, int threads, size_t smem, cudaStream_t st, const StridedArgs &a) {
  static SmemOptIn configured;
  cudaError_t e = ensure_smem(fft_strided_kernel<T, S, LG, NV>, smem, configured);
  if (e != cudaSuccess) return e;
  return launch_pdl(fft_strided_kernel<T, S, LG, NV>, blocks, threads, smem, st, a.data, LG, a.lgTI, a.inner,
                    a.tiles, a.tw, a.active, a.outer_per_rep, a.pitch, a.rev);
}

template <typename T, int S, int LG>
static cudaError_t strided_nv(int nv, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                              const StridedArgs &a) {
  if constexpr (LG >= 4) {
    if (nv == 16) return strided_lg<T, S, LG, 16>(blocks, threads, smem, st, a);
  }
  if (nv != 8) return cudaErrorInvalidValue;
  return strided_lg<T, S, LG, 8>(blocks, threads, smem, st, a);
}

template <typename T, int S>
static cudaError_t strided_t(int lgL, int nv, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                             const StridedArgs &a) {
  switch (lgL) {
    case 0: return strided_nv<T, S, 0>(nv, blocks, threads, smem, st, a);
    case 1: return strided_nv<T, S, 1>(nv, blocks, threads, smem, st, a);
    case 2: return strided_nv<T, S, 2>(nv, blocks, threads, smem, st, a);
    case 3: return strided_nv<T, S, 3>(nv, blocks, threads, smem, st, a);
    case 4: return strided_nv<T, S, 4>(nv, blocks, threads, smem, st, a);
    case 5: return strided_nv<T, S, 5>(nv, blocks, threads, smem, st, a);
    case 6: return strided_nv<T, S, 6>(nv, blocks, threads, smem, st, a);
    case 7: return strided_nv<T, S, 7>(nv, blocks, threads, smem, st, a);
    case 8: return strided_nv<T, S, 8>(nv, blocks, threads, smem, st, a);
    case 9: return strided_nv<T, S, 9>(nv, blocks, threads, smem, st, a);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_strided(int prec, int sign, int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                           void *data, int lgTI, long long inner, long long tiles_per_outer, const void *tw,
                           const uint8_t *active, long long outer_per_rep, int pitch, bool rev, int nv) {
  const StridedArgs a{data, lgTI, inner, tiles_per_outer, tw, active, outer_per_rep, pitch, rev ? 1 : 0};
  if (nv == 0) nv = fft_nv(lgL);
  if (prec == 0)
    return sign < 0 ? strided_t<double, -1>(lgL, nv, blocks, threads, smem, st, a)
                    : strided_t<double, +1>(lgL, nv, blocks, threads, smem, st, a);
  return sign < 0 ? strided_t<float, -1>(lgL, nv, blocks, threads, smem, st, a)
                  : strided_t<float, +1>(lgL, nv, blocks, threads, smem, st, a);
}

}  // namespace pfdd
