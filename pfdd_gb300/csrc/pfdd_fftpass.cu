// pfdd_fftpass.cu -- instantiations of the z-pass and strided FFT passes for
// every line length 2^0 .. 2^9 and both spectral precisions.
#include "pfdd_launch.h"

namespace pfdd {

template <typename T, int LG>
static cudaError_t zpass_lg(unsigned blocks, int threads, size_t smem, cudaStream_t st, const ZParams &p) {
  static SmemOptIn configured;
  cudaError_t e = ensure_smem(zpass_kernel<T, LG>, smem, configured);
  if (e != cudaSuccess) return e;
  return launch_pdl(zpass_kernel<T, LG>, blocks, threads, smem, st, p);
}

template <typename T>
static cudaError_t zpass_t(int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st, const ZParams &p) {
  switch (lgL) {
    case 0: return zpass_lg<T, 0>(blocks, threads, smem, st, p);
    case 1: return zpass_lg<T, 1>(blocks, threads, smem, st, p);
    case 2: return zpass_lg<T, 2>(blocks, threads, smem, st, p);
    case 3: return zpass_lg<T, 3>(blocks, threads, smem, st, p);
    case 4: return zpass_lg<T, 4>(blocks, threads, smem, st, p);
    case 5: return zpass_lg<T, 5>(blocks, threads, smem, st, p);
    case 6: return zpass_lg<T, 6>(blocks, threads, smem, st, p);
    case 7: return zpass_lg<T, 7>(blocks, threads, smem, st, p);
    case 8: return zpass_lg<T, 8>(blocks, threads, smem, st, p);
    case 9: return zpass_lg<T, 9>(blocks, threads, smem, st, p);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_zpass(int prec, int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                         const ZParams &p) {
  return prec == 0 ? zpass_t<double>(lgL, blocks, threads, smem, st, p)
                   : zpass_t<float>(lgL, blocks, threads, smem, st, p);
}

struct StridedArgs {
  void *data;
  int lgTI;
  long long inner, tiles;
  const void *tw;
  const uint8_t *active;
  long long outer_per_rep;
  int pitch, rev;
};

template <typename T, int S, int LG>
static cudaError_t strided_lg(unsigned blocks, int threads, size_t smem, cudaStream_t st, const StridedArgs &a) {
  static SmemOptIn configured;
  cudaError_t e = ensure_smem(fft_strided_kernel<T, S, LG>, smem, configured);
  if (e != cudaSuccess) return e;
  return launch_pdl(fft_strided_kernel<T, S, LG>, blocks, threads, smem, st, a.data, LG, a.lgTI, a.inner, a.tiles,
                    a.tw, a.active, a.outer_per_rep, a.pitch, a.rev);
}

template <typename T, int S>
static cudaError_t strided_t(int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                             const StridedArgs &a) {
  switch (lgL) {
    case 0: return strided_lg<T, S, 0>(blocks, threads, smem, st, a);
    case 1: return strided_lg<T, S, 1>(blocks, threads, smem, st, a);
    case 2: return strided_lg<T, S, 2>(blocks, threads, smem, st, a);
    case 3: return strided_lg<T, S, 3>(blocks, threads, smem, st, a);
    case 4: return strided_lg<T, S, 4>(blocks, threads, smem, st, a);
    case 5: return strided_lg<T, S, 5>(blocks, threads, smem, st, a);
    case 6: return strided_lg<T, S, 6>(blocks, threads, smem, st, a);
    case 7: return strided_lg<T, S, 7>(blocks, threads, smem, st, a);
    case 8: return strided_lg<T, S, 8>(blocks, threads, smem, st, a);
    case 9: return strided_lg<T, S, 9>(blocks, threads, smem, st, a);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_strided(int prec, int sign, int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                           void *data, int lgTI, long long inner, long long tiles_per_outer, const void *tw,
                           const uint8_t *active, long long outer_per_rep, int pitch, bool rev) {
  const StridedArgs a{data, lgTI, inner, tiles_per_outer, tw, active, outer_per_rep, pitch, rev ? 1 : 0};
  if (prec == 0)
    return sign < 0 ? strided_t<double, -1>(lgL, blocks, threads, smem, st, a)
                    : strided_t<double, +1>(lgL, blocks, threads, smem, st, a);
  return sign < 0 ? strided_t<float, -1>(lgL, blocks, threads, smem, st, a)
                  : strided_t<float, +1>(lgL, blocks, threads, smem, st, a);
}

}  // namespace pfdd
