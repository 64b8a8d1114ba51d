// pfdd_zpass.cu -- instantiations of the z-pass for every line length
// 2^0 .. 2^9, both spectral precisions and both radix plans (8 or 16 values a
// thread; 16 from L = 16 on).
#include "pfdd_launch.h"

namespace pfdd {

template <typename T, int LG, int NV>
static cudaError_t zpass_lg(unsigned blocks, int threads, size_t smem, cudaStream_t st, const ZParams &p) {
  static SmemOptIn configured;
  cudaError_t e = ensure_smem(zpass_kernel<T, LG, NV>, smem, configured);
  if (e != cudaSuccess) return e;
  return launch_pdl(zpass_kernel<T, LG, NV>, blocks, threads, smem, st, p);
}

template <typename T, int LG>
static cudaError_t zpass_nv_lg(int nv, unsigned blocks, int threads, size_t smem, cudaStream_t st, const ZParams &p) {
  if constexpr (LG >= 4) {
    if (nv == 16) return zpass_lg<T, LG, 16>(blocks, threads, smem, st, p);
  }
  if (nv != 8) return cudaErrorInvalidValue;
  return zpass_lg<T, LG, 8>(blocks, threads, smem, st, p);
}

template <typename T>
static cudaError_t zpass_t(int lgL, int nv, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                           const ZParams &p) {
  switch (lgL) {
    case 0: return zpass_nv_lg<T, 0>(nv, blocks, threads, smem, st, p);
    case 1: return zpass_nv_lg<T, 1>(nv, blocks, threads, smem, st, p);
    case 2: return zpass_nv_lg<T, 2>(nv, blocks, threads, smem, st, p);
    case 3: return zpass_nv_lg<T, 3>(nv, blocks, threads, smem, st, p);
    case 4: return zpass_nv_lg<T, 4>(nv, blocks, threads, smem, st, p);
    case 5: return zpass_nv_lg<T, 5>(nv, blocks, threads, smem, st, p);
    case 6: return zpass_nv_lg<T, 6>(nv, blocks, threads, smem, st, p);
    case 7: return zpass_nv_lg<T, 7>(nv, blocks, threads, smem, st, p);
    case 8: return zpass_nv_lg<T, 8>(nv, blocks, threads, smem, st, p);
    case 9: return zpass_nv_lg<T, 9>(nv, blocks, threads, smem, st, p);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_zpass(int prec, int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                         const ZParams &p, int nv) {
  if (nv == 0) nv = zpass_nv(lgL, prec == 0 ? 16 : 8);
  return prec == 0 ? zpass_t<double>(lgL, nv, blocks, threads, smem, st, p)
                   : zpass_t<float>(lgL, nv, blocks, threads, smem, st, p);
}

}  // namespace pfdd
