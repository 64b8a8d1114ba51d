// pfdd_xpass_warp.cu -- instantiations of the warp-team fused x-pass (FP32
// spectra, stored or register-evaluated B(k)): every ns in [1, 12], N1 = 32..256.
#include "pfdd_launch.h"

namespace pfdd {

template <int NS, int LG, bool BFLY>
static cudaError_t launch_lg(unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p) {
  static SmemOptIn configured;
  cudaError_t e = ensure_smem(x_warp_kernel<NS, LG, BFLY>, smem, configured);
  if (e != cudaSuccess) return e;
  return launch_pdl(x_warp_kernel<NS, LG, BFLY>, blocks, threads, smem, st, p);
}

template <int NS, bool BFLY>
static cudaError_t launch_ns(unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p) {
  switch (p.lgL) {
    case 5: return launch_lg<NS, 5, BFLY>(blocks, threads, smem, st, p);
    case 6: return launch_lg<NS, 6, BFLY>(blocks, threads, smem, st, p);
    case 7: return launch_lg<NS, 7, BFLY>(blocks, threads, smem, st, p);
    case 8: return launch_lg<NS, 8, BFLY>(blocks, threads, smem, st, p);
    default: return cudaErrorInvalidValue;
  }
}

template <bool BFLY>
static cudaError_t launch_form(int ns, unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p) {
  switch (ns) {
    case 1: return launch_ns<1, BFLY>(blocks, threads, smem, st, p);
    case 2: return launch_ns<2, BFLY>(blocks, threads, smem, st, p);
    case 3: return launch_ns<3, BFLY>(blocks, threads, smem, st, p);
    case 4: return launch_ns<4, BFLY>(blocks, threads, smem, st, p);
    case 5: return launch_ns<5, BFLY>(blocks, threads, smem, st, p);
    case 6: return launch_ns<6, BFLY>(blocks, threads, smem, st, p);
    case 7: return launch_ns<7, BFLY>(blocks, threads, smem, st, p);
    case 8: return launch_ns<8, BFLY>(blocks, threads, smem, st, p);
    case 9: return launch_ns<9, BFLY>(blocks, threads, smem, st, p);
    case 10: return launch_ns<10, BFLY>(blocks, threads, smem, st, p);
    case 11: return launch_ns<11, BFLY>(blocks, threads, smem, st, p);
    case 12: return launch_ns<12, BFLY>(blocks, threads, smem, st, p);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_x_warp_f32(int ns, bool bfly, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                              const XParams &p) {
  return bfly ? launch_form<true>(ns, blocks, threads, smem, st, p)
              : launch_form<false>(ns, blocks, threads, smem, st, p);
}

}  // namespace pfdd
