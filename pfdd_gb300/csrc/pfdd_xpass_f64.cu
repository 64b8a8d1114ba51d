// pfdd_xpass_f64.cu -- instantiations of the fused x-pass for double spectra:
// every ns in [1, 12]; N1 = 32..256 with the line length fixed at compile
// time, any other power of two through the run-time-length variant.
#include "pfdd_launch.h"

namespace pfdd {

template <int NS, int LG>
static cudaError_t launch_lg(unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p) {
  static SmemOptIn configured;
  cudaError_t e = ensure_smem(x_fused_kernel<double, NS, false, LG, false>, smem, configured);
  if (e != cudaSuccess) return e;
  return launch_pdl(x_fused_kernel<double, NS, false, LG, false>, blocks, threads, smem, st, p);
}

template <int NS>
static cudaError_t launch_ns(unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p) {
  switch (p.lgL) {
    case 5: return launch_lg<NS, 5>(blocks, threads, smem, st, p);
    case 6: return launch_lg<NS, 6>(blocks, threads, smem, st, p);
    case 7: return launch_lg<NS, 7>(blocks, threads, smem, st, p);
    case 8: return launch_lg<NS, 8>(blocks, threads, smem, st, p);
    default: return launch_lg<NS, -1>(blocks, threads, smem, st, p);
  }
}

cudaError_t launch_x_fused_f64(int ns, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                                 const XParams &p) {
  switch (ns) {
    case 1: return launch_ns<1>(blocks, threads, smem, st, p);
    case 2: return launch_ns<2>(blocks, threads, smem, st, p);
    case 3: return launch_ns<3>(blocks, threads, smem, st, p);
    case 4: return launch_ns<4>(blocks, threads, smem, st, p);
    case 5: return launch_ns<5>(blocks, threads, smem, st, p);
    case 6: return launch_ns<6>(blocks, threads, smem, st, p);
    case 7: return launch_ns<7>(blocks, threads, smem, st, p);
    case 8: return launch_ns<8>(blocks, threads, smem, st, p);
    case 9: return launch_ns<9>(blocks, threads, smem, st, p);
    case 10: return launch_ns<10>(blocks, threads, smem, st, p);
    case 11: return launch_ns<11>(blocks, threads, smem, st, p);
    case 12: return launch_ns<12>(blocks, threads, smem, st, p);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pfdd
