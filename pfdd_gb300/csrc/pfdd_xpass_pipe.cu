// pfdd_xpass_pipe.cu -- instantiations of the persistent pipelined x-pass
// (FP32 spectra, B(k) tile table with line pairs): every ns in [1, 12],
// N1 = 32..256.  The grid holds as many CTAs as the device runs at once.
#include "pfdd_launch.h"

namespace pfdd {

template <int NS, int LG>
static cudaError_t launch_lg(long long items, int threads, size_t smem, cudaStream_t st, const XParams &p) {
  static SmemOptIn configured;
  cudaError_t e = ensure_smem(x_pipe_kernel<NS, LG>, smem, configured);
  if (e != cudaSuccess) return e;
  int per_sm = 0, sms = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, x_pipe_kernel<NS, LG>, threads, smem);
  if (e != cudaSuccess) return e;
  if ((e = device_sm_count(&sms)) != cudaSuccess) return e;
  const long long resident = (long long)std::max(1, per_sm) * sms;
  const unsigned blocks = (unsigned)std::max(1LL, std::min(items, resident));
  return launch_pdl(x_pipe_kernel<NS, LG>, blocks, threads, smem, st, p);
}

template <int NS>
static cudaError_t launch_ns(long long items, int threads, size_t smem, cudaStream_t st, const XParams &p) {
  switch (p.lgL) {
    case 5: return launch_lg<NS, 5>(items, threads, smem, st, p);
    case 6: return launch_lg<NS, 6>(items, threads, smem, st, p);
    case 7: return launch_lg<NS, 7>(items, threads, smem, st, p);
    case 8: return launch_lg<NS, 8>(items, threads, smem, st, p);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_x_pipe_f32(int ns, long long items, int threads, size_t smem, cudaStream_t st, const XParams &p) {
  switch (ns) {
    case 1: return launch_ns<1>(items, threads, smem, st, p);
    case 2: return launch_ns<2>(items, threads, smem, st, p);
    case 3: return launch_ns<3>(items, threads, smem, st, p);
    case 4: return launch_ns<4>(items, threads, smem, st, p);
    case 5: return launch_ns<5>(items, threads, smem, st, p);
    case 6: return launch_ns<6>(items, threads, smem, st, p);
    case 7: return launch_ns<7>(items, threads, smem, st, p);
    case 8: return launch_ns<8>(items, threads, smem, st, p);
    case 9: return launch_ns<9>(items, threads, smem, st, p);
    case 10: return launch_ns<10>(items, threads, smem, st, p);
    case 11: return launch_ns<11>(items, threads, smem, st, p);
    case 12: return launch_ns<12>(items, threads, smem, st, p);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pfdd
