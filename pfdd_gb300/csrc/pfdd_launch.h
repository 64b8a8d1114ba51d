// pfdd_launch.h -- host launchers of the templated kernels.  Each kernel is
// instantiated for every power-of-two line length it runs (log2 L known at
// compile time) in its own translation unit, so the build compiles in
// parallel: pfdd_fftpass.cu (z-pass, strided passes), pfdd_xpass_f32.cu and
// pfdd_xpass_f64.cu (fused x-pass).
#pragma once
#include <cuda_runtime.h>

#include "pfdd_kernels.cuh"

namespace pfdd {
// z-pass for lgL in [0, 9]; prec 0 = FP64 spectra, 1 = FP32
cudaError_t launch_zpass(int prec, int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                         const ZParams &p);
// strided line FFT (sign -1 forward, +1 inverse) for lgL in [0, 9]
cudaError_t launch_strided(int prec, int sign, int lgL, unsigned blocks, int threads, size_t smem, cudaStream_t st,
                           void *data, int lgTI, long long inner, long long tiles_per_outer, const void *tw,
                           const uint8_t *active, long long outer_per_rep, int pitch);
// fused x-pass (x-forward FFT, contraction, x-inverse FFT) for ns in [1, 12]
cudaError_t launch_x_fused_f32(int ns, unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p);
cudaError_t launch_x_fused_f64(int ns, unsigned blocks, int threads, size_t smem, cudaStream_t st, const XParams &p);

// opts a kernel into `smem` bytes of dynamic shared memory once per size increase
template <typename K>
inline cudaError_t ensure_smem(K kernel, size_t smem, size_t &configured) {
  if (smem <= configured) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) configured = smem;
  return e;
}
}  // namespace pfdd
