// pfdd_noalloc.cu -- in-place 3D FFT of device-resident fields that performs
// no device allocation.
//
// The regular FFT boundary (pfdd_fft_plan_create + pfdd_fft_forward/backward)
// allocates its twiddle tables and a staging buffer when the plan is created.
// Some callers cannot do that: code that runs inside a data region whose device
// memory belongs to another runtime (the reference calls its FFT from OpenACC
// `host_data use_device` regions, F:4446-4450), or a process that must stay
// within a device-memory budget fixed by someone else.  This entry point works
// on the caller's device buffer in place and keeps its only scratch -- the
// twiddle tables of the three axes -- in a file-scope static device array.
#include <cstring>
#include <mutex>

#include "../../include/pfdd_gpu.h"
#include "pfdd_launch.h"

namespace {

constexpr int kNoAllocMaxLen = 512;      // largest N1, N2 or N3
constexpr int kNoAllocMaxDevices = 64;

// twiddles of the three axes; slot ax holds kNoAllocMaxLen complex128 values
// (FP32 transforms use the first half of each slot as complex64)
__device__ __align__(256) unsigned char g_noalloc_twiddles[3 * kNoAllocMaxLen * 16];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[kNoAllocMaxDevices] = {};

// Host code cannot take the address of a __device__ array directly: its
// device address comes from cudaGetSymbolAddress, once per device, with that
// device current.
cudaError_t noalloc_scratch(int dev, void **out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" pfdd_status pfdd_fft_device_noalloc(void *data, int n1, int n2, int n3, int batch, int precision,
                                               int sign, void *stream) {
  using namespace pfdd;
  if (!data || batch < 1 || (sign != -1 && sign != 1) || (precision != PFDD_FP64 && precision != PFDD_FFT_FP32))
    return PFDD_EINVAL;
  const int n[3] = {n1, n2, n3};
  for (int ax = 0; ax < 3; ++ax) {
    if (n[ax] < 1 || (n[ax] & (n[ax] - 1)) != 0) return PFDD_EINVAL;
    if (n[ax] > kNoAllocMaxLen) return PFDD_ELIMIT;  // beyond the static twiddle table
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return PFDD_ECUDA;
  void *scratch = nullptr;
  if (noalloc_scratch(dev, &scratch) != cudaSuccess) return PFDD_ECUDA;
  cudaStream_t st = (cudaStream_t)stream;
  const int pc = precision == PFDD_FP64 ? 0 : 1;
  const size_t vsize = pc == 0 ? sizeof(double2) : sizeof(float2);
  // every call rewrites the tables of its three lengths before using them
  void *tw[3];
  for (int ax = 0; ax < 3; ++ax) {
    tw[ax] = (unsigned char *)scratch + (size_t)ax * kNoAllocMaxLen * 16;
    if (pc == 0) twiddle_kernel<double><<<(n[ax] + 127) / 128, 128, 0, st>>>(tw[ax], n[ax]);
    else twiddle_kernel<float><<<(n[ax] + 127) / 128, 128, 0, st>>>(tw[ax], n[ax]);
  }
  if (cudaGetLastError() != cudaSuccess) return PFDD_ECUDA;
  const Geometry g = make_geometry(n1, n2, n3, 0, vsize, pc == 0 ? 8 : 4);
  ZParams zp;
  memset(&zp, 0, sizeof zp);
  zp.S = data; zp.tw = tw[2]; zp.N = (long long)n1 * n2 * n3; zp.lines_per_field = (long long)n1 * n2;
  zp.L = n3; zp.lgL = g.lgL3; zp.ns = batch; zp.R = 1; zp.TL = g.zTL; zp.nparts = g.zNparts; zp.pitch = g.zPitch;
  const unsigned zblocks = (unsigned)((long long)batch * g.zNparts);
  auto strided = [&](int ax, int s) -> cudaError_t {  // ax 0: y, 1: x
    const int L = ax == 0 ? n2 : n1;
    if (L == 1) return cudaSuccess;
    const long long inner = ax == 0 ? (long long)n3 : (long long)n2 * n3;
    const long long outer = ax == 0 ? (long long)batch * n1 : (long long)batch;
    return launch_strided(pc, s, ilog2(L), (unsigned)(outer * g.tiles[ax]), g.threads[ax], g.smem[ax], st, data,
                          g.lgTI[ax], inner, g.tiles[ax], tw[ax == 0 ? 1 : 0], nullptr, outer, g.pitch[ax]);
  };
  cudaError_t e;
  if (sign < 0) {
    zp.flags = Z_FWD | Z_STORE;
    e = launch_zpass(pc, g.lgL3, zblocks, g.zThreads, g.zSmem, st, zp);
    if (e == cudaSuccess) e = strided(0, -1);
    if (e == cudaSuccess) e = strided(1, -1);
  } else {
    e = strided(1, +1);
    if (e == cudaSuccess) e = strided(0, +1);
    zp.flags = Z_INV | Z_STORE;
    if (e == cudaSuccess) e = launch_zpass(pc, g.lgL3, zblocks, g.zThreads, g.zSmem, st, zp);
  }
  return e == cudaSuccess ? PFDD_OK : PFDD_ECUDA;
}
