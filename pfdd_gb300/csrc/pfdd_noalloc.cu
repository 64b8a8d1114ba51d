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
#include <climits>
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
// the array's device address per device, with the CUDA context it belongs to
struct ScratchSlot {
  void *ctx = nullptr;
  void *addr = nullptr;
};
ScratchSlot g_noalloc_slot[kNoAllocMaxDevices];

// cuCtxGetCurrent through the runtime's driver entry point (no link to the
// driver library): the context current on this thread, null if none yet.
cudaError_t current_context(void **ctx) {
  using Fn = int (*)(void **);
  static Fn fn = nullptr;  // resolved under g_noalloc_mu
  if (!fn) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !f) return cudaErrorNotSupported;
    fn = reinterpret_cast<Fn>(f);
  }
  *ctx = nullptr;
  return fn(ctx) == 0 ? cudaSuccess : cudaErrorDeviceUninitialized;
}

// Host code cannot take the address of a __device__ array directly: its
// device address comes from cudaGetSymbolAddress, with the device current.
// It is looked up on the first call on a device and again whenever the
// current context is not the one it was looked up in (another context of the
// same device, or the device's primary context created anew).
cudaError_t noalloc_scratch(int dev, void **out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  ScratchSlot &slot = g_noalloc_slot[dev];
  void *ctx = nullptr;
  cudaError_t e = current_context(&ctx);
  if (e != cudaSuccess) return e;
  if (!slot.addr || !ctx || ctx != slot.ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);  // makes the device's context current if none was
    if (e != cudaSuccess) return e;
    e = current_context(&ctx);
    if (e != cudaSuccess) return e;
    slot.ctx = ctx;
    slot.addr = p;
  }
  *out = slot.addr;
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
  const Geometry g = make_geometry(n1, n2, n3, 0, precision == PFDD_FP64 ? sizeof(double2) : sizeof(float2),
                                   precision == PFDD_FP64 ? 8 : 4);
  // grid sizes of the three passes: every launch covers all the data or none runs
  if ((long long)batch * g.zNparts > INT_MAX || (long long)batch * n1 * g.tiles[0] > INT_MAX ||
      (long long)batch * g.tiles[1] > INT_MAX)
    return PFDD_EINVAL;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return PFDD_ECUDA;
  void *scratch = nullptr;
  if (noalloc_scratch(dev, &scratch) != cudaSuccess) return PFDD_ECUDA;
  cudaStream_t st = (cudaStream_t)stream;
  const int pc = precision == PFDD_FP64 ? 0 : 1;
  // every call rewrites the tables of its three lengths before using them
  void *tw[3];
  for (int ax = 0; ax < 3; ++ax) {
    tw[ax] = (unsigned char *)scratch + (size_t)ax * kNoAllocMaxLen * 16;
    if (pc == 0) twiddle_kernel<double><<<(n[ax] + 127) / 128, 128, 0, st>>>(tw[ax], n[ax]);
    else twiddle_kernel<float><<<(n[ax] + 127) / 128, 128, 0, st>>>(tw[ax], n[ax]);
  }
  if (cudaGetLastError() != cudaSuccess) return PFDD_ECUDA;
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
