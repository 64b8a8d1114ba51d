// pfdd_tma.cuh -- bulk global -> shared copies on the TMA engine
// (cp.async.bulk, completion counted in bytes on an mbarrier), with
// time-bounded waits.
//
// A CTA stages a contiguous block (a B(k) tile, an FP64 state tile) with a
// handful of bulk copies issued by one thread instead of thousands of per-
// thread cp.async requests.  Every wait on the mbarrier is bounded by the
// global timer: if the bytes have not arrived within kWaitNs the kernel
// records an error in `err` (reported by the host as PFDD_ETIMEOUT) instead
// of spinning forever.
#pragma once
#include <stdint.h>

namespace pfdd {

constexpr unsigned long long kWaitNs = 500ull * 1000 * 1000;  // 0.5 s
constexpr unsigned kBulkChunk = 16384;                        // bytes per bulk copy

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of the barrier for at most limit_ns; false (and
// *err set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, int *err,
                                          unsigned long long limit_ns = kWaitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > limit_ns) {
      if (err) atomicOr(err, 1);
      return false;
    }
  }
  return true;
}

// One thread: copies `bytes` (multiple of 16, both addresses 16-byte aligned)
// completing on `bar` without raising its expected byte count (the caller
// announced the total of all its copies with one mbar_arrive_expect_tx).
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  for (unsigned off = 0; off < bytes; off += kBulkChunk) {
    const unsigned n = bytes - off < kBulkChunk ? bytes - off : kBulkChunk;
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32((const char *)dst + off)),
        "l"((const char *)src + off), "r"(n), "r"(smem_u32(bar))
        : "memory");
  }
}

// One thread: copies `bytes` (multiple of 16, both addresses 16-byte aligned)
// in chunks, all completing on `bar`, whose expected byte count it raises.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  mbar_arrive_expect_tx(bar, bytes);
  for (unsigned off = 0; off < bytes; off += kBulkChunk) {
    const unsigned n = bytes - off < kBulkChunk ? bytes - off : kBulkChunk;
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32((const char *)dst + off)),
        "l"((const char *)src + off), "r"(n), "r"(smem_u32(bar))
        : "memory");
  }
}

// The same with an L2 evict-first policy: for data read once (a B(k) tile),
// so that it does not push out of L2 what the previous pass wrote last.
__device__ __forceinline__ void bulk_load_evict_first(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  mbar_arrive_expect_tx(bar, bytes);
  for (unsigned off = 0; off < bytes; off += kBulkChunk) {
    const unsigned n = bytes - off < kBulkChunk ? bytes - off : kBulkChunk;
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32((const char *)dst + off)),
        "l"((const char *)src + off), "r"(n), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
  }
}

// Programmatic dependent launch (kernels launched with launch_pdl): a kernel
// may be launched while the previous kernel on its stream finishes, does the
// work that does not depend on it (constant tables, TMA copies of data written
// earlier) and waits here before it reads what that kernel wrote (the wait
// returns once that kernel has completed and its writes are visible).  The
// kernels signal no early completion: measured at 128^3 x 12, letting the next
// kernel in once every CTA of this one had started cost 3% (its CTAs waited
// on SMs the tail needed); launching it at completion gains 0.4%.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

}  // namespace pfdd
