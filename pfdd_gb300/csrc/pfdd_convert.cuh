// pfdd_convert.cuh -- binary64 <-> binary32 conversions done with integer
// operations on the IEEE-754 bit patterns.
//
// GB300 executes FP64 instructions (including the F2F conversions) at 1/58 of
// the FP32 rate, so the FP32-FFT form's update, which converts every state
// element between the FP64 state and the FP32 spectral buffer, keeps those
// conversions on the integer pipe.  Both functions are exact IEEE conversions
// for normal numbers (round to nearest even on narrowing), flush subnormal
// inputs/results to signed zero, and map Inf/NaN to Inf/NaN.  They are
// __host__ __device__ so the host test suite checks them against the C
// compiler's own conversions.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PFDD_HD __host__ __device__ __forceinline__
#else
#define PFDD_HD static inline
#endif

namespace pfdd {

PFDD_HD uint64_t f64_bits(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
#endif
}
PFDD_HD double bits_f64(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}
PFDD_HD uint32_t f32_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
PFDD_HD float bits_f32(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

// binary32 -> binary64 bit pattern (exact for normal numbers)
PFDD_HD uint64_t f32_to_f64bits_int(float f) {
  const uint32_t u = f32_bits(f);
  const uint64_t sign = (uint64_t)(u >> 31) << 63;
  const uint32_t e = (u >> 23) & 0xffu;
  const uint64_t m = (uint64_t)(u & 0x7fffffu) << 29;
  if (e == 0u) return sign;
  if (e == 0xffu) return sign | (0x7ffull << 52) | m;
  return sign | ((uint64_t)(e + (1023u - 127u)) << 52) | m;
}

// binary32 -> binary64 (exact for normal numbers)
PFDD_HD double f32_to_f64_int(float f) {
  const uint32_t u = f32_bits(f);
  const uint64_t sign = (uint64_t)(u >> 31) << 63;
  const uint32_t e = (u >> 23) & 0xffu;
  const uint64_t m = (uint64_t)(u & 0x7fffffu) << 29;
  if (e == 0u) return bits_f64(sign);                               // zero / subnormal -> signed zero
  if (e == 0xffu) return bits_f64(sign | (0x7ffull << 52) | m);      // Inf / NaN
  return bits_f64(sign | ((uint64_t)(e + (1023u - 127u)) << 52) | m);
}

// binary64 bit pattern -> binary32, round to nearest even
PFDD_HD float f64bits_to_f32_int(uint64_t u) {
  const uint32_t sign = (uint32_t)(u >> 63) << 31;
  const uint64_t mag = u & 0x7fffffffffffffffull;
  const uint32_t e11 = (uint32_t)(mag >> 52);
  if (e11 == 0x7ffu) {  // Inf / NaN (keep NaNs quiet and non-zero)
    const uint32_t nan = (mag & 0xfffffffffffffull) ? 0x400000u : 0u;
    return bits_f32(sign | 0x7f800000u | nan);
  }
  // round the 52-bit mantissa to 23 bits: add half an ulp (minus one unless the
  // kept lsb is odd) so that ties go to even; a carry moves into the exponent
  const uint64_t lsb = (mag >> 29) & 1ull;
  const uint64_t r = mag + ((1ull << 28) - 1ull) + lsb;
  const int64_t e = (int64_t)(r >> 52) - (1023 - 127);
  if (e >= 255) return bits_f32(sign | 0x7f800000u);  // overflow -> Inf
  if (e <= 0) return bits_f32(sign);                  // underflow -> signed zero
  return bits_f32(sign | ((uint32_t)e << 23) | (uint32_t)((r >> 29) & 0x7fffffull));
}

// binary64 -> binary32, round to nearest even
PFDD_HD float f64_to_f32_int(double d) { return f64bits_to_f32_int(f64_bits(d)); }

// The same two conversions on 32-bit words, with a short path for the common
// case (a binary32-normal result) and the general functions above otherwise.
// Results are identical to f64bits_to_f32_int / f32_to_f64bits_int.
PFDD_HD float f64bits_to_f32_fast(uint64_t u) {
  const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
  const uint32_t mhi = hi & 0x7fffffffu;
  // binary64 exponents 897..1150 give binary32 exponents 1..254
  if (mhi - (897u << 20) < (254u << 20)) {
    uint32_t v = ((mhi - (896u << 20)) << 3) | (lo >> 29);  // exponent and 23 mantissa bits
    const uint32_t rem = lo & 0x1fffffffu;                   // the 29 dropped bits
    v += (uint32_t)(rem > 0x10000000u) | ((uint32_t)(rem == 0x10000000u) & v);  // ties to even
    return bits_f32(v | (hi & 0x80000000u));
  }
  return f64bits_to_f32_int(u);
}

PFDD_HD uint64_t f32_to_f64bits_fast(float f) {
  const uint32_t u = f32_bits(f);
  const uint32_t e8 = (u >> 23) & 0xffu;
  if (e8 == 0xffu) return f32_to_f64bits_int(f);
  const uint32_t sign = u & 0x80000000u;
  const uint32_t hi = e8 ? sign | (((u & 0x7fffffffu) >> 3) + (896u << 20)) : sign;
  const uint32_t lo = e8 ? u << 29 : 0u;
  return ((uint64_t)hi << 32) | lo;
}

}  // namespace pfdd
