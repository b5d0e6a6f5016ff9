// exact_sqrt.cuh -- correctly rounded double square root on the integer and
// FP32 pipes.
//
// The BETA rule's sampled mean distance (kernel.cu:357-364) needs, per
// sampled pair, the double square root of a double, rounded to nearest.
// GB300's FP64 pipe is a small fraction of its FP32 pipe, and that root was
// most of the estimator's time.  This computes the same value with FP32 and
// 64-bit integer operations only:
//
//   x = m * 2^E (m the 53-bit significand); k in {52, 53} with E - k even;
//   M = m * 2^k in [2^104, 2^106); sqrt(x) = S * 2^((E-k)/2), S = sqrt(M).
//   A = M / 2^52 = m * 2^(k-52) < 2^54 (an integer), sqrt(A) = S / 2^26.
//
//   1. y0 = RN(sqrt(a_hi)) in float, a_hi = A cut to its top 24 bits; y0 =
//      j * 2^(ey-23) with j a 24-bit integer, so T = A - y0^2 is an exact
//      64-bit integer with |T| < 2^31.
//   2. One Newton step in float, with its quadratic term: d = T / (2 y0),
//      d -= d^2 / (2 y0); s1 = y0 * 2^26 + RN(d * 2^26).  Three float
//      roundings of relative size 2^-24 on |d| <= 16 leave |s1 - S| <= 193.
//   3. r1 = M - s1^2 is exact modulo 2^64 (|r1| < 2^62); its high word gives
//      the second correction r1 / (2 s1) to within 2^-14, so s = s1 +
//      RN(r1 / (2 s1)) has |s - S| < 1.
//   4. r = M - s^2 (mod 2^64, |r| <= 2^54) fixes floor(S) with one step
//      either way, leaving 0 <= r <= 2 floor(S).  Since (s + 1/2)^2 =
//      s^2 + s + 1/4 and M is an integer, S rounds up exactly when r > s
//      (no ties occur).
//
// Every floating-point step is an IEEE round-to-nearest operation (sqrt,
// reciprocal, multiply, fma, int<->float conversions of 32-bit values), so
// host and device compute the same bits; tests compare the host build with
// the C library's correctly rounded sqrt, and the device build with the
// GPU's.  64-bit integer <-> float conversions, which run on the FP64 pipe
// of this GPU, are not used.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__  // plain C++ (host tests)
#define __host__
#define __device__
#endif

namespace knnsj {

__host__ __device__ inline int es_clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

__host__ __device__ inline uint64_t es_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}

__host__ __device__ inline double es_from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

__host__ __device__ inline float es_float_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  std::memcpy(&f, &b, 4);
  return f;
#endif
}

__host__ __device__ inline uint32_t es_bits_of_float(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t b;
  std::memcpy(&b, &f, 4);
  return b;
#endif
}

// IEEE round-to-nearest float operations, the same on host and device.
__host__ __device__ inline float es_sqrtf(float a) {
#ifdef __CUDA_ARCH__
  return __fsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
__host__ __device__ inline float es_rcp(float a) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(a);
#else
  return 1.0f / a;
#endif
}
__host__ __device__ inline float es_fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ inline float es_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
__host__ __device__ inline float es_i2f(int32_t v) {
#ifdef __CUDA_ARCH__
  return __int2float_rn(v);
#else
  return (float)v;
#endif
}
__host__ __device__ inline int32_t es_f2i_rn(float f) {
#ifdef __CUDA_ARCH__
  return __float2int_rn(f);
#else
  return (int32_t)std::nearbyint(f);
#endif
}

// The double of a float, exactly, assembled from bits: a float-to-double
// conversion instruction runs on the FP64 pipe of this GPU.
__host__ __device__ inline double es_f2d(float f) {
  const uint32_t b = es_bits_of_float(f);
  const uint32_t ef = (b >> 23) & 0xffu;
  // normal floats: rebias the exponent (by 896, in place) and widen the
  // significand -- one 64-bit shift and an add
  if (ef - 1u < 254u)
    return es_from_bits((((uint64_t)(b & 0x7fffffffu)) << 29) + (896ull << 52) + ((uint64_t)(b >> 31) << 63));
  const uint64_t sign = (uint64_t)(b >> 31) << 63;
  uint32_t mf = b & 0x7fffffu;
  if (ef == 0xffu) return es_from_bits(sign | (0x7ffull << 52) | ((uint64_t)mf << 29));  // inf, nan
  if (ef == 0) {
    if (mf == 0) return es_from_bits(sign);  // +-0
    // subnormal: mf * 2^-149, normalised to a leading one at bit 23
    const int sh = es_clz64((uint64_t)mf) - 40;
    mf <<= sh;
    return es_from_bits(sign | ((uint64_t)(1023 - 126 - sh) << 52) | ((uint64_t)(mf & 0x7fffffu) << 29));
  }
  return es_from_bits(sign | ((uint64_t)(ef - 127 + 1023) << 52) | ((uint64_t)mf << 29));
}

// sqrt(x) rounded to nearest, for finite x >= 0 (any other input returns x).
__host__ __device__ inline double exact_sqrt(double x) {
  const uint64_t b = es_bits(x);
  // +-0, negative, inf and nan are returned as they are (integer tests: no FP64 compare)
  if ((b << 1) == 0 || (b >> 63) || ((b >> 52) & 0x7ff) == 0x7ff) return x;
  int e = (int)(b >> 52);
  uint64_t m = b & ((1ull << 52) - 1);
  if (e == 0) {  // subnormal: normalise
    const int sh = es_clz64(m) - 11;
    m <<= sh;
    e = 1 - sh;
  } else {
    m |= 1ull << 52;
  }
  const int E = e - 1075;  // x = m * 2^E, m in [2^52, 2^53)
  const int k = ((E - 52) & 1) ? 53 : 52;
  const uint64_t A = m << (k - 52);  // M / 2^52
  // 1. float seed and the exact remainder of A
  const float a_hi = es_float_bits((uint32_t)((127 + k) << 23) | (uint32_t)((m >> 29) & 0x7fffffu));
  const float y0 = es_sqrtf(a_hi);  // in [2^26, 2^27]
  const uint32_t yb = es_bits_of_float(y0);
  const int ey = (int)((yb >> 23) & 0xffu) - 127;  // 26 or 27
  const uint64_t j = (uint64_t)((yb & 0x7fffffu) | 0x800000u);
  const int64_t T = (int64_t)(A - ((j * j) << (2 * (ey - 23))));
  // 2. Newton step with its quadratic term
  const float inv = es_rcp(2.0f * y0);
  float d = es_fmul(es_i2f((int32_t)T), inv);
  d = es_fma(-es_fmul(d, inv), d, d);
  const int64_t s1 = (int64_t)(j << (ey + 3)) + es_f2i_rn(es_fmul(d, 67108864.0f));
  // 3. second correction from the exact remainder's high word
  const uint64_t Mlo = m << k;  // M mod 2^64
  const int64_t r1 = (int64_t)(Mlo - (uint64_t)s1 * (uint64_t)s1);
  const float d2 = es_fmul(es_fmul(es_i2f((int32_t)(r1 >> 32)), inv), 64.0f);
  int64_t s = s1 + es_f2i_rn(d2);
  // 4. floor and rounding
  int64_t r = (int64_t)(Mlo - (uint64_t)s * (uint64_t)s);
  if (r < 0) {
    r += 2 * s - 1;
    s -= 1;
  } else if (r > 2 * s) {
    r -= 2 * s + 1;
    s += 1;
  }
  uint64_t q = (uint64_t)s + (r > s ? 1u : 0u);
  int ex = (E - k) / 2 + 52 + 1023;  // q in [2^52, 2^53]
  if (q >> 53) {
    q >>= 1;
    ex++;
  }
  return es_from_bits(((uint64_t)ex << 52) | (q & ((1ull << 52) - 1)));
}

}  // namespace knnsj
