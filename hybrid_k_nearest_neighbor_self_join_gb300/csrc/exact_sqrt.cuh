// exact_sqrt.cuh -- correctly rounded double square root on the integer and
// FP32 pipes.
//
// The BETA rule's sampled mean distance (kernel.cu:357-364) needs, per
// sampled pair, the double square root of a double, rounded to nearest.
// GB300's FP64 pipe is a small fraction of its FP32 pipe, and that root was
// most of the estimator's time.  This computes the same value from integers:
// with x = m * 2^E (m the 53-bit significand), M = m * 2^k (k = 52 or 53,
// E - k even) lies in [2^104, 2^106), and sqrt(x) = sqrt(M) * 2^((E-k)/2).
// s = floor(sqrt(M)) (53 bits) comes from a float seed refined by two Newton
// steps on the exact 128-bit remainder M - y^2 (the division by 2y done in
// float, whose error the next step absorbs), then a final +-1 correction
// that leaves 0 <= r = M - s^2 <= 2s.  Since (s + 1/2)^2 = s^2 + s + 1/4 and
// M is an integer, sqrt(M) rounds up exactly when r > s (no ties occur).
// Host and device run the same integer arithmetic; tests compare it with the
// C library's correctly rounded sqrt on the host.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__  // plain C++ (host tests)
#define __host__
#define __device__
#endif

namespace knnsj {

struct U128 {
  uint64_t lo, hi;
};

__host__ __device__ inline uint64_t es_mulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

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

// M - y*y as a signed 128-bit value (hi word signed); y < 2^54.
__host__ __device__ inline U128 es_rem(U128 M, uint64_t y) {
  const uint64_t plo = y * y, phi = es_mulhi(y, y);
  U128 r;
  r.lo = M.lo - plo;
  r.hi = M.hi - phi - (M.lo < plo ? 1u : 0u);
  return r;
}

// Conversions between 64-bit integers and floats run on the FP64 pipe on this
// GPU, which is what this file avoids: floats are assembled from and taken
// apart into bits with integer operations (truncating; Newton absorbs it).
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

// A float close to (within 2^-23 of) the unsigned value v = hi:lo > 0.
__host__ __device__ inline float es_u128_to_float(uint64_t hi, uint64_t lo) {
  int p;  // index of the leading one
  uint64_t top;
  if (hi) {
    p = 127 - es_clz64(hi);
    top = p >= 64 + 23 ? (hi >> (p - 64 - 23)) : ((hi << (64 + 23 - p)) | (lo >> (p - 23)));
  } else {
    p = 63 - es_clz64(lo);
    top = p >= 23 ? (lo >> (p - 23)) : (lo << (23 - p));
  }
  return es_float_bits((uint32_t)((p + 127) << 23) | (uint32_t)(top & 0x7fffffu));
}

// A float close to the signed 128-bit value r.
__host__ __device__ inline float es_to_float(U128 r) {
  const bool neg = (int64_t)r.hi < 0;
  uint64_t lo = r.lo, hi = r.hi;
  if (neg) {  // two's complement negate
    lo = ~lo + 1;
    hi = ~hi + (lo == 0 ? 1 : 0);
  }
  if (!hi && !lo) return 0.0f;
  const float f = es_u128_to_float(hi, lo);
  return neg ? -f : f;
}

// The integer nearest below |f| (truncation toward zero), with f's sign.
__host__ __device__ inline int64_t es_float_to_i64(float f) {
  const uint32_t b = es_bits_of_float(f);
  const int e = (int)((b >> 23) & 0xff) - 127;
  if (e < 0) return 0;
  const uint64_t mant = (uint64_t)((b & 0x7fffffu) | 0x800000u);
  const uint64_t v = e >= 23 ? mant << (e - 23) : mant >> (23 - e);
  return (b >> 31) ? -(int64_t)v : (int64_t)v;
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
  U128 M;
  M.lo = m << k;
  M.hi = m >> (64 - k);
  // float seed: sqrt(m * 2^(k-52)) * 2^26, m truncated to 24 bits
  const float mf = es_float_bits((uint32_t)((127 + k) << 23) | (uint32_t)((m >> 29) & 0x7fffffu));
  const uint32_t sb = es_bits_of_float(sqrtf(mf));  // in [2^26, 2^27)
  uint64_t y = (uint64_t)((sb & 0x7fffffu) | 0x800000u) << ((int)((sb >> 23) & 0xff) - 127 + 3);
  for (int it = 0; it < 2; it++) {
    const U128 r = es_rem(M, y);
    const float d = es_to_float(r) / (2.0f * es_u128_to_float(0, y));
    y = (uint64_t)((int64_t)y + es_float_to_i64(d));
  }
  // final correction: 0 <= r <= 2y
  int64_t r = (int64_t)es_rem(M, y).lo;  // |r| < 2^63 here
  while (r < 0) {
    y--;
    r += (int64_t)(2 * y + 1);
  }
  while (r > (int64_t)(2 * y)) {
    r -= (int64_t)(2 * y + 1);
    y++;
  }
  uint64_t q = y + (r > (int64_t)y ? 1u : 0u);
  int ex = (E - k) / 2 + 52 + 1023;  // q in [2^52, 2^53]
  if (q >> 53) {
    q >>= 1;
    ex++;
  }
  return es_from_bits(((uint64_t)ex << 52) | (q & ((1ull << 52) - 1)));
}

}  // namespace knnsj
