// knnsj_device.cuh -- device-side building blocks shared by the kernels.
//
// All floating-point arithmetic on the result path goes through explicit
// round-to-nearest intrinsics so that nvcc cannot contract or reassociate it:
// the squared distance is exactly fma(p-q, p-q, acc) per dimension, the form
// nvcc gives the reference's `runningTotalDist += (p-q)*(p-q)`
// (kernel.cu:139-140), and cell coordinates are exactly
// (unsigned)((x - min) / eps) (kernel.cu:91, kernel.cu:1690).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace knnsj {

constexpr unsigned FULL = 0xffffffffu;
constexpr int MAX_DI = 8;      // indexed dimensions supported by the ring search
constexpr int MAX_D = 256;     // data dimensions supported

template <typename T>
struct Num;

template <>
struct Num<float> {
  using Bits = uint32_t;
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
  static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
  static __device__ __forceinline__ Bits bits(float a) { return __float_as_uint(a); }
  static __device__ __forceinline__ float from_bits(Bits b) { return __uint_as_float(b); }
  static __device__ __forceinline__ float down(double v) { return __double2float_rd(v); }
  static __device__ __forceinline__ float up(double v) { return __double2float_ru(v); }
  // relative slack covering the rounding of a d <= 256 term distance
  static constexpr double ring_margin = 1.0 + 1.0 / 65536.0;
};

template <>
struct Num<double> {
  using Bits = unsigned long long;
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
  static __device__ __forceinline__ double sqrt(double a) { return __dsqrt_rn(a); }
  static __device__ __forceinline__ Bits bits(double a) { return (Bits)__double_as_longlong(a); }
  static __device__ __forceinline__ double from_bits(Bits b) { return __longlong_as_double((long long)b); }
  static __device__ __forceinline__ double down(double v) { return v; }
  static __device__ __forceinline__ double up(double v) { return v; }
  static constexpr double ring_margin = 1.0 + 1.0 / 1099511627776.0;  // 1 + 2^-40
};

// Grid geometry as the kernels see it (cell width eps, NUMINDEXEDDIM = di).
template <typename T>
struct GridGeom {
  T minv[MAX_DI];
  uint32_t ncell[MAX_DI];
  unsigned long long mult[MAX_DI];  // row-major multipliers, dimension 0 fastest
  T width;
  uint32_t di;
  unsigned long long total_cells;
};

// Cell coordinate of a data point: kernel.cu:1690 / kernel.cu:91.
template <typename T>
__device__ __forceinline__ uint32_t point_cell_coord(T x, T minv, T width) {
  return (uint32_t)Num<T>::div(Num<T>::sub(x, minv), width);
}

// The same formula for an arbitrary bound v, clamped into [0, ncell-1].  It
// is monotone in v, so every point with coordinate in [lo, hi] lies in a cell
// between clamped_cell(lo) and clamped_cell(hi).
template <typename T>
__device__ __forceinline__ uint32_t clamped_cell(T v, T minv, T width, uint32_t ncell) {
  if (!(v > minv)) return 0;
  const T u = Num<T>::div(Num<T>::sub(v, minv), width);
  if (!(u < (T)ncell)) return ncell - 1;
  const uint32_t c = (uint32_t)u;
  return c < ncell ? c : ncell - 1;
}

// A lower (up = false) or upper (up = true) bound of the grid cell of
// coordinate v, clamped to [0, ncell-1], from float arithmetic with a
// reciprocal: (v - minf) * invw is within 2^-22 relative of (v - min) / width
// (the rounding of v - minf, of 1/width, of the product, and of min and
// width to float), plus 2^-24 |minf| * invw from rounding min; the bound
// moves by twice that, so the true cell of any coordinate on the far side
// of v (the grid's own monotone division in the data type) is never cut off.
__device__ __forceinline__ uint32_t ring_cell(float v, float minf, float invw, uint32_t ncell, bool up) {
  const float u = (v - minf) * invw;
  const float tol = (fabsf(u) + fabsf(minf) * invw) * (1.0f / 2097152.0f) + (1.0f / 1048576.0f);
  const float ub = up ? u + tol : u - tol;
  if (!(ub > 0.0f)) return 0;
  if (!(ub < (float)ncell)) return ncell - 1;
  const uint32_t c = (uint32_t)ub;
  return c < ncell ? c : ncell - 1;
}

// Largest squared distance accepted at radius r: the reference keeps a point
// when acc <= fl(r*r) (SHORTCIRCUIT, kernel.cu:131-135) and sqrt(acc) <= r
// (kernel.cu:146).  Both are monotone in acc, so one threshold decides both.
__device__ __forceinline__ float within_threshold(float r) {
  const float r2 = __fmul_rn(r, r);
  uint32_t b = __float_as_uint(r2);
  if (__fsqrt_rn(r2) > r) {
    for (int i = 0; i < 16 && b > 0 && __fsqrt_rn(__uint_as_float(b)) > r; i++) b--;
  } else {
    for (int i = 0; i < 16 && __fsqrt_rn(__uint_as_float(b + 1)) <= r; i++) b++;
  }
  const float t = __uint_as_float(b);
  return t < r2 ? t : r2;
}
__device__ __forceinline__ double within_threshold(double r) {
  const double r2 = __dmul_rn(r, r);
  unsigned long long b = (unsigned long long)__double_as_longlong(r2);
  if (__dsqrt_rn(r2) > r) {
    for (int i = 0; i < 16 && b > 0 && __dsqrt_rn(__longlong_as_double((long long)b)) > r; i++) b--;
  } else {
    for (int i = 0; i < 16 && __dsqrt_rn(__longlong_as_double((long long)(b + 1))) <= r; i++) b++;
  }
  const double t = __longlong_as_double((long long)b);
  return t < r2 ? t : r2;
}

// Selection keys: ascending (squared distance, original point id).  Squared
// distances are non-negative, so their IEEE bit patterns order like the values.
template <typename T>
struct Key;

template <>
struct Key<float> {
  using type = unsigned long long;
  static __device__ __forceinline__ type make(float acc, uint32_t id) {
    return ((type)__float_as_uint(acc) << 32) | id;
  }
  static __device__ __forceinline__ type bound(float thr) {
    return ((type)__float_as_uint(thr) << 32) | 0xffffffffull;
  }
  static __device__ __forceinline__ type maxv() { return ~0ull; }
  static __device__ __forceinline__ bool less(const type& x, const type& y) { return x < y; }
  static __device__ __forceinline__ float acc(const type& x) { return __uint_as_float((uint32_t)(x >> 32)); }
  static __device__ __forceinline__ uint32_t id(const type& x) { return (uint32_t)x; }
};

struct KeyF64 {
  unsigned long long a;
  unsigned int id;
  unsigned int pad;
};

template <>
struct Key<double> {
  using type = KeyF64;
  static __device__ __forceinline__ type make(double acc, uint32_t id) {
    type k;
    k.a = (unsigned long long)__double_as_longlong(acc);
    k.id = id;
    k.pad = 0;
    return k;
  }
  static __device__ __forceinline__ type bound(double thr) {
    type k;
    k.a = (unsigned long long)__double_as_longlong(thr);
    k.id = 0xffffffffu;
    k.pad = 0;
    return k;
  }
  static __device__ __forceinline__ type maxv() {
    type k;
    k.a = ~0ull;
    k.id = 0xffffffffu;
    k.pad = 0;
    return k;
  }
  static __device__ __forceinline__ bool less(const type& x, const type& y) {
    return x.a < y.a || (x.a == y.a && x.id < y.id);
  }
  static __device__ __forceinline__ double acc(const type& x) { return __longlong_as_double((long long)x.a); }
  static __device__ __forceinline__ uint32_t id(const type& x) { return x.id; }
};

// The verification sum of one result row (the reference adds dist * dist,
// GPU.cu:3690-3693): each lane's partial sum in the data type, reduced across
// the warp in a fixed butterfly order; lane 0 stores it widened to double.
template <typename T>
__device__ __forceinline__ void store_row_sum(double* __restrict__ rowsum, uint64_t row, T part, int lane) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) part = Num<T>::add(part, __shfl_xor_sync(0xffffffffu, part, off));
  if (lane == 0) rowsum[row] = (double)part;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Bitonic sort of n (a power of two) keys in shared memory by one warp.
template <typename T>
__device__ __forceinline__ void warp_bitonic_sort(typename Key<T>::type* buf, int n, int lane) {
  using K = Key<T>;
  for (int size = 2; size <= n; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = lane; i < (n >> 1); i += 32) {
        const int lo = ((i & ~(stride - 1)) << 1) | (i & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const typename K::type x = buf[lo];
        const typename K::type y = buf[hi];
        if (K::less(y, x) == up) {
          buf[lo] = y;
          buf[hi] = x;
        }
      }
      __syncwarp();
    }
  }
}

}  // namespace knnsj
