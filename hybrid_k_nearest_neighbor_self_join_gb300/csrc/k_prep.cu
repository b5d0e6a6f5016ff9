// k_prep.cu -- input preparation on the device.
//
//  * transpose_reorder: row-major N x d input -> d column arrays in the
//    variance order chosen by ReorderByDimension (main.cu:2521-2615; the
//    reference permutes its host vectors, main.cu:2596-2605), flagging NaN /
//    infinite coordinates on the way.
//  * minmax: per-dimension minimum and maximum of the indexed dimensions, the
//    first half of generateNDGridDimensions (main.cu:2425-2460).

#include <cfloat>

#include "exact_sqrt.cuh"
#include "knnsj_internal.h"

namespace knnsj {

namespace {

template <typename T>
__global__ void transpose_reorder_kernel(const T* __restrict__ aos, T* __restrict__ soa, uint64_t n,
                                         uint32_t d, const uint32_t* __restrict__ perm,
                                         uint32_t* __restrict__ nonfinite) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    for (uint32_t j = 0; j < d; j++) {
      const T v = aos[i * d + perm[j]];
      bad |= !isfinite(v);
      soa[(uint64_t)j * n + i] = v;
    }
  }
  if (__any_sync(FULL, bad) && (threadIdx.x & 31) == 0) atomicOr(nonfinite, 1u);
}

template <typename T>
__device__ __forceinline__ T tmin(T a, T b) { return b < a ? b : a; }
template <typename T>
__device__ __forceinline__ T tmax(T a, T b) { return b > a ? b : a; }

// Stage 1: per-block min/max of each indexed dimension into part[block][2*di].
template <typename T>
__global__ void minmax_kernel(const T* __restrict__ soa, uint64_t n, uint32_t di, T* __restrict__ part) {
  __shared__ T smin[32], smax[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (uint32_t j = 0; j < di; j++) {
    T mn = soa[(uint64_t)j * n], mx = mn;
    const T* col = soa + (uint64_t)j * n;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
      const T v = col[i];
      mn = tmin(mn, v);
      mx = tmax(mx, v);
    }
    for (int off = 16; off > 0; off >>= 1) {
      mn = tmin(mn, __shfl_xor_sync(FULL, mn, off));
      mx = tmax(mx, __shfl_xor_sync(FULL, mx, off));
    }
    if (lane == 0) {
      smin[w] = mn;
      smax[w] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 1; k < (int)(blockDim.x >> 5); k++) {
        mn = tmin(mn, smin[k]);
        mx = tmax(mx, smax[k]);
      }
      part[(uint64_t)blockIdx.x * 2 * di + 2 * j] = mn;
      part[(uint64_t)blockIdx.x * 2 * di + 2 * j + 1] = mx;
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void minmax_final_kernel(const T* __restrict__ part, uint32_t nblocks, uint32_t di,
                                    T* __restrict__ out) {
  const uint32_t j = threadIdx.x;
  if (j >= di) return;
  T mn = part[2 * j], mx = part[2 * j + 1];
  for (uint32_t b = 1; b < nblocks; b++) {
    mn = tmin(mn, part[(uint64_t)b * 2 * di + 2 * j]);
    mx = tmax(mx, part[(uint64_t)b * 2 * di + 2 * j + 1]);
  }
  out[2 * j] = mn;
  out[2 * j + 1] = mx;
}

constexpr unsigned CHECKSUM_BLOCKS = 1024;

// Squared distance in DTYPE, widened and added in double (GPU.cu:3690-3693);
// fixed grid, fixed per-thread order and a fixed tree, so the figure is the
// same on every run.
// exact widening to double (float: assembled from bits, off the FP64 pipe)
__device__ __forceinline__ double widen(float x) { return es_f2d(x); }
__device__ __forceinline__ double widen(double x) { return x; }

template <typename T>
__global__ void checksum_kernel(const T* __restrict__ v, uint64_t count, double* __restrict__ part) {
  __shared__ double ws[32];
  double s = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const T x = v[i];
    s = __dadd_rn(s, widen(Num<T>::mul(x, x)));
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(FULL, s, off);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += ws[k];
    part[blockIdx.x] = t;
  }
}

__global__ void checksum_final_kernel(const double* __restrict__ part, unsigned nb, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double t = 0.0;
  for (unsigned b = 0; b < nb; b++) t += part[b];
  *out = t;
}

// Sum of n doubles in a fixed order: grid-stride partial sums per thread,
// warp butterflies, block partials summed in block order.
__global__ void sum_f64_kernel(const double* __restrict__ v, uint64_t count, double* __restrict__ part) {
  __shared__ double ws[32];
  double s = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x)
    s = __dadd_rn(s, v[i]);
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(FULL, s, off);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += ws[k];
    part[blockIdx.x] = t;
  }
}

}  // namespace

void launch_sum_f64(const double* v, uint64_t count, double* d_partial, double* d_out, cudaStream_t s) {
  sum_f64_kernel<<<CHECKSUM_BLOCKS, 256, 0, s>>>(v, count, d_partial);
  KNNSJ_CHECK_LAUNCH();
  checksum_final_kernel<<<1, 32, 0, s>>>(d_partial, CHECKSUM_BLOCKS, d_out);
  KNNSJ_CHECK_LAUNCH();
}

template <typename T>
void launch_checksum(const T* dists, uint64_t count, double* d_partial, double* d_out, cudaStream_t s) {
  checksum_kernel<T><<<CHECKSUM_BLOCKS, 256, 0, s>>>(dists, count, d_partial);
  KNNSJ_CHECK_LAUNCH();
  checksum_final_kernel<<<1, 32, 0, s>>>(d_partial, CHECKSUM_BLOCKS, d_out);
  KNNSJ_CHECK_LAUNCH();
}
template void launch_checksum<float>(const float*, uint64_t, double*, double*, cudaStream_t);
template void launch_checksum<double>(const double*, uint64_t, double*, double*, cudaStream_t);

constexpr uint32_t MINMAX_BLOCKS = 1024;

template <typename T>
void launch_transpose_reorder(const T* aos, T* soa, uint64_t n, uint32_t d, const uint32_t* d_perm,
                              cudaStream_t s, uint32_t* d_nonfinite) {
  uint64_t blocks = (n + 255) / 256;
  if (blocks > 152ull * 32) blocks = 152ull * 32;
  transpose_reorder_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(aos, soa, n, d, d_perm, d_nonfinite);
  KNNSJ_CHECK_LAUNCH();
}

template <typename T>
void launch_minmax(const T* soa, uint64_t n, uint32_t di, T* d_minmax, T* scratch, cudaStream_t s) {
  uint32_t blocks = (uint32_t)((n + 255) / 256);
  if (blocks > MINMAX_BLOCKS) blocks = MINMAX_BLOCKS;
  if (blocks < 1) blocks = 1;
  minmax_kernel<T><<<blocks, 256, 0, s>>>(soa, n, di, scratch);
  KNNSJ_CHECK_LAUNCH();
  minmax_final_kernel<T><<<1, 32, 0, s>>>(scratch, blocks, di, d_minmax);
  KNNSJ_CHECK_LAUNCH();
}

template void launch_transpose_reorder<float>(const float*, float*, uint64_t, uint32_t, const uint32_t*,
                                              cudaStream_t, uint32_t*);
template void launch_transpose_reorder<double>(const double*, double*, uint64_t, uint32_t,
                                               const uint32_t*, cudaStream_t, uint32_t*);
template void launch_minmax<float>(const float*, uint64_t, uint32_t, float*, float*, cudaStream_t);
template void launch_minmax<double>(const double*, uint64_t, uint32_t, double*, double*, cudaStream_t);

}  // namespace knnsj
