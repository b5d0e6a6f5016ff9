// Device check of knnsj::exact_sqrt (csrc/exact_sqrt.cuh): every result must
// equal the GPU's correctly rounded double sqrt bit for bit, on 2^28 inputs
// per kind: hashed bit patterns over the whole positive range (subnormals
// included), sums of two squared floats (the BETA estimator's own terms),
// and perfect squares with their neighbours.  Built and run by
// tests/test_exact_sqrt.py on a GPU.
#include "exact_sqrt.cuh"
#include <cstdio>
#include <cuda_runtime.h>

__device__ unsigned long long g_bad = 0;
__device__ unsigned long long g_first[4];

__device__ __forceinline__ uint64_t mix(uint64_t z) {  // splitmix64 finaliser
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ void check(double x) {
  const double a = knnsj::exact_sqrt(x), b = __dsqrt_rn(x);
  if (__double_as_longlong(a) != __double_as_longlong(b)) {
    const unsigned long long i = atomicAdd(&g_bad, 1ull);
    if (i < 4) g_first[i] = (unsigned long long)__double_as_longlong(x);
  }
}

__global__ void check_kernel(uint64_t n, int kind) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t h = mix(i * 4 + (uint64_t)kind);
    if (kind == 0) {
      check(__longlong_as_double((long long)(h & 0x7fefffffffffffffull)));
    } else if (kind == 1) {
      const float a = __uint_as_float((uint32_t)(h & 0x7f7fffffu) % 0x4b000000u);  // below 2^23
      const float c = __uint_as_float((uint32_t)(h >> 32) % 0x4b000000u);
      check(__dadd_rn((double)__fmul_rn(a, a), (double)__fmul_rn(c, c)));
    } else {
      const double s = (double)(h >> 11);  // exact: < 2^53
      const double q = __dmul_rn(s, s);
      check(q);
      check(__longlong_as_double(__double_as_longlong(q) - 1));
      check(__longlong_as_double(__double_as_longlong(q) + 1));
    }
  }
}

int main() {
  const uint64_t n = 1ull << 28;
  for (int kind = 0; kind < 3; kind++) check_kernel<<<1024, 256>>>(n, kind);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    printf("cuda error\n");
    return 2;
  }
  unsigned long long bad = 0, first[4] = {0, 0, 0, 0};
  cudaMemcpyFromSymbol(&bad, g_bad, sizeof(bad));
  cudaMemcpyFromSymbol(first, g_first, sizeof(first));
  for (unsigned long long i = 0; i < bad && i < 4; i++) printf("x bits %016llx\n", first[i]);
  printf("n=%llu bad=%llu\n", (unsigned long long)(n * 5), bad);
  return bad != 0;
}
