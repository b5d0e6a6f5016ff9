// k_eps.cu -- the starting radius eps0 from BETA.
//
// Restates sampleNeighborsBruteForce (GPU.cu:3088-3566) and its kernels:
//   * kernelEstimateAvgDistBruteForce (kernel.cu:343-381): sample thread g
//     takes point 1000*g and sums its distances to points t, t+1000, ...
//     (t = g mod 256) in double.  The reference adds every distance to one
//     double with atomicAdd, so its mean varies in the last bits from run to
//     run; here each thread sums in loop order and one thread then adds the
//     per-thread sums in thread order, a fixed order the oracle repeats.
//   * kernelKDistBruteForce (kernel.cu:450-523): block b takes point
//     b*offset and bins its distances below the mean to every 8th block of
//     256 points into 10 000 buckets of width mean/10000, 8 counts per hit.
//     Reads past N (the reference leaves i+threadIdx.x unchecked,
//     kernel.cu:486-492) are skipped and a bucket index that rounds up to
//     10000 is dropped.
// The host then picks eps0 from the cumulative histogram (GPU.cu:3480-3527).
//
// For float data each histogram distance is first bracketed in float: when
// the bracket decides the bucket (and the below-mean test) unambiguously, the
// double sqrt and division of the reference are skipped; otherwise they are
// computed exactly as the reference does.  Either way the bucket equals the
// reference's double-precision bucket.

#include "knnsj_internal.h"

namespace knnsj {

namespace {

constexpr int EPS_BLOCK = 256;
constexpr uint32_t NBUCKETS = 10000;

// One squared-distance term as the reference's double accumulator receives
// it: a float product widened (no contraction across the type change) or a
// double fma.
__device__ __forceinline__ double eps_term(double acc, float a, float b) {
  const float df = __fsub_rn(a, b);
  return __dadd_rn(acc, (double)__fmul_rn(df, df));
}
__device__ __forceinline__ double eps_term(double acc, double a, double b) {
  const double df = __dsub_rn(a, b);
  return __fma_rn(df, df, acc);
}

template <typename T>
__global__ void eps_avg_kernel(const T* __restrict__ soa, uint64_t n, uint32_t d, uint64_t nthr,
                               double* __restrict__ partial, unsigned long long* __restrict__ pcount) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nthr) return;
  const uint64_t tid = g * 1000;
  if (tid >= n) {
    partial[g] = 0.0;
    pcount[g] = 0;
    return;
  }
  const uint64_t t = g % EPS_BLOCK;
  double s = 0.0;
  unsigned long long c = 0;
  for (uint64_t i = t; i < n; i += 1000) {
    double rd = 0.0;
    for (uint32_t l = 0; l < d; l++) rd = eps_term(rd, soa[(uint64_t)l * n + i], soa[(uint64_t)l * n + tid]);
    s = __dadd_rn(s, __dsqrt_rn(rd));
    c++;
  }
  partial[g] = s;
  pcount[g] = c;
}

__global__ void eps_avg_final_kernel(const double* __restrict__ partial,
                                     const unsigned long long* __restrict__ pcount, uint64_t nthr,
                                     double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double tot = 0.0;
  unsigned long long cnt = 0;
  for (uint64_t g = 0; g < nthr; g++) {
    tot = __dadd_rn(tot, partial[g]);
    cnt += pcount[g];
  }
  out[0] = __ddiv_rn(tot, (double)cnt);  // GPU.cu:3339: total/(cnt*1.0)
  out[1] = (double)cnt;
}

// Exact reference bucket of a squared distance rd (double).  Returns
// NBUCKETS when the pair is not counted.
__device__ __forceinline__ uint32_t exact_bucket(double rd, double avg, double bw) {
  const double s = __dsqrt_rn(rd);
  if (!(s < avg)) return NBUCKETS;
  const uint32_t b = (uint32_t)__ddiv_rn(s, bw);
  return b < NBUCKETS ? b : NBUCKETS;
}

template <typename T>
__global__ void __launch_bounds__(EPS_BLOCK) eps_hist_kernel(const T* __restrict__ soa, uint64_t n,
                                                             uint32_t d, uint32_t offset,
                                                             const double* __restrict__ avg_in,
                                                             uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[NBUCKETS];
  for (uint32_t i = threadIdx.x; i < NBUCKETS; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const double avg = avg_in[0];
  const double bw = __ddiv_rn(avg, NBUCKETS * 1.0);  // GPU.cu:3356
  const uint64_t sid = (uint64_t)blockIdx.x * offset;
  // float bracket (used for float data only)
  const float inv_bw = (float)(1.0 / bw);
  const float errc = (float)(2 * d + 8) * 5.9604645e-8f;  // (2d+8) * 2^-24
  const float q_far = 10000.5f;
  for (uint64_t i = 0; i < n; i += (uint64_t)EPS_BLOCK * 8) {
    const uint64_t p = i + threadIdx.x;
    if (p >= n || p == sid) continue;
    uint32_t bucket = NBUCKETS;
    if constexpr (sizeof(T) == 4) {
      float s32 = 0.0f;
      for (uint32_t l = 0; l < d; l++) {
        const float df = __fsub_rn((float)soa[(uint64_t)l * n + p], (float)soa[(uint64_t)l * n + sid]);
        s32 = __fadd_rn(s32, __fmul_rn(df, df));
      }
      const float q32 = __fmul_rn(__fsqrt_rn(s32), inv_bw);
      const float del = __fmaf_rn(errc, q32, 1e-4f);
      if (q32 - del > q_far) continue;  // certainly not below the mean
      const float fb = floorf(q32);
      if (q32 + del < 9999.9f && q32 - del > fb && q32 + del < fb + 1.0f) {
        bucket = (uint32_t)fb;
      } else {
        double rd = 0.0;
        for (uint32_t l = 0; l < d; l++) rd = eps_term(rd, soa[(uint64_t)l * n + p], soa[(uint64_t)l * n + sid]);
        bucket = exact_bucket(rd, avg, bw);
      }
    } else {
      double rd = 0.0;
      for (uint32_t l = 0; l < d; l++) rd = eps_term(rd, soa[(uint64_t)l * n + p], soa[(uint64_t)l * n + sid]);
      bucket = exact_bucket(rd, avg, bw);
    }
    if (bucket < NBUCKETS) atomicAdd(&sh[bucket], 8u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < NBUCKETS; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

}  // namespace

uint64_t eps_avg_threads(uint64_t n) {
  // GPU.cu:3275: TOTALBLOCKS = ceil((0.001*N)/(1.0*BLOCKSIZE))
  const int blocks = (int)std::ceil((0.001 * (double)(uint32_t)n) / (1.0 * EPS_BLOCK));
  return (uint64_t)blocks * EPS_BLOCK;
}

uint32_t eps_sample_offset(uint64_t n) {
  // GPU.cu:3400-3412
  const uint32_t N = (uint32_t)n;
  const double offsetRate = 0.01;
  if (N >= 50000) {
    const double frac = (50000.0 / N) * offsetRate;
    return (uint32_t)(1.0 / frac);
  }
  return (uint32_t)(1.0 / offsetRate);
}

template <typename T>
void launch_eps(const T* soa, uint64_t n, uint32_t d, const EpsScratch& sc, cudaStream_t s) {
  const uint64_t nthr = eps_avg_threads(n);
  if (nthr > 0) {
    eps_avg_kernel<T><<<(unsigned)(nthr / EPS_BLOCK), EPS_BLOCK, 0, s>>>(soa, n, d, nthr, sc.partial,
                                                                      sc.pcount);
    KNNSJ_CHECK_LAUNCH();
  }
  eps_avg_final_kernel<<<1, 32, 0, s>>>(sc.partial, sc.pcount, nthr, sc.avg_out);
  KNNSJ_CHECK_LAUNCH();
  KNNSJ_CUDA(cudaMemsetAsync(sc.hist, 0, NBUCKETS * sizeof(uint32_t), s));
  const uint32_t offset = eps_sample_offset(n);
  const uint32_t blocks2 = (uint32_t)n / offset;  // GPU.cu:3440 (integer division)
  if (blocks2 > 0) {
    eps_hist_kernel<T><<<blocks2, EPS_BLOCK, 0, s>>>(soa, n, d, offset, sc.avg_out, sc.hist);
    KNNSJ_CHECK_LAUNCH();
  }
}

template void launch_eps<float>(const float*, uint64_t, uint32_t, const EpsScratch&, cudaStream_t);
template void launch_eps<double>(const double*, uint64_t, uint32_t, const EpsScratch&, cudaStream_t);

}  // namespace knnsj
