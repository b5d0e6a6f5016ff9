// k_eps.cu -- the starting radius eps0 from BETA.
//
// Restates sampleNeighborsBruteForce (GPU.cu:3088-3566) and its kernels:
//   * kernelEstimateAvgDistBruteForce (kernel.cu:343-381): sample thread g
//     takes point 1000*g and sums, in double, its distances to points
//     t, t+1000, ... (t = g mod 256).  The reference adds every distance to
//     one double with atomicAdd, so its mean varies in the last bits from run
//     to run.  Here the order is fixed: sample g's distances are summed in
//     chunks of EPS_CHUNK consecutive terms, the chunk sums in chunk order,
//     then the per-sample sums in 32 contiguous groups of samples (each in
//     sample order, the group sums in group order) -- the oracle's order.
//   * kernelKDistBruteForce (kernel.cu:450-523): block b takes point
//     b*offset and bins its distances below the mean to every 8th block of
//     256 points into 10 000 buckets of width mean/10000, 8 counts per hit.
//     Reads past N (the reference leaves i+threadIdx.x unchecked,
//     kernel.cu:486-492) are skipped and a bucket index that rounds up to
//     10000 is dropped.
// eps0 depends only on the cumulative histogram up to the first bucket whose
// neighbours per sampled point exceed k + (100k - k) * BETA (GPU.cu:3480-
// 3527), so the histogram is built in two bucket ranges: [0, 256) first and
// the rest only when the crossing is not in the first range.
//
// Each histogram distance is first bracketed with float arithmetic and a
// rigorous error bound; when the bracket settles the bucket (and the
// below-mean test) the double sqrt and division are skipped, otherwise they
// are computed exactly as the reference does.  The bucket is always the
// reference's double-precision bucket.

#include "exact_sqrt.cuh"
#include "knnsj_internal.h"

namespace knnsj {

namespace {

constexpr int EPS_BLOCK = 256;
constexpr uint32_t NBUCKETS = 10000;
constexpr uint32_t EPS_CHUNK = 256;
#ifndef KNNSJ_HIST_SPLIT
#define KNNSJ_HIST_SPLIT 16
#endif
constexpr uint32_t HIST_SPLIT = KNNSJ_HIST_SPLIT;  // blocks per histogram sample point
#ifndef KNNSJ_EPS_UNROLL
#define KNNSJ_EPS_UNROLL 4
#endif

// One squared-distance term as the reference's double accumulator receives
// it: a float product widened (no contraction across the type change; the
// widening is assembled from bits, off the FP64 pipe) or a double fma.
__device__ __forceinline__ double eps_term(double acc, float a, float b) {
  const float df = __fsub_rn(a, b);
  return __dadd_rn(acc, es_f2d(__fmul_rn(df, df)));
}
__device__ __forceinline__ double eps_term(double acc, double a, double b) {
  const double df = __dsub_rn(a, b);
  return __fma_rn(df, df, acc);
}

// The first term of the sum, which the reference adds to 0.0: the same value
// without the FP64 addition.
__device__ __forceinline__ double eps_first(float a, float b) {
  const float df = __fsub_rn(a, b);
  return es_f2d(__fmul_rn(df, df));
}
__device__ __forceinline__ double eps_first(double a, double b) {
  const double df = __dsub_rn(a, b);
  return __dmul_rn(df, df);
}

__host__ __device__ __forceinline__ uint64_t terms_of_sample(uint64_t g, uint64_t n) {
  const uint64_t t = g % EPS_BLOCK;
  return t < n ? (n - t + 999) / 1000 : 0;
}

template <typename T>
__global__ void eps_avg_chunk_kernel(const T* __restrict__ soa, uint64_t n, uint32_t d, uint64_t nthr,
                                     uint32_t nchunks, double* __restrict__ partial) {
  // neighbouring lanes take neighbouring samples (the same chunk): their
  // candidates t + 1000 m are neighbouring points, so each load is coalesced
  const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nthr * nchunks) return;
  const uint64_t g = w % nthr;
  const uint32_t c = (uint32_t)(w / nthr);
  const uint64_t tid = g * 1000;
  double s = 0.0;
  if (tid < n) {
    const uint64_t t = g % EPS_BLOCK;
    const uint64_t m_end = min(terms_of_sample(g, n), (uint64_t)(c + 1) * EPS_CHUNK);
    // the sample point's first two coordinates stay in registers
    const T q0 = soa[tid];
    const T q1 = d > 1 ? soa[n + tid] : (T)0;
    // U terms at a time: their loads and square roots are independent; the
    // sum still runs term by term in ascending order
    constexpr int U = KNNSJ_EPS_UNROLL;
    for (uint64_t m = (uint64_t)c * EPS_CHUNK; m < m_end; m += U) {
      double rd[U];
#pragma unroll
      for (int u = 0; u < U; u++) rd[u] = m + u < m_end ? eps_first(soa[t + 1000 * (m + u)], q0) : 0.0;
      for (uint32_t l = 1; l < d; l++) {
        const T ql = l == 1 ? q1 : soa[(uint64_t)l * n + tid];
#pragma unroll
        for (int u = 0; u < U; u++)
          if (m + u < m_end) rd[u] = eps_term(rd[u], soa[(uint64_t)l * n + t + 1000 * (m + u)], ql);
      }
      // the correctly rounded double root, computed on the integer pipes
#pragma unroll
      for (int u = 0; u < U; u++)
        if (m + u < m_end) s = __dadd_rn(s, exact_sqrt(rd[u]));
    }
  }
  partial[g * nchunks + c] = s;
}

__global__ void eps_avg_sample_kernel(const double* __restrict__ partial, uint64_t nthr, uint32_t nchunks,
                                      double* __restrict__ sample_sum) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nthr) return;
  double s = 0.0;
  for (uint32_t c = 0; c < nchunks; c++) s = __dadd_rn(s, partial[g * nchunks + c]);
  sample_sum[g] = s;
}

// One warp: lane j adds the per-sample sums of the j-th of 32 contiguous
// groups of samples in sample order, then the 32 group sums are added in
// group order; cnt = number of terms.
__global__ void eps_avg_final_kernel(const double* __restrict__ sample_sum, uint64_t nthr, unsigned long long cnt,
                                     double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const uint64_t group = (nthr + 31) / 32;
  const uint64_t g_end = min(nthr, (uint64_t)(lane + 1) * group);
  double gs = 0.0;
  for (uint64_t g = (uint64_t)lane * group; g < g_end; g++) gs = __dadd_rn(gs, sample_sum[g]);
  double tot = 0.0;
  for (int j = 0; j < 32; j++) tot = __dadd_rn(tot, __shfl_sync(FULL, gs, j));
  if (lane == 0) {
    out[0] = __ddiv_rn(tot, (double)cnt);  // GPU.cu:3339: total/(cnt*1.0)
    out[1] = (double)cnt;
  }
}

// Exact reference bucket of a squared distance rd (double).  Returns
// NBUCKETS when the pair is not counted.
__device__ __forceinline__ uint32_t exact_bucket(double rd, double avg, double bw) {
  const double s = __dsqrt_rn(rd);
  if (!(s < avg)) return NBUCKETS;
  const uint32_t b = (uint32_t)__ddiv_rn(s, bw);
  return b < NBUCKETS ? b : NBUCKETS;
}

// Counts the buckets in [b_lo, b_hi) of sample blocks.  abs_err bounds the
// float bracket's absolute distance error from rounding the coordinates to
// float (0 for float data).
template <typename T>
__global__ void __launch_bounds__(EPS_BLOCK) eps_hist_kernel(const T* __restrict__ soa, uint64_t n, uint32_t d,
                                                             uint32_t offset, const double* __restrict__ avg_in,
                                                             uint32_t* __restrict__ hist, uint32_t b_lo,
                                                             uint32_t b_hi, double abs_err) {
  extern __shared__ uint32_t sh[];  // the b_hi - b_lo counted buckets
  const uint32_t nb = b_hi - b_lo;
  for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const double avg = avg_in[0];
  const double bw = __ddiv_rn(avg, NBUCKETS * 1.0);  // GPU.cu:3356
  // HIST_SPLIT blocks share one sample point, each taking every
  // HIST_SPLIT-th round of candidates (integer counts: the order of the
  // additions does not matter)
  const uint64_t sid = (uint64_t)(blockIdx.x / HIST_SPLIT) * offset;
  const uint32_t part = blockIdx.x % HIST_SPLIT;
  const float inv_bw = (float)(1.0 / bw);
  const float errc = (float)(2 * d + 8) * 5.9604645e-8f;  // (2d+8) * 2^-24, relative
  const float abs_q = (float)(abs_err / bw) * 1.0001f + 1e-4f;
  const float flo = (float)b_lo, fhi = (float)b_hi;
  // squared-distance prefilter: a pair whose float squared distance is at
  // least s_hi has q32 - del >= fhi (the bracket below puts it above the
  // counted range) -- q32 is within 2^-23 of sqrt(s32) / bw, and s_hi is
  // widened by 2^-20 for its own rounding -- so it is skipped without a root
  const double q_need = ((double)fhi + (double)abs_q) / (1.0 - (double)errc);
  const double sq_bw = q_need * bw / ((1.0 - 1.0 / 8388608.0) * (1.0 - 1.0 / 8388608.0));
  const float s_hi = __double2float_ru(sq_bw * sq_bw * (1.0 + 1.0 / 1048576.0));
  // the sample point's coordinates once per block; four candidates per
  // thread and round so that their loads overlap
  __shared__ T qs[MAX_D];
  for (uint32_t l = threadIdx.x; l < d; l += blockDim.x) qs[l] = soa[(uint64_t)l * n + sid];
  __syncthreads();
  constexpr uint64_t STEP = (uint64_t)EPS_BLOCK * 8;
  constexpr int U = 4;
  for (uint64_t i0 = (uint64_t)part * STEP * U; i0 < n; i0 += STEP * U * HIST_SPLIT) {
    float s4[U];
#pragma unroll
    for (int u = 0; u < U; u++) s4[u] = 0.0f;
    for (uint32_t l = 0; l < d; l++) {
      const float qf = (float)qs[l];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const uint64_t p = i0 + u * STEP + threadIdx.x;
        if (p < n) {
          const float df = __fsub_rn((float)soa[(uint64_t)l * n + p], qf);
          s4[u] = __fadd_rn(s4[u], __fmul_rn(df, df));
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const uint64_t p = i0 + u * STEP + threadIdx.x;
      if (p >= n || p == sid) continue;
      const float s32 = s4[u];
      if (s32 >= s_hi) continue;
      const float q32 = __fmul_rn(__fsqrt_rn(s32), inv_bw);
      const float del = __fmaf_rn(errc, q32, abs_q);
      if (q32 - del >= 10000.5f) continue;  // certainly not below the mean
      if (q32 + del < flo) continue;        // below this bucket range
      if (q32 - del >= fhi) continue;       // above this bucket range
      uint32_t bucket;
      const float fb = floorf(q32);
      if (q32 + del < 9999.9f && q32 - del > fb && q32 + del < fb + 1.0f) {
        bucket = (uint32_t)fb;
      } else {
        double rd = 0.0;
        for (uint32_t l = 0; l < d; l++) rd = eps_term(rd, soa[(uint64_t)l * n + p], qs[l]);
        bucket = exact_bucket(rd, avg, bw);
      }
      if (bucket >= b_lo && bucket < b_hi) atomicAdd(&sh[bucket - b_lo], 8u);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[b_lo + i], sh[i]);
}

}  // namespace

uint64_t eps_avg_threads(uint64_t n) {
  // GPU.cu:3275: TOTALBLOCKS = ceil((0.001*N)/(1.0*BLOCKSIZE))
  const int blocks = (int)std::ceil((0.001 * (double)(uint32_t)n) / (1.0 * EPS_BLOCK));
  return (uint64_t)blocks * EPS_BLOCK;
}

uint32_t eps_avg_chunks(uint64_t n) {
  const uint64_t m = terms_of_sample(0, n);
  return (uint32_t)std::max<uint64_t>(1, (m + EPS_CHUNK - 1) / EPS_CHUNK);
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
void launch_eps_avg(const T* soa, uint64_t n, uint32_t d, const EpsScratch& sc, cudaStream_t s) {
  const uint64_t nthr = eps_avg_threads(n);
  const uint32_t nch = eps_avg_chunks(n);
  const uint64_t work = nthr * nch;
  if (work > 0) {
    eps_avg_chunk_kernel<T><<<(unsigned)((work + 255) / 256), 256, 0, s>>>(soa, n, d, nthr, nch, sc.partial);
    KNNSJ_CHECK_LAUNCH();
    eps_avg_sample_kernel<<<(unsigned)((nthr + 255) / 256), 256, 0, s>>>(sc.partial, nthr, nch, sc.sample_sum);
    KNNSJ_CHECK_LAUNCH();
  }
  // number of distances summed (the reference counts them with an atomic,
  // kernel.cu:366): every sample thread g with 1000*g < N
  unsigned long long cnt = 0;
  for (uint64_t g = 0; g < nthr; g++)
    if (g * 1000 < n) cnt += terms_of_sample(g, n);
  eps_avg_final_kernel<<<1, 32, 0, s>>>(sc.sample_sum, nthr, cnt, sc.avg_out);
  KNNSJ_CHECK_LAUNCH();
}

template <typename T>
void launch_eps_hist(const T* soa, uint64_t n, uint32_t d, const EpsScratch& sc, uint32_t b_lo, uint32_t b_hi,
                     double abs_err, cudaStream_t s) {
  const uint32_t offset = eps_sample_offset(n);
  const uint32_t blocks2 = (uint32_t)n / offset;  // GPU.cu:3440 (integer division)
  if (blocks2 > 0 && b_hi > b_lo) {
    // shared memory for the counted bucket range only (256 buckets on the
    // first try: a small footprint lets more blocks share an SM)
    eps_hist_kernel<T><<<blocks2 * HIST_SPLIT, EPS_BLOCK, (size_t)(b_hi - b_lo) * 4, s>>>(
        soa, n, d, offset, sc.avg_out, sc.hist, b_lo, b_hi, abs_err);
    KNNSJ_CHECK_LAUNCH();
  }
}

template void launch_eps_avg<float>(const float*, uint64_t, uint32_t, const EpsScratch&, cudaStream_t);
template void launch_eps_avg<double>(const double*, uint64_t, uint32_t, const EpsScratch&, cudaStream_t);
template void launch_eps_hist<float>(const float*, uint64_t, uint32_t, const EpsScratch&, uint32_t, uint32_t,
                                     double, cudaStream_t);
template void launch_eps_hist<double>(const double*, uint64_t, uint32_t, const EpsScratch&, uint32_t, uint32_t,
                                      double, cudaStream_t);

}  // namespace knnsj
