// k_outlier.cu -- outlier scores of a finished result table on the device.
//
// Restates printOutlierScores (main.cu:952-1067) on the GPU for a table that
// is already in device memory:
//   criterion 1: each point's total distance to its K table entries, summed
//     in the data type in entry order (main.cu:963-968: a thread per row, the
//     same additions in the same order, so the totals are bit-identical), and
//     the mean total / (K - 1) widened to double as the reference prints it;
//     its rank: position in the order of decreasing total (main.cu:980-989);
//   criterion 2: each point's in-degree, the number of table entries naming
//     it (main.cu:1013-1022), by atomics (exact integers); its rank: position
//     in the order of increasing in-degree (main.cu:1025-1033).
// The orders come from the library's stable LSD radix sort, so equal scores
// are ranked by ascending point id.  The reference ranks equal scores in
// whatever order std::sort leaves them (an unstable sort); the file writer
// knnsj_write_outlier_scores keeps that order for byte-identical output, and
// these device ranks equal it wherever scores are distinct.

#include <cstring>

#include "knnsj_internal.h"

namespace knnsj {

namespace {

template <typename T>
__global__ void row_total_kernel(const T* __restrict__ dists, uint64_t n, uint32_t K, T* __restrict__ total,
                                 double* __restrict__ mean) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    T t = 0;
    const T* r = dists + i * K;
    for (uint32_t j = 0; j < K; j++) t = Num<T>::add(t, r[j]);
    total[i] = t;
    mean[i] = __ddiv_rn((double)t, __dsub_rn((double)K * 1.0, 1.0));
  }
}

__global__ void in_degree_kernel(const int32_t* __restrict__ ids, uint64_t count, uint64_t n,
                                 unsigned long long* __restrict__ indeg) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t id = ids[i];
    if (id >= 0 && (uint64_t)id < n) atomicAdd(&indeg[id], 1ull);
  }
}

// Sort keys: decreasing total (an order-preserving map of the non-negative
// float bits, complemented) and increasing in-degree; values = point ids.
template <typename T>
__global__ void total_keys_kernel(const T* __restrict__ total, uint64_t n, unsigned long long* __restrict__ keys,
                                  uint32_t* __restrict__ vals) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    unsigned long long b = (unsigned long long)Num<T>::bits(total[i]);
    const unsigned long long sign = sizeof(T) == 4 ? 0x80000000ull : 0x8000000000000000ull;
    const unsigned long long mask = sizeof(T) == 4 ? 0xffffffffull : ~0ull;
    // IEEE order as unsigned: flip every bit of negatives, the sign of positives
    b = (b & sign) ? (~b & mask) : (b | sign);
    keys[i] = ~b & mask;  // decreasing
    vals[i] = (uint32_t)i;
  }
}

__global__ void degree_keys_kernel(const unsigned long long* __restrict__ indeg, uint64_t n,
                                   unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    keys[i] = indeg[i];
    vals[i] = (uint32_t)i;
  }
}

template <typename R>
__global__ void rank_scatter_kernel(const uint32_t* __restrict__ sorted_ids, uint64_t n, R* __restrict__ rank) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    rank[sorted_ids[i]] = (R)i;
}

unsigned blocks_for(uint64_t n) {
  uint64_t b = (n + 255) / 256;
  if (b > 152ull * 32) b = 152ull * 32;
  return (unsigned)(b ? b : 1);
}

int bits_of(unsigned long long v) {
  int b = 0;
  while (b < 64 && (v >> b) != 0) b++;
  return b;
}

}  // namespace

template <typename T>
void outlier_scores_device(Workspace& w, const int32_t* ids, const T* dists, uint64_t n, uint32_t K, double* mean,
                           int32_t* dist_rank, unsigned long long* indeg, uint32_t* degree_rank, cudaStream_t s) {
  GridScratch sc;
  sc.keys[0] = (unsigned long long*)w.keys0.get(n * 8);
  sc.keys[1] = (unsigned long long*)w.keys1.get(n * 8);
  sc.vals[0] = (uint32_t*)w.vals0.get(n * 4);
  sc.vals[1] = (uint32_t*)w.vals1.get(n * 4);
  sc.hist_elems = radix_hist_elems(n);
  sc.hist = (uint32_t*)w.hist.get(sc.hist_elems * 4);
  sc.scan_tmp_elems = scan_tmp_elems(std::max<size_t>(sc.hist_elems, n + 1));
  sc.scan_tmp = (uint32_t*)w.scan_tmp.get(sc.scan_tmp_elems * 4);
  T* total = (T*)w.xs.get(n * sizeof(T));
  // criterion 1: totals, means and the order of decreasing total
  row_total_kernel<T><<<blocks_for(n), 256, 0, s>>>(dists, n, K, total, mean);
  KNNSJ_CHECK_LAUNCH();
  total_keys_kernel<T><<<blocks_for(n), 256, 0, s>>>(total, n, sc.keys[0], sc.vals[0]);
  KNNSJ_CHECK_LAUNCH();
  int cur = radix_sort_pairs(sc, n, (int)(8 * sizeof(T)), s);
  rank_scatter_kernel<int32_t><<<blocks_for(n), 256, 0, s>>>(sc.vals[cur], n, dist_rank);
  KNNSJ_CHECK_LAUNCH();
  // criterion 2: in-degrees and the order of increasing in-degree
  KNNSJ_CUDA(cudaMemsetAsync(indeg, 0, n * sizeof(unsigned long long), s));
  in_degree_kernel<<<blocks_for(n * K), 256, 0, s>>>(ids, n * K, n, indeg);
  KNNSJ_CHECK_LAUNCH();
  degree_keys_kernel<<<blocks_for(n), 256, 0, s>>>(indeg, n, sc.keys[0], sc.vals[0]);
  KNNSJ_CHECK_LAUNCH();
  cur = radix_sort_pairs(sc, n, std::max(bits_of(n * (unsigned long long)K), 1), s);
  rank_scatter_kernel<uint32_t><<<blocks_for(n), 256, 0, s>>>(sc.vals[cur], n, degree_rank);
  KNNSJ_CHECK_LAUNCH();
}

template void outlier_scores_device<float>(Workspace&, const int32_t*, const float*, uint64_t, uint32_t, double*,
                                           int32_t*, unsigned long long*, uint32_t*, cudaStream_t);
template void outlier_scores_device<double>(Workspace&, const int32_t*, const double*, uint64_t, uint32_t, double*,
                                            int32_t*, unsigned long long*, uint32_t*, cudaStream_t);

}  // namespace knnsj
