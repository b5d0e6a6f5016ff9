// knnsj_host.h -- host-side pieces of the reference pipeline shared by the
// GPU pipeline (join.cu), the host-only C-ABI helpers (hostio.cpp) and the
// CLI.  Everything here is plain C++; the library is compiled with
// -ffp-contract=off so these computations round exactly as written, on x86
// and on Arm alike.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/knnsj.h"

namespace knnsj {

// Per-call configuration after defaults and environment overrides.
struct JoinConfig {
  uint32_t num_indexed_dims = 0;
  double beta = 0.05;
  int no_reorder = 0;
  int radius_mode = KNNSJ_RADIUS_BETA;
  int max_iterations = 0;
  int verbose = 0;
  int dense_mode = 1;  // 0 never, 1 auto, 2 always (testing)
  double radius_offset = 0.0;  // added to the learned log-radius
  unsigned long long dense_cells_cap = 0;  // largest grid given a dense cell table; 0 = default
  int use_graph = 1;                       // retry passes after the first inside a CUDA graph
  int float_prefilter = 1;                 // double data: float distances screen candidates first
  int search_warps = 0;                    // search launch shape (0 = default), see SearchShape
  int search_qchunk = 0;
  int search_buffer = 0;
  int tail_brute = 1;                      // a few queries whose radius outgrew the grid are finished by
                                           // an exact scan over all points (2: at any due rebuild; 0: off)
  int row_chunks = 32;                     // with direct_rows 0: rows streamed out of the device table
                                           // in this many blocks while the join runs (< 2: at the end)
  int tile_search = 1;                     // first pass of 2-D / 3-D float data over a finer grid: 0 off,
                                           // 1 query tiles (k_tile.cu) for per-query radii and one warp
                                           // per query for a uniform radius, 2 always one warp per query,
                                           // 3 always query tiles
  int tile_fine = 0;                       // that grid's cells: eps0 / tile_fine (0: 4 for tiles, 2 else)
  int direct_rows = 2;                     // pinned outputs: 2 a device table copied into them by an SM
                                           // kernel after the join, 1 rows straight from the search
                                           // kernels, 0 a device table streamed by the copy engines
  unsigned long long device_table_cap = 0; // largest device result table (bytes) before pageable outputs
                                           // are registered and written directly; 0 = free memory less 2 GB
};

// ReorderByDimension (main.cu:2521-2615).  `sample` holds rows 0, 100, 200,
// ... of the n x d input (ns = ceil(n/100) rows).  Sums run in DTYPE in row
// order; the denominators use the full n as the reference does
// (main.cu:2569, 2579); dimensions are ordered by std::sort with the
// reference's comparator (compareByDimVariance, main.cu:44-47), so ties fall
// exactly where the reference's std::sort puts them.
template <typename T>
struct DimVar {
  unsigned int dim;
  T variance;
};

template <typename T>
void reorder_from_sample(const T* sample, uint64_t ns, uint64_t n, uint32_t d, uint32_t* perm,
                         T* variances) {
  const int sample_stride = 100;
  const T inv_sample = (T)(1.0 / (sample_stride * 1.0));
  std::vector<DimVar<T>> dv(d);
  for (uint32_t i = 0; i < d; i++) {
    T sum = 0;
    for (uint64_t j = 0; j < ns; j++) sum += sample[j * d + i];
    const T denom = (T)n * inv_sample;
    const T average = sum / denom;
    sum = 0;
    for (uint64_t j = 0; j < ns; j++) {
      const T t = sample[j * d + i] - average;
      const T sq = t * t;
      sum += sq;
    }
    dv[i].variance = sum / denom;
    dv[i].dim = i;
  }
  std::sort(dv.begin(), dv.end(),
            [](const DimVar<T>& a, const DimVar<T>& b) { return a.variance > b.variance; });
  for (uint32_t j = 0; j < d; j++) {
    perm[j] = dv[j].dim;
    if (variances) variances[j] = dv[j].variance;
  }
}

// eps0 from the 10 000-bucket histogram (GPU.cu:3480-3527): the first bucket
// whose cumulative neighbours per sampled point exceed
// k + (100k - k) * BETA (truncated), else the last bucket.
struct EpsChoice {
  double eps;
  int bucket;
  uint32_t sample_blocks;
  bool complete;  // false: the crossing lies beyond the buckets counted so far
};

inline uint32_t eps_offset_host(uint64_t n) {
  const uint32_t N = (uint32_t)n;
  const double offsetRate = 0.01;
  if (N >= 50000) {
    const double frac = (50000.0 / N) * offsetRate;
    return (uint32_t)(1.0 / frac);
  }
  return (uint32_t)(1.0 / offsetRate);
}

// `valid` buckets of hist are counted; when the crossing is not among them
// (and valid < 10000) the choice is marked incomplete.
inline EpsChoice choose_eps(const uint32_t* hist, uint32_t valid, double avg, uint64_t n, uint32_t k,
                            double beta) {
  const uint32_t nbuckets = 10000;
  const double bw = avg / (nbuckets * 1.0);
  const uint32_t blocks2 = (uint32_t)n / eps_offset_host(n);
  uint32_t cumulative = 0;
  EpsChoice c{0.0, -1, blocks2, true};
  bool flag = false;
  const unsigned long min_pts = (unsigned long)(k * 1.0);
  const unsigned long max_pts = (unsigned long)(k * 100.0);
  const unsigned long thr = (unsigned long)(min_pts + (max_pts - min_pts) * beta);
  for (uint32_t i = 0; i < nbuckets; i++) {
    if (i >= valid) {
      if (!flag) c.complete = false;
      break;
    }
    cumulative += hist[i];
    const double cpp = cumulative / (1.0 * blocks2);
    if (cpp > (double)thr && !flag) {
      c.eps = bw * (i + 1.0);
      c.bucket = (int)i;
      flag = true;
    }
    if (i == nbuckets - 1 && c.bucket == -1) {
      c.eps = bw * (i + 1.0);
      c.bucket = (int)i;
    }
  }
  return c;
}

// generateNDGridDimensions (main.cu:2425-2488) on row-major data.
template <typename T>
void grid_dims_host(const T* data, uint64_t n, uint32_t d, uint32_t di, T eps, T* minArr, T* maxArr,
                    uint32_t* nCells, uint64_t* totalCells) {
  for (uint32_t j = 0; j < di; j++) {
    minArr[j] = data[j];
    maxArr[j] = data[j];
  }
  for (uint64_t i = 1; i < n; i++)
    for (uint32_t j = 0; j < di; j++) {
      const T v = data[i * d + j];
      if (v < minArr[j]) minArr[j] = v;
      if (v > maxArr[j]) maxArr[j] = v;
    }
  for (uint32_t j = 0; j < di; j++) {
    minArr[j] -= eps;
    maxArr[j] += eps;
  }
  uint64_t tc = 1;
  for (uint32_t j = 0; j < di; j++) {
    const T q = (maxArr[j] - minArr[j]) / eps;
    nCells[j] = (uint32_t)std::ceil(q);
    tc *= nCells[j];
  }
  *totalCells = tc;
}

}  // namespace knnsj
