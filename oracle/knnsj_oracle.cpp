// knnsj_oracle.cpp -- CPU oracle for the exact kNN self-join.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, on the CPU, the algorithm of
// the reference GPU-only kNN self-join (mgowanlock/hybrid_k_nearest_neighbor_
// self_join).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline / reference arm may load it, and only as the checker or the timed
// CPU baseline.  The product library never links, loads or calls it.
//
// Parity status: the dimension reorder, the grid dimensions, the grid index
// (cell ids, non-empty cell table, point lookup array), the CSV parse, the
// KNN_out text format and the outlier scores are pinned against the
// reference's own host code compiled from its sources (tests/golden/, made by
// tests/golden/make_golden.py through oracle/build_ref_host.sh).  The
// epsilon estimator and the range search live in the reference only as CUDA
// kernels; their restatement below follows kernel.cu / GPU.cu line by line
// and is cross-checked against an independent brute-force definition.  The
// range search's arithmetic is also pinned on the GPU against the reference
// kernel itself: tests/test_reference_kernel.py runs kernelNDGridIndexGlobalkNN
// (compiled from the reference's kernel.cu by build_ref_kernel.sh, launched
// by ref_kernel_runner.cpp) and requires its within-epsilon pairs to equal
// orc_range_* bit for bit.
//
// Arithmetic conventions (shared with the CUDA path):
//   * squared distance: acc = fma(p_l - q_l, p_l - q_l, acc) for l = 0..d-1
//     over the variance-reordered dimensions, starting at acc = 0.  This is
//     how nvcc (default --fmad=true) compiles
//     `runningTotalDist += (p-q)*(p-q)` in evalPoint (kernel.cu:116-161).
//   * reported distance: IEEE sqrt of acc in DTYPE (kernel.cu:144).
//   * within-epsilon test: acc <= fl(eps*eps) (the SHORTCIRCUIT exit at
//     kernel.cu:131-135 fires exactly when the final acc exceeds it, because
//     partial sums never decrease) and sqrt(acc) <= eps (kernel.cu:146).
//   * neighbour order: ascending (acc, point id).  The reference sorts by
//     distance and leaves equal distances in atomic-append order
//     (GPU.cu:1629-1634); ordering ties by id is one of its possible outputs.
//
// Build: oracle/build_oracle.sh (g++ -O2 -fopenmp -ffp-contract=off).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>
#include <omp.h>
#include <parallel/algorithm>

namespace {

// ---------------------------------------------------------------------------
// ReorderByDimension, main.cu:2521-2615.
// Variance of every dimension over every 100th point, DTYPE accumulation in
// serial order, then std::sort descending by variance (compareByDimVariance,
// main.cu:44-47).  Returns perm[j] = original dimension placed at slot j.
// ---------------------------------------------------------------------------
template <typename T>
struct DimVariance {
  unsigned int dim;
  T variance;
};

template <typename T>
void reorder_permutation(const T* data, uint64_t n, uint32_t d, uint32_t* perm,
                         T* variance_out) {
  const int sample = 100;
  const T inv_sample = (T)(1.0 / (sample * 1.0));
  std::vector<DimVariance<T>> dv(d);
  for (uint32_t i = 0; i < d; i++) {
    T sum = 0;
    for (uint64_t j = 0; j < n; j += sample) sum += data[j * d + i];
    const T denom = (T)n * inv_sample;
    const T average = sum / denom;
    sum = 0;
    for (uint64_t j = 0; j < n; j += sample) {
      const T t = data[j * d + i] - average;
      const T sq = t * t;
      sum += sq;
    }
    dv[i].variance = sum / denom;
    dv[i].dim = i;
  }
  std::sort(dv.begin(), dv.end(),
            [](const DimVariance<T>& a, const DimVariance<T>& b) {
              return a.variance > b.variance;
            });
  for (uint32_t j = 0; j < d; j++) {
    perm[j] = dv[j].dim;
    if (variance_out) variance_out[j] = dv[j].variance;
  }
}

template <typename T>
std::vector<T> apply_permutation(const T* data, uint64_t n, uint32_t d,
                                 const uint32_t* perm) {
  std::vector<T> out((size_t)n * d);
  for (uint64_t i = 0; i < n; i++)
    for (uint32_t j = 0; j < d; j++) out[i * d + j] = data[i * d + perm[j]];
  return out;
}

// Squared-distance term as the reference's double accumulators receive it:
// for DTYPE=float the product is rounded to float and then widened
// (kernel.cu:360-362, 480-482 -- no contraction across the type change);
// for DTYPE=double the statement contracts to one fma.
inline double accum_term(double acc, float a, float b) {
  const float df = a - b;
  const float pr = df * df;
  return acc + (double)pr;
}
inline double accum_term(double acc, double a, double b) {
  const double df = a - b;
  return std::fma(df, df, acc);
}

inline float fma_t(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double fma_t(double a, double b, double c) { return std::fma(a, b, c); }

// ---------------------------------------------------------------------------
// sampleNeighborsBruteForce, GPU.cu:3088-3566, with its two kernels
// kernelEstimateAvgDistBruteForce (kernel.cu:343-381) and
// kernelKDistBruteForce (kernel.cu:450-523).
//
// Deviations, all documented in the returned statistics' meaning:
//   * the mean distance is summed per sample thread in chunks of 256 terms
//     (chunk sums added in order), then over sample threads: 32 contiguous
//     groups of threads each in thread order, the group sums in group order
//     (the reference uses a double atomicAdd, whose order -- and so the last
//     bits of the mean -- varies run to run);
//   * histogram reads past N (kernel.cu:486-492 leaves i+threadIdx.x
//     unchecked) are skipped, and a bucket index that rounds up to nbuckets
//     is dropped instead of written past the histogram.
// ---------------------------------------------------------------------------
struct EpsResult {
  double avg;
  uint64_t pair_count;
  double bucket_width;
  uint32_t offset;
  uint32_t n_sample_blocks;
  int bucket;
  double eps_double;
};

template <typename T>
EpsResult estimate_epsilon(const T* X, uint64_t n, uint32_t d, uint32_t k,
                           double beta, std::vector<uint32_t>* hist_out,
                           int nthreads) {
  EpsResult r{};
  const uint32_t N = (uint32_t)n;
  const int BLOCK = 256;
  // GPU.cu:3275: TOTALBLOCKS=ceil((0.001*N)/(1.0*BLOCKSIZE))
  const int total_blocks = (int)std::ceil((0.001 * N) / (1.0 * BLOCK));
  const uint64_t nthr = (uint64_t)total_blocks * BLOCK;
  std::vector<double> partial(nthr, 0.0);
  std::vector<uint64_t> pcount(nthr, 0);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
  for (int64_t g = 0; g < (int64_t)nthr; g++) {
    const uint64_t tid = (uint64_t)g * 1000;  // kernel.cu:349
    if (tid >= N) continue;
    const uint32_t t = (uint32_t)(g % BLOCK);  // threadIdx.x
    // fixed summation order: chunks of 256 consecutive terms, chunk sums in
    // chunk order (the CUDA path sums in exactly this order)
    const uint64_t chunk = 256;
    double s = 0.0, cs = 0.0;
    uint64_t c = 0;
    for (uint64_t i = t; i < N; i += 1000) {  // kernel.cu:360
      double rd = 0.0;
      for (uint32_t j = 0; j < d; j++) rd = accum_term(rd, X[i * d + j], X[tid * d + j]);
      rd = std::sqrt(rd);
      cs += rd;
      c++;
      if (c % chunk == 0) {
        s += cs;
        cs = 0.0;
      }
    }
    if (c % chunk != 0) s += cs;
    partial[g] = s;
    pcount[g] = c;
  }
  // per-thread sums: 32 contiguous groups of threads, each summed in thread
  // order, then the 32 group sums in group order (the CUDA path's order)
  double total = 0.0;
  uint64_t cnt = 0;
  const uint64_t group = (nthr + 31) / 32;
  for (uint64_t j = 0; j < 32; j++) {
    double gs = 0.0;
    for (uint64_t g = j * group; g < std::min(nthr, (j + 1) * group); g++) gs += partial[g];
    total += gs;
  }
  for (uint64_t g = 0; g < nthr; g++) cnt += pcount[g];
  r.pair_count = cnt;
  r.avg = total / (cnt * 1.0);  // GPU.cu:3339

  const uint32_t nbuckets = 10000;
  r.bucket_width = r.avg / (nbuckets * 1.0);  // GPU.cu:3356
  // GPU.cu:3400-3412
  const double offsetRate = 0.01;
  uint32_t offset;
  if (N >= 50000) {
    const double frac = (50000.0 / N) * offsetRate;
    offset = (uint32_t)(1.0 / frac);
  } else {
    offset = (uint32_t)(1.0 / offsetRate);
  }
  r.offset = offset;
  const uint32_t blocks2 = N / offset;  // GPU.cu:3440 (integer division)
  r.n_sample_blocks = blocks2;

  std::vector<uint32_t> hist(nbuckets, 0);
  const double avg = r.avg;
  const double bw = r.bucket_width;
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<uint32_t> local(nbuckets, 0);
#pragma omp for schedule(dynamic, 1)
    for (int64_t b = 0; b < (int64_t)blocks2; b++) {
      const uint64_t sid = (uint64_t)b * offset;  // kernel.cu:459
      if (sid >= N) continue;
      const int samplePnts = 8;
      for (uint64_t i = 0; i < N; i += (uint64_t)BLOCK * samplePnts) {  // kernel.cu:479
        for (uint32_t t = 0; t < (uint32_t)BLOCK; t++) {
          const uint64_t p = i + t;
          if (p >= N) continue;  // deviation: the reference reads past N here
          double rd = 0.0;
          // The per-dimension early exit (kernel.cu:484-487) cannot change
          // the outcome: a partial sum whose sqrt exceeds avg leaves a final
          // sum whose sqrt exceeds it too, and both fail the test below.
          for (uint32_t j = 0; j < d; j++) rd = accum_term(rd, X[p * d + j], X[sid * d + j]);
          rd = std::sqrt(rd);
          if (rd < avg && p != sid) {
            const uint32_t bucket = (uint32_t)(rd / bw);
            if (bucket < nbuckets) local[bucket] += (uint32_t)samplePnts;
          }
        }
      }
    }
#pragma omp critical
    for (uint32_t i = 0; i < nbuckets; i++) hist[i] += local[i];
  }

  // GPU.cu:3480-3527: first bucket whose cumulative neighbours per sampled
  // point exceed k + (100k - k) * BETA (truncated to an integer).
  uint32_t cumulative = 0;
  double best = 0.0;
  int found = -1;
  bool flag = false;
  for (uint32_t i = 0; i < nbuckets; i++) {
    cumulative += hist[i];
    const double cpp = cumulative / (1.0 * blocks2);
    const unsigned long min_pts = (unsigned long)(k * 1.0);
    const unsigned long max_pts = (unsigned long)(k * 100.0);
    const unsigned long thr = (unsigned long)(min_pts + (max_pts - min_pts) * beta);
    if (cpp > (double)thr && !flag) {
      best = bw * (i + 1.0);
      found = (int)i;
      flag = true;
    }
    if (i == nbuckets - 1 && found == -1) {
      best = bw * (i + 1.0);
      found = (int)i;
    }
  }
  r.bucket = found;
  r.eps_double = best;
  if (hist_out) *hist_out = hist;
  return r;
}

// ---------------------------------------------------------------------------
// generateNDGridDimensions, main.cu:2425-2488 and the grid index of
// populateNDGridIndexAndLookupArrayGPU (GPU.cu:3715-4067) /
// populateNDGridIndexAndLookupArrayParallel (main.cu:1968-2377).
// ---------------------------------------------------------------------------
template <typename T>
struct Grid {
  uint32_t di = 0;
  T eps = 0;
  std::vector<T> minArr, maxArr;
  std::vector<uint32_t> nCells;
  uint64_t totalCells = 0;
  std::vector<uint64_t> cellKeys;   // sorted non-empty linear ids
  std::vector<int32_t> indexmin;    // grid[c].indexmin
  std::vector<int32_t> indexmax;    // grid[c].indexmax
  std::vector<uint32_t> lookup;     // indexLookupArr
};

template <typename T>
void grid_dimensions(const T* X, uint64_t n, uint32_t d, uint32_t di, T eps, Grid<T>* g) {
  g->di = di;
  g->eps = eps;
  g->minArr.assign(di, 0);
  g->maxArr.assign(di, 0);
  g->nCells.assign(di, 0);
  for (uint32_t j = 0; j < di; j++) {
    g->minArr[j] = X[j];
    g->maxArr[j] = X[j];
  }
  for (uint64_t i = 1; i < n; i++)
    for (uint32_t j = 0; j < di; j++) {
      const T v = X[i * d + j];
      if (v < g->minArr[j]) g->minArr[j] = v;
      if (v > g->maxArr[j]) g->maxArr[j] = v;
    }
  for (uint32_t j = 0; j < di; j++) {
    g->minArr[j] -= eps;
    g->maxArr[j] += eps;
  }
  for (uint32_t j = 0; j < di; j++) {
    const T ext = g->maxArr[j] - g->minArr[j];
    const T q = ext / eps;
    g->nCells[j] = (uint32_t)std::ceil(q);
  }
  uint64_t tc = g->nCells[0];
  for (uint32_t j = 1; j < di; j++) tc *= g->nCells[j];
  g->totalCells = tc;
}

// kernel.cu:1673-1697 and kernel.cu:31-47 (row-major, dimension 0 fastest).
template <typename T>
inline uint64_t point_cell(const T* x, const Grid<T>& g) {
  uint64_t lin = 0, mult = 1;
  for (uint32_t j = 0; j < g.di; j++) {
    const T u = (x[j] - g.minArr[j]) / g.eps;
    const uint32_t c = (uint32_t)u;
    lin += (uint64_t)c * mult;
    mult *= g.nCells[j];
  }
  return lin;
}

template <typename T>
void build_grid(const T* X, uint64_t n, uint32_t d, Grid<T>* g, int nthreads) {
  std::vector<std::pair<uint64_t, uint32_t>> kv(n);
#pragma omp parallel for num_threads(nthreads)
  for (int64_t i = 0; i < (int64_t)n; i++) kv[i] = {point_cell(X + (uint64_t)i * d, *g), (uint32_t)i};
  // stable by construction: the pair sort orders equal cells by point id,
  // as the reference's radix sort_by_key does (GPU.cu:3959).  Parallel as
  // the reference's host grid sort (par_sort.cpp:7-10); pairs are unique, so
  // the order does not depend on the sorting algorithm.
  __gnu_parallel::sort(kv.begin(), kv.end());
  g->lookup.resize(n);
  g->cellKeys.clear();
  g->indexmin.clear();
  g->indexmax.clear();
  for (uint64_t i = 0; i < n; i++) {
    g->lookup[i] = kv[i].second;
    if (i == 0 || kv[i].first != kv[i - 1].first) {
      if (i > 0) g->indexmax.push_back((int32_t)(i - 1));
      g->cellKeys.push_back(kv[i].first);
      g->indexmin.push_back((int32_t)i);
    }
  }
  if (n > 0) g->indexmax.push_back((int32_t)(n - 1));
}

// ---------------------------------------------------------------------------
// One search pass: kernelNDGridIndexGlobalkNN (kernel.cu:61-113) +
// evaluateCell (kernel.cu:180-225) + evalPoint (kernel.cu:116-161), then the
// per-query sort and K-row extraction of GPU.cu:1629-1634 and
// storeNeighborTableForkNNOnTheFly (GPU.cu:3610-3704).
// Returns true and fills the row when at least K points lie within eps.
// ---------------------------------------------------------------------------
template <typename T>
struct Cand {
  T acc;
  uint32_t id;
  bool operator<(const Cand& o) const { return acc < o.acc || (acc == o.acc && id < o.id); }
};

template <typename T>
inline T sqdist(const T* a, const T* b, uint32_t d) {
  T acc = 0;
  for (uint32_t l = 0; l < d; l++) {
    const T df = a[l] - b[l];
    acc = fma_t(df, df, acc);
  }
  return acc;
}

template <typename T>
bool search_query(const T* X, uint32_t d, const Grid<T>& g, uint32_t q, uint32_t K,
                  std::vector<Cand<T>>& cands, int32_t* out_ids, T* out_d,
                  uint64_t* n_cand_scanned) {
  const uint32_t di = g.di;
  const T* xq = X + (uint64_t)q * d;
  uint32_t lo[64], hi[64], cur[64];
  for (uint32_t j = 0; j < di; j++) {
    const uint32_t c = (uint32_t)((xq[j] - g.minArr[j]) / g.eps);
    lo[j] = (uint32_t)std::max(0, (int)c - 1);
    hi[j] = std::min(g.nCells[j] - 1, c + 1);
    cur[j] = lo[j];
  }
  const T eps = g.eps;
  const T eps2 = eps * eps;
  cands.clear();
  uint64_t scanned = 0;
  while (true) {
    uint64_t lin = 0, mult = 1;
    for (uint32_t j = 0; j < di; j++) {
      lin += (uint64_t)cur[j] * mult;
      mult *= g.nCells[j];
    }
    auto it = std::lower_bound(g.cellKeys.begin(), g.cellKeys.end(), lin);
    if (it != g.cellKeys.end() && *it == lin) {
      const size_t c = (size_t)(it - g.cellKeys.begin());
      for (int32_t kk = g.indexmin[c]; kk <= g.indexmax[c]; kk++) {
        const uint32_t p = g.lookup[kk];
        scanned++;
        const T acc = sqdist(X + (uint64_t)p * d, xq, d);
        if (acc > eps2) continue;
        const T dist = std::sqrt(acc);
        if (dist <= eps) cands.push_back({acc, p});
      }
    }
    // odometer over the 3^di neighbourhood, dimension 0 innermost
    uint32_t j = 0;
    while (j < di) {
      if (cur[j] < hi[j]) {
        cur[j]++;
        break;
      }
      cur[j] = lo[j];
      j++;
    }
    if (j == di) break;
  }
  *n_cand_scanned += scanned;
  if (cands.size() < K) return false;
  std::partial_sort(cands.begin(), cands.begin() + K, cands.end());
  for (uint32_t i = 0; i < K; i++) {
    out_ids[i] = (int32_t)cands[i].id;
    out_d[i] = std::sqrt(cands[i].acc);
  }
  return true;
}

}  // namespace

// Statistics of one oracle join.  Field meanings follow the reference's
// printouts (main.cu:205-210, 440-452).
extern "C" {
typedef struct {
  double avg_distance;      // mean sampled pairwise distance
  double bucket_width;
  double eps0;              // initial epsilon, as DTYPE widened to double
  double eps_final;
  double total_distance;    // sum of squared kNN distances, row-major order
  uint64_t pair_count;
  uint64_t candidates;      // points scanned over all iterations
  int32_t bucket;
  int32_t iterations;       // reference loop iterations (main.cu:312-430)
  int32_t reindexes;        // epsilon growths
  uint32_t eps_offset;
  uint32_t eps_sample_blocks;
  uint32_t perm[64];        // dimension order after ReorderByDimension
  double seconds_prep;      // reorder + epsilon + first grid
  double seconds_regrid;    // grid rebuilds on epsilon growth
  double seconds_search;    // search passes
} orc_stats;
}

namespace {

int clamp_threads(int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  return nthreads;
}

// The reference pipeline of main() / KNNJoinPy (main.cu:109-510, 514-907):
// reorder, estimate epsilon, grid, then the retry loop of main.cu:312-430.
// Returns 0, or 1 (bad argument), 3 (k+1 > N), 6 (iteration cap), 10 (eps 0).
template <typename T>
int join_impl(const T* data, uint64_t n, uint32_t d, uint32_t k, int32_t di, double beta,
              int32_t reorder, const uint32_t* queries, uint64_t nq, int32_t max_iterations,
              int32_t* out_ids, T* out_dists, orc_stats* s, int nthreads) {
  if (!data || !out_ids || !out_dists || n == 0 || d == 0 || d > 64) return 1;
  if ((uint64_t)k + 1 > n) return 3;
  if (di <= 0) di = (int32_t)std::min<uint32_t>(d, 6);
  if ((uint32_t)di > d) return 1;
  nthreads = clamp_threads(nthreads);
  std::memset(s, 0, sizeof(*s));
  const double t_start = omp_get_wtime();
  std::vector<uint32_t> perm(d);
  for (uint32_t j = 0; j < d; j++) perm[j] = j;
  if (reorder) reorder_permutation<T>(data, n, d, perm.data(), (T*)nullptr);
  for (uint32_t j = 0; j < d; j++) s->perm[j] = perm[j];
  std::vector<T> X = apply_permutation<T>(data, n, d, perm.data());
  EpsResult er = estimate_epsilon<T>(X.data(), n, d, k, beta, nullptr, nthreads);
  const T eps0 = (T)er.eps_double;
  s->avg_distance = er.avg;
  s->bucket_width = er.bucket_width;
  s->bucket = er.bucket;
  s->pair_count = er.pair_count;
  s->eps_offset = er.offset;
  s->eps_sample_blocks = er.n_sample_blocks;
  if (!(eps0 > 0) || !std::isfinite((double)eps0)) return 10;
  s->eps0 = (double)eps0;
  const uint32_t K = k + 1;
  std::vector<uint32_t> active;
  if (queries) {
    active.assign(queries, queries + nq);
  } else {
    active.resize(n);
    for (uint64_t i = 0; i < n; i++) active[i] = (uint32_t)i;
  }
  T eps = eps0;
  Grid<T> g;
  grid_dimensions<T>(X.data(), n, d, (uint32_t)di, eps, &g);
  build_grid<T>(X.data(), n, d, &g, nthreads);
  s->seconds_prep = omp_get_wtime() - t_start;
  double failPrev = 0.0;
  int iter = 0;
  uint64_t scanned_total = 0;
  while (!active.empty()) {
    if (max_iterations > 0 && iter >= max_iterations) return 6;
    bool repeat_same = false;
    if (iter != 0 && failPrev > 0.25) {
      const double t0 = omp_get_wtime();
      eps = (T)((double)eps + (double)eps0 * 0.5);  // main.cu:336
      if (eps == 0) return 10;                       // main.cu:338-342
      grid_dimensions<T>(X.data(), n, d, (uint32_t)di, eps, &g);
      build_grid<T>(X.data(), n, d, &g, nthreads);
      s->reindexes++;
      s->seconds_regrid += omp_get_wtime() - t0;
    } else if (iter != 0) {
      // main.cu:330: at most 25% failed, so the failed queries run again at
      // the same epsilon.  That pass is deterministic and fails them all, so
      // it is counted without being recomputed.
      repeat_same = true;
    }
    const uint64_t nactive = active.size();
    std::vector<uint8_t> ok(nactive, 0);
    if (!repeat_same) {
      const double t0 = omp_get_wtime();
      uint64_t sc = 0;
#pragma omp parallel num_threads(nthreads) reduction(+ : sc)
      {
        std::vector<Cand<T>> cands;
#pragma omp for schedule(dynamic, 64)
        for (int64_t a = 0; a < (int64_t)nactive; a++) {
          const uint32_t q = active[a];
          ok[a] = search_query<T>(X.data(), d, g, q, K, cands, out_ids + (uint64_t)q * K,
                                  out_dists + (uint64_t)q * K, &sc);
        }
      }
      scanned_total += sc;
      s->seconds_search += omp_get_wtime() - t0;
    }
    std::vector<uint32_t> failed;
    for (uint64_t a = 0; a < nactive; a++)
      if (!ok[a]) failed.push_back(active[a]);
    failPrev = (failed.size() * 1.0) / (nactive * 1.0);  // main.cu:402
    active.swap(failed);
    iter++;
  }
  s->iterations = iter;
  s->eps_final = (double)eps;
  s->candidates = scanned_total;
  // verification sum of squared distances (GPU.cu:3690-3693), row-major
  double tot = 0.0;
  const uint64_t nrows = queries ? nq : n;
  for (uint64_t a = 0; a < nrows; a++) {
    const uint64_t q = queries ? queries[a] : a;
    for (uint32_t i = 0; i < K; i++) {
      const T dv = out_dists[q * K + i];
      const T sq = dv * dv;
      tot += sq;
    }
  }
  s->total_distance = tot;
  return 0;
}

template <typename T>
int grid_impl(const T* data, uint64_t n, uint32_t d, uint32_t di, T eps, T* minArr,
              uint32_t* nCells, uint64_t* totalCells, uint64_t* cellKeys, int32_t* indexmin,
              int32_t* indexmax, uint32_t* lookup, uint64_t* n_nonempty, int nthreads) {
  if (!data || n == 0 || di == 0 || di > d || di > 64) return 1;
  Grid<T> g;
  grid_dimensions<T>(data, n, d, di, eps, &g);
  build_grid<T>(data, n, d, &g, clamp_threads(nthreads));
  for (uint32_t j = 0; j < di; j++) {
    minArr[j] = g.minArr[j];
    nCells[j] = g.nCells[j];
  }
  *totalCells = g.totalCells;
  *n_nonempty = g.cellKeys.size();
  std::copy(g.cellKeys.begin(), g.cellKeys.end(), cellKeys);
  std::copy(g.indexmin.begin(), g.indexmin.end(), indexmin);
  std::copy(g.indexmax.begin(), g.indexmax.end(), indexmax);
  std::copy(g.lookup.begin(), g.lookup.end(), lookup);
  return 0;
}

template <typename T>
int eps_impl(const T* data, uint64_t n, uint32_t d, uint32_t k, double beta, double* out6,
             uint32_t* hist10000, int nthreads) {
  if (!data || !out6 || n == 0 || d == 0) return 1;
  std::vector<uint32_t> h;
  EpsResult r = estimate_epsilon<T>(data, n, d, k, beta, &h, clamp_threads(nthreads));
  out6[0] = r.avg;
  out6[1] = r.bucket_width;
  out6[2] = (double)(T)r.eps_double;
  out6[3] = (double)r.bucket;
  out6[4] = (double)r.pair_count;
  out6[5] = (double)r.offset;
  if (hist10000) std::memcpy(hist10000, h.data(), sizeof(uint32_t) * 10000);
  return 0;
}

// Brute-force definition: for each listed query, the first K points in
// ascending (acc, id) order over ALL points, with the same arithmetic.
template <typename T>
int bruteforce_impl(const T* data, uint64_t n, uint32_t d, uint32_t K, const uint32_t* queries,
                    uint64_t nq, int32_t* out_ids, T* out_dists, int nthreads) {
  if (!data || !queries || K == 0 || K > n) return 1;
  nthreads = clamp_threads(nthreads);
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<Cand<T>> c(n);
#pragma omp for schedule(dynamic, 4)
    for (int64_t a = 0; a < (int64_t)nq; a++) {
      const uint32_t q = queries[a];
      for (uint64_t p = 0; p < n; p++)
        c[p] = {sqdist(data + p * d, data + (uint64_t)q * d, d), (uint32_t)p};
      std::partial_sort(c.begin(), c.begin() + K, c.end());
      for (uint32_t i = 0; i < K; i++) {
        out_ids[a * K + i] = (int32_t)c[i].id;
        out_dists[a * K + i] = std::sqrt(c[i].acc);
      }
    }
  }
  return 0;
}

// Brute-force range query with the reference's within-epsilon rule
// (evalPoint, kernel.cu:116-161: acc <= fl(eps*eps) on the way, then
// sqrt(acc) <= eps): for each listed query, every point within eps in
// ascending (acc, id) order, at most maxper of them (counts are exact).
template <typename T>
int range_impl(const T* data, uint64_t n, uint32_t d, T eps, const uint32_t* queries, uint64_t nq,
               uint32_t maxper, uint32_t* counts, int32_t* out_ids, T* out_dists, int nthreads) {
  if (!data || !queries || !counts) return 1;
  nthreads = clamp_threads(nthreads);
  const T eps2 = eps * eps;
  int bad = 0;
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<Cand<T>> c;
#pragma omp for schedule(dynamic, 4) reduction(| : bad)
    for (int64_t a = 0; a < (int64_t)nq; a++) {
      const uint32_t q = queries[a];
      c.clear();
      for (uint64_t p = 0; p < n; p++) {
        const T acc = sqdist(data + p * d, data + (uint64_t)q * d, d);
        if (acc <= eps2 && std::sqrt(acc) <= eps) c.push_back({acc, (uint32_t)p});
      }
      std::sort(c.begin(), c.end());
      counts[a] = (uint32_t)c.size();
      if (c.size() > maxper) {
        bad = 1;
        continue;
      }
      for (size_t i = 0; i < c.size(); i++) {
        out_ids[a * maxper + i] = (int32_t)c[i].id;
        out_dists[a * maxper + i] = std::sqrt(c[i].acc);
      }
    }
  }
  return bad ? 2 : 0;
}

}  // namespace

extern "C" {

#define ORC_DEFINE(SUFFIX, T)                                                                \
  int orc_reorder_##SUFFIX(const T* data, uint64_t n, uint32_t d, uint32_t* perm,            \
                           T* variances) {                                                   \
    if (!data || !perm || n == 0 || d == 0) return 1;                                        \
    reorder_permutation<T>(data, n, d, perm, variances);                                     \
    return 0;                                                                                \
  }                                                                                          \
  int orc_eps_##SUFFIX(const T* data, uint64_t n, uint32_t d, uint32_t k, double beta,       \
                       double* out6, uint32_t* hist10000, int nthreads) {                    \
    return eps_impl<T>(data, n, d, k, beta, out6, hist10000, nthreads);                      \
  }                                                                                          \
  int orc_grid_##SUFFIX(const T* data, uint64_t n, uint32_t d, uint32_t di, T eps,           \
                        T* minArr, uint32_t* nCells, uint64_t* totalCells,                   \
                        uint64_t* cellKeys, int32_t* indexmin, int32_t* indexmax,            \
                        uint32_t* lookup, uint64_t* n_nonempty, int nthreads) {              \
    return grid_impl<T>(data, n, d, di, eps, minArr, nCells, totalCells, cellKeys,           \
                        indexmin, indexmax, lookup, n_nonempty, nthreads);                   \
  }                                                                                          \
  int orc_join_##SUFFIX(const T* data, uint64_t n, uint32_t d, uint32_t k, int32_t di,       \
                        double beta, int32_t reorder, const uint32_t* queries, uint64_t nq,  \
                        int32_t max_iterations, int32_t* out_ids, T* out_dists,              \
                        orc_stats* st, int nthreads) {                                       \
    orc_stats local;                                                                         \
    return join_impl<T>(data, n, d, k, di, beta, reorder, queries, nq, max_iterations,       \
                        out_ids, out_dists, st ? st : &local, nthreads);                     \
  }                                                                                          \
  int orc_range_##SUFFIX(const T* data, uint64_t n, uint32_t d, T eps, const uint32_t* queries, \
                         uint64_t nq, uint32_t maxper, uint32_t* counts, int32_t* out_ids,          \
                         T* out_dists, int nthreads) {                                              \
    return range_impl<T>(data, n, d, eps, queries, nq, maxper, counts, out_ids, out_dists,        \
                         nthreads);                                                                 \
  }                                                                                                 \
  int orc_bruteforce_##SUFFIX(const T* data, uint64_t n, uint32_t d, uint32_t K,             \
                              const uint32_t* queries, uint64_t nq, int32_t* out_ids,        \
                              T* out_dists, int nthreads) {                                  \
    return bruteforce_impl<T>(data, n, d, K, queries, nq, out_ids, out_dists, nthreads);     \
  }

ORC_DEFINE(f32, float)
ORC_DEFINE(f64, double)

int orc_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
