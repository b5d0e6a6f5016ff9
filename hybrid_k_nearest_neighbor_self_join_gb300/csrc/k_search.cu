// k_search.cu -- epsilon-range search over the cell ring with the k+1
// nearest neighbours selected inside the kernel.
//
// Replaces kernelNDGridIndexGlobalkNN (kernel.cu:61-113) with evaluateCell
// (kernel.cu:180-225) and evalPoint (kernel.cu:116-161), the pair buffer, the
// two thrust::stable_sort_by_key calls (GPU.cu:1629-1634), the device->host
// copy of all pairs (GPU.cu:1671-1676) and the host K-row extraction
// storeNeighborTableForkNNOnTheFly (GPU.cu:3610-3704).
//
// One warp owns one query at a time (dynamic work fetching in chunks).  The
// warp walks the rows of the query's cell ring -- each row is a run of
// consecutive linear cell ids, hence one contiguous run of the cell-ordered
// point array -- with one lane per row doing the cell lookup (dense table or
// binary search over the non-empty cells, as gridCellLookup does), then
// streams the concatenated runs 32 points at a time.  Each lane computes one
// squared distance with the reference's fma chain; points under the current
// threshold are appended to the warp's shared-memory buffer with one ballot.
// When the buffer fills, a bitonic sort keeps the K best and tightens the
// threshold.  A query is accepted when at least K = k+1 points lie within its
// radius (the reference's acceptance, GPU.cu:3659-3669); otherwise its
// original id is appended to the failure list for the next, larger radius.
//
// Exactness: the ring covers every cell that can hold a point within the
// radius, including rounding (see cell_range below), so an accepted query's
// K rows are its exact K nearest by (distance, id).

#include "knnsj_internal.h"

namespace knnsj {

namespace {

constexpr int SEARCH_THREADS = 256;
constexpr int QCHUNK = 4;

template <typename T>
struct SearchParams {
  GridGeom<T> g;
  const T* __restrict__ ps;
  const T* __restrict__ xs;
  const uint32_t* __restrict__ pid;
  const unsigned long long* __restrict__ ckeys;
  const uint32_t* __restrict__ coff;
  const uint32_t* __restrict__ dstart;
  unsigned long long C;
  int dense;
  uint64_t n;
  uint32_t d;
  uint32_t K;
  uint32_t B;
  const uint32_t* __restrict__ qlist;
  uint32_t nq;
  T radius;
  T* qradius;
  double step;
  int32_t* out_ids;
  T* out_d;
  uint32_t* fail_list;
  uint32_t* fail_count;
  unsigned long long* cand_count;
  uint32_t* work_counter;
};

__device__ __forceinline__ unsigned long long lower_bound_u64(const unsigned long long* __restrict__ a,
                                                              unsigned long long n,
                                                              unsigned long long key) {
  unsigned long long lo = 0, hi = n;
  while (lo < hi) {
    const unsigned long long mid = (lo + hi) >> 1;
    if (a[mid] < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

template <typename T, int D>
__global__ void __launch_bounds__(SEARCH_THREADS) search_kernel(const SearchParams<T> p) {
  using K = Key<T>;
  using KT = typename K::type;
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  KT* buf = reinterpret_cast<KT*>(smem) + (size_t)wib * p.B;
  uint32_t* rowS = reinterpret_cast<uint32_t*>(reinterpret_cast<KT*>(smem) + (size_t)wpb * p.B) + wib * 64;
  uint32_t* rowP = rowS + 32;
  T* qsm = reinterpret_cast<T*>(reinterpret_cast<uint32_t*>(reinterpret_cast<KT*>(smem) + (size_t)wpb * p.B) +
                                wpb * 64) +
           (size_t)wib * MAX_D;
  const uint64_t n = p.n;
  const uint32_t di = p.g.di;
  unsigned long long scanned = 0;

  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(p.work_counter, (uint32_t)QCHUNK);
    base = __shfl_sync(FULL, base, 0);
    if (base >= p.nq) break;
    const uint32_t qend = min(base + (uint32_t)QCHUNK, p.nq);
    for (uint32_t qi = base; qi < qend; ++qi) {
      // first pass: every point in cell order; later passes: the failed
      // queries by original id (valid across grid rebuilds)
      const uint32_t qid = p.qlist ? p.qlist[qi] : p.pid[qi];
      const T* qsrc = p.qlist ? p.xs : p.ps;
      const uint32_t qcol = p.qlist ? qid : qi;
      T q[D > 0 ? D : 1];
      if (D > 0) {
#pragma unroll
        for (int l = 0; l < (D > 0 ? D : 1); l++) q[l] = qsrc[(uint64_t)l * n + qcol];
      } else {
        for (uint32_t l = lane; l < p.d; l += 32) qsm[l] = qsrc[(uint64_t)l * n + qcol];
        __syncwarp();
      }
      const T r = p.qradius ? p.qradius[qid] : p.radius;
      const T thr = within_threshold(r);

      // cell_range: any point whose computed squared distance is <= thr
      // differs from the query by at most r * (1 + 2^-16) (float) in every
      // coordinate; widen by that, round outward, and map both ends through
      // the (monotone) cell formula of the grid build.
      uint32_t lo[MAX_DI], hi[MAX_DI];
      const double rr = __dmul_ru((double)r, Num<T>::ring_margin);
#pragma unroll
      for (int j = 0; j < MAX_DI; j++) {
        if (j < (int)di) {
          const T qj = (D > 0) ? q[j < D ? j : 0] : qsm[j];
          const T lov = Num<T>::down(__dsub_rd((double)qj, rr));
          const T hiv = Num<T>::up(__dadd_ru((double)qj, rr));
          lo[j] = clamped_cell(lov, p.g.minv[j], p.g.width, p.g.ncell[j]);
          hi[j] = clamped_cell(hiv, p.g.minv[j], p.g.width, p.g.ncell[j]);
        } else {
          lo[j] = 0;
          hi[j] = 0;
        }
      }
      unsigned long long nrows = 1;
#pragma unroll
      for (int j = 1; j < MAX_DI; j++)
        if (j < (int)di) nrows *= (unsigned long long)(hi[j] - lo[j] + 1);

      KT tau = K::bound(thr);
      uint32_t len = 0;
      for (unsigned long long g0 = 0; g0 < nrows; g0 += 32) {
        const unsigned long long ridx = g0 + lane;
        uint32_t s = 0, e = 0;
        if (ridx < nrows) {
          unsigned long long rem = ridx, lin = 0;
#pragma unroll
          for (int j = 1; j < MAX_DI; j++) {
            if (j < (int)di) {
              const unsigned long long ext = hi[j] - lo[j] + 1;
              const unsigned long long c = lo[j] + rem % ext;
              rem /= ext;
              lin += c * p.g.mult[j];
            }
          }
          const unsigned long long Llo = lin + lo[0];
          const unsigned long long Lhi = lin + hi[0];
          if (p.dense) {
            s = p.dstart[Llo];
            e = p.dstart[Lhi + 1];
          } else {
            const unsigned long long a = lower_bound_u64(p.ckeys, p.C, Llo);
            const unsigned long long b = lower_bound_u64(p.ckeys, p.C, Lhi + 1);
            s = p.coff[a];
            e = p.coff[b];
          }
        }
        const uint32_t rlen = e - s;
        uint32_t incl = rlen;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const uint32_t t = __shfl_up_sync(FULL, incl, off);
          if (lane >= off) incl += t;
        }
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        rowS[lane] = s;
        rowP[lane] = incl - rlen;
        __syncwarp();
        int row = 0;
        for (uint32_t v0 = 0; v0 < total; v0 += 32) {
          const uint32_t v = v0 + lane;
          bool pass = false;
          KT key = K::maxv();
          if (v < total) {
            while (row < 31 && rowP[row + 1] <= v) row++;
            const uint32_t j = rowS[row] + (v - rowP[row]);
            T acc = 0;
            if (D > 0) {
#pragma unroll
              for (int l = 0; l < (D > 0 ? D : 1); l++) {
                const T t = Num<T>::sub(p.ps[(uint64_t)l * n + j], q[l]);
                acc = Num<T>::fma(t, t, acc);
              }
            } else {
              for (uint32_t l = 0; l < p.d; l++) {
                const T t = Num<T>::sub(p.ps[(uint64_t)l * n + j], qsm[l]);
                acc = Num<T>::fma(t, t, acc);
              }
            }
            key = K::make(acc, p.pid[j]);
            pass = K::less(key, tau);
          }
          const unsigned m = __ballot_sync(FULL, pass);
          if (m) {
            if (pass) buf[len + __popc(m & lanemask_lt())] = key;
            len += __popc(m);
            if (len > p.B - 32) {
              __syncwarp();
              for (uint32_t i = len + lane; i < p.B; i += 32) buf[i] = K::maxv();
              __syncwarp();
              warp_bitonic_sort<T>(buf, (int)p.B, lane);
              len = p.K;
              tau = buf[p.K - 1];
            }
          }
        }
        scanned += total;
        __syncwarp();
      }
      __syncwarp();
      if (len >= p.K) {
        const uint32_t n2 = len <= 1 ? 1u : (1u << (32 - __clz(len - 1)));
        for (uint32_t i = len + lane; i < n2; i += 32) buf[i] = K::maxv();
        __syncwarp();
        warp_bitonic_sort<T>(buf, (int)n2, lane);
        const uint64_t row_base = (uint64_t)qid * p.K;
        for (uint32_t i = lane; i < p.K; i += 32) {
          const KT kk = buf[i];
          p.out_ids[row_base + i] = (int32_t)K::id(kk);
          p.out_d[row_base + i] = Num<T>::sqrt(K::acc(kk));
        }
      } else if (lane == 0) {
        const uint32_t slot = atomicAdd(p.fail_count, 1u);
        p.fail_list[slot] = qid;
        if (p.qradius) p.qradius[qid] = (T)((double)r + p.step);
      }
      __syncwarp();
    }
  }
  if (lane == 0 && scanned) atomicAdd(p.cand_count, scanned);
}

template <typename T, int D>
void launch_one(const SearchParams<T>& prm, int sm_count, cudaStream_t s) {
  // per-warp shared memory: selection buffer, row table, query copy (generic d)
  const size_t per_warp =
      (size_t)prm.B * sizeof(typename Key<T>::type) + 64 * 4 + (D == 0 ? (size_t)MAX_D * sizeof(T) : 0);
  int wpb = SEARCH_THREADS / 32;
  while (wpb > 1 && per_warp * wpb > 200 * 1024) wpb--;
  const size_t smem = per_warp * wpb;
  auto kern = search_kernel<T, D>;
  KNNSJ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  KNNSJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, wpb * 32, smem));
  if (per_sm < 1) throw StatusError{KNNSJ_ERR_UNSUPPORTED, "search kernel does not fit"};
  const uint64_t warps_needed = (prm.nq + QCHUNK - 1) / QCHUNK;
  uint64_t blocks = (uint64_t)per_sm * sm_count;
  const uint64_t need_blocks = (warps_needed + wpb - 1) / wpb;
  if (need_blocks < blocks) blocks = need_blocks;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, wpb * 32, smem, s>>>(prm);
  KNNSJ_CHECK_LAUNCH();
}

}  // namespace

int search_buffer_capacity(uint32_t K) {
  uint32_t b = 64;
  while (b < K + 32) b <<= 1;
  return (int)b;
}

template <typename T>
void launch_search(const SearchLaunch<T>& a, int sm_count, cudaStream_t s) {
  if (a.nq == 0) return;
  SearchParams<T> p;
  p.g = a.grid.geom;
  p.ps = a.grid.ps;
  p.xs = a.xs;
  p.pid = a.grid.pid;
  p.ckeys = a.grid.ckeys;
  p.coff = a.grid.coff;
  p.dstart = a.grid.dstart;
  p.C = a.grid.C;
  p.dense = a.grid.dense;
  p.n = a.n;
  p.d = a.d;
  p.K = a.K;
  p.B = (uint32_t)search_buffer_capacity(a.K);
  p.qlist = a.qlist;
  p.nq = a.nq;
  p.radius = a.radius;
  p.qradius = a.qradius;
  p.step = (double)a.step;
  p.out_ids = a.out_ids;
  p.out_d = a.out_d;
  p.fail_list = a.fail_list;
  p.fail_count = a.fail_count;
  p.cand_count = a.cand_count;
  p.work_counter = a.work_counter;
  KNNSJ_CUDA(cudaMemsetAsync(a.work_counter, 0, sizeof(uint32_t), s));
  switch (a.d) {
    case 2: launch_one<T, 2>(p, sm_count, s); break;
    case 3: launch_one<T, 3>(p, sm_count, s); break;
    case 4: launch_one<T, 4>(p, sm_count, s); break;
    case 5: launch_one<T, 5>(p, sm_count, s); break;
    case 6: launch_one<T, 6>(p, sm_count, s); break;
    case 7: launch_one<T, 7>(p, sm_count, s); break;
    case 8: launch_one<T, 8>(p, sm_count, s); break;
    default: launch_one<T, 0>(p, sm_count, s); break;
  }
}

template void launch_search<float>(const SearchLaunch<float>&, int, cudaStream_t);
template void launch_search<double>(const SearchLaunch<double>&, int, cudaStream_t);

}  // namespace knnsj
