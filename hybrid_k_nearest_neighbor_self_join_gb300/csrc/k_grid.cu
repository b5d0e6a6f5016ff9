// k_grid.cu -- grid index build on the device.
//
// Replaces populateNDGridIndexAndLookupArrayGPU (GPU.cu:3715-4067):
//   cell ids (kernelIndexComputeNonemptyCells, kernel.cu:1673-1697, with the
//   row-major linear id of kernel.cu:31-47), point ids (kernelInitEnumerateDB,
//   kernel.cu:1699-1713), thrust::sort / unique / sort_by_key and the host scan
//   into grid{indexmin,indexmax}.
// Here: one coalesced pass computes (cell id, point id) pairs, a hand-written
// stable LSD radix sort orders them by cell id (points of a cell stay in
// ascending id, as with the reference's stable radix sort_by_key), a scan
// compacts the non-empty cells into a sorted key table with start offsets
// (gridCellLookup + grid), and the coordinates are gathered into cell order so
// every cell -- and every run of consecutive cells -- is one contiguous slice.
// When the grid is small enough a dense start table replaces the binary
// search over non-empty cells.

#include "knnsj_internal.h"

namespace knnsj {

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 8;                       // rounds of 32 keys per warp
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;    // keys per block tile
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__global__ void cell_id_kernel(const T* __restrict__ soa, uint64_t n, const GridGeom<T> g,
                               unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    unsigned long long lin = 0;
    for (uint32_t j = 0; j < g.di; j++) {
      const uint32_t c = point_cell_coord(soa[(uint64_t)j * n + i], g.minv[j], g.width);
      lin += (unsigned long long)c * g.mult[j];
    }
    keys[i] = lin;
    vals[i] = (uint32_t)i;
  }
}

__global__ void radix_hist_kernel(const unsigned long long* __restrict__ keys, uint64_t n, int shift,
                                  uint32_t ntiles, uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    const uint64_t idx = base + (uint64_t)r * RS_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 0xff], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter: warp w owns keys [tile + w*256, tile + w*256 + 256) and
// visits them in order, 32 at a time; equal digits within a round are ranked
// by lane, rounds by order, warps by index, tiles by the scanned histogram.
__global__ void radix_scatter_kernel(const unsigned long long* __restrict__ kin,
                                     const uint32_t* __restrict__ vin, unsigned long long* __restrict__ kout,
                                     uint32_t* __restrict__ vout, uint64_t n, int shift, uint32_t ntiles,
                                     const uint32_t* __restrict__ offs) {
  __shared__ uint32_t wc[RS_WARPS][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&wc[0][0])[i] = 0;
  __syncthreads();
  const uint64_t wbase = (uint64_t)blockIdx.x * RS_TILE + (uint64_t)w * (RS_ITEMS * 32);
  unsigned long long k[RS_ITEMS];
  uint32_t v[RS_ITEMS];
  uint32_t dg[RS_ITEMS];
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    const uint64_t idx = wbase + (uint64_t)r * 32 + lane;
    if (idx < n) {
      k[r] = kin[idx];
      v[r] = vin[idx];
      dg[r] = (uint32_t)((k[r] >> shift) & 0xff);
    } else {
      k[r] = 0;
      v[r] = 0;
      dg[r] = 256;
    }
    const unsigned peers = __match_any_sync(FULL, dg[r]);
    const int leader = __ffs(peers) - 1;
    if (lane == leader && dg[r] < 256) wc[w][dg[r]] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    const int digit = threadIdx.x;  // RS_THREADS == 256
    uint32_t run = offs[(uint64_t)digit * ntiles + blockIdx.x];
    for (int ww = 0; ww < RS_WARPS; ww++) {
      const uint32_t c = wc[ww][digit];
      wc[ww][digit] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    const unsigned peers = __match_any_sync(FULL, dg[r]);
    const int leader = __ffs(peers) - 1;
    if (dg[r] < 256) {
      const uint32_t dst = wc[w][dg[r]] + __popc(peers & lanemask_lt());
      kout[dst] = k[r];
      vout[dst] = v[r];
    }
    __syncwarp();
    if (lane == leader && dg[r] < 256) wc[w][dg[r]] += __popc(peers);
    __syncwarp();
  }
}

// ---- exclusive scan of uint32 (three kernels) ----------------------------
__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, size_t n, uint32_t* __restrict__ sums) {
  __shared__ uint32_t ws[32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE;
  uint32_t s = 0;
#pragma unroll
  for (int r = 0; r < SCAN_ITEMS; r++) {
    const size_t i = base + (size_t)r * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(FULL, s, off);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = ws[threadIdx.x];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(FULL, s, off);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
  }
}

// Block-wide exclusive scan of SCAN_TILE items held SCAN_ITEMS per thread in
// blocked order; returns the tile total.
__device__ uint32_t block_scan_tile(uint32_t (&x)[SCAN_ITEMS], uint32_t* ws) {
  uint32_t tsum = 0;
#pragma unroll
  for (int r = 0; r < SCAN_ITEMS; r++) {
    const uint32_t t = x[r];
    x[r] = tsum;
    tsum += t;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t incl = tsum;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL, incl, off);
    if (lane >= off) incl += t;
  }
  if (lane == 31) ws[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t v = ws[lane];
    uint32_t vi = v;
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t t = __shfl_up_sync(FULL, vi, off);
      if (lane >= off) vi += t;
    }
    ws[lane] = vi - v;
    if (lane == 31) ws[32] = vi;
  }
  __syncthreads();
  const uint32_t excl = incl - tsum + ws[w];
#pragma unroll
  for (int r = 0; r < SCAN_ITEMS; r++) x[r] += excl;
  const uint32_t total = ws[32];
  __syncthreads();
  return total;
}

// Single block: in-place exclusive scan of the block sums.
__global__ void scan_sums_kernel(uint32_t* __restrict__ sums, size_t nb) {
  __shared__ uint32_t ws[33];
  uint32_t carry = 0;
  for (size_t base = 0; base < nb; base += SCAN_TILE) {
    uint32_t x[SCAN_ITEMS];
#pragma unroll
    for (int r = 0; r < SCAN_ITEMS; r++) {
      const size_t i = base + (size_t)threadIdx.x * SCAN_ITEMS + r;
      x[r] = i < nb ? sums[i] : 0;
    }
    const uint32_t total = block_scan_tile(x, ws);
#pragma unroll
    for (int r = 0; r < SCAN_ITEMS; r++) {
      const size_t i = base + (size_t)threadIdx.x * SCAN_ITEMS + r;
      if (i < nb) sums[i] = x[r] + carry;
    }
    carry += total;
    __syncthreads();
  }
}

__global__ void scan_apply_kernel(const uint32_t* __restrict__ in, size_t n, const uint32_t* __restrict__ sums,
                                  uint32_t* __restrict__ out) {
  __shared__ uint32_t ws[33];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE;
  uint32_t x[SCAN_ITEMS];
#pragma unroll
  for (int r = 0; r < SCAN_ITEMS; r++) {
    const size_t i = base + (size_t)threadIdx.x * SCAN_ITEMS + r;
    x[r] = i < n ? in[i] : 0;
  }
  block_scan_tile(x, ws);
  const uint32_t add = sums[blockIdx.x];
#pragma unroll
  for (int r = 0; r < SCAN_ITEMS; r++) {
    const size_t i = base + (size_t)threadIdx.x * SCAN_ITEMS + r;
    if (i < n) out[i] = x[r] + add;
  }
}

// ---- non-empty cell table --------------------------------------------------
__global__ void cell_flags_kernel(const unsigned long long* __restrict__ sk, uint64_t n,
                                  uint32_t* __restrict__ flags) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    flags[i] = (i == 0 || sk[i] != sk[i - 1]) ? 1u : 0u;
}

__global__ void cell_compact_kernel(const unsigned long long* __restrict__ sk, uint64_t n,
                                    const uint32_t* __restrict__ pos, unsigned long long* __restrict__ ckeys,
                                    uint32_t* __restrict__ coff) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (i == 0 || sk[i] != sk[i - 1]) {
      ckeys[pos[i]] = sk[i];
      coff[pos[i]] = (uint32_t)i;
    }
  }
}

__global__ void cell_count_kernel(const unsigned long long* __restrict__ sk, uint64_t n,
                                  const uint32_t* __restrict__ pos, uint32_t* __restrict__ coff,
                                  unsigned long long* __restrict__ dC) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint32_t last = (n == 1 || sk[n - 1] != sk[n - 2]) ? 1u : 0u;
  const unsigned long long C = (unsigned long long)pos[n - 1] + last;
  coff[C] = (uint32_t)n;
  *dC = C;
}

__global__ void dense_table_kernel(const unsigned long long* __restrict__ ckeys,
                                   const uint32_t* __restrict__ coff, unsigned long long C,
                                   unsigned long long total, uint32_t* __restrict__ dstart) {
  for (unsigned long long L = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; L <= total;
       L += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long lo = 0, hi = C;
    while (lo < hi) {
      const unsigned long long mid = (lo + hi) >> 1;
      if (ckeys[mid] < L)
        lo = mid + 1;
      else
        hi = mid;
    }
    dstart[L] = coff[lo];
  }
}

template <typename T>
__global__ void gather_sorted_kernel(const T* __restrict__ soa, uint64_t n, uint32_t d,
                                     const uint32_t* __restrict__ ids, T* __restrict__ ps, float* __restrict__ psf) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t src = ids[i];
    for (uint32_t j = 0; j < d; j++) {
      const T v = soa[(uint64_t)j * n + src];
      ps[(uint64_t)j * n + i] = v;
      if (psf) psf[(uint64_t)j * n + i] = (float)v;  // round to nearest
    }
  }
}

// Position of a point's cell along a space-filling curve over the di indexed
// dimensions, `bits` bits per dimension (a code of bits * di bits).  Two
// dimensions: the Hilbert curve (the published xy-to-d conversion: per level
// from the top, the quadrant's index (3 rx) ^ ry, then the quadrant is
// rotated or flipped into the curve's frame), whose consecutive cells are
// always adjacent; otherwise the Morton (Z-order) code, bit b of cell
// coordinate j at bit b*di + j.
template <typename T>
__global__ void morton_key_kernel(const T* __restrict__ ps, uint64_t n, const GridGeom<T> g, int bits,
                                  unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    unsigned long long code = 0;
    if (g.di == 2) {
      // (bits <= 21: coordinates and their flips stay in 32 bits; the
      // quadrant indices enter the code two bits per level from the top)
      const uint32_t last = (1u << bits) - 1u;  // cell coordinates are at most this
      uint32_t x = point_cell_coord(ps[i], g.minv[0], g.width) & last;
      uint32_t y = point_cell_coord(ps[n + i], g.minv[1], g.width) & last;
      for (int l = bits - 1; l >= 0; l--) {
        const uint32_t rx = (x >> l) & 1u, ry = (y >> l) & 1u;
        code = (code << 2) | ((3u * rx) ^ ry);
        if (ry == 0) {
          if (rx == 1) {
            x = last - x;
            y = last - y;
          }
          const uint32_t t = x;
          x = y;
          y = t;
        }
      }
    } else {
      for (uint32_t j = 0; j < g.di; j++) {
        const uint32_t c = point_cell_coord(ps[(uint64_t)j * n + i], g.minv[j], g.width);
        for (int b = 0; b < bits; b++) code |= (unsigned long long)((c >> b) & 1u) << (b * g.di + j);
      }
    }
    keys[i] = code;
    vals[i] = (uint32_t)i;
  }
}

// Counting sort of points into the cells of a grid (any order within a
// cell).  The points are visited in the order of src (cell-ordered columns of
// a coarser grid keep neighbours together), and the lanes of a warp that
// fall in one cell take their counts or positions with one atomic:
// tbl[L + 1] counts cell L, ...
template <typename T>
__device__ __forceinline__ unsigned long long cell_of(const T* __restrict__ src, uint64_t n, uint64_t i,
                                                      const GridGeom<T>& g) {
  unsigned long long lin = 0;
  for (uint32_t j = 0; j < g.di; j++)
    lin += (unsigned long long)point_cell_coord(src[(uint64_t)j * n + i], g.minv[j], g.width) * g.mult[j];
  return lin;
}

template <typename T>
__global__ void cell_count_atomic_kernel(const T* __restrict__ src, uint64_t n, const GridGeom<T> g,
                                         uint32_t* __restrict__ tbl) {
  const int lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint64_t i = base + threadIdx.x;
    const bool live = i < n;
    const unsigned long long lin = live ? cell_of(src, n, i, g) : ~0ull;
    const unsigned peers = __match_any_sync(FULL, lin);
    if (live && lane == __ffs(peers) - 1) atomicAdd(&tbl[lin + 1], (uint32_t)__popc(peers));
  }
}

// ... after the exclusive scan tbl[L + 1] is the first position of cell L;
// each point takes the next position of its cell (leaving tbl[L + 1] at the
// cell's end, which is where cell L + 1 starts: tbl becomes the start table).
template <typename T>
__global__ void cell_scatter_atomic_kernel(const T* __restrict__ src, const uint32_t* __restrict__ src_ids, uint64_t n,
                                           uint32_t d, const GridGeom<T> g, uint32_t* __restrict__ tbl,
                                           T* __restrict__ ps, uint32_t* __restrict__ pid) {
  const int lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b0 = (uint64_t)blockIdx.x * blockDim.x; b0 < n; b0 += stride) {
    const uint64_t i = b0 + threadIdx.x;
    const bool live = i < n;
    const unsigned long long lin = live ? cell_of(src, n, i, g) : ~0ull;
    const unsigned peers = __match_any_sync(FULL, lin);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (live && lane == leader) base = atomicAdd(&tbl[lin + 1], (uint32_t)__popc(peers));
    base = __shfl_sync(FULL, base, leader);
    if (live) {
      const uint32_t pos = base + __popc(peers & lanemask_lt());
      for (uint32_t j = 0; j < d; j++) ps[(uint64_t)j * n + pos] = src[(uint64_t)j * n + i];
      pid[pos] = src_ids ? src_ids[i] : (uint32_t)i;
    }
  }
}

unsigned grid_blocks(uint64_t n, int threads = 256) {
  uint64_t b = (n + threads - 1) / threads;
  if (b > 152ull * 64) b = 152ull * 64;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

size_t radix_hist_elems(uint64_t n) { return (size_t)256 * ((n + RS_TILE - 1) / RS_TILE); }

size_t scan_tmp_elems(size_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

void scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp, cudaStream_t s) {
  if (n == 0) return;
  const size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  scan_reduce_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, tmp);
  KNNSJ_CHECK_LAUNCH();
  scan_sums_kernel<<<1, SCAN_THREADS, 0, s>>>(tmp, nb);
  KNNSJ_CHECK_LAUNCH();
  scan_apply_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, tmp, out);
  KNNSJ_CHECK_LAUNCH();
}

template <typename T>
void launch_cell_ids(const T* soa, uint64_t n, const GridGeom<T>& g, unsigned long long* keys,
                     uint32_t* vals, cudaStream_t s) {
  cell_id_kernel<T><<<grid_blocks(n), 256, 0, s>>>(soa, n, g, keys, vals);
  KNNSJ_CHECK_LAUNCH();
}

int radix_sort_pairs(GridScratch& sc, uint64_t n, int bits, cudaStream_t s) {
  int cur = 0;
  const uint32_t ntiles = (uint32_t)((n + RS_TILE - 1) / RS_TILE);
  const size_t nh = (size_t)256 * ntiles;
  for (int shift = 0; shift < bits; shift += 8) {
    radix_hist_kernel<<<ntiles, RS_THREADS, 0, s>>>(sc.keys[cur], n, shift, ntiles, sc.hist);
    KNNSJ_CHECK_LAUNCH();
    scan_exclusive_u32(sc.hist, sc.hist, nh, sc.scan_tmp, s);
    radix_scatter_kernel<<<ntiles, RS_THREADS, 0, s>>>(sc.keys[cur], sc.vals[cur], sc.keys[cur ^ 1],
                                                       sc.vals[cur ^ 1], n, shift, ntiles, sc.hist);
    KNNSJ_CHECK_LAUNCH();
    cur ^= 1;
  }
  return cur;
}

void launch_compact_cells(const unsigned long long* skeys, uint64_t n, uint32_t* flags, uint32_t* pos,
                          uint32_t* scan_tmp, unsigned long long* ckeys, uint32_t* coff,
                          unsigned long long* d_C, cudaStream_t s) {
  cell_flags_kernel<<<grid_blocks(n), 256, 0, s>>>(skeys, n, flags);
  KNNSJ_CHECK_LAUNCH();
  scan_exclusive_u32(flags, pos, n, scan_tmp, s);
  cell_compact_kernel<<<grid_blocks(n), 256, 0, s>>>(skeys, n, pos, ckeys, coff);
  KNNSJ_CHECK_LAUNCH();
  cell_count_kernel<<<1, 32, 0, s>>>(skeys, n, pos, coff, d_C);
  KNNSJ_CHECK_LAUNCH();
}

void launch_dense_table(const unsigned long long* ckeys, const uint32_t* coff, unsigned long long C,
                        unsigned long long total_cells, uint32_t* dstart, cudaStream_t s) {
  dense_table_kernel<<<grid_blocks(total_cells + 1), 256, 0, s>>>(ckeys, coff, C, total_cells, dstart);
  KNNSJ_CHECK_LAUNCH();
}

template <typename T>
void launch_morton_keys(const T* ps, uint64_t n, const GridGeom<T>& g, int bits, unsigned long long* keys,
                        uint32_t* vals, cudaStream_t s) {
  morton_key_kernel<T><<<grid_blocks(n), 256, 0, s>>>(ps, n, g, bits, keys, vals);
  KNNSJ_CHECK_LAUNCH();
}

template <typename T>
void launch_counting_grid(const T* src, const uint32_t* src_ids, uint64_t n, uint32_t d, const GridGeom<T>& g,
                          uint32_t* tbl, uint32_t* scan_tmp, T* ps, uint32_t* pid, cudaStream_t s) {
  launch_zero_words(tbl, (g.total_cells + 1) * 4, s);
  cell_count_atomic_kernel<T><<<grid_blocks(n), 256, 0, s>>>(src, n, g, tbl);
  KNNSJ_CHECK_LAUNCH();
  scan_exclusive_u32(tbl + 1, tbl + 1, g.total_cells, scan_tmp, s);
  cell_scatter_atomic_kernel<T><<<grid_blocks(n), 256, 0, s>>>(src, src_ids, n, d, g, tbl, ps, pid);
  KNNSJ_CHECK_LAUNCH();
}

template <typename T>
void launch_gather_sorted(const T* soa, uint64_t n, uint32_t d, const uint32_t* sorted_ids, T* ps, float* psf,
                          cudaStream_t s) {
  gather_sorted_kernel<T><<<grid_blocks(n), 256, 0, s>>>(soa, n, d, sorted_ids, ps, psf);
  KNNSJ_CHECK_LAUNCH();
}

template void launch_cell_ids<float>(const float*, uint64_t, const GridGeom<float>&, unsigned long long*,
                                     uint32_t*, cudaStream_t);
template void launch_cell_ids<double>(const double*, uint64_t, const GridGeom<double>&, unsigned long long*,
                                      uint32_t*, cudaStream_t);
template void launch_morton_keys<float>(const float*, uint64_t, const GridGeom<float>&, int, unsigned long long*,
                                        uint32_t*, cudaStream_t);
template void launch_morton_keys<double>(const double*, uint64_t, const GridGeom<double>&, int,
                                         unsigned long long*, uint32_t*, cudaStream_t);
template void launch_counting_grid<float>(const float*, const uint32_t*, uint64_t, uint32_t, const GridGeom<float>&,
                                          uint32_t*, uint32_t*, float*, uint32_t*, cudaStream_t);
template void launch_counting_grid<double>(const double*, const uint32_t*, uint64_t, uint32_t, const GridGeom<double>&,
                                           uint32_t*, uint32_t*, double*, uint32_t*, cudaStream_t);
template void launch_gather_sorted<float>(const float*, uint64_t, uint32_t, const uint32_t*, float*, float*,
                                          cudaStream_t);
template void launch_gather_sorted<double>(const double*, uint64_t, uint32_t, const uint32_t*, double*, float*,
                                           cudaStream_t);

}  // namespace knnsj
