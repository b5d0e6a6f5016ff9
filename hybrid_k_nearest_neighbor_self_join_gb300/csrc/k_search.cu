// k_search.cu -- epsilon-range search over the cell ring with the k+1
// nearest neighbours selected inside the kernel.
//
// Replaces kernelNDGridIndexGlobalkNN (kernel.cu:61-113) with evaluateCell
// (kernel.cu:180-225) and evalPoint (kernel.cu:116-161), the pair buffer, the
// two thrust::stable_sort_by_key calls (GPU.cu:1629-1634), the device->host
// copy of all pairs (GPU.cu:1671-1676) and the host K-row extraction
// storeNeighborTableForkNNOnTheFly (GPU.cu:3610-3704).
//
// One warp owns one query at a time (dynamic work fetching in chunks):
//   1. In dense-table mode the warp first counts the points of every cell in
//      the ring (two table reads per row); fewer than K = k+1 means the
//      query cannot be accepted at this radius and it fails without a scan.
//   2. The query's own cell is scanned first.
//   3. The other rows of the ring (a row = consecutive linear cell ids along
//      dimension 0, one contiguous run of the cell-ordered point array) are
//      sorted by a lower bound of their distance to the query and scanned in
//      waves of a few rows.  Once K points are held, a row whose lower bound
//      exceeds the current K-th distance is skipped, and every row is cut to
//      the dimension-0 interval that can still hold a better point.
//   Each lane computes one squared distance with the reference's fma chain
//   (kernel.cu:139-140); points under the current threshold go to the warp's
//   shared-memory buffer with one ballot.  When the buffer fills, a 32-bin
//   histogram of the buffered distances finds a new threshold that keeps at
//   least K keys (an exact sort when the histogram cannot split them).
// A query is accepted when at least K points lie within its radius (the
// reference's acceptance, GPU.cu:3659-3669); its row is then sorted by
// (distance, id) and written.  Otherwise its original id goes to the failure
// list for the next, larger radius.
//
// Exactness: the ring covers every cell that can hold a point within the
// radius, including rounding (cell ranges are widened and rounded outward and
// mapped through the grid's own monotone cell formula), and every skipped row
// or cut provably holds no point that could enter the K best, with slack for
// the rounding of the computed distance.  An accepted query's K rows are its
// exact K nearest by (computed distance, id) -- the oracle's definition.

#include <cmath>

#include "knnsj_internal.h"

namespace knnsj {

namespace {

constexpr int SEARCH_THREADS = 256;  // largest block; the launch may use fewer warps
constexpr int QCHUNK = 4;            // default queries per work fetch
// per-query radii: queries per work fetch up to three indexed dimensions
// (2 measured best on 2-D and 3-D joins) and beyond (1: uneven work per query)
#ifndef KNNSJ_QCHUNK_PER_QUERY_RADIUS_LO
#define KNNSJ_QCHUNK_PER_QUERY_RADIUS_LO 2
#endif
#ifndef KNNSJ_QCHUNK_PER_QUERY_RADIUS
#define KNNSJ_QCHUNK_PER_QUERY_RADIUS 1
#endif
// ring rows per wave (each row is one run of points): for one or two indexed
// dimensions, and for more (wider rings of shorter rows)
#ifndef KNNSJ_WAVE_ROWS_LO
#define KNNSJ_WAVE_ROWS_LO 16
#endif
#ifndef KNNSJ_WAVE_ROWS_HI
#define KNNSJ_WAVE_ROWS_HI 32
#endif
#ifndef KNNSJ_EARLY_FAIL
#define KNNSJ_EARLY_FAIL 1
#endif
#ifndef KNNSJ_SORT_ROWS
#define KNNSJ_SORT_ROWS 1
#endif
// intermediate threshold tightening once K keys are held: 0 only when the
// buffer fills, 1 after every wave, 2 after every wave for a uniform radius
// only (a per-query starting radius is already close to the K-th distance)
// reduce before the output sort when more than 2K keys are held (the counting
// sort handles up to 256 keys by itself)
#ifndef KNNSJ_PRE_WRITE_REDUCE
#define KNNSJ_PRE_WRITE_REDUCE 0
#endif
// per-query radii of failed queries grow toward K points from the count
// they found (1) or by eps0/2 per pass like the plain schedule (0)
#ifndef KNNSJ_GUIDED_GROWTH
#define KNNSJ_GUIDED_GROWTH 1
#endif
#ifndef KNNSJ_TIGHTEN
#define KNNSJ_TIGHTEN 2
#endif
constexpr int MAX_WAVE_ROWS = KNNSJ_WAVE_ROWS_LO > KNNSJ_WAVE_ROWS_HI ? KNNSJ_WAVE_ROWS_LO : KNNSJ_WAVE_ROWS_HI;
constexpr int MAX_RUNS = MAX_WAVE_ROWS;  // one run of points per row
static_assert(MAX_WAVE_ROWS <= 32, "a wave is at most one row per lane");
template <int DI>
constexpr int wave_rows() {
  return (DI > 0 && DI <= 2) ? KNNSJ_WAVE_ROWS_LO : KNNSJ_WAVE_ROWS_HI;
}
constexpr uint32_t HIST_MAX_B = 256;  // histogram reduce for buffers up to this size
constexpr int WARP_WORDS = 256 + 2 * MAX_RUNS + 8;  // per-warp u32 scratch: bins, runS, runP
constexpr int FILTER_QUEUE = 64;  // double data: candidates that passed the float prefilter
template <typename T>
constexpr int warp_words() {
  return WARP_WORDS + (sizeof(T) == 8 ? FILTER_QUEUE : 0);
}

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
  uint32_t qchunk;
  const uint32_t* __restrict__ qlist;
  uint32_t nq;
  const uint32_t* nq_dev;  // non-null: the query count is read here
  const LoopCtl* ctl;
  T radius;
  T* qradius;
  double step;
  int32_t* out_ids;
  T* out_d;
  double* rowsum;  // per-row verification sums (nullptr: none)
  uint32_t* fail_list;
  uint32_t* fail_count;
  unsigned long long* cand_count;
  uint32_t* work_counter;
  FailRadii* fail_radii;
  const float* __restrict__ psf;  // double data: float copy of ps for the prefilter (nullptr: off)
  float filt_e1;                  // bound of the distance change from rounding coordinates to float
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

// Points of cells [Llo, Lhi] (consecutive linear ids): one contiguous run.
template <typename T>
__device__ __forceinline__ void run_of(const SearchParams<T>& p, unsigned long long Llo, unsigned long long Lhi,
                                       uint32_t& s, uint32_t& e) {
  if (Llo > Lhi) {
    s = e = 0;
    return;
  }
  if (p.dense) {
    s = p.dstart[Llo];
    e = p.dstart[Lhi + 1];
  } else {
    s = p.coff[lower_bound_u64(p.ckeys, p.C, Llo)];
    e = p.coff[lower_bound_u64(p.ckeys, p.C, Lhi + 1)];
  }
}

__device__ __forceinline__ unsigned long long shfl_key(unsigned long long v, int src) {
  return __shfl_sync(FULL, v, src);
}
__device__ __forceinline__ KeyF64 shfl_key(KeyF64 v, int src) {
  KeyF64 r;
  r.a = __shfl_sync(FULL, v.a, src);
  r.id = __shfl_sync(FULL, v.id, src);
  r.pad = 0;
  return r;
}
__device__ __forceinline__ unsigned long long key_min() { return 0ull; }
__device__ __forceinline__ KeyF64 key_min_f64() {
  KeyF64 k;
  k.a = 0;
  k.id = 0;
  k.pad = 0;
  return k;
}

__device__ __forceinline__ float to_float_up(float x) { return x; }
__device__ __forceinline__ float to_float_up(double x) { return __double2float_ru(x); }

template <typename T>
struct Sel {
  using K = Key<T>;
  using KT = typename K::type;
  uint32_t len;
  KT tau;     // pass iff key < tau
  bool tight; // tau came from a reduce (an upper bound of the K-th best)
};

template <typename T>
__device__ __forceinline__ void sort_reduce(typename Key<T>::type* buf, Sel<T>& st, uint32_t K, uint32_t B,
                                            int lane) {
  __syncwarp();
  for (uint32_t i = st.len + lane; i < B; i += 32) buf[i] = Key<T>::maxv();
  __syncwarp();
  warp_bitonic_sort<T>(buf, (int)B, lane);
  st.len = K;
  st.tau = buf[K - 1];
  st.tight = true;
  __syncwarp();
}

// Row-index divisors of small ring extents: 0xffffffff / e + 1 (0 for e <= 1),
// read from the constant cache instead of divided per query.
constexpr uint32_t MAGIC_TAB = 64;
struct MagicTable {
  uint32_t v[MAGIC_TAB + 1];
};
constexpr MagicTable make_magic_table() {
  MagicTable t{};
  for (uint32_t e = 0; e <= MAGIC_TAB; e++) t.v[e] = e > 1 ? 0xffffffffu / e + 1u : 0u;
  return t;
}
__constant__ MagicTable c_magic = make_magic_table();

// Monotone bin of a squared distance, round(a * scale) clamped to top, on
// the FMA pipe (a float-to-int conversion runs on a narrower pipe): with
// 1.5 * 2^23 added, the integer lands in the low mantissa bits.  Both users
// only need a monotone map that sends the largest kept key to a bin <= top.
__device__ __forceinline__ int acc_bin(float a, float scale, int top) {
  return min(__float_as_int(__fmaf_rn(a, scale, 12582912.0f)) - 0x4b400000, top);
}
// scale that maps [0, tacc] onto [0, nb] (0 when tacc is 0 or huge)
__device__ __forceinline__ float bin_scale(float nb, float tacc) {
  return (tacc > 0.0f && tacc < 3.0e38f) ? __fdividef(nb, tacc) : 0.0f;
}

// Keeps the keys of the lowest histogram bins that hold at least K keys
// (bins split [0, acc(tau)] evenly); the new threshold is the largest kept
// key.  Needs st.len >= K and B <= HIST_MAX_B.
template <typename T>
__device__ void hist_reduce(typename Key<T>::type* buf, uint32_t* hist, Sel<T>& st, uint32_t K, uint32_t B,
                            int lane) {
  using Kt = Key<T>;
  using KT = typename Kt::type;
  // bins by a monotone float map of the distance: equal distances share a bin
  const float tacc = to_float_up(Kt::acc(st.tau));
  const float scale = bin_scale(32.0f, tacc);
  __syncwarp();
  hist[lane] = 0;
  __syncwarp();
  for (uint32_t i = lane; i < st.len; i += 32) {
    const int b = acc_bin((float)Kt::acc(buf[i]), scale, 31);
    atomicAdd(&hist[b], 1u);
  }
  __syncwarp();
  uint32_t cum = hist[lane];
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL, cum, off);
    if (lane >= off) cum += t;
  }
  const int bst = __ffs(__ballot_sync(FULL, cum >= K)) - 1;
  const uint32_t kept = __shfl_sync(FULL, cum, bst);
  if (kept + 32 > B) {  // one bin holds too much: exact reduce
    sort_reduce<T>(buf, st, K, B, lane);
    return;
  }
  // in-place compaction: a round writes only below the end of what has been
  // read, so reading the round before writing it is enough
  uint32_t nl = 0;
  KT mx;
  if constexpr (sizeof(KT) == 8)
    mx = key_min();
  else
    mx = key_min_f64();
  for (uint32_t base = 0; base < st.len; base += 32) {
    const uint32_t i = base + lane;
    KT v = Kt::maxv();
    if (i < st.len) v = buf[i];
    const bool keep = i < st.len && acc_bin((float)Kt::acc(v), scale, 31) <= bst;
    const unsigned m = __ballot_sync(FULL, keep);
    __syncwarp();
    if (keep) {
      buf[nl + __popc(m & lanemask_lt())] = v;
      if (Kt::less(mx, v)) mx = v;
    }
    nl += __popc(m);
    __syncwarp();
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const KT o = shfl_key(mx, lane ^ off);
    if (Kt::less(mx, o)) mx = o;
  }
  st.len = nl;
  st.tau = mx;
  st.tight = true;
  __syncwarp();
}

// Rare paths are kept out of line so the hot loop stays small in the
// instruction cache.
#ifndef KNNSJ_REDUCE_CALLED
#define KNNSJ_REDUCE_CALLED 1
#endif
#if KNNSJ_REDUCE_CALLED
#define KNNSJ_REDUCE_LINKAGE __noinline__
#else
#define KNNSJ_REDUCE_LINKAGE __forceinline__
#endif
template <typename T>
__device__ KNNSJ_REDUCE_LINKAGE Sel<T> reduce(typename Key<T>::type* buf, uint32_t* hist, Sel<T> st, uint32_t K, uint32_t B,
                                      int lane) {
  if (B <= HIST_MAX_B)
    hist_reduce<T>(buf, hist, st, K, B, lane);
  else
    sort_reduce<T>(buf, st, K, B, lane);
  return st;
}

// the output sort is inlined (0: measured faster) or a called function (1)
#ifndef KNNSJ_WRITE_CALLED
#define KNNSJ_WRITE_CALLED 0
#endif
#if KNNSJ_WRITE_CALLED
#define KNNSJ_WRITE_LINKAGE __noinline__
#else
#define KNNSJ_WRITE_LINKAGE __forceinline__
#endif

// Writes the K smallest of buf[0..len) in ascending (distance, id) order by a
// counting sort over 256 bins of a monotone map of the distance (all keys are
// <= acc(top)), ranking keys that share a bin among themselves.  len <= 256.
template <typename T>
__device__ KNNSJ_WRITE_LINKAGE void write_sorted_row(typename Key<T>::type* buf, uint32_t* cnt, uint32_t len,
                                              typename Key<T>::type top, uint32_t K, int32_t* __restrict__ out_ids,
                                              T* __restrict__ out_d, uint64_t row_out, int lane,
                                              double* __restrict__ rowsum) {
  using Kt = Key<T>;
  using KT = typename Kt::type;
  constexpr int R = HIST_MAX_B / 32;
  const float tacc = to_float_up(Kt::acc(top));
  const float scale = bin_scale(256.0f, tacc);
  __syncwarp();
  reinterpret_cast<uint4*>(cnt)[lane] = make_uint4(0u, 0u, 0u, 0u);
  reinterpret_cast<uint4*>(cnt)[lane + 32] = make_uint4(0u, 0u, 0u, 0u);
  __syncwarp();
  KT v[R];
  uint32_t slot[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const uint32_t i = r * 32 + lane;
    v[r] = Kt::maxv();
    slot[r] = 0;
    if (r * 32 < (int)len && i < len) {
      v[r] = buf[i];
      const int b = acc_bin((float)Kt::acc(v[r]), scale, 255);
      slot[r] = atomicAdd(&cnt[b], 1u);
    }
  }
  __syncwarp();
  // exclusive scan of the 256 bin counts, 8 consecutive bins per lane
  uint32_t c[8], s = 0;
  {
    const uint4 c0 = reinterpret_cast<const uint4*>(cnt)[lane * 2];
    const uint4 c1 = reinterpret_cast<const uint4*>(cnt)[lane * 2 + 1];
    c[0] = c0.x, c[1] = c0.y, c[2] = c0.z, c[3] = c0.w;
    c[4] = c1.x, c[5] = c1.y, c[6] = c1.z, c[7] = c1.w;
  }
#pragma unroll
  for (int t = 0; t < 8; t++) s += c[t];
  uint32_t incl = s;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL, incl, off);
    if (lane >= off) incl += t;
  }
  uint32_t run = incl - s;
  __syncwarp();
  {
    uint32_t o[8];
#pragma unroll
    for (int t = 0; t < 8; t++) {
      o[t] = run;
      run += c[t];
    }
    reinterpret_cast<uint4*>(cnt)[lane * 2] = make_uint4(o[0], o[1], o[2], o[3]);
    reinterpret_cast<uint4*>(cnt)[lane * 2 + 1] = make_uint4(o[4], o[5], o[6], o[7]);
  }
  __syncwarp();
  // scatter by bin (order inside a bin still arbitrary)
  uint32_t pos[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const uint32_t i = r * 32 + lane;
    pos[r] = 0xffffffffu;
    if (r * 32 < (int)len && i < len) {
      const int b = acc_bin((float)Kt::acc(v[r]), scale, 255);
      pos[r] = cnt[b] + slot[r];
      buf[pos[r]] = v[r];
    }
  }
  __syncwarp();
  // buf is now in bin order, and the K smallest keys lie in the bins that
  // start below K: only positions below the end of the bin holding position
  // K-1 are ranked inside their bin and written
  uint32_t end = 0;
  {
    uint32_t st = incl - s;  // start of this lane's first bin
    uint32_t e = 0;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const uint32_t nx = st + c[t];
      if (st < K && K <= nx) e = nx;  // bin t holds position K-1
      st = nx;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) e = max(e, __shfl_xor_sync(FULL, e, off));
    end = e ? e : len;
  }
  T rsq = 0;
  for (uint32_t p0 = 0; p0 < end; p0 += 32) {
    const uint32_t pp = p0 + lane;
    if (pp < end) {
      const KT w = buf[pp];
      const int b = acc_bin((float)Kt::acc(w), scale, 255);
      const uint32_t first = cnt[b];
      const uint32_t last = b < 255 ? cnt[b + 1] : len;
      uint32_t rank = 0;
      if (last - first > 1)  // a key alone in its bin is ranked by the bin
        for (uint32_t j = first; j < last; j++) rank += Kt::less(buf[j], w) ? 1u : 0u;
      const uint32_t fin = first + rank;
      if (fin < K) {
        const T dist = Num<T>::sqrt(Kt::acc(w));
        out_ids[row_out + fin] = (int32_t)Kt::id(w);
        out_d[row_out + fin] = dist;
        rsq = Num<T>::add(rsq, Num<T>::mul(dist, dist));
      }
    }
  }
  if (rowsum) store_row_sum<T>(rowsum, row_out / K, rsq, lane);
  __syncwarp();
}

// Writes the K smallest of buf[0..len) by a full bitonic sort (any len <= B).
template <typename T>
__device__ __noinline__ void write_sorted_row_bitonic(typename Key<T>::type* buf, uint32_t len, uint32_t K,
                                                      int32_t* __restrict__ out_ids, T* __restrict__ out_d,
                                                      uint64_t row_out, int lane, double* __restrict__ rowsum) {
  using Kt = Key<T>;
  const uint32_t n2 = len <= 1 ? 1u : (1u << (32 - __clz(len - 1)));
  __syncwarp();
  for (uint32_t i = len + lane; i < n2; i += 32) buf[i] = Kt::maxv();
  __syncwarp();
  warp_bitonic_sort<T>(buf, (int)n2, lane);
  T rsq = 0;
  for (uint32_t i = lane; i < K; i += 32) {
    const typename Kt::type kk = buf[i];
    const T dist = Num<T>::sqrt(Kt::acc(kk));
    out_ids[row_out + i] = (int32_t)Kt::id(kk);
    out_d[row_out + i] = dist;
    rsq = Num<T>::add(rsq, Num<T>::mul(dist, dist));
  }
  if (rowsum) store_row_sum<T>(rowsum, row_out / K, rsq, lane);
  __syncwarp();
}

// Bitonic sort of one 64-bit value per lane across the warp (ascending).
__device__ __forceinline__ unsigned long long warp_sort32(unsigned long long v, int lane) {
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const unsigned long long o = __shfl_xor_sync(FULL, v, j);
      const bool up = (lane & k) == 0;
      const bool low = (lane & j) == 0;
      const unsigned long long mn = v < o ? v : o;
      const unsigned long long mx = v < o ? o : v;
      v = (low == up) ? mn : mx;
    }
  }
  return v;
}

// resident blocks per SM the register budget is cut for: float data in low
// dimensions (d <= 3, all indexed) fits 64 registers, the rest needs more
#ifndef KNNSJ_MINB_LO
#define KNNSJ_MINB_LO 4
#endif
#ifndef KNNSJ_MINB_HI
#define KNNSJ_MINB_HI 3
#endif
template <typename T, int D, int DI>
constexpr int search_min_blocks() {
  return (sizeof(T) == 4 && D > 0 && D <= 3 && DI > 0) ? KNNSJ_MINB_LO : KNNSJ_MINB_HI;
}

// D: data dimensions (0 = runtime); DI: indexed dimensions (0 = runtime, <= MAX_DI).
template <typename T, int D, int DI>
__global__ void __launch_bounds__(SEARCH_THREADS, search_min_blocks<T, D, DI>()) search_kernel(const SearchParams<T> p) {
  constexpr int WAVE_ROWS = wave_rows<DI>();
  constexpr int NDI = DI > 0 ? DI : MAX_DI;
  using Kt = Key<T>;
  using KT = typename Kt::type;
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  KT* buf = reinterpret_cast<KT*>(smem) + (size_t)wib * p.B;
  uint32_t* words = reinterpret_cast<uint32_t*>(reinterpret_cast<KT*>(smem) + (size_t)wpb * p.B) + wib * warp_words<T>();
  uint32_t* hist = words;                   // [256]: reduce bins / output counting sort
  uint32_t* runS = words + 256;             // [MAX_RUNS]
  uint32_t* runP = words + 256 + MAX_RUNS;  // [MAX_RUNS + 1]
  T* qsm = reinterpret_cast<T*>(reinterpret_cast<uint32_t*>(reinterpret_cast<KT*>(smem) + (size_t)wpb * p.B) +
                                wpb * warp_words<T>()) +
           (size_t)wib * MAX_D;
  const uint64_t n = p.n;
  const uint32_t di = DI > 0 ? (uint32_t)DI : p.g.di;
  const uint32_t K = p.K;
  const uint32_t B = p.B;
  unsigned long long scanned = 0;
  // the pass's queries, failure list and radius: from the launch, or from
  // the loop state when the pass runs inside the retry graph (kept in shared
  // memory, not in registers, which the scan loop needs)
  __shared__ uint32_t s_nq;
  __shared__ const uint32_t* s_qlist;
  __shared__ uint32_t* s_fail;
  __shared__ T s_radius;
  // the grid's origin and inverse cell width in float, for ring bounds
  __shared__ float s_minf[NDI];
  __shared__ float s_invw;
  if (threadIdx.x < (unsigned)NDI) s_minf[threadIdx.x] = threadIdx.x < p.g.di ? (float)p.g.minv[threadIdx.x] : 0.0f;
  if (threadIdx.x == 0) {
    s_invw = 1.0f / (float)p.g.width;
    if (p.ctl) {
      s_nq = p.ctl->nq;
      s_qlist = p.ctl->list[p.ctl->cur];
      s_fail = p.ctl->list[p.ctl->cur ^ 1];
      s_radius = (T)p.ctl->r;
    } else {
      s_nq = p.nq_dev ? *p.nq_dev : p.nq;
      s_qlist = p.qlist;
      s_fail = p.fail_list;
      s_radius = p.radius;
    }
  }
  __syncthreads();

  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(p.work_counter, p.qchunk);
    base = __shfl_sync(FULL, base, 0);
    if (base >= s_nq) break;
    const uint32_t qend = min(base + p.qchunk, s_nq);
    for (uint32_t qi = base; qi < qend; ++qi) {
      // first pass: every point in cell order; later passes: the failed
      // queries by original id (valid across grid rebuilds)
      const uint32_t* qlist = s_qlist;
      const uint32_t qid = qlist ? qlist[qi] : p.pid[qi];
      const T* qsrc = qlist ? p.xs : p.ps;
      const uint32_t qcol = qlist ? qid : qi;
      T q[D > 0 ? D : 1];
      if (D > 0) {
#pragma unroll
        for (int l = 0; l < (D > 0 ? D : 1); l++) q[l] = qsrc[(uint64_t)l * n + qcol];
      } else {
        for (uint32_t l = lane; l < p.d; l += 32) qsm[l] = qsrc[(uint64_t)l * n + qcol];
        __syncwarp();
      }
      auto qdim = [&](int j) -> T { return (D > 0) ? q[j < D ? j : 0] : qsm[j]; };
      const T r = p.qradius ? p.qradius[qid] : s_radius;
      const T thr = within_threshold(r);

      // All bound arithmetic below is float, widened by explicit slack so
      // that float rounding (and, for double data, the rounding of the
      // coordinates to float) only ever enlarges what is searched.
      // Cell ring: a point whose computed squared distance is <= thr differs
      // from the query by at most r * (1 + 2^-16) per coordinate.
      const float rf = to_float_up(r) * (1.0f + 1.0f / 8192.0f);
      uint32_t lo[NDI], hi[NDI], magic[NDI];
      float qf[NDI];
#pragma unroll
      for (int j = 0; j < NDI; j++) {
        lo[j] = hi[j] = magic[j] = 0;
        qf[j] = 0.0f;
        if (j < (int)di) {
          const T qj = qdim(j);
          qf[j] = (float)qj;
          const float slack = (fabsf(qf[j]) + rf) * (1.0f / 2097152.0f);
          lo[j] = ring_cell(qf[j] - rf - slack, s_minf[j], s_invw, p.g.ncell[j], false);
          hi[j] = ring_cell(qf[j] + rf + slack, s_minf[j], s_invw, p.g.ncell[j], true);
          const uint32_t ext = hi[j] - lo[j] + 1;
          // x / ext == umulhi(x, magic) for small x; rows are indexed by dims 1..
          if (j > 0) magic[j] = ext <= MAGIC_TAB ? c_magic.v[ext] : 0xffffffffu / ext + 1u;
        }
      }
      unsigned long long nrows = 1;
#pragma unroll
      for (int j = 1; j < NDI; j++)
        if (j < (int)di) nrows *= (unsigned long long)(hi[j] - lo[j] + 1);
      const float wf = (float)p.g.width;

      // Row ridx of the ring: linear id of its dimension-0 origin and a lower
      // bound of the computed squared distance of any of its points
      // (dimensions 1..di-1, less 2^-14 for the rounding of the distance).
      auto row_info = [&](uint32_t ridx, unsigned long long& rbase) -> float {
        uint32_t rem = ridx;
        unsigned long long lin = 0;
        float lbf = 0.0f;
#pragma unroll
        for (int j = 1; j < NDI; j++) {
          if (j < (int)di) {
            const uint32_t ext = hi[j] - lo[j] + 1;
            uint32_t qq = ext > 1 ? __umulhi(rem, magic[j]) : rem;
            int rj = (int)(rem - qq * ext);
            if (rj < 0) {
              qq--;
              rj += (int)ext;
            } else if (rj >= (int)ext) {
              qq++;
              rj -= (int)ext;
            }
            rem = qq;
            const uint32_t c = lo[j] + (uint32_t)rj;
            lin += (unsigned long long)c * p.g.mult[j];
            const float mv = (float)p.g.minv[j];
            const float slo = mv + (float)c * wf;
            const float shi = slo + wf;
            const float m = (fabsf(mv) + ((float)c + 1.0f) * wf + fabsf(qf[j])) * (1.0f / 524288.0f);
            const float gap = fmaxf(0.0f, fmaxf(slo - m - qf[j], qf[j] - shi - m));
            lbf += gap * gap;
          }
        }
        rbase = lin;
        return lbf * (1.0f - 1.0f / 16384.0f);
      };

      // The dimension-0 cells [xl, xh] of a row with lower bound lbs that can
      // hold a point whose computed squared distance is <= tupv (float,
      // rounded up); false when none can.
      auto cut_row = [&](float lbs, float tupv, uint32_t& xl, uint32_t& xh) -> bool {
        if (lbs > tupv) return false;
        const float avail = tupv * (1.0f + 1.0f / 16384.0f) - lbs;
        const float g = sqrtf(fmaxf(avail, 0.0f)) * (1.0f + 1.0f / 1048576.0f);
        const float slack = (fabsf(qf[0]) + g) * (1.0f / 2097152.0f);
        xl = max(xl, ring_cell(qf[0] - g - slack, s_minf[0], s_invw, p.g.ncell[0], false));
        xh = min(xh, ring_cell(qf[0] + g + slack, s_minf[0], s_invw, p.g.ncell[0], true));
        return xl <= xh;
      };

      Sel<T> st;
      st.len = 0;
      st.tau = Kt::bound(thr);
      st.tight = false;
      // a uniform radius tightens the threshold after each wave (the first
      // wave being the query's own row alone), so rows are visited nearest
      // first; per-query radii are already close to the K-th distance
      const bool tighten = KNNSJ_TIGHTEN == 1 || (KNNSJ_TIGHTEN == 2 && p.qradius == nullptr);
      // rows are sorted when a later wave can be pruned: with a per-query
      // radius a ring of one wave is scanned in its natural order
      const bool sorted_rows = KNNSJ_SORT_ROWS && (tighten ? nrows > 1 : nrows > (unsigned long long)WAVE_ROWS);

      bool fail_now = false;
      uint32_t ring_cnt = 0;  // points in the ring's cells, when counted
      if (KNNSJ_EARLY_FAIL && p.dense && nrows > 32) {
        // fewer than K points in the whole ring: this radius cannot succeed
        // (rings of one group are counted from the runs loaded below)
        uint32_t cnt = 0;
        for (unsigned long long g0 = 0; g0 < nrows; g0 += 32) {
          const unsigned long long ridx = g0 + lane;
          if (ridx < nrows) {
            unsigned long long rb;
            row_info((uint32_t)ridx, rb);
            cnt += p.dstart[rb + hi[0] + 1] - p.dstart[rb + lo[0]];
          }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(FULL, cnt, off);
        fail_now = cnt < K;
        ring_cnt = cnt;
      }

      // Producer of run lists: the rows of the ring in groups of 32, each
      // lane loading its row's full dimension-0 run (one memory round trip
      // per group), sorted by lower bound when that can prune, consumed a
      // wave of rows at a time; a row is cut to a narrower run only once K
      // keys are held.  One scan loop consumes the runs.
      unsigned long long g0 = 0;  // first row of the current group
      int nvalid = 0, w0 = 0;     // rows in the group, next wave start
      unsigned long long skey = 0, rbase = 0;
      uint32_t rs = 0, re = 0;    // this lane's row of the group: its full run
      bool first_wave = true;
      const unsigned long long groups_end = fail_now ? 0 : nrows;
      for (;;) {
        uint32_t total = 0;
        int nr = 1;
        if (w0 >= nvalid) {  // next group of rows
          if (nvalid > 0) g0 += 32;
          if (g0 >= groups_end) break;
          const unsigned long long ridx = g0 + lane;
          float rlb = __int_as_float(0x7f800000);
          rbase = 0;
          rs = re = 0;
          if (ridx < nrows) {
            rlb = row_info((uint32_t)ridx, rbase);
            // three or more indexed dimensions: only the row's dimension-0
            // interval that can hold a point under the current threshold (the
            // radius, until K keys are held) -- the corners of a cube of
            // cells hold most of its points; with two, rows are cut only once
            // K keys are held (measured: the cut costs more than it saves)
            uint32_t xl = lo[0], xh = hi[0];
            const bool cut = DI >= 3 || (DI == 0 && di >= 3);
            if (!cut || cut_row(rlb, to_float_up(Kt::acc(st.tau)), xl, xh)) run_of(p, rbase + xl, rbase + xh, rs, re);
          }
          if (KNNSJ_EARLY_FAIL && nrows <= 32) {
            uint32_t cnt = re - rs;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(FULL, cnt, off);
            if (cnt < K) {  // the whole ring holds fewer than K points
              ring_cnt = cnt;
              fail_now = true;
              break;
            }
          }
          skey = ((unsigned long long)__float_as_uint(rlb) << 32) | (unsigned long long)(uint32_t)lane;
          if (sorted_rows) skey = warp_sort32(skey, lane);
          nvalid = (int)min(32ull, nrows - g0);
          w0 = 0;
        }
        const int wave = (tighten && first_wave) ? 1 : WAVE_ROWS;
        first_wave = false;
        const unsigned long long myk = __shfl_sync(FULL, skey, (w0 + lane) & 31);
        const int srcl = (int)(myk & 31u);
        const unsigned long long lb = __shfl_sync(FULL, rbase, srcl);
        const uint32_t s0 = __shfl_sync(FULL, rs, srcl);
        const uint32_t e0 = __shfl_sync(FULL, re, srcl);
        const float lbs = __uint_as_float((uint32_t)(myk >> 32));
        const bool active = lane < wave && w0 + lane < nvalid;
        const float tup = to_float_up(Kt::acc(st.tau));
        const bool have = st.len >= K;
        // rows come in ascending lower bound: the rest of the group can go
        const float first_lb = __shfl_sync(FULL, lbs, 0);
        if (sorted_rows && have && first_lb > tup) {
          w0 = nvalid;
          continue;
        }
        uint32_t sA = 0, eA = 0;
        if (active) {
          uint32_t xl = lo[0], xh = hi[0];
          // (the group's run already holds the row cut to the threshold of
          // its loading; with K keys held the row is cut again)
          const bool empty = have && !cut_row(lbs, tup, xl, xh);
          if (!empty) {
            if (xl == lo[0] && xh == hi[0]) {
              sA = s0;
              eA = e0;
            } else {
              run_of(p, lb + xl, lb + xh, sA, eA);
            }
          }
        }
        const uint32_t la = eA - sA;
        uint32_t incl = la;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const uint32_t t = __shfl_up_sync(FULL, incl, off);
          if (lane >= off) incl += t;
        }
        total = __shfl_sync(FULL, incl, WAVE_ROWS - 1);
        if (lane < WAVE_ROWS) {
          runS[lane] = sA;
          runP[lane] = incl - la;
        }
        nr = WAVE_ROWS;
        w0 += wave;
        __syncwarp();
        int row = 0;
        if constexpr (sizeof(T) == 8) {
          if (p.psf) {
            // double data: float squared distances first; only candidates
            // under the float bound (queued in shared memory) get the exact
            // double distance, 32 at a time
            uint32_t* queue = words + WARP_WORDS;
            auto filt_thr = [&]() -> float {
              const double t = (double)Kt::acc(st.tau);
              const double sq = sqrt(t * (1.0 + 1.0 / 1099511627776.0)) + (double)p.filt_e1;
              return __double2float_ru((1.0 + (double)(p.d + 4) * 1.1920928955078125e-07) * sq * sq);
            };
            float tf = filt_thr();
            uint32_t qn = 0;
            auto exact_batch = [&](uint32_t cnt_q, uint32_t base_q) {
              bool pass = false;
              KT key = Kt::maxv();
              if (lane < cnt_q) {
                const uint32_t j = queue[base_q + lane];
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
                if (acc <= Kt::acc(st.tau)) {
                  key = Kt::make(acc, p.pid[j]);
                  pass = Kt::less(key, st.tau);
                }
              }
              const unsigned m = __ballot_sync(FULL, pass);
              if (m) {
                if (pass) buf[st.len + __popc(m & lanemask_lt())] = key;
                st.len += __popc(m);
                if (st.len > B - 32) {
                  st = reduce<T>(buf, hist, st, K, B, lane);
                  tf = filt_thr();
                }
              }
            };
            for (uint32_t v0 = 0; v0 < total; v0 += 32) {
              const uint32_t v = v0 + lane;
              bool surv = false;
              uint32_t j = 0;
              if (v < total) {
                while (row < nr - 1 && runP[row + 1] <= v) row++;
                j = runS[row] + (v - runP[row]);
                float af = 0.0f;
                if (D > 0) {
#pragma unroll
                  for (int l = 0; l < (D > 0 ? D : 1); l++) {
                    const float t = __fsub_rn(p.psf[(uint64_t)l * n + j], (float)q[l]);
                    af = __fmaf_rn(t, t, af);
                  }
                } else {
                  for (uint32_t l = 0; l < p.d; l++) {
                    const float t = __fsub_rn(p.psf[(uint64_t)l * n + j], (float)qsm[l]);
                    af = __fmaf_rn(t, t, af);
                  }
                }
                surv = af <= tf;
              }
              const unsigned m = __ballot_sync(FULL, surv);
              if (surv) queue[qn + __popc(m & lanemask_lt())] = j;
              qn += __popc(m);
              __syncwarp();
              if (qn >= 32) {
                exact_batch(32, qn - 32);
                qn -= 32;
                __syncwarp();
              }
            }
            if (qn) exact_batch(qn, 0);
            scanned += total;
            __syncwarp();
            if (tighten && !st.tight && st.len >= K) st = reduce<T>(buf, hist, st, K, B, lane);
            continue;
          }
        }
        // the scan: one squared distance per lane, ballot-append under tau
        for (uint32_t v0 = 0; v0 < total; v0 += 32) {
          const uint32_t v = v0 + lane;
          bool pass = false;
          KT key = Kt::maxv();
          if (v < total) {
            while (row < nr - 1 && runP[row + 1] <= v) row++;
            const uint32_t j = runS[row] + (v - runP[row]);
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
            if (acc <= Kt::acc(st.tau)) {
              key = Kt::make(acc, p.pid[j]);
              pass = Kt::less(key, st.tau);
            }
          }
          const unsigned m = __ballot_sync(FULL, pass);
          if (m) {
            if (pass) buf[st.len + __popc(m & lanemask_lt())] = key;
            st.len += __popc(m);
            if (st.len > B - 32) st = reduce<T>(buf, hist, st, K, B, lane);
          }
        }
        scanned += total;
        __syncwarp();
        if (tighten && !st.tight && st.len >= K) st = reduce<T>(buf, hist, st, K, B, lane);
      }

      __syncwarp();
      if (st.len >= K) {
        const uint64_t row_out = (uint64_t)qid * K;
        if (B <= HIST_MAX_B) {
#if KNNSJ_PRE_WRITE_REDUCE
          if (st.len > 2 * K && st.len > 64) st = reduce<T>(buf, hist, st, K, B, lane);
#endif
          write_sorted_row<T>(buf, hist, st.len, st.tau, K, p.out_ids, p.out_d, row_out, lane, p.rowsum);
        } else {
          write_sorted_row_bitonic<T>(buf, st.len, K, p.out_ids, p.out_d, row_out, lane, p.rowsum);
        }
      } else if (lane == 0) {
        const uint32_t slot = atomicAdd(p.fail_count, 1u);
        s_fail[slot] = qid;
        if (p.qradius) {
          // Per-query radii grow by at least eps0/2 (the plain schedule's
          // step).  With guided growth the points found -- within the radius
          // after a scan, or in the whole ring when it failed its count --
          // give the local density, and the radius is scaled toward K points:
          // (K / found)^(1/indexed dims), at most 4x per pass.  Any radius is
          // exact; this only saves passes.
          double rn = (double)r + p.step;
          if (KNNSJ_GUIDED_GROWTH) {
            const uint32_t found = fail_now ? ring_cnt : st.len;
            const float f = exp2f(log2f((float)K / (float)max(found, 1u)) / (float)di) * 1.05f;
            rn = fmax(rn, (double)r * (double)fminf(fmaxf(f, 1.0f), 4.0f));
          }
          const T rt = (T)rn;
          p.qradius[qid] = rt;
          atomicMax(&p.fail_radii->rmax_bits, (unsigned long long)Num<T>::bits(rt));
          const float oct = log2f((float)rt / (2.0f * (float)p.step));  // log2(r / eps0)
          const int bin = min(max((int)floorf(4.0f * oct) + 16, 0), FAIL_RADIUS_BINS - 1);
          atomicAdd(&p.fail_radii->hist[bin], 1u);
        }
      }
      __syncwarp();
    }
  }
  if (lane == 0 && scanned) atomicAdd(p.cand_count, scanned);
}

template <typename T, int D, int DI>
void launch_one(const SearchParams<T>& prm, int wpb_req, int sm_count, cudaStream_t s) {
  // per-warp shared memory: selection buffer, u32 scratch, query copy (generic d)
  const size_t per_warp = (size_t)prm.B * sizeof(typename Key<T>::type) + warp_words<T>() * 4 +
                          (D == 0 ? (size_t)MAX_D * sizeof(T) : 0);
  int wpb = SEARCH_THREADS / 32;
  if (wpb_req > 0 && wpb_req < wpb) wpb = wpb_req;
  while (wpb > 1 && per_warp * wpb > 200 * 1024) wpb--;
  const size_t smem = per_warp * wpb;
  auto kern = search_kernel<T, D, DI>;
  KNNSJ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  KNNSJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, wpb * 32, smem));
  if (per_sm < 1) throw StatusError{KNNSJ_ERR_UNSUPPORTED, "search kernel does not fit"};
  const uint64_t warps_needed = (prm.nq + prm.qchunk - 1) / prm.qchunk;
  uint64_t blocks = (uint64_t)per_sm * sm_count;
  const uint64_t need_blocks = (warps_needed + wpb - 1) / wpb;
  // inside the retry graph the pass size is known only on the device: the
  // full persistent grid, whose surplus warps find no work and leave
  if (!prm.ctl && !prm.nq_dev && need_blocks < blocks) blocks = need_blocks;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, wpb * 32, smem, s>>>(prm);
  KNNSJ_CHECK_LAUNCH();
}

// Sparse-query tail: the exact K nearest points of each listed query by a
// scan over every point (one CTA per query; its warps take equal shares of
// the cell-ordered columns with the search kernel's selection, then warp 0
// merges their selections and writes the row).  The distances use the search
// kernel's arithmetic, so rows equal those of a ring search.
constexpr int BRUTE_THREADS = 1024;

template <typename T>
__global__ void __launch_bounds__(BRUTE_THREADS) brute_kernel(const SearchParams<T> p) {
  using Kt = Key<T>;
  using KT = typename Kt::type;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t s_len[BRUTE_THREADS / 32];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const uint32_t B = p.B, K = p.K;
  const uint64_t n = p.n;
  KT* bufs = reinterpret_cast<KT*>(smem);
  KT* buf = bufs + (size_t)wib * B;
  uint32_t* hist = reinterpret_cast<uint32_t*>(bufs + (size_t)wpb * B) + wib * 256;
  T* qs = reinterpret_cast<T*>(reinterpret_cast<uint32_t*>(bufs + (size_t)wpb * B) + wpb * 256);
  const uint32_t qid = p.qlist[blockIdx.x];
  for (uint32_t l = threadIdx.x; l < p.d; l += blockDim.x) qs[l] = p.xs[(uint64_t)l * n + qid];
  __syncthreads();
  Sel<T> st;
  st.len = 0;
  st.tau = Kt::bound((T)INFINITY);
  st.tight = false;
  const uint64_t share = (n + wpb - 1) / wpb;
  const uint64_t j0 = (uint64_t)wib * share;
  const uint64_t j1 = min(n, j0 + share);
  for (uint64_t v0 = j0; v0 < j1; v0 += 32) {
    const uint64_t j = v0 + lane;
    bool pass = false;
    KT key = Kt::maxv();
    if (j < j1) {
      T acc = 0;
      for (uint32_t l = 0; l < p.d; l++) {
        const T t = Num<T>::sub(p.ps[(uint64_t)l * n + j], qs[l]);
        acc = Num<T>::fma(t, t, acc);
      }
      key = Kt::make(acc, p.pid[j]);
      pass = Kt::less(key, st.tau);
    }
    const unsigned m = __ballot_sync(FULL, pass);
    if (m) {
      if (pass) buf[st.len + __popc(m & lanemask_lt())] = key;
      st.len += __popc(m);
      if (st.len > B - 32) st = reduce<T>(buf, hist, st, K, B, lane);
    }
  }
  if (lane == 0) s_len[wib] = st.len;
  __syncthreads();
  if (wib != 0) return;
  for (int w = 1; w < wpb; w++) {
    const KT* ob = bufs + (size_t)w * B;
    const uint32_t lw = s_len[w];
    for (uint32_t b0 = 0; b0 < lw; b0 += 32) {
      bool pass = false;
      KT key = Kt::maxv();
      if (b0 + lane < lw) {
        key = ob[b0 + lane];
        pass = Kt::less(key, st.tau);
      }
      const unsigned m = __ballot_sync(FULL, pass);
      if (m) {
        if (pass) buf[st.len + __popc(m & lanemask_lt())] = key;
        st.len += __popc(m);
        if (st.len > B - 32) st = reduce<T>(buf, hist, st, K, B, lane);
      }
    }
  }
  write_sorted_row_bitonic<T>(buf, st.len, K, p.out_ids, p.out_d, (uint64_t)qid * K, lane, p.rowsum);
}

}  // namespace

template <typename T>
void launch_brute(const SearchLaunch<T>& a, cudaStream_t s) {
  if (a.nq == 0) return;
  SearchParams<T> p{};
  p.ps = a.grid.ps;
  p.xs = a.xs;
  p.pid = a.grid.pid;
  p.n = a.n;
  p.d = a.d;
  p.K = a.K;
  p.B = (uint32_t)search_buffer_capacity(a.K);
  p.qlist = a.qlist;
  p.nq = a.nq;
  p.out_ids = a.out_ids;
  p.out_d = a.out_d;
  p.rowsum = a.rowsum;
  const size_t per_warp = (size_t)p.B * sizeof(typename Key<T>::type) + 256 * 4;
  int wpb = BRUTE_THREADS / 32;
  while (wpb > 1 && per_warp * wpb + a.d * sizeof(T) > 200 * 1024) wpb--;
  const size_t smem = per_warp * wpb + a.d * sizeof(T);
  KNNSJ_CUDA(cudaFuncSetAttribute(brute_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  brute_kernel<T><<<a.nq, wpb * 32, smem, s>>>(p);
  KNNSJ_CHECK_LAUNCH();
}

// Selection buffer per warp: room for K keys plus a full chunk of 32, and at
// least HIST_MAX_B so the histogram reduce runs rarely.
int search_buffer_capacity(uint32_t K) {
  uint32_t b = HIST_MAX_B;
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
  if (a.shape.buffer > 0 && (uint32_t)a.shape.buffer > p.B && (a.shape.buffer & (a.shape.buffer - 1)) == 0 &&
      a.shape.buffer <= 4096)
    p.B = (uint32_t)a.shape.buffer;
  // per-query radii make the work per query uneven: finer work fetching
  p.qchunk = a.shape.qchunk > 0 ? (uint32_t)a.shape.qchunk
                                : (uint32_t)(!a.qradius               ? QCHUNK
                                             : a.grid.geom.di <= 3 ? KNNSJ_QCHUNK_PER_QUERY_RADIUS_LO
                                                                   : KNNSJ_QCHUNK_PER_QUERY_RADIUS);
  const int wpb = a.shape.warps_per_block;
  p.qlist = a.qlist;
  p.nq = a.nq;
  p.nq_dev = a.nq_dev;
  p.ctl = a.ctl;
  p.radius = a.radius;
  p.qradius = a.qradius;
  p.step = (double)a.step;
  p.out_ids = a.out_ids;
  p.out_d = a.out_d;
  p.rowsum = a.rowsum;
  p.fail_list = a.fail_list;
  p.fail_count = a.fail_count;
  p.cand_count = a.cand_count;
  p.work_counter = a.work_counter;
  p.fail_radii = a.fail_radii;
  // Float prefilter for double data: a candidate is skipped when its float
  // squared distance exceeds a bound that every candidate within the radius
  // respects.  Rounding coordinates of magnitude <= M to float moves a
  // distance by at most sqrt(d) * M * 2^-23 (plus subnormal slack).  Off
  // when the coordinates could overflow a float square.
  p.psf = nullptr;
  p.filt_e1 = 0.0f;
  if (sizeof(T) == 8 && a.grid.psf && std::isfinite(a.coord_bound) &&
      2.0 * std::sqrt((double)a.d) * a.coord_bound < 1e18) {
    p.psf = a.grid.psf;
    const double e1 = std::sqrt((double)a.d) * (a.coord_bound * std::ldexp(1.0, -23) + std::ldexp(1.0, -140));
    p.filt_e1 = (float)(e1 * (1.0 + 1e-6));
  }
  launch_zero_words(a.work_counter, sizeof(uint32_t), s);
  const bool full = a.grid.geom.di == a.d;  // every dimension indexed
  switch (a.d) {
    case 2: full ? launch_one<T, 2, 2>(p, wpb, sm_count, s) : launch_one<T, 2, 0>(p, wpb, sm_count, s); break;
    case 3: full ? launch_one<T, 3, 3>(p, wpb, sm_count, s) : launch_one<T, 3, 0>(p, wpb, sm_count, s); break;
    case 4: full ? launch_one<T, 4, 4>(p, wpb, sm_count, s) : launch_one<T, 4, 0>(p, wpb, sm_count, s); break;
    case 5: full ? launch_one<T, 5, 5>(p, wpb, sm_count, s) : launch_one<T, 5, 0>(p, wpb, sm_count, s); break;
    case 6: full ? launch_one<T, 6, 6>(p, wpb, sm_count, s) : launch_one<T, 6, 0>(p, wpb, sm_count, s); break;
    case 7: full ? launch_one<T, 7, 7>(p, wpb, sm_count, s) : launch_one<T, 7, 0>(p, wpb, sm_count, s); break;
    case 8: full ? launch_one<T, 8, 8>(p, wpb, sm_count, s) : launch_one<T, 8, 0>(p, wpb, sm_count, s); break;
    default: launch_one<T, 0, 0>(p, wpb, sm_count, s); break;
  }
}

template void launch_search<float>(const SearchLaunch<float>&, int, cudaStream_t);
template void launch_search<double>(const SearchLaunch<double>&, int, cudaStream_t);
template void launch_brute<float>(const SearchLaunch<float>&, cudaStream_t);
template void launch_brute<double>(const SearchLaunch<double>&, cudaStream_t);

}  // namespace knnsj
