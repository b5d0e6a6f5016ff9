// k_tile.cu -- range search of low-dimensional float data by tiles of
// queries: one warp owns QPT queries (4 by default) that are neighbours in
// Morton order of their cells, 32 / QPT lanes per query, and the tile's
// queries share one pass over the candidates of the union of their rings.
//
// Replaces, for the first search pass of float data with two or three
// dimensions (all indexed) and k+1 <= 65, the same reference steps as
// search_kernel (k_search.cu): kernelNDGridIndexGlobalkNN with evaluateCell
// and evalPoint (kernel.cu:61-225), the pair buffer and the two
// thrust::stable_sort_by_key (GPU.cu:1629-1634), and the K-row extraction of
// storeNeighborTableForkNNOnTheFly (GPU.cu:3610-3704).
//
// Per tile (one warp):
//   1. each query's cell ring, the union box of the tile's rings (a query
//      whose ring is much wider than the tile's mean is handed to
//      search_kernel instead, so one outlier does not widen everyone's
//      scan); each row of the box (consecutive cells along dimension 0) is
//      one contiguous run of the cell-ordered columns;
//   2. the box's candidates are staged in shared memory 64 at a time
//      (coalesced loads: coordinates and id in one 16-byte record, the next
//      chunk in flight while the current one is evaluated); lane (slot q,
//      phase p) evaluates candidates p, p + 32 / QPT, ... for query q;
//   3. the single pass over the candidates: every key (squared distance,
//      id) within the query's radius goes to the query's list in shared
//      memory, its slot from a ballot over the query's lanes (no atomics);
//      a query that finds more keys than the list holds (0.2 % of the sky
//      join) is handed to search_kernel, one that finds fewer than K fails
//      (the reference's acceptance rule, GPU.cu:3659-3669);
//   4. a histogram of the list in 128 bins of squared distance (a monotone
//      map of [0, r^2]; 8-bit counts, four to a word, scanned bytewise),
//      the bin holding the K-th smallest key and the count below it; a
//      boundary bin with more keys than the 16-entry overflow list is split
//      32 ways (at most two refinements; beyond, only exact ties, the query
//      goes to search_kernel);
//   5. placement: the list index of every key below the boundary bin goes
//      to its bin's running slot of the row (a counting sort by bin), keys
//      of the boundary bin to the overflow list; the few bins holding two
//      keys or more are sorted, and so is the overflow list;
//   6. the warp writes each query's row with coalesced stores (distances
//      as sqrt in the data type), the first K - c_lo overflow keys last.
// Squared distances use the reference's fma chain in dimension order
// (kernel.cu:139-140) exactly as search_kernel does, so rows are identical.
// Keys are (squared distance bits, id) in one u64: ties are ordered by id.

#include <cmath>
#include <cstdlib>

#include "knnsj_internal.h"

namespace knnsj {

namespace {

constexpr int TILE_WARPS = 4;                    // warps per block
constexpr int TILE_THREADS = TILE_WARPS * 32;
constexpr int TILE_CH = 64;                      // staged candidates per chunk
constexpr int TILE_BINS0 = 128;                  // level-0 bins (8-bit counts, four to a word)
constexpr int TILE_BINS = 32;                    // bins of a refinement level (32-bit counts)
constexpr int TILE_OV = 16;                      // overflow keys per query
constexpr uint32_t TILE_MAX_ROWS = 4096;         // larger union boxes go to search_kernel

struct alignas(16) Cand {
  float x[3];
  uint32_t id;
};

// Capacity of a query's key list: more than twice k+1 (the learned radius
// finds 1.4 (k+1) keys on average; the few queries that find more are
// handed to search_kernel: 1.1 % of the sky join with 132 entries for
// k+1 = 65, about 0.2 % with 148, the most that 8 blocks of 4 warps of 4
// queries leave room for), the pitch in u64 words = 4 (mod 16) so that the
// lists of a warp's queries spread over the banks.
constexpr int tile_list_cap(int kmax) { return kmax >= 65 ? 148 : kmax >= 33 ? 84 : 52; }

// shared memory of one warp (bytes): QPT queries with rows of up to KMAX
// keys.  The staging chunk, the refinement histograms and the rows' u16
// list indices share one region (used one after another); a query's sorted
// row is assembled at the start of its own list.
template <int QPT, int KMAX>
struct TileSmem {
  static constexpr int C = tile_list_cap(KMAX);                 // list capacity per query (u64 keys)
  static constexpr int HP = TILE_BINS + 1;                      // histogram pitch (u32 words)
  static constexpr int RP = KMAX + 1;                           // row index pitch (u16)
  static constexpr int SHARED_BYTES =
      (TILE_CH * 16 > QPT * HP * 4 ? (TILE_CH * 16 > QPT * RP * 2 ? TILE_CH * 16 : QPT * RP * 2)
                                   : (QPT * HP * 4 > QPT * RP * 2 ? QPT * HP * 4 : QPT * RP * 2));
  static constexpr int LIST = 0;                                // [QPT][C] u64
  static constexpr int CAND = LIST + QPT * C * 8;               // staging chunk | refinement bins | row indices
  static constexpr int AUX = CAND;
  static constexpr int RIDX = CAND;
  static constexpr int HIST = (CAND + SHARED_BYTES + 15) / 16 * 16;  // [QPT][HP] u32
  static constexpr int OVC = HIST + QPT * HP * 4;               // [QPT] u32 overflow counts
  static constexpr int OVI = OVC + QPT * 4;                     // [QPT][TILE_OV] u16 overflow indices
  static constexpr int RUNS = (OVI + QPT * TILE_OV * 2 + 15) / 16 * 16;  // 2 x 32 u32
  static constexpr int BYTES = RUNS + 2 * 32 * 4;
};

struct TileParams {
  GridGeom<float> g;                    // candidate grid
  const float* __restrict__ ps;         // candidate columns in cell order (d x n)
  const uint32_t* __restrict__ pid;     // original id of each cell-ordered position
  const uint32_t* __restrict__ dstart;  // first position of every linear cell id (dense table)
  uint64_t n;
  uint32_t K;
  const float* __restrict__ qps;        // query columns: cell order (qlist null) or input order
  const uint32_t* __restrict__ qpid;    // ids of qps positions (qlist null)
  const uint32_t* __restrict__ qlist;   // query ids, or null: the positions of qps in qorder
  const uint32_t* __restrict__ qorder;  // positions of qps in tile order (null: 0, 1, ...)
  uint32_t nq;
  float radius;                         // uniform radius (qradius null)
  float* qradius;                       // per-query radius by id
  double step;                          // least growth of a failed per-query radius
  int32_t* out_ids;
  float* out_d;
  double* rowsum;                       // per-row verification sums (null: none)
  uint32_t* fail_list;
  uint32_t* fail_count;
  uint32_t* defer_list;                 // queries handed to search_kernel at the same radius
  uint32_t* defer_count;
  unsigned long long* cand_count;
  uint32_t* work_counter;
  FailRadii* fail_radii;
};

// round(a * s + c) clamped to [0, NB - 1], with the integer read from the
// low mantissa bits of a + 1.5 * 2^23 (one FMA); monotone in a.  c must be
// an integer (exact in float).
template <int NB>
__device__ __forceinline__ int tbin(float a, float s, float cm) {
  const int v = __float_as_int(__fmaf_rn(a, s, cm)) - 0x4b400000;
  return min(max(v, 0), NB - 1);
}

// Warp-aggregated append of this lane's value to a global list.
__device__ __forceinline__ void warp_append(bool want, uint32_t v, uint32_t* list, uint32_t* count, int lane) {
  const unsigned m = __ballot_sync(FULL, want);
  if (!m) return;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
  base = __shfl_sync(FULL, base, leader);
  if (want) list[base + __popc(m & lanemask_lt())] = v;
}

// QPT queries per warp (4, 8 or 16), LPQ = 32 / QPT lanes per query: lane
// (slot qs = lane % QPT, phase ph = lane / QPT) evaluates the staged
// candidates ph, ph + LPQ, ... for query qs.  The query's lanes share its
// list, histogram, row indices and overflow list in shared memory; the lane
// of phase 0 does the query's serial steps.  With 4 queries per warp the
// kernel is held to 64 registers: 8 blocks of 4 warps fit an SM.
template <int D, int KMAX, int QPT>
__global__ void __launch_bounds__(TILE_THREADS, QPT == 4 ? 8 : 5) tile_kernel(const TileParams p) {
  using SM = TileSmem<QPT, KMAX>;
  constexpr int LPQ = 32 / QPT;
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int qs = lane % QPT;
  const int ph = lane / QPT;
  const bool lead = ph == 0;
  unsigned char* ws = smem + (size_t)wib * SM::BYTES;
  Cand* cand = reinterpret_cast<Cand*>(ws + SM::CAND);
  unsigned long long* lists = reinterpret_cast<unsigned long long*>(ws + SM::LIST);  // [QPT][C]
  unsigned long long* mylist = lists + (size_t)qs * SM::C;  // this query's keys, later its row
  uint32_t* hq = reinterpret_cast<uint32_t*>(ws + SM::HIST) + qs * SM::HP;  // this query's bins
  uint32_t* aq = reinterpret_cast<uint32_t*>(ws + SM::AUX) + qs * SM::HP;
  uint16_t* rowix = reinterpret_cast<uint16_t*>(ws + SM::RIDX);  // [QPT][RP] list indices by row slot
  uint32_t* ovcs = reinterpret_cast<uint32_t*>(ws + SM::OVC);
  uint32_t* ovc = ovcs + qs;
  uint16_t* ovi = reinterpret_cast<uint16_t*>(ws + SM::OVI);  // [QPT][TILE_OV] list indices
  uint32_t* runS = reinterpret_cast<uint32_t*>(ws + SM::RUNS);
  uint32_t* runP = runS + 32;
  // this query's lanes, and those of them below this lane
  unsigned qmask = 0;
#pragma unroll
  for (int pp = 0; pp < LPQ; pp++) qmask |= 1u << (qs + QPT * pp);
  const unsigned qbelow = qmask & lanemask_lt();

  __shared__ float s_minf[3];
  __shared__ float s_invw;
  if (threadIdx.x < 3) s_minf[threadIdx.x] = threadIdx.x < (unsigned)D ? (float)p.g.minv[threadIdx.x] : 0.0f;
  if (threadIdx.x == 0) s_invw = 1.0f / (float)p.g.width;
  __syncthreads();

  const uint64_t n = p.n;
  const uint32_t K = p.K;
  const uint32_t ntiles = (p.nq + QPT - 1) / QPT;
  unsigned long long scanned = 0;

  for (;;) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(p.work_counter, 1u);
    t = __shfl_sync(FULL, t, 0);
    if (t >= ntiles) break;
    const uint32_t qi = t * (uint32_t)QPT + (uint32_t)qs;
    const bool valid = qi < p.nq;
    uint32_t qid = 0;
    float q[D];
    float r = 0.0f;
#pragma unroll
    for (int j = 0; j < D; j++) q[j] = 0.0f;
    if (valid) {
      const uint32_t pos = p.qorder ? p.qorder[qi] : qi;
      qid = p.qlist ? p.qlist[qi] : p.qpid[pos];
      const uint64_t col = p.qlist ? (uint64_t)qid : (uint64_t)pos;
#pragma unroll
      for (int j = 0; j < D; j++) q[j] = p.qps[(uint64_t)j * n + col];
      r = p.qradius ? p.qradius[qid] : p.radius;
    }

    // 1. the query's ring (as search_kernel computes it) and the union box
    const float rf = r * (1.0f + 1.0f / 8192.0f);
    uint32_t lo[D], hi[D];
    uint32_t ext = 0;
#pragma unroll
    for (int j = 0; j < D; j++) {
      const float slack = (fabsf(q[j]) + rf) * (1.0f / 2097152.0f);
      lo[j] = ring_cell(q[j] - rf - slack, s_minf[j], s_invw, p.g.ncell[j], false);
      hi[j] = ring_cell(q[j] + rf + slack, s_minf[j], s_invw, p.g.ncell[j], true);
      ext = max(ext, hi[j] - lo[j] + 1);
    }
    // queries whose ring is far wider than the tile's mean go to search_kernel
    // (one outlier would widen every query's scan)
    bool defer = false;
    {
      const uint32_t nv = __popc(__ballot_sync(FULL, valid));  // (each query counted LPQ times)
      const uint32_t sum = __reduce_add_sync(FULL, valid ? ext : 0u);
      const uint32_t mean = (sum + nv - 1) / nv;
      defer = valid && ext > 2u * mean + 2u;
    }
    bool in = valid && !defer;  // queries searched by this tile
    uint32_t LO[D], HI[D];
#pragma unroll
    for (int j = 0; j < D; j++) {
      LO[j] = __reduce_min_sync(FULL, in ? lo[j] : 0xffffffffu);
      HI[j] = __reduce_max_sync(FULL, in ? hi[j] : 0u);
    }
    uint32_t ext1 = HI[1] - LO[1] + 1;
    uint32_t ext2 = D == 3 ? HI[D - 1] - LO[D - 1] + 1 : 1u;
    uint64_t nrows64 = __ballot_sync(FULL, in) ? (uint64_t)ext1 * ext2 : 0;
    if (nrows64 > TILE_MAX_ROWS) {  // (uniform) the whole tile goes to search_kernel
      defer = valid;
      in = false;
      nrows64 = 0;
    }
    uint32_t nrows = (uint32_t)nrows64;
    warp_append(defer && lead, qid, p.defer_list, p.defer_count, lane);

    const float thr = in ? within_threshold(r) : -1.0f;  // acc <= thr never holds off the tile
    const float s0 = (thr > 0.0f && thr < 3.0e38f) ? __fdividef((float)TILE_BINS0, thr) : 0.0f;
    const float MAG = 12582912.0f;  // 1.5 * 2^23

    // Visits every candidate of the union box; body(c, live) runs on every
    // lane, live when c is a candidate of this lane's phase.
    auto for_each_candidate = [&](auto&& body) -> uint32_t {
      uint32_t visited = 0;
      for (uint32_t g0 = 0; g0 < nrows; g0 += 32) {
        const uint32_t ridx = g0 + (uint32_t)lane;
        uint32_t rs = 0, len = 0;
        if (ridx < nrows) {
          unsigned long long rbase;
          if constexpr (D == 2) {
            rbase = (unsigned long long)(LO[1] + ridx) * p.g.mult[1];
          } else {
            const uint32_t a1 = ridx % ext1, a2 = ridx / ext1;
            rbase = (unsigned long long)(LO[1] + a1) * p.g.mult[1] + (unsigned long long)(LO[D - 1] + a2) * p.g.mult[D - 1];
          }
          rs = p.dstart[rbase + LO[0]];
          len = p.dstart[rbase + HI[0] + 1] - rs;
        }
        uint32_t incl = len;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const uint32_t tt = __shfl_up_sync(FULL, incl, off);
          if (lane >= off) incl += tt;
        }
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        visited += total;
        __syncwarp();
        runS[lane] = rs;
        runP[lane] = incl - len;
        __syncwarp();
        // chunks are loaded one ahead: the loads of chunk c + 1 are in flight
        // while chunk c is evaluated
        int row = 0;
        Cand pre[TILE_CH / 32];
        auto fetch = [&](uint32_t c0) {
#pragma unroll
          for (int m = 0; m < TILE_CH / 32; m++) {
            const uint32_t v = c0 + (uint32_t)(m * 32 + lane);
            if (v < total) {
              while (row < 31 && runP[row + 1] <= v) row++;
              const uint32_t pos = runS[row] + (v - runP[row]);
#pragma unroll
              for (int j = 0; j < 3; j++) pre[m].x[j] = j < D ? p.ps[(uint64_t)j * n + pos] : 0.0f;
              pre[m].id = p.pid[pos];
            }
          }
        };
        if (total) fetch(0);
        for (uint32_t c0 = 0; c0 < total; c0 += TILE_CH) {
          const uint32_t cnt = min((uint32_t)TILE_CH, total - c0);
          __syncwarp();
#pragma unroll
          for (int m = 0; m < TILE_CH / 32; m++)
            if (c0 + (uint32_t)(m * 32 + lane) < total) cand[m * 32 + lane] = pre[m];
          __syncwarp();
          if (c0 + TILE_CH < total) fetch(c0 + TILE_CH);
          const uint32_t steps = (cnt + LPQ - 1) / LPQ;
          uint32_t st = 0;
          for (; st + 4 <= steps; st += 4) {
            Cand c4[4];
            bool l4[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const uint32_t j = (st + u) * LPQ + ph;
              l4[u] = j < cnt;
              c4[u] = cand[l4[u] ? j : 0];
            }
#pragma unroll
            for (int u = 0; u < 4; u++) body(c4[u], l4[u]);
          }
          for (; st < steps; st++) {
            const uint32_t j = st * LPQ + ph;
            const bool live = j < cnt;
            const Cand cc = cand[live ? j : 0];
            body(cc, live);
          }
        }
        __syncwarp();
      }
      return visited;
    };
    auto sqdist = [&](const Cand& c) -> float {
      float acc = 0.0f;
#pragma unroll
      for (int j = 0; j < D; j++) {
        const float tt = __fsub_rn(c.x[j], q[j]);
        acc = __fmaf_rn(tt, tt, acc);
      }
      return acc;
    };
    // zeroes a query's 32 histogram words (its LPQ lanes share the work)
    auto clear_bins = [&](uint32_t* h) {
      for (int b = ph; b < TILE_BINS; b += LPQ) h[b] = 0u;
    };

    // The boundary search over one query's 128 level-0 bins, 8-bit counts
    // packed four to a word (h[w] holds bins 4w .. 4w+3; every count and
    // every prefix is at most the list capacity, below 256, so bytewise sums
    // never carry): each of the query's LPQ lanes takes 32 / LPQ consecutive
    // words, one multiply by 0x01010101 gives a word's inclusive prefix per
    // byte, a scan over the query's lanes gives each lane its starting
    // count, and the bins become their exclusive prefix.  Outputs as for
    // walk_bins below; `multi` gets a bit for each of this lane's bins
    // (32 / LPQ words from bin 128 / LPQ * ph on) holding two keys or more.
    auto walk_bytes = [&](uint32_t* h, uint32_t& total, uint32_t& lo_cnt, uint32_t& mb, uint32_t& bstar,
                          unsigned long long& multi) {
      constexpr int WPL = 32 / LPQ;
      uint32_t wv[WPL];
      uint32_t part = 0;
      multi = 0;
#pragma unroll
      for (int i = 0; i < WPL; i++) {
        wv[i] = h[ph * WPL + i];
        part += (wv[i] * 0x01010101u) >> 24;
        // bytes of 2 or more, 4 bits per word (a byte's carry only reaches
        // bins above one of 130 keys or more, which lies at or above the
        // boundary bin: the bins that get sorted hold fewer than K keys)
        const uint32_t two = (wv[i] + 0x7e7e7e7eu) & 0x80808080u;
        const uint32_t nib = ((two >> 7) & 1u) | ((two >> 14) & 2u) | ((two >> 21) & 4u) | ((two >> 28) & 8u);
        multi |= (unsigned long long)nib << (4 * i);
      }
      uint32_t incl = part;
#pragma unroll
      for (int off = 1; off < LPQ; off <<= 1) {
        const uint32_t tt = __shfl_up_sync(FULL, incl, off * QPT);
        if (ph >= off) incl += tt;
      }
      uint32_t cum = incl - part;
      uint32_t fb = TILE_BINS0, flo = 0, fm = 0;
#pragma unroll
      for (int i = 0; i < WPL; i++) {
        const uint32_t w = wv[i];
        const uint32_t pin = w * 0x01010101u;  // inclusive prefix within the word, per byte
        h[ph * WPL + i] = (pin - w) + cum * 0x01010101u;
        if (fb == TILE_BINS0 && cum + (pin >> 24) >= K) {
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const uint32_t cj = (pin >> (8 * j)) & 0xffu;
            if (fb == TILE_BINS0 && cum + cj >= K) {
              fb = (uint32_t)(4 * (ph * WPL + i) + j);
              fm = (w >> (8 * j)) & 0xffu;
              flo = cum + cj - fm;
            }
          }
        }
        cum += pin >> 24;
      }
      total = __shfl_sync(FULL, incl, qs + QPT * (LPQ - 1));
      const unsigned hit = __ballot_sync(FULL, fb != TILE_BINS0);
      const unsigned mine = hit & qmask;
      const int src = mine ? __ffs(mine) - 1 : qs;
      bstar = __shfl_sync(FULL, fb, src);
      lo_cnt = __shfl_sync(FULL, flo, src);
      mb = __shfl_sync(FULL, fm, src);
    };

    // The boundary search over one query's 32 bins (counts h[b], base keys
    // below bin 0), shared by its LPQ lanes: each lane sums its 32 / LPQ
    // consecutive bins, a scan over the query's lanes gives each lane its
    // starting count, and the lane holding the bin where the count reaches K
    // reports it.  With `prefix` the bins are replaced by their exclusive
    // prefix (plus base).  Outputs are the query's (same on its lanes).
    auto walk_bins = [&](uint32_t* h, uint32_t base, bool prefix, uint32_t& total, uint32_t& lo_cnt,
                         uint32_t& mb, uint32_t& bstar) {
      constexpr int BPL = TILE_BINS / LPQ;
      uint32_t part = 0;
#pragma unroll
      for (int i = 0; i < BPL; i++) part += h[ph * BPL + i];
      uint32_t incl = part;
#pragma unroll
      for (int off = 1; off < LPQ; off <<= 1) {
        const uint32_t tt = __shfl_up_sync(FULL, incl, off * QPT);
        if (ph >= off) incl += tt;
      }
      uint32_t cum = base + incl - part;
      uint32_t fb = TILE_BINS, flo = 0, fm = 0;
#pragma unroll
      for (int i = 0; i < BPL; i++) {
        const int b = ph * BPL + i;
        const uint32_t hh = h[b];
        if (prefix) h[b] = cum;
        if (fb == TILE_BINS && cum + hh >= K) {
          fb = (uint32_t)b;
          flo = cum;
          fm = hh;
        }
        cum += hh;
      }
      total = __shfl_sync(FULL, base + incl, qs + QPT * (LPQ - 1)) - base;
      // the first lane of the query (by phase) that found the boundary
      const unsigned hit = __ballot_sync(FULL, fb != TILE_BINS);
      const unsigned mine = hit & qmask;
      const int src = mine ? __ffs(mine) - 1 : qs;
      bstar = __shfl_sync(FULL, fb, src);
      lo_cnt = __shfl_sync(FULL, flo, src);
      mb = __shfl_sync(FULL, fm, src);
    };

    // 3. pass 1: every key within the radius is appended to the query's
    // list (slots from a ballot over the query's lanes: no atomics); the
    // count goes on past the capacity, so `found` is exact
    uint32_t found = 0;
    const uint32_t box_points = for_each_candidate([&](const Cand& c, bool live) {
      const float acc = sqdist(c);
      const bool want = live && acc <= thr;
      const unsigned bal = __ballot_sync(FULL, want);
      const uint32_t slot = found + (uint32_t)__popc(bal & qbelow);
      if (want && slot < (uint32_t)SM::C)
        mylist[slot] = ((unsigned long long)__float_as_uint(acc) << 32) | c.id;
      found += (uint32_t)__popc(bal & qmask);
    });
    // candidates evaluated: the union box's points for every query it serves
    scanned += (unsigned long long)box_points * (unsigned)__popc(__ballot_sync(FULL, in && lead));
    // a query with more keys than its list holds goes to search_kernel
    const bool big = in && found > (uint32_t)SM::C;
    warp_append(big && lead, qid, p.defer_list, p.defer_count, lane);
    bool ok = in && found >= K && !big;
    const uint32_t nl = ok ? found : 0u;  // list entries of an accepted query
    __syncwarp();

    // 128 bins of squared distance over the list (8-bit counts), the
    // boundary bin of level 0 and the counts below it; the bins become their
    // exclusive prefix
    clear_bins(hq);
    __syncwarp();
    for (uint32_t e = (uint32_t)ph; e < nl; e += LPQ) {
      const int b = tbin<TILE_BINS0>(__uint_as_float((uint32_t)(mylist[e] >> 32)), s0, MAG);
      atomicAdd(&hq[b >> 2], 1u << (8 * (b & 3)));
    }
    __syncwarp();
    uint32_t listed = 0, c_lo = 0, m = 0, bs0 = TILE_BINS0;
    unsigned long long multi = 0;
    walk_bytes(hq, listed, c_lo, m, bs0, multi);

    // refinement of the boundary bin while it overflows the overflow list
    int lev = 0;
    int bs[3] = {(int)bs0, TILE_BINS, TILE_BINS};
    float sl[3] = {s0, 0.0f, 0.0f}, cl[3] = {0.0f, 0.0f, 0.0f};  // scale and integer offset per level
#pragma unroll
    for (int L = 1; L < 3; L++) {
      const bool need = ok && lev == L - 1 && m > (uint32_t)TILE_OV;
      if (!__any_sync(FULL, need)) break;
      if (need) {
        sl[L] = sl[L - 1] * (float)TILE_BINS;
        cl[L] = (float)TILE_BINS * (cl[L - 1] - ((float)bs[L - 1] - 0.5f));
        clear_bins(aq);
      }
      __syncwarp();
      if (need) {
        for (uint32_t e = (uint32_t)ph; e < nl; e += LPQ) {
          const float acc = __uint_as_float((uint32_t)(mylist[e] >> 32));
          if (tbin<TILE_BINS0>(acc, sl[0], MAG) != bs[0]) continue;
          bool member = true;
#pragma unroll
          for (int l2 = 1; l2 < L; l2++)
            if (tbin<TILE_BINS>(acc, sl[l2], MAG + cl[l2]) != bs[l2]) member = false;
          if (member) atomicAdd(&aq[tbin<TILE_BINS>(acc, sl[L], MAG + cl[L])], 1u);
        }
      }
      __syncwarp();
      uint32_t nb = TILE_BINS, nlo = c_lo, nm = m, ntot = 0;
      walk_bins(aq, c_lo, false, ntot, nlo, nm, nb);
      if (need) {
        bs[L] = (int)nb;
        c_lo = nlo;
        m = nm;
        lev = L;
      }
      __syncwarp();
    }
    // still more boundary keys than the overflow list holds (exact ties):
    // search_kernel takes the query
    const bool tie_defer = ok && m > (uint32_t)TILE_OV;
    warp_append(tie_defer && lead, qid, p.defer_list, p.defer_count, lane);
    ok = ok && !tie_defer;

    // 4. placement: the list index of every key below the boundary bin goes
    // to its bin's running slot of the row (a counting sort by bin), the
    // keys of the boundary bin to the overflow list
    if (lead) *ovc = 0u;
    __syncwarp();
    if (ok) {
      uint16_t* myridx = rowix + qs * SM::RP;
      uint16_t* myovi = ovi + qs * TILE_OV;
      for (uint32_t e = (uint32_t)ph; e < nl; e += LPQ) {
        const float acc = __uint_as_float((uint32_t)(mylist[e] >> 32));
        const int b0 = tbin<TILE_BINS0>(acc, sl[0], MAG);
        bool place = b0 < bs[0];
        bool over = b0 == bs[0] && lev == 0;
        if (b0 == bs[0] && lev > 0) {  // (refined boundary bins only)
          const int b1 = tbin<TILE_BINS>(acc, sl[1], MAG + cl[1]);
          if (b1 < bs[1]) {
            place = true;
          } else if (b1 == bs[1]) {
            if (lev == 1) {
              over = true;
            } else {
              const int b2 = tbin<TILE_BINS>(acc, sl[2], MAG + cl[2]);
              place = b2 < bs[2];
              over = b2 == bs[2];
            }
          }
        }
        if (place) {
          const int sh = 8 * (b0 & 3);
          myridx[(atomicAdd(&hq[b0 >> 2], 1u << sh) >> sh) & 0xffu] = (uint16_t)e;
        }
        if (over) myovi[atomicAdd(ovc, 1u)] = (uint16_t)e;
      }
    }
    __syncwarp();

    // 5. rows in order: after placement the byte of bin b <= bs0 holds the
    // end of its slots (its start is the end of bin b - 1); only the bins
    // the histogram found with two keys or more need ordering (the bins are
    // narrow: 0.7 keys on average), and one lane sorts the overflow indices,
    // whose smallest complete the row
    auto isort_idx = [&](uint16_t* a, uint32_t lo, uint32_t hi) {
      for (uint32_t i = lo + 1; i < hi; i++) {
        const uint16_t ix = a[i];
        const unsigned long long key = mylist[ix];
        uint32_t j = i;
        while (j > lo) {
          const uint16_t pix = a[j - 1];
          if (mylist[pix] <= key) break;
          a[j] = pix;
          j--;
        }
        a[j] = ix;
      }
    };
    auto sort_idx = [&](uint16_t* a, uint32_t lo, uint32_t hi) {
      if (hi - lo == 2) {
        const uint16_t i0 = a[lo], i1 = a[lo + 1];
        if (mylist[i1] < mylist[i0]) {
          a[lo] = i1;
          a[lo + 1] = i0;
        }
      } else if (hi - lo > 2) {
        isort_idx(a, lo, hi);
      }
    };
    if (ok) {
      constexpr int BPL = TILE_BINS0 / LPQ;  // bins per lane
      uint16_t* myridx = rowix + qs * SM::RP;
      // this lane's bins with placed keys: up to bs0 (bs0 itself only when
      // refined: otherwise its keys are in the overflow list)
      const int top = bs[0] - (lev == 0 ? 1 : 0) - BPL * ph;
      unsigned long long mm = top < 0 ? 0ull : (top >= BPL - 1 ? multi : multi & ((2ull << top) - 1ull));
      // a refined boundary bin is sorted whatever its count (a count above
      // 129 would not show in the bytewise test)
      if (lev > 0 && top >= 0 && top < BPL) mm |= 1ull << top;
      while (mm) {
        const int b = BPL * ph + __ffsll((long long)mm) - 1;
        mm &= mm - 1;
        const uint32_t w = hq[b >> 2];
        const int j = b & 3;
        const uint32_t hi = (w >> (8 * j)) & 0xffu;
        const uint32_t lo = j ? (w >> (8 * (j - 1))) & 0xffu : (b ? hq[(b >> 2) - 1] >> 24 : 0u);
        sort_idx(myridx, lo, hi);
      }
      if (ph == LPQ - 1) sort_idx(ovi + qs * TILE_OV, 0u, *ovc);
    }
    __syncwarp();
    // coalesced row writes: the warp writes each accepted query's row, slot
    // s from the list entry of row index s (s < c_lo) or of overflow index
    // s - c_lo
    {
      unsigned mask = __ballot_sync(FULL, ok && lead);
      while (mask) {
        const int rl = __ffs(mask) - 1;  // (a lead lane: its index is the query slot)
        mask &= mask - 1;
        const uint32_t rid = __shfl_sync(FULL, qid, rl);
        const uint32_t rclo = __shfl_sync(FULL, c_lo, rl);
        const unsigned long long* rlist = lists + (size_t)rl * SM::C;
        const uint16_t* rix = rowix + rl * SM::RP;
        const uint16_t* rov = ovi + rl * TILE_OV;
        const uint64_t base = (uint64_t)rid * K;
        float rsq = 0.0f;
        for (uint32_t s = (uint32_t)lane; s < K; s += 32) {
          const unsigned long long key = rlist[s < rclo ? rix[s] : rov[s - rclo]];
          const float dist = __fsqrt_rn(__uint_as_float((uint32_t)(key >> 32)));
          p.out_ids[base + s] = (int32_t)(uint32_t)key;
          p.out_d[base + s] = dist;
          rsq = __fadd_rn(rsq, __fmul_rn(dist, dist));
        }
        if (p.rowsum) store_row_sum<float>(p.rowsum, rid, rsq, lane);
      }
    }
    // failures: fewer than K points within the radius
    const bool fail = in && found < K;
    warp_append(fail && lead, qid, p.fail_list, p.fail_count, lane);
    if (fail && lead && p.qradius) {
      // per-query radii grow by at least eps0/2, toward K points from the
      // count found within the radius: (K / found)^(1/dims), at most 4x
      double rn = (double)r + p.step;
      const float f = exp2f(log2f((float)K / (float)max(found, 1u)) / (float)D) * 1.05f;
      rn = fmax(rn, (double)r * (double)fminf(fmaxf(f, 1.0f), 4.0f));
      const float rt = (float)rn;
      p.qradius[qid] = rt;
      atomicMax(&p.fail_radii->rmax_bits, (unsigned long long)__float_as_uint(rt));
      const float oct = log2f(rt / (2.0f * (float)p.step));  // log2(r / eps0)
      const int bin = min(max((int)floorf(4.0f * oct) + 16, 0), FAIL_RADIUS_BINS - 1);
      atomicAdd(&p.fail_radii->hist[bin], 1u);
    }
    __syncwarp();
  }
  if (lane == 0 && scanned) atomicAdd(p.cand_count, scanned);
}

template <int D, int KMAX, int QPT>
void launch_tile_kernel(const TileParams& prm, int sm_count, cudaStream_t s) {
  using SM = TileSmem<QPT, KMAX>;
  const size_t smem = (size_t)SM::BYTES * TILE_WARPS;
  auto kern = tile_kernel<D, KMAX, QPT>;
  KNNSJ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  KNNSJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TILE_THREADS, smem));
  if (per_sm < 1) throw StatusError{KNNSJ_ERR_UNSUPPORTED, "tile kernel does not fit"};
  const uint64_t tiles = ((uint64_t)prm.nq + QPT - 1) / QPT;
  uint64_t blocks = (uint64_t)per_sm * sm_count;
  const uint64_t need = (tiles + TILE_WARPS - 1) / TILE_WARPS;
  if (need < blocks) blocks = need;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, TILE_THREADS, smem, s>>>(prm);
  KNNSJ_CHECK_LAUNCH();
}

}  // namespace

bool tile_search_applies(uint32_t d, uint32_t di, uint32_t K, int dense, size_t elem) {
  return elem == 4 && (d == 2 || d == 3) && di == d && K <= 65 && dense;
}

template <typename T>
void launch_tile_search(const SearchLaunch<T>& a, uint32_t* defer_list, uint32_t* defer_count, int sm_count,
                        cudaStream_t s) {
  if constexpr (sizeof(T) != 4) {
    throw StatusError{KNNSJ_ERR_UNSUPPORTED, "tile search is float only"};
  } else {
    if (a.nq == 0) return;
    TileParams p{};
    p.g = a.grid.geom;
    p.ps = a.grid.ps;
    p.pid = a.grid.pid;
    p.dstart = a.grid.dstart;
    p.n = a.n;
    p.K = a.K;
    p.qlist = a.qlist;
    p.qps = a.qlist ? a.xs : (a.qps ? a.qps : a.grid.ps);
    p.qpid = a.qps ? a.qpid : a.grid.pid;
    p.qorder = a.qlist ? nullptr : a.qorder;
    p.nq = a.nq;
    p.radius = a.radius;
    p.qradius = a.qradius;
    p.step = (double)a.step;
    p.out_ids = a.out_ids;
    p.out_d = a.out_d;
    p.rowsum = a.rowsum;
    p.fail_list = a.fail_list;
    p.fail_count = a.fail_count;
    p.defer_list = defer_list;
    p.defer_count = defer_count;
    p.cand_count = a.cand_count;
    p.work_counter = a.work_counter;
    p.fail_radii = a.fail_radii;
    launch_zero_words(a.work_counter, sizeof(uint32_t), s);
    const bool d3 = a.d == 3;
    // queries per tile: 8 share a box best (fewest candidates per query),
    // but their lists need twice the shared memory of 4; with 4 (64
    // registers, 8 blocks of 4 warps per SM) the kernel keeps 32 warps per
    // SM against 20, and the tile kernel is bound by latency: 4 is faster
    int qpt = 4;
    if (const char* e = std::getenv("KNNSJ_TILE_QPT")) qpt = std::atoi(e);
#define KNNSJ_TILE_LAUNCH(QPT)                                                                 \
  do {                                                                                        \
    if (a.K <= 16)                                                                            \
      d3 ? launch_tile_kernel<3, 16, QPT>(p, sm_count, s) : launch_tile_kernel<2, 16, QPT>(p, sm_count, s); \
    else if (a.K <= 33)                                                                       \
      d3 ? launch_tile_kernel<3, 33, QPT>(p, sm_count, s) : launch_tile_kernel<2, 33, QPT>(p, sm_count, s); \
    else                                                                                      \
      d3 ? launch_tile_kernel<3, 65, QPT>(p, sm_count, s) : launch_tile_kernel<2, 65, QPT>(p, sm_count, s); \
  } while (0)
    if (qpt == 16)
      KNNSJ_TILE_LAUNCH(16);
    else if (qpt == 4)
      KNNSJ_TILE_LAUNCH(4);
    else
      KNNSJ_TILE_LAUNCH(8);
#undef KNNSJ_TILE_LAUNCH
  }
}

template void launch_tile_search<float>(const SearchLaunch<float>&, uint32_t*, uint32_t*, int, cudaStream_t);
template void launch_tile_search<double>(const SearchLaunch<double>&, uint32_t*, uint32_t*, int, cudaStream_t);

}  // namespace knnsj
