// join.cu -- the self-join pipeline on one GPU.
//
// Host side of the reference's main()/KNNJoinPy (main.cu:109-510, 514-907),
// re-planned for one resident dataset:
//   1. dimension order (ReorderByDimension, main.cu:2521-2615) on the host,
//      from every 100th point, in the reference's float/double arithmetic;
//   2. one transpose into column arrays in that order (device);
//   3. eps0 from BETA (sampleNeighborsBruteForce, GPU.cu:3088-3566);
//   4. grid dimensions (generateNDGridDimensions, main.cu:2425-2488) and the
//      grid index at width eps0 (populateNDGridIndexAndLookupArrayGPU,
//      GPU.cu:3715-4067), built once and kept in HBM;
//   5. the retry loop (main.cu:312-430): search all queries at eps0, then the
//      failed ones at eps0 + m*eps0/2 over the widened cell ring of the same
//      grid.  The reference repeats a pass at an unchanged radius when at
//      most 25% failed (main.cu:330); that pass cannot succeed, so here the
//      radius grows every pass.  When the ring would need many more cells
//      than 3^NUMINDEXEDDIM, the grid is rebuilt at the current radius, as
//      the reference does on every growth (main.cu:353).
// Every device buffer lives in a per-device workspace reused across calls.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <vector>

#include "knnsj_internal.h"
#include "knnsj_host.h"
#include "radius_model.cuh"
#include "ring_policy.h"

namespace knnsj {

thread_local unsigned long long g_launches = 0;
thread_local bool g_forbid_alloc = false;

void* Arena::take(size_t bytes) {
  const size_t at = (used + 255) & ~(size_t)255;
  if (at + bytes > cap)
    throw StatusError{KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH, "problem exceeds the fixed scratch array"};
  used = at + bytes;
  return base + at;
}

void Workspace::attach_arena(Arena* a) {
  DevBuf* bufs[] = {&model, &in, &ids, &dists, &xs, &ps, &psf, &pid, &keys0, &keys1, &vals0, &vals1, &hist,
                    &scan_tmp, &flags, &pos, &ckeys, &coff, &dstart, &list0, &list1, &small,
                    &eps_partial, &eps_sample, &perm, &minmax_part, &qradius, &chunk_list, &patch_rows, &defer_list,
                    &fps, &fpid, &fdstart, &qorder, &rowsum};
  for (DevBuf* b : bufs) {
    b->arena = a;
    b->p = nullptr;
    b->bytes = 0;
  }
  model_version = 0;
}

void* DevBuf::get(size_t need) {
  if (need == 0) need = 16;
  if (arena) {
    if (need > bytes) {
      unsigned char* b = (unsigned char*)p;
      if (b && b + bytes == arena->base + arena->used && (size_t)(b - arena->base) + need <= arena->cap) {
        arena->used = (size_t)(b - arena->base) + need;  // the last block carved grows in place
      } else {
        p = arena->take(need);
      }
      bytes = need;
    }
    return p;
  }
  if (need > bytes) {
    if (g_forbid_alloc) throw StatusError{KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH, "buffer outside the fixed scratch array"};
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      throw StatusError{KNNSJ_ERR_OUT_OF_MEMORY, "cudaMalloc"};
    }
    bytes = need;
  }
  return p;
}

void DevBuf::release() {
  if (p && !arena) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

Workspace& workspace(int device) {
  static std::vector<Workspace*> all;
  static std::mutex m;
  std::lock_guard<std::mutex> g(m);
  if ((int)all.size() <= device) all.resize(device + 1, nullptr);
  if (!all[device]) all[device] = new Workspace();
  return *all[device];
}

void Workspace::release_all() {
  model_version = 0;
  DevBuf* bufs[] = {&model, &in, &ids, &dists, &xs, &ps, &psf, &pid, &keys0, &keys1, &vals0, &vals1, &hist,
                    &scan_tmp, &flags, &pos, &ckeys, &coff, &dstart, &list0, &list1, &small,
                    &eps_partial, &eps_sample, &perm, &minmax_part, &qradius, &chunk_list, &patch_rows, &defer_list,
                    &fps, &fpid, &fdstart, &qorder, &rowsum};
  for (DevBuf* b : bufs) b->release();
  if (stream) cudaStreamDestroy(stream);
  stream = nullptr;
  if (copy_stream) cudaStreamDestroy(copy_stream);
  copy_stream = nullptr;
  for (auto& e : ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  for (auto& e : chunk_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  if (mail_host) cudaFreeHost(mail_host);
  mail_host = mail_dev = nullptr;
  mail = false;
  pinned_release();
}

void Workspace::pinned_release() {
  if (h_pinned) cudaFreeHost(h_pinned);
  h_pinned = nullptr;
  h_pinned_bytes = 0;
}

void* Workspace::pinned(size_t need) {
  if (need > h_pinned_bytes) {
    if (g_forbid_alloc) throw StatusError{KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH, "pinned buffer in a fixed-scratch join"};
    pinned_release();
    KNNSJ_CUDA(cudaMallocHost(&h_pinned, need));
    h_pinned_bytes = need;
  }
  return h_pinned;
}

void Workspace::ensure_stream() {
  if (g_forbid_alloc && !stream) throw StatusError{KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH, "stream in a fixed-scratch join"};
  if (!stream) KNNSJ_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  for (auto& e : ev)
    if (!e) KNNSJ_CUDA(cudaEventCreate(&e));
}

void Workspace::ensure_copy_stream() {
  if (g_forbid_alloc) throw StatusError{KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH, "copy stream in a fixed-scratch join"};
  if (!copy_stream) KNNSJ_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
  for (auto& e : chunk_ev)
    if (!e) KNNSJ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  if (!mail_host) {
    KNNSJ_CUDA(cudaHostAlloc(&mail_host, MAIL_BYTES, cudaHostAllocMapped));
    KNNSJ_CUDA(cudaHostGetDevicePointer(&mail_dev, mail_host, 0));
  }
}

namespace {

__global__ void copy_words_kernel(uint32_t* __restrict__ dst, const uint32_t* __restrict__ src, uint64_t words) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

__global__ void zero_words_kernel(uint32_t* __restrict__ p, uint64_t words) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = 0u;
}

void launch_copy_words(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  const uint64_t words = bytes / 4;
  const uint64_t blocks = std::min<uint64_t>((words + 255) / 256, 1024);
  if (blocks == 0) return;
  copy_words_kernel<<<(unsigned)blocks, 256, 0, s>>>((uint32_t*)dst, (const uint32_t*)src, words);
  KNNSJ_CHECK_LAUNCH();
}

__global__ void copy_vec16_kernel(uint4* __restrict__ dst, const uint4* __restrict__ src, uint64_t n16) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

}  // namespace

// Copies a device table into mapped pinned host memory with an SM kernel:
// 16-byte loads and stores in address order, so the host receives whole
// cache lines (13 GB of rows in 67 ms on GB300, the rate of a copy-engine
// copy).  Unaligned buffers fall back to 4-byte words, then to a copy.
void launch_copy_to_mapped(void* dst, const void* src, size_t bytes, int sm_count, cudaStream_t s) {
  const uintptr_t a = (uintptr_t)dst | (uintptr_t)src;
  if ((a & 15) == 0) {
    const uint64_t n16 = bytes / 16;
    if (n16) {
      const uint64_t blocks = std::min<uint64_t>((n16 + 511) / 512, (uint64_t)std::max(sm_count, 1) * 2);
      copy_vec16_kernel<<<(unsigned)blocks, 512, 0, s>>>((uint4*)dst, (const uint4*)src, n16);
      KNNSJ_CHECK_LAUNCH();
    }
    const size_t done = n16 * 16;
    if (bytes > done && (bytes - done) % 4 == 0)
      launch_copy_words((char*)dst + done, (const char*)src + done, bytes - done, s);
    else if (bytes > done)
      KNNSJ_CUDA(cudaMemcpyAsync((char*)dst + done, (const char*)src + done, bytes - done, cudaMemcpyDefault, s));
  } else if ((a & 3) == 0 && bytes % 4 == 0) {
    launch_copy_words(dst, src, bytes, s);
  } else {
    KNNSJ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s));
  }
}

void launch_zero_words(void* p, size_t bytes, cudaStream_t s) {
  const uint64_t words = bytes / 4;
  const uint64_t blocks = std::min<uint64_t>((words + 255) / 256, 1024);
  if (blocks == 0) return;
  zero_words_kernel<<<(unsigned)blocks, 256, 0, s>>>((uint32_t*)p, words);
  KNNSJ_CHECK_LAUNCH();
}

// Device-to-device copy (bytes a multiple of 4).
static void dev_copy(Workspace& w, void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (w.mail)
    launch_copy_words(dst, src, bytes, s);
  else
    KNNSJ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s));
}

// Device-to-host read of a few bytes (a multiple of 4); synchronises s.
static void read_small(Workspace& w, void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (w.mail) {
    if (bytes > MAIL_BYTES / 2) throw StatusError{KNNSJ_ERR_UNSUPPORTED, "mailbox read too large"};
    launch_copy_words(w.mail_dev, src, bytes, s);
    KNNSJ_CUDA(cudaStreamSynchronize(s));
    std::memcpy(dst, w.mail_host, bytes);
    return;
  }
  KNNSJ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
  KNNSJ_CUDA(cudaStreamSynchronize(s));
}

// Host-to-device write of a few bytes (a multiple of 4); the source may be
// reused on return.
static void write_small(Workspace& w, void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (w.mail) {
    if (bytes > MAIL_BYTES / 2) throw StatusError{KNNSJ_ERR_UNSUPPORTED, "mailbox write too large"};
    unsigned char* in_host = (unsigned char*)w.mail_host + MAIL_BYTES / 2;
    std::memcpy(in_host, src, bytes);
    launch_copy_words(dst, (unsigned char*)w.mail_dev + MAIL_BYTES / 2, bytes, s);
    KNNSJ_CUDA(cudaStreamSynchronize(s));  // the mailbox is free again
    return;
  }
  KNNSJ_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  KNNSJ_CUDA(cudaStreamSynchronize(s));
}

namespace {

struct SmallDev {  // layout of Workspace::small
  uint32_t nonfinite;
  uint32_t fail_count;
  uint32_t work_counter;
  uint32_t defer_count;  // queries the tile search handed to search_kernel (current launch)
  unsigned long long C;
  unsigned long long cand;
  double avg[2];
  uint32_t hist[10000];
  double csum;
  double cpart[1024];
  FailRadii fr;
  LoopCtl ctl;
  uint32_t mlp_err;  // the tensor-core radius MLP timed out
  uint32_t chunk_fill[MAX_ROW_CHUNKS];  // streamed rows: queries placed per id block
  uint32_t patch_count;                 // streamed rows: first-pass failures
  unsigned long long defer_total;       // all queries handed over by the tile search in this join
};

template <typename T>
T host_fallback_eps(const std::vector<T>& mn, const std::vector<T>& mx, uint64_t n, uint32_t K) {
  double ext = 0.0;
  for (size_t j = 0; j < mn.size(); j++) ext = std::max(ext, (double)mx[j] - (double)mn[j]);
  if (!(ext > 0)) return (T)1;
  const double per_dim = std::max(1.0, std::floor(std::pow((double)n / K, 1.0 / mn.size())));
  return (T)(ext / per_dim);
}

}  // namespace

template <typename T>
static void build_grid(Workspace& w, const JoinConfig& cfg, uint64_t n, uint32_t d, uint32_t di,
                       const std::vector<T>& mn, const std::vector<T>& mx, T width, DeviceGrid<T>* out,
                       cudaStream_t s) {
  // generateNDGridDimensions (main.cu:2425-2488), in DTYPE.
  GridGeom<T> g{};
  g.di = di;
  g.width = width;
  unsigned long long mult = 1;
  bool overflow = false;
  for (uint32_t j = 0; j < di; j++) {
    const T lo = mn[j] - width;
    const T hi = mx[j] + width;
    const T cells = std::ceil((hi - lo) / width);
    if (!(cells < 4294967295.0)) throw StatusError{KNNSJ_ERR_UNSUPPORTED, "grid too fine"};
    g.minv[j] = lo;
    g.ncell[j] = (uint32_t)cells;
    if (g.ncell[j] == 0) g.ncell[j] = 1;
    g.mult[j] = mult;
    if (mult > ~0ull / g.ncell[j]) overflow = true;
    mult *= g.ncell[j];
  }
  if (overflow) throw StatusError{KNNSJ_ERR_UNSUPPORTED, "more than 2^64 grid cells"};
  g.total_cells = mult;
  int bits = 0;
  while (bits < 64 && ((mult - 1) >> bits) != 0) bits++;

  GridScratch sc;
  sc.keys[0] = (unsigned long long*)w.keys0.get(n * 8);
  sc.keys[1] = (unsigned long long*)w.keys1.get(n * 8);
  sc.vals[0] = (uint32_t*)w.vals0.get(n * 4);
  sc.vals[1] = (uint32_t*)w.vals1.get(n * 4);
  sc.hist_elems = radix_hist_elems(n);
  sc.hist = (uint32_t*)w.hist.get(sc.hist_elems * 4);
  sc.scan_tmp_elems = scan_tmp_elems(std::max<size_t>(sc.hist_elems, n + 1));
  sc.scan_tmp = (uint32_t*)w.scan_tmp.get(sc.scan_tmp_elems * 4);
  const T* xs = (const T*)w.xs.p;
  launch_cell_ids<T>(xs, n, g, sc.keys[0], sc.vals[0], s);
  const int cur = radix_sort_pairs(sc, n, bits, s);
  const unsigned long long* skeys = sc.keys[cur];
  const uint32_t* sids = sc.vals[cur];
  uint32_t* flags = (uint32_t*)w.flags.get(n * 4);
  uint32_t* pos = (uint32_t*)w.pos.get(n * 4);
  unsigned long long* ckeys = (unsigned long long*)w.ckeys.get(n * 8);
  uint32_t* coff = (uint32_t*)w.coff.get((n + 1) * 4);
  SmallDev* sm = (SmallDev*)w.small.p;
  launch_compact_cells(skeys, n, flags, pos, sc.scan_tmp, ckeys, coff, &sm->C, s);
  T* ps = (T*)w.ps.get(n * d * sizeof(T));
  float* psf = sizeof(T) == 8 ? (float*)w.psf.get(n * d * sizeof(float)) : nullptr;
  uint32_t* pid = (uint32_t*)w.pid.get(n * 4);
  dev_copy(w, pid, sids, n * 4, s);
  launch_gather_sorted<T>(xs, n, d, sids, ps, psf, s);
  unsigned long long C = 0;
  read_small(w, &C, &sm->C, sizeof(C), s);
  out->geom = g;
  out->ps = ps;
  out->psf = psf;
  out->pid = pid;
  out->ckeys = ckeys;
  out->coff = coff;
  out->C = C;
  const unsigned long long dense_limit =
      cfg.dense_cells_cap ? cfg.dense_cells_cap : std::max<unsigned long long>(4ull * n, 1ull << 24);
  out->dense = (cfg.dense_mode != 0) && (g.total_cells <= dense_limit) && g.total_cells < (1ull << 31);
  // (forced dense tables still respect an explicit cap: a fixed scratch array sets one)
  if (cfg.dense_mode == 2) out->dense = g.total_cells < (1ull << 31) && (!cfg.dense_cells_cap || g.total_cells <= dense_limit);
  out->dstart = nullptr;
  if (out->dense) {
    uint32_t* dstart = (uint32_t*)w.dstart.get((g.total_cells + 1) * 4);
    launch_dense_table(ckeys, coff, C, g.total_cells, dstart, s);
    out->dstart = dstart;
  }
}

// The radius a rebuilt grid is sized for when queries carry their own radii:
// the median grown radius of the failed queries (bin upper edge, at most the
// largest), so that most of them search small rings; the few with far larger
// radii search wider rings of the same grid.
__host__ __device__ inline double median_fail_radius(const uint32_t* hist, uint32_t nfail, const double* redge,
                                                     double rmax) {
  const uint32_t target = (nfail + 1) / 2;
  uint32_t cum = 0;
  for (int b = 0; b < FAIL_RADIUS_BINS; b++) {
    cum += hist[b];
    if (cum >= target) return redge[b] < rmax ? redge[b] : rmax;
  }
  return rmax;
}

namespace {

// One pass's bookkeeping inside the retry graph, mirroring the host loop of
// run_join: count the pass, swap the lists, grow the radius, and let the next
// pass run unless every query is done, a rebuild is due or the pass budget
// of this graph launch is spent (the loop always ends: iter grows by one per
// pass and stop_iter is finite).
template <typename T>
__global__ void loop_step_kernel(LoopCtl* c, const uint32_t* __restrict__ fail_count,
                                 const FailRadii* __restrict__ fr, cudaGraphConditionalHandle handle,
                                 int in_graph) {
  const uint32_t nfail = *fail_count;
  c->queries_run += c->nq;
  c->accepted += c->nq - nfail;
  c->iter++;
  c->cur ^= 1u;
  c->nq = nfail;
  if (nfail > 0) {
    if (c->per_query) {
      const unsigned long long b = fr->rmax_bits;
      c->rmax = sizeof(T) == 4 ? (double)__uint_as_float((uint32_t)b) : __longlong_as_double((long long)b);
      c->rgrid = median_fail_radius(fr->hist, nfail, c->redge, c->rmax);
    } else {
      c->r = (double)(T)__dadd_rn(c->r, c->step);  // main.cu:336
      c->rmax = c->r;
      c->rgrid = c->r;
    }
    c->rmax_seen = fmax(c->rmax_seen, c->rmax);
  }
  const bool regrid = regrid_due(c->rgrid, c->rmax, c->r_limit, c->width, c->ring_div);
  c->go = (nfail > 0 && c->iter < c->stop_iter && !regrid) ? 1 : 0;
  if (in_graph) cudaGraphSetConditional(handle, c->go ? 1u : 0u);
}

// First node of the retry graph: the loop runs while the loop state says so.
__global__ void loop_cond_kernel(const LoopCtl* c, cudaGraphConditionalHandle handle) {
  cudaGraphSetConditional(handle, c->go ? 1u : 0u);
}

// Streamed rows: the queries of each block of crow consecutive ids, in the
// cell order they have in pid, visited in `order` when given (nearby queries
// stay together), block c at
// lists[c * crow ...].  Lanes of a warp with the same block take consecutive
// slots from one atomic.
__global__ void chunk_lists_kernel(const uint32_t* __restrict__ pid, const uint32_t* __restrict__ order, uint32_t n,
                                   uint32_t crow, uint32_t* __restrict__ fill, uint32_t* __restrict__ lists) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool live = i < n;
  const uint32_t id = live ? pid[order ? order[i] : i] : 0u;
  const uint32_t c = live ? id / crow : 0xffffffffu;
  const unsigned peers = __match_any_sync(0xffffffffu, c);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (live && lane == leader) base = atomicAdd(&fill[c], (uint32_t)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (live) lists[(uint64_t)c * crow + base + __popc(peers & ((1u << lane) - 1u))] = id;
}

// Streamed rows: the first pass's failures (count on the device), kept for
// the patch after the lists are reused by later passes.
__global__ void save_fail_list_kernel(const uint32_t* __restrict__ src, const uint32_t* __restrict__ count,
                                      uint32_t* __restrict__ dst, uint32_t* __restrict__ saved) {
  const uint32_t nf = *count;
  if (blockIdx.x == 0 && threadIdx.x == 0) *saved = nf;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

// Streamed rows: rows finished after the first pass, copied from the device
// table into the host buffers (one warp per row).
template <typename T>
__global__ void patch_rows_kernel(const uint32_t* __restrict__ rows, const uint32_t* __restrict__ count,
                                  const int32_t* __restrict__ ids, const T* __restrict__ dists, uint32_t K,
                                  int32_t* h_ids, T* h_d) {
  const uint32_t nrows = *count;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t wid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; wid < nrows; wid += nwarps) {
    const uint64_t base = (uint64_t)rows[wid] * K;
    for (uint32_t j = lane; j < K; j += 32) {
      h_ids[base + j] = ids[base + j];
      h_d[base + j] = dists[base + j];
    }
  }
}

// Adds the tile search's hand-over count to the join's total and clears it
// for the next launch.
__global__ void defer_roll_kernel(uint32_t* __restrict__ count, unsigned long long* __restrict__ total) {
  *total += *count;
  *count = 0u;
}

}  // namespace

// Set-up of the tile search for the first pass: the order in which tiles
// take the queries (Hilbert or Morton order of their cells on a grid 16
// times finer than eps0, so that consecutive queries are close in every
// dimension) and
// the grid the candidates come from (a finer grid of width eps0 / f when its
// dense table fits).
template <typename T>
struct TileSetup {
  bool on = false;
  DeviceGrid<T> cand;                 // candidate grid
  const uint32_t* qorder = nullptr;   // positions of the eps0 grid's cell order, in tile order
  int fine = 1;                       // eps0 / candidate cell width
  bool per_query = false;             // search_kernel (one warp per query) on the candidate grid
};

template <typename T>
static void prepare_tile(Workspace& w, bool tiles, int fine_max, const DeviceGrid<T>& g, const T* xs, uint64_t n,
                         uint32_t d, T eps0, const std::vector<T>& mx, TileSetup<T>* t, cudaStream_t s) {
  const uint32_t di = g.geom.di;
  GridScratch sc;
  sc.hist_elems = radix_hist_elems(n);
  sc.scan_tmp_elems = scan_tmp_elems(std::max<size_t>(sc.hist_elems, n + 1));
  t->per_query = !tiles;
  if (tiles) {
  // 1. order of the points' cells along a space-filling curve (Hilbert in
  // two dimensions, Morton otherwise) on a grid 16 times finer than eps0
  // (stable: cell order within a cell), so that the few queries of a tile
  // lie close together, not anywhere in one eps0 cell: the union box of
  // their rings then stays near the size of one ring
  constexpr int ORDER_FINE = 16;
  GridGeom<T> gm = g.geom;
  gm.width = (T)((double)eps0 / ORDER_FINE);
  int bits = 1;
  for (uint32_t j = 0; j < di; j++)
    while (bits < 21 && (1ull << bits) < (unsigned long long)g.geom.ncell[j] * ORDER_FINE) bits++;
  sc.keys[0] = (unsigned long long*)w.keys0.get(n * 8);
  sc.keys[1] = (unsigned long long*)w.keys1.get(n * 8);
  sc.vals[0] = (uint32_t*)w.vals0.get(n * 4);
  sc.vals[1] = (uint32_t*)w.vals1.get(n * 4);
  sc.hist = (uint32_t*)w.hist.get(sc.hist_elems * 4);
  sc.scan_tmp = (uint32_t*)w.scan_tmp.get(sc.scan_tmp_elems * 4);
  launch_morton_keys<T>(g.ps, n, gm, bits, sc.keys[0], sc.vals[0], s);
  const int cur = radix_sort_pairs(sc, n, bits * (int)di, s);
  uint32_t* qorder = (uint32_t*)w.qorder.get(n * 4);
  dev_copy(w, qorder, sc.vals[cur], n * 4, s);
  t->qorder = qorder;
  }
  // 2. candidate grid: width eps0 / f, the largest f <= fine_max whose
  // dense table stays within max(8 n, 2^24) cells
  t->cand = g;
  t->fine = 1;
  const unsigned long long limit = std::max<unsigned long long>(8ull * n, 1ull << 24);
  for (int f = fine_max; f >= 2; f--) {
    GridGeom<T> gf = g.geom;
    gf.width = (T)((double)eps0 / (double)f);
    if (!(gf.width > 0)) continue;
    unsigned long long mult = 1;
    bool fits = true;
    for (uint32_t j = 0; j < di && fits; j++) {
      const T hi = mx[j] + eps0;
      const T cells = std::ceil((hi - gf.minv[j]) / gf.width);
      if (!(cells < 4294967295.0)) {
        fits = false;
        break;
      }
      gf.ncell[j] = std::max<uint32_t>((uint32_t)cells, 1u);
      gf.mult[j] = mult;
      if (mult > limit / gf.ncell[j]) fits = false;
      mult *= gf.ncell[j];
    }
    if (!fits || mult > limit) continue;
    gf.total_cells = mult;
    uint32_t* tbl = (uint32_t*)w.fdstart.get((mult + 1) * 4);
    uint32_t* tmp = (uint32_t*)w.scan_tmp.get(std::max(sc.scan_tmp_elems, scan_tmp_elems(mult)) * 4);
    T* fps = (T*)w.fps.get(n * d * sizeof(T));
    uint32_t* fpid = (uint32_t*)w.fpid.get(n * 4);
    // (points visited in eps0-cell order: neighbours fall in the same cells)
    launch_counting_grid<T>(g.ps, g.pid, n, d, gf, tbl, tmp, fps, fpid, s);
    t->cand.geom = gf;
    t->cand.ps = fps;
    t->cand.psf = nullptr;
    t->cand.pid = fpid;
    t->cand.ckeys = nullptr;
    t->cand.coff = nullptr;
    t->cand.C = 0;
    t->cand.dense = 1;
    t->cand.dstart = tbl;
    t->fine = f;
    break;
  }
  t->on = true;
}

// One search pass over the queries of a.qlist (or all points in cell order):
// the tile search where it is set up, then search_kernel over the queries it
// handed over, at the same radius on the eps0 grid; otherwise search_kernel
// alone.
template <typename T>
static void first_pass_search(Workspace& w, const SearchLaunch<T>& a, const TileSetup<T>& tile, SmallDev* sm,
                              cudaStream_t s) {
  if (tile.on && tile.per_query) {  // search_kernel over the finer candidate grid, queries in its cell order
    SearchLaunch<T> t = a;
    t.grid = tile.cand;
    launch_search<T>(t, w.sm_count, s);
    return;
  }
  if (tile.on) {
    uint32_t* defer = (uint32_t*)w.defer_list.get(a.n * 4);
    SearchLaunch<T> t = a;
    t.grid = tile.cand;
    t.qps = a.grid.ps;
    t.qpid = a.grid.pid;
    t.qorder = tile.qorder;
    launch_tile_search<T>(t, defer, &sm->defer_count, w.sm_count, s);
    SearchLaunch<T> b = a;
    b.qlist = defer;
    b.nq_dev = &sm->defer_count;
    launch_search<T>(b, w.sm_count, s);
    defer_roll_kernel<<<1, 1, 0, s>>>(&sm->defer_count, &sm->defer_total);
    KNNSJ_CHECK_LAUNCH();
    return;
  }
  launch_search<T>(a, w.sm_count, s);
}

// Steps 1-4 of the pipeline: dimension order, column transpose, eps0 and
// the grid index at eps0.
template <typename T>
struct Prepared {
  DeviceGrid<T> grid;
  T* xs = nullptr;
  T eps0 = 0;
  int bucket = -1;
  double avg = 0.0;
  double max_abs = 0.0;  // largest |coordinate| over all dimensions
  std::vector<T> mn, mx;
};

template <typename T>
static void prepare(Workspace& w, const JoinConfig& cfg, const T* d_aos, const T* h_aos, uint64_t n, uint32_t d,
                    uint32_t k, knnsj_stats* st, cudaStream_t s, Prepared<T>* P) {
  const uint32_t K = k + 1;
  const uint32_t di = cfg.num_indexed_dims;

  // 1. dimension order
  std::vector<uint32_t> perm(d);
  for (uint32_t j = 0; j < d; j++) perm[j] = j;
  if (!cfg.no_reorder) {
    const uint64_t ns = (n + 99) / 100;
    std::vector<T> sample(ns * d);
    if (h_aos) {
      for (uint64_t i = 0; i < ns; i++)
        std::memcpy(&sample[i * d], h_aos + i * 100 * d, d * sizeof(T));
    } else {
      KNNSJ_CUDA(cudaMemcpy2DAsync(sample.data(), d * sizeof(T), d_aos, 100 * d * sizeof(T),
                                   d * sizeof(T), ns, cudaMemcpyDeviceToHost, s));
      KNNSJ_CUDA(cudaStreamSynchronize(s));
    }
    reorder_from_sample<T>(sample.data(), ns, n, d, perm.data(), nullptr);
  }
  if (st)
    for (uint32_t j = 0; j < d && j < 64; j++) st->perm[j] = perm[j];

  // 2. transpose into column arrays
  uint32_t* d_perm = (uint32_t*)w.perm.get(d * 4);
  SmallDev* sm = (SmallDev*)w.small.get(sizeof(SmallDev));
  KNNSJ_CUDA(cudaMemsetAsync(sm, 0, offsetof(SmallDev, hist), s));
  launch_zero_words(&sm->defer_total, sizeof(sm->defer_total), s);
  KNNSJ_CUDA(cudaMemcpyAsync(d_perm, perm.data(), d * 4, cudaMemcpyHostToDevice, s));
  T* xs = (T*)w.xs.get(n * d * sizeof(T));
  launch_transpose_reorder<T>(d_aos, xs, n, d, d_perm, s, &sm->nonfinite);
  T* mm_part = (T*)w.minmax_part.get(1024 * 2 * d * sizeof(T) + 2 * d * sizeof(T));
  T* d_minmax = mm_part + 1024 * 2 * d;
  launch_minmax<T>(xs, n, d, d_minmax, mm_part, s);

  // 3. eps0 (GPU.cu:3088-3566)
  EpsScratch es;
  const uint64_t nthr = eps_avg_threads(n);
  es.partial = (double*)w.eps_partial.get(std::max<uint64_t>(nthr * eps_avg_chunks(n), 1) * 8);
  es.sample_sum = (double*)w.eps_sample.get(std::max<uint64_t>(nthr, 1) * 8);
  es.avg_out = sm->avg;
  es.hist = sm->hist;
  launch_eps_avg<T>(xs, n, d, es, s);
  KNNSJ_CUDA(cudaMemsetAsync(sm->hist, 0, sizeof(sm->hist), s));
  struct Head {
    uint32_t nonfinite, fail_count, work_counter, defer_count;
    unsigned long long C, cand;
    double avg[2];
  } head;
  std::vector<T> hmm(2 * d);
  KNNSJ_CUDA(cudaMemcpyAsync(hmm.data(), d_minmax, 2 * d * sizeof(T), cudaMemcpyDeviceToHost, s));
  KNNSJ_CUDA(cudaMemcpyAsync(&head, sm, sizeof(head), cudaMemcpyDeviceToHost, s));
  KNNSJ_CUDA(cudaStreamSynchronize(s));
  if (head.nonfinite) throw StatusError{KNNSJ_ERR_NONFINITE_INPUT, "NaN or infinite coordinate"};
  // float bracket error from rounding double coordinates to float
  double max_abs = 0.0;
  for (uint32_t j = 0; j < 2 * d; j++) max_abs = std::max(max_abs, std::fabs((double)hmm[j]));
  const double abs_err = sizeof(T) == 8 ? std::sqrt((double)d) * std::ldexp(max_abs, -22) : 0.0;
  P->max_abs = max_abs;
  // buckets [0, 256) first; the rest only if the crossing lies beyond
  std::vector<uint32_t> hh(10000, 0);
  const uint32_t first_range = 256;
  launch_eps_hist<T>(xs, n, d, es, 0, first_range, abs_err, s);
  KNNSJ_CUDA(cudaMemcpyAsync(hh.data(), sm->hist, first_range * 4, cudaMemcpyDeviceToHost, s));
  KNNSJ_CUDA(cudaStreamSynchronize(s));
  EpsChoice ec = choose_eps(hh.data(), first_range, head.avg[0], n, k, cfg.beta);
  if (!ec.complete) {
    launch_eps_hist<T>(xs, n, d, es, first_range, 10000, abs_err, s);
    KNNSJ_CUDA(cudaMemcpyAsync(hh.data(), sm->hist, 10000 * 4, cudaMemcpyDeviceToHost, s));
    KNNSJ_CUDA(cudaStreamSynchronize(s));
    ec = choose_eps(hh.data(), 10000, head.avg[0], n, k, cfg.beta);
  }
  T eps0 = (T)ec.eps;
  P->mn.assign(di, 0);
  P->mx.assign(di, 0);
  for (uint32_t j = 0; j < di; j++) {
    P->mn[j] = hmm[2 * j];
    P->mx[j] = hmm[2 * j + 1];
  }
  int bucket = ec.bucket;
  if (!(eps0 > 0) || !std::isfinite((double)eps0)) {
    // The reference divides by a zero epsilon here (N <= 1000 gives a zero
    // sampled mean); any positive width keeps the join exact.
    eps0 = host_fallback_eps<T>(P->mn, P->mx, n, K);
    bucket = -1;
  }
  P->eps0 = eps0;
  P->bucket = bucket;
  P->avg = head.avg[0];
  P->xs = xs;
  if (st) {
    st->eps0 = (double)eps0;
    st->eps_bucket = bucket;
    st->avg_distance = head.avg[0];
  }

  // 4. grid at eps0
  build_grid<T>(w, cfg, n, d, di, P->mn, P->mx, eps0, &P->grid, s);
  if (st) st->nonempty_cells = P->grid.C;
}

// The radius model used by the learned starting radius, uploaded to the
// device when it changed since the last call.
static const float* device_model(Workspace& w, cudaStream_t s) {
  std::vector<float> m;
  const unsigned v = radius_model_snapshot(&m);
  float* dm = (float*)w.model.get(MODEL_FLOATS * 4);
  if (w.model_version != v) {
    KNNSJ_CUDA(cudaMemcpyAsync(dm, m.data(), MODEL_FLOATS * 4, cudaMemcpyHostToDevice, s));
    KNNSJ_CUDA(cudaStreamSynchronize(s));
    w.model_version = v;
  }
  return dm;
}

template <typename T>
static double decode_radius(unsigned long long bits) {
  if (sizeof(T) == 4) {
    const uint32_t b = (uint32_t)bits;
    float f;
    std::memcpy(&f, &b, 4);
    return (double)f;
  }
  double x;
  std::memcpy(&x, &bits, 8);
  return x;
}

// Runs retry passes on the device: a CUDA graph whose conditional while node
// repeats [clear the pass counters, search, loop_step_kernel] until the step
// kernel stops it.  c holds the loop state on entry and is updated on return.
// Returns false, having run nothing, when conditional graph nodes are not
// available.
template <typename T>
static bool run_graph_passes(Workspace& w, SearchLaunch<T> a, LoopCtl& c, LoopCtl* dctl, SmallDev* sm,
                             int sm_count, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, double* kernel_ms,
                             bool upload = true, uint32_t iter_before = 0,
                             const std::function<void()>& after_launch = {}) {
  // launches are counted as they ran: the body's once per pass, the
  // condition node once
  if (upload) iter_before = c.iter;
  unsigned long long body = 0;
  cudaGraph_t g = nullptr;
  KNNSJ_CUDA(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) {
    cudaGetLastError();
    cudaGraphDestroy(g);
    return false;
  }
  // the loop state decides whether the first pass runs at all
  cudaGraphNode_t cond_node;
  {
    const LoopCtl* cp = dctl;
    void* args[] = {(void*)&cp, (void*)&h};
    cudaKernelNodeParams kp{};
    kp.func = (void*)loop_cond_kernel;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(1);
    kp.kernelParams = args;
    if (cudaGraphAddKernelNode(&cond_node, g, nullptr, 0, &kp) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphDestroy(g);
      return false;
    }
  }
  // (the parameter union has no default constructor: zeroed raw storage)
  alignas(cudaGraphNodeParams) unsigned char np_raw[sizeof(cudaGraphNodeParams)];
  std::memset(np_raw, 0, sizeof(np_raw));
  cudaGraphNodeParams* np = reinterpret_cast<cudaGraphNodeParams*>(np_raw);
  np->type = cudaGraphNodeTypeConditional;
  np->conditional.handle = h;
  np->conditional.type = cudaGraphCondTypeWhile;
  np->conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, &cond_node, nullptr, 1, np) != cudaSuccess) {
    cudaGetLastError();
    cudaGraphDestroy(g);
    return false;
  }
  cudaGraph_t body_graph = np->conditional.phGraph_out[0];
  cudaGraphExec_t ex = nullptr;
  try {
    if (upload) write_small(w, dctl, &c, sizeof(LoopCtl), s);
    const unsigned long long l0 = g_launches;
    KNNSJ_CUDA(cudaStreamBeginCaptureToGraph(s, body_graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    try {
      a.ctl = dctl;
      a.qlist = c.list[c.cur];  // placeholders: the kernel reads the live values from dctl
      a.fail_list = c.list[c.cur ^ 1];
      a.nq = c.nq;
      launch_zero_words(&sm->fail_count, 4, s);
      launch_zero_words(&sm->fr, sizeof(FailRadii), s);
      launch_search<T>(a, sm_count, s);
      loop_step_kernel<T><<<1, 1, 0, s>>>(dctl, &sm->fail_count, &sm->fr, h, 1);
      KNNSJ_CHECK_LAUNCH();
    } catch (...) {
      cudaGraph_t dummy = nullptr;
      cudaStreamEndCapture(s, &dummy);
      throw;
    }
    KNNSJ_CUDA(cudaStreamEndCapture(s, &body_graph));
    body = g_launches - l0;
    KNNSJ_CUDA(cudaGraphInstantiate(&ex, g, 0));
    KNNSJ_CUDA(cudaEventRecord(e0, s));
    KNNSJ_CUDA(cudaGraphLaunch(ex, s));
    KNNSJ_CUDA(cudaEventRecord(e1, s));
    if (after_launch) after_launch();  // device work that can precede the host's look at the state
    read_small(w, &c, dctl, sizeof(LoopCtl), s);
    const unsigned long long passes = c.iter - iter_before;
    g_launches = g_launches - body + body * passes + 1;
  } catch (...) {
    if (ex) cudaGraphExecDestroy(ex);
    cudaGraphDestroy(g);
    throw;
  }
  float ms = 0.f;
  KNNSJ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  *kernel_ms += ms;
  cudaGraphExecDestroy(ex);
  cudaGraphDestroy(g);
  return true;
}

template <typename T>
void run_join(Workspace& w, const JoinConfig& cfg, const T* d_aos, const T* h_aos, uint64_t n, uint32_t d,
              uint32_t k, int32_t* d_ids, T* d_dists, knnsj_stats* st, cudaStream_t s, RowStream* rows,
              double* rowsum) {
  const uint32_t K = k + 1;
  const uint32_t di = cfg.num_indexed_dims;
  cudaEvent_t* ev = w.ev;
  // a workspace without events (fixed-scratch calls) records no timings
  auto rec = [&](int i) {
    if (ev[i]) KNNSJ_CUDA(cudaEventRecord(ev[i], s));
  };
  auto elapsed = [&](int a, int b) -> float {
    float ms = 0.f;
    if (ev[a] && ev[b]) KNNSJ_CUDA(cudaEventElapsedTime(&ms, ev[a], ev[b]));
    return ms;
  };
  g_launches = 0;
  rec(0);
  Prepared<T> P;
  prepare<T>(w, cfg, d_aos, h_aos, n, d, k, st, s, &P);
  SmallDev* sm = (SmallDev*)w.small.p;
  rec(1);

  // 5. starting radii: eps0 for every query (plain), or one per query
  T* qrad = nullptr;
  double rmax = (double)P.eps0;
  if (cfg.radius_mode == KNNSJ_RADIUS_LEARNED) {
    qrad = (T*)w.qradius.get(n * sizeof(T));
    KNNSJ_CUDA(cudaMemsetAsync(&sm->mlp_err, 0, 4, s));
    launch_radius_assign<T>(P.grid, n, d, k, (float)cfg.beta, device_model(w, s), (double)P.eps0,
                            (float)cfg.radius_offset, qrad, &sm->mlp_err, w.sm_count, s);
    rmax = (double)P.eps0 * learned_max_cells(di);
  }
  // 5b. the first pass's tile search (2-D / 3-D float data, all indexed)
  TileSetup<T> tile;
  const bool will_stream = rows && rows->chunks >= 2 && n >= (uint64_t)rows->chunks;
  if (cfg.tile_search && tile_search_applies(d, di, K, P.grid.dense, sizeof(T))) {
    // per-query starting radii: query tiles over a grid of width eps0/4; a
    // uniform radius: one warp per query over a grid of width eps0/2
    // (measured best for each on the 25M-point sky-like set).  Streamed rows
    // search blocks of query ids, spread over the whole dataset: one warp
    // per query there.
    const bool tiles = !will_stream && (cfg.tile_search == 3 || (cfg.tile_search == 1 && qrad != nullptr));
    const int fine = cfg.tile_fine > 0 ? cfg.tile_fine : (tiles ? 4 : 2);
    prepare_tile<T>(w, tiles, fine, P.grid, P.xs, n, d, P.eps0, P.mx, &tile, s);
  }

  // 6. retry loop (main.cu:312-430)
  uint32_t* list[2] = {(uint32_t*)w.list0.get(n * 4), (uint32_t*)w.list1.get(n * 4)};
  SearchLaunch<T> a;
  a.grid = P.grid;
  a.xs = P.xs;
  a.n = n;
  a.d = d;
  a.K = K;
  a.out_ids = d_ids;
  a.out_d = d_dists;
  a.rowsum = rowsum;
  a.fail_count = &sm->fail_count;
  a.cand_count = &sm->cand;
  a.work_counter = &sm->work_counter;
  a.fail_radii = &sm->fr;
  a.qradius = qrad;
  a.shape.warps_per_block = cfg.search_warps;
  a.shape.qchunk = cfg.search_qchunk;
  a.shape.buffer = cfg.search_buffer;
  a.coord_bound = cfg.float_prefilter ? P.max_abs : INFINITY;
  T r = P.eps0;
  const double step = (double)P.eps0 * 0.5;
  a.step = (T)step;
  uint32_t nq = (uint32_t)n;
  int iter = 0, regrids = 0, cur = 0;
  uint64_t queries_run = 0;
  double kernel_ms = 0.0, alg_bytes = 0.0, rmax_seen = rmax;
  double rgrid = rmax;  // the radius a rebuilt grid is sized for
  double redge[FAIL_RADIUS_BINS];
  for (int b = 0; b < FAIL_RADIUS_BINS; b++) redge[b] = (double)P.eps0 * std::exp2((b - 15) / 4.0);
  const int max_iter = cfg.max_iterations > 0 ? cfg.max_iterations : 100000;
  double r_limit = regrid_limit((double)a.grid.geom.width, di);
  const double ring_div = ring_div_of(di);
  // passes after the first run inside a CUDA graph (no host round trip per
  // pass) unless the stream cannot be captured (the legacy default stream)
  bool graph_ok = cfg.use_graph && s != nullptr && ev[4] != nullptr && cfg.verbose < 2;
  LoopCtl* dctl = &sm->ctl;

  // 6a. streamed rows: the first pass in blocks of query ids, each block's
  // rows copied into the host buffers while the next block searches.  The
  // copies keep the host link busy, so the pass bookkeeping stays on the
  // device (the step kernel, then the retry graph) with no host round trip
  // until the graph stops.
  // (the caller waits for the copies and patches the late rows in:
  // finish_row_stream)
  const bool streamed = rows && rows->chunks >= 2 && n >= (uint64_t)rows->chunks;
  bool checksum_done = false;  // streamed rows: the checksum of the final table is launched
  if (streamed) {
    w.ensure_copy_stream();
    w.mail = true;
    rows->active = true;
    const int C = std::min(rows->chunks, MAX_ROW_CHUNKS);
    const uint32_t crow = (uint32_t)((n + C - 1) / C);
    uint32_t* clist = (uint32_t*)w.chunk_list.get(n * 4);
    const bool dev_loop = graph_ok;
    LoopCtl c{};
    c.nq = (uint32_t)n;
    c.iter = 0;
    c.cur = 0;
    c.stop_iter = (uint32_t)std::min<int64_t>((int64_t)max_iter, 256);
    c.list[0] = list[0];
    c.list[1] = list[1];
    c.r = (double)r;
    c.step = step;
    c.rmax = rmax;
    c.rgrid = rgrid;
    c.rmax_seen = rmax_seen;
    for (int b = 0; b < FAIL_RADIUS_BINS; b++) c.redge[b] = redge[b];
    c.r_limit = r_limit;
    c.width = (double)a.grid.geom.width;
    c.per_query = qrad ? 1 : 0;
    c.ring_div = ring_div;
    c.go = 0;
    if (dev_loop) write_small(w, dctl, &c, sizeof(LoopCtl), s);
    launch_zero_words(sm->chunk_fill, sizeof(sm->chunk_fill), s);
    chunk_lists_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a.grid.pid, nullptr, (uint32_t)n, crow,
                                                                   sm->chunk_fill, clist);
    KNNSJ_CHECK_LAUNCH();
    launch_zero_words(&sm->fail_count, 4, s);
    launch_zero_words(&sm->fr, sizeof(FailRadii), s);
    a.radius = r;
    a.fail_list = list[1];
    KNNSJ_CUDA(cudaEventRecord(ev[6], s));
    for (int ch = 0; ch < C; ch++) {
      const uint64_t r0 = (uint64_t)ch * crow;
      if (r0 >= n) break;
      const uint64_t nr = std::min<uint64_t>(crow, n - r0);
      a.qlist = clist + r0;
      a.nq = (uint32_t)nr;
      // (the queries of a block of ids are spread over the whole dataset:
      // the per-query search, over the finer grid when one is set up)
      SearchLaunch<T> c = a;
      if (tile.on) c.grid = tile.cand;
      launch_search<T>(c, w.sm_count, s);
      KNNSJ_CUDA(cudaEventRecord(w.chunk_ev[ch], s));
      KNNSJ_CUDA(cudaStreamWaitEvent(w.copy_stream, w.chunk_ev[ch], 0));
      KNNSJ_CUDA(cudaMemcpyAsync((int32_t*)rows->ids_host + r0 * K, d_ids + r0 * K, nr * K * 4,
                                 cudaMemcpyDeviceToHost, w.copy_stream));
      KNNSJ_CUDA(cudaMemcpyAsync((T*)rows->d_host + r0 * K, d_dists + r0 * K, nr * K * sizeof(T),
                                 cudaMemcpyDeviceToHost, w.copy_stream));
    }
    KNNSJ_CUDA(cudaEventRecord(ev[7], s));
    // the block lists are spent: they keep the failures for the patch
    save_fail_list_kernel<<<(unsigned)(w.sm_count * 4), 256, 0, s>>>(list[1], &sm->fail_count, clist,
                                                                    &sm->patch_count);
    KNNSJ_CHECK_LAUNCH();
    alg_bytes += (double)n * d * sizeof(T);  // the pass's candidate columns; the rest is counted below
    bool ran = false;
    if (dev_loop) {
      loop_step_kernel<T><<<1, 1, 0, s>>>(dctl, &sm->fail_count, &sm->fr, 0, 0);
      KNNSJ_CHECK_LAUNCH();
      // the result checksum goes right behind the graph: if the graph
      // finishes the join, it overlaps the row copies (the host's read of the
      // loop state waits behind them)
      auto early_checksum = [&]() {
        if (rows->checksum) {
          launch_checksum<T>(d_dists, n * K, sm->cpart, &sm->csum, s);
          checksum_done = true;
        }
      };
      ran = run_graph_passes<T>(w, a, c, dctl, sm, w.sm_count, s, ev[4], ev[5], &kernel_ms, false, 1,
                                early_checksum);
      if (ran) {
        const int passes = (int)c.iter - 1;
        alg_bytes += (double)passes * n * d * sizeof(T);
      } else {
        graph_ok = false;
        read_small(w, &c, dctl, sizeof(LoopCtl), s);
      }
    } else {  // host bookkeeping, as after any host-driven pass
      uint32_t nfail = 0;
      FailRadii fr{};
      read_small(w, &nfail, &sm->fail_count, 4, s);
      if (qrad) read_small(w, &fr, &sm->fr, sizeof(FailRadii), s);
      c.queries_run = n;
      c.accepted = n - nfail;
      c.nq = nfail;
      c.iter = 1;
      c.cur = 1;
      if (nfail > 0) {
        if (qrad) {
          c.rmax = decode_radius<T>(fr.rmax_bits);
          c.rgrid = median_fail_radius(fr.hist, nfail, redge, c.rmax);
        } else {
          c.r = (double)(T)((double)r + step);  // main.cu:336
          c.rmax = c.r;
          c.rgrid = c.rmax;
        }
        c.rmax_seen = std::max(c.rmax_seen, c.rmax);
      }
    }
    float first_ms = 0.f;
    KNNSJ_CUDA(cudaEventSynchronize(ev[7]));
    KNNSJ_CUDA(cudaEventElapsedTime(&first_ms, ev[6], ev[7]));
    kernel_ms += first_ms;
    alg_bytes += (double)c.queries_run * d * sizeof(T) + (double)c.accepted * K * (4.0 + sizeof(T));
    queries_run += c.queries_run;
    iter = (int)c.iter;
    cur = (int)c.cur;
    nq = c.nq;
    r = (T)c.r;
    rmax = c.rmax;
    rgrid = c.rgrid;
    rmax_seen = c.rmax_seen;
  }

  while (nq > 0) {
    checksum_done = false;  // more passes change the table
    if (iter >= max_iter) throw StatusError{KNNSJ_ERR_NO_CONVERGENCE, "iteration cap reached"};
    // learned starting radii are clamped so their rings stay small on the
    // eps0 grid: no rebuild for the first pass
    const bool first_learned = qrad && iter == 0;
    if (!first_learned && regrid_due(rgrid, rmax, r_limit, (double)a.grid.geom.width, ring_div)) {
      // sparse-query tail: when the largest radius has outgrown the grid
      // (its ring would pass the row cap) and only a handful of queries are
      // left (nq * n <= 2^32 distances), they are finished exactly by a scan
      // over all points instead of a grid coarse enough for that radius
      // (tail_brute 2, for tests: at any due rebuild)
      const bool outgrown = ring_too_wide(rmax, (double)a.grid.geom.width, ring_div) || cfg.tail_brute == 2;
      if (cfg.tail_brute && outgrown && nq <= 4096 && (uint64_t)nq * n <= (1ull << 32)) {
        a.qlist = list[cur];
        a.nq = nq;
        rec(4);
        launch_brute<T>(a, s);
        rec(5);
        KNNSJ_CUDA(cudaStreamSynchronize(s));
        kernel_ms += elapsed(4, 5);
        alg_bytes += (double)nq * n * d * sizeof(T) + (double)nq * K * (4.0 + sizeof(T));
        queries_run += nq;
        iter++;
        nq = 0;
        break;
      }
      // coarser grid for the radius in flight (like main.cu:333-356); the
      // widened width keeps that radius's ring at three cells per dimension
      const T wnew = (T)(rgrid * (1.0 + 1.0 / 32768.0));
      build_grid<T>(w, cfg, n, d, di, P.mn, P.mx, wnew, &a.grid, s);
      r_limit = regrid_limit((double)a.grid.geom.width, di);
      regrids++;
    }
    if (graph_ok && iter >= 1) {
      LoopCtl c{};
      c.nq = nq;
      c.iter = (uint32_t)iter;
      c.cur = (uint32_t)cur;
      c.stop_iter = (uint32_t)std::min<int64_t>((int64_t)max_iter, (int64_t)iter + 256);
      c.list[0] = list[0];
      c.list[1] = list[1];
      c.r = (double)r;
      c.step = step;
      c.rmax = rmax;
      c.rgrid = rgrid;
      c.rmax_seen = rmax_seen;
      for (int b = 0; b < FAIL_RADIUS_BINS; b++) c.redge[b] = redge[b];
      c.r_limit = r_limit;
      c.width = (double)a.grid.geom.width;
      c.per_query = qrad ? 1 : 0;
      c.ring_div = ring_div;
      c.go = 1;
      if (run_graph_passes<T>(w, a, c, dctl, sm, w.sm_count, s, ev[4], ev[5], &kernel_ms)) {
        const int passes = (int)c.iter - iter;
        alg_bytes += (double)passes * n * d * sizeof(T) + (double)c.queries_run * d * sizeof(T) +
                     (double)c.accepted * K * (4.0 + sizeof(T));
        queries_run += c.queries_run;
        iter = (int)c.iter;
        cur = (int)c.cur;
        nq = c.nq;
        r = (T)c.r;
        rmax = c.rmax;
        rgrid = c.rgrid;
        rmax_seen = c.rmax_seen;
        continue;
      }
      graph_ok = false;  // conditional graphs unavailable: host-driven passes
    }
    a.qlist = iter == 0 ? nullptr : list[cur];
    a.nq = nq;
    a.radius = r;
    a.fail_list = list[cur ^ 1];
    launch_zero_words(&sm->fail_count, 4, s);
    launch_zero_words(&sm->fr, sizeof(FailRadii), s);
    rec(4);
    if (iter == 0)
      first_pass_search<T>(w, a, tile, sm, s);
    else
      launch_search<T>(a, w.sm_count, s);
    rec(5);
    struct {
      uint32_t fail;
      uint32_t pad;
      FailRadii fr;
    } tail;
    read_small(w, &tail.fail, &sm->fail_count, 4, s);
    if (qrad) read_small(w, &tail.fr, &sm->fr, sizeof(FailRadii), s);
    const uint32_t nfail = tail.fail;
    const float pass_ms = elapsed(4, 5);
    kernel_ms += pass_ms;
    if (cfg.verbose >= 2) {  // one line per pass
      unsigned long long cand_now = 0;
      KNNSJ_CUDA(cudaMemcpy(&cand_now, &sm->cand, 8, cudaMemcpyDeviceToHost));
      fprintf(stderr, "knnsj: pass %d: %u queries, %u failed, radius %g (largest %g), grid width %g, %.3f ms, "
              "candidates so far %llu\n", iter, nq, nfail, (double)r, rmax, (double)a.grid.geom.width, pass_ms,
              cand_now);
    }
    // candidate columns read once, query rows read, accepted rows written
    alg_bytes += (double)n * d * sizeof(T) + (double)nq * d * sizeof(T) +
                 (double)(nq - nfail) * K * (4.0 + sizeof(T));
    queries_run += nq;
    nq = nfail;
    cur ^= 1;
    iter++;
    if (nq > 0) {
      if (qrad) {
        rmax = decode_radius<T>(tail.fr.rmax_bits);  // largest grown radius among the failures
        rgrid = median_fail_radius(tail.fr.hist, nfail, redge, rmax);
      } else {
        r = (T)((double)r + step);  // main.cu:336
        rmax = (double)r;
        rgrid = rmax;
      }
      rmax_seen = std::max(rmax_seen, rmax);
    }
  }
  rec(2);
  if (streamed) {
    // the result checksum runs while the last row copies are in flight; the
    // wait for them and the late rows follow, and the small reads below come
    // after the copies instead of queueing behind them
    if (rows->checksum && !checksum_done) launch_checksum<T>(d_dists, n * K, sm->cpart, &sm->csum, s);
    finish_row_stream<T>(w, *rows, d_ids, d_dists, K, s);
    rec(3);
    w.mail = false;
    if (rows->checksum) read_small(w, &rows->total_distance, &sm->csum, sizeof(double), s);
  }
  if (rowsum && st) {
    launch_sum_f64(rowsum, n, sm->cpart, &sm->csum, s);
    read_small(w, &st->total_distance, &sm->csum, sizeof(double), s);
  }
  unsigned long long cand = 0, deferred = 0;
  uint32_t mlp_err = 0;
  read_small(w, &cand, &sm->cand, 8, s);
  read_small(w, &deferred, &sm->defer_total, 8, s);
  if (qrad) read_small(w, &mlp_err, &sm->mlp_err, 4, s);
  if (mlp_err && cfg.verbose)  // rows are still exact: the affected queries started at eps0
    fprintf(stderr, "knnsj: the tensor-core radius model timed out (%u); those queries started at eps0\n", mlp_err);
  if (st) {
    st->iterations = iter;
    st->regrids = regrids;
    st->eps_final = qrad ? rmax_seen : (double)r;
    st->candidates = cand;
    st->queries_run = queries_run;
    st->kernel_launches = g_launches;
    st->ms_search_kernels = kernel_ms;
    st->search_alg_bytes = alg_bytes;
    st->search_alg_flops = 3.0 * d * (double)cand;
    st->radius_model_error = (double)mlp_err;
    st->tile_handovers = (double)deferred;
    const float a01 = elapsed(0, 1), a12 = elapsed(1, 2);
    st->ms_prep = a01;
    st->ms_search = a12;
    st->ms_total = a01 + a12;
    if (streamed) st->ms_transfer = elapsed(2, 3);  // the row copies that outlast the join
  }
}

// Features of the learned starting radius for every point (by input row),
// on the eps0 grid of a (plain) join of the same data and k.
template <typename T>
void run_features(Workspace& w, const JoinConfig& cfg, const T* d_aos, const T* h_aos, uint64_t n, uint32_t d,
                  uint32_t k, float* d_out, double* eps0_out, cudaStream_t s) {
  g_launches = 0;
  Prepared<T> P;
  prepare<T>(w, cfg, d_aos, h_aos, n, d, k, nullptr, s, &P);
  launch_radius_features<T>(P.grid, n, d, k, (float)cfg.beta, d_out, s);
  KNNSJ_CUDA(cudaStreamSynchronize(s));
  if (eps0_out) *eps0_out = (double)P.eps0;
}

template <typename T>
double device_checksum(Workspace& w, const T* d_vals, uint64_t count, cudaStream_t s) {
  SmallDev* sm = (SmallDev*)w.small.get(sizeof(SmallDev));
  launch_checksum<T>(d_vals, count, sm->cpart, &sm->csum, s);
  double v = 0.0;
  read_small(w, &v, &sm->csum, sizeof(v), s);
  return v;
}
template double device_checksum<float>(Workspace&, const float*, uint64_t, cudaStream_t);
template double device_checksum<double>(Workspace&, const double*, uint64_t, cudaStream_t);

// Streamed rows: waits (on s) for every block copy, then writes the rows
// that passes after the first finished into the host buffers.  The caller
// synchronises s.
template <typename T>
void finish_row_stream(Workspace& w, const RowStream& rows, const int32_t* d_ids, const T* d_dists, uint32_t K,
                       cudaStream_t s) {
  SmallDev* sm = (SmallDev*)w.small.p;
  KNNSJ_CUDA(cudaEventRecord(w.chunk_ev[MAX_ROW_CHUNKS], w.copy_stream));
  KNNSJ_CUDA(cudaStreamWaitEvent(s, w.chunk_ev[MAX_ROW_CHUNKS], 0));
  patch_rows_kernel<T><<<(unsigned)(w.sm_count * 8), 256, 0, s>>>((const uint32_t*)w.chunk_list.p, &sm->patch_count,
                                                                  d_ids, d_dists, K, (int32_t*)rows.ids_dev,
                                                                  (T*)rows.d_dev);
  KNNSJ_CHECK_LAUNCH();
}

template void finish_row_stream<float>(Workspace&, const RowStream&, const int32_t*, const float*, uint32_t,
                                       cudaStream_t);
template void finish_row_stream<double>(Workspace&, const RowStream&, const int32_t*, const double*, uint32_t,
                                        cudaStream_t);

template void run_join<float>(Workspace&, const JoinConfig&, const float*, const float*, uint64_t, uint32_t,
                              uint32_t, int32_t*, float*, knnsj_stats*, cudaStream_t, RowStream*, double*);
template void run_join<double>(Workspace&, const JoinConfig&, const double*, const double*, uint64_t,
                               uint32_t, uint32_t, int32_t*, double*, knnsj_stats*, cudaStream_t,
                               RowStream*, double*);
template void run_features<float>(Workspace&, const JoinConfig&, const float*, const float*, uint64_t, uint32_t,
                                  uint32_t, float*, double*, cudaStream_t);
template void run_features<double>(Workspace&, const JoinConfig&, const double*, const double*, uint64_t,
                                   uint32_t, uint32_t, float*, double*, cudaStream_t);

}  // namespace knnsj
