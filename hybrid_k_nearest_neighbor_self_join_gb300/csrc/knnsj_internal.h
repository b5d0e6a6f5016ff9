// knnsj_internal.h -- host-side declarations shared by the library's
// translation units (kernel launchers, pipeline, host I/O).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>
#include <vector>

#include "../../include/knnsj.h"
#include "knnsj_device.cuh"

namespace knnsj {

// ---- error plumbing ------------------------------------------------------
struct CudaError {
  cudaError_t err;
  const char* where;
};

#define KNNSJ_CUDA(call)                                                   \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) throw ::knnsj::CudaError{e_, #call};            \
  } while (0)

struct StatusError {
  knnsj_status st;
  const char* what;
};

// Kernel launches of this host thread since the last reset (reported in
// knnsj_stats; batched joins run sets on several host threads).
extern thread_local unsigned long long g_launches;
// Set while a fixed-scratch join runs on this thread: any cudaMalloc-backed
// buffer, pinned host buffer or stream creation then fails with
// KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH instead of allocating.
extern thread_local bool g_forbid_alloc;
#define KNNSJ_CHECK_LAUNCH()                 \
  do {                                       \
    KNNSJ_CUDA(cudaGetLastError());          \
    ++::knnsj::g_launches;                   \
  } while (0)

// ---- device buffers of one join (cached across calls, grow-only) --------
// A fixed device region carved out by bump allocation (no cudaMalloc).
struct Arena {
  unsigned char* base = nullptr;
  size_t cap = 0;
  size_t used = 0;
  void* take(size_t bytes);  // 256-byte aligned; throws when the region is full
};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  Arena* arena = nullptr;  // non-null: carve from the arena instead of cudaMalloc
  void* get(size_t need);  // grows (contents not kept)
  void release();
};

// Grid index on the device, in cell order.
template <typename T>
struct DeviceGrid {
  GridGeom<T> geom;
  const T* ps = nullptr;                  // SoA coords in cell order: d x n
  const float* psf = nullptr;             // the same rounded to float (double data only)
  const uint32_t* pid = nullptr;          // original id of each sorted position
  const unsigned long long* ckeys = nullptr;  // sorted non-empty cell ids [C]
  const uint32_t* coff = nullptr;         // first sorted position of each cell [C+1]
  const uint32_t* dstart = nullptr;       // dense: first position of cell L [total+1]
  unsigned long long C = 0;
  int dense = 0;
};

// ---- kernel launchers (k_*.cu) -------------------------------------------
template <typename T>
void launch_transpose_reorder(const T* aos, T* soa, uint64_t n, uint32_t d, const uint32_t* d_perm,
                              cudaStream_t s, uint32_t* d_nonfinite);
template <typename T>
void launch_minmax(const T* soa, uint64_t n, uint32_t di, T* d_minmax /*2*di*/, T* scratch /*1024*2*di*/,
                   cudaStream_t s);

struct EpsScratch {
  double* partial = nullptr;     // [eps_avg_threads * eps_avg_chunks]
  double* sample_sum = nullptr;  // [eps_avg_threads]
  double* avg_out = nullptr;     // [2]: mean distance, pair count
  uint32_t* hist = nullptr;      // [10000]
};
uint64_t eps_avg_threads(uint64_t n);
uint32_t eps_avg_chunks(uint64_t n);
uint32_t eps_sample_offset(uint64_t n);
template <typename T>
void launch_eps_avg(const T* soa, uint64_t n, uint32_t d, const EpsScratch& sc, cudaStream_t s);
template <typename T>
void launch_eps_hist(const T* soa, uint64_t n, uint32_t d, const EpsScratch& sc, uint32_t b_lo, uint32_t b_hi,
                     double abs_err, cudaStream_t s);
// Sum of squared result distances (the reference's verification figure,
// GPU.cu:3690-3693) in a fixed order; result in *d_out.
template <typename T>
void launch_checksum(const T* dists, uint64_t count, double* d_partial, double* d_out, cudaStream_t s);
// Sum of count doubles (the per-row verification sums) in a fixed order.
void launch_sum_f64(const double* v, uint64_t count, double* d_partial, double* d_out, cudaStream_t s);

struct GridScratch {
  unsigned long long* keys[2] = {nullptr, nullptr};
  uint32_t* vals[2] = {nullptr, nullptr};
  uint32_t* hist = nullptr;   // radix tile histograms
  uint32_t* scan_tmp = nullptr;
  uint32_t* flags = nullptr;
  size_t hist_elems = 0;
  size_t scan_tmp_elems = 0;
};
size_t radix_hist_elems(uint64_t n);
size_t scan_tmp_elems(size_t n);
void scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp, cudaStream_t s);

template <typename T>
void launch_cell_ids(const T* soa, uint64_t n, const GridGeom<T>& g, unsigned long long* keys,
                     uint32_t* vals, cudaStream_t s);
// Stable LSD radix sort of (key, value) by the low `bits` bits of key.
// Returns the index (0/1) of the buffers holding the result.
int radix_sort_pairs(GridScratch& sc, uint64_t n, int bits, cudaStream_t s);
// Non-empty cell table from sorted keys; writes C to *d_C.
void launch_compact_cells(const unsigned long long* skeys, uint64_t n, uint32_t* flags,
                          uint32_t* pos, uint32_t* scan_tmp, unsigned long long* ckeys,
                          uint32_t* coff, unsigned long long* d_C, cudaStream_t s);
void launch_dense_table(const unsigned long long* ckeys, const uint32_t* coff,
                        unsigned long long C, unsigned long long total_cells, uint32_t* dstart,
                        cudaStream_t s);
// Morton (Z-order) codes of the cells of points given in cell-ordered
// columns ps (keys) and their positions (vals), `bits` bits per dimension.
template <typename T>
void launch_morton_keys(const T* ps, uint64_t n, const GridGeom<T>& g, int bits, unsigned long long* keys,
                        uint32_t* vals, cudaStream_t s);
// Grid by counting sort (points in any order within a cell): tbl (total+1
// entries) becomes the dense start table, ps/pid the cell-ordered columns and
// ids of the points given as columns src with ids src_ids (null: 0, 1, ...).
// scan_tmp: scan_tmp_elems(total).
template <typename T>
void launch_counting_grid(const T* src, const uint32_t* src_ids, uint64_t n, uint32_t d, const GridGeom<T>& g,
                          uint32_t* tbl, uint32_t* scan_tmp, T* ps, uint32_t* pid, cudaStream_t s);
template <typename T>
// psf (optional): the same columns rounded to float (double data: the
// search's float prefilter)
void launch_gather_sorted(const T* soa, uint64_t n, uint32_t d, const uint32_t* sorted_ids, T* ps, float* psf,
                          cudaStream_t s);

// ---- range search with fused top-K --------------------------------------
// State of the retry loop in device memory, for passes that run inside a
// CUDA graph (a conditional while node): the search kernel reads the pass's
// query count, lists and radius from here, and a one-thread step kernel
// advances it and decides whether another pass runs.
struct LoopCtl {
  uint32_t nq;         // queries of the next pass
  uint32_t iter;       // passes done
  uint32_t cur;        // list[cur] holds the next pass's queries
  uint32_t stop_iter;  // the graph stops before this pass
  uint32_t* list[2];
  double r;            // uniform radius (a value of the data type)
  double step;         // radius growth per pass
  double rmax;         // largest radius the next pass searches
  double rmax_seen;    // largest radius of any pass
  double rgrid;        // radius the grid must suit (plain: r; per-query: median failing radius)
  double r_limit;      // a grid rebuild is due when rgrid > r_limit and rgrid > width
  double width;
  unsigned long long queries_run;
  unsigned long long accepted;
  int per_query;       // per-query radii (learned starting radius)
  int go;              // the next pass runs (set by each pass's step)
  double ring_div;     // radii above width * ring_div / 2 force a rebuild (0: none)
  double redge[64];    // upper radius of each bin of the failing-radius histogram
};

// Grown radii of the queries that failed a pass (per-query radius mode):
// their largest value and a histogram in quarter octaves of eps0, bin
// floor(4 log2(r / eps0)) + 16 clamped to [0, 63].
struct FailRadii {
  unsigned long long rmax_bits;
  uint32_t hist[64];
};
constexpr int FAIL_RADIUS_BINS = 64;

// Launch shape of the search kernel; 0 = the default.
struct SearchShape {
  int warps_per_block = 0;  // 2..8
  int qchunk = 0;           // queries a warp takes per work fetch
  int buffer = 0;           // selection buffer capacity (power of two >= K+32)
};
template <typename T>
struct SearchLaunch {
  DeviceGrid<T> grid;
  const T* xs = nullptr;            // SoA coords in input order (failed queries)
  uint64_t n = 0;
  uint32_t d = 0;
  uint32_t K = 0;
  const uint32_t* qlist = nullptr;  // original ids; nullptr = all, in cell order
  uint32_t nq = 0;
  T radius = 0;                     // uniform radius (qradius == nullptr)
  T* qradius = nullptr;             // per-query radius by original id
  T step = 0;                       // radius growth written back on failure
  int32_t* out_ids = nullptr;
  T* out_d = nullptr;
  double* rowsum = nullptr;                 // per-row verification sums, by id (nullptr: none)
  uint32_t* fail_list = nullptr;
  uint32_t* fail_count = nullptr;
  unsigned long long* cand_count = nullptr;
  uint32_t* work_counter = nullptr;
  FailRadii* fail_radii = nullptr;          // grown radii of the failures (per-query radii)
  double coord_bound = 0.0;                 // largest |coordinate|: enables the float prefilter when finite
  SearchShape shape;                        // launch shape (autotuned for batched joins)
  const LoopCtl* ctl = nullptr;             // non-null: nq, lists and radius come from here (graph passes)
  const uint32_t* nq_dev = nullptr;         // non-null: the pass's query count is read here (nq is a bound)
  // tile search only: queries from these cell-ordered columns and ids (when
  // the candidates come from another grid), visited in qorder
  const T* qps = nullptr;
  const uint32_t* qpid = nullptr;
  const uint32_t* qorder = nullptr;
};
template <typename T>
void launch_search(const SearchLaunch<T>& a, int sm_count, cudaStream_t s);
// Tile search (k_tile.cu): the first pass of float data with two or three
// dimensions, all indexed, K <= 65 and a dense cell table.  Queries it hands
// over (ring far wider than its tile's, exact ties at the K-th distance) are
// appended to defer_list / *defer_count for search_kernel at the same radius.
bool tile_search_applies(uint32_t d, uint32_t di, uint32_t K, int dense, size_t elem);
template <typename T>
void launch_tile_search(const SearchLaunch<T>& a, uint32_t* defer_list, uint32_t* defer_count, int sm_count,
                        cudaStream_t s);
// Clears bytes (a multiple of 4) with a kernel: unlike a runtime memset it
// never waits behind copies in flight on another stream.
void launch_zero_words(void* p, size_t bytes, cudaStream_t s);
void launch_copy_to_mapped(void* dst, const void* src, size_t bytes, int sm_count, cudaStream_t s);
int search_buffer_capacity(uint32_t K);
// Exact rows of the queries a.qlist[0..a.nq) by a scan over all points.
template <typename T>
void launch_brute(const SearchLaunch<T>& a, cudaStream_t s);

// Rows delivered to host buffers while the join runs (host-pointer calls
// whose output buffers are pinned): the first pass runs in chunks of query
// ids, each chunk's block of rows is copied out on a second stream as soon as
// its search is done, and the rows that later passes finish are written into
// the host buffers by a kernel at the end, after every chunk copy.
constexpr int MAX_ROW_CHUNKS = 32;
constexpr size_t MAIL_BYTES = 4096;  // mailbox: reads in the first half, writes in the second
struct RowStream {
  void* ids_host = nullptr;  // the host buffers
  void* d_host = nullptr;
  void* ids_dev = nullptr;   // their device-accessible addresses
  void* d_dev = nullptr;
  int chunks = 0;            // blocks of query ids in the first pass (>= 2)
  bool checksum = false;     // also compute the result's verification sum
  bool active = false;       // set by run_join when it streamed (rows complete on return)
  double total_distance = 0.0;
};

// ---- per-device workspace --------------------------------------------------
struct Workspace {
  DevBuf model;                          // radius model (learned starting radius)
  unsigned model_version = 0;
  DevBuf in, ids, dists;                 // staging for host-pointer calls
  DevBuf xs, ps, psf, pid;               // input-order columns, cell-order columns (+ float copy), ids
  DevBuf keys0, keys1, vals0, vals1, hist, scan_tmp, flags, pos;  // grid build
  DevBuf ckeys, coff, dstart;            // cell tables
  DevBuf list0, list1, small, eps_partial, eps_sample, perm, minmax_part, qradius;
  DevBuf chunk_list, patch_rows;         // streamed rows: queries by id block, rows finished late
  DevBuf defer_list;                     // queries the tile search hands to search_kernel
  DevBuf rowsum;                         // per-row verification sums (host-pointer calls)
  DevBuf fps, fpid, fdstart;             // tile search: the finer candidate grid (columns, ids, start table)
  DevBuf qorder;                         // tile search: cell-ordered positions in Morton order of their cells
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  cudaStream_t copy_stream = nullptr;    // streamed rows: device-to-host copies
  cudaEvent_t chunk_ev[MAX_ROW_CHUNKS + 1] = {};
  // While rows stream out, the copy engines are busy for tens of ms: the
  // join's small reads and writes of host memory then go through the mailbox
  // (mapped pinned memory that kernels read and write), device copies run on
  // the SMs, and none of them queues behind the row copies.
  void* mail_host = nullptr;
  void* mail_dev = nullptr;
  bool mail = false;
  int sm_count = 0;
  void* h_pinned = nullptr;
  size_t h_pinned_bytes = 0;
  void ensure_stream();
  void ensure_copy_stream();  // and the mailbox
  void* pinned(size_t need);
  void pinned_release();
  void release_all();
  void attach_arena(Arena* a);  // every buffer carves from `a` from now on
};
Workspace& workspace(int device);

struct JoinConfig;
// Full join of n x d row-major data already on the device.  h_aos (optional)
// is the same data on the host, used for the dimension-order sample.
// rowsum (optional, n doubles): each result row's verification sum, and
// st->total_distance their sum.  d_ids / d_dists may be device-mapped host
// memory: the kernels then write the rows straight into the host buffers.
template <typename T>
void run_join(Workspace& w, const JoinConfig& cfg, const T* d_aos, const T* h_aos, uint64_t n, uint32_t d,
              uint32_t k, int32_t* d_ids, T* d_dists, knnsj_stats* st, cudaStream_t s,
              RowStream* rows = nullptr, double* rowsum = nullptr);
template <typename T>
void finish_row_stream(Workspace& w, const RowStream& rows, const int32_t* d_ids, const T* d_dists, uint32_t K,
                       cudaStream_t s);
template <typename T>
void run_features(Workspace& w, const JoinConfig& cfg, const T* d_aos, const T* h_aos, uint64_t n, uint32_t d,
                  uint32_t k, float* d_out, double* eps0_out, cudaStream_t s);

// ---- learned starting radius (k_radius.cu, k_mlp.cu) -----------------------
double learned_max_cells(uint32_t di);
template <typename T>
void launch_radius_assign(const DeviceGrid<T>& g, uint64_t n, uint32_t d, uint32_t k, float beta,
                          const float* d_model, double eps0, float offset, T* qradius, uint32_t* d_err, int sm_count,
                          cudaStream_t s);
template <typename T>
void launch_radius_features(const DeviceGrid<T>& g, uint64_t n, uint32_t d, uint32_t k, float beta, float* out,
                            cudaStream_t s);
// d_err is set to 1 if a tensor-core wait timed out (the outputs then hold
// the fallback: eps0 radii, NaN predictions).
void launch_mlp_predict(const float* d_model, const float* d_feat, uint64_t n, float* d_out, uint32_t* d_err,
                        int sm_count, cudaStream_t s);
// Active model: a copy and its version (changes on every set).
unsigned radius_model_snapshot(std::vector<float>* out);
void radius_model_set(const float* model);  // nullptr restores the built-in model
void mlp_grad_device(const float* d_model, const float* d_X, const float* d_Y, const uint32_t* d_idx, uint64_t n,
                     float quantile, float inv_batch, float* d_part, double* d_part_loss, float* d_grad,
                     cudaStream_t s);
size_t mlp_grad_partials(uint64_t n);  // floats of d_part for n samples
void train_model(const float* hX, const float* hY, uint64_t n, int epochs, uint32_t batch, float lr,
                 float quantile, uint64_t seed, float* model_out, float* loss_out, cudaStream_t s);

// Outlier scores of a result table on the device (k_outlier.cu): per point
// the mean table distance and its rank (decreasing), the in-degree and its
// rank (increasing); equal scores ranked by point id.
template <typename T>
void outlier_scores_device(Workspace& w, const int32_t* ids, const T* dists, uint64_t n, uint32_t K, double* mean,
                           int32_t* dist_rank, unsigned long long* indeg, uint32_t* degree_rank, cudaStream_t s);

// Verification figure of a result table on the device (synchronises s).
template <typename T>
double device_checksum(Workspace& w, const T* d_vals, uint64_t count, cudaStream_t s);

}  // namespace knnsj
