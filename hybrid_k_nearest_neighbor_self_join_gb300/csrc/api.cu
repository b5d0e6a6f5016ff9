// api.cu -- the C ABI (include/knnsj.h): KNNJoinPy and the status-returning
// entry points.  Validation, defaults, device selection, host<->device
// staging and error translation live here; the join itself is run_join
// (join.cu).

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#ifdef KNNSJ_BUILD_DTYPE_DOUBLE
#define KNNSJ_KNNJOINPY_DOUBLE 1
#endif
#include "knnsj_host.h"
#include "knnsj_internal.h"

#ifndef KNNSJ_BUILD_DTYPE_DOUBLE
typedef float knnjoinpy_t;
#define KNNSJ_PY_DTYPE KNNSJ_F32
#else
typedef double knnjoinpy_t;
#define KNNSJ_PY_DTYPE KNNSJ_F64
#endif

using namespace knnsj;

namespace {

std::mutex g_call_mutex;

const char* env(const char* name) {
  const char* v = std::getenv(name);
  return (v && *v) ? v : nullptr;
}

knnsj_status make_config(const knnsj_options* o, uint32_t d, JoinConfig* c) {
  // params.h defaults, then environment, then explicit options
  c->beta = 0.05;
  c->num_indexed_dims = d < 6 ? d : 6;
  if (const char* e = env("KNNSJ_BETA")) c->beta = std::atof(e);
  if (const char* e = env("KNNSJ_NUMINDEXEDDIM")) c->num_indexed_dims = (uint32_t)std::atoi(e);
  if (const char* e = env("KNNSJ_VERBOSE")) c->verbose = std::atoi(e);
  if (const char* e = env("KNNSJ_DENSE")) c->dense_mode = std::atoi(e);
  if (const char* e = env("KNNSJ_GRAPH")) c->use_graph = std::atoi(e);
  if (const char* e = env("KNNSJ_FLOAT_PREFILTER")) c->float_prefilter = std::atoi(e);
  if (const char* e = env("KNNSJ_ROW_CHUNKS")) c->row_chunks = std::atoi(e);
  if (const char* e = env("KNNSJ_TAIL_BRUTE")) c->tail_brute = std::atoi(e);
  if (const char* e = env("KNNSJ_TILE")) c->tile_search = std::atoi(e);
  if (const char* e = env("KNNSJ_TILE_FINE")) c->tile_fine = std::max(0, std::atoi(e));
  if (const char* e = env("KNNSJ_DIRECT_ROWS")) c->direct_rows = std::atoi(e);
  if (const char* e = env("KNNSJ_DEVICE_TABLE_MB")) c->device_table_cap = (unsigned long long)std::atoll(e) << 20;
  if (const char* e = env("KNNSJ_SEARCH_SHAPE")) {  // "warps,qchunk,buffer" (0 = default)
    int a = 0, b = 0, bb = 0;
    if (std::sscanf(e, "%d,%d,%d", &a, &b, &bb) >= 1) {
      c->search_warps = a;
      c->search_qchunk = b;
      c->search_buffer = bb;
    }
  }
  if (o) {
    if (o->struct_size < sizeof(uint32_t)) return KNNSJ_ERR_INVALID_ARGUMENT;
    if (o->num_indexed_dims > 0) c->num_indexed_dims = (uint32_t)o->num_indexed_dims;
    if (o->beta >= 0) c->beta = o->beta;
    c->no_reorder = o->no_reorder;
    c->radius_mode = o->radius_mode;
    c->max_iterations = o->max_iterations;
    if (o->verbose) c->verbose = o->verbose;
    if (o->struct_size >= offsetof(knnsj_options, radius_offset) + sizeof(double))
      c->radius_offset = o->radius_offset;
    if (o->struct_size >= offsetof(knnsj_options, device_table_mb) + sizeof(int32_t) && o->device_table_mb > 0)
      c->device_table_cap = (unsigned long long)o->device_table_mb << 20;
  }
  if (const char* e = env("KNNSJ_RADIUS_MODE")) c->radius_mode = std::atoi(e);
  if (c->num_indexed_dims == 0 || c->num_indexed_dims > d) c->num_indexed_dims = d < 6 ? d : 6;
  if (c->num_indexed_dims > (uint32_t)MAX_DI) return KNNSJ_ERR_UNSUPPORTED;
  if (!(c->beta >= 0.0) || !(c->beta <= 1.0)) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (c->radius_mode != KNNSJ_RADIUS_BETA && c->radius_mode != KNNSJ_RADIUS_LEARNED)
    return KNNSJ_ERR_INVALID_ARGUMENT;
  return KNNSJ_OK;
}

knnsj_status validate(const void* data, uint64_t n, uint32_t d, uint32_t k, const void* ids,
                      const void* dists) {
  if (!data || !ids || !dists) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (n == 0 || d == 0 || d > (uint32_t)MAX_D) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (n >= (1ull << 31)) return KNNSJ_ERR_TOO_MANY_POINTS;
  if ((uint64_t)k + 1 > n) return KNNSJ_ERR_K_TOO_LARGE;
  return KNNSJ_OK;
}

// Largest k+1 of a join.  The search kernels keep each query's selection in
// a shared-memory buffer of the next power of two >= k+1 + 32 keys (8-byte
// keys for float data, 16-byte for double); one warp per block holds up to
// 128 KB of it: k+1 up to 16352 (float) or 8160 (double).  The reference
// has no such limit (its rows come from pair buffers on the host).
constexpr uint32_t MAX_K_F32 = (128u << 10) / 8 - 32;
constexpr uint32_t MAX_K_F64 = (128u << 10) / 16 - 32;

knnsj_status k_supported(uint32_t k, knnsj_dtype dt) {
  return (uint64_t)k + 1 <= (dt == KNNSJ_F64 ? MAX_K_F64 : MAX_K_F32) ? KNNSJ_OK : KNNSJ_ERR_UNSUPPORTED;
}

int select_device(const knnsj_options* o) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    throw StatusError{KNNSJ_ERR_NO_DEVICE, "no CUDA device"};
  }
  int dev = 0;
  if (o && o->device >= 0) {
    if (o->device >= count) throw StatusError{KNNSJ_ERR_INVALID_ARGUMENT, "device ordinal"};
    dev = o->device;
    KNNSJ_CUDA(cudaSetDevice(dev));
  } else {
    KNNSJ_CUDA(cudaGetDevice(&dev));
  }
  return dev;
}

Workspace& ready_workspace(int dev) {
  Workspace& w = workspace(dev);
  w.ensure_stream();
  if (!w.sm_count) KNNSJ_CUDA(cudaDeviceGetAttribute(&w.sm_count, cudaDevAttrMultiProcessorCount, dev));
  return w;
}

bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

template <typename F>
knnsj_status guarded(F&& f, knnsj_stats* st) {
  try {
    f();
    return KNNSJ_OK;
  } catch (const StatusError& e) {
    if (std::getenv("KNNSJ_VERBOSE")) fprintf(stderr, "knnsj: %s\n", e.what);
    return e.st;
  } catch (const CudaError& e) {
    fprintf(stderr, "knnsj: CUDA error %s in %s\n", cudaGetErrorString(e.err), e.where);
    cudaGetLastError();
    if (e.err == cudaErrorMemoryAllocation) return KNNSJ_ERR_OUT_OF_MEMORY;
    return KNNSJ_ERR_CUDA;
  } catch (const std::bad_alloc&) {
    return KNNSJ_ERR_OUT_OF_MEMORY;
  }
  (void)st;
}

void init_stats(knnsj_stats* st) {
  if (!st) return;
  const uint32_t sz = st->struct_size;
  std::memset(st, 0, sizeof(*st));
  st->struct_size = sz ? sz : (uint32_t)sizeof(*st);
}

// Where the rows of a host-pointer call go:
//  * pinned output buffers (cfg.direct_rows 2, the default): a device
//    result table, copied into them after the join by an SM kernel through
//    their mapped addresses (whole cache lines in address order);
//  * direct rows: pinned buffers with cfg.direct_rows 1, and any outputs
//    whose device result table would not fit (more than the free device
//    memory less a margin, or cfg.device_table_cap), take every row
//    straight from the search kernels, pageable ones being registered with
//    the device for the duration of the call; the device then holds no
//    result table at all, which bounds device memory by the input and the
//    index;
//  * otherwise a device result table whose rows are streamed into pinned
//    buffers by the copy engines in blocks of query ids while the join runs
//    (cfg.direct_rows 0, n >= 2^18, cfg.row_chunks >= 2), or copied out
//    after the join.
// Measured on the 25M-point sky-like join (13 GB of rows) with the query-tile
// first pass: the SM copy after the join 116 ms per join (37 ms search, 67 ms
// copy, the link's rate); direct rows 149 ms (rows land in scattered 260-byte
// pieces, partial cache lines); streamed 86 ms on some boxes, but 150-350 ms
// steps on others, where the copy engines' device-to-host rate fell to
// ~50 GB/s for seconds at a time (the SM writes of direct rows were steady
// there).
constexpr uint64_t ROW_STREAM_MIN_ROWS = 1u << 18;

// Device-visible address of a host buffer, when it is pinned and mapped.
void* mapped_host_pointer(void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // an unregistered pointer is not an error here
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Registers pageable host buffers with the device for one call (mapped);
// unregisters on destruction.
struct HostRegistration {
  cudaStream_t stream = nullptr;  // finished before the buffers are unregistered
  std::vector<void*> regs;
  bool add(void* p, size_t bytes) {
    if (cudaHostRegister(p, bytes, cudaHostRegisterMapped) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    regs.push_back(p);
    return true;
  }
  ~HostRegistration() {
    if (!regs.empty() && stream) cudaStreamSynchronize(stream);
    for (void* p : regs) cudaHostUnregister(p);
  }
};

// Waits for a stream when leaving a scope, also on an error: no kernel is
// left writing into the caller's buffers after the call returns.
struct SyncOnExit {
  cudaStream_t s;
  ~SyncOnExit() { cudaStreamSynchronize(s); }
};

template <typename T>
void host_join_ws(Workspace& w, const T* data, uint64_t n, uint32_t d, uint32_t k, const JoinConfig& cfg,
                  int32_t* out_ids, T* out_d, knnsj_stats* st, bool checksum) {
  cudaStream_t s = w.stream;
  const uint64_t K = (uint64_t)k + 1;
  const uint64_t table_bytes = n * K * (4 + sizeof(T));
  T* din = (T*)w.in.get(n * d * sizeof(T));
  cudaEvent_t t0, t1;
  KNNSJ_CUDA(cudaEventCreate(&t0));
  KNNSJ_CUDA(cudaEventCreate(&t1));
  KNNSJ_CUDA(cudaEventRecord(t0, s));
  KNNSJ_CUDA(cudaMemcpyAsync(din, data, n * d * sizeof(T), cudaMemcpyHostToDevice, s));
  KNNSJ_CUDA(cudaEventRecord(t1, s));
  double* rowsum = (st && checksum) ? (double*)w.rowsum.get(n * 8) : nullptr;
  // 1. direct rows into pinned buffers, or into pageable buffers registered
  // for this call when the result table does not fit on the device
  int32_t* ids_dev = nullptr;
  T* d_dev = nullptr;
  HostRegistration reg;
  reg.stream = s;
  int32_t* mi = (int32_t*)mapped_host_pointer(out_ids);
  T* md = (T*)mapped_host_pointer(out_d);
  const bool pinned = mi && md;
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) cudaGetLastError();
    const uint64_t cap = cfg.device_table_cap ? cfg.device_table_cap
                                              : (free_b > (2ull << 30) ? (uint64_t)free_b - (2ull << 30) : 0ull);
    const bool fits = table_bytes <= cap;
    // pinned: direct rows when asked for or when the table does not fit;
    // otherwise a device table (below)
    if (pinned && (cfg.direct_rows == 1 || !fits)) {
      ids_dev = mi;
      d_dev = md;
    } else if (!pinned && !fits && reg.add(out_ids, n * K * 4) && reg.add(out_d, n * K * sizeof(T))) {
      ids_dev = (int32_t*)mapped_host_pointer(out_ids);
      d_dev = (T*)mapped_host_pointer(out_d);
      if (!ids_dev || !d_dev) ids_dev = nullptr, d_dev = nullptr;
    }
  }
  if (ids_dev && d_dev) {
    SyncOnExit guard{s};
    run_join<T>(w, cfg, din, data, n, d, k, ids_dev, d_dev, st, s, nullptr, rowsum);
    KNNSJ_CUDA(cudaStreamSynchronize(s));
    if (st) {
      float a = 0;
      cudaEventElapsedTime(&a, t0, t1);
      st->ms_transfer = a;  // the rows needed no copy
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (cfg.verbose && st)
      fprintf(stderr, "knnsj: n=%llu d=%u k=%u rows written to host memory; prep=%.3f ms search=%.3f ms\n",
              (unsigned long long)n, d, k, st->ms_prep, st->ms_search);
    return;
  }
  // 2. a device result table, streamed or copied after the join
  int32_t* dids = (int32_t*)w.ids.get(n * K * 4);
  T* ddist = (T*)w.dists.get(n * K * sizeof(T));
  RowStream rs;
  RowStream* rsp = nullptr;
  if (cfg.direct_rows == 0 && cfg.row_chunks >= 2 && n >= ROW_STREAM_MIN_ROWS) {
    cudaPointerAttributes ai{}, ad{};
    if (cudaPointerGetAttributes(&ai, out_ids) == cudaSuccess && cudaPointerGetAttributes(&ad, out_d) == cudaSuccess &&
        ai.type == cudaMemoryTypeHost && ad.type == cudaMemoryTypeHost && ai.devicePointer && ad.devicePointer) {
      rs.ids_host = out_ids;
      rs.d_host = out_d;
      rs.ids_dev = ai.devicePointer;
      rs.d_dev = ad.devicePointer;
      rs.chunks = cfg.row_chunks;
      rsp = &rs;
    }
    cudaGetLastError();  // an unregistered pointer is not an error here
  }
  struct CopyWait {  // no copy into the caller's buffers outlives this call
    Workspace* w = nullptr;
    ~CopyWait() {
      if (!w) return;
      cudaStreamSynchronize(w->copy_stream);
      w->mail = false;
    }
  } copy_wait;
  if (rsp) copy_wait.w = &w;
  run_join<T>(w, cfg, din, data, n, d, k, dids, ddist, st, s, rsp, rowsum);
  const bool streamed = rsp && rsp->active;  // rows already in place
  cudaEvent_t t2, t3;
  KNNSJ_CUDA(cudaEventCreate(&t2));
  KNNSJ_CUDA(cudaEventCreate(&t3));
  KNNSJ_CUDA(cudaEventRecord(t2, s));
  if (!streamed && pinned && cfg.direct_rows == 2) {
    launch_copy_to_mapped(mi, dids, n * K * 4, w.sm_count, s);
    launch_copy_to_mapped(md, ddist, n * K * sizeof(T), w.sm_count, s);
  } else if (!streamed) {
    KNNSJ_CUDA(cudaMemcpyAsync(out_ids, dids, n * K * 4, cudaMemcpyDeviceToHost, s));
    KNNSJ_CUDA(cudaMemcpyAsync(out_d, ddist, n * K * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
  KNNSJ_CUDA(cudaEventRecord(t3, s));
  KNNSJ_CUDA(cudaStreamSynchronize(s));
  if (st) {  // (streamed rows: run_join counted the copies that outlast the join)
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, t0, t1);
    cudaEventElapsedTime(&b, t2, t3);
    st->ms_transfer = a + (streamed ? st->ms_transfer : b);
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaEventDestroy(t2);
  cudaEventDestroy(t3);
  if (cfg.verbose && st)
    fprintf(stderr,
            "knnsj: n=%llu d=%u k=%u eps0=%g bucket=%d iterations=%d regrids=%d candidates=%llu "
            "prep=%.3f ms search=%.3f ms transfer=%.3f ms\n",
            (unsigned long long)n, d, k, st->eps0, st->eps_bucket, st->iterations, st->regrids,
            (unsigned long long)st->candidates, st->ms_prep, st->ms_search, st->ms_transfer);
}

template <typename T>
void host_join(const T* data, uint64_t n, uint32_t d, uint32_t k, const JoinConfig& cfg, int dev,
               int32_t* out_ids, T* out_d, knnsj_stats* st) {
  host_join_ws<T>(ready_workspace(dev), data, n, d, k, cfg, out_ids, out_d, st, true);
}

template <typename T>
void device_join(const T* data, uint64_t n, uint32_t d, uint32_t k, const JoinConfig& cfg, int dev,
                 int32_t* out_ids, T* out_d, knnsj_stats* st) {
  Workspace& w = ready_workspace(dev);
  run_join<T>(w, cfg, data, nullptr, n, d, k, out_ids, out_d, st, w.stream);
  KNNSJ_CUDA(cudaStreamSynchronize(w.stream));
}

// ---- batched self-joins (knnsj_selfjoin_batched) ---------------------------
// Many independent joins of uneven sizes.  One small set keeps the GPU busy
// for a fraction of the time its launches and host synchronisations take, so
// worker host threads, each with its own workspace and stream, take the sets
// largest first and run them side by side.  The search kernel's launch shape
// (warps per block, queries per work fetch, selection buffer) is chosen per
// (dtype, d, indexed dims, K) class by an autotuner: the first time a class
// appears in the process, every candidate shape runs the class's largest set
// and the fastest search is kept.  Shapes change only speed: every set's
// result equals that of a knnsj_selfjoin call on it.

struct ShapeKey {
  int dtype;
  uint32_t d, di, K;
  bool operator<(const ShapeKey& o) const {
    if (dtype != o.dtype) return dtype < o.dtype;
    if (d != o.d) return d < o.d;
    if (di != o.di) return di < o.di;
    return K < o.K;
  }
};

std::map<ShapeKey, SearchShape> g_tuned;  // guarded by g_call_mutex

std::vector<SearchShape> candidate_shapes(uint32_t K) {
  std::vector<SearchShape> v;
  for (int wpb : {4, 8})
    for (int qc : {1, 4, 16}) {
      SearchShape sh;
      sh.warps_per_block = wpb;
      sh.qchunk = qc;
      v.push_back(sh);
    }
  if (K + 32 <= 256) {  // the sorted-buffer selection instead of the histogram one
    SearchShape sh;
    sh.warps_per_block = 8;
    sh.qchunk = 4;
    sh.buffer = 512;
    v.push_back(sh);
  }
  return v;
}

// Tuned shapes persist across processes in a text file named by
// KNNSJ_TUNE_CACHE: one line per class, "<device> dtype d di K warps qchunk
// buffer" (the device's name with blanks replaced by '_'); lines of other
// devices are kept as they are.  The file is read the first time the batched
// join runs on a device, and rewritten (through a temporary file and a
// rename) whenever classes were tuned.  Only shapes the tuner itself would
// try are taken from it.
std::set<int> g_tune_loaded;   // devices whose cache file was read; guarded by g_call_mutex
std::set<ShapeKey> g_measured;  // classes tuned by measurement here or in the file's process

std::string device_tag(int dev) {
  cudaDeviceProp p{};
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  std::string t = p.name;
  for (char& c : t)
    if (c == ' ' || c == '\t') c = '_';
  return t.empty() ? "unknown" : t;
}

bool tunable_shape(uint32_t K, const SearchShape& sh) {
  if (sh.warps_per_block == 0 && sh.qchunk == 0 && sh.buffer == 0) return true;  // the default shape
  for (const SearchShape& c : candidate_shapes(K))
    if (c.warps_per_block == sh.warps_per_block && c.qchunk == sh.qchunk && c.buffer == sh.buffer) return true;
  return false;
}

void load_tune_cache(int dev) {
  const char* path = env("KNNSJ_TUNE_CACHE");
  if (!path || !*path || g_tune_loaded.count(dev)) return;
  g_tune_loaded.insert(dev);
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  const std::string tag = device_tag(dev);
  char name[256];
  int dt = 0;
  unsigned d = 0, di = 0, K = 0;
  SearchShape sh;
  while (std::fscanf(f, "%255s %d %u %u %u %d %d %d", name, &dt, &d, &di, &K, &sh.warps_per_block, &sh.qchunk,
                     &sh.buffer) == 8) {
    if (tag == name && tunable_shape(K, sh)) {
      g_tuned[ShapeKey{dt, d, di, K}] = sh;
      g_measured.insert(ShapeKey{dt, d, di, K});
    }
  }
  std::fclose(f);
}

void save_tune_cache(int dev) {
  const char* path = env("KNNSJ_TUNE_CACHE");
  if (!path || !*path) return;
  const std::string tag = device_tag(dev);
  std::string keep;  // other devices' lines
  if (FILE* f = std::fopen(path, "r")) {
    char line[512];
    while (std::fgets(line, sizeof(line), f)) {
      char name[256];
      if (std::sscanf(line, "%255s", name) == 1 && tag != name) keep += line;
    }
    std::fclose(f);
  }
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) return;
  std::fputs(keep.c_str(), f);
  for (const auto& kv : g_tuned)
    if (g_measured.count(kv.first))
      std::fprintf(f, "%s %d %u %u %u %d %d %d\n", tag.c_str(), kv.first.dtype, kv.first.d, kv.first.di, kv.first.K,
                 kv.second.warps_per_block, kv.second.qchunk, kv.second.buffer);
  const bool ok = std::fclose(f) == 0;
  if (ok) std::rename(tmp.c_str(), path);
  else std::remove(tmp.c_str());
}

struct BatchPool {
  std::vector<Workspace*> ws;  // one per worker, kept across calls
};

BatchPool& batch_pool(int dev) {
  static std::vector<BatchPool*> all;
  if ((int)all.size() <= dev) all.resize(dev + 1, nullptr);
  if (!all[dev]) all[dev] = new BatchPool();
  return *all[dev];
}

int batch_workers(uint32_t n_sets) {
  int w = 8;
  if (const char* e = env("KNNSJ_BATCH_WORKERS")) w = std::max(1, std::atoi(e));
  return (int)std::min<uint32_t>((uint32_t)w, std::max<uint32_t>(n_sets, 1));
}

template <typename T>
void run_batched(knnsj_set* sets, const std::vector<uint32_t>& order, const std::vector<JoinConfig>& cfgs,
                 int dev, knnsj_stats* agg) {
  BatchPool& pool = batch_pool(dev);
  const int nw = batch_workers((uint32_t)order.size());
  while ((int)pool.ws.size() < nw) pool.ws.push_back(new Workspace());
  for (int i = 0; i < nw; i++) {
    pool.ws[i]->ensure_stream();
    if (!pool.ws[i]->sm_count)
      KNNSJ_CUDA(cudaDeviceGetAttribute(&pool.ws[i]->sm_count, cudaDevAttrMultiProcessorCount, dev));
  }
  const int code = sizeof(T) == 4 ? KNNSJ_F32 : KNNSJ_F64;
  auto key_of = [&](uint32_t i) {
    return ShapeKey{code, sets[i].d, cfgs[i].num_indexed_dims, sets[i].k + 1};
  };
  auto join_one = [&](Workspace& w, uint32_t i, const SearchShape& sh, knnsj_stats* st) {
    JoinConfig c = cfgs[i];
    c.search_warps = sh.warps_per_block;
    c.search_qchunk = sh.qchunk;
    c.search_buffer = sh.buffer;
    host_join_ws<T>(w, (const T*)sets[i].data, sets[i].n, sets[i].d, sets[i].k, c, sets[i].out_ids,
                    (T*)sets[i].out_dists, st, false);
  };
  // autotune the classes seen for the first time, on their largest set
  load_tune_cache(dev);
  bool tuned_now = false;
  const char* at = env("KNNSJ_AUTOTUNE");
  const bool tune = !(at && std::atoi(at) == 0);
  std::map<ShapeKey, uint32_t> largest;
  for (uint32_t i : order) {
    if (sets[i].status != KNNSJ_OK) continue;
    const ShapeKey kk = key_of(i);
    if (!largest.count(kk) || sets[i].n > sets[largest[kk]].n) largest[kk] = i;
  }
  for (const auto& kv : largest) {
    if (g_tuned.count(kv.first)) continue;
    SearchShape best;
    if (tune && sets[kv.second].n >= 20000) {
      Workspace& w = *pool.ws[0];
      knnsj_stats st;
      std::memset(&st, 0, sizeof(st));
      st.struct_size = sizeof(st);
      try {
        join_one(w, kv.second, best, &st);  // warm-up with the default shape
        double best_ms = st.ms_search_kernels;
        for (const SearchShape& sh : candidate_shapes(kv.first.K)) {
          join_one(w, kv.second, sh, &st);
          if (st.ms_search_kernels < best_ms * 0.98) {
            best_ms = st.ms_search_kernels;
            best = sh;
          }
        }
        g_measured.insert(kv.first);
        tuned_now = true;
      } catch (...) {
        best = SearchShape();  // the set itself reports its error below
      }
    }
    g_tuned[kv.first] = best;
  }
  if (tuned_now) save_tune_cache(dev);
  // run every set; workers take them largest first
  std::atomic<uint32_t> next{0};
  std::vector<knnsj_stats> per(order.size());
  auto worker = [&](int wi) {
    cudaSetDevice(dev);
    Workspace& w = *pool.ws[wi];
    for (;;) {
      const uint32_t slot = next.fetch_add(1);
      if (slot >= order.size()) break;
      const uint32_t i = order[slot];
      if (sets[i].status != KNNSJ_OK) continue;
      knnsj_stats& st = per[slot];
      std::memset(&st, 0, sizeof(st));
      st.struct_size = sizeof(st);
      const SearchShape sh = g_tuned.find(key_of(i))->second;  // every valid set's class is tuned above
      sets[i].status = guarded([&] { join_one(w, i, sh, &st); }, nullptr);
    }
  };
  std::vector<std::thread> th;
  for (int wi = 1; wi < nw; wi++) th.emplace_back(worker, wi);
  worker(0);
  for (auto& t : th) t.join();
  for (const knnsj_stats& st : per) {
    agg->iterations += st.iterations;
    agg->regrids += st.regrids;
    agg->candidates += st.candidates;
    agg->queries_run += st.queries_run;
    agg->ms_prep += st.ms_prep;
    agg->ms_search += st.ms_search;
    agg->ms_transfer += st.ms_transfer;
    agg->ms_search_kernels += st.ms_search_kernels;
    agg->search_alg_bytes += st.search_alg_bytes;
    agg->search_alg_flops += st.search_alg_flops;
    agg->kernel_launches += st.kernel_launches;
  }
}

// ---- fixed-scratch join (knnsj_selfjoin_device_noalloc) --------------------
// For callers that may not allocate device memory: a join inside CUDA stream
// capture (cudaMalloc is illegal there), runtimes whose allocator owns all of
// device memory and forbids raw cudaMalloc/cudaFree, and hosts that size every
// allocation before they start.  All scratch of such a join is carved from this
// array; each device that loads the library holds it until the process exits.
// In host code `g_fixed_scratch` only names the symbol: its device address
// comes from cudaGetSymbolAddress, looked up once per device.
static __device__ __align__(256) unsigned char g_fixed_scratch[KNNSJ_NOALLOC_SCRATCH_BYTES];

struct FixedScratchDevice {
  bool ready = false;
  Arena arena;
  Workspace w;  // never given a stream or events: works on the legacy stream
};

// Set-up on the current device `dev` (the first call there): symbol address and
// SM count.  Neither allocates; both must run outside stream capture.
FixedScratchDevice& fixed_scratch_device(int dev) {
  static std::vector<FixedScratchDevice*> all;
  if ((int)all.size() <= dev) all.resize(dev + 1, nullptr);
  if (!all[dev]) all[dev] = new FixedScratchDevice();
  FixedScratchDevice& f = *all[dev];
  if (!f.ready) {
    unsigned char* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_fixed_scratch);
    if (e != cudaSuccess) throw CudaError{e, "cudaGetSymbolAddress(g_fixed_scratch)"};
    KNNSJ_CUDA(cudaDeviceGetAttribute(&f.w.sm_count, cudaDevAttrMultiProcessorCount, dev));
    f.arena.base = ptr;
    f.arena.cap = KNNSJ_NOALLOC_SCRATCH_BYTES;
    f.ready = true;
  }
  return f;
}

template <typename T>
void fixed_scratch_join(const T* data, uint64_t n, uint32_t d, uint32_t k, JoinConfig cfg, int dev,
                        int32_t* out_ids, T* out_d) {
  FixedScratchDevice& f = fixed_scratch_device(dev);
  // every buffer is carved afresh from the start of the array; the pipeline
  // clears what must start at zero, so the previous call's contents do not matter
  f.arena.used = 0;
  f.w.attach_arena(&f.arena);
  cfg.dense_cells_cap = 4ull * n;  // keeps the dense cell table within the array
  const cudaStream_t s = 0;
  struct Forbid {  // a buffer the array does not cover fails instead of allocating
    Forbid() { g_forbid_alloc = true; }
    ~Forbid() { g_forbid_alloc = false; }
  } forbid;
  run_join<T>(f.w, cfg, data, nullptr, n, d, k, out_ids, out_d, nullptr, s);
  KNNSJ_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

extern "C" {

const char* knnsj_version(void) { return "knnsj 1.0 (sm_103a)"; }

const char* knnsj_status_string(knnsj_status s) {
  switch (s) {
    case KNNSJ_OK: return "ok";
    case KNNSJ_ERR_INVALID_ARGUMENT: return "invalid argument";
    case KNNSJ_ERR_DIM_MISMATCH: return "number of dimensions differs from GPUNUMDIM";
    case KNNSJ_ERR_K_TOO_LARGE: return "k+1 exceeds the number of points";
    case KNNSJ_ERR_NONFINITE_INPUT: return "NaN or infinite coordinate";
    case KNNSJ_ERR_TOO_MANY_POINTS: return "more than 2^31-1 points";
    case KNNSJ_ERR_NO_CONVERGENCE: return "iteration cap reached";
    case KNNSJ_ERR_CUDA: return "CUDA error";
    case KNNSJ_ERR_OUT_OF_MEMORY: return "out of device memory";
    case KNNSJ_ERR_NO_DEVICE: return "no CUDA device";
    case KNNSJ_ERR_UNSUPPORTED: return "unsupported configuration";
    case KNNSJ_ERR_IO: return "file I/O error";
    case KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH:
      return "problem exceeds the fixed scratch array (n <= 65536, d <= 8, k+1 <= 128)";
  }
  return "unknown status";
}

knnsj_dtype knnsj_build_dtype(void) { return KNNSJ_PY_DTYPE; }

knnsj_status knnsj_selfjoin(const void* data, knnsj_dtype dtype, uint64_t n, uint32_t d, uint32_t k,
                            const knnsj_options* opts, int32_t* out_ids, void* out_dists,
                            knnsj_stats* stats) {
  knnsj_status v = validate(data, n, d, k, out_ids, out_dists);
  if (v != KNNSJ_OK) return v;
  if (dtype != KNNSJ_F32 && dtype != KNNSJ_F64) return KNNSJ_ERR_INVALID_ARGUMENT;
  v = k_supported(k, dtype);
  if (v != KNNSJ_OK) return v;
  JoinConfig cfg;
  v = make_config(opts, d, &cfg);
  if (v != KNNSJ_OK) return v;
  std::lock_guard<std::mutex> lock(g_call_mutex);
  init_stats(stats);
  return guarded(
      [&] {
        const int dev = select_device(opts);
        if (dtype == KNNSJ_F32)
          host_join<float>((const float*)data, n, d, k, cfg, dev, out_ids, (float*)out_dists, stats);
        else
          host_join<double>((const double*)data, n, d, k, cfg, dev, out_ids, (double*)out_dists, stats);
      },
      stats);
}

knnsj_status knnsj_selfjoin_device(const void* d_data, knnsj_dtype dtype, uint64_t n, uint32_t d,
                                   uint32_t k, const knnsj_options* opts, int32_t* d_out_ids,
                                   void* d_out_dists, knnsj_stats* stats) {
  knnsj_status v = validate(d_data, n, d, k, d_out_ids, d_out_dists);
  if (v != KNNSJ_OK) return v;
  if (dtype != KNNSJ_F32 && dtype != KNNSJ_F64) return KNNSJ_ERR_INVALID_ARGUMENT;
  v = k_supported(k, dtype);
  if (v != KNNSJ_OK) return v;
  JoinConfig cfg;
  v = make_config(opts, d, &cfg);
  if (v != KNNSJ_OK) return v;
  std::lock_guard<std::mutex> lock(g_call_mutex);
  init_stats(stats);
  return guarded(
      [&] {
        const int dev = select_device(opts);
        if (dtype == KNNSJ_F32)
          device_join<float>((const float*)d_data, n, d, k, cfg, dev, d_out_ids, (float*)d_out_dists, stats);
        else
          device_join<double>((const double*)d_data, n, d, k, cfg, dev, d_out_ids, (double*)d_out_dists,
                              stats);
      },
      stats);
}

// The device join without any allocation (declared in include/knnsj.h).  All
// calls share one array; calls whose GPU work overlapped would race on it.
// This one holds the library's call lock and returns only after its GPU work
// is done, so calls through it follow one another.
knnsj_status knnsj_selfjoin_device_noalloc(const void* d_data, knnsj_dtype dtype, uint64_t n, uint32_t d,
                                           uint32_t k, const knnsj_options* opts, int32_t* d_out_ids,
                                           void* d_out_dists) {
  knnsj_status v = validate(d_data, n, d, k, d_out_ids, d_out_dists);
  if (v != KNNSJ_OK) return v;
  if (dtype != KNNSJ_F32 && dtype != KNNSJ_F64) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (n > KNNSJ_NOALLOC_MAX_POINTS || d > 8 || k + 1 > 128) {
    if (std::getenv("KNNSJ_VERBOSE"))
      fprintf(stderr, "knnsj: fixed-scratch join limited to n <= %u, d <= 8, k+1 <= 128\n",
              KNNSJ_NOALLOC_MAX_POINTS);
    return KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH;
  }
  JoinConfig cfg;
  v = make_config(opts, d, &cfg);
  if (v != KNNSJ_OK) return v;
  std::lock_guard<std::mutex> lock(g_call_mutex);
  return guarded(
      [&] {
        const int dev = select_device(opts);
        if (dtype == KNNSJ_F32)
          fixed_scratch_join<float>((const float*)d_data, n, d, k, cfg, dev, d_out_ids, (float*)d_out_dists);
        else
          fixed_scratch_join<double>((const double*)d_data, n, d, k, cfg, dev, d_out_ids,
                                     (double*)d_out_dists);
      },
      nullptr);
}

knnsj_status knnsj_selfjoin_batched(uint32_t n_sets, knnsj_set* sets, knnsj_dtype dtype,
                                    const knnsj_options* opts, knnsj_stats* stats) {
  if (n_sets > 0 && !sets) return KNNSJ_ERR_INVALID_ARGUMENT;
  if (dtype != KNNSJ_F32 && dtype != KNNSJ_F64) return KNNSJ_ERR_INVALID_ARGUMENT;
  std::vector<JoinConfig> cfgs(n_sets);
  std::vector<uint32_t> order;
  for (uint32_t i = 0; i < n_sets; i++) {
    knnsj_set& st = sets[i];
    st.status = validate(st.data, st.n, st.d, st.k, st.out_ids, st.out_dists);
    if (st.status == KNNSJ_OK) st.status = k_supported(st.k, dtype);
    if (st.status == KNNSJ_OK) st.status = make_config(opts, st.d, &cfgs[i]);
    order.push_back(i);
  }
  // largest first: the long sets start early and the short ones fill the gaps
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return sets[a].n > sets[b].n; });
  std::lock_guard<std::mutex> lock(g_call_mutex);
  knnsj_stats agg;
  std::memset(&agg, 0, sizeof(agg));
  const auto t0 = std::chrono::steady_clock::now();
  knnsj_status call = guarded(
      [&] {
        const int dev = select_device(opts);
        if (dtype == KNNSJ_F32)
          run_batched<float>(sets, order, cfgs, dev, &agg);
        else
          run_batched<double>(sets, order, cfgs, dev, &agg);
      },
      nullptr);
  agg.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) {
    agg.struct_size = stats->struct_size ? stats->struct_size : (uint32_t)sizeof(agg);
    *stats = agg;
  }
  if (call != KNNSJ_OK) return call;
  for (uint32_t i = 0; i < n_sets; i++)
    if (sets[i].status != KNNSJ_OK) return sets[i].status;
  return KNNSJ_OK;
}

knnsj_status knnsj_get_radius_model(float* out) {
  if (!out) return KNNSJ_ERR_INVALID_ARGUMENT;
  std::vector<float> m;
  radius_model_snapshot(&m);
  std::memcpy(out, m.data(), m.size() * sizeof(float));
  return KNNSJ_OK;
}

knnsj_status knnsj_set_radius_model(const float* model) {
  if (model)
    for (int i = 0; i < KNNSJ_RADIUS_MODEL_FLOATS; i++)
      if (!std::isfinite(model[i])) return KNNSJ_ERR_INVALID_ARGUMENT;
  radius_model_set(model);
  return KNNSJ_OK;
}

knnsj_status knnsj_radius_features(const void* data, knnsj_dtype dtype, uint64_t n, uint32_t d, uint32_t k,
                                   const knnsj_options* opts, float* out_features, double* out_eps0) {
  knnsj_status v = validate(data, n, d, k, out_features, out_features);
  if (v != KNNSJ_OK) return v;
  JoinConfig cfg;
  v = make_config(opts, d, &cfg);
  if (v != KNNSJ_OK) return v;
  std::lock_guard<std::mutex> lock(g_call_mutex);
  return guarded(
      [&] {
        const int dev = select_device(opts);
        Workspace& w = ready_workspace(dev);
        cudaStream_t s = w.stream;
        const size_t es = dtype == KNNSJ_F32 ? 4 : 8;
        void* din = w.in.get(n * d * es);
        float* dout = (float*)w.dists.get(n * KNNSJ_RADIUS_FEATURES * 4);
        KNNSJ_CUDA(cudaMemcpyAsync(din, data, n * d * es, cudaMemcpyHostToDevice, s));
        if (dtype == KNNSJ_F32)
          run_features<float>(w, cfg, (const float*)din, (const float*)data, n, d, k, dout, out_eps0, s);
        else
          run_features<double>(w, cfg, (const double*)din, (const double*)data, n, d, k, dout, out_eps0, s);
        KNNSJ_CUDA(cudaMemcpyAsync(out_features, dout, n * KNNSJ_RADIUS_FEATURES * 4, cudaMemcpyDeviceToHost, s));
        KNNSJ_CUDA(cudaStreamSynchronize(s));
      },
      nullptr);
}

knnsj_status knnsj_radius_predict(const float* model, const float* features, uint64_t n, float* out) {
  if (!model || !features || !out) return KNNSJ_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_call_mutex);
  return guarded(
      [&] {
        const int dev = select_device(nullptr);
        Workspace& w = ready_workspace(dev);
        cudaStream_t s = w.stream;
        float* dm = (float*)w.perm.get(KNNSJ_RADIUS_MODEL_FLOATS * 4);
        float* df = (float*)w.in.get(std::max<uint64_t>(n, 1) * KNNSJ_RADIUS_FEATURES * 4);
        float* dy = (float*)w.dists.get(std::max<uint64_t>(n, 1) * 4);
        KNNSJ_CUDA(cudaMemcpyAsync(dm, model, KNNSJ_RADIUS_MODEL_FLOATS * 4, cudaMemcpyHostToDevice, s));
        KNNSJ_CUDA(cudaMemcpyAsync(df, features, n * KNNSJ_RADIUS_FEATURES * 4, cudaMemcpyHostToDevice, s));
        uint32_t* derr = (uint32_t*)w.flags.get(4);
        KNNSJ_CUDA(cudaMemsetAsync(derr, 0, 4, s));
        launch_mlp_predict(dm, df, n, dy, derr, w.sm_count, s);
        uint32_t herr = 0;
        KNNSJ_CUDA(cudaMemcpyAsync(out, dy, n * 4, cudaMemcpyDeviceToHost, s));
        KNNSJ_CUDA(cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, s));
        KNNSJ_CUDA(cudaStreamSynchronize(s));
        if (herr) throw StatusError{KNNSJ_ERR_CUDA, "tensor-core radius model timed out"};
      },
      nullptr);
}

knnsj_status knnsj_radius_grad(const float* model, const float* features, const float* targets, uint64_t n,
                               float quantile, float* out_grad, double* out_loss) {
  if (!model || !features || !targets || !out_grad || n == 0 || !(quantile > 0.0f && quantile < 1.0f))
    return KNNSJ_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_call_mutex);
  return guarded(
      [&] {
        const int dev = select_device(nullptr);
        Workspace& w = ready_workspace(dev);
        cudaStream_t s = w.stream;
        float* dm = (float*)w.perm.get(KNNSJ_RADIUS_MODEL_FLOATS * 4);
        float* df = (float*)w.in.get(n * KNNSJ_RADIUS_FEATURES * 4);
        float* dt = (float*)w.ids.get(n * 4);
        const size_t np = mlp_grad_partials(n);
        float* dpart = (float*)w.dists.get(np * 4);
        double* dpl = (double*)w.eps_partial.get(((n + 63) / 64) * 8);
        float* dg = (float*)w.eps_sample.get(KNNSJ_RADIUS_MODEL_FLOATS * 4);
        KNNSJ_CUDA(cudaMemcpyAsync(dm, model, KNNSJ_RADIUS_MODEL_FLOATS * 4, cudaMemcpyHostToDevice, s));
        KNNSJ_CUDA(cudaMemcpyAsync(df, features, n * KNNSJ_RADIUS_FEATURES * 4, cudaMemcpyHostToDevice, s));
        KNNSJ_CUDA(cudaMemcpyAsync(dt, targets, n * 4, cudaMemcpyHostToDevice, s));
        mlp_grad_device(dm, df, dt, nullptr, n, quantile, 1.0f / (float)n, dpart, dpl, dg, s);
        const size_t ntrain = KNNSJ_RADIUS_MODEL_FLOATS - 2 * KNNSJ_RADIUS_FEATURES;
        KNNSJ_CUDA(cudaMemcpyAsync(out_grad, dg, ntrain * 4, cudaMemcpyDeviceToHost, s));
        std::vector<double> pl((n + 63) / 64);
        KNNSJ_CUDA(cudaMemcpyAsync(pl.data(), dpl, pl.size() * 8, cudaMemcpyDeviceToHost, s));
        KNNSJ_CUDA(cudaStreamSynchronize(s));
        if (out_loss) {
          double l = 0.0;
          for (double x : pl) l += x;
          *out_loss = l / (double)n;
        }
      },
      nullptr);
}

knnsj_status knnsj_radius_train(const float* features, const float* targets, uint64_t n,
                                const knnsj_train_options* o, float* model_out, float* loss_per_epoch) {
  if (!features || !targets || !model_out || n == 0) return KNNSJ_ERR_INVALID_ARGUMENT;
  int epochs = 8;
  uint32_t batch = 8192;
  float lr = 1e-3f, quantile = 0.9f;
  uint64_t seed = 1;
  if (o) {
    if (o->epochs > 0) epochs = o->epochs;
    if (o->batch > 0) batch = o->batch;
    if (o->lr > 0) lr = o->lr;
    if (o->quantile > 0) quantile = o->quantile;
    seed = o->seed;
  }
  if (!(quantile > 0.0f && quantile < 1.0f)) return KNNSJ_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_call_mutex);
  return guarded(
      [&] {
        const int dev = select_device(nullptr);
        Workspace& w = ready_workspace(dev);
        train_model(features, targets, n, epochs, batch, lr, quantile, seed, model_out, loss_per_epoch, w.stream);
      },
      nullptr);
}

knnsj_status knnsj_outlier_scores_device(const int32_t* d_ids, const void* d_dists, knnsj_dtype dtype, uint64_t n,
                                         uint32_t K, double* d_mean, int32_t* d_dist_rank, uint64_t* d_in_degree,
                                         uint32_t* d_degree_rank) {
  if (!d_ids || !d_dists || !d_mean || !d_dist_rank || !d_in_degree || !d_degree_rank || n == 0 || K < 2)
    return KNNSJ_ERR_INVALID_ARGUMENT;
  if (n >= (1ull << 31)) return KNNSJ_ERR_TOO_MANY_POINTS;
  if (dtype != KNNSJ_F32 && dtype != KNNSJ_F64) return KNNSJ_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_call_mutex);
  return guarded(
      [&] {
        const int dev = select_device(nullptr);
        Workspace& w = ready_workspace(dev);
        if (dtype == KNNSJ_F32)
          outlier_scores_device<float>(w, d_ids, (const float*)d_dists, n, K, d_mean, d_dist_rank,
                                       (unsigned long long*)d_in_degree, d_degree_rank, w.stream);
        else
          outlier_scores_device<double>(w, d_ids, (const double*)d_dists, n, K, d_mean, d_dist_rank,
                                        (unsigned long long*)d_in_degree, d_degree_rank, w.stream);
        KNNSJ_CUDA(cudaStreamSynchronize(w.stream));
      },
      nullptr);
}

void knnsj_release(void) {
  std::lock_guard<std::mutex> lock(g_call_mutex);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  workspace(dev).release_all();
  for (Workspace* w : batch_pool(dev).ws) w->release_all();
}

// KNNJoinPy (main.cu:514): same symbol and arguments; returns nothing.
void KNNJoinPy(knnjoinpy_t* dataset, unsigned int NUMPOINTS, unsigned int kNN, unsigned int NDIM,
               int* outNearestNeighborTable, knnjoinpy_t* outNearestNeighborTableDistances) {
#ifdef GPUNUMDIM
  if (GPUNUMDIM != NDIM) {
    // main.cu:526-530
    printf(
        "\nERROR: The number of dimensions defined for the GPU is not the same as the number of "
        "dimensions\n \t\t passed from the Python Interface. GPUNUMDIM=%d, NDIM=%d Exiting!!!",
        GPUNUMDIM, NDIM);
    return;
  }
#endif
  knnsj_options o;
  std::memset(&o, 0, sizeof(o));
  o.struct_size = sizeof(o);
  o.beta = -1.0;
  o.device = -1;
#ifdef NUMINDEXEDDIM
  o.num_indexed_dims = NUMINDEXEDDIM;
#endif
#ifdef BETA
  o.beta = BETA;
#endif
  knnsj_stats st;
  std::memset(&st, 0, sizeof(st));
  st.struct_size = sizeof(st);
  const knnsj_status s = knnsj_selfjoin(dataset, KNNSJ_PY_DTYPE, NUMPOINTS, NDIM, kNN, &o,
                                        outNearestNeighborTable, outNearestNeighborTableDistances, &st);
  if (s != KNNSJ_OK) {
    printf("\nERROR: knnsj: %s\n", knnsj_status_string(s));
    return;
  }
  // main.cu:851 prints the same checksum line
  printf("\n[Verification] Total distance (without sqaure root): %f", st.total_distance);
  fflush(stdout);
}

}  // extern "C"
