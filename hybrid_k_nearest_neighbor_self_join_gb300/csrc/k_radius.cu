// k_radius.cu -- radius assignment for the learned starting radius: the
// features of radius_model.cuh and the MLP evaluated in one pass, one thread
// per query, queries in cell order (neighbouring threads read neighbouring
// points and the same cell-table entries).  The model lives in shared memory.

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "knnsj_internal.h"
#include "mlp_tc.cuh"
#include "radius_model.cuh"

namespace knnsj {

// kRadiusModelDefault[MODEL_FLOATS]: the model trained by
// hybrid_k_nearest_neighbor_self_join_gb300/train_radius.py.
#include "radius_model_weights.inc"

namespace {
std::mutex g_model_mu;
std::vector<float> g_model;
unsigned g_model_version = 0;
}  // namespace

unsigned radius_model_snapshot(std::vector<float>* out) {
  std::lock_guard<std::mutex> lock(g_model_mu);
  if (g_model.empty()) {
    g_model.assign(kRadiusModelDefault, kRadiusModelDefault + MODEL_FLOATS);
    g_model_version = 1;
  }
  *out = g_model;
  return g_model_version;
}

void radius_model_set(const float* model) {
  std::lock_guard<std::mutex> lock(g_model_mu);
  if (model)
    g_model.assign(model, model + MODEL_FLOATS);
  else
    g_model.assign(kRadiusModelDefault, kRadiusModelDefault + MODEL_FLOATS);
  g_model_version = g_model_version + 1 == 0 ? 1 : g_model_version + 1;
}

namespace {

constexpr int RA_THREADS = 128;

template <typename T>
CellTable<T> table_of(const DeviceGrid<T>& g) {
  CellTable<T> t;
  t.g = g.geom;
  t.ckeys = g.ckeys;
  t.coff = g.coff;
  t.dstart = g.dstart;
  t.C = g.C;
  t.dense = g.dense;
  return t;
}

template <typename T>
__global__ void __launch_bounds__(RA_THREADS) radius_assign_kernel(const CellTable<T> t, const T* __restrict__ ps,
                                                                   const uint32_t* __restrict__ pid, uint64_t n,
                                                                   uint32_t d, uint32_t k, float beta,
                                                                   const float* __restrict__ model, float eps0f,
                                                                   float log_lo, float log_hi, float offset,
                                                                   T* __restrict__ qradius) {
  __shared__ __align__(16) float sm[MODEL_FLOATS + 3];
  for (int i = threadIdx.x; i < MODEL_FLOATS; i += blockDim.x) sm[i] = model[i];
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T q[MAX_DI];
  for (uint32_t j = 0; j < t.g.di; j++) q[j] = ps[(uint64_t)j * n + i];
  float f[NFEAT];
  radius_features(t, q, d, k, beta, n, f);
  float y = mlp_eval_blocked(sm, f) + offset;
  y = fminf(fmaxf(y, log_lo), log_hi);
  qradius[pid[i]] = (T)(eps0f * expf(y));
}

template <typename T>
__global__ void __launch_bounds__(RA_THREADS) radius_features_kernel(const CellTable<T> t, const T* __restrict__ ps,
                                                                     const uint32_t* __restrict__ pid, uint64_t n,
                                                                     uint32_t d, uint32_t k, float beta,
                                                                     float* __restrict__ out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T q[MAX_DI];
  for (uint32_t j = 0; j < t.g.di; j++) q[j] = ps[(uint64_t)j * n + i];
  float f[NFEAT];
  radius_features(t, q, d, k, beta, n, f);
  float* o = out + (uint64_t)pid[i] * NFEAT;
  for (int j = 0; j < NFEAT; j++) o[j] = f[j];
}

__global__ void __launch_bounds__(RA_THREADS) mlp_predict_kernel(const float* __restrict__ model,
                                                                 const float* __restrict__ feat, uint64_t n,
                                                                 float* __restrict__ out) {
  __shared__ __align__(16) float sm[MODEL_FLOATS + 3];
  for (int i = threadIdx.x; i < MODEL_FLOATS; i += blockDim.x) sm[i] = model[i];
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float f[NFEAT];
  for (int j = 0; j < NFEAT; j++) f[j] = feat[i * NFEAT + j];
  out[i] = mlp_eval_blocked(sm, f);
}

// Front-ends of the tensor-core MLP (mlp_tc.cuh).
// Radius assignment: features from the cell table, radius written by
// original id; the fallback is the plain starting radius eps0.
template <typename T>
struct AssignSrc {
  CellTable<T> t;
  const T* ps;
  const uint32_t* pid;
  uint64_t n;
  uint32_t d, k;
  float beta, eps0f, log_lo, log_hi, offset;
  T* qradius;
  __device__ void features(uint64_t i, float* f) {
    T q[MAX_DI];
    for (uint32_t j = 0; j < t.g.di; j++) q[j] = ps[(uint64_t)j * n + i];
    radius_features(t, q, d, k, beta, n, f);
  }
  __device__ void store(uint64_t i, float y) {
    y = fminf(fmaxf(y + offset, log_lo), log_hi);
    qradius[pid[i]] = (T)(eps0f * expf(y));
  }
  __device__ void fallback(uint64_t i) { qradius[pid[i]] = (T)eps0f; }
};

// Prediction from stored features (knnsj_radius_predict).
struct PredictSrc {
  const float* feat;
  float* out;
  __device__ void features(uint64_t i, float* f) {
    for (int j = 0; j < NFEAT; j++) f[j] = feat[i * NFEAT + j];
  }
  __device__ void store(uint64_t i, float y) { out[i] = y; }
  __device__ void fallback(uint64_t i) { out[i] = __int_as_float(0x7fc00000); }
};

template <typename Src>
__global__ void __launch_bounds__(TC_ROWS) mlp_tc_kernel(Src src, const float* __restrict__ model, uint64_t n,
                                                          uint32_t* err, TcCtl ctl) {
  mlp_tc_tiles(src, model, n, err, ctl);
}

// KNNSJ_TEST_MLP_TIMEOUT=1 (tests only): the tensor-core MLP issues no MMA and
// waits at most 1024 polls, so every tile takes the timeout path (eps0
// radii for a join, NaN predictions, the error flag set).
static TcCtl tc_ctl() {
  TcCtl c;
  const char* e = std::getenv("KNNSJ_TEST_MLP_TIMEOUT");
  if (e && std::atoi(e) == 1) {
    c.no_issue = 1;
    c.wait_limit = 1024;
  }
  return c;
}

template <typename Src>
void launch_mlp_tc(const Src& src, const float* model, uint64_t n, uint32_t* err, int sm_count, cudaStream_t s) {
  if (n == 0) return;
  // the largest shared-memory carveout, so that several CTAs share an SM
  // (each holds 64 of the SM's 512 TMEM columns: at most 8 fit)
  KNNSJ_CUDA(cudaFuncSetAttribute(mlp_tc_kernel<Src>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
  // CTAs per SM by registers and shared memory (the occupancy query does not
  // count co-resident CTAs of a kernel that allocates TMEM), at most what
  // the SM's TMEM holds
  cudaFuncAttributes fa;
  KNNSJ_CUDA(cudaFuncGetAttributes(&fa, mlp_tc_kernel<Src>));
  const int regs = std::max(fa.numRegs, 1) * TC_ROWS;
  int per_sm = std::min(65536 / regs, (int)((227 * 1024) / std::max<size_t>(fa.sharedSizeBytes + 1024, 1)));
  per_sm = std::max(1, std::min(per_sm, 512 / TC_TMEM_COLS));
  const uint64_t tiles = (n + TC_ROWS - 1) / TC_ROWS;
  uint64_t blocks = (uint64_t)std::max(per_sm, 1) * (uint64_t)std::max(sm_count, 1);
  if (blocks > tiles) blocks = tiles;
  mlp_tc_kernel<Src><<<(unsigned)blocks, TC_ROWS, 0, s>>>(src, model, n, err, tc_ctl());
  KNNSJ_CHECK_LAUNCH();
}

}  // namespace

constexpr float LEARNED_LOG_MARGIN = 0.08f;

// Largest ring half-width (in cells of the eps0 grid) a learned radius may
// start with: keeps a ring at most ~1024 rows; growth beyond is handled by
// the retry schedule and grid rebuilds.
double learned_max_cells(uint32_t di) {
  if (const char* e = std::getenv("KNNSJ_LEARNED_MAX_CELLS")) {  // tuning override
    const double v = std::atof(e);
    if (v >= 1.0) return v;
  }
  switch (di) {
    case 1: return 64.0;
    case 2: return 64.0;
    case 3: return 15.0;
    default: return 1.0;  // beyond three indexed dimensions a larger first ring
                          // costs more than the passes it saves (measured on
                          // 4-D and 6-D mixtures): large radii grow in retries
  }
}

// The MLP runs on the tensor cores (BF16 operands, FP32 accumulation) unless
// KNNSJ_RADIUS_MLP=fp32 selects the CUDA-core FP32 evaluation.
static bool mlp_on_tensor_cores() {
  const char* e = std::getenv("KNNSJ_RADIUS_MLP");
  return !(e && std::strcmp(e, "fp32") == 0);
}

template <typename T>
void launch_radius_assign(const DeviceGrid<T>& g, uint64_t n, uint32_t d, uint32_t k, float beta,
                          const float* d_model, double eps0, float offset, T* qradius, uint32_t* d_err, int sm_count,
                          cudaStream_t s) {
  const float log_lo = std::log(1.0f / 16.0f);
  const float log_hi = (float)std::log(learned_max_cells(g.geom.di) * (1.0 - 1.0 / 4096.0));
  // the model predicts the 0.9 quantile of log(r_K / eps0); a failed first
  // pass costs a second scan at a larger radius, so starting 8% wider (in
  // radius) is cheaper overall (measured on 2-D, 3-D and 4-D joins, k 32-64)
  offset += LEARNED_LOG_MARGIN;
  if (mlp_on_tensor_cores()) {
    AssignSrc<T> src{table_of(g), g.ps, g.pid, n, d, k, beta, (float)eps0, log_lo, log_hi, offset, qradius};
    launch_mlp_tc(src, d_model, n, d_err, sm_count, s);
    return;
  }
  radius_assign_kernel<T><<<(unsigned)((n + RA_THREADS - 1) / RA_THREADS), RA_THREADS, 0, s>>>(
      table_of(g), g.ps, g.pid, n, d, k, beta, d_model, (float)eps0, log_lo, log_hi, offset, qradius);
  KNNSJ_CHECK_LAUNCH();
}

template <typename T>
void launch_radius_features(const DeviceGrid<T>& g, uint64_t n, uint32_t d, uint32_t k, float beta, float* out,
                            cudaStream_t s) {
  radius_features_kernel<T><<<(unsigned)((n + RA_THREADS - 1) / RA_THREADS), RA_THREADS, 0, s>>>(
      table_of(g), g.ps, g.pid, n, d, k, beta, out);
  KNNSJ_CHECK_LAUNCH();
}

void launch_mlp_predict(const float* d_model, const float* d_feat, uint64_t n, float* d_out, uint32_t* d_err,
                        int sm_count, cudaStream_t s) {
  if (n == 0) return;
  if (mlp_on_tensor_cores()) {
    PredictSrc src{d_feat, d_out};
    launch_mlp_tc(src, d_model, n, d_err, sm_count, s);
    return;
  }
  mlp_predict_kernel<<<(unsigned)((n + RA_THREADS - 1) / RA_THREADS), RA_THREADS, 0, s>>>(d_model, d_feat, n, d_out);
  KNNSJ_CHECK_LAUNCH();
}

template void launch_radius_assign<float>(const DeviceGrid<float>&, uint64_t, uint32_t, uint32_t, float,
                                          const float*, double, float, float*, uint32_t*, int, cudaStream_t);
template void launch_radius_assign<double>(const DeviceGrid<double>&, uint64_t, uint32_t, uint32_t, float,
                                           const float*, double, float, double*, uint32_t*, int, cudaStream_t);
template void launch_radius_features<float>(const DeviceGrid<float>&, uint64_t, uint32_t, uint32_t, float, float*,
                                            cudaStream_t);
template void launch_radius_features<double>(const DeviceGrid<double>&, uint64_t, uint32_t, uint32_t, float, float*,
                                             cudaStream_t);

}  // namespace knnsj
