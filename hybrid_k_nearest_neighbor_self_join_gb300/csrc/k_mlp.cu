// k_mlp.cu -- training of the radius MLP (radius_model.cuh) on the GPU with
// hand-written kernels: forward + backward of the pinball (quantile) loss,
// a deterministic gradient reduction and Adam.  No reference counterpart.
//
// One block handles TR_BLOCK samples, one thread per sample: the forward
// pass keeps each sample's hidden activations in shared memory, the backward
// pass the activation gradients; parameter gradients are then summed over
// the block's samples in sample order, written as one partial per block and
// summed over blocks in block order -- every run gives the same bits.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "knnsj_internal.h"
#include "radius_model.cuh"

namespace knnsj {

constexpr int NPARAM = MODEL_FLOATS - M_W1;  // trainable: W1..b3 (5825)

namespace {

constexpr int TR_BLOCK = 64;

// grads: per-block partial [gridDim.x][NPARAM]; loss: per-block partial sum
__global__ void __launch_bounds__(TR_BLOCK) mlp_fwd_bwd_kernel(const float* __restrict__ model,
                                                               const float* __restrict__ X,
                                                               const float* __restrict__ Y,
                                                               const uint32_t* __restrict__ idx, uint64_t n,
                                                               float quantile, float inv_batch,
                                                               float* __restrict__ part_grad,
                                                               double* __restrict__ part_loss) {
  extern __shared__ float shm[];
  float* xs = shm;                         // [TR_BLOCK][NFEAT]  normalised inputs
  float* h1 = xs + TR_BLOCK * NFEAT;       // [TR_BLOCK][NHID]   post-ReLU layer 1
  float* h2 = h1 + TR_BLOCK * NHID;        // [TR_BLOCK][NHID]   post-ReLU layer 2
  float* g1 = h2 + TR_BLOCK * NHID;        // [TR_BLOCK][NHID]   dL/d(pre-activation 1)
  float* g2 = g1 + TR_BLOCK * NHID;        // [TR_BLOCK][NHID]   dL/d(pre-activation 2)
  float* g3 = g2 + TR_BLOCK * NHID;        // [TR_BLOCK]         dL/dy
  __shared__ double lsum[TR_BLOCK];
  const int t = threadIdx.x;
  const uint64_t s = (uint64_t)blockIdx.x * TR_BLOCK + t;
  const bool valid = s < n;
  float loss = 0.0f;
  if (valid) {
    const uint64_t row = idx ? idx[s] : s;
    for (int i = 0; i < NFEAT; i++)
      xs[t * NFEAT + i] = (X[row * NFEAT + i] - model[M_MEAN + i]) * model[M_ISTD + i];
    for (int h = 0; h < NHID; h++) {
      float a = model[M_B1 + h];
      for (int i = 0; i < NFEAT; i++) a = fmaf(xs[t * NFEAT + i], model[M_W1 + i * NHID + h], a);
      h1[t * NHID + h] = fmaxf(a, 0.0f);
    }
    float y = model[M_B3];
    for (int o = 0; o < NHID; o++) {
      float a = model[M_B2 + o];
      for (int i = 0; i < NHID; i++) a = fmaf(h1[t * NHID + i], model[M_W2 + i * NHID + o], a);
      const float r = fmaxf(a, 0.0f);
      h2[t * NHID + o] = r;
      y = fmaf(r, model[M_W3 + o], y);
    }
    // pinball loss at `quantile`: L = max(q e, (q - 1) e), e = target - y
    const float e = Y[row] - y;
    loss = e > 0.0f ? quantile * e : (quantile - 1.0f) * e;
    const float dy = (e > 0.0f ? -quantile : (1.0f - quantile)) * inv_batch;
    g3[t] = dy;
    for (int o = 0; o < NHID; o++) g2[t * NHID + o] = h2[t * NHID + o] > 0.0f ? dy * model[M_W3 + o] : 0.0f;
    for (int i = 0; i < NHID; i++) {
      float a = 0.0f;
      if (h1[t * NHID + i] > 0.0f)
        for (int o = 0; o < NHID; o++) a = fmaf(model[M_W2 + i * NHID + o], g2[t * NHID + o], a);
      g1[t * NHID + i] = a;
    }
  } else {
    for (int i = 0; i < NFEAT; i++) xs[t * NFEAT + i] = 0.0f;
    for (int h = 0; h < NHID; h++) {
      h1[t * NHID + h] = 0.0f;
      h2[t * NHID + h] = 0.0f;
      g1[t * NHID + h] = 0.0f;
      g2[t * NHID + h] = 0.0f;
    }
    g3[t] = 0.0f;
  }
  lsum[t] = (double)loss;
  __syncthreads();
  float* pg = part_grad + (uint64_t)blockIdx.x * NPARAM;
  // parameter gradients, each a sum over this block's samples in order
  for (int p = t; p < NPARAM; p += TR_BLOCK) {
    const int m = p + M_W1;
    float a = 0.0f;
    if (m < M_B1) {
      const int i = (m - M_W1) / NHID, h = (m - M_W1) % NHID;
      for (int r = 0; r < TR_BLOCK; r++) a = fmaf(xs[r * NFEAT + i], g1[r * NHID + h], a);
    } else if (m < M_W2) {
      const int h = m - M_B1;
      for (int r = 0; r < TR_BLOCK; r++) a += g1[r * NHID + h];
    } else if (m < M_B2) {
      const int i = (m - M_W2) / NHID, o = (m - M_W2) % NHID;
      for (int r = 0; r < TR_BLOCK; r++) a = fmaf(h1[r * NHID + i], g2[r * NHID + o], a);
    } else if (m < M_W3) {
      const int o = m - M_B2;
      for (int r = 0; r < TR_BLOCK; r++) a += g2[r * NHID + o];
    } else if (m < M_B3) {
      const int o = m - M_W3;
      for (int r = 0; r < TR_BLOCK; r++) a = fmaf(h2[r * NHID + o], g3[r], a);
    } else {
      for (int r = 0; r < TR_BLOCK; r++) a += g3[r];
    }
    pg[p] = a;
  }
  if (t == 0) {
    double l = 0.0;
    for (int r = 0; r < TR_BLOCK; r++) l += lsum[r];
    part_loss[blockIdx.x] = l;
  }
}

__global__ void grad_reduce_kernel(const float* __restrict__ part, uint32_t nblocks, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  float a = 0.0f;
  for (uint32_t b = 0; b < nblocks; b++) a += part[(uint64_t)b * NPARAM + p];
  grad[p] = a;
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  const float gp = g[p];
  const float a = b1 * m1[p] + (1.0f - b1) * gp;
  const float v = b2 * m2[p] + (1.0f - b2) * gp * gp;
  m1[p] = a;
  m2[p] = v;
  const float mh = a / c1, vh = v / c2;
  w[p] -= lr * mh / (sqrtf(vh) + eps);
}

size_t fwd_bwd_smem() { return (size_t)TR_BLOCK * (NFEAT + 4 * NHID + 1) * sizeof(float); }

}  // namespace

size_t mlp_grad_partials(uint64_t n) { return (size_t)((n + TR_BLOCK - 1) / TR_BLOCK) * NPARAM; }

// Full gradient (sum over the batch of the pinball loss / n) and loss of
// `model` on n samples already on the device.
void mlp_grad_device(const float* d_model, const float* d_X, const float* d_Y, const uint32_t* d_idx, uint64_t n,
                     float quantile, float inv_batch, float* d_part, double* d_part_loss, float* d_grad,
                     cudaStream_t s) {
  const uint32_t nb = (uint32_t)((n + TR_BLOCK - 1) / TR_BLOCK);
  const size_t sm = fwd_bwd_smem();
  KNNSJ_CUDA(cudaFuncSetAttribute(mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  mlp_fwd_bwd_kernel<<<nb, TR_BLOCK, sm, s>>>(d_model, d_X, d_Y, d_idx, n, quantile, inv_batch, d_part, d_part_loss);
  KNNSJ_CHECK_LAUNCH();
  grad_reduce_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(d_part, nb, d_grad);
  KNNSJ_CHECK_LAUNCH();
}

struct TrainBuffers {
  DevBuf model, X, Y, idx, part, ploss, grad, m1, m2;
};

// Seeded initial model: feature standardisation from the data, He-normal
// weights, zero biases, output bias at the target's `quantile` quantile.
void init_model(const float* X, const float* Y, uint64_t n, float quantile, uint64_t seed, float* model) {
  std::memset(model, 0, sizeof(float) * MODEL_FLOATS);
  for (int i = 0; i < NFEAT; i++) {
    double s = 0, s2 = 0;
    for (uint64_t r = 0; r < n; r++) {
      const double v = X[r * NFEAT + i];
      s += v;
      s2 += v * v;
    }
    const double mean = n ? s / n : 0.0;
    const double var = n ? std::max(0.0, s2 / n - mean * mean) : 0.0;
    model[M_MEAN + i] = (float)mean;
    model[M_ISTD + i] = (float)(var > 1e-12 ? 1.0 / std::sqrt(var) : 1.0);
  }
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  for (int i = 0; i < NFEAT * NHID; i++) model[M_W1 + i] = (float)(nd(rng) * std::sqrt(2.0 / NFEAT));
  for (int i = 0; i < NHID * NHID; i++) model[M_W2 + i] = (float)(nd(rng) * std::sqrt(2.0 / NHID));
  for (int i = 0; i < NHID; i++) model[M_W3 + i] = (float)(nd(rng) * std::sqrt(1.0 / NHID) * 0.1);
  if (n) {
    std::vector<float> ys(Y, Y + n);
    const size_t at = std::min<size_t>(n - 1, (size_t)(quantile * (n - 1)));
    std::nth_element(ys.begin(), ys.begin() + at, ys.end());
    model[M_B3] = ys[at];
  }
}

void train_model(const float* hX, const float* hY, uint64_t n, int epochs, uint32_t batch, float lr,
                 float quantile, uint64_t seed, float* model_out, float* loss_out, cudaStream_t s) {
  static TrainBuffers b;
  std::vector<float> model(MODEL_FLOATS);
  init_model(hX, hY, n, quantile, seed, model.data());
  float* d_model = (float*)b.model.get(MODEL_FLOATS * 4);
  float* d_X = (float*)b.X.get(n * NFEAT * 4);
  float* d_Y = (float*)b.Y.get(n * 4);
  uint32_t* d_idx = (uint32_t*)b.idx.get(n * 4);
  const uint32_t nbmax = (batch + TR_BLOCK - 1) / TR_BLOCK;
  float* d_part = (float*)b.part.get((size_t)nbmax * NPARAM * 4);
  double* d_pl = (double*)b.ploss.get((size_t)nbmax * 8);
  float* d_grad = (float*)b.grad.get(NPARAM * 4);
  float* d_m1 = (float*)b.m1.get(NPARAM * 4);
  float* d_m2 = (float*)b.m2.get(NPARAM * 4);
  KNNSJ_CUDA(cudaMemcpyAsync(d_model, model.data(), MODEL_FLOATS * 4, cudaMemcpyHostToDevice, s));
  KNNSJ_CUDA(cudaMemcpyAsync(d_X, hX, n * NFEAT * 4, cudaMemcpyHostToDevice, s));
  KNNSJ_CUDA(cudaMemcpyAsync(d_Y, hY, n * 4, cudaMemcpyHostToDevice, s));
  KNNSJ_CUDA(cudaMemsetAsync(d_m1, 0, NPARAM * 4, s));
  KNNSJ_CUDA(cudaMemsetAsync(d_m2, 0, NPARAM * 4, s));
  std::vector<uint32_t> perm(n);
  std::iota(perm.begin(), perm.end(), 0u);
  std::mt19937_64 rng(seed ^ 0x9e3779b97f4a7c15ull);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  int step = 0;
  std::vector<double> pl(nbmax);
  for (int e = 0; e < epochs; e++) {
    std::shuffle(perm.begin(), perm.end(), rng);
    KNNSJ_CUDA(cudaMemcpyAsync(d_idx, perm.data(), n * 4, cudaMemcpyHostToDevice, s));
    KNNSJ_CUDA(cudaStreamSynchronize(s));
    double epoch_loss = 0.0;
    for (uint64_t off = 0; off < n; off += batch) {
      const uint64_t nb = std::min<uint64_t>(batch, n - off);
      mlp_grad_device(d_model, d_X, d_Y, d_idx + off, nb, quantile, 1.0f / (float)nb, d_part, d_pl, d_grad, s);
      step++;
      const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
      adam_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(d_model + M_W1, d_grad, d_m1, d_m2, lr, b1, b2, eps, c1, c2);
      KNNSJ_CHECK_LAUNCH();
      const uint32_t nblk = (uint32_t)((nb + TR_BLOCK - 1) / TR_BLOCK);
      KNNSJ_CUDA(cudaMemcpyAsync(pl.data(), d_pl, nblk * 8, cudaMemcpyDeviceToHost, s));
      KNNSJ_CUDA(cudaStreamSynchronize(s));
      for (uint32_t i = 0; i < nblk; i++) epoch_loss += pl[i];
    }
    if (loss_out) loss_out[e] = (float)(epoch_loss / (double)n);
  }
  KNNSJ_CUDA(cudaMemcpyAsync(model_out, d_model, MODEL_FLOATS * 4, cudaMemcpyDeviceToHost, s));
  KNNSJ_CUDA(cudaStreamSynchronize(s));
}

}  // namespace knnsj
