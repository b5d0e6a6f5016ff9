// radius_model.cuh -- the learned starting radius: feature layout, model
// layout and the per-query device functions shared by inference (radius
// assignment before the first search pass) and training-data extraction.
//
// No counterpart in the reference: it starts every query at the same eps0
// (GPU.cu:3088-3566) and grows it by eps0/2 per pass (main.cu:336).  Here a
// small MLP predicts each query's radius from cell counts around it; the
// acceptance rule is unchanged (a query is accepted only with at least k+1
// points inside its searched radius), so results stay exact.
//
// Features (24 floats per query), all from the eps0 grid.  Let c_j be the
// query's cell along indexed dimension j, u_j = (x_j - min_j) / eps0, and
// m = min(NUMINDEXEDDIM, 2) the "shell" dimensions (the two of largest
// variance).  B1(R) is the block of cells with |c'_j - c_j| <= R for j < m
// and c'_j = c_j otherwise; B2(R) is the same on the grid of width 2*eps0
// (cell pairs 2C, 2C+1 along each shell dimension, C = c_j >> 1).
//   0..2   log1p of the points in B1(0), B1(1) \ B1(0), B1(2) \ B1(1)
//   3..5   the same for B2
//   6      d / 8          7  log(k)        8  NUMINDEXEDDIM / 8    9  m / 2
//   10..15 u_j - c_j - 1/2 for j < min(NUMINDEXEDDIM, 6), else 0
//   16..21 u_j/2 - (c_j >> 1) - 1/2 for j < min(NUMINDEXEDDIM, 6), else 0
//   22     BETA           23 reserved, 0
// Model (KNNSJ_MODEL_FLOATS floats): feature mean[24], feature 1/std[24],
// W1[24][64], b1[64], W2[64][64], b2[64], W3[64], b3; ReLU after layers 1
// and 2.  Output y estimates a high quantile of log(r_K / eps0), r_K being
// the distance to the (k+1)-th nearest point (self included).
#pragma once

#include "knnsj_device.cuh"

namespace knnsj {

constexpr int NFEAT = 24;
constexpr int NHID = 64;
constexpr int M_MEAN = 0;
constexpr int M_ISTD = M_MEAN + NFEAT;
constexpr int M_W1 = M_ISTD + NFEAT;
constexpr int M_B1 = M_W1 + NFEAT * NHID;
constexpr int M_W2 = M_B1 + NHID;
constexpr int M_B2 = M_W2 + NHID * NHID;
constexpr int M_W3 = M_B2 + NHID;
constexpr int M_B3 = M_W3 + NHID;
constexpr int MODEL_FLOATS = M_B3 + 1;  // 5873
static_assert(MODEL_FLOATS == 5873, "model layout");

// Dense or sparse cell table, as the search uses it.
template <typename T>
struct CellTable {
  GridGeom<T> g;
  const unsigned long long* ckeys;
  const uint32_t* coff;
  const uint32_t* dstart;
  unsigned long long C;
  int dense;
};

template <typename T>
__device__ __forceinline__ uint32_t table_run_count(const CellTable<T>& t, unsigned long long Llo,
                                                    unsigned long long Lhi) {
  if (Llo > Lhi) return 0;
  if (t.dense) return t.dstart[Lhi + 1] - t.dstart[Llo];
  unsigned long long lo = 0, hi = t.C;
  while (lo < hi) {
    const unsigned long long mid = (lo + hi) >> 1;
    if (t.ckeys[mid] < Llo) lo = mid + 1; else hi = mid;
  }
  const unsigned long long a = lo;
  hi = t.C;
  while (lo < hi) {
    const unsigned long long mid = (lo + hi) >> 1;
    if (t.ckeys[mid] < Lhi + 1) lo = mid + 1; else hi = mid;
  }
  return t.coff[lo] - t.coff[a];
}

// Points in the block [lo_j, hi_j] for j < m (m <= 2) with the other indexed
// dimensions fixed at the query's cell.
template <typename T>
__device__ __forceinline__ uint32_t block_count(const CellTable<T>& t, const uint32_t* c, uint32_t m,
                                                const uint32_t* lo, const uint32_t* hi) {
  unsigned long long fixed = 0;
  for (uint32_t j = m; j < t.g.di; j++) fixed += (unsigned long long)c[j] * t.g.mult[j];
  if (m <= 1) return table_run_count(t, fixed + lo[0], fixed + hi[0]);
  uint32_t s = 0;
  for (uint32_t r1 = lo[1]; r1 <= hi[1]; r1++) {
    const unsigned long long base = fixed + (unsigned long long)r1 * t.g.mult[1];
    s += table_run_count(t, base + lo[0], base + hi[0]);
  }
  return s;
}

// The 24 features of a query with coordinates q (indexed dims first).
template <typename T>
__device__ void radius_features(const CellTable<T>& t, const T* q, uint32_t d, uint32_t k, float beta, uint64_t n,
                                float* f) {
  const uint32_t di = t.g.di;
  const uint32_t m = di < 2 ? di : 2;
  uint32_t c[MAX_DI];
  float u[MAX_DI];
  for (uint32_t j = 0; j < di; j++) {
    const T uj = Num<T>::div(Num<T>::sub(q[j], t.g.minv[j]), t.g.width);
    const uint32_t cj = clamped_cell(q[j], t.g.minv[j], t.g.width, t.g.ncell[j]);
    c[j] = cj;
    u[j] = (float)uj;
  }
  uint32_t cnt1[3], cnt2[3];
  for (int R = 0; R < 3; R++) {
    uint32_t lo[2], hi[2];
    for (uint32_t j = 0; j < m; j++) {
      const int n1 = (int)t.g.ncell[j];
      lo[j] = (uint32_t)max(0, (int)c[j] - R);
      hi[j] = (uint32_t)min(n1 - 1, (int)c[j] + R);
    }
    cnt1[R] = block_count(t, c, m, lo, hi);
    for (uint32_t j = 0; j < m; j++) {
      const int n1 = (int)t.g.ncell[j];
      const int C = (int)(c[j] >> 1);
      lo[j] = (uint32_t)max(0, 2 * (C - R));
      hi[j] = (uint32_t)min(n1 - 1, 2 * (C + R) + 1);
    }
    cnt2[R] = block_count(t, c, m, lo, hi);
  }
  f[0] = log1pf((float)cnt1[0]);
  f[1] = log1pf((float)(cnt1[1] - cnt1[0]));
  f[2] = log1pf((float)(cnt1[2] - cnt1[1]));
  f[3] = log1pf((float)cnt2[0]);
  f[4] = log1pf((float)(cnt2[1] - cnt2[0]));
  f[5] = log1pf((float)(cnt2[2] - cnt2[1]));
  f[6] = (float)d / 8.0f;
  f[7] = logf((float)(k > 0 ? k : 1));
  f[8] = (float)di / 8.0f;
  f[9] = (float)m / 2.0f;
  for (int j = 0; j < 6; j++) {
    float a = 0.0f, b = 0.0f;
    if (j < (int)di) {
      a = (u[j] - (float)c[j]) - 0.5f;
      b = 0.5f * ((float)(c[j] & 1u) + (u[j] - (float)c[j])) - 0.5f;
    }
    f[10 + j] = a;
    f[16 + j] = b;
  }
  f[22] = beta;
  f[23] = 0.0f;  // reserved (kept 0 so models stay independent of N)
  (void)n;
}

// Model output for one feature vector (one thread).  Every sum runs in a
// fixed order: first layer h = b1 + sum_i x_i W1[i][h] (i ascending), second
// layer a = b2 + sum_i relu(h_i) W2[i][o] (i ascending), y = b3 + sum_o
// relu(a_o) W3[o] (o ascending), so the training kernels and a numpy
// restatement reproduce it.  The loops are turned so that the weights are
// read as vector rows: the 64 second-layer sums stay in registers while the
// first layer is produced 16 hidden units at a time and consumed at once.
// The model must be 16-byte aligned (shared memory in practice).
__device__ __forceinline__ float mlp_eval_blocked(const float* __restrict__ model, const float* f) {
  float x[NFEAT];
#pragma unroll
  for (int i = 0; i < NFEAT; i++) x[i] = (f[i] - model[M_MEAN + i]) * model[M_ISTD + i];
  float a[NHID];
#pragma unroll
  for (int o = 0; o < NHID; o++) a[o] = model[M_B2 + o];
#pragma unroll 1
  for (int hc = 0; hc < NHID; hc += 16) {
    float h1[16];
#pragma unroll
    for (int h = 0; h < 16; h++) h1[h] = model[M_B1 + hc + h];
#pragma unroll
    for (int i = 0; i < NFEAT; i++) {
      const float4* w = reinterpret_cast<const float4*>(model + M_W1 + i * NHID + hc);
#pragma unroll
      for (int h4 = 0; h4 < 4; h4++) {
        const float4 wv = w[h4];
        h1[4 * h4 + 0] = fmaf(x[i], wv.x, h1[4 * h4 + 0]);
        h1[4 * h4 + 1] = fmaf(x[i], wv.y, h1[4 * h4 + 1]);
        h1[4 * h4 + 2] = fmaf(x[i], wv.z, h1[4 * h4 + 2]);
        h1[4 * h4 + 3] = fmaf(x[i], wv.w, h1[4 * h4 + 3]);
      }
    }
#pragma unroll
    for (int h = 0; h < 16; h++) {
      const float hv = fmaxf(h1[h], 0.0f);
      const float4* w = reinterpret_cast<const float4*>(model + M_W2 + (hc + h) * NHID);
#pragma unroll
      for (int o4 = 0; o4 < NHID / 4; o4++) {
        const float4 wv = w[o4];
        a[4 * o4 + 0] = fmaf(hv, wv.x, a[4 * o4 + 0]);
        a[4 * o4 + 1] = fmaf(hv, wv.y, a[4 * o4 + 1]);
        a[4 * o4 + 2] = fmaf(hv, wv.z, a[4 * o4 + 2]);
        a[4 * o4 + 3] = fmaf(hv, wv.w, a[4 * o4 + 3]);
      }
    }
  }
  float y = model[M_B3];
#pragma unroll
  for (int o = 0; o < NHID; o++) y = fmaf(fmaxf(a[o], 0.0f), model[M_W3 + o], y);
  return y;
}

}  // namespace knnsj
