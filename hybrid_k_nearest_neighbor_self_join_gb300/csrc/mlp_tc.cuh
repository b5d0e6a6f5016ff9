// mlp_tc.cuh -- the radius MLP (24 -> 64 -> 64 -> 1, radius_model.cuh) on
// the 5th-generation tensor cores: tcgen05.mma with BF16 operands in shared
// memory and FP32 accumulators in tensor memory (TMEM).
//
// A CTA of 128 threads evaluates 128 queries at a time (one query = one row
// of the MMA's M = 128, one thread per row):
//   1. each thread writes its query's normalised features, BF16, into row r
//      of A1 (128 x 32, the 24 features padded with zeros);
//   2. one elected thread issues D = A1 . W1 (two K = 16 MMAs, N = 64) into
//      64 TMEM columns and commits them to an mbarrier;
//   3. every warp reads its 32 TMEM lanes (tcgen05.ld 32x32b), adds b1,
//      applies ReLU and writes the row, BF16, into A2 (128 x 64);
//   4. D = A2 . W2 (four K = 16 MMAs) into the same TMEM columns;
//   5. every thread reads its row, adds b2, applies ReLU and takes the dot
//      product with W3 plus b3 in FP32: its query's log-radius.
// W1 and W2 are converted to BF16 once per CTA; CTAs are persistent over
// tiles.  Operands use the no-swizzle K-major layout of 8 x 16-byte core
// matrices: byte offset ((row/8) * (K/8) + k/8) * 128 + (row%8) * 16 +
// (k%8) * 2, so consecutive K core matrices are 128 bytes apart (leading
// byte offset) and consecutive 8-row groups K/8 * 128 bytes apart (stride
// byte offset).
//
// Every wait on the mbarrier is bounded.  The parity a wait uses flips only
// after every thread of the CTA saw that phase complete, so after a timeout
// `phase` still names the commit that has not been seen to complete.  On a
// timeout the CTA records an error (1), falls back to the plain eps0 radius
// for its queries (any radius gives exact results), waits once more, bounded,
// on that same phase when a commit is in flight -- recording error 2 if the
// tensor core still has not finished -- then frees its TMEM and stops.
// TcCtl::no_issue (a test switch) makes thread 0 skip the MMAs and their
// commit: nothing is then in flight, and the first bounded wait runs out.
#pragma once

#include <cuda_bf16.h>

#include "radius_model.cuh"

namespace knnsj {

constexpr int TC_ROWS = 128;   // queries per tile = MMA M
constexpr int TC_K1 = 32;      // features padded to two K = 16 steps
constexpr int TC_TMEM_COLS = 64;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;  // mbarrier polls before giving up

// Wait bound and the test switch of one launch.
struct TcCtl {
  uint32_t wait_limit = TC_WAIT_LIMIT;  // mbarrier polls before a wait gives up
  uint32_t no_issue = 0;                // 1: issue no MMA and no commit (tests the timeout path)
};

// shared memory of one CTA (bytes)
constexpr int TC_OFF_A1 = 0;                          // 128 x 32 bf16
constexpr int TC_OFF_A2 = TC_OFF_A1 + TC_ROWS * TC_K1 * 2;  // 128 x 64 bf16
constexpr int TC_OFF_B1 = TC_OFF_A2 + TC_ROWS * NHID * 2;   // 64 x 32 bf16
constexpr int TC_OFF_B2 = TC_OFF_B1 + NHID * TC_K1 * 2;     // 64 x 64 bf16
constexpr int TC_OFF_P = TC_OFF_B2 + NHID * NHID * 2;       // fp32: mean, istd, b1, b2, w3, b3
constexpr int TC_NPARAM = 2 * NFEAT + 3 * NHID + 1;
constexpr int TC_OFF_BAR = TC_OFF_P + ((TC_NPARAM * 4 + 15) / 16) * 16;
constexpr int TC_SMEM = TC_OFF_BAR + 16;

__device__ __forceinline__ uint32_t tc_cm_off(uint32_t row, uint32_t k, uint32_t kchunks) {
  return (((row >> 3) * kchunks + (k >> 3)) << 7) + ((row & 7u) << 4) + ((k & 7u) << 1);
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all in 16-byte units), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 64, M = 128.
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NHID >> 3) << 17) |
                              ((uint32_t)(TC_ROWS >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// Polls the mbarrier for the given phase parity; false after `limit` polls.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t phase, uint32_t limit) {
  for (uint32_t it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_proxy() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ uint32_t tc_saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Writes 8 consecutive K values of one row (16 bytes) of a BF16 operand.
__device__ __forceinline__ void tc_put8(unsigned char* base, uint32_t row, uint32_t k0, uint32_t kchunks,
                                        const float* v) {
  __nv_bfloat162 h[4];
#pragma unroll
  for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
  *reinterpret_cast<uint4*>(base + tc_cm_off(row, k0, kchunks)) = *reinterpret_cast<uint4*>(h);
}

// The MLP over persistent tiles.  Src supplies, for query i < n, its 24 raw
// features (features(i, f)) and receives its log-radius (store(i, y)) or,
// after a timeout, the fallback (fallback(i)).
template <typename Src>
__device__ void mlp_tc_tiles(Src& src, const float* __restrict__ model, uint64_t n, uint32_t* err, TcCtl ctl) {
  __shared__ __align__(128) unsigned char sm[TC_SMEM];
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  float* prm = reinterpret_cast<float*>(sm + TC_OFF_P);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + TC_OFF_BAR + 8);
  const uint32_t bar = tc_saddr(sm + TC_OFF_BAR);
  // weights: W1 (n = hidden, k = feature) and W2 (n = output, k = hidden), BF16
  for (uint32_t e = tid; e < NHID * (TC_K1 / 8); e += blockDim.x) {
    const uint32_t h = e / (TC_K1 / 8), k0 = (e % (TC_K1 / 8)) * 8;
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = (k0 + i) < (uint32_t)NFEAT ? model[M_W1 + (k0 + i) * NHID + h] : 0.0f;
    tc_put8(sm + TC_OFF_B1, h, k0, TC_K1 / 8, v);
  }
  for (uint32_t e = tid; e < NHID * (NHID / 8); e += blockDim.x) {
    const uint32_t o = e / (NHID / 8), k0 = (e % (NHID / 8)) * 8;
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = model[M_W2 + (k0 + i) * NHID + o];
    tc_put8(sm + TC_OFF_B2, o, k0, NHID / 8, v);
  }
  for (uint32_t e = tid; e < (uint32_t)TC_NPARAM; e += blockDim.x) {
    float v;
    if (e < 2 * NFEAT) v = model[M_MEAN + e];  // mean, istd
    else if (e < 2 * NFEAT + NHID) v = model[M_B1 + (e - 2 * NFEAT)];
    else if (e < 2 * NFEAT + 2 * NHID) v = model[M_B2 + (e - 2 * NFEAT - NHID)];
    else if (e < 2 * NFEAT + 3 * NHID) v = model[M_W3 + (e - 2 * NFEAT - 2 * NHID)];
    else v = model[M_B3];
    prm[e] = v;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_saddr(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_addr = tmem + ((warp * 32u) << 16);
  const float* mean = prm;
  const float* istd = prm + NFEAT;
  const float* b1 = prm + 2 * NFEAT;
  const float* b2 = b1 + NHID;
  const float* w3 = b2 + NHID;
  const float b3 = w3[NHID];
  const uint32_t a1 = tc_saddr(sm + TC_OFF_A1), a2 = tc_saddr(sm + TC_OFF_A2);
  const uint32_t bb1 = tc_saddr(sm + TC_OFF_B1), bb2 = tc_saddr(sm + TC_OFF_B2);
  uint32_t phase = 0;       // parity of the next completion to wait for
  bool inflight = false;    // a commit has been issued whose completion was not yet seen by all
  bool failed = false;
  const uint64_t ntiles = (n + TC_ROWS - 1) / TC_ROWS;
  uint64_t tile = blockIdx.x;
  for (; tile < ntiles && !failed; tile += gridDim.x) {
    const uint64_t i = tile * TC_ROWS + tid;
    const bool valid = i < n;
    // 1. normalised features, row tid of A1
    {
      float f[TC_K1];
#pragma unroll
      for (int j = 0; j < TC_K1; j++) f[j] = 0.0f;
      if (valid) {
        float raw[NFEAT];
        src.features(i, raw);
#pragma unroll
        for (int j = 0; j < NFEAT; j++) f[j] = (raw[j] - mean[j]) * istd[j];
      }
#pragma unroll
      for (int c = 0; c < TC_K1 / 8; c++) tc_put8(sm + TC_OFF_A1, tid, c * 8, TC_K1 / 8, f + c * 8);
    }
    tc_fence_proxy();
    tc_fence_before();
    __syncthreads();
    // 2. first layer
    if (tid == 0 && !ctl.no_issue) {
      tc_fence_after();
#pragma unroll
      for (int s = 0; s < TC_K1 / 16; s++)
        tc_mma(tmem, tc_desc(a1 + s * 256, 128, (TC_K1 / 8) * 128), tc_desc(bb1 + s * 256, 128, (TC_K1 / 8) * 128),
               s > 0);
      tc_commit(bar);
    }
    inflight = !ctl.no_issue;
    bool ok = tc_wait(bar, phase, ctl.wait_limit);
    ok = __syncthreads_and(ok);  // uniform: tcgen05.ld is warp-collective
    if (ok) {                    // every thread saw this phase complete
      phase ^= 1u;
      inflight = false;
    }
    tc_fence_after();
    // 3. ReLU(h + b1) into A2
    if (ok) {
#pragma unroll
      for (int c = 0; c < NHID / 16; c++) {
        float h[16];
        tc_ld16(lane_addr + c * 16, h);
        tc_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; j++) h[j] = fmaxf(h[j] + b1[c * 16 + j], 0.0f);
        tc_put8(sm + TC_OFF_A2, tid, c * 16, NHID / 8, h);
        tc_put8(sm + TC_OFF_A2, tid, c * 16 + 8, NHID / 8, h + 8);
      }
    }
    tc_fence_proxy();
    tc_fence_before();
    ok = __syncthreads_and(ok);
    // 4. second layer, into the same TMEM columns
    if (ok && tid == 0 && !ctl.no_issue) {
      tc_fence_after();
#pragma unroll
      for (int s = 0; s < NHID / 16; s++)
        tc_mma(tmem, tc_desc(a2 + s * 256, 128, (NHID / 8) * 128), tc_desc(bb2 + s * 256, 128, (NHID / 8) * 128),
               s > 0);
      tc_commit(bar);
    }
    if (ok) {  // (ok is uniform here: every thread takes this branch or none)
      inflight = !ctl.no_issue;
      const bool seen = __syncthreads_and(tc_wait(bar, phase, ctl.wait_limit));
      if (seen) {
        phase ^= 1u;
        inflight = false;
      }
      ok = seen;
    }
    ok = __syncthreads_and(ok);
    tc_fence_after();
    // 5. y = b3 + sum relu(a + b2) w3
    if (ok) {
      float y = b3;
#pragma unroll
      for (int c = 0; c < NHID / 16; c++) {
        float a[16];
        tc_ld16(lane_addr + c * 16, a);
        tc_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; j++) y = fmaf(fmaxf(a[j] + b2[c * 16 + j], 0.0f), w3[c * 16 + j], y);
      }
      if (valid) src.store(i, y);
    }
    tc_fence_before();
    ok = __syncthreads_and(ok);
    if (!ok) {
      // an MMA did not complete in time: plain radius for this tile, error
      // recorded; if a commit is in flight, one more bounded wait on the
      // phase that timed out (so that TMEM is freed only once the tensor core
      // is done with it), then stop
      if (valid) src.fallback(i);
      if (tid == 0) atomicMax(err, 1u);
      if (inflight) {
        const bool drained = __syncthreads_and(tc_wait(bar, phase, ctl.wait_limit));
        if (!drained && tid == 0) atomicMax(err, 2u);  // TMEM released with the MMA unconfirmed
        inflight = false;
      }
      failed = true;
    }
  }
  // the remaining tiles of a failed CTA get the fallback too (the loop has
  // already stepped past the failed tile)
  if (failed) {
    for (; tile < ntiles; tile += gridDim.x) {
      const uint64_t i = tile * TC_ROWS + tid;
      if (i < n) src.fallback(i);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

}  // namespace knnsj
