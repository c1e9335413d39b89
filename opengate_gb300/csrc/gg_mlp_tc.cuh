// gg_mlp_tc.cuh - ARF network forward on the 5th-generation tensor cores.
//
// Same network and parameter layout as gg_mlp.cuh (garf ARF model of the
// reference's ARFActor, opengate/actors/arfactors.py:349-415).  A CTA holds the
// BF16 weights of layers 2-4 once, as tcgen05 B operands (K-major core
// matrices, gg_tc.cuh), and runs kTcGroups independent warpgroups.  A
// warpgroup evaluates a tile of 128 rows, one row per thread:
//   layer 1 (3 inputs) on the CUDA cores, written as the BF16 A operand;
//   layers 2-4: one thread issues 8 tcgen05.mma (K = 16 each, M = 128,
//   N = 128 or 16) into the group's 128 TMEM columns and commits to the
//   group's mbarrier; after the wait every thread reads its own row from TMEM
//   (tcgen05.ld 32x32b), adds the bias, applies ReLU and writes the next A
//   operand in place;
//   the output layer leaves each thread with its row's 16 logits, so the
//   softmax needs no exchange between threads.
// Groups synchronise with named barriers only, so they overlap each other's
// MMA and epilogue phases.  Every wait is bounded; a wait that runs out ends
// the group's work with an error status.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_mlp.cuh"
#include "gg_tc.cuh"

namespace gg {

constexpr int kTcGroups = 4;                         // warpgroups per CTA
constexpr int kTcRows = 128;                         // rows per warpgroup tile (MMA M)
constexpr int kTcThreads = 128 * kTcGroups;          // threads per CTA
constexpr uint32_t kTcCols = 128u * kTcGroups;       // TMEM columns (power of two, <= 512)
constexpr uint32_t kTcWaitLimit = 1u << 22;          // mbarrier tries before a wait gives up
constexpr int kTcBytesHid = kHid * kHid * 2;         // one 128 x 128 BF16 operand
constexpr int kTcBytesOut = kOutPad * kHid * 2;      // the 16 x 128 output-layer operand

struct TcNetSmem {
  alignas(1024) uint8_t w2[kTcBytesHid];             // B operands: W[out][in], K = in
  alignas(1024) uint8_t w3[kTcBytesHid];
  alignas(1024) uint8_t w4[kTcBytesOut];
  alignas(1024) uint8_t act[kTcGroups][kTcBytesHid]; // A operand of each group: [row][unit]
  float w1[kHid * 3], b1[kHid], b2[kHid], b3[kHid], b4[kOutPad];
  uint64_t mbar[kTcGroups];
  uint64_t mbar_load;                                 // bulk copy of the weight operands
  unsigned long long claim[kTcGroups];
  uint32_t tmem_base;
};

// Named barrier of the 128 threads of a group that also returns whether any of
// them passed pred = true (bar.red.or).
__device__ __forceinline__ bool named_bar_any(int id, int count, bool pred) {
  uint32_t out;
  asm volatile(
      "{\n"
      ".reg .pred p, q;\n"
      "setp.ne.u32 p, %1, 0;\n"
      "bar.red.or.pred q, %2, %3, p;\n"
      "selp.u32 %0, 1, 0, q;\n"
      "}\n"
      : "=r"(out)
      : "r"((uint32_t)pred), "r"(id), "r"(count)
      : "memory");
  return out != 0u;
}

// Weights into shared memory and the CTA's tensor memory; every thread of the
// CTA calls it.  W2, W3, W4 arrive as three bulk asynchronous copies of their
// tensor-core copies (`wtc`, the K-major core-matrix layout, 16-byte aligned)
// completing on one mbarrier; layer 1 and the biases are plain FP32 loads.
// Warp 0 allocates kTcCols TMEM columns.  False (for every thread) when the
// copies did not complete within the bounded wait.
__device__ __forceinline__ bool tc_net_prepare(TcNetSmem &sm, const float *params, const __nv_bfloat16 *wtc) {
  if (threadIdx.x == 0) {
#pragma unroll
    for (int g = 0; g < kTcGroups; ++g) mbar_init(&sm.mbar[g], 1u);
    mbar_init(&sm.mbar_load, 1u);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&sm.mbar_load, (uint32_t)(2 * kTcBytesHid + kTcBytesOut));
    bulk_load(sm.w2, wtc + kBfW2, (uint32_t)kTcBytesHid, &sm.mbar_load);
    bulk_load(sm.w3, wtc + kBfW3, (uint32_t)kTcBytesHid, &sm.mbar_load);
    bulk_load(sm.w4, wtc + kBfW4, (uint32_t)kTcBytesOut, &sm.mbar_load);
  }
  for (int e = threadIdx.x; e < kHid * 3; e += blockDim.x) sm.w1[e] = params[kOffW1 + e];
  for (int e = threadIdx.x; e < kHid; e += blockDim.x) {
    sm.b1[e] = params[kOffB1 + e];
    sm.b2[e] = params[kOffB2 + e];
    sm.b3[e] = params[kOffB3 + e];
  }
  for (int e = threadIdx.x; e < kOutPad; e += blockDim.x) sm.b4[e] = params[kOffB4 + e];
  if (threadIdx.x < 32) {
    tmem_alloc(&sm.tmem_base, kTcCols);
    tmem_relinquish();
  }
  bool ok = mbar_wait(&sm.mbar_load, 0u, kTcWaitLimit);
  if (!ok) mbar_wait(&sm.mbar_load, 0u, kTcWaitLimit);  // let the copies land before the CTA can leave
  tc_fence_before();
  ok = __syncthreads_and(ok) != 0;
  tc_fence_after();
  return ok;
}

// Frees the TMEM columns; every thread of the CTA calls it once its group is done.
__device__ __forceinline__ void tc_net_teardown(TcNetSmem &sm) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32) tmem_dealloc(sm.tmem_base, kTcCols);
}

// Bias + ReLU of 32 accumulator columns (col0 ..) of row r into the A operand.
__device__ __forceinline__ void tc_store_relu32(uint8_t *act, int r, int col0, const float (&v)[32], const float *b) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int j = col0 + 8 * c + 2 * i;
      const float z0 = v[8 * c + 2 * i] + b[j];
      const float z1 = v[8 * c + 2 * i + 1] + b[j + 1];
      __nv_bfloat162 h = __floats2bfloat162_rn(z0 > 0.0f ? z0 : 0.0f, z1 > 0.0f ? z1 : 0.0f);
      w[i] = *reinterpret_cast<uint32_t *>(&h);
    }
    *reinterpret_cast<uint4 *>(act + tc_offset(r, col0 + 8 * c, kHid)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// One layer's MMAs (K = 128 in 8 steps) into the group's TMEM columns, then a commit to its mbarrier.
__device__ __forceinline__ void tc_issue_layer(uint32_t d_tmem, const uint8_t *a, const uint8_t *b, int n,
                                               uint64_t *mbar) {
  tc_fence_after();
  const uint32_t a0 = tc_smem(a), b0 = tc_smem(b), idesc = tc_idesc_bf16(kTcRows, n);
#pragma unroll
  for (int ks = 0; ks < kHid / 16; ++ks)
    tc_mma_bf16(d_tmem, tc_desc(a0 + 256u * ks, kTcLbo, tc_sbo(kHid)), tc_desc(b0 + 256u * ks, kTcLbo, tc_sbo(kHid)),
                idesc, ks > 0 ? 1u : 0u);
  tc_commit(mbar);
}

// Network forward for group g's tile: thread r (0..127 inside the group)
// holds row r, inputs x0..x2 already standardised; on return logit[c] holds
// its row's output-layer value (bias included) for c < 16.  `phase` counts
// the group's completed MMA batches (the mbarrier parity).  Every thread of
// the group calls it; false (for the whole group) when a wait ran out.
__device__ __forceinline__ bool tc_net_forward(TcNetSmem &sm, int g, int r, uint32_t &phase, float x0, float x1,
                                               float x2, float (&logit)[16]) {
  uint8_t *act = sm.act[g];
  const int bar = 1 + g;
  const uint32_t tcol = sm.tmem_base + 128u * (uint32_t)g;
  const uint32_t tlane = (uint32_t)(32 * ((threadIdx.x >> 5) & 3)) << 16;
  // layer 1: row r of the A operand
#pragma unroll 4
  for (int j0 = 0; j0 < kHid; j0 += 8) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int j = j0 + 2 * i;
      float z0 = sm.b1[j];
      z0 = fmaf(sm.w1[3 * j + 0], x0, z0);
      z0 = fmaf(sm.w1[3 * j + 1], x1, z0);
      z0 = fmaf(sm.w1[3 * j + 2], x2, z0);
      float z1 = sm.b1[j + 1];
      z1 = fmaf(sm.w1[3 * j + 3], x0, z1);
      z1 = fmaf(sm.w1[3 * j + 4], x1, z1);
      z1 = fmaf(sm.w1[3 * j + 5], x2, z1);
      __nv_bfloat162 h = __floats2bfloat162_rn(z0 > 0.0f ? z0 : 0.0f, z1 > 0.0f ? z1 : 0.0f);
      w[i] = *reinterpret_cast<uint32_t *>(&h);
    }
    *reinterpret_cast<uint4 *>(act + tc_offset(r, j0, kHid)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
#pragma unroll 1
  for (int layer = 0; layer < 3; ++layer) {
    fence_async_smem();
    tc_fence_before();
    named_bar(bar, kTcRows);
    if (r == 0)
      tc_issue_layer(tcol, act, layer == 0 ? sm.w2 : (layer == 1 ? sm.w3 : sm.w4), layer == 2 ? kOutPad : kHid,
                     &sm.mbar[g]);
    const bool ok = mbar_wait(&sm.mbar[g], phase & 1u, kTcWaitLimit);
    ++phase;
    if (named_bar_any(bar, kTcRows, !ok)) {
      // let the MMAs in flight finish (bounded) before the caller frees TMEM
      mbar_wait(&sm.mbar[g], (phase - 1u) & 1u, kTcWaitLimit);
      return false;
    }
    tc_fence_after();
    if (layer < 2) {
      const float *b = layer == 0 ? sm.b2 : sm.b3;
#pragma unroll 1
      for (int c = 0; c < 4; ++c) {
        float v[32];
        tmem_ld32(tcol + tlane + 32u * c, v);
        tc_store_relu32(act, r, 32 * c, v, b);
      }
    } else {
      float v[16];
      tmem_ld16(tcol + tlane, v);
#pragma unroll
      for (int c = 0; c < 16; ++c) logit[c] = v[c] + sm.b4[c];
    }
  }
  tc_fence_before();
  return true;
}

// Softmax over the first n_classes logits of one row (in place; the rest 0).
__device__ __forceinline__ void tc_softmax(float (&p)[16], int n_classes) {
  float mx = -INFINITY;
#pragma unroll
  for (int c = 0; c < 16; ++c)
    if (c < n_classes) mx = fmaxf(mx, p[c]);
  float sum = 0.0f;
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    p[c] = c < n_classes ? expf(p[c] - mx) : 0.0f;
    sum += p[c];
  }
  const float inv = 1.0f / sum;
#pragma unroll
  for (int c = 0; c < 16; ++c) p[c] *= inv;
}

}  // namespace gg
