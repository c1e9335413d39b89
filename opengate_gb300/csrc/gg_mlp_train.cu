// gg_mlp_train.cu - one training step of the ARF network on the 5th-generation
// tensor cores.
//
// Same network, loss and storage points as the inference kernels (garf ARF
// model, opengate/actors/arfactors.py:349-415; softmax cross-entropy on the
// (E, theta, phi, class) rows of GateARFTrainingDatasetActor).  One CTA (one
// warpgroup, 128 threads) takes a tile of 128 rows; thread r owns row r in the
// forward pass and unit r when it reads a weight gradient back.
//
//   forward: layer 1 on the CUDA cores; layers 2-4 as tcgen05.mma (M 128,
//     K 16 per instruction) from BF16 K-major operands into TMEM, epilogue per
//     thread (bias, ReLU, BF16) writing the next A operand [row][unit] and,
//     for H1 and H2, the transposed copy [unit][row]; ReLU masks stay in
//     registers;
//   output: softmax, loss, dL/dlogits = (p - onehot) / B in BF16 [row][class];
//   backward, per hidden layer l (dZ = BF16 gradient at the layer's output):
//     dW_l = dZ^T H_{l-1}: A = dZ^T [unit][row], B = H_{l-1}^T [unit][row],
//     dH_{l-1} = dZ W_l: A = dZ [row][unit], B = W_l^T (a bulk-loaded copy),
//     both issued back to back into two TMEM column ranges, one commit;
//     dW_l read back lane by lane into the tile's partial gradient; biases
//     and the small output / input layers on the CUDA cores.
// The per-tile gradients are summed in tile order by k_mlp_adam (gg_mlp.cu).
// Every mbarrier wait is bounded; a wait that runs out sets kStatusWaitTimeout
// and the tile stops (its tensor memory is freed).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_internal.h"
#include "gg_mlp.cuh"
#include "gg_mlp_tc.cuh"
#include "gg_tc.cuh"

namespace gg {

constexpr int kTrThreads = kTrainRows;             // one warpgroup
constexpr int kTrBytesDz4 = kTrainRows * kOutPad * 2;  // dL/dlogits, [row][class], K = 16

struct TrainSmem {
  alignas(1024) uint8_t w2[kTcBytesHid];  // forward W2 [out][in]; backward W2^T [in][out]
  alignas(1024) uint8_t w3[kTcBytesHid];  // forward W3; backward W3^T
  alignas(1024) uint8_t w4[kTcBytesOut];  // forward W4 [16][128]; backward W4^T [128][16]
  alignas(1024) uint8_t act[kTcBytesHid]; // [row][unit]: H1, H2, H3, then dZ3, dZ2
  alignas(1024) uint8_t h1t[kTcBytesHid]; // H1^T [unit][row]
  alignas(1024) uint8_t h2t[kTcBytesHid]; // H2^T
  alignas(1024) uint8_t dzt[kTcBytesHid]; // dZ^T [unit][row] of the current layer
  alignas(1024) uint8_t dz4[kTrBytesDz4]; // dL/dlogits [row][class]
  float w1[kHid * 3], b1[kHid], b2[kHid], b3[kHid], b4[kOutPad];
  float x[kTrainRows][3];
  float loss[kTrainRows];
  uint64_t mbar_mma, mbar_load;
  uint32_t tmem_base;
};

constexpr uint32_t kTrCols = 256;  // TMEM: columns [0, 128) dW / forward, [128, 256) dH

__device__ __forceinline__ uint32_t bf2_pack(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&h);
}

// Writes unit values v[0..31] (units col0 ..) of row r: BF16 into the A operand
// [row][unit] (16-byte stores) and, when t != nullptr, into the transposed
// operand [unit][row] (one element per unit).
__device__ __forceinline__ void tr_store32(uint8_t *act, uint8_t *t, int r, int col0, const float (&v)[32]) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = bf2_pack(v[8 * c + 2 * i], v[8 * c + 2 * i + 1]);
    *reinterpret_cast<uint4 *>(act + tc_offset(r, col0 + 8 * c, kHid)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  if (t) {
#pragma unroll
    for (int i = 0; i < 32; ++i)
      *reinterpret_cast<__nv_bfloat16 *>(t + tc_offset(col0 + i, r, kTrainRows)) = __float2bfloat16_rn(v[i]);
  }
}

// Sum over the tile's rows of row j of a transposed operand [unit][row].
__device__ __forceinline__ float tr_row_sum(const uint8_t *t, int j) {
  float s = 0.0f;
#pragma unroll 4
  for (int c = 0; c < kTrainRows / 8; ++c) {
    const uint4 q = *reinterpret_cast<const uint4 *>(t + tc_offset(j, 8 * c, kTrainRows));
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&q);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 f = __bfloat1622float2(h[i]);
      s += f.x;
      s += f.y;
    }
  }
  return s;
}

// Issues the MMAs of D (+)= A B^T, K = kk in steps of 16, into d_tmem (no commit).
__device__ __forceinline__ void tr_mma(uint32_t d_tmem, const uint8_t *a, const uint8_t *b, int n, int kk) {
  const uint32_t a0 = tc_smem(a), b0 = tc_smem(b), idesc = tc_idesc_bf16(kTrainRows, n);
  const uint32_t sbo = tc_sbo(kk);
  for (int ks = 0; ks < kk / 16; ++ks)
    tc_mma_bf16(d_tmem, tc_desc(a0 + 256u * ks, kTcLbo, sbo), tc_desc(b0 + 256u * ks, kTcLbo, sbo), idesc,
                ks > 0 ? 1u : 0u);
}

// Waits for MMA batch `phase` of the CTA; the result is the same for every thread.
__device__ __forceinline__ bool tr_wait(TrainSmem &sm, uint32_t &phase) {
  bool ok = mbar_wait(&sm.mbar_mma, phase & 1u, kTcWaitLimit);
  if (!ok) mbar_wait(&sm.mbar_mma, phase & 1u, kTcWaitLimit);  // let MMAs in flight finish
  ++phase;
  ok = __syncthreads_and(ok) != 0;
  tc_fence_after();
  return ok;
}

// Generic-proxy shared-memory writes visible to the tensor core, TMEM reads
// ordered, all threads past this point; then thread 0 may issue MMAs.
__device__ __forceinline__ void tr_publish() {
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
}


__global__ void __launch_bounds__(kTrThreads, 1) k_mlp_train(MlpTrainArgs a) {
  extern __shared__ __align__(1024) unsigned char tr_smem_raw[];
  TrainSmem &sm = *reinterpret_cast<TrainSmem *>(tr_smem_raw);
  const int t = threadIdx.x;  // row t (forward), unit t (gradient read-back)
  const int tile = blockIdx.x;
  float *part = a.partial + (size_t)tile * kNParams;
  const uint32_t tlane = (uint32_t)(32 * (t >> 5)) << 16;  // the warp's TMEM lane quarter

  // ---- set-up: mbarriers, forward weights (bulk copies), inputs, TMEM ----
  if (t == 0) {
    mbar_init(&sm.mbar_mma, 1u);
    mbar_init(&sm.mbar_load, 1u);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  const __nv_bfloat16 *wtc = a.wbf + kTcBf, *wtt = a.wbf + kTcTBf;
  if (t == 0) {
    mbar_expect_tx(&sm.mbar_load, (uint32_t)(2 * kTcBytesHid + kTcBytesOut));
    bulk_load(sm.w2, wtc + kBfW2, (uint32_t)kTcBytesHid, &sm.mbar_load);
    bulk_load(sm.w3, wtc + kBfW3, (uint32_t)kTcBytesHid, &sm.mbar_load);
    bulk_load(sm.w4, wtc + kBfW4, (uint32_t)kTcBytesOut, &sm.mbar_load);
  }
  for (int e = t; e < kHid * 3; e += kTrThreads) sm.w1[e] = a.params[kOffW1 + e];
  sm.b1[t] = a.params[kOffB1 + t];
  sm.b2[t] = a.params[kOffB2 + t];
  sm.b3[t] = a.params[kOffB3 + t];
  if (t < kOutPad) sm.b4[t] = a.params[kOffB4 + t];
  const float4 row = a.rows[(a.row0 + (uint64_t)tile * kTrainRows + (uint64_t)t) % a.n_rows];
  const float x0 = (row.y - a.mean[0]) * a.inv_std[0];
  const float x1 = (row.z - a.mean[1]) * a.inv_std[1];
  const float x2 = (row.x - a.mean[2]) * a.inv_std[2];
  const int y = (int)row.w;
  sm.x[t][0] = x0;
  sm.x[t][1] = x1;
  sm.x[t][2] = x2;
  if (t < 32) {
    tmem_alloc(&sm.tmem_base, kTrCols);
    tmem_relinquish();
  }
  bool ok = mbar_wait(&sm.mbar_load, 0u, kTcWaitLimit);
  if (!ok) mbar_wait(&sm.mbar_load, 0u, kTcWaitLimit);
  tc_fence_before();
  ok = __syncthreads_and(ok) != 0;
  tc_fence_after();
  const uint32_t d_a = sm.tmem_base, d_b = sm.tmem_base + 128u;
  uint32_t phase = 0;
  uint32_t mask1[4] = {0, 0, 0, 0}, mask2[4] = {0, 0, 0, 0}, mask3[4] = {0, 0, 0, 0};

  if (ok) {
    // ---- layer 1 (CUDA cores): H1 -> act, H1^T -> h1t ----
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float v[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int j = 32 * c + i;
        float z = sm.b1[j];
        z = fmaf(sm.w1[3 * j + 0], x0, z);
        z = fmaf(sm.w1[3 * j + 1], x1, z);
        z = fmaf(sm.w1[3 * j + 2], x2, z);
        const bool on = z > 0.0f;
        v[i] = on ? z : 0.0f;
        if (on) mask1[c] |= 1u << i;
      }
      tr_store32(sm.act, sm.h1t, t, 32 * c, v);
    }
    // ---- layers 2, 3 (tensor cores) ----
#pragma unroll 1
    for (int layer = 0; layer < 2 && ok; ++layer) {
      tr_publish();
      if (t == 0) {
        tc_fence_after();
        tr_mma(d_a, sm.act, layer == 0 ? sm.w2 : sm.w3, kHid, kHid);
        tc_commit(&sm.mbar_mma);
      }
      ok = tr_wait(sm, phase);
      if (!ok) break;
      const float *b = layer == 0 ? sm.b2 : sm.b3;
      uint32_t *mask = layer == 0 ? mask2 : mask3;
#pragma unroll 1
      for (int c = 0; c < 4; ++c) {
        float v[32];
        tmem_ld32(d_a + tlane + 32u * c, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float z = v[i] + b[32 * c + i];
          const bool on = z > 0.0f;
          v[i] = on ? z : 0.0f;
          if (on) mask[c] |= 1u << i;
        }
        tr_store32(sm.act, layer == 0 ? sm.h2t : nullptr, t, 32 * c, v);
      }
    }
  }
  if (ok) {
    // ---- output layer, softmax, loss, dL/dlogits ----
    tr_publish();
    if (t == 0) {
      tc_fence_after();
      tr_mma(d_a, sm.act, sm.w4, kOutPad, kHid);
      tc_commit(&sm.mbar_mma);
    }
    ok = tr_wait(sm, phase);
  }
  if (ok) {
    float p[16];
    {
      float v[16];
      tmem_ld16(d_a + tlane, v);
#pragma unroll
      for (int c = 0; c < 16; ++c) p[c] = v[c] + sm.b4[c];
    }
    tc_softmax(p, a.n_classes);
    float py = 1.0f;
#pragma unroll
    for (int c = 0; c < 16; ++c)
      if (c == y) py = p[c];
    sm.loss[t] = -logf(fmaxf(py, 1e-30f));
    uint32_t w[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      float g0 = 2 * c < a.n_classes ? (p[2 * c] - (2 * c == y ? 1.0f : 0.0f)) * a.inv_batch : 0.0f;
      float g1 = 2 * c + 1 < a.n_classes ? (p[2 * c + 1] - (2 * c + 1 == y ? 1.0f : 0.0f)) * a.inv_batch : 0.0f;
      w[c] = bf2_pack(g0, g1);
    }
    *reinterpret_cast<uint4 *>(sm.dz4 + tc_offset(t, 0, kOutPad)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4 *>(sm.dz4 + tc_offset(t, 8, kOutPad)) = make_uint4(w[4], w[5], w[6], w[7]);
    tc_fence_before();
    __syncthreads();
    // the backward weight copies replace the forward ones (all forward MMAs are complete)
    if (t == 0) {
      mbar_expect_tx(&sm.mbar_load, (uint32_t)(2 * kTcBytesHid + kTcBytesOut));
      bulk_load(sm.w2, wtt + kBfW2, (uint32_t)kTcBytesHid, &sm.mbar_load);
      bulk_load(sm.w3, wtt + kBfW3, (uint32_t)kTcBytesHid, &sm.mbar_load);
      bulk_load(sm.w4, wtt + kBfW4, (uint32_t)kTcBytesOut, &sm.mbar_load);
    }
    // ---- output layer gradients (CUDA cores): dW4[o][t] = sum_r dz4[r][o] H3[r][t], db4 ----
    float g[16];
#pragma unroll
    for (int o = 0; o < 16; ++o) g[o] = 0.0f;
#pragma unroll 2
    for (int r = 0; r < kTrainRows; ++r) {
      const float h = __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(sm.act + tc_offset(r, t, kHid)));
      const uint4 q0 = *reinterpret_cast<const uint4 *>(sm.dz4 + tc_offset(r, 0, kOutPad));
      const uint4 q1 = *reinterpret_cast<const uint4 *>(sm.dz4 + tc_offset(r, 8, kOutPad));
      const __nv_bfloat162 *d0 = reinterpret_cast<const __nv_bfloat162 *>(&q0);
      const __nv_bfloat162 *d1 = reinterpret_cast<const __nv_bfloat162 *>(&q1);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float2 f0 = __bfloat1622float2(d0[i]);
        const float2 f1 = __bfloat1622float2(d1[i]);
        g[2 * i] = fmaf(f0.x, h, g[2 * i]);
        g[2 * i + 1] = fmaf(f0.y, h, g[2 * i + 1]);
        g[8 + 2 * i] = fmaf(f1.x, h, g[8 + 2 * i]);
        g[8 + 2 * i + 1] = fmaf(f1.y, h, g[8 + 2 * i + 1]);
      }
    }
#pragma unroll
    for (int o = 0; o < 16; ++o) part[kOffW4 + o * kHid + t] = g[o];
    if (t < kOutPad) {
      float sb = 0.0f;
      for (int r = 0; r < kTrainRows; ++r)
        sb += __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(sm.dz4 + tc_offset(r, t, kOutPad)));
      part[kOffB4 + t] = sb;
    }
    ok = mbar_wait(&sm.mbar_load, 1u, kTcWaitLimit);
    if (!ok) mbar_wait(&sm.mbar_load, 1u, kTcWaitLimit);
    fence_async_smem();
    tc_fence_before();
    ok = __syncthreads_and(ok) != 0;  // every thread is done with H3 in act
  }
  if (ok) {
    // ---- dH3 = dL W4 (K = 16) ----
    if (t == 0) {
      tc_fence_after();
      tr_mma(d_b, sm.dz4, sm.w4, kHid, kOutPad);
      tc_commit(&sm.mbar_mma);
    }
    ok = tr_wait(sm, phase);
  }
  // ---- hidden layers 3, 2: dZ = dH * mask -> act and dzt; dW = dZ^T H_in, dH_in = dZ W ----
#pragma unroll 1
  for (int layer = 0; layer < 2 && ok; ++layer) {
    const uint32_t *mask = layer == 0 ? mask3 : mask2;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float v[32];
      tmem_ld32(d_b + tlane + 32u * c, v);
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = (mask[c] >> i) & 1u ? v[i] : 0.0f;
      tr_store32(sm.act, sm.dzt, t, 32 * c, v);
    }
    tr_publish();
    if (t == 0) {
      tc_fence_after();
      tr_mma(d_a, sm.dzt, layer == 0 ? sm.h2t : sm.h1t, kHid, kTrainRows);  // dW
      tr_mma(d_b, sm.act, layer == 0 ? sm.w3 : sm.w2, kHid, kHid);          // dH of the layer below
      tc_commit(&sm.mbar_mma);
    }
    ok = tr_wait(sm, phase);
    if (!ok) break;
    // dW (lane t = output unit t) and db into the tile's partial gradient
    const int off_w = layer == 0 ? kOffW3 : kOffW2, off_b = layer == 0 ? kOffB3 : kOffB2;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float v[32];
      tmem_ld32(d_a + tlane + 32u * c, v);
      float4 *dst = reinterpret_cast<float4 *>(part + off_w + t * kHid + 32 * c);
#pragma unroll
      for (int i = 0; i < 8; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    }
    part[off_b + t] = tr_row_sum(sm.dzt, t);
    __syncthreads();  // dzt and act are read; the next dZ may overwrite them
  }
  if (ok) {
    // ---- layer 1 (CUDA cores): dZ1 = dH1 * mask1 -> dzt; dW1[t][c] = sum_r dZ1[r][t] x[r][c], db1 ----
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float v[32];
      tmem_ld32(d_b + tlane + 32u * c, v);
#pragma unroll
      for (int i = 0; i < 32; ++i)
        *reinterpret_cast<__nv_bfloat16 *>(sm.dzt + tc_offset(32 * c + i, t, kTrainRows)) =
            __float2bfloat16_rn((mask1[c] >> i) & 1u ? v[i] : 0.0f);
    }
    __syncthreads();
    float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, gb = 0.0f;
#pragma unroll 4
    for (int r = 0; r < kTrainRows; ++r) {
      const float dz =
          __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(sm.dzt + tc_offset(t, r, kTrainRows)));
      g0 = fmaf(dz, sm.x[r][0], g0);
      g1 = fmaf(dz, sm.x[r][1], g1);
      g2 = fmaf(dz, sm.x[r][2], g2);
      gb += dz;
    }
    part[kOffW1 + 3 * t + 0] = g0;
    part[kOffW1 + 3 * t + 1] = g1;
    part[kOffW1 + 3 * t + 2] = g2;
    part[kOffB1 + t] = gb;
    if (t == 0) {
      float s = 0.0f;
      for (int r = 0; r < kTrainRows; ++r) s += sm.loss[r];
      a.loss_part[tile] = s;
    }
  }
  if (!ok && t == 0 && a.status) atomicOr(a.status, kStatusWaitTimeout);
  tc_fence_before();
  __syncthreads();
  if (t < 32) tmem_dealloc(sm.tmem_base, kTrCols);
}

size_t mlp_train_smem_bytes() { return sizeof(TrainSmem); }

cudaError_t launch_mlp_train(const MlpTrainArgs &a, int n_tiles, cudaStream_t st) {
  static unsigned long long configured = 0;
  cudaError_t e = configure_smem(k_mlp_train, (int)sizeof(TrainSmem), configured);
  if (e != cudaSuccess) return e;
  k_mlp_train<<<n_tiles, kTrThreads, sizeof(TrainSmem), st>>>(a);
  return cudaGetLastError();
}

}  // namespace gg
