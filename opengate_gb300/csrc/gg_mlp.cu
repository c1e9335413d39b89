// gg_mlp.cu - training and batch inference of the ARF network.
//
// One training step over a batch of B rows (B a multiple of kTileM):
//   k_mlp_train: one CTA per tile of kTileM rows - forward pass, softmax
//     cross-entropy, and the backward pass of every layer; each CTA writes
//     its tile's parameter gradient (FP32, all kNParams) and loss sum;
//   k_mlp_adam: one thread per parameter - the tile gradients summed in tile
//     order (deterministic), Adam update of the FP32 parameters, and the BF16
//     copies of W2 / W3 / W4 refreshed for the next step.
// The weight-gradient GEMMs reduce over the tile's samples on the tensor
// cores (dW = dZ^T H: both operands read transposed by ldmatrix.trans).
// Batch inference (k_mlp_predict) runs the forward pass on tcgen05 (gg_mlp_tc.cuh).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_internal.h"
#include "gg_mlp.cuh"
#include "gg_mlp_tc.cuh"

namespace gg {

// Input features of a row: standardised (theta, phi, E); class label.
__device__ __forceinline__ void mlp_tile_inputs(MlpSmem &sm, const float4 *rows, uint64_t row0, uint64_t n_rows,
                                                const MlpTrainArgs &a) {
  for (int r = threadIdx.x; r < kTileM; r += blockDim.x) {
    const float4 v = rows[(row0 + (uint64_t)r) % n_rows];
    sm.x[r][0] = (v.y - a.mean[0]) * a.inv_std[0];
    sm.x[r][1] = (v.z - a.mean[1]) * a.inv_std[1];
    sm.x[r][2] = (v.x - a.mean[2]) * a.inv_std[2];
    sm.y[r] = (int)v.w;
  }
}

__global__ void __launch_bounds__(kMlpThreads) k_mlp_train(MlpTrainArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpSmem &sm = *reinterpret_cast<MlpSmem *>(smem_raw);
  const int warp = threadIdx.x >> 5;
  const int m0 = 16 * warp;
  const int tile = blockIdx.x;
  float *part = a.partial + (size_t)tile * kNParams;

  mlp_load_weights(sm, a.params, a.wbf);
  mlp_tile_inputs(sm, a.rows, a.row0 + (uint64_t)tile * kTileM, a.n_rows, a);
  __syncthreads();
  // ---- forward ----
  mlp_layer1(sm);
  __syncthreads();
  mlp_hidden(sm.h1, sm.w2, sm.b2, sm.h2);
  __syncthreads();
  mlp_hidden(sm.h2, sm.w3, sm.b3, sm.h3);
  __syncthreads();
  {
    float acc[1][2][4];
    mlp_logits(sm, acc);
    mlp_softmax(acc, a.n_classes);
    // dL/dlogit = (p - onehot(y)) / B; the loss of row r is -log p[y]
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int rr, cc;
        acc_pos(q, rr, cc);
        const int row = m0 + rr, col = 8 * nt + cc;
        const float p = acc[0][nt][q];
        const bool hit = col == sm.y[row];
        if (hit) sm.loss[row] = -logf(fmaxf(p, 1e-30f));
        const float g = col < a.n_classes ? (p - (hit ? 1.0f : 0.0f)) * a.inv_batch : 0.0f;
        sm.dl[row * 24 + col] = __float2bfloat16_rn(g);
      }
  }
  __syncthreads();
  // ---- backward ----
  // output layer: dW4 = dl^T h3 (16 x 128), db4 = column sums of dl
  {
    float acc[1][4][4];
    zero_acc(acc);
    warp_gemm<1, 4, true, true>(acc, sm.dl, 24, 0, sm.h3, kLds, 32 * warp, kTileM);
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int rr, cc;
        acc_pos(q, rr, cc);
        part[kOffW4 + rr * kHid + 32 * warp + 8 * nt + cc] = acc[0][nt][q];
      }
    if (threadIdx.x < kOutPad) {
      float s = 0.0f;
      for (int r = 0; r < kTileM; ++r) s += __bfloat162float(sm.dl[r * 24 + threadIdx.x]);
      part[kOffB4 + threadIdx.x] = s;
    }
  }
  // dh3 = dl W4, dz3 = dh3 * (h3 > 0)
  {
    float acc[1][16][4];
    zero_acc(acc);
    warp_gemm<1, 16, false, true>(acc, sm.dl, 24, m0, sm.w4, kLds, 0, kOutPad);
#pragma unroll
    for (int nt = 0; nt < 16; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int rr, cc;
        acc_pos(q, rr, cc);
        const int idx = (m0 + rr) * kLds + 8 * nt + cc;
        const bool on = __bfloat162float(sm.h3[idx]) > 0.0f;
        sm.d[idx] = __float2bfloat16_rn(on ? acc[0][nt][q] : 0.0f);
      }
  }
  __syncthreads();
  // two hidden layers: (d = dz of layer L, h_in = input of layer L, W_L)
  const __nv_bfloat16 *h_in[2] = {sm.h2, sm.h1};
  const __nv_bfloat16 *w_l[2] = {sm.w3, sm.w2};
  const int off_w[2] = {kOffW3, kOffW2}, off_b[2] = {kOffB3, kOffB2};
#pragma unroll
  for (int layer = 0; layer < 2; ++layer) {
    // dW = d^T h_in (128 x 128, reduction over the tile's rows), two column halves
    for (int half = 0; half < 2; ++half) {
      float acc[2][8][4];
      zero_acc(acc);
      warp_gemm<2, 8, true, true>(acc, sm.d, kLds, 32 * warp, h_in[layer], kLds, 64 * half, kTileM);
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            int rr, cc;
            acc_pos(q, rr, cc);
            part[off_w[layer] + (32 * warp + 16 * mt + rr) * kHid + 64 * half + 8 * nt + cc] = acc[mt][nt][q];
          }
    }
    {
      float s = 0.0f;
      for (int r = 0; r < kTileM; ++r) s += __bfloat162float(sm.d[r * kLds + threadIdx.x]);
      part[off_b[layer] + threadIdx.x] = s;
    }
    __syncthreads();  // every warp has read all rows of d
    // dh_in = d W, dz_in = dh_in * (h_in > 0): each warp rewrites its own rows of d
    {
      float acc[1][16][4];
      zero_acc(acc);
      warp_gemm<1, 16, false, true>(acc, sm.d, kLds, m0, w_l[layer], kLds, 0, kHid);
      __syncwarp();
#pragma unroll
      for (int nt = 0; nt < 16; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          int rr, cc;
          acc_pos(q, rr, cc);
          const int idx = (m0 + rr) * kLds + 8 * nt + cc;
          const bool on = __bfloat162float(h_in[layer][idx]) > 0.0f;
          sm.d[idx] = __float2bfloat16_rn(on ? acc[0][nt][q] : 0.0f);
        }
    }
    __syncthreads();
  }
  // layer 1 on the CUDA cores: dW1[j][c] = sum_r dz1[r][j] x[r][c], db1[j] = sum_r dz1[r][j]
  {
    const int j = threadIdx.x;
    float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, gb = 0.0f;
    for (int r = 0; r < kTileM; ++r) {
      const float dz = __bfloat162float(sm.d[r * kLds + j]);
      g0 = fmaf(dz, sm.x[r][0], g0);
      g1 = fmaf(dz, sm.x[r][1], g1);
      g2 = fmaf(dz, sm.x[r][2], g2);
      gb += dz;
    }
    part[kOffW1 + 3 * j + 0] = g0;
    part[kOffW1 + 3 * j + 1] = g1;
    part[kOffW1 + 3 * j + 2] = g2;
    part[kOffB1 + j] = gb;
  }
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int r = 0; r < kTileM; ++r) s += sm.loss[r];
    a.loss_part[tile] = s;
  }
}

// Sum of the tile gradients (tile order) and one Adam step; refreshes the BF16 copies.
__global__ void k_mlp_adam(MlpAdamArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0 && a.loss_acc) {
    double s = 0.0;
    for (int t = 0; t < a.n_tiles; ++t) s += (double)a.loss_part[t];
    *a.loss_acc += s;
  }
  if (p >= kNParams) return;
  float g = 0.0f;
  for (int t = 0; t < a.n_tiles; ++t) g += a.partial[(size_t)t * kNParams + p];
  if (a.grad_out) a.grad_out[p] = g;
  if (a.lr == 0.0f) return;  // gradient only
  float m = a.m[p], v = a.v[p];
  m = a.beta1 * m + (1.0f - a.beta1) * g;
  v = a.beta2 * v + (1.0f - a.beta2) * g * g;
  a.m[p] = m;
  a.v[p] = v;
  const float mh = m * a.c1, vh = v * a.c2;
  const float w = a.params[p] - a.lr * mh / (sqrtf(vh) + a.eps);
  a.params[p] = w;
  bf16_store_weight(a.wbf, p, w);
}

// BF16 copies of W2 / W3 / W4 from the FP32 parameters.
__global__ void k_mlp_to_bf16(const float *params, __nv_bfloat16 *wbf) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < kHid * kHid) {
    bf16_store_weight(wbf, kOffW2 + e, params[kOffW2 + e]);
    bf16_store_weight(wbf, kOffW3 + e, params[kOffW3 + e]);
  }
  if (e < kOutPad * kHid) bf16_store_weight(wbf, kOffW4 + e, params[kOffW4 + e]);
}

// Class probabilities of n rows on the 5th-generation tensor cores
// (gg_mlp_tc.cuh): each warpgroup of a CTA takes tiles of 128 rows in turn.
__global__ void __launch_bounds__(kTcThreads, 1)
    k_mlp_predict(MlpTrainArgs a, float *out, uint64_t n, unsigned int *status) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  TcNetSmem &sm = *reinterpret_cast<TcNetSmem *>(tc_smem_raw);
  const bool ready = tc_net_prepare(sm, a.params, a.wbf + kTcBf);
  const int g = threadIdx.x >> 7, r = threadIdx.x & 127;
  uint32_t phase = 0;
  const uint64_t n_tiles = (n + kTcRows - 1) / kTcRows;
  if (!ready && threadIdx.x == 0) atomicOr(status, kStatusWaitTimeout);
  for (uint64_t t = (uint64_t)blockIdx.x * kTcGroups + g; ready && t < n_tiles;
       t += (uint64_t)gridDim.x * kTcGroups) {
    const uint64_t row = t * kTcRows + r;
    const float4 v = row < n ? a.rows[row] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float x0 = (v.y - a.mean[0]) * a.inv_std[0];
    const float x1 = (v.z - a.mean[1]) * a.inv_std[1];
    const float x2 = (v.x - a.mean[2]) * a.inv_std[2];
    float p[16];
    if (!tc_net_forward(sm, g, r, phase, x0, x1, x2, p)) {
      if (r == 0) atomicOr(status, kStatusWaitTimeout);
      break;
    }
    tc_softmax(p, a.n_classes);
    if (row < n) {
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (c < a.n_classes) out[row * a.n_classes + c] = p[c];
    }
  }
  tc_net_teardown(sm);
}

size_t mlp_smem_bytes() { return sizeof(MlpSmem); }

cudaError_t launch_mlp_train(const MlpTrainArgs &a, int n_tiles, cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(MlpSmem));
    if (e != cudaSuccess) return e;
    configured = true;
  }
  k_mlp_train<<<n_tiles, kMlpThreads, sizeof(MlpSmem), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(const MlpAdamArgs &a, cudaStream_t st) {
  k_mlp_adam<<<(kNParams + 255) / 256, 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mlp_to_bf16(const float *params, __nv_bfloat16 *wbf, cudaStream_t st) {
  k_mlp_to_bf16<<<(kHid * kHid + 255) / 256, 256, 0, st>>>(params, wbf);
  return cudaGetLastError();
}

size_t mlp_tc_smem_bytes() { return sizeof(TcNetSmem); }

cudaError_t launch_mlp_predict(const MlpTrainArgs &a, float *out, uint64_t n, int grid, unsigned int *status,
                               cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(TcNetSmem));
    if (e != cudaSuccess) return e;
    configured = true;
  }
  k_mlp_predict<<<grid, kTcThreads, sizeof(TcNetSmem), st>>>(a, out, n, status);
  return cudaGetLastError();
}

}  // namespace gg
