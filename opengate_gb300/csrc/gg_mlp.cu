// gg_mlp.cu - optimiser step and batch inference of the ARF network.
//
// One training step over a batch of B rows (B a multiple of kTrainRows):
//   k_mlp_train (gg_mlp_train.cu): one CTA per tile of 128 rows on the
//     5th-generation tensor cores - forward, softmax cross-entropy, backward;
//     each CTA writes its tile's parameter gradient (FP32, all kNParams) and
//     loss sum;
//   k_mlp_adam: one thread per parameter - the tile gradients summed in tile
//     order (deterministic), Adam update of the FP32 parameters, and the BF16
//     copies of W2 / W3 / W4 (row-major, tensor-core operands, transposed
//     operands) refreshed for the next step.
// Batch inference (k_mlp_predict) runs the forward pass on tcgen05 (gg_mlp_tc.cuh).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gg_internal.h"
#include "gg_mlp.cuh"
#include "gg_mlp_tc.cuh"

namespace gg {

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
  static unsigned long long configured = 0;
  cudaError_t e = configure_smem(k_mlp_predict, (int)sizeof(TcNetSmem), configured);
  if (e != cudaSuccess) return e;
  k_mlp_predict<<<grid, kTcThreads, sizeof(TcNetSmem), st>>>(a, out, n, status);
  return cudaGetLastError();
}

}  // namespace gg
