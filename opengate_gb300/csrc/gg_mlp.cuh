// gg_mlp.cuh - the ARF network: parameter layout and BF16 weight copies.
//
// Network (restating the garf ARF model used by the reference's ARFActor,
// opengate/actors/arfactors.py:349-415): input x = (theta deg, phi deg, E MeV)
// standardised with the training-set mean / std, three hidden layers of 128
// ReLU units, a linear output of n_classes logits (class 0 = no energy
// window, class k = window k) and a softmax.
//
// Parameters are one FP32 array (offsets below).  Layers 2-4 run on the
// 5th-generation tensor cores (gg_mlp_tc.cuh, gg_mlp_train.cu) from BF16
// copies of their weights with FP32 accumulation; layer 1 (3 inputs) runs on
// the CUDA cores in FP32.  Activations between layers are stored as BF16.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace gg {

constexpr int kHid = 128;     // hidden units
constexpr int kOutPad = 16;   // output logits padded to one n16 tile pair

// FP32 parameter layout
constexpr int kOffW1 = 0;                        // [128][3]
constexpr int kOffB1 = kOffW1 + kHid * 3;        // [128]
constexpr int kOffW2 = kOffB1 + kHid;            // [128][128] (out, in)
constexpr int kOffB2 = kOffW2 + kHid * kHid;     // [128]
constexpr int kOffW3 = kOffB2 + kHid;            // [128][128]
constexpr int kOffB3 = kOffW3 + kHid * kHid;     // [128]
constexpr int kOffW4 = kOffB3 + kHid;            // [16][128] (rows >= n_classes stay 0)
constexpr int kOffB4 = kOffW4 + kOutPad * kHid;  // [16]
constexpr int kNParams = kOffB4 + kOutPad;       // 35600

// BF16 weight copies used by the tensor cores: W2, W3, W4 back to back,
// row-major [out][in] (the training kernel's ldmatrix operands), then the same
// three matrices again as 5th-generation tensor-core operands (K-major core
// matrices, gg_tc.cuh) starting at element kTcBf, so that one bulk copy per
// matrix stages them in shared memory
constexpr int kBfW2 = 0;
constexpr int kBfW3 = kHid * kHid;
constexpr int kBfW4 = 2 * kHid * kHid;
constexpr int kNBf = 2 * kHid * kHid + kOutPad * kHid;
constexpr int kTcBf = kNBf;
// ... and transposed, W^T[in][out] (K = out; W4^T is 128 x 16), the B operands
// of the backward pass dH = dZ W, starting at element kTcTBf
constexpr int kTcTBf = 2 * kNBf;
constexpr int kNBfAll = 3 * kNBf;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Element offset of (n, k) in a K-major core-matrix operand with kk columns:
// the byte offset of the layout (gg_tc.cuh) / 2.
__host__ __device__ constexpr int tc_elem_k(int n, int k, int kk) {
  return (n >> 3) * (kk / 8) * 64 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7);
}
__host__ __device__ constexpr int tc_elem(int n, int k) { return tc_elem_k(n, k, kHid); }

// Stores parameter p (a weight of W2, W3 or W4, value w) as BF16 in both copies.
__device__ __forceinline__ void bf16_store_weight(__nv_bfloat16 *wbf, int p, float w) {
  const __nv_bfloat16 b = __float2bfloat16_rn(w);
  int base, tc, q;
  if (p >= kOffW2 && p < kOffB2) base = kBfW2, tc = kTcBf + kBfW2, q = p - kOffW2;
  else if (p >= kOffW3 && p < kOffB3) base = kBfW3, tc = kTcBf + kBfW3, q = p - kOffW3;
  else if (p >= kOffW4 && p < kOffB4) base = kBfW4, tc = kTcBf + kBfW4, q = p - kOffW4;
  else return;
  const int o = q / kHid, i = q % kHid;
  wbf[base + q] = b;
  wbf[tc + tc_elem(o, i)] = b;
  // transposed: W^T[i][o], K = out units (128, or 16 for W4)
  const int kk = base == kBfW4 ? kOutPad : kHid;
  wbf[tc - kTcBf + kTcTBf + tc_elem_k(i, o, kk)] = b;
}

}  // namespace gg
