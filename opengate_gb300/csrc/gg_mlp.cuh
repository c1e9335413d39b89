// gg_mlp.cuh - the ARF network on the tensor cores (device side).
//
// Network (restating the garf ARF model used by the reference's ARFActor,
// opengate/actors/arfactors.py:349-415): input x = (theta deg, phi deg, E MeV)
// standardised with the training-set mean / std, three hidden layers of 128
// ReLU units, a linear output of n_classes logits (class 0 = no energy
// window, class k = window k) and a softmax.
//
// Parameters are one FP32 array (offsets below).  Layers 2-4 run on the
// tensor cores from BF16 copies of their weights with FP32 accumulation
// (mma.sync m16n8k16, operands from padded shared memory by ldmatrix);
// layer 1 (3 inputs) runs on the CUDA cores in FP32.  Activations between
// layers are stored as BF16.  One CTA works on a tile of kTileM samples; each
// of its 4 warps owns 16 rows of the tile.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace gg {

constexpr int kHid = 128;     // hidden units
constexpr int kOutPad = 16;   // output logits padded to one n16 tile pair
constexpr int kTileM = 64;    // samples per CTA tile
constexpr int kLds = 136;     // shared-memory row stride in BF16 elements (272 B: ldmatrix without bank conflicts)
constexpr int kMlpThreads = 128;

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
constexpr int kNBfAll = 2 * kNBf;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Element offset of W(n, k) (n < rows, k < kHid) in the tensor-core copy of a
// matrix: the byte offset of the K-major core-matrix layout / 2.
__host__ __device__ constexpr int tc_elem(int n, int k) {
  return (n >> 3) * (kHid / 8) * 64 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7);
}

// Stores parameter p (a weight of W2, W3 or W4, value w) as BF16 in both copies.
__device__ __forceinline__ void bf16_store_weight(__nv_bfloat16 *wbf, int p, float w) {
  const __nv_bfloat16 b = __float2bfloat16_rn(w);
  int base, tc, q;
  if (p >= kOffW2 && p < kOffB2) base = kBfW2, tc = kTcBf + kBfW2, q = p - kOffW2;
  else if (p >= kOffW3 && p < kOffB3) base = kBfW3, tc = kTcBf + kBfW3, q = p - kOffW3;
  else if (p >= kOffW4 && p < kOffB4) base = kBfW4, tc = kTcBf + kBfW4, q = p - kOffW4;
  else return;
  wbf[base + q] = b;
  wbf[tc + tc_elem(q / kHid, q % kHid)] = b;
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc[mt][nt] (16 x 8 tiles) += A[m0 + 16 mt .., k] * B[k, n0 + 8 nt ..] for k in [0, K).
// A_KM: A is stored [k][m] (else [m][k]); B_KN: B is stored [k][n] (else [n][k]).
// Row strides lda / ldb in elements; every address stays inside the stored
// [M or K][lda] / [N or K][ldb] blocks the caller passes.
template <int MT, int NT, bool A_KM, bool B_KN>
__device__ __forceinline__ void warp_gemm(float (&acc)[MT][NT][4], const __nv_bfloat16 *A, int lda, int m0,
                                          const __nv_bfloat16 *B, int ldb, int n0, int K) {
  static_assert(NT % 2 == 0, "n tiles in pairs");
  const int lane = threadIdx.x & 31, i = lane >> 3, r = lane & 7;
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
      if (!A_KM) ldsm_x4(a[mt], A + (size_t)(m0 + 16 * mt + (lane & 15)) * lda + k0 + (lane >> 4) * 8);
      else ldsm_x4_t(a[mt], A + (size_t)(k0 + r + (i >> 1) * 8) * lda + m0 + 16 * mt + (i & 1) * 8);
    }
#pragma unroll
    for (int nt = 0; nt < NT; nt += 2) {
      uint32_t b[4];
      if (!B_KN) ldsm_x4(b, B + (size_t)(n0 + 8 * nt + r + (i >> 1) * 8) * ldb + k0 + (i & 1) * 8);
      else ldsm_x4_t(b, B + (size_t)(k0 + r + (i & 1) * 8) * ldb + n0 + 8 * nt + (i >> 1) * 8);
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        mma_bf16(acc[mt][nt], a[mt], b[0], b[1]);
        mma_bf16(acc[mt][nt + 1], a[mt], b[2], b[3]);
      }
    }
  }
}

template <int MT, int NT>
__device__ __forceinline__ void zero_acc(float (&acc)[MT][NT][4]) {
#pragma unroll
  for (int mt = 0; mt < MT; ++mt)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[mt][nt][q] = 0.0f;
}

// Position of accumulator element q of tile (mt, nt): row m0 + 16 mt + rr, column n0 + 8 nt + cc.
__device__ __forceinline__ void acc_pos(int q, int &rr, int &cc) {
  const int lane = threadIdx.x & 31;
  rr = (lane >> 2) + ((q >> 1) << 3);
  cc = ((lane & 3) << 1) + (q & 1);
}

// Shared-memory plan of the MLP kernels (BF16 unless noted).
struct MlpSmem {
  __nv_bfloat16 w2[kHid * kLds], w3[kHid * kLds], w4[kOutPad * kLds];
  __nv_bfloat16 h1[kTileM * kLds], h2[kTileM * kLds], h3[kTileM * kLds];
  __nv_bfloat16 d[kTileM * kLds];    // back-propagated gradient of the current layer
  __nv_bfloat16 dl[kTileM * 24];     // output gradient (16 used, stride 24)
  float w1[kHid * 3], b1[kHid], b2[kHid], b3[kHid], b4[kOutPad];
  float x[kTileM][3];
  float xn_mean[3], xn_inv_std[3];
  int y[kTileM];
  float loss[kTileM];
};

// Weights of the tile kernels into shared memory (BF16 copies + FP32 layer 1 and biases).
__device__ __forceinline__ void mlp_load_weights(MlpSmem &sm, const float *params, const __nv_bfloat16 *wbf) {
  for (int e = threadIdx.x; e < kHid * kHid; e += blockDim.x) {
    const int row = e / kHid, col = e % kHid;
    sm.w2[row * kLds + col] = wbf[kBfW2 + e];
    sm.w3[row * kLds + col] = wbf[kBfW3 + e];
  }
  for (int e = threadIdx.x; e < kOutPad * kHid; e += blockDim.x) {
    const int row = e / kHid, col = e % kHid;
    sm.w4[row * kLds + col] = wbf[kBfW4 + e];
  }
  for (int e = threadIdx.x; e < kHid * 3; e += blockDim.x) sm.w1[e] = params[kOffW1 + e];
  for (int e = threadIdx.x; e < kHid; e += blockDim.x) {
    sm.b1[e] = params[kOffB1 + e];
    sm.b2[e] = params[kOffB2 + e];
    sm.b3[e] = params[kOffB3 + e];
  }
  for (int e = threadIdx.x; e < kOutPad; e += blockDim.x) sm.b4[e] = params[kOffB4 + e];
}

// Layer 1 on the CUDA cores: h1 = bf16(relu(W1 x + b1)) for the tile's rows.
__device__ __forceinline__ void mlp_layer1(MlpSmem &sm) {
  for (int e = threadIdx.x; e < kTileM * kHid; e += blockDim.x) {
    const int srow = e / kHid, j = e % kHid;
    float z = sm.b1[j];
    z = fmaf(sm.w1[3 * j + 0], sm.x[srow][0], z);
    z = fmaf(sm.w1[3 * j + 1], sm.x[srow][1], z);
    z = fmaf(sm.w1[3 * j + 2], sm.x[srow][2], z);
    sm.h1[srow * kLds + j] = __float2bfloat16_rn(z > 0.0f ? z : 0.0f);
  }
}

// Hidden layer on the tensor cores: out = bf16(relu(in W^T + b)) for the warp's 16 rows.
__device__ __forceinline__ void mlp_hidden(const __nv_bfloat16 *in, const __nv_bfloat16 *w, const float *b,
                                           __nv_bfloat16 *out) {
  const int m0 = 16 * (threadIdx.x >> 5);
  float acc[1][16][4];
  zero_acc(acc);
  warp_gemm<1, 16, false, false>(acc, in, kLds, m0, w, kLds, 0, kHid);
#pragma unroll
  for (int nt = 0; nt < 16; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int rr, cc;
      acc_pos(q, rr, cc);
      const int col = 8 * nt + cc;
      const float z = acc[0][nt][q] + b[col];
      out[(m0 + rr) * kLds + col] = __float2bfloat16_rn(z > 0.0f ? z : 0.0f);
    }
}

// Output layer and softmax for the warp's 16 rows: p[r][c] (c < n_classes)
// in the accumulator layout; returns the logits tile in acc.
__device__ __forceinline__ void mlp_logits(const MlpSmem &sm, float (&acc)[1][2][4]) {
  const int m0 = 16 * (threadIdx.x >> 5);
  zero_acc(acc);
  warp_gemm<1, 2, false, false>(acc, sm.h3, kLds, m0, sm.w4, kLds, 0, kHid);
#pragma unroll
  for (int nt = 0; nt < 2; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int rr, cc;
      acc_pos(q, rr, cc);
      acc[0][nt][q] += sm.b4[8 * nt + cc];
    }
}

// Softmax over the first n_classes columns of each row of the logits tile
// (the 4 lanes of a quad hold one row's 16 columns); in place.
__device__ __forceinline__ void mlp_softmax(float (&acc)[1][2][4], int n_classes) {
#pragma unroll
  for (int half = 0; half < 2; ++half) {  // rows rr (q = 0, 1) and rr + 8 (q = 2, 3)
    float mx = -INFINITY;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 2 * half; q < 2 * half + 2; ++q) {
        int rr, cc;
        acc_pos(q, rr, cc);
        if (8 * nt + cc < n_classes) mx = fmaxf(mx, acc[0][nt][q]);
      }
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
    float sum = 0.0f;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 2 * half; q < 2 * half + 2; ++q) {
        int rr, cc;
        acc_pos(q, rr, cc);
        const float ev = 8 * nt + cc < n_classes ? expf(acc[0][nt][q] - mx) : 0.0f;
        acc[0][nt][q] = ev;
        sum += ev;
      }
    sum += __shfl_xor_sync(0xffffffffu, sum, 1);
    sum += __shfl_xor_sync(0xffffffffu, sum, 2);
    const float inv = 1.0f / sum;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 2 * half; q < 2 * half + 2; ++q) acc[0][nt][q] *= inv;
  }
}

}  // namespace gg
